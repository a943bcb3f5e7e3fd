// Gate engine: direct sweep kernels, the fused tile kernel and the planner
// that turns a gate list into full-state passes.
//
// Reference semantics: every gate is quantumflow/backend/numpybk.py:159-214
// tensormul -- contract the gate's bra axes with the state axes `indices`
// and write the ket axes back in place -- applied in list order as
// quantumflow/circuits.py:87-99 Circuit.run does.  Nothing here is a
// translation of that einsum: the state is swept once per fused block.
#include "engine.cuh"
#include "regops.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace qf {

__device__ int g_qf_device_error = 0;

thread_local int t_last_cuda_error = 0;

int check_cuda(cudaError_t e) {
  if (e != cudaSuccess) {
    t_last_cuda_error = static_cast<int>(e);
    return QF_ERR_CUDA;
  }
  return QF_OK;
}

int read_clear_device_error(int* flags, cudaStream_t stream) {
  int rc = check_cuda(cudaMemcpyFromSymbolAsync(flags, g_qf_device_error, sizeof(int), 0,
                                                cudaMemcpyDeviceToHost, stream));
  if (rc) return rc;
  rc = check_cuda(cudaStreamSynchronize(stream));
  if (rc) return rc;
  static const int zero = 0;
  rc = check_cuda(cudaMemcpyToSymbolAsync(g_qf_device_error, &zero, sizeof(int), 0,
                                          cudaMemcpyHostToDevice, stream));
  if (rc) return rc;
  return check_cuda(cudaStreamSynchronize(stream));
}

// Device address of the error word, for kernels in other translation units.
int* device_error_word() {
  static int* addr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_qf_device_error) != cudaSuccess) return nullptr;
    addr[dev] = static_cast<int*>(p);
  }
  return addr[dev];
}

int device_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int v = cache[dev].load();
  if (v == 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
    cache[dev].store(v);
  }
  return v;
}

QF_D int ins0(int v, int b) { return ((v >> b) << (b + 1)) | (v & ((1 << b) - 1)); }

struct CoefArr4 {
  Coef c[4];
};
struct CoefArr16 {
  Coef c[16];
};

// ============================================================ direct sweeps
// 1-qubit dense gate on bit b (any b): each thread owns pairs (i0, i0|2^b),
// two pairs per iteration so four 16-byte loads are in flight per thread.
template <int LAY>
__global__ void __launch_bounds__(256) k_dense1(const typename Types<LAY>::E* in,
                                                typename Types<LAY>::E* out, int64_t npairs, int b,
                                                const __grid_constant__ CoefArr4 u) {
  using E = typename Types<LAY>::E;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int64_t bit = int64_t(1) << b;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < npairs; t += 2 * nthr) {
    const int64_t t2 = t + nthr;
    const bool has2 = t2 < npairs;
    const int64_t i0 = insert0(t, b);
    const int64_t j0 = has2 ? insert0(t2, b) : i0;
    E a[2], c[2];
    a[0] = in[i0];
    a[1] = in[i0 | bit];
    if (has2) {
      c[0] = in[j0];
      c[1] = in[j0 | bit];
    }
    out[i0] = cdot<2>(&u.c[0], a);
    out[i0 | bit] = cdot<2>(&u.c[2], a);
    if (has2) {
      out[j0] = cdot<2>(&u.c[0], c);
      out[j0 | bit] = cdot<2>(&u.c[2], c);
    }
  }
}

// 1-qubit dense gate on a low bit b < 5: fully coalesced one-amplitude-per-
// thread loads, partner amplitude fetched with a warp shuffle.
// Requires namps and the thread count to be multiples of 32.
template <int LAY>
__global__ void __launch_bounds__(256) k_dense1_low(const typename Types<LAY>::E* in,
                                                    typename Types<LAY>::E* out, int64_t namps, int b,
                                                    const __grid_constant__ CoefArr4 u) {
  using E = typename Types<LAY>::E;
  const int lane = threadIdx.x & 31;
  const int hi = (lane >> b) & 1;
  E* tag = nullptr;
  const E c_self = coef_e(u.c[hi * 3], tag);
  const E c_other = coef_e(u.c[hi ? 2 : 1], tag);
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < namps; i += 2 * nthr) {
    const int64_t i2 = i + nthr;
    const bool has2 = i2 < namps;  // warp-uniform: namps, nthr multiples of 32
    E a = in[i], a2;
    if (has2) a2 = in[i2];
    E p = shfl_xor(a, 1 << b);
    out[i] = cmul_add2(c_self, a, c_other, p);
    if (has2) {
      E p2 = shfl_xor(a2, 1 << b);
      out[i2] = cmul_add2(c_self, a2, c_other, p2);
    }
  }
}

// 2-qubit dense gate on bits q0 (matrix MSB) and q1.  IT: the index type
// (uint32_t for states of at most 2^31 amplitudes, int64_t above).
template <int LAY, typename IT>
__global__ void __launch_bounds__(256) k_dense2(const typename Types<LAY>::E* in,
                                                typename Types<LAY>::E* out, IT nquads, int q0,
                                                int q1, const __grid_constant__ CoefArr16 u, int dense) {
  using E = typename Types<LAY>::E;
  const int lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0;
  const IT b0 = IT(1) << q0, b1 = IT(1) << q1;
  const IT nthr = (IT)gridDim.x * blockDim.x;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < nquads; t += nthr) {
    const IT base = insert0(insert0(t, lo), hi);
    const IT idx[4] = {base, base | b1, base | b0, base | b0 | b1};
    E a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = in[idx[r]];
    if constexpr (LAY == FF) {
      if (dense) {  // every coefficient part nonzero (merged Haar blocks): tree sums
#pragma unroll
        for (int r = 0; r < 4; ++r) out[idx[r]] = ff_cdot4_dense(&u.c[4 * r], a);
        continue;
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) out[idx[r]] = cdot<4>(&u.c[4 * r], a);
  }
}

// Generalised permutation (one nonzero per row) on k <= 3 bits.
struct MonoParams {
  int k;
  int gb[3];     // global bits, matrix MSB first
  int sb[3];     // sorted ascending
  int perm[8];   // output row r takes input row perm[r]
  int unit[8];   // coefficient is exactly 1
  Coef c[8];
};
template <int LAY>
__global__ void __launch_bounds__(256) k_mono(const typename Types<LAY>::E* in,
                                              typename Types<LAY>::E* out, int64_t ngroups,
                                              const __grid_constant__ MonoParams m) {
  using E = typename Types<LAY>::E;
  const int G = 1 << m.k;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ngroups; t += nthr) {
    int64_t base = t;
    for (int i = 0; i < m.k; ++i) base = insert0(base, m.sb[i]);
    int64_t idx[8];
    E a[8];
    for (int r = 0; r < G; ++r) {
      int64_t x = base;
      for (int i = 0; i < m.k; ++i)
        if ((r >> (m.k - 1 - i)) & 1) x |= int64_t(1) << m.gb[i];
      idx[r] = x;
      a[r] = in[x];
    }
    for (int r = 0; r < G; ++r) {
      const E v = a[m.perm[r]];
      out[idx[r]] = m.unit[r] ? v : cmul(m.c[r], v);
    }
  }
}

// Element-wise ops (diagonal, sign, cut-phase, scalar) fused in one sweep.
constexpr int ELEM_MAX_OPS = 32;
struct ElemOp {
  int type;
  int k;
  int gb[3];
  int coef;
  int ncoef;
};
struct ElemParams {
  const uint16_t* cuts;
  int nops;
  ElemOp ops[ELEM_MAX_OPS];
  Coef coef[TILE_MAX_COEF / 2];
};

template <typename E>
QF_D E elem_apply(const ElemOp& op, const Coef* coef, const uint16_t* cuts, int64_t x, E v) {
  switch (op.type) {
    case OP_DIAG: {
      int idx = 0;
      for (int i = 0; i < op.k; ++i) idx = (idx << 1) | int((x >> op.gb[i]) & 1);
      return cmul_v(coef[op.coef + idx], v);
    }
    case OP_SIGN: {
      bool all = true;
      for (int i = 0; i < op.k; ++i) all = all && ((x >> op.gb[i]) & 1);
      return all ? cneg(v) : v;
    }
    case OP_CUT: {
      const int c = min((int)cuts[x], op.ncoef - 1);  // a foreign cut table cannot overrun
      return cmul_v(coef[op.coef + c], v);
    }
    case OP_PHASE:
      return cmul(coef[op.coef], v);
    default:
      return v;
  }
}

template <int LAY>
__global__ void __launch_bounds__(256) k_elem(const typename Types<LAY>::E* in,
                                              typename Types<LAY>::E* out, int64_t namps,
                                              const __grid_constant__ ElemParams P) {
  using E = typename Types<LAY>::E;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    E v = in[x];
    for (int o = 0; o < P.nops; ++o) v = elem_apply(P.ops[o], P.coef, P.cuts, x, v);
    out[x] = v;
  }
}

// ============================================================ tile kernel
// A fused block: all its non-elementwise gates act on the tile bits (a low
// run of L contiguous bits plus nh high bits).  Each CTA loops over tiles;
// tiles are staged into shared memory with bulk async copies (one copy per
// contiguous 2^L-amplitude chunk, completion on an mbarrier), double
// buffered so the next tile streams in while this one is processed, and
// written back with bulk async stores.
QF_D int64_t tile_base_of(const TileParams& P, int64_t t) {
  int64_t v = t << P.L;
  for (int r = 0; r < P.nh; ++r) v = insert0(v, P.hb[r]);
  return v;
}
QF_D int64_t chunk_off_of(const TileParams& P, int c) {
  int64_t o = 0;
  for (int r = 0; r < P.nh; ++r)
    if ((c >> r) & 1) o |= int64_t(1) << P.hb[r];
  return o;
}
QF_D int64_t global_of(const TileParams& P, int64_t base, int l) {
  int64_t x = base | (l & ((1 << P.L) - 1));
  for (int r = 0; r < P.nh; ++r)
    if ((l >> (P.L + r)) & 1) x |= int64_t(1) << P.hb[r];
  return x;
}

// One op applied to a tile held in shared memory (all threads of the CTA;
// the caller synchronises afterwards).
template <int LAY>
__device__ void smem_op(const TileParams& P, const TileOp& op, const Coef* cf,
                        typename Types<LAY>::E* s, int64_t base, int tbits) {
  using E = typename Types<LAY>::E;
  const int T = 1 << tbits;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  switch (op.type) {
    case OP_DENSE1: {
      const int q = op.lb[0], bit = 1 << q;
      for (int p = tid; p < (T >> 1); p += nthr) {
        const int i0 = ins0(p, q);
        E a[2] = {s[i0], s[i0 | bit]};
        s[i0] = cdot<2>(cf, a);
        s[i0 | bit] = cdot<2>(cf + 2, a);
      }
      break;
    }
    case OP_DENSE2: {
      const int q0 = op.lb[0], q1 = op.lb[1];
      const int lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0;
      for (int p = tid; p < (T >> 2); p += nthr) {
        const int b = ins0(ins0(p, lo), hi);
        const int idx[4] = {b, b | (1 << q1), b | (1 << q0), b | (1 << q0) | (1 << q1)};
        E a[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = s[idx[r]];
#pragma unroll
        for (int r = 0; r < 4; ++r) s[idx[r]] = cdot<4>(cf + 4 * r, a);
      }
      break;
    }
    case OP_DENSEK: {
      const int k = op.k, G = 1 << k;
      for (int g = warp; g < (T >> k); g += nwarps) {
        int b = g;
        for (int i = 0; i < k; ++i) b = ins0(b, op.slb[i]);
        E acc;
        int mine = b;
        if (lane < G) {
          for (int i = 0; i < k; ++i)
            if ((lane >> (k - 1 - i)) & 1) mine |= 1 << op.lb[i];
          FFAcc ar, ai;  // accumulate in float-float for every layout
          ar.zero();
          ai.zero();
          for (int j = 0; j < G; ++j) {
            int src = b;
            for (int i = 0; i < k; ++i)
              if ((j >> (k - 1 - i)) & 1) src |= 1 << op.lb[i];
            const float4 pf = to_ff(cmul_v(cf[lane * G + j], s[src]));
            ar.add(pf.x, pf.y);
            ai.add(pf.z, pf.w);
          }
          float rh, rl, ih, il;
          ar.finish(rh, rl);
          ai.finish(ih, il);
          if constexpr (LAY == C64) {
            acc = make_float2(rh + rl, ih + il);
          } else if constexpr (LAY == C128) {
            acc = make_double2((double)rh + (double)rl, (double)ih + (double)il);
          } else {
            acc = make_float4(rh, rl, ih, il);
          }
        }
        __syncwarp();
        if (lane < G) s[mine] = acc;
        __syncwarp();
      }
      break;
    }
    case OP_MONO: {
      const int k = op.k, G = 1 << k;
      for (int g = tid; g < (T >> k); g += nthr) {
        int b = g;
        for (int i = 0; i < k; ++i) b = ins0(b, op.slb[i]);
        int idx[8];
        E a[8];
        for (int r = 0; r < G; ++r) {
          int x = b;
          for (int i = 0; i < k; ++i)
            if ((r >> (k - 1 - i)) & 1) x |= 1 << op.lb[i];
          idx[r] = x;
          a[r] = s[x];
        }
        for (int r = 0; r < G; ++r) s[idx[r]] = cmul(cf[r], a[op.perm[r]]);
      }
      break;
    }
    default: {  // element-wise ops
      ElemOp eo;
      eo.type = op.type;
      eo.k = op.k;
      eo.gb[0] = op.gb[0];
      eo.gb[1] = op.gb[1];
      eo.gb[2] = op.gb[2];
      eo.coef = 0;
      eo.ncoef = op.ncoef;
      for (int l = tid; l < T; l += nthr) {
        const int64_t x = global_of(P, base, l);
        s[l] = elem_apply(eo, cf, P.cuts, x, s[l]);
      }
      break;
    }
  }
}

template <int LAY>
__device__ void tile_apply(const TileParams& P, typename Types<LAY>::E* s, int64_t base, int tbits) {
  for (int o = 0; o < P.nops; ++o) {
    const TileOp& op = P.ops[o];
    smem_op<LAY>(P, op, &P.coef[op.coef], s, base, tbits);
    __syncthreads();
  }
}

// ------------------------------------------- register-resident programs ----
template <int RB>
QF_D int reg_local(const TMap& m, int r) {
  int o = 0;
#pragma unroll
  for (int j = 0; j < RB; ++j)
    if ((r >> j) & 1) o |= 1 << m.rpos[j];
  return o;
}
template <int RB>
QF_D int64_t reg_global(const TMap& m, int r) {
  int64_t o = 0;
#pragma unroll
  for (int j = 0; j < RB; ++j)
    if ((r >> j) & 1) o |= int64_t(1) << m.rglob[j];
  return o;
}
QF_D int warp_local(const TMap& m, int warp) {
  return (((warp >> 0) & 1) << m.wpos[0]) | (((warp >> 1) & 1) << m.wpos[1]) |
         (((warp >> 2) & 1) << m.wpos[2]);
}
QF_D int64_t warp_global(const TMap& m, int warp) {
  return (int64_t((warp >> 0) & 1) << m.wglob[0]) | (int64_t((warp >> 1) & 1) << m.wglob[1]) |
         (int64_t((warp >> 2) & 1) << m.wglob[2]);
}

template <int RB, typename E>
QF_D void regs_load(const E* s, const TMap& m, E (&a)[1 << RB], int lane, int warp) {
  const int base = lane | warp_local(m, warp);
#pragma unroll
  for (int r = 0; r < (1 << RB); ++r) a[r] = s[base | reg_local<RB>(m, r)];
}
template <int RB, typename E>
QF_D void regs_store(E* s, const TMap& m, const E (&a)[1 << RB], int lane, int warp) {
  const int base = lane | warp_local(m, warp);
#pragma unroll
  for (int r = 0; r < (1 << RB); ++r) s[base | reg_local<RB>(m, r)] = a[r];
}

template <int RB, typename E>
QF_D void g1_lane(int l, const Coef* cf, E (&a)[1 << RB], int lane) {
  const int hi = (lane >> l) & 1;
  E* tag = nullptr;
  const E cs = coef_e(cf[hi * 3], tag);
  const E co = coef_e(cf[hi ? 2 : 1], tag);
#pragma unroll
  for (int r = 0; r < (1 << RB); ++r) {
    const E p = shfl_xor(a[r], 1 << l);
    a[r] = cmul_add2(cs, a[r], co, p);
  }
}

// element-wise segment: x computed once per amplitude, sign ops folded into
// one parity, phase ops multiplied in order
template <int RB, typename E>
QF_D void seg_apply(const TileParams& P, const TInstr& in, const TMap& m, const Coef* scoef,
                    int64_t xbase, E (&a)[1 << RB]) {
#pragma unroll
  for (int r = 0; r < (1 << RB); ++r) {
    const int64_t x = xbase | reg_global<RB>(m, r);
    E v = a[r];
    bool neg = false;
    for (int o = in.a; o < in.a + in.b; ++o) {
      const SegOp& so = P.segs[o];
      switch (so.type) {
        case OP_SIGN:
          neg ^= ((uint64_t)x & so.mask) == so.mask;
          break;
        case OP_DIAG: {
          int idx = 0;
          for (int i = 0; i < so.k; ++i) idx = (idx << 1) | int((x >> so.gb[i]) & 1);
          v = cmul_v(scoef[so.coef + idx], v);
          break;
        }
        case OP_CUT: {
          const int c = min((int)P.cuts[x], so.ncoef - 1);
          v = cmul_v(scoef[so.coef + c], v);
          break;
        }
        case OP_PHASE:
          v = cmul_v(scoef[so.coef], v);
          break;
      }
    }
    a[r] = neg ? cneg(v) : v;
  }
}

QF_D uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded mbarrier wait on wall-clock time (4 s): on timeout the device
// error word is raised and false returned.
QF_D bool mbar_wait_timed(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023u) == 0 && globaltimer_ns() - t0 > 4000000000ull) {
      atomicOr(&g_qf_device_error, 1);
      return false;
    }
  }
}

template <int LAY>
__global__ void __launch_bounds__(256) k_tile(const __grid_constant__ TileParams P) {
  using E = typename Types<LAY>::E;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  const int tbits = P.L + P.nh;
  const int T = 1 << tbits;
  E* stage[2] = {reinterpret_cast<E*>(smem_raw), reinterpret_cast<E*>(smem_raw) + T};
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t ntiles = int64_t(1) << (P.n - tbits);
  const uint32_t chunk_amps = 1u << P.L;
  const uint32_t chunk_bytes = chunk_amps * (uint32_t)sizeof(E);
  const int nchunks = 1 << P.nh;
  const E* gin = reinterpret_cast<const E*>(P.in);
  E* gout = reinterpret_cast<E*>(P.out);

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue_load = [&](int64_t t, int s) {  // all 32 lanes of warp 0
    if (lane == 0) mbar_arrive_expect_tx(&bars[s], (uint32_t)T * (uint32_t)sizeof(E));
    __syncwarp();
    const int64_t base = tile_base_of(P, t);
    for (int c = lane; c < nchunks; c += 32)
      bulk_g2s(stage[s] + (size_t)c * chunk_amps, gin + base + chunk_off_of(P, c), chunk_bytes, &bars[s]);
  };

  int64_t t = blockIdx.x;
  if (tid < 32 && t < ntiles) issue_load(t, 0);
  uint32_t it = 0;
  for (; t < ntiles; t += gridDim.x, ++it) {
    const int s = it & 1;
    const int64_t nxt = t + gridDim.x;
    if (tid < 32 && nxt < ntiles) {
      bulk_wait_read0();  // stores issued from stage s^1 have read their source
      __syncwarp();
      issue_load(nxt, s ^ 1);
    }
    const bool ok = mbar_wait_timed(&bars[s], (it >> 1) & 1);
    if (__syncthreads_or(!ok)) break;
    const int64_t base = tile_base_of(P, t);
    tile_apply<LAY>(P, stage[s], base, tbits);
    fence_proxy_async_smem();
    __syncthreads();
    if (tid < 32) {
      for (int c = lane; c < nchunks; c += 32)
        bulk_s2g(gout + base + chunk_off_of(P, c), stage[s] + (size_t)c * chunk_amps, chunk_bytes);
      bulk_commit();
    }
  }
  if (tid < 32) bulk_wait0();
}

template <int LAY, int RB>
__global__ void __launch_bounds__(256) k_tile2(const __grid_constant__ TileParams P) {
  using E = typename Types<LAY>::E;
  constexpr int TBITS = RB + 8;
  constexpr int T = 1 << TBITS;
  // three tile buffers: while tile i is processed, tile i+1 streams in and
  // tile i-1 streams out, so the prefetch never waits on a fresh store
  constexpr int NST = 3;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[NST];
  E* stage0 = reinterpret_cast<E*>(smem_raw);
  Coef* scoef = reinterpret_cast<Coef*>(stage0 + NST * T);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t ntiles = int64_t(1) << (P.n - TBITS);
  const uint32_t chunk_amps = 1u << P.L;
  const uint32_t chunk_bytes = chunk_amps * (uint32_t)sizeof(E);
  const int nchunks = 1 << P.nh;
  const E* gin = reinterpret_cast<const E*>(P.in);
  E* gout = reinterpret_cast<E*>(P.out);

  for (int i = tid; i < P.necoef; i += blockDim.x) scoef[i] = P.coef[i];
  if (tid == 0) {
    for (int i = 0; i < NST; ++i) mbar_init(&bars[i], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue_load = [&](int64_t t, int s) {  // all 32 lanes of warp 0
    if (lane == 0) mbar_arrive_expect_tx(&bars[s], (uint32_t)T * (uint32_t)sizeof(E));
    __syncwarp();
    const int64_t base = tile_base_of(P, t);
    E* dst = stage0 + (size_t)s * T;
    for (int c = lane; c < nchunks; c += 32)
      bulk_g2s(dst + (size_t)c * chunk_amps, gin + base + chunk_off_of(P, c), chunk_bytes, &bars[s]);
  };

  E a[1 << RB];
  int64_t t = blockIdx.x;
  if (tid < 32 && t < ntiles) issue_load(t, 0);
  uint32_t it = 0;
  for (; t < ntiles; t += gridDim.x, ++it) {
    const int s = it % NST;
    const int64_t nxt = t + gridDim.x;
    if (tid < 32 && nxt < ntiles) {
      // the next load reuses the buffer of tile it-2: its store (the older
      // of the two pending groups) must have finished reading
      bulk_wait_read1();
      __syncwarp();
      issue_load(nxt, (it + 1) % NST);
    }
    const bool ok = mbar_wait_timed(&bars[s], (it / NST) & 1);
    if (__syncthreads_or(!ok)) break;
    E* st = stage0 + (size_t)s * T;
    const int64_t base = tile_base_of(P, t);
    int map = 0;
    int64_t xbase = 0;
    for (int pc = 0; pc < P.nprog; ++pc) {
      const TInstr in = P.prog[pc];
      switch (in.code) {
        case I_MAP: {
          if (pc > 0) {
            regs_store<RB>(st, P.maps[map], a, lane, warp);
            __syncthreads();
          }
          map = in.a;
          regs_load<RB>(st, P.maps[map], a, lane, warp);
          __syncthreads();
          xbase = base | lane | warp_global(P.maps[map], warp);
          break;
        }
        case I_G1R:
          g1_reg_dispatch<RB>(in.a, &P.coef[in.coef], a);
          break;
        case I_G1L:
          g1_lane<RB>(in.a, &P.coef[in.coef], a, lane);
          break;
        case I_G2R:
          g2_reg_dispatch<RB>(in.a, in.b, &P.coef[in.coef], a);
          break;
        case I_SEG:
          seg_apply<RB>(P, in, P.maps[map], scoef, xbase, a);
          break;
        case I_SMEM: {
          regs_store<RB>(st, P.maps[map], a, lane, warp);
          __syncthreads();
          const TileOp& op = P.ops[in.a];
          smem_op<LAY>(P, op, &P.coef[op.coef], st, base, TBITS);
          __syncthreads();
          regs_load<RB>(st, P.maps[map], a, lane, warp);
          __syncthreads();
          break;
        }
      }
    }
    regs_store<RB>(st, P.maps[map], a, lane, warp);
    fence_proxy_async_smem();
    __syncthreads();
    if (tid < 32) {
      for (int c = lane; c < nchunks; c += 32)
        bulk_s2g(gout + base + chunk_off_of(P, c), st + (size_t)c * chunk_amps, chunk_bytes);
      bulk_commit();
    }
  }
  if (tid < 32) bulk_wait0();
}

// -------------------------------------------------------------- k_warp ----
// Exchange register-index bits J and K: a register permutation (moves only).
template <int RB, int J, int K, typename E>
QF_D void rswap(E (&a)[1 << RB]) {
#pragma unroll
  for (int r = 0; r < (1 << RB); ++r) {
    const int bj = (r >> J) & 1, bk = (r >> K) & 1;
    if (bj == 0 && bk == 1) {
      const int q = r ^ (1 << J) ^ (1 << K);
      const E t = a[r];
      a[r] = a[q];
      a[q] = t;
    }
  }
}
template <int RB, typename E>
QF_D void rswap_dispatch(int j, int k, E (&a)[1 << RB]) {
  switch (j * 4 + k) {
    case 1: rswap<RB, 0, 1>(a); break;
    case 2: if constexpr (RB > 2) rswap<RB, 0, 2>(a); break;
    case 3: if constexpr (RB > 3) rswap<RB, 0, 3>(a); break;
    case 6: if constexpr (RB > 2) rswap<RB, 1, 2>(a); break;
    case 7: if constexpr (RB > 3) rswap<RB, 1, 3>(a); break;
    case 11: if constexpr (RB > 3) rswap<RB, 2, 3>(a); break;
  }
}

// Exchange lane bit l with register-index bit J: the lane whose bit l is h
// keeps its registers with bit J = h and trades the others with its partner.
template <int RB, int J, typename E>
QF_D void lswap(int l, int lane, E (&a)[1 << RB]) {
  const bool hi = (lane >> l) & 1;
#pragma unroll
  for (int i = 0; i < (1 << (RB - 1)); ++i) {
    const int i0 = ((i >> J) << (J + 1)) | (i & ((1 << J) - 1));
    const int i1 = i0 | (1 << J);
    const E x0 = a[i0], x1 = a[i1];
    const E recv = shfl_xor(hi ? x0 : x1, 1 << l);
    a[i0] = hi ? recv : x0;
    a[i1] = hi ? x1 : recv;
  }
}
template <int RB, typename E>
QF_D void lswap_dispatch(int l, int j, int lane, E (&a)[1 << RB]) {
  switch (j) {
    case 0: lswap<RB, 0>(l, lane, a); break;
    case 1: if constexpr (RB > 1) lswap<RB, 1>(l, lane, a); break;
    case 2: if constexpr (RB > 2) lswap<RB, 2>(l, lane, a); break;
    case 3: if constexpr (RB > 3) lswap<RB, 3>(l, lane, a); break;
  }
}

template <int RB, typename E>
QF_D void seg_apply_w(const WarpParams& P, const TInstr& in, const Coef* scoef, int64_t base, int64_t lx, int lane,
                      uint32_t pb, E (&a)[1 << RB]) {
  constexpr int R = 1 << RB;
  // Sign ops (CZ-like) as one parity mask over the registers, from the
  // host's resolution of each op against the sub-tile layout (tile bits
  // tested on the base, lane bits on the lane, register bits as a register
  // mask); all ops of a segment are diagonal and commute, so the signs are
  // applied last.
  uint32_t negmask = 0;
  bool other = false;
  for (int o = in.a; o < in.a + in.b; ++o) {
    const SegOp& so = P.segs[o];
    if (so.type != OP_SIGN) {
      other = true;
      continue;
    }
    if (((uint64_t)base & so.tmask) == so.tmask && ((uint32_t)lane & so.lmask) == so.lmask) negmask ^= so.rmask;
  }
  if (other) {
    // register r holds global index base | lx | hoff[r]
    int64_t hoff[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      int64_t o = 0;
#pragma unroll
      for (int j = 0; j < RB; ++j)
        if ((r >> j) & 1) o |= int64_t(1) << ((pb >> (8 * j)) & 255u);
      hoff[r] = o;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int64_t x = base | lx | hoff[r];
      E v = a[r];
      for (int o = in.a; o < in.a + in.b; ++o) {
        const SegOp& so = P.segs[o];
        switch (so.type) {
          case OP_DIAG: {
            int idx = 0;
            for (int i = 0; i < so.k; ++i) idx = (idx << 1) | int((x >> so.gb[i]) & 1);
            v = cmul_v(scoef[so.coef + idx], v);
            break;
          }
          case OP_CUT: {
            const int c = min((int)P.cuts[x], so.ncoef - 1);
            v = cmul_v(scoef[so.coef + c], v);
            break;
          }
          case OP_PHASE:
            v = cmul_v(scoef[so.coef], v);
            break;
          default:
            break;
        }
      }
      a[r] = v;
    }
  }
  if (negmask != 0) {
#pragma unroll
    for (int r = 0; r < R; ++r)
      if ((negmask >> r) & 1u) a[r] = cneg(a[r]);
  }
}

// SWAP = true: every register-bit gate runs one code variant on the top
// register bit and the host inserts register-bit exchanges (small code,
// for the long float-float gate bodies); SWAP = false: one variant per
// register bit (no exchanges; for the short FP32 bodies).
constexpr int WARP_STAGES = 3;  // per-warp prefetch ring depth (sub-tiles)

template <int LAY, int RB>
constexpr size_t warp_ring_bytes() {
  return (size_t)8 * WARP_STAGES * (32 << RB) * sizeof(typename Types<LAY>::E);
}

template <int LAY, int RB, bool SWAP>
__global__ void __launch_bounds__(256) k_warp(const __grid_constant__ WarpParams P) {
  using E = typename Types<LAY>::E;
  constexpr int R = 1 << RB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Coef* scoef = reinterpret_cast<Coef*>(smem_raw);
  for (int i = threadIdx.x; i < P.necoef; i += blockDim.x) scoef[i] = P.coef[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // this warp's ring of prefetched sub-tiles: [stage][register][lane]
  E* ring = reinterpret_cast<E*>(smem_raw + (((size_t)P.necoef * sizeof(Coef) + 127) & ~size_t(127))) +
            (size_t)warp * WARP_STAGES * R * 32;
  const int64_t nsub = int64_t(1) << (P.n - 5 - RB);
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  const E* gin = reinterpret_cast<const E*>(P.in);
  E* gout = reinterpret_cast<E*>(P.out);
  const uint32_t pb0 = (uint32_t)P.hb[0] | ((uint32_t)P.hb[1] << 8) | ((uint32_t)P.hb[2] << 16) |
                       ((uint32_t)P.hb[3] << 24);
  int64_t hoff0[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int64_t o = 0;
#pragma unroll
    for (int j = 0; j < RB; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << P.hb[j];
    hoff0[r] = o;
  }
  auto sub_base = [&](int64_t st) {
    int64_t base = st << 5;
#pragma unroll
    for (int j = 0; j < RB; ++j) base = insert0(base, P.hb[j]);
    return base;
  };
  auto issue = [&](int64_t st, int sg) {
    if (st < nsub) {
      const int64_t xb = sub_base(st) | lane;
      E* sp = ring + (size_t)sg * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) cp_async_amp(sp + r * 32, gin + (xb | hoff0[r]));
    }
    cp_async_commit();
  };
  int64_t st = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  __syncthreads();  // coefficient table staged
#pragma unroll
  for (int k = 0; k < WARP_STAGES - 1; ++k) issue(st + k * wstride, k);
  int sg = 0;
  for (; st < nsub; st += wstride) {
    cp_async_wait<WARP_STAGES - 2>();
    const int64_t base = sub_base(st);
    // register-index bit j holds global bit (pb >> 8j) & 255, lane bit l
    // global bit (lm >> 8l) & 255; lx = the lane's share of the global index
    uint32_t pb = pb0;
    uint64_t lm = 0x0403020100ull;
    int64_t lx = lane;
    E a[R];
    {
      const E* sp = ring + (size_t)sg * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = sp[r * 32];
    }
    // refill the stage read one iteration ago (its values are in registers)
    issue(st + (WARP_STAGES - 1) * wstride, sg == 0 ? WARP_STAGES - 1 : sg - 1);
    sg = sg + 1 == WARP_STAGES ? 0 : sg + 1;
    for (int pc = 0; pc < P.nprog; ++pc) {
      const TInstr in = P.prog[pc];
      switch (in.code) {
        case I_G1R:
          if constexpr (SWAP) g1_reg<RB, RB - 1>(&P.coef[in.coef], a);
          else g1_reg_dispatch<RB>(in.a, &P.coef[in.coef], a);
          break;
        case I_G1L:
          g1_lane<RB>(in.a, &P.coef[in.coef], a, lane);
          break;
        case I_G2R:
          if constexpr (SWAP) {
            if constexpr (RB >= 2) g2_reg<RB, RB - 1, RB - 2>(&P.coef[in.coef], a, in.c != 0);
          } else {
            g2_reg_dispatch<RB>(in.a, in.b, &P.coef[in.coef], a);
          }
          break;
        case I_RSWAP: {
          rswap_dispatch<RB>(in.a, in.b, a);
          const uint32_t sa = 8u * in.a, sb = 8u * in.b;
          const uint32_t va = (pb >> sa) & 255u, vb = (pb >> sb) & 255u;
          pb = (pb & ~((255u << sa) | (255u << sb))) | (vb << sa) | (va << sb);
          break;
        }
        case I_SEG:
          seg_apply_w<RB>(P, in, scoef, base, lx, lane, pb, a);
          break;
        case I_LSWAP: {
          lswap_dispatch<RB>(in.a, in.b, lane, a);
          const uint32_t sl = 8u * in.a, sj = 8u * in.b;
          const uint32_t gl = (uint32_t)(lm >> sl) & 255u, gj = (pb >> sj) & 255u;
          lm = (lm & ~(uint64_t(255) << sl)) | (uint64_t(gj) << sl);
          pb = (pb & ~(255u << sj)) | (gl << sj);
          lx = (lx & ~(int64_t(1) << gl)) | (int64_t((lane >> in.a) & 1) << gj);
          break;
        }
      }
    }
    // the program ends with every lane and register bit back on its own
    // global bit: the stores reuse the prefetch offsets
#pragma unroll
    for (int r = 0; r < R; ++r) gout[base | lane | hoff0[r]] = a[r];
  }
  cp_async_wait<0>();
}

// ============================================================== host side
// Optional per-launch timing (qf_timing_enable): a CUDA event pair recorded
// on the launch stream around every engine kernel, summed per kernel class
// by qf_timing_collect.
namespace {
std::mutex g_timing_mu;
bool g_timing_on = false;
struct TimedLaunch {
  int kind;
  cudaEvent_t start, stop;
};
std::vector<TimedLaunch> g_timed;
std::vector<cudaEvent_t> g_event_pool;

cudaEvent_t pooled_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

LaunchTimer::LaunchTimer(int k, cudaStream_t stream) {
  std::lock_guard<std::mutex> g(g_timing_mu);
  if (!g_timing_on) return;
  on = true;
  s = stream;
  kind = k;
  start = pooled_event();
  stop = pooled_event();
  cudaEventRecord(start, s);
}
LaunchTimer::~LaunchTimer() {
  if (!on) return;
  cudaEventRecord(stop, s);
  std::lock_guard<std::mutex> g(g_timing_mu);
  g_timed.push_back(TimedLaunch{kind, start, stop});
}

int timing_enable(int on) {
  std::lock_guard<std::mutex> g(g_timing_mu);
  g_timing_on = on != 0;
  return QF_OK;
}

int timing_collect(double* ms, int64_t* counts, int nkinds) {
  std::vector<TimedLaunch> done;
  {
    std::lock_guard<std::mutex> g(g_timing_mu);
    done.swap(g_timed);
  }
  for (int k = 0; k < nkinds; ++k) {
    ms[k] = 0.0;
    counts[k] = 0;
  }
  int rc = QF_OK;
  for (auto& t : done) {
    float e = 0.f;
    if (cudaEventSynchronize(t.stop) != cudaSuccess || cudaEventElapsedTime(&e, t.start, t.stop) != cudaSuccess)
      rc = QF_ERR_CUDA;
    if (t.kind >= 0 && t.kind < nkinds) {
      ms[t.kind] += e;
      counts[t.kind] += 1;
    }
  }
  std::lock_guard<std::mutex> g(g_timing_mu);
  for (auto& t : done) {
    g_event_pool.push_back(t.start);
    g_event_pool.push_back(t.stop);
  }
  return rc;
}

static int grid_for(int64_t items, int per_sm = 16) {
  const int64_t cap = (int64_t)device_sm_count() * per_sm;
  int64_t g = (items + 255) / 256;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return static_cast<int>(g);
}

static bool is_zero(cplx v) { return v.real() == 0.0 && v.imag() == 0.0; }

int classify_op(int k, const int* gbits, const double* mat, HostOp& op) {
  if (k < 1 || k > KMAX_DENSE) return QF_ERR_NOT_SUPPORTED;
  op.k = k;
  for (int i = 0; i < k; ++i) op.gb[i] = gbits[i];
  for (int i = 0; i < k; ++i)
    for (int j = i + 1; j < k; ++j)
      if (gbits[i] == gbits[j]) return QF_ERR_INVALID_ARGUMENT;
  const int G = 1 << k;
  op.m.assign((size_t)G * G, cplx(0, 0));
  for (int i = 0; i < G * G; ++i) op.m[i] = cplx(mat[2 * i], mat[2 * i + 1]);
  // monomial test: exactly one nonzero per row, distinct columns
  bool mono = k <= 3;
  int perm[8] = {0};
  if (mono) {
    unsigned used = 0;
    for (int r = 0; r < G && mono; ++r) {
      int nz = -1, cnt = 0;
      for (int c = 0; c < G; ++c)
        if (!is_zero(op.m[r * G + c])) {
          nz = c;
          ++cnt;
        }
      if (cnt != 1 || (used >> nz) & 1u) mono = false;
      else {
        used |= 1u << nz;
        perm[r] = nz;
      }
    }
  }
  if (mono) {
    bool diag = true;
    for (int r = 0; r < G; ++r) diag = diag && perm[r] == r;
    op.diag.resize(G);
    for (int r = 0; r < G; ++r) {
      op.diag[r] = op.m[r * G + perm[r]];
      op.perm[r] = perm[r];
    }
    if (diag) {
      bool sign = true;  // 1 everywhere except -1 at the all-ones row
      for (int r = 0; r < G; ++r) {
        const cplx want = (r == G - 1) ? cplx(-1, 0) : cplx(1, 0);
        sign = sign && op.diag[r] == want;
      }
      op.type = sign ? OP_SIGN : OP_DIAG;
    } else {
      op.type = OP_MONO;
    }
    return QF_OK;
  }
  op.type = (k == 1) ? OP_DENSE1 : (k == 2) ? OP_DENSE2 : OP_DENSEK;
  return QF_OK;
}

static bool is_elementwise(uint8_t t) {
  return t == OP_DIAG || t == OP_SIGN || t == OP_CUT || t == OP_PHASE;
}

static int coef_count(const HostOp& op) {
  switch (op.type) {
    case OP_DENSE1: return 4;
    case OP_DENSE2: return 16;
    case OP_DENSEK: return 1 << (2 * op.k);
    case OP_MONO: return 1 << op.k;
    case OP_DIAG: return 1 << op.k;
    case OP_SIGN: return 0;
    case OP_CUT: return (int)op.table.size();
    case OP_PHASE: return 1;
  }
  return 0;
}

template <int LAY>
static int launch_elem_t(const void* in, void* out, int n, const std::vector<HostOp>& ops,
                         const std::vector<int>& idx, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  ElemParams P;
  std::memset(&P, 0, sizeof(P));
  P.nops = 0;
  int nc = 0;
  for (int i : idx) {
    const HostOp& op = ops[i];
    if (P.nops >= ELEM_MAX_OPS) return QF_ERR_TOO_LARGE;
    ElemOp& e = P.ops[P.nops++];
    e.type = op.type;
    e.k = op.k;
    for (int j = 0; j < 3; ++j) e.gb[j] = j < op.k ? op.gb[j] : 0;
    e.coef = nc;
    const int need = coef_count(op);
    e.ncoef = need;
    if (nc + need > TILE_MAX_COEF / 2) return QF_ERR_TOO_LARGE;
    if (op.type == OP_DIAG)
      for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.diag[r], LAY);
    if (op.type == OP_CUT) {
      for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.table[r], LAY);
      P.cuts = op.cuts;
    }
    if (op.type == OP_PHASE) P.coef[nc] = make_coef(op.scalar, LAY);
    nc += need;
  }
  const int64_t namps = int64_t(1) << n;
  k_elem<LAY><<<grid_for(namps), 256, 0, stream>>>(reinterpret_cast<const E*>(in),
                                                      reinterpret_cast<E*>(out), namps, P);
  return check_cuda(cudaGetLastError());
}

template <int LAY>
static int launch_single_t(const void* in, void* out, int n, const HostOp& op, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  const E* src = reinterpret_cast<const E*>(in);
  E* dst = reinterpret_cast<E*>(out);
  switch (op.type) {
    case OP_DENSE1: {
      CoefArr4 u;
      for (int i = 0; i < 4; ++i) u.c[i] = make_coef(op.m[i], LAY);
      const int b = op.gb[0];
      if (b < 5 && n >= 5) {
        const int64_t namps = int64_t(1) << n;
        k_dense1_low<LAY><<<grid_for(namps / 2), 256, 0, stream>>>(src, dst, namps, b, u);
      } else {
        const int64_t np = int64_t(1) << (n - 1);
        k_dense1<LAY><<<grid_for(np / 2), 256, 0, stream>>>(src, dst, np, b, u);
      }
      return check_cuda(cudaGetLastError());
    }
    case OP_DENSE2: {
      CoefArr16 u;
      for (int i = 0; i < 16; ++i) u.c[i] = make_coef(op.m[i], LAY);
      const int64_t nq = int64_t(1) << (n - 2);
      int dense = 1;
      for (int i = 0; i < 16; ++i) dense &= (op.m[i].real() != 0.0 && op.m[i].imag() != 0.0) ? 1 : 0;
      if (n <= 31)
        k_dense2<LAY, uint32_t><<<grid_for(nq), 256, 0, stream>>>(src, dst, (uint32_t)nq, op.gb[0], op.gb[1], u,
                                                                  dense);
      else
        k_dense2<LAY, int64_t><<<grid_for(nq), 256, 0, stream>>>(src, dst, nq, op.gb[0], op.gb[1], u, dense);
      return check_cuda(cudaGetLastError());
    }
    case OP_MONO: {
      MonoParams m;
      std::memset(&m, 0, sizeof(m));
      m.k = op.k;
      for (int i = 0; i < op.k; ++i) m.gb[i] = m.sb[i] = op.gb[i];
      std::sort(m.sb, m.sb + op.k);
      for (int r = 0; r < (1 << op.k); ++r) {
        m.perm[r] = op.perm[r];
        m.c[r] = make_coef(op.diag[r], LAY);
        m.unit[r] = op.diag[r] == cplx(1, 0);
      }
      const int64_t ng = int64_t(1) << (n - op.k);
      k_mono<LAY><<<grid_for(ng), 256, 0, stream>>>(src, dst, ng, m);
      return check_cuda(cudaGetLastError());
    }
    default:
      break;
  }
  return QF_ERR_INVALID_ARGUMENT;
}

int launch_single(const void* in, void* out, int n, int layout, const HostOp& op, cudaStream_t stream) {
  switch (layout) {
    case C64: return launch_single_t<C64>(in, out, n, op, stream);
    case C128: return launch_single_t<C128>(in, out, n, op, stream);
    case FF: return launch_single_t<FF>(in, out, n, op, stream);
  }
  return QF_ERR_LAYOUT;
}

static int launch_elem(const void* in, void* out, int n, int layout, const std::vector<HostOp>& ops,
                       const std::vector<int>& idx, cudaStream_t stream) {
  switch (layout) {
    case C64: return launch_elem_t<C64>(in, out, n, ops, idx, stream);
    case C128: return launch_elem_t<C128>(in, out, n, ops, idx, stream);
    case FF: return launch_elem_t<FF>(in, out, n, ops, idx, stream);
  }
  return QF_ERR_LAYOUT;
}

// Tile geometry for a block whose in-tile bits are `hmask`.
static void tile_geometry(int n, int layout, uint64_t hmask, int& L, int& nh, uint8_t hb[8]) {
  const int Lmin = layout == C64 ? 6 : 5;  // 512-byte chunks
  const int TB = layout == C64 ? 12 : 11;  // 32 KiB tiles
  if (n <= TB) {
    L = n;
    nh = 0;
    return;
  }
  L = Lmin;
  for (int iter = 0; iter < 16; ++iter) {
    int cnt = 0;
    for (int b = L; b < n; ++b)
      if ((hmask >> b) & 1) ++cnt;
    int want = std::max(Lmin, TB - cnt);
    want = std::min(want, n - cnt);
    if (want == L) break;
    L = want;
  }
  nh = 0;
  for (int b = L; b < n; ++b)
    if ((hmask >> b) & 1) hb[nh++] = (uint8_t)b;
}

// Compile a fused block into a k_tile2 register program.  Returns false
// when the block does not fit the register scheme (the shared-memory kernel
// k_tile then runs it).
static bool compile_program(TileParams& P, const std::vector<HostOp>& ops, const std::vector<int>& idx,
                            const std::vector<int>& local_bits_flat, int RB) {
  const int tb = P.L + P.nh;
  if (tb != RB + 8) return false;
  auto gpos = [&](int lb) -> int { return lb < P.L ? lb : P.hb[lb - P.L]; };
  const int nop = (int)idx.size();
  std::vector<TInstr> prog;
  std::vector<TMap> maps;
  std::vector<SegOp> segs;
  std::vector<int> regset;  // local bits held in registers (size RB) under the current map
  auto lb_of = [&](int i, int j) { return local_bits_flat[i * KMAX_DENSE + j]; };

  auto lookahead = [&](int from, std::vector<int> must) {
    std::vector<int> set = must;
    auto add = [&](int b) {
      if ((int)set.size() < RB && b >= 5 && std::find(set.begin(), set.end(), b) == set.end()) set.push_back(b);
    };
    for (int i = from; i < nop && (int)set.size() < RB; ++i) {
      const HostOp& op = ops[idx[i]];
      if (op.type == OP_DENSE1) add(lb_of(i, 0));
      if (op.type == OP_DENSE2 && lb_of(i, 0) >= 5 && lb_of(i, 1) >= 5 && (int)set.size() + 2 <= RB) {
        add(lb_of(i, 0));
        add(lb_of(i, 1));
      }
    }
    for (int b = 5; b < tb && (int)set.size() < RB; ++b) add(b);
    return set;
  };
  auto emit_map = [&](const std::vector<int>& set) -> bool {
    if ((int)maps.size() >= TILE_MAX_MAPS) return false;
    TMap m;
    std::memset(&m, 0, sizeof(m));
    int w = 0;
    for (int j = 0; j < RB; ++j) {
      m.rpos[j] = (uint8_t)set[j];
      m.rglob[j] = (uint8_t)gpos(set[j]);
    }
    for (int b = 5; b < tb; ++b)
      if (std::find(set.begin(), set.end(), b) == set.end()) {
        if (w >= 3) return false;
        m.wpos[w] = (uint8_t)b;
        m.wglob[w] = (uint8_t)gpos(b);
        ++w;
      }
    if (w != 3) return false;
    maps.push_back(m);
    TInstr in{I_MAP, (uint8_t)(maps.size() - 1), 0, 0, 0, 0};
    prog.push_back(in);
    regset = set;
    return true;
  };
  auto ensure_map = [&](int from) -> bool {
    if (!regset.empty()) return true;
    return emit_map(lookahead(from, {}));
  };
  auto reg_index = [&](int b) -> int {
    for (int j = 0; j < (int)regset.size(); ++j)
      if (regset[j] == b) return j;
    return -1;
  };
  for (int i = 0; i < nop; ++i) {
    const HostOp& op = ops[idx[i]];
    const TileOp& top = P.ops[i];
    if (is_elementwise(op.type)) {
      if (!ensure_map(i)) return false;
      if ((int)segs.size() >= TILE_MAX_SEGS) return false;
      SegOp so;
      std::memset(&so, 0, sizeof(so));
      so.type = op.type;
      so.k = (uint8_t)op.k;
      for (int j = 0; j < op.k && j < 3; ++j) {
        so.gb[j] = (uint8_t)op.gb[j];
        so.mask |= uint64_t(1) << op.gb[j];
      }
      so.coef = top.coef;
      so.ncoef = top.ncoef;
      segs.push_back(so);
      if (!prog.empty() && prog.back().code == I_SEG && prog.back().a + prog.back().b == (int)segs.size() - 1 &&
          prog.back().b < 255) {
        prog.back().b++;
      } else {
        TInstr in{I_SEG, (uint8_t)(segs.size() - 1), 1, 0, 0, 0};
        prog.push_back(in);
      }
      continue;
    }
    if (op.type == OP_DENSE1) {
      const int q = lb_of(i, 0);
      if (q < 5) {
        if (!ensure_map(i)) return false;
        prog.push_back(TInstr{I_G1L, (uint8_t)q, 0, 0, top.coef, 0});
        continue;
      }
      if (reg_index(q) < 0 && !emit_map(lookahead(i, {q}))) return false;
      prog.push_back(TInstr{I_G1R, (uint8_t)reg_index(q), 0, 0, top.coef, 0});
      continue;
    }
    if (op.type == OP_DENSE2 && lb_of(i, 0) >= 5 && lb_of(i, 1) >= 5) {
      const int q0 = lb_of(i, 0), q1 = lb_of(i, 1);
      if (reg_index(q0) < 0 || reg_index(q1) < 0) {
        if (!emit_map(lookahead(i, {q0, q1}))) return false;
      }
      prog.push_back(TInstr{I_G2R, (uint8_t)reg_index(q0), (uint8_t)reg_index(q1), 0, top.coef, 0});
      continue;
    }
    if (!ensure_map(i)) return false;
    prog.push_back(TInstr{I_SMEM, (uint8_t)i, 0, 0, 0, 0});
  }
  if ((int)prog.size() > TILE_MAX_PROG) return false;
  P.nprog = (int)prog.size();
  std::copy(prog.begin(), prog.end(), P.prog);
  std::copy(maps.begin(), maps.end(), P.maps);
  std::copy(segs.begin(), segs.end(), P.segs);
  return true;
}

template <typename K>
static int set_smem_attr(K kernel, std::atomic<bool>* flags) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !flags[dev].load()) {
    // the opt-in maximum less the kernel's static shared memory
    int optin = 0;
    int rc = check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (rc) return rc;
    cudaFuncAttributes fa;
    rc = check_cuda(cudaFuncGetAttributes(&fa, kernel));
    if (rc) return rc;
    rc = check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         optin - (int)fa.sharedSizeBytes));
    if (rc) return rc;
    flags[dev].store(true);
  }
  return QF_OK;
}

int g_force_smem_tile = 0;    // qf_set_tile_kernel: 1 = shared-memory tile kernels only
int g_warp_rb_override = 0;  // qf_set_tile_kernel: register bits of k_warp (0 = per layout)

template <int LAY>
static int launch_tile_t(const void* in, void* out, int n, const std::vector<HostOp>& ops,
                         const std::vector<int>& idx, uint64_t hmask, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  constexpr int RB = LAY == C64 ? 4 : 3;
  static thread_local TileParams P;  // ~25 KiB: kept off the stack
  std::memset(&P, 0, sizeof(TileParams));
  P.in = in;
  P.out = out;
  P.n = n;
  int L = 0, nh = 0;
  tile_geometry(n, LAY, hmask, L, nh, P.hb);
  if (nh > 8) return QF_ERR_TOO_LARGE;
  P.L = L;
  P.nh = nh;
  auto local_of = [&](int b) -> int {
    if (b < L) return b;
    for (int r = 0; r < nh; ++r)
      if (P.hb[r] == b) return L + r;
    return -1;
  };
  if ((int)idx.size() > TILE_MAX_OPS) return QF_ERR_TOO_LARGE;
  std::vector<int> local_bits(idx.size() * KMAX_DENSE, -1);
  // coefficients: element-wise ops first (k_tile2 stages them in shared
  // memory), then the rest
  int nc = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (size_t i = 0; i < idx.size(); ++i) {
      const HostOp& op = ops[idx[i]];
      if (is_elementwise(op.type) != (pass == 0)) continue;
      TileOp& t = P.ops[i];
      t.type = op.type;
      t.k = (uint8_t)op.k;
      t.coef = (uint16_t)nc;
      t.ncoef = (uint16_t)coef_count(op);
      if (!is_elementwise(op.type)) {
        int sl[KMAX_DENSE];
        for (int j = 0; j < op.k; ++j) {
          const int lb = local_of(op.gb[j]);
          if (lb < 0) return QF_ERR_INVALID_ARGUMENT;
          t.lb[j] = (uint8_t)lb;
          sl[j] = lb;
          local_bits[i * KMAX_DENSE + j] = lb;
        }
        std::sort(sl, sl + op.k);
        for (int j = 0; j < op.k; ++j) t.slb[j] = (uint8_t)sl[j];
      } else {
        for (int j = 0; j < op.k && j < 3; ++j) t.gb[j] = (uint8_t)op.gb[j];
      }
      const int need = coef_count(op);
      if (nc + need > TILE_MAX_COEF) return QF_ERR_TOO_LARGE;
      switch (op.type) {
        case OP_DENSE1:
        case OP_DENSE2:
        case OP_DENSEK:
          for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.m[r], LAY);
          break;
        case OP_MONO:
          for (int r = 0; r < need; ++r) {
            P.coef[nc + r] = make_coef(op.diag[r], LAY);
            t.perm[r] = (uint8_t)op.perm[r];
          }
          break;
        case OP_DIAG:
          for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.diag[r], LAY);
          break;
        case OP_CUT:
          for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.table[r], LAY);
          P.cuts = op.cuts;
          break;
        case OP_PHASE:
          P.coef[nc] = make_coef(op.scalar, LAY);
          break;
        default:
          break;
      }
      nc += need;
    }
    if (pass == 0) P.necoef = nc;
  }
  P.nops = (int)idx.size();
  P.threads = 256;
  const int tbits = L + nh;
  const int64_t ntiles = int64_t(1) << (n - tbits);
  static std::atomic<bool> attr1[64], attr2[64];
  if (!g_force_smem_tile && compile_program(P, ops, idx, local_bits, RB)) {
    const size_t smem = 3 * (size_t(1) << tbits) * sizeof(E) + (size_t)P.necoef * sizeof(Coef);
    if (smem <= 200 * 1024) {
      int rc = set_smem_attr(k_tile2<LAY, RB>, attr2);
      if (rc) return rc;
      int64_t grid = (int64_t)device_sm_count() * 2;
      if (grid > ntiles) grid = ntiles;
      k_tile2<LAY, RB><<<(int)grid, 256, smem, stream>>>(P);
      return check_cuda(cudaGetLastError());
    }
  }
  P.nprog = 0;
  const size_t smem = 2 * (size_t(1) << tbits) * sizeof(E);
  int rc = set_smem_attr(k_tile<LAY>, attr1);
  if (rc) return rc;
  int64_t grid = (int64_t)device_sm_count() * (smem > 80 * 1024 ? 2 : 3);
  if (grid > ntiles) grid = ntiles;
  k_tile<LAY><<<(int)grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

// Compile and launch a block on k_warp.  Returns QF_ERR_NOT_SUPPORTED (and
// launches nothing) when the block does not fit the warp-tile scheme.
template <int LAY, int RB>
static int launch_warp_t(const void* in, void* out, int n, const std::vector<HostOp>& ops,
                         const std::vector<int>& idx, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  constexpr bool SWAP = LAY != C64;
  if (n < 5 + RB) return QF_ERR_NOT_SUPPORTED;
  static thread_local WarpParams P;
  std::memset(&P, 0, sizeof(P));
  P.in = in;
  P.out = out;
  P.n = n;
  P.rb = RB;
  // register bits: the block's high bits, padded with unused bits >= 5
  std::vector<int> hb;
  for (int i : idx) {
    const HostOp& op = ops[i];
    if (is_elementwise(op.type)) continue;
    if (op.type != OP_DENSE1 && op.type != OP_DENSE2) return QF_ERR_NOT_SUPPORTED;
    if (op.type == OP_DENSE2 && RB < 2) return QF_ERR_NOT_SUPPORTED;
    for (int j = 0; j < op.k; ++j)
      if (op.gb[j] >= 5 && std::find(hb.begin(), hb.end(), op.gb[j]) == hb.end()) hb.push_back(op.gb[j]);
  }
  if ((int)hb.size() > RB) return QF_ERR_NOT_SUPPORTED;
  for (int b = 5; b < n && (int)hb.size() < RB; ++b)
    if (std::find(hb.begin(), hb.end(), b) == hb.end()) hb.push_back(b);
  std::sort(hb.begin(), hb.end());
  for (int j = 0; j < RB; ++j) P.hb[j] = (uint8_t)hb[j];
  // where each global bit of the sub-tile lives while the program runs:
  // reg[p] = global bit of register-index bit p, lanes[l] = of lane bit l.
  // Register exchanges (SWAP kernels) bring a gate's bit to the top register
  // bit (a 2-qubit gate's LSB below it); lane exchanges bring a lane bit of
  // a 2-qubit gate into the registers, and the program ends with the lanes
  // restored (coalesced stores).
  int reg[4] = {0, 0, 0, 0}, lanes[5] = {0, 1, 2, 3, 4};
  for (int j = 0; j < RB; ++j) reg[j] = hb[j];
  auto reg_pos = [&](int g) {
    for (int j = 0; j < RB; ++j)
      if (reg[j] == g) return j;
    return -1;
  };
  auto lane_pos = [&](int g) {
    for (int l = 0; l < 5; ++l)
      if (lanes[l] == g) return l;
    return -1;
  };
  // element-wise coefficients first (staged in shared memory), then dense
  int nc = 0, nprog = 0, nseg = 0;
  std::vector<int> coef_at(idx.size(), 0);
  for (int pass = 0; pass < 2; ++pass) {
    for (size_t i = 0; i < idx.size(); ++i) {
      const HostOp& op = ops[idx[i]];
      if (is_elementwise(op.type) != (pass == 0)) continue;
      const int need = coef_count(op);
      if (nc + need > 1152) return QF_ERR_NOT_SUPPORTED;
      coef_at[i] = nc;
      switch (op.type) {
        case OP_DENSE1:
        case OP_DENSE2:
          for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.m[r], LAY);
          break;
        case OP_DIAG:
          for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.diag[r], LAY);
          break;
        case OP_CUT:
          for (int r = 0; r < need; ++r) P.coef[nc + r] = make_coef(op.table[r], LAY);
          P.cuts = op.cuts;
          break;
        case OP_PHASE:
          P.coef[nc] = make_coef(op.scalar, LAY);
          break;
        default:
          break;
      }
      nc += need;
    }
    if (pass == 0) P.necoef = nc;
  }
  bool ok = true;
  auto emit = [&](TInstr t) {
    if (nprog >= 160) {
      ok = false;
      return;
    }
    P.prog[nprog++] = t;
  };
  auto rswap = [&](int j, int target) {  // exchange register-index bits j and target
    if (j == target) return;
    const int lo = j < target ? j : target, hi = j < target ? target : j;
    emit(TInstr{I_RSWAP, (uint8_t)lo, (uint8_t)hi, 0, 0, 0});
    std::swap(reg[j], reg[target]);
  };
  auto lswap = [&](int l, int j) {  // exchange lane bit l with register-index bit j
    emit(TInstr{I_LSWAP, (uint8_t)l, (uint8_t)j, 0, 0, 0});
    std::swap(lanes[l], reg[j]);
  };
  // bring global bit g into the registers, not evicting global bit keep
  auto to_reg = [&](int g, int keep) {
    if (reg_pos(g) >= 0) return;
    const int l = lane_pos(g);
    int j = SWAP ? RB - 1 : 0;
    if (reg[j] == keep) j = SWAP ? RB - 2 : 1;
    lswap(l, j);
  };
  for (size_t i = 0; i < idx.size() && ok; ++i) {
    const HostOp& op = ops[idx[i]];
    if (is_elementwise(op.type)) {
      if (nseg >= 64) return QF_ERR_NOT_SUPPORTED;
      SegOp& so = P.segs[nseg];
      std::memset(&so, 0, sizeof(so));
      so.type = op.type;
      so.k = (uint8_t)op.k;
      for (int j = 0; j < op.k && j < 3; ++j) {
        so.gb[j] = (uint8_t)op.gb[j];
        so.mask |= uint64_t(1) << op.gb[j];
      }
      so.coef = (uint16_t)coef_at[i];
      so.ncoef = (uint16_t)coef_count(op);
      if (op.type == OP_SIGN) {
        // where the op's bits are at this point of the program
        uint32_t jm = 0;
        for (int j = 0; j < op.k; ++j) {
          const int g = op.gb[j], p = reg_pos(g), l = lane_pos(g);
          if (p >= 0) jm |= 1u << p;
          else if (l >= 0) so.lmask |= (uint8_t)(1u << l);
          else so.tmask |= uint64_t(1) << g;
        }
        for (int r = 0; r < (1 << RB); ++r)
          if ((r & jm) == jm) so.rmask |= (uint16_t)(1u << r);
      }
      if (nprog > 0 && P.prog[nprog - 1].code == I_SEG && P.prog[nprog - 1].b < 255 &&
          P.prog[nprog - 1].a + P.prog[nprog - 1].b == nseg) {
        P.prog[nprog - 1].b++;
      } else {
        emit(TInstr{I_SEG, (uint8_t)nseg, 1, 0, 0, 0});
      }
      ++nseg;
    } else if (op.type == OP_DENSE1) {
      const int g = op.gb[0];
      const int l = lane_pos(g);
      if (l >= 0) {
        emit(TInstr{I_G1L, (uint8_t)l, 0, 0, (uint16_t)coef_at[i], 0});
      } else {
        if (SWAP) rswap(reg_pos(g), RB - 1);
        emit(TInstr{I_G1R, (uint8_t)(SWAP ? 0 : reg_pos(g)), 0, 0, (uint16_t)coef_at[i], 0});
      }
    } else {
      const int g0 = op.gb[0], g1 = op.gb[1];
      to_reg(g0, g1);
      to_reg(g1, g0);
      if (SWAP) {
        rswap(reg_pos(g0), RB - 1);
        rswap(reg_pos(g1), RB - 2);
      }
      bool dense = true;
      for (int e = 0; e < 16; ++e) dense = dense && op.m[e].real() != 0.0 && op.m[e].imag() != 0.0;
      emit(TInstr{I_G2R, (uint8_t)(SWAP ? 0 : reg_pos(g0)), (uint8_t)(SWAP ? 0 : reg_pos(g1)),
                  (uint8_t)(dense ? 1 : 0), (uint16_t)coef_at[i], 0});
    }
  }
  // restore the lanes in order; a lane fixed here stays fixed (the bit
  // fetched for lane l is never in a lane < l)
  for (int l = 0; l < 5 && ok; ++l) {
    if (lanes[l] == l) continue;
    if (reg_pos(l) < 0) lswap(lane_pos(l), SWAP ? RB - 1 : 0);
    lswap(l, reg_pos(l));
  }
  // and the register bits (register moves), so that the stores use the
  // offsets of the loads
  for (int j = 0; j < RB && ok; ++j) {
    const int p = reg_pos(hb[j]);
    if (p != j) rswap(p, j);
  }
  if (!ok) return QF_ERR_NOT_SUPPORTED;
  P.nprog = nprog;
  const size_t smem = (((size_t)P.necoef * sizeof(Coef) + 127) & ~size_t(127)) + warp_ring_bytes<LAY, RB>();
  static std::atomic<bool> attr[64];
  int rc = set_smem_attr(k_warp<LAY, RB, SWAP>, attr);
  if (rc) return rc;
  const int64_t nsub = int64_t(1) << (n - 5 - RB);
  int64_t grid = (nsub + 7) / 8;
  const int64_t cap = (int64_t)device_sm_count() * 4;
  if (grid > cap) grid = cap;
  k_warp<LAY, RB, SWAP><<<(int)grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

int warp_rb(int layout) { return layout == C64 ? 4 : 2; }

int launch_warp_block(const void* in, void* out, int n, int layout, const std::vector<HostOp>& ops,
                      const std::vector<int>& idx, int rb, cudaStream_t stream) {
#define QF_WARP_CASE(LAYV)                                                    \
  switch (rb) {                                                               \
    case 2: return launch_warp_t<LAYV, 2>(in, out, n, ops, idx, stream);      \
    case 3: return launch_warp_t<LAYV, 3>(in, out, n, ops, idx, stream);      \
    case 4: return launch_warp_t<LAYV, 4>(in, out, n, ops, idx, stream);      \
  }                                                                           \
  return QF_ERR_NOT_SUPPORTED;
  switch (layout) {
    case C64: { QF_WARP_CASE(C64) }
    case C128: { QF_WARP_CASE(C128) }
    case FF: { QF_WARP_CASE(FF) }
  }
#undef QF_WARP_CASE
  return QF_ERR_LAYOUT;
}

int launch_tile_block(const void* in, void* out, int n, int layout, const std::vector<HostOp>& ops,
                      const std::vector<int>& idx, uint64_t hmask, cudaStream_t stream) {
  switch (layout) {
    case C64: return launch_tile_t<C64>(in, out, n, ops, idx, hmask, stream);
    case C128: return launch_tile_t<C128>(in, out, n, ops, idx, hmask, stream);
    case FF: return launch_tile_t<FF>(in, out, n, ops, idx, hmask, stream);
  }
  return QF_ERR_LAYOUT;
}

// ------------------------------------------------------- gate merging ----
// Consecutive gates are multiplied into blocks of at most two qubits on the
// host (in double precision) before the passes are planned: a 1-qubit gate
// joins the last gate on its qubit when that gate is dense (a product costs
// nothing extra), and a 2-qubit gate absorbs the pending 1-qubit gates on
// its qubits when it is dense or when both qubits have one (a diagonal CZ
// between two dense layers becomes one dense 4x4 instead of two 2x2 gates
// and a sign).  Only gates that commute are reordered: a gate moves past
// another only when they share no qubit.
static bool mergeable(const HostOp& op) {
  switch (op.type) {
    case OP_DENSE1:
    case OP_DENSE2:
      return true;
    case OP_DIAG:
    case OP_SIGN:
    case OP_MONO:
      return op.k <= 2;
  }
  return false;
}

static std::vector<cplx> dense_of(const HostOp& op) {
  const int G = 1 << op.k;
  if ((int)op.m.size() == G * G) return op.m;
  std::vector<cplx> m((size_t)G * G, cplx(0, 0));
  if (op.type == OP_DIAG) {
    for (int r = 0; r < G; ++r) m[r * G + r] = op.diag[r];
  } else if (op.type == OP_SIGN) {
    for (int r = 0; r < G; ++r) m[r * G + r] = r == G - 1 ? cplx(-1, 0) : cplx(1, 0);
  } else if (op.type == OP_MONO) {
    for (int r = 0; r < G; ++r) m[r * G + op.perm[r]] = op.diag[r];
  }
  return m;
}

// the matrix of `op` (k = 1 or 2) acting on the bits `bits` (MSB first, 2 bits)
static std::vector<cplx> embed2(const HostOp& op, const int bits[2]) {
  const std::vector<cplx> m = dense_of(op);
  std::vector<cplx> e(16, cplx(0, 0));
  if (op.k == 1) {
    const bool msb = op.gb[0] == bits[0];
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        const int rs = msb ? r >> 1 : r & 1, cs = msb ? c >> 1 : c & 1;  // acted-on bit
        const int ro = msb ? r & 1 : r >> 1, co = msb ? c & 1 : c >> 1;  // other bit
        if (ro == co) e[r * 4 + c] = m[rs * 2 + cs];
      }
    return e;
  }
  if (op.gb[0] == bits[0]) return m;
  auto sw = [](int v) { return ((v & 1) << 1) | (v >> 1); };  // exchange the two index bits
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) e[r * 4 + c] = m[sw(r) * 4 + sw(c)];
  return e;
}

static std::vector<cplx> matmul_n(const std::vector<cplx>& a, const std::vector<cplx>& b, int G) {
  std::vector<cplx> c((size_t)G * G, cplx(0, 0));
  for (int i = 0; i < G; ++i)
    for (int k = 0; k < G; ++k) {
      const cplx v = a[i * G + k];
      if (v == cplx(0, 0)) continue;
      for (int j = 0; j < G; ++j) c[i * G + j] += v * b[k * G + j];
    }
  return c;
}

// rebuild `op` as the gate with matrix m on bits (k = 1 or 2), re-classified
static void set_matrix(HostOp& op, int k, const int* bits, const std::vector<cplx>& m) {
  std::vector<double> flat(2 * m.size());
  for (size_t i = 0; i < m.size(); ++i) {
    flat[2 * i] = m[i].real();
    flat[2 * i + 1] = m[i].imag();
  }
  HostOp r;
  classify_op(k, bits, flat.data(), r);
  op = r;
}

static bool dense_cost(const HostOp& op) { return op.type == OP_DENSE1 || op.type == OP_DENSE2; }

void merge_ops(std::vector<HostOp>& ops, int n) {
  std::vector<HostOp> out;
  std::vector<char> alive;
  std::vector<int> last(n, -1);
  out.reserve(ops.size());
  for (HostOp& o : ops) {
    if (!mergeable(o)) {
      const int idx = (int)out.size();
      if (o.type == OP_CUT || o.type == OP_PHASE) {
        for (int q = 0; q < n; ++q) last[q] = idx;
      } else {
        for (int j = 0; j < o.k; ++j) last[o.gb[j]] = idx;
      }
      out.push_back(std::move(o));
      alive.push_back(1);
      continue;
    }
    if (o.k == 1) {
      const int q = o.gb[0];
      const int t = last[q];
      if (t >= 0 && alive[t] && mergeable(out[t]) && (dense_cost(out[t]) || out[t].k == 1)) {
        HostOp& d = out[t];
        if (d.k == 1) {
          const int bits[1] = {q};
          set_matrix(d, 1, bits, matmul_n(dense_of(o), dense_of(d), 2));
        } else {
          const int bits[2] = {d.gb[0], d.gb[1]};
          set_matrix(d, 2, bits, matmul_n(embed2(o, bits), dense_of(d), 4));
        }
        continue;
      }
      last[q] = (int)out.size();
      out.push_back(std::move(o));
      alive.push_back(1);
      continue;
    }
    // two qubits
    const int a = o.gb[0], b = o.gb[1];
    const int bits[2] = {a, b};
    const int ta = last[a], tb = last[b];
    if (ta >= 0 && ta == tb && alive[ta] && mergeable(out[ta]) && out[ta].k == 2) {
      HostOp& d = out[ta];
      const int dbits[2] = {d.gb[0], d.gb[1]};
      set_matrix(d, 2, dbits, matmul_n(embed2(o, dbits), dense_of(d), 4));
      continue;
    }
    std::vector<cplx> m = dense_of(o);
    auto pending = [&](int t) {  // a live 1-qubit gate that is the last on its qubit
      return t >= 0 && alive[t] && mergeable(out[t]) && out[t].k == 1;
    };
    const bool pa = pending(ta), pb = pending(tb);
    const bool cheap_a = pa && !dense_cost(out[ta]), cheap_b = pb && !dense_cost(out[tb]);
    const bool take_all = dense_cost(o) || (pa && pb);
    if (pa && (take_all || cheap_a)) {
      m = matmul_n(m, embed2(out[ta], bits), 4);
      alive[ta] = 0;
    }
    if (pb && (take_all || cheap_b)) {
      m = matmul_n(m, embed2(out[tb], bits), 4);
      alive[tb] = 0;
    }
    HostOp r;
    set_matrix(r, 2, bits, m);
    last[a] = last[b] = (int)out.size();
    out.push_back(std::move(r));
    alive.push_back(1);
  }
  ops.clear();
  for (size_t i = 0; i < out.size(); ++i)
    if (alive[i]) ops.push_back(std::move(out[i]));
}

// Greedy fusion: walk the ops in order; element-wise ops join the current
// block unconditionally (they need no tile bits), every other op joins while
// the union of high bits (>= Lmin) stays within fusion_k.
int g_default_fusion[3] = {4, 2, 2};  // per layout (C64, C128, FF): warp-tile capacity
int g_group_kernel = 1;               // qf_set_tile_kernel(5) turns the group kernel off

// Group passes are the default fused kernel for the passes they fit; the
// diagnostic kernel selections (forced shared-memory tiles, warp register
// widths) and tile mode 5 leave them out.
static bool group_pass_enabled() {
  return g_group_kernel && !g_force_smem_tile && g_warp_rb_override == 0;
}
// The interpreted group kernel takes passes of dense gates and signs only
// (those the shape split leaves whole, or all of them when shape passes are
// off); passes with diagonal phases (QFT's CPHASE) stay on warp tiles, which
// ran QFT at N=26 in 87.7 ms against 90.1 ms on the group kernel.
static bool group_pass_fits(const std::vector<HostOp>& ops, const std::vector<int>& idx) {
  for (int i : idx) {
    const uint8_t t = ops[i].type;
    if (t != OP_DENSE1 && t != OP_DENSE2 && t != OP_SIGN) return false;
  }
  return true;
}
int g_merge_gates = 1;                 // qf_set_gate_merging: 0 off, 1 merge, 2 merge + pack passes

// Pass packing (optional, qf_set_gate_merging(2)): after merging, the gates
// are re-ordered (within the freedom of their dependences -- a gate only
// moves past gates on other qubits) so that each pass gathers as many gates
// as its high-bit budget allows: a list scheduler that keeps adding ready
// gates whose high bits fit the current pass (gates that add no new high bit
// first, then the fewest new bits, then program order), and opens a new
// pass when none fits.  Fewer passes, but on the random-layer workload the
// packed warp-tile passes cost more than the lone 4x4 sweeps they replace
// (measured 197 vs 157 ms per 10 layers at N=28), so it is off by default.
static void schedule_ops(std::vector<HostOp>& ops, int n, int fusion_k) {
  const int m = (int)ops.size();
  if (m < 3) return;
  std::vector<std::vector<int>> succ(m);
  std::vector<int> indeg(m, 0);
  std::vector<int> last(n, -1);
  std::vector<uint64_t> hbits(m, 0);
  for (int i = 0; i < m; ++i) {
    const HostOp& op = ops[i];
    std::vector<int> qs;
    if (op.type == OP_CUT || op.type == OP_PHASE) {
      for (int q = 0; q < n; ++q) qs.push_back(q);
    } else {
      for (int j = 0; j < op.k; ++j) qs.push_back(op.gb[j]);
    }
    std::vector<int> preds;
    for (int q : qs) {
      if (last[q] >= 0 && std::find(preds.begin(), preds.end(), last[q]) == preds.end()) preds.push_back(last[q]);
      last[q] = i;
    }
    for (int p : preds) succ[p].push_back(i);
    indeg[i] = (int)preds.size();
    if (!is_elementwise(op.type))
      for (int j = 0; j < op.k; ++j)
        if (op.gb[j] >= 5) hbits[i] |= uint64_t(1) << op.gb[j];
  }
  std::vector<int> ready;
  for (int i = 0; i < m; ++i)
    if (indeg[i] == 0) ready.push_back(i);
  std::vector<int> order;
  order.reserve(m);
  uint64_t cur = 0;
  while (!ready.empty()) {
    int best = -1, best_new = 99;
    for (int k = 0; k < (int)ready.size(); ++k) {
      const int i = ready[k];
      const uint64_t u = cur | hbits[i];
      if (__builtin_popcountll(u) > fusion_k) continue;
      const int nw = __builtin_popcountll(hbits[i] & ~cur);
      if (nw < best_new || (nw == best_new && i < ready[best])) {
        best = k;
        best_new = nw;
      }
    }
    if (best < 0) {  // nothing fits: open a new pass with the earliest ready gate
      cur = 0;
      best = (int)(std::min_element(ready.begin(), ready.end()) - ready.begin());
    }
    const int i = ready[best];
    ready.erase(ready.begin() + best);
    order.push_back(i);
    cur |= hbits[i];
    for (int s2 : succ[i])
      if (--indeg[s2] == 0) ready.push_back(s2);
  }
  if ((int)order.size() != m) return;  // (cannot happen: the dependences form a DAG)
  std::vector<HostOp> out;
  out.reserve(m);
  for (int i : order) out.push_back(std::move(ops[i]));
  ops.swap(out);
}

struct PlanBlock {
  std::vector<int> idx;
  uint64_t hmask = 0;
  int ncoef = 0;
  bool elem_only = true;
};

// Float-float fused passes of dense gates and sign ops are cut where their
// next dense gate would leave the shape table (group.cu), so that each
// piece runs as one straight-line shape kernel: on this layout a pass is
// bound by FP32 issue, and two such sweeps cost less than one interpreted
// pass over both gates (also for passes of 2x2 gates alone: unmerged layers
// of 2x2 gates and CZs at N=26 ran 23.7 ms split against 29.9 ms on warp
// tiles and 119.3 against 114.6 ms per 10 merged random layers at N=28 when
// such passes stayed whole).  Blocks with other ops stay whole.
// max_chunks > 0: a block that would become more shape passes than this
// stays whole (complex64: a state sweep per shape pass costs more than one
// interpreted warp-tile pass of many gates).
static void split_for_shapes(std::vector<PlanBlock>& blocks, const std::vector<HostOp>& ops, int max_bits,
                             int max_chunks) {
  std::vector<PlanBlock> out;
  out.reserve(blocks.size());
  for (PlanBlock& b : blocks) {
    bool ok = !b.elem_only && b.idx.size() > 1;
    for (int i : b.idx) {
      const uint8_t t = ops[i].type;
      ok = ok && (t == OP_DENSE1 || t == OP_DENSE2 || t == OP_SIGN);
    }
    if (!ok) {
      out.push_back(std::move(b));
      continue;
    }
    std::vector<PlanBlock> chunks;
    PlanBlock cur;
    int dense[3], nd = 0;
    auto close = [&]() {
      if (!cur.idx.empty()) chunks.push_back(std::move(cur));
      cur = PlanBlock();
      nd = 0;
    };
    for (int i : b.idx) {
      const HostOp& op = ops[i];
      if (op.type != OP_SIGN) {
        dense[nd] = i;
        if (nd > 0 && (nd == 2 || shape_of(ops, dense, nd + 1, max_bits) < 0)) {
          close();
          dense[0] = i;
        }
        ++nd;
        cur.elem_only = false;
        for (int j = 0; j < op.k; ++j) cur.hmask |= uint64_t(1) << op.gb[j];
      }
      cur.idx.push_back(i);
      cur.ncoef += coef_count(op);
    }
    close();
    if (max_chunks > 0 && (int)chunks.size() > max_chunks) {
      out.push_back(std::move(b));
      continue;
    }
    for (PlanBlock& c : chunks) out.push_back(std::move(c));
  }
  blocks.swap(out);
}

// Gate merging, then greedy blocking into passes (see above); host only.
static std::vector<PlanBlock> plan_blocks(std::vector<HostOp>& ops, int n, int layout, int& fusion_k) {
  const int Lmin = 5;  // bits 0..4 are the lane bits of every fused kernel
  if (fusion_k <= 0) fusion_k = g_default_fusion[layout];
  if (fusion_k > 8) fusion_k = 8;
  if (fusion_k > 1 && g_merge_gates) merge_ops(ops, n);
  if (fusion_k > 1 && g_merge_gates == 2) schedule_ops(ops, n, fusion_k);
  std::vector<PlanBlock> blocks;
  PlanBlock cur;
  for (int i = 0; i < (int)ops.size(); ++i) {
    const HostOp& op = ops[i];
    const int need = coef_count(op);
    uint64_t bits = 0;
    if (!is_elementwise(op.type))
      for (int j = 0; j < op.k; ++j) bits |= uint64_t(1) << op.gb[j];
    const uint64_t newmask = cur.hmask | bits;
    const uint64_t highmask = newmask & ~((uint64_t(1) << Lmin) - 1);
    const bool fits = fusion_k > 1 && __builtin_popcountll(highmask) <= fusion_k &&
                      (int)cur.idx.size() < (cur.elem_only ? ELEM_MAX_OPS : TILE_MAX_OPS) &&
                      cur.ncoef + need <= (cur.elem_only ? TILE_MAX_COEF / 2 : TILE_MAX_COEF);
    if (!cur.idx.empty() && !fits) {
      blocks.push_back(cur);
      cur = PlanBlock();
    }
    cur.idx.push_back(i);
    cur.hmask |= bits;
    cur.ncoef += need;
    cur.elem_only = cur.elem_only && is_elementwise(op.type);
  }
  if (!cur.idx.empty()) blocks.push_back(cur);
  if (layout == FF && group_pass_enabled() && g_shape_max_bits > 0)
    split_for_shapes(blocks, ops, shape_max_bits(FF), 0);
  // complex64: a three-gate pass with CZ signs ran 1.55 ms on a warp tile at
  // N=28 against 0.67 ms per two-gate shape pass
  if (layout == C64 && group_pass_enabled() && shape_max_bits(C64) > 0)
    split_for_shapes(blocks, ops, shape_max_bits(C64), 2);
  return blocks;
}

// Per planned pass: ops, dense 1-qubit, dense 2-qubit (of which with a lane
// bit), element-wise, other, high bits, kernel (0 element-wise, 1 direct
// single-gate sweep, 2 fused warp-tile or shared-memory pass, 3 group pass,
// 4 shape pass).
int plan_stats(int n, int layout, std::vector<HostOp>& ops, int fusion_k, int32_t* stats, int max_blocks,
               int* nblocks) {
  if (layout == FX) return fx_plan_stats(n, ops, fusion_k, stats, max_blocks, nblocks);
  std::vector<PlanBlock> blocks = plan_blocks(ops, n, layout, fusion_k);
  *nblocks = (int)blocks.size();
  for (int b = 0; b < (int)blocks.size() && b < max_blocks; ++b) {
    const PlanBlock& B = blocks[b];
    int32_t* st = stats + 8 * b;
    std::memset(st, 0, 8 * sizeof(int32_t));
    st[0] = (int32_t)B.idx.size();
    for (int i : B.idx) {
      const HostOp& op = ops[i];
      if (op.type == OP_DENSE1) st[1]++;
      else if (op.type == OP_DENSE2) {
        st[2]++;
        if (op.gb[0] < 5 || op.gb[1] < 5) st[3]++;
      } else if (is_elementwise(op.type)) st[4]++;
      else st[5]++;
    }
    st[6] = __builtin_popcountll(B.hmask & ~uint64_t(31));
    const HostOp& first = ops[B.idx[0]];
    st[7] = B.elem_only ? 0
            : (B.idx.size() == 1 && (first.type == OP_DENSE1 || first.type == OP_MONO || first.type == OP_DENSE2))
                ? 1 : 2;
    static thread_local GroupParams gp;
    static thread_local ShapeParams sp;
    int G = 0;
    if (st[7] == 2 && group_pass_enabled()) {
      if (shape_prepare(n, layout, ops, B.idx, sp) == QF_OK) st[7] = 4;
      else if (group_pass_fits(ops, B.idx) && group_prepare(n, layout, ops, B.idx, gp, G) == QF_OK) st[7] = 3;
    }
  }
  return QF_OK;
}

int run_ops(const void* in, void* out, int n, int layout, std::vector<HostOp>& ops, int fusion_k,
            cudaStream_t stream, int* passes_out) {
  if (layout == FX) return fx_run_ops(in, out, n, ops, fusion_k, stream, passes_out);
  const int Lmin = 5;
  std::vector<PlanBlock> blocks = plan_blocks(ops, n, layout, fusion_k);
  int passes = 0;
  const void* src = in;
  if (blocks.empty()) {
    if (in != out) {
      const size_t bytes = (size_t(1) << n) * elem_bytes(layout);
      int rc = check_cuda(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, stream));
      if (rc) return rc;
      passes = 1;
    }
    if (passes_out) *passes_out = passes;
    return QF_OK;
  }
  for (const PlanBlock& b : blocks) {
    int rc;
    const HostOp& first = ops[b.idx[0]];
    if (b.elem_only) {
      LaunchTimer timer(QF_KERNEL_ELEMENTWISE, stream);
      rc = launch_elem(src, out, n, layout, ops, b.idx, stream);
    } else if (b.idx.size() == 1 &&
               (first.type == OP_DENSE1 || first.type == OP_DENSE2 || first.type == OP_MONO)) {
      LaunchTimer timer(first.type == OP_DENSE1 ? QF_KERNEL_DENSE1
                        : first.type == OP_DENSE2 ? QF_KERNEL_DENSE2 : QF_KERNEL_PERMUTATION,
                        stream);
      rc = launch_single(src, out, n, layout, first, stream);
    } else {
      int hb = __builtin_popcountll(b.hmask & ~((uint64_t(1) << Lmin) - 1));
      int rb = g_warp_rb_override > 0 ? g_warp_rb_override : warp_rb(layout);
      rc = QF_ERR_NOT_SUPPORTED;
      static thread_local GroupParams gp;  // ~11 KiB: kept off the stack
      static thread_local ShapeParams sp;
      int G = 0;
      if (group_pass_enabled() && shape_prepare(n, layout, ops, b.idx, sp) == QF_OK) {
        sp.in = src;
        sp.out = out;
        LaunchTimer timer(QF_KERNEL_SHAPE, stream);
        rc = shape_launch(sp, stream);
      } else if (group_pass_enabled() && group_pass_fits(ops, b.idx) &&
                 group_prepare(n, layout, ops, b.idx, gp, G) == QF_OK) {
        gp.in = src;
        gp.out = out;
        LaunchTimer timer(QF_KERNEL_GROUP, stream);
        rc = group_launch(gp, G, stream);
      } else if (!g_force_smem_tile && hb <= rb) {
        LaunchTimer timer(QF_KERNEL_WARP_TILE, stream);
        rc = launch_warp_block(src, out, n, layout, ops, b.idx, rb, stream);
      }
      if (rc == QF_ERR_NOT_SUPPORTED) {
        LaunchTimer timer(QF_KERNEL_FUSED_TILE, stream);
        rc = launch_tile_block(src, out, n, layout, ops, b.idx, b.hmask, stream);
      }
    }
    if (rc) return rc;
    ++passes;
    src = out;
  }
  if (passes_out) *passes_out = passes;
  return QF_OK;
}

}  // namespace qf
