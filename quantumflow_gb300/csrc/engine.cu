// Gate engine: direct sweep kernels, the fused tile kernel and the planner
// that turns a gate list into full-state passes.
//
// Reference semantics: every gate is quantumflow/backend/numpybk.py:159-214
// tensormul -- contract the gate's bra axes with the state axes `indices`
// and write the ket axes back in place -- applied in list order as
// quantumflow/circuits.py:87-99 Circuit.run does.  Nothing here is a
// translation of that einsum: the state is swept once per fused block.
#include "engine.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>

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

// ------------------------------------------------ per-thread coefficients --
QF_D float2 coef_e(const Coef& c, float2*) { return make_float2(c.f[0], c.f[2]); }
QF_D double2 coef_e(const Coef& c, double2*) { return make_double2(c.d[0], c.d[1]); }
QF_D float4 coef_e(const Coef& c, float4*) { return make_float4(c.f[0], c.f[1], c.f[2], c.f[3]); }

QF_D float2 cmul_v(const Coef& c, float2 a) {
  const float ur = c.f[0], ui = c.f[2];
  return make_float2(fmaf(ur, a.x, -ui * a.y), fmaf(ur, a.y, ui * a.x));
}
QF_D double2 cmul_v(const Coef& c, double2 a) {
  const double ur = c.d[0], ui = c.d[1];
  return make_double2(fma(ur, a.x, -ui * a.y), fma(ur, a.y, ui * a.x));
}
QF_D float4 cmul_v(const Coef& c, float4 a) {
  FFAcc re, im;
  re.zero();
  im.zero();
  re.add_prod(c.f[0], c.f[1], a.x, a.y);
  re.add_prod(-c.f[2], -c.f[3], a.z, a.w);
  im.add_prod(c.f[0], c.f[1], a.z, a.w);
  im.add_prod(c.f[2], c.f[3], a.x, a.y);
  float4 r;
  re.finish(r.x, r.y);
  im.finish(r.z, r.w);
  return r;
}

QF_D float2 shfl_xor(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
QF_D double2 shfl_xor(double2 v, int m) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
QF_D float4 shfl_xor(float4 v, int m) {
  return make_float4(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m),
                     __shfl_xor_sync(0xffffffffu, v.z, m), __shfl_xor_sync(0xffffffffu, v.w, m));
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

// 2-qubit dense gate on bits q0 (matrix MSB) and q1.
template <int LAY>
__global__ void __launch_bounds__(256) k_dense2(const typename Types<LAY>::E* in,
                                                typename Types<LAY>::E* out, int64_t nquads, int q0,
                                                int q1, const __grid_constant__ CoefArr16 u) {
  using E = typename Types<LAY>::E;
  const int lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0;
  const int64_t b0 = int64_t(1) << q0, b1 = int64_t(1) << q1;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nquads; t += nthr) {
    const int64_t base = insert0(insert0(t, lo), hi);
    const int64_t idx[4] = {base, base | b1, base | b0, base | b0 | b1};
    E a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = in[idx[r]];
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

template <int LAY>
__device__ void tile_apply(const TileParams& P, typename Types<LAY>::E* s, int64_t base, int tbits) {
  using E = typename Types<LAY>::E;
  const int T = 1 << tbits;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  for (int o = 0; o < P.nops; ++o) {
    const TileOp& op = P.ops[o];
    const Coef* cf = &P.coef[op.coef];
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
        E* tag = nullptr;
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
              const E prod = cmul_v(cf[lane * G + j], s[src]);
              const float4 pf = to_ff(prod);
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
          (void)tag;
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
    __syncthreads();
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

struct LaunchTimer {
  bool on = false;
  TimedLaunch t{};
  cudaStream_t s = nullptr;
  LaunchTimer(int kind, cudaStream_t stream) {
    std::lock_guard<std::mutex> g(g_timing_mu);
    if (!g_timing_on) return;
    on = true;
    s = stream;
    t.kind = kind;
    t.start = pooled_event();
    t.stop = pooled_event();
    cudaEventRecord(t.start, s);
  }
  ~LaunchTimer() {
    if (!on) return;
    cudaEventRecord(t.stop, s);
    std::lock_guard<std::mutex> g(g_timing_mu);
    g_timed.push_back(t);
  }
};

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
      k_dense2<LAY><<<grid_for(nq), 256, 0, stream>>>(src, dst, nq, op.gb[0], op.gb[1], u);
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

template <int LAY>
static int launch_tile_t(const void* in, void* out, int n, const std::vector<HostOp>& ops,
                         const std::vector<int>& idx, uint64_t hmask, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  static thread_local TileParams P;  // ~20 KiB: kept off the stack
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
  int nc = 0;
  P.nops = 0;
  for (int i : idx) {
    const HostOp& op = ops[i];
    if (P.nops >= TILE_MAX_OPS) return QF_ERR_TOO_LARGE;
    TileOp& t = P.ops[P.nops++];
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
  const int tbits = L + nh;
  const size_t smem = 2 * (size_t(1) << tbits) * sizeof(E);
  static std::atomic<bool> attr_set[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr_set[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_tile<LAY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024));
    if (rc) return rc;
    attr_set[dev].store(true);
  }
  const int64_t ntiles = int64_t(1) << (n - tbits);
  int64_t grid = (int64_t)device_sm_count() * (smem > 80 * 1024 ? 2 : 3);
  if (grid > ntiles) grid = ntiles;
  P.threads = 256;
  k_tile<LAY><<<(int)grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
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

// Greedy fusion: walk the ops in order; element-wise ops join the current
// block unconditionally (they need no tile bits), every other op joins while
// the union of high bits (>= Lmin) stays within fusion_k.
int run_ops(const void* in, void* out, int n, int layout, std::vector<HostOp>& ops, int fusion_k,
            cudaStream_t stream, int* passes_out) {
  const int Lmin = layout == C64 ? 6 : 5;
  if (fusion_k <= 0) fusion_k = 6;
  if (fusion_k > 8) fusion_k = 8;
  int passes = 0;
  const void* src = in;
  struct Block {
    std::vector<int> idx;
    uint64_t hmask = 0;
    int ncoef = 0;
    bool elem_only = true;
  };
  std::vector<Block> blocks;
  Block cur;
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
      cur = Block();
    }
    cur.idx.push_back(i);
    cur.hmask |= bits;
    cur.ncoef += need;
    cur.elem_only = cur.elem_only && is_elementwise(op.type);
  }
  if (!cur.idx.empty()) blocks.push_back(cur);
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
  for (const Block& b : blocks) {
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
      LaunchTimer timer(QF_KERNEL_FUSED_TILE, stream);
      rc = launch_tile_block(src, out, n, layout, ops, b.idx, b.hmask, stream);
    }
    if (rc) return rc;
    ++passes;
    src = out;
  }
  if (passes_out) *passes_out = passes;
  return QF_OK;
}

}  // namespace qf
