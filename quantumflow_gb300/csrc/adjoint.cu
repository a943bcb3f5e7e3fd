// Adjoint (reverse-mode) gradient of the QAOA MAXCUT expectation
// <C> = <psi|C|psi>, psi = prod_l [RX(beta_l)^n  exp(i gamma_l (E/2 - C))] |+>^n
// (the qubo_circuit of quantumflow/qaoa.py:22-64; the reference obtains this
// gradient only through TensorFlow autodiff, examples/qaoa_maxcut.py:56-64).
//
// After the forward state psi, lambda = C psi, and the layers are undone in
// reverse order on both vectors at once.  For layer l, with psi and lambda
// taken right after its mixer:
//   d<C>/d beta_l  = sum_j Im <lambda| X_j |psi>
// and right after its cost layer:
//   d<C>/d gamma_l = -2 Im <lambda| (E/2 - C) |psi>.
// Only two state vectors are held, whatever the depth.
//
// Each pass is a dual-state tile kernel: tiles of psi and lambda are staged
// into shared memory with bulk async copies, the pass's ops run on both, and
// reductions accumulate per warp; every CTA adds its totals into its own row
// of the caller's workspace (rows stay fixed across passes because the grid
// size is fixed for a given n), and a final kernel sums the rows.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "state.cuh"

namespace qf {

enum AdjOpType : uint8_t {
  A_INIT = 1,    // lambda = c * psi, and out[slot] += sum c |psi|^2
  A_REDX = 2,    // out[slot] += scale * Im sum_x conj(lambda_x) psi_{x ^ bit}
  A_REDCUT = 3,  // out[slot] += scale * Im sum_x conj(lambda_x) (wref - c_x) psi_x
  A_G1 = 4,      // 2x2 gate on a tile bit, both vectors
  A_CUT = 5,     // psi_x *= table[c_x], both vectors
  A_DIAG1 = 6,   // 1-qubit diagonal on a global bit, both vectors
};

constexpr int ADJ_MAX_OPS = 64;
constexpr int ADJ_MAX_COEF = 1200;
constexpr int ADJ_MAX_SLOTS = 64;

struct AdjOp {
  uint8_t type;
  uint8_t lb;  // tile-local bit (A_G1, A_REDX)
  uint8_t gb;  // global bit (A_DIAG1)
  uint8_t pad;
  uint16_t slot;
  uint16_t coef;
  uint16_t ncoef;
  uint16_t pad2;
  float scale;
  float wref;
};

struct AdjParams {
  void* psi;
  void* lam;
  const uint16_t* cuts;
  double* rows;  // [gridDim.x][nslots]
  int32_t n, L, nh, nops, nslots, load_lambda;
  uint8_t hb[8];
  AdjOp ops[ADJ_MAX_OPS];
  Coef coef[ADJ_MAX_COEF];
};

QF_D int64_t adj_global(const AdjParams& P, int64_t base, int l) {
  int64_t x = base | (l & ((1 << P.L) - 1));
  for (int r = 0; r < P.nh; ++r)
    if ((l >> (P.L + r)) & 1) x |= int64_t(1) << P.hb[r];
  return x;
}

QF_D bool adj_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023u) == 0) {
      uint64_t t1;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
      if (t1 - t0 > 4000000000ull) return false;
    }
  }
}

template <int LAY>
__global__ void __launch_bounds__(256) k_adj(const __grid_constant__ AdjParams P) {
  using E = typename Types<LAY>::E;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ double acc[8][ADJ_MAX_SLOTS];  // per-warp running sums
  const int tbits = P.L + P.nh;
  const int T = 1 << tbits;
  // stage s: psi tile at 2*s, lambda tile at 2*s+1
  E* buf = reinterpret_cast<E*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nthr = blockDim.x;
  const int64_t ntiles = int64_t(1) << (P.n - tbits);
  const uint32_t chunk_amps = 1u << P.L;
  const uint32_t chunk_bytes = chunk_amps * (uint32_t)sizeof(E);
  const int nchunks = 1 << P.nh;
  E* gpsi = reinterpret_cast<E*>(P.psi);
  E* glam = reinterpret_cast<E*>(P.lam);
  const int nvec = P.load_lambda ? 2 : 1;

  for (int i = tid; i < 8 * ADJ_MAX_SLOTS; i += nthr) (&acc[0][0])[i] = 0.0;
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto tile_base = [&](int64_t t) {
    int64_t v = t << P.L;
    for (int r = 0; r < P.nh; ++r) v = insert0(v, P.hb[r]);
    return v;
  };
  auto chunk_off = [&](int c) {
    int64_t o = 0;
    for (int r = 0; r < P.nh; ++r)
      if ((c >> r) & 1) o |= int64_t(1) << P.hb[r];
    return o;
  };
  auto issue_load = [&](int64_t t, int s) {
    if (lane == 0) mbar_arrive_expect_tx(&bars[s], (uint32_t)(nvec * T * sizeof(E)));
    __syncwarp();
    const int64_t base = tile_base(t);
    for (int c = lane; c < nchunks; c += 32) {
      const int64_t off = base + chunk_off(c);
      bulk_g2s(buf + (size_t)(2 * s) * T + (size_t)c * chunk_amps, gpsi + off, chunk_bytes, &bars[s]);
      if (nvec == 2)
        bulk_g2s(buf + (size_t)(2 * s + 1) * T + (size_t)c * chunk_amps, glam + off, chunk_bytes, &bars[s]);
    }
  };

  int64_t t = blockIdx.x;
  if (tid < 32 && t < ntiles) issue_load(t, 0);
  uint32_t it = 0;
  bool failed = false;
  for (; t < ntiles; t += gridDim.x, ++it) {
    const int s = it & 1;
    const int64_t nxt = t + gridDim.x;
    if (tid < 32 && nxt < ntiles) {
      bulk_wait_read0();
      __syncwarp();
      issue_load(nxt, s ^ 1);
    }
    const bool ok = adj_wait(&bars[s], (it >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    E* sp = buf + (size_t)(2 * s) * T;
    E* sl = sp + T;
    const int64_t base = tile_base(t);
    for (int o = 0; o < P.nops; ++o) {
      const AdjOp& op = P.ops[o];
      const Coef* cf = &P.coef[op.coef];
      switch (op.type) {
        case A_INIT: {
          FFAcc e;
          e.zero();
          for (int l = tid; l < T; l += nthr) {
            const int64_t x = adj_global(P, base, l);
            const float c = (float)P.cuts[x];
            const E v = sp[l];
            sl[l] = scale_ff(v, c);
            FFAcc tmp;
            tmp.zero();
            acc_norm2(tmp, v);
            e.add_prod(c, 0.f, tmp.s, tmp.e);
          }
          double v = warp_sum((double)e.s + (double)e.e);
          if (lane == 0) acc[warp][op.slot] += v;
          break;
        }
        case A_REDX: {
          const int q = op.lb, bit = 1 << q;
          FFAcc a;
          a.zero();
          for (int p = tid; p < (T >> 1); p += nthr) {
            const int i0 = ((p >> q) << (q + 1)) | (p & (bit - 1));
            const int i1 = i0 | bit;
            acc_imconj(a, sl[i0], sp[i1], 1.f);
            acc_imconj(a, sl[i1], sp[i0], 1.f);
          }
          double v = warp_sum((double)a.s + (double)a.e);
          if (lane == 0) acc[warp][op.slot] += v * op.scale;
          break;
        }
        case A_REDCUT: {
          FFAcc a;
          a.zero();
          for (int l = tid; l < T; l += nthr) {
            const int64_t x = adj_global(P, base, l);
            const float w = op.wref - (float)P.cuts[x];  // half-integer: exact
            acc_imconj(a, sl[l], sp[l], w);
          }
          double v = warp_sum((double)a.s + (double)a.e);
          if (lane == 0) acc[warp][op.slot] += v * op.scale;
          break;
        }
        case A_G1: {
          const int q = op.lb, bit = 1 << q;
          for (int p = tid; p < (T >> 1); p += nthr) {
            const int i0 = ((p >> q) << (q + 1)) | (p & (bit - 1));
            const int i1 = i0 | bit;
            E a[2] = {sp[i0], sp[i1]};
            sp[i0] = cdot<2>(cf, a);
            sp[i1] = cdot<2>(cf + 2, a);
            E b[2] = {sl[i0], sl[i1]};
            sl[i0] = cdot<2>(cf, b);
            sl[i1] = cdot<2>(cf + 2, b);
          }
          break;
        }
        case A_CUT: {
          for (int l = tid; l < T; l += nthr) {
            const int64_t x = adj_global(P, base, l);
            const int c = min((int)P.cuts[x], op.ncoef - 1);
            sp[l] = cmul_v(cf[c], sp[l]);
            sl[l] = cmul_v(cf[c], sl[l]);
          }
          break;
        }
        case A_DIAG1: {
          for (int l = tid; l < T; l += nthr) {
            const int64_t x = adj_global(P, base, l);
            const Coef& c = cf[(x >> op.gb) & 1];
            sp[l] = cmul_v(c, sp[l]);
            sl[l] = cmul_v(c, sl[l]);
          }
          break;
        }
      }
      __syncthreads();
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid < 32) {
      for (int c = lane; c < nchunks; c += 32) {
        const int64_t off = base + chunk_off(c);
        bulk_s2g(gpsi + off, sp + (size_t)c * chunk_amps, chunk_bytes);
        bulk_s2g(glam + off, sl + (size_t)c * chunk_amps, chunk_bytes);
      }
      bulk_commit();
    }
  }
  if (tid < 32) bulk_wait0();
  __syncthreads();
  if (failed) return;  // rows keep their old values; the host sees the error word
  for (int sidx = tid; sidx < P.nslots; sidx += nthr) {
    double v = 0.0;
    for (int w = 0; w < (nthr >> 5); ++w) v += acc[w][sidx];
    P.rows[(size_t)blockIdx.x * P.nslots + sidx] += v;
  }
}

// ------------------------------------------------- warp-tile adjoint ----
// The same passes as k_adj with psi and lambda held in registers: a warp
// owns a sub-tile of 32 lanes (global bits 0..4) x 2^RB registers (the
// pass's high bits), gates on lane bits use shuffles, and nothing waits on
// another warp.  The pass structure is fixed by the QAOA layer: optionally
// lambda = C psi (the sweep's first pass), the mixer on the lane bits (a
// layer's first pass) and on up to RB register bits, and the cost layer (a
// layer's last pass).  Each sub-tile is prefetched two sub-tiles ahead into
// a per-warp shared-memory ring with per-thread async copies.
constexpr int ADJW_MAX_COEF = 1100;
constexpr int ADJW_STAGES = 2;  // per-warp prefetch ring depth (sub-tiles)

struct AdjWParams {
  void* psi;
  void* lam;
  const uint16_t* cuts;
  double* rows;
  int32_t n, nslots;
  int32_t init;   // lambda = c psi; <C> accumulator += c |psi|^2
  int32_t lanes;  // mixer reduction + RX(-beta) on lane bits 0..4
  int32_t nact;   // ... and on register bits 0..nact-1
  int32_t last;   // cut reduction, node phases (ndiag), cut phase (ncut entries)
  int32_t ndiag, ncut;
  int32_t hasB, nactB;               // stage B: the previous layer's mixer on lanes + bits 0..nactB-1
  int32_t slot_x, slot_cut, slot_e, slot_xb;  // output slots of the four accumulators (-1: unused)
  float wref;                        // E/2
  uint8_t hb[4];                     // global bit of each register index bit
  uint8_t hs[4];                     // the same bits in ascending order
  uint8_t diag_bit[QF_MAX_QUBITS];   // global bit of each node phase
  Coef rx_c, rx_s;                   // RX(-beta) = [[c, i s], [i s, c]]
  Coef b_c, b_s;                     // the same for stage B's layer
  Coef coef[ADJW_MAX_COEF];          // node phase pairs, then the cut table
};

template <int LAY, int RB>
constexpr size_t adjw_ring_bytes() {
  return (size_t)8 * ADJW_STAGES * 2 * (32 << RB) * sizeof(typename Types<LAY>::E);
}

template <int LAY, int RB>
__global__ void __launch_bounds__(256) k_adjw(const __grid_constant__ AdjWParams P) {
  using E = typename Types<LAY>::E;
  constexpr int R = 1 << RB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Coef* scoef = reinterpret_cast<Coef*>(smem_raw);
  __shared__ double red[8][4];
  const int necoef = 2 * P.ndiag + P.ncut;
  for (int i = threadIdx.x; i < necoef; i += blockDim.x) scoef[i] = P.coef[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // this warp's ring: [stage][vector][register][lane]
  E* ring = reinterpret_cast<E*>(smem_raw + (((size_t)necoef * sizeof(Coef) + 127) & ~size_t(127))) +
            (size_t)warp * ADJW_STAGES * 2 * R * 32;
  const int64_t nsub = int64_t(1) << (P.n - 5 - RB);
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  E* gp = reinterpret_cast<E*>(P.psi);
  E* gl = reinterpret_cast<E*>(P.lam);
  const bool load_lambda = !P.init;
  int64_t hoff[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int64_t o = 0;
#pragma unroll
    for (int j = 0; j < RB; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << P.hb[j];
    hoff[r] = o;
  }
  auto sub_base = [&](int64_t st) {
    int64_t base = st << 5;
#pragma unroll
    for (int j = 0; j < RB; ++j) base = insert0(base, P.hs[j]);
    return base | lane;
  };
  // prefetch sub-tile st into ring stage sg (an empty group past the end)
  auto issue = [&](int64_t st, int sg) {
    if (st < nsub) {
      const int64_t xb = sub_base(st);
      E* sp = ring + (size_t)sg * 2 * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) cp_async_amp(sp + r * 32, gp + (xb | hoff[r]));
      if (load_lambda) {
#pragma unroll
        for (int r = 0; r < R; ++r) cp_async_amp(sp + (R + r) * 32, gl + (xb | hoff[r]));
      }
    }
    cp_async_commit();
  };
  FFAcc ax, ac, ae, axb;
  ax.zero();
  ac.zero();
  ae.zero();
  axb.zero();
  const Coef rc = P.rx_c, rs = P.rx_s;
  int64_t st = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  __syncthreads();  // coefficient table staged
#pragma unroll
  for (int k = 0; k < ADJW_STAGES - 1; ++k) issue(st + k * wstride, k);
  int sg = 0;
  for (; st < nsub; st += wstride) {
    cp_async_wait<ADJW_STAGES - 2>();  // this sub-tile's group has landed
    const int64_t xb = sub_base(st);
    E a[R], l[R];
    {
      const E* sp = ring + (size_t)sg * 2 * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        a[r] = sp[r * 32];
        if (load_lambda) l[r] = sp[(R + r) * 32];
      }
    }
    // refill the stage read one iteration ago (its values are in registers)
    issue(st + (ADJW_STAGES - 1) * wstride, sg == 0 ? ADJW_STAGES - 1 : sg - 1);
    sg = sg + 1 == ADJW_STAGES ? 0 : sg + 1;

    if (P.init) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float c = (float)P.cuts[xb | hoff[r]];
        FFAcc t;
        t.zero();
        acc_norm2(t, a[r]);
        ae.add_prod(c, 0.f, t.s, t.e);
        l[r] = scale_ff(a[r], c);
      }
    }
    // mixer: each bit's reduction precedes its own RX(-beta); the
    // reduction on bit j is unchanged by RX already undone on other bits
    // (same unitary on both vectors) and commutes with X_j
    // complex64: a sub-tile's reduction terms are summed in FP32 and added
    // to the compensated accumulator once
    constexpr bool F32 = LAY == C64;
    auto redx = [&](FFAcc& acc, float& part, const E& lv, const E& pv) {
      if constexpr (F32) {
        part = fmaf(lv.x, pv.y, part);
        part = fmaf(-lv.y, pv.x, part);
      } else {
        redx_acc(acc, lv, pv);
      }
    };
    auto mixer = [&](const Coef& mc, const Coef& ms, bool lanes, int nact, FFAcc& acc) {
      float part = 0.f;
      if (lanes) {
        for (int b = 0; b < 5; ++b) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const E pa = shfl_xor(a[r], 1 << b);
            const E pl = shfl_xor(l[r], 1 << b);
            redx(acc, part, l[r], pa);
            a[r] = rx_one(mc, ms, a[r], pa);
            l[r] = rx_one(mc, ms, l[r], pl);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        if (j < nact) {
#pragma unroll
          for (int i = 0; i < R / 2; ++i) {
            const int i0 = ((i >> j) << (j + 1)) | (i & ((1 << j) - 1));
            const int i1 = i0 | (1 << j);
            redx(acc, part, l[i0], a[i1]);
            redx(acc, part, l[i1], a[i0]);
            const E a0 = a[i0], l0 = l[i0];
            a[i0] = rx_one(mc, ms, a0, a[i1]);
            a[i1] = rx_one(mc, ms, a[i1], a0);
            l[i0] = rx_one(mc, ms, l0, l[i1]);
            l[i1] = rx_one(mc, ms, l[i1], l0);
          }
        }
      }
      if constexpr (F32) acc.add(part, 0.f);
    };
    mixer(rc, rs, P.lanes != 0, P.nact, ax);
    if (P.last) {
      uint32_t cv[R];
#pragma unroll
      for (int r = 0; r < R; ++r) cv[r] = P.cuts[xb | hoff[r]];
      if constexpr (F32) {
        float part = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r)
          part = fmaf(P.wref - (float)cv[r], fmaf(l[r].x, a[r].y, -l[r].y * a[r].x), part);
        ac.add(part, 0.f);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) acc_imconj(ac, to_ff(l[r]), to_ff(a[r]), P.wref - (float)cv[r]);
      }
      for (int d = 0; d < P.ndiag; ++d) {
        const int gb = P.diag_bit[d];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const Coef& c = scoef[2 * d + (((xb | hoff[r]) >> gb) & 1)];
          a[r] = cmul_v(c, a[r]);
          l[r] = cmul_v(c, l[r]);
        }
      }
      const Coef* tab = scoef + 2 * P.ndiag;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const Coef& c = tab[min((int)cv[r], P.ncut - 1)];
        a[r] = cmul_v(c, a[r]);
        l[r] = cmul_v(c, l[r]);
      }
    }
    if (P.hasB) mixer(P.b_c, P.b_s, true, P.nactB, axb);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      gp[xb | hoff[r]] = a[r];
      gl[xb | hoff[r]] = l[r];
    }
  }
  cp_async_wait<0>();
  // per-CTA sums of the four accumulators into this CTA's row
  const double v[4] = {warp_sum((double)ax.s + (double)ax.e), warp_sum((double)ac.s + (double)ac.e),
                       warp_sum((double)ae.s + (double)ae.e), warp_sum((double)axb.s + (double)axb.e)};
  if (lane == 0)
    for (int k = 0; k < 4; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 4) {
    const int k = threadIdx.x;
    const int slot = k == 0 ? P.slot_x : k == 1 ? P.slot_cut : k == 2 ? P.slot_e : P.slot_xb;
    if (slot >= 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
      const float sc = threadIdx.x == 1 ? -2.f : 1.f;
      P.rows[(size_t)blockIdx.x * P.nslots + slot] += sc * t;
    }
  }
}

// out[s] = sum over rows of rows[r][s]; one warp per slot, fixed order
__global__ void k_rows_sum(const double* rows, int nrows, int nslots, double* out) {
  const int s = blockIdx.x;
  if (s >= nslots) return;
  double v = 0.0;
  for (int r = threadIdx.x; r < nrows; r += 32) v += rows[(size_t)r * nslots + s];
  v = warp_sum(v);
  if (threadIdx.x == 0) out[s] = v;
}

void qaoa_layer_ops(int n, const uint16_t* cuts, int nedges, double beta, double gamma,
                    const double* node_theta, std::vector<HostOp>& ops);

int g_adjoint_smem_only = 0;  // qf_set_tile_kernel(1): shared-memory adjoint kernel only

int adj_grid(int n, int layout) {
  const int TB = layout == C64 ? 11 : 10;
  const int tb = n < TB ? n : TB;
  const int64_t ntiles = int64_t(1) << (n - tb);
  int64_t g = device_sm_count();
  if (g > ntiles) g = (int)ntiles;
  return (int)g;
}

extern int g_warp_rb_override;

// register bits of k_adjw: 2 or 3 for FP64/float-float, 3 or 4 for complex64
int adjw_rb(int layout) {
  const int o = g_warp_rb_override;
  if (layout == C64) return (o == 3 || o == 4) ? o : 3;
  return (o == 2 || o == 3) ? o : 2;
}

int adjw_grid(int n, int layout) {
  const int rb = adjw_rb(layout);
  if (n < 5 + rb) return 0;
  const int64_t nsub = int64_t(1) << (n - 5 - rb);
  int64_t g = (nsub + 7) / 8;
  const int64_t cap = (int64_t)device_sm_count() * 4;
  return (int)(g < cap ? g : cap);
}

size_t qaoa_grad_workspace_bytes(int n, int p, int layout) {
  const size_t amps = size_t(1) << n;
  const int nslots = 2 * p + 1;
  const int rows = std::max(adj_grid(n, layout), adjw_grid(n, layout));
  return amps * elem_bytes(layout) + (size_t)rows * nslots * sizeof(double) + 512;
}

template <int LAY, int RB>
static int launch_adjw(AdjWParams& P, int grid, cudaStream_t stream) {
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_adjw<LAY, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(adjw_ring_bytes<LAY, RB>() + ADJW_MAX_COEF * sizeof(Coef) + 128)));
    if (rc) return rc;
    attr[dev].store(true);
  }
  const size_t necoef = (size_t)(2 * P.ndiag + P.ncut);
  const size_t smem = ((necoef * sizeof(Coef) + 127) & ~size_t(127)) + adjw_ring_bytes<LAY, RB>();
  k_adjw<LAY, RB><<<grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

// Warp-tile adjoint sweep (k_adjw); psi holds the forward state.  Per layer
// the high bits 5..n-1 are taken RB at a time (the last group may act on
// fewer, its register index padded with other high bits that are carried
// unchanged); the first pass also undoes the mixer on the lane bits, the
// last one the cost layer.
static int qaoa_grad_warp(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p, const double* beta,
                          const double* gamma, const double* node_theta, void* lam, double* rows, int nslots,
                          cudaStream_t stream) {
  const int RB = adjw_rb(layout);
  const int grid = adjw_grid(n, layout);
  static thread_local AdjWParams P;
  std::vector<std::vector<int>> groups;
  for (int b = 5; b < n; b += RB) {
    std::vector<int> g;
    for (int k = b; k < std::min(n, b + RB); ++k) g.push_back(k);
    groups.push_back(g);
  }
  const double half_e = 0.5 * nedges;
  std::memset(&P, 0, sizeof(P));
  P.psi = psi;
  P.lam = lam;
  P.cuts = cuts;
  P.rows = rows;
  P.n = n;
  P.nslots = nslots;
  P.wref = (float)half_e;
  int nd = 0;
  if (node_theta != nullptr) {
    for (int q = 0; q < n; ++q) {
      if (std::isnan(node_theta[q])) continue;
      P.diag_bit[nd] = (uint8_t)(n - 1 - q);
      P.coef[2 * nd] = make_coef(std::polar(1.0, 0.5 * node_theta[q]), layout);
      P.coef[2 * nd + 1] = make_coef(std::polar(1.0, -0.5 * node_theta[q]), layout);
      ++nd;
    }
  }
  P.ndiag = nd;
  P.ncut = nedges + 1;
  if (2 * nd + P.ncut > ADJW_MAX_COEF) return QF_ERR_TOO_LARGE;
  const int m = (int)groups.size();
  // layer l (counted from the last) visits the groups forwards or backwards
  // so that its last group is the next layer's first: that pass also runs
  // the next layer's mixer on the lanes and the same group (stage B)
  auto order = [&](int l, int k) { return ((p - 1 - l) & 1) ? m - 1 - k : k; };
  auto set_group = [&](int gi) {
    std::vector<int> hb = groups[gi];
    for (int b = 5; b < n && (int)hb.size() < RB; ++b)
      if (std::find(hb.begin(), hb.end(), b) == hb.end()) hb.push_back(b);
    for (int j = 0; j < RB; ++j) P.hb[j] = (uint8_t)hb[j];  // acted-on bits first
    std::sort(hb.begin(), hb.end());
    for (int j = 0; j < RB; ++j) P.hs[j] = (uint8_t)hb[j];
    return (int)groups[gi].size();
  };
  auto launch = [&]() {
    switch (layout * 8 + RB) {
      case C64 * 8 + 3: return launch_adjw<C64, 3>(P, grid, stream);
      case C64 * 8 + 4: return launch_adjw<C64, 4>(P, grid, stream);
      case C128 * 8 + 2: return launch_adjw<C128, 2>(P, grid, stream);
      case C128 * 8 + 3: return launch_adjw<C128, 3>(P, grid, stream);
      case FF * 8 + 2: return launch_adjw<FF, 2>(P, grid, stream);
      case FF * 8 + 3: return launch_adjw<FF, 3>(P, grid, stream);
    }
    return (int)QF_ERR_LAYOUT;
  };
  bool first = true;
  bool lanes_done = false;  // the layer's lane bits were undone by the previous pass's stage B
  for (int l = p - 1; l >= 0; --l) {
    P.rx_c = make_coef(cplx(std::cos(0.5 * beta[l]), 0.0), layout);
    P.rx_s = make_coef(cplx(std::sin(0.5 * beta[l]), 0.0), layout);
    for (int cv = 0; cv <= nedges; ++cv)
      P.coef[2 * nd + cv] = make_coef(std::polar(1.0, -gamma[l] * (half_e - cv)), layout);
    for (int k = lanes_done ? 1 : 0; k < m; ++k) {
      const int nact = set_group(order(l, k));
      P.init = first ? 1 : 0;
      P.lanes = k == 0 ? 1 : 0;
      P.nact = nact;
      P.last = k == m - 1 ? 1 : 0;
      P.slot_x = p + l;
      P.slot_cut = P.last ? l : -1;
      P.slot_e = first ? 2 * p : -1;
      P.hasB = 0;
      P.slot_xb = -1;
      if (P.last && l > 0 && m > 1) {  // order(l-1, 0) == order(l, m-1)
        P.hasB = 1;
        P.nactB = nact;
        P.b_c = make_coef(cplx(std::cos(0.5 * beta[l - 1]), 0.0), layout);
        P.b_s = make_coef(cplx(std::sin(0.5 * beta[l - 1]), 0.0), layout);
        P.slot_xb = p + l - 1;
      }
      const int rc = launch();
      if (rc) return rc;
      first = false;
    }
    lanes_done = m > 1;
  }
  return QF_OK;
}

template <int LAY>
static int launch_adj(AdjParams& P, int grid, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  const size_t smem = 4 * (size_t(1) << (P.L + P.nh)) * sizeof(E);
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_adj<LAY>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    if (rc) return rc;
    attr[dev].store(true);
  }
  k_adj<LAY><<<grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

// out[0..p) = d<C>/d gamma, out[p..2p) = d<C>/d beta, out[2p] = <C>.
// psi must hold the forward QAOA state; it is consumed (left at |+>^n).
int qaoa_grad(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p, const double* beta,
              const double* gamma, const double* node_theta, double* out, void* ws, cudaStream_t stream) {
  const int TB = layout == C64 ? 11 : 10;
  const int KH = TB - (layout == C64 ? 6 : 5);  // high bits per pass
  const int Lmin = layout == C64 ? 6 : 5;
  const size_t amps = size_t(1) << n;
  void* lam = ws;
  double* rows = reinterpret_cast<double*>(reinterpret_cast<char*>(ws) + ((amps * elem_bytes(layout) + 255) & ~size_t(255)));
  const int nslots = 2 * p + 1;
  if (nslots > ADJ_MAX_SLOTS) return QF_ERR_TOO_LARGE;
  const int wgrid = adjw_grid(n, layout);
  const bool wfits = 4 + 2 * n + nedges + 1 <= ADJW_MAX_COEF;  // coefficient table of one pass
  if (wgrid > 0 && p > 0 && wfits && !g_adjoint_smem_only) {
    int rc = check_cuda(cudaMemsetAsync(rows, 0, (size_t)wgrid * nslots * sizeof(double), stream));
    if (rc) return rc;
    rc = qaoa_grad_warp(psi, n, layout, cuts, nedges, p, beta, gamma, node_theta, lam, rows, nslots, stream);
    if (rc) return rc;
    k_rows_sum<<<nslots, 32, 0, stream>>>(rows, wgrid, nslots, out);
    return check_cuda(cudaGetLastError());
  }
  const int grid = adj_grid(n, layout);
  int rc = check_cuda(cudaMemsetAsync(rows, 0, (size_t)grid * nslots * sizeof(double), stream));
  if (rc) return rc;
  static thread_local AdjParams P;

  // pass plan for one layer: groups of tile bits
  std::vector<std::vector<int>> groups;  // each: high bits (>= Lmin) of a pass
  {
    std::vector<int> high;
    for (int b = Lmin; b < n; ++b) high.push_back(b);
    if (n <= TB) {
      groups.push_back({});
    } else {
      for (size_t i = 0; i < high.size(); i += KH)
        groups.push_back(std::vector<int>(high.begin() + i, high.begin() + std::min(high.size(), i + KH)));
    }
  }
  const double half_e = 0.5 * nedges;
  bool first = true;
  for (int l = p - 1; l >= 0; --l) {
    const double c = std::cos(0.5 * beta[l]), s = std::sin(0.5 * beta[l]);
    // RX(beta)^dagger = RX(-beta) = [[c, is], [is, c]]
    const cplx rxd[4] = {cplx(c, 0), cplx(0, s), cplx(0, s), cplx(c, 0)};
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      std::memset(&P, 0, sizeof(P));
      P.psi = psi;
      P.lam = lam;
      P.cuts = cuts;
      P.rows = rows;
      P.n = n;
      P.nslots = nslots;
      P.load_lambda = first ? 0 : 1;
      // geometry: tile bits = low run + this group's high bits
      int L, nh;
      if (n <= TB) {
        L = n;
        nh = 0;
      } else {
        nh = (int)groups[gi].size();
        L = TB - nh;
        // the low run must not swallow the group's bits: groups hold bits >= Lmin,
        // so use L = Lmin and pad with the next free low bits instead
        L = Lmin;
        for (int b : groups[gi]) (void)b;
      }
      P.L = L;
      P.nh = nh;
      for (int r = 0; r < nh; ++r) P.hb[r] = (uint8_t)groups[gi][r];
      int nops = 0, nc = 0;
      auto push = [&](AdjOp o) { P.ops[nops++] = o; };
      if (first) {
        AdjOp o{};
        o.type = A_INIT;
        o.slot = (uint16_t)(2 * p);
        push(o);
        first = false;
      }
      // tile bits of this pass: low run [0, L) plus hb
      std::vector<int> tile_global;
      for (int b = 0; b < L; ++b) tile_global.push_back(b);
      for (int r = 0; r < nh; ++r) tile_global.push_back(P.hb[r]);
      // mixer: bits handled in this pass = the group's high bits, plus all
      // low bits in the layer's first pass
      std::vector<std::pair<int, int>> mbits;  // (global bit, local bit)
      if (gi == 0)
        for (int b = 0; b < std::min(L, n); ++b) mbits.push_back({b, b});
      for (int r = 0; r < nh; ++r) mbits.push_back({P.hb[r], L + r});
      if (n <= TB) {
        mbits.clear();
        for (int b = 0; b < n; ++b) mbits.push_back({b, b});
      }
      for (auto& bl : mbits) {
        AdjOp o{};
        o.type = A_REDX;
        o.lb = (uint8_t)bl.second;
        o.slot = (uint16_t)(p + l);
        o.scale = 1.f;
        push(o);
      }
      for (auto& bl : mbits) {
        AdjOp o{};
        o.type = A_G1;
        o.lb = (uint8_t)bl.second;
        o.coef = (uint16_t)nc;
        for (int k = 0; k < 4; ++k) P.coef[nc + k] = make_coef(rxd[k], layout);
        nc += 4;
        push(o);
      }
      if (gi + 1 == groups.size()) {
        // cost layer of step l: gradient, then undo node RZ and the phase
        AdjOp g{};
        g.type = A_REDCUT;
        g.slot = (uint16_t)l;
        g.scale = -2.f;
        g.wref = (float)half_e;
        push(g);
        if (node_theta != nullptr) {
          for (int q = 0; q < n; ++q) {
            if (std::isnan(node_theta[q])) continue;
            AdjOp o{};
            o.type = A_DIAG1;
            o.gb = (uint8_t)(n - 1 - q);
            o.coef = (uint16_t)nc;
            P.coef[nc] = make_coef(std::polar(1.0, 0.5 * node_theta[q]), layout);
            P.coef[nc + 1] = make_coef(std::polar(1.0, -0.5 * node_theta[q]), layout);
            nc += 2;
            push(o);
          }
        }
        AdjOp o{};
        o.type = A_CUT;
        o.coef = (uint16_t)nc;
        o.ncoef = (uint16_t)(nedges + 1);
        if (nc + nedges + 1 > ADJ_MAX_COEF) return QF_ERR_TOO_LARGE;
        for (int cv = 0; cv <= nedges; ++cv)
          P.coef[nc + cv] = make_coef(std::polar(1.0, -gamma[l] * (half_e - cv)), layout);
        nc += nedges + 1;
        push(o);
      }
      if (nops > ADJ_MAX_OPS) return QF_ERR_TOO_LARGE;
      P.nops = nops;
      switch (layout) {
        case C64: rc = launch_adj<C64>(P, grid, stream); break;
        case C128: rc = launch_adj<C128>(P, grid, stream); break;
        case FF: rc = launch_adj<FF>(P, grid, stream); break;
        default: rc = QF_ERR_LAYOUT;
      }
      if (rc) return rc;
    }
  }
  if (p == 0) {  // <C> only
    return reduce_diag(psi, n, layout, 1, cuts, nullptr, out + 2 * p, rows, stream);
  }
  k_rows_sum<<<nslots, 32, 0, stream>>>(rows, grid, nslots, out);
  return check_cuda(cudaGetLastError());
}

}  // namespace qf
