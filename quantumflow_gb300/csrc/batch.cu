// Batched QAOA MAXCUT: forward expectation and adjoint gradient of many
// independent instances (uneven qubit counts, graphs and depths) in one
// persistent launch.
//
// Each CTA takes instances from an atomic work counter (the host orders them
// largest first) and processes one instance at a time with all its threads:
//   - cut table c(x) = sum_e [x_a != x_b]   (quantumflow/qaoa.py:68-81)
//   - psi = |+>^n, then per layer: psi_x *= exp(i gamma (E/2 - c_x)) and
//     RX(beta) on every qubit             (quantumflow/qaoa.py:22-64)
//   - <C> = sum c |psi|^2, lambda = C psi, and the layers undone in reverse
//     on psi and lambda with the gradient reductions of the adjoint method
//     (see adjoint.cu for the formulas).
// Instances with n <= TS (tile bits) keep psi, lambda and c in shared memory
// for their whole life.  Larger instances keep them in the CTA's slice of
// global scratch and are processed in tiles of 2^TS amplitudes: pass A
// covers bits [0, TS), pass B bits [TS, n) plus the low bits that fill the
// tile.  Nothing waits on another CTA, so no launch-order assumptions exist.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "engine.cuh"
#include "state.cuh"

namespace qf {

struct BatchInstanceDev {
  int32_t n, p, nedges, edge_offset, angle_offset, out_offset;
};
static_assert(sizeof(BatchInstanceDev) == sizeof(qf_batch_instance), "layout mismatch");

constexpr int BATCH_MAX_EDGES = 1023;
constexpr int BATCH_THREADS = 256;
constexpr int BATCH_CLUSTER = 8;  // CTAs that share one large instance

// ---------------------------------------------------------- arithmetic ----
template <int LAY>
QF_D Coef coef_dev(double re, double im) {
  Coef c;
  if constexpr (LAY == C64) {
    c.f[0] = (float)re;
    c.f[1] = 0.f;
    c.f[2] = (float)im;
    c.f[3] = 0.f;
  } else {
    split_d(re, c.f[0], c.f[1]);
    split_d(im, c.f[2], c.f[3]);
  }
  return c;
}
// RX(theta) = [[c, -i s], [-i s, c]] with c = cos(theta/2), s = sin(theta/2)
QF_D void rx_pair(float2& a0, float2& a1, const Coef& c, const Coef& s) {
  const float cc = c.f[0], ss = s.f[0];
  const float2 b0 = a0, b1 = a1;
  a0 = make_float2(fmaf(cc, b0.x, ss * b1.y), fmaf(cc, b0.y, -ss * b1.x));
  a1 = make_float2(fmaf(cc, b1.x, ss * b0.y), fmaf(cc, b1.y, -ss * b0.x));
}
QF_D void ff2(float ah, float al, float bh, float bl, float ch, float cl, float dh, float dl, float& rh,
              float& rl) {  // (a*b + c*d) in float-float
  FFAcc t;
  t.zero();
  t.add_prod(ah, al, bh, bl);
  t.add_prod(ch, cl, dh, dl);
  t.finish(rh, rl);
}
QF_D void rx_pair(float4& a0, float4& a1, const Coef& c, const Coef& s) {
  const float ch = c.f[0], cl = c.f[1], sh = s.f[0], sl = s.f[1];
  const float4 b0 = a0, b1 = a1;
  ff2(ch, cl, b0.x, b0.y, sh, sl, b1.z, b1.w, a0.x, a0.y);    // c re0 + s im1
  ff2(ch, cl, b0.z, b0.w, -sh, -sl, b1.x, b1.y, a0.z, a0.w);  // c im0 - s re1
  ff2(ch, cl, b1.x, b1.y, sh, sl, b0.z, b0.w, a1.x, a1.y);
  ff2(ch, cl, b1.z, b1.w, -sh, -sl, b0.x, b0.y, a1.z, a1.w);
}
QF_D float2 cmulc(const Coef& c, float2 a) {
  const float ur = c.f[0], ui = c.f[2];
  return make_float2(fmaf(ur, a.x, -ui * a.y), fmaf(ur, a.y, ui * a.x));
}
QF_D float4 cmulc(const Coef& c, float4 a) {
  float4 r;
  ff2(c.f[0], c.f[1], a.x, a.y, -c.f[2], -c.f[3], a.z, a.w, r.x, r.y);
  ff2(c.f[0], c.f[1], a.z, a.w, c.f[2], c.f[3], a.x, a.y, r.z, r.w);
  return r;
}
QF_D float2 scalec(float2 a, float c) { return make_float2(a.x * c, a.y * c); }
QF_D float4 scalec(float4 a, float c) {
  float4 r;
  FFAcc t;
  t.zero();
  t.add_prod(c, 0.f, a.x, a.y);
  t.finish(r.x, r.y);
  t.zero();
  t.add_prod(c, 0.f, a.z, a.w);
  t.finish(r.z, r.w);
  return r;
}
// acc += w * Im(conj(l) p)
QF_D void imconj(FFAcc& acc, float2 l, float2 p, float w) {
  FFAcc t;
  t.zero();
  t.add_prod(l.x, 0.f, p.y, 0.f);
  t.add_prod(-l.y, 0.f, p.x, 0.f);
  acc.add_prod(w, 0.f, t.s, t.e);
}
QF_D void imconj(FFAcc& acc, float4 l, float4 p, float w) {
  FFAcc t;
  t.zero();
  t.add_prod(l.x, l.y, p.z, p.w);
  t.add_prod(-l.z, -l.w, p.x, p.y);
  acc.add_prod(w, 0.f, t.s, t.e);
}
QF_D void norm2acc(FFAcc& acc, float2 a, float w) {
  FFAcc t;
  t.zero();
  acc_norm2(t, a);
  acc.add_prod(w, 0.f, t.s, t.e);
}
QF_D void norm2acc(FFAcc& acc, float4 a, float w) {
  FFAcc t;
  t.zero();
  acc_norm2(t, a);
  acc.add_prod(w, 0.f, t.s, t.e);
}

// Block-wide sum of a float-float accumulator (all threads call; result on
// every thread).
QF_D double block_sum(const FFAcc& a, double* red) {
  double v = warp_sum((double)a.s + (double)a.e);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// ------------------------------------------------------------- passes ----
// One tile of 2^tb amplitudes of psi (sp) and lambda (sl) with cut values
// (sc) in shared memory; local bit j of the tile is global bit gpos[j].
struct TileOpsB {
  int tb;
  int nbits;       // mixer bits handled in this pass (local positions)
  int lbits[24];
  bool phase;      // forward: apply cost phase
  bool init;       // backward first pass: lambda = c psi, E reduction
  bool dual;       // lambda present
  int dir;         // +1 forward (RX(beta), phase), -1 backward (RX(-beta), phase^*)
};

template <typename E>
__device__ void tile_apply_b(const TileOpsB& T, E* sp, E* sl, const uint16_t* sc, const Coef* phase_tab,
                             const Coef& rc, const Coef& rs, float half_e, FFAcc& accx, FFAcc& acccut,
                             FFAcc& acce) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int N = 1 << T.tb;
  if (T.dir > 0) {
    if (T.phase) {
      for (int x = tid; x < N; x += nthr) sp[x] = cmulc(phase_tab[sc[x]], sp[x]);
      __syncthreads();
    }
    for (int i = 0; i < T.nbits; ++i) {
      const int q = T.lbits[i], bit = 1 << q;
      for (int pr = tid; pr < (N >> 1); pr += nthr) {
        const int i0 = ((pr >> q) << (q + 1)) | (pr & (bit - 1));
        rx_pair(sp[i0], sp[i0 | bit], rc, rs);
      }
      __syncthreads();
    }
    return;
  }
  if (T.init) {
    for (int x = tid; x < N; x += nthr) {
      const float c = (float)sc[x];
      const E v = sp[x];
      sl[x] = scalec(v, c);
      norm2acc(acce, v, c);
    }
    __syncthreads();
  }
  // mixer gradient terms for this pass's bits, then undo RX on them.  In
  // FP32 arithmetic each thread sums its few pairs of one bit in FP32 and
  // folds the partial into the compensated accumulator once per bit.
  for (int i = 0; i < T.nbits; ++i) {
    const int q = T.lbits[i], bit = 1 << q;
    if constexpr (sizeof(E) == sizeof(float2)) {
      float part = 0.f;
      for (int pr = tid; pr < (N >> 1); pr += nthr) {
        const int i0 = ((pr >> q) << (q + 1)) | (pr & (bit - 1));
        const float2 l0 = sl[i0], l1 = sl[i0 | bit], p0 = sp[i0], p1 = sp[i0 | bit];
        part = fmaf(l0.x, p1.y, part);
        part = fmaf(-l0.y, p1.x, part);
        part = fmaf(l1.x, p0.y, part);
        part = fmaf(-l1.y, p0.x, part);
      }
      accx.add(part, 0.f);
    } else {
      for (int pr = tid; pr < (N >> 1); pr += nthr) {
        const int i0 = ((pr >> q) << (q + 1)) | (pr & (bit - 1));
        imconj(accx, sl[i0], sp[i0 | bit], 1.f);
        imconj(accx, sl[i0 | bit], sp[i0], 1.f);
      }
    }
  }
  __syncthreads();
  for (int i = 0; i < T.nbits; ++i) {
    const int q = T.lbits[i], bit = 1 << q;
    for (int pr = tid; pr < (N >> 1); pr += nthr) {
      const int i0 = ((pr >> q) << (q + 1)) | (pr & (bit - 1));
      rx_pair(sp[i0], sp[i0 | bit], rc, rs);
      rx_pair(sl[i0], sl[i0 | bit], rc, rs);
    }
    __syncthreads();
  }
  if (T.phase) {  // cost-layer gradient, then undo the phase
    float part = 0.f;
    for (int x = tid; x < N; x += nthr) {
      const float c = (float)sc[x];
      if constexpr (sizeof(E) == sizeof(float2)) {
        const float2 l = sl[x], v = sp[x];
        part = fmaf(half_e - c, fmaf(l.x, v.y, -l.y * v.x), part);
      } else {
        imconj(acccut, sl[x], sp[x], half_e - c);
      }
      sp[x] = cmulc(phase_tab[sc[x]], sp[x]);
      sl[x] = cmulc(phase_tab[sc[x]], sl[x]);
    }
    if constexpr (sizeof(E) == sizeof(float2)) acccut.add(part, 0.f);
    __syncthreads();
  }
}

struct BatchParams {
  const BatchInstanceDev* inst;
  int ninst;
  int nlarge;            // instances [0, nlarge) are processed by whole clusters
  const uint8_t* edges;  // axis pairs
  const double* angles;  // per instance: beta[p], gamma[p]
  double* out;           // per instance: dgamma[p], dbeta[p], <C>
  char* scratch;         // per CTA: psi, lambda, cuts for n > TS
  size_t scratch_per_cta;
  int* counter;          // [0]: large-instance queue, [1]: the rest
  int ts;                // tile bits
  int max_n;             // scratch is sized for this many qubits
  int* error;            // device error word (bit 1: malformed instance skipped)
};

namespace cg = cooperative_groups;

// One instance, processed by `csize` CTAs of a cluster (csize == 1: this CTA
// alone).  All CTAs of the group call it with the same idx.
template <int LAY>
__device__ void run_instance(const BatchParams& B, int idx, int crank, int csize, typename Types<LAY>::E* sp,
                             typename Types<LAY>::E* sl, uint16_t* sc, Coef* tab, double* red, uint8_t* s_edges,
                             double* part, char* scratch) {
  using E = typename Types<LAY>::E;
  const int TS = B.ts;
  const int NT = 1 << TS;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const bool coop = csize > 1;
  cg::cluster_group cluster = cg::this_cluster();
  auto group_sync = [&]() {
    if (coop) cluster.sync();
    else __syncthreads();
  };
  __shared__ int s_bad;
  const BatchInstanceDev I = B.inst[idx];
  const int n = I.n, p = I.p, ne = I.nedges;
  // a malformed instance is skipped: NaN outputs and the error word
  if (tid == 0)
    s_bad = n < 1 || n > B.max_n || n > 2 * TS || p < 0 || p > 64 || ne < 0 || ne > BATCH_MAX_EDGES;
  __syncthreads();
  for (int e = tid; e < 2 * ne && !s_bad; e += nthr)
    if (B.edges[2 * I.edge_offset + e] >= n) s_bad = 1;
  __syncthreads();
  if (s_bad) {
    if (tid == 0 && crank == 0) {
      if (p >= 0 && p <= 64)
        for (int k = 0; k <= 2 * p; ++k) B.out[I.out_offset + k] = __longlong_as_double(0x7ff8000000000000ll);
      atomicOr(B.error, 2);
    }
    group_sync();
    return;
  }
  const int64_t namps = int64_t(1) << n;
  for (int e = tid; e < 2 * ne; e += nthr) s_edges[e] = (uint8_t)(n - 1 - B.edges[2 * I.edge_offset + e]);
  __syncthreads();
  const double* beta = B.angles + I.angle_offset;
  const double* gamma = beta + p;
  const float half_e = 0.5f * ne;
  const bool small = n <= TS;
  E* gp = reinterpret_cast<E*>(scratch);
  E* gl = gp + namps;
  uint16_t* gc = reinterpret_cast<uint16_t*>(gl + namps);

  const E plus = [&] {
    const double a = 1.0 / sqrt((double)namps);
    if constexpr (LAY == C64) return make_float2((float)a, 0.f);
    else {
      float h, l;
      split_d(a, h, l);
      return make_float4(h, l, 0.f, 0.f);
    }
  }();
  for (int64_t x = (int64_t)crank * nthr + tid; x < namps; x += (int64_t)csize * nthr) {
    unsigned c = 0;
    for (int e = 0; e < ne; ++e) c += (unsigned)(((x >> s_edges[2 * e]) ^ (x >> s_edges[2 * e + 1])) & 1);
    if (small) {
      sc[x] = (uint16_t)c;
      sp[x] = plus;
    } else {
      gc[x] = (uint16_t)c;
      gp[x] = plus;
    }
  }
  group_sync();

  const int hcount = small ? 0 : n - TS;
  const int lowB = TS - hcount;
  auto pass = [&](bool passA, const TileOpsB& T, const Coef& rc, const Coef& rs, FFAcc& ax, FFAcc& acut,
                  FFAcc& ae) {
    if (small) {
      tile_apply_b<E>(T, sp, sl, sc, tab, rc, rs, half_e, ax, acut, ae);
      return;
    }
    const int64_t ntile = int64_t(1) << (n - TS);
    for (int64_t t = crank; t < ntile; t += csize) {
      for (int l = tid; l < NT; l += nthr) {
        int64_t x;
        if (passA) x = (t << TS) | l;
        else x = (int64_t(l >> lowB) << TS) | (t << lowB) | (l & ((1 << lowB) - 1));
        sp[l] = gp[x];
        if (T.dual && !T.init) sl[l] = gl[x];
        sc[l] = gc[x];
      }
      __syncthreads();
      tile_apply_b<E>(T, sp, sl, sc, tab, rc, rs, half_e, ax, acut, ae);
      for (int l = tid; l < NT; l += nthr) {
        int64_t x;
        if (passA) x = (t << TS) | l;
        else x = (int64_t(l >> lowB) << TS) | (t << lowB) | (l & ((1 << lowB) - 1));
        gp[x] = sp[l];
        if (T.dual) gl[x] = sl[l];
      }
      __syncthreads();
    }
    group_sync();
  };
  auto fill_phase = [&](double g, int sign) {
    for (int c = tid; c <= ne; c += nthr) {
      double sn, cs;
      sincos(sign * g * (0.5 * ne - c), &sn, &cs);
      tab[c] = coef_dev<LAY>(cs, sn);
    }
    __syncthreads();
  };
  auto rx_coefs = [&](double b, Coef& rc, Coef& rs) {
    rc = coef_dev<LAY>(cos(0.5 * b), 0.0);
    rs = coef_dev<LAY>(sin(0.5 * b), 0.0);
  };
  // sum of a per-CTA value over the group, delivered to rank 0
  auto group_total = [&](double v, int slot) -> double {
    if (!coop) return v;
    if (tid == 0) part[slot] = v;
    cluster.sync();
    double s = 0.0;
    if (crank == 0 && tid == 0)
      for (int r = 0; r < csize; ++r) s += *cluster.map_shared_rank(&part[slot], r);
    cluster.sync();
    return s;
  };

  // ---- forward
  FFAcc dummy;
  dummy.zero();
  for (int l = 0; l < p; ++l) {
    fill_phase(gamma[l], +1);
    Coef rc, rs;
    rx_coefs(beta[l], rc, rs);
    TileOpsB T{};
    T.dir = 1;
    T.dual = false;
    if (small) {
      T.tb = n;
      T.phase = true;
      T.nbits = n;
      for (int b = 0; b < n; ++b) T.lbits[b] = b;
      pass(true, T, rc, rs, dummy, dummy, dummy);
    } else {
      T.tb = TS;
      T.phase = true;
      T.nbits = TS;
      for (int b = 0; b < TS; ++b) T.lbits[b] = b;
      pass(true, T, rc, rs, dummy, dummy, dummy);
      T.phase = false;
      T.nbits = hcount;
      for (int b = 0; b < hcount; ++b) T.lbits[b] = lowB + b;
      pass(false, T, rc, rs, dummy, dummy, dummy);
    }
  }
  // ---- backward (adjoint)
  double* o = B.out + I.out_offset;
  FFAcc ae;
  ae.zero();
  bool first = true;
  for (int l = p - 1; l >= 0; --l) {
    fill_phase(gamma[l], -1);
    Coef rc, rs;
    rx_coefs(-beta[l], rc, rs);
    FFAcc ax, acut;
    ax.zero();
    acut.zero();
    TileOpsB T{};
    T.dir = -1;
    T.dual = true;
    if (small) {
      T.tb = n;
      T.init = first;
      T.phase = true;
      T.nbits = n;
      for (int b = 0; b < n; ++b) T.lbits[b] = b;
      pass(true, T, rc, rs, ax, acut, ae);
    } else {
      T.tb = TS;
      T.init = first;
      T.phase = false;
      T.nbits = hcount;
      for (int b = 0; b < hcount; ++b) T.lbits[b] = lowB + b;
      pass(false, T, rc, rs, ax, acut, ae);
      T.init = false;
      T.phase = true;
      T.nbits = TS;
      for (int b = 0; b < TS; ++b) T.lbits[b] = b;
      pass(true, T, rc, rs, ax, acut, ae);
    }
    first = false;
    const double gx = group_total(block_sum(ax, red), 0);
    const double gc2 = group_total(block_sum(acut, red), 1);
    if (tid == 0 && crank == 0) {
      o[p + l] = gx;
      o[l] = -2.0 * gc2;
    }
  }
  if (p == 0) {
    for (int64_t x = (int64_t)crank * nthr + tid; x < namps; x += (int64_t)csize * nthr)
      norm2acc(ae, small ? sp[x] : gp[x], (float)(small ? sc[x] : gc[x]));
  }
  const double e = group_total(block_sum(ae, red), 2);
  if (tid == 0 && crank == 0) o[2 * p] = e;
  __syncthreads();
}

template <int LAY>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch(const __grid_constant__ BatchParams B) {
  using E = typename Types<LAY>::E;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TS = B.ts;
  const int NT = 1 << TS;
  E* sp = reinterpret_cast<E*>(smem_raw);
  E* sl = sp + NT;
  uint16_t* sc = reinterpret_cast<uint16_t*>(sl + NT);
  Coef* tab = reinterpret_cast<Coef*>(sc + NT);  // BATCH_MAX_EDGES + 1 entries
  __shared__ double red[32];
  __shared__ double part[4];
  __shared__ int s_item;
  __shared__ uint8_t s_edges[2 * BATCH_MAX_EDGES];
  const int tid = threadIdx.x;
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank();
  const int csize = (int)cluster.num_blocks();
  // the cluster leader's scratch slice holds a cooperative instance
  const size_t cl_first = blockIdx.x - crank;
  char* lead_scratch = B.scratch + cl_first * B.scratch_per_cta;
  char* own_scratch = B.scratch + (size_t)blockIdx.x * B.scratch_per_cta;

  // phase 1: large instances, one cluster each
  if (B.nlarge > 0) {
    for (;;) {
      if (crank == 0 && tid == 0) s_item = atomicAdd(&B.counter[0], 1);
      cluster.sync();
      const int item = *cluster.map_shared_rank(&s_item, 0);
      cluster.sync();
      if (item >= B.nlarge) break;
      run_instance<LAY>(B, item, crank, csize, sp, sl, sc, tab, red, s_edges, part, lead_scratch);
    }
  }
  // phase 2: everything else, one CTA each
  for (;;) {
    if (tid == 0) s_item = B.nlarge + atomicAdd(&B.counter[1], 1);
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= B.ninst) break;
    run_instance<LAY>(B, idx, 0, 1, sp, sl, sc, tab, red, s_edges, part, own_scratch);
  }
}

size_t batch_smem_bytes(int layout, int ts) {
  const size_t NT = size_t(1) << ts;
  return NT * 2 * elem_bytes(layout) + NT * 2 + (BATCH_MAX_EDGES + 1) * sizeof(Coef);
}

size_t batch_workspace_bytes(int max_n, int layout, int ctas) {
  const size_t amps = size_t(1) << max_n;
  const size_t per = ((amps * (2 * elem_bytes(layout) + 2)) + 255) & ~size_t(255);
  return 256 + per * (size_t)ctas;
}

int* device_error_word();

int batch_qaoa(const qf_batch_instance* inst, int ninst, int nlarge, const uint8_t* edges, const double* angles,
               double* out, int layout, int max_n, int ts, int ctas, void* ws, size_t ws_bytes,
               cudaStream_t stream) {
  BatchParams B;
  std::memset(&B, 0, sizeof(B));
  B.max_n = max_n;
  B.error = device_error_word();
  if (B.error == nullptr) return QF_ERR_CUDA;
  B.inst = reinterpret_cast<const BatchInstanceDev*>(inst);
  B.ninst = ninst;
  B.nlarge = nlarge;
  B.edges = edges;
  B.angles = angles;
  B.out = out;
  B.counter = reinterpret_cast<int*>(ws);
  B.scratch = reinterpret_cast<char*>(ws) + 256;
  const size_t amps = size_t(1) << max_n;
  B.scratch_per_cta = ((amps * (2 * elem_bytes(layout) + 2)) + 255) & ~size_t(255);
  B.ts = ts;
  if (ws_bytes < batch_workspace_bytes(max_n, layout, ctas)) return QF_ERR_WORKSPACE;
  int rc = check_cuda(cudaMemsetAsync(B.counter, 0, 2 * sizeof(int), stream));
  if (rc) return rc;
  const size_t smem = batch_smem_bytes(layout, ts);
  static std::atomic<bool> attr[2][64];
  int dev = 0;
  cudaGetDevice(&dev);
  void (*kern)(BatchParams) = layout == C64 ? k_batch<C64> : k_batch<FF>;
  const int li = layout == C64 ? 0 : 1;
  if (layout != C64 && layout != FF) return QF_ERR_LAYOUT;
  if (dev < 64 && !attr[li][dev].load()) {
    rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    if (rc) return rc;
    rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    if (rc) return rc;
    attr[li][dev].store(true);
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(BATCH_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = BATCH_CLUSTER;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  rc = check_cuda(cudaLaunchKernelEx(&cfg, kern, B));
  return rc;
}

}  // namespace qf
