// QAOA on the gate engine: the qubo_circuit of quantumflow/qaoa.py:22-64 as
// fused passes.  The cost layer prod_e ZZ(-gamma/pi) of an unweighted graph
// is exp(i*gamma*(E/2 - C(x))) (quantumflow/stdgates.py ZZ: diag
// cis(-pi t/2), cis(pi t/2), cis(pi t/2), cis(-pi t/2)), i.e. one diagonal
// phase per amplitude looked up by its cut value C(x).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "state.cuh"

namespace qf {

void qaoa_layer_ops(int n, const uint16_t* cuts, int nedges, double beta, double gamma,
                    const double* node_theta, std::vector<HostOp>& ops) {
  HostOp cut;
  cut.type = OP_CUT;
  cut.k = 0;
  cut.cuts = cuts;
  cut.table.resize(nedges + 1);
  for (int c = 0; c <= nedges; ++c) cut.table[c] = std::polar(1.0, gamma * (0.5 * nedges - c));
  ops.push_back(cut);
  if (node_theta != nullptr) {
    for (int q = 0; q < n; ++q) {
      const double th = node_theta[q];
      if (std::isnan(th)) continue;
      HostOp rz;  // RZ(theta) = diag(exp(-i theta/2), exp(i theta/2))
      rz.type = OP_DIAG;
      rz.k = 1;
      rz.gb[0] = n - 1 - q;
      rz.diag = {std::polar(1.0, -0.5 * th), std::polar(1.0, 0.5 * th)};
      ops.push_back(rz);
    }
  }
  const double c = std::cos(0.5 * beta), s = std::sin(0.5 * beta);
  for (int q = 0; q < n; ++q) {  // RX(beta) = [[c, -is], [-is, c]]
    HostOp rx;
    rx.type = OP_DENSE1;
    rx.k = 1;
    rx.gb[0] = n - 1 - q;
    rx.m = {cplx(c, 0), cplx(0, -s), cplx(0, -s), cplx(c, 0)};
    ops.push_back(rx);
  }
}

// ------------------------------------------------ warp-tile QAOA passes --
// A warp owns a sub-tile of 32 lanes (global bits 0..4) x 2^RB registers
// (RB high bits chosen per pass), prefetched two sub-tiles ahead into a
// per-warp shared-memory ring with per-thread async copies.  A pass runs
// stage A, the mixer RX(beta_A) on the register bits of a group, then
// optionally stage B, the next layer's cost layer (cut phase, node phases)
// and its mixer on the lane bits and the same register bits.  With the
// group order reversed on alternate layers a layer boundary costs no extra
// pass: p layers over m groups take 1 + p (m - 1) passes.
constexpr int QW_MAX_COEF = 1100;
constexpr int QW_STAGES = 2;

struct QaoaWParams {
  void* psi;
  const uint16_t* cuts;
  int32_t n;
  int32_t init;   // the pass generates |+>^n instead of loading psi
  int32_t nactA;  // stage A on register bits 0..nactA-1 (0: no stage A)
  int32_t hasB;   // stage B present
  int32_t nactB;
  int32_t ndiag, ncut;
  uint8_t hb[4];  // global bit of each register index bit
  uint8_t hs[4];  // the same bits in ascending order
  uint8_t diag_bit[QF_MAX_QUBITS];
  Coef amp0;               // 2^(-n/2)
  Coef a_c, a_s, b_c, b_s;  // RX(beta) = [[c, i s], [i s, c]] with s = -sin(beta/2)
  Coef coef[QW_MAX_COEF];   // stage B: node phase pairs, then the cut table
};

template <int LAY, int RB>
constexpr size_t qw_ring_bytes() {
  return (size_t)8 * QW_STAGES * (32 << RB) * sizeof(typename Types<LAY>::E);
}

template <int RB, typename E>
QF_D void rx_regs(const Coef& c, const Coef& s, int nact, E (&a)[1 << RB]) {
#pragma unroll
  for (int j = 0; j < RB; ++j) {
    if (j < nact) {
#pragma unroll
      for (int i = 0; i < (1 << (RB - 1)); ++i) {
        const int i0 = ((i >> j) << (j + 1)) | (i & ((1 << j) - 1));
        const int i1 = i0 | (1 << j);
        const E a0 = a[i0];
        a[i0] = rx_one(c, s, a0, a[i1]);
        a[i1] = rx_one(c, s, a[i1], a0);
      }
    }
  }
}

template <int LAY, int RB>
__global__ void __launch_bounds__(256) k_qaoaw(const __grid_constant__ QaoaWParams P) {
  using E = typename Types<LAY>::E;
  constexpr int R = 1 << RB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Coef* scoef = reinterpret_cast<Coef*>(smem_raw);
  const int necoef = P.hasB ? 2 * P.ndiag + P.ncut : 0;
  for (int i = threadIdx.x; i < necoef; i += blockDim.x) scoef[i] = P.coef[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  E* ring = reinterpret_cast<E*>(smem_raw + (((size_t)necoef * sizeof(Coef) + 127) & ~size_t(127))) +
            (size_t)warp * QW_STAGES * R * 32;
  const int64_t nsub = int64_t(1) << (P.n - 5 - RB);
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  E* gp = reinterpret_cast<E*>(P.psi);
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
  auto issue = [&](int64_t st, int sg) {
    if (!P.init && st < nsub) {
      const int64_t xb = sub_base(st);
      E* sp = ring + (size_t)sg * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) cp_async_amp(sp + r * 32, gp + (xb | hoff[r]));
    }
    cp_async_commit();
  };
  E* tag = nullptr;
  const E amp0 = coef_e(P.amp0, tag);
  int64_t st = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < QW_STAGES - 1; ++k) issue(st + k * wstride, k);
  int sg = 0;
  for (; st < nsub; st += wstride) {
    cp_async_wait<QW_STAGES - 2>();
    const int64_t xb = sub_base(st);
    E a[R];
    if (P.init) {
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = amp0;
    } else {
      const E* sp = ring + (size_t)sg * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = sp[r * 32];
    }
    issue(st + (QW_STAGES - 1) * wstride, sg == 0 ? QW_STAGES - 1 : sg - 1);
    sg = sg + 1 == QW_STAGES ? 0 : sg + 1;

    rx_regs<RB>(P.a_c, P.a_s, P.nactA, a);
    if (P.hasB) {
      const Coef* tab = scoef + 2 * P.ndiag;
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = cmul_v(tab[min((int)P.cuts[xb | hoff[r]], P.ncut - 1)], a[r]);
      for (int d = 0; d < P.ndiag; ++d) {
        const int gb = P.diag_bit[d];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = cmul_v(scoef[2 * d + (((xb | hoff[r]) >> gb) & 1)], a[r]);
      }
      const Coef bc = P.b_c, bs = P.b_s;
      for (int b = 0; b < 5; ++b) {
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = rx_one(bc, bs, a[r], shfl_xor(a[r], 1 << b));
      }
      rx_regs<RB>(bc, bs, P.nactB, a);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) gp[xb | hoff[r]] = a[r];
  }
  cp_async_wait<0>();
}

extern int g_force_smem_tile;
extern int g_warp_rb_override;

// register bits of k_qaoaw: 2 or 3 for FP64/float-float, 3 or 4 for complex64
static int qw_rb(int layout) {
  const int o = g_warp_rb_override;
  if (layout == C64) return (o == 3 || o == 4) ? o : 4;
  return (o == 2 || o == 3) ? o : 3;
}

template <int LAY, int RB>
static int launch_qw(QaoaWParams& P, cudaStream_t stream) {
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_qaoaw<LAY, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(qw_ring_bytes<LAY, RB>() + QW_MAX_COEF * sizeof(Coef) + 128)));
    if (rc) return rc;
    attr[dev].store(true);
  }
  const size_t necoef = P.hasB ? (size_t)(2 * P.ndiag + P.ncut) : 0;
  const size_t smem = ((necoef * sizeof(Coef) + 127) & ~size_t(127)) + qw_ring_bytes<LAY, RB>();
  const int64_t nsub = int64_t(1) << (P.n - 5 - RB);
  int64_t grid = (nsub + 7) / 8;
  const int64_t cap = (int64_t)device_sm_count() * 4;
  if (grid > cap) grid = cap;
  k_qaoaw<LAY, RB><<<(int)grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

static int qaoa_state_warp(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p,
                           const double* beta, const double* gamma, const double* node_theta, int RB,
                           cudaStream_t stream) {
  static thread_local QaoaWParams P;
  std::memset(&P, 0, sizeof(P));
  P.psi = psi;
  P.cuts = cuts;
  P.n = n;
  P.amp0 = make_coef(cplx(std::ldexp(1.0, -n / 2) / ((n & 1) ? std::sqrt(2.0) : 1.0), 0.0), layout);
  int nd = 0;
  if (node_theta != nullptr) {
    for (int q = 0; q < n; ++q) {
      if (std::isnan(node_theta[q])) continue;
      P.diag_bit[nd] = (uint8_t)(n - 1 - q);
      P.coef[2 * nd] = make_coef(std::polar(1.0, -0.5 * node_theta[q]), layout);  // RZ(theta)
      P.coef[2 * nd + 1] = make_coef(std::polar(1.0, 0.5 * node_theta[q]), layout);
      ++nd;
    }
  }
  P.ndiag = nd;
  P.ncut = nedges + 1;
  if (2 * nd + P.ncut > QW_MAX_COEF) return QF_ERR_TOO_LARGE;
  std::vector<std::vector<int>> groups;
  for (int b = 5; b < n; b += RB) {
    std::vector<int> g;
    for (int k = b; k < std::min(n, b + RB); ++k) g.push_back(k);
    groups.push_back(g);
  }
  const int m = (int)groups.size();
  auto order = [&](int l, int k) { return (l & 1) ? m - 1 - k : k; };
  auto set_group = [&](int gi) {
    std::vector<int> hb = groups[gi];
    for (int b = 5; b < n && (int)hb.size() < RB; ++b)
      if (std::find(hb.begin(), hb.end(), b) == hb.end()) hb.push_back(b);
    for (int j = 0; j < RB; ++j) P.hb[j] = (uint8_t)hb[j];
    std::sort(hb.begin(), hb.end());
    for (int j = 0; j < RB; ++j) P.hs[j] = (uint8_t)hb[j];
    return (int)groups[gi].size();
  };
  auto rx = [&](int l, Coef& c, Coef& s) {
    c = make_coef(cplx(std::cos(0.5 * beta[l]), 0.0), layout);
    s = make_coef(cplx(-std::sin(0.5 * beta[l]), 0.0), layout);
  };
  auto stage_b = [&](int l, int nact) {
    P.hasB = 1;
    P.nactB = nact;
    rx(l, P.b_c, P.b_s);
    for (int cv = 0; cv <= nedges; ++cv)
      P.coef[2 * nd + cv] = make_coef(std::polar(1.0, gamma[l] * (0.5 * nedges - cv)), layout);
  };
  auto launch = [&]() {
    switch (layout * 8 + RB) {
      case C64 * 8 + 3: return launch_qw<C64, 3>(P, stream);
      case C64 * 8 + 4: return launch_qw<C64, 4>(P, stream);
      case C128 * 8 + 2: return launch_qw<C128, 2>(P, stream);
      case C128 * 8 + 3: return launch_qw<C128, 3>(P, stream);
      case FF * 8 + 2: return launch_qw<FF, 2>(P, stream);
      case FF * 8 + 3: return launch_qw<FF, 3>(P, stream);
    }
    return (int)QF_ERR_LAYOUT;
  };
  // first pass: |+>^n, layer 0's cost layer and mixer on lanes + group order(0, 0)
  P.init = 1;
  P.nactA = 0;
  stage_b(0, set_group(order(0, 0)));
  int rc = launch();
  if (rc) return rc;
  P.init = 0;
  for (int l = 0; l < p; ++l) {
    if (m == 1) {
      if (l == 0) continue;
      P.nactA = 0;
      stage_b(l, set_group(0));
      if ((rc = launch())) return rc;
      continue;
    }
    for (int k = 1; k < m; ++k) {
      const int nact = set_group(order(l, k));
      P.nactA = nact;
      rx(l, P.a_c, P.a_s);
      P.hasB = 0;
      if (k == m - 1 && l + 1 < p) stage_b(l + 1, nact);  // order(l+1, 0) == order(l, m-1)
      if ((rc = launch())) return rc;
    }
  }
  return QF_OK;
}

int qaoa_state(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p, const double* beta,
               const double* gamma, const double* node_theta, int fusion_k, cudaStream_t stream) {
  const int RB = qw_rb(layout);
  if (p > 0 && fusion_k == 0 && !g_force_smem_tile && n >= 5 + RB && nedges + 1 + 2 * n <= QW_MAX_COEF)
    return qaoa_state_warp(psi, n, layout, cuts, nedges, p, beta, gamma, node_theta, RB, stream);
  int rc = fill_uniform(psi, n, layout, stream);
  if (rc) return rc;
  std::vector<HostOp> ops;
  for (int l = 0; l < p; ++l) qaoa_layer_ops(n, cuts, nedges, beta[l], gamma[l], node_theta, ops);
  if (ops.empty()) return QF_OK;
  return run_ops(psi, psi, n, layout, ops, fusion_k, stream, nullptr);
}

}  // namespace qf
