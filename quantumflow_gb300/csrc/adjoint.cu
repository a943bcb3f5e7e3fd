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

QF_D float2 cmulv(const Coef& c, float2 a) {
  const float ur = c.f[0], ui = c.f[2];
  return make_float2(fmaf(ur, a.x, -ui * a.y), fmaf(ur, a.y, ui * a.x));
}
QF_D double2 cmulv(const Coef& c, double2 a) {
  const double ur = c.d[0], ui = c.d[1];
  return make_double2(fma(ur, a.x, -ui * a.y), fma(ur, a.y, ui * a.x));
}
QF_D float4 cmulv(const Coef& c, float4 a) {
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
QF_D float4 scale_ff(float4 a, float c) {  // exact-product scaling by a small integer-valued float
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
QF_D float2 scale_ff(float2 a, float c) { return make_float2(a.x * c, a.y * c); }
QF_D double2 scale_ff(double2 a, float c) { return make_double2(a.x * (double)c, a.y * (double)c); }

// acc += w * Im(conj(l) * p), with Im(conj(l) p) formed in float-float
// first and then multiplied by w exactly (w is a small half-integer).
QF_D void acc_imconj(FFAcc& acc, float4 l, float4 p, float w) {
  FFAcc t;
  t.zero();
  t.add_prod(l.x, l.y, p.z, p.w);
  t.add_prod(-l.z, -l.w, p.x, p.y);
  if (w == 1.f) {
    acc.add(t.s, t.e);
  } else {
    acc.add_prod(w, 0.f, t.s, t.e);
  }
}
QF_D void acc_imconj(FFAcc& acc, float2 l, float2 p, float w) {
  FFAcc t;
  t.zero();
  t.add_prod(l.x, 0.f, p.y, 0.f);
  t.add_prod(-l.y, 0.f, p.x, 0.f);
  acc.add_prod(w, 0.f, t.s, t.e);
}
QF_D void acc_imconj(FFAcc& acc, double2 l, double2 p, float w) {
  acc_imconj(acc, to_ff(l), to_ff(p), w);
}

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
            sp[l] = cmulv(cf[c], sp[l]);
            sl[l] = cmulv(cf[c], sl[l]);
          }
          break;
        }
        case A_DIAG1: {
          for (int l = tid; l < T; l += nthr) {
            const int64_t x = adj_global(P, base, l);
            const Coef& c = cf[(x >> op.gb) & 1];
            sp[l] = cmulv(c, sp[l]);
            sl[l] = cmulv(c, sl[l]);
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

__global__ void k_rows_sum(const double* rows, int nrows, int nslots, double* out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslots; s += gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int r = 0; r < nrows; ++r) v += rows[(size_t)r * nslots + s];
    out[s] = v;
  }
}

void qaoa_layer_ops(int n, const uint16_t* cuts, int nedges, double beta, double gamma,
                    const double* node_theta, std::vector<HostOp>& ops);

int adj_grid(int n, int layout) {
  const int TB = layout == C64 ? 11 : 10;
  const int tb = n < TB ? n : TB;
  const int64_t ntiles = int64_t(1) << (n - tb);
  int64_t g = device_sm_count();
  if (g > ntiles) g = (int)ntiles;
  return (int)g;
}

size_t qaoa_grad_workspace_bytes(int n, int p, int layout) {
  const size_t amps = size_t(1) << n;
  const int nslots = 2 * p + 1;
  return amps * elem_bytes(layout) + (size_t)adj_grid(n, layout) * nslots * sizeof(double) + 256;
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
  k_rows_sum<<<1, 64, 0, stream>>>(rows, grid, nslots, out);
  return check_cuda(cudaGetLastError());
}

}  // namespace qf
