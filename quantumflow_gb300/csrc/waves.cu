// Multi-instance QAOA passes ("waves") for the large instances of a batch.
//
// Each instance keeps psi, lambda and its uint16 cut table in its own region
// of the caller's device workspace.  Its forward sweep and adjoint sweep are
// the pass sequences of the single-instance warp-tile kernels (qaoa.cu
// k_qaoaw, adjoint.cu k_adjw): warp sub-tiles of 32 lanes x 2^RB registers
// prefetched through a per-warp async-copy ring, layer boundaries merged into
// one pass.  Wave w launches the w-th pass of every instance that has
// one -- forward items in one launch, adjoint items in another -- so one
// launch covers all instances and the launch count is the longest
// instance's pass count, whatever the batch size.  Every launch reads its
// angles-dependent coefficients (RX cos/sin, cut-phase tables) from device
// tables that one small kernel refreshes from the angle array, so the whole
// evaluation replays from a CUDA graph while the angles change on the
// device.  Gradient partial sums go to one row per adjoint block; a final
// kernel adds each output's rows in a fixed order (deterministic).
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "state.cuh"

namespace qf {

constexpr int WV_MAX_EDGES = 1023;

struct WvInst {           // per instance, device copy
  int64_t psi, lam;       // element offsets in the state region
  int64_t cuts;           // element offset in the cut region
  int64_t tab;            // Coef offset of this instance's tables
  int32_t n, p, nedges, edge_offset, angle_offset, out_offset;
};
struct WvFwd {            // one forward pass of one instance
  int32_t inst, block_begin;
  int8_t init, nactA, hasB, nactB;
  int16_t layerA, layerB;
  uint8_t hb[4], hs[4];
};
struct WvAdj {            // one adjoint pass of one instance
  int32_t inst, block_begin, prow;
  int8_t init, lanes, nact, last, hasB, nactB;
  int16_t layer;
  uint8_t hb[4], hs[4];
};
struct WvSeg {            // out[o] += sum of rows [row, row + nrows) column k
  int32_t row, nrows, k, pad;
};

// Coefficient tables of one instance (Coef units), at WvInst::tab:
//   [l * 3 + 0] cos(beta_l / 2), [+1] -sin(beta_l / 2), [+2] +sin(beta_l / 2)
//   then p forward cut tables exp(+i gamma_l (E/2 - c)), then p adjoint ones
//   exp(-i gamma_l (E/2 - c)), each E + 1 entries.
static inline int64_t wv_tab_size(int p, int nedges) { return (int64_t)p * 3 + 2 * (int64_t)p * (nedges + 1); }

template <int LAY>
QF_D Coef wv_coef(double re, double im) {
  Coef c;
  if constexpr (LAY == C64) {
    c.f[0] = (float)re;
    c.f[1] = 0.f;
    c.f[2] = (float)im;
    c.f[3] = 0.f;
  } else if constexpr (LAY == C128) {
    c.d[0] = re;
    c.d[1] = im;
  } else {
    split_d(re, c.f[0], c.f[1]);
    split_d(im, c.f[2], c.f[3]);
  }
  return c;
}

// cut values of every instance (once per batch)
__global__ void k_wave_cuts(const WvInst* inst, int ninst, const uint8_t* edges, uint16_t* cuts) {
  const int i = blockIdx.y;
  if (i >= ninst) return;
  const WvInst I = inst[i];
  __shared__ uint8_t se[2 * WV_MAX_EDGES];
  const int ne = min(I.nedges, WV_MAX_EDGES);
  for (int e = threadIdx.x; e < 2 * ne; e += blockDim.x) se[e] = (uint8_t)(I.n - 1 - edges[2 * I.edge_offset + e]);
  __syncthreads();
  const int64_t namps = int64_t(1) << I.n;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += (int64_t)gridDim.x * blockDim.x) {
    unsigned c = 0;
    for (int e = 0; e < ne; ++e) c += (unsigned)(((x >> se[2 * e]) ^ (x >> se[2 * e + 1])) & 1);
    cuts[I.cuts + x] = (uint16_t)c;
  }
}

// angle-dependent tables of every instance (once per evaluation)
template <int LAY>
__global__ void k_wave_coefs(const WvInst* inst, int ninst, const double* angles, Coef* tab, const int32_t* skip) {
  const int i = blockIdx.x;
  if (i >= ninst || (skip != nullptr && skip[i] != 0)) return;
  const WvInst I = inst[i];
  const double* beta = angles + I.angle_offset;
  const double* gamma = beta + I.p;
  Coef* t = tab + I.tab;
  const int E1 = I.nedges + 1;
  for (int l = threadIdx.x; l < I.p; l += blockDim.x) {
    double s, c;
    sincos(0.5 * beta[l], &s, &c);
    t[3 * l] = wv_coef<LAY>(c, 0.0);
    t[3 * l + 1] = wv_coef<LAY>(-s, 0.0);
    t[3 * l + 2] = wv_coef<LAY>(s, 0.0);
  }
  Coef* fw = t + 3 * I.p;
  Coef* bw = fw + (int64_t)I.p * E1;
  for (int j = threadIdx.x; j < I.p * E1; j += blockDim.x) {
    const int l = j / E1, cv = j - l * E1;
    double s, c;
    sincos(gamma[l] * (0.5 * I.nedges - cv), &s, &c);
    fw[j] = wv_coef<LAY>(c, s);
    bw[j] = wv_coef<LAY>(c, -s);
  }
}

// item of this block: the last item whose block_begin <= blockIdx.x
template <typename T>
QF_D int wv_find(const T* items, int nitems) {
  int lo = 0, hi = nitems - 1;
  const int b = (int)blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].block_begin <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int RB, typename E>
QF_D void wv_rx_regs(const Coef& c, const Coef& s, int nact, E (&a)[1 << RB]) {
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

// A block owns WV_SUB x 8 sub-tiles of one item; each warp walks WV_SUB of
// them through a 2-stage per-warp async-copy ring (measured: 2 stages x 8
// sub-tiles beat 3 x 4 on both the 32 x n=20 and the 4096-instance batch).
constexpr int WV_SUB = 8;
constexpr int WV_STAGES = 2;
constexpr int WV_SUBS_PER_BLOCK = 8 * WV_SUB;

template <int LAY, int RB>
constexpr size_t wv_ring_bytes(int vectors) {
  return (size_t)8 * WV_STAGES * vectors * (32 << RB) * sizeof(typename Types<LAY>::E);
}

// ------------------------------------------------------------- forward ----
template <int LAY, int RB>
__global__ void __launch_bounds__(256) k_wave_fwd(const WvFwd* items, int nitems, const WvInst* inst, void* states,
                                                  const uint16_t* cuts, const Coef* tab, int cutb,
                                                  const int32_t* skip) {
  using E = typename Types<LAY>::E;
  constexpr int R = 1 << RB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ WvFwd s_it;
  __shared__ WvInst s_in;
  if (threadIdx.x == 0) {
    s_it = items[wv_find(items, nitems)];
    s_in = inst[s_it.inst];
  }
  __syncthreads();
  // a skipped instance keeps its states and partial rows from its last evaluation
  if (skip != nullptr && skip[s_it.inst] != 0) return;
  const WvFwd& F = s_it;
  const WvInst& I = s_in;
  const int E1 = I.nedges + 1;
  Coef* scut = reinterpret_cast<Coef*>(smem_raw);  // cutb bytes: the batch's largest table
  const Coef* ttab = tab + I.tab;
  if (F.hasB)
    for (int j = threadIdx.x; j < E1; j += blockDim.x) scut[j] = ttab[3 * I.p + (int64_t)F.layerB * E1 + j];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  E* ring = reinterpret_cast<E*>(smem_raw + cutb) + (size_t)warp * WV_STAGES * R * 32;
  E* gp = reinterpret_cast<E*>(states) + I.psi;
  const uint16_t* gc = cuts + I.cuts;
  const int64_t nsub = int64_t(1) << (I.n - 5 - RB);
  const int64_t first = (int64_t)(blockIdx.x - F.block_begin) * WV_SUBS_PER_BLOCK + warp;
  int64_t hoff[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int64_t o = 0;
#pragma unroll
    for (int j = 0; j < RB; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << F.hb[j];
    hoff[r] = o;
  }
  auto sub_xb = [&](int64_t st) {
    int64_t base = st << 5;
#pragma unroll
    for (int j = 0; j < RB; ++j) base = insert0(base, F.hs[j]);
    return base | lane;
  };
  auto issue = [&](int k, int sg) {
    const int64_t st = first + 8 * k;
    if (!F.init && k < WV_SUB && st < nsub) {
      const int64_t xb = sub_xb(st);
      E* sp = ring + (size_t)sg * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) cp_async_amp(sp + r * 32, gp + (xb | hoff[r]));
    }
    cp_async_commit();
  };
  __syncthreads();  // cut table staged
  E* tag = nullptr;
  const E amp0 = coef_e(wv_coef<LAY>(1.0 / sqrt((double)(int64_t(1) << I.n)), 0.0), tag);
  const Coef ac = ttab[3 * F.layerA], as = ttab[3 * F.layerA + 1];
  const Coef bc = ttab[3 * F.layerB], bs = ttab[3 * F.layerB + 1];
#pragma unroll
  for (int k = 0; k < WV_STAGES - 1; ++k) issue(k, k);
  int sg = 0;
  for (int k = 0; k < WV_SUB; ++k) {
    const int64_t st = first + 8 * k;
    cp_async_wait<WV_STAGES - 2>();
    if (st >= nsub) break;
    const int64_t xb = sub_xb(st);
    E a[R];
    if (F.init) {
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = amp0;
    } else {
      const E* sp = ring + (size_t)sg * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = sp[r * 32];
    }
    issue(k + WV_STAGES - 1, sg == 0 ? WV_STAGES - 1 : sg - 1);
    sg = sg + 1 == WV_STAGES ? 0 : sg + 1;
    if (F.nactA > 0) wv_rx_regs<RB>(ac, as, F.nactA, a);
    if (F.hasB) {
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = cmul_v(scut[min((int)gc[xb | hoff[r]], E1 - 1)], a[r]);
      for (int b = 0; b < 5; ++b) {
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = rx_one(bc, bs, a[r], shfl_xor(a[r], 1 << b));
      }
      wv_rx_regs<RB>(bc, bs, F.nactB, a);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) gp[xb | hoff[r]] = a[r];
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------------- adjoint ----
template <int LAY, int RB>
__global__ void __launch_bounds__(256) k_wave_adj(const WvAdj* items, int nitems, const WvInst* inst, void* states,
                                                  const uint16_t* cuts, const Coef* tab, double* partials,
                                                  int cutb, const int32_t* skip) {
  using E = typename Types<LAY>::E;
  constexpr int R = 1 << RB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ WvAdj s_it;
  __shared__ WvInst s_in;
  __shared__ double red[8][4];
  if (threadIdx.x == 0) {
    s_it = items[wv_find(items, nitems)];
    s_in = inst[s_it.inst];
  }
  __syncthreads();
  if (skip != nullptr && skip[s_it.inst] != 0) return;
  const WvAdj& A = s_it;
  const WvInst& I = s_in;
  const int E1 = I.nedges + 1;
  Coef* scut = reinterpret_cast<Coef*>(smem_raw);  // cutb bytes: the batch's largest table
  const Coef* ttab = tab + I.tab;
  if (A.last)
    for (int j = threadIdx.x; j < E1; j += blockDim.x)
      scut[j] = ttab[3 * I.p + (int64_t)I.p * E1 + (int64_t)A.layer * E1 + j];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  E* ring = reinterpret_cast<E*>(smem_raw + cutb) + (size_t)warp * WV_STAGES * 2 * R * 32;
  E* gp = reinterpret_cast<E*>(states) + I.psi;
  E* gl = reinterpret_cast<E*>(states) + I.lam;
  const uint16_t* gc = cuts + I.cuts;
  const int64_t nsub = int64_t(1) << (I.n - 5 - RB);
  const int64_t first = (int64_t)(blockIdx.x - A.block_begin) * WV_SUBS_PER_BLOCK + warp;
  int64_t hoff[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int64_t o = 0;
#pragma unroll
    for (int j = 0; j < RB; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << A.hb[j];
    hoff[r] = o;
  }
  auto sub_xb = [&](int64_t st) {
    int64_t base = st << 5;
#pragma unroll
    for (int j = 0; j < RB; ++j) base = insert0(base, A.hs[j]);
    return base | lane;
  };
  auto issue = [&](int k, int sg) {
    const int64_t st = first + 8 * k;
    if (k < WV_SUB && st < nsub) {
      const int64_t xb = sub_xb(st);
      E* sp = ring + (size_t)sg * 2 * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) cp_async_amp(sp + r * 32, gp + (xb | hoff[r]));
      if (!A.init) {
#pragma unroll
        for (int r = 0; r < R; ++r) cp_async_amp(sp + (R + r) * 32, gl + (xb | hoff[r]));
      }
    }
    cp_async_commit();
  };
  FFAcc ax, acu, ae, axb;
  ax.zero();
  acu.zero();
  ae.zero();
  axb.zero();
  // RX(-beta) = [[c, i s], [i s, c]]: entries (c, +sin) of the tables
  const Coef mc = ttab[3 * A.layer], ms = ttab[3 * A.layer + 2];
  const int lb = A.layer > 0 ? A.layer - 1 : 0;
  const Coef bc = ttab[3 * lb], bs = ttab[3 * lb + 2];
  const float wref = 0.5f * (float)I.nedges;
  __syncthreads();  // cut table staged
#pragma unroll
  for (int k = 0; k < WV_STAGES - 1; ++k) issue(k, k);
  int sg = 0;
  for (int k = 0; k < WV_SUB; ++k) {
    const int64_t st = first + 8 * k;
    cp_async_wait<WV_STAGES - 2>();
    if (st >= nsub) break;
    const int64_t xb = sub_xb(st);
    E a[R], l[R];
    {
      const E* sp = ring + (size_t)sg * 2 * R * 32 + lane;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        a[r] = sp[r * 32];
        if (!A.init) l[r] = sp[(R + r) * 32];
      }
    }
    issue(k + WV_STAGES - 1, sg == 0 ? WV_STAGES - 1 : sg - 1);
    sg = sg + 1 == WV_STAGES ? 0 : sg + 1;
    uint32_t cv[R];
#pragma unroll
    for (int r = 0; r < R; ++r) cv[r] = gc[xb | hoff[r]];
    // complex64: each thread sums one sub-tile's terms of a reduction in
    // FP32 and adds that partial to the compensated accumulator once
    constexpr bool F32 = LAY == C64;
    if (A.init) {
      float part = 0.f;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float c = (float)cv[r];
        if constexpr (F32) {
          part = fmaf(c, fmaf(a[r].x, a[r].x, a[r].y * a[r].y), part);
        } else {
          FFAcc t;
          t.zero();
          acc_norm2(t, a[r]);
          ae.add_prod(c, 0.f, t.s, t.e);
        }
        l[r] = scale_ff(a[r], c);
      }
      if constexpr (F32) ae.add(part, 0.f);
    }
    auto redx = [&](FFAcc& acc, float& part, const E& lv, const E& pv) {
      if constexpr (F32) {
        part = fmaf(lv.x, pv.y, part);
        part = fmaf(-lv.y, pv.x, part);
      } else {
        redx_acc(acc, lv, pv);
      }
    };
    auto mixer = [&](const Coef& c0, const Coef& s0, bool lanes, int nact, FFAcc& acc) {
      float part = 0.f;
      if (lanes) {
        for (int b = 0; b < 5; ++b) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const E pa = shfl_xor(a[r], 1 << b);
            const E pl = shfl_xor(l[r], 1 << b);
            redx(acc, part, l[r], pa);
            a[r] = rx_one(c0, s0, a[r], pa);
            l[r] = rx_one(c0, s0, l[r], pl);
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
            a[i0] = rx_one(c0, s0, a0, a[i1]);
            a[i1] = rx_one(c0, s0, a[i1], a0);
            l[i0] = rx_one(c0, s0, l0, l[i1]);
            l[i1] = rx_one(c0, s0, l[i1], l0);
          }
        }
      }
      if constexpr (F32) acc.add(part, 0.f);
    };
    mixer(mc, ms, A.lanes != 0, A.nact, ax);
    if (A.last) {
      if constexpr (F32) {
        float part = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r)
          part = fmaf(wref - (float)cv[r], fmaf(l[r].x, a[r].y, -l[r].y * a[r].x), part);
        acu.add(part, 0.f);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) acc_imconj(acu, to_ff(l[r]), to_ff(a[r]), wref - (float)cv[r]);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const Coef& c = scut[min((int)cv[r], E1 - 1)];
        a[r] = cmul_v(c, a[r]);
        l[r] = cmul_v(c, l[r]);
      }
    }
    if (A.hasB) mixer(bc, bs, true, A.nactB, axb);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      gp[xb | hoff[r]] = a[r];
      gl[xb | hoff[r]] = l[r];
    }
  }
  cp_async_wait<0>();
  const double v[4] = {warp_sum((double)ax.s + (double)ax.e), warp_sum((double)acu.s + (double)acu.e),
                       warp_sum((double)ae.s + (double)ae.e), warp_sum((double)axb.s + (double)axb.e)};
  if (lane == 0)
    for (int k = 0; k < 4; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
    if (threadIdx.x == 1) t *= -2.0;
    partials[(int64_t)(A.prow + (blockIdx.x - A.block_begin)) * 4 + threadIdx.x] = t;
  }
}

// out[o] = sum of its segments, in order (one warp per output)
__global__ void k_wave_reduce(const int32_t* seg_begin, const WvSeg* segs, int nout_total, const int32_t* out_index,
                              const double* partials, double* out) {
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nout_total) return;
  double total = 0.0;
  for (int s = seg_begin[w]; s < seg_begin[w + 1]; ++s) {
    const WvSeg g = segs[s];
    double v = 0.0;
    for (int r = lane; r < g.nrows; r += 32) v += partials[(int64_t)(g.row + r) * 4 + g.k];
    total += warp_sum(v);
  }
  if (lane == 0) out[out_index[w]] = total;
}

// ------------------------------------------------------------ host plan ----
struct WvPlanHeader {
  int32_t magic, layout, rbf, rba;
  int32_t ninst, nwaves, nfwd, nadj, nsegs, nout;
  int64_t state_elems, cut_elems, tab_coefs, prows;
  // device byte offsets inside the workspace
  int64_t off_inst, off_fwd, off_adj, off_segbeg, off_segs, off_outidx, off_tab, off_part, off_cuts, off_states;
  int64_t device_bytes;
};
struct WvWave {
  int32_t fwd_begin, fwd_count, fwd_blocks;
  int32_t adj_begin, adj_count, adj_blocks;
};
constexpr int32_t WV_MAGIC = 0x51465756;

static int wv_rb_fwd(int layout) { return layout == C64 ? 4 : 3; }
static int wv_rb_adj(int layout) { return layout == C64 ? 3 : 2; }
int wave_min_qubits(int layout) { return 5 + std::max(wv_rb_fwd(layout), wv_rb_adj(layout)); }

static size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

namespace {
struct PlanBuild {
  WvPlanHeader h{};
  std::vector<WvInst> inst;
  std::vector<WvFwd> fwd;
  std::vector<WvAdj> adj;
  std::vector<WvWave> waves;
  std::vector<int32_t> segbeg, outidx;
  std::vector<WvSeg> segs;
};

std::vector<std::vector<int>> wv_groups(int n, int RB) {
  std::vector<std::vector<int>> groups;
  for (int b = 5; b < n; b += RB) {
    std::vector<int> g;
    for (int k = b; k < std::min(n, b + RB); ++k) g.push_back(k);
    groups.push_back(g);
  }
  return groups;
}

void wv_set_bits(int n, int RB, const std::vector<int>& group, uint8_t* hb, uint8_t* hs) {
  std::vector<int> bits = group;
  for (int b = 5; b < n && (int)bits.size() < RB; ++b)
    if (std::find(bits.begin(), bits.end(), b) == bits.end()) bits.push_back(b);
  for (int j = 0; j < RB; ++j) hb[j] = (uint8_t)bits[j];
  std::sort(bits.begin(), bits.end());
  for (int j = 0; j < RB; ++j) hs[j] = (uint8_t)bits[j];
}

// per-instance pass lists (same schedules as qaoa_state_warp / qaoa_grad_warp)
void wv_fwd_passes(int n, int p, int RB, std::vector<WvFwd>& out) {
  const auto groups = wv_groups(n, RB);
  const int m = (int)groups.size();
  auto order = [&](int l, int k) { return (l & 1) ? m - 1 - k : k; };
  WvFwd f{};
  wv_set_bits(n, RB, groups[order(0, 0)], f.hb, f.hs);
  f.init = 1;
  f.nactA = 0;
  f.hasB = 1;
  f.layerB = 0;
  f.nactB = (int8_t)groups[order(0, 0)].size();
  out.push_back(f);
  for (int l = 0; l < p; ++l) {
    if (m == 1) {
      if (l == 0) continue;
      WvFwd g{};
      wv_set_bits(n, RB, groups[0], g.hb, g.hs);
      g.hasB = 1;
      g.layerB = (int16_t)l;
      g.nactB = (int8_t)groups[0].size();
      out.push_back(g);
      continue;
    }
    for (int k = 1; k < m; ++k) {
      WvFwd g{};
      const auto& grp = groups[order(l, k)];
      wv_set_bits(n, RB, grp, g.hb, g.hs);
      g.nactA = (int8_t)grp.size();
      g.layerA = (int16_t)l;
      if (k == m - 1 && l + 1 < p) {
        g.hasB = 1;
        g.layerB = (int16_t)(l + 1);
        g.nactB = (int8_t)grp.size();
      }
      out.push_back(g);
    }
  }
}

// adjoint passes with, per pass, the output slots of its four accumulators
void wv_adj_passes(int n, int p, int RB, std::vector<WvAdj>& out, std::vector<std::array<int, 4>>& slots) {
  const auto groups = wv_groups(n, RB);
  const int m = (int)groups.size();
  auto order = [&](int l, int k) { return ((p - 1 - l) & 1) ? m - 1 - k : k; };
  bool first = true, lanes_done = false;
  for (int l = p - 1; l >= 0; --l) {
    for (int k = lanes_done ? 1 : 0; k < m; ++k) {
      WvAdj a{};
      const auto& grp = groups[order(l, k)];
      wv_set_bits(n, RB, grp, a.hb, a.hs);
      a.init = first ? 1 : 0;
      a.lanes = k == 0 ? 1 : 0;
      a.nact = (int8_t)grp.size();
      a.last = k == m - 1 ? 1 : 0;
      a.layer = (int16_t)l;
      std::array<int, 4> s = {p + l, a.last ? l : -1, first ? 2 * p : -1, -1};
      if (a.last && l > 0 && m > 1) {
        a.hasB = 1;
        a.nactB = (int8_t)grp.size();
        s[3] = p + l - 1;
      }
      out.push_back(a);
      slots.push_back(s);
      first = false;
    }
    lanes_done = m > 1;
  }
}
}  // namespace

int wave_plan(const qf_batch_instance* hinst, int ninst, int layout, void* host_plan, size_t host_bytes,
              size_t* need_host, size_t* need_device) {
  if (layout != C64 && layout != FF) return QF_ERR_LAYOUT;
  const int RBf = wv_rb_fwd(layout), RBa = wv_rb_adj(layout);
  const size_t S = elem_bytes(layout);
  PlanBuild P;
  P.h.magic = WV_MAGIC;
  P.h.layout = layout;
  P.h.rbf = RBf;
  P.h.rba = RBa;
  P.h.ninst = ninst;
  std::vector<std::vector<WvFwd>> fw(ninst);
  std::vector<std::vector<WvAdj>> ad(ninst);
  std::vector<std::vector<std::array<int, 4>>> sl(ninst);
  int64_t st = 0, ct = 0, tb = 0;
  int nw = 0;
  for (int i = 0; i < ninst; ++i) {
    const qf_batch_instance& q = hinst[i];
    if (q.n < wave_min_qubits(layout) || q.n > QF_MAX_QUBITS || q.p < 1 || q.p > 64 || q.nedges < 0 ||
        q.nedges > WV_MAX_EDGES)
      return QF_ERR_INVALID_ARGUMENT;
    WvInst w{};
    w.n = q.n;
    w.p = q.p;
    w.nedges = q.nedges;
    w.edge_offset = q.edge_offset;
    w.angle_offset = q.angle_offset;
    w.out_offset = q.out_offset;
    const int64_t amps = int64_t(1) << q.n;
    w.psi = st;
    w.lam = st + amps;
    st += 2 * amps;
    w.cuts = ct;
    ct += amps;
    w.tab = tb;
    tb += wv_tab_size(q.p, q.nedges);
    P.inst.push_back(w);
    wv_fwd_passes(q.n, q.p, RBf, fw[i]);
    wv_adj_passes(q.n, q.p, RBa, ad[i], sl[i]);
    nw = std::max(nw, (int)(fw[i].size() + ad[i].size()));
  }
  // waves: pass w of every instance; adjoint blocks get consecutive rows
  int64_t prow = 0;
  std::vector<std::vector<int64_t>> rows(ninst);  // first row of each adjoint pass
  for (int w = 0; w < nw; ++w) {
    WvWave wave{};
    wave.fwd_begin = (int32_t)P.fwd.size();
    wave.adj_begin = (int32_t)P.adj.size();
    int32_t fb = 0, ab = 0;
    for (int i = 0; i < ninst; ++i) {
      const int nf = (int)fw[i].size();
      const int n = P.inst[i].n;
      if (w < nf) {
        WvFwd f = fw[i][w];
        f.inst = i;
        f.block_begin = fb;
        fb += (int32_t)(((int64_t(1) << (n - 5 - RBf)) + WV_SUBS_PER_BLOCK - 1) / WV_SUBS_PER_BLOCK);
        P.fwd.push_back(f);
      } else if (w < nf + (int)ad[i].size()) {
        WvAdj a = ad[i][w - nf];
        a.inst = i;
        a.block_begin = ab;
        const int32_t nb =
            (int32_t)(((int64_t(1) << (n - 5 - RBa)) + WV_SUBS_PER_BLOCK - 1) / WV_SUBS_PER_BLOCK);
        ab += nb;
        a.prow = (int32_t)prow;
        rows[i].push_back(prow);
        prow += nb;
        P.adj.push_back(a);
      }
    }
    wave.fwd_count = (int32_t)P.fwd.size() - wave.fwd_begin;
    wave.adj_count = (int32_t)P.adj.size() - wave.adj_begin;
    wave.fwd_blocks = fb;
    wave.adj_blocks = ab;
    P.waves.push_back(wave);
  }
  if (prow > INT32_MAX / 2) return QF_ERR_TOO_LARGE;
  // final reduction: per output, the segments of adjoint rows feeding it
  for (int i = 0; i < ninst; ++i) {
    const int p = P.inst[i].p, n = P.inst[i].n;
    const int32_t nb = (int32_t)(((int64_t(1) << (n - 5 - RBa)) + WV_SUBS_PER_BLOCK - 1) / WV_SUBS_PER_BLOCK);
    for (int slot = 0; slot <= 2 * p; ++slot) {
      P.segbeg.push_back((int32_t)P.segs.size());
      P.outidx.push_back(P.inst[i].out_offset + slot);
      for (size_t j = 0; j < sl[i].size(); ++j)
        for (int k = 0; k < 4; ++k)
          if (sl[i][j][k] == slot) P.segs.push_back(WvSeg{(int32_t)rows[i][j], nb, k, 0});
    }
  }
  P.segbeg.push_back((int32_t)P.segs.size());
  P.h.nwaves = nw;
  P.h.nfwd = (int32_t)P.fwd.size();
  P.h.nadj = (int32_t)P.adj.size();
  P.h.nsegs = (int32_t)P.segs.size();
  P.h.nout = (int32_t)P.outidx.size();
  P.h.state_elems = st;
  P.h.cut_elems = ct;
  P.h.tab_coefs = tb;
  P.h.prows = prow;
  // device layout
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = al256(off + std::max<size_t>(bytes, 1));
    return (int64_t)o;
  };
  P.h.off_inst = take(P.inst.size() * sizeof(WvInst));
  P.h.off_fwd = take(P.fwd.size() * sizeof(WvFwd));
  P.h.off_adj = take(P.adj.size() * sizeof(WvAdj));
  P.h.off_segbeg = take(P.segbeg.size() * sizeof(int32_t));
  P.h.off_segs = take(P.segs.size() * sizeof(WvSeg));
  P.h.off_outidx = take(P.outidx.size() * sizeof(int32_t));
  P.h.off_tab = take((size_t)tb * sizeof(Coef));
  P.h.off_part = take((size_t)prow * 4 * sizeof(double));
  P.h.off_cuts = take((size_t)ct * sizeof(uint16_t));
  P.h.off_states = take((size_t)st * S);
  P.h.device_bytes = (int64_t)off;
  // host image: header, waves, then the arrays that are uploaded
  const size_t hbytes = sizeof(WvPlanHeader) + P.waves.size() * sizeof(WvWave) + P.inst.size() * sizeof(WvInst) +
                        P.fwd.size() * sizeof(WvFwd) + P.adj.size() * sizeof(WvAdj) +
                        P.segbeg.size() * sizeof(int32_t) + P.segs.size() * sizeof(WvSeg) +
                        P.outidx.size() * sizeof(int32_t);
  if (need_host) *need_host = hbytes;
  if (need_device) *need_device = (size_t)off;
  if (host_plan == nullptr) return QF_OK;
  if (host_bytes < hbytes) return QF_ERR_WORKSPACE;
  char* h = reinterpret_cast<char*>(host_plan);
  auto put = [&](const void* src, size_t bytes) {
    std::memcpy(h, src, bytes);
    h += bytes;
  };
  put(&P.h, sizeof(P.h));
  put(P.waves.data(), P.waves.size() * sizeof(WvWave));
  put(P.inst.data(), P.inst.size() * sizeof(WvInst));
  put(P.fwd.data(), P.fwd.size() * sizeof(WvFwd));
  put(P.adj.data(), P.adj.size() * sizeof(WvAdj));
  put(P.segbeg.data(), P.segbeg.size() * sizeof(int32_t));
  put(P.segs.data(), P.segs.size() * sizeof(WvSeg));
  put(P.outidx.data(), P.outidx.size() * sizeof(int32_t));
  return QF_OK;
}

namespace {
struct PlanView {
  const WvPlanHeader* h;
  const WvWave* waves;
  const WvInst* inst;
  const WvFwd* fwd;
  const WvAdj* adj;
  const int32_t* segbeg;
  const WvSeg* segs;
  const int32_t* outidx;
};
bool view_plan(const void* host_plan, PlanView& v) {
  const char* h = reinterpret_cast<const char*>(host_plan);
  v.h = reinterpret_cast<const WvPlanHeader*>(h);
  if (v.h->magic != WV_MAGIC) return false;
  h += sizeof(WvPlanHeader);
  v.waves = reinterpret_cast<const WvWave*>(h);
  h += v.h->nwaves * sizeof(WvWave);
  v.inst = reinterpret_cast<const WvInst*>(h);
  h += v.h->ninst * sizeof(WvInst);
  v.fwd = reinterpret_cast<const WvFwd*>(h);
  h += v.h->nfwd * sizeof(WvFwd);
  v.adj = reinterpret_cast<const WvAdj*>(h);
  h += v.h->nadj * sizeof(WvAdj);
  v.segbeg = reinterpret_cast<const int32_t*>(h);
  h += (v.h->nout + 1) * sizeof(int32_t);
  v.segs = reinterpret_cast<const WvSeg*>(h);
  h += v.h->nsegs * sizeof(WvSeg);
  v.outidx = reinterpret_cast<const int32_t*>(h);
  return true;
}
}  // namespace

int wave_prepare(const void* host_plan, const uint8_t* edges, void* ws, size_t ws_bytes, cudaStream_t stream) {
  PlanView v;
  if (!view_plan(host_plan, v)) return QF_ERR_INVALID_ARGUMENT;
  const WvPlanHeader& h = *v.h;
  if (ws_bytes < (size_t)h.device_bytes) return QF_ERR_WORKSPACE;
  char* d = reinterpret_cast<char*>(ws);
  auto up = [&](int64_t off, const void* src, size_t bytes) {
    return bytes ? check_cuda(cudaMemcpyAsync(d + off, src, bytes, cudaMemcpyHostToDevice, stream)) : QF_OK;
  };
  int rc;
  if ((rc = up(h.off_inst, v.inst, h.ninst * sizeof(WvInst)))) return rc;
  if ((rc = up(h.off_fwd, v.fwd, h.nfwd * sizeof(WvFwd)))) return rc;
  if ((rc = up(h.off_adj, v.adj, h.nadj * sizeof(WvAdj)))) return rc;
  if ((rc = up(h.off_segbeg, v.segbeg, (h.nout + 1) * sizeof(int32_t)))) return rc;
  if ((rc = up(h.off_segs, v.segs, h.nsegs * sizeof(WvSeg)))) return rc;
  if ((rc = up(h.off_outidx, v.outidx, h.nout * sizeof(int32_t)))) return rc;
  if (h.ninst > 0) {
    int maxn = 0;
    for (int i = 0; i < h.ninst; ++i) maxn = std::max(maxn, v.inst[i].n);
    const int64_t per = std::min<int64_t>((int64_t(1) << maxn) / 256 + 1, 1024);
    k_wave_cuts<<<dim3((unsigned)per, (unsigned)h.ninst), 256, 0, stream>>>(
        reinterpret_cast<const WvInst*>(d + h.off_inst), h.ninst, edges, reinterpret_cast<uint16_t*>(d + h.off_cuts));
    if ((rc = check_cuda(cudaGetLastError()))) return rc;
  }
  return QF_OK;
}

template <int LAY, int RBF, int RBA>
static int wave_run_t(const PlanView& v, char* d, const double* angles, double* out, const int32_t* skip,
                      cudaStream_t stream) {
  const WvPlanHeader& h = *v.h;
  const WvInst* dinst = reinterpret_cast<const WvInst*>(d + h.off_inst);
  const Coef* dtab = reinterpret_cast<const Coef*>(d + h.off_tab);
  const uint16_t* dcuts = reinterpret_cast<const uint16_t*>(d + h.off_cuts);
  void* dstates = d + h.off_states;
  double* dpart = reinterpret_cast<double*>(d + h.off_part);
  int maxe = 0;
  for (int i = 0; i < h.ninst; ++i) maxe = std::max(maxe, v.inst[i].nedges);
  const size_t cutb = (((size_t)(maxe + 1) * sizeof(Coef)) + 127) & ~size_t(127);
  const size_t smem_max = ((((size_t)(WV_MAX_EDGES + 1) * sizeof(Coef)) + 127) & ~size_t(127));
  const size_t smem_f = cutb + wv_ring_bytes<LAY, RBF>(1), smem_a = cutb + wv_ring_bytes<LAY, RBA>(2);
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_wave_fwd<LAY, RBF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(smem_max + wv_ring_bytes<LAY, RBF>(1))));
    if (rc) return rc;
    rc = check_cuda(cudaFuncSetAttribute(k_wave_adj<LAY, RBA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(smem_max + wv_ring_bytes<LAY, RBA>(2))));
    if (rc) return rc;
    attr[dev].store(true);
  }
  k_wave_coefs<LAY><<<h.ninst, 128, 0, stream>>>(dinst, h.ninst, angles, const_cast<Coef*>(dtab), skip);
  int rc = check_cuda(cudaGetLastError());
  if (rc) return rc;
  const WvFwd* dfwd = reinterpret_cast<const WvFwd*>(d + h.off_fwd);
  const WvAdj* dadj = reinterpret_cast<const WvAdj*>(d + h.off_adj);
  for (int w = 0; w < h.nwaves; ++w) {
    const WvWave& W = v.waves[w];
    if (W.fwd_count > 0) {
      k_wave_fwd<LAY, RBF><<<W.fwd_blocks, 256, smem_f, stream>>>(
          dfwd + W.fwd_begin, W.fwd_count, dinst, dstates, dcuts, dtab, (int)cutb, skip);
      if ((rc = check_cuda(cudaGetLastError()))) return rc;
    }
    if (W.adj_count > 0) {
      k_wave_adj<LAY, RBA><<<W.adj_blocks, 256, smem_a, stream>>>(
          dadj + W.adj_begin, W.adj_count, dinst, dstates, dcuts, dtab, dpart, (int)cutb, skip);
      if ((rc = check_cuda(cudaGetLastError()))) return rc;
    }
  }
  if (h.nout > 0) {
    k_wave_reduce<<<(h.nout * 32 + 255) / 256, 256, 0, stream>>>(
        reinterpret_cast<const int32_t*>(d + h.off_segbeg), reinterpret_cast<const WvSeg*>(d + h.off_segs), h.nout,
        reinterpret_cast<const int32_t*>(d + h.off_outidx), dpart, out);
    rc = check_cuda(cudaGetLastError());
  }
  return rc;
}

int wave_run(const void* host_plan, void* ws, size_t ws_bytes, const double* angles, double* out,
             const int32_t* skip, cudaStream_t stream) {
  PlanView v;
  if (!view_plan(host_plan, v)) return QF_ERR_INVALID_ARGUMENT;
  if (ws_bytes < (size_t)v.h->device_bytes) return QF_ERR_WORKSPACE;
  char* d = reinterpret_cast<char*>(ws);
  if (v.h->layout == C64) return wave_run_t<C64, 4, 3>(v, d, angles, out, skip, stream);
  if (v.h->layout == FF) return wave_run_t<FF, 3, 2>(v, d, angles, out, skip, stream);
  return QF_ERR_LAYOUT;
}

}  // namespace qf
