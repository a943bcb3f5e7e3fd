// Float-float fused passes whose dense gates touch at most four bits:
// shape kernels (k_shape, the default) and group kernels (k_group).
//
// The warp-tile kernel (k_warp) keeps bits 0..4 on the lanes and moves a
// gate's lane bits into registers with shuffles; each of its decoded
// instructions serves the 4 amplitudes a thread holds (float-float, RB=2),
// so on passes with one or two dense gates and a row of CZ signs the
// decoding and exchanges cost as much as the arithmetic.  Here a thread
// holds all 2^G amplitudes that differ in the pass's gate bits, wherever
// those bits are, so no amplitude leaves its thread: dense gates run on
// register bits, and the lanes of a warp fall on the lowest remaining bits
// (coalesced 16-byte accesses).  k_shape compiles one or two gates on fixed
// register bits as straight-line code (the planner cuts passes to fit);
// k_group interprets any op list, decoding each op once per 2^G amplitudes.
//
// Semantics are those of quantumflow/backend/numpybk.py:159-214 tensormul
// applied in list order (quantumflow/circuits.py:87-99), as in every pass.
#include "engine.cuh"
#include "regops.cuh"

#include <algorithm>
#include <cstring>

namespace qf {

// 4x4 gate with its MSB on register bit a and LSB on b, a > b (the host
// exchanges the matrix's qubit order to make it so)
template <int G>
QF_D void group_g2(int a, int b, const Coef* cf, float4 (&v)[1 << G], bool dense) {
  switch (a * 4 + b) {
    case 4: g2_reg<G, 1, 0>(cf, v, dense); break;
    case 8: if constexpr (G > 2) g2_reg<G, 2, 0>(cf, v, dense); break;
    case 9: if constexpr (G > 2) g2_reg<G, 2, 1>(cf, v, dense); break;
    case 12: if constexpr (G > 3) g2_reg<G, 3, 0>(cf, v, dense); break;
    case 13: if constexpr (G > 3) g2_reg<G, 3, 1>(cf, v, dense); break;
    case 14: if constexpr (G > 3) g2_reg<G, 3, 2>(cf, v, dense); break;
  }
}

// negate the registers whose bit is set in neg (sign-bit flips on all four
// float-float words, or both words of a complex64 amplitude)
template <int R>
QF_D void apply_negmask(uint32_t neg, float4 (&v)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint32_t s = (neg << (31 - r)) & 0x80000000u;
    v[r].x = __uint_as_float(__float_as_uint(v[r].x) ^ s);
    v[r].y = __uint_as_float(__float_as_uint(v[r].y) ^ s);
    v[r].z = __uint_as_float(__float_as_uint(v[r].z) ^ s);
    v[r].w = __uint_as_float(__float_as_uint(v[r].w) ^ s);
  }
}
template <int R>
QF_D void apply_negmask(uint32_t neg, float2 (&v)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint32_t s = (neg << (31 - r)) & 0x80000000u;
    v[r].x = __uint_as_float(__float_as_uint(v[r].x) ^ s);
    v[r].y = __uint_as_float(__float_as_uint(v[r].y) ^ s);
  }
}

template <int G>
__global__ void __launch_bounds__(256) k_group(const __grid_constant__ GroupParams P) {
  constexpr int R = 1 << G;
  const float4* gin = reinterpret_cast<const float4*>(P.in);
  float4* gout = reinterpret_cast<float4*>(P.out);
  const int64_t ngroups = int64_t(1) << (P.n - G);
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ngroups; t += nthr) {
    int64_t xb = t;
#pragma unroll
    for (int j = 0; j < G; ++j) xb = insert0(xb, P.sbits[j]);
    float4 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = gin[xb | P.off[r]];
    uint32_t neg = 0;
    for (int o = 0; o < P.nops; ++o) {
      const GroupOp& op = P.ops[o];
      switch (op.type) {
        case OP_SIGN:
          if ((xb & (int64_t)op.mout) == (int64_t)op.mout) neg ^= op.rmask;
          break;
        case OP_DENSE1:
          if (op.flush) {
            apply_negmask<R>(neg, v);
            neg = 0;
          }
          g1_reg_dispatch<G>(op.a, &P.coef[op.coef], v);
          break;
        case OP_DENSE2:
          if constexpr (G >= 2) {
            if (op.flush) {
              apply_negmask<R>(neg, v);
              neg = 0;
            }
            group_g2<G>(op.a, op.b, &P.coef[op.coef], v, op.flag != 0);
          }
          break;
        case OP_DIAG:
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int64_t x = xb | P.off[r];
            int idx = 0;
            for (int i = 0; i < op.flag; ++i) idx = (idx << 1) | int((x >> op.gb[i]) & 1);
            v[r] = cmul_v(P.coef[op.coef + idx], v[r]);
          }
          break;
        case OP_PHASE:
#pragma unroll
          for (int r = 0; r < R; ++r) v[r] = cmul_v(P.coef[op.coef], v[r]);
          break;
        default:
          break;
      }
    }
    if (P.final_flush) apply_negmask<R>(neg, v);
#pragma unroll
    for (int r = 0; r < R; ++r) gout[xb | P.off[r]] = v[r];
  }
}

int group_prepare(int n, int layout, const std::vector<HostOp>& ops, const std::vector<int>& idx,
                  GroupParams& P, int& G) {
  if (layout != FF) return QF_ERR_NOT_SUPPORTED;
  // gate bits in order of first use; the first gate's bits take the top
  // register bits
  int order[4], G_ = 0;
  for (int i : idx) {
    const HostOp& op = ops[i];
    switch (op.type) {
      case OP_DENSE1:
      case OP_DENSE2:
        for (int j = 0; j < op.k; ++j) {
          if (std::find(order, order + G_, op.gb[j]) != order + G_) continue;
          if (G_ == 4) return QF_ERR_NOT_SUPPORTED;
          order[G_++] = op.gb[j];
        }
        break;
      case OP_SIGN:
      case OP_PHASE:
        break;
      case OP_DIAG:
        if (op.k > 3) return QF_ERR_NOT_SUPPORTED;
        break;
      default:
        return QF_ERR_NOT_SUPPORTED;  // permutations, cut tables, wider gates
    }
  }
  if (G_ == 0 || n - G_ < 8 || (int)idx.size() > GROUP_MAX_OPS) return QF_ERR_NOT_SUPPORTED;
  std::memset(&P, 0, sizeof(GroupParams));
  P.n = n;
  int reg_of[64];
  std::fill(reg_of, reg_of + 64, -1);
  uint64_t gmask = 0;
  for (int k = 0; k < G_; ++k) {
    const int j = G_ - 1 - k;
    P.rbits[j] = (uint8_t)order[k];
    reg_of[order[k]] = j;
    gmask |= uint64_t(1) << order[k];
  }
  for (int j = 0; j < G_; ++j) P.sbits[j] = P.rbits[j];
  std::sort(P.sbits, P.sbits + G_);
  for (int r = 0; r < (1 << G_); ++r) {
    int64_t o = 0;
    for (int j = 0; j < G_; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << P.rbits[j];
    P.off[r] = o;
  }
  int nc = 0, no = 0;
  bool pending = false;
  auto put = [&](cplx v) { P.coef[nc++] = make_coef(v, FF); };
  for (int i : idx) {
    const HostOp& op = ops[i];
    GroupOp& g = P.ops[no++];
    g.type = op.type;
    const int need = op.type == OP_DENSE1 ? 4 : op.type == OP_DENSE2 ? 16
                     : op.type == OP_DIAG ? (1 << op.k) : op.type == OP_PHASE ? 1 : 0;
    if (nc + need > GROUP_MAX_COEF) return QF_ERR_NOT_SUPPORTED;
    g.coef = (uint16_t)nc;
    switch (op.type) {
      case OP_DENSE1:
        g.a = (uint8_t)reg_of[op.gb[0]];
        g.flush = pending ? 1 : 0;
        pending = false;
        for (int e = 0; e < 4; ++e) put(op.m[e]);
        break;
      case OP_DENSE2: {
        const int ja = reg_of[op.gb[0]], jb = reg_of[op.gb[1]];
        const bool swap = ja < jb;
        g.a = (uint8_t)(swap ? jb : ja);
        g.b = (uint8_t)(swap ? ja : jb);
        g.flush = pending ? 1 : 0;
        pending = false;
        bool dense = true;
        for (int e = 0; e < 16; ++e) dense = dense && op.m[e].real() != 0.0 && op.m[e].imag() != 0.0;
        g.flag = dense ? 1 : 0;
        auto sw = [](int x) { return ((x & 1) << 1) | (x >> 1); };  // exchange the two index bits
        for (int r = 0; r < 4; ++r)
          for (int c = 0; c < 4; ++c) put(swap ? op.m[sw(r) * 4 + sw(c)] : op.m[r * 4 + c]);
        break;
      }
      case OP_SIGN: {
        uint64_t m = 0;
        int jm = 0;
        for (int j = 0; j < op.k; ++j) {
          m |= uint64_t(1) << op.gb[j];
          if (reg_of[op.gb[j]] >= 0) jm |= 1 << reg_of[op.gb[j]];
        }
        g.mout = m & ~gmask;
        uint32_t rm = 0;
        for (int r = 0; r < (1 << G_); ++r)
          if ((r & jm) == jm) rm |= 1u << r;
        g.rmask = (uint16_t)rm;
        pending = true;
        break;
      }
      case OP_DIAG:
        g.flag = (uint8_t)op.k;
        for (int j = 0; j < op.k; ++j) g.gb[j] = (uint8_t)op.gb[j];
        for (int e = 0; e < (1 << op.k); ++e) put(op.diag[e]);
        break;
      case OP_PHASE:
        put(op.scalar);
        break;
    }
  }
  P.nops = no;
  P.final_flush = pending ? 1 : 0;
  G = G_;
  return QF_OK;
}

int group_launch(const GroupParams& P, int G, cudaStream_t stream) {
  const int64_t ngroups = int64_t(1) << (P.n - G);
  int64_t grid = ngroups / 256;
  const int64_t cap = (int64_t)device_sm_count() * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  switch (G) {
    case 1: k_group<1><<<(int)grid, 256, 0, stream>>>(P); break;
    case 2: k_group<2><<<(int)grid, 256, 0, stream>>>(P); break;
    case 3: k_group<3><<<(int)grid, 256, 0, stream>>>(P); break;
    case 4: k_group<4><<<(int)grid, 256, 0, stream>>>(P); break;
    default: return QF_ERR_NOT_SUPPORTED;
  }
  return check_cuda(cudaGetLastError());
}


// ------------------------------------------------------------ shape passes
// The table of straight-line programs.  Slot codes: 0 none, 10 + j a 2x2
// gate on register bit j, 100 + 10 j0 + j1 a 4x4 gate with its MSB on j0
// and LSB on j1 (j0 > j1).  Register bits are named in order of first use
// from the top, so e.g. "4x4 on (a,b), then 2x2 on c" is {3, 121, 10} for
// any three distinct bits a, b, c.
struct ShapeDef {
  int G, s0, s1;
};
static const ShapeDef kShapes[] = {
    {1, 10, 0},   {2, 110, 0},   {1, 10, 10},   {2, 11, 10},   {2, 11, 110},
    {3, 12, 110}, {2, 110, 11},  {2, 110, 10},  {3, 121, 10},  {2, 110, 110},
    {3, 121, 120}, {3, 121, 110}, {4, 132, 110},
};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

template <int G, int S, typename E>
QF_D void slot_apply(const Coef* cf, E (&v)[1 << G], bool dense) {
  if constexpr (S >= 100) {
    g2_reg<G, (S / 10) % 10, S % 10>(cf, v, dense);
  } else if constexpr (S >= 10) {
    g1_reg<G, S - 10>(cf, v);
  }
}

// LAY: FF (float4 amplitudes) or C64 (float2); IT: index type (uint32_t
// for states of at most 2^31 amplitudes)
template <int LAY, int G, int S0, int S1, typename IT>
__global__ void __launch_bounds__(256) k_shape(const __grid_constant__ ShapeParams P) {
  using E = typename Types<LAY>::E;
  constexpr int R = 1 << G;
  const E* gin = reinterpret_cast<const E*>(P.in);
  E* gout = reinterpret_cast<E*>(P.out);
  const IT ngroups = IT(1) << (P.n - G);
  const IT nthr = (IT)gridDim.x * blockDim.x;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < ngroups; t += nthr) {
    IT xb = t;
#pragma unroll
    for (int j = 0; j < G; ++j) xb = insert0(xb, P.sbits[j]);
    E v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = gin[xb | (IT)P.off[r]];
    auto signs = [&](int s0, int s1) {
      uint32_t m = 0;
      for (int s = s0; s < s1; ++s)
        if ((xb & (IT)P.mout[s]) == (IT)P.mout[s]) m ^= P.rmask[s];
      apply_negmask<R>(m, v);
    };
    if (P.sign_end[0] > 0) signs(0, P.sign_end[0]);
    slot_apply<G, S0>(&P.coef[0], v, P.dense[0] != 0);
    if constexpr (S1 != 0) {
      if (P.sign_end[1] > P.sign_end[0]) signs(P.sign_end[0], P.sign_end[1]);
      slot_apply<G, S1>(&P.coef[16], v, P.dense[1] != 0);
    }
    if (P.sign_end[2] > P.sign_end[1]) signs(P.sign_end[1], P.sign_end[2]);
#pragma unroll
    for (int r = 0; r < R; ++r) gout[xb | (IT)P.off[r]] = v[r];
  }
}

using ShapeKernel = void (*)(ShapeParams);
#define QF_SHAPES(L, IT)                                                                                \
  {                                                                                                    \
    k_shape<L, 1, 10, 0, IT>, k_shape<L, 2, 110, 0, IT>, k_shape<L, 1, 10, 10, IT>,                      \
        k_shape<L, 2, 11, 10, IT>, k_shape<L, 2, 11, 110, IT>, k_shape<L, 3, 12, 110, IT>,               \
        k_shape<L, 2, 110, 11, IT>, k_shape<L, 2, 110, 10, IT>, k_shape<L, 3, 121, 10, IT>,              \
        k_shape<L, 2, 110, 110, IT>, k_shape<L, 3, 121, 120, IT>, k_shape<L, 3, 121, 110, IT>,           \
        k_shape<L, 4, 132, 110, IT>,                                                                   \
  }
static const ShapeKernel kShapeKernelsFF32[kNumShapes] = QF_SHAPES(FF, uint32_t);
static const ShapeKernel kShapeKernelsFF64[kNumShapes] = QF_SHAPES(FF, int64_t);
static const ShapeKernel kShapeKernelsC64_32[kNumShapes] = QF_SHAPES(C64, uint32_t);
static const ShapeKernel kShapeKernelsC64_64[kNumShapes] = QF_SHAPES(C64, int64_t);
#undef QF_SHAPES

// Register naming of a dense-op program: bits in order of first use get
// register bits G-1, G-2, ...; codes[] the slot codes; swap[s] when a 4x4
// gate's MSB lands on the lower register bit (its matrix is then given
// with the qubit order exchanged).  Returns the table index or -1.
static int shape_name(const std::vector<HostOp>& ops, const int* dense, int nd, int* order, int& G,
                      bool* swap) {
  if (nd < 1 || nd > 2) return -1;
  G = 0;
  for (int s = 0; s < nd; ++s) {
    const HostOp& op = ops[dense[s]];
    if (op.type != OP_DENSE1 && op.type != OP_DENSE2) return -1;
    for (int j = 0; j < op.k; ++j) {
      if (std::find(order, order + G, op.gb[j]) != order + G) continue;
      if (G == 4) return -1;
      order[G++] = op.gb[j];
    }
  }
  auto reg = [&](int bit) { return G - 1 - (int)(std::find(order, order + G, bit) - order); };
  int codes[2] = {0, 0};
  for (int s = 0; s < nd; ++s) {
    const HostOp& op = ops[dense[s]];
    if (op.type == OP_DENSE1) {
      codes[s] = 10 + reg(op.gb[0]);
      swap[s] = false;
    } else {
      const int ja = reg(op.gb[0]), jb = reg(op.gb[1]);
      swap[s] = ja < jb;
      codes[s] = 100 + 10 * std::max(ja, jb) + std::min(ja, jb);
    }
  }
  for (int i = 0; i < kNumShapes; ++i)
    if (kShapes[i].G == G && kShapes[i].s0 == codes[0] && kShapes[i].s1 == codes[1]) return i;
  return -1;
}

// Widest shape in gate bits (qf_set_shape_bits).  Measured on the
// random-layer circuit at N=28 (10 layers, ms per step): 114.6 with 3 bits,
// 115.2 with 2, 118.1 with 4 -- the two-4x4 shape on four bits is about 6k
// straight-line instructions and stalls on instruction fetch, so two
// single-gate sweeps beat it.
int g_shape_max_bits = 3;

int shape_lookup(const std::vector<HostOp>& ops, const int* dense, int nd, int* order, int& G, bool* swap,
                 int* s0, int* s1) {
  const int i = shape_name(ops, dense, nd, order, G, swap);
  if (i < 0) return -1;
  *s0 = kShapes[i].s0;
  *s1 = kShapes[i].s1;
  return i;
}

int shape_of(const std::vector<HostOp>& ops, const int* dense, int nd, int max_bits) {
  int order[4], G = 0;
  bool swap[2];
  const int s = shape_name(ops, dense, nd, order, G, swap);
  return G <= max_bits ? s : -1;
}

// Complex64 passes take every shape of the table: their FP32 bodies are a
// quarter of the float-float ones (the four-bit two-4x4 shape is short), and
// a pass that moves the state once for two gates is what an HBM-bound
// layout wants.  Measured at N=28 (100 random layers): 342.7 ms per step on
// warp tiles alone.  qf_set_shape_bits(0) turns shape passes off for both.
int shape_max_bits(int layout) { return layout == C64 && g_shape_max_bits > 0 ? 4 : g_shape_max_bits; }

int shape_prepare(int n, int layout, const std::vector<HostOp>& ops, const std::vector<int>& idx,
                  ShapeParams& P) {
  if (layout != FF && layout != C64) return QF_ERR_NOT_SUPPORTED;
  int dense[2], nd = 0, nsign = 0;
  for (int i : idx) {
    const HostOp& op = ops[i];
    if (op.type == OP_SIGN) {
      ++nsign;
    } else if (op.type == OP_DENSE1 || op.type == OP_DENSE2) {
      if (nd == 2) return QF_ERR_NOT_SUPPORTED;
      dense[nd++] = i;
    } else {
      return QF_ERR_NOT_SUPPORTED;
    }
  }
  int order[4], G = 0;
  bool swap[2] = {false, false};
  const int shape = shape_name(ops, dense, nd, order, G, swap);
  if (shape < 0 || G > shape_max_bits(layout) || nsign > SHAPE_MAX_SIGNS || n - G < 8) return QF_ERR_NOT_SUPPORTED;
  std::memset(&P, 0, sizeof(ShapeParams));
  P.n = n;
  P.shape = shape;
  P.layout = layout;
  int reg_of[64];
  std::fill(reg_of, reg_of + 64, -1);
  uint64_t gmask = 0;
  int rbits[4];
  for (int k = 0; k < G; ++k) {
    rbits[G - 1 - k] = order[k];
    reg_of[order[k]] = G - 1 - k;
    gmask |= uint64_t(1) << order[k];
  }
  for (int j = 0; j < G; ++j) P.sbits[j] = (uint8_t)rbits[j];
  std::sort(P.sbits, P.sbits + G);
  for (int r = 0; r < (1 << G); ++r) {
    int64_t o = 0;
    for (int j = 0; j < G; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << rbits[j];
    P.off[r] = o;
  }
  int slot = 0, ns = 0;
  for (int i : idx) {
    const HostOp& op = ops[i];
    if (op.type == OP_SIGN) {
      uint64_t m = 0;
      int jm = 0;
      for (int j = 0; j < op.k; ++j) {
        m |= uint64_t(1) << op.gb[j];
        if (reg_of[op.gb[j]] >= 0) jm |= 1 << reg_of[op.gb[j]];
      }
      uint32_t rm = 0;
      for (int r = 0; r < (1 << G); ++r)
        if ((r & jm) == jm) rm |= 1u << r;
      P.mout[ns] = m & ~gmask;
      P.rmask[ns] = (uint16_t)rm;
      ++ns;
      continue;
    }
    // a dense slot closes the sign list before it
    for (int b = slot; b < 3; ++b) P.sign_end[b] = ns;
    Coef* c = &P.coef[16 * slot];
    if (op.type == OP_DENSE1) {
      for (int e = 0; e < 4; ++e) c[e] = make_coef(op.m[e], layout);
    } else {
      bool all = true;
      for (int e = 0; e < 16; ++e) all = all && op.m[e].real() != 0.0 && op.m[e].imag() != 0.0;
      P.dense[slot] = all ? 1 : 0;
      auto sw = [](int x) { return ((x & 1) << 1) | (x >> 1); };  // exchange the two index bits
      for (int r = 0; r < 4; ++r)
        for (int col = 0; col < 4; ++col)
          c[4 * r + col] = make_coef(swap[slot] ? op.m[sw(r) * 4 + sw(col)] : op.m[r * 4 + col], layout);
    }
    ++slot;
  }
  // signs after the last slot act at the end (boundary 2); with one slot
  // boundary 1 is the end as well
  if (nd == 1) P.sign_end[1] = P.sign_end[0];
  P.sign_end[2] = ns;
  return QF_OK;
}

int shape_launch(const ShapeParams& P, cudaStream_t stream) {
  if (P.shape < 0 || P.shape >= kNumShapes) return QF_ERR_INVALID_ARGUMENT;
  const int G = kShapes[P.shape].G;
  const int64_t ngroups = int64_t(1) << (P.n - G);
  int64_t grid = ngroups / 256;
  const int64_t cap = (int64_t)device_sm_count() * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  const ShapeKernel* table = P.layout == C64 ? (P.n <= 31 ? kShapeKernelsC64_32 : kShapeKernelsC64_64)
                                             : (P.n <= 31 ? kShapeKernelsFF32 : kShapeKernelsFF64);
  table[P.shape]<<<(int)grid, 256, 0, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

}  // namespace qf
