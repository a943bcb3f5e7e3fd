// Gate passes on complex128 states in 64-bit integer fixed-point arithmetic
// (QF_LAYOUT_FX; the arithmetic is described in fx.cuh).
//
// Semantics are those of quantumflow/backend/numpybk.py:159-214 tensormul
// applied in list order (quantumflow/circuits.py:87-99): the state is swept
// once per pass, each pass applying a run of gates whose dense qubits fit one
// thread's register group.
//
// Kernels:
//   k_fxdense1  one 2x2 gate on any bit (a thread holds two amplitude pairs)
//   k_fxdense2  one 4x4 gate on any two bits (a thread holds one quad)
//   k_fxgroup<G> an op program on a group of 2^G amplitudes per thread (the
//               pass's dense gate bits, G <= 4): 2x2 and 4x4 gates at one
//               canonical register place with register-bit exchanges
//               between them, sign (CZ-like), diagonal and phase ops; G = 0
//               is a pass of element-wise ops only
// Each kernel converts the amplitudes it holds to fixed point once, applies
// its gates, and rounds to FP64 once.
#include <algorithm>
#include <cstring>

#include "engine.cuh"
#include "fx.cuh"

namespace qf {

int* device_error_word();

// ------------------------------------------------------------- device ----
// largest FP64 exponent field among the parts of v[]
template <int R>
QF_D int fx_group_exp_raw(const double2 (&v)[R]) {
  uint32_t m = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    m = max(m, fx_hiword(v[r].x) & 0x7fffffffu);
    m = max(m, fx_hiword(v[r].y) & 0x7fffffffu);
  }
  return static_cast<int>(m >> 20);
}
// the group exponent fx_in takes: a group of parts below 2^-959 becomes all
// zero (an exponent no part reaches shifts every part out)
QF_D int fx_exp_final(int e) { return e < FX_EMIN ? 4095 : e; }
template <int R>
QF_D int fx_group_exp(const double2 (&v)[R]) {
  return fx_exp_final(fx_group_exp_raw<R>(v));
}

template <int M>
QF_D FxAmp fx_load_amp(double2 v, int E) {
  FxAmp a;
  fx_in<M>(v.x, E, a.rh, a.rl);
  fx_in<M>(v.y, E, a.ih, a.il);
  return a;
}
template <int M>
QF_D double2 fx_store_amp(const FxAmp& a, int E) {
  return make_double2(fx_out<M>(fx_t_of(a.rh, a.rl), E), fx_out<M>(fx_t_of(a.ih, a.il), E));
}
// flip the FP64 sign of both parts (a pending CZ-like sign at store time)
// as an integer XOR of the sign bits: a floating-point negation can take the
// FP64 pipe, a few lanes per clock on this part
QF_D double2 fx_flip(double2 v, bool neg) {
  const uint32_t s = neg ? 0x80000000u : 0u;
  return make_double2(fx_double(fx_hiword(v.x) ^ s, fx_loword(v.x)), fx_double(fx_hiword(v.y) ^ s, fx_loword(v.y)));
}

struct FxCoef4 {
  FxC c[4];
};
struct FxCoef16 {
  FxC c[16];
};

// 2x2 gate on bit b: each thread takes pairs t and t + nthr per iteration
template <typename IT>
__global__ void __launch_bounds__(256) k_fxdense1(const double2* __restrict__ in, double2* out, IT npairs, int b,
                                                  const __grid_constant__ FxCoef4 u) {
  constexpr int M = 57;
  const IT nthr = (IT)gridDim.x * blockDim.x;
  const IT bit = IT(1) << b;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < npairs; t += 2 * nthr) {
    const IT t2 = t + nthr;
    const bool has2 = t2 < npairs;
    const IT i0 = insert0(t, b);
    const IT j0 = has2 ? insert0(t2, b) : i0;
    double2 a[2] = {in[i0], in[i0 | bit]};
    double2 c[2];
    if (has2) {
      c[0] = in[j0];
      c[1] = in[j0 | bit];
    }
    {
      const int E = fx_group_exp<2>(a);
      FxAmp f[2] = {fx_load_amp<M>(a[0], E), fx_load_amp<M>(a[1], E)};
      int64_t tr, ti;
      fx_cdot<2>(&u.c[0], f, tr, ti);
      out[i0] = make_double2(fx_out_br<M>(tr, E), fx_out_br<M>(ti, E));
      fx_cdot<2>(&u.c[2], f, tr, ti);
      out[i0 | bit] = make_double2(fx_out_br<M>(tr, E), fx_out_br<M>(ti, E));
    }
    if (has2) {
      const int E = fx_group_exp<2>(c);
      FxAmp f[2] = {fx_load_amp<M>(c[0], E), fx_load_amp<M>(c[1], E)};
      int64_t tr, ti;
      fx_cdot<2>(&u.c[0], f, tr, ti);
      out[j0] = make_double2(fx_out_br<M>(tr, E), fx_out_br<M>(ti, E));
      fx_cdot<2>(&u.c[2], f, tr, ti);
      out[j0 | bit] = make_double2(fx_out_br<M>(tr, E), fx_out_br<M>(ti, E));
    }
  }
}

// 4x4 gate on bits q0 (matrix MSB) and q1
template <typename IT>
__global__ void __launch_bounds__(256) k_fxdense2(const double2* __restrict__ in, double2* out, IT nquads, int q0,
                                                  int q1, const __grid_constant__ FxCoef16 u) {
  constexpr int M = 57;
  const int lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0;
  const IT b0 = IT(1) << q0, b1 = IT(1) << q1;
  const IT nthr = (IT)gridDim.x * blockDim.x;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < nquads; t += nthr) {
    const IT base = insert0(insert0(t, lo), hi);
    const IT idx[4] = {base, base | b1, base | b0, base | b0 | b1};
    double2 a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = in[idx[r]];
    const int E = fx_group_exp<4>(a);
    FxAmp f[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) f[r] = fx_load_amp<M>(a[r], E);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int64_t tr, ti;
      fx_cdot<4>(&u.c[4 * r], f, tr, ti);
      out[idx[r]] = make_double2(fx_out_br<M>(tr, E), fx_out_br<M>(ti, E));
    }
  }
}

// ----------------------------------------------------------- group pass ----
// A thread holds the 2^G amplitudes of the pass's gate bits; register-index
// bit j holds one of those global bits, as the host tracks it.  Gates run in
// one canonical place -- a 2x2 gate on register bit G-1, a 4x4 gate with
// its matrix MSB on bit G-1 and LSB on bit G-2 -- and the host inserts
// register-bit exchanges (FXI_SWAP) to bring each gate's bits there, so the
// kernel holds one body per gate kind instead of one per bit combination.
constexpr int FXG_MAX_OPS = 96;
constexpr int FXG_MAX_COEF = 640;
enum FxInstr : uint8_t {
  FXI_SWAP = 1,    // exchange register-index bits a < b
  FXI_DENSE1 = 2,  // 2x2 on register bit G-1
  FXI_DENSE2 = 3,  // 4x4, MSB on bit G-1, LSB on bit G-2
  FXI_SIGN = 4,    // negate registers rmask when the bits mout of xb are set
  FXI_DIAG = 5,    // diagonal on k <= 3 bits (register bit rb[i], or global bit gb[i] of xb)
  FXI_PHASE = 6,   // global scalar
};
struct FxGroupOp {
  uint8_t type;
  uint8_t a, b;    // SWAP: register bits, a < b
  uint8_t k;       // DIAG: qubits
  int8_t rb[3];    // DIAG: register bit of the op's bit i (MSB first), -1 outside the group
  uint8_t gb[3];   // DIAG: global bit of the op's bit i
  uint16_t coef;   // first coefficient
  uint16_t rmask;  // SIGN: registers whose group bits of the op are all set
  uint64_t mout;   // SIGN: the op's global bits outside the group
};
struct FxGroupParams {
  const double2* in;
  double2* out;
  int32_t n, nops;
  uint8_t sbits[4];     // the group bits, ascending
  int32_t pad;
  int64_t off_in[16];   // global offset of register index r at load
  int64_t off_out[16];  // ... at store (after the pass's exchanges)
  FxGroupOp ops[FXG_MAX_OPS];
  FxC coef[FXG_MAX_COEF];
};

// 2x2 on register bit G-1
template <int G>
QF_D void fxg_dense1(const FxC* cf, FxAmp (&v)[1 << G]) {
  constexpr int H = 1 << (G - 1);
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const FxAmp p[2] = {v[i], v[i + H]};
    int64_t tr, ti;
    fx_cdot<2>(cf, p, tr, ti);
    v[i] = fx_amp_from_t(tr, ti);
    fx_cdot<2>(cf + 2, p, tr, ti);
    v[i + H] = fx_amp_from_t(tr, ti);
  }
}
// 4x4 with its MSB on register bit G-1 and LSB on bit G-2
template <int G>
QF_D void fxg_dense2(const FxC* cf, FxAmp (&v)[1 << G]) {
  constexpr int Q = 1 << (G - 2);
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const FxAmp p[4] = {v[i], v[i + Q], v[i + 2 * Q], v[i + 3 * Q]};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int64_t tr, ti;
      fx_cdot<4>(cf + 4 * r, p, tr, ti);
      v[i + r * Q] = fx_amp_from_t(tr, ti);
    }
  }
}
// exchange register-index bits A < B (register moves only)
template <int G, int A, int B>
QF_D void fxg_swap(FxAmp (&v)[1 << G]) {
#pragma unroll
  for (int r = 0; r < (1 << G); ++r)
    if (((r >> A) & 1) && !((r >> B) & 1)) {
      const int s = r ^ (1 << A) ^ (1 << B);
      const FxAmp t = v[r];
      v[r] = v[s];
      v[s] = t;
    }
}
template <int G>
QF_D void fxg_swap_dispatch(int a, int b, FxAmp (&v)[1 << G]) {
  if constexpr (G >= 2) {
    switch (a * 4 + b) {
      case 1: fxg_swap<G, 0, 1>(v); break;
      case 2: if constexpr (G > 2) fxg_swap<G, 0, 2>(v); break;
      case 6: if constexpr (G > 2) fxg_swap<G, 1, 2>(v); break;
      case 3: if constexpr (G > 3) fxg_swap<G, 0, 3>(v); break;
      case 7: if constexpr (G > 3) fxg_swap<G, 1, 3>(v); break;
      case 11: if constexpr (G > 3) fxg_swap<G, 2, 3>(v); break;
    }
  }
}

template <int G>
QF_D void fxg_negate(uint32_t neg, FxAmp (&v)[1 << G]) {
#pragma unroll
  for (int r = 0; r < (1 << G); ++r)
    if ((neg >> r) & 1u) v[r] = fx_neg(v[r]);
}

// one coefficient per amplitude: v *= c
QF_D FxAmp fx_mul1(const FxC& c, const FxAmp& a) {
  int64_t tr, ti;
  fx_cdot<1>(&c, &a, tr, ti);
  return fx_amp_from_t(tr, ti);
}

constexpr int FXG_THREADS = 128;

template <int G, typename IT>
__global__ void __launch_bounds__(FXG_THREADS) k_fxgroup(const __grid_constant__ FxGroupParams P) {
  constexpr int R = 1 << G;
  constexpr int M = G <= 2 ? 57 : 56;
  const IT ngroups = IT(1) << (P.n - G);
  const IT nthr = (IT)gridDim.x * blockDim.x;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < ngroups; t += nthr) {
    IT xb = t;
#pragma unroll
    for (int j = 0; j < G; ++j) xb = insert0(xb, (int)P.sbits[j]);
    double2 a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = P.in[xb | (IT)P.off_in[r]];
    const int E = fx_group_exp<R>(a);
    FxAmp v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = fx_load_amp<M>(a[r], E);
    uint32_t neg = 0;  // CZ-like signs not yet applied (register mask)
    for (int o = 0; o < P.nops; ++o) {
      const FxGroupOp& op = P.ops[o];
      switch (op.type) {
        case FXI_SIGN:
          if ((xb & (IT)op.mout) == (IT)op.mout) neg ^= op.rmask;
          break;
        case FXI_SWAP:
          fxg_negate<G>(neg, v);
          neg = 0;
          fxg_swap_dispatch<G>(op.a, op.b, v);
          break;
        case FXI_DENSE1:
          if constexpr (G >= 1) {
            fxg_negate<G>(neg, v);
            neg = 0;
            fxg_dense1<G>(&P.coef[op.coef], v);
          }
          break;
        case FXI_DENSE2:
          if constexpr (G >= 2) {
            fxg_negate<G>(neg, v);
            neg = 0;
            fxg_dense2<G>(&P.coef[op.coef], v);
          }
          break;
        case FXI_DIAG:
#pragma unroll
          for (int r = 0; r < R; ++r) {
            int idx = 0;
            for (int i = 0; i < op.k; ++i) {
              const int bit = op.rb[i] >= 0 ? (r >> op.rb[i]) & 1 : int((xb >> op.gb[i]) & 1);
              idx = (idx << 1) | bit;
            }
            v[r] = fx_mul1(P.coef[op.coef + idx], v[r]);
          }
          break;
        case FXI_PHASE:
#pragma unroll
          for (int r = 0; r < R; ++r) v[r] = fx_mul1(P.coef[op.coef], v[r]);
          break;
        default:
          break;
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      P.out[xb | (IT)P.off_out[r]] = fx_flip(fx_store_amp<M>(v[r], E), (neg >> r) & 1u);
  }
}

// ---------------------------------------------------------- shape passes ----
// Straight-line passes for the common programs: one or two dense gates
// (slots) at fixed register bits -- the shape table shared with the
// float-float engine (group.cu): slot code 10 + j is a 2x2 gate on register
// bit j, 100 + 10 j0 + j1 a 4x4 gate with its matrix MSB on bit j0 and LSB on
// j1 -- with CZ-like signs before, between and after the slots.  The
// coefficients sit at fixed parameter offsets (slot s at coef[16 s]), so the
// products read them as constant operands.  Signs before the first slot and
// after the last flip FP64 sign bits (exact); only signs between the slots
// negate fixed-point registers.
constexpr int FXS_THREADS = 128;
struct FxShapeParams {
  const double2* in;
  double2* out;
  int32_t n, shape;
  int32_t sign_end[3];  // signs [sign_end[b-1], sign_end[b]) act before slot b (b = 2: after the last)
  int32_t pad;
  uint8_t sbits[4];     // the group bits, ascending
  int32_t pad2;
  int64_t off[16];      // global offset of register index r
  uint16_t rmask[SHAPE_MAX_SIGNS];
  uint64_t mout[SHAPE_MAX_SIGNS];
  FxC coef[32];         // slot s at coef[16 s]
};

// 2x2 on register bit J / 4x4 with MSB on register bit J0 and LSB on J1
template <int G, int J>
QF_D void fxs_dense1(const FxC* cf, FxAmp (&v)[1 << G]) {
#pragma unroll
  for (int i = 0; i < (1 << (G - 1)); ++i) {
    const int i0 = ((i >> J) << (J + 1)) | (i & ((1 << J) - 1));
    const int i1 = i0 | (1 << J);
    const FxAmp p[2] = {v[i0], v[i1]};
    int64_t tr, ti;
    fx_cdot<2>(cf, p, tr, ti);
    v[i0] = fx_amp_from_t(tr, ti);
    fx_cdot<2>(cf + 2, p, tr, ti);
    v[i1] = fx_amp_from_t(tr, ti);
  }
}
template <int G, int J0, int J1>
QF_D void fxs_dense2(const FxC* cf, FxAmp (&v)[1 << G]) {
  constexpr int LO = J0 < J1 ? J0 : J1, HI = J0 < J1 ? J1 : J0;
#pragma unroll
  for (int i = 0; i < (1 << (G - 2)); ++i) {
    int b = ((i >> LO) << (LO + 1)) | (i & ((1 << LO) - 1));
    b = ((b >> HI) << (HI + 1)) | (b & ((1 << HI) - 1));
    const int idx[4] = {b, b | (1 << J1), b | (1 << J0), b | (1 << J0) | (1 << J1)};
    const FxAmp p[4] = {v[idx[0]], v[idx[1]], v[idx[2]], v[idx[3]]};
    int64_t tr[4], ti[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) fx_cdot<4>(cf + 4 * r, p, tr[r], ti[r]);
#pragma unroll
    for (int r = 0; r < 4; ++r) v[idx[r]] = fx_amp_from_t(tr[r], ti[r]);
  }
}
template <int G, int S>
QF_D void fxs_slot(const FxC* cf, FxAmp (&v)[1 << G]) {
  if constexpr (S >= 100) {
    fxs_dense2<G, (S / 10) % 10, S % 10>(cf, v);
  } else if constexpr (S >= 10) {
    fxs_dense1<G, S - 10>(cf, v);
  }
}

// the last slot of a pass: results stay as T values (units of A / 4) and are
// rounded to FP64 straight from there
template <int G, int J>
QF_D void fxs_dense1_t(const FxC* cf, const FxAmp (&v)[1 << G], int64_t (&tr)[1 << G], int64_t (&ti)[1 << G]) {
#pragma unroll
  for (int i = 0; i < (1 << (G - 1)); ++i) {
    const int i0 = ((i >> J) << (J + 1)) | (i & ((1 << J) - 1));
    const int i1 = i0 | (1 << J);
    const FxAmp p[2] = {v[i0], v[i1]};
    fx_cdot<2>(cf, p, tr[i0], ti[i0]);
    fx_cdot<2>(cf + 2, p, tr[i1], ti[i1]);
  }
}
template <int G, int J0, int J1>
QF_D void fxs_dense2_t(const FxC* cf, const FxAmp (&v)[1 << G], int64_t (&tr)[1 << G], int64_t (&ti)[1 << G]) {
  constexpr int LO = J0 < J1 ? J0 : J1, HI = J0 < J1 ? J1 : J0;
#pragma unroll
  for (int i = 0; i < (1 << (G - 2)); ++i) {
    int b = ((i >> LO) << (LO + 1)) | (i & ((1 << LO) - 1));
    b = ((b >> HI) << (HI + 1)) | (b & ((1 << HI) - 1));
    const int idx[4] = {b, b | (1 << J1), b | (1 << J0), b | (1 << J0) | (1 << J1)};
    const FxAmp p[4] = {v[idx[0]], v[idx[1]], v[idx[2]], v[idx[3]]};
#pragma unroll
    for (int r = 0; r < 4; ++r) fx_cdot<4>(cf + 4 * r, p, tr[idx[r]], ti[idx[r]]);
  }
}
template <int G, int S>
QF_D void fxs_slot_t(const FxC* cf, const FxAmp (&v)[1 << G], int64_t (&tr)[1 << G], int64_t (&ti)[1 << G]) {
  if constexpr (S >= 100) {
    fxs_dense2_t<G, (S / 10) % 10, S % 10>(cf, v, tr, ti);
  } else {
    fxs_dense1_t<G, S - 10>(cf, v, tr, ti);
  }
}

// MINB: resident CTAs per SM the register allocation must allow (narrow
// shapes need few registers; the widest are tuned by qf_set_fx_occupancy)
template <int G, int S0, int S1, typename IT, int MINB = (G <= 1 ? 8 : G == 2 ? 4 : 1)>
__global__ void __launch_bounds__(FXS_THREADS, MINB) k_fxshape(const __grid_constant__ FxShapeParams P) {
  constexpr int R = 1 << G;
  constexpr int M = G <= 2 ? 56 : 55;
  const IT ngroups = IT(1) << (P.n - G);
  const IT nthr = (IT)gridDim.x * blockDim.x;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < ngroups; t += nthr) {
    IT xb = t;
#pragma unroll
    for (int j = 0; j < G; ++j) xb = insert0(xb, (int)P.sbits[j]);
    double2 a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = P.in[xb | (IT)P.off[r]];
    auto signs = [&](int s0, int s1) {
      uint32_t m = 0;
      for (int s = s0; s < s1; ++s)
        if ((xb & (IT)P.mout[s]) == (IT)P.mout[s]) m ^= P.rmask[s];
      return m;
    };
    if (P.sign_end[0] > 0) {
      const uint32_t m = signs(0, P.sign_end[0]);
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = fx_flip(a[r], (m >> r) & 1u);
    }
    const int E = fx_group_exp<R>(a);
    FxAmp v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = fx_load_amp<M>(a[r], E);
    int64_t tr[R], ti[R];
    if constexpr (S1 != 0) {
      fxs_slot<G, S0>(&P.coef[0], v);
      if (P.sign_end[1] > P.sign_end[0]) {
        const uint32_t m = signs(P.sign_end[0], P.sign_end[1]);
#pragma unroll
        for (int r = 0; r < R; ++r)
          if ((m >> r) & 1u) v[r] = fx_neg(v[r]);
      }
      fxs_slot_t<G, S1>(&P.coef[16], v, tr, ti);
    } else {
      fxs_slot_t<G, S0>(&P.coef[0], v, tr, ti);
    }
    const uint32_t m = P.sign_end[2] > P.sign_end[1] ? signs(P.sign_end[1], P.sign_end[2]) : 0u;
#pragma unroll
    for (int r = 0; r < R; ++r)
      P.out[xb | (IT)P.off[r]] = fx_flip(make_double2(fx_out<M>(tr[r], E), fx_out<M>(ti[r], E)), (m >> r) & 1u);
  }
}


// The widest shape (a 4x4 gate on register bits (3,2), then one on (1,0)) on
// a pair of threads: each holds 8 of the group's 16 amplitudes, so a thread
// needs about half the registers and twice as many warps fit an SM.  For the
// first gate a thread holds the amplitudes whose register bit 0 is its half
// p; the pair then trades four amplitudes through warp shuffles so that for
// the second gate a thread holds those whose register bit 3 is p.  Both
// halves use the group's common exponent (a shuffled maximum).  Every lane of
// a warp runs the same number of iterations (the thread count is a multiple
// of 32), as the shuffles require.
template <typename IT>
__global__ void __launch_bounds__(FXS_THREADS, 3) k_fxpair(const __grid_constant__ FxShapeParams P) {
  constexpr int M = 55;
  const IT nitems = IT(2) << (P.n - 4);  // two threads per group
  const IT nthr = (IT)gridDim.x * blockDim.x;
  for (IT t = (IT)blockIdx.x * blockDim.x + threadIdx.x; t < nitems; t += nthr) {
    const int p = (int)(t & 1);
    IT xb = t >> 1;
#pragma unroll
    for (int j = 0; j < 4; ++j) xb = insert0(xb, (int)P.sbits[j]);
    auto signs = [&](int s0, int s1) {
      uint32_t m = 0;
      for (int s = s0; s < s1; ++s)
        if ((xb & (IT)P.mout[s]) == (IT)P.mout[s]) m ^= P.rmask[s];
      return m;
    };
    // phase 1: local i (bits 3,2,1 of the register) <-> register 2 i + p
    double2 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = P.in[xb | (IT)P.off[2 * i + p]];
    if (P.sign_end[0] > 0) {
      const uint32_t m = signs(0, P.sign_end[0]);
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = fx_flip(a[i], (m >> (2 * i + p)) & 1u);
    }
    // the exponent of all 16 amplitudes (maximum of the raw exponents first)
    const int e_own = fx_group_exp_raw<8>(a);
    const int e_oth = __shfl_xor_sync(0xffffffffu, e_own, 1);
    const int E = fx_exp_final(e_own > e_oth ? e_own : e_oth);
    FxAmp v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = fx_load_amp<M>(a[i], E);
    fxs_dense2<3, 2, 1>(&P.coef[0], v);  // register bits (3,2) are local bits (2,1)
    if (P.sign_end[1] > P.sign_end[0]) {
      const uint32_t m = signs(P.sign_end[0], P.sign_end[1]);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if ((m >> (2 * i + p)) & 1u) v[i] = fx_neg(v[i]);
    }
    // exchange: keep register bit 3 == p, send bit 3 == !p; phase 2 local j
    // (bits 2,1,0 of the register) <-> register 8 p + j
    FxAmp w[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const FxAmp keep = p ? v[4 + k] : v[k];
      const FxAmp send = p ? v[k] : v[4 + k];
      FxAmp recv;
      recv.rh = __shfl_xor_sync(0xffffffffu, send.rh, 1);
      recv.rl = __shfl_xor_sync(0xffffffffu, send.rl, 1);
      recv.ih = __shfl_xor_sync(0xffffffffu, send.ih, 1);
      recv.il = __shfl_xor_sync(0xffffffffu, send.il, 1);
      w[2 * k] = p ? recv : keep;      // register bit 0 = 0
      w[2 * k + 1] = p ? keep : recv;  // register bit 0 = 1
    }
    int64_t tr[8], ti[8];
    fxs_dense2_t<3, 1, 0>(&P.coef[16], w, tr, ti);
    const uint32_t m = P.sign_end[2] > P.sign_end[1] ? signs(P.sign_end[1], P.sign_end[2]) : 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int r = 8 * p + j;
      P.out[xb | (IT)P.off[r]] = fx_flip(make_double2(fx_out<M>(tr[j], E), fx_out<M>(ti[j], E)), (m >> r) & 1u);
    }
  }
}

using FxShapeKernel = void (*)(FxShapeParams);
#define QF_FX_SHAPES(IT)                                                                                    \
  {                                                                                                        \
    k_fxshape<1, 10, 0, IT>, k_fxshape<2, 110, 0, IT>, k_fxshape<1, 10, 10, IT>, k_fxshape<2, 11, 10, IT>,       \
        k_fxshape<2, 11, 110, IT>, k_fxshape<3, 12, 110, IT>, k_fxshape<2, 110, 11, IT>,                         \
        k_fxshape<2, 110, 10, IT>, k_fxshape<3, 121, 10, IT>, k_fxshape<2, 110, 110, IT>,                        \
        k_fxshape<3, 121, 120, IT>, k_fxshape<3, 121, 110, IT>, k_fxshape<4, 132, 110, IT>,                      \
  }
// the same order as the shape table of group.cu
static const FxShapeKernel kFxShapes32[] = QF_FX_SHAPES(uint32_t);
static const FxShapeKernel kFxShapes64[] = QF_FX_SHAPES(int64_t);
#undef QF_FX_SHAPES
// register-capped forms of the widest shapes (more resident warps, fewer
// registers each; qf_set_fx_occupancy)
#define QF_FX_WIDE(IT, B)                                                                              \
  { k_fxshape<3, 121, 120, IT, B>, k_fxshape<3, 121, 110, IT, B>, k_fxshape<4, 132, 110, IT, B> }
static const FxShapeKernel kFxWide32[3][3] = {QF_FX_WIDE(uint32_t, 2), QF_FX_WIDE(uint32_t, 3),
                                              QF_FX_WIDE(uint32_t, 4)};
#undef QF_FX_WIDE
int g_fx_min_blocks = 1;  // CTAs of the widest shape kernels per SM the registers must allow (1..4)
static const int kFxShapeG[] = {1, 2, 1, 2, 2, 3, 2, 2, 3, 2, 3, 3, 4};

// --------------------------------------------------------------- host ----
namespace {

constexpr double FX_UNIT_TOL = 1e-9;

bool unit_modulus(cplx c) { return std::abs(std::abs(c) - 1.0) <= FX_UNIT_TOL; }

// the fixed-point kernels take unitary gates only (their overflow bound
// rests on the group norm being preserved)
bool unitary(const std::vector<cplx>& m, int G) {
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j) {
      cplx d(0, 0);
      for (int k = 0; k < G; ++k) d += m[i * G + k] * std::conj(m[j * G + k]);
      if (std::abs(d - (i == j ? cplx(1, 0) : cplx(0, 0))) > FX_UNIT_TOL) return false;
    }
  return true;
}

// kinds of op for the fixed-point planner
enum FxKind { FXK_DENSE = 1, FXK_ELEM = 2, FXK_NATIVE = 3 };

FxKind fx_kind(const HostOp& op) {
  switch (op.type) {
    case OP_DENSE1:
    case OP_DENSE2:
      return unitary(op.m, 1 << op.k) ? FXK_DENSE : FXK_NATIVE;
    case OP_MONO:  // generalised permutations on <= 2 bits run as dense gates
      if (op.k > 2) return FXK_NATIVE;
      for (int r = 0; r < (1 << op.k); ++r)
        if (!unit_modulus(op.diag[r])) return FXK_NATIVE;
      return FXK_DENSE;
    case OP_SIGN:
      return FXK_ELEM;
    case OP_DIAG:
      if (op.k > 3) return FXK_NATIVE;
      for (int r = 0; r < (1 << op.k); ++r)
        if (!unit_modulus(op.diag[r])) return FXK_NATIVE;
      return FXK_ELEM;
    case OP_PHASE:
      return unit_modulus(op.scalar) ? FXK_ELEM : FXK_NATIVE;
    default:  // dense gates on 3..5 qubits, QAOA cut-table phases
      return FXK_NATIVE;  // dense gates on 3..5 qubits
  }
}

int fx_coef_count(const HostOp& op) {
  switch (op.type) {
    case OP_DENSE1: return 4;
    case OP_DENSE2: return 16;
    case OP_MONO: return op.k == 1 ? 4 : 16;
    case OP_DIAG: return 1 << op.k;
    case OP_PHASE: return 1;
  }
  return 0;
}

std::vector<cplx> dense_matrix(const HostOp& op) {
  const int D = 1 << op.k;
  if (op.type != OP_MONO) return op.m;
  std::vector<cplx> m((size_t)D * D, cplx(0, 0));
  for (int r = 0; r < D; ++r) m[r * D + op.perm[r]] = op.diag[r];
  return m;
}

struct FxBlock {
  std::vector<int> idx;
  int order[4] = {0, 0, 0, 0};  // dense bits in order of first use
  int G = 0;
  bool native = false;  // one op run by the native FP64 kernels
  bool wide = false;    // one unitary gate on 3 or 4 qubits for the tensor-core pass
  int ncoef = 0;
  int shape = -1;       // table shape of a straight-line pass (-1: other kernels)
};

// A unitary gate on 3 or 4 qubits (dense, or a generalised permutation
// with unit-modulus entries on 3): the CUDA-core fixed-point kernels do not
// take it, but it is one 16x16 window of the tensor-core pass.
bool tx_wide(const HostOp& op) {
  if (op.type == OP_DENSEK) return op.k <= 4 && unitary(op.m, 1 << op.k);
  if (op.type == OP_MONO && op.k == 3) {
    for (int r = 0; r < 8; ++r)
      if (!unit_modulus(op.diag[r])) return false;
    return true;
  }
  return false;
}

constexpr int FX_G_MAX = 4;

// Greedy passes: element-wise ops join the current pass; a dense op joins
// while the pass's dense bits stay within gmax; ops the fixed-point kernels
// do not take close the pass and run alone in native FP64.
std::vector<FxBlock> fx_split_shapes(std::vector<FxBlock>& blocks, const std::vector<HostOp>& ops);

std::vector<FxBlock> fx_plan(std::vector<HostOp>& ops, int n, int& fusion_k, bool split = true,
                             bool wide_ok = false) {
  if (fusion_k <= 0) fusion_k = FX_G_MAX;
  if (fusion_k > 1 && g_merge_gates) merge_ops(ops, n);
  // generalised permutations on <= 2 qubits with unit-modulus entries run as
  // dense gates here (one code path for the fixed-point passes)
  for (HostOp& op : ops)
    if (op.type == OP_MONO && fx_kind(op) == FXK_DENSE) {
      op.m = dense_matrix(op);
      op.type = op.k == 1 ? OP_DENSE1 : OP_DENSE2;
    }
  const int gmax = std::min(fusion_k, FX_G_MAX);
  const bool fuse = fusion_k > 1;
  std::vector<FxBlock> blocks;
  FxBlock cur;
  auto close = [&]() {
    if (!cur.idx.empty()) blocks.push_back(cur);
    cur = FxBlock();
  };
  for (int i = 0; i < (int)ops.size(); ++i) {
    const HostOp& op = ops[i];
    const FxKind kind = fx_kind(op);
    const int need = fx_coef_count(op);
    if (kind == FXK_NATIVE) {
      close();
      cur.idx.push_back(i);
      if (wide_ok && tx_wide(op)) {
        cur.wide = true;
        cur.G = op.k;
        for (int j = 0; j < op.k; ++j) cur.order[j] = op.gb[j];
      } else {
        cur.native = true;
      }
      close();
      continue;
    }
    int add[2], nadd = 0;
    if (kind == FXK_DENSE)
      for (int j = 0; j < op.k; ++j)
        if (std::find(cur.order, cur.order + cur.G, op.gb[j]) == cur.order + cur.G) add[nadd++] = op.gb[j];
    const bool fits = cur.G + nadd <= gmax && (int)cur.idx.size() < FXG_MAX_OPS / 3 &&
                      cur.ncoef + need <= FXG_MAX_COEF;
    if (!cur.idx.empty() && (!fuse || !fits)) close();
    if (kind == FXK_DENSE) {
      for (int j = 0; j < op.k; ++j)
        if (std::find(cur.order, cur.order + cur.G, op.gb[j]) == cur.order + cur.G) cur.order[cur.G++] = op.gb[j];
    }
    cur.idx.push_back(i);
    cur.ncoef += need;
  }
  close();
  return split ? fx_split_shapes(blocks, ops) : blocks;
}

// Passes made of dense gates and signs only are cut where their next dense
// gate would leave the shape table, so each piece runs straight-line.
std::vector<FxBlock> fx_split_shapes(std::vector<FxBlock>& blocks, const std::vector<HostOp>& ops) {
  std::vector<FxBlock> out;
  out.reserve(blocks.size());
  for (FxBlock& b : blocks) {
    bool ok = !b.native && b.G > 0;
    for (int i : b.idx) {
      const uint8_t t = ops[i].type;
      ok = ok && (t == OP_DENSE1 || t == OP_DENSE2 || t == OP_SIGN);
    }
    if (!ok) {
      out.push_back(std::move(b));
      continue;
    }
    FxBlock cur;
    int dense[3], nd = 0;
    auto finish = [&]() {
      if (cur.idx.empty()) return;
      int order[4], G = 0, s0 = 0, s1 = 0;
      bool swap[2];
      cur.shape = shape_lookup(ops, dense, nd, order, G, swap, &s0, &s1);
      cur.G = G;
      for (int k = 0; k < G; ++k) cur.order[k] = order[k];
      out.push_back(std::move(cur));
      cur = FxBlock();
      nd = 0;
    };
    for (int i : b.idx) {
      if (ops[i].type != OP_SIGN) {
        if (nd > 0) {
          int order[4], G = 0, s0 = 0, s1 = 0;
          bool swap[2];
          dense[nd] = i;
          if (nd == 2 || shape_lookup(ops, dense, nd + 1, order, G, swap, &s0, &s1) < 0) finish();
        }
        dense[nd++] = i;
      }
      cur.idx.push_back(i);
    }
    finish();
  }
  return out;
}

int grid_cap(int64_t items) {
  const int64_t cap = (int64_t)device_sm_count() * 8;
  int64_t g = (items + 255) / 256;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}


int launch_fx_single(const void* in, void* out, int n, const HostOp& op, cudaStream_t stream) {
  const double2* src = reinterpret_cast<const double2*>(in);
  double2* dst = reinterpret_cast<double2*>(out);
  const std::vector<cplx> m = dense_matrix(op);
  if (op.k == 1) {
    FxCoef4 u;
    for (int i = 0; i < 4; ++i) u.c[i] = make_fxc(m[i].real(), m[i].imag());
    const int64_t np = int64_t(1) << (n - 1);
    const int grid = grid_cap((np + 1) / 2);
    if (n <= 31)
      k_fxdense1<uint32_t><<<grid, 256, 0, stream>>>(src, dst, (uint32_t)np, op.gb[0], u);
    else
      k_fxdense1<int64_t><<<grid, 256, 0, stream>>>(src, dst, np, op.gb[0], u);
  } else {
    FxCoef16 u;
    for (int i = 0; i < 16; ++i) u.c[i] = make_fxc(m[i].real(), m[i].imag());
    const int64_t nq = int64_t(1) << (n - 2);
    if (n <= 31)
      k_fxdense2<uint32_t><<<grid_cap(nq), 256, 0, stream>>>(src, dst, (uint32_t)nq, op.gb[0], op.gb[1], u);
    else
      k_fxdense2<int64_t><<<grid_cap(nq), 256, 0, stream>>>(src, dst, nq, op.gb[0], op.gb[1], u);
  }
  return check_cuda(cudaGetLastError());
}

// Fill the group parameters of block B: its dense bits are the register
// bits, placed so that the first dense gate needs no exchange; before every
// later dense gate the exchanges that bring its bits to the canonical
// register bits are emitted, and the host follows the register <-> global
// bit map through them (element-wise ops and the store use the map in force
// at their point of the program).
int fx_group_prepare(int n, const std::vector<HostOp>& ops, const FxBlock& B, FxGroupParams& P) {
  const int G = B.G;
  if (n - G < 0 || (int)B.idx.size() * 3 > FXG_MAX_OPS) return QF_ERR_NOT_SUPPORTED;
  std::memset(&P, 0, sizeof(FxGroupParams));
  P.n = n;
  int pos[4] = {0, 0, 0, 0};  // global bit held by register-index bit j
  {
    int first = -1;
    for (int i : B.idx)
      if (fx_kind(ops[i]) == FXK_DENSE) {
        first = i;
        break;
      }
    int placed = 0;
    auto place = [&](int bit) {
      for (int j = G - placed; j < G; ++j)
        if (pos[j] == bit) return;
      pos[G - 1 - placed] = bit;
      ++placed;
    };
    if (first >= 0)
      for (int j = 0; j < ops[first].k; ++j) place(ops[first].gb[j]);
    for (int k = 0; k < G; ++k) place(B.order[k]);
  }
  auto reg_of = [&](int bit) {
    for (int j = 0; j < G; ++j)
      if (pos[j] == bit) return j;
    return -1;
  };
  auto offsets = [&](int64_t* off) {
    for (int r = 0; r < (1 << G); ++r) {
      int64_t o = 0;
      for (int j = 0; j < G; ++j)
        if ((r >> j) & 1) o |= int64_t(1) << pos[j];
      off[r] = o;
    }
  };
  uint64_t gmask = 0;
  int sb[4];
  for (int j = 0; j < G; ++j) {
    gmask |= uint64_t(1) << pos[j];
    sb[j] = pos[j];
  }
  std::sort(sb, sb + G);
  for (int j = 0; j < G; ++j) P.sbits[j] = (uint8_t)sb[j];
  offsets(P.off_in);
  int nc = 0, no = 0;
  auto put = [&](cplx v) { P.coef[nc++] = make_fxc(v.real(), v.imag()); };
  auto swap_to = [&](int j, int target) {
    if (j == target) return;
    FxGroupOp& g = P.ops[no++];
    g.type = FXI_SWAP;
    g.a = (uint8_t)std::min(j, target);
    g.b = (uint8_t)std::max(j, target);
    std::swap(pos[j], pos[target]);
  };
  for (int i : B.idx) {
    const HostOp& op = ops[i];
    const int need = fx_coef_count(op);
    if (nc + need > FXG_MAX_COEF || no + 3 > FXG_MAX_OPS) return QF_ERR_NOT_SUPPORTED;
    if (fx_kind(op) == FXK_DENSE) {
      const std::vector<cplx> m = dense_matrix(op);
      if (op.k == 1) {
        swap_to(reg_of(op.gb[0]), G - 1);
        FxGroupOp& g = P.ops[no++];
        g.type = FXI_DENSE1;
        g.coef = (uint16_t)nc;
        for (int e = 0; e < 4; ++e) put(m[e]);
      } else {
        // matrix MSB on the top register bit, or (matrix qubits exchanged)
        // its LSB: whichever needs fewer exchanges
        const int jm = reg_of(op.gb[0]), jl = reg_of(op.gb[1]);
        const int cost_a = (jm != G - 1) + (jl != G - 2), cost_b = (jl != G - 1) + (jm != G - 2);
        const bool exch = cost_b < cost_a;
        const int top = exch ? op.gb[1] : op.gb[0], second = exch ? op.gb[0] : op.gb[1];
        swap_to(reg_of(top), G - 1);
        swap_to(reg_of(second), G - 2);
        FxGroupOp& g = P.ops[no++];
        g.type = FXI_DENSE2;
        g.coef = (uint16_t)nc;
        auto sw = [](int x) { return ((x & 1) << 1) | (x >> 1); };  // exchange the two index bits
        for (int r = 0; r < 4; ++r)
          for (int c = 0; c < 4; ++c) put(exch ? m[sw(r) * 4 + sw(c)] : m[r * 4 + c]);
      }
      continue;
    }
    FxGroupOp& g = P.ops[no++];
    g.coef = (uint16_t)nc;
    switch (op.type) {
      case OP_SIGN: {
        g.type = FXI_SIGN;
        uint64_t msk = 0;
        int jm = 0;
        for (int j = 0; j < op.k; ++j) {
          msk |= uint64_t(1) << op.gb[j];
          const int r = reg_of(op.gb[j]);
          if (r >= 0) jm |= 1 << r;
        }
        g.mout = msk & ~gmask;
        uint32_t rm = 0;
        for (int r = 0; r < (1 << G); ++r)
          if ((r & jm) == jm) rm |= 1u << r;
        g.rmask = (uint16_t)rm;
        break;
      }
      case OP_DIAG:
        g.type = FXI_DIAG;
        g.k = (uint8_t)op.k;
        for (int j = 0; j < op.k; ++j) {
          g.gb[j] = (uint8_t)op.gb[j];
          g.rb[j] = (int8_t)reg_of(op.gb[j]);
        }
        for (int e = 0; e < (1 << op.k); ++e) put(op.diag[e]);
        break;
      case OP_PHASE:
        g.type = FXI_PHASE;
        put(op.scalar);
        break;
      default:
        return QF_ERR_NOT_SUPPORTED;
    }
  }
  offsets(P.off_out);
  P.nops = no;
  return QF_OK;
}

using FxGroupKernel = void (*)(FxGroupParams);
const FxGroupKernel kFxGroup32[5] = {k_fxgroup<0, uint32_t>, k_fxgroup<1, uint32_t>, k_fxgroup<2, uint32_t>,
                                     k_fxgroup<3, uint32_t>, k_fxgroup<4, uint32_t>};
const FxGroupKernel kFxGroup64[5] = {k_fxgroup<0, int64_t>, k_fxgroup<1, int64_t>, k_fxgroup<2, int64_t>,
                                     k_fxgroup<3, int64_t>, k_fxgroup<4, int64_t>};

int fx_group_launch(const FxGroupParams& P, int G, cudaStream_t stream) {
  const int64_t ngroups = int64_t(1) << (P.n - G);
  int64_t grid = (ngroups + FXG_THREADS - 1) / FXG_THREADS;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (grid > cap) grid = cap;
  (P.n <= 31 ? kFxGroup32 : kFxGroup64)[G]<<<(int)grid, FXG_THREADS, 0, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

// kernel used by a block: 0 element-wise group pass, 1 direct sweep,
// 3 group pass, 4 shape pass, 5 native FP64 op, 6 tensor-core pass
int fx_block_kernel(const std::vector<HostOp>& ops, const FxBlock& B) {
  if (B.shape == -2) return 6;
  if (B.native) return 5;
  if (B.G == 0) return 0;
  if (B.idx.size() == 1) return 1;
  if (B.shape >= 0) return 4;
  return 3;
}

// Parameters of a shape pass (dense gates and signs; the shape table names
// the gates' bits in order of first use from the top register bit).
int fx_shape_prepare(int n, const std::vector<HostOp>& ops, const FxBlock& B, FxShapeParams& P) {
  int dense[2], nd = 0, nsign = 0;
  for (int i : B.idx) {
    if (ops[i].type == OP_SIGN) {
      ++nsign;
    } else {
      if (nd == 2) return QF_ERR_NOT_SUPPORTED;
      dense[nd++] = i;
    }
  }
  int order[4], G = 0, s0 = 0, s1 = 0;
  bool swap[2] = {false, false};
  const int shape = shape_lookup(ops, dense, nd, order, G, swap, &s0, &s1);
  if (shape < 0 || nsign > SHAPE_MAX_SIGNS || n - G < 0) return QF_ERR_NOT_SUPPORTED;
  std::memset(&P, 0, sizeof(FxShapeParams));
  P.n = n;
  P.shape = shape;
  int reg_of[64];
  std::fill(reg_of, reg_of + 64, -1);
  uint64_t gmask = 0;
  int rbits[4];
  for (int k = 0; k < G; ++k) {
    rbits[G - 1 - k] = order[k];
    reg_of[order[k]] = G - 1 - k;
    gmask |= uint64_t(1) << order[k];
  }
  int sb[4];
  for (int j = 0; j < G; ++j) sb[j] = rbits[j];
  std::sort(sb, sb + G);
  for (int j = 0; j < G; ++j) P.sbits[j] = (uint8_t)sb[j];
  for (int r = 0; r < (1 << G); ++r) {
    int64_t o = 0;
    for (int j = 0; j < G; ++j)
      if ((r >> j) & 1) o |= int64_t(1) << rbits[j];
    P.off[r] = o;
  }
  int slot = 0, ns = 0;
  for (int i : B.idx) {
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
    for (int b = slot; b < 3; ++b) P.sign_end[b] = ns;  // a dense slot closes the signs before it
    FxC* c = &P.coef[16 * slot];
    if (op.type == OP_DENSE1) {
      for (int e = 0; e < 4; ++e) c[e] = make_fxc(op.m[e].real(), op.m[e].imag());
    } else {
      auto sw = [](int x) { return ((x & 1) << 1) | (x >> 1); };  // exchange the two index bits
      for (int r = 0; r < 4; ++r)
        for (int col = 0; col < 4; ++col) {
          const cplx v = swap[slot] ? op.m[sw(r) * 4 + sw(col)] : op.m[r * 4 + col];
          c[4 * r + col] = make_fxc(v.real(), v.imag());
        }
    }
    ++slot;
  }
  if (nd == 1) P.sign_end[1] = P.sign_end[0];
  P.sign_end[2] = ns;
  return QF_OK;
}

int fx_shape_launch(const FxShapeParams& P, cudaStream_t stream) {
  const int G = kFxShapeG[P.shape];
  const int64_t ngroups = int64_t(1) << (P.n - G);
  int64_t grid = (ngroups + FXS_THREADS - 1) / FXS_THREADS;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  FxShapeKernel kern = (P.n <= 31 ? kFxShapes32 : kFxShapes64)[P.shape];
  if (P.n <= 31 && g_fx_min_blocks > 1 && P.shape >= 10) kern = kFxWide32[g_fx_min_blocks - 2][P.shape - 10];
  if (P.shape == 12 && g_fx_min_blocks == 1 && P.n >= 9) {
    // two threads per group (the thread count, 2^(n-3), is a multiple of 32)
    int64_t g2 = (int64_t(2) << (P.n - 4)) / FXS_THREADS;
    if (g2 > cap) g2 = cap;
    if (g2 < 1) g2 = 1;
    kern = P.n <= 31 ? k_fxpair<uint32_t> : k_fxpair<int64_t>;
    grid = g2;
  }
  kern<<<(int)grid, FXS_THREADS, 0, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

// Double-double complex arithmetic for the pass unitary: products of the
// gates' FP64 entries carried to ~106 bits with FMA-based error-free
// transformations, the same on every host.
struct Dd {
  double hi = 0.0, lo = 0.0;
};
inline Dd dd_norm(double a, double b) {  // |a| >= |b| or a == 0
  const double s = a + b;
  return {s, b - (s - a)};
}
inline Dd dd_add(Dd a, Dd b) {
  const double s = a.hi + b.hi, bb = s - a.hi;
  const double e = (a.hi - (s - bb)) + (b.hi - bb) + a.lo + b.lo;
  return dd_norm(s, e);
}
inline Dd dd_neg(Dd a) { return {-a.hi, -a.lo}; }
inline Dd dd_mul_d(Dd a, double b) {
  const double p = a.hi * b;
  return dd_norm(p, std::fma(a.hi, b, -p) + a.lo * b);
}
struct Cdd {
  Dd re, im;
};
inline bool cdd_zero(const Cdd& v) { return v.re.hi == 0.0 && v.im.hi == 0.0; }
// g * v for an FP64 complex g
inline Cdd cdd_mul(cplx g, const Cdd& v) {
  return {dd_add(dd_mul_d(v.re, g.real()), dd_neg(dd_mul_d(v.im, g.imag()))),
          dd_add(dd_mul_d(v.im, g.real()), dd_mul_d(v.re, g.imag()))};
}
inline Cdd cdd_add(const Cdd& a, const Cdd& b) { return {dd_add(a.re, b.re), dd_add(a.im, b.im)}; }
// v * 2^62 of a double-double rounded to the nearest integer, ties away
// from zero
inline int64_t dd_fixed62(Dd v) {
  const double h = std::ldexp(v.hi, 62), l = std::ldexp(v.lo, 62);
  const double fh = std::floor(h);
  const double frac = (h - fh) + l;  // h - fh is exact; |l| is below half an ulp of h
  int64_t r = static_cast<int64_t>(fh);
  if (frac > 0.5 || (frac == 0.5 && h > 0.0)) ++r;
  else if (frac < -0.5 || (frac == -0.5 && h < 0.0)) --r;
  return r;
}

// Fill the tensor-core pass of block B (dense unitary gates, unit-modulus
// diagonals and phases on its window, sign ops), or return
// QF_ERR_NOT_SUPPORTED.  The window is the block's dense bits, padded to
// four with the highest bits outside them (the rows then keep the low
// bits, so a warp's accesses stay contiguous).  A sign op with bits outside
// the window is moved to the inputs when no earlier dense gate of the block
// touches its window bits, else to the outputs when no later one does.
// With `matrix` false only the structure is checked (the planner's test);
// with it, U is multiplied up in double-double from the gates in block
// order and rounded to the 2^-62 integers of the kernel.
int tx_prepare(int n, const std::vector<HostOp>& ops, const FxBlock& B, TxParams& P, bool matrix = true) {
  if (B.native || B.G < 1 || B.G > 4 || n < 11) return QF_ERR_NOT_SUPPORTED;
  auto dense_op = [](const HostOp& op) {
    return op.type == OP_DENSE1 || op.type == OP_DENSE2 || op.type == OP_DENSEK || op.type == OP_MONO;
  };
  int wb[4], nw = 0;
  for (int j = 0; j < B.G; ++j) wb[nw++] = B.order[j];
  for (int bit = n - 1; nw < 4 && bit >= 0; --bit)
    if (std::find(wb, wb + nw, bit) == wb + nw) wb[nw++] = bit;
  auto pos = [&](int bit) {
    for (int j = 0; j < 4; ++j)
      if (wb[j] == bit) return j;
    return -1;
  };
  std::memset(&P, 0, sizeof(TxParams));
  P.n = n;
  int sb[4] = {wb[0], wb[1], wb[2], wb[3]};
  std::sort(sb, sb + 4);
  for (int j = 0; j < 4; ++j) P.sbits[j] = sb[j];
  for (int c = 0; c < 16; ++c) {
    int64_t o = 0;
    for (int j = 0; j < 4; ++j)
      if ((c >> j) & 1) o |= int64_t(1) << wb[j];
    P.off[c] = o;
  }
  std::vector<Cdd> U, T;
  bool identity = true;  // U is still the identity (the first dense gate is copied, not multiplied)
  if (matrix) {
    U.assign(256, Cdd());
    T.assign(256, Cdd());
    for (int c = 0; c < 16; ++c) U[c * 16 + c].re.hi = 1.0;
  }
  // window bits each dense op of the block touches, for the sign placement
  std::vector<int> dense_pos;
  std::vector<uint32_t> dense_bits;
  for (int k = 0; k < (int)B.idx.size(); ++k) {
    const HostOp& op = ops[B.idx[k]];
    if (dense_op(op)) {
      uint32_t m = 0;
      for (int j = 0; j < op.k; ++j) m |= 1u << pos(op.gb[j]);
      dense_pos.push_back(k);
      dense_bits.push_back(m);
    }
  }
  for (int k = 0; k < (int)B.idx.size(); ++k) {
    const HostOp& op = ops[B.idx[k]];
    if (fx_kind(op) == FXK_NATIVE && !tx_wide(op)) return QF_ERR_NOT_SUPPORTED;
    if (dense_op(op)) {
      int jp[4];
      for (int j = 0; j < op.k; ++j) {
        jp[j] = pos(op.gb[j]);
        if (jp[j] < 0) return QF_ERR_NOT_SUPPORTED;
      }
      if (!matrix) continue;
      const int D = 1 << op.k;
      const std::vector<cplx> gm = dense_matrix(op);
      uint32_t om = 0;
      for (int j = 0; j < op.k; ++j) om |= 1u << jp[j];
      auto local = [&](int c) {  // the gate's matrix index of window index c (gate qubit 0 = MSB)
        int r = 0;
        for (int j = 0; j < op.k; ++j) r = (r << 1) | ((c >> jp[j]) & 1);
        return r;
      };
      auto spread = [&](int r, int m) {  // window index r with the gate's bits set to m
        int cm = r & ~static_cast<int>(om);
        for (int j = 0; j < op.k; ++j)
          if ((m >> (op.k - 1 - j)) & 1) cm |= 1 << jp[j];
        return cm;
      };
      if (identity) {  // U = E: the gate embedded in the window
        for (int r = 0; r < 16; ++r)
          for (int c = 0; c < 16; ++c) {
            Cdd v;
            if ((r & ~static_cast<int>(om)) == (c & ~static_cast<int>(om))) {
              const cplx g = gm[local(r) * D + local(c)];
              v.re.hi = g.real();
              v.im.hi = g.imag();
            }
            U[r * 16 + c] = v;
          }
        identity = false;
        continue;
      }
      // T = E U
      for (int r = 0; r < 16; ++r) {
        const int lr = local(r);
        for (int c = 0; c < 16; ++c) {
          Cdd acc;
          for (int m = 0; m < D; ++m) {
            const cplx g = gm[lr * D + m];
            const Cdd& u = U[spread(r, m) * 16 + c];
            if ((g.real() == 0.0 && g.imag() == 0.0) || cdd_zero(u)) continue;
            acc = cdd_add(acc, cdd_mul(g, u));
          }
          T[r * 16 + c] = acc;
        }
      }
      U.swap(T);
      continue;
    }
    if (op.type == OP_PHASE) {
      if (!matrix) continue;
      for (Cdd& v : U) v = cdd_mul(op.scalar, v);
      identity = false;
      continue;
    }
    if (op.type == OP_DIAG) {
      int jp[3];
      for (int j = 0; j < op.k; ++j) {
        jp[j] = pos(op.gb[j]);
        if (jp[j] < 0) return QF_ERR_NOT_SUPPORTED;
      }
      if (!matrix) continue;
      for (int r = 0; r < 16; ++r) {
        int e = 0;
        for (int j = 0; j < op.k; ++j) e = (e << 1) | ((r >> jp[j]) & 1);
        for (int c = 0; c < 16; ++c) U[r * 16 + c] = cdd_mul(op.diag[e], U[r * 16 + c]);
      }
      identity = false;
      continue;
    }
    if (op.type != OP_SIGN) return QF_ERR_NOT_SUPPORTED;
    uint32_t jm = 0;
    uint64_t mo = 0;
    for (int j = 0; j < op.k; ++j) {
      const int p = pos(op.gb[j]);
      if (p >= 0) jm |= 1u << p;
      else mo |= uint64_t(1) << op.gb[j];
    }
    uint32_t rm = 0;
    for (int c = 0; c < 16; ++c)
      if ((c & jm) == jm) rm |= 1u << c;
    if (mo == 0) {  // inside the window: a diagonal of U
      if (!matrix) continue;
      for (int r = 0; r < 16; ++r)
        if ((rm >> r) & 1)
          for (int c = 0; c < 16; ++c) U[r * 16 + c] = {dd_neg(U[r * 16 + c].re), dd_neg(U[r * 16 + c].im)};
      identity = false;
      continue;
    }
    bool before = false, after = false;
    for (size_t d = 0; d < dense_pos.size(); ++d) {
      if (!(dense_bits[d] & jm)) continue;
      if (dense_pos[d] < k) before = true;
      else after = true;
    }
    if (!before) {
      if (P.nin >= TX_MAX_SIGNS) return QF_ERR_NOT_SUPPORTED;
      P.in_mout[P.nin] = mo;
      P.in_rmask[P.nin++] = (uint16_t)rm;
    } else if (!after) {
      if (P.nout >= TX_MAX_SIGNS) return QF_ERR_NOT_SUPPORTED;
      P.out_mout[P.nout] = mo;
      P.out_rmask[P.nout++] = (uint16_t)rm;
    } else {
      return QF_ERR_NOT_SUPPORTED;
    }
  }
  if (!matrix) return QF_OK;
  for (int r = 0; r < 16; ++r)
    for (int c = 0; c < 16; ++c) {
      const Cdd& v = U[r * 16 + c];
      // unit rows of a product of gates unitary to 1e-9: well inside the
      // digits' bounds (|G| < 2^62.9 keeps G + bias below 2^64)
      if (std::abs(v.re.hi) > 1.0 + 1e-6 || std::abs(v.im.hi) > 1.0 + 1e-6) return QF_ERR_NOT_SUPPORTED;
      P.g[r][c][0] = dd_fixed62(v.re);
      P.g[r][c][1] = dd_fixed62(v.im);
    }
  return QF_OK;
}

}  // namespace

// The passes to run: blocks the tensor-core pass takes stay whole (shape
// -2), the others are cut into straight-line shapes as before.
std::vector<FxBlock> fx_plan_final(std::vector<HostOp>& ops, int n, int& fusion_k) {
  if (!g_fx_tensor || n < 11) return fx_plan(ops, n, fusion_k);
  std::vector<FxBlock> blocks = fx_plan(ops, n, fusion_k, false, true);
  std::vector<FxBlock> out;
  out.reserve(blocks.size());
  static thread_local TxParams tp;  // ~5 KiB: kept off the stack
  for (FxBlock& B : blocks) {
    if (B.wide) {  // a 3- or 4-qubit gate: alone on the tensor cores, else native FP64
      if (tx_prepare(n, ops, B, tp, false) == QF_OK) B.shape = -2;
      else B.native = true;
      out.push_back(std::move(B));
      continue;
    }
    // a lone 2x2 gate streams faster through the CUDA-core sweep
    const bool lone2x2 = B.idx.size() == 1 && ops[B.idx[0]].type == OP_DENSE1;
    if (!lone2x2 && tx_prepare(n, ops, B, tp, false) == QF_OK) {
      B.shape = -2;
      out.push_back(std::move(B));
      continue;
    }
    std::vector<FxBlock> one(1, std::move(B));
    for (FxBlock& b : fx_split_shapes(one, ops)) out.push_back(std::move(b));
  }
  return out;
}

int fx_run_ops(const void* in, void* out, int n, std::vector<HostOp>& ops, int fusion_k, cudaStream_t stream,
               int* passes_out) {
  std::vector<FxBlock> blocks = fx_plan_final(ops, n, fusion_k);
  int passes = 0;
  const void* src = in;
  if (blocks.empty()) {
    if (in != out) {
      const size_t bytes = (size_t(1) << n) * 16;
      int rc = check_cuda(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, stream));
      if (rc) return rc;
      passes = 1;
    }
    if (passes_out) *passes_out = passes;
    return QF_OK;
  }
  static thread_local FxGroupParams gp;  // ~18 KiB: kept off the stack
  static thread_local FxShapeParams sp;
  static thread_local TxParams tp;
  for (FxBlock& B : blocks) {
    int rc;
    switch (fx_block_kernel(ops, B)) {
      case 6: {
        rc = tx_prepare(n, ops, B, tp);
        if (rc) return rc;
        tp.in = src;
        tp.out = out;
        tp.err = device_error_word();
        if (tp.err == nullptr) return QF_ERR_CUDA;
        LaunchTimer timer(QF_KERNEL_FX_TENSOR, stream);
        rc = tx_launch(tp, stream);
        break;
      }
      case 4: {
        rc = fx_shape_prepare(n, ops, B, sp);
        if (rc) return rc;
        sp.in = reinterpret_cast<const double2*>(src);
        sp.out = reinterpret_cast<double2*>(out);
        LaunchTimer timer(QF_KERNEL_FX_SHAPE, stream);
        rc = fx_shape_launch(sp, stream);
        break;
      }
      case 5: {
        std::vector<HostOp> one(1, ops[B.idx[0]]);
        int p = 0;
        rc = run_ops(src, out, n, C128, one, 1, stream, &p);
        break;
      }
      case 1: {
        LaunchTimer timer(ops[B.idx[0]].k == 1 ? QF_KERNEL_FX_DENSE1 : QF_KERNEL_FX_DENSE2, stream);
        rc = launch_fx_single(src, out, n, ops[B.idx[0]], stream);
        break;
      }
      default: {
        rc = fx_group_prepare(n, ops, B, gp);
        if (rc) return rc;
        gp.in = reinterpret_cast<const double2*>(src);
        gp.out = reinterpret_cast<double2*>(out);
        LaunchTimer timer(B.G == 0 ? QF_KERNEL_FX_ELEMENTWISE : QF_KERNEL_FX_GROUP, stream);
        rc = fx_group_launch(gp, B.G, stream);
        break;
      }
    }
    if (rc) return rc;
    ++passes;
    src = out;
  }
  if (passes_out) *passes_out = passes;
  return QF_OK;
}

int fx_plan_stats(int n, std::vector<HostOp>& ops, int fusion_k, int32_t* stats, int max_blocks, int* nblocks) {
  std::vector<FxBlock> blocks = fx_plan_final(ops, n, fusion_k);
  *nblocks = (int)blocks.size();
  for (int b = 0; b < (int)blocks.size() && b < max_blocks; ++b) {
    const FxBlock& B = blocks[b];
    int32_t* st = stats + 8 * b;
    std::memset(st, 0, 8 * sizeof(int32_t));
    st[0] = (int32_t)B.idx.size();
    for (int i : B.idx) {
      const HostOp& op = ops[i];
      const bool dense = op.type == OP_DENSE1 || op.type == OP_DENSE2 || op.type == OP_MONO;
      if (dense && op.k == 1) st[1]++;
      else if (dense && op.k == 2) {
        st[2]++;
        if (op.gb[0] < 5 || op.gb[1] < 5) st[3]++;
      } else if (op.type == OP_DIAG || op.type == OP_SIGN || op.type == OP_PHASE || op.type == OP_CUT) st[4]++;
      else st[5]++;
    }
    uint64_t hm = 0;
    for (int j = 0; j < B.G; ++j) hm |= uint64_t(1) << B.order[j];
    st[6] = __builtin_popcountll(hm & ~uint64_t(31));
    st[7] = fx_block_kernel(ops, B);
  }
  return QF_OK;
}

}  // namespace qf
