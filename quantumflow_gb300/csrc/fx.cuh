// Integer fixed-point arithmetic for complex128 states (QF_LAYOUT_FX).
//
// Storage is the complex128 layout itself (interleaved FP64 re, im); only the
// arithmetic differs.  GB300 issues FP64 FMAs at about 2 per clock per SM
// but 32x32->64-bit integer multiply-adds (IMAD.WIDE) at 64, so a gate is
// applied in 64-bit integer arithmetic:
//
//  * load: the 2^G amplitudes a thread holds share one exponent E (the
//    largest FP64 exponent among their real and imaginary parts); every part
//    becomes a fixed-point integer A = v * 2^(1022 + M - E) (truncated), so
//    the largest part has M significant bits (M = 56 or 57) and the rest
//    keep theirs down to the same absolute quantum;
//  * gates: a coefficient c (|c| <= 1, unitary gates only) is the integer
//    C = round(c * 2^58).  Both are held as two int32 pieces,
//    A = Ah * 2^28 + Al and C = Ch * 2^28 + Cl, and a real dot product is
//        sum_k A_k C_k = 2^56 sum Ah Ch + 2^28 sum (Ah Cl + Al Ch) + sum Al Cl
//    accumulated exactly in two int64 registers (three IMAD.WIDE per real
//    product); the last term (< 2^56 per product, a quarter of the result's
//    quantum) is dropped and the result is rounded to the quantum of A.  A
//    complex row sum_j u_j a_j takes three real dot products (Gauss's
//    three-multiplication complex product): P1 = sum ur ar, P2 = sum ui ai,
//    P3 = sum (ur + ui)(ar + ai); re = P1 - P2, im = P3 - P1 - P2;
//  * store: each part is rounded once to the nearest FP64 value.
//
// Unitary gates preserve the 2-norm of a thread's amplitude group, so no
// part exceeds 2^(M + 0.5 + G/2) and no sum ar + ai exceeds 2^(M + 1 + G/2)
// <= 2^58.5 (M = 56 for G <= 2, 55 for G <= 4): the pieces fit int32 and the
// accumulators int64.  The error of one pass is below a quarter of the
// quantum per product plus the final FP64 rounding: at least 55 significant
// bits relative to the group's largest part, against the 53 of FP64
// arithmetic.  Gates that are not unitary run in native FP64 (the host
// planner routes them).  Parts must stay below 2^1000 in magnitude.
#pragma once
#include <cstdint>
#include <cmath>

#include "qf_common.cuh"

namespace qf {

constexpr int FX_F = 58;  // coefficient fraction bits
constexpr int FX_L = 28;  // piece split position
constexpr uint32_t FX_LMASK = (1u << FX_L) - 1u;

// One complex coefficient: re, im and re + im, each as (hi, lo) pieces with
// C = hi * 2^28 + lo, 0 <= lo < 2^28.
struct FxC {
  int32_t rh, rl, ih, il, sh, sl;
};

// Host: pieces of C = round(v * 2^58), |v| <= 1.5.
inline void fx_pieces(long long c, int32_t& h, int32_t& l) {
  h = static_cast<int32_t>(c >> FX_L);  // arithmetic shift: floor
  l = static_cast<int32_t>(c & static_cast<long long>(FX_LMASK));
}
inline FxC make_fxc(double re, double im) {
  FxC c;
  const long long cr = std::llround(std::ldexp(re, FX_F)), ci = std::llround(std::ldexp(im, FX_F));
  fx_pieces(cr, c.rh, c.rl);
  fx_pieces(ci, c.ih, c.il);
  fx_pieces(cr + ci, c.sh, c.sl);  // exactly the sum of the rounded parts
  return c;
}

// ------------------------------------------------------- bit primitives ----
// low 32 bits of (hi:lo) >> min(n, 32)
QF_HD uint32_t fx_shr64lo(uint32_t lo, uint32_t hi, uint32_t n) {
#ifdef __CUDA_ARCH__
  return __funnelshift_rc(lo, hi, n);
#else
  n = n > 32 ? 32 : n;
  return static_cast<uint32_t>(((static_cast<uint64_t>(hi) << 32) | lo) >> n);
#endif
}
// high 32 bits of (hi:lo) << min(n, 32)
QF_HD uint32_t fx_shl64hi(uint32_t lo, uint32_t hi, uint32_t n) {
#ifdef __CUDA_ARCH__
  return __funnelshift_lc(lo, hi, n);
#else
  n = n > 32 ? 32 : n;
  return static_cast<uint32_t>((((static_cast<uint64_t>(hi) << 32) | lo) << n) >> 32);
#endif
}
// x >> n, 0 when n >= 32
QF_HD uint32_t fx_shr(uint32_t x, uint32_t n) { return fx_shr64lo(x, 0u, n); }
QF_HD int fx_clz(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz(x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}
// d = a * b + c, 32x32 -> 64 bits signed (one IMAD.WIDE)
QF_HD int64_t fx_mad(int32_t a, int32_t b, int64_t c) {
#ifdef __CUDA_ARCH__
  int64_t d;
  asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
  return d;
#else
  return static_cast<int64_t>(a) * b + c;
#endif
}
// d = a * b + c, 32x32 -> 64 bits unsigned (one IMAD.WIDE.U32)
QF_HD uint64_t fx_madu(uint32_t a, uint32_t b, uint64_t c) {
#ifdef __CUDA_ARCH__
  uint64_t d;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
  return d;
#else
  return static_cast<uint64_t>(a) * b + c;
#endif
}
QF_HD uint32_t fx_hiword(double v) {
#ifdef __CUDA_ARCH__
  return static_cast<uint32_t>(__double2hiint(v));
#else
  uint64_t b;
  __builtin_memcpy(&b, &v, 8);
  return static_cast<uint32_t>(b >> 32);
#endif
}
QF_HD uint32_t fx_loword(double v) {
#ifdef __CUDA_ARCH__
  return static_cast<uint32_t>(__double2loint(v));
#else
  uint64_t b;
  __builtin_memcpy(&b, &v, 8);
  return static_cast<uint32_t>(b);
#endif
}
QF_HD double fx_double(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
#else
  const uint64_t b = (static_cast<uint64_t>(hi) << 32) | lo;
  double v;
  __builtin_memcpy(&v, &b, 8);
  return v;
#endif
}

// ------------------------------------------------------------ conversion ----
// FP64 exponent field of a part (0 for zeros and subnormals).
QF_HD int fx_exp(double v) { return static_cast<int>((fx_hiword(v) >> 20) & 0x7ffu); }

// Group exponents below this are treated as all-zero groups (parts below
// 2^-959): it keeps every stored exponent in the normal range.
constexpr int FX_EMIN = 64;

// The part v as A = ah * 2^28 + al relative to the group exponent E >= e(v):
// A = v * 2^(1022 + M - E), truncated toward zero; |al| < 2^28.
// E comes from fx_group_exp, which raises groups below FX_EMIN out of range
// (every part of such a group becomes 0).
template <int M>
QF_HD void fx_in(double v, int E, int32_t& ah, int32_t& al) {
  const uint32_t hi = fx_hiword(v), lo = fx_loword(v);
  const int e = static_cast<int>((hi >> 20) & 0x7ffu);
  // right shift of the 64-bit mantissa with its hidden bit at bit 63
  // (zeros and subnormals carry no hidden bit and become 0)
  const uint32_t r = static_cast<uint32_t>(E - e) + static_cast<uint32_t>(64 - M);
  const uint32_t mh = fx_shl64hi(lo, hi, 11) | (e != 0 ? 0x80000000u : 0u);
  const uint32_t ml = lo << 11;
  const uint32_t h = fx_shr(mh, r - 4u);        // A >> 28 (r >= 64 - M >= 7)
  const uint32_t x = fx_shr64lo(ml, mh, r);     // low word of A for r < 32
  const uint32_t y = fx_shr(mh, r - 32u);       // low word of A for 32 <= r (0 for r < 32 or r >= 64)
  const uint32_t l = (r < 32u ? x : y) & FX_LMASK;
  const int32_t s = static_cast<int32_t>(hi) >> 31;
  ah = (static_cast<int32_t>(h) ^ s) - s;
  al = (static_cast<int32_t>(l) ^ s) - s;
}

// FP64 value of T * 2^(E - 1024 - M) (T = 4 A after a gate), rounded to
// nearest even.
template <int M>
QF_HD double fx_out(int64_t T, int E) {
  const uint32_t thi = static_cast<uint32_t>(static_cast<uint64_t>(T) >> 32);
  const uint32_t tlo = static_cast<uint32_t>(T);
  const uint32_t s = static_cast<uint32_t>(static_cast<int32_t>(thi) >> 31);
  // |T| as (mh:ml)
  const uint64_t mag = ((static_cast<uint64_t>(thi ^ s) << 32) | (tlo ^ s)) - static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(s)));
  const uint32_t mh = static_cast<uint32_t>(mag >> 32), ml = static_cast<uint32_t>(mag);
  // normalise without branches (a branch here would cut the unrolled
  // conversions of a thread's amplitudes into blocks the scheduler cannot
  // interleave): lz = leading zeros of the 64-bit |T| (64 when T = 0)
  const bool big = mh != 0u;
  const int zh = fx_clz(mh), zl = fx_clz(ml);
  const int lz = big ? zh : 32 + zl;
  const uint32_t nh = big ? fx_shl64hi(ml, mh, static_cast<uint32_t>(zh)) : fx_shl64hi(0u, ml, static_cast<uint32_t>(zl));
  const uint32_t nl = big ? (ml << (zh & 31)) : 0u;
  // n = |T| << lz has its leading one at bit 63
  uint32_t qh = nh >> 11;
  uint32_t ql = fx_shr64lo(nl, nh, 11);
  const uint32_t rest = nl & 0x7ffu;  // dropped bits; 0x400 is the half
  const uint32_t inc = (rest > 0x400u || (rest == 0x400u && (ql & 1u))) ? 1u : 0u;
  const uint64_t q = ((static_cast<uint64_t>(qh) << 32) | ql) + inc;
  qh = static_cast<uint32_t>(q >> 32);
  ql = static_cast<uint32_t>(q);
  const int eb = E + 62 - M - lz;  // biased exponent; the hidden bit of q adds one
  const uint32_t bits_hi = (qh + (static_cast<uint32_t>(eb - 1) << 20)) | (s & 0x80000000u);
  const bool zero = (mh | ml) == 0u;
  return fx_double(zero ? 0u : bits_hi, zero ? 0u : ql);
}

// The same conversion with a branch on the normalisation: fewer
// instructions, for kernels that convert only a few values per thread (the
// single-gate sweeps), where the branch costs no scheduling freedom.
template <int M>
QF_HD double fx_out_br(int64_t T, int E) {
  const uint32_t thi = static_cast<uint32_t>(static_cast<uint64_t>(T) >> 32);
  const uint32_t tlo = static_cast<uint32_t>(T);
  const uint32_t s = static_cast<uint32_t>(static_cast<int32_t>(thi) >> 31);
  const uint64_t mag = ((static_cast<uint64_t>(thi ^ s) << 32) | (tlo ^ s)) - static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(s)));
  const uint32_t mh = static_cast<uint32_t>(mag >> 32), ml = static_cast<uint32_t>(mag);
  int lz;
  uint32_t nh, nl;
  if (mh != 0u) {
    lz = fx_clz(mh);
    nh = fx_shl64hi(ml, mh, static_cast<uint32_t>(lz));
    nl = ml << lz;
  } else {
    if (ml == 0u) return 0.0;
    const int z = fx_clz(ml);
    lz = 32 + z;
    nh = ml << z;
    nl = 0u;
  }
  uint32_t qh = nh >> 11;
  uint32_t ql = fx_shr64lo(nl, nh, 11);
  const uint32_t rest = nl & 0x7ffu;
  const uint32_t inc = (rest > 0x400u || (rest == 0x400u && (ql & 1u))) ? 1u : 0u;
  const uint64_t q = ((static_cast<uint64_t>(qh) << 32) | ql) + inc;
  qh = static_cast<uint32_t>(q >> 32);
  ql = static_cast<uint32_t>(q);
  const int eb = E + 62 - M - lz;
  const uint32_t bits_hi = (qh + (static_cast<uint32_t>(eb - 1) << 20)) | (s & 0x80000000u);
  return fx_double(bits_hi, ql);
}

// ------------------------------------------------------------- products ----
// Row accumulator: H = sum Ah Ch, X = sum (Ah Cl + Al Ch).
struct FxAcc {
  int64_t H, X;
  QF_HD void zero() {
    H = 0;
    X = 0;
  }
  QF_HD void add(int32_t ah, int32_t al, int32_t ch, int32_t cl) {
    H = fx_mad(ah, ch, H);
    X = fx_mad(ah, cl, X);
    X = fx_mad(al, ch, X);
  }
  // T = (sum A C) / 2^56 = H + floor(X / 2^28), i.e. four times the result
  // in units of A.  With X = xh 2^32 + xl (xl unsigned), floor(X / 2^28) =
  // 16 xh + (xl >> 28): two multiply-adds on the IMAD pipe instead of a
  // 64-bit shift and add on the integer ALU, the busier pipe of these passes.
  QF_HD int64_t total() const {
    const int32_t xh = static_cast<int32_t>(static_cast<uint64_t>(X) >> 32);
    const uint32_t xl = static_cast<uint32_t>(X);
    const int64_t t = fx_mad(xh, 16, H);
    return static_cast<int64_t>(fx_madu(xl >> FX_L, 1u, static_cast<uint64_t>(t)));
  }
};

// Split a result T (units of A / 4) into the pieces of A = round(T / 4).
QF_HD void fx_resplit(int64_t T, int32_t& ah, int32_t& al) {
  const int64_t t = T + 2;
  const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(t) >> 32), lo = static_cast<uint32_t>(t);
  ah = static_cast<int32_t>(fx_shr64lo(lo, hi, 30));
  al = static_cast<int32_t>((lo >> 2) & FX_LMASK);
}

// A complex amplitude in fixed point: real and imaginary pieces.
struct FxAmp {
  int32_t rh, rl, ih, il;
};

// out = sum_j u[j] a[j] (J terms) as T values (units of A / 4): three real
// dot products (P1 = sum ur ar, P2 = sum ui ai, P3 = sum (ur+ui)(ar+ai)).
template <int J>
QF_HD void fx_cdot(const FxC* u, const FxAmp* a, int64_t& tre, int64_t& tim) {
  FxAcc p1, p2, p3;
  p1.zero();
  p2.zero();
  p3.zero();
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const FxC c = u[j];
    p1.add(a[j].rh, a[j].rl, c.rh, c.rl);
    p2.add(a[j].ih, a[j].il, c.ih, c.il);
    p3.add(a[j].rh + a[j].ih, a[j].rl + a[j].il, c.sh, c.sl);
  }
  const int64_t t1 = p1.total(), t2 = p2.total(), t3 = p3.total();
  tre = t1 - t2;
  tim = t3 - t1 - t2;
}

QF_HD FxAmp fx_amp_from_t(int64_t tre, int64_t tim) {
  FxAmp r;
  fx_resplit(tre, r.rh, r.rl);
  fx_resplit(tim, r.ih, r.il);
  return r;
}
QF_HD FxAmp fx_neg(FxAmp a) { return FxAmp{-a.rh, -a.rl, -a.ih, -a.il}; }

// A part loaded as A (not yet through a gate) back to FP64: T = 4 A.
QF_HD int64_t fx_t_of(int32_t ah, int32_t al) {
  return (static_cast<int64_t>(ah) << (FX_L + 2)) + (static_cast<int64_t>(al) << 2);
}

}  // namespace qf
