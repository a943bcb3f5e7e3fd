// Shared device-side building blocks for the GB300 state-vector engine.
//
// State layout.  A state of n qubits is 2^n amplitudes in C order: flat index
// x, with reference axis a stored at bit position (n-1-a) of x (axis 0 is the
// most significant bit, quantumflow/qubits.py:63-69).  Three element layouts:
//
//   QF_LAYOUT_C64   complex64   float2  {re, im}                 8 B
//   QF_LAYOUT_C128  complex128  double2 {re, im}                16 B
//   QF_LAYOUT_FF    float-float float4  {re_hi, re_lo, im_hi, im_lo}  16 B
//
// FF carries a complex128 value as two unevaluated float sums
// (value = hi + lo, |lo| <= ulp(hi)/2), a 48-bit significand.  GB300 issues
// FP64 FMAs at ~1/64 of the FP32 rate, so a dense 2x2 complex gate in native
// FP64 cannot keep up with HBM; the same gate in float-float arithmetic on
// the FP32 pipes can.  Error-free transforms below (two_sum, two_prod) follow
// Knuth (TAOCP vol. 2, 4.2.2) and Dekker (1971); the dot-product accumulation
// is the compensated scheme of Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26 (2005).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define QF_HD __host__ __device__ __forceinline__
#define QF_D __device__ __forceinline__

namespace qf {

enum Layout : int { C64 = 0, C128 = 1, FF = 2, FX = 3 };  // FX: C128 storage, fixed-point gates

// ---------------------------------------------------------------- types ----
template <int L> struct Types;
template <> struct Types<C64>  { using E = float2;  };
template <> struct Types<C128> { using E = double2; };
template <> struct Types<FF>   { using E = float4;  };

// A complex gate coefficient in the layout's arithmetic: for FF the four
// floats are (re_hi, re_lo, im_hi, im_lo); for C64 only .x/.z are used
// (re, im) and for C128 the double pair.  16 bytes in every case; the host
// fills it for the layout of the kernel it launches (engine.cuh make_coef).
struct Coef {
  union {
    double d[2];
    float f[4];
  };
};

// ---------------------------------------------------- error-free transforms
QF_D void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
QF_D void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// Compensated accumulator for sums of float-float products.
struct FFAcc {
  float s, e;
  QF_D void zero() { s = 0.f; e = 0.f; }
  // += (ah + al) * (bh + bl); the al*bl term (2^-48 relative) is dropped.
  QF_D void add_prod(float ah, float al, float bh, float bl) {
    float p = __fmul_rn(ah, bh);
    float pe = __fmaf_rn(ah, bh, -p);
    float t;
    two_sum(s, p, s, t);
    float cross = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, pe));
    e = __fadd_rn(e, __fadd_rn(t, cross));
  }
  QF_D void add(float h, float l) {
    float t;
    two_sum(s, h, s, t);
    e = __fadd_rn(e, __fadd_rn(t, l));
  }
  QF_D void finish(float& hi, float& lo) const { fast_two_sum(s, e, hi, lo); }
};

// ---------------------------------------------------- complex dot products
// out = sum_j u[j] * a[j] for J terms.  u comes from kernel parameters (warp
// uniform), so the zero tests below are uniform branches: real or imaginary
// coefficient parts that are exactly zero (RX, RZ, H, CNOT ...) cost nothing.
template <int J>
QF_D float2 cdot(const Coef* u, const float2* a) {
  float re = 0.f, im = 0.f;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const float ur = u[j].f[0], ui = u[j].f[2];
    re = fmaf(ur, a[j].x, re);
    re = fmaf(-ui, a[j].y, re);
    im = fmaf(ur, a[j].y, im);
    im = fmaf(ui, a[j].x, im);
  }
  return make_float2(re, im);
}

template <int J>
QF_D double2 cdot(const Coef* u, const double2* a) {
  double re = 0.0, im = 0.0;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const double ur = u[j].d[0], ui = u[j].d[1];
    if (ur != 0.0) {
      re = fma(ur, a[j].x, re);
      im = fma(ur, a[j].y, im);
    }
    if (ui != 0.0) {
      re = fma(-ui, a[j].y, re);
      im = fma(ui, a[j].x, im);
    }
  }
  return make_double2(re, im);
}

// Error-free product terms: p = ah*bh rounded, c = its rounding error plus
// the ah*bl and al*bh cross terms (the al*bl term, 2^-48 relative, is
// dropped).
QF_D void ff_term(float ah, float al, float bh, float bl, float& p, float& c) {
  p = __fmul_rn(ah, bh);
  c = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, __fmaf_rn(ah, bh, -p)));
}
// Float-float sum of four product terms, summed as a TwoSum tree (depth 2)
// with all rounding errors gathered into the low word.
QF_D void ff_sum4(const float (&p)[4], const float (&c)[4], float& hi, float& lo) {
  float s01, t01, s23, t23, s, t;
  two_sum(p[0], p[1], s01, t01);
  two_sum(p[2], p[3], s23, t23);
  two_sum(s01, s23, s, t);
  const float e = __fadd_rn(__fadd_rn(__fadd_rn(c[0], c[1]), __fadd_rn(c[2], c[3])),
                            __fadd_rn(__fadd_rn(t01, t23), t));
  fast_two_sum(s, e, hi, lo);
}
// (u0 a0 + u1 a1) for float-float complex values, all parts dense.
QF_D float4 ff_cmac2(float4 u0, float4 a0, float4 u1, float4 a1) {
  float p[4], c[4];
  float4 r;
  ff_term(u0.x, u0.y, a0.x, a0.y, p[0], c[0]);
  ff_term(-u0.z, -u0.w, a0.z, a0.w, p[1], c[1]);
  ff_term(u1.x, u1.y, a1.x, a1.y, p[2], c[2]);
  ff_term(-u1.z, -u1.w, a1.z, a1.w, p[3], c[3]);
  ff_sum4(p, c, r.x, r.y);
  ff_term(u0.x, u0.y, a0.z, a0.w, p[0], c[0]);
  ff_term(u0.z, u0.w, a0.x, a0.y, p[1], c[1]);
  ff_term(u1.x, u1.y, a1.z, a1.w, p[2], c[2]);
  ff_term(u1.z, u1.w, a1.x, a1.y, p[3], c[3]);
  ff_sum4(p, c, r.z, r.w);
  return r;
}

// float-float a*x + b*y: both products exact to 2^-48, one TwoSum, one
// renormalisation
QF_D void ff_dot2(float ah, float al, float xh, float xl, float bh, float bl, float yh, float yl, float& rh,
                  float& rl) {
  float p0, c0, p1, c1, s, t;
  ff_term(ah, al, xh, xl, p0, c0);
  ff_term(bh, bl, yh, yl, p1, c1);
  two_sum(p0, p1, s, t);
  fast_two_sum(s, __fadd_rn(__fadd_rn(c0, c1), t), rh, rl);
}

// Float-float sum of eight product terms: a TwoSum tree (depth 3) on the
// rounded products, all rounding errors and cross terms gathered in the low
// word, one renormalisation.
QF_D void ff_sum8(const float (&p)[8], const float (&c)[8], float& hi, float& lo) {
  float s[4], t[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) two_sum(p[2 * i], p[2 * i + 1], s[i], t[i]);
  float s01, t01, s23, t23, ss, tt;
  two_sum(s[0], s[1], s01, t01);
  two_sum(s[2], s[3], s23, t23);
  two_sum(s01, s23, ss, tt);
  float e = __fadd_rn(__fadd_rn(__fadd_rn(c[0], c[1]), __fadd_rn(c[2], c[3])),
                      __fadd_rn(__fadd_rn(c[4], c[5]), __fadd_rn(c[6], c[7])));
  e = __fadd_rn(e, __fadd_rn(__fadd_rn(__fadd_rn(t[0], t[1]), __fadd_rn(t[2], t[3])),
                             __fadd_rn(__fadd_rn(t01, t23), tt)));
  fast_two_sum(ss, e, hi, lo);
}
// sum_j u[j] a[j] over four terms with every coefficient part nonzero
QF_D float4 ff_cdot4_dense(const Coef* u, const float4* a) {
  float p[8], c[8];
  float4 r;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    ff_term(u[j].f[0], u[j].f[1], a[j].x, a[j].y, p[2 * j], c[2 * j]);
    ff_term(-u[j].f[2], -u[j].f[3], a[j].z, a[j].w, p[2 * j + 1], c[2 * j + 1]);
  }
  ff_sum8(p, c, r.x, r.y);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    ff_term(u[j].f[0], u[j].f[1], a[j].z, a[j].w, p[2 * j], c[2 * j]);
    ff_term(u[j].f[2], u[j].f[3], a[j].x, a[j].y, p[2 * j + 1], c[2 * j + 1]);
  }
  ff_sum8(p, c, r.z, r.w);
  return r;
}

template <int J>
QF_D float4 cdot(const Coef* u, const float4* a) {
  if constexpr (J == 2) {
    // dense 2x2 rows (Haar-random gates): the tree form; rows with zero
    // parts (RX, RY, H ...) take the skipping loop below
    if (u[0].f[0] != 0.f && u[0].f[2] != 0.f && u[1].f[0] != 0.f && u[1].f[2] != 0.f) {
      const float4 u0 = make_float4(u[0].f[0], u[0].f[1], u[0].f[2], u[0].f[3]);
      const float4 u1 = make_float4(u[1].f[0], u[1].f[1], u[1].f[2], u[1].f[3]);
      return ff_cmac2(u0, a[0], u1, a[1]);
    }
  }
  FFAcc re, im;
  re.zero();
  im.zero();
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const float urh = u[j].f[0], url = u[j].f[1], uih = u[j].f[2], uil = u[j].f[3];
    if (urh != 0.f) {
      re.add_prod(urh, url, a[j].x, a[j].y);
      im.add_prod(urh, url, a[j].z, a[j].w);
    }
    if (uih != 0.f) {
      re.add_prod(-uih, -uil, a[j].z, a[j].w);
      im.add_prod(uih, uil, a[j].x, a[j].y);
    }
  }
  float4 r;
  re.finish(r.x, r.y);
  im.finish(r.z, r.w);
  return r;
}

// Per-thread (non-uniform) coefficient variants, no zero skipping.
QF_D float2 cmul_add2(float2 u0, float2 a0, float2 u1, float2 a1) {
  float re = u0.x * a0.x;
  re = fmaf(-u0.y, a0.y, re);
  re = fmaf(u1.x, a1.x, re);
  re = fmaf(-u1.y, a1.y, re);
  float im = u0.x * a0.y;
  im = fmaf(u0.y, a0.x, im);
  im = fmaf(u1.x, a1.y, im);
  im = fmaf(u1.y, a1.x, im);
  return make_float2(re, im);
}
QF_D double2 cmul_add2(double2 u0, double2 a0, double2 u1, double2 a1) {
  double re = u0.x * a0.x;
  re = fma(-u0.y, a0.y, re);
  re = fma(u1.x, a1.x, re);
  re = fma(-u1.y, a1.y, re);
  double im = u0.x * a0.y;
  im = fma(u0.y, a0.x, im);
  im = fma(u1.x, a1.y, im);
  im = fma(u1.y, a1.x, im);
  return make_double2(re, im);
}
QF_D float4 cmul_add2(float4 u0, float4 a0, float4 u1, float4 a1) { return ff_cmac2(u0, a0, u1, a1); }

// single complex multiply by a uniform coefficient
QF_D float2 cmul(const Coef& u, float2 a) { return cdot<1>(&u, &a); }
QF_D double2 cmul(const Coef& u, double2 a) { return cdot<1>(&u, &a); }
QF_D float4 cmul(const Coef& u, float4 a) { return cdot<1>(&u, &a); }

QF_D float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }
QF_D double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
QF_D float4 cneg(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }

// |a|^2 accumulated into a float-float accumulator (all layouts).
QF_D void acc_norm2(FFAcc& acc, float2 a) {
  acc.add_prod(a.x, 0.f, a.x, 0.f);
  acc.add_prod(a.y, 0.f, a.y, 0.f);
}
QF_D void acc_norm2(FFAcc& acc, float4 a) {
  acc.add_prod(a.x, a.y, a.x, a.y);
  acc.add_prod(a.z, a.w, a.z, a.w);
}
// double amplitudes: split each component into float-float first
QF_D void split_d(double d, float& h, float& l) {
  h = __double2float_rn(d);
  l = __double2float_rn(d - (double)h);
}
QF_D void acc_norm2(FFAcc& acc, double2 a) {
  float rh, rl, ih, il;
  split_d(a.x, rh, rl);
  split_d(a.y, ih, il);
  acc.add_prod(rh, rl, rh, rl);
  acc.add_prod(ih, il, ih, il);
}
QF_D float4 to_ff(double2 a) {
  float4 r;
  split_d(a.x, r.x, r.y);
  split_d(a.y, r.z, r.w);
  return r;
}
QF_D float4 to_ff(float2 a) { return make_float4(a.x, 0.f, a.y, 0.f); }
QF_D float4 to_ff(float4 a) { return a; }

// ------------------------------------------------------------- indexing ----
// Insert a zero bit at position b of v.
QF_HD int64_t insert0(int64_t v, int b) {
  const int64_t lo = v & ((int64_t(1) << b) - 1);
  return ((v >> b) << (b + 1)) | lo;
}
// 32-bit form for states of at most 2^31 amplitudes (b <= 30)
QF_HD uint32_t insert0(uint32_t v, int b) {
  const uint32_t lo = v & ((1u << b) - 1u);
  return ((v >> b) << (b + 1)) | lo;
}


// ------------------------------------ per-amplitude helpers (all layouts) --
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
  float4 r;
  ff_dot2(c.f[0], c.f[1], a.x, a.y, -c.f[2], -c.f[3], a.z, a.w, r.x, r.y);
  ff_dot2(c.f[0], c.f[1], a.z, a.w, c.f[2], c.f[3], a.x, a.y, r.z, r.w);
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


// c a + i s p for real c, s (RX(-beta) row applied to self a and partner p)
QF_D float4 rx_one(const Coef& c, const Coef& s, float4 a, float4 p) {
  float4 o;
  ff_dot2(c.f[0], c.f[1], a.x, a.y, -s.f[0], -s.f[1], p.z, p.w, o.x, o.y);
  ff_dot2(c.f[0], c.f[1], a.z, a.w, s.f[0], s.f[1], p.x, p.y, o.z, o.w);
  return o;
}
QF_D double2 rx_one(const Coef& c, const Coef& s, double2 a, double2 p) {
  return make_double2(fma(c.d[0], a.x, -s.d[0] * p.y), fma(c.d[0], a.y, s.d[0] * p.x));
}
QF_D float2 rx_one(const Coef& c, const Coef& s, float2 a, float2 p) {
  return make_float2(fmaf(c.f[0], a.x, -s.f[0] * p.y), fmaf(c.f[0], a.y, s.f[0] * p.x));
}
// acc += Im(conj(l) p)
QF_D void redx_acc(FFAcc& acc, float4 l, float4 p) {
  acc.add_prod(l.x, l.y, p.z, p.w);
  acc.add_prod(-l.z, -l.w, p.x, p.y);
}
QF_D void redx_acc(FFAcc& acc, double2 l, double2 p) { acc_imconj(acc, l, p, 1.f); }
QF_D void redx_acc(FFAcc& acc, float2 l, float2 p) {
  acc.add_prod(l.x, 0.f, p.y, 0.f);
  acc.add_prod(-l.y, 0.f, p.x, 0.f);
}


// ---------------------------------------- mbarrier + bulk async copies -----
QF_D uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
QF_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
QF_D void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
QF_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
QF_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared bulk copy completing on an mbarrier (16-byte aligned,
// size a multiple of 16)
QF_D void bulk_g2s(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(sdst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// shared -> global bulk copy tracked in the issuing thread's bulk group
QF_D void bulk_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(smem_u32(ssrc)), "r"(bytes)
               : "memory");
}
QF_D void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
QF_D void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
QF_D void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
QF_D void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
QF_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Per-thread asynchronous global -> shared copies of one amplitude (8 or 16
// bytes), tracked in the issuing thread's cp.async groups.  A thread that
// reads back only what it copied itself needs no barrier, only wait_group.
QF_D void cp_async_amp(float4* s, const float4* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(s)), "l"(g) : "memory");
}
QF_D void cp_async_amp(double2* s, const double2* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(s)), "l"(g) : "memory");
}
QF_D void cp_async_amp(float2* s, const float2* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(s)), "l"(g) : "memory");
}
QF_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
QF_D void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }


// ---------------------------------------------------- warp reductions ----
QF_D double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace qf
