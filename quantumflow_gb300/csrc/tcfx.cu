// Complex128 gate passes on the 5th-generation tensor cores at FP64-class
// precision: integer digits of a fixed-point form, multiplied by fp16 MMAs
// (tcgen05.mma kind::f16) whose FP32 accumulators stay exact.
//
// Reference semantics: quantumflow/backend/numpybk.py:159-214 tensormul
// applied gate by gate (quantumflow/circuits.py:87-99).  A pass applies a
// run of unitary gates whose dense qubits lie in a window of four bits,
// with CZ-like sign ops around them (or one unitary gate on 3 or 4
// qubits): the host multiplies them into one 16x16 unitary U (double-double)
// and the pass computes y = U x for every "row" x, the 16 amplitudes that
// differ only in the window bits.
//
// Arithmetic (an integer form of the Ozaki splitting scheme: Ozaki, Ogita,
// Oishi and Rump, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication", Numer. Algorithms 59, 2012):
//
//  * a row's 32 real parts share one exponent E (the largest FP64 exponent
//    field among them); each part becomes A = v * 2^(1022 + 61 - E)
//    truncated toward zero, |A| < 2^61, with integer bit operations (the
//    FP64 pipe is the narrowest unit on this part);
//  * U's real form (32 x 32) is G = round(g * 2^62), |G| <= 2^62;
//  * both are written in base 256 with balanced digits: X + 0x8080..80 =
//    sum_t (d_t + 128) 256^(7-t), d_t in [-128, 127] (the amplitudes'
//    top byte is biased by 0x40 instead, which keeps it below 0x80), so a
//    byte of the biased integer is a digit (one byte permute per digit
//    pair) and every digit is exact in fp16;
//  * A.G = sum_delta acc_delta 256^(14 - delta), acc_delta = sum over the
//    digit pairs t + u = delta of the digit GEMMs; delta = 0..7 are kept
//    (36 of the 64 digit products).  With K = 32 terms per output every
//    acc_delta is an integer below 2^22 (the top digits are small:
//    |d_0(A)| <= 33, |d_0(G)| <= 65; the largest, acc_7, is at most
//    32 (33 128 + 6 128^2 + 128 65) < 2^21.8), so the FP32 accumulation is
//    exact and so is a float-to-integer conversion by the 1.5 * 2^23
//    addition trick;
//  * Z = A.G / 2^63 = sum acc_delta 2^(49 - 8 delta) (two's complement
//    int64; |Z| <= 2^62.5 because U is unitary), converted to FP64 once,
//    exactly rounded, and scaled by 2^(E - 1082).
//
// Error per output, relative to the row's largest part: the truncation of
// the inputs (each below 2^-59 of it; through a unit row of U at most
// sqrt(32) 2^-59 = 2^-56.5), the dropped digit products (delta >= 8: a few
// 2^-63 typically) and one FP64 rounding of the output -- below the error of
// FP64 arithmetic on the same row.  The CPU model of this arithmetic
// (tests/txarith.py) measures it against exact rational arithmetic.
//
// Kernel: one CTA of 640 threads per SM, persistent over tiles of 128 rows
// (the MMA's M); three stages of the A operand, two of the accumulators.
// Warps 0-7 convert: two threads per row (lanes l and l ^ 8, eight
// amplitudes each; the row exponent is a shuffle away) turn their
// amplitudes into digits and store them as the A operand, K-major rows of
// 8 digits x 32 reals in four 128-byte swizzled chunks.  The gate's digits
// (B: 8 digit blocks x 32 output reals, K = 32 input reals) are built once
// per CTA.  Once every converter has arrived on the stage's mbarrier, the
// first thread of warps 16-19 issues, per amplitude digit t, two MMAs
// (K = 16 each) against the first 32 (8 - t) rows of B into tensor-memory
// columns [32 t, 256) of the accumulator stage: column block delta
// receives every digit product of its weight.  Warps 8-15 run the
// epilogue: the thread of TMEM lane r (two per row, 16 output reals each)
// reads the eight accumulators of each output, combines them into Z and
// stores FP64.  Conversion, MMAs and epilogue of consecutive tiles overlap.
// Every wait is bounded (4 s): on expiry the kernel raises the device error
// word and every thread leaves its loop.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <cuda_fp16.h>

#include "engine.cuh"
#include "fx.cuh"

namespace qf {

int* device_error_word();
int g_fx_tensor = 1;  // qf_set_fx_tensor_cores

namespace {

constexpr int TX_ROWS = 128;     // rows per tile (MMA M)
constexpr int TX_KD = 32;        // real width of a row (GEMM K) and of U (GEMM N per digit)
constexpr int TX_ND = 8;         // base-256 digits per integer
constexpr int TX_MB = 61;        // amplitude integers: |A| < 2^61
constexpr uint64_t TX_BIAS = 0x8080808080808080ull;
// the amplitudes' bias: the top byte of A + bias stays below 0x80 (|A| <
// 2^61 moves it by at most 32), so a sign-replicating byte permute of it
// gives a zero byte; the digits are the same as with TX_BIAS
constexpr uint64_t TX_BIAS_A = 0x4080808080808080ull;
constexpr uint32_t TX_A_CHUNK = TX_ROWS * 128;         // 64 fp16 of K per row, 128-byte rows
constexpr uint32_t TX_A_BYTES = 4 * TX_A_CHUNK;        // 8 digits x 32 reals = 256 K per row
constexpr uint32_t TX_B_BYTES = TX_ND * TX_KD * 128;   // 256 N-rows, 32 K used of each 128-byte row
constexpr float TX_MAGIC = 12582912.0f;  // 1.5 * 2^23
constexpr int32_t TX_MAGIC_BITS = 0x4B400000;

QF_D uint32_t tx_smem(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// canonical K-major, 128-byte swizzled shared-memory matrix descriptor
QF_D uint64_t tx_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);  // start address
  d |= static_cast<uint64_t>(1) << 16;                   // leading byte offset (unused when swizzled)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;           // stride byte offset: 8 rows x 128 B
  d |= static_cast<uint64_t>(1) << 46;                   // descriptor version
  d |= static_cast<uint64_t>(2) << 61;                   // 128-byte swizzle
  return d;
}
// instruction descriptor: D f32, A and B f16, both K-major, M = 128
QF_D uint32_t tx_idesc(int N) {
  return (1u << 4) | (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(TX_ROWS >> 4) << 24);
}
// byte offset of the 16-byte piece p (0..7) of row r in a 128-byte swizzled chunk
QF_D uint32_t tx_piece(int r, int p) { return static_cast<uint32_t>(r * 128 + ((p ^ (r & 7)) << 4)); }

QF_D void tx_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
QF_D void tx_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tx_smem(bar))
               : "memory");
}
QF_D void tx_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
QF_D void tx_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
QF_D void tx_alloc(uint32_t* slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tx_smem(slot)), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
QF_D void tx_bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tx_smem(bar)), "r"(count) : "memory");
}
QF_D void tx_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tx_smem(bar)) : "memory");
}

// waits for the phase to complete, suspended up to about 100 us per try
QF_D bool tx_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(tx_smem(bar)), "r"(parity), "r"(100000u)
      : "memory");
  return ok != 0;
}
QF_D uint64_t tx_now() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// bounded wait (4 s of wall clock); false (and the error word raised) on expiry
QF_D bool tx_wait(uint64_t* bar, uint32_t parity, int* err) {
  if (tx_try_wait(bar, parity)) return true;
  const uint64_t t0 = tx_now();
  while (!tx_try_wait(bar, parity)) {
    if (tx_now() - t0 > 4000000000ull) {
      atomicOr(err, 1);
      return false;
    }
  }
  return true;
}

// 4 consecutive fp32 accumulator columns of this warp's 32 TMEM lanes
// (the caller waits with tx_wait_ld before reading)
QF_D void tx_ld4(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
// wait for this thread's tensor-memory loads; the registers pass through the
// asm so that no use of them is scheduled before the wait
QF_D void tx_wait_ld(uint32_t (&a)[8][4]) {
  asm volatile(
      "tcgen05.wait::ld.sync.aligned;"
      : "+r"(a[0][0]), "+r"(a[0][1]), "+r"(a[0][2]), "+r"(a[0][3]), "+r"(a[1][0]), "+r"(a[1][1]), "+r"(a[1][2]),
        "+r"(a[1][3]), "+r"(a[2][0]), "+r"(a[2][1]), "+r"(a[2][2]), "+r"(a[2][3]), "+r"(a[3][0]), "+r"(a[3][1]),
        "+r"(a[3][2]), "+r"(a[3][3]), "+r"(a[4][0]), "+r"(a[4][1]), "+r"(a[4][2]), "+r"(a[4][3]), "+r"(a[5][0]),
        "+r"(a[5][1]), "+r"(a[5][2]), "+r"(a[5][3]), "+r"(a[6][0]), "+r"(a[6][1]), "+r"(a[6][2]), "+r"(a[6][3]),
        "+r"(a[7][0]), "+r"(a[7][1]), "+r"(a[7][2]), "+r"(a[7][3])
      :
      : "memory");
}

// Biased fixed-point integer of one part: A + TX_BIAS_A, A = v * 2^(1022 +
// 61 - E) truncated toward zero (Ep = E + 3 >= the part's exponent field +
// 3).  The 64-bit mantissa with its hidden bit at bit 63 is shifted right by
// n = Ep - e in one 64-bit shift, whose amount clamps at 64 (zeros and
// subnormals, n >= 67, shift out completely).  The sign and the bias are
// one add: (t ^ neg) - neg + BIAS = (t ^ neg) + BIAS + (neg & 1).
QF_D uint64_t tx_biased(double v, uint32_t Ep) {
  const uint32_t hi = fx_hiword(v), lo = fx_loword(v);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  const uint64_t m = (static_cast<uint64_t>(__funnelshift_l(lo, hi, 11) | 0x80000000u) << 32) | (lo << 11);
  uint64_t t;
  asm("shr.b64 %0, %1, %2;" : "=l"(t) : "l"(m), "r"(Ep - e));
  const uint64_t neg = static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(hi) >> 31));
  return (t ^ neg) + TX_BIAS_A + (neg & 1u);
}

// fp16x2 word of digit t (0 = most significant) of two biased integers:
// low half from x, high half from y; each half is the fp16 number
// byte - 128 (byte | 0x6400 is the fp16 value 1024 + byte).
template <int T>
QF_D uint32_t tx_digit_pair(uint64_t x, uint64_t y) {
  constexpr int byte = 7 - T;  // little-endian byte index within the 64-bit integer
  const uint32_t xw = byte >= 4 ? static_cast<uint32_t>(x >> 32) : static_cast<uint32_t>(x);
  const uint32_t yw = byte >= 4 ? static_cast<uint32_t>(y >> 32) : static_cast<uint32_t>(y);
  constexpr uint32_t b = byte & 3;
  // selector: byte b of xw into byte 0, byte b of yw (source bytes 4..7) into byte 2
  // selector nibbles: result byte 0 <- byte b of xw, result byte 2 <- byte b of yw
  const uint32_t w = __byte_perm(xw, yw, b | ((4u + b) << 8)) & 0x00FF00FFu;
  const uint32_t biased = w | 0x64006400u;
  __half2 r = *reinterpret_cast<const __half2*>(&biased);
  r = __hsub2(r, __halves2half2(__float2half_rn(1152.f), __float2half_rn(1152.f)));
  return *reinterpret_cast<uint32_t*>(&r);
}

// The same fp16x2 digit word for the amplitudes (biased by TX_BIAS_A).
// Digits 0-3 (the high words): one byte permute puts the digit bytes in
// the low byte of each half and zeros above them (sign copies of the top
// byte), i.e. the fp16 subnormals byte * 2^-24; two exact half-precision
// multiply-adds make them byte - bias, leaving the integer ALU (the
// busiest unit) one instruction per word.  Digits 4-7 as tx_digit_pair.
template <int T>
QF_D uint32_t tx_digit_pair_a(uint64_t x, uint64_t y) {
  if constexpr (T >= 4) {
    return tx_digit_pair<T>(x, y);
  } else {
    constexpr uint32_t b = 3 - T;  // byte of the high word
    const uint32_t xw = static_cast<uint32_t>(x >> 32), yw = static_cast<uint32_t>(y >> 32);
    // result bytes: byte b of xw, sign of byte 3 of xw, byte b of yw, sign of byte 3 of yw
    // (prmt's sign-replicating selectors: the __byte_perm intrinsic takes
    // only the byte index bits of each selector)
    uint32_t w;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(w) : "r"(xw), "r"(yw), "r"(b | (0xBu << 4) | ((4u + b) << 8) | (0xFu << 12)));
    constexpr float bias = T == 0 ? 64.f : 128.f;
    __half2 h = *reinterpret_cast<const __half2*>(&w);
    const __half2 k = __float2half2_rn(4096.f);
    h = __hfma2(__hmul2(h, k), k, __float2half2_rn(-bias));
    return *reinterpret_cast<uint32_t*>(&h);
  }
}

// Z = sum_delta acc_delta 2^(49 - 8 delta) (= A.G / 2^63) from the eight
// accumulator words (FP32 integers below 2^22): each becomes 1.5 * 2^23 +
// acc exactly, whose bit pattern is TX_MAGIC_BITS + acc.  A pair joins in
// uint32 as b_2j 256 + b_2j+1 = p_j + K2 with p_j = acc_2j 256 + acc_2j+1
// (|p_j| < 2^30 + 2^22) and K2 = 257 TX_MAGIC_BITS mod 2^32 = 0x8B400000,
// which never wraps; K2 is a multiple of 128, so the biases of the four
// pairs leave one constant, subtracted once.  The shifts and adds are
// multiply-adds (the FMA pipe), the integer ALU being the busiest unit.
QF_D int64_t tx_combine(const uint32_t (&w)[8]) {
  uint32_t b[8];
#pragma unroll
  for (int d = 0; d < 8; ++d) b[d] = __float_as_uint(__uint_as_float(w[d]) + TX_MAGIC);
  constexpr uint32_t K2 = static_cast<uint32_t>(TX_MAGIC_BITS) * 257u;
  static_assert(K2 == 0x8B400000u && K2 % 128u == 0u, "pair bias");
  constexpr uint64_t C = (static_cast<uint64_t>(K2) << 41) + (static_cast<uint64_t>(K2) << 25) +
                         (static_cast<uint64_t>(K2) << 9) + (K2 >> 7);
  const uint32_t q0 = b[0] * 256u + b[1], q1 = b[2] * 256u + b[3];
  const uint32_t q2 = b[4] * 256u + b[5], q3 = b[6] * 256u + b[7];
  // sums wrap mod 2^64; the true Z fits int64
  uint64_t z = fx_madu(q2, 1u << 9, static_cast<uint64_t>(q3 >> 7) - C);
  z = fx_madu(q1, 1u << 25, z);
  const uint32_t zh = static_cast<uint32_t>(z >> 32) + q0 * 512u;
  return static_cast<int64_t>((static_cast<uint64_t>(zh) << 32) | static_cast<uint32_t>(z));
}

// FP64 value of Z * 2^(E - 1082), its sign flipped when the sign bit of ds
// is set: Z is converted exactly rounded by the FP64 pipe's convert, and
// the power of two (delta = (E - 1082) << 20) and the sign flip (adding
// 2^31 mod 2^32) are one multiply-add on the high word, ds = delta ^ sign,
// scaled by min(hi, 1) so that Z = 0 stays 0 without a compare and select
// on the integer ALU.  E >= 64 and |Z| >= 1 keep the result normal.
QF_D double tx_out(int64_t Z, uint32_t ds) {
  const double d = __ll2double_rn(Z);
  const uint32_t hi = fx_hiword(d);
  return fx_double(hi + min(hi, 1u) * ds, fx_loword(d));
}

// ------------------------------------------------------------ pass parts ----
// B: row 32 u + o (digit u of output real o = 2 r + p), K = input real
// 2 c + q; one fp16x2 word (q = 0, 1) per (u, r, c, p)
QF_D void tx_build_b(const TxParams& P, unsigned char* sb, int tid, int nthreads) {
  for (int w = tid; w < TX_ND * 16 * 16 * 2; w += nthreads) {
    const int p = w & 1, c = (w >> 1) & 15, r = (w >> 5) & 15, u = w >> 9;
    const int64_t gre = P.g[r][c][0], gim = P.g[r][c][1];
    // real form: re out = (Re, -Im) . (re, im); im out = (Im, Re) . (re, im)
    const uint64_t x = static_cast<uint64_t>(p == 0 ? gre : gim) + TX_BIAS;
    const uint64_t y = static_cast<uint64_t>(p == 0 ? -gim : gre) + TX_BIAS;
    uint32_t word;
    switch (u) {
      case 0: word = tx_digit_pair<0>(x, y); break;
      case 1: word = tx_digit_pair<1>(x, y); break;
      case 2: word = tx_digit_pair<2>(x, y); break;
      case 3: word = tx_digit_pair<3>(x, y); break;
      case 4: word = tx_digit_pair<4>(x, y); break;
      case 5: word = tx_digit_pair<5>(x, y); break;
      case 6: word = tx_digit_pair<6>(x, y); break;
      default: word = tx_digit_pair<7>(x, y); break;
    }
    const int row = 32 * u + 2 * r + p, k = 2 * c;  // fp16 element k, k + 1 of the row
    *reinterpret_cast<uint32_t*>(sb + tx_piece(row, k >> 3) + (k & 7) * 2) = word;
  }
}

// Global index of a row with its window bits zero: the row index's bits
// are spread over the non-window bits.  The tile part (tile * 128, the same
// for every thread) and the row-in-tile part map independently.
QF_D int64_t tx_spread(const TxParams& P, int64_t x) {
#pragma unroll
  for (int j = 0; j < 4; ++j) x = insert0(x, P.sbits[j]);
  return x;
}


// Row exponent shared by the AP-amplitude groups of one row (lanes l, l ^ 8
// and, for AP = 4, l ^ 16, l ^ 24): the largest FP64 exponent field (4095
// for rows below 2^-959, which become 0).
template <int AP>
QF_D int tx_rowexp(const double2 (&x)[AP]) {
  uint32_t mx = 0u;
#pragma unroll
  for (int j = 0; j < AP; ++j) {
    mx = max(mx, fx_hiword(x[j].x) & 0x7fffffffu);
    mx = max(mx, fx_hiword(x[j].y) & 0x7fffffffu);
  }
  mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
  if (AP == 4) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
  return static_cast<int>(mx >> 20) < FX_EMIN ? 4095 : static_cast<int>(mx >> 20);
}

// Input group of one thread: its AP amplitudes (window indices AP q + j)
// of row irow, after the input-side signs, become digits in A (sa), scaled
// by the row exponent E (tx_rowexp), which goes to rowE[irow].  b is the
// group's base (the input-side signs test it).  As soon as four amplitudes
// have become integers, their registers take the loads of the same
// amplitudes of the next tile (group base nb; none when nb < 0), so those
// are in flight during the rest of this conversion and the MMAs.
template <int AP>
QF_D void tx_convert(const TxParams& P, const double2* __restrict__ in, double2 (&x)[AP], unsigned char* sa,
                     uint16_t* rowE, int64_t b, int irow, int q, int E, int64_t nb) {
  if (P.nin > 0) {
    uint32_t fl = 0u;
    for (int s = 0; s < P.nin; ++s)
      if ((static_cast<uint64_t>(b) & P.in_mout[s]) == P.in_mout[s]) fl ^= P.in_rmask[s];
    fl >>= AP * q;
#pragma unroll
    for (int j = 0; j < AP; ++j) {
      const uint32_t sg = ((fl >> j) & 1u) << 31;
      x[j] = make_double2(fx_double(fx_hiword(x[j].x) ^ sg, fx_loword(x[j].x)),
                          fx_double(fx_hiword(x[j].y) ^ sg, fx_loword(x[j].y)));
    }
  }
  if (q == 0) rowE[irow] = static_cast<uint16_t>(E);
  const uint32_t Ep = static_cast<uint32_t>(E + 64 - TX_MB);
#pragma unroll
  for (int j0 = 0; j0 < AP; j0 += 4) {
    uint64_t ur[4], ui[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      ur[j] = tx_biased(x[j0 + j].x, Ep);
      ui[j] = tx_biased(x[j0 + j].y, Ep);
    }
    if (nb >= 0) {
#pragma unroll
      for (int j = 0; j < 4; ++j) x[j0 + j] = in[nb | P.off[j0 + j]];
    }
    // digit t of amplitudes c = AP q + j0 .. + 3: fp16 elements (t & 1) 32 + 2c
    // of chunk t >> 1, one 16-byte piece
#define QF_TX_STORE(T)                                                                                   \
  {                                                                                                      \
    uint4 v;                                                                                             \
    v.x = tx_digit_pair_a<T>(ur[0], ui[0]);                                                             \
    v.y = tx_digit_pair_a<T>(ur[1], ui[1]);                                                             \
    v.z = tx_digit_pair_a<T>(ur[2], ui[2]);                                                             \
    v.w = tx_digit_pair_a<T>(ur[3], ui[3]);                                                             \
    const int piece = ((T & 1) * 32 + 2 * (AP * q + j0)) >> 3;                                          \
    *reinterpret_cast<uint4*>(sa + (T >> 1) * TX_A_CHUNK + tx_piece(irow, piece)) = v;                  \
  }
    QF_TX_STORE(0)
    QF_TX_STORE(1)
    QF_TX_STORE(2)
    QF_TX_STORE(3)
    QF_TX_STORE(4)
    QF_TX_STORE(5)
    QF_TX_STORE(6)
    QF_TX_STORE(7)
#undef QF_TX_STORE
  }
}

// The MMAs of one tile: amplitude digit t against gate digits 0 .. 7 - t,
// into accumulator columns [acc + 32 t, acc + 256)
QF_D void tx_issue(uint32_t abase, uint32_t bbase, uint32_t acc) {
#pragma unroll
  for (int t = 0; t < TX_ND; ++t) {
    const uint32_t idesc = tx_idesc(TX_KD * (TX_ND - t));
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const uint32_t a = abase + (t >> 1) * TX_A_CHUNK + (t & 1) * 64 + ks * 32;
      const uint32_t b = bbase + ks * 32;
      tx_mma(acc + static_cast<uint32_t>(TX_KD * t), tx_desc(a), tx_desc(b), idesc, (t > 0 || ks > 0) ? 1u : 0u);
    }
  }
}

// Epilogue of one thread: 16 output reals (amplitudes c = 8 oh + j) of its
// row (half-row base b) from the accumulators at tensor-memory address acc
// (lane field set), with the output-side signs, stored as FP64.  The tensor-memory loads of
// the next four reals are in flight while four are converted.  As soon as
// the last of them has landed, the warp releases the accumulators (one
// arrival on tmem_free), before its last conversions and stores.
template <bool DB>
QF_D void tx_epilogue(const TxParams& P, double2* out, uint32_t acc, int E, int64_t b, int oh, uint64_t* tmem_free) {
  const uint32_t delta = static_cast<uint32_t>(E - 1082) << 20;
  uint32_t fl = 0u;
  for (int s = 0; s < P.nout; ++s)
    if ((static_cast<uint64_t>(b) & P.out_mout[s]) == P.out_mout[s]) fl ^= P.out_rmask[s];
  fl = (fl >> (8 * oh)) & 0xFFu;
  uint32_t a4[DB ? 2 : 1][8][4];
#pragma unroll
  for (int d = 0; d < 8; ++d) tx_ld4(acc + static_cast<uint32_t>(TX_KD * d + 16 * oh), a4[0][d]);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (!DB && q > 0) {
#pragma unroll
      for (int d = 0; d < 8; ++d) tx_ld4(acc + static_cast<uint32_t>(TX_KD * d + 16 * oh + 4 * q), a4[0][d]);
    }
    tx_wait_ld(a4[DB ? (q & 1) : 0]);
    if (q == 3) {
      tx_fence_before();
      __syncwarp();
      if ((threadIdx.x & 31) == 0) tx_arrive(tmem_free);
    }
    if (DB && q < 3) {
#pragma unroll
      for (int d = 0; d < 8; ++d)
        tx_ld4(acc + static_cast<uint32_t>(TX_KD * d + 16 * oh + 4 * (q + 1)), a4[DB ? ((q + 1) & 1) : 0][d]);
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int j = 2 * q + a;
      uint32_t wr[8], wi[8];
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        wr[d] = a4[DB ? (q & 1) : 0][d][2 * a];
        wi[d] = a4[DB ? (q & 1) : 0][d][2 * a + 1];
      }
      const uint32_t ds = delta ^ (((fl >> j) & 1u) << 31);
      out[b | P.off[j]] = make_double2(tx_out(tx_combine(wr), ds), tx_out(tx_combine(wi), ds));
    }
  }
}

// ------------------------------------------------ warp-specialised kernel ----
// One CTA per SM; three stages of the A operand (tile i in A stage i % 3),
// two of the accumulators (tensor-memory stage i & 1: 2 x 256 of its 512
// columns).  The converter warps (AP amplitudes per thread: 8 -> 8 warps,
// 4 -> 16 warps) convert tile i into its A stage once the MMAs of tile i - 3
// have read it (a_free) and arrive on a_full.  One thread of the last warp
// issues the MMAs: it waits for the converters of tile i and for the
// epilogue of tile i - 2 to release the accumulators (tmem_free), issues
// the tile's MMAs and commits them to a_free and mma_done.  An MMA issue
// holds its thread about as long as the tensor core takes to run it, so
// that thread does nothing else.  The 8 epilogue warps wait for the MMAs
// (and for the issuer's e_ready, which passes on the converters' row
// exponents), run the epilogue from the accumulators and release them
// (tmem_free, one arrival per warp).  The converters wait only for the
// tensor core, the epilogue only for the MMAs.
constexpr int TX_AST = 3;   // A-operand stages
constexpr int TX_ESL = 5;   // row-exponent slots: tile i + 5 is converted only after the epilogue of tile i
constexpr uint32_t TP_SMEM = TX_AST * TX_A_BYTES + TX_B_BYTES + 1024;
constexpr int TP_TMEM_COLS = 512;

template <int AP>
struct TxShape {
  static constexpr int CW = 128 * (16 / AP) / 32;  // converter warps
  // converters, epilogue, and one warpgroup whose first thread issues the MMAs
  static constexpr int THREADS = 32 * (CW + 8 + 4);
  static constexpr bool DB = AP == 8;               // double-buffered tensor-memory reads (registers allow)
};
// Register split (AP = 8: 640 threads launched at 96 registers, 61440 in
// all): the issuer's warpgroup gives its registers up (24 each), the
// converters take 120 and the epilogue 104: 256 x 120 + 256 x 104 + 128 x 24
// = 60416 (at N=28, 128 / 96 ran 1.5% and 112 / 112 0.7% slower).
constexpr int TX_REG_LAUNCH = 96, TX_REG_CONV = 120, TX_REG_EPI = 104, TX_REG_ISSUE = 24;
static_assert(256 * TX_REG_CONV + 256 * TX_REG_EPI + 128 * TX_REG_ISSUE <= 640 * TX_REG_LAUNCH,
              "register split above the launch's registers");
static_assert(32 * (2 * TX_REG_CONV + 2 * TX_REG_EPI + TX_REG_ISSUE) <= 16384,
              "register split above one scheduler partition's registers");

template <int AP>
__global__ void __launch_bounds__(TxShape<AP>::THREADS, 1) k_txpipe(const __grid_constant__ TxParams P) {
  constexpr int CW = TxShape<AP>::CW;
  extern __shared__ __align__(1024) unsigned char tx_raw[];
  unsigned char* sm = tx_raw + ((1024u - (tx_smem(tx_raw) & 1023u)) & 1023u);  // 1024-byte aligned
  unsigned char* sb = sm + TX_AST * TX_A_BYTES;
  __shared__ __align__(8) uint64_t a_full[TX_AST], a_free[TX_AST], mma_done[2], e_ready[2], tmem_free[2];
  __shared__ uint32_t tmem_slot;
  __shared__ uint16_t rowE[TX_ESL][TX_ROWS];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  tx_build_b(P, sb, tid, TxShape<AP>::THREADS);
  if (warp == 0) tx_alloc(&tmem_slot, TP_TMEM_COLS);
  if (tid == 0) {
    for (int a = 0; a < TX_AST; ++a) {
      tx_bar_init(&a_full[a], 32 * CW);
      tx_bar_init(&a_free[a], 1);
    }
    for (int t = 0; t < 2; ++t) {
      tx_bar_init(&mma_done[t], 1);
      tx_bar_init(&e_ready[t], 1);
      tx_bar_init(&tmem_free[t], 8);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tx_fence_before();
  __syncthreads();
  tx_fence_after();
  const uint32_t tmem = tmem_slot;
  const int64_t ntiles = (int64_t(1) << (P.n - 4)) / TX_ROWS;
  if (warp < CW) {
    if constexpr (AP == 8) asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(TX_REG_CONV));
    // ---- converters.  Row irow, group q (window
    // indices AP q .. AP q + AP - 1); the lanes of one 8-lane shared-store
    // phase hold 8 consecutive rows (distinct swizzle phases) and the groups
    // of a row are lanes l ^ 8 (and l ^ 16, l ^ 24)
    const double2* __restrict__ in = static_cast<const double2*>(P.in);
    const int irow = AP == 8 ? warp * 16 + (lane & 7) + ((lane >> 4) << 3) : warp * 8 + (lane & 7);
    const int q = AP == 8 ? (lane >> 3) & 1 : lane >> 3;
    const int64_t grow = tx_spread(P, irow) | P.off[AP * q];  // this group within its tile
    const int64_t step = gridDim.x;
    double2 x[AP];
    int64_t tile = blockIdx.x;
    if (tile < ntiles) {
      const int64_t b = tx_spread(P, tile * TX_ROWS) | grow;
#pragma unroll
      for (int j = 0; j < AP; ++j) x[j] = in[b | P.off[j]];
    }
    int a = 0, ar = 0;  // A stage (it % 3) and its round (it / 3)
    for (int it = 0; tile < ntiles; tile += step, ++it) {
      bool ok = true;
      if (ar > 0) ok = tx_wait(&a_free[a], static_cast<uint32_t>(ar - 1) & 1u, P.err);
      if (!__all_sync(0xffffffffu, ok)) break;  // warp-uniform: the row exponent shuffles within the warp
      tx_fence_after();
      unsigned char* sa = sm + a * TX_A_BYTES;
      const int64_t nb = tile + step < ntiles ? tx_spread(P, (tile + step) * TX_ROWS) | grow : -1;
      tx_convert<AP>(P, in, x, sa, rowE[it % TX_ESL], tx_spread(P, tile * TX_ROWS) | grow, irow, q,
                     tx_rowexp<AP>(x), nb);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tx_arrive(&a_full[a]);  // this thread's digits and row exponent are written
      if (++a == TX_AST) {
        a = 0;
        ++ar;
      }
    }
  } else if (warp >= CW + 8) {
    // ---- MMA issuer (one thread of this warpgroup)
    if constexpr (AP == 8) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(TX_REG_ISSUE));
    if (warp == CW + 8 && lane == 0) {
      const uint32_t bbase = tx_smem(sb);
      int a = 0, ar = 0;
      int64_t last = -1;  // the last tile whose MMAs were issued
      for (int64_t it = 0, tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int t = static_cast<int>(it & 1);
        if (!tx_wait(&a_full[a], static_cast<uint32_t>(ar) & 1u, P.err)) break;
        if (it >= 2 && !tx_wait(&tmem_free[t], static_cast<uint32_t>((it >> 1) - 1) & 1u, P.err)) break;
        // the converters' row exponents, passed on to the epilogue (after
        // tmem_free, so that e_ready is never two phases ahead of it)
        tx_arrive(&e_ready[t]);
        tx_fence_after();
        tx_issue(tx_smem(sm + a * TX_A_BYTES), bbase, tmem + static_cast<uint32_t>(256 * t));
        tx_commit(&a_free[a]);
        tx_commit(&mma_done[t]);
        last = it;
        if (++a == TX_AST) {
          a = 0;
          ++ar;
        }
      }
      // every MMA issued has finished before the accumulators are freed (on
      // the normal path the epilogue has already seen this phase; after an
      // expired wait the epilogue may have left its loop early)
      if (last >= 0) tx_wait(&mma_done[last & 1], static_cast<uint32_t>(last >> 1) & 1u, P.err);
    }
  } else {
    // ---- epilogue
    if constexpr (AP == 8) asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(TX_REG_EPI));
    double2* out = static_cast<double2*>(P.out);
    const int ew = warp - CW;
    const int orow = 32 * (ew & 3) + lane, oh = ew >> 2;
    const int64_t hrow = tx_spread(P, orow) | (oh ? P.off[8] : 0);
    const uint32_t lane_addr = static_cast<uint32_t>(32 * (ew & 3)) << 16;
    int64_t tile = blockIdx.x;
    for (int it = 0; tile < ntiles; tile += gridDim.x, ++it) {
      const int t = it & 1;
      const uint32_t par = static_cast<uint32_t>(it >> 1) & 1u;
      const bool ok = tx_wait(&e_ready[t], par, P.err) && tx_wait(&mma_done[t], par, P.err);
      if (!__all_sync(0xffffffffu, ok)) break;
      tx_fence_after();
      tx_epilogue<TxShape<AP>::DB>(P, out, tmem + lane_addr + static_cast<uint32_t>(256 * t),
                                   rowE[it % TX_ESL][orow], tx_spread(P, tile * TX_ROWS) | hrow, oh, &tmem_free[t]);
    }
  }
  tx_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TP_TMEM_COLS) : "memory");
}

template <int AP>
int tx_launch_ap(const TxParams& P, cudaStream_t stream) {
  static std::atomic<int> attr_set[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!attr_set[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_txpipe<AP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TP_SMEM));
    if (rc) return rc;
    attr_set[dev].store(1);
  }
  const int64_t ntiles = (int64_t(1) << (P.n - 4)) / TX_ROWS;
  int64_t grid = device_sm_count();
  if (grid > ntiles) grid = ntiles;
  k_txpipe<AP><<<(int)grid, TxShape<AP>::THREADS, TP_SMEM, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

}  // namespace

// Launch one tensor-core pass (P.in/out/err set by the caller); the state
// must have at least 2^11 amplitudes.  Every row is read completely before
// its outputs are written, by the same CTA, so the pass may run in place.
int tx_launch(const TxParams& P, cudaStream_t stream) {
  if (P.n < 11) return QF_ERR_NOT_SUPPORTED;
  // eight amplitudes per converter thread: 8 converter warps at 128
  // registers; four per thread (16 converter warps, 80 registers) issued 12%
  // more instructions and ran 7% slower at N=28
  return tx_launch_ap<8>(P, stream);
}

}  // namespace qf
