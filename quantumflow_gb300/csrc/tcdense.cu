// Dense K-qubit gates (K = 5, 6) on complex64 states on the 5th-generation
// tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// Reference semantics: quantumflow/backend/numpybk.py:159-214 tensormul
// with a wide gate.  A dense gate on K qubits costs 2^K complex
// multiply-adds per amplitude -- 64 at K = 6 -- which makes the sweep
// compute-bound on the FP32 pipes; as a real GEMM it is
//     Y[g, :] = X[g, :] . Gr^T,   X[g, 2c + {0,1}] = (re, im) of amplitude c
// of column group g (the 2^K amplitudes that differ only in the gate's
// bits), Gr the 2^(K+1) x 2^(K+1) real form of the gate.  A CTA takes 128
// column groups per tile (the MMA's M), the whole real gate width as N (128
// at K = 6) and walks K in chunks of 32 elements.
//
// Precision: the MMAs run kind::tf32 (11 significant bits per operand), so
// each operand is split exactly into hi = x with its low 13 mantissa bits
// cleared and lo = x - hi, and three MMAs accumulate hi.hi + hi.lo + lo.hi
// in FP32 (relative error ~2^-22 per product, the complex64 result's own
// precision).
//
// Shared memory holds the gate (hi and lo planes, built once per CTA from the
// caller's complex128 device matrix) and a two-stage ring of X chunks (hi and
// lo), all in the canonical K-major layout with 128-byte swizzling: row r of
// a 32-element chunk is 128 bytes at r * 128, its 16-byte pieces permuted by
// XOR with (r mod 8); groups of 8 rows are 1024 bytes apart.  Two threads
// share a tile row (8 amplitudes of each chunk apiece) and hold the whole
// next tile of their row in registers: the loads of tile t+1's chunk c are
// issued as soon as chunk c of tile t is in shared memory, so one tile of
// reads (64 KB at K = 6) is in flight per SM while the tensor cores work.
// One thread issues the MMAs and commits them to the stage's mbarrier.  The
// accumulators alternate between two tensor-memory regions by tile, so the
// epilogue of tile t (tcgen05.ld, scattered stores) runs while the MMAs of
// tile t+1's first chunk execute.  Every wait is bounded (4 s); on expiry the
// kernel raises the device error word and stops, with every thread leaving
// the loop at the same barrier (__syncthreads_or of the failures).
#include <algorithm>
#include <atomic>
#include <cstring>

#include "engine.cuh"

namespace qf {

int* device_error_word();

namespace {

constexpr int TC_M = 128;        // column groups per tile (MMA M)
constexpr int TC_THREADS = 256;  // two threads per tile row
constexpr int TC_KC = 32;        // K elements per chunk (128 bytes of fp32)
constexpr int TC_AH = TC_KC / 4; // amplitudes per thread per chunk

struct TcParams {
  const float2* in;
  float2* out;
  const double2* mat;  // 2^K x 2^K complex, row-major (device)
  int* err;            // device error word
  int32_t n, k;
  int32_t sbits[6];    // gate bits ascending
  int32_t gb[6];       // gate bits, matrix MSB first
};

QF_D uint32_t tc_smem(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// canonical K-major, 128B-swizzled shared-memory matrix descriptor
QF_D uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);  // start address
  d |= static_cast<uint64_t>(1) << 16;                   // leading byte offset (unused when swizzled)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;           // stride byte offset: 8 rows x 128 B
  d |= static_cast<uint64_t>(1) << 46;                   // descriptor version
  d |= static_cast<uint64_t>(2) << 61;                   // 128-byte swizzle
  return d;
}
// instruction descriptor: D f32, A and B tf32, both K-major, M = 128
QF_D uint32_t tc_idesc(int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(TC_M >> 4) << 24);
}
// byte offset of element (row, k) (k < 32) of a 128B-swizzled chunk
QF_D uint32_t tc_swz(int row, int k) {
  return static_cast<uint32_t>(row * 128 + ((((k >> 2) ^ (row & 7)) << 4) | ((k & 3) << 2)));
}
QF_D float tc_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

QF_D void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
QF_D void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(bar))
               : "memory");
}
QF_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
QF_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

QF_D bool tc_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(tc_smem(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
QF_D uint64_t tc_now() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// bounded wait (4 s of wall clock); false (and the error word raised) on expiry
QF_D bool tc_wait(uint64_t* bar, uint32_t parity, int* err) {
  if (tc_try_wait(bar, parity)) return true;
  const uint64_t t0 = tc_now();
  while (!tc_try_wait(bar, parity)) {
    if (tc_now() - t0 > 4000000000ull) {
      atomicOr(err, 1);
      return false;
    }
  }
  return true;
}

// 32 consecutive fp32 accumulator columns of this warp's 32 TMEM lanes
QF_D void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <int K>
struct TcGeom {
  static constexpr int D = 1 << K;          // amplitudes per column group
  static constexpr int KD = 2 * D;          // real width (GEMM K and N)
  static constexpr int NCH = KD / TC_KC;    // K chunks (2 or 4: even, so stage = chunk parity)
  static constexpr uint32_t B_CHUNK = KD * 128;        // one 32-wide chunk of the gate: N rows x 128 B
  static constexpr uint32_t B_BYTES = NCH * B_CHUNK;   // one plane (hi or lo)
  static constexpr uint32_t A_CHUNK = TC_M * 128;      // one 32-wide chunk of X: 128 rows x 128 B
  // layout: B hi | B lo | A stage 0 hi | A stage 0 lo | A stage 1 hi | A stage 1 lo
  static constexpr uint32_t A_OFF = 2 * B_BYTES;
  static constexpr uint32_t BYTES = A_OFF + 4 * A_CHUNK;
  static constexpr int TMEM_COLS = 2 * KD;  // two fp32 accumulators (by tile parity)
};

template <int K>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tcdense(const __grid_constant__ TcParams P) {
  using Geo = TcGeom<K>;
  constexpr int D = Geo::D, KD = Geo::KD, NCH = Geo::NCH;
  static_assert(NCH % 2 == 0, "the stage of a chunk is its parity within the tile");
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  // 1024-byte alignment of the swizzled regions
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int64_t offs[D];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (TC_M - 1), half = tid >> 7;

  for (int c = tid; c < D; c += TC_THREADS) {
    int64_t o = 0;
    for (int j = 0; j < K; ++j)
      if ((c >> (K - 1 - j)) & 1) o |= int64_t(1) << P.gb[j];
    offs[c] = o;
  }
  // the gate's real form, hi and lo planes: B row n = output real n, column
  // k = input real k (Gr[2r][2c] = Re, [2r][2c+1] = -Im, [2r+1][2c] = Im,
  // [2r+1][2c+1] = Re of G[r][c]); one complex entry per iteration
  for (int e = tid; e < D * D; e += TC_THREADS) {
    const double2 g = P.mat[e];
    const int r = e >> K, c = e & (D - 1);
    const float re = static_cast<float>(g.x), im = static_cast<float>(g.y);
    const uint32_t chunk = static_cast<uint32_t>((2 * c) / TC_KC) * Geo::B_CHUNK;
    const uint32_t o0 = chunk + tc_swz(2 * r, (2 * c) % TC_KC), o1 = chunk + tc_swz(2 * r + 1, (2 * c) % TC_KC);
    const float2 h0 = make_float2(tc_hi(re), tc_hi(-im)), h1 = make_float2(tc_hi(im), tc_hi(re));
    *reinterpret_cast<float2*>(sm + o0) = h0;
    *reinterpret_cast<float2*>(sm + o1) = h1;
    *reinterpret_cast<float2*>(sm + Geo::B_BYTES + o0) = make_float2(re - h0.x, -im - h0.y);
    *reinterpret_cast<float2*>(sm + Geo::B_BYTES + o1) = make_float2(im - h1.x, re - h1.y);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_slot)),
                 "r"(Geo::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc_idesc(KD);
  const uint32_t sbase = tc_smem(sm);
  // this thread's TMEM lanes (its warp's quarter of the rows) and output columns
  const uint32_t lane_addr = static_cast<uint32_t>(32 * (warp & 3)) << 16;
  uint32_t phase = 0u;    // bit s: the parity stage s's next wait expects
  uint32_t pending = 0u;  // bit s: a commit on stage s not yet waited for
  int fail = 0;           // this thread saw a wait expire

  const int64_t ngroups = int64_t(1) << (P.n - K);
  const int64_t ntiles = ngroups / TC_M;  // the host launches only when TC_M divides ngroups
  auto row_base = [&](int64_t tile) {
    int64_t b = tile * TC_M + row;
    for (int j = 0; j < K; ++j) b = insert0(b, P.sbits[j]);
    return b;
  };
  // stores the accumulator of a finished tile (rows of base b) to the output
  auto epilogue = [&](int64_t b, uint32_t acc) {
#pragma unroll
    for (int c0 = 0; c0 < KD / 2; c0 += 32) {
      float v[32];
      tc_ld32(acc + lane_addr + static_cast<uint32_t>(half * (KD / 2) + c0), v);
      const int a0 = (half * (KD / 2) + c0) / 2;
#pragma unroll
      for (int i = 0; i < 16; ++i) P.out[b | offs[a0 + i]] = make_float2(v[2 * i], v[2 * i + 1]);
    }
  };

  // registers: this thread's 8 amplitudes of every chunk of its row's next tile
  float2 x[NCH][TC_AH];
  int64_t tile = blockIdx.x;
  int64_t cur_b = 0, prev_b = 0;
  if (tile < ntiles) {
    cur_b = row_base(tile);
#pragma unroll
    for (int kc = 0; kc < NCH; ++kc)
#pragma unroll
      for (int j = 0; j < TC_AH; ++j) x[kc][j] = P.in[cur_b | offs[kc * (TC_KC / 2) + half * TC_AH + j]];
  }
  int it = 0;
  bool stopped = false;
  for (; tile < ntiles && !stopped; tile += gridDim.x, ++it) {
    const bool has_next = tile + gridDim.x < ntiles;
    const int64_t nb = has_next ? row_base(tile + gridDim.x) : 0;
    const uint32_t acc = tmem + static_cast<uint32_t>((it & 1) * KD);
#pragma unroll
    for (int kc = 0; kc < NCH; ++kc) {
      const int s = kc & 1;
      // the MMAs that last read this stage must be done before it is rewritten
      if ((pending >> s) & 1u) {
        if (!tc_wait(&bar[s], (phase >> s) & 1u, P.err)) fail = 1;
        phase ^= 1u << s;
        pending &= ~(1u << s);
      }
      // split this thread's amplitudes of chunk kc into the stage's hi and lo
      // rows, two amplitudes (one 16-byte piece) at a time
      unsigned char* ahi = sm + Geo::A_OFF + (2 * s) * Geo::A_CHUNK;
      unsigned char* alo = ahi + Geo::A_CHUNK;
#pragma unroll
      for (int j = 0; j < TC_AH; j += 2) {
        const float2 v0 = x[kc][j], v1 = x[kc][j + 1];
        const float4 h = make_float4(tc_hi(v0.x), tc_hi(v0.y), tc_hi(v1.x), tc_hi(v1.y));
        const uint32_t o = tc_swz(row, 2 * (half * TC_AH + j));
        *reinterpret_cast<float4*>(ahi + o) = h;
        *reinterpret_cast<float4*>(alo + o) = make_float4(v0.x - h.x, v0.y - h.y, v1.x - h.z, v1.y - h.w);
      }
      // the same chunk of the next tile: in flight until this chunk comes round again
      if (has_next) {
#pragma unroll
        for (int j = 0; j < TC_AH; ++j) x[kc][j] = P.in[nb | offs[kc * (TC_KC / 2) + half * TC_AH + j]];
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_before();
      if (__syncthreads_or(fail)) {
        stopped = true;
        break;
      }
      tc_fence_after();
      if (tid == 0) {
        const uint32_t a_hi = sbase + Geo::A_OFF + (2 * s) * Geo::A_CHUNK, a_lo = a_hi + Geo::A_CHUNK;
        const uint32_t b_hi = sbase + kc * Geo::B_CHUNK, b_lo = b_hi + Geo::B_BYTES;
#pragma unroll
        for (int ks = 0; ks < TC_KC / 8; ++ks) {  // 8 tf32 (32 bytes) per MMA
          const uint32_t koff = ks * 32;
          const uint32_t accumulate = (kc > 0 || ks > 0) ? 1u : 0u;
          tc_mma(acc, tc_desc(a_hi + koff), tc_desc(b_hi + koff), idesc, accumulate);
          tc_mma(acc, tc_desc(a_hi + koff), tc_desc(b_lo + koff), idesc, 1u);
          tc_mma(acc, tc_desc(a_lo + koff), tc_desc(b_hi + koff), idesc, 1u);
        }
        tc_commit(&bar[s]);
      }
      pending |= 1u << s;
      if (kc == 0 && it > 0) {
        // the previous tile: the commit of its last chunk (stage 1) covers
        // all of its MMAs; its accumulator is read while this tile's first
        // chunk is on the tensor cores
        if (!tc_wait(&bar[1], (phase >> 1) & 1u, P.err)) fail = 1;
        phase ^= 2u;
        pending &= ~2u;
        if (__all_sync(0xffffffffu, fail == 0)) epilogue(prev_b, tmem + static_cast<uint32_t>(((it - 1) & 1) * KD));
      }
    }
    prev_b = cur_b;
    cur_b = nb;
  }
  // drain: MMAs still reading shared memory or writing tensor memory finish
  // before the last tile's epilogue and the CTA's exit
  for (int s = 0; s < 2; ++s)
    if ((pending >> s) & 1u) {
      if (!tc_wait(&bar[s], (phase >> s) & 1u, P.err)) fail = 1;
    }
  tc_fence_before();
  const int any_fail = __syncthreads_or(fail);
  tc_fence_after();
  if (!stopped && !any_fail && it > 0) epilogue(prev_b, tmem + static_cast<uint32_t>(((it - 1) & 1) * KD));
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Geo::TMEM_COLS) : "memory");
}

template <int K>
int tc_launch(const TcParams& P, cudaStream_t stream) {
  static std::atomic<int> attr_set[64];
  constexpr size_t smem = TcGeom<K>::BYTES + 1024;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!attr_set[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_tcdense<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (rc) return rc;
    attr_set[dev].store(1);
  }
  const int64_t ntiles = (int64_t(1) << (P.n - K)) / TC_M;
  int64_t grid = device_sm_count();
  if (grid > ntiles) grid = ntiles;
  k_tcdense<K><<<(int)grid, TC_THREADS, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

}  // namespace

// Tensor-core path of qf_apply_dense_gate for complex64 states; returns
// QF_ERR_NOT_SUPPORTED (launching nothing) outside its domain: K = 5 or 6,
// at least one full tile of 128 column groups.  Every column group is read
// completely before its outputs are written, by the same thread, so the
// gate may be applied in place.
int tc_dense_gate(const void* in, void* out, int n, int k, const int* bits, const double* mat, cudaStream_t stream) {
  if ((k != 5 && k != 6) || n - k < 7) return QF_ERR_NOT_SUPPORTED;
  TcParams P;
  std::memset(&P, 0, sizeof(P));
  P.in = reinterpret_cast<const float2*>(in);
  P.out = reinterpret_cast<float2*>(out);
  P.mat = reinterpret_cast<const double2*>(mat);
  P.err = device_error_word();
  if (P.err == nullptr) return QF_ERR_CUDA;
  P.n = n;
  P.k = k;
  for (int j = 0; j < k; ++j) P.gb[j] = P.sbits[j] = bits[j];
  std::sort(P.sbits, P.sbits + k);
  return k == 5 ? tc_launch<5>(P, stream) : tc_launch<6>(P, stream);
}

}  // namespace qf
