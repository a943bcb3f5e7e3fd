// State preparation, layout conversion, reductions, sampling and the QAOA
// cut table.
//
// Reference: quantumflow/states.py:113-147 (probabilities, sample,
// expectation), :186-191 (zero_state), quantumflow/qubits.py:180-182 (norm),
// quantumflow/backend/numpybk.py:125-128 (inner), quantumflow/qaoa.py:68-81
// (graph_cuts).
#include "engine.cuh"
#include "state.cuh"

#include <cmath>
#include <cstring>

namespace qf {

// ------------------------------------------------------------- fills -------
template <typename E> QF_D E make_amp(double re, double im);
template <> QF_D float2 make_amp<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <> QF_D double2 make_amp<double2>(double re, double im) { return make_double2(re, im); }
template <> QF_D float4 make_amp<float4>(double re, double im) {
  float rh, rl, ih, il;
  split_d(re, rh, rl);
  split_d(im, ih, il);
  return make_float4(rh, rl, ih, il);
}

template <int LAY>
__global__ void k_fill_basis(typename Types<LAY>::E* psi, int64_t namps, int64_t index) {
  using E = typename Types<LAY>::E;
  const E zero = make_amp<E>(0.0, 0.0), one = make_amp<E>(1.0, 0.0);
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr)
    psi[x] = (x == index) ? one : zero;
}

template <int LAY>
__global__ void k_fill_uniform(typename Types<LAY>::E* psi, int64_t namps, double amp) {
  using E = typename Types<LAY>::E;
  const E v = make_amp<E>(amp, 0.0);
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) psi[x] = v;
}

// --------------------------------------------------------- conversion ------
QF_D double2 as_c128(float2 a) { return make_double2(a.x, a.y); }
QF_D double2 as_c128(double2 a) { return a; }
QF_D double2 as_c128(float4 a) {
  return make_double2((double)a.x + (double)a.y, (double)a.z + (double)a.w);
}
template <typename E> QF_D E from_c128(double2 a);
template <> QF_D float2 from_c128<float2>(double2 a) { return make_float2((float)a.x, (float)a.y); }
template <> QF_D double2 from_c128<double2>(double2 a) { return a; }
template <> QF_D float4 from_c128<float4>(double2 a) { return make_amp<float4>(a.x, a.y); }

template <int SL, int DL>
__global__ void k_convert(const typename Types<SL>::E* src, typename Types<DL>::E* dst, int64_t namps) {
  using DE = typename Types<DL>::E;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr)
    dst[x] = from_c128<DE>(as_c128(src[x]));
}

template <int LAY>
__global__ void k_scale(typename Types<LAY>::E* psi, int64_t namps, double s) {
  using E = typename Types<LAY>::E;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    if constexpr (LAY == C64) {
      psi[x] = make_float2(psi[x].x * (float)s, psi[x].y * (float)s);
    } else if constexpr (LAY == C128) {
      psi[x] = make_double2(psi[x].x * s, psi[x].y * s);
    } else {
      float sh, sl;
      split_d(s, sh, sl);
      const float4 a = psi[x];
      FFAcc re, im;
      re.zero();
      im.zero();
      re.add_prod(sh, sl, a.x, a.y);
      im.add_prod(sh, sl, a.z, a.w);
      float4 r;
      re.finish(r.x, r.y);
      im.finish(r.z, r.w);
      psi[x] = r;
    }
  }
}

// --------------------------------------------------------- reductions ------
// |a|^2 as a float-float value
QF_D void norm2_ff(float2 a, float& h, float& l) {
  FFAcc t;
  t.zero();
  acc_norm2(t, a);
  t.finish(h, l);
}
QF_D void norm2_ff(float4 a, float& h, float& l) {
  FFAcc t;
  t.zero();
  acc_norm2(t, a);
  t.finish(h, l);
}
QF_D void norm2_ff(double2 a, float& h, float& l) {
  FFAcc t;
  t.zero();
  acc_norm2(t, a);
  t.finish(h, l);
}

QF_D void split_any(float v, float& h, float& l) {
  h = v;
  l = 0.f;
}
QF_D void split_any(double v, float& h, float& l) { split_d(v, h, l); }

// Block reduction of two float-float accumulators into partials[2*block].
QF_D void block_reduce2(const FFAcc& a0, const FFAcc& a1, double* partials) {
  __shared__ double sh[2][32];
  double v0 = (double)a0.s + (double)a0.e;
  double v1 = (double)a1.s + (double)a1.e;
  v0 = warp_sum(v0);
  v1 = warp_sum(v1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][warp] = v0;
    sh[1][warp] = v1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) {
      s0 += sh[0][w];
      s1 += sh[1][w];
    }
    partials[2 * blockIdx.x] = s0;
    partials[2 * blockIdx.x + 1] = s1;
  }
}

// kind: 0 = norm2, 1 = expectation with uint16 cuts, 2 = expectation with
// double diagonal.
template <int LAY, int KIND>
__global__ void __launch_bounds__(256) k_reduce_diag(const typename Types<LAY>::E* psi, int64_t namps,
                                                     const uint16_t* cuts, const double* diag,
                                                     double* partials) {
  FFAcc acc, unused;
  acc.zero();
  unused.zero();
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    float ph, pl;
    norm2_ff(psi[x], ph, pl);
    if (KIND == 0) {
      acc.add(ph, pl);
    } else if (KIND == 1) {
      const float c = (float)cuts[x];
      acc.add_prod(c, 0.f, ph, pl);
    } else {
      float dh, dl;
      split_d(diag[x], dh, dl);
      acc.add_prod(dh, dl, ph, pl);
    }
  }
  block_reduce2(acc, unused, partials);
}

template <int LAY>
__global__ void __launch_bounds__(256) k_reduce_inner(const typename Types<LAY>::E* a,
                                                      const typename Types<LAY>::E* b, int64_t namps,
                                                      double* partials) {
  FFAcc re, im;
  re.zero();
  im.zero();
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    const float4 u = to_ff(a[x]), v = to_ff(b[x]);
    // conj(u) v = (ur ur' ...) : re = ur vr + ui vi, im = ur vi - ui vr
    re.add_prod(u.x, u.y, v.x, v.y);
    re.add_prod(u.z, u.w, v.z, v.w);
    im.add_prod(u.x, u.y, v.z, v.w);
    im.add_prod(-u.z, -u.w, v.x, v.y);
  }
  block_reduce2(re, im, partials);
}

// Probabilities of global bit `bit` being 0 and 1 (the single-qubit
// measurement of quantumflow/stdops.py:53-64, without the projected copy).
template <int LAY>
__global__ void __launch_bounds__(256) k_reduce_bit(const typename Types<LAY>::E* psi, int64_t namps, int bit,
                                                    double* partials) {
  FFAcc p0, p1;
  p0.zero();
  p1.zero();
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    float ph, pl;
    norm2_ff(psi[x], ph, pl);
    if ((x >> bit) & 1) p1.add(ph, pl);
    else p0.add(ph, pl);
  }
  block_reduce2(p0, p1, partials);
}

// Fixed-order final pass over the block partials.
__global__ void k_finish2(const double* partials, int nblocks, double* out, int nout) {
  __shared__ double sh[2][256];
  double s0 = 0.0, s1 = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
    s0 += partials[2 * i];
    s1 += partials[2 * i + 1];
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sh[0][0];
    if (nout > 1) out[1] = sh[1][0];
  }
}

int reduce_blocks(int64_t namps) {
  int64_t b = (namps + 1023) / 1024;
  const int64_t cap = (int64_t)device_sm_count() * 8;
  if (b > cap) b = cap;
  if (b > REDUCE_MAX_BLOCKS) b = REDUCE_MAX_BLOCKS;
  if (b < 1) b = 1;
  return (int)b;
}

template <int LAY>
static int reduce_diag_t(const void* psi, int n, int kind, const uint16_t* cuts, const double* diag,
                         double* out, double* partials, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  const int64_t namps = int64_t(1) << n;
  const int nb = reduce_blocks(namps);
  const E* p = reinterpret_cast<const E*>(psi);
  if (kind == 0) k_reduce_diag<LAY, 0><<<nb, 256, 0, stream>>>(p, namps, cuts, diag, partials);
  else if (kind == 1) k_reduce_diag<LAY, 1><<<nb, 256, 0, stream>>>(p, namps, cuts, diag, partials);
  else k_reduce_diag<LAY, 2><<<nb, 256, 0, stream>>>(p, namps, cuts, diag, partials);
  k_finish2<<<1, 256, 0, stream>>>(partials, nb, out, 1);
  return check_cuda(cudaGetLastError());
}

template <int LAY>
static int reduce_bit_t(const void* psi, int n, int bit, double* out, double* partials, cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  const int64_t namps = int64_t(1) << n;
  const int nb = reduce_blocks(namps);
  k_reduce_bit<LAY><<<nb, 256, 0, stream>>>(reinterpret_cast<const E*>(psi), namps, bit, partials);
  k_finish2<<<1, 256, 0, stream>>>(partials, nb, out, 2);
  return check_cuda(cudaGetLastError());
}

int reduce_bit(const void* psi, int n, int layout, int bit, double* out, double* partials, cudaStream_t stream) {
  switch (layout) {
    case C64: return reduce_bit_t<C64>(psi, n, bit, out, partials, stream);
    case C128: return reduce_bit_t<C128>(psi, n, bit, out, partials, stream);
    case FF: return reduce_bit_t<FF>(psi, n, bit, out, partials, stream);
  }
  return QF_ERR_LAYOUT;
}

int reduce_diag(const void* psi, int n, int layout, int kind, const uint16_t* cuts, const double* diag,
                double* out, double* partials, cudaStream_t stream) {
  switch (layout) {
    case C64: return reduce_diag_t<C64>(psi, n, kind, cuts, diag, out, partials, stream);
    case C128: return reduce_diag_t<C128>(psi, n, kind, cuts, diag, out, partials, stream);
    case FF: return reduce_diag_t<FF>(psi, n, kind, cuts, diag, out, partials, stream);
  }
  return QF_ERR_LAYOUT;
}

template <int LAY>
static int reduce_inner_t(const void* a, const void* b, int n, double* out, double* partials,
                          cudaStream_t stream) {
  using E = typename Types<LAY>::E;
  const int64_t namps = int64_t(1) << n;
  const int nb = reduce_blocks(namps);
  k_reduce_inner<LAY><<<nb, 256, 0, stream>>>(reinterpret_cast<const E*>(a),
                                               reinterpret_cast<const E*>(b), namps, partials);
  k_finish2<<<1, 256, 0, stream>>>(partials, nb, out, 2);
  return check_cuda(cudaGetLastError());
}

int reduce_inner(const void* a, const void* b, int n, int layout, double* out, double* partials,
                 cudaStream_t stream) {
  switch (layout) {
    case C64: return reduce_inner_t<C64>(a, b, n, out, partials, stream);
    case C128: return reduce_inner_t<C128>(a, b, n, out, partials, stream);
    case FF: return reduce_inner_t<FF>(a, b, n, out, partials, stream);
  }
  return QF_ERR_LAYOUT;
}

// ------------------------------------------------------ probabilities ------
template <int LAY>
__global__ void k_probs(const typename Types<LAY>::E* psi, int64_t namps, double* probs) {
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    if constexpr (LAY == C128) {
      const double2 a = psi[x];
      probs[x] = fma(a.x, a.x, a.y * a.y);
    } else {
      float h, l;
      norm2_ff(psi[x], h, l);
      probs[x] = (double)h + (double)l;
    }
  }
}

static int grid_for(int64_t items) {
  int64_t g = (items + 255) / 256;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

int probabilities(const void* psi, int n, int layout, double* probs, cudaStream_t stream) {
  const int64_t namps = int64_t(1) << n;
  switch (layout) {
    case C64:
      k_probs<C64><<<grid_for(namps), 256, 0, stream>>>(reinterpret_cast<const float2*>(psi), namps, probs);
      break;
    case C128:
      k_probs<C128><<<grid_for(namps), 256, 0, stream>>>(reinterpret_cast<const double2*>(psi), namps, probs);
      break;
    case FF:
      k_probs<FF><<<grid_for(namps), 256, 0, stream>>>(reinterpret_cast<const float4*>(psi), namps, probs);
      break;
    default:
      return QF_ERR_LAYOUT;
  }
  return check_cuda(cudaGetLastError());
}

// ----------------------------------------------------------- sampling ------
// Inclusive scan of probabilities in three launches: per-block totals,
// a single-block scan of the totals, then per-block scans with offsets.
constexpr int SCAN_BLOCK = 1024;  // amplitudes per scan block (256 threads x 4)

__global__ void k_scan_totals(const double* p, int64_t namps, double* totals) {
  __shared__ double sh[256];
  const int64_t base = (int64_t)blockIdx.x * SCAN_BLOCK;
  double s = 0.0;
  for (int i = threadIdx.x; i < SCAN_BLOCK; i += blockDim.x) {
    const int64_t x = base + i;
    if (x < namps) s += p[x];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = sh[0];
}

// exclusive scan of totals in place (single block, sequential chunks)
__global__ void k_scan_offsets(double* totals, int64_t nblocks) {
  __shared__ double sh[1024];
  double carry = 0.0;
  for (int64_t c0 = 0; c0 < nblocks; c0 += 1024) {
    const int64_t i = c0 + threadIdx.x;
    const double v = i < nblocks ? totals[i] : 0.0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
      double t = ((int)threadIdx.x >= o) ? sh[threadIdx.x - o] : 0.0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nblocks) totals[i] = carry + sh[threadIdx.x] - v;
    const double chunk_total = sh[1023];
    __syncthreads();
    carry += chunk_total;
  }
}

__global__ void k_scan_blocks(double* p, int64_t namps, const double* offsets) {
  __shared__ double sh[SCAN_BLOCK];
  const int64_t base = (int64_t)blockIdx.x * SCAN_BLOCK;
  for (int i = threadIdx.x; i < SCAN_BLOCK; i += blockDim.x) {
    const int64_t x = base + i;
    sh[i] = x < namps ? p[x] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // sequential within the block: 1024 adds
    double c = offsets[blockIdx.x];
    for (int i = 0; i < SCAN_BLOCK; ++i) {
      c += sh[i];
      sh[i] = c;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SCAN_BLOCK; i += blockDim.x) {
    const int64_t x = base + i;
    if (x < namps) p[x] = sh[i];
  }
}

// splitmix64 (Steele, Lea, Flood 2014) as a counter-based generator
QF_D uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_draw(const double* cdf, int64_t namps, int64_t trials, uint64_t seed, int64_t* counts) {
  const double total = cdf[namps - 1];
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < trials; j += nthr) {
    const uint64_t r = mix64(seed ^ mix64((uint64_t)j));
    const double u = (double)(r >> 11) * (1.0 / 9007199254740992.0) * total;  // [0, total)
    int64_t lo = 0, hi = namps - 1;  // first x with cdf[x] > u
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (cdf[mid] > u) hi = mid;
      else lo = mid + 1;
    }
    atomicAdd(reinterpret_cast<unsigned long long*>(counts + lo), 1ull);
  }
}

size_t sample_workspace_bytes(int n) {
  const int64_t namps = int64_t(1) << n;
  const int64_t nb = (namps + SCAN_BLOCK - 1) / SCAN_BLOCK;
  return (size_t)namps * 8 + (size_t)nb * 8 + 256;
}

int sample(const void* psi, int n, int layout, int64_t trials, uint64_t seed, int64_t* counts,
           void* ws, cudaStream_t stream) {
  const int64_t namps = int64_t(1) << n;
  const int64_t nb = (namps + SCAN_BLOCK - 1) / SCAN_BLOCK;
  double* cdf = reinterpret_cast<double*>(ws);
  double* totals = cdf + namps;
  int rc = probabilities(psi, n, layout, cdf, stream);
  if (rc) return rc;
  k_scan_totals<<<(unsigned)nb, 256, 0, stream>>>(cdf, namps, totals);
  k_scan_offsets<<<1, 1024, 0, stream>>>(totals, nb);
  k_scan_blocks<<<(unsigned)nb, 256, 0, stream>>>(cdf, namps, totals);
  rc = check_cuda(cudaMemsetAsync(counts, 0, (size_t)namps * sizeof(int64_t), stream));
  if (rc) return rc;
  if (trials > 0) {
    int64_t g = (trials + 255) / 256;
    const int64_t cap = (int64_t)device_sm_count() * 16;
    if (g > cap) g = cap;
    k_draw<<<(unsigned)g, 256, 0, stream>>>(cdf, namps, trials, seed, counts);
  }
  return check_cuda(cudaGetLastError());
}

// ------------------------------------------------------------ cuts ---------
struct EdgeList {
  int nedges;
  uint8_t bits[2 * CUT_MAX_EDGES];  // global bit positions
};

__global__ void k_cuts(uint16_t* cuts, int64_t namps, const __grid_constant__ EdgeList e) {
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    unsigned c = 0;
    for (int i = 0; i < e.nedges; ++i)
      c += (unsigned)(((x >> e.bits[2 * i]) ^ (x >> e.bits[2 * i + 1])) & 1);
    cuts[x] = (uint16_t)c;
  }
}

struct WEdgeList {
  int nedges;
  uint8_t bits[2 * CUT_MAX_EDGES];
  double w[CUT_MAX_EDGES];
};

__global__ void k_cuts_w(double* cuts, int64_t namps, const __grid_constant__ WEdgeList e) {
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < namps; x += nthr) {
    double c = 0.0;
    for (int i = 0; i < e.nedges; ++i)
      if (((x >> e.bits[2 * i]) ^ (x >> e.bits[2 * i + 1])) & 1) c += e.w[i];
    cuts[x] = c;
  }
}

int cut_values(uint16_t* cuts, int n, int nedges, const int* edges, cudaStream_t stream) {
  static thread_local EdgeList e;
  e.nedges = nedges;
  for (int i = 0; i < 2 * nedges; ++i) e.bits[i] = (uint8_t)(n - 1 - edges[i]);
  const int64_t namps = int64_t(1) << n;
  k_cuts<<<grid_for(namps), 256, 0, stream>>>(cuts, namps, e);
  return check_cuda(cudaGetLastError());
}

int cut_values_weighted(double* cuts, int n, int nedges, const int* edges, const double* w,
                        cudaStream_t stream) {
  static thread_local WEdgeList e;
  e.nedges = nedges;
  for (int i = 0; i < 2 * nedges; ++i) e.bits[i] = (uint8_t)(n - 1 - edges[i]);
  for (int i = 0; i < nedges; ++i) e.w[i] = w[i];
  const int64_t namps = int64_t(1) << n;
  k_cuts_w<<<grid_for(namps), 256, 0, stream>>>(cuts, namps, e);
  return check_cuda(cudaGetLastError());
}

// ---------------------------------------------------------- dispatch -------
int fill_basis(void* psi, int n, int layout, int64_t index, cudaStream_t stream) {
  const int64_t namps = int64_t(1) << n;
  switch (layout) {
    case C64: k_fill_basis<C64><<<grid_for(namps), 256, 0, stream>>>((float2*)psi, namps, index); break;
    case C128: k_fill_basis<C128><<<grid_for(namps), 256, 0, stream>>>((double2*)psi, namps, index); break;
    case FF: k_fill_basis<FF><<<grid_for(namps), 256, 0, stream>>>((float4*)psi, namps, index); break;
    default: return QF_ERR_LAYOUT;
  }
  return check_cuda(cudaGetLastError());
}

int fill_uniform(void* psi, int n, int layout, cudaStream_t stream) {
  const int64_t namps = int64_t(1) << n;
  const double amp = 1.0 / std::sqrt((double)namps);
  switch (layout) {
    case C64: k_fill_uniform<C64><<<grid_for(namps), 256, 0, stream>>>((float2*)psi, namps, amp); break;
    case C128: k_fill_uniform<C128><<<grid_for(namps), 256, 0, stream>>>((double2*)psi, namps, amp); break;
    case FF: k_fill_uniform<FF><<<grid_for(namps), 256, 0, stream>>>((float4*)psi, namps, amp); break;
    default: return QF_ERR_LAYOUT;
  }
  return check_cuda(cudaGetLastError());
}

template <int SL>
static int convert_from(const void* src, void* dst, int dl, int64_t namps, cudaStream_t stream) {
  using SE = typename Types<SL>::E;
  const SE* s = reinterpret_cast<const SE*>(src);
  switch (dl) {
    case C64: k_convert<SL, C64><<<grid_for(namps), 256, 0, stream>>>(s, (float2*)dst, namps); break;
    case C128: k_convert<SL, C128><<<grid_for(namps), 256, 0, stream>>>(s, (double2*)dst, namps); break;
    case FF: k_convert<SL, FF><<<grid_for(namps), 256, 0, stream>>>(s, (float4*)dst, namps); break;
    default: return QF_ERR_LAYOUT;
  }
  return check_cuda(cudaGetLastError());
}

int convert(const void* src, int sl, void* dst, int dl, int n, cudaStream_t stream) {
  const int64_t namps = int64_t(1) << n;
  switch (sl) {
    case C64: return convert_from<C64>(src, dst, dl, namps, stream);
    case C128: return convert_from<C128>(src, dst, dl, namps, stream);
    case FF: return convert_from<FF>(src, dst, dl, namps, stream);
  }
  return QF_ERR_LAYOUT;
}

int scale(void* psi, int n, int layout, double s, cudaStream_t stream) {
  const int64_t namps = int64_t(1) << n;
  switch (layout) {
    case C64: k_scale<C64><<<grid_for(namps), 256, 0, stream>>>((float2*)psi, namps, s); break;
    case C128: k_scale<C128><<<grid_for(namps), 256, 0, stream>>>((double2*)psi, namps, s); break;
    case FF: k_scale<FF><<<grid_for(namps), 256, 0, stream>>>((float4*)psi, namps, s); break;
    default: return QF_ERR_LAYOUT;
  }
  return check_cuda(cudaGetLastError());
}

}  // namespace qf
