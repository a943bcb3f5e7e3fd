// Dense gates on many qubits with a device-resident matrix:
// qf_apply_dense_gate.
//
// Reference semantics: quantumflow/backend/numpybk.py:159-214 tensormul for
// any K (the reference's einsum takes up to the state's rank; wide gates
// come from Gate.__matmul__, quantumflow/ops.py:187-198, and
// Circuit.asgate, quantumflow/circuits.py:111-118).  A 2^K x 2^K matrix is
// too large for kernel parameters beyond K = 5, so the caller passes it in
// device memory.
//
// Kernel k_densek: a CTA takes CPG column groups at a time -- a column group
// is the 2^K amplitudes that differ only in the gate's bits -- stages them in
// shared memory, and then each warp computes output rows: lanes split the
// row's 2^K columns (coalesced reads of the row-major matrix, which stays
// in L2 across CTAs), multiply against all CPG staged groups, and reduce
// with shuffles.  Every group is owned by one CTA and fully staged before
// its outputs are written, so the gate may be applied in place.
// complex64 states compute in FP32, complex128 in FP64; float-float states
// are converted to complex128 in place around the FP64 kernel.  Dense
// complex64 gates on 5 or 6 qubits take the tensor cores instead
// (tcdense.cu) unless qf_set_dense_tensor_cores(0).
#include <algorithm>
#include <atomic>
#include <cstring>

#include "engine.cuh"

namespace qf {

int convert(const void* src, int sl, void* dst, int dl, int n, cudaStream_t stream);
int tc_dense_gate(const void* in, void* out, int n, int k, const int* bits, const double* mat, cudaStream_t stream);
int g_dense_tensor_cores = 1;  // qf_set_dense_tensor_cores

constexpr int DENSEK_MAX = QF_MAX_DENSE_QUBITS;

struct DenseKParams {
  const void* in;
  void* out;
  const double2* mat;  // row-major 2^K x 2^K, (re, im)
  int32_t n, k;
  int32_t sbits[DENSEK_MAX];  // gate bits, ascending
  int32_t gb[DENSEK_MAX];     // gate bits, matrix MSB first
};

template <typename E>
struct DkAcc;
template <>
struct DkAcc<float2> {
  using T = float;
};
template <>
struct DkAcc<double2> {
  using T = double;
};

template <typename E, int CPG>
__global__ void __launch_bounds__(256) k_densek(const __grid_constant__ DenseKParams P) {
  using T = typename DkAcc<E>::T;
  extern __shared__ __align__(16) unsigned char dk_smem[];
  const int K = P.k;
  const int D = 1 << K;
  int64_t* offs = reinterpret_cast<int64_t*>(dk_smem);  // [D] offset of row index r
  int64_t* bases = offs + D;                             // [CPG]
  E* s = reinterpret_cast<E*>(bases + CPG);              // [CPG][D]
  const E* in = reinterpret_cast<const E*>(P.in);
  E* out = reinterpret_cast<E*>(P.out);
  const int64_t ngroups = int64_t(1) << (P.n - K);
  for (int r = threadIdx.x; r < D; r += blockDim.x) {
    int64_t o = 0;
    for (int j = 0; j < K; ++j)
      if ((r >> (K - 1 - j)) & 1) o |= int64_t(1) << P.gb[j];
    offs[r] = o;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t g0 = (int64_t)blockIdx.x * CPG; g0 < ngroups; g0 += (int64_t)gridDim.x * CPG) {
    __syncthreads();  // offs ready / previous batch's reads of s done
    if (threadIdx.x < CPG) {
      int64_t b = g0 + threadIdx.x;
      for (int j = 0; j < K; ++j) b = insert0(b, P.sbits[j]);
      bases[threadIdx.x] = g0 + threadIdx.x < ngroups ? b : -1;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < CPG * D; i += blockDim.x) {
      const int g = i >> K, r = i & (D - 1);
      const int64_t b = bases[g];
      E v;
      if (b >= 0) {
        v = in[b | offs[r]];
      } else {
        v.x = 0;
        v.y = 0;
      }
      s[i] = v;
    }
    __syncthreads();
    for (int r = warp; r < D; r += nwarps) {
      T re[CPG], im[CPG];
#pragma unroll
      for (int g = 0; g < CPG; ++g) re[g] = im[g] = T(0);
      const double2* row = P.mat + (int64_t)r * D;
      for (int c = lane; c < D; c += 32) {
        const double2 m = row[c];
        const T mr = static_cast<T>(m.x), mi = static_cast<T>(m.y);
#pragma unroll
        for (int g = 0; g < CPG; ++g) {
          const E a = s[g * D + c];
          re[g] = fma(mr, a.x, re[g]);
          re[g] = fma(-mi, a.y, re[g]);
          im[g] = fma(mr, a.y, im[g]);
          im[g] = fma(mi, a.x, im[g]);
        }
      }
#pragma unroll
      for (int g = 0; g < CPG; ++g) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          re[g] += __shfl_xor_sync(0xffffffffu, re[g], o);
          im[g] += __shfl_xor_sync(0xffffffffu, im[g], o);
        }
      }
      if (lane < CPG) {
        T vr = re[0], vi = im[0];
#pragma unroll
        for (int g = 1; g < CPG; ++g)
          if (lane == g) {
            vr = re[g];
            vi = im[g];
          }
        const int64_t b = bases[lane];
        if (b >= 0) {
          E v;
          v.x = vr;
          v.y = vi;
          out[b | offs[r]] = v;
        }
      }
    }
  }
}

namespace {

template <typename E, int CPG>
size_t densek_smem(int k) {
  return (size_t(1) << k) * sizeof(int64_t) + CPG * sizeof(int64_t) + CPG * (size_t(1) << k) * sizeof(E);
}

template <typename E, int CPG>
int densek_launch(const DenseKParams& P, cudaStream_t stream) {
  static std::atomic<int> attr_set[64];
  const size_t smem = densek_smem<E, CPG>(P.k);
  if (smem > 200 * 1024) return QF_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!attr_set[dev].load()) {
    int rc = check_cuda(cudaFuncSetAttribute(k_densek<E, CPG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024));
    if (rc) return rc;
    attr_set[dev].store(1);
  }
  const int64_t ngroups = int64_t(1) << (P.n - P.k);
  int64_t grid = (ngroups + CPG - 1) / CPG;
  const int64_t cap = (int64_t)device_sm_count() * 4;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  k_densek<E, CPG><<<(int)grid, 256, smem, stream>>>(P);
  return check_cuda(cudaGetLastError());
}

// widest group batch whose staging fits ~64 KiB
template <typename E>
int densek_dispatch(const DenseKParams& P, cudaStream_t stream) {
  const size_t group = (size_t(1) << P.k) * sizeof(E);
  if (group * 8 <= 64 * 1024) return densek_launch<E, 8>(P, stream);
  if (group * 4 <= 64 * 1024) return densek_launch<E, 4>(P, stream);
  if (group * 2 <= 64 * 1024) return densek_launch<E, 2>(P, stream);
  return densek_launch<E, 1>(P, stream);
}

}  // namespace

int apply_dense_gate(const void* in, void* out, int n, int layout, int k, const int* bits, const double* mat,
                     cudaStream_t stream) {
  DenseKParams P;
  std::memset(&P, 0, sizeof(P));
  P.in = in;
  P.out = out;
  P.mat = reinterpret_cast<const double2*>(mat);
  P.n = n;
  P.k = k;
  for (int j = 0; j < k; ++j) P.gb[j] = P.sbits[j] = bits[j];
  std::sort(P.sbits, P.sbits + k);
  switch (layout) {
    case C64:
      if (g_dense_tensor_cores) {
        const int rc = tc_dense_gate(in, out, n, k, bits, mat, stream);
        if (rc != QF_ERR_NOT_SUPPORTED) return rc;
      }
      return densek_dispatch<float2>(P, stream);
    case C128:
    case FX:
      return densek_dispatch<double2>(P, stream);
    case FF: {
      // float-float <-> complex128 in place (both 16 bytes per amplitude)
      int rc = convert(in, FF, out, C128, n, stream);
      if (rc) return rc;
      P.in = out;
      rc = densek_dispatch<double2>(P, stream);
      if (rc) return rc;
      return convert(out, C128, out, FF, n, stream);
    }
  }
  return QF_ERR_LAYOUT;
}

}  // namespace qf
