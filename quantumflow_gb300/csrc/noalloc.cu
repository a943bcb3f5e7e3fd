// Allocation-free expectation value: qf_expectation_cuts_noalloc.
//
// Who needs this: a caller that can hand the library the state, the cut
// table and an output slot, but cannot obtain any further device memory for
// it.  Examples are a host application whose memory pool owns every byte of
// the GPU and forbids outside allocations, or a latency-critical loop that
// must not call cudaMalloc (which can synchronise the device and stall
// other streams).  The regular qf_expectation_cuts needs a caller-supplied
// workspace for its per-block partial sums; this variant keeps those partial
// sums in a fixed array compiled into the library instead.
//
// Limits and sharing:
//   - The array holds QF_NOALLOC_MAX_PARTIALS (2048) block partial sums,
//     i.e. 2048 * 2 doubles = 32 KiB on every GPU that loads the library,
//     kept until the process exits.  A launch never uses more than 2048
//     blocks, so every state size up to QF_MAX_QUBITS fits; larger n is
//     rejected with QF_ERR_TOO_LARGE.
//   - Every call, on every stream, uses the same array.  Each block
//     overwrites its own slot before the final pass reads it, so nothing
//     needs clearing between calls, but two calls whose kernels overlap on
//     the GPU (different streams, or different host threads) race on the
//     array and may return wrong values.  Serialise such calls.
//   - Every call that is not being captured into a CUDA graph looks up the
//     array's device address (cudaGetSymbolAddress) with the calling device
//     current, so the address stays right after a device reset reloads the
//     library's module; a call made while its stream is capturing reuses
//     the address its device's last uncaptured call found.  Make one call
//     on each device before any stream capture begins.
#include <mutex>

#include "engine.cuh"
#include "state.cuh"

namespace qf {

static __device__ __align__(256) double g_noalloc_partials[2 * QF_NOALLOC_MAX_PARTIALS];

// Every reduction launch fits the array: the header's promise (any n up to
// QF_MAX_QUBITS) holds as long as this does.
static_assert(REDUCE_MAX_BLOCKS <= QF_NOALLOC_MAX_PARTIALS,
              "reduction block count exceeds the no-allocation partial-sum array");

namespace {

// Device address of g_noalloc_partials per device.  In host code the symbol
// names a host-side stand-in, not device memory, so the kernel must be given
// the address returned by cudaGetSymbolAddress instead.
std::mutex g_noalloc_mu;
double* g_noalloc_addr[64] = {nullptr};

int noalloc_scratch(cudaStream_t stream, double** out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev));
  if (rc) return rc;
  if (dev < 0 || dev >= 64) return QF_ERR_NOT_SUPPORTED;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  rc = check_cuda(cudaStreamIsCapturing(stream, &cap));
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone || g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_partials));
    if (rc) return rc;
    g_noalloc_addr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_addr[dev];
  return QF_OK;
}

}  // namespace
}  // namespace qf

extern "C" int qf_expectation_cuts_noalloc(const void* psi, int n, int layout, const uint16_t* cuts,
                                           double* out, void* stream) {
  using namespace qf;
  if (layout != C64 && layout != C128 && layout != FF && layout != FX) return QF_ERR_LAYOUT;
  if (layout == FX) layout = C128;  // the same complex128 bytes
  if (n > QF_MAX_QUBITS) return QF_ERR_TOO_LARGE;
  if (n < 1 || psi == nullptr || cuts == nullptr || out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(psi) & 15u) != 0) return QF_ERR_ALIGNMENT;
  if (reduce_blocks(int64_t(1) << n) > QF_NOALLOC_MAX_PARTIALS) return QF_ERR_TOO_LARGE;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  double* partials = nullptr;
  int rc = noalloc_scratch(s, &partials);
  if (rc) return rc;
  return reduce_diag(psi, n, layout, 1, cuts, nullptr, out, partials, s);
}
