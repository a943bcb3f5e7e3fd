// extern "C" entry points declared in include/qf_gb300.h: argument checks,
// status codes, and dispatch into the engine.  No entry point allocates
// device memory; callers pass workspaces where one is needed.
#include <cmath>
#include <cstdint>
#include <vector>

#include "engine.cuh"
#include "state.cuh"

namespace qf {
extern thread_local int t_last_cuda_error;
extern int g_force_smem_tile;
extern int g_adjoint_smem_only;
extern int g_warp_rb_override;
extern int g_merge_gates;
extern int g_group_kernel;
extern int g_shape_max_bits;
extern int g_dense_tensor_cores;
extern int g_fx_tensor;
extern int g_fx_min_blocks;
int read_clear_device_error(int* flags, cudaStream_t stream);
int apply_dense_gate(const void* in, void* out, int n, int layout, int k, const int* bits, const double* mat,
                     cudaStream_t stream);
int qaoa_state(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p, const double* beta,
               const double* gamma, const double* node_theta, int fusion_k, cudaStream_t stream);
size_t qaoa_grad_workspace_bytes(int n, int p, int layout);
size_t batch_workspace_bytes(int max_n, int layout, int ctas);
int batch_qaoa(const qf_batch_instance* inst, int ninst, int nlarge, const uint8_t* edges, const double* angles,
               double* out, int layout, int max_n, int ts, int ctas, void* ws, size_t ws_bytes,
               cudaStream_t stream);
int qaoa_grad(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p, const double* beta,
              const double* gamma, const double* node_theta, double* out, void* ws, cudaStream_t stream);
int wave_min_qubits(int layout);
int plan_stats(int n, int layout, std::vector<HostOp>& ops, int fusion_k, int32_t* stats, int max_blocks,
               int* nblocks);
int wave_plan(const qf_batch_instance* hinst, int ninst, int layout, void* host_plan, size_t host_bytes,
              size_t* need_host, size_t* need_device);
int wave_prepare(const void* host_plan, const uint8_t* edges, void* ws, size_t ws_bytes, cudaStream_t stream);
int wave_run(const void* host_plan, void* ws, size_t ws_bytes, const double* angles, double* out,
             const int32_t* skip, cudaStream_t stream);
}  // namespace qf

using namespace qf;

namespace {

bool valid_layout(int layout) { return layout == C64 || layout == C128 || layout == FF || layout == FX; }

// Storage layout of a buffer: QF_LAYOUT_FX holds complex128 values in the
// QF_LAYOUT_C128 bytes; only the gate engine computes differently on it.
int st(int layout) { return layout == FX ? C128 : layout; }

int check_state(const void* p, int n, int layout) {
  if (!valid_layout(layout)) return QF_ERR_LAYOUT;
  if (n > QF_MAX_QUBITS) return QF_ERR_TOO_LARGE;
  if (n < 1) return QF_ERR_INVALID_ARGUMENT;
  if (p == nullptr) return QF_ERR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(p) & 15u) != 0) return QF_ERR_ALIGNMENT;
  return QF_OK;
}

int check_ws(const void* ws, size_t have, size_t need) {
  if (ws == nullptr || have < need) return QF_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(ws) & 15u) != 0) return QF_ERR_ALIGNMENT;
  return QF_OK;
}

int axes_to_bits(int n, int k, const int* axes, int* bits) {
  if (axes == nullptr || k < 1) return QF_ERR_INVALID_ARGUMENT;
  if (k > QF_MAX_GATE_QUBITS) return QF_ERR_NOT_SUPPORTED;
  if (k > n) return QF_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < k; ++i) {
    if (axes[i] < 0 || axes[i] >= n) return QF_ERR_INVALID_ARGUMENT;
    for (int j = 0; j < i; ++j)
      if (axes[j] == axes[i]) return QF_ERR_INVALID_ARGUMENT;
    bits[i] = n - 1 - axes[i];
  }
  return QF_OK;
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace

extern "C" {

int qf_abi_version(void) { return QF_ABI_VERSION; }

const char* qf_status_string(int status) {
  switch (status) {
    case QF_OK: return "ok";
    case QF_ERR_INVALID_ARGUMENT: return "invalid argument";
    case QF_ERR_LAYOUT: return "unknown element layout";
    case QF_ERR_CUDA: return "CUDA runtime error";
    case QF_ERR_ALIGNMENT: return "device pointer not 16-byte aligned";
    case QF_ERR_TOO_LARGE: return "size above the supported maximum";
    case QF_ERR_NOT_SUPPORTED: return "operation not supported";
    case QF_ERR_DEVICE: return "a bounded device-side wait gave up";
    case QF_ERR_WORKSPACE: return "workspace missing or too small";
  }
  return "unknown status";
}

int qf_last_cuda_error(void) { return t_last_cuda_error; }

int qf_get_device_error(int* flags, void* stream) {
  if (flags == nullptr) return QF_ERR_INVALID_ARGUMENT;
  return read_clear_device_error(flags, as_stream(stream));
}

int qf_set_shape_bits(int bits) {
  if (bits < 0 || bits > 4) return QF_ERR_INVALID_ARGUMENT;
  g_shape_max_bits = bits;
  return QF_OK;
}

int qf_set_tile_kernel(int mode) {
  if (mode < 0 || mode > 5) return QF_ERR_INVALID_ARGUMENT;
  g_force_smem_tile = mode == 1;
  g_adjoint_smem_only = mode == 1;
  g_warp_rb_override = mode >= 2 && mode <= 4 ? mode : 0;
  g_group_kernel = mode == 5 ? 0 : 1;
  return QF_OK;
}

int qf_set_fx_occupancy(int min_blocks) {
  if (min_blocks < 1 || min_blocks > 4) return QF_ERR_INVALID_ARGUMENT;
  g_fx_min_blocks = min_blocks;
  return QF_OK;
}

int qf_set_fx_tensor_cores(int on) {
  if (on < 0 || on > 1) return QF_ERR_INVALID_ARGUMENT;
  g_fx_tensor = on;
  return QF_OK;
}

int qf_set_dense_tensor_cores(int on) {
  if (on < 0 || on > 1) return QF_ERR_INVALID_ARGUMENT;
  g_dense_tensor_cores = on;
  return QF_OK;
}

int qf_set_gate_merging(int on) {
  if (on < 0 || on > 2) return QF_ERR_INVALID_ARGUMENT;
  g_merge_gates = on;
  return QF_OK;
}

int qf_timing_enable(int on) { return timing_enable(on); }

int qf_timing_collect(double* ms, int64_t* launches, int nkinds) {
  if (ms == nullptr || launches == nullptr || nkinds < 0) return QF_ERR_INVALID_ARGUMENT;
  return timing_collect(ms, launches, nkinds);
}

size_t qf_reduce_workspace_bytes(int n) {
  (void)n;
  return (size_t)REDUCE_MAX_BLOCKS * 2 * sizeof(double);
}

size_t qf_sample_workspace_bytes(int n) {
  if (n < 1 || n > QF_MAX_QUBITS) return 0;
  return sample_workspace_bytes(n);
}

int qf_fill_basis(void* psi, int n, int layout, int64_t index, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (index < 0 || index >= (int64_t(1) << n)) return QF_ERR_INVALID_ARGUMENT;
  return fill_basis(psi, n, st(layout), index, as_stream(stream));
}

int qf_fill_uniform(void* psi, int n, int layout, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  return fill_uniform(psi, n, st(layout), as_stream(stream));
}

int qf_convert(const void* src, int src_layout, void* dst, int dst_layout, int n, void* stream) {
  int rc = check_state(src, n, src_layout);
  if (rc) return rc;
  rc = check_state(dst, n, dst_layout);
  if (rc) return rc;
  if (src == dst) return QF_ERR_INVALID_ARGUMENT;
  return convert(src, st(src_layout), dst, st(dst_layout), n, as_stream(stream));
}

int qf_scale(void* psi, int n, int layout, double s, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  return scale(psi, n, st(layout), s, as_stream(stream));
}

int qf_apply_gate(const void* psi_in, void* psi_out, int n, int layout, int k, const int* axes,
                  const double* matrix, void* stream) {
  int rc = check_state(psi_in, n, layout);
  if (rc) return rc;
  rc = check_state(psi_out, n, layout);
  if (rc) return rc;
  if (matrix == nullptr) return QF_ERR_INVALID_ARGUMENT;
  int bits[QF_MAX_GATE_QUBITS];
  rc = axes_to_bits(n, k, axes, bits);
  if (rc) return rc;
  std::vector<HostOp> ops(1);
  rc = classify_op(k, bits, matrix, ops[0]);
  if (rc) return rc;
  return run_ops(psi_in, psi_out, n, layout, ops, 1, as_stream(stream), nullptr);
}

int qf_apply_dense_gate(const void* psi_in, void* psi_out, int n, int layout, int k, const int* axes,
                        const double* matrix, void* stream) {
  int rc = check_state(psi_in, n, layout);
  if (rc) return rc;
  rc = check_state(psi_out, n, layout);
  if (rc) return rc;
  if (matrix == nullptr || axes == nullptr || k < 1 || k > n) return QF_ERR_INVALID_ARGUMENT;
  if (k > QF_MAX_DENSE_QUBITS) return QF_ERR_NOT_SUPPORTED;
  if ((reinterpret_cast<uintptr_t>(matrix) & 15u) != 0) return QF_ERR_ALIGNMENT;
  int bits[QF_MAX_DENSE_QUBITS];
  for (int i = 0; i < k; ++i) {
    if (axes[i] < 0 || axes[i] >= n) return QF_ERR_INVALID_ARGUMENT;
    for (int j = 0; j < i; ++j)
      if (axes[j] == axes[i]) return QF_ERR_INVALID_ARGUMENT;
    bits[i] = n - 1 - axes[i];
  }
  return apply_dense_gate(psi_in, psi_out, n, layout, k, bits, matrix, as_stream(stream));
}

int qf_run_circuit(const void* psi_in, void* psi_out, int n, int layout, int nops, const int* op_k,
                   const int* op_axes, const double* op_mats, int fusion_k, int* passes, void* stream) {
  int rc = check_state(psi_in, n, layout);
  if (rc) return rc;
  rc = check_state(psi_out, n, layout);
  if (rc) return rc;
  if (nops < 0) return QF_ERR_INVALID_ARGUMENT;
  if (nops > 0 && (op_k == nullptr || op_axes == nullptr || op_mats == nullptr))
    return QF_ERR_INVALID_ARGUMENT;
  std::vector<HostOp> ops(nops);
  size_t ax = 0, mo = 0;
  for (int i = 0; i < nops; ++i) {
    const int k = op_k[i];
    int bits[QF_MAX_GATE_QUBITS];
    rc = axes_to_bits(n, k, op_axes + ax, bits);
    if (rc) return rc;
    rc = classify_op(k, bits, op_mats + mo, ops[i]);
    if (rc) return rc;
    ax += k;
    mo += size_t(2) << (2 * k);
  }
  return run_ops(psi_in, psi_out, n, layout, ops, fusion_k, as_stream(stream), passes);
}

int qf_plan_circuit(int n, int layout, int nops, const int* op_k, const int* op_axes, const double* op_mats,
                    int fusion_k, int32_t* stats, int max_blocks, int* nblocks) {
  if (!valid_layout(layout)) return QF_ERR_LAYOUT;
  if (n < 1 || n > QF_MAX_QUBITS) return QF_ERR_INVALID_ARGUMENT;
  if (nops < 0 || nblocks == nullptr || max_blocks < 0 || (max_blocks > 0 && stats == nullptr))
    return QF_ERR_INVALID_ARGUMENT;
  if (nops > 0 && (op_k == nullptr || op_axes == nullptr || op_mats == nullptr)) return QF_ERR_INVALID_ARGUMENT;
  std::vector<HostOp> ops(nops);
  size_t ax = 0, mo = 0;
  for (int i = 0; i < nops; ++i) {
    const int k = op_k[i];
    int bits[QF_MAX_GATE_QUBITS];
    int rc = axes_to_bits(n, k, op_axes + ax, bits);
    if (rc) return rc;
    rc = classify_op(k, bits, op_mats + mo, ops[i]);
    if (rc) return rc;
    ax += k;
    mo += size_t(2) << (2 * k);
  }
  return plan_stats(n, layout, ops, fusion_k, stats, max_blocks, nblocks);
}

int qf_cut_values(uint16_t* cuts, int n, int nedges, const int* edges, void* stream) {
  if (cuts == nullptr || n < 1) return QF_ERR_INVALID_ARGUMENT;
  if (n > QF_MAX_QUBITS) return QF_ERR_TOO_LARGE;
  if (nedges < 0 || (nedges > 0 && edges == nullptr)) return QF_ERR_INVALID_ARGUMENT;
  if (nedges > CUT_MAX_EDGES) return QF_ERR_TOO_LARGE;
  for (int i = 0; i < 2 * nedges; ++i)
    if (edges[i] < 0 || edges[i] >= n) return QF_ERR_INVALID_ARGUMENT;
  return cut_values(cuts, n, nedges, edges, as_stream(stream));
}

int qf_cut_values_weighted(double* cuts, int n, int nedges, const int* edges, const double* weights,
                           void* stream) {
  if (cuts == nullptr || n < 1) return QF_ERR_INVALID_ARGUMENT;
  if (n > QF_MAX_QUBITS) return QF_ERR_TOO_LARGE;
  if (nedges < 0 || (nedges > 0 && (edges == nullptr || weights == nullptr))) return QF_ERR_INVALID_ARGUMENT;
  if (nedges > CUT_MAX_EDGES) return QF_ERR_TOO_LARGE;
  for (int i = 0; i < 2 * nedges; ++i)
    if (edges[i] < 0 || edges[i] >= n) return QF_ERR_INVALID_ARGUMENT;
  return cut_values_weighted(cuts, n, nedges, edges, weights, as_stream(stream));
}

int qf_qaoa_state(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p,
                  const double* beta, const double* gamma, const double* node_theta, int fusion_k,
                  void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (cuts == nullptr || p < 0 || nedges < 0) return QF_ERR_INVALID_ARGUMENT;
  if (p > 0 && (beta == nullptr || gamma == nullptr)) return QF_ERR_INVALID_ARGUMENT;
  if (nedges + 1 > 1024) return QF_ERR_TOO_LARGE;
  return qaoa_state(psi, n, st(layout), cuts, nedges, p, beta, gamma, node_theta, fusion_k,
                    as_stream(stream));
}

int qf_wave_min_qubits(int layout) {
  if (layout != QF_LAYOUT_C64 && layout != QF_LAYOUT_FF) return -QF_ERR_LAYOUT;
  return wave_min_qubits(layout);
}

int qf_wave_plan(const qf_batch_instance* instances, int ninstances, int layout, void* host_plan,
                 size_t host_bytes, size_t* host_bytes_needed, size_t* device_bytes_needed) {
  if (ninstances < 0 || (ninstances > 0 && instances == nullptr)) return QF_ERR_INVALID_ARGUMENT;
  if (host_plan == nullptr && host_bytes_needed == nullptr && device_bytes_needed == nullptr)
    return QF_ERR_INVALID_ARGUMENT;
  return wave_plan(instances, ninstances, layout, host_plan, host_bytes, host_bytes_needed, device_bytes_needed);
}

int qf_wave_prepare(const void* host_plan, const uint8_t* edges, void* workspace, size_t workspace_bytes,
                    void* stream) {
  if (host_plan == nullptr || edges == nullptr) return QF_ERR_INVALID_ARGUMENT;
  if (workspace == nullptr) return QF_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return QF_ERR_ALIGNMENT;
  return wave_prepare(host_plan, edges, workspace, workspace_bytes, as_stream(stream));
}

int qf_wave_qaoa_grad(const void* host_plan, void* workspace, size_t workspace_bytes, const double* angles,
                      double* out, const int32_t* skip, void* stream) {
  if (host_plan == nullptr || angles == nullptr || out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  if (workspace == nullptr) return QF_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return QF_ERR_ALIGNMENT;
  return wave_run(host_plan, workspace, workspace_bytes, angles, out, skip, as_stream(stream));
}

size_t qf_batch_workspace_bytes(int max_n, int layout, int ctas) {
  if (max_n < 1 || max_n > 26 || ctas < 1 || (layout != C64 && layout != FF)) return 0;
  return batch_workspace_bytes(max_n, layout, ctas);
}

int qf_batch_qaoa_grad(const qf_batch_instance* instances, int ninstances, int nlarge, const uint8_t* edges,
                       const double* angles, double* out, int layout, int max_n, int tile_bits, int ctas,
                       void* workspace, size_t workspace_bytes, void* stream) {
  if (layout != C64 && layout != FF) return QF_ERR_LAYOUT;
  if (ninstances < 0 || (ninstances > 0 && (instances == nullptr || angles == nullptr || out == nullptr)))
    return QF_ERR_INVALID_ARGUMENT;
  if (nlarge < 0 || nlarge > ninstances) return QF_ERR_INVALID_ARGUMENT;
  if (max_n < 1 || max_n > 26 || ctas < 8 || ctas > 65535 || ctas % 8 != 0) return QF_ERR_INVALID_ARGUMENT;
  const int ts_max = layout == C64 ? 12 : 11;
  if (tile_bits < 8 || tile_bits > ts_max || max_n > 2 * tile_bits) return QF_ERR_INVALID_ARGUMENT;
  int rc = check_ws(workspace, workspace_bytes, batch_workspace_bytes(max_n, layout, ctas));
  if (rc) return rc;
  if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return QF_ERR_ALIGNMENT;
  if (ninstances == 0) return QF_OK;
  return batch_qaoa(instances, ninstances, nlarge, edges, angles, out, layout, max_n, tile_bits, ctas, workspace,
                    workspace_bytes, as_stream(stream));
}

size_t qf_qaoa_grad_workspace_bytes(int n, int p, int layout) {
  if (n < 1 || n > QF_MAX_QUBITS || p < 0 || !valid_layout(layout)) return 0;
  return qaoa_grad_workspace_bytes(n, p, st(layout));
}

int qf_qaoa_expectation_grad(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p,
                             const double* beta, const double* gamma, const double* node_theta,
                             int fusion_k, double* out, void* workspace, size_t workspace_bytes,
                             void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (cuts == nullptr || out == nullptr || p < 0 || nedges < 0) return QF_ERR_INVALID_ARGUMENT;
  if (p > 0 && (beta == nullptr || gamma == nullptr)) return QF_ERR_INVALID_ARGUMENT;
  if (nedges + 1 > 1024 || 2 * p + 1 > 64) return QF_ERR_TOO_LARGE;
  layout = st(layout);
  rc = check_ws(workspace, workspace_bytes, qaoa_grad_workspace_bytes(n, p, layout));
  if (rc) return rc;
  if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return QF_ERR_ALIGNMENT;
  cudaStream_t s = as_stream(stream);
  rc = qaoa_state(psi, n, layout, cuts, nedges, p, beta, gamma, node_theta, fusion_k, s);
  if (rc) return rc;
  return qaoa_grad(psi, n, layout, cuts, nedges, p, beta, gamma, node_theta, out, workspace, s);
}

int qf_expectation_cuts(const void* psi, int n, int layout, const uint16_t* cuts, double* out,
                        void* workspace, size_t workspace_bytes, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (cuts == nullptr || out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  rc = check_ws(workspace, workspace_bytes, qf_reduce_workspace_bytes(n));
  if (rc) return rc;
  return reduce_diag(psi, n, st(layout), 1, cuts, nullptr, out, reinterpret_cast<double*>(workspace),
                     as_stream(stream));
}

int qf_expectation_diag(const void* psi, int n, int layout, const double* diag, double* out,
                        void* workspace, size_t workspace_bytes, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (diag == nullptr || out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  rc = check_ws(workspace, workspace_bytes, qf_reduce_workspace_bytes(n));
  if (rc) return rc;
  return reduce_diag(psi, n, st(layout), 2, nullptr, diag, out, reinterpret_cast<double*>(workspace),
                     as_stream(stream));
}

int qf_qubit_probabilities(const void* psi, int n, int layout, int axis, double* out, void* workspace,
                           size_t workspace_bytes, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (out == nullptr || axis < 0 || axis >= n) return QF_ERR_INVALID_ARGUMENT;
  rc = check_ws(workspace, workspace_bytes, qf_reduce_workspace_bytes(n));
  if (rc) return rc;
  return reduce_bit(psi, n, st(layout), n - 1 - axis, out, reinterpret_cast<double*>(workspace), as_stream(stream));
}

int qf_norm2(const void* psi, int n, int layout, double* out, void* workspace, size_t workspace_bytes,
             void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  rc = check_ws(workspace, workspace_bytes, qf_reduce_workspace_bytes(n));
  if (rc) return rc;
  return reduce_diag(psi, n, st(layout), 0, nullptr, nullptr, out, reinterpret_cast<double*>(workspace),
                     as_stream(stream));
}

int qf_inner(const void* a, const void* b, int n, int layout, double* out, void* workspace,
             size_t workspace_bytes, void* stream) {
  int rc = check_state(a, n, layout);
  if (rc) return rc;
  rc = check_state(b, n, layout);
  if (rc) return rc;
  if (out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  rc = check_ws(workspace, workspace_bytes, qf_reduce_workspace_bytes(n));
  if (rc) return rc;
  return reduce_inner(a, b, n, st(layout), out, reinterpret_cast<double*>(workspace), as_stream(stream));
}

int qf_probabilities(const void* psi, int n, int layout, double* probs, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (probs == nullptr) return QF_ERR_INVALID_ARGUMENT;
  return probabilities(psi, n, st(layout), probs, as_stream(stream));
}

int qf_sample(const void* psi, int n, int layout, int64_t trials, uint64_t seed, int64_t* counts,
              void* workspace, size_t workspace_bytes, void* stream) {
  int rc = check_state(psi, n, layout);
  if (rc) return rc;
  if (counts == nullptr || trials < 0) return QF_ERR_INVALID_ARGUMENT;
  rc = check_ws(workspace, workspace_bytes, sample_workspace_bytes(n));
  if (rc) return rc;
  return sample(psi, n, st(layout), trials, seed, counts, workspace, as_stream(stream));
}

}  // extern "C"
