/*
 * qf_gb300.h -- C ABI of the GB300 state-vector backend for QuantumFlow.
 *
 * Plain pointers and sizes only: device pointers are CUDA global-memory
 * addresses (any allocator), `stream` is a cudaStream_t (NULL = legacy default
 * stream).  Every entry point returns a status code (QF_OK = 0); none aborts,
 * traps or prints.  Calls are asynchronous on `stream` unless stated.
 *
 * Conventions shared with the reference (rigetti/quantumflow):
 *   - A state on n qubits is 2^n complex amplitudes in C order, i.e. the
 *     reference tensor of shape [2]*n flattened (quantumflow/qubits.py:63-84).
 *     Reference axis a lives at bit (n-1-a) of the flat index: axis 0 is the
 *     most significant bit.
 *   - Qubit arguments are AXIS indices in that convention (the `indices`
 *     argument of quantumflow/backend/numpybk.py:159 tensormul).
 *   - A k-qubit gate matrix is the reference gate tensor [2]*(2k) reshaped to
 *     (2^k, 2^k), row-major, gate qubit 0 the most significant bit of the row
 *     and column index (quantumflow/qubits.py:70-80), passed as interleaved
 *     (re, im) doubles: 2 * 4^k doubles.
 *
 * Element layouts (bytes per amplitude):
 *   QF_LAYOUT_C64   complex64  (float re, float im)                 8
 *   QF_LAYOUT_C128  complex128 (double re, double im), FP64 math   16
 *   QF_LAYOUT_FF    complex128 value held as float-float pairs
 *                   (re_hi, re_lo, im_hi, im_lo), 48-bit significand,
 *                   float-float math on the FP32 pipes            16
 *   QF_LAYOUT_FX    complex128 (double re, double im), the same bytes as
 *                   QF_LAYOUT_C128; gates computed in fixed point: fused
 *                   passes as 61-bit integer digits on the tensor cores
 *                   (qf_set_fx_tensor_cores), the rest in 64-bit integer
 *                   arithmetic on the CUDA cores (each amplitude group
 *                   shares one exponent, >= 55 significant bits relative
 *                   to the group's largest part, one FP64 rounding per
 *                   pass).  Unitary gates only take this arithmetic; other
 *                   gates, and every entry point other than qf_apply_gate /
 *                   qf_run_circuit / qf_plan_circuit, treat the buffer as
 *                   QF_LAYOUT_C128 (native FP64)                  16
 */
#ifndef QF_GB300_H
#define QF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QF_ABI_VERSION 1

#define QF_LAYOUT_C64 0
#define QF_LAYOUT_C128 1
#define QF_LAYOUT_FF 2
#define QF_LAYOUT_FX 3

#define QF_OK 0
#define QF_ERR_INVALID_ARGUMENT 1 /* bad qubit index, k, n, null pointer, ... */
#define QF_ERR_LAYOUT 2           /* unknown element layout                    */
#define QF_ERR_CUDA 3             /* a CUDA runtime call failed                 */
#define QF_ERR_ALIGNMENT 4        /* device pointer not 16-byte aligned         */
#define QF_ERR_TOO_LARGE 5        /* n above QF_MAX_QUBITS or table too large   */
#define QF_ERR_NOT_SUPPORTED 6    /* e.g. dense gate on more than 5 qubits      */
#define QF_ERR_DEVICE 7           /* a bounded device-side wait gave up         */
#define QF_ERR_WORKSPACE 8        /* workspace missing or too small             */

#define QF_MAX_QUBITS 34
#define QF_MAX_GATE_QUBITS 5
#define QF_MAX_DENSE_QUBITS 12

/* ------------------------------------------------------------ utilities -- */
int qf_abi_version(void);
const char* qf_status_string(int status);
/* cudaError_t of the most recent failing CUDA call made by this thread. */
int qf_last_cuda_error(void);
/* Read and clear the device error word (bit 0: a bounded wait gave up).
 * Synchronises `stream`. */
int qf_get_device_error(int* flags, void* stream);
/* Bytes of workspace the reductions below need for an n-qubit state. */
size_t qf_reduce_workspace_bytes(int n);

/* ------------------------------------------------- kernel timing ---------- */
/* Instrumentation with no counterpart in the reference (whose only timing is
 * timeit in tools/benchmark.py:48-53).  While enabled, every engine kernel
 * launched by qf_apply_gate / qf_run_circuit / qf_qaoa_state is bracketed by
 * a CUDA event pair on its launch stream.  qf_timing_collect synchronises on
 * the recorded events and returns, per kernel class, the summed milliseconds
 * and the launch count since the previous collect. */
#define QF_KERNEL_FUSED_TILE 0
#define QF_KERNEL_DENSE1 1
#define QF_KERNEL_DENSE2 2
#define QF_KERNEL_PERMUTATION 3
#define QF_KERNEL_ELEMENTWISE 4
#define QF_KERNEL_WARP_TILE 5
#define QF_KERNEL_GROUP 6
#define QF_KERNEL_SHAPE 7
#define QF_KERNEL_FX_DENSE1 8      /* fixed-point 2x2 sweep (QF_LAYOUT_FX)        */
#define QF_KERNEL_FX_DENSE2 9      /* fixed-point 4x4 sweep                       */
#define QF_KERNEL_FX_GROUP 10      /* fixed-point fused pass on a register group  */
#define QF_KERNEL_FX_ELEMENTWISE 11 /* fixed-point pass of element-wise ops only  */
#define QF_KERNEL_FX_SHAPE 12      /* fixed-point straight-line pass (1-2 gates)  */
#define QF_KERNEL_FX_TENSOR 13     /* complex128 pass on the tensor cores         */
#define QF_KERNEL_CLASSES 14
int qf_timing_enable(int on);
/* Fused-pass kernel selection (diagnostics and tests; no reference
 * counterpart), process-wide: 0 = default (float-float group passes --
 * every thread holding the amplitudes of a pass's <= 4 gate bits -- then
 * warp tiles, then shared-memory register programs, then the shared-memory
 * kernel, whichever first fits the block); 1 = shared-memory kernels only
 * (gate passes and the QAOA adjoint); 2, 3, 4 = no group passes, warp tiles
 * of 2^mode registers per thread (the adjoint's warp tiles take 2 or 3 for
 * complex128 and float-float, 3 or 4 for complex64, else their default);
 * 5 = default order without group passes. */
int qf_set_tile_kernel(int mode);
/* Widest float-float shape pass, in gate bits (0..4, default 3),
 * process-wide (tuning; no reference counterpart).  A fused pass of dense
 * gates and CZ-like signs is cut into straight-line shape kernels of at
 * most this many gate bits each; 0 = no shape passes (fused passes stay
 * whole and run the interpreted group or warp-tile kernels).  Complex64
 * passes that form one table shape (one or two dense gates on at most four
 * bits, with signs) run as shape kernels unless this is 0; they are never
 * cut. */
int qf_set_shape_bits(int bits);
/* Gate merging before pass planning (diagnostics and tests; no reference
 * counterpart), process-wide, whenever fusion_k > 1: 1 (default) =
 * consecutive gates are multiplied into blocks of at most two qubits on the
 * host; 2 = merging, then re-ordering within the gates' dependences to pack
 * each pass with as many gates as its high-bit budget allows; 0 = every
 * gate is applied as given. */
int qf_set_gate_merging(int on);
/* The pass plan qf_run_circuit would execute, without touching the GPU
 * (diagnostics; no reference counterpart).  For each planned pass, 8 ints
 * in stats[8*b ..]: ops, dense 1-qubit, dense 2-qubit, of those with a lane
 * bit (< 5), element-wise, other, high bits (>= 5), kernel (0 element-wise,
 * 1 direct single-gate sweep, 2 fused warp-tile or shared-memory pass,
 * 3 group pass, 4 shape pass, 5 one gate in native FP64 inside a
 * QF_LAYOUT_FX circuit, 6 tensor-core complex128 pass).  *nblocks gets the pass count; at most max_blocks
 * rows are written. */
int qf_plan_circuit(int n, int layout, int nops, const int* op_k, const int* op_axes, const double* op_mats,
                    int fusion_k, int32_t* stats, int max_blocks, int* nblocks);
int qf_timing_collect(double* ms, int64_t* launches, int nkinds);

/* ------------------------------------------------- state preparation ------ */
/* psi = |index> (quantumflow/states.py:186-191 zero_state for index 0). */
int qf_fill_basis(void* psi, int n, int layout, int64_t index, void* stream);
/* psi = |+>^n = H^n |0..0>, the state after the H layer of
 * quantumflow/qaoa.py:43-44. */
int qf_fill_uniform(void* psi, int n, int layout, void* stream);
/* Element-wise layout conversion (src and dst must not alias). */
int qf_convert(const void* src, int src_layout, void* dst, int dst_layout, int n, void* stream);
/* psi *= scale (real).  Used by State.normalize (quantumflow/states.py:108-111). */
int qf_scale(void* psi, int n, int layout, double scale, void* stream);

/* ------------------------------------------------- gate application ------- */
/* psi_out = gate (.) psi_in on the given axes.  Replaces
 * quantumflow/backend/numpybk.py:159-214 tensormul (called from
 * quantumflow/ops.py:161-166 Gate.run).  psi_out may equal psi_in (in place).
 * k = 1..QF_MAX_GATE_QUBITS, matrix = 2*4^k interleaved doubles (host). */
int qf_apply_gate(const void* psi_in, void* psi_out, int n, int layout, int k, const int* axes,
                  const double* matrix, void* stream);

/* psi_out = gate (.) psi_in for a dense gate on k = 1..QF_MAX_DENSE_QUBITS
 * axes whose matrix is in DEVICE memory (2 * 4^k interleaved doubles,
 * row-major, the convention of qf_apply_gate; 16-byte aligned).  Replaces
 * quantumflow/backend/numpybk.py:159-214 tensormul for gates wider than
 * qf_apply_gate takes (Gate.__matmul__, quantumflow/ops.py:187-198;
 * Circuit.asgate, quantumflow/circuits.py:111-118).  psi_out may equal
 * psi_in.  complex64 computes in FP32, the complex128 layouts in FP64 (a
 * float-float state is converted to complex128 in psi_out and back). */
int qf_apply_dense_gate(const void* psi_in, void* psi_out, int n, int layout, int k, const int* axes,
                        const double* matrix, void* stream);
/* Dense complex64 gates on 5 or 6 qubits (n >= k + 7) run on the tensor
 * cores (tcgen05 MMAs, TF32 operands split into hi + lo parts, FP32
 * accumulation) unless this is 0 (then the CUDA-core kernel); default 1.
 * Process-wide; diagnostics and tests, no reference counterpart. */
int qf_set_dense_tensor_cores(int on);
/* Fixed-point (QF_LAYOUT_FX) straight-line passes on 3 and 4 gate bits:
 * compile them for at least min_blocks resident CTAs of 128 threads per SM
 * (1..4; the register cap trades per-thread registers for warps), states of
 * at most 2^31 amplitudes.  Process-wide tuning, no reference counterpart. */
int qf_set_fx_occupancy(int min_blocks);
/* Complex128 (QF_LAYOUT_FX) fused passes on the tensor cores (default 1):
 * a pass of unitary gates on at most four bits, with CZ-like signs around
 * them, or one unitary gate on 3 or 4 qubits, runs as one 16 x 16 unitary
 * applied by fp16 tcgen05 MMAs to base-256 integer digits of a 61-bit
 * fixed-point form of each row of 16 amplitudes (exact FP32 accumulation,
 * one FP64 rounding per pass; states of at least 2^11 amplitudes); 0 = the
 * CUDA-core fixed-point kernels (3- and 4-qubit gates in native FP64).
 * Process-wide; no reference counterpart. */
int qf_set_fx_tensor_cores(int on);

/* Apply nops gates in order with gate fusion.  Replaces the per-gate loop of
 * quantumflow/circuits.py:87-99 Circuit.run.  Gate i acts on op_k[i] axes
 * taken consecutively from op_axes; its matrix is the next 2*4^k doubles of
 * op_mats (host arrays).  fusion_k = maximum number of non-contiguous high
 * qubits per fused pass (0 = library default, 1 = no fusion).  *passes (may
 * be NULL) receives the number of full-state passes launched. */
int qf_run_circuit(const void* psi_in, void* psi_out, int n, int layout, int nops, const int* op_k,
                   const int* op_axes, const double* op_mats, int fusion_k, int* passes,
                   void* stream);

/* ------------------------------------------------------------- QAOA ------- */
/* cuts[x] = number of edges cut by basis state x (unweighted graph),
 * the table quantumflow/qaoa.py:68-81 graph_cuts builds in Python.
 * edges = 2*nedges axis indices (device-independent host array). */
int qf_cut_values(uint16_t* cuts, int n, int nedges, const int* edges, void* stream);
/* Weighted variant: cuts[x] = sum of weights of cut edges (double). */
int qf_cut_values_weighted(double* cuts, int n, int nedges, const int* edges, const double* weights,
                           void* stream);

/* The QAOA state of quantumflow/qaoa.py:22-64 qubo_circuit for an
 * unweighted graph given its cut table: |+>^n, then for each of p steps the
 * cost layer prod_e ZZ(-gamma/pi) = exp(i*gamma*(E/2 - C(x))) as one
 * diagonal-phase pass, RZ(node_theta[q]) on nodes whose theta is not NaN
 * (node_theta may be NULL), then RX(beta) on every node.  nedges = E. */
int qf_qaoa_state(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p,
                  const double* beta, const double* gamma, const double* node_theta, int fusion_k,
                  void* stream);

/* <C> and its gradient by the adjoint method: the forward state is built in
 * psi (state-sized device buffer, left at |+>^n on return), lambda = C psi,
 * then every layer is undone in reverse on both vectors while
 *   d<C>/d beta_l  = sum_j Im <lambda|X_j|psi>          (after the mixer)
 *   d<C>/d gamma_l = -2 Im <lambda|(E/2 - C)|psi>       (after the cost layer)
 * accumulate.  Two state vectors regardless of p.  out (device, 2p+1
 * doubles): out[0..p) = d/d gamma, out[p..2p) = d/d beta, out[2p] = <C>.
 * Workspace: qf_qaoa_grad_workspace_bytes(n, p, layout), 256-byte aligned.
 * The reference differentiates only through TensorFlow
 * (examples/qaoa_maxcut.py:56-64, quantumflow/backend/tensorflowbk.py). */
size_t qf_qaoa_grad_workspace_bytes(int n, int p, int layout);
int qf_qaoa_expectation_grad(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p,
                             const double* beta, const double* gamma, const double* node_theta,
                             int fusion_k, double* out, void* workspace, size_t workspace_bytes,
                             void* stream);

/* ------------------------------------------------- batched QAOA ---------- */
/* Many independent QAOA MAXCUT instances (uneven n, graphs, depths) in one
 * persistent launch: forward <C> and its adjoint gradient per instance.  No
 * reference counterpart (the reference evaluates one circuit at a time,
 * quantumflow/qaoa.py:22-81, examples/qaoa_maxcut.py:37-87).  All pointers
 * are device pointers; the launch is asynchronous and contains only device
 * work (a counter reset and one kernel), so it can be captured in a CUDA
 * graph and replayed after the angles are updated in place. */
typedef struct qf_batch_instance {
  int32_t n;            /* qubits, 1..max_n (and <= 2*tile_bits)              */
  int32_t p;            /* QAOA layers, 0..64                                 */
  int32_t nedges;       /* unweighted edges, 0..1023                          */
  int32_t edge_offset;  /* first edge: axis pairs at edges[2*edge_offset]     */
  int32_t angle_offset; /* beta[p] then gamma[p] at angles[angle_offset]      */
  int32_t out_offset;   /* d/dgamma[p], d/dbeta[p], <C> at out[out_offset]    */
} qf_batch_instance;
/* Workspace for `ctas` persistent CTAs and instances of up to max_n qubits. */
size_t qf_batch_workspace_bytes(int max_n, int layout, int ctas);
/* layout QF_LAYOUT_C64 or QF_LAYOUT_FF; tile_bits 8..12 (C64) / 8..11 (FF):
 * instances with n <= tile_bits stay in shared memory.  The first nlarge
 * instances are each processed by a cluster of 8 CTAs (hardware cluster
 * barriers between passes); the rest by one CTA each.  ctas must be a
 * multiple of 8.  Order instances largest first within each group.  A
 * malformed instance gets NaN outputs and raises bit 1 of the device error
 * word. */
int qf_batch_qaoa_grad(const qf_batch_instance* instances, int ninstances, int nlarge, const uint8_t* edges,
                       const double* angles, double* out, int layout, int max_n, int tile_bits, int ctas,
                       void* workspace, size_t workspace_bytes, void* stream);

/* Multi-instance passes for the batch instances too large for one CTA's
 * shared memory (no reference counterpart: the reference evaluates one
 * circuit at a time, quantumflow/qaoa.py:22-81).  Each instance keeps psi,
 * lambda and its cut table in the caller's device workspace; wave w runs
 * pass w of every instance (forward and adjoint warp-tile passes), so the
 * launch count is the longest instance's pass count.
 *   qf_wave_min_qubits: smallest n accepted for `layout` (C64 or FF).
 *   qf_wave_plan: `instances` is a HOST array (same fields as for
 *     qf_batch_qaoa_grad; p >= 1, nedges <= 1023).  With host_plan == NULL
 *     it only reports the host and device bytes needed; otherwise it writes
 *     the plan into host_plan, which must stay unchanged while it is used.
 *   qf_wave_prepare: uploads the plan into the device workspace (256-byte
 *     aligned) and computes the cut tables from the device edge array;
 *     once per plan, before any stream capture.
 *   qf_wave_qaoa_grad: one evaluation: out gets, per instance,
 *     dgamma[p], dbeta[p], <C> at out_offset, from the device angle array.
 *     skip: NULL, or a DEVICE array of one int32 per planned instance (plan
 *     order); a nonzero entry leaves that instance out of the evaluation and
 *     its outputs at their values from its last evaluation (an optimiser
 *     that stops instances at a target ratio).  No host synchronisation; may
 *     be captured in a CUDA graph. */
int qf_wave_min_qubits(int layout);
int qf_wave_plan(const qf_batch_instance* instances, int ninstances, int layout, void* host_plan,
                 size_t host_bytes, size_t* host_bytes_needed, size_t* device_bytes_needed);
int qf_wave_prepare(const void* host_plan, const uint8_t* edges, void* workspace, size_t workspace_bytes,
                    void* stream);
int qf_wave_qaoa_grad(const void* host_plan, void* workspace, size_t workspace_bytes, const double* angles,
                      double* out, const int32_t* skip, void* stream);

/* ------------------------------------------ learned angle initialiser ----- */
/* A 3-layer message-passing graph network (hidden width 64, FP32) mapping a
 * graph to 2p QAOA angles (beta_0..beta_{p-1}, gamma_0..gamma_{p-1}); no
 * reference counterpart (the reference draws initial angles at random,
 * examples/qaoa_maxcut.py:47-51).  Graph batches are CSR on the device:
 * graph g owns nodes [node_offset[g], node_offset[g+1]) (1..32 nodes), node
 * i's neighbours are adj[adj_offset[i] .. adj_offset[i+1]) (global node ids,
 * both directions listed).  params holds qf_gnn_param_count(p) floats. */
#define QF_GNN_HIDDEN 64
#define QF_GNN_MAX_NODES 32
size_t qf_gnn_param_count(int p);
/* Activation buffer size (floats) for the backward pass. */
size_t qf_gnn_activation_floats(int total_nodes, int ngraphs);
/* out[g][2p] = network(graph g); activations may be NULL (inference). */
int qf_gnn_forward(const float* params, int p, int ngraphs, int total_nodes, const int32_t* node_offset,
                   const int32_t* adj_offset, const int32_t* adj, float* out, float* activations, void* stream);
/* grad += d/dparams of mean((out - target)^2) over the batch (grad must be
 * zeroed by the caller before the first batch); loss += sum (out-target)^2. */
int qf_gnn_backward(const float* params, int p, int ngraphs, int total_nodes, const int32_t* node_offset,
                    const int32_t* adj_offset, const int32_t* adj, const float* out, const float* target,
                    const float* activations, float* grad, float* loss, void* stream);
/* One Adam step (Kingma & Ba 2015) on count floats; step counts from 1. */
int qf_adam_update(float* params, const float* grad, float* m, float* v, int count, float lr, float beta1,
                   float beta2, float eps, int step, void* stream);

/* ------------------------------------------------------- reductions ------- */
/* All reductions write their result to DEVICE memory `out` and need a
 * workspace of qf_reduce_workspace_bytes(n) bytes (device, 256-byte aligned).
 * Results are deterministic (fixed-order two-pass reduction). */

/* out[0] = sum_x cuts[x] |psi_x|^2 -- State.expectation
 * (quantumflow/states.py:131-147) with the diagonal of graph_cuts. */
int qf_expectation_cuts(const void* psi, int n, int layout, const uint16_t* cuts, double* out,
                        void* workspace, size_t workspace_bytes, void* stream);
/* Allocation-free variant of qf_expectation_cuts (same result, same
 * arguments minus the workspace).  No counterpart in the reference.  It is
 * for callers that cannot allocate or hand over device workspace -- e.g. a
 * host whose memory pool owns the whole GPU, or a loop that must not call
 * cudaMalloc because it can synchronise the device.  The partial sums live
 * in a fixed array compiled into the library: QF_NOALLOC_MAX_PARTIALS block
 * partials (32 KiB per GPU, held until exit), enough for every n up to
 * QF_MAX_QUBITS (larger n: QF_ERR_TOO_LARGE).  All calls share that array,
 * so calls whose kernels overlap on the GPU race; serialise them.  A call
 * whose stream is not capturing looks up the array's device address with
 * the calling device current (so the address survives a device reset); a
 * call made during stream capture reuses the last address found on that
 * device, so make one call per device before any stream capture. */
#define QF_NOALLOC_MAX_PARTIALS 2048
int qf_expectation_cuts_noalloc(const void* psi, int n, int layout, const uint16_t* cuts, double* out,
                                void* stream);
/* out[0] = sum_x diag[x] |psi_x|^2 for a real device array diag[2^n]. */
int qf_expectation_diag(const void* psi, int n, int layout, const double* diag, double* out,
                        void* workspace, size_t workspace_bytes, void* stream);
/* out[0] = probability that the qubit on reference axis `axis` reads 0,
 * out[1] = that it reads 1 (unnormalised: their sum is the squared norm).
 * Replaces the projected copy + norm of Measure.run,
 * quantumflow/stdops.py:53-54 (prob_zero = P0(qubit).run(ket).norm()). */
int qf_qubit_probabilities(const void* psi, int n, int layout, int axis, double* out, void* workspace,
                           size_t workspace_bytes, void* stream);
/* out[0] = sum_x |psi_x|^2 (quantumflow/qubits.py:180-182 norm). */
int qf_norm2(const void* psi, int n, int layout, double* out, void* workspace,
             size_t workspace_bytes, void* stream);
/* out[0..1] = (re, im) of <a|b> = sum_x conj(a_x) b_x
 * (quantumflow/backend/numpybk.py:125-128 inner). */
int qf_inner(const void* a, const void* b, int n, int layout, double* out, void* workspace,
             size_t workspace_bytes, void* stream);
/* probs[x] = |psi_x|^2 as double (quantumflow/states.py:113-119). */
int qf_probabilities(const void* psi, int n, int layout, double* probs, void* stream);
/* Multinomial sampling, quantumflow/states.py:121-129 State.sample:
 * counts[x] (int64, device, 2^n, zeroed by the call) = number of the
 * `trials` draws that gave x.  Draws use a counter-based generator keyed by
 * `seed`.  Needs qf_sample_workspace_bytes(n) of workspace. */
size_t qf_sample_workspace_bytes(int n);
int qf_sample(const void* psi, int n, int layout, int64_t trials, uint64_t seed, int64_t* counts,
              void* workspace, size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QF_GB300_H */
