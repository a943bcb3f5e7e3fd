// Host+device interface of the gate engine shared by the .cu files.
#pragma once
#include <cstdint>
#include <complex>
#include <vector>
#include <cuda_runtime.h>
#include "qf_common.cuh"
#include "qf_gb300.h"

namespace qf {

using cplx = std::complex<double>;

// ---------------------------------------------------------- op classes ----
enum OpType : uint8_t {
  OP_DENSE1 = 1,  // 2x2 on one in-tile bit
  OP_DENSE2 = 2,  // 4x4 on two in-tile bits
  OP_DENSEK = 3,  // 2^k x 2^k (k = 3..5) on in-tile bits, warp per group
  OP_MONO = 4,    // generalised permutation on k<=3 in-tile bits
  OP_DIAG = 5,    // diagonal on k<=3 bits anywhere (elementwise)
  OP_SIGN = 6,    // -1 where all k bits are set (CZ, CCZ); elementwise
  OP_CUT = 7,     // psi_x *= table[cut[x]]  (QAOA cost layer); elementwise
  OP_PHASE = 8,   // psi_x *= c (global scalar); elementwise
};

constexpr int TILE_MAX_OPS = 96;
constexpr int TILE_MAX_COEF = 1152;
constexpr int KMAX_DENSE = 5;

struct TileOp {
  uint8_t type;
  uint8_t k;
  uint8_t lb[5];    // local (tile) bit positions, matrix MSB first
  uint8_t slb[5];   // the same, sorted ascending (group enumeration)
  uint8_t gb[3];    // global bit positions (elementwise ops), MSB first
  uint8_t perm[8];  // OP_MONO: source row for each output row
  uint16_t coef;    // index of first coefficient
  uint16_t ncoef;   // number of coefficients (OP_CUT: table size, index clamp)
};

// Register-resident tile program (k_tile2).  Each of the 256 threads owns
// 2^RB amplitudes of the 2^(RB+8)-amplitude tile: local bits 0..4 are the
// lane index, RB local bits index the thread's registers and 3 index the
// warp, as given by the current TMap.  Gates on register bits run in
// registers, gates on lane bits through warp shuffles; a MAP instruction
// re-distributes the tile through shared memory.
enum TInstrCode : uint8_t {
  I_MAP = 1,   // a: map index; (re)load registers under that bit map
  I_G1R = 2,   // a: register bit; coef: 4 coefficients
  I_G1L = 3,   // a: lane bit; coef: 4 coefficients
  I_G2R = 4,   // a: register bit of the matrix MSB, b: of the LSB; 16 coefs
  I_SEG = 5,   // a: first SegOp, b: count (element-wise ops in registers)
  I_SMEM = 6,  // a: index into ops[] -- applied in shared memory
  I_RSWAP = 7, // a, b: exchange register-index bits a and b (k_warp)
  I_LSWAP = 8, // a: lane bit, b: register-index bit; exchange the global bits they hold (k_warp)
};
struct TInstr {
  uint8_t code, a, b, c;
  uint16_t coef;
  uint16_t pad;
};
struct TMap {
  uint8_t rpos[4];  // local bit of register-index bit j
  uint8_t wpos[3];  // local bit of warp-index bit i
  uint8_t pad0;
  uint8_t rglob[4];  // global bit positions of the same bits
  uint8_t wglob[3];
  uint8_t pad1;
};
struct SegOp {
  uint8_t type, k;
  uint8_t gb[3];
  uint8_t pad[3];
  uint16_t coef, ncoef;  // into the element-wise coefficient table
  // OP_SIGN in warp-tile programs, resolved by the host against the
  // sub-tile layout at the op's program point: rmask = the registers whose
  // index has every register bit of the op set, lmask = the lane bits that
  // hold op bits, tmask = the op bits in the sub-tile base
  uint16_t rmask;
  uint8_t lmask, pad2;
  uint64_t mask;  // OP_SIGN: the k global bits
  uint64_t tmask;
};
// Warp-tile programs (k_warp): a sub-tile is 32 lanes (global bits 0..4)
// x 2^RB registers (the block's RB high bits hb[]), streamed straight from
// global memory; warps never synchronise with each other.
struct WarpParams {
  const void* in;
  void* out;
  const uint16_t* cuts;
  int32_t n, rb, nprog, necoef;
  uint8_t hb[4];  // global bits indexing the registers, ascending
  TInstr prog[160];
  SegOp segs[64];
  Coef coef[1152];
};

constexpr int TILE_MAX_PROG = 160;
constexpr int TILE_MAX_MAPS = 48;
constexpr int TILE_MAX_SEGS = 64;

struct TileParams {
  const void* in;
  void* out;
  const uint16_t* cuts;  // OP_CUT source (device), may be null
  int32_t n;             // qubits
  int32_t L;             // contiguous low bits in a tile
  int32_t nh;            // extra high tile bits
  int32_t nops;
  int32_t threads;
  int32_t nprog;         // k_tile2 program length (0: use k_tile)
  int32_t necoef;        // element-wise coefficients at coef[0, necoef)
  uint8_t hb[8];         // high tile bits (global positions), ascending
  TileOp ops[TILE_MAX_OPS];
  TInstr prog[TILE_MAX_PROG];
  TMap maps[TILE_MAX_MAPS];
  SegOp segs[TILE_MAX_SEGS];
  Coef coef[TILE_MAX_COEF];
};

// A host-side classified op (one gate).
struct HostOp {
  int k = 0;
  int gb[KMAX_DENSE] = {0, 0, 0, 0, 0};  // global bit positions, matrix MSB first
  uint8_t type = 0;
  std::vector<cplx> m;        // dense: row-major 2^k x 2^k
  std::vector<cplx> diag;     // OP_DIAG / OP_MONO phases (per output row)
  int perm[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  const uint16_t* cuts = nullptr;  // OP_CUT
  std::vector<cplx> table;         // OP_CUT phase per cut value
  cplx scalar{1.0, 0.0};           // OP_PHASE
};

// Fill one coefficient in the arithmetic of `layout`.
inline Coef make_coef(cplx v, int layout) {
  Coef c;
  c.d[0] = 0.0;
  c.d[1] = 0.0;
  if (layout == C128) {
    c.d[0] = v.real();
    c.d[1] = v.imag();
  } else if (layout == FF) {
    float rh = static_cast<float>(v.real());
    float rl = static_cast<float>(v.real() - static_cast<double>(rh));
    float ih = static_cast<float>(v.imag());
    float il = static_cast<float>(v.imag() - static_cast<double>(ih));
    c.f[0] = rh;
    c.f[1] = rl;
    c.f[2] = ih;
    c.f[3] = il;
  } else {
    c.f[0] = static_cast<float>(v.real());
    c.f[1] = 0.f;
    c.f[2] = static_cast<float>(v.imag());
    c.f[3] = 0.f;
  }
  return c;
}

inline size_t elem_bytes(int layout) { return layout == C64 ? 8 : 16; }

// Classify a k-qubit matrix into DIAG / SIGN / MONO / DENSE and fill HostOp.
// Returns QF_OK or an error status.
int classify_op(int k, const int* gbits, const double* mat_interleaved, HostOp& op);

// Plan + launch a sequence of ops on one state (in -> out, may alias).
int run_ops(const void* in, void* out, int n, int layout, std::vector<HostOp>& ops, int fusion_k,
            cudaStream_t stream, int* passes_out);

// Launch helpers used by other translation units.
int launch_tile_block(const void* in, void* out, int n, int layout, const std::vector<HostOp>& ops,
                      const std::vector<int>& idx, uint64_t hmask, cudaStream_t stream);
int launch_single(const void* in, void* out, int n, int layout, const HostOp& op, cudaStream_t stream);

// Group passes (k_group, float-float layout): a fused pass whose dense
// gates touch at most four bits.  Every thread holds the 2^G amplitudes
// that differ only in those G bits (register-index bit j = global bit
// rbits[j]), applies the pass's ops to them in order and writes them back;
// sign ops (CZ-like) become one per-thread register mask, applied before
// the next dense gate.
constexpr int GROUP_MAX_OPS = 96;
constexpr int GROUP_MAX_COEF = 512;
struct GroupOp {
  uint8_t type;    // OP_DENSE1 / OP_DENSE2 / OP_SIGN / OP_DIAG / OP_PHASE
  uint8_t a, b;    // dense: register-index bits (DENSE2: a = matrix MSB, a > b)
  uint8_t flag;    // DENSE2: every coefficient part nonzero; DIAG: k
  uint8_t flush;   // dense: apply the pending sign mask first
  uint8_t gb[3];   // DIAG: global bits, matrix MSB first
  uint16_t coef;   // first coefficient
  uint16_t rmask;  // SIGN: registers whose group bits of the op are all set
  uint32_t pad;
  uint64_t mout;   // SIGN: the op's global bits outside the group
};
struct GroupParams {
  const void* in;
  void* out;
  int32_t n, nops;
  int32_t final_flush, pad;
  uint8_t rbits[4];  // global bit of register-index bit j
  uint8_t sbits[4];  // the same bits, ascending
  int64_t off[16];   // global offset of register index r
  GroupOp ops[GROUP_MAX_OPS];
  Coef coef[GROUP_MAX_COEF];
};
// Fill P for the pass ops[idx] and return QF_OK with its group size G, or
// QF_ERR_NOT_SUPPORTED when the pass does not fit a group kernel.
int group_prepare(int n, int layout, const std::vector<HostOp>& ops, const std::vector<int>& idx,
                  GroupParams& P, int& G);
int group_launch(const GroupParams& P, int G, cudaStream_t stream);

// Shape passes (k_shape, float-float and complex64 layouts): the
// straight-line form of a group pass for the common programs -- one or two
// dense gates (slots) on fixed register bits, with sign ops (CZ-like)
// between and around them as per-thread register masks.  The host renames
// the pass's gate bits to register bits in order of first use (top first),
// which maps every program of the table in group.cu to one compiled kernel.
constexpr int SHAPE_MAX_SIGNS = 64;
struct ShapeParams {
  const void* in;
  void* out;
  int32_t n, shape;
  int32_t sign_end[3];  // signs [sign_end[b-1], sign_end[b]) act before slot b (b = 2: after the last)
  int32_t layout;       // FF or C64
  uint8_t sbits[4];     // the group bits, ascending
  uint8_t dense[2];     // slot s: every coefficient part nonzero
  uint8_t pad2[2];
  int64_t off[16];      // global offset of register index r
  uint16_t rmask[SHAPE_MAX_SIGNS];
  uint64_t mout[SHAPE_MAX_SIGNS];
  Coef coef[32];        // slot s at coef[16 s]
};
// Which table shape of at most max_bits gate bits the dense ops
// ops[dense[0..nd)] form (-1: none); the planner splits fused float-float
// and complex64 passes at the points where the next dense gate would leave
// the table.
int shape_of(const std::vector<HostOp>& ops, const int* dense, int nd, int max_bits);
// Widest shape in gate bits for a layout (0: no shape passes).
int shape_max_bits(int layout);
// The table shape of ops[dense[0..nd)] whatever the width limit: returns its
// index (or -1), the bits in order of first use (order[0] is register bit
// G-1), G, which 4x4 slots have their matrix MSB on the lower register bit
// (swap[]), and the slot codes.
int shape_lookup(const std::vector<HostOp>& ops, const int* dense, int nd, int* order, int& G, bool* swap,
                 int* s0, int* s1);
// Fill P for the pass ops[idx] (dense gates and sign ops only) and launch
// it; QF_ERR_NOT_SUPPORTED when it is not a table shape.
int shape_prepare(int n, int layout, const std::vector<HostOp>& ops, const std::vector<int>& idx,
                  ShapeParams& P);
int shape_launch(const ShapeParams& P, cudaStream_t stream);
extern int g_shape_max_bits;  // qf_set_shape_bits (0: no shape passes, blocks stay whole)

// While qf_timing_enable is on, a CUDA event pair brackets the launches made
// during this object's lifetime on `stream`, summed under kernel class `kind`.
struct LaunchTimer {
  bool on = false;
  int kind = 0;
  cudaEvent_t start = nullptr, stop = nullptr;
  cudaStream_t s = nullptr;
  LaunchTimer(int kind, cudaStream_t stream);
  ~LaunchTimer();
  LaunchTimer(const LaunchTimer&) = delete;
  LaunchTimer& operator=(const LaunchTimer&) = delete;
};

// Consecutive gates multiplied into blocks of at most two qubits (host).
void merge_ops(std::vector<HostOp>& ops, int n);
extern int g_merge_gates;

// Passes of complex128 states in 64-bit integer fixed-point arithmetic
// (fxengine.cu); ops the fixed-point kernels do not take run in native FP64.
int fx_run_ops(const void* in, void* out, int n, std::vector<HostOp>& ops, int fusion_k, cudaStream_t stream,
               int* passes_out);
int fx_plan_stats(int n, std::vector<HostOp>& ops, int fusion_k, int32_t* stats, int max_blocks, int* nblocks);

// Tensor-core complex128 passes (tcfx.cu): the unitary U (16 x 16) of a run
// of gates and window sign ops on four window bits, applied to every row of
// 16 amplitudes in an integer-digit fixed-point arithmetic on fp16 MMAs.
// Sign ops with bits outside the window run on the inputs (before every
// dense gate on their window bits) or on the outputs.
constexpr int TX_MAX_SIGNS = 48;
struct TxParams {
  const void* in;
  void* out;
  int* err;
  int32_t n, nin, nout, pad;
  int32_t sbits[4];                 // window bits, ascending
  int64_t off[16];                  // global offset of window index c
  int64_t g[16][16][2];             // U as round(entry * 2^62): [out c][in c][re, im]
  uint64_t in_mout[TX_MAX_SIGNS];   // input-side sign ops: their bits outside the window
  uint64_t out_mout[TX_MAX_SIGNS];  // output-side sign ops
  uint16_t in_rmask[TX_MAX_SIGNS];  // window indices c that carry all of the op's window bits
  uint16_t out_rmask[TX_MAX_SIGNS];
};
int tx_launch(const TxParams& P, cudaStream_t stream);
extern int g_fx_tensor;  // qf_set_fx_tensor_cores (1: tensor-core passes where they apply)

int device_sm_count();
int timing_enable(int on);
int timing_collect(double* ms, int64_t* counts, int nkinds);
int check_cuda(cudaError_t e);

}  // namespace qf
