// Declarations of the state-level helpers in state.cu and qaoa.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace qf {

constexpr int REDUCE_MAX_BLOCKS = 2048;
constexpr int CUT_MAX_EDGES = 2048;

int fill_basis(void* psi, int n, int layout, int64_t index, cudaStream_t stream);
int fill_uniform(void* psi, int n, int layout, cudaStream_t stream);
int convert(const void* src, int sl, void* dst, int dl, int n, cudaStream_t stream);
int scale(void* psi, int n, int layout, double s, cudaStream_t stream);

int reduce_blocks(int64_t namps);
// kind 0: norm2, 1: uint16 cuts, 2: double diagonal
int reduce_diag(const void* psi, int n, int layout, int kind, const uint16_t* cuts, const double* diag,
                double* out, double* partials, cudaStream_t stream);
int reduce_bit(const void* psi, int n, int layout, int bit, double* out, double* partials, cudaStream_t stream);
int reduce_inner(const void* a, const void* b, int n, int layout, double* out, double* partials,
                 cudaStream_t stream);
int probabilities(const void* psi, int n, int layout, double* probs, cudaStream_t stream);
size_t sample_workspace_bytes(int n);
int sample(const void* psi, int n, int layout, int64_t trials, uint64_t seed, int64_t* counts, void* ws,
           cudaStream_t stream);
int cut_values(uint16_t* cuts, int n, int nedges, const int* edges, cudaStream_t stream);
int cut_values_weighted(double* cuts, int n, int nedges, const int* edges, const double* w,
                        cudaStream_t stream);

}  // namespace qf
