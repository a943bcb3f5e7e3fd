// Learned QAOA angle initialiser: a message-passing graph network that maps
// a MAXCUT graph to 2p angles (beta_0..beta_{p-1}, gamma_0..gamma_{p-1}).
// No reference counterpart: the reference initialises angles at random
// (examples/qaoa_maxcut.py:47-51).
//
// Architecture (FP32, hidden width H = 64):
//   x_v   = [1, deg_v / 8, n / 16]
//   h0_v  = relu(W0 x_v + b0)
//   a_v   = mean_{u in N(v)} h_{l-1,u}          (0 for isolated nodes)
//   h_l,v = relu(Ws_l h_{l-1,v} + Wn_l a_v + b_l),   l = 1, 2, 3
//   g     = mean_v h_3,v
//   r     = relu(Wr g + br)
//   out   = Wo r + bo                            (2p values)
// One CTA per graph (n <= 32).  Forward keeps every activation in a caller
// buffer so the backward kernel can form the exact gradient of the mean
// squared error; each CTA sums a weight's gradient over its graph's nodes
// and adds it to the caller's gradient buffer with one atomic per weight.
#include <cmath>
#include <cstring>

#include "engine.cuh"

namespace qf {

constexpr int GH = QF_GNN_HIDDEN;
constexpr int GMAXN = QF_GNN_MAX_NODES;
constexpr int GLAYERS = 3;
constexpr int GTHREADS = 256;

// parameter block offsets (floats)
struct GnnLayout {
  int p, nout;
  int W0, b0, Ws[GLAYERS], Wn[GLAYERS], bl[GLAYERS], Wr, br, Wo, bo, total;
  __host__ __device__ explicit GnnLayout(int p_) : p(p_), nout(2 * p_) {
    int o = 0;
    W0 = o; o += GH * 3;
    b0 = o; o += GH;
    for (int l = 0; l < GLAYERS; ++l) {
      Ws[l] = o; o += GH * GH;
      Wn[l] = o; o += GH * GH;
      bl[l] = o; o += GH;
    }
    Wr = o; o += GH * GH;
    br = o; o += GH;
    Wo = o; o += nout * GH;
    bo = o; o += nout;
    total = o;
  }
};

// activations per node: h0..h3 then a1..a3 (7 x H); per graph: g, r (2 x H)
constexpr int GACT_NODE = 7 * GH;
constexpr int GACT_GRAPH = 2 * GH;

struct GnnArgs {
  const float* params;
  int p;
  int ngraphs;
  const int32_t* node_offset;  // [ngraphs + 1]
  const int32_t* adj_offset;   // [total_nodes + 1]
  const int32_t* adj;          // neighbour global node ids
  float* out;                  // [ngraphs][2p]
  float* acts;                 // activations, may be null for inference
  const float* target;         // backward: labels [ngraphs][2p]
  float* grad;                 // backward: accumulated parameter gradient
  float* loss;                 // backward: accumulated sum of squared errors
  int total_nodes;
};

// y[v][j] = act(sum_k A[j][k] x[v][k] + B[j][k] x2[v][k] + bias[j]) for nv
// rows; AT, BT hold the matrices transposed (AT[k][j]) so the 32 lanes of a
// warp (consecutive j) read consecutive banks.
__device__ void dense_rows(const float* __restrict__ AT, const float* __restrict__ xin, const float* __restrict__ BT,
                           const float* __restrict__ xin2, const float* __restrict__ bias, float* y, int nv,
                           bool relu_on) {
  for (int t = threadIdx.x; t < nv * GH; t += blockDim.x) {
    const int v = t / GH, j = t % GH;
    float s = bias[j];
    const float* x = xin + v * GH;
#pragma unroll 8
    for (int k = 0; k < GH; ++k) s = fmaf(AT[k * GH + j], x[k], s);
    if (BT != nullptr) {
      const float* x2 = xin2 + v * GH;
#pragma unroll 8
      for (int k = 0; k < GH; ++k) s = fmaf(BT[k * GH + j], x2[k], s);
    }
    y[t] = relu_on ? fmaxf(s, 0.f) : s;
  }
}

__global__ void __launch_bounds__(GTHREADS) k_gnn_forward(const __grid_constant__ GnnArgs A) {
  const GnnLayout L(A.p);
  extern __shared__ __align__(16) float gsm[];
  float* Wa = gsm;                   // GH*GH
  float* Wb = Wa + GH * GH;          // GH*GH
  float* hs = Wb + GH * GH;          // GMAXN*GH  (h_{l-1})
  float* as = hs + GMAXN * GH;       // GMAXN*GH  (a_l)
  float* hn = as + GMAXN * GH;       // GMAXN*GH  (h_l)
  float* vec = hn + GMAXN * GH;      // 4*GH
  __shared__ int s_deg[GMAXN];
  const int g = blockIdx.x;
  const int v0 = A.node_offset[g], nv = A.node_offset[g + 1] - v0;
  const float* P = A.params;
  const int tid = threadIdx.x;
  if (nv < 1 || nv > GMAXN) return;
  for (int v = tid; v < nv; v += blockDim.x) s_deg[v] = A.adj_offset[v0 + v + 1] - A.adj_offset[v0 + v];
  __syncthreads();
  // h0
  for (int t = tid; t < nv * GH; t += blockDim.x) {
    const int v = t / GH, j = t % GH;
    const float x1 = s_deg[v] / 8.f, x2 = nv / 16.f;
    const float* w = P + L.W0 + j * 3;
    hs[t] = fmaxf(fmaf(w[0], 1.f, fmaf(w[1], x1, fmaf(w[2], x2, P[L.b0 + j]))), 0.f);
  }
  __syncthreads();
  float* acts = A.acts;
  auto save = [&](const float* src, int slot) {
    if (acts == nullptr) return;
    for (int t = tid; t < nv * GH; t += blockDim.x)
      acts[(size_t)(v0 + t / GH) * GACT_NODE + slot * GH + t % GH] = src[t];
  };
  save(hs, 0);
  for (int l = 0; l < GLAYERS; ++l) {
    for (int t = tid; t < GH * GH; t += blockDim.x) {  // transposed copies
      const int j = t / GH, k = t % GH;
      Wa[k * GH + j] = P[L.Ws[l] + t];
      Wb[k * GH + j] = P[L.Wn[l] + t];
    }
    // mean aggregation over neighbours
    for (int t = tid; t < nv * GH; t += blockDim.x) {
      const int v = t / GH, j = t % GH;
      const int b = A.adj_offset[v0 + v], e = A.adj_offset[v0 + v + 1];
      float s = 0.f;
      for (int k = b; k < e; ++k) s += hs[(A.adj[k] - v0) * GH + j];
      as[t] = (e > b) ? s / (float)(e - b) : 0.f;
    }
    __syncthreads();
    dense_rows(Wa, hs, Wb, as, P + L.bl[l], hn, nv, true);
    __syncthreads();
    save(hn, 1 + l);
    save(as, 4 + l);
    for (int t = tid; t < nv * GH; t += blockDim.x) hs[t] = hn[t];
    __syncthreads();
  }
  // readout
  float* gv = vec;
  float* rv = vec + GH;
  for (int j = tid; j < GH; j += blockDim.x) {
    float s = 0.f;
    for (int v = 0; v < nv; ++v) s += hs[v * GH + j];
    gv[j] = s / (float)nv;
  }
  __syncthreads();
  for (int j = tid; j < GH; j += blockDim.x) {
    float s = P[L.br + j];
    for (int k = 0; k < GH; ++k) s = fmaf(P[L.Wr + j * GH + k], gv[k], s);
    rv[j] = fmaxf(s, 0.f);
  }
  __syncthreads();
  for (int j = tid; j < L.nout; j += blockDim.x) {
    float s = P[L.bo + j];
    for (int k = 0; k < GH; ++k) s = fmaf(P[L.Wo + j * GH + k], rv[k], s);
    A.out[(size_t)g * L.nout + j] = s;
  }
  if (acts != nullptr) {
    float* ga = acts + (size_t)A.total_nodes * GACT_NODE + (size_t)g * GACT_GRAPH;
    for (int j = tid; j < GH; j += blockDim.x) {
      ga[j] = gv[j];
      ga[GH + j] = rv[j];
    }
  }
}

// dW[j][k] += sum_v dz[v][j] * x[v][k] (and the bias row sums), one atomic
// add per weight per CTA.
__device__ void add_outer(float* gW, float* gb, const float* dz, const float* x, int nv, int ncols) {
  for (int t = threadIdx.x; t < GH * ncols; t += blockDim.x) {
    const int j = t / ncols, k = t % ncols;
    float s = 0.f;
    for (int v = 0; v < nv; ++v) s = fmaf(dz[v * GH + j], x[v * ncols + k], s);
    atomicAdd(gW + t, s);
  }
  if (gb != nullptr)
    for (int j = threadIdx.x; j < GH; j += blockDim.x) {
      float s = 0.f;
      for (int v = 0; v < nv; ++v) s += dz[v * GH + j];
      atomicAdd(gb + j, s);
    }
}

__global__ void __launch_bounds__(GTHREADS) k_gnn_backward(const __grid_constant__ GnnArgs A) {
  const GnnLayout L(A.p);
  extern __shared__ __align__(16) float gsm[];
  float* dh = gsm;                  // GMAXN*GH: dL/dh_l
  float* dz = dh + GMAXN * GH;      // GMAXN*GH
  float* hprev = dz + GMAXN * GH;   // GMAXN*GH
  float* aggr = hprev + GMAXN * GH; // GMAXN*GH
  float* da = aggr + GMAXN * GH;    // GMAXN*GH
  float* vec = da + GMAXN * GH;     // 4*GH + nout
  __shared__ int s_deg[GMAXN];
  const int g = blockIdx.x;
  const int v0 = A.node_offset[g], nv = A.node_offset[g + 1] - v0;
  const float* P = A.params;
  float* G = A.grad;
  const int tid = threadIdx.x;
  if (nv < 1 || nv > GMAXN) return;
  for (int v = tid; v < nv; v += blockDim.x) s_deg[v] = A.adj_offset[v0 + v + 1] - A.adj_offset[v0 + v];
  const float* ga = A.acts + (size_t)A.total_nodes * GACT_NODE + (size_t)g * GACT_GRAPH;
  float* gv = vec;
  float* rv = vec + GH;
  float* dr = vec + 2 * GH;
  float* dgv = vec + 3 * GH;
  float* dout = vec + 4 * GH;
  const float scale = 2.f / (float)(A.ngraphs * L.nout);
  for (int j = tid; j < GH; j += blockDim.x) {
    gv[j] = ga[j];
    rv[j] = ga[GH + j];
  }
  for (int j = tid; j < L.nout; j += blockDim.x) {
    const float d = A.out[(size_t)g * L.nout + j] - A.target[(size_t)g * L.nout + j];
    dout[j] = scale * d;
    atomicAdd(A.loss, d * d);
  }
  __syncthreads();
  // output layer
  for (int t = tid; t < L.nout * GH; t += blockDim.x) atomicAdd(G + L.Wo + t, dout[t / GH] * rv[t % GH]);
  for (int j = tid; j < L.nout; j += blockDim.x) atomicAdd(G + L.bo + j, dout[j]);
  for (int k = tid; k < GH; k += blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < L.nout; ++j) s = fmaf(P[L.Wo + j * GH + k], dout[j], s);
    dr[k] = rv[k] > 0.f ? s : 0.f;
  }
  __syncthreads();
  for (int t = tid; t < GH * GH; t += blockDim.x) atomicAdd(G + L.Wr + t, dr[t / GH] * gv[t % GH]);
  for (int j = tid; j < GH; j += blockDim.x) atomicAdd(G + L.br + j, dr[j]);
  for (int k = tid; k < GH; k += blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < GH; ++j) s = fmaf(P[L.Wr + j * GH + k], dr[j], s);
    dgv[k] = s;
  }
  __syncthreads();
  // dL/dh3 = dg / n for every node
  for (int t = tid; t < nv * GH; t += blockDim.x) dh[t] = dgv[t % GH] / (float)nv;
  __syncthreads();
  auto load = [&](float* dst, int slot) {
    for (int t = tid; t < nv * GH; t += blockDim.x)
      dst[t] = A.acts[(size_t)(v0 + t / GH) * GACT_NODE + slot * GH + t % GH];
  };
  for (int l = GLAYERS - 1; l >= 0; --l) {
    // dz = dh * relu'(h_l)
    for (int t = tid; t < nv * GH; t += blockDim.x) {
      const float h = A.acts[(size_t)(v0 + t / GH) * GACT_NODE + (1 + l) * GH + t % GH];
      dz[t] = h > 0.f ? dh[t] : 0.f;
    }
    load(hprev, l);
    load(aggr, 4 + l);
    __syncthreads();
    add_outer(G + L.Ws[l], G + L.bl[l], dz, hprev, nv, GH);
    add_outer(G + L.Wn[l], nullptr, dz, aggr, nv, GH);
    // da = Wn^T dz ; dh_{l-1} = Ws^T dz + scatter(da / deg)
    for (int t = tid; t < nv * GH; t += blockDim.x) {
      const int v = t / GH, k = t % GH;
      float s1 = 0.f, s2 = 0.f;
      for (int j = 0; j < GH; ++j) {
        const float d = dz[v * GH + j];
        s1 = fmaf(P[L.Ws[l] + j * GH + k], d, s1);
        s2 = fmaf(P[L.Wn[l] + j * GH + k], d, s2);
      }
      dh[t] = s1;
      da[t] = s_deg[v] > 0 ? s2 / (float)s_deg[v] : 0.f;
    }
    __syncthreads();
    for (int t = tid; t < nv * GH; t += blockDim.x) {  // h_u feeds a_w for every neighbour w
      const int u = t / GH, k = t % GH;
      const int b = A.adj_offset[v0 + u], e = A.adj_offset[v0 + u + 1];
      float s = 0.f;
      for (int q = b; q < e; ++q) s += da[(A.adj[q] - v0) * GH + k];
      dh[t] += s;
    }
    __syncthreads();
  }
  // input layer
  for (int t = tid; t < nv * GH; t += blockDim.x) {
    const float h = A.acts[(size_t)(v0 + t / GH) * GACT_NODE + t % GH];
    dz[t] = h > 0.f ? dh[t] : 0.f;
  }
  __syncthreads();
  for (int t = tid; t < GH * 3; t += blockDim.x) {
    const int j = t / 3, k = t % 3;
    float s = 0.f;
    for (int v = 0; v < nv; ++v) {
      const float x = k == 0 ? 1.f : (k == 1 ? s_deg[v] / 8.f : nv / 16.f);
      s = fmaf(dz[v * GH + j], x, s);
    }
    atomicAdd(G + L.W0 + t, s);
  }
  for (int j = tid; j < GH; j += blockDim.x) {
    float s = 0.f;
    for (int v = 0; v < nv; ++v) s += dz[v * GH + j];
    atomicAdd(G + L.b0 + j, s);
  }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int count, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

size_t gnn_param_count(int p) { return (size_t)GnnLayout(p).total; }
size_t gnn_act_floats(int total_nodes, int ngraphs) {
  return (size_t)total_nodes * GACT_NODE + (size_t)ngraphs * GACT_GRAPH;
}

static const size_t kFwdSmem = (2 * GH * GH + 3 * GMAXN * GH + 4 * GH) * sizeof(float);
static const size_t kBwdSmem = (5 * GMAXN * GH + 4 * GH + 64) * sizeof(float);

int gnn_forward(const GnnArgs& A, cudaStream_t stream) {
  static bool attr = false;
  if (!attr) {
    int rc = check_cuda(cudaFuncSetAttribute(k_gnn_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem));
    if (rc) return rc;
    attr = true;
  }
  if (A.ngraphs == 0) return QF_OK;
  k_gnn_forward<<<A.ngraphs, GTHREADS, kFwdSmem, stream>>>(A);
  return check_cuda(cudaGetLastError());
}

int gnn_backward(const GnnArgs& A, cudaStream_t stream) {
  static bool attr = false;
  if (!attr) {
    int rc = check_cuda(cudaFuncSetAttribute(k_gnn_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem));
    if (rc) return rc;
    attr = true;
  }
  if (A.ngraphs == 0) return QF_OK;
  k_gnn_backward<<<A.ngraphs, GTHREADS, kBwdSmem, stream>>>(A);
  return check_cuda(cudaGetLastError());
}

int adam_update(float* w, const float* g, float* m, float* v, int count, float lr, float b1, float b2, float eps,
                int step, cudaStream_t stream) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  int grid = (count + 255) / 256;
  if (grid > 1024) grid = 1024;
  if (grid < 1) grid = 1;
  k_adam<<<grid, 256, 0, stream>>>(w, g, m, v, count, lr, b1, b2, eps, c1, c2);
  return check_cuda(cudaGetLastError());
}

}  // namespace qf

// ---------------------------------------------------------------- C ABI ----
using namespace qf;

extern "C" size_t qf_gnn_param_count(int p) { return (p < 1 || p > 32) ? 0 : gnn_param_count(p); }

extern "C" size_t qf_gnn_activation_floats(int total_nodes, int ngraphs) {
  return (total_nodes < 0 || ngraphs < 0) ? 0 : gnn_act_floats(total_nodes, ngraphs);
}

static int gnn_check(const float* params, int p, int ngraphs, const int32_t* node_offset, const int32_t* adj_offset,
                     const int32_t* adj, const float* out) {
  if (params == nullptr || node_offset == nullptr || adj_offset == nullptr || out == nullptr) return QF_ERR_INVALID_ARGUMENT;
  if (p < 1 || p > 32 || ngraphs < 0) return QF_ERR_INVALID_ARGUMENT;
  (void)adj;
  return QF_OK;
}

extern "C" int qf_gnn_forward(const float* params, int p, int ngraphs, int total_nodes, const int32_t* node_offset,
                              const int32_t* adj_offset, const int32_t* adj, float* out, float* activations,
                              void* stream) {
  int rc = gnn_check(params, p, ngraphs, node_offset, adj_offset, adj, out);
  if (rc) return rc;
  GnnArgs A;
  std::memset(&A, 0, sizeof(A));
  A.params = params;
  A.p = p;
  A.ngraphs = ngraphs;
  A.node_offset = node_offset;
  A.adj_offset = adj_offset;
  A.adj = adj;
  A.out = out;
  A.acts = activations;
  A.total_nodes = total_nodes;
  return gnn_forward(A, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qf_gnn_backward(const float* params, int p, int ngraphs, int total_nodes, const int32_t* node_offset,
                               const int32_t* adj_offset, const int32_t* adj, const float* out, const float* target,
                               const float* activations, float* grad, float* loss, void* stream) {
  int rc = gnn_check(params, p, ngraphs, node_offset, adj_offset, adj, out);
  if (rc) return rc;
  if (target == nullptr || activations == nullptr || grad == nullptr || loss == nullptr) return QF_ERR_INVALID_ARGUMENT;
  GnnArgs A;
  std::memset(&A, 0, sizeof(A));
  A.params = params;
  A.p = p;
  A.ngraphs = ngraphs;
  A.node_offset = node_offset;
  A.adj_offset = adj_offset;
  A.adj = adj;
  A.out = const_cast<float*>(out);
  A.acts = const_cast<float*>(activations);
  A.target = target;
  A.grad = grad;
  A.loss = loss;
  A.total_nodes = total_nodes;
  return gnn_backward(A, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int qf_adam_update(float* params, const float* grad, float* m, float* v, int count, float lr, float beta1,
                              float beta2, float eps, int step, void* stream) {
  if (params == nullptr || grad == nullptr || m == nullptr || v == nullptr || count < 0 || step < 1)
    return QF_ERR_INVALID_ARGUMENT;
  return adam_update(params, grad, m, v, count, lr, beta1, beta2, eps, step, reinterpret_cast<cudaStream_t>(stream));
}
