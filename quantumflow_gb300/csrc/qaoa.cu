// QAOA on the gate engine: the qubo_circuit of quantumflow/qaoa.py:22-64 as
// fused passes.  The cost layer prod_e ZZ(-gamma/pi) of an unweighted graph
// is exp(i*gamma*(E/2 - C(x))) (quantumflow/stdgates.py ZZ: diag
// cis(-pi t/2), cis(pi t/2), cis(pi t/2), cis(-pi t/2)), i.e. one diagonal
// phase per amplitude looked up by its cut value C(x).
#include <cmath>
#include <vector>

#include "engine.cuh"
#include "state.cuh"

namespace qf {

void qaoa_layer_ops(int n, const uint16_t* cuts, int nedges, double beta, double gamma,
                    const double* node_theta, std::vector<HostOp>& ops) {
  HostOp cut;
  cut.type = OP_CUT;
  cut.k = 0;
  cut.cuts = cuts;
  cut.table.resize(nedges + 1);
  for (int c = 0; c <= nedges; ++c) cut.table[c] = std::polar(1.0, gamma * (0.5 * nedges - c));
  ops.push_back(cut);
  if (node_theta != nullptr) {
    for (int q = 0; q < n; ++q) {
      const double th = node_theta[q];
      if (std::isnan(th)) continue;
      HostOp rz;  // RZ(theta) = diag(exp(-i theta/2), exp(i theta/2))
      rz.type = OP_DIAG;
      rz.k = 1;
      rz.gb[0] = n - 1 - q;
      rz.diag = {std::polar(1.0, -0.5 * th), std::polar(1.0, 0.5 * th)};
      ops.push_back(rz);
    }
  }
  const double c = std::cos(0.5 * beta), s = std::sin(0.5 * beta);
  for (int q = 0; q < n; ++q) {  // RX(beta) = [[c, -is], [-is, c]]
    HostOp rx;
    rx.type = OP_DENSE1;
    rx.k = 1;
    rx.gb[0] = n - 1 - q;
    rx.m = {cplx(c, 0), cplx(0, -s), cplx(0, -s), cplx(c, 0)};
    ops.push_back(rx);
  }
}

int qaoa_state(void* psi, int n, int layout, const uint16_t* cuts, int nedges, int p, const double* beta,
               const double* gamma, const double* node_theta, int fusion_k, cudaStream_t stream) {
  int rc = fill_uniform(psi, n, layout, stream);
  if (rc) return rc;
  std::vector<HostOp> ops;
  for (int l = 0; l < p; ++l) qaoa_layer_ops(n, cuts, nedges, beta[l], gamma[l], node_theta, ops);
  if (ops.empty()) return QF_OK;
  return run_ops(psi, psi, n, layout, ops, fusion_k, stream, nullptr);
}

}  // namespace qf
