// Gates on register-held amplitudes, shared by the fused-pass kernels: a
// thread holds 2^RB amplitudes whose register index r carries RB bits of
// the global index (bit j of r = one global bit).  g1_reg applies a 2x2
// gate on register bit J; g2_reg a 4x4 gate with its matrix MSB on
// register bit J0 and LSB on J1 (row index = 2 * bit(J0) + bit(J1)).
#pragma once
#include <type_traits>

#include "qf_common.cuh"

namespace qf {

template <int RB, int J, typename E>
QF_D void g1_reg(const Coef* cf, E (&a)[1 << RB]) {
#pragma unroll
  for (int i = 0; i < (1 << (RB - 1)); ++i) {
    const int i0 = ((i >> J) << (J + 1)) | (i & ((1 << J) - 1));
    const int i1 = i0 | (1 << J);
    E p[2] = {a[i0], a[i1]};
    a[i0] = cdot<2>(cf, p);
    a[i1] = cdot<2>(cf + 2, p);
  }
}
template <int RB, typename E>
QF_D void g1_reg_dispatch(int j, const Coef* cf, E (&a)[1 << RB]) {
  switch (j) {
    case 0: g1_reg<RB, 0>(cf, a); break;
    case 1: if constexpr (RB > 1) g1_reg<RB, 1>(cf, a); break;
    case 2: if constexpr (RB > 2) g1_reg<RB, 2>(cf, a); break;
    case 3: if constexpr (RB > 3) g1_reg<RB, 3>(cf, a); break;
  }
}

template <int RB, int J0, int J1, typename E>
QF_D void g2_reg(const Coef* cf, E (&a)[1 << RB], bool dense = false) {
  constexpr int LO = J0 < J1 ? J0 : J1, HI = J0 < J1 ? J1 : J0;
#pragma unroll
  for (int i = 0; i < (1 << (RB - 2)); ++i) {
    int b = ((i >> LO) << (LO + 1)) | (i & ((1 << LO) - 1));
    b = ((b >> HI) << (HI + 1)) | (b & ((1 << HI) - 1));
    const int idx[4] = {b, b | (1 << J1), b | (1 << J0), b | (1 << J0) | (1 << J1)};
    E p[4] = {a[idx[0]], a[idx[1]], a[idx[2]], a[idx[3]]};
    if constexpr (sizeof(E) == sizeof(float4) && std::is_same<E, float4>::value) {
      if (dense) {  // every coefficient part nonzero: float-float TwoSum trees
#pragma unroll
        for (int r = 0; r < 4; ++r) a[idx[r]] = ff_cdot4_dense(cf + 4 * r, p);
        continue;
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) a[idx[r]] = cdot<4>(cf + 4 * r, p);
  }
}
template <int RB, typename E>
QF_D void g2_reg_dispatch(int j0, int j1, const Coef* cf, E (&a)[1 << RB]) {
  switch (j0 * 4 + j1) {
    case 1: g2_reg<RB, 0, 1>(cf, a); break;
    case 4: g2_reg<RB, 1, 0>(cf, a); break;
    case 2: if constexpr (RB > 2) g2_reg<RB, 0, 2>(cf, a); break;
    case 8: if constexpr (RB > 2) g2_reg<RB, 2, 0>(cf, a); break;
    case 6: if constexpr (RB > 2) g2_reg<RB, 1, 2>(cf, a); break;
    case 9: if constexpr (RB > 2) g2_reg<RB, 2, 1>(cf, a); break;
    case 3: if constexpr (RB > 3) g2_reg<RB, 0, 3>(cf, a); break;
    case 12: if constexpr (RB > 3) g2_reg<RB, 3, 0>(cf, a); break;
    case 7: if constexpr (RB > 3) g2_reg<RB, 1, 3>(cf, a); break;
    case 13: if constexpr (RB > 3) g2_reg<RB, 3, 1>(cf, a); break;
    case 11: if constexpr (RB > 3) g2_reg<RB, 2, 3>(cf, a); break;
    case 14: if constexpr (RB > 3) g2_reg<RB, 3, 2>(cf, a); break;
  }
}

}  // namespace qf
