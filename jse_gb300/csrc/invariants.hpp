// Three- and four-body invariants of a spherical expansion A[l^2 + l + m] (the l3max /
// l4max descriptor columns of the spherical-Chebyshev basis, calSphL3 / calSphL4 in
// basis_SphericalUtil.hpp:395-467).
#pragma once

#include <vector>

namespace nnapgb {

// coeff * A[idx[0]] * ... * A[idx[order-1]]
struct InvTerm {
    int order;
    int idx[4];
    double coeff;
};

// Number of invariant columns per channel for l3max (0..6) and l4max (0..3).
int invariant_count(int l3max, int l4max);

// Term lists of every invariant column of (l3max, l4max), in descriptor order:
//   l3: 222 112 | 233 123 | 444 224 334 244 134 | 255 455 235 145 345 |
//       666 336 446 556 266 466 246 156 356
//   l4: 1111 | 2222 1122 | 3333 1133 2233 1113 1333 1223
// With a the complex-basis coefficients of A (a_{l,0} = A_{l,0},
// a_{l,m} = (-1)^m (A_{l,m} + i A_{l,-m})/sqrt2, a_{l,-m} = (A_{l,m} - i A_{l,-m})/sqrt2):
//   L3(l1 l2 l3)    = sum (l1 l2 l3; m1 m2 m3) a a a                      (Wigner 3j)
//   L4(l1 l2 l3 l4) = sum_L (-1)^(l1+l2+L)/(2L+1) sum_M X12_LM conj(X34_LM),
//                     X12_LM = sum <l1 m1 l2 m2|L M> a a                 (Clebsch-Gordan)
// Index tuples are sorted and repeated products folded into one term.
std::vector<std::vector<InvTerm>> invariant_columns(int l3max, int l4max);

}  // namespace nnapgb
