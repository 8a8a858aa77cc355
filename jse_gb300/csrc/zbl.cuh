// NEP's ZBL short-range term (k_zbl.cu).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace nnapgb {

constexpr float kZblMaxR = 2.5f;  // pairs at or beyond this distance carry no ZBL term

struct ZblArgs {
    int flexible, T;
    double rc_inner, rc_outer;  // fixed form
    const double* z;            // [T] atomic numbers
    const double* zp;           // [T] Z^0.23
    const double* para;         // flexible: [T (T + 1) / 2][10]
    const double* rc_pair;      // fixed form with type-wise radii: [T][T][2] (rc_inner, rc_outer), or NULL
};

// Adds each atom's half of its pairs' ZBL energies to e_atom and the ZBL part of each
// entry's pair gradient to P.g (rows indexed like e_atom).
cudaError_t launch_nep_zbl(const PairBufs& P, int n, const int* type, const ZblArgs& z, double* e_atom,
                           cudaStream_t st);

}  // namespace nnapgb
