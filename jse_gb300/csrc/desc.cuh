// Launch interfaces of the descriptor and network kernels.
#pragma once

#include "common.cuh"

namespace nnapgb {

// Arguments of one descriptor launch: one sub-basis over a contiguous range of
// species-sorted slots [s0, s1) whose species share the sub-basis shape.
struct DescArgs {
    const int* perm;        // slot -> atom
    int s0, s1;
    const int* type;        // 1-based species per atom
    PairBufs P;
    const float* W;         // [T][T][NP][N1] radial-fuse matrices, centre species major
    int T;
    float rcut;
    float* fp;              // descriptors by slot, row stride fp_stride
    int fp_stride, fp_off;  // column offset of this sub-basis
    float* A;               // spherical only: [s - s0][NP][K] expansion coefficients
    const float* gfp;       // backward: dE/dfp by slot (same layout as fp)
    int accumulate;         // backward: add into P.g instead of overwriting
};

cudaError_t upload_sh_constants();
bool desc_supported(int kind, int lmax, int np, int n1);
cudaError_t launch_descriptor(int kind, int lmax, int np, int n1, const DescArgs& a, bool fwd, cudaStream_t st);

// Network over the slots [s0, s1) of one species.
struct NetArgs {
    const int* perm;
    int s0, s1;
    const float* fp;        // descriptors by slot
    int fp_stride;
    int D, nlayer;
    int H[4];
    const float* w;         // packed FP32 parameters of the species (see net_pack_layout)
    double mu_e, sigma_e;
    double* e_atom;         // energy per atom (by atom index)
    float* gfp;             // dE/dfp by slot
};

// FP32 SIMT network (plain precision).
cudaError_t launch_net_fp32(const NetArgs& a, cudaStream_t st);

}  // namespace nnapgb
