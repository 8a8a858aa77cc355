// Launch interfaces of the force-training kernels: parameter gradients of
//   L = sum_i bE_i E_i + sum_i bF_i . F_i + sum_ab bW_ab W_ab
// (E per-atom energies, F forces, W the total virial of each structure).
#pragma once

#include "common.cuh"
#include "desc.cuh"

namespace nnapgb {

// Descriptor directional derivative of one sub-basis over a run of species:
//   u_i = sum_j S_ij b_ij,   S_ij the map with g_ij = S_ij^T dE_i/dfp_i,
// with b_ij = bF_j - bF_i + bW(struct)^T dx_ij the upstream gradient of g_ij.  u has
// the layout of the descriptors (by slot, row stride fp_stride, column offset fp_off).
struct JvpArgs {
    DescArgs d;             // d.A: the forward's expansion coefficients (spherical)
    const float4* bF;       // [n] upstream force gradients (x, y, z, 0) or NULL
    const float* bW;        // [nstruct][9] upstream virial gradients or NULL
    const int* sid;         // [n] structure of each atom
    float* u;               // [slots][fp_stride] directional derivatives
    float* dA;              // spherical, or NULL: D_b A stored like d.A
};

// Per-slot records of one species' network pass (see k_net_train):
//   for each hidden layer l: aZ_l[H_l] | dZ_l[H_l] | U_l[in_l] | X_l[in_l]
//   then wo[H_L] | bo[1]
// so that dL/dW_l = sum_slots aZ_l (x) U_l + dZ_l (x) X_l, dL/db_l = sum dZ_l,
// dL/dw_out = sum wo, dL/db_out = sum bo.
struct NetTrainArgs {
    const int* perm;
    const int* range;       // device: first slot of each species, [ntypes + 1]
    int t;                  // species (0-based)
    int nmax;               // upper bound of the slot count (grid sizing)
    const float* fp;        // descriptors by slot
    const float* u;         // descriptor directional derivatives by slot
    int fp_stride;
    int D, nlayer;
    int H[4];
    const float* w;         // packed FP32 parameters (the FP32 network's layout)
    float sigma_e;
    const double* bE;       // [n] upstream per-atom energy gradients (by atom) or NULL
    float* rec;             // [slots][V]
    int V;
    float* gfp;             // or NULL: dE/dfp by slot (fp layout)
    float* dfp;             // or NULL: dL/dfp by slot, energy and force terms (fp layout)
};

// Gradient of the radial-fuse matrices W[tc][tn][p][n] of one sub-basis over a run of
// species, from the per-atom dE/dfp (gfp), dL/dfp (dfp) and, spherical, A and D_b A:
//   dL/dW[tc][tn][p][n] = sum over pairs (i, j) with types (tc, tn) of
//       Gc_j[p] fc T_n(r_j) + Gdc_j[p] D_b(fc T_n)(r_j)
// with Gc, Gdc the loss gradients of c_j = fc Rnp_j and of its directional derivative.
// Warp w processes slots s0 + w, s0 + w + G, ... and owns partial[w][tc - t0][T][NP][N1].
struct WgradArgs {
    JvpArgs j;              // geometry, upstream gradients and j.d.A
    const float* dA;        // spherical: D_b A from the directional-derivative pass
    const float* gfp;
    const float* dfp;
    float* partial;         // [G][t1 - t0][T][NP][N1], zeroed before the launch
    int G;                  // warps of the launch
    // spherical with invariant columns, or NULL: their part of M1 (dL/dA at fixed D_b A)
    // and M2 (dL/dD_b A), laid out like A
    const float* M1x;
    const float* M2x;
};

// One tile of a species' parameter gradient: a 64 x 64 block (o0, i0) of layer `layer`'s
// weight gradient, or (layer = -1) every bias and output-layer entry.
struct GradTile {
    int layer, o0, i0;
};

struct ReduceArgs {
    const int* range;
    int T;
    const float* rec;       // per-slot records, row stride V[t]
    int chunk;              // slots per partial sum
    int nchunk;             // upper bound of the chunks of one species
    float* partial;         // [T][nchunk][Pmax]
    int Pmax;
    const GradTile* tiles;  // [T][tmax]
    int tmax;
    int ntiles[kMaxTypes];
    int V[kMaxTypes];
    int D[kMaxTypes], nlayer[kMaxTypes], H[kMaxTypes][4];
    int P[kMaxTypes];       // parameter count of each species' network
    double* grad;           // concatenated per-species gradients (FP64)
    int goff[kMaxTypes];    // offset of each species in grad
};

cudaError_t upload_sh_constants_train();
cudaError_t launch_train_prep(const double* bF, int n, float4* bFf, cudaStream_t st);
cudaError_t launch_jvp(int kind, int lmax, int np, int n1, const JvpArgs& a, cudaStream_t st);
cudaError_t launch_net_train(const NetTrainArgs& a, cudaStream_t st);
cudaError_t launch_train_reduce(const ReduceArgs& a, cudaStream_t st);
cudaError_t launch_wgrad(int kind, int lmax, int np, int n1, const WgradArgs& a, cudaStream_t st);
// out[e] = sum over w < G of partial[w * per + e] (FP64, in w order), e < per.
cudaError_t launch_wgrad_final(const float* partial, int G, int per, double* out, cudaStream_t st);

}  // namespace nnapgb
