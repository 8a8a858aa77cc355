// Launch interfaces of the descriptor and network kernels.
#pragma once

#include "common.cuh"

namespace nnapgb {

// Arguments of one descriptor launch: one sub-basis over the contiguous range of
// species-sorted slots of a run of species sharing the sub-basis shape.  The range is
// read on the device, so launches need no host knowledge of the species counts.
struct DescArgs {
    const int* perm;        // slot -> atom
    const int* range;       // device: first slot of each species, [ntypes + 1]
    int t0, t1;             // species run [t0, t1): slots range[t0] .. range[t1]
    int nmax;               // upper bound of the slot count (grid sizing)
    const int* type;        // 1-based species per atom
    PairBufs P;
    const float* W;         // [T][T][NP][N1] radial-fuse matrices, centre species major
    int T;
    float rcut;
    float* fp;              // descriptors by slot, row stride fp_stride
    int fp_stride, fp_off;  // column offset of this sub-basis
    float* A;               // spherical only: [slot - range[t0]][NP][K] expansion coefficients
    const float* gfp;       // backward: dE/dfp by slot (same layout as fp)
    int accumulate;         // backward: add into P.g instead of overwriting
    int warps;              // warps per CTA (2, 4 or 8; one atom slot per warp)
    // spherical backward: sparse form of W, [T][T][N1][kNz] nonzero rows p (-1: none) and
    // their weights, or NULL (the kernel then works in the space of the NP channels)
    const int* nz_p;
    const float* nz_w;
    // spherical forward: alpha[tc][tn][p] with W[tc][tn][p][n] = alpha delta(n, p mod N1),
    // [T][kFwdTypes][NP], or NULL (the forward then accumulates the NP channels)
    const float* fwd_alpha;
    // spherical: power-spectrum columns per channel (l < nl2) and descriptor columns per
    // channel (sl = nl2 + invariant columns); Gx, or NULL: the invariant columns' part of
    // dE/dA, [slot - range[t0]][NP][K] like A, added to the power-spectrum part
    int nl2, sl;
    const float* Gx;
    // spherical p-space kernels of an accumulating call: compact rows of the entries within
    // rcut (dx, position in the full row; capacity P.M per atom) and their count per atom,
    // or NULL: the kernels then scan the full rows
    const float4* sub_dx;
    const int* sub_pos;
    const int* sub_count;
    // NEP type-wise cutoffs: (rc, 1/rc) of each species pair, [T][T] centre species major,
    // or NULL: every pair uses rcut
    const float2* pair_rc = nullptr;
    // spherical forward on the tensor cores: the device's SM count when the evaluation may
    // use them (mixed precision), else 0; err receives ERRBIT_TIMEOUT if one of the
    // kernel's bounded waits gives up
    int tc_sms = 0;
    int* err = nullptr;
};

// Invariant (l3max / l4max) columns of one spherical sub-basis over a run of species:
// one warp per atom slot, lanes over channels.
struct InvArgs {
    const int* perm;
    const int* range;
    int t0, t1, nmax;
    const float* A;          // [slot - range[t0]][NP][K]
    int NP, K;
    const int4* idx;         // term factors (indices into a channel's K entries, -1 unused)
    const float* coef;
    const int* start;        // [ncol + 1] first term of each column
    int ncol;
    float* fp;               // forward output (by slot)
    const float* gfp;        // backward input: dE/dfp (by slot)
    int fp_stride, fp_off, nl2, sl;
    float* Gx;               // backward output, layout of A
    // training: D_b A (layout of A), the directional derivatives u (descriptor layout),
    // dL/dfp (descriptor layout) and the outputs M1x, M2x (layout of A)
    const float* dA;
    float* u;
    const float* dfp;
    float* M1x;
    float* M2x;
};
cudaError_t launch_invariants(const InvArgs& a, bool fwd, cudaStream_t st);
// u of the invariant columns: -sum over terms of the column's derivative along D_b A.
cudaError_t launch_invariants_jvp(const InvArgs& a, cudaStream_t st);
// M1x = sum_c dfp_c dcol_c/dA - gfp_c (d2col_c/dA2) D_b A,  M2x = -sum_c gfp_c dcol_c/dA.
cudaError_t launch_invariants_wgrad(const InvArgs& a, cudaStream_t st);

constexpr int kNz = 4;        // nonzero rows per column (or columns per row) of a fuse matrix in sparse form
constexpr int kFwdTypes = 3;  // most species for the radial-space forward (per-species accumulators)
constexpr float kTcAlphaMax = 1024.f;  // largest |alpha| the tensor-core forward takes (FP16 operand range)

// Compiled shapes.  Radial: (NP, N1).  Spherical: (L, NP, N1).
#define NNAP_RADIAL_SHAPES(X) X(11, 11) X(12, 6) X(4, 4) X(8, 4) X(12, 4) X(18, 9)
#define NNAP_SPH_SHAPES(X)                                                                    \
    X(6, 18, 9) X(4, 18, 9) X(4, 5, 5) X(2, 4, 4) X(2, 8, 4) X(2, 12, 4) X(3, 5, 4) X(2, 16, 4) \
    X(3, 10, 5) X(6, 9, 9) X(4, 9, 9) X(3, 8, 4) X(4, 10, 5)

// Radial functions of a sub-basis: the NNAP Chebyshev basis or the NEP basis (radial_f /
// radial_g in sph_math.cuh).
enum { kRbNNAP = 0, kRbNEP = 1 };
// Hidden-layer activation of a species network.
enum { kActSiLU = 0, kActTanh = 1 };

// Shapes compiled for the NEP radial functions (basis kRbNEP of sph_math.cuh): radial
// (n_max_R + 1, basis_size_R + 1) and angular (L, n_max_A + 1, basis_size_A + 1).
#define NEP_RADIAL_SHAPES(X) X(5, 9) X(7, 9) X(9, 9)
#define NEP_SPH_SHAPES(X) X(4, 5, 9) X(4, 7, 9) X(4, 9, 9)

cudaError_t upload_sh_constants();
// Compact rows of the entries within rc (k_subrows): sdx / spos [n][P.M], scount [n].
cudaError_t launch_subrows(const PairBufs& P, int n, float rc, float4* sdx, int* spos, int* scount,
                           cudaStream_t st);
// basis: kRbNNAP or kRbNEP (the radial functions of the sub-basis).
// desc_compiled: a shape-specialised instance exists (NNAP_*_SHAPES / NEP_*_SHAPES);
// desc_supported: that, or the any-shape kernels of k_desc_gen.cu fit in shared memory.
bool desc_compiled(int kind, int basis, int lmax, int np, int n1);
bool desc_supported(int kind, int basis, int lmax, int np, int n1);
// Specialised instance when there is one, else the any-shape kernels.
cudaError_t launch_descriptor(int kind, int basis, int lmax, int np, int n1, const DescArgs& a, bool fwd,
                              cudaStream_t st);
// The any-shape kernels (k_desc_gen.cu): runtime NP and N1 <= 21, L <= 12.
bool desc_generic_fits(int kind, int lmax, int np, int n1);
cudaError_t launch_descriptor_generic(int kind, int basis, int lmax, int np, int n1, const DescArgs& a, bool fwd,
                                      cudaStream_t st);
cudaError_t upload_sh_constants_gen();

// Network over the slots of one species.
constexpr int kNetMaxLayers = 16;  // hidden layers of a network
struct NetArgs {
    const int* perm;
    const int* range;       // device: first slot of each species, [ntypes + 1]
    int t;                  // species (0-based): slots range[t] .. range[t+1]
    int nmax;               // upper bound of the slot count (grid sizing)
    const float* fp;        // descriptors by slot
    int fp_stride;
    int D, nlayer;
    int H[kNetMaxLayers];
    const float* w;         // packed FP32 parameters of the species (see net_pack_layout)
    double mu_e, sigma_e;
    double* e_atom;         // energy per atom (by atom index)
    float* gfp;             // dE/dfp by slot
    int act;                // hidden activation: kActSiLU (NNAP) or kActTanh (NEP)
};

// FP32 SIMT network (plain precision).
cudaError_t launch_net_fp32(const NetArgs& a, cudaStream_t st);
// Whether the FP32 network of this shape fits in shared memory (at least one warp per CTA).
bool net_fp32_fits(int D, int nlayer, const int* H);

}  // namespace nnapgb
