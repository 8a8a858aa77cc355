// Descriptor kernels (FP32): radial Chebyshev and spherical-Chebyshev power spectrum,
// forward (descriptors) and backward (pair gradients from dE/dfp).
//
// Mathematics restated from the reference (see the oracle for an FP64 copy):
//   x = 1 - 2r/rc, R_n = T_n(x), fc = (1 - (r/rc)^2)^4            nnap_util.hpp:226-271
//   Rnp[p] = sum_n W[t_i][t_j][p][n] R_n  (internal fuse matrix)    nnap_util.hpp:273-280
//   radial:     fp[p] = sum_j fc Rnp[p]                             basis_Chebyshev.hpp:82-133
//   spherical:  A[p][lm] = sum_j fc Rnp[p] Y_lm,
//               fp[p][l] = 4 pi/(2l+1) sum_m A[p][l,m]^2            basis_SphericalChebyshev.hpp:264-351
//   backward:   g_j = -dE_i/d(x_j - x_i) through fc, R_n, theta, phi  basis_SphericalChebyshev.hpp:353-525
// Real spherical harmonics use normalised associated Legendre functions with the
// Condon-Shortley phase, Y_{l,m>0} = sqrt2 P_lm cos(m phi), Y_{l,-m} = sqrt2 P_lm sin(m phi)
// (basis_SphericalUtil.hpp:12-101); dY/dtheta uses
//   dP_lm/dtheta = 1/2 [sqrt((l-m)(l+m+1)) P_{l,m+1} - sqrt((l+m)(l-m+1)) P_{l,m-1}],
// and the pole branch (dxy == 0) takes phi = 0 and drops the phi terms like
// calYPthetaPphi (basis_SphericalUtil.hpp:160-181).
//
// Layout: one warp per atom slot (atoms are processed in species-sorted slot order);
// forward lanes first evaluate one neighbour each into a shared-memory tile, then own
// columns lm of the P x K accumulator A; backward lanes own one neighbour each and
// stream G = dE/dA from shared memory.  The radial-fuse matrices of the basis live in
// shared memory for the whole block.  In mixed precision the spherical forward of the
// one-nonzero-per-row fuse matrices runs on the tensor cores (k_sph_tc.cuh).
#include <math_constants.h>

#include "common.cuh"
#include "pdl.cuh"
#include "desc.cuh"
#include "sph_math.cuh"
#include "k_sph_tc.cuh"

namespace nnapgb {

cudaError_t upload_sh_constants() { return upload_sh_tables(); }

namespace {

constexpr int kDescMaxWarps = 8;  // warps per CTA are a launch parameter (2, 4 or 8)

__device__ __forceinline__ int atom_of(const DescArgs& a, int s0, int warp) { return a.perm[s0 + warp]; }

}  // namespace

// NEP type-wise cutoffs (find_descriptor, nep_core.hpp:1074-1082 and 1117-1125): a pair's
// radial functions use its own cutoff min(rc, (R_cov,i + R_cov,j) factor), and a pair at or
// beyond it adds nothing. Sets rc / irc to the pair's values; false when r is beyond them.
template <int RB>
__device__ __forceinline__ bool pair_cut(const DescArgs& a, int tc, int tn, float r, float& rc, float& irc) {
    if constexpr (RB == kRbNEP) {
        if (a.pair_rc) {
            const float2 q = a.pair_rc[tc * a.T + tn];
            rc = q.x;
            irc = q.y;
            return r < rc;
        }
    }
    return true;
}

// =========================================================================== radial
template <int NP, int N1, int RB>
__global__ void __launch_bounds__(32 * kDescMaxWarps) k_radial_fwd(DescArgs a) {
    pdl_enter();
    extern __shared__ float sW[];
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    const int at = atom_of(a, s0, w);
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut, irc = 1.f / a.rcut;
    float acc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p] = 0.f;
    for (int k = lane; k < cnt; k += 32) {
        const float4 d = a.P.dx[(size_t)at * M + k];
        const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        if (r >= rc) continue;
        const int tn = __float_as_int(d.w) - 1;
        float rcp = rc, ircp = irc;
        if (!pair_cut<RB>(a, tc, tn, r, rcp, ircp)) continue;
        float T[N1], sv[NP];
        const float fc = radial_f<RB, N1>(r, ircp, T);
        fuse_apply<NP, N1>(sW + (size_t)(tc * a.T + tn) * NP * Fuse<N1>::N1P, T, sv);
#pragma unroll
        for (int p = 0; p < NP; ++p) acc[p] += fc * sv[p];
    }
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[p] += __shfl_xor_sync(0xffffffffu, acc[p], o);
    float* out = a.fp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
#pragma unroll
    for (int p = 0; p < NP; ++p)
        if (lane == (p & 31)) out[p] = acc[p];
}

template <int NP, int N1, int RB>
__global__ void __launch_bounds__(32 * kDescMaxWarps) k_radial_bwd(DescArgs a) {
    pdl_enter();
    extern __shared__ float sW[];
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    const int at = atom_of(a, s0, w);
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut, irc = 1.f / a.rcut;
    const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    float gfp[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) gfp[p] = gf[p];
    for (int k = lane; k < cnt; k += 32) {
        const size_t e = (size_t)at * M + k;
        const float4 d = a.P.dx[e];
        const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        const int tn = __float_as_int(d.w) - 1;
        float rcp = rc, ircp = irc;
        if (r < rc && pair_cut<RB>(a, tc, tn, r, rcp, ircp)) {
            float T[N1], TG[N1], fcg;
            const float fc = radial_g<RB, N1>(r, rcp, ircp, T, TG, &fcg);
            float v[N1];
            fuse_apply_t<NP, N1>(sW + (size_t)(tc * a.T + tn) * NP * Fuse<N1>::N1P, gfp, v);
            float dfc = 0.f, drn = 0.f;
#pragma unroll
            for (int n = 0; n < N1; ++n) {
                dfc += v[n] * T[n];
                drn += v[n] * TG[n];
            }
            const float gr = dfc * fcg + fc * drn;
            g = make_float4(gr * d.x, gr * d.y, gr * d.z, 0.f);
        }
        if (a.accumulate) {
            float4 o = a.P.g[e];
            a.P.g[e] = make_float4(o.x + g.x, o.y + g.y, o.z + g.z, 0.f);
        } else {
            a.P.g[e] = g;
        }
    }
}

// =========================================================================== spherical
template <int L, int NP>
struct SphShape {
    static constexpr int K = (L + 1) * (L + 1);
    static constexpr int COLS = (K + 31) / 32;
    static constexpr int KS = K | 1;                 // odd row stride: conflict-free lane writes
    static constexpr int NPS = (NP + 3) & ~3;        // 16-byte rows for broadcast float4 reads
    static constexpr int FWD_WARP_FLOATS =
        (((32 * KS + 32 * NPS) > NP * K ? (32 * KS + 32 * NPS) : NP * K) + 3) & ~3;
    static constexpr int BWD_WARP_FLOATS = K * NPS + 2 * K * 32;
};

template <int L, int NP, int N1, int RB>
__global__ void __launch_bounds__(32 * kDescMaxWarps) k_sph_fwd(DescArgs a) {
    pdl_enter();
    using S = SphShape<L, NP>;
    extern __shared__ float smem[];
    const int nW = a.T * a.T * NP * Fuse<N1>::N1P;
    float* sW = smem;
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sY = smem + ((nW + 3) & ~3) + wl * S::FWD_WARP_FLOATS;  // [32][KS]
    float* sC = sY + 32 * S::KS;                                       // [32][NPS]
    const int at = atom_of(a, s0, w);
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = a.sub_dx ? a.sub_count[at] : min(a.P.count[at], M);
    const float4* rdx = (a.sub_dx ? a.sub_dx : a.P.dx) + (size_t)at * M;
    const float rc = a.rcut, irc = 1.f / a.rcut;
    // accumulators in packed pairs of channels (p = 2h, 2h + 1) for paired FP32 FMAs
    constexpr int NH = (NP + 1) / 2;
    float2 acc[NH][S::COLS];
#pragma unroll
    for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int c = 0; c < S::COLS; ++c) acc[h][c] = make_float2(0.f, 0.f);
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float c[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) c[p] = 0.f;
        float* y = sY + lane * S::KS;
        bool valid = false;
        if (k < cnt) {
            const float4 d = rdx[k];
            const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            const int tn = __float_as_int(d.w) - 1;
            float rcp = rc, ircp = irc;
            if (r < rc && pair_cut<RB>(a, tc, tn, r, rcp, ircp)) {
                valid = true;
                float T[N1], sv[NP];
                const float fc = radial_f<RB, N1>(r, ircp, T);
                fuse_apply<NP, N1>(sW + (size_t)(tc * a.T + tn) * NP * Fuse<N1>::N1P, T, sv);
#pragma unroll
                for (int p = 0; p < NP; ++p) c[p] = fc * sv[p];
                const Angles an = angles_f(d.x, d.y, d.z, r);
                sph_harm<L, false>(an, y, nullptr, 1);
            }
        }
        if (!valid)
#pragma unroll
            for (int q = 0; q < S::K; ++q) y[q] = 0.f;
#pragma unroll
        for (int p = 0; p < S::NPS; ++p) sC[lane * S::NPS + p] = p < NP ? c[p] : 0.f;
        __syncwarp();
        const int nk = min(32, cnt - base);
#pragma unroll 4
        for (int kk = 0; kk < nk; ++kk) {
            float2 cv[NH];
            const float4* crow = reinterpret_cast<const float4*>(sC + kk * S::NPS);
#pragma unroll
            for (int q = 0; q < S::NPS / 4; ++q) {
                const float4 v = crow[q];
                if (2 * q < NH) cv[2 * q] = make_float2(v.x, v.y);
                if (2 * q + 1 < NH) cv[2 * q + 1] = make_float2(v.z, v.w);
            }
            const float* yrow = sY + kk * S::KS;
#pragma unroll
            for (int col = 0; col < S::COLS; ++col) {
                const int lm = lane + 32 * col;
                const float yv = lm < S::K ? yrow[lm] : 0.f;
                const float2 yy = make_float2(yv, yv);
#pragma unroll
                for (int h = 0; h < NH; ++h) acc[h][col] = __ffma2_rn(cv[h], yy, acc[h][col]);
            }
        }
        __syncwarp();
    }
    // A to global (backward input) and squared to shared memory for the power spectrum
    float* Aout = a.A + (size_t)w * NP * S::K;
    float* sA2 = sY;
#pragma unroll
    for (int col = 0; col < S::COLS; ++col) {
        const int lm = lane + 32 * col;
        if (lm < S::K)
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float v = (p & 1) ? acc[p >> 1][col].y : acc[p >> 1][col].x;
                Aout[p * S::K + lm] = v;
                sA2[p * S::K + lm] = v * v;
            }
    }
    __syncwarp();
    float* out = a.fp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int e = lane; e < NP * a.nl2; e += 32) {
        const int p = e / a.nl2, l = e - p * a.nl2;
        float s = 0.f;
        for (int m = 0; m <= 2 * l; ++m) s += sA2[p * S::K + l * l + m];
        out[p * a.sl + l] = kPi4 / (float)(2 * l + 1) * s;
    }
}

// Forward in the space of the radial functions, for at most kFwdTypes species and fuse
// matrices whose row p has its only nonzero in column p mod N1 (every weight type but
// rfuse): W[tc][tn][p][n] = alpha[tc][tn][p] delta(n, p mod N1).  Per neighbour species
// tn the warp accumulates
//   Ah[tn][n][lm] = sum_{j of species tn} fc_j T_n(r_j) Y_j[lm]
// (N1 instead of NP products per neighbour and lm; the neighbour's species is uniform
// across the warp in the accumulation loop, so the branch does not diverge), then
//   A[p][lm] = sum_tn alpha[tc][tn][p] Ah[tn][p mod N1][lm]
// straight from the accumulator registers.  fc Rnp is never formed.
template <int L, int NP, int N1>
struct SphFNShape {
    static constexpr int K = (L + 1) * (L + 1);
    static constexpr int COLS = (K + 31) / 32;
    static constexpr int KS = K | 1;
    static constexpr int N1P = (N1 + 3) & ~3;
    static constexpr int H = (N1 + 1) / 2;
    static constexpr int EVAL = 32 * KS + 32 * N1P + 32;   // Y, fc T, species
    static constexpr int POST = NP * K;                     // A^2
    static constexpr int WARP_FLOATS = ((EVAL > POST ? EVAL : POST) + 3) & ~3;
};

template <int L, int NP, int N1>
__global__ void __launch_bounds__(32 * kDescMaxWarps) k_sph_fwd_n(DescArgs a) {
    pdl_enter();
    using S = SphFNShape<L, NP, N1>;
    extern __shared__ float smem[];
    const int T = a.T;
    const int ntab = T * kFwdTypes * NP;  // alpha[tc][tn][p], zero for tn >= T
    float* sAl = smem;
    for (int q = threadIdx.x; q < ntab; q += blockDim.x) sAl[q] = a.fwd_alpha[q];
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* base = smem + ((ntab + 3) & ~3) + (size_t)wl * S::WARP_FLOATS;
    float* sY = base;                                       // [32][KS]
    float* sF = sY + 32 * S::KS;                            // [32][N1P] fc T_n
    int* sTn = reinterpret_cast<int*>(sF + 32 * S::N1P);    // [32]
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut, irc = 1.f / a.rcut;
    float2 acc[kFwdTypes][S::H][S::COLS];
#pragma unroll
    for (int t = 0; t < kFwdTypes; ++t)
#pragma unroll
        for (int h = 0; h < S::H; ++h)
#pragma unroll
            for (int c = 0; c < S::COLS; ++c) acc[t][h][c] = make_float2(0.f, 0.f);
    for (int b0 = 0; b0 < cnt; b0 += 32) {
        const int k = b0 + lane;
        float fT[S::N1P];
#pragma unroll
        for (int n = 0; n < S::N1P; ++n) fT[n] = 0.f;
        float* y = sY + lane * S::KS;
        int tn = 0;
        bool valid = false;
        if (k < cnt) {
            const float4 d = a.P.dx[(size_t)at * M + k];
            const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            if (r < rc) {
                valid = true;
                tn = __float_as_int(d.w) - 1;
                const float u = r * irc, fc1 = 1.f - u * u, fc2 = fc1 * fc1, fc = fc2 * fc2;
                cheby_f<N1>(1.f - 2.f * u, fT);
#pragma unroll
                for (int n = 0; n < N1; ++n) fT[n] *= fc;
                const Angles an = angles_f(d.x, d.y, d.z, r);
                sph_harm<L, false>(an, y, nullptr, 1);
            }
        }
        if (!valid)
#pragma unroll 7
            for (int q = 0; q < S::K; ++q) y[q] = 0.f;
        float4* frow = reinterpret_cast<float4*>(sF + lane * S::N1P);
#pragma unroll
        for (int q = 0; q < S::N1P / 4; ++q) frow[q] = make_float4(fT[4 * q], fT[4 * q + 1], fT[4 * q + 2], fT[4 * q + 3]);
        sTn[lane] = tn;
        __syncwarp();
        const int nk = min(32, cnt - b0);
        // unrolled so the loads of the next neighbours overlap the FMAs of this one
#pragma unroll 4
        for (int kk = 0; kk < nk; ++kk) {
            float2 f2[S::N1P / 2];
            const float4* fr = reinterpret_cast<const float4*>(sF + kk * S::N1P);
#pragma unroll
            for (int q = 0; q < S::N1P / 4; ++q) {
                const float4 v = fr[q];
                f2[2 * q] = make_float2(v.x, v.y);
                f2[2 * q + 1] = make_float2(v.z, v.w);
            }
            float2 yy[S::COLS];
#pragma unroll
            for (int col = 0; col < S::COLS; ++col) {
                const int lm = lane + 32 * col;
                const float yv = lm < S::K ? sY[kk * S::KS + lm] : 0.f;
                yy[col] = make_float2(yv, yv);
            }
            const int t = sTn[kk];
#pragma unroll
            for (int tt = 0; tt < kFwdTypes; ++tt) {
                if (t != tt) continue;  // uniform across the warp
#pragma unroll
                for (int h = 0; h < S::H; ++h)
#pragma unroll
                    for (int col = 0; col < S::COLS; ++col) acc[tt][h][col] = __ffma2_rn(f2[h], yy[col], acc[tt][h][col]);
            }
        }
        __syncwarp();
    }
    // A from the accumulators and alpha; A to global memory, A^2 to shared memory
    float* sA2 = base;
    float* Aout = a.A + (size_t)w * NP * S::K;
    const float* al = sAl + (size_t)tc * kFwdTypes * NP;
#pragma unroll
    for (int col = 0; col < S::COLS; ++col) {
        const int lm = lane + 32 * col;
        if (lm < S::K) {
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const int n = p % N1;  // a constant once the loop is unrolled
                float v = 0.f;
#pragma unroll
                for (int t = 0; t < kFwdTypes; ++t)
                    v += al[t * NP + p] * ((n & 1) ? acc[t][n >> 1][col].y : acc[t][n >> 1][col].x);
                Aout[p * S::K + lm] = v;
                sA2[p * S::K + lm] = v * v;
            }
        }
    }
    __syncwarp();
    float* out = a.fp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int e = lane; e < NP * a.nl2; e += 32) {
        const int p = e / a.nl2, l = e - p * a.nl2;
        float s = 0.f;
        for (int m = 0; m <= 2 * l; ++m) s += sA2[p * S::K + l * l + m];
        out[p * a.sl + l] = kPi4 / (float)(2 * l + 1) * s;
    }
}

// Backward, one warp per atom slot, one neighbour per lane.  For each neighbour,
//   dY_lm = sum_p c_p G[p][lm]        (chain into theta and phi),
//   dc_p  = sum_lm G[p][lm] Y_lm      (chain into fc and the radial functions),
// with c_p = fc Rnp_p.  G rows are read from shared memory as broadcast float4 loads;
// Y and dY/dtheta of the lane's neighbour sit in a lane column of shared memory.  Only
// c and dc stay live through the lm loop: the radial sums are formed again afterwards
// as v_n = sum_p dc_p W[p][n], so dfc = v . T and drn = v . dT.  Registers stay at or
// below 128 per thread (four CTAs of four warps per SM).
template <int L, int NP, int N1, int RB>
__global__ void __launch_bounds__(32 * kDescMaxWarps, 2) k_sph_bwd(DescArgs a) {
    pdl_enter();
    using S = SphShape<L, NP>;
    extern __shared__ float smem[];
    const int nW = a.T * a.T * NP * Fuse<N1>::N1P;
    float* sW = smem;
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sG = smem + nW + wl * S::BWD_WARP_FLOATS;  // [K][NPS]
    float* sY = sG + S::K * S::NPS;                  // [K][32]
    float* sYt = sY + S::K * 32;                     // [K][32]
    const int at = atom_of(a, s0, w);
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = a.sub_dx ? a.sub_count[at] : min(a.P.count[at], M);
    const float4* rdx = (a.sub_dx ? a.sub_dx : a.P.dx) + (size_t)at * M;
    const float rc = a.rcut, irc = 1.f / a.rcut;
    // G[p][lm] = 2 * 4pi/(2l+1) * dE/dfp[p][l] * A[p][lm], stored transposed
    {
        const float* Ain = a.A + (size_t)w * NP * S::K;
        const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
        for (int lm = lane; lm < S::K; lm += 32) {
            int l = 0;
            while ((l + 1) * (l + 1) <= lm) ++l;
            const float coef = l < a.nl2 ? 2.f * kPi4 / (float)(2 * l + 1) : 0.f;
            const int lc = l < a.nl2 ? l : 0;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                float v = coef * gf[p * a.sl + lc] * Ain[p * S::K + lm];
                if (a.Gx) v += a.Gx[(size_t)w * NP * S::K + p * S::K + lm];
                sG[lm * S::NPS + p] = v;
            }
#pragma unroll
            for (int p = NP; p < S::NPS; ++p) sG[lm * S::NPS + p] = 0.f;
        }
        __syncwarp();
    }
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float c[NP];
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        float r = 1.f, rcp = rc, ircp = irc;
        bool valid = false;
        if (k < cnt) {
            d = rdx[k];
            r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            valid = r < rc;
        }
        const int tn = valid ? __float_as_int(d.w) - 1 : 0;
        if (valid) valid = pair_cut<RB>(a, tc, tn, r, rcp, ircp);
        const float* Wt = sW + (size_t)(tc * a.T + tn) * NP * Fuse<N1>::N1P;
        if (valid) {
            float T[N1], sv[NP];
            const float fc = radial_f<RB, N1>(r, ircp, T);
            fuse_apply<NP, N1>(Wt, T, sv);
#pragma unroll
            for (int p = 0; p < NP; ++p) c[p] = fc * sv[p];
            const Angles an = angles_f(d.x, d.y, d.z, r);
            sph_harm<L, true>(an, sY + lane, sYt + lane, 32);
        } else {
#pragma unroll
            for (int p = 0; p < NP; ++p) c[p] = 0.f;
#pragma unroll 7
            for (int q = 0; q < S::K; ++q) { sY[q * 32 + lane] = 0.f; sYt[q * 32 + lane] = 0.f; }
        }
        // c and dc in packed channel pairs (p = 2h, 2h + 1); padded G columns are zero
        constexpr int NH = (NP + 1) / 2;
        float2 c2[NH], dc2[NH];
#pragma unroll
        for (int h = 0; h < NH; ++h) {
            c2[h] = make_float2(c[2 * h], 2 * h + 1 < NP ? c[2 * h + 1] : 0.f);
            dc2[h] = make_float2(0.f, 0.f);
        }
        float gth = 0.f, gph = 0.f;
        // one G row: returns dY_lm and adds G[.][lm] * Y_lm into dc
        auto row = [&](int lm) -> float {
            const float4* gr = reinterpret_cast<const float4*>(sG + lm * S::NPS);
            const float yv = sY[lm * 32 + lane];
            const float2 yy = make_float2(yv, yv);
            // two independent partial sums keep the dependent FMA chain short
            float2 dYa = make_float2(0.f, 0.f), dYb = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < S::NPS / 4; ++q) {
                const float4 g = gr[q];
                if (2 * q < NH) {
                    const float2 ga = make_float2(g.x, g.y);
                    dYa = __ffma2_rn(c2[2 * q], ga, dYa);
                    dc2[2 * q] = __ffma2_rn(ga, yy, dc2[2 * q]);
                }
                if (2 * q + 1 < NH) {
                    const float2 gb = make_float2(g.z, g.w);
                    dYb = __ffma2_rn(c2[2 * q + 1], gb, dYb);
                    dc2[2 * q + 1] = __ffma2_rn(gb, yy, dc2[2 * q + 1]);
                }
            }
            return (dYa.x + dYb.x) + (dYa.y + dYb.y);
        };
#pragma unroll 1
        for (int l = 0; l <= L; ++l) {
            const int c0 = l * l + l;
            gth += row(c0) * sYt[c0 * 32 + lane];
#pragma unroll 1
            for (int m = 1; m <= l; ++m) {
                const float dYp = row(c0 + m);
                const float dYm = row(c0 - m);
                gth += dYp * sYt[(c0 + m) * 32 + lane] + dYm * sYt[(c0 - m) * 32 + lane];
                gph += (float)m * (dYm * sY[(c0 + m) * 32 + lane] - dYp * sY[(c0 - m) * 32 + lane]);
            }
        }
        if (k < cnt) {
            const size_t e = (size_t)at * M + (a.sub_dx ? a.sub_pos[(size_t)at * M + k] : k);
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                float T[N1], TG[N1], v[N1], fcg;
                const float fc = radial_g<RB, N1>(r, rcp, ircp, T, TG, &fcg);
                float dc[NP];
#pragma unroll
                for (int p = 0; p < NP; ++p) dc[p] = (p & 1) ? dc2[p >> 1].y : dc2[p >> 1].x;
                fuse_apply_t<NP, N1>(Wt, dc, v);
                float dfc = 0.f, drn = 0.f;
#pragma unroll
                for (int n = 0; n < N1; ++n) {
                    dfc += v[n] * T[n];
                    drn += v[n] * TG[n];
                }
                const float gr = dfc * fcg + fc * drn;
                const Angles an = angles_f(d.x, d.y, d.z, r);
                const float ir = 1.f / r;
                const float tpx = -an.ct * an.cp * ir, tpy = -an.ct * an.sp * ir, tpz = an.st * ir;
                const float ppx = an.pole ? 0.f : an.sp / an.dxy, ppy = an.pole ? 0.f : -an.cp / an.dxy;
                g.x = gr * d.x + gth * tpx + gph * ppx;
                g.y = gr * d.y + gth * tpy + gph * ppy;
                g.z = gr * d.z + gth * tpz;
            }
            if (a.accumulate) {
                if (valid) {
                    const float4 o = a.P.g[e];
                    a.P.g[e] = make_float4(o.x + g.x, o.y + g.y, o.z + g.z, 0.f);
                }
            } else {
                a.P.g[e] = g;
            }
        }
        __syncwarp();
    }
}

// Backward in the space of the radial functions (used when every column of the fuse
// matrices has at most kNz nonzero rows and N1 < NP, e.g. the default, full, exfull and
// fuse weight types).  With Gh[tn][lm][n] = sum_p W[tc][tn][p][n] G[p][lm], formed once per
// atom from the sparse fuse table,
//   dY_lm = sum_p c_p G[p][lm] = fc sum_n T_n Gh[tn][lm][n],
//   v_n   = sum_p W[p][n] dc_p = sum_lm Gh[tn][lm][n] Y_lm,
// so the per-neighbour products run over N1 instead of NP channels, and c, dc are never
// formed.  Y and dY/dtheta are formed row by row from the lane's Legendre column in
// shared memory with cos/sin(m phi) recurrences, instead of being stored.  The Gh rows of
// m != 0 are stored times sqrt2 (the factor of those Y_lm) and the Chebyshev values times
// fc, so the per-neighbour loop multiplies by neither.
template <int L, int NP, int N1>
struct SphNShape {
    static constexpr int K = (L + 1) * (L + 1);
    static constexpr int NT = L * (L + 1) / 2 + L + 1;      // Legendre entries
    static constexpr int N1P = (N1 + 3) & ~3;
    static constexpr int NPS = (NP + 3) & ~3;
    static constexpr int SCR = ((K * NP > NT * 32 ? K * NP : NT * 32) + 3) & ~3;  // keeps float4 rows aligned
    static int warp_floats(int T) { return T * K * N1P + SCR; }
};

template <int L, int NP, int N1>
__global__ void __launch_bounds__(32 * kDescMaxWarps, 2) k_sph_bwd_n(DescArgs a) {
    pdl_enter();
    using S = SphNShape<L, NP, N1>;
    extern __shared__ float smem[];
    const int T = a.T;
    const int ntab = T * T * N1 * kNz;
    int* sNp = reinterpret_cast<int*>(smem);
    float* sNw = smem + ntab;
    for (int q = threadIdx.x; q < ntab; q += blockDim.x) {
        sNp[q] = a.nz_p[q];
        sNw[q] = a.nz_w[q];
    }
    // fuse rows with their one nonzero in column p mod N1: alpha[tc][tn][p] in shared memory
    const bool diag = a.fwd_alpha != nullptr && T <= kFwdTypes;
    const int nal = diag ? T * kFwdTypes * NP : 0;
    float* sAl = smem + ((2 * ntab + 3) & ~3);
    for (int q = threadIdx.x; q < nal; q += blockDim.x) sAl[q] = a.fwd_alpha[q];
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sGh = sAl + ((nal + 3) & ~3) + (size_t)wl * (T * S::K * S::N1P + S::SCR);  // [T][K][N1P]
    float* scr = sGh + T * S::K * S::N1P;   // G [NP][K], then the Legendre columns [NT][32]
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut, irc = 1.f / a.rcut;
    if (diag) {
        // Gh[tn][lm][n] = sum over p = n mod N1 of alpha[tc][tn][p] G[p][lm], with
        // G[p][lm] = 2 * 4pi/(2l+1) * dE/dfp[p][l] * A[p][lm] held in registers: lanes over lm
        const float* Ain = a.A + (size_t)w * NP * S::K;
        const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
        const float* al = sAl + (size_t)tc * kFwdTypes * NP;
        for (int lm = lane; lm < S::K; lm += 32) {
            int l = 0;
            while ((l + 1) * (l + 1) <= lm) ++l;
            const float coef = l < a.nl2 ? 2.f * kPi4 / (float)(2 * l + 1) : 0.f;
            const int lc = l < a.nl2 ? l : 0;
            float g[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                g[p] = coef * gf[p * a.sl + lc] * Ain[p * S::K + lm];
                if (a.Gx) g[p] += a.Gx[(size_t)w * NP * S::K + p * S::K + lm];
            }
            for (int tn = 0; tn < T; ++tn) {
                float v[S::N1P];
#pragma unroll
                for (int n = 0; n < S::N1P; ++n) {
                    v[n] = 0.f;
#pragma unroll
                    for (int p = n; p < NP; p += N1)
                        if (n < N1) v[n] += al[tn * NP + p] * g[p];
                }
                const float rs = lm != l * l + l ? kSqrt2 : 1.f;  // rows m != 0 carry sqrt2
                float4* out = reinterpret_cast<float4*>(sGh + (size_t)(tn * S::K + lm) * S::N1P);
#pragma unroll
                for (int q = 0; q < S::N1P / 4; ++q)
                    out[q] = make_float4(rs * v[4 * q], rs * v[4 * q + 1], rs * v[4 * q + 2], rs * v[4 * q + 3]);
            }
        }
        __syncwarp();
    } else {
        // G[p][lm] = 2 * 4pi/(2l+1) * dE/dfp[p][l] * A[p][lm], transposed into scr
        const float* Ain = a.A + (size_t)w * NP * S::K;
        const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
        for (int lm = lane; lm < S::K; lm += 32) {
            int l = 0;
            while ((l + 1) * (l + 1) <= lm) ++l;
            const float coef = l < a.nl2 ? 2.f * kPi4 / (float)(2 * l + 1) : 0.f;
            const int lc = l < a.nl2 ? l : 0;
#pragma unroll
            for (int p = 0; p < NP; ++p) {  // lanes over lm: conflict-free [p][K] stores
                float v = coef * gf[p * a.sl + lc] * Ain[p * S::K + lm];
                if (a.Gx) v += a.Gx[(size_t)w * NP * S::K + p * S::K + lm];
                scr[p * S::K + lm] = v;
            }
        }
        __syncwarp();
        // Gh[tn][lm][n] from the sparse fuse table of (tc, tn); lanes over lm read G rows
        // without conflicts and write their Gh rows as float4
        for (int idx = lane; idx < T * S::K; idx += 32) {
            const int tn = idx / S::K, lm = idx - tn * S::K;
            const int* np_ = sNp + (size_t)(tc * T + tn) * N1 * kNz;
            const float* nw = sNw + (size_t)(tc * T + tn) * N1 * kNz;
            float v[S::N1P];
#pragma unroll
            for (int n = 0; n < S::N1P; ++n) {
                v[n] = 0.f;
                if (n < N1) {
#pragma unroll
                    for (int z = 0; z < kNz; ++z) {
                        const int pp = np_[n * kNz + z];
                        if (pp >= 0) v[n] += nw[n * kNz + z] * scr[pp * S::K + lm];
                    }
                }
            }
            int l = 0;
            while ((l + 1) * (l + 1) <= lm) ++l;
            const float rs = lm != l * l + l ? kSqrt2 : 1.f;  // rows m != 0 carry sqrt2
            float4* out = reinterpret_cast<float4*>(sGh + (size_t)idx * S::N1P);
#pragma unroll
            for (int q = 0; q < S::N1P / 4; ++q)
                out[q] = make_float4(rs * v[4 * q], rs * v[4 * q + 1], rs * v[4 * q + 2], rs * v[4 * q + 3]);
        }
        __syncwarp();
    }
    float* sP = scr;  // [NT][32], one Legendre column per lane
    constexpr int H2 = S::N1P / 2;
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        float r = 1.f;
        bool valid = false;
        if (k < cnt) {
            d = a.P.dx[(size_t)at * M + k];
            r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            valid = r < rc;
        }
        const int tn = valid ? __float_as_int(d.w) - 1 : 0;
        const float u = r * irc, fc1 = 1.f - u * u, fc2 = fc1 * fc1, fc = valid ? fc2 * fc2 : 0.f;
        const float x = 1.f - 2.f * u;
        float Tn[S::N1P];
        cheby_f<N1>(x, Tn);
#pragma unroll
        for (int n = N1; n < S::N1P; ++n) Tn[n] = 0.f;
        const Angles an = angles_f(d.x, d.y, d.z, r);
        {
            float Pv[S::NT];
            legendre_f<L>(an.ct, an.st, Pv);
#pragma unroll
            for (int q = 0; q < S::NT; ++q) sP[q * 32 + lane] = valid ? Pv[q] : 0.f;
        }
        __syncwarp();
        float2 T2[H2], v2[H2];
#pragma unroll
        for (int h = 0; h < H2; ++h) {
            T2[h] = make_float2(fc * Tn[2 * h], fc * Tn[2 * h + 1]);
            v2[h] = make_float2(0.f, 0.f);
        }
        const float* gh = sGh + (size_t)tn * S::K * S::N1P;
        // one Gh row: returns dY_lm and adds Gh[lm][n] * y into v.  Whole float4 groups of
        // the N1 radial functions, then the remainder (the row's padding is never multiplied)
        auto row = [&](int lm, float y) -> float {
            const float4* gr = reinterpret_cast<const float4*>(gh + lm * S::N1P);
            const float2 yy = make_float2(y, y);
            float2 da = make_float2(0.f, 0.f), db = make_float2(0.f, 0.f);
            constexpr int NQ = N1 / 4, NR = N1 - 4 * (N1 / 4);
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const float4 g = gr[q];
                const float2 ga = make_float2(g.x, g.y), gb = make_float2(g.z, g.w);
                da = __ffma2_rn(T2[2 * q], ga, da);
                db = __ffma2_rn(T2[2 * q + 1], gb, db);
                v2[2 * q] = __ffma2_rn(ga, yy, v2[2 * q]);
                v2[2 * q + 1] = __ffma2_rn(gb, yy, v2[2 * q + 1]);
            }
            if (NR >= 2) {
                const float2 ga = reinterpret_cast<const float2*>(gr + NQ)[0];
                da = __ffma2_rn(T2[2 * NQ], ga, da);
                v2[2 * NQ] = __ffma2_rn(ga, yy, v2[2 * NQ]);
            }
            if (NR & 1) {
                constexpr int n = N1 - 1;
                const float g = gh[lm * S::N1P + n];
                if (n & 1) {
                    db.y = fmaf(T2[n >> 1].y, g, db.y);
                    v2[n >> 1].y = fmaf(g, y, v2[n >> 1].y);
                } else {
                    db.x = fmaf(T2[n >> 1].x, g, db.x);
                    v2[n >> 1].x = fmaf(g, y, v2[n >> 1].x);
                }
            }
            return (da.x + db.x) + (da.y + db.y);
        };
        const float cp = an.cp, sp = an.sp;
        float gth = 0.f, gph = 0.f;
#pragma unroll
        for (int l = 0; l <= L; ++l) {
            const int c0 = l * l + l, tl = l * (l + 1) / 2;
            const float p0 = sP[tl * 32 + lane];
            const float p1 = l >= 1 ? sP[(tl + 1) * 32 + lane] : 0.f;
            // m = 0: dP/dtheta = (dup P_{l,1} + ddn P_{l,1}) / 2 (P_{l,-1} = -P_{l,1})
            gth += row(c0, p0) * (0.5f * (c_dup[tl] + c_ddn[tl]) * p1);
            float cmm = 1.f, cmv = cp, smm = 0.f, smv = sp;
            float pmm = p0, pmv = p1;
#pragma unroll
            for (int m = 1; m <= l; ++m) {
                const int t = tl + m;
                const float pmp = m + 1 <= l ? sP[(t + 1) * 32 + lane] : 0.f;
                const float dpt = 0.5f * (c_dup[t] * pmp - c_ddn[t] * pmm);
                const float yp = pmv * cmv, ym = pmv * smv;  // Y / sqrt2 (the Gh rows carry sqrt2)
                const float dYp = row(c0 + m, yp);
                const float dYm = row(c0 - m, ym);
                gth += dpt * (dYp * cmv + dYm * smv);
                gph += (float)m * (dYm * yp - dYp * ym);
                const float cn = 2.f * cp * cmv - cmm, sn = 2.f * cp * smv - smm;
                cmm = cmv; cmv = cn; smm = smv; smv = sn;
                pmm = pmv; pmv = pmp;
            }
        }
        __syncwarp();  // the Legendre columns are rewritten by the next batch
        if (k < cnt) {
            const size_t e = (size_t)at * M + k;
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                const float fcg = 8.f * fc1 * fc2 * irc * irc;
                float TG[N1], Tr[N1];  // T_n formed again: fc T_n went into the row products
                cheby_grad_f<N1>(x, 2.f / (r * rc), TG);
                cheby_f<N1>(x, Tr);
                float dfc = 0.f, drn = 0.f;
#pragma unroll
                for (int n = 0; n < N1; ++n) {
                    const float vn = (n & 1) ? v2[n >> 1].y : v2[n >> 1].x;
                    dfc += vn * Tr[n];
                    drn += vn * TG[n];
                }
                const float gr = dfc * fcg + fc * drn;
                const float ir = 1.f / r;
                const float tpx = -an.ct * an.cp * ir, tpy = -an.ct * an.sp * ir, tpz = an.st * ir;
                const float ppx = an.pole ? 0.f : an.sp / an.dxy, ppy = an.pole ? 0.f : -an.cp / an.dxy;
                g.x = gr * d.x + gth * tpx + gph * ppx;
                g.y = gr * d.y + gth * tpy + gph * ppy;
                g.z = gr * d.z + gth * tpz;
            }
            if (a.accumulate) {
                if (valid) {
                    const float4 o = a.P.g[e];
                    a.P.g[e] = make_float4(o.x + g.x, o.y + g.y, o.z + g.z, 0.f);
                }
            } else {
                a.P.g[e] = g;
            }
        }
    }
}

// =========================================================================== sub-rows
// Compact copy of the entries of each row within cutoff rc (same FP32 test as the
// descriptor kernels), with their positions in the full row: the spherical kernels of a
// sub-basis whose cutoff is well inside the neighbour cutoff scan these instead of the
// full rows.  One warp per atom; entries keep their row order.
__global__ void __launch_bounds__(256) k_subrows(PairBufs P, int n, float rc, float4* __restrict__ sdx,
                                                 int* __restrict__ spos, int* __restrict__ scount) {
    pdl_enter();
    const int at = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (at >= n) return;
    const int M = P.M, cnt = min(P.count[at], M);
    int c = 0;
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        bool in = false;
        if (k < cnt) {
            d = P.dx[(size_t)at * M + k];
            in = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z) < rc;
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (in) {
            const size_t q = (size_t)at * M + c + __popc(m & ((1u << lane) - 1u));
            sdx[q] = d;
            spos[q] = k;
        }
        c += __popc(m);
    }
    if (lane == 0) scount[at] = c;
}

cudaError_t launch_subrows(const PairBufs& P, int n, float rc, float4* sdx, int* spos, int* scount,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    return launch_pdl(&k_subrows, dim3((unsigned)(((size_t)n * 32 + 255) / 256)), dim3(256), 0, st, P, n, rc, sdx,
                      spos, scount);
}

// =========================================================================== invariants
// Columns: sum over the column's terms of coefficient x product of a channel's A entries
// (calSphL3 / calSphL4, basis_SphericalUtil.hpp:395-467).  Backward: dE/dA of each
// product, one factor at a time (calGradSphL3 / L4).  One thread owns one (atom slot,
// channel) row of A, so each sum runs in term order and the results do not depend on
// scheduling.  The rows of a block are contiguous in A; the block stages them in shared
// memory with an odd row stride: the lanes of a warp apply the same term at the same time,
// so their reads of one index fall in distinct banks.
constexpr int kInvThreads = 128;

__device__ __forceinline__ int inv_stage(const InvArgs& a, float* sA, long long& r0) {
    const long long nrows = (long long)(a.range[a.t1] - a.range[a.t0]) * a.NP;
    r0 = (long long)blockIdx.x * kInvThreads;
    if (r0 >= nrows) return 0;
    const int nr = (int)min((long long)kInvThreads, nrows - r0);
    const int KS = a.K | 1;
    const float* Ab = a.A + r0 * a.K;
    for (int e = threadIdx.x; e < nr * a.K; e += kInvThreads) {
        const int r = e / a.K;
        sA[r * KS + (e - r * a.K)] = Ab[e];
    }
    return nr;
}

__global__ void __launch_bounds__(kInvThreads) k_inv_fwd(InvArgs a) {
    pdl_enter();
    extern __shared__ float sA[];  // [kInvThreads][K | 1]
    long long r0;
    const int nr = inv_stage(a, sA, r0);
    if (!nr) return;
    __syncthreads();
    const int r = threadIdx.x;
    if (r >= nr) return;
    const long long row = r0 + r;
    const int w = (int)(row / a.NP), p = (int)(row - (long long)w * a.NP);
    const float* Ap = sA + r * (a.K | 1);
    float* out = a.fp + (size_t)(a.range[a.t0] + w) * a.fp_stride + a.fp_off + p * a.sl + a.nl2;
    for (int c = 0; c < a.ncol; ++c) {
        float s = 0.f;
        for (int q = a.start[c]; q < a.start[c + 1]; ++q) {
            const int4 t = a.idx[q];
            float v = a.coef[q] * Ap[t.x] * Ap[t.y] * Ap[t.z];
            if (t.w >= 0) v *= Ap[t.w];
            s += v;
        }
        out[c] = s;
    }
}

__global__ void __launch_bounds__(kInvThreads) k_inv_bwd(InvArgs a) {
    pdl_enter();
    extern __shared__ float sA[];  // [kInvThreads][K | 1] A rows, then as many dE/dA rows
    const int KS = a.K | 1;
    float* sG = sA + kInvThreads * KS;
    long long r0;
    const int nr = inv_stage(a, sA, r0);
    if (!nr) return;
    for (int e = threadIdx.x; e < kInvThreads * KS; e += kInvThreads) sG[e] = 0.f;
    __syncthreads();
    const int r = threadIdx.x;
    if (r < nr) {
        const long long row = r0 + r;
        const int w = (int)(row / a.NP), p = (int)(row - (long long)w * a.NP);
        const float* Ap = sA + r * KS;
        float* Gp = sG + r * KS;
        const float* gf = a.gfp + (size_t)(a.range[a.t0] + w) * a.fp_stride + a.fp_off + p * a.sl + a.nl2;
        for (int c = 0; c < a.ncol; ++c) {
            const float g = gf[c];
            for (int q = a.start[c]; q < a.start[c + 1]; ++q) {
                const int4 t = a.idx[q];
                const float cg = g * a.coef[q];
                const float x = Ap[t.x], y = Ap[t.y], z = Ap[t.z];
                if (t.w < 0) {
                    Gp[t.x] += cg * y * z;
                    Gp[t.y] += cg * x * z;
                    Gp[t.z] += cg * x * y;
                } else {
                    const float u = Ap[t.w];
                    Gp[t.x] += cg * y * z * u;
                    Gp[t.y] += cg * x * z * u;
                    Gp[t.z] += cg * x * y * u;
                    Gp[t.w] += cg * x * y * z;
                }
            }
        }
    }
    __syncthreads();
    float* Gb = a.Gx + r0 * a.K;
    for (int e = threadIdx.x; e < nr * a.K; e += kInvThreads) {
        const int rr = e / a.K;
        Gb[e] = sG[rr * KS + (e - rr * a.K)];
    }
}

// u[p][nl2 + c] = -sum_terms coef sum_f (prod of the other factors) D_b A[factor f]
__global__ void __launch_bounds__(128) k_inv_jvp(InvArgs a) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* out = a.u + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int p = lane; p < a.NP; p += 32) {
        const float* Ap = a.A + ((size_t)w * a.NP + p) * a.K;
        const float* dAp = a.dA + ((size_t)w * a.NP + p) * a.K;
        for (int c = 0; c < a.ncol; ++c) {
            float s = 0.f;
            for (int q = a.start[c]; q < a.start[c + 1]; ++q) {
                const int4 t = a.idx[q];
                const float x = Ap[t.x], y = Ap[t.y], z = Ap[t.z];
                const float dx = dAp[t.x], dy = dAp[t.y], dz = dAp[t.z];
                float v;
                if (t.w < 0) {
                    v = dx * y * z + x * dy * z + x * y * dz;
                } else {
                    const float u = Ap[t.w], du = dAp[t.w];
                    v = (dx * y * z + x * dy * z + x * y * dz) * u + x * y * z * du;
                }
                s += a.coef[q] * v;
            }
            out[p * a.sl + a.nl2 + c] = -s;
        }
    }
}

// Per channel: M1x and M2x of the radial-fuse gradient (the invariant columns' parts).
__global__ void __launch_bounds__(128) k_inv_wgrad(InvArgs a) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    const float* df = a.dfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int p = lane; p < a.NP; p += 32) {
        const size_t row = ((size_t)w * a.NP + p) * a.K;
        const float* Ap = a.A + row;
        const float* dAp = a.dA + row;
        float* M1 = a.M1x + row;
        float* M2 = a.M2x + row;
        for (int k = 0; k < a.K; ++k) { M1[k] = 0.f; M2[k] = 0.f; }
        for (int c = 0; c < a.ncol; ++c) {
            const float gv = gf[p * a.sl + a.nl2 + c], dv = df[p * a.sl + a.nl2 + c];
            for (int q = a.start[c]; q < a.start[c + 1]; ++q) {
                const int4 t = a.idx[q];
                const float cf = a.coef[q];
                const int ord = t.w < 0 ? 3 : 4;
                const int id[4] = {t.x, t.y, t.z, t.w};
                float v[4], dvv[4];
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    v[f] = f < ord ? Ap[id[f]] : 1.f;
                    dvv[f] = f < ord ? dAp[id[f]] : 0.f;
                }
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    if (f >= ord) continue;
                    // d term / d A[f] and its derivative along D_b A
                    float prod = 1.f, hd = 0.f;
#pragma unroll
                    for (int o = 0; o < 4; ++o) {
                        if (o == f || o >= ord) continue;
                        float pr = dvv[o];
#pragma unroll
                        for (int o2 = 0; o2 < 4; ++o2)
                            if (o2 != f && o2 != o && o2 < ord) pr *= v[o2];
                        hd += pr;
                        prod *= v[o];
                    }
                    M1[id[f]] += cf * (dv * prod - gv * hd);
                    M2[id[f]] -= cf * gv * prod;
                }
            }
        }
    }
}

cudaError_t launch_invariants_jvp(const InvArgs& a, cudaStream_t st) {
    if (a.nmax <= 0 || a.ncol <= 0) return cudaSuccess;
    k_inv_jvp<<<(a.nmax + 3) / 4, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_invariants_wgrad(const InvArgs& a, cudaStream_t st) {
    if (a.nmax <= 0 || a.ncol <= 0) return cudaSuccess;
    k_inv_wgrad<<<(a.nmax + 3) / 4, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_invariants(const InvArgs& a, bool fwd, cudaStream_t st) {
    if (a.nmax <= 0 || a.ncol <= 0) return cudaSuccess;
    const int grid = (int)(((long long)a.nmax * a.NP + kInvThreads - 1) / kInvThreads);
    const size_t sm = sizeof(float) * kInvThreads * (a.K | 1) * (fwd ? 1 : 2);
    static int limit_fwd = 0, limit_bwd = 0;  // raised once, before any graph capture
    int& lim = fwd ? limit_fwd : limit_bwd;
    if ((int)sm > lim && sm > 48 * 1024) {
        const cudaError_t e = fwd ? cudaFuncSetAttribute(k_inv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)
                                  : cudaFuncSetAttribute(k_inv_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    if (fwd) return launch_pdl(&k_inv_fwd, dim3(grid), dim3(kInvThreads), sm, st, a);
    return launch_pdl(&k_inv_bwd, dim3(grid), dim3(kInvThreads), sm, st, a);
}

// =========================================================================== dispatch
namespace {

template <int NP, int N1, int RB>
cudaError_t launch_radial(const DescArgs& a, bool fwd, cudaStream_t st) {
    const int n = a.nmax;
    if (n <= 0) return cudaSuccess;
    const int wpc = a.warps;
    const int grid = (n + wpc - 1) / wpc;
    const size_t sm = sizeof(float) * a.T * a.T * NP * Fuse<N1>::N1P;
    static int limit_fwd = 0, limit_bwd = 0;  // raised once, before any graph capture
    int& lim = fwd ? limit_fwd : limit_bwd;
    if ((int)sm > lim && sm > 48 * 1024) {
        const cudaError_t e =
            fwd ? cudaFuncSetAttribute(k_radial_fwd<NP, N1, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)
                : cudaFuncSetAttribute(k_radial_bwd<NP, N1, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    if (fwd) return launch_pdl(&k_radial_fwd<NP, N1, RB>, dim3(grid), dim3(32 * wpc), sm, st, a);
    return launch_pdl(&k_radial_bwd<NP, N1, RB>, dim3(grid), dim3(32 * wpc), sm, st, a);
}

template <int L, int NP, int N1>
cudaError_t launch_sph_bwd_n(const DescArgs& a, cudaStream_t st) {
    using S = SphNShape<L, NP, N1>;
    const int wpc = a.warps;
    const int grid = (a.nmax + wpc - 1) / wpc;
    const size_t nal = (a.fwd_alpha && a.T <= kFwdTypes) ? (size_t)a.T * kFwdTypes * NP : 0;
    const size_t sm = sizeof(float) * (((size_t)2 * a.T * a.T * N1 * kNz + 3) / 4 * 4 + (nal + 3) / 4 * 4 +
                                       (size_t)wpc * S::warp_floats(a.T));
    if (sm > 227 * 1024) return cudaErrorInvalidValue;
    static int lim = 0;
    if ((int)sm > lim) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_sph_bwd_n<L, NP, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    return launch_pdl(&k_sph_bwd_n<L, NP, N1>, dim3(grid), dim3(32 * wpc), sm, st, a);
}

template <int L, int NP, int N1>
cudaError_t launch_sph_fwd_n(const DescArgs& a, cudaStream_t st) {
    using S = SphFNShape<L, NP, N1>;
    const int wpc = a.warps;
    const int grid = (a.nmax + wpc - 1) / wpc;
    const size_t sm = sizeof(float) * (((size_t)a.T * kFwdTypes * NP + 3) / 4 * 4 + (size_t)wpc * S::WARP_FLOATS);
    if (sm > 227 * 1024) return cudaErrorInvalidValue;
    static int lim = 0;
    if ((int)sm > lim) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_sph_fwd_n<L, NP, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    return launch_pdl(&k_sph_fwd_n<L, NP, N1>, dim3(grid), dim3(32 * wpc), sm, st, a);
}

template <int L, int NP, int N1, int RB>
cudaError_t launch_sph(const DescArgs& a, bool fwd, cudaStream_t st) {
    using S = SphShape<L, NP>;
    const int n = a.nmax;
    if (n <= 0) return cudaSuccess;
    if constexpr (RB == kRbNNAP) {   // the radial-space kernels are written for the NNAP radial functions
        if (!fwd && a.nz_p && a.nz_w && N1 < NP) return launch_sph_bwd_n<L, NP, N1>(a, st);
        if (fwd && a.fwd_alpha && N1 < NP && a.T <= kFwdTypes) {
            if constexpr (SphTcShape<L, NP>::fits)
                if (a.tc_sms > 0) return launch_sph_fwd_tc<L, NP, N1>(a, st);
            return launch_sph_fwd_n<L, NP, N1>(a, st);
        }
    }
    const int wpc = a.warps;
    const int grid = (n + wpc - 1) / wpc;
    const size_t wbytes = sizeof(float) * ((size_t)a.T * a.T * NP * Fuse<N1>::N1P);
    const size_t sm = wbytes + sizeof(float) * wpc * (fwd ? S::FWD_WARP_FLOATS : S::BWD_WARP_FLOATS);
    // the shared-memory limit is raised once per kernel (before any graph capture: the
    // first evaluation of a layout always runs eagerly)
    static int limit_fwd = 0, limit_bwd = 0;
    int& lim = fwd ? limit_fwd : limit_bwd;
    if ((int)sm > lim) {
        const cudaError_t e =
            fwd ? cudaFuncSetAttribute(k_sph_fwd<L, NP, N1, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)
                : cudaFuncSetAttribute(k_sph_bwd<L, NP, N1, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    if (fwd) return launch_pdl(&k_sph_fwd<L, NP, N1, RB>, dim3(grid), dim3(32 * wpc), sm, st, a);
    return launch_pdl(&k_sph_bwd<L, NP, N1, RB>, dim3(grid), dim3(32 * wpc), sm, st, a);
}

}  // namespace


bool desc_supported(int kind, int basis, int lmax, int np, int n1) {
    return desc_compiled(kind, basis, lmax, np, n1) || desc_generic_fits(kind, lmax, np, n1);
}

bool desc_compiled(int kind, int basis, int lmax, int np, int n1) {
#define R_CASE(P_, N_) if (kind == 0 && np == P_ && n1 == N_) return true;
#define S_CASE(L_, P_, N_) if (kind == 1 && lmax == L_ && np == P_ && n1 == N_) return true;
    if (basis == kRbNNAP) {
        NNAP_RADIAL_SHAPES(R_CASE)
        NNAP_SPH_SHAPES(S_CASE)
    } else if (basis == kRbNEP) {
        NEP_RADIAL_SHAPES(R_CASE)
        NEP_SPH_SHAPES(S_CASE)
    }
#undef R_CASE
#undef S_CASE
    return false;
}

cudaError_t launch_descriptor(int kind, int basis, int lmax, int np, int n1, const DescArgs& a, bool fwd,
                              cudaStream_t st) {
#define R_CASE(P_, N_) if (kind == 0 && np == P_ && n1 == N_) return launch_radial<P_, N_, RB_>(a, fwd, st);
#define S_CASE(L_, P_, N_) \
    if (kind == 1 && lmax == L_ && np == P_ && n1 == N_) return launch_sph<L_, P_, N_, RB_>(a, fwd, st);
    if (basis == kRbNNAP) {
        constexpr int RB_ = kRbNNAP;
        NNAP_RADIAL_SHAPES(R_CASE)
        NNAP_SPH_SHAPES(S_CASE)
    } else if (basis == kRbNEP) {
        constexpr int RB_ = kRbNEP;
        NEP_RADIAL_SHAPES(R_CASE)
        NEP_SPH_SHAPES(S_CASE)
    }
#undef R_CASE
#undef S_CASE
    return launch_descriptor_generic(kind, basis, lmax, np, n1, a, fwd, st);
}

}  // namespace nnapgb
