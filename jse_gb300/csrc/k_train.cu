// Force-training double backward (FP32): parameter gradients of
//   L = sum_i bE_i E_i + sum_i bF_i . F_i + sum_ab bW_ab W_ab.
//
// The reference computes these per atom with jse_nnap_forwardEnergyForce /
// jse_nnap_backwardEnergyForce (nnap_interface.cpp:142-232): fpBackwardBackward
// (nnap_main.hpp:398-445, basis_SphericalChebyshev.hpp:527-656, basis_Chebyshev.hpp)
// turns the upstream pair gradients b_ij = dL/dg_ij into a descriptor-space vector,
// normedNnBackwardBackward + normedNnBackward (nnap_main.hpp:447-495,
// nn_FeedForward.hpp:184-320) carry it and bE through the network.  Restated here:
//
//   u_i = sum_j S_ij b_ij, where g_ij = S_ij^T dE_i/dfp_i, i.e. u_i = -D_b fp_i, the
//   derivative of the descriptors along the displacement perturbation b:
//     radial      u[p]    = sum_j (dx . b) sum_n W[p][n] (fcg T_n + fc TG_n)
//     spherical   dA[p][lm] = sum_j D_b(c_j[p]) Y_j[lm] + c_j[p] D_b(Y_j[lm]),
//                 u[p][l] = -2 * 4 pi/(2l+1) * sum_m A[p][lm] dA[p][lm]
//   with c = fc Rnp, fcg = -(dfc/dr)/r, TG_n = -(dT_n/dr)/r,
//   D_b c[p] = -(dx . b) sum_n W[p][n] (fcg T_n + fc TG_n),
//   D_b Y = dY/dtheta (grad theta . b) + dY/dphi (grad phi . b).
//
//   Network (x = (fp - mu)/sigma, z_l = W_l h_{l-1} + b_l, h_l = silu(z_l),
//   E = sigma_E (w . h_L + b_out) + mu_E), with ux = u / sigma:
//     first backward     aH_L = sigma_E w,  aZ_l = aH_l silu'(z_l),  aH_{l-1} = W_l^T aZ_l
//     force term         U_0 = ux;  v_l = W_l U_{l-1};  U_l = v_l silu'(z_l);
//                        bz_l = v_l aH_l silu''(z_l);  dL/dW_l += aZ_l (x) U_{l-1};
//                        dL/dw += sigma_E U_L
//     energy term + bz   dZ_L = bE sigma_E w silu'(z_L) + bz_L;
//                        dZ_{l-1} = (W_l^T dZ_l) silu'(z_{l-1}) + bz_{l-1};
//                        dL/dW_l += dZ_l (x) h_{l-1};  dL/db_l += dZ_l;
//                        dL/dw += bE sigma_E h_L;  dL/db_out += bE sigma_E
// The per-atom vectors go to per-slot records; k_train_reduce sums their outer
// products over fixed chunks of slots and adds the chunks in FP64 in chunk order, so the
// result does not depend on scheduling.
#include "common.cuh"
#include "desc.cuh"
#include "sph_math.cuh"
#include "train.cuh"

namespace nnapgb {

cudaError_t upload_sh_constants_train() { return upload_sh_tables(); }

namespace {

constexpr int kJvpWarps = 4;

__global__ void k_train_prep(const double* __restrict__ bF, int n, float4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_float4((float)bF[3 * (size_t)i], (float)bF[3 * (size_t)i + 1], (float)bF[3 * (size_t)i + 2], 0.f);
}

// Upstream gradient of g for row entry e of atom `at`: bF_j - bF_i + bW^T dx, with the
// virial components ordered xx, yy, zz, xy, xz, yz, yx, zx, zy (W_ab = sum dx_a g_b).
__device__ __forceinline__ float3 pair_upstream(const JvpArgs& a, int at, size_t e, float4 d) {
    float3 b = make_float3(0.f, 0.f, 0.f);
    if (a.bF) {
        const int j = (int)(a.d.P.key[e] >> 32);
        const float4 fj = a.bF[j], fi = a.bF[at];
        b = make_float3(fj.x - fi.x, fj.y - fi.y, fj.z - fi.z);
    }
    if (a.bW) {
        const float* w = a.bW + 9 * (size_t)a.sid[at];
        b.x += w[0] * d.x + w[6] * d.y + w[7] * d.z;
        b.y += w[3] * d.x + w[1] * d.y + w[8] * d.z;
        b.z += w[4] * d.x + w[5] * d.y + w[2] * d.z;
    }
    return b;
}

// D_b (fc T_n) for every n: -(dx . b) (fcg T_n + fc TG_n)
template <int N1>
__device__ __forceinline__ void radial_dir(float r, float rc, float db, float* T, float* v) {
    const float irc = 1.f / rc;
    const float u = r * irc, fc1 = 1.f - u * u, fc2 = fc1 * fc1, fc = fc2 * fc2;
    const float fcg = 8.f * fc1 * fc2 * irc * irc;
    const float x = 1.f - 2.f * u;
    float TG[N1];
    cheby_f<N1>(x, T);
    cheby_grad_f<N1>(x, 2.f / (r * rc), TG);
#pragma unroll
    for (int n = 0; n < N1; ++n) v[n] = -db * (fcg * T[n] + fc * TG[n]);
#pragma unroll
    for (int n = 0; n < N1; ++n) T[n] *= fc;  // T becomes fc T_n
}

}  // namespace

// =========================================================================== radial
// One warp per atom slot, lanes over neighbours; u[p] = -sum_j D_b c_j[p].
template <int NP, int N1>
__global__ void __launch_bounds__(32 * kJvpWarps) k_radial_jvp(JvpArgs ja) {
    const DescArgs& a = ja.d;
    extern __shared__ float sW[];
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut;
    float acc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p] = 0.f;
    for (int k = lane; k < cnt; k += 32) {
        const size_t e = (size_t)at * M + k;
        const float4 d = a.P.dx[e];
        const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        if (!(r < rc)) continue;
        const float3 b = pair_upstream(ja, at, e, d);
        const float db = d.x * b.x + d.y * b.y + d.z * b.z;
        float T[N1], v[N1], dc[NP];
        radial_dir<N1>(r, rc, db, T, v);
        fuse_apply<NP, N1>(sW + (size_t)(tc * a.T + __float_as_int(d.w) - 1) * NP * Fuse<N1>::N1P, v, dc);
#pragma unroll
        for (int p = 0; p < NP; ++p) acc[p] -= dc[p];
    }
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[p] += __shfl_xor_sync(0xffffffffu, acc[p], off);
    float* out = ja.u + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
#pragma unroll
    for (int p = 0; p < NP; ++p)
        if (lane == p % 32) out[p] = acc[p];
}

// =========================================================================== spherical
template <int L, int NP>
struct JvpShape {
    static constexpr int K = (L + 1) * (L + 1);
    static constexpr int COLS = (K + 31) / 32;
    static constexpr int KS = K | 1;            // odd row stride: conflict-free lane writes
    static constexpr int NPS = (NP + 3) & ~3;   // 16-byte rows for broadcast float4 reads
    static constexpr int WARP_FLOATS = 2 * 32 * KS + 2 * 32 * NPS;
    static_assert(NP <= 64, "the A dA products reuse the two Y tiles");
};

// One warp per atom slot.  Lanes first evaluate one neighbour each (c, D_b c, Y, D_b Y
// into shared-memory tiles), then own columns lm of the P x K accumulator dA, as the
// forward kernel owns those of A.  A itself is the forward's stored copy.
template <int L, int NP, int N1>
__global__ void __launch_bounds__(32 * kJvpWarps) k_sph_jvp(JvpArgs ja) {
    using S = JvpShape<L, NP>;
    const DescArgs& a = ja.d;
    extern __shared__ float smem[];
    const int nW = a.T * a.T * NP * Fuse<N1>::N1P;
    float* sW = smem;
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sY = smem + ((nW + 3) & ~3) + wl * S::WARP_FLOATS;  // [32][KS] Y
    float* sD = sY + 32 * S::KS;                                 // [32][KS] D_b Y
    float* sC = sD + 32 * S::KS;                                 // [32][NPS] c
    float* sDC = sC + 32 * S::NPS;                               // [32][NPS] D_b c
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut;
    constexpr int NH = (NP + 1) / 2;
    float2 acc[NH][S::COLS];
#pragma unroll
    for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int c = 0; c < S::COLS; ++c) acc[h][c] = make_float2(0.f, 0.f);
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float c[NP], dc[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) { c[p] = 0.f; dc[p] = 0.f; }
        float* y = sY + lane * S::KS;
        float* dy = sD + lane * S::KS;
        bool valid = false;
        if (k < cnt) {
            const size_t e = (size_t)at * M + k;
            const float4 d = a.P.dx[e];
            const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            if (r < rc) {
                valid = true;
                const float3 b = pair_upstream(ja, at, e, d);
                const float db = d.x * b.x + d.y * b.y + d.z * b.z;
                float T[N1], v[N1];
                radial_dir<N1>(r, rc, db, T, v);
                const float* Wt = sW + (size_t)(tc * a.T + __float_as_int(d.w) - 1) * NP * Fuse<N1>::N1P;
                fuse_apply<NP, N1>(Wt, T, c);
                fuse_apply<NP, N1>(Wt, v, dc);
                const Angles an = angles_f(d.x, d.y, d.z, r);
                sph_harm<L, true>(an, y, dy, 1);
                // derivatives of theta and phi along b (phi terms dropped at the pole)
                const float ir = 1.f / r;
                const float dth = an.ct * an.cp * ir * b.x + an.ct * an.sp * ir * b.y - an.st * ir * b.z;
                const float dph = an.pole ? 0.f : (-an.sp * b.x + an.cp * b.y) / an.dxy;
#pragma unroll
                for (int l = 0; l <= L; ++l) {
                    const int c0 = l * l + l;
                    dy[c0] *= dth;
#pragma unroll
                    for (int m = 1; m <= l; ++m) {
                        const float yp = y[c0 + m], ym = y[c0 - m];
                        dy[c0 + m] = dy[c0 + m] * dth - (float)m * ym * dph;
                        dy[c0 - m] = dy[c0 - m] * dth + (float)m * yp * dph;
                    }
                }
            }
        }
        if (!valid)
#pragma unroll 7
            for (int q = 0; q < S::K; ++q) { y[q] = 0.f; dy[q] = 0.f; }
#pragma unroll
        for (int p = 0; p < S::NPS; ++p) {
            sC[lane * S::NPS + p] = p < NP ? c[p] : 0.f;
            sDC[lane * S::NPS + p] = p < NP ? dc[p] : 0.f;
        }
        __syncwarp();
        const int nk = min(32, cnt - base);
        for (int kk = 0; kk < nk; ++kk) {
            float2 cv[NH], dv[NH];
            const float4* crow = reinterpret_cast<const float4*>(sC + kk * S::NPS);
            const float4* drow = reinterpret_cast<const float4*>(sDC + kk * S::NPS);
#pragma unroll
            for (int q = 0; q < S::NPS / 4; ++q) {
                const float4 v = crow[q], g = drow[q];
                if (2 * q < NH) { cv[2 * q] = make_float2(v.x, v.y); dv[2 * q] = make_float2(g.x, g.y); }
                if (2 * q + 1 < NH) { cv[2 * q + 1] = make_float2(v.z, v.w); dv[2 * q + 1] = make_float2(g.z, g.w); }
            }
            const float* yrow = sY + kk * S::KS;
            const float* drow2 = sD + kk * S::KS;
#pragma unroll
            for (int col = 0; col < S::COLS; ++col) {
                const int lm = lane + 32 * col;
                const float yv = lm < S::K ? yrow[lm] : 0.f;
                const float dyv = lm < S::K ? drow2[lm] : 0.f;
                const float2 yy = make_float2(yv, yv), dd = make_float2(dyv, dyv);
#pragma unroll
                for (int h = 0; h < NH; ++h) {
                    acc[h][col] = __ffma2_rn(dv[h], yy, acc[h][col]);
                    acc[h][col] = __ffma2_rn(cv[h], dd, acc[h][col]);
                }
            }
        }
        __syncwarp();
    }
    // A dA products (A from the forward pass) into the freed Y tiles, then the l sums
    const float* Ain = a.A + (size_t)w * NP * S::K;
    float* dAout = ja.dA ? ja.dA + (size_t)w * NP * S::K : nullptr;
    float* sP = sY;  // [NP][K]
#pragma unroll
    for (int col = 0; col < S::COLS; ++col) {
        const int lm = lane + 32 * col;
        if (lm < S::K)
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float v = (p & 1) ? acc[p >> 1][col].y : acc[p >> 1][col].x;
                sP[p * S::K + lm] = Ain[p * S::K + lm] * v;
                if (dAout) dAout[p * S::K + lm] = v;
            }
    }
    __syncwarp();
    float* out = ja.u + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int e = lane; e < NP * a.nl2; e += 32) {
        const int p = e / a.nl2, l = e - p * a.nl2;
        float s = 0.f;
        for (int m = 0; m <= 2 * l; ++m) s += sP[p * S::K + l * l + m];
        out[p * a.sl + l] = -2.f * kPi4 / (float)(2 * l + 1) * s;
    }
}

// Directional derivative in the space of the radial functions (fuse matrices whose row p
// has its only nonzero alpha[tc][tn][p] in column p mod N1, at most kFwdTypes species):
//   dAh[tn][n][lm] = sum_{j of species tn} D_b(fc T_n) Y_lm + fc T_n D_b(Y_lm),
//   dA[p][lm] = sum_tn alpha[tc][tn][p] dAh[tn][p mod N1][lm]
// (2 N1 instead of 2 NP products per neighbour and lm, as the radial-space forward).
template <int L, int NP, int N1>
struct JvpNShape {
    static constexpr int K = (L + 1) * (L + 1);
    static constexpr int COLS = (K + 31) / 32;
    static constexpr int KS = K | 1;
    static constexpr int N1P = (N1 + 3) & ~3;
    static constexpr int H = (N1 + 1) / 2;
    static constexpr int EVAL = 2 * 32 * KS + 2 * 32 * N1P + 32;  // Y, D_b Y, fc T, D_b(fc T), species
    static constexpr int POST = NP * K;
    static constexpr int WARP_FLOATS = ((EVAL > POST ? EVAL : POST) + 3) & ~3;
};

template <int L, int NP, int N1>
__global__ void __launch_bounds__(32 * kJvpWarps, 3) k_sph_jvp_n(JvpArgs ja) {
    using S = JvpNShape<L, NP, N1>;
    const DescArgs& a = ja.d;
    extern __shared__ float smem[];
    const int T = a.T;
    const int ntab = T * kFwdTypes * NP;
    float* sAl = smem;
    for (int q = threadIdx.x; q < ntab; q += blockDim.x) sAl[q] = a.fwd_alpha[q];
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* base = smem + ((ntab + 3) & ~3) + (size_t)wl * S::WARP_FLOATS;
    float* sY = base;                       // [32][KS]
    float* sD = sY + 32 * S::KS;            // [32][KS]
    float* sF = sD + 32 * S::KS;            // [32][N1P] fc T_n
    float* sV = sF + 32 * S::N1P;           // [32][N1P] D_b(fc T_n)
    int* sTn = reinterpret_cast<int*>(sV + 32 * S::N1P);
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut;
    float2 acc[kFwdTypes][S::H][S::COLS];
#pragma unroll
    for (int t = 0; t < kFwdTypes; ++t)
#pragma unroll
        for (int h = 0; h < S::H; ++h)
#pragma unroll
            for (int c = 0; c < S::COLS; ++c) acc[t][h][c] = make_float2(0.f, 0.f);
    for (int b0 = 0; b0 < cnt; b0 += 32) {
        const int k = b0 + lane;
        float* y = sY + lane * S::KS;
        float* dy = sD + lane * S::KS;
        int tn = 0;
        bool valid = false;
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        float3 b = make_float3(0.f, 0.f, 0.f);
        float r = 1.f;
        if (k < cnt) {
            const size_t e = (size_t)at * M + k;
            d = a.P.dx[e];
            r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            if (r < rc) {
                valid = true;
                tn = __float_as_int(d.w) - 1;
                b = pair_upstream(ja, at, e, d);
            }
        }
        {
            // radial rows first, so they hold no registers during the harmonics
            float fT[S::N1P], v[S::N1P];
#pragma unroll
            for (int n = 0; n < S::N1P; ++n) { fT[n] = 0.f; v[n] = 0.f; }
            if (valid) radial_dir<N1>(r, rc, d.x * b.x + d.y * b.y + d.z * b.z, fT, v);
            float4* fr = reinterpret_cast<float4*>(sF + lane * S::N1P);
            float4* vr = reinterpret_cast<float4*>(sV + lane * S::N1P);
#pragma unroll
            for (int q = 0; q < S::N1P / 4; ++q) {
                fr[q] = make_float4(fT[4 * q], fT[4 * q + 1], fT[4 * q + 2], fT[4 * q + 3]);
                vr[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
        if (valid) {
            {
                const Angles an = angles_f(d.x, d.y, d.z, r);
                sph_harm<L, true>(an, y, dy, 1);
                const float ir = 1.f / r;
                const float dth = an.ct * an.cp * ir * b.x + an.ct * an.sp * ir * b.y - an.st * ir * b.z;
                const float dph = an.pole ? 0.f : (-an.sp * b.x + an.cp * b.y) / an.dxy;
#pragma unroll
                for (int l = 0; l <= L; ++l) {
                    const int c0 = l * l + l;
                    dy[c0] *= dth;
#pragma unroll
                    for (int m = 1; m <= l; ++m) {
                        const float yp = y[c0 + m], ym = y[c0 - m];
                        dy[c0 + m] = dy[c0 + m] * dth - (float)m * ym * dph;
                        dy[c0 - m] = dy[c0 - m] * dth + (float)m * yp * dph;
                    }
                }
            }
        }
        if (!valid)
#pragma unroll 7
            for (int q = 0; q < S::K; ++q) { y[q] = 0.f; dy[q] = 0.f; }
        sTn[lane] = tn;
        __syncwarp();
        const int nk = min(32, cnt - b0);
        for (int kk = 0; kk < nk; ++kk) {
            float2 f2[S::N1P / 2], v2[S::N1P / 2];
            const float4* fk = reinterpret_cast<const float4*>(sF + kk * S::N1P);
            const float4* vk = reinterpret_cast<const float4*>(sV + kk * S::N1P);
#pragma unroll
            for (int q = 0; q < S::N1P / 4; ++q) {
                const float4 x = fk[q], z = vk[q];
                f2[2 * q] = make_float2(x.x, x.y);
                f2[2 * q + 1] = make_float2(x.z, x.w);
                v2[2 * q] = make_float2(z.x, z.y);
                v2[2 * q + 1] = make_float2(z.z, z.w);
            }
            float2 yy[S::COLS], dd[S::COLS];
#pragma unroll
            for (int col = 0; col < S::COLS; ++col) {
                const int lm = lane + 32 * col;
                const float yv = lm < S::K ? sY[kk * S::KS + lm] : 0.f;
                const float dv = lm < S::K ? sD[kk * S::KS + lm] : 0.f;
                yy[col] = make_float2(yv, yv);
                dd[col] = make_float2(dv, dv);
            }
            const int t = sTn[kk];
#pragma unroll
            for (int tt = 0; tt < kFwdTypes; ++tt) {
                if (t != tt) continue;  // uniform across the warp
#pragma unroll
                for (int h = 0; h < S::H; ++h)
#pragma unroll
                    for (int col = 0; col < S::COLS; ++col) {
                        acc[tt][h][col] = __ffma2_rn(v2[h], yy[col], acc[tt][h][col]);
                        acc[tt][h][col] = __ffma2_rn(f2[h], dd[col], acc[tt][h][col]);
                    }
            }
        }
        __syncwarp();
    }
    // dA from the accumulators; A dA products into shared memory, then the l sums
    const float* Ain = a.A + (size_t)w * NP * S::K;
    float* dAout = ja.dA ? ja.dA + (size_t)w * NP * S::K : nullptr;
    const float* al = sAl + (size_t)tc * kFwdTypes * NP;
    float* sP = base;  // [NP][K]
#pragma unroll
    for (int col = 0; col < S::COLS; ++col) {
        const int lm = lane + 32 * col;
        if (lm < S::K) {
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const int n = p % N1;  // a constant once the loop is unrolled
                float dv = 0.f;
#pragma unroll
                for (int t = 0; t < kFwdTypes; ++t)
                    dv += al[t * NP + p] * ((n & 1) ? acc[t][n >> 1][col].y : acc[t][n >> 1][col].x);
                sP[p * S::K + lm] = Ain[p * S::K + lm] * dv;
                if (dAout) dAout[p * S::K + lm] = dv;
            }
        }
    }
    __syncwarp();
    float* out = ja.u + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int e = lane; e < NP * a.nl2; e += 32) {
        const int p = e / a.nl2, l = e - p * a.nl2;
        float s = 0.f;
        for (int m = 0; m <= 2 * l; ++m) s += sP[p * S::K + l * l + m];
        out[p * a.sl + l] = -2.f * kPi4 / (float)(2 * l + 1) * s;
    }
}

// =========================================================================== network
namespace {

constexpr int kTrainAtoms = 8;  // atoms per warp: every weight load is used 8 times

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float silu_f(float z) { return z * sigm(z); }
__device__ __forceinline__ float silu_g(float z) {
    const float s = sigm(z);
    return s * (1.f + z * (1.f - s));
}
__device__ __forceinline__ float silu_gg(float z) {
    const float s = sigm(z);
    return s * (1.f - s) * (2.f + z * (1.f - 2.f * s));
}

// out[o][q] = sum_i WT[i][o] in[i][q] (+ bias[o]); lanes own outputs o and o + 32, so each
// pair of 8-atom input loads from shared memory feeds 16 FMAs per weight pair.
__device__ __forceinline__ void mv_fwd(const float* __restrict__ WT, const float* __restrict__ bias, int in, int H,
                                       const float* vin, float* out, int lane) {
    for (int o0 = 0; o0 < H; o0 += 64) {
        const int oa = o0 + lane, ob = o0 + 32 + lane;
        const bool ha = oa < H, hb = ob < H;
        float za[kTrainAtoms], zb[kTrainAtoms];
#pragma unroll
        for (int q = 0; q < kTrainAtoms; ++q) {
            za[q] = (bias && ha) ? bias[oa] : 0.f;
            zb[q] = (bias && hb) ? bias[ob] : 0.f;
        }
#pragma unroll 4
        for (int i = 0; i < in; ++i) {
            const float wa = ha ? WT[(size_t)i * H + oa] : 0.f;
            const float wb = hb ? WT[(size_t)i * H + ob] : 0.f;
            const float4 x0 = *reinterpret_cast<const float4*>(vin + i * kTrainAtoms);
            const float4 x1 = *reinterpret_cast<const float4*>(vin + i * kTrainAtoms + 4);
            za[0] += wa * x0.x; za[1] += wa * x0.y; za[2] += wa * x0.z; za[3] += wa * x0.w;
            za[4] += wa * x1.x; za[5] += wa * x1.y; za[6] += wa * x1.z; za[7] += wa * x1.w;
            zb[0] += wb * x0.x; zb[1] += wb * x0.y; zb[2] += wb * x0.z; zb[3] += wb * x0.w;
            zb[4] += wb * x1.x; zb[5] += wb * x1.y; zb[6] += wb * x1.z; zb[7] += wb * x1.w;
        }
#pragma unroll
        for (int q = 0; q < kTrainAtoms; ++q) {
            if (ha) out[oa * kTrainAtoms + q] = za[q];
            if (hb) out[ob * kTrainAtoms + q] = zb[q];
        }
    }
}

// out[i][q] = sum_o W[o][i] in[o][q]; lanes own inputs i, i + 32, i + 64 and i + 96.
__device__ __forceinline__ void mv_bwd(const float* __restrict__ W, int in, int H, const float* vin, float* out,
                                       int lane) {
    for (int i0 = 0; i0 < in; i0 += 128) {
        float g[4][kTrainAtoms];
        bool has[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            has[r] = i0 + 32 * r + lane < in;
#pragma unroll
            for (int q = 0; q < kTrainAtoms; ++q) g[r][q] = 0.f;
        }
#pragma unroll 2
        for (int o = 0; o < H; ++o) {
            const float4 d0 = *reinterpret_cast<const float4*>(vin + o * kTrainAtoms);
            const float4 d1 = *reinterpret_cast<const float4*>(vin + o * kTrainAtoms + 4);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float wv = has[r] ? W[(size_t)o * in + i0 + 32 * r + lane] : 0.f;
                g[r][0] += wv * d0.x; g[r][1] += wv * d0.y; g[r][2] += wv * d0.z; g[r][3] += wv * d0.w;
                g[r][4] += wv * d1.x; g[r][5] += wv * d1.y; g[r][6] += wv * d1.z; g[r][7] += wv * d1.w;
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (has[r])
#pragma unroll
                for (int q = 0; q < kTrainAtoms; ++q) out[(i0 + 32 * r + lane) * kTrainAtoms + q] = g[r][q];
    }
}

// Record columns [off, off + len) of the warp's atoms from a [len][8] buffer.
__device__ __forceinline__ void put_rec(float* rec, int V, int slot0, int na, int off, int len, const float* buf,
                                        int lane) {
    for (int q = 0; q < na; ++q)
        for (int k = lane; k < len; k += 32) rec[(size_t)(slot0 + q) * V + off + k] = buf[k * kTrainAtoms + q];
}

}  // namespace

// One warp per 8 atom slots of one species.  Shared memory per warp (units x 8 atoms):
// x, ux [D]; z_l, aH_l [H_l] per layer; two work buffers [Hmax].
__global__ void __launch_bounds__(128) k_net_train(NetTrainArgs a, int warp_floats) {
    extern __shared__ float smem[];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s0 = a.range[a.t], s1 = a.range[a.t + 1];
    const int slot0 = s0 + (blockIdx.x * (blockDim.x >> 5) + wl) * kTrainAtoms;
    if (slot0 >= s1) return;
    const int na = min(kTrainAtoms, s1 - slot0);
    const int L = a.nlayer, D = a.D;
    int Hmax = D, Hsum = 0;
    for (int l = 0; l < L; ++l) { Hmax = max(Hmax, a.H[l]); Hsum += a.H[l]; }
    float* x = smem + (size_t)wl * warp_floats;  // [D][8]
    float* ux = x + D * kTrainAtoms;              // [D][8]
    float* zb = ux + D * kTrainAtoms;             // z_l at zb + 8 * (sum of H before l)
    float* ab = zb + Hsum * kTrainAtoms;          // aH_l, later bz_l, same offsets
    float* t0 = ab + Hsum * kTrainAtoms;          // [Hmax][8]
    float* t1 = t0 + Hmax * kTrainAtoms;          // [Hmax][8]
    // packed parameters: mu | 1/sigma | per layer W^T[in][H] | W[H][in] | b[H] | w_out | b_out
    const float* mu = a.w;
    const float* isig = mu + D;
    const float* WT[4];
    const float* Wr[4];
    const float* bb[4];
    int zoff[4], roff[4], in_of[4];
    {
        const float* p = isig + D;
        int in = D, zo = 0, ro = 0;
        for (int l = 0; l < L; ++l) {
            const int H = a.H[l];
            WT[l] = p;
            Wr[l] = p + (size_t)in * H;
            bb[l] = Wr[l] + (size_t)H * in;
            p = bb[l] + H;
            zoff[l] = zo;
            roff[l] = ro;
            in_of[l] = in;
            zo += H * kTrainAtoms;
            ro += 2 * H + 2 * in;
            in = H;
        }
    }
    const int HL = a.H[L - 1];
    const float* wo = bb[L - 1] + HL;
    const int rwo = roff[L - 1] + 2 * HL + 2 * in_of[L - 1];  // wo columns, then bo
    const float se = a.sigma_e;
    // bE of atom (lane & 7): the element loops below give each thread atoms q = lane & 7
    const int myq = lane & (kTrainAtoms - 1);
    const float be = (a.bE && myq < na) ? (float)a.bE[a.perm[slot0 + myq]] : 0.f;
    // inputs: x = (fp - mu)/sigma, ux = u/sigma
    for (int i = lane; i < D; i += 32)
#pragma unroll
        for (int q = 0; q < kTrainAtoms; ++q) {
            const size_t r = (size_t)(slot0 + q) * a.fp_stride + i;
            x[i * kTrainAtoms + q] = q < na ? (a.fp[r] - mu[i]) * isig[i] : 0.f;
            ux[i * kTrainAtoms + q] = q < na ? a.u[r] * isig[i] : 0.f;
        }
    __syncwarp();
    // forward: z_l; layer inputs recorded as X_l
    {
        const float* cur = x;
        float* nxt = t0;
        for (int l = 0; l < L; ++l) {
            const int H = a.H[l], in = in_of[l];
            put_rec(a.rec, a.V, slot0, na, roff[l] + 2 * H + in, in, cur, lane);
            float* z = zb + zoff[l];
            mv_fwd(WT[l], bb[l], in, H, cur, z, lane);
            __syncwarp();
            if (l + 1 < L) {
                for (int k = lane; k < H * kTrainAtoms; k += 32) nxt[k] = silu_f(z[k]);
                __syncwarp();
                cur = nxt;
                nxt = (nxt == t0) ? t1 : t0;
            }
        }
    }
    // first backward: aH_l (upstream sigma_E on the output); aZ_l recorded
    for (int k = lane; k < HL * kTrainAtoms; k += 32) ab[zoff[L - 1] + k] = se * wo[k / kTrainAtoms];
    __syncwarp();
    for (int l = L - 1; l >= 0; --l) {
        const int H = a.H[l];
        const float* z = zb + zoff[l];
        const float* aH = ab + zoff[l];
        for (int k = lane; k < H * kTrainAtoms; k += 32) t0[k] = aH[k] * silu_g(z[k]);
        __syncwarp();
        put_rec(a.rec, a.V, slot0, na, roff[l], H, t0, lane);
        if (l > 0) {
            mv_bwd(Wr[l], in_of[l], H, t0, ab + zoff[l - 1], lane);
        } else if (a.gfp) {  // dE/dfp = (W_1^T aZ_1) / sigma
            mv_bwd(Wr[0], D, H, t0, t1, lane);
            __syncwarp();
            for (int q = 0; q < na; ++q)
                for (int i = lane; i < D; i += 32)
                    a.gfp[(size_t)(slot0 + q) * a.fp_stride + i] = t1[i * kTrainAtoms + q] * isig[i];
        }
        __syncwarp();
    }
    // force term: U_l forward, bz_l into the aH_l buffers
    {
        const float* U = ux;
        for (int l = 0; l < L; ++l) {
            const int H = a.H[l], in = in_of[l];
            put_rec(a.rec, a.V, slot0, na, roff[l] + 2 * H, in, U, lane);
            float* v = (U == t1) ? t0 : t1;  // not U's buffer
            mv_fwd(WT[l], nullptr, in, H, U, v, lane);
            __syncwarp();
            const float* z = zb + zoff[l];
            float* aH = ab + zoff[l];
            for (int k = lane; k < H * kTrainAtoms; k += 32) {
                const float zz = z[k], vv = v[k];
                aH[k] = vv * aH[k] * silu_gg(zz);  // bz_l
                v[k] = vv * silu_g(zz);             // U_l
            }
            __syncwarp();
            U = v;
        }
        // wo = sigma_E U_L + bE sigma_E h_L (energy part added below)
        for (int k = lane; k < HL * kTrainAtoms; k += 32) {
            const float zz = zb[zoff[L - 1] + k];
            t0[k] = se * (U[k] + be * silu_f(zz));
        }
        __syncwarp();
        put_rec(a.rec, a.V, slot0, na, rwo, HL, t0, lane);
        if (lane < na) a.rec[(size_t)(slot0 + lane) * a.V + rwo + HL] = se * be;
        __syncwarp();
    }
    // energy backward with the bz terms: dZ_l recorded
    {
        float* dz = t0;
        for (int k = lane; k < HL * kTrainAtoms; k += 32) {
            const float zz = zb[zoff[L - 1] + k];
            dz[k] = be * se * wo[k / kTrainAtoms] * silu_g(zz) + ab[zoff[L - 1] + k];
        }
        __syncwarp();
        for (int l = L - 1; l >= 0; --l) {
            const int H = a.H[l];
            put_rec(a.rec, a.V, slot0, na, roff[l] + H, H, dz, lane);
            if (l == 0) {
                if (a.dfp) {  // dL/dfp = (W_1^T dZ_1) / sigma
                    float* nd = (dz == t0) ? t1 : t0;
                    mv_bwd(Wr[0], D, H, dz, nd, lane);
                    __syncwarp();
                    for (int q = 0; q < na; ++q)
                        for (int i = lane; i < D; i += 32)
                            a.dfp[(size_t)(slot0 + q) * a.fp_stride + i] = nd[i * kTrainAtoms + q] * isig[i];
                }
                break;
            }
            float* nd = (dz == t0) ? t1 : t0;
            mv_bwd(Wr[l], in_of[l], H, dz, nd, lane);
            __syncwarp();
            const int Hp = a.H[l - 1];
            const float* z = zb + zoff[l - 1];
            const float* bz = ab + zoff[l - 1];
            for (int k = lane; k < Hp * kTrainAtoms; k += 32) nd[k] = nd[k] * silu_g(z[k]) + bz[k];
            __syncwarp();
            dz = nd;
        }
    }
}

// =========================================================================== reductions
namespace {

constexpr int kRedThreads = 256;
constexpr int kStage = 32;  // slots staged in shared memory per step

struct NetGeom {
    int L, H[4], in[4], roff[4], woff[4], hoff[4], HW, HL, Hsum, rwo;
};

__device__ __forceinline__ NetGeom geom(const ReduceArgs& a, int t) {
    NetGeom g;
    g.L = a.nlayer[t];
    int in = a.D[t], ro = 0, wo = 0, ho = 0;
    for (int l = 0; l < 4; ++l) {
        if (l >= g.L) { g.H[l] = g.in[l] = g.roff[l] = g.woff[l] = g.hoff[l] = 0; continue; }
        const int H = a.H[t][l];
        g.H[l] = H;
        g.in[l] = in;
        g.roff[l] = ro;
        g.woff[l] = wo;
        g.hoff[l] = ho;
        ro += 2 * H + 2 * in;
        wo += H * in;
        ho += H;
        in = H;
    }
    g.HW = wo;
    g.HL = g.H[g.L - 1];
    g.Hsum = ho;
    g.rwo = ro;
    return g;
}

}  // namespace

// Partial gradient of one tile over one chunk of one species' slots.  Weight tiles: each
// thread owns a 4 x 4 block of the 64 x 64 tile, with the chunk's aZ/dZ rows and U/X
// columns staged through shared memory 32 slots at a time.
__global__ void __launch_bounds__(kRedThreads) k_train_reduce(ReduceArgs a) {
    const int c = blockIdx.x, t = blockIdx.y, z = blockIdx.z;
    if (z >= a.ntiles[t]) return;
    const int s0 = a.range[t], s1 = a.range[t + 1];
    const int b0 = s0 + c * a.chunk;
    if (b0 >= s1) return;
    const int b1 = min(b0 + a.chunk, s1);
    const GradTile tile = a.tiles[t * a.tmax + z];
    const NetGeom g = geom(a, t);
    const int V = a.V[t];
    float* part = a.partial + ((size_t)t * a.nchunk + c) * a.Pmax;
    if (tile.layer < 0) {
        const int nvec = g.Hsum + g.HL + 1;
        for (int e = threadIdx.x; e < nvec; e += kRedThreads) {
            int col, pidx;
            if (e < g.Hsum) {
                int l = 0;
                while (l + 1 < g.L && e >= g.hoff[l + 1]) ++l;
                col = g.roff[l] + g.H[l] + (e - g.hoff[l]);
                pidx = g.HW + g.HL + e;
            } else if (e < g.Hsum + g.HL) {
                col = g.rwo + (e - g.Hsum);
                pidx = g.HW + (e - g.Hsum);
            } else {
                col = g.rwo + g.HL;
                pidx = g.HW + g.HL + g.Hsum;
            }
            float s = 0.f;
            for (int q = b0; q < b1; ++q) s += a.rec[(size_t)q * V + col];
            part[pidx] = s;
        }
        return;
    }
    __shared__ __align__(16) float sO[2][kStage][64];
    __shared__ __align__(16) float sI[2][kStage][64];
    const int l = tile.layer, H = g.H[l], in = g.in[l];
    const int o0 = tile.o0, i0 = tile.i0;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] = 0.f;
    for (int sb = b0; sb < b1; sb += kStage) {
        const int ns = min(kStage, b1 - sb);
        for (int q = threadIdx.x; q < kStage * 64; q += kRedThreads) {
            const int s = q >> 6, k = q & 63;
            float ao = 0.f, dz = 0.f, uu = 0.f, xx = 0.f;
            if (s < ns) {
                const float* r = a.rec + (size_t)(sb + s) * V + g.roff[l];
                if (o0 + k < H) { ao = r[o0 + k]; dz = r[H + o0 + k]; }
                if (i0 + k < in) { uu = r[2 * H + i0 + k]; xx = r[2 * H + in + i0 + k]; }
            }
            sO[0][s][k] = ao;
            sO[1][s][k] = dz;
            sI[0][s][k] = uu;
            sI[1][s][k] = xx;
        }
        __syncthreads();
        for (int s = 0; s < ns; ++s) {
            const float4 oa = *reinterpret_cast<const float4*>(&sO[0][s][ty * 4]);
            const float4 od = *reinterpret_cast<const float4*>(&sO[1][s][ty * 4]);
            const float4 iu = *reinterpret_cast<const float4*>(&sI[0][s][tx * 4]);
            const float4 ix = *reinterpret_cast<const float4*>(&sI[1][s][tx * 4]);
            const float ov[4] = {oa.x, oa.y, oa.z, oa.w}, dv[4] = {od.x, od.y, od.z, od.w};
            const float uv[4] = {iu.x, iu.y, iu.z, iu.w}, xv[4] = {ix.x, ix.y, ix.z, ix.w};
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[r][q] += ov[r] * uv[q] + dv[r] * xv[q];
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int o = o0 + ty * 4 + r, i = i0 + tx * 4 + q;
            if (o < H && i < in) part[g.woff[l] + (size_t)o * in + i] = acc[r][q];
        }
}

// grad[t][p] = sum over the species' chunks, in chunk order, in FP64.
__global__ void k_train_final(ReduceArgs a) {
    const int t = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P[t]) return;
    const int s0 = a.range[t], s1 = a.range[t + 1];
    const int nck = (s1 - s0 + a.chunk - 1) / a.chunk;
    double s = 0.0;
    for (int c = 0; c < nck; ++c) s += (double)a.partial[((size_t)t * a.nchunk + c) * a.Pmax + p];
    a.grad[a.goff[t] + p] = s;
}

// =========================================================================== radial-fuse gradients
namespace {

constexpr int kWgWarps = 4;

template <int L, int NP, int N1, bool SPH>
struct WgShape {
    static constexpr int K = SPH ? (L + 1) * (L + 1) : 1;
    static constexpr int KS = K | 1;
    static constexpr int NPS = (NP + 3) & ~3;
    static constexpr int N1P = (N1 + 3) & ~3;
    static constexpr int PN = NP * N1;
    // M1, M2 [K][NPS] | Y, D_b Y [32][KS] | Gc, Gdc [32][NPS] | fc T, D_b(fc T) [32][N1P] | tn [32]
    static constexpr int FIXED = (SPH ? 2 * K * NPS + 2 * 32 * KS : 0) + 2 * 32 * NPS + 2 * 32 * N1P + 32;
    __host__ __device__ static int warp_floats(int T) { return (FIXED + T * PN + 3) & ~3; }
};

}  // namespace

// One warp per atom slot (slots s0 + w, s0 + w + G, ... of warp w).  Lanes evaluate one
// neighbour each: fc T_n and D_b(fc T_n), and the loss gradients of c_j and D_b c_j,
//   spherical  Gc[p] = sum_lm M1[lm][p] Y_lm + M2[lm][p] D_b Y_lm,  Gdc[p] = sum_lm M2[lm][p] Y_lm,
//              M1 = 2 k_l (dfp[p][l] A - gfp[p][l] D_b A),  M2 = -2 k_l gfp[p][l] A,  k_l = 4 pi/(2l+1)
//   radial     Gc[p] = dfp[p],  Gdc[p] = -gfp[p]
// (restating backwardAnlm with GRAD_PARAM and backwardBackwardAnlm, basis_SphericalChebyshev.hpp:353-617,
// with backwardRnp / backwardBackwardRnp, nnap_util.hpp:282-313).  Lanes then own entries
// (p, n) of the [T][NP][N1] block of the centre's species and add Gc fcT + Gdc D_b(fcT) of
// each neighbour into the entry of its species, in neighbour order.
template <int L, int NP, int N1, bool SPH>
__global__ void __launch_bounds__(32 * kWgWarps) k_wgrad(WgradArgs g) {
    using S = WgShape<L, NP, N1, SPH>;
    const DescArgs& a = g.j.d;
    extern __shared__ float smem[];
    const int nW = a.T * a.T * NP * Fuse<N1>::N1P;
    float* sW = smem;
    load_fuse<NP, N1>(a.W, sW, a.T);
    __syncthreads();
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    if (w >= g.G) return;
    float* base = smem + ((nW + 3) & ~3) + (size_t)wl * S::warp_floats(a.T);
    float* sM1 = base;
    float* sM2 = sM1 + (SPH ? S::K * S::NPS : 0);
    float* sY = sM2 + (SPH ? S::K * S::NPS : 0);
    float* sD = sY + (SPH ? 32 * S::KS : 0);
    float* sGc = sD + (SPH ? 32 * S::KS : 0);
    float* sGd = sGc + 32 * S::NPS;
    float* sF = sGd + 32 * S::NPS;
    float* sV = sF + 32 * S::N1P;
    int* sTn = reinterpret_cast<int*>(sV + 32 * S::N1P);
    float* sAcc = reinterpret_cast<float*>(sTn + 32);
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    const int Tr = a.t1 - a.t0;
    const int TPN = a.T * S::PN;
    float* part = g.partial + (size_t)w * Tr * TPN;
    const float rc = a.rcut;
    for (int slot = s0 + w; slot < s1; slot += g.G) {
        const int at = a.perm[slot];
        const int tc = a.type[at] - 1;
        const int M = a.P.M, cnt = min(a.P.count[at], M);
        const float* gf = g.gfp + (size_t)slot * a.fp_stride + a.fp_off;
        const float* df = g.dfp + (size_t)slot * a.fp_stride + a.fp_off;
        if (SPH) {
            const float* Ain = a.A + (size_t)(slot - s0) * NP * S::K;
            const float* dAin = g.dA + (size_t)(slot - s0) * NP * S::K;
            const float* M1x = g.M1x ? g.M1x + (size_t)(slot - s0) * NP * S::K : nullptr;
            const float* M2x = g.M2x ? g.M2x + (size_t)(slot - s0) * NP * S::K : nullptr;
            for (int lm = lane; lm < S::K; lm += 32) {
                int l = 0;
                while ((l + 1) * (l + 1) <= lm) ++l;
                const float k2 = l < a.nl2 ? 2.f * kPi4 / (float)(2 * l + 1) : 0.f;
                const int lc = l < a.nl2 ? l : 0;
                for (int p = 0; p < S::NPS; ++p) {
                    float m1 = 0.f, m2 = 0.f;
                    if (p < NP) {
                        const float av = Ain[p * S::K + lm], dav = dAin[p * S::K + lm];
                        const float gv = gf[p * a.sl + lc], dv = df[p * a.sl + lc];
                        m1 = k2 * (dv * av - gv * dav);
                        m2 = -k2 * gv * av;
                        if (M1x) {  // the invariant columns' part
                            m1 += M1x[p * S::K + lm];
                            m2 += M2x[p * S::K + lm];
                        }
                    }
                    sM1[lm * S::NPS + p] = m1;
                    sM2[lm * S::NPS + p] = m2;
                }
            }
        }
        for (int e = lane; e < TPN; e += 32) sAcc[e] = 0.f;
        __syncwarp();
        for (int b0 = 0; b0 < cnt; b0 += 32) {
            const int k = b0 + lane;
            float gc[NP], gd[NP], fT[N1], v[N1];
#pragma unroll
            for (int p = 0; p < NP; ++p) { gc[p] = 0.f; gd[p] = 0.f; }
#pragma unroll
            for (int n = 0; n < N1; ++n) { fT[n] = 0.f; v[n] = 0.f; }
            int tn = 0;
            bool valid = false;
            float* y = sY + lane * S::KS;
            float* dy = sD + lane * S::KS;
            if (k < cnt) {
                const size_t e = (size_t)at * M + k;
                const float4 d = a.P.dx[e];
                const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
                if (r < rc) {
                    valid = true;
                    tn = __float_as_int(d.w) - 1;
                    const float3 b = pair_upstream(g.j, at, e, d);
                    const float db = d.x * b.x + d.y * b.y + d.z * b.z;
                    radial_dir<N1>(r, rc, db, fT, v);
                    if (SPH) {
                        const Angles an = angles_f(d.x, d.y, d.z, r);
                        sph_harm<(SPH ? L : 0), true>(an, y, dy, 1);
                        const float ir = 1.f / r;
                        const float dth = an.ct * an.cp * ir * b.x + an.ct * an.sp * ir * b.y - an.st * ir * b.z;
                        const float dph = an.pole ? 0.f : (-an.sp * b.x + an.cp * b.y) / an.dxy;
#pragma unroll
                        for (int l = 0; l <= (SPH ? L : 0); ++l) {
                            const int c0 = l * l + l;
                            dy[c0] *= dth;
#pragma unroll
                            for (int m = 1; m <= l; ++m) {
                                const float yp = y[c0 + m], ym = y[c0 - m];
                                dy[c0 + m] = dy[c0 + m] * dth - (float)m * ym * dph;
                                dy[c0 - m] = dy[c0 - m] * dth + (float)m * yp * dph;
                            }
                        }
#pragma unroll 1
                        for (int lm = 0; lm < S::K; ++lm) {
                            const float yv = y[lm], dyv = dy[lm];
                            const float4* m1 = reinterpret_cast<const float4*>(sM1 + lm * S::NPS);
                            const float4* m2 = reinterpret_cast<const float4*>(sM2 + lm * S::NPS);
#pragma unroll
                            for (int q = 0; q < S::NPS / 4; ++q) {
                                const float4 x1 = m1[q], x2 = m2[q];
                                const float a1[4] = {x1.x, x1.y, x1.z, x1.w}, a2[4] = {x2.x, x2.y, x2.z, x2.w};
#pragma unroll
                                for (int c = 0; c < 4; ++c) {
                                    const int p = 4 * q + c;
                                    if (p < NP) {
                                        gc[p] += a1[c] * yv + a2[c] * dyv;
                                        gd[p] += a2[c] * yv;
                                    }
                                }
                            }
                        }
                    } else {
#pragma unroll
                        for (int p = 0; p < NP; ++p) { gc[p] = df[p]; gd[p] = -gf[p]; }
                    }
                }
            }
            (void)valid;
#pragma unroll
            for (int p = 0; p < S::NPS; ++p) {
                sGc[lane * S::NPS + p] = p < NP ? gc[p] : 0.f;
                sGd[lane * S::NPS + p] = p < NP ? gd[p] : 0.f;
            }
#pragma unroll
            for (int n = 0; n < S::N1P; ++n) {
                sF[lane * S::N1P + n] = n < N1 ? fT[n] : 0.f;
                sV[lane * S::N1P + n] = n < N1 ? v[n] : 0.f;
            }
            sTn[lane] = tn;
            __syncwarp();
            const int nk = min(32, cnt - b0);
            for (int e = lane; e < S::PN; e += 32) {
                const int p = e / N1, n = e - p * N1;
                for (int kk = 0; kk < nk; ++kk) {
                    const float c = sGc[kk * S::NPS + p] * sF[kk * S::N1P + n] + sGd[kk * S::NPS + p] * sV[kk * S::N1P + n];
                    sAcc[sTn[kk] * S::PN + e] += c;
                }
            }
            __syncwarp();
        }
        float* dst = part + (size_t)(tc - a.t0) * TPN;
        for (int e = lane; e < TPN; e += 32) dst[e] += sAcc[e];
        __syncwarp();
    }
}

__global__ void k_wgrad_final(const float* __restrict__ partial, int G, int per, double* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= per) return;
    double s = 0.0;
    for (int w = 0; w < G; ++w) s += (double)partial[(size_t)w * per + e];
    out[e] = s;
}

// =========================================================================== launchers
namespace {

template <int NP, int N1>
cudaError_t launch_radial_jvp(const JvpArgs& a, cudaStream_t st) {
    const int n = a.d.nmax;
    if (n <= 0) return cudaSuccess;
    const size_t sm = sizeof(float) * a.d.T * a.d.T * NP * Fuse<N1>::N1P;
    static int lim = 0;
    if ((int)sm > lim && sm > 48 * 1024) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_radial_jvp<NP, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    k_radial_jvp<NP, N1><<<(n + kJvpWarps - 1) / kJvpWarps, 32 * kJvpWarps, sm, st>>>(a);
    return cudaGetLastError();
}

template <int L, int NP, int N1>
cudaError_t launch_sph_jvp_n(const JvpArgs& a, cudaStream_t st) {
    using S = JvpNShape<L, NP, N1>;
    const size_t sm = sizeof(float) * (((size_t)a.d.T * kFwdTypes * NP + 3) / 4 * 4 + (size_t)kJvpWarps * S::WARP_FLOATS);
    if (sm > 227 * 1024) return cudaErrorInvalidValue;
    static int lim = 0;
    if ((int)sm > lim) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_sph_jvp_n<L, NP, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    k_sph_jvp_n<L, NP, N1><<<(a.d.nmax + kJvpWarps - 1) / kJvpWarps, 32 * kJvpWarps, sm, st>>>(a);
    return cudaGetLastError();
}

template <int L, int NP, int N1>
cudaError_t launch_sph_jvp(const JvpArgs& a, cudaStream_t st) {
    using S = JvpShape<L, NP>;
    const int n = a.d.nmax;
    if (n <= 0) return cudaSuccess;
    if (a.d.fwd_alpha && N1 < NP && a.d.T <= kFwdTypes) return launch_sph_jvp_n<L, NP, N1>(a, st);
    const size_t wf = ((size_t)a.d.T * a.d.T * NP * Fuse<N1>::N1P + 3) & ~(size_t)3;
    const size_t sm = sizeof(float) * (wf + (size_t)kJvpWarps * S::WARP_FLOATS);
    static int lim = 0;
    if ((int)sm > lim) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_sph_jvp<L, NP, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    k_sph_jvp<L, NP, N1><<<(n + kJvpWarps - 1) / kJvpWarps, 32 * kJvpWarps, sm, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

namespace {

template <int L, int NP, int N1, bool SPH>
cudaError_t launch_wgrad_t(const WgradArgs& g, cudaStream_t st) {
    using S = WgShape<L, NP, N1, SPH>;
    if (g.G <= 0) return cudaSuccess;
    const size_t wf = ((size_t)g.j.d.T * g.j.d.T * NP * Fuse<N1>::N1P + 3) & ~(size_t)3;
    const size_t sm = sizeof(float) * (wf + (size_t)kWgWarps * S::warp_floats(g.j.d.T));
    if (sm > 227 * 1024) return cudaErrorInvalidValue;
    static int lim = 0;
    if ((int)sm > lim) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_wgrad<L, NP, N1, SPH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    k_wgrad<L, NP, N1, SPH><<<(g.G + kWgWarps - 1) / kWgWarps, 32 * kWgWarps, sm, st>>>(g);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_wgrad(int kind, int lmax, int np, int n1, const WgradArgs& a, cudaStream_t st) {
#define R_CASE(P_, N_) if (kind == 0 && np == P_ && n1 == N_) return launch_wgrad_t<0, P_, N_, false>(a, st);
#define S_CASE(L_, P_, N_) if (kind == 1 && lmax == L_ && np == P_ && n1 == N_) return launch_wgrad_t<L_, P_, N_, true>(a, st);
    NNAP_RADIAL_SHAPES(R_CASE)
    NNAP_SPH_SHAPES(S_CASE)
#undef R_CASE
#undef S_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_wgrad_final(const float* partial, int G, int per, double* out, cudaStream_t st) {
    if (per <= 0) return cudaSuccess;
    k_wgrad_final<<<(per + 255) / 256, 256, 0, st>>>(partial, G, per, out);
    return cudaGetLastError();
}

cudaError_t launch_train_prep(const double* bF, int n, float4* bFf, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_train_prep<<<(n + 255) / 256, 256, 0, st>>>(bF, n, bFf);
    return cudaGetLastError();
}

cudaError_t launch_jvp(int kind, int lmax, int np, int n1, const JvpArgs& a, cudaStream_t st) {
#define R_CASE(P_, N_) if (kind == 0 && np == P_ && n1 == N_) return launch_radial_jvp<P_, N_>(a, st);
#define S_CASE(L_, P_, N_) if (kind == 1 && lmax == L_ && np == P_ && n1 == N_) return launch_sph_jvp<L_, P_, N_>(a, st);
    NNAP_RADIAL_SHAPES(R_CASE)
    NNAP_SPH_SHAPES(S_CASE)
#undef R_CASE
#undef S_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_net_train(const NetTrainArgs& a, cudaStream_t st) {
    const int n = a.nmax;
    if (n <= 0) return cudaSuccess;
    int Hmax = a.D, Hsum = 0;
    for (int l = 0; l < a.nlayer; ++l) {
        Hmax = Hmax > a.H[l] ? Hmax : a.H[l];
        Hsum += a.H[l];
    }
    const int warp_floats = kTrainAtoms * (2 * a.D + 2 * Hsum + 2 * Hmax);
    int wpc = 4;
    while (wpc > 1 && (size_t)wpc * warp_floats * sizeof(float) > 200 * 1024) --wpc;
    const size_t sm = sizeof(float) * (size_t)warp_floats * wpc;
    if (sm > 227 * 1024) return cudaErrorInvalidValue;
    static int lim = 0;
    if ((int)sm > lim) {
        const cudaError_t e = cudaFuncSetAttribute(k_net_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = (int)sm;
    }
    const int per_block = kTrainAtoms * wpc;
    k_net_train<<<(n + per_block - 1) / per_block, 32 * wpc, sm, st>>>(a, warp_floats);
    return cudaGetLastError();
}

cudaError_t launch_train_reduce(const ReduceArgs& a, cudaStream_t st) {
    if (a.nchunk <= 0) return cudaSuccess;
    k_train_reduce<<<dim3(a.nchunk, a.T, a.tmax), kRedThreads, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_train_final<<<dim3((a.Pmax + 255) / 256, a.T), 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace nnapgb
