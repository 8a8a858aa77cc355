// Device mathematics shared by the descriptor kernels: Chebyshev polynomials and their
// radial gradients, normalised associated Legendre functions, real spherical harmonics
// with dY/dtheta, and the radial-fuse matrix products.  Included by each translation
// unit that evaluates descriptors; every such unit holds its own copy of the Legendre
// recursion tables in constant memory and fills it with upload_sh_tables().
#pragma once

#include <cuda_runtime.h>

#include "desc.cuh"

#include <cmath>

namespace nnapgb {
namespace {

__constant__ float c_shA[91], c_shB[91], c_dup[91], c_ddn[91];
__constant__ float c_diag[13], c_sub[13];

// Recursion coefficients of the normalised associated Legendre functions for l <= 12.
cudaError_t upload_sh_tables() {
    float A[91] = {0}, B[91] = {0}, up[91] = {0}, dn[91] = {0}, dg[13] = {0}, sb[13] = {0};
    for (int l = 0; l <= 12; ++l)
        for (int m = 0; m <= l; ++m) {
            const int t = l * (l + 1) / 2 + m;
            if (l >= m + 2) {
                A[t] = (float)sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
                B[t] = (float)-sqrt(((double)(l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
            }
            up[t] = (float)sqrt((double)(l - m) * (l + m + 1));
            dn[t] = (float)sqrt((double)(l + m) * (l - m + 1));
        }
    for (int m = 0; m <= 12; ++m) {
        dg[m] = m ? (float)sqrt(1.0 + 0.5 / m) : 0.f;
        sb[m] = (float)sqrt(2.0 * m + 3.0);
    }
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(c_shA, A, sizeof(A))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_shB, B, sizeof(B))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_dup, up, sizeof(up))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_ddn, dn, sizeof(dn))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_diag, dg, sizeof(dg))) != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_sub, sb, sizeof(sb));
}

constexpr float kPi4 = 12.566370614359172f;
constexpr float kSqrt2 = 1.41421356237309515f;

__host__ __device__ constexpr int tri(int l, int m) { return l * (l + 1) / 2 + m; }

template <int N1>
__device__ __forceinline__ void cheby_f(float x, float* T) {
    T[0] = 1.f;
    if (N1 > 1) T[1] = x;
#pragma unroll
    for (int n = 2; n < N1; ++n) T[n] = 2.f * x * T[n - 1] - T[n - 2];
}
// -(1/r) d/dr T_n(1 - 2r/rc) = (2/(r rc)) n U_{n-1}(x)
template <int N1>
__device__ __forceinline__ void cheby_grad_f(float x, float mul, float* G) {
    G[0] = 0.f;
    float um2 = 0.f, um1 = mul;
#pragma unroll
    for (int n = 1; n < N1; ++n) {
        const float u = (n == 1) ? mul : ((n == 2) ? 2.f * mul * x : 2.f * x * um1 - um2);
        if (n >= 2) { um2 = um1; um1 = u; }
        G[n] = (float)n * u;
    }
}

// Radial functions of the two bases the p-space descriptor kernels serve (template
// parameter RB); a neighbour's channel value is c_p = fc sum_n W[p][n] R_n.
//   kRbNNAP (nnap_util.hpp:226-271):            u = r/rc, fc = (1 - u^2)^4, R_n = T_n(1 - 2u)
//   kRbNEP  (find_fc / find_fn, nep_core.hpp):  fc = (cos(pi u) + 1)/2,
//                                               R_n = (T_n(2(u - 1)^2 - 1) + 1)/2
// radial_f returns fc and fills R; radial_g also fills RG_n = -(1/r) dR_n/dr and sets
// fcg = -(1/r) dfc/dr.
template <int RB, int N1>
__device__ __forceinline__ float radial_f(float r, float irc, float* R) {
    const float u = r * irc;
    if (RB == kRbNEP) {
        cheby_f<N1>(2.f * (u - 1.f) * (u - 1.f) - 1.f, R);
#pragma unroll
        for (int n = 0; n < N1; ++n) R[n] = 0.5f * (R[n] + 1.f);
        return 0.5f * cospif(u) + 0.5f;
    }
    const float fc1 = 1.f - u * u, fc2 = fc1 * fc1;
    cheby_f<N1>(1.f - 2.f * u, R);
    return fc2 * fc2;
}

template <int RB, int N1>
__device__ __forceinline__ float radial_g(float r, float rc, float irc, float* R, float* RG, float* fcg) {
    const float u = r * irc;
    if (RB == kRbNEP) {
        const float x = 2.f * (u - 1.f) * (u - 1.f) - 1.f;
        cheby_f<N1>(x, R);
        cheby_grad_f<N1>(x, 2.f * (1.f - u) / (r * rc), RG);   // dx/dr = 4 (u - 1)/rc
#pragma unroll
        for (int n = 0; n < N1; ++n) R[n] = 0.5f * (R[n] + 1.f);
        float sn, cs;
        sincospif(u, &sn, &cs);
        *fcg = 0.5f * 3.14159265358979f * sn * irc / r;
        return 0.5f * cs + 0.5f;
    }
    const float fc1 = 1.f - u * u, fc2 = fc1 * fc1;
    *fcg = 8.f * fc1 * fc2 * irc * irc;
    const float x = 1.f - 2.f * u;
    cheby_f<N1>(x, R);
    cheby_grad_f<N1>(x, 2.f / (r * rc), RG);
    return fc2 * fc2;
}

// Normalised associated Legendre functions P[tri(l,m)], Condon-Shortley phase included.
template <int L>
__device__ __forceinline__ void legendre_f(float ct, float st, float* P) {
    P[0] = 0.28209479177387814f;
#pragma unroll
    for (int m = 1; m <= L; ++m) P[tri(m, m)] = -c_diag[m] * st * P[tri(m - 1, m - 1)];
#pragma unroll
    for (int m = 0; m < L; ++m) P[tri(m + 1, m)] = c_sub[m] * ct * P[tri(m, m)];
#pragma unroll
    for (int m = 0; m <= L; ++m)
#pragma unroll
        for (int l = m + 2; l <= L; ++l)
            P[tri(l, m)] = c_shA[tri(l, m)] * (ct * P[tri(l - 1, m)] + c_shB[tri(l, m)] * P[tri(l - 2, m)]);
}

struct Angles {
    float ct, st, cp, sp, dxy;
    bool pole;
};

__device__ __forceinline__ Angles angles_f(float dx, float dy, float dz, float r) {
    Angles a;
    a.dxy = hypotf(dx, dy);
    a.ct = dz / r;
    a.st = a.dxy / r;
    a.pole = a.dxy < 8.f * 1.17549435e-38f;  // numericEqual(dxy, 0) in single precision
    if (a.pole) { a.cp = 1.f; a.sp = 0.f; } else { a.cp = dx / a.dxy; a.sp = dy / a.dxy; }
    return a;
}

// Y (and optionally dY/dtheta) written to Y[lm*ys], Yt[lm*ys].
template <int L, bool DTHETA>
__device__ __forceinline__ void sph_harm(const Angles& an, float* Y, float* Yt, int ys) {
    float P[tri(L, L) + 1];
    legendre_f<L>(an.ct, an.st, P);
    float cm[L + 1], sm[L + 1];
    cm[0] = 1.f; sm[0] = 0.f;
    if (L >= 1) { cm[1] = an.cp; sm[1] = an.sp; }
#pragma unroll
    for (int m = 2; m <= L; ++m) {
        cm[m] = 2.f * an.cp * cm[m - 1] - cm[m - 2];
        sm[m] = 2.f * an.cp * sm[m - 1] - sm[m - 2];
    }
    const float r2 = 1.41421356237309515f;
#pragma unroll
    for (int l = 0; l <= L; ++l) {
        const int c0 = l * l + l;
        Y[c0 * ys] = P[tri(l, 0)];
#pragma unroll
        for (int m = 1; m <= l; ++m) {
            Y[(c0 + m) * ys] = r2 * P[tri(l, m)] * cm[m];
            Y[(c0 - m) * ys] = r2 * P[tri(l, m)] * sm[m];
        }
        if (DTHETA) {
#pragma unroll
            for (int m = 0; m <= l; ++m) {
                const float upv = (m + 1 <= l) ? c_dup[tri(l, m)] * P[tri(l, m + 1)] : 0.f;
                const float pm1 = (m >= 1) ? P[tri(l, m - 1)] : (l >= 1 ? -P[tri(l, 1)] : 0.f);
                const float dPt = 0.5f * (upv - c_ddn[tri(l, m)] * pm1);
                if (m == 0) {
                    Yt[c0 * ys] = dPt;
                } else {
                    Yt[(c0 + m) * ys] = r2 * dPt * cm[m];
                    Yt[(c0 - m) * ys] = r2 * dPt * sm[m];
                }
            }
        }
    }
}

// Radial-fuse matrices in shared memory with rows padded to N1P = N1 rounded up to 4,
// so a row is read with float4 loads: sW[(tc * T + tn) * NP * N1P + p * N1P + n].
template <int N1>
struct Fuse {
    static constexpr int N1P = (N1 + 3) & ~3;
};

template <int NP, int N1>
__device__ __forceinline__ void load_fuse(const float* __restrict__ Wg, float* sW, int T) {
    constexpr int N1P = Fuse<N1>::N1P;
    const int count = T * T * NP * N1P;
    for (int q = threadIdx.x; q < count; q += blockDim.x) {
        const int row = q / N1P, n = q - row * N1P;
        sW[q] = n < N1 ? Wg[row * N1 + n] : 0.f;
    }
}

// out[p] = sum_n Wt[p][n] * v[n]
template <int NP, int N1>
__device__ __forceinline__ void fuse_apply(const float* __restrict__ Wt, const float* v, float* out) {
    constexpr int N1P = Fuse<N1>::N1P;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float4* row = reinterpret_cast<const float4*>(Wt + p * N1P);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < N1P / 4; ++q) {
            const float4 w = row[q];
            s += w.x * v[4 * q];
            if (4 * q + 1 < N1) s += w.y * v[4 * q + 1];
            if (4 * q + 2 < N1) s += w.z * v[4 * q + 2];
            if (4 * q + 3 < N1) s += w.w * v[4 * q + 3];
        }
        out[p] = s;
    }
}

// out[n] = sum_p u[p] * Wt[p][n]
template <int NP, int N1>
__device__ __forceinline__ void fuse_apply_t(const float* __restrict__ Wt, const float* u, float* out) {
    constexpr int N1P = Fuse<N1>::N1P;
#pragma unroll
    for (int n = 0; n < N1; ++n) out[n] = 0.f;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float4* row = reinterpret_cast<const float4*>(Wt + p * N1P);
#pragma unroll
        for (int q = 0; q < N1P / 4; ++q) {
            const float4 w = row[q];
            out[4 * q] += u[p] * w.x;
            if (4 * q + 1 < N1) out[4 * q + 1] += u[p] * w.y;
            if (4 * q + 2 < N1) out[4 * q + 2] += u[p] * w.z;
            if (4 * q + 3 < N1) out[4 * q + 3] += u[p] * w.w;
        }
    }
}

}  // namespace
}  // namespace nnapgb
