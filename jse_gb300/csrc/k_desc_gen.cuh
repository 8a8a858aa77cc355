// Descriptor kernels for any basis shape the model format allows: the channel count NP
// and the radial-function count N1 = nmax + 1 (<= 21) are launch arguments, only the
// expansion degree L (<= 12) is a template parameter.  They serve every sub-basis shape
// that has no compiled instance in k_desc.cu (radial and spherical, NNAP and NEP radial
// functions), with the same mathematics, data layout and accumulation rules:
//   c_p = fc sum_n W[t_i][t_j][p][n] R_n(r)                        nnap_util.hpp:273-280
//   radial:    fp[p] = sum_j c_p                                    basis_Chebyshev.hpp:82-133
//   spherical: A[p][lm] = sum_j c_p Y_lm,
//              fp[p][l] = 4 pi/(2l+1) sum_m A[p][l,m]^2             basis_SphericalChebyshev.hpp:264-351
//   backward:  G[p][lm] = 2 4pi/(2l+1) dE/dfp[p][l] A[p][lm] (+ invariant part),
//              dY_lm = sum_p c_p G[p][lm], dc_p = sum_lm G[p][lm] Y_lm,
//              chained through fc, R_n, theta and phi               basis_SphericalChebyshev.hpp:353-525
// Layout: one warp per atom slot.  The accumulators live in shared memory (A and G as
// [rows p][K]); lanes own neighbours while the radial functions and spherical harmonics
// are evaluated, then own columns lm (forward) or keep their neighbour (backward) while
// channels are contracted in register blocks of 8.  The radial-fuse matrices are read
// through the cache.
#pragma once

#include "common.cuh"
#include "desc.cuh"
#include "pdl.cuh"
#include "sph_math.cuh"

namespace nnapgb {
namespace gen {

constexpr int kMaxN1 = 21;       // nmax <= 20 (WTypeBasis.java:56)
constexpr int kMaxWarps = 8;
constexpr int kBlk = 8;          // channels per register block

__host__ __device__ inline int r8(int v) { return (v + 7) & ~7; }
__host__ __device__ inline int r4(int v) { return (v + 3) & ~3; }

// Floats of shared memory one warp uses.
__host__ __device__ inline int sph_fwd_floats(int L, int NP) {
    const int K = (L + 1) * (L + 1), KS = K | 1;
    return r4(32 * KS) + 32 * r8(NP) + r8(NP) * K;
}
__host__ __device__ inline int sph_bwd_floats(int L, int NP) {
    const int K = (L + 1) * (L + 1), KS = K | 1;
    return r4(r8(NP) * K) + r4(3 * 32 * KS) + 32 * (r8(NP) | 1);
}
__host__ __device__ inline int rad_fwd_floats(int NP, int N1) { return 32 * r4(N1) + 32; }
__host__ __device__ inline int rad_bwd_floats(int NP) { return r4(NP); }

template <int RB>
__device__ __forceinline__ bool pair_cut_g(const DescArgs& a, int tc, int tn, float r, float& rc, float& irc) {
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

// c[p] = fc sum_n Wt[p][n] R[n] for p < NP into a shared row (zero up to NP8).
__device__ __forceinline__ void channel_row(const float* __restrict__ Wt, int NP, int NP8, int N1, float fc,
                                            const float* R, float* row) {
    for (int p = 0; p < NP; ++p) {
        const float* w = Wt + (size_t)p * N1;
        float s = 0.f;
#pragma unroll
        for (int n = 0; n < kMaxN1; ++n)
            if (n < N1) s += __ldg(w + n) * R[n];
        row[p] = fc * s;
    }
    for (int p = NP; p < NP8; ++p) row[p] = 0.f;
}

// =========================================================================== radial
template <int RB>
__global__ void __launch_bounds__(32 * kMaxWarps) k_radial_fwd_g(DescArgs a, int NP, int N1) {
    pdl_enter();
    extern __shared__ float smem[];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    const int N1P = r4(N1);
    float* sR = smem + (size_t)wl * rad_fwd_floats(NP, N1);  // [32][N1P] fc R_n per neighbour
    int* sT = reinterpret_cast<int*>(sR + 32 * N1P);          // [32] neighbour species (-1: none)
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut, irc = 1.f / a.rcut;
    const float* W = a.W + (size_t)tc * a.T * NP * N1;
    float* out = a.fp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    // lanes own channels p = lane + 32 q; the sums run over neighbours in row order
    for (int p0 = 0; p0 < NP; p0 += 32 * 4) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int base = 0; base < cnt; base += 32) {
            const int k = base + lane;
            int tn = -1;
            float R[kMaxN1];
#pragma unroll
            for (int n = 0; n < kMaxN1; ++n) R[n] = 0.f;
            if (k < cnt) {
                const float4 d = a.P.dx[(size_t)at * M + k];
                const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
                const int t = __float_as_int(d.w) - 1;
                float rcp = rc, ircp = irc;
                if (r < rc && pair_cut_g<RB>(a, tc, t, r, rcp, ircp)) {
                    tn = t;
                    const float fc = radial_f<RB, kMaxN1>(r, ircp, R);
#pragma unroll
                    for (int n = 0; n < kMaxN1; ++n) R[n] *= fc;
                }
            }
#pragma unroll
            for (int n = 0; n < kMaxN1; ++n)
                if (n < N1) sR[lane * N1P + n] = R[n];
            sT[lane] = tn;
            __syncwarp();
            const int nk = min(32, cnt - base);
            for (int kk = 0; kk < nk; ++kk) {
                const int t = sT[kk];
                if (t < 0) continue;  // uniform across the warp
                const float* Rk = sR + kk * N1P;
                const float* Wt = W + (size_t)t * NP * N1;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int p = p0 + lane + 32 * q;
                    if (p < NP) {
                        float s = 0.f;
                        for (int n = 0; n < N1; ++n) s += __ldg(Wt + (size_t)p * N1 + n) * Rk[n];
                        acc[q] += s;
                    }
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int p = p0 + lane + 32 * q;
            if (p < NP) out[p] = acc[q];
        }
    }
}

template <int RB>
__global__ void __launch_bounds__(32 * kMaxWarps) k_radial_bwd_g(DescArgs a, int NP, int N1) {
    pdl_enter();
    extern __shared__ float smem[];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sg = smem + (size_t)wl * rad_bwd_floats(NP);
    const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int p = lane; p < NP; p += 32) sg[p] = gf[p];
    __syncwarp();
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = min(a.P.count[at], M);
    const float rc = a.rcut, irc = 1.f / a.rcut;
    for (int k = lane; k < cnt; k += 32) {
        const size_t e = (size_t)at * M + k;
        const float4 d = a.P.dx[e];
        const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        const int tn = __float_as_int(d.w) - 1;
        float rcp = rc, ircp = irc;
        if (r < rc && pair_cut_g<RB>(a, tc, tn, r, rcp, ircp)) {
            float R[kMaxN1], RG[kMaxN1], fcg;
            const float fc = radial_g<RB, kMaxN1>(r, rcp, ircp, R, RG, &fcg);
            const float* Wt = a.W + ((size_t)tc * a.T + tn) * NP * N1;
            float v[kMaxN1];
#pragma unroll
            for (int n = 0; n < kMaxN1; ++n) v[n] = 0.f;
            for (int p = 0; p < NP; ++p) {
                const float gp = sg[p];
#pragma unroll
                for (int n = 0; n < kMaxN1; ++n)
                    if (n < N1) v[n] += gp * __ldg(Wt + (size_t)p * N1 + n);
            }
            float dfc = 0.f, drn = 0.f;
#pragma unroll
            for (int n = 0; n < kMaxN1; ++n)
                if (n < N1) {
                    dfc += v[n] * R[n];
                    drn += v[n] * RG[n];
                }
            const float gr = dfc * fcg + fc * drn;
            g = make_float4(gr * d.x, gr * d.y, gr * d.z, 0.f);
        }
        if (a.accumulate) {
            const float4 o = a.P.g[e];
            a.P.g[e] = make_float4(o.x + g.x, o.y + g.y, o.z + g.z, 0.f);
        } else {
            a.P.g[e] = g;
        }
    }
}

// =========================================================================== spherical
template <int L, int RB>
__global__ void __launch_bounds__(32 * kMaxWarps) k_sph_fwd_g(DescArgs a, int NP, int N1) {
    pdl_enter();
    constexpr int K = (L + 1) * (L + 1), KS = K | 1;
    extern __shared__ float smem[];
    const int NP8 = r8(NP);
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sY = smem + (size_t)wl * sph_fwd_floats(L, NP);  // [32][KS] Y of each lane's neighbour
    float* sC = sY + r4(32 * KS);                             // [32][NP8] c of each lane's neighbour
    float* sA = sC + 32 * NP8;                                // [NP8][K] accumulators
    for (int q = lane; q < NP8 * K; q += 32) sA[q] = 0.f;
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = a.sub_dx ? a.sub_count[at] : min(a.P.count[at], M);
    const float4* rdx = (a.sub_dx ? a.sub_dx : a.P.dx) + (size_t)at * M;
    const float rc = a.rcut, irc = 1.f / a.rcut;
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float* y = sY + lane * KS;
        float* cr = sC + lane * NP8;
        bool valid = false;
        if (k < cnt) {
            const float4 d = rdx[k];
            const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            const int tn = __float_as_int(d.w) - 1;
            float rcp = rc, ircp = irc;
            if (r < rc && pair_cut_g<RB>(a, tc, tn, r, rcp, ircp)) {
                valid = true;
                float R[kMaxN1];
                const float fc = radial_f<RB, kMaxN1>(r, ircp, R);
                channel_row(a.W + ((size_t)tc * a.T + tn) * NP * N1, NP, NP8, N1, fc, R, cr);
                sph_harm<L, false>(angles_f(d.x, d.y, d.z, r), y, nullptr, 1);
            }
        }
        if (!valid) {
            for (int q = 0; q < K; ++q) y[q] = 0.f;
            for (int p = 0; p < NP8; ++p) cr[p] = 0.f;
        }
        __syncwarp();
        const int nk = min(32, cnt - base);
        for (int lm = lane; lm < K; lm += 32) {
            for (int p0 = 0; p0 < NP8; p0 += kBlk) {
                float acc[kBlk];
#pragma unroll
                for (int q = 0; q < kBlk; ++q) acc[q] = sA[(p0 + q) * K + lm];
#pragma unroll 4
                for (int kk = 0; kk < nk; ++kk) {
                    const float yv = sY[kk * KS + lm];
                    const float4 c0 = *reinterpret_cast<const float4*>(sC + kk * NP8 + p0);
                    const float4 c1 = *reinterpret_cast<const float4*>(sC + kk * NP8 + p0 + 4);
                    acc[0] = fmaf(c0.x, yv, acc[0]); acc[1] = fmaf(c0.y, yv, acc[1]);
                    acc[2] = fmaf(c0.z, yv, acc[2]); acc[3] = fmaf(c0.w, yv, acc[3]);
                    acc[4] = fmaf(c1.x, yv, acc[4]); acc[5] = fmaf(c1.y, yv, acc[5]);
                    acc[6] = fmaf(c1.z, yv, acc[6]); acc[7] = fmaf(c1.w, yv, acc[7]);
                }
#pragma unroll
                for (int q = 0; q < kBlk; ++q) sA[(p0 + q) * K + lm] = acc[q];
            }
        }
        __syncwarp();
    }
    // A to global memory (rows p < NP of sA are exactly A[p][lm]), power spectrum
    float* Aout = a.A + (size_t)w * NP * K;
    for (int q = lane; q < NP * K; q += 32) Aout[q] = sA[q];
    float* out = a.fp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
    for (int e = lane; e < NP * a.nl2; e += 32) {
        const int p = e / a.nl2, l = e - p * a.nl2;
        float s = 0.f;
        for (int m = 0; m <= 2 * l; ++m) {
            const float v = sA[p * K + l * l + m];
            s += v * v;
        }
        out[p * a.sl + l] = kPi4 / (float)(2 * l + 1) * s;
    }
}

template <int L, int RB>
__global__ void __launch_bounds__(32 * kMaxWarps) k_sph_bwd_g(DescArgs a, int NP, int N1) {
    pdl_enter();
    constexpr int K = (L + 1) * (L + 1), KS = K | 1;
    extern __shared__ float smem[];
    const int NP8 = r8(NP), NPS = NP8 | 1;
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + wl;
    const int s0 = a.range[a.t0], s1 = a.range[a.t1];
    if (s0 + w >= s1) return;
    float* sG = smem + (size_t)wl * sph_bwd_floats(L, NP);  // [NP8][K] G rows
    float* sY = sG + r4(NP8 * K);                            // [32][KS] Y
    float* sYt = sY + 32 * KS;                               // [32][KS] dY/dtheta
    float* sdY = sYt + 32 * KS;                              // [32][KS] dE/dY
    float* sC = sY + r4(3 * 32 * KS);                        // [32][NPS] c
    const int at = a.perm[s0 + w];
    const int tc = a.type[at] - 1;
    const int M = a.P.M, cnt = a.sub_dx ? a.sub_count[at] : min(a.P.count[at], M);
    const float4* rdx = (a.sub_dx ? a.sub_dx : a.P.dx) + (size_t)at * M;
    const float rc = a.rcut, irc = 1.f / a.rcut;
    {
        const float* Ain = a.A + (size_t)w * NP * K;
        const float* gf = a.gfp + (size_t)(s0 + w) * a.fp_stride + a.fp_off;
        for (int q = lane; q < NP8 * K; q += 32) {
            const int p = q / K, lm = q - p * K;
            float v = 0.f;
            if (p < NP) {
                int l = 0;
                while ((l + 1) * (l + 1) <= lm) ++l;
                if (l < a.nl2) v = 2.f * kPi4 / (float)(2 * l + 1) * gf[p * a.sl + l] * Ain[p * K + lm];
                if (a.Gx) v += a.Gx[(size_t)w * NP * K + p * K + lm];
            }
            sG[q] = v;
        }
        __syncwarp();
    }
    float* y = sY + lane * KS;
    float* yt = sYt + lane * KS;
    float* dy = sdY + lane * KS;
    float* cr = sC + lane * NPS;
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        float r = 1.f, rcp = rc, ircp = irc;
        bool valid = false;
        if (k < cnt) {
            d = rdx[k];
            r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
            valid = r < rc;
        }
        const int tn = valid ? __float_as_int(d.w) - 1 : 0;
        if (valid) valid = pair_cut_g<RB>(a, tc, tn, r, rcp, ircp);
        const float* Wt = a.W + ((size_t)tc * a.T + tn) * NP * N1;
        if (valid) {
            float R[kMaxN1];
            const float fc = radial_f<RB, kMaxN1>(r, ircp, R);
            channel_row(Wt, NP, NP8, N1, fc, R, cr);
            sph_harm<L, true>(angles_f(d.x, d.y, d.z, r), y, yt, 1);
        } else {
            for (int p = 0; p < NP8; ++p) cr[p] = 0.f;
            for (int q = 0; q < K; ++q) { y[q] = 0.f; yt[q] = 0.f; }
        }
        for (int q = 0; q < K; ++q) dy[q] = 0.f;
        // channel blocks: dY_lm += sum_p c_p G[p][lm]; dc_p = sum_lm G[p][lm] Y_lm; then
        // v_n += sum_p dc_p W[p][n]
        float v[kMaxN1];
#pragma unroll
        for (int n = 0; n < kMaxN1; ++n) v[n] = 0.f;
        for (int p0 = 0; p0 < NP8; p0 += kBlk) {
            float c8[kBlk], dc8[kBlk];
#pragma unroll
            for (int q = 0; q < kBlk; ++q) {
                c8[q] = cr[p0 + q];
                dc8[q] = 0.f;
            }
#pragma unroll 7
            for (int lm = 0; lm < K; ++lm) {
                const float yv = y[lm];
                float s = 0.f;
#pragma unroll
                for (int q = 0; q < kBlk; ++q) {
                    const float gq = sG[(p0 + q) * K + lm];
                    s = fmaf(c8[q], gq, s);
                    dc8[q] = fmaf(gq, yv, dc8[q]);
                }
                dy[lm] += s;
            }
            if (valid) {
#pragma unroll
                for (int q = 0; q < kBlk; ++q) {
                    if (p0 + q >= NP) break;
                    const float* wr = Wt + (size_t)(p0 + q) * N1;
#pragma unroll
                    for (int n = 0; n < kMaxN1; ++n)
                        if (n < N1) v[n] = fmaf(dc8[q], __ldg(wr + n), v[n]);
                }
            }
        }
        if (k < cnt) {
            const size_t e = (size_t)at * M + (a.sub_dx ? a.sub_pos[(size_t)at * M + k] : k);
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                float gth = 0.f, gph = 0.f;
#pragma unroll
                for (int l = 0; l <= L; ++l) {
                    const int c0 = l * l + l;
                    gth += dy[c0] * yt[c0];
#pragma unroll
                    for (int m = 1; m <= l; ++m) {
                        const float dYp = dy[c0 + m], dYm = dy[c0 - m];
                        gth += dYp * yt[c0 + m] + dYm * yt[c0 - m];
                        gph += (float)m * (dYm * y[c0 + m] - dYp * y[c0 - m]);
                    }
                }
                float R[kMaxN1], RG[kMaxN1], fcg;
                const float fc = radial_g<RB, kMaxN1>(r, rcp, ircp, R, RG, &fcg);
                float dfc = 0.f, drn = 0.f;
#pragma unroll
                for (int n = 0; n < kMaxN1; ++n)
                    if (n < N1) {
                        dfc += v[n] * R[n];
                        drn += v[n] * RG[n];
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

}  // namespace gen
}  // namespace nnapgb
