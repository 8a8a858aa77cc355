// Spherical-Chebyshev forward on the tensor cores (tcgen05, kind::f16, FP32 accumulation in
// TMEM).  Included by k_desc.cu after the FP32-pipe kernels.
//
// For fuse matrices of the form W[tc][tn][p][n] = alpha[tc][tn][p] delta(n, p mod N1) the
// expansion coefficients of one atom are a single product over its neighbours,
//   A[p][lm] = sum_j Y_j[lm] c_j[p],   c_j[p] = alpha[tc][tn_j][p] fc_j T_{p mod N1}(r_j)
// (basis_SphericalChebyshev.hpp:264-351 with the fuse step of nnap_util.hpp:273-280), i.e.
// D = Y^T C with M = 64 rows (lm; (L+1)^2 <= 64), N = NP rounded up to 8 columns (p) and
// K = 16 neighbours per MMA.  The descriptors are then fp[p][l] = 4 pi/(2l+1) sum_m A^2 as
// in k_sph_fwd_n.
//
// Precision.  Each FP32 operand x is split into FP16 hi = fp16(x) and lo = fp16(x - hi), and
// each product is formed as hi*hi + lo*hi + hi*lo: about 22 significant bits per operand
// where lo is a normal FP16 number (|x| >= 2^-3) and an absolute error below 2^-25
// otherwise, well inside FP32 descriptor accuracy.  The operands are bounded (|Y_lm| <= 1.5
// for l <= 12, |fc T_n| <= 1), and the host uses this kernel only when every |alpha| is at
// most kTcAlphaMax, so hi never overflows FP16.
//
// Organisation.  A CTA of 4 warps takes 4 atom slots per round, one per warp.  A warp walks
// its atom's row 32 neighbours at a time (lane = neighbour): it evaluates fc T_n, c and Y
// into registers, waits for its own previous MMAs, stores the split operands into its two
// 16-neighbour chunks of shared memory (MN-major, no swizzle: core matrices of 8
// neighbours x 16 bytes, LBO = the stride between neighbour groups, SBO = 128 bytes between
// groups of 8 rows or columns), and one lane issues the 3 MMAs of each chunk into the
// atom's 32 TMEM columns and commits them to the warp's mbarrier.  After the round's last
// MMAs all 4 warps read the 4 tiles back: an M = 64 tile keeps rows 16q..16q+15 in TMEM
// lanes 32q..32q+15, which warp q reads.  They write A and form the power spectrum from
// A^2 in shared memory (the operand buffers, free once the MMAs are done).  Every wait on
// an mbarrier is bounded; a wait that gives up raises ERRBIT_TIMEOUT.
#pragma once

#include <cuda_fp16.h>

#include "tc_util.cuh"

namespace nnapgb {
namespace {

constexpr int kFwdTcWarps = 4;

template <int L, int NP>
struct SphTcShape {
    static constexpr int KM = (L + 1) * (L + 1);   // tile rows in use
    static constexpr int NPN = (NP + 7) & ~7;       // MMA N
    static constexpr int NCA = (KM + 7) / 8;        // 8-row groups of Y a neighbour writes
    static constexpr int NCB = NPN / 8;             // 8-column groups of c a neighbour writes
    static constexpr int ABYTES = 64 * 16 * 2;      // one FP16 image of a chunk's Y^T
    static constexpr int BBYTES = 16 * NPN * 2;     // one FP16 image of a chunk's C
    static constexpr int CHUNK = 2 * ABYTES + 2 * BBYTES;
    static constexpr int WARP_BYTES = 2 * CHUNK;
    static constexpr int AL_BYTES = (kFwdTypes * kFwdTypes * NP * 4 + 127) & ~127;
    static constexpr int A2_BYTES = kFwdTcWarps * NP * KM * 4;
    static constexpr int OPS = kFwdTcWarps * WARP_BYTES > A2_BYTES ? kFwdTcWarps * WARP_BYTES : A2_BYTES;
    // at least 46 KB, so that at most four CTAs (4 x 128 TMEM columns) share an SM
    static constexpr int SMEM = AL_BYTES + OPS > 47104 ? AL_BYTES + OPS : 47104;
    // lmax 6 or 7: the tile's 64 rows are mostly in use.  Below that the FP32-pipe kernel,
    // whose work scales with (L+1)^2, is faster (lmax 4, 131k-atom glass: 0.34 against
    // 0.41 ms; lmax 6, 1024-structure batch: 2.41 against 2.08 ms on the tensor cores)
    static constexpr bool fits = KM >= 49 && KM <= 64 && NPN <= 32;
};

__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for this architecture; no swizzle
    return d;
}

// 8 FP32 values -> FP16 hi and lo images (16 bytes each, element 0 at the lowest address).
__device__ __forceinline__ void split_f16x8(const float* v, uint4& hi, uint4& lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __half2 hh = __floats2half2_rn(v[2 * q], v[2 * q + 1]);
        const float2 hf = __half22float2(hh);
        const __half2 ll = __floats2half2_rn(v[2 * q] - hf.x, v[2 * q + 1] - hf.y);
        h[q] = *reinterpret_cast<const uint32_t*>(&hh);
        l[q] = *reinterpret_cast<const uint32_t*>(&ll);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// 32 TMEM columns of this warp's lane quarter, waited for in the same statement.
__device__ __forceinline__ void tmem_ld32_wait(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

template <int L, int NP, int N1>
__global__ void __launch_bounds__(32 * kFwdTcWarps, 4) k_sph_fwd_tc(DescArgs a) {
    pdl_enter();
    using S = SphTcShape<L, NP>;
    constexpr int KM = S::KM, NPN = S::NPN;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[kFwdTcWarps];
    __shared__ uint32_t s_tmem;
    __shared__ int s_cnt[kFwdTcWarps];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntab = a.T * kFwdTypes * NP;
    float* sAl = reinterpret_cast<float*>(smem);
    uint8_t* ops = smem + S::AL_BYTES;
    float* sA2 = reinterpret_cast<float*>(ops);  // [warp][NP][KM] once a round's MMAs are done
    for (int q = tid; q < ntab; q += blockDim.x) sAl[q] = a.fwd_alpha[q];
    if (tid == 0) {
        for (int q = 0; q < kFwdTcWarps; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::smem_u32(&mbar[q])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(&s_tmem)),
                     "r"(32 * kFwdTcWarps)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = s_tmem;
    const uint32_t mb = tc::smem_u32(&mbar[warp]);
    uint32_t phase = 0;
    bool ok = true;
    const int s0 = a.range[a.t0], nslot = a.range[a.t1] - s0;
    const int M = a.P.M;
    const float rc = a.rcut, irc = 1.f / a.rcut;
    uint8_t* wops = ops + warp * S::WARP_BYTES;
    const uint32_t wops_s = tc::smem_u32(wops);
    // kind::f16: D F32, A = B = F16, both MN-major, N = NPN, M = 64
    const uint32_t idesc = (1u << 4) | (1u << 15) | (1u << 16) | ((uint32_t)(NPN >> 3) << 17) | (4u << 24);
    const uint32_t dcol = tbase + 32u * warp;
    const int ch = lane >> 4, kk = lane & 15;
    uint8_t* cbase = wops + ch * S::CHUNK;
    const int aoff = (kk >> 3) * 1024 + (kk & 7) * 16;
    const int boff = (kk >> 3) * (NPN / 8) * 128 + (kk & 7) * 16;

    for (int r0 = blockIdx.x * kFwdTcWarps; r0 < nslot; r0 += gridDim.x * kFwdTcWarps) {
        const int slot = r0 + warp;
        int at = 0, tc = 0, cnt = 0;
        if (slot < nslot) {
            at = a.perm[s0 + slot];
            tc = a.type[at] - 1;
            cnt = min(a.P.count[at], M);
        }
        if (lane == 0) s_cnt[warp] = cnt;
        const float* al = sAl + tc * kFwdTypes * NP;
        for (int b0 = 0; b0 < cnt; b0 += 32) {
            const int k = b0 + lane;
            float y[KM];
            float c[NPN];
#pragma unroll
            for (int p = 0; p < NPN; ++p) c[p] = 0.f;
            bool valid = false;
            if (k < cnt) {
                const float4 d = a.P.dx[(size_t)at * M + k];
                const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
                if (r < rc) {
                    valid = true;
                    const int tn = __float_as_int(d.w) - 1;
                    const float u = r * irc, fc1 = 1.f - u * u, fc2 = fc1 * fc1, fc = fc2 * fc2;
                    float fT[N1];
                    cheby_f<N1>(1.f - 2.f * u, fT);
#pragma unroll
                    for (int p = 0; p < NP; ++p) c[p] = al[tn * NP + p] * (fc * fT[p % N1]);
                    const Angles an = angles_f(d.x, d.y, d.z, r);
                    sph_harm<L, false>(an, y, nullptr, 1);
                }
            }
            if (!valid) {
#pragma unroll
                for (int q = 0; q < KM; ++q) y[q] = 0.f;
            }
            // the warp's previous MMAs read these chunks
            if (b0 > 0) {
                ok = tc::mbar_wait(mb, phase) && ok;
                phase ^= 1;
            }
#pragma unroll
            for (int g = 0; g < S::NCA; ++g) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = 8 * g + e < KM ? y[8 * g + e] : 0.f;
                uint4 hi, lo;
                split_f16x8(v, hi, lo);
                *reinterpret_cast<uint4*>(cbase + g * 128 + aoff) = hi;
                *reinterpret_cast<uint4*>(cbase + S::ABYTES + g * 128 + aoff) = lo;
            }
#pragma unroll
            for (int g = 0; g < S::NCB; ++g) {
                uint4 hi, lo;
                split_f16x8(c + 8 * g, hi, lo);
                *reinterpret_cast<uint4*>(cbase + 2 * S::ABYTES + g * 128 + boff) = hi;
                *reinterpret_cast<uint4*>(cbase + 2 * S::ABYTES + S::BBYTES + g * 128 + boff) = lo;
            }
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0) {
                tc::fence_after();
                const int nch = min(2, (cnt - b0 + 15) >> 4);
                for (int q = 0; q < nch; ++q) {
                    const uint32_t cb = wops_s + q * S::CHUNK;
                    const uint64_t ah = tc_sdesc(cb, 1024, 128), alo = tc_sdesc(cb + S::ABYTES, 1024, 128);
                    const uint64_t bh = tc_sdesc(cb + 2 * S::ABYTES, (NPN / 8) * 128, 128);
                    const uint64_t bl = tc_sdesc(cb + 2 * S::ABYTES + S::BBYTES, (NPN / 8) * 128, 128);
                    tc::mma_bf16(dcol, ah, bh, idesc, (b0 > 0 || q > 0) ? 1u : 0u);
                    tc::mma_bf16(dcol, alo, bh, idesc, 1u);
                    tc::mma_bf16(dcol, ah, bl, idesc, 1u);
                }
                tc::mma_commit(mb);
            }
            __syncwarp();
        }
        if (cnt > 0) {
            ok = tc::mbar_wait(mb, phase) && ok;
            phase ^= 1;
        }
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        // the 4 tiles: warp q holds rows lm = 16q + lane (lanes 0..15)
        for (int w4 = 0; w4 < kFwdTcWarps; ++w4) {
            const int sl = r0 + w4;
            if (sl >= nslot) break;
            float v[32];
            tmem_ld32_wait(tbase + ((uint32_t)(32 * warp) << 16) + 32u * w4, v);
            const int lm = 16 * warp + lane;
            if (lane < 16 && lm < KM) {
                const bool any = s_cnt[w4] > 0;
                float* Aout = a.A + (size_t)sl * NP * KM;
                float* a2 = sA2 + w4 * NP * KM;
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    const float x = any ? v[p] : 0.f;
                    Aout[p * KM + lm] = x;
                    a2[p * KM + lm] = x * x;
                }
            }
        }
        __syncthreads();
        const int nout = NP * a.nl2;
        for (int e = tid; e < kFwdTcWarps * nout; e += blockDim.x) {
            const int w4 = e / nout, rr = e - w4 * nout;
            const int sl = r0 + w4;
            if (sl >= nslot) continue;
            const int p = rr / a.nl2, l = rr - p * a.nl2;
            const float* a2 = sA2 + w4 * NP * KM + p * KM + l * l;
            float s = 0.f;
            for (int m = 0; m <= 2 * l; ++m) s += a2[m];
            a.fp[(size_t)(s0 + sl) * a.fp_stride + a.fp_off + p * a.sl + l] = kPi4 / (float)(2 * l + 1) * s;
        }
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    }
    if (!ok && lane == 0 && a.err) atomicOr(a.err, ERRBIT_TIMEOUT);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(32 * kFwdTcWarps)
                     : "memory");
}

template <int L, int NP, int N1>
cudaError_t launch_sph_fwd_tc(const DescArgs& a, cudaStream_t st) {
    using S = SphTcShape<L, NP>;
    static int lim = 0;
    if (S::SMEM > lim) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_sph_fwd_tc<L, NP, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
        if (e != cudaSuccess) return e;
        lim = S::SMEM;
    }
    const int rounds = (a.nmax + kFwdTcWarps - 1) / kFwdTcWarps;
    const int grid = rounds < 4 * a.tc_sms ? rounds : 4 * a.tc_sms;
    return launch_pdl(&k_sph_fwd_tc<L, NP, N1>, dim3(grid), dim3(32 * kFwdTcWarps), (size_t)S::SMEM, st, a);
}

}  // namespace
}  // namespace nnapgb
