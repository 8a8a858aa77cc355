// Tensor-core evaluation of the per-species network and its input gradient (the
// mixed-precision path), on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// Mathematics: normedNnForward / normedNnBackward (nnap_main.hpp:267-323) with two SiLU
// hidden layers (nn_FeedForward.hpp:8-261):
//   X  = (fp - mu)/sigma                      [128 x Dp]   Dp = D rounded up to 16
//   Z1 = X W1^T + b1, A1 = silu(Z1)           [128 x H1]   GEMM 1 (N = H1, K = Dp)
//   Z2 = A1 W2^T + b2, A2 = silu(Z2)          [128 x H2]   GEMM 2 (N = H2, K = H1)
//   E  = (w_o . A2 + b_o) sigma_E + mu_E      (FP32 on the CUDA cores, FP64 output)
//   dZ2 = sigma_E w_o * silu'(Z2)
//   dA1 = dZ2 W2                              [128 x H1]   GEMM 3 (N = H1, K = H2)
//   dZ1 = dA1 * silu'(Z1)
//   dX  = dZ1 W1                              [128 x Dp]   GEMM 4 (N = Dp, K = H1)
//   dE/dfp = dX / sigma
// Operands are BF16 and every product is split as hi*hi + lo*hi + hi*lo with
// x = hi + lo (both BF16), accumulated in FP32 in TMEM: three kind::f16 MMAs per
// 16-wide K step keep the network error near FP32 level (about 1e-6 eV per atom)
// while the arithmetic stays on the BF16 tensor pipe.
//
// One CTA of 128 threads owns a 128-atom tile; thread t owns row t (one atom) in every
// epilogue, so TMEM lane t is read by thread t with tcgen05.ld 32x32b.  One thread
// issues the MMAs; completion is signalled through an mbarrier (tcgen05.commit) whose
// waits are bounded in time and raise ERRBIT_TIMEOUT instead of hanging.
// Shared-memory operands use the no-swizzle K-major canonical layout: 8x8 core
// matrices of 128 bytes, adjacent in K at LBO = 128 bytes and in M/N at
// SBO = (K/8)*128 bytes.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "net_tc.cuh"
#include "pdl.cuh"
#include "tc_util.cuh"

namespace nnapgb {

namespace {

using namespace ::nnapgb::tc;

// SPLIT threads per tile row in the epilogues (a launch parameter: 2 or 4); warp w
// reads TMEM lanes 32 * (w % 4) .. 32 * (w % 4) + 31.

struct TCLayout {
    int Dp, H1, H2;
    // byte offsets inside the weight image (all multiples of 1024)
    int w1, w2, w2t, w1t, fvec, bytes;  // each operand image holds hi then lo
    int fmu, fisig, fb1, fb2, fwo;      // float offsets inside the FP32 vector block
    int ncols;                          // TMEM columns allocated
    int z1, z2, da1, dx;                // TMEM column offsets
};

__host__ __device__ inline int align1k(int b) { return (b + 1023) & ~1023; }

TCLayout make_layout(int D, int H1, int H2) {
    TCLayout L;
    L.Dp = (D + 15) & ~15;
    L.H1 = H1;
    L.H2 = H2;
    int off = 0;
    L.w1 = off; off = align1k(off + 2 * 2 * H1 * L.Dp);
    L.w2 = off; off = align1k(off + 2 * 2 * H2 * H1);
    L.w2t = off; off = align1k(off + 2 * 2 * H1 * H2);
    L.w1t = off; off = align1k(off + 2 * 2 * L.Dp * H1);
    L.fvec = off;
    L.fmu = 0;
    L.fisig = L.Dp;
    L.fb1 = 2 * L.Dp;
    L.fb2 = L.fb1 + H1;
    L.fwo = L.fb2 + H2;
    off = align1k(off + 4 * (L.fwo + H2 + 4));
    L.bytes = off;
    L.z1 = 0;
    L.z2 = H1;
    L.da1 = H1 + H2;
    L.dx = 2 * H1 + H2;
    const int need = L.dx + L.Dp;
    L.ncols = 32;
    while (L.ncols < need) L.ncols *= 2;
    return L;
}

// Element (r, k) of an R x K K-major operand in the no-swizzle core-matrix layout.
inline size_t cm_index(int r, int k, int K) { return ((size_t)(r >> 3) * (K >> 3) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7); }

uint16_t bf16_bits(float f) {
    __nv_bfloat16 b = __float2bfloat16_rn(f);
    uint16_t u;
    std::memcpy(&u, &b, 2);
    return u;
}
float bf16_val(uint16_t u) {
    uint32_t w = (uint32_t)u << 16;
    float f;
    std::memcpy(&f, &w, 4);
    return f;
}

// Write the hi and lo images of an R x K matrix M(r, k) (zero outside rows/cols given).
template <class F>
void put_operand(std::vector<uint8_t>& img, int byte_off, int R, int K, F&& M) {
    uint16_t* hi = reinterpret_cast<uint16_t*>(img.data() + byte_off);
    uint16_t* lo = hi + (size_t)R * K;
    for (int r = 0; r < R; ++r)
        for (int k = 0; k < K; ++k) {
            const float v = (float)M(r, k);
            const uint16_t h = bf16_bits(v);
            const uint16_t l = bf16_bits(v - bf16_val(h));
            hi[cm_index(r, k, K)] = h;
            lo[cm_index(r, k, K)] = l;
        }
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }

// Species t0 .. t0+nt-1 of one launch; all share one layout (D, H1, H2).  Tiles are
// numbered species by species; a CTA stages a species' weights when its next tile
// belongs to another species than the last one.
struct TcParams {
    const int* perm;
    const int* range;     // device: first slot of each species
    int t0, nt;
    const float* fp;
    int fp_stride, D;
    float* gfp;
    double* e_atom;
    const uint8_t* img[kMaxTypes];  // weight image per species (global)
    float bo[kMaxTypes];
    double mu_e[kMaxTypes], sigma_e[kMaxTypes];
    int* err;
};

template <int SPLIT>
__global__ void __launch_bounds__(128 * SPLIT, 1) k_net_tc(TcParams p, TCLayout L) {
    pdl_enter();
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_tstart[kMaxTypes + 1];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int part = tid >> 7;  // column share of this thread in the epilogues
    __shared__ float s_e[SPLIT][128];
    const int Dp = L.Dp, H1 = L.H1, H2 = L.H2;
    uint8_t* sw = smem;                                       // weight image
    uint8_t* sx = smem + L.bytes;                             // X / dZ1 operand (hi, lo)
    const int xbytes = align1k(2 * 2 * 128 * (Dp > H1 ? Dp : H1));
    uint8_t* sa = sx + xbytes;                                // A1 / dZ2 operand (hi, lo)
    const int ab = 2 * 128 * (H1 > H2 ? H1 : H2);             // bytes of one (hi or lo) activation image
    const float* fv = reinterpret_cast<const float*>(sw + L.fvec);

    if (tid == 0) {
        s_tstart[0] = 0;
        for (int t = 0; t < p.nt; ++t)
            s_tstart[t + 1] = s_tstart[t] + (p.range[p.t0 + t + 1] - p.range[p.t0 + t] + 127) / 128;
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(L.ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = tmem_base;
    const uint32_t tlane = tbase + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t mb = smem_u32(&mbar);
    uint32_t phase = 0;
    bool ok = true;

    const uint32_t w1h = smem_u32(sw + L.w1), w1l = w1h + 2 * H1 * Dp;
    const uint32_t w2h = smem_u32(sw + L.w2), w2l = w2h + 2 * H2 * H1;
    const uint32_t w2th = smem_u32(sw + L.w2t), w2tl = w2th + 2 * H1 * H2;
    const uint32_t w1th = smem_u32(sw + L.w1t), w1tl = w1th + 2 * Dp * H1;
    const uint32_t xh = smem_u32(sx), xl = xh + 2 * 128 * (Dp > H1 ? Dp : H1);
    const uint32_t ah = smem_u32(sa), al = ah + ab;
    uint8_t* sx_lo = sx + 2 * 128 * (Dp > H1 ? Dp : H1);
    uint8_t* sa_lo = sa + ab;

    const int total = s_tstart[p.nt];
    int staged = -1;
    for (int gt = blockIdx.x; gt < total && ok; gt += gridDim.x) {
        int ts = 0;
        while (gt >= s_tstart[ts + 1]) ++ts;
        const int tile = gt - s_tstart[ts];
        if (ts != staged) {  // stage this species' weight image (no MMA is in flight here)
            __syncthreads();
            const uint4* src = reinterpret_cast<const uint4*>(p.img[ts]);
            uint4* dst = reinterpret_cast<uint4*>(sw);
            for (int q = tid; q < L.bytes / 16; q += (128 * SPLIT)) dst[q] = src[q];
            fence_async_smem();
            __syncthreads();
            staged = ts;
        }
        const int s0 = p.range[p.t0 + ts], s1 = p.range[p.t0 + ts + 1];
        const int row = tid & 127;
        const int slot = s0 + tile * 128 + row;
        const bool valid = slot < s1;
        // ---- X = (fp - mu) / sigma, split into hi / lo.  Warp-cooperative: the lanes of a
        // warp take 8 rows (one core-matrix block) x 4 chunks of 8 columns, so the global
        // reads are 128-byte row segments and the shared stores fill 512 contiguous bytes
        {
            const int nch = Dp >> 3, ngr = (nch + 3) >> 2;
            const int r8 = lane & 7, cq = lane >> 3;
            for (int it = warp; it < 16 * ngr; it += 4 * SPLIT) {
                const int rb = it / ngr, c = 4 * (it - rb * ngr) + cq;
                if (c >= nch) continue;
                const int r = rb * 8 + r8, k0 = 8 * c;
                const int sl = s0 + tile * 128 + r;
                float v[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = 0.f;
                if (sl < s1) {
                    const float* fr = p.fp + (size_t)sl * p.fp_stride + k0;
                    if (k0 + 8 <= p.D) {
                        const float4 a = reinterpret_cast<const float4*>(fr)[0];
                        const float4 b = reinterpret_cast<const float4*>(fr)[1];
                        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
                        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
                    } else {
#pragma unroll
                        for (int q = 0; q < 8; ++q) v[q] = k0 + q < p.D ? fr[q] : 0.f;
                    }
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int k = k0 + q;
                        v[q] = k < p.D ? (v[q] - fv[L.fmu + k]) * fv[L.fisig + k] : 0.f;
                    }
                }
                store_split8(sx, sx_lo, r, k0, Dp, v);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            issue_gemm(tbase + L.z1, xh, xl, w1h, w1l, Dp, H1);
            mma_commit(mb);
        }
        ok = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
        // ---- A1 = silu(Z1 + b1)
        for (int c0 = 16 * part; c0 < H1; c0 += 16 * SPLIT) {
            float z[16];
            tmem_ld16(tlane + L.z1 + c0, z);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const float zz = z[q] + fv[L.fb1 + c0 + q];
                z[q] = zz * sigmoidf_(zz);
            }
            store_split8(sa, sa_lo, row, c0, H1, z);
            store_split8(sa, sa_lo, row, c0 + 8, H1, z + 8);
        }
        fence_before();
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            issue_gemm(tbase + L.z2, ah, al, w2h, w2l, H1, H2);
            mma_commit(mb);
        }
        ok = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
        // ---- energy and dZ2 = sigma_E w_o silu'(Z2 + b2)
        const float se = (float)p.sigma_e[ts];
        float e = 0.f;
        for (int c0 = 16 * part; c0 < H2; c0 += 16 * SPLIT) {
            float z[16];
            tmem_ld16(tlane + L.z2 + c0, z);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const float zz = z[q] + fv[L.fb2 + c0 + q];
                const float s = sigmoidf_(zz);
                const float wo = fv[L.fwo + c0 + q];
                e += wo * (zz * s);
                z[q] = se * wo * (s * (1.f + zz * (1.f - s)));
            }
            store_split8(sa, sa_lo, row, c0, H2, z);
            store_split8(sa, sa_lo, row, c0 + 8, H2, z + 8);
        }
        s_e[part][row] = e;
        fence_before();
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            issue_gemm(tbase + L.da1, ah, al, w2th, w2tl, H2, H1);
            mma_commit(mb);
        }
        ok = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
        if (part == 0 && valid) {  // energy: the four column shares added in a fixed order
            float e = s_e[0][row];
#pragma unroll
            for (int q = 1; q < SPLIT; ++q) e += s_e[q][row];
            p.e_atom[p.perm[slot]] = ((double)e + (double)p.bo[ts]) * p.sigma_e[ts] + p.mu_e[ts];
        }
        // ---- dZ1 = dA1 * silu'(Z1 + b1)
        for (int c0 = 16 * part; c0 < H1; c0 += 16 * SPLIT) {
            float g[16], z[16];
            tmem_ld16(tlane + L.da1 + c0, g);
            tmem_ld16(tlane + L.z1 + c0, z);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const float zz = z[q] + fv[L.fb1 + c0 + q];
                const float s = sigmoidf_(zz);
                g[q] *= s * (1.f + zz * (1.f - s));
            }
            store_split8(sx, sx_lo, row, c0, H1, g);
            store_split8(sx, sx_lo, row, c0 + 8, H1, g + 8);
        }
        fence_before();
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            issue_gemm(tbase + L.dx, xh, xl, w1th, w1tl, H1, Dp);
            mma_commit(mb);
        }
        ok = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
        // ---- dE/dfp = dX / sigma.  Staged in shared memory over the X and A operand areas
        // (free once GEMM 4 has completed; rows padded to Dp + 4 floats against bank
        // conflicts), then written row by row with coalesced float4 stores
        {
            const int Dps = Dp + 4;
            float* sg = reinterpret_cast<float*>(sx);  // [128][Dps]
            for (int c0 = 16 * part; c0 < Dp; c0 += 16 * SPLIT) {
                float g[16];
                tmem_ld16(tlane + L.dx + c0, g);
                float4* o = reinterpret_cast<float4*>(sg + (size_t)row * Dps + c0);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    o[q] = make_float4(g[4 * q] * fv[L.fisig + c0 + 4 * q], g[4 * q + 1] * fv[L.fisig + c0 + 4 * q + 1],
                                       g[4 * q + 2] * fv[L.fisig + c0 + 4 * q + 2],
                                       g[4 * q + 3] * fv[L.fisig + c0 + 4 * q + 3]);
            }
            __syncthreads();
            for (int r = warp; r < 128; r += 4 * SPLIT) {
                const int sl = s0 + tile * 128 + r;
                if (sl >= s1) continue;  // uniform across the warp
                float* gr = p.gfp + (size_t)sl * p.fp_stride;
                const float* src = sg + (size_t)r * Dps;
                for (int k = 4 * lane; k < p.D; k += 128) {
                    const float4 v = *reinterpret_cast<const float4*>(src + k);
                    if (k + 4 <= p.D) {
                        *reinterpret_cast<float4*>(gr + k) = v;
                    } else {
                        const float w[4] = {v.x, v.y, v.z, v.w};
                        for (int q = 0; k + q < p.D; ++q) gr[k + q] = w[q];
                    }
                }
            }
        }
        fence_before();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicOr(p.err, ERRBIT_TIMEOUT);
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(L.ncols) : "memory");
}

}  // namespace

bool net_tc_prepare(const Species& sp, NetTC& tc, std::string& why) {
    tc.ready = false;
    if (sp.hidden.size() != 2) {
        why = "the tensor-core network needs exactly two hidden layers";
        return false;
    }
    const int D = sp.D, H1 = sp.hidden[0], H2 = sp.hidden[1];
    if (D > 128 || H1 % 16 || H2 % 16 || H1 > 128 || H2 > 128 || H1 < 16 || H2 < 16) {
        why = "the tensor-core network needs D <= 128 and hidden widths that are multiples of 16 up to 128";
        return false;
    }
    const TCLayout L = make_layout(D, H1, H2);
    std::vector<uint8_t> img(L.bytes, 0);
    const int Dp = L.Dp;
    auto W1 = [&](int o, int i) { return i < D ? sp.Wh[0][(size_t)o * D + i] : 0.0; };
    auto W2 = [&](int o, int i) { return sp.Wh[1][(size_t)o * H1 + i]; };
    put_operand(img, L.w1, H1, Dp, [&](int r, int k) { return W1(r, k); });         // GEMM1 B: [H1][Dp]
    put_operand(img, L.w2, H2, H1, [&](int r, int k) { return W2(r, k); });         // GEMM2 B: [H2][H1]
    put_operand(img, L.w2t, H1, H2, [&](int r, int k) { return W2(k, r); });        // GEMM3 B: [H1][H2]
    put_operand(img, L.w1t, Dp, H1, [&](int r, int k) { return W1(k, r); });        // GEMM4 B: [Dp][H1]
    float* fv = reinterpret_cast<float*>(img.data() + L.fvec);
    for (int k = 0; k < Dp; ++k) {
        fv[L.fmu + k] = k < D ? (float)sp.mu[k] : 0.f;
        fv[L.fisig + k] = k < D ? (float)(1.0 / sp.sigma[k]) : 0.f;
    }
    for (int o = 0; o < H1; ++o) fv[L.fb1 + o] = (float)sp.bh[0][o];
    for (int o = 0; o < H2; ++o) fv[L.fb2 + o] = (float)sp.bh[1][o];
    for (int o = 0; o < H2; ++o) fv[L.fwo + o] = (float)sp.wo[o];
    if (cudaMalloc(&tc.blob, img.size()) != cudaSuccess) {
        why = "device allocation failed";
        return false;
    }
    if (cudaMemcpy(tc.blob, img.data(), img.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        why = "copy of the network image failed";
        return false;
    }
    tc.blob_bytes = img.size();
    tc.D = D;
    tc.Dp = Dp;
    tc.H1 = H1;
    tc.H2 = H2;
    tc.bo = (float)sp.bo;
    tc.ready = true;
    return true;
}

void net_tc_release(NetTC& tc) {
    if (tc.blob) cudaFree(tc.blob);
    tc.blob = nullptr;
    tc.ready = false;
}

cudaError_t launch_net_tc(const NetArgs* a, const NetTC* const* tc, int nt, int* err, int sm_count, int split,
                          cudaStream_t st) {
    if (nt < 1 || nt > kMaxTypes) return cudaErrorInvalidValue;
    for (int k = 0; k < nt; ++k) {
        if (!tc[k]->ready) return cudaErrorNotSupported;
        if (tc[k]->D != tc[0]->D || tc[k]->H1 != tc[0]->H1 || tc[k]->H2 != tc[0]->H2) return cudaErrorInvalidValue;
    }
    const int n = a[0].nmax;
    if (n <= 0) return cudaSuccess;
    const TCLayout L = make_layout(tc[0]->D, tc[0]->H1, tc[0]->H2);
    const int xbytes = align1k(2 * 2 * 128 * (L.Dp > L.H1 ? L.Dp : L.H1));
    const int abytes = align1k(2 * 2 * 128 * (L.H1 > L.H2 ? L.H1 : L.H2));
    const size_t sm = (size_t)L.bytes + xbytes + abytes;
    if (split != 2 && split != 4) return cudaErrorInvalidValue;
    static int limit2 = 0, limit4 = 0;  // raised once per instantiation, before any graph capture
    int& limit = split == 2 ? limit2 : limit4;
    if ((int)sm > limit) {
        const cudaError_t e =
            split == 2 ? cudaFuncSetAttribute(k_net_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)
                       : cudaFuncSetAttribute(k_net_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        limit = (int)sm;
    }
    TcParams p;
    std::memset(&p, 0, sizeof p);
    p.perm = a[0].perm;
    p.range = a[0].range;
    p.t0 = a[0].t;
    p.nt = nt;
    p.fp = a[0].fp;
    p.fp_stride = a[0].fp_stride;
    p.D = tc[0]->D;
    p.gfp = a[0].gfp;
    p.e_atom = a[0].e_atom;
    for (int k = 0; k < nt; ++k) {
        p.img[k] = reinterpret_cast<const uint8_t*>(tc[k]->blob);
        p.bo[k] = tc[k]->bo;
        p.mu_e[k] = a[k].mu_e;
        p.sigma_e[k] = a[k].sigma_e;
    }
    p.err = err;
    const int ntiles = (n + 127) / 128 + nt;  // upper bound of the tiles over all species
    const int grid = ntiles < sm_count ? ntiles : sm_count;
    if (split == 2) return launch_pdl(&k_net_tc<2>, dim3(grid), dim3(256), sm, st, p, L);
    return launch_pdl(&k_net_tc<4>, dim3(grid), dim3(512), sm, st, p, L);
}

}  // namespace nnapgb
