// Tensor-core evaluation of the per-species network and its input gradient (the
// mixed-precision path), on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// Mathematics: normedNnForward / normedNnBackward (nnap_main.hpp:267-323) with L >= 1
// SiLU hidden layers (nn_FeedForward.hpp:8-261), widths padded to multiples of 16:
//   X   = (fp - mu)/sigma                       [128 x Dp]
//   Z_l = A_{l-1} W_l^T + b_l, A_l = silu(Z_l)   [128 x Hp_l]  GEMM (N = Hp_l, K = K_l), A_0 = X
//   E   = (w_o . A_L + b_o) sigma_E + mu_E       (FP32 on the CUDA cores, FP64 output)
//   dZ_L = sigma_E w_o * silu'(Z_L)
//   dA_{l-1} = dZ_l W_l                          [128 x K_l]   GEMM (N = K_l, K = Hp_l)
//   dZ_{l-1} = dA_{l-1} * silu'(Z_{l-1})
//   dE/dfp = dA_0 / sigma
// Padded units have zero weights and biases, so they stay zero through every layer.
// Operands are BF16 and every product is split as hi*hi + lo*hi + hi*lo with x = hi + lo
// (both BF16), accumulated in FP32 in TMEM: three kind::f16 MMAs per 16-wide K step keep
// the network error near FP32 level (about 1e-6 eV per atom) while the arithmetic stays
// on the BF16 tensor pipe.
//
// One CTA of 128 x SPLIT threads owns a 128-atom tile; the SPLIT threads of row t read
// TMEM lane t with tcgen05.ld 32x32b, each a share of the columns.  One thread issues the
// MMAs; completion is signalled through an mbarrier (tcgen05.commit) whose waits are
// bounded in time and raise ERRBIT_TIMEOUT instead of hanging.  Z_l of every layer stays
// in TMEM for the backward pass; dA and dX share one column range.  One shared-memory
// operand buffer holds the activation of the current GEMM and is overwritten by the next
// layer's once that GEMM has completed.  The weight images of a species are staged in
// shared memory once per species when they fit, otherwise the B operand of each GEMM is
// copied in before it (the images are small and stay in L2).
// Shared-memory operands use the no-swizzle K-major canonical layout: 8x8 core
// matrices of 128 bytes, adjacent in K at LBO = 128 bytes and in M/N at
// SBO = (K/8)*128 bytes.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "net_tc.cuh"
#include "pdl.cuh"
#include "tc_util.cuh"

namespace nnapgb {

bool TCLayout::same(const TCLayout& o) const {
    if (nl != o.nl || Dp != o.Dp) return false;
    for (int l = 0; l < nl; ++l)
        if (Hp[l] != o.Hp[l]) return false;
    return true;
}

namespace {

using namespace ::nnapgb::tc;

constexpr int kTcSmemMax = 220 * 1024;  // dynamic shared memory; the static part (mbarrier, energies) comes on top
constexpr int kTcWidthMax = 256;       // widest padded layer (one MMA N, one operand buffer)
constexpr int kTcOperandMax = 96 * 1024;  // largest single weight operand image (hi + lo)
constexpr int kOutCols = 64;           // columns of dE/dfp staged per pass

__host__ __device__ inline int align1k(int b) { return (b + 1023) & ~1023; }
inline int r16(int v) { return (v + 15) & ~15; }

// Layout of a network with descriptor length D and hidden widths H[0..nl-1]; false with a
// reason when the kernel cannot take it.
bool make_layout(int D, const std::vector<int>& H, TCLayout& L, std::string& why) {
    const int nl = (int)H.size();
    if (nl < 1 || nl > kTcMaxLayers) {
        why = "the tensor-core network takes 1 to 8 hidden layers";
        return false;
    }
    L.nl = nl;
    L.Dp = r16(D);
    L.Wmax = L.Dp;
    int in = L.Dp, off = 0, wimg = 0;
    for (int l = 0; l < nl; ++l) {
        L.K[l] = in;
        L.Hp[l] = r16(H[l]);
        L.Wmax = std::max(L.Wmax, L.Hp[l]);
        const int img = 4 * L.Hp[l] * in;  // hi + lo BF16
        wimg = std::max(wimg, img);
        L.wf[l] = off; off = align1k(off + img);
        L.wb[l] = off; off = align1k(off + img);
        in = L.Hp[l];
    }
    if (L.Wmax > kTcWidthMax) {
        why = "the tensor-core network takes descriptors and hidden layers of at most 256 (padded) columns";
        return false;
    }
    if (wimg > kTcOperandMax) {
        why = "a tensor-core weight operand would exceed 96 KiB";
        return false;
    }
    L.fvec = off;
    L.fmu = 0;
    L.fisig = L.Dp;
    int f = 2 * L.Dp;
    for (int l = 0; l < nl; ++l) { L.fb[l] = f; f += L.Hp[l]; }
    L.fwo = f;
    f += L.Hp[nl - 1];
    L.nvec = (f + 3) & ~3;
    off = align1k(off + 4 * L.nvec);
    L.bytes = off;
    L.wimg = align1k(wimg);
    // TMEM: Z of every layer, then one range for dA / dX
    int cols = 0, dmax = 0;
    for (int l = 0; l < nl; ++l) { L.z[l] = cols; cols += L.Hp[l]; dmax = std::max(dmax, L.K[l]); }
    L.dacc = cols;
    cols += dmax;
    if (cols > 512) {
        why = "the tensor-core network's accumulators would exceed the 512 TMEM columns";
        return false;
    }
    L.ncols = 32;
    while (L.ncols < cols) L.ncols *= 2;
    L.act = align1k(std::max(4 * 128 * L.Wmax, 4 * 128 * (kOutCols + 4)));
    const int staged = L.bytes + L.act;
    const int streamed = align1k(4 * L.nvec) + L.wimg + L.act;
    if (staged <= kTcSmemMax) {
        L.staged = 1;
        L.smem = staged;
    } else if (streamed <= kTcSmemMax) {
        L.staged = 0;
        L.smem = streamed;
    } else {
        why = "the tensor-core network's operands exceed shared memory";
        return false;
    }
    return true;
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

// Write the hi and lo images of an R x K matrix M(r, k).
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

// Species t0 .. t0+nt-1 of one launch; all share one layout.  Tiles are numbered species
// by species; a CTA stages a species' image (or its FP32 vectors, in streamed mode) when
// its next tile belongs to another species than the last one.
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

// Copy n bytes (a multiple of 16) from global to shared memory with every thread.
__device__ __forceinline__ void copy16(uint8_t* dst, const uint8_t* src, int n, int tid, int nthr) {
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int q = tid; q < n / 16; q += nthr) d[q] = s[q];
}

template <int SPLIT>
__global__ void __launch_bounds__(128 * SPLIT, 1) k_net_tc(TcParams p, TCLayout L) {
    pdl_enter();
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_tstart[kMaxTypes + 1];
    __shared__ float s_e[SPLIT][128];
    constexpr int NT = 128 * SPLIT;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int part = tid >> 7;  // column share of this thread in the epilogues
    const int row = tid & 127;
    const int nl = L.nl, Dp = L.Dp;
    // shared memory: staged [image | act]; streamed [FP32 vectors | one operand | act]
    uint8_t* sw = smem;
    uint8_t* swb = smem + (L.staged ? 0 : align1k(4 * L.nvec));  // per-GEMM operand (streamed)
    uint8_t* sact = smem + (L.staged ? L.bytes : align1k(4 * L.nvec) + L.wimg);
    const float* fv = reinterpret_cast<const float*>(L.staged ? sw + L.fvec : sw);
    const int half = 2 * 128 * L.Wmax;  // bytes of the hi (or lo) activation image
    uint8_t* sact_lo = sact + half;

    if (tid == 0) {
        s_tstart[0] = 0;
        for (int t = 0; t < p.nt; ++t)
            s_tstart[t + 1] = s_tstart[t] + (p.range[p.t0 + t + 1] - p.range[p.t0 + t] + 127) / 128;
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
    const uint32_t ah = smem_u32(sact), al = ah + half;

    // one GEMM: D (TMEM column dcol) = act [128 x K] * B [N x K]^T, B the image at byte
    // offset boff of the species image (staged) or copied from global first (streamed)
    auto gemm = [&](int ts, int boff, int N, int K, int dcol) -> bool {
        uint32_t bh;
        if (L.staged) {
            bh = smem_u32(sw + boff);
        } else {
            copy16(swb, p.img[ts] + boff, 4 * N * K, tid, NT);
            bh = smem_u32(swb);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            issue_gemm(tbase + dcol, ah, al, bh, bh + 2 * N * K, K, N);
            mma_commit(mb);
        }
        const bool done = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1;
        if (done) fence_after();
        return done;
    };

    const int total = s_tstart[p.nt];
    int staged = -1;
    for (int gt = blockIdx.x; gt < total && ok; gt += gridDim.x) {
        int ts = 0;
        while (gt >= s_tstart[ts + 1]) ++ts;
        const int tile = gt - s_tstart[ts];
        if (ts != staged) {  // stage this species' image or FP32 vectors (no MMA is in flight here)
            __syncthreads();
            if (L.staged) copy16(sw, p.img[ts], L.bytes, tid, NT);
            else copy16(sw, p.img[ts] + L.fvec, 4 * L.nvec, tid, NT);
            fence_async_smem();
            __syncthreads();
            staged = ts;
        }
        const int s0 = p.range[p.t0 + ts], s1 = p.range[p.t0 + ts + 1];
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
                store_split8(sact, sact_lo, r, k0, Dp, v);
            }
        }
        // ---- forward through the hidden layers
        const float se = (float)p.sigma_e[ts];
        float e = 0.f;
        for (int l = 0; l < nl && ok; ++l) {
            const int H = L.Hp[l];
            ok = gemm(ts, L.wf[l], H, L.K[l], L.z[l]);
            if (!ok) break;
            const float* b = fv + L.fb[l];
            const bool last = l == nl - 1;
            for (int c0 = 16 * part; c0 < H; c0 += 16 * SPLIT) {
                float z[16];
                tmem_ld16(tlane + L.z[l] + c0, z);
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const float zz = z[q] + b[c0 + q];
                    const float s = sigmoidf_(zz);
                    if (last) {  // energy share and dZ_L = sigma_E w_o silu'(Z_L)
                        const float wo = fv[L.fwo + c0 + q];
                        e += wo * (zz * s);
                        z[q] = se * wo * (s * (1.f + zz * (1.f - s)));
                    } else {
                        z[q] = zz * s;
                    }
                }
                store_split8(sact, sact_lo, row, c0, H, z);
                store_split8(sact, sact_lo, row, c0 + 8, H, z + 8);
            }
            fence_before();
        }
        if (!ok) break;
        s_e[part][row] = e;
        // ---- backward: dA_{l-1} = dZ_l W_l; dZ_{l-1} = dA_{l-1} silu'(Z_{l-1})
        for (int l = nl - 1; l >= 1 && ok; --l) {
            ok = gemm(ts, L.wb[l], L.K[l], L.Hp[l], L.dacc);
            if (!ok) break;
            if (l == nl - 1 && part == 0 && valid) {  // energy: the column shares added in a fixed order
                float et = s_e[0][row];
#pragma unroll
                for (int q = 1; q < SPLIT; ++q) et += s_e[q][row];
                p.e_atom[p.perm[slot]] = ((double)et + (double)p.bo[ts]) * p.sigma_e[ts] + p.mu_e[ts];
            }
            const int H = L.Hp[l - 1];
            const float* b = fv + L.fb[l - 1];
            for (int c0 = 16 * part; c0 < H; c0 += 16 * SPLIT) {
                float g[16], z[16];
                tmem_ld16(tlane + L.dacc + c0, g);
                tmem_ld16(tlane + L.z[l - 1] + c0, z);
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const float zz = z[q] + b[c0 + q];
                    const float s = sigmoidf_(zz);
                    g[q] *= s * (1.f + zz * (1.f - s));
                }
                store_split8(sact, sact_lo, row, c0, H, g);
                store_split8(sact, sact_lo, row, c0 + 8, H, g + 8);
            }
            fence_before();
        }
        if (!ok) break;
        // ---- dX = dZ_1 W_1
        ok = gemm(ts, L.wb[0], Dp, L.Hp[0], L.dacc);
        if (!ok) break;
        if (nl == 1 && part == 0 && valid) {
            float et = s_e[0][row];
#pragma unroll
            for (int q = 1; q < SPLIT; ++q) et += s_e[q][row];
            p.e_atom[p.perm[slot]] = ((double)et + (double)p.bo[ts]) * p.sigma_e[ts] + p.mu_e[ts];
        }
        // ---- dE/dfp = dX / sigma, staged through the (now free) operand buffer kOutCols
        // columns at a time (rows padded by 4 floats against bank conflicts) and written
        // row by row with coalesced stores
        {
            constexpr int CS = kOutCols + 4;
            float* sg = reinterpret_cast<float*>(sact);  // [128][CS]
            for (int cb = 0; cb < Dp; cb += kOutCols) {
                const int cw = Dp - cb < kOutCols ? Dp - cb : kOutCols;
                for (int c0 = 16 * part; c0 < cw; c0 += 16 * SPLIT) {
                    float g[16];
                    tmem_ld16(tlane + L.dacc + cb + c0, g);
                    float4* o = reinterpret_cast<float4*>(sg + (size_t)row * CS + c0);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        o[q] = make_float4(g[4 * q] * fv[L.fisig + cb + c0 + 4 * q],
                                           g[4 * q + 1] * fv[L.fisig + cb + c0 + 4 * q + 1],
                                           g[4 * q + 2] * fv[L.fisig + cb + c0 + 4 * q + 2],
                                           g[4 * q + 3] * fv[L.fisig + cb + c0 + 4 * q + 3]);
                }
                __syncthreads();
                const int lim = p.D - cb < cw ? p.D - cb : cw;  // columns of this pass that exist
                for (int r = warp; r < 128; r += 4 * SPLIT) {
                    const int sl = s0 + tile * 128 + r;
                    if (sl >= s1 || lim <= 0) continue;  // uniform across the warp
                    float* gr = p.gfp + (size_t)sl * p.fp_stride + cb;
                    const float* src = sg + (size_t)r * CS;
                    for (int k = 4 * lane; k < lim; k += 128) {
                        const float4 v = *reinterpret_cast<const float4*>(src + k);
                        if (k + 4 <= lim) {
                            *reinterpret_cast<float4*>(gr + k) = v;
                        } else {
                            const float w[4] = {v.x, v.y, v.z, v.w};
                            for (int q = 0; k + q < lim; ++q) gr[k + q] = w[q];
                        }
                    }
                }
                __syncthreads();
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
    const int D = sp.D;
    TCLayout L;
    if (!make_layout(D, sp.hidden, L, why)) return false;
    std::vector<uint8_t> img(L.bytes, 0);
    int in = D;
    for (int l = 0; l < L.nl; ++l) {
        const int H = sp.hidden[l], Hp = L.Hp[l], K = L.K[l];
        const std::vector<double>& W = sp.Wh[l];  // [H][in]
        auto Wf = [&](int o, int i) { return o < H && i < in ? W[(size_t)o * in + i] : 0.0; };
        put_operand(img, L.wf[l], Hp, K, [&](int r, int k) { return Wf(r, k); });  // [Hp][K]
        put_operand(img, L.wb[l], K, Hp, [&](int r, int k) { return Wf(k, r); });  // [K][Hp]
        in = H;
    }
    float* fv = reinterpret_cast<float*>(img.data() + L.fvec);
    for (int k = 0; k < L.Dp; ++k) {
        fv[L.fmu + k] = k < D ? (float)sp.mu[k] : 0.f;
        fv[L.fisig + k] = k < D ? (float)(1.0 / sp.sigma[k]) : 0.f;
    }
    for (int l = 0; l < L.nl; ++l)
        for (int o = 0; o < sp.hidden[l]; ++o) fv[L.fb[l] + o] = (float)sp.bh[l][o];
    for (int o = 0; o < sp.hidden.back(); ++o) fv[L.fwo + o] = (float)sp.wo[o];
    if (cudaMalloc(&tc.blob, img.size()) != cudaSuccess) {
        cudaGetLastError();
        why = "device allocation failed";
        return false;
    }
    if (cudaMemcpy(tc.blob, img.data(), img.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        why = "copy of the network image failed";
        return false;
    }
    tc.blob_bytes = img.size();
    tc.D = D;
    tc.L = L;
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
        if (tc[k]->D != tc[0]->D || !tc[k]->L.same(tc[0]->L)) return cudaErrorInvalidValue;
    }
    const int n = a[0].nmax;
    if (n <= 0) return cudaSuccess;
    const TCLayout& L = tc[0]->L;
    const size_t sm = (size_t)L.smem;
    if (split != 2 && split != 4) return cudaErrorInvalidValue;
    static int limit2 = 0, limit4 = 0;  // raised once per instantiation, before any graph capture
    int& limit = split == 2 ? limit2 : limit4;
    if ((int)sm > limit) {
        const cudaError_t e =
            split == 2 ? cudaFuncSetAttribute(k_net_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemMax)
                       : cudaFuncSetAttribute(k_net_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemMax);
        if (e != cudaSuccess) return e;
        limit = kTcSmemMax;
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
