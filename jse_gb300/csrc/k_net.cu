// FP32 SIMT evaluation of the per-species SiLU feed-forward network and of its input
// gradient (the plain-precision path; also the tanh network of NEP models).
//
// Restates normedNnForward / normedNnBackward (nnap_main.hpp:267-323) and
// nnForward / nnBackward (nn_FeedForward.hpp:8-21, 131-261):
//   x = (fp - mu) / sigma;  h_l = silu(W_l h_{l-1} + b_l);  o = w_out . h_L + b_out;
//   E = o * sigma_E + mu_E;  dE/dfp = (sigma_E * d o / d x) / sigma.
// One warp evaluates 8 atoms of one species together so every weight it loads is
// used 8 times; lanes own output units in the forward pass and input units in the
// backward pass, so all weight loads are coalesced (W^T rows forward, W rows backward).
//
// Packed FP32 parameters of a species (net_pack in nnap_api.cu):
//   mu[D] | 1/sigma[D] | for each layer: W^T[in][H] | W[H][in] | b[H] | w_out[H_L] | b_out
#include "desc.cuh"
#include "pdl.cuh"

namespace nnapgb {
namespace {

constexpr int kNetAtoms = 8;
constexpr int kNetWarps = 4;

__device__ __forceinline__ float silu_and_grad(float z, float* grad) {
    const float s = 1.f / (1.f + expf(-z));
    *grad = s * (1.f + z * (1.f - s));
    return z * s;
}

// tanh for NEP networks (apply_ann_one_layer, nep_core.hpp:267-305)
__device__ __forceinline__ float act_and_grad(float z, float* grad, int act) {
    if (act == kActTanh) {
        const float t = tanhf(z);
        *grad = 1.f - t * t;
        return t;
    }
    return silu_and_grad(z, grad);
}

__global__ void __launch_bounds__(32 * kNetWarps) k_net_fp32(NetArgs a, int warp_floats) {
    pdl_enter();
    extern __shared__ float smem[];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s0 = a.range[a.t], s1 = a.range[a.t + 1];
    const int slot0 = s0 + (blockIdx.x * (blockDim.x >> 5) + wl) * kNetAtoms;
    if (slot0 >= s1) return;
    const int na = min(kNetAtoms, s1 - slot0);
    int Hmax = a.D;
    for (int l = 0; l < a.nlayer; ++l) Hmax = max(Hmax, a.H[l]);
    float* buf0 = smem + (size_t)wl * warp_floats;        // [Hmax][8]
    float* buf1 = buf0 + Hmax * kNetAtoms;                  // [Hmax][8]
    float* sd = buf1 + Hmax * kNetAtoms;                    // [nlayer][Hmax][8] silu'
    const float* mu = a.w;
    const float* isig = mu + a.D;
    // normalised input, layout [i][atom]
    for (int i = lane; i < a.D; i += 32)
#pragma unroll
        for (int q = 0; q < kNetAtoms; ++q)
            buf0[i * kNetAtoms + q] = q < na ? (a.fp[(size_t)(slot0 + q) * a.fp_stride + i] - mu[i]) * isig[i] : 0.f;
    __syncwarp();
    const float* p = isig + a.D;
    const float* layerW[kNetMaxLayers];
    int in = a.D;
    float* cur = buf0;
    float* nxt = buf1;
    for (int l = 0; l < a.nlayer; ++l) {
        const int H = a.H[l];
        const float* WT = p;
        layerW[l] = p + (size_t)in * H;
        const float* b = layerW[l] + (size_t)H * in;
        for (int o = lane; o < H; o += 32) {
            float z[kNetAtoms];
#pragma unroll
            for (int q = 0; q < kNetAtoms; ++q) z[q] = b[o];
#pragma unroll 8
            for (int i = 0; i < in; ++i) {
                const float wv = WT[(size_t)i * H + o];
                const float4 x0 = *reinterpret_cast<const float4*>(cur + i * kNetAtoms);
                const float4 x1 = *reinterpret_cast<const float4*>(cur + i * kNetAtoms + 4);
                z[0] += wv * x0.x; z[1] += wv * x0.y; z[2] += wv * x0.z; z[3] += wv * x0.w;
                z[4] += wv * x1.x; z[5] += wv * x1.y; z[6] += wv * x1.z; z[7] += wv * x1.w;
            }
#pragma unroll
            for (int q = 0; q < kNetAtoms; ++q) {
                float gz;
                nxt[o * kNetAtoms + q] = act_and_grad(z[q], &gz, a.act);
                sd[((size_t)l * Hmax + o) * kNetAtoms + q] = gz;
            }
        }
        __syncwarp();
        p = b + H;
        in = H;
        float* t = cur; cur = nxt; nxt = t;
    }
    const float* wo = p;
    const float bo = wo[in];
    // output layer and energies
    float part[kNetAtoms];
#pragma unroll
    for (int q = 0; q < kNetAtoms; ++q) part[q] = 0.f;
    for (int o = lane; o < in; o += 32)
#pragma unroll
        for (int q = 0; q < kNetAtoms; ++q) part[q] += wo[o] * cur[o * kNetAtoms + q];
#pragma unroll
    for (int q = 0; q < kNetAtoms; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) part[q] += __shfl_xor_sync(0xffffffffu, part[q], off);
    if (lane < na) {
        float outv = part[0];
#pragma unroll
        for (int q = 1; q < kNetAtoms; ++q) if (lane == q) outv = part[q];
        a.e_atom[a.perm[slot0 + lane]] = ((double)outv + (double)bo) * a.sigma_e + a.mu_e;
    }
    __syncwarp();
    // backward: dz_L = sigma_E * w_out * silu'(z_L)
    const float se = (float)a.sigma_e;
    const int L = a.nlayer;
    for (int o = lane; o < in; o += 32)
#pragma unroll
        for (int q = 0; q < kNetAtoms; ++q)
            cur[o * kNetAtoms + q] = se * wo[o] * sd[((size_t)(L - 1) * Hmax + o) * kNetAtoms + q];
    __syncwarp();
    for (int l = L - 1; l >= 0; --l) {
        const int H = a.H[l];
        const int lin = l ? a.H[l - 1] : a.D;
        const float* W = layerW[l];
        for (int i = lane; i < lin; i += 32) {
            float g[kNetAtoms];
#pragma unroll
            for (int q = 0; q < kNetAtoms; ++q) g[q] = 0.f;
#pragma unroll 8
            for (int o = 0; o < H; ++o) {
                const float wv = W[(size_t)o * lin + i];
                const float4 d0 = *reinterpret_cast<const float4*>(cur + o * kNetAtoms);
                const float4 d1 = *reinterpret_cast<const float4*>(cur + o * kNetAtoms + 4);
                g[0] += wv * d0.x; g[1] += wv * d0.y; g[2] += wv * d0.z; g[3] += wv * d0.w;
                g[4] += wv * d1.x; g[5] += wv * d1.y; g[6] += wv * d1.z; g[7] += wv * d1.w;
            }
            if (l > 0) {
#pragma unroll
                for (int q = 0; q < kNetAtoms; ++q)
                    nxt[i * kNetAtoms + q] = g[q] * sd[((size_t)(l - 1) * Hmax + i) * kNetAtoms + q];
            } else {
#pragma unroll
                for (int q = 0; q < kNetAtoms; ++q)
                    if (q < na) a.gfp[(size_t)(slot0 + q) * a.fp_stride + i] = g[q] * isig[i];
            }
        }
        __syncwarp();
        float* t = cur; cur = nxt; nxt = t;
    }
}

}  // namespace

namespace {
int net_warp_floats(int D, int nlayer, const int* H) {
    int Hmax = D;
    for (int l = 0; l < nlayer; ++l) Hmax = Hmax > H[l] ? Hmax : H[l];
    return (2 + nlayer) * Hmax * kNetAtoms;
}
constexpr size_t kNetSmemMax = 227 * 1024;
}  // namespace

bool net_fp32_fits(int D, int nlayer, const int* H) {
    return nlayer >= 1 && nlayer <= kNetMaxLayers && sizeof(float) * (size_t)net_warp_floats(D, nlayer, H) <= kNetSmemMax;
}

cudaError_t launch_net_fp32(const NetArgs& a, cudaStream_t st) {
    const int n = a.nmax;
    if (n <= 0) return cudaSuccess;
    if (!net_fp32_fits(a.D, a.nlayer, a.H)) return cudaErrorInvalidValue;
    const int warp_floats = net_warp_floats(a.D, a.nlayer, a.H);
    int wpc = kNetWarps;  // fewer warps per CTA for wide networks
    while (wpc > 1 && sizeof(float) * (size_t)warp_floats * wpc > kNetSmemMax) wpc >>= 1;
    const size_t sm = sizeof(float) * (size_t)warp_floats * wpc;
    static int limit = 0;
    if ((int)sm > limit) {
        const cudaError_t e = cudaFuncSetAttribute(k_net_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        limit = (int)sm;
    }
    const int per_block = kNetAtoms * wpc;
    return launch_pdl(&k_net_fp32, dim3((n + per_block - 1) / per_block), dim3(32 * wpc), sm, st, a, warp_floats);
}

}  // namespace nnapgb
