// Tensor-core (tcgen05, BF16 operands, FP32 accumulation in TMEM) evaluation of the
// per-species network and its input gradient: the mixed-precision path.
#pragma once

#include <string>

#include "desc.cuh"
#include "model.hpp"

namespace nnapgb {

constexpr int kTcMaxLayers = 8;  // hidden layers of a tensor-core network

// Operand images, FP32 vectors, TMEM columns and shared memory of one network shape.
struct TCLayout {
    int nl = 0;                    // hidden layers
    int Dp = 0;                    // descriptor length rounded up to 16
    int K[kTcMaxLayers];           // input width of layer l (Dp, then Hp[l - 1])
    int Hp[kTcMaxLayers];          // output width of layer l rounded up to 16
    int Wmax = 0;                  // widest activation
    // byte offsets inside the species image (multiples of 1024): W_l as a [Hp x K] B
    // operand and W_l^T as a [K x Hp] B operand, each BF16 hi then lo
    int wf[kTcMaxLayers], wb[kTcMaxLayers];
    int fvec = 0;                  // FP32 vectors: mu[Dp] | 1/sigma[Dp] | b_l[Hp_l] ... | w_out[Hp_last]
    int fmu = 0, fisig = 0, fb[kTcMaxLayers], fwo = 0, nvec = 0;
    int bytes = 0;                 // whole image
    int wimg = 0;                  // largest single operand image (hi + lo), bytes
    int ncols = 0;                 // TMEM columns allocated (power of two, <= 512)
    int z[kTcMaxLayers];           // TMEM column of Z_l
    int dacc = 0;                  // TMEM column of dA_{l-1} / dX
    int staged = 0;                // whole image in shared memory once per species (else per GEMM)
    int act = 0;                   // bytes of the activation operand buffer (hi + lo)
    int smem = 0;                  // dynamic shared memory bytes
    bool same(const TCLayout& o) const;
};

struct NetTC {
    bool ready = false;
    int D = 0;
    TCLayout L;
    float bo = 0.f;           // output bias
    void* blob = nullptr;     // device: packed operand images and FP32 vectors
    size_t blob_bytes = 0;
};

// Pack a species' network for the tensor-core kernel; false (with a reason) when the
// shape is outside what the kernel implements (the species then evaluates its network
// with the FP32 kernel).
bool net_tc_prepare(const Species& sp, NetTC& tc, std::string& why);
void net_tc_release(NetTC& tc);
// One launch over nt consecutive species a[k].t = a[0].t + k, all with the same layout.
// err receives ERRBIT_TIMEOUT if a bounded wait on the tensor cores gave up.
// split: threads per tile row in the epilogues (2 or 4).
cudaError_t launch_net_tc(const NetArgs* a, const NetTC* const* tc, int nt, int* err, int sm_count, int split,
                          cudaStream_t st);

}  // namespace nnapgb
