// Tensor-core (tcgen05, BF16 operands, FP32 accumulation in TMEM) evaluation of the
// per-species network and its input gradient: the mixed-precision path.
#pragma once

#include <string>

#include "desc.cuh"
#include "model.hpp"

namespace nnapgb {

struct NetTC {
    bool ready = false;
    int D = 0, Dp = 0, H1 = 0, H2 = 0;
    float bo = 0.f;           // output bias
    void* blob = nullptr;     // device: packed operand images and FP32 vectors
    size_t blob_bytes = 0;
};

// Pack a species' network for the tensor-core kernel; false (with a reason) when the
// shape is outside what the kernel implements.
bool net_tc_prepare(const Species& sp, NetTC& tc, std::string& why);
void net_tc_release(NetTC& tc);
// One launch over nt consecutive species a[k].t = a[0].t + k, all with the same network
// shape (D, H1, H2).  err receives ERRBIT_TIMEOUT if a bounded wait on the tensor cores
// gave up.
// split: threads per tile row in the epilogues (2 or 4).
cudaError_t launch_net_tc(const NetArgs* a, const NetTC* const* tc, int nt, int* err, int sm_count, int split,
                          cudaStream_t st);

}  // namespace nnapgb
