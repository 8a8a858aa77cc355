// Tensor-core network kernel (mixed precision).  See net_tc.cuh.
#include "net_tc.cuh"

namespace nnapgb {

bool net_tc_prepare(const Species& sp, NetTC& tc, std::string& why) {
    (void)sp;
    tc.ready = false;
    why = "the tensor-core network kernel is not available in this build";
    return false;
}

void net_tc_release(NetTC& tc) {
    if (tc.blob) cudaFree(tc.blob);
    tc.blob = nullptr;
    tc.ready = false;
}

cudaError_t launch_net_tc(const NetArgs& a, const NetTC& tc, cudaStream_t st) {
    (void)a;
    (void)tc;
    (void)st;
    return cudaErrorNotSupported;
}

}  // namespace nnapgb
