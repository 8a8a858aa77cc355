// Instances and launch of the any-shape descriptor kernels (k_desc_gen.cuh): radial
// bases and spherical bases of every expansion degree L = 0 .. 12, for the NNAP and NEP
// radial functions.  A launch uses as many warps per CTA as its launch shape asks for and
// shared memory allows (one atom slot per warp).
#include <map>

#include "k_desc_gen.cuh"

namespace nnapgb {

cudaError_t upload_sh_constants_gen() { return upload_sh_tables(); }

namespace {

constexpr size_t kSmemMax = 227 * 1024;

size_t warp_bytes(int kind, bool fwd, int lmax, int np, int n1) {
    if (kind == 0) return sizeof(float) * (size_t)(fwd ? gen::rad_fwd_floats(np, n1) : gen::rad_bwd_floats(np));
    return sizeof(float) * (size_t)(fwd ? gen::sph_fwd_floats(lmax, np) : gen::sph_bwd_floats(lmax, np));
}

template <class Kern>
cudaError_t launch_g(Kern kern, const DescArgs& a, size_t per_warp, int np, int n1, cudaStream_t st) {
    int wpc = a.warps < 1 ? 1 : (a.warps > gen::kMaxWarps ? gen::kMaxWarps : a.warps);
    while (wpc > 1 && per_warp * wpc > kSmemMax) wpc >>= 1;
    const size_t sm = per_warp * wpc;
    if (sm > kSmemMax) return cudaErrorInvalidValue;
    // the shared-memory limit is raised once per kernel and size (the first evaluation of a
    // layout runs eagerly, before any graph capture)
    static std::map<const void*, size_t> limits;
    size_t& lim = limits[reinterpret_cast<const void*>(kern)];
    if (sm > 48 * 1024 && sm > lim) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        lim = sm;
    }
    const int grid = (a.nmax + wpc - 1) / wpc;
    return launch_pdl(kern, dim3(grid), dim3(32 * wpc), sm, st, a, np, n1);
}

template <int RB>
cudaError_t launch_sph_g(int L, const DescArgs& a, bool fwd, int np, int n1, size_t pw, cudaStream_t st) {
    switch (L) {
#define L_CASE(L_) \
    case L_: return fwd ? launch_g(gen::k_sph_fwd_g<L_, RB>, a, pw, np, n1, st) : launch_g(gen::k_sph_bwd_g<L_, RB>, a, pw, np, n1, st);
        L_CASE(0) L_CASE(1) L_CASE(2) L_CASE(3) L_CASE(4) L_CASE(5) L_CASE(6)
        L_CASE(7) L_CASE(8) L_CASE(9) L_CASE(10) L_CASE(11) L_CASE(12)
#undef L_CASE
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool desc_generic_fits(int kind, int lmax, int np, int n1) {
    if (np < 1 || n1 < 1 || n1 > gen::kMaxN1) return false;
    if (kind == 1 && (lmax < 0 || lmax > 12)) return false;
    return warp_bytes(kind, true, lmax, np, n1) <= kSmemMax && warp_bytes(kind, false, lmax, np, n1) <= kSmemMax;
}

cudaError_t launch_descriptor_generic(int kind, int basis, int lmax, int np, int n1, const DescArgs& a, bool fwd,
                                      cudaStream_t st) {
    if (a.nmax <= 0) return cudaSuccess;
    if (!desc_generic_fits(kind, lmax, np, n1)) return cudaErrorInvalidValue;
    const size_t pw = warp_bytes(kind, fwd, lmax, np, n1);
    if (kind == 0) {
        if (basis == kRbNEP)
            return fwd ? launch_g(gen::k_radial_fwd_g<kRbNEP>, a, pw, np, n1, st)
                       : launch_g(gen::k_radial_bwd_g<kRbNEP>, a, pw, np, n1, st);
        return fwd ? launch_g(gen::k_radial_fwd_g<kRbNNAP>, a, pw, np, n1, st)
                   : launch_g(gen::k_radial_bwd_g<kRbNNAP>, a, pw, np, n1, st);
    }
    if (basis == kRbNEP) return launch_sph_g<kRbNEP>(lmax, a, fwd, np, n1, pw, st);
    return launch_sph_g<kRbNNAP>(lmax, a, fwd, np, n1, pw, st);
}

}  // namespace nnapgb
