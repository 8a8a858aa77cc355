// NEP's ZBL short-range term over the pair rows (find_force_ZBL, nep_core.hpp:1321-1386).
//
// For every row entry (i -> j) with r < 2.5 A:
//   f(r)  = k Z_i Z_j / r * phi(r / a) * fc(r),   1/a = 2.134563 (Z_i^0.23 + Z_j^0.23),
//   phi(x) = sum_k a_k exp(-b_k x)   (the universal ZBL screening coefficients, or the
//                                     file's per-pair a_k, b_k in the flexible form),
//   fc = 1 below rc_inner, (cos(pi (r - rc_inner)/(rc_outer - rc_inner)) + 1)/2 up to
//        rc_outer, 0 beyond,
// atom i takes f/2 of its energy and the entry's pair gradient gets -dx f'(r) / (2 r): the
// full rows hold each pair in both directions, as the reference's neighbour lists do.
// One warp per atom row; the row's energy is summed in a fixed order and added once.
// The pair terms are evaluated in FP64 from the displacement carried to ~48 bits (its FP32
// value and the low part the row builders store for ZBL models): an atom's ZBL energy
// reaches tens of eV at short range, where an FP32 displacement alone would cost up to
// 1e-5 eV per atom.
#include "common.cuh"
#include "pdl.cuh"
#include "zbl.cuh"

namespace nnapgb {

namespace {

__device__ __forceinline__ void zbl_term(double a, double b, double x, double& phi, double& dphi) {
    const double t = a * exp(-b * x);
    phi += t;
    dphi -= b * t;
}

}  // namespace

__global__ void __launch_bounds__(256) k_nep_zbl(PairBufs P, int n, const int* __restrict__ type, ZblArgs z,
                                                 double* __restrict__ e_atom) {
    pdl_enter();
    const int at = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (at >= n) return;
    const int M = P.M, cnt = min(P.count[at], M);
    const int ti = type[at] - 1;
    double esum = 0.0;
    for (int k = lane; k < cnt; k += 32) {
        const size_t e = (size_t)at * M + k;
        const float4 d = P.dx[e];
        const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
        if (r2 >= kZblMaxR * kZblMaxR) continue;
        const int tj = __float_as_int(d.w) - 1;
        // the displacement to ~48 bits: FP32 value plus its stored low part
        double dx = d.x, dy = d.y, dz = d.z;
        if (P.dxlo) {
            const float4 lo = P.dxlo[e];
            dx += lo.x;
            dy += lo.y;
            dz += lo.z;
        }
        const double r = sqrt(dx * dx + dy * dy + dz * dz), rinv = 1.0 / r;
        const double a_inv = (z.zp[ti] + z.zp[tj]) * 2.134563;
        const double zizj = 14.399645 * z.z[ti] * z.z[tj];
        const double x = r * a_inv;
        double phi = 0.0, dphi = 0.0, rin = z.rc_inner, rout = z.rc_outer;
        if (z.flexible) {
            const int t1 = min(ti, tj), t2 = max(ti, tj);
            const double* p = z.para + 10 * (t1 * z.T - t1 * (t1 - 1) / 2 + (t2 - t1));
            rin = p[0];
            rout = p[1];
#pragma unroll
            for (int q = 0; q < 4; ++q) zbl_term(p[2 + 2 * q], p[3 + 2 * q], x, phi, dphi);
        } else {
            if (z.rc_pair) {
                rin = z.rc_pair[2 * (ti * z.T + tj)];
                rout = z.rc_pair[2 * (ti * z.T + tj) + 1];
            }
            zbl_term(0.18175, 3.1998, x, phi, dphi);
            zbl_term(0.50986, 0.94229, x, phi, dphi);
            zbl_term(0.28022, 0.4029, x, phi, dphi);
            zbl_term(0.02817, 0.20162, x, phi, dphi);
        }
        // f = zizj phi / r and its r-derivative, then the switch
        double f = zizj * phi * rinv;
        double fp = zizj * a_inv * dphi * rinv - f * rinv;
        double fc = 0.0, fcp = 0.0;
        if (r < rin) {
            fc = 1.0;
        } else if (r < rout) {
            double sn, cs;
            sincospi((r - rin) / (rout - rin), &sn, &cs);
            fc = 0.5 * cs + 0.5;
            fcp = -0.5 * (3.141592653589793 / (rout - rin)) * sn;
        }
        fp = fp * fc + f * fcp;
        f *= fc;
        const double s = 0.5 * fp * rinv;
        const float4 g = P.g[e];
        P.g[e] = make_float4(g.x - (float)(s * dx), g.y - (float)(s * dy), g.z - (float)(s * dz), g.w);
        esum += 0.5 * f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(0xffffffffu, esum, o);
    if (lane == 0) e_atom[at] += esum;
}

cudaError_t launch_nep_zbl(const PairBufs& P, int n, const int* type, const ZblArgs& z, double* e_atom,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    return launch_pdl(&k_nep_zbl, dim3((unsigned)(((size_t)n * 32 + 255) / 256)), dim3(256), 0, st, P, n, type, z,
                      e_atom);
}

}  // namespace nnapgb
