// Kernels of the LAMMPS-style boundary: rows built from a caller's full neighbour list
// over local and ghost atoms, and an atomic-free, deterministic scatter of the pair
// gradients onto every atom, ghosts included (their forces go back to their owners by
// the caller's reverse communication).
//
// Reference behaviour restated (nnap_interface_cuda.cu:12-169, 319-483):
//   rows        for local atom ii (i = ilist[ii]) and each listed j: dx = x_j - x_i and
//               the pair is kept when |dx|^2 < rcut^2 (initLammpsNeiKernel);
//   scatter     F_j += g, F_i -= g, per-atom virial dx (x) g on j in the order
//               xx, yy, zz, xy, xz, yz, yx, zx, zy (collectLammpsResultsKernel).
// The reference scatters with float atomics; here every atom gathers its incoming
// entries, sorted by entry index, so the sums have a fixed order.
#include "box_math.cuh"
#include "common.cuh"

namespace nnapgb {

// One warp per local atom: keep the listed neighbours within rcut (FP64 test), compacted
// in list order.  Rows are indexed by the position ii in ilist.
__global__ void k_lmp_rows(int inum, int nall, const int* __restrict__ ilist, const int* __restrict__ noff,
                           const int* __restrict__ nidx, const double* __restrict__ x, const int* __restrict__ type,
                           int ntypes, double rc2, PairBufs P, int* __restrict__ row_type, int* __restrict__ err,
                           int* __restrict__ max_count) {
    const int ii = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (ii >= inum) return;
    const int i = ilist[ii];
    if (i < 0 || i >= nall) {
        if (lane == 0) {
            atomicOr(err, ERRBIT_CELLS);
            P.count[ii] = 0;
            row_type[ii] = 1;
        }
        return;
    }
    const int ti = type[i];
    if (lane == 0) {
        row_type[ii] = ti;
        if (ti < 1 || ti > ntypes) atomicOr(err, ERRBIT_BAD_TYPE);
    }
    const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    const int b = noff[ii], e = noff[ii + 1];
    const int M = P.M;
    int cnt = 0;
    for (int k0 = b; k0 < e; k0 += 32) {
        const int k = k0 + lane;
        bool acc = false;
        int j = 0;
        double dx = 0.0, dy = 0.0, dz = 0.0;
        if (k < e) {
            j = nidx[k];
            if (j < 0 || j >= nall) {
                atomicOr(err, ERRBIT_CELLS);
            } else {
                dx = ds(x[3 * j], xi);
                dy = ds(x[3 * j + 1], yi);
                dz = ds(x[3 * j + 2], zi);
                acc = da(da(dm(dx, dx), dm(dy, dy)), dm(dz, dz)) < rc2;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        if (acc) {
            const int pos = cnt + __popc(m & ((1u << lane) - 1u));
            if (pos < M) {
                const size_t q = (size_t)ii * M + pos;
                P.key[q] = pair_key(j, pack_img(0, 0, 0));
                const int tj = type[j];
                if (tj < 1 || tj > ntypes) atomicOr(err, ERRBIT_BAD_TYPE);
                P.dx[q] = make_float4((float)dx, (float)dy, (float)dz, __int_as_float(min(max(tj, 1), ntypes)));
                if (P.dxlo)
                    P.dxlo[q] = make_float4((float)(dx - (double)(float)dx), (float)(dy - (double)(float)dy),
                                            (float)(dz - (double)(float)dz), 0.f);
                P.grp[q] = 0;
            }
        }
        cnt += __popc(m);
    }
    if (lane == 0) {
        P.count[ii] = cnt;
        if (cnt > M) atomicOr(err, ERRBIT_CAPACITY);
        atomicMax(max_count, cnt);
    }
}

// Number of row entries aimed at each atom (local or ghost).
__global__ void k_lmp_count(PairBufs P, int inum, int* __restrict__ tcount) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int M = P.M;
    const int ii = (int)(t / M), k = (int)(t % M);
    if (ii >= inum || k >= min(P.count[ii], M)) return;
    atomicAdd(&tcount[(int)(P.key[t] >> 32)], 1);
}

// Entry indices grouped by target atom (order inside a group fixed afterwards by sorting).
__global__ void k_lmp_fill(PairBufs P, int inum, const int* __restrict__ tstart, int* __restrict__ tfill,
                           int* __restrict__ tlist) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int M = P.M;
    const int ii = (int)(t / M), k = (int)(t % M);
    if (ii >= inum || k >= min(P.count[ii], M)) return;
    const int j = (int)(P.key[t] >> 32);
    tlist[tstart[j] + atomicAdd(&tfill[j], 1)] = (int)t;
}

// One thread per atom a: F_a = sum of incoming g - sum of g over a's own row (a local
// atom); per-atom virial W_a = sum over incoming entries of dx (x) g.  Float-float sums,
// FP64 output.
__global__ void k_lmp_gather(PairBufs P, int nall, const int* __restrict__ row_of, const int* __restrict__ tstart,
                             const int* __restrict__ tlist, double* __restrict__ forces, double* __restrict__ virials) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nall) return;
    const int M = P.M;
    float fh[3] = {0.f, 0.f, 0.f}, fl[3] = {0.f, 0.f, 0.f};
    float vh[9], vl[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) { vh[d] = 0.f; vl[d] = 0.f; }
    for (int q = tstart[a]; q < tstart[a + 1]; ++q) {
        const int e = tlist[q];
        const float4 g = P.g[e];
        const float4 d = P.dx[e];
        ff_acc(fh[0], fl[0], g.x);
        ff_acc(fh[1], fl[1], g.y);
        ff_acc(fh[2], fl[2], g.z);
        ff_acc_prod(vh[0], vl[0], d.x, g.x);
        ff_acc_prod(vh[1], vl[1], d.y, g.y);
        ff_acc_prod(vh[2], vl[2], d.z, g.z);
        ff_acc_prod(vh[3], vl[3], d.x, g.y);
        ff_acc_prod(vh[4], vl[4], d.x, g.z);
        ff_acc_prod(vh[5], vl[5], d.y, g.z);
        ff_acc_prod(vh[6], vl[6], d.y, g.x);
        ff_acc_prod(vh[7], vl[7], d.z, g.x);
        ff_acc_prod(vh[8], vl[8], d.z, g.y);
    }
    const int r = row_of[a];
    if (r >= 0) {
        const int c = min(P.count[r], M);
        for (int k = 0; k < c; ++k) {
            const float4 g = P.g[(size_t)r * M + k];
            ff_acc(fh[0], fl[0], -g.x);
            ff_acc(fh[1], fl[1], -g.y);
            ff_acc(fh[2], fl[2], -g.z);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) forces[3 * (size_t)a + d] = (double)fh[d] + (double)fl[d];
#pragma unroll
    for (int d = 0; d < 9; ++d) virials[9 * (size_t)a + d] = (double)vh[d] + (double)vl[d];
}

}  // namespace nnapgb

namespace nnapgb {

// Global virial: the first six components of every atom's virial summed in double in a
// fixed order (thread t takes atoms t, t + blockDim, ...; then a tree over the threads).
__global__ void __launch_bounds__(kLmpSumThreads) k_lmp_virial_sum(const double* __restrict__ virials, int nall,
                                                                   double* __restrict__ out) {
    __shared__ double s[6][kLmpSumThreads];
    const int t = threadIdx.x;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int a = t; a < nall; a += kLmpSumThreads)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] += virials[9 * (size_t)a + c];
#pragma unroll
    for (int c = 0; c < 6; ++c) s[c][t] = acc[c];
    __syncthreads();
    for (int w = kLmpSumThreads / 2; w > 0; w >>= 1) {
        if (t < w)
#pragma unroll
            for (int c = 0; c < 6; ++c) s[c][t] += s[c][t + w];
        __syncthreads();
    }
    if (t < 6) out[t] = s[t][0];
}

}  // namespace nnapgb
