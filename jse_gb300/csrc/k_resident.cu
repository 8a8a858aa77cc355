// Kernels of the resident (served) path: neighbour lists kept on the device between
// evaluations of the same structure.
//
// A rebuild runs the ordinary cell-list kernels at rc + skin and stores each row
// (k_verlet_store).  Every evaluation then wraps the new positions exactly as
// IBox.wrapPBC does (IBox.java:145-151), corrects each stored pair image by the change
// of the two atoms' wrap counts, and keeps the pairs with d^2 < rc^2 under the same
// FP64 rule as the full search (NeighborListGetter.java:1018-1050).  As long as no
// atom moved more than skin/2 since the rebuild, every pair within rc is among the
// stored ones, so the kept set equals the full search's set exactly.  Kept rows keep
// the stored (cell-offset group, atom) order, which the mirror search relies on.
#include "box_math.cuh"
#include "common.cuh"
#include "resident.cuh"

namespace nnapgb {

// Structure index and species of every atom of the tick (one CTA per structure).
__global__ void k_tick_atoms(const SlotDev* __restrict__ slots, int* __restrict__ sid, int* __restrict__ type_b) {
    const int s = blockIdx.x;
    const SlotDev sl = slots[s];
    for (int i = threadIdx.x; i < sl.n; i += blockDim.x) {
        sid[sl.a0 + i] = s;
        type_b[sl.a0 + i] = sl.type[i];
    }
}

// Wrap every atom into its box (same operations as k_wrap_bin) and record the lattice
// counts subtracted per direction.
__global__ void k_wrap_resident(const StructDev* __restrict__ S, const int* __restrict__ sid,
                                const double* __restrict__ x, const int* __restrict__ type, int n, int ntypes,
                                double* __restrict__ xw, float4* __restrict__ xf, float4* __restrict__ xlo,
                                int4* __restrict__ kw, int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StructDev& st = S[sid[i]];
    const int t = type[i];
    if (t < 1 || t > ntypes) atomicOr(err, ERRBIT_BAD_TYPE);
    double p[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    to_direct(st, p);
    int k[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        k[d] = 0;
        if (p[d] < 0.0 || p[d] >= 1.0) {
            const double f = floor(p[d]);
            k[d] = (int)fmax(fmin(f, 1.0e6), -1.0e6);
            p[d] = ds(p[d], f);
        }
    }
    to_cartesian(st, p);
    xw[3 * i] = p[0]; xw[3 * i + 1] = p[1]; xw[3 * i + 2] = p[2];
    const float hx = (float)p[0], hy = (float)p[1], hz = (float)p[2];
    xf[i] = make_float4(hx, hy, hz, __int_as_float(min(max(t, 1), ntypes)));  // clamped as in k_wrap_bin
    xlo[i] = make_float4((float)ds(p[0], (double)hx), (float)ds(p[1], (double)hy), (float)ds(p[2], (double)hz), 0.f);
    kw[i] = make_int4(k[0], k[1], k[2], 0);
}

// Copy the rebuilt rows (batch rows of capacity Mv, atoms [0, nbuild) of the tick) into
// the structures' resident arrays, with neighbour indices made local.  One warp per atom.
__global__ void k_verlet_store(const SlotDev* __restrict__ slots, const int* __restrict__ sid, PairBufs P, int nbuild,
                               const int4* __restrict__ kw) {
    const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (a >= nbuild) return;
    const SlotDev sl = slots[sid[a]];
    const int i = a - sl.a0;
    const int M = P.M;
    const int cnt = P.count[a];
    const int c = min(cnt, M);
    const size_t src = (size_t)a * M, dst = (size_t)i * M;
    for (int k = lane; k < c; k += 32) {
        const uint64_t key = P.key[src + k];
        const uint32_t j = (uint32_t)(key >> 32) - (uint32_t)sl.a0;
        sl.vkey[dst + k] = ((uint64_t)j << 32) | (uint32_t)key;
        sl.vgrp[dst + k] = P.grp[src + k];
    }
    if (lane == 0) {
        sl.vcnt[i] = cnt;
        sl.kb[i] = kw[a];
    }
}

// Keep the stored pairs that are within rc at the current positions.  One warp per
// atom; 32 stored entries per step, compacted with a ballot in stored order.  The
// image of entry (i -> j, n) becomes n + (m_j - mb_j) - (m_i - mb_i), m the current
// and mb the rebuild's wrap counts.  The test is the full search's: an FP32 screen,
// float-float d^2, and the exact FP64 test within 1e-10 * rc^2 of the cutoff.
constexpr int kFilterWarps = 4;

__global__ void __launch_bounds__(32 * kFilterWarps)
k_filter(const StructDev* __restrict__ S, const SlotDev* __restrict__ slots, const int* __restrict__ sid,
         const double* __restrict__ xw, const float4* __restrict__ xf, const float4* __restrict__ xlo,
         const int4* __restrict__ kw, int n, int Mv, PairBufs P, int* __restrict__ err, int* __restrict__ max_count) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.x * kFilterWarps + w;
    if (a >= n) return;
    const int s = sid[a];
    const StructDev& st = S[s];
    const SlotDev sl = slots[s];
    const int i = a - sl.a0;
    const int cv = min(sl.vcnt[i], Mv);
    const int M = P.M;
    const int4 mi = kw[a], bi = sl.kb[i];
    const int dia = mi.x - bi.x, dib = mi.y - bi.y, dic = mi.z - bi.z;
    const double xi = xw[3 * a], yi = xw[3 * a + 1], zi = xw[3 * a + 2];
    const float4 fi = xf[a];
    const float4 li = xlo[a];
    const float rc2h = (float)st.rc2, rc2l = (float)(st.rc2 - (double)(float)st.rc2);
    const float tol = 1e-10f * rc2h;
    const uint64_t* vrow = sl.vkey + (size_t)i * Mv;
    const uint16_t* grow = sl.vgrp + (size_t)i * Mv;
    int cnt = 0;
    for (int k0 = 0; k0 < cv; k0 += 32) {
        const int k = k0 + lane;
        bool acc = false;
        int jb = 0, na = 0, nb = 0, nc = 0;
        float ox = 0.f, oy = 0.f, oz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
        uint16_t g = 0;
        if (k < cv) {
            const uint64_t key = vrow[k];
            g = grow[k];
            const int jl = (int)(key >> 32);
            jb = sl.a0 + jl;
            unpack_img((uint32_t)key, na, nb, nc);
            const int4 mj = kw[jb], bj = sl.kb[jl];
            na += (mj.x - bj.x) - dia;
            nb += (mj.y - bj.y) - dib;
            nc += (mj.z - bj.z) - dic;
            if (max(abs(na), max(abs(nb), abs(nc))) >= kImgBias) {
                atomicOr(err, ERRBIT_CELLS);  // image beyond the packed range
            } else {
                // shift = na*a + nb*b + nc*c as float-float (exact products of the
                // integer counts with the split box rows)
                const float fna = (float)na, fnb = (float)nb, fnc = (float)nc;
                float shh[3], shl[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    float h = 0.f, l = 0.f;
                    ff_acc_prod(h, l, fna, st.fa[d]);
                    l += fna * st.la[d];
                    ff_acc_prod(h, l, fnb, st.fb[d]);
                    l += fnb * st.lb[d];
                    ff_acc_prod(h, l, fnc, st.fc[d]);
                    l += fnc * st.lc[d];
                    two_sum(h, l, shh[d], shl[d]);
                }
                const float4 fj = xf[jb];
                const float fx = (fj.x + shh[0]) - fi.x;
                const float fy = (fj.y + shh[1]) - fi.y;
                const float fz = (fj.z + shh[2]) - fi.z;
                if (fx * fx + fy * fy + fz * fz < st.rc2_hi) {
                    const float4 lj = xlo[jb];
                    float dh[3], dl[3];
                    const float ajh[3] = {fj.x, fj.y, fj.z}, ajl[3] = {lj.x, lj.y, lj.z};
                    const float aih[3] = {fi.x, fi.y, fi.z}, ail[3] = {li.x, li.y, li.z};
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        float s1, e1, s2, e2;
                        two_sum(ajh[d], shh[d], s1, e1);
                        two_sum(s1, -aih[d], s2, e2);
                        const float lo = ((ajl[d] + shl[d]) - ail[d]) + (e1 + e2);
                        two_sum(s2, lo, dh[d], dl[d]);
                    }
                    float d2h = 0.f, d2l = 0.f;
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        ff_acc_prod(d2h, d2l, dh[d], dh[d]);
                        d2l += 2.f * dh[d] * dl[d];
                    }
                    const float diff = (d2h - rc2h) + (d2l - rc2l);
                    if (fabsf(diff) > tol) {
                        acc = diff < 0.f;
                    } else {  // within 1e-10 of the cutoff: the exact FP64 test
                        double sh[3];
                        image_shift(st, na, nb, nc, sh);
                        const double dxv = ds(da(xw[3 * jb], sh[0]), xi);
                        const double dyv = ds(da(xw[3 * jb + 1], sh[1]), yi);
                        const double dzv = ds(da(xw[3 * jb + 2], sh[2]), zi);
                        acc = da(da(dm(dxv, dxv), dm(dyv, dyv)), dm(dzv, dzv)) < st.rc2;
                    }
                    two_sum(dh[0], dl[0], ox, lx);
                    two_sum(dh[1], dl[1], oy, ly);
                    two_sum(dh[2], dl[2], oz, lz);
                }
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        if (acc) {
            const int pos = cnt + __popc(m & ((1u << lane) - 1u));
            if (pos < M) {
                const size_t e = (size_t)a * M + pos;
                P.key[e] = pair_key(jb, pack_img(na, nb, nc));
                P.dx[e] = make_float4(ox, oy, oz, xf[jb].w);
                if (P.dxlo) P.dxlo[e] = make_float4(lx, ly, lz, 0.f);
                P.grp[e] = g;
            }
        }
        cnt += __popc(m);
    }
    if (lane == 0) {
        P.count[a] = cnt;
        if (cnt > M) atomicOr(err, ERRBIT_CAPACITY);
        atomicMax(max_count, cnt);
    }
}

}  // namespace nnapgb
