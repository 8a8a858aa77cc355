// Structure kernels: FP64 wrapping and cell binning, the full neighbour list,
// the mirror index used by the atomic-free scatter, the species sort of atoms,
// the force / per-atom virial gather and the per-structure FP64 reductions.
//
// Reference behaviour restated here:
//   wrapping        IBox.wrapPBC / toDirect / toCartesian (IBox.java:145-222,
//                   BoxPrism.java:162-175), including the snap of direct coordinates
//                   within 1e-10 of an integer (MathEX.java:1213).  All FP64 operations
//                   use explicit round-to-nearest intrinsics so that no multiply-add is
//                   contracted and every rounding matches the reference's Java doubles.
//   neighbours      NeighborListGetter.forEachNeighbor_ with check=true, half=false
//                   (NeighborListGetter.java:1018-1050): all periodic images j' with
//                   |(x_j + shift) - x_i|^2 < rcut^2 evaluated in FP64, images of i
//                   itself included, (i, zero image) excluded (NeighborListGetter.java:119-173).
//   scatter         NNAP.calEnergyForceVirial + IPairPotential accumulators
//                   (NNAP.java:571-592, IPairPotential.java:919-1006): F_i -= g_ij,
//                   F_j += g_ij, per-atom virial dx_ij (x) g_ij on j; computed here as a
//                   gather over each atom's own row and the mirrored entries, without atomics.
#include "box_math.cuh"
#include "common.cuh"
#include "pdl.cuh"

namespace nnapgb {

// ----------------------------------------------------------------- wrap + cell binning
// One thread per atom: wrap into the box, record the float copy used by the
// candidate screen and the atom's cell, and count atoms per cell.
__global__ void k_wrap_bin(const StructDev* __restrict__ S, const int* __restrict__ sid, const double* __restrict__ x,
                           const int* __restrict__ type, int n, int ntypes, double* __restrict__ xw,
                           float4* __restrict__ xf, float4* __restrict__ xlo, int* __restrict__ cell_of,
                           int* __restrict__ cell_count, int* __restrict__ err) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StructDev& st = S[sid[i]];
    const int t = type[i];
    if (t < 1 || t > ntypes) atomicOr(err, ERRBIT_BAD_TYPE);
    double p[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    to_direct(st, p);
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (p[d] < 0.0 || p[d] >= 1.0) p[d] = ds(p[d], floor(p[d]));
    // the cell comes from these wrapped direct coordinates: every atom is binned by the same
    // rule, and the stencil's slack (R cells cover at least rc plus 1e-6 of a cell) dwarfs
    // their rounding, so no second conversion of the wrapped position is needed
    const double f[3] = {p[0], p[1], p[2]};
    to_cartesian(st, p);
    xw[3 * i] = p[0]; xw[3 * i + 1] = p[1]; xw[3 * i + 2] = p[2];
    const float hx = (float)p[0], hy = (float)p[1], hz = (float)p[2];
    // the species the pair rows carry, clamped into 1..ntypes: a bad species fails the call
    // (ERRBIT_BAD_TYPE) and indexes nothing out of range meanwhile
    xf[i] = make_float4(hx, hy, hz, __int_as_float(min(max(t, 1), ntypes)));
    // x = hi + lo exactly to 48 bits: the float-float form used by the neighbour test
    xlo[i] = make_float4((float)ds(p[0], (double)hx), (float)ds(p[1], (double)hy), (float)ds(p[2], (double)hz), 0.f);
    int c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int ci = (int)floor(f[d] * (double)st.nc[d]);
        c[d] = min(max(ci, 0), st.nc[d] - 1);
    }
    const int cid = st.c0 + c[0] + st.nc[0] * (c[1] + st.nc[1] * c[2]);
    cell_of[i] = cid;
    atomicAdd(&cell_count[cid], 1);
}

// Exclusive scan of n ints (one CTA of 1024 threads, sequential chunks); out has n+1 entries.
__global__ void k_scan_excl(const int* __restrict__ in, int n, int* __restrict__ out) {
    pdl_enter();
    __shared__ int warp_tot[32];
    __shared__ int carry;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + tid;
        int v = i < n ? in[i] : 0;
        int s = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += u;
        }
        if (lane == 31) warp_tot[w] = s;
        __syncthreads();
        if (w == 0) {
            int t = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int u = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += u;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const int before = (w ? warp_tot[w - 1] : 0) + carry;
        if (i < n) out[i] = before + s - v;
        __syncthreads();
        if (tid == 1023) carry = before + s;
        __syncthreads();
    }
    if (tid == 0) out[n] = carry;
}

__global__ void k_fill_cells(const int* __restrict__ cell_of, int n, const int* __restrict__ cell_start,
                             int* __restrict__ cell_fill, int* __restrict__ cell_atoms) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell_of[i];
    cell_atoms[cell_start[c] + atomicAdd(&cell_fill[c], 1)] = i;
}

// Order each cell's atoms by index so that every neighbour row is deterministic.
// One warp per cell (8 per CTA of 256 threads): up to 32 atoms are placed by rank from
// registers; up to kSortCellMax atoms by rank from a copy of the cell in shared memory (the
// small boxes of a batch have cells of a hundred atoms); larger cells are sorted by lane 0.
constexpr int kSortCellMax = 1024;

__global__ void k_sort_cells(const int* __restrict__ cell_start, int ncells, int* __restrict__ cell_atoms) {
    pdl_enter();
    __shared__ int s_cell[8][kSortCellMax];
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, w = (threadIdx.x >> 5) & 7;
    if (c >= ncells) return;
    const int b = cell_start[c], e = cell_start[c + 1], m = e - b;
    if (m <= 32) {
        const int v = lane < m ? cell_atoms[b + lane] : 0x7fffffff;
        int rank = 0;
        for (int q = 0; q < m; ++q) {
            const int u = __shfl_sync(0xffffffffu, v, q);
            rank += (u < v) ? 1 : 0;
        }
        __syncwarp();
        if (lane < m) cell_atoms[b + rank] = v;
    } else if (m <= kSortCellMax) {
        for (int t = lane; t < m; t += 32) s_cell[w][t] = cell_atoms[b + t];
        __syncwarp();
        for (int t = lane; t < m; t += 32) {
            const int v = s_cell[w][t];
            int rank = 0;
            for (int q = 0; q < m; ++q) rank += s_cell[w][q] < v ? 1 : 0;
            cell_atoms[b + rank] = v;
        }
    } else if (lane == 0) {
        for (int k = b + 1; k < e; ++k) {
            const int v = cell_atoms[k];
            int q = k - 1;
            while (q >= b && cell_atoms[q] > v) { cell_atoms[q + 1] = cell_atoms[q]; --q; }
            cell_atoms[q + 1] = v;
        }
    }
}

// ----------------------------------------------------------------- neighbour rows
// One warp per atom.  Candidate cells are visited in a fixed order; within a batch
// of 32 cells the candidates are spread over the lanes, screened in FP32 against
// rc^2 plus a rounding margin, and confirmed with the exact FP64 test.  Accepted
// pairs are compacted in candidate order with a ballot, so rows are deterministic.
// Candidate positions are read from the cell-ordered copies xfc / xloc (k_cell_order), so
// a lane's atom index and position loads are independent and a cell's candidates are
// contiguous in memory.
constexpr int kNbMaxWarps = 8;  // warps per CTA are a launch parameter (2, 4 or 8)

// floor(a / b) for b >= 1 and |a| < 2^22, from a float reciprocal of b and one correction
// step (the float quotient is within one of the true one).
__device__ __forceinline__ int floor_div(int a, int b, float inv_b) {
    int q = __float2int_rd((float)a * inv_b);
    const int r = a - q * b;
    if (r < 0) --q;
    else if (r >= b) ++q;
    return q;
}

// xfc[k] = xf[cell_atoms[k]], xloc[k] = xlo[cell_atoms[k]] for the n binned atoms.
__global__ void __launch_bounds__(256) k_cell_order(const int* __restrict__ cell_atoms, int n,
                                                    const float4* __restrict__ xf, const float4* __restrict__ xlo,
                                                    float4* __restrict__ xfc, float4* __restrict__ xloc) {
    pdl_enter();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int a = cell_atoms[k];
    xfc[k] = xf[a];
    xloc[k] = xlo[a];
}

// Renumber the atoms of an evaluation in cell order: position k of the sorted cell lists
// takes the float positions and low parts (xfc / xloc), the FP64 wrapped position, the cell
// and the species of the atom there, and orig[k] records that atom; the cell lists become
// the identity.  Rows, pair keys and per-atom work arrays then use cell-order numbers, so
// the rows of atoms close in space are close in memory (the mirror search and the gather
// read the rows of each atom's neighbours).  A structure's atoms keep their index range.
__global__ void __launch_bounds__(256) k_renumber(int* __restrict__ cell_atoms, int n, const float4* __restrict__ xf,
                                                  const float4* __restrict__ xlo, const double* __restrict__ xw,
                                                  const int* __restrict__ cell_of, const int* __restrict__ type,
                                                  float4* __restrict__ xfc, float4* __restrict__ xloc,
                                                  double* __restrict__ xw2, int* __restrict__ cell_of2,
                                                  int* __restrict__ type2, int* __restrict__ orig) {
    pdl_enter();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int a = cell_atoms[k];
    xfc[k] = xf[a];
    xloc[k] = xlo[a];
    xw2[3 * (size_t)k] = xw[3 * (size_t)a];
    xw2[3 * (size_t)k + 1] = xw[3 * (size_t)a + 1];
    xw2[3 * (size_t)k + 2] = xw[3 * (size_t)a + 2];
    cell_of2[k] = cell_of[a];
    type2[k] = type[a];
    orig[k] = a;
    cell_atoms[k] = k;
}

// out[orig[k]] = in[k]: a per-atom array of a cell-ordered evaluation back in atom order.
__global__ void k_unpermute(const double* __restrict__ in, const int* __restrict__ orig, int n,
                            double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[orig[k]] = in[k];
}

__global__ void __launch_bounds__(32 * kNbMaxWarps, 4)
k_neighbors(const StructDev* __restrict__ S, const int* __restrict__ sid, const double* __restrict__ xw,
            const float4* __restrict__ xf, const float4* __restrict__ xlo, const float4* __restrict__ xfc,
            const float4* __restrict__ xloc, const int* __restrict__ cell_of, const int* __restrict__ cell_start,
            const int* __restrict__ cell_atoms, int n, PairBufs P, int* __restrict__ err,
            int* __restrict__ max_count) {
    pdl_enter();
    __shared__ int s_base[kNbMaxWarps][32];     // per cell slot: cell-order start minus candidate start
    __shared__ int s_slot_at[kNbMaxWarps][32];  // cell slot starting at each position of a window
    // per cell slot: the image shift's high parts and the packed image (one 16-byte load in
    // the candidate loop), and the shift's low parts (the float-float test)
    __shared__ float4 s_sh4[kNbMaxWarps][32];
    __shared__ float s_flo[kNbMaxWarps][32][3];
    __shared__ int s_acc[kNbMaxWarps][32];  // accepted entries per cell-offset group of the batch
    __shared__ int s_qs[kNbMaxWarps][64];   // candidates passing the FP32 screen: cell slot,
    __shared__ int s_qk[kNbMaxWarps][64];   // position in cell order
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + w;
    if (i >= n) return;
    const StructDev& st = S[sid[i]];
    const int M = P.M;
    const int cl = cell_of[i] - st.c0;
    const int ci0 = cl % st.nc[0], ci1 = (cl / st.nc[0]) % st.nc[1], ci2 = cl / (st.nc[0] * st.nc[1]);
    const int wa = 2 * st.R[0] + 1, wb = 2 * st.R[1] + 1;
    const int noff = wa * wb * (2 * st.R[2] + 1);
    const float4 fi = xf[i];
    const float4 li = xlo[i];

    const float rc2h = (float)st.rc2, rc2l = (float)(st.rc2 - (double)(float)st.rc2);
    const float rc2_hi = st.rc2_hi;
    const float tol = 1e-10f * rc2h;  // float-float d^2 is accurate to ~1e-12 relative
    int cnt = 0;
    const bool keep_groups = P.GS > noff;
    for (int o0 = 0; o0 < noff; o0 += 32) {
        const int o = o0 + lane;
        const int cnt0 = cnt;
        s_acc[w][lane] = 0;
        int ccount = 0, cs = 0;
        if (o < noff) {
            const float inv_wa = __frcp_rn((float)wa), inv_wb = __frcp_rn((float)wb);
            const float inv_nc0 = __frcp_rn((float)st.nc[0]), inv_nc1 = __frcp_rn((float)st.nc[1]),
                        inv_nc2 = __frcp_rn((float)st.nc[2]);
            const int oab = floor_div(o, wa, inv_wa), ocr = floor_div(oab, wb, inv_wb);
            const int oa = o - oab * wa - st.R[0], ob = oab - ocr * wb - st.R[1], oc = ocr - st.R[2];
            const int q0 = ci0 + oa, q1 = ci1 + ob, q2 = ci2 + oc;
            const int na = floor_div(q0, st.nc[0], inv_nc0);
            const int nb = floor_div(q1, st.nc[1], inv_nc1);
            const int nc = floor_div(q2, st.nc[2], inv_nc2);
            const int c0 = q0 - na * st.nc[0], c1 = q1 - nb * st.nc[1], c2 = q2 - nc * st.nc[2];
            const int cid = st.c0 + c0 + st.nc[0] * (c1 + st.nc[1] * c2);
            cs = cell_start[cid];
            ccount = cell_start[cid + 1] - cs;
            if (st.kind == 0) {
                // orthogonal box: a lower bound of the distance from atom i to the target
                // cell (unwrapped cell q spans [q, q+1) cell widths); cells beyond the screen
                // bound (rc^2 plus its rounding margin) hold no neighbour and are skipped
                const float wx = st.fa[0] / (float)st.nc[0], wy = st.fb[1] / (float)st.nc[1],
                            wz = st.fc[2] / (float)st.nc[2];
                const float gx = fmaxf(0.f, fmaxf((float)q0 * wx - fi.x, fi.x - (float)(q0 + 1) * wx));
                const float gy = fmaxf(0.f, fmaxf((float)q1 * wy - fi.y, fi.y - (float)(q1 + 1) * wy));
                const float gz = fmaxf(0.f, fmaxf((float)q2 * wz - fi.z, fi.z - (float)(q2 + 1) * wz));
                if (gx * gx + gy * gy + gz * gz > rc2_hi) ccount = 0;
            } else if (st.smin2 > 0.f) {
                // skewed box: the gap in direct coordinates times the box's smallest
                // singular value bounds the Cartesian distance from below (the atom's
                // direct coordinates are formed here, so they hold no register in the
                // candidate loop)
                const int q[3] = {q0, q1, q2};
                float g2 = 0.f;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float ui = st.iv[d][0] * fi.x + st.iv[d][1] * fi.y + st.iv[d][2] * fi.z;
                    const float inv_n = 1.f / (float)st.nc[d];
                    const float g = fmaxf(0.f, fmaxf((float)q[d] * inv_n - ui, ui - (float)(q[d] + 1) * inv_n));
                    g2 += g * g;
                }
                if (st.smin2 * g2 > rc2_hi) ccount = 0;
            }

            // the image shift as float-float on the FP32 pipe (the exact test forms the FP64
            // shift itself); the zero image has an exactly zero shift
            float hi[3], lo[3];
            image_shift_ff(st, na, nb, nc, hi, lo);
            s_sh4[w][lane] = make_float4(hi[0], hi[1], hi[2], __uint_as_float(pack_img(na, nb, nc)));
#pragma unroll
            for (int d = 0; d < 3; ++d) s_flo[w][lane][d] = lo[d];
        }
        int incl = ccount;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += u;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int before = incl - ccount;  // candidates of the earlier cell slots
        s_base[w][lane] = cs - before;
        __syncwarp();
        // Candidates are screened 32 at a time in FP32; the ones that pass (about one in four
        // or five) queue in candidate order in shared memory and take the exact test 32 at a
        // time, so its lanes stay busy.  Accepted entries keep candidate order.
        int qn = 0;  // queued candidates (warp-uniform)
        auto exact_batch = [&](int k) {  // the first k queued candidates
            bool acc = false;
            int j = 0, slot = 0;
            uint32_t img = 0;
            float4 fj = make_float4(0.f, 0.f, 0.f, 0.f);
            float ox = 0.f, oy = 0.f, oz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
            if (lane < k) {
                slot = s_qs[w][lane];
                const int kp = s_qk[w][lane];
                j = cell_atoms[kp];
                const float4 s4 = s_sh4[w][slot];
                const float sh[3] = {s4.x, s4.y, s4.z};
                img = __float_as_uint(s4.w);
                fj = xfc[kp];
                const float4 lj = xloc[kp];
                // (x_j + shift) - x_i in float-float, then d^2 in float-float
                float dh[3], dl[3];
                const float ajh[3] = {fj.x, fj.y, fj.z}, ajl[3] = {lj.x, lj.y, lj.z};
                const float aih[3] = {fi.x, fi.y, fi.z}, ail[3] = {li.x, li.y, li.z};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    float s1, e1, s2, e2;
                    two_sum(ajh[d], sh[d], s1, e1);
                    two_sum(s1, -aih[d], s2, e2);
                    const float lo = ((ajl[d] + s_flo[w][slot][d]) - ail[d]) + (e1 + e2);
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
                    int na, nb, nc;
                    unpack_img(img, na, nb, nc);
                    double sh[3] = {0.0, 0.0, 0.0};
                    if (na | nb | nc) image_shift(st, na, nb, nc, sh);
                    const double dxv = ds(da(xw[3 * j], sh[0]), xw[3 * i]);
                    const double dyv = ds(da(xw[3 * j + 1], sh[1]), xw[3 * i + 1]);
                    const double dzv = ds(da(xw[3 * j + 2], sh[2]), xw[3 * i + 2]);
                    acc = da(da(dm(dxv, dxv), dm(dyv, dyv)), dm(dzv, dzv)) < st.rc2;
                }
                if (j == i && img == pack_img(0, 0, 0)) acc = false;  // the atom itself
                two_sum(dh[0], dl[0], ox, lx);
                two_sum(dh[1], dl[1], oy, ly);
                two_sum(dh[2], dl[2], oz, lz);
            }
            const unsigned m = __ballot_sync(0xffffffffu, acc);
            if (acc) {
                const int pos = cnt + __popc(m & ((1u << lane) - 1u));
                if (pos < M) {
                    const size_t e = (size_t)i * M + pos;
                    P.key[e] = pair_key(j, img);
                    P.dx[e] = make_float4(ox, oy, oz, fj.w);
                    if (P.dxlo) P.dxlo[e] = make_float4(lx, ly, lz, 0.f);
                    P.grp[e] = (uint16_t)(o0 + slot);
                }
                if (keep_groups) atomicAdd(&s_acc[w][slot], 1);
            }
            cnt += __popc(m);
        };
        // The cell slot of candidate cidx: the last nonempty slot starting at or before it.
        // Per window of 32 candidates the starting positions form a bit mask (one OR
        // reduction); a lane takes the highest start at or below its position, or the slot
        // that ran into the window from the one before.
        int carry = 0;
        for (int cb = 0; cb < total; cb += 32) {
            const int cidx = cb + lane;
            const bool starts = ccount > 0 && before >= cb && before < cb + 32;
            const unsigned smask = __reduce_or_sync(0xffffffffu, starts ? 1u << (before - cb) : 0u);
            if (starts) s_slot_at[w][before - cb] = lane;
            __syncwarp();
            const unsigned mine = smask & (0xffffffffu >> (31 - lane));
            const int slot = mine ? s_slot_at[w][31 - __clz(mine)] : carry;
            carry = __shfl_sync(0xffffffffu, slot, 31);
            // the screen reads only the candidate's cell-order position; its atom index is
            // loaded by the exact test, which also drops the atom itself (zero image)
            bool pass = false;
            int kp = 0;
            if (cidx < total) {
                kp = s_base[w][slot] + cidx;
                const float4 fj = xfc[kp];
                const float4 sh = s_sh4[w][slot];
                const float fx = (fj.x + sh.x) - fi.x;
                const float fy = (fj.y + sh.y) - fi.y;
                const float fz = (fj.z + sh.z) - fi.z;
                pass = fx * fx + fy * fy + fz * fz < rc2_hi;
            }
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (pass) {
                const int q = qn + __popc(m & ((1u << lane) - 1u));
                s_qs[w][q] = slot;
                s_qk[w][q] = kp;
            }
            qn += __popc(m);
            __syncwarp();
            if (qn >= 32) {
                exact_batch(32);
                // move the overflow (at most 31 entries) to the front of the queue
                int rs = 0, rk = 0;
                if (lane < qn - 32) {
                    rs = s_qs[w][32 + lane];
                    rk = s_qk[w][32 + lane];
                }
                __syncwarp();
                if (lane < qn - 32) {
                    s_qs[w][lane] = rs;
                    s_qk[w][lane] = rk;
                }
                qn -= 32;
                __syncwarp();
            }
        }
        if (qn > 0) exact_batch(qn);
        __syncwarp();
        if (keep_groups) {  // start of each group of this batch: cnt0 + accepted entries of earlier groups
            const int a = s_acc[w][lane];
            int incl2 = a;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl2, d);
                if (lane >= d) incl2 += u;
            }
            if (o < noff) P.gstart[(size_t)i * P.GS + o] = cnt0 + incl2 - a;
        }
        __syncwarp();
    }
    if (lane == 0) {
        if (keep_groups) P.gstart[(size_t)i * P.GS + noff] = cnt;
        P.count[i] = cnt;
        if (cnt > M) atomicOr(err, ERRBIT_CAPACITY);
        atomicMax(max_count, cnt);
    }
}

// Mirror index: for entry (i -> j, image n) the position of (j -> i, image -n) in j's row.
// Rows are ordered by (cell-offset group, atom index); the mirrored entry lies in group
// noff-1-g of j's row (the negated cell offset).  With group starts kept, it is found
// by a scan of that group (a few entries); otherwise by binary search on (group, atom).
// One warp per row.
__global__ void k_mirror(const StructDev* __restrict__ S, const int* __restrict__ sid, PairBufs P, int n,
                         int* __restrict__ err) {
    pdl_enter();
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const int M = P.M;
    const int ci = min(P.count[i], M);
    const StructDev& st = S[sid[i]];
    const int noff = (2 * st.R[0] + 1) * (2 * st.R[1] + 1) * (2 * st.R[2] + 1);
    const bool groups = P.GS > noff;
    for (int k = lane; k < ci; k += 32) {
        const size_t e = (size_t)i * M + k;
        const uint64_t key = P.key[e];
        const int j = (int)(key >> 32);
        const int want_g = noff - 1 - P.grp[e];
        int na, nb, nc;
        unpack_img((uint32_t)key, na, nb, nc);
        const uint64_t target = pair_key(i, pack_img(-na, -nb, -nc));
        const int cj = min(P.count[j], M);
        const uint64_t* row = P.key + (size_t)j * M;
        int found = -1;
        if (groups) {
            const int* gs = P.gstart + (size_t)j * P.GS;
            const int lo = min(gs[want_g], cj), hi = min(gs[want_g + 1], cj);
            for (int q = lo; q < hi; ++q)
                if (row[q] == target) {
                    found = q;
                    break;
                }
        } else {
            const uint16_t* grow = P.grp + (size_t)j * M;
            const uint64_t want = ((uint64_t)(uint32_t)want_g << 32) | (uint32_t)i;
            int lo = 0, hi = cj;  // first q with composite(q) >= want
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                const uint64_t c = ((uint64_t)grow[mid] << 32) | (uint32_t)(row[mid] >> 32);
                if (c < want) lo = mid + 1; else hi = mid;
            }
            if (lo < cj && row[lo] == target) found = lo;
        }
        if (found >= 0) {
            P.rev[e] = (int)((size_t)j * M + found);
        } else {
            atomicOr(err, ERRBIT_NO_MIRROR);
            P.rev[e] = (int)e;
        }
    }
}

// ----------------------------------------------------------------- species sort
constexpr int kSortBlock = 256;

__global__ void k_type_hist(const int* __restrict__ type, int n, int T, int* __restrict__ block_counts) {
    pdl_enter();
    __shared__ int h[kMaxTypes];
    if (threadIdx.x < kMaxTypes) h[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * kSortBlock + threadIdx.x;
    if (i < n) {
        const int t = type[i] - 1;
        if (t >= 0 && t < T) atomicAdd(&h[t], 1);
    }
    __syncthreads();
    if (threadIdx.x < T) block_counts[blockIdx.x * T + threadIdx.x] = h[threadIdx.x];
}

// In place: block_counts -> exclusive offsets in (type, block) order; type_start[T+1].
__global__ void k_type_offsets(int* __restrict__ block_counts, int nb, int T, int* __restrict__ type_start) {
    pdl_enter();
    __shared__ int warp_tot[32];
    __shared__ int carry;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int t = 0; t < T; ++t) {
        if (tid == 0) type_start[t] = carry;
        __syncthreads();
        for (int base = 0; base < nb; base += 1024) {
            const int b = base + tid;
            const int v = b < nb ? block_counts[b * T + t] : 0;
            int s = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int u = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += u;
            }
            if (lane == 31) warp_tot[w] = s;
            __syncthreads();
            if (w == 0) {
                int q = warp_tot[lane];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int u = __shfl_up_sync(0xffffffffu, q, o);
                    if (lane >= o) q += u;
                }
                warp_tot[lane] = q;
            }
            __syncthreads();
            const int before = (w ? warp_tot[w - 1] : 0) + carry;
            if (b < nb) block_counts[b * T + t] = before + s - v;
            __syncthreads();
            if (tid == 1023) carry = before + s;
            __syncthreads();
        }
    }
    if (tid == 0) type_start[T] = carry;
}

// Stable scatter: slot = offset(type, block) + rank of the atom among same-type atoms of its block.
__global__ void k_type_scatter(const int* __restrict__ type, int n, int T, const int* __restrict__ block_offsets,
                               int* __restrict__ perm) {
    pdl_enter();
    __shared__ int wc[kSortBlock / 32][kMaxTypes];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * kSortBlock + threadIdx.x;
    const int t = i < n ? type[i] - 1 : -1;
    unsigned mine = 0;
    for (int q = 0; q < T; ++q) {
        const unsigned m = __ballot_sync(0xffffffffu, t == q);
        if (lane == 0) wc[w][q] = __popc(m);
        if (t == q) mine = m;
    }
    __syncthreads();
    if (t < 0 || t >= T) return;
    int rank = __popc(mine & ((1u << lane) - 1u));
    for (int q = 0; q < w; ++q) rank += wc[q][t];
    perm[block_offsets[blockIdx.x * T + t] + rank] = i;
}

// ----------------------------------------------------------------- gather
// kGatherLanes lanes per atom a: F_a = sum_k (g[mirror(a,k)] - g[a,k]);
// W_a = sum_k dx[mirror(a,k)] (x) g[mirror(a,k)], with dx[mirror(a,k)] = -dx[a,k] (the
// mirrored displacement is the negated one; both are the same exact value rounded to
// nearest, which is symmetric under negation).  Each lane sums every kGatherLanes-th entry
// of the row as float-float pairs (exact products, error-free additions); the partial sums
// are combined by a fixed xor butterfly, so the result does not depend on timing.
// Own-row loads are coalesced; only g of the mirrored entry is a scattered load.  Four
// lanes per atom (eight atoms per warp) beat eight: 0.416 -> 0.347 ms on the batch.
constexpr int kGatherLanes = 4;

__device__ __forceinline__ void ff_merge(float& h, float& l, unsigned mask, int off) {
    const float oh = __shfl_xor_sync(mask, h, off), ol = __shfl_xor_sync(mask, l, off);
    float s, e;
    two_sum(h, oh, s, e);
    h = s;
    l = (l + ol) + e;
}

// orig: the atom of each row (rows in cell order), or NULL (rows are atoms).
__global__ void k_gather(PairBufs P, int n, const int* __restrict__ orig, double* __restrict__ forces,
                         double* __restrict__ virials) {
    pdl_enter();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = t / kGatherLanes, sub = t & (kGatherLanes - 1);
    if (a >= n) return;  // all lanes of an atom leave together
    const unsigned mask = ((1u << kGatherLanes) - 1u) << ((threadIdx.x & 31) & ~(kGatherLanes - 1));
    const int M = P.M;
    const int cnt = min(P.count[a], M);
    float fh[3] = {0.f, 0.f, 0.f}, fl[3] = {0.f, 0.f, 0.f};
    float vh[9], vl[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) { vh[d] = 0.f; vl[d] = 0.f; }
    const size_t row = (size_t)a * M;
    // two entries per step: both mirrored-gradient loads (an index load, then a gather) are
    // in flight before either is used; the second entry's terms are added after the first's,
    // so the summation order is that of one entry per step
    for (int k0 = sub; k0 < cnt; k0 += 2 * kGatherLanes) {
        const int k1 = k0 + kGatherLanes;
        const bool two = k1 < cnt;
        const int r0 = P.rev[row + k0], r1 = two ? P.rev[row + k1] : r0;
        const float4 gr0 = P.g[r0], gr1 = P.g[r1];
        const float4 go0 = P.g[row + k0], go1 = two ? P.g[row + k1] : go0;
        const float4 dn0 = P.dx[row + k0], dn1 = two ? P.dx[row + k1] : dn0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (h == 1 && !two) break;
            const float4 go = h ? go1 : go0;
            const float4 dn = h ? dn1 : dn0;
            const float4 gr = h ? gr1 : gr0;
            const float dx = -dn.x, dy = -dn.y, dz = -dn.z;
            ff_acc(fh[0], fl[0], gr.x); ff_acc(fh[0], fl[0], -go.x);
            ff_acc(fh[1], fl[1], gr.y); ff_acc(fh[1], fl[1], -go.y);
            ff_acc(fh[2], fl[2], gr.z); ff_acc(fh[2], fl[2], -go.z);
            ff_acc_prod(vh[0], vl[0], dx, gr.x);
            ff_acc_prod(vh[1], vl[1], dy, gr.y);
            ff_acc_prod(vh[2], vl[2], dz, gr.z);
            ff_acc_prod(vh[3], vl[3], dx, gr.y);
            ff_acc_prod(vh[4], vl[4], dx, gr.z);
            ff_acc_prod(vh[5], vl[5], dy, gr.z);
            ff_acc_prod(vh[6], vl[6], dy, gr.x);
            ff_acc_prod(vh[7], vl[7], dz, gr.x);
            ff_acc_prod(vh[8], vl[8], dz, gr.y);
        }
    }
#pragma unroll
    for (int off = kGatherLanes / 2; off > 0; off >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) ff_merge(fh[d], fl[d], mask, off);
#pragma unroll
        for (int d = 0; d < 9; ++d) ff_merge(vh[d], vl[d], mask, off);
    }
    if (sub == 0) {
        const size_t o = orig ? (size_t)orig[a] : (size_t)a;
#pragma unroll
        for (int d = 0; d < 3; ++d) forces[3 * o + d] = (double)fh[d] + (double)fl[d];
#pragma unroll
        for (int d = 0; d < 9; ++d) virials[9 * o + d] = (double)vh[d] + (double)vl[d];
    }
}

// ----------------------------------------------------------------- per-structure totals
// chunk c covers atoms [cb[c], ce[c]); partial[c][0] = sum E, partial[c][1..9] = sum W.
constexpr int kRedBlock = 256;

__global__ void k_reduce_chunks(const int* __restrict__ cb, const int* __restrict__ ce,
                                const double* __restrict__ e_atom, const double* __restrict__ virials,
                                double* __restrict__ partial) {
    pdl_enter();
    __shared__ double sm[10][kRedBlock / 32];
    const int c = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = cb[c] + threadIdx.x; a < ce[c]; a += kRedBlock) {
        s[0] += e_atom[a];
#pragma unroll
        for (int d = 0; d < 9; ++d) s[1 + d] += virials[9 * (size_t)a + d];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int d = 0; d < 10; ++d) s[d] += __shfl_xor_sync(0xffffffffu, s[d], o);
    if (lane == 0)
#pragma unroll
        for (int d = 0; d < 10; ++d) sm[d][w] = s[d];
    __syncthreads();
    if (threadIdx.x < 10) {
        double t = 0.0;
        for (int q = 0; q < kRedBlock / 32; ++q) t += sm[threadIdx.x][q];
        partial[10 * (size_t)c + threadIdx.x] = t;
    }
}

// structure s owns chunks [sc[s], sc[s+1]); one warp per structure, fixed summation order.
__global__ void k_reduce_structs(const int* __restrict__ sc, int nstruct, const double* __restrict__ partial,
                                 double* __restrict__ energy, double* __restrict__ virial) {
    pdl_enter();
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nstruct) return;
    double t = 0.0;
    const int nv = 10;
    // lanes 0..9 each own one of the 10 totals and add the chunks in order
    if (lane < nv)
        for (int c = sc[s]; c < sc[s + 1]; ++c) t += partial[10 * (size_t)c + lane];
    if (lane == 0) energy[s] = t;
    else if (lane < nv) virial[9 * (size_t)s + lane - 1] = t;
}

}  // namespace nnapgb
