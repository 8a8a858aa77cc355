// C ABI of the force-training gradients (the double backward of training with forces).
//
// Replaces, for whole structures, the per-atom training pair of the reference:
// jse_nnap_forwardEnergyForce + jse_nnap_backwardEnergyForce (nnap_interface.cpp:142-232)
// called atom by atom by TrainerNNAP's force branch (TrainerNNAP.java:1006-1175), whose
// per-pair upstream gradient is bF_j - bF_i plus the stress terms.  One call evaluates the
// neighbour rows and descriptors of the batch (the evaluation pipeline with fp_only), then
// the descriptor directional derivatives, the network passes and the parameter-gradient
// reductions (k_train.cu).  Gradients are FP64 sums of FP32 chunk partials over a fixed
// chunking, so repeated calls return identical results.
#include <cstring>

#include "api_internal.hpp"
#include "train.cuh"

namespace nnapgb {
namespace {

constexpr int kTrainChunk = 256;  // slots per partial sum

int net_params(const Species& sp) {
    int p = 0, in = sp.D;
    for (int H : sp.hidden) { p += H * in + H; in = H; }
    return p + in + 1;
}

int record_floats(const Species& sp) {
    int v = 0, in = sp.D;
    for (int H : sp.hidden) { v += 2 * H + 2 * in; in = H; }
    return v + in + 1;
}

int fp_params(const Species& sp) {
    size_t p = 0;
    for (auto& b : sp.subs) p += b.W.size();
    return (int)p;
}

// Tiles of one species' gradient: 64 x 64 blocks of every weight matrix, then the
// vector tile (biases, output weights, output bias).
std::vector<GradTile> grad_tiles(const Species& sp) {
    std::vector<GradTile> t;
    int in = sp.D;
    for (size_t l = 0; l < sp.hidden.size(); ++l) {
        const int H = sp.hidden[l];
        for (int o0 = 0; o0 < H; o0 += 64)
            for (int i0 = 0; i0 < in; i0 += 64) t.push_back({(int)l, o0, i0});
        in = H;
    }
    t.push_back({-1, 0, 0});
    return t;
}

// Invariant-column arguments of sub-basis k of run r (A: that sub's expansion arena).
InvArgs inv_args(nnap_handle* h, const Run& r, size_t k, int n, const float* A, const SubShape& s) {
    InvArgs ia;
    std::memset(&ia, 0, sizeof ia);
    ia.perm = h->perm.p;
    ia.range = h->type_start.p;
    ia.t0 = r.t0;
    ia.t1 = r.t1;
    ia.nmax = n;
    ia.A = A;
    ia.NP = s.np;
    ia.K = (s.lmax + 1) * (s.lmax + 1);
    ia.idx = r.inv_idx[k].p;
    ia.coef = r.inv_coef[k].p;
    ia.start = r.inv_start[k].p;
    ia.ncol = s.ninv;
    ia.fp = h->fp.p;
    ia.gfp = h->gfp.p;
    ia.fp_stride = h->fp_stride;
    ia.fp_off = r.fp_off[k];
    ia.nl2 = s.nl2;
    ia.sl = s.nl2 + s.ninv;
    return ia;
}

bool any_fused(const Model& m) {
    for (auto& sp : m.sp)
        for (auto& b : sp.subs)
            if (b.fused) return true;
    return false;
}

// Queue the training passes.  With want_w, also the radial-fuse gradients: one FP64
// block [t1 - t0][T][NP][N1] per run of species and sub-basis in h->twgrad, in run order.
void train_enqueue(nnap_handle* h, const Batch& B, const double* bE, const double* bF, const double* bW,
                   bool want_w) {
    const Model& m = h->model;
    const int n = B.natoms, T = m.ntypes(), n1 = std::max(n, 1);
    cudaStream_t st = h->stream;
    // record and gradient geometry
    int Vmax = 1, Pmax = 1, tmax = 1;
    std::vector<std::vector<GradTile>> tiles(T);
    for (int t = 0; t < T; ++t) {
        Vmax = std::max(Vmax, record_floats(m.sp[t]));
        Pmax = std::max(Pmax, net_params(m.sp[t]));
        tiles[t] = grad_tiles(m.sp[t]);
        tmax = std::max(tmax, (int)tiles[t].size());
    }
    const int nchunk = (n + kTrainChunk - 1) / kTrainChunk;
    h->tu.ensure((size_t)n1 * h->fp_stride);
    h->trec.ensure((size_t)n1 * Vmax);
    h->tpart.ensure((size_t)T * std::max(nchunk, 1) * Pmax);
    h->ttiles.ensure((size_t)T * tmax);
    h->tbW.ensure(9 * (size_t)B.nstruct);
    int Ptot = 0;
    for (int t = 0; t < T; ++t) Ptot += net_params(m.sp[t]);
    h->tgrad.ensure(std::max(Ptot, 1));
    std::vector<GradTile> flat((size_t)T * tmax, GradTile{-1, 0, 0});
    for (int t = 0; t < T; ++t) std::copy(tiles[t].begin(), tiles[t].end(), flat.begin() + (size_t)t * tmax);
    CK(cudaMemcpyAsync(h->ttiles.p, flat.data(), sizeof(GradTile) * flat.size(), cudaMemcpyHostToDevice, st));
    // upstream gradients
    const float4* dbF = nullptr;
    const float* dbW = nullptr;
    const double* dbE = nullptr;
    if (bF && n) {
        h->tbFd.ensure(3 * (size_t)n);
        h->tbF.ensure(n);
        CK(cudaMemcpyAsync(h->tbFd.p, bF, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        CK(launch_train_prep(h->tbFd.p, n, h->tbF.p, st));
        ++h->launches;
        dbF = h->tbF.p;
    }
    std::vector<float> wf;
    if (bW) {
        wf.assign(bW, bW + 9 * (size_t)B.nstruct);
        CK(cudaMemcpyAsync(h->tbW.p, wf.data(), sizeof(float) * wf.size(), cudaMemcpyHostToDevice, st));
        dbW = h->tbW.p;
    }
    if (bE && n) {
        h->tbE.ensure(n);
        CK(cudaMemcpyAsync(h->tbE.p, bE, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        dbE = h->tbE.p;
    }
    if (n) CK(cudaMemsetAsync(h->tu.p, 0, sizeof(float) * (size_t)n * h->fp_stride, st));
    bool inv = false;
    for (auto& r : h->runs)
        for (auto& sh : r.subs) inv = inv || sh.ninv > 0;
    const bool want_dA = want_w || inv;  // D_b A: the fuse gradients and the invariant columns
    if (want_dA) {
        const size_t an = std::max<size_t>(a_arena_size(h, n), 1);
        h->tdA.ensure(an);
        CK(cudaMemsetAsync(h->tdA.p, 0, sizeof(float) * an, st));
    }
    if (want_w && inv) {
        const size_t an = std::max<size_t>(a_arena_size(h, n), 1);
        h->tM1x.ensure(an);
        h->tM2x.ensure(an);
    }
    if (want_w) {
        const size_t an = std::max<size_t>(a_arena_size(h, n), 1);
        h->tdA.ensure(an);
        h->tgfp.ensure((size_t)n1 * h->fp_stride);
        h->tdfp.ensure((size_t)n1 * h->fp_stride);
        CK(cudaMemsetAsync(h->tdA.p, 0, sizeof(float) * an, st));
        CK(cudaMemsetAsync(h->tgfp.p, 0, sizeof(float) * (size_t)n1 * h->fp_stride, st));
        CK(cudaMemsetAsync(h->tdfp.p, 0, sizeof(float) * (size_t)n1 * h->fp_stride, st));
    }
    // descriptor directional derivatives, per run of species and sub-basis (A arena as the forward)
    size_t a_off = 0;
    for (auto& r : h->runs) {
        for (size_t k = 0; k < r.subs.size(); ++k) {
            const SubShape& s = r.subs[k];
            JvpArgs ja;
            DescArgs& a = ja.d;
            a.perm = h->perm.p;
            a.range = h->type_start.p;
            a.t0 = r.t0;
            a.t1 = r.t1;
            a.nmax = n;
            a.type = h->type.p;
            a.P = pair_bufs(h);
            a.W = r.W[k].p;
            a.T = T;
            a.rcut = (float)s.rcut;
            a.fp = h->fp.p;
            a.fp_stride = h->fp_stride;
            a.fp_off = r.fp_off[k];
            a.A = nullptr;
            if (s.kind == KIND_SPHERICAL) {
                a.A = h->A.p + a_off;
                a_off += (size_t)n * s.np * (s.lmax + 1) * (s.lmax + 1);
            }
            a.gfp = nullptr;
            a.accumulate = 0;
            a.warps = 4;
            a.nz_p = nullptr;
            a.nz_w = nullptr;
            a.fwd_alpha = r.falpha[k].p;
            a.nl2 = s.nl2;
            a.sl = s.nl2 + s.ninv;
            a.Gx = nullptr;
            a.sub_dx = nullptr;
            a.sub_pos = nullptr;
            a.sub_count = nullptr;
            ja.bF = dbF;
            ja.bW = dbW;
            ja.sid = h->sid.p;
            ja.u = h->tu.p;
            ja.dA = (want_dA && s.kind == KIND_SPHERICAL) ? h->tdA.p + (a.A - h->A.p) : nullptr;
            if (n > 0 && (dbF || dbW)) {
                CK(launch_jvp(s.kind, s.lmax, s.np, s.n1, ja, st));
                ++h->launches;
                if (s.ninv) {  // the invariant columns' directional derivatives
                    InvArgs ia = inv_args(h, r, k, n, a.A, s);
                    ia.dA = ja.dA;
                    ia.u = h->tu.p;
                    CK(launch_invariants_jvp(ia, st));
                    ++h->launches;
                }
            }
        }
    }
    // network passes, one launch per species
    for (int t = 0; t < T && n > 0; ++t) {
        const NetDev& nd = h->nets[t];
        NetTrainArgs a;
        a.perm = h->perm.p;
        a.range = h->type_start.p;
        a.t = t;
        a.nmax = n;
        a.fp = h->fp.p;
        a.u = h->tu.p;
        a.fp_stride = h->fp_stride;
        a.D = nd.D;
        a.nlayer = nd.nlayer;
        for (int l = 0; l < 4; ++l) a.H[l] = l < nd.nlayer ? nd.H[l] : 0;  // at most 4 (checked at entry)
        a.w = nd.w32.p;
        a.sigma_e = (float)nd.sigma_e;
        a.bE = dbE;
        a.rec = h->trec.p;
        a.V = Vmax;
        a.gfp = want_w ? h->tgfp.p : nullptr;
        a.dfp = want_w ? h->tdfp.p : nullptr;
        CK(launch_net_train(a, st));
        ++h->launches;
    }
    // chunk partials and their FP64 sums
    ReduceArgs ra;
    std::memset(&ra, 0, sizeof ra);
    ra.range = h->type_start.p;
    ra.T = T;
    ra.rec = h->trec.p;
    ra.chunk = kTrainChunk;
    ra.nchunk = nchunk;
    ra.partial = h->tpart.p;
    ra.Pmax = Pmax;
    ra.tiles = h->ttiles.p;
    ra.tmax = tmax;
    ra.grad = h->tgrad.p;
    int goff = 0;
    for (int t = 0; t < T; ++t) {
        const Species& sp = m.sp[t];
        ra.ntiles[t] = (int)tiles[t].size();
        ra.V[t] = Vmax;
        ra.D[t] = sp.D;
        ra.nlayer[t] = (int)sp.hidden.size();
        for (int l = 0; l < 4; ++l) ra.H[t][l] = l < (int)sp.hidden.size() ? sp.hidden[l] : 0;
        ra.P[t] = net_params(sp);
        ra.goff[t] = goff;
        goff += ra.P[t];
    }
    CK(cudaMemsetAsync(h->tgrad.p, 0, sizeof(double) * std::max(Ptot, 1), st));
    if (nchunk) {
        CK(launch_train_reduce(ra, st));
        h->launches += 2;
    }
    if (want_w) {
        // warps of the radial-fuse gradient launches: enough to fill the GPU, with the
        // partial blocks bounded to about 64 M floats
        size_t wtot = 0, per_max = 1;
        for (auto& r : h->runs)
            for (auto& sh : r.subs) {
                const size_t per = (size_t)(r.t1 - r.t0) * T * sh.np * sh.n1;
                wtot += per;
                per_max = std::max(per_max, per);
            }
        int G = (int)std::min<size_t>(4096, std::max<size_t>(1, ((size_t)64 << 20) / per_max));
        G = std::max(4, std::min(G, ((n + 3) / 4) * 4));
        h->twpart.ensure((size_t)G * per_max);
        h->twgrad.ensure(std::max<size_t>(wtot, 1));
        size_t a_off = 0, w_off = 0;
        for (auto& r : h->runs) {
            for (size_t k = 0; k < r.subs.size(); ++k) {
                const SubShape& sh = r.subs[k];
                const size_t per = (size_t)(r.t1 - r.t0) * T * sh.np * sh.n1;
                WgradArgs g;
                DescArgs& a = g.j.d;
                a.perm = h->perm.p;
                a.range = h->type_start.p;
                a.t0 = r.t0;
                a.t1 = r.t1;
                a.nmax = n;
                a.type = h->type.p;
                a.P = pair_bufs(h);
                a.W = r.W[k].p;
                a.T = T;
                a.rcut = (float)sh.rcut;
                a.fp = h->fp.p;
                a.fp_stride = h->fp_stride;
                a.fp_off = r.fp_off[k];
                a.A = nullptr;
                g.dA = nullptr;
                if (sh.kind == KIND_SPHERICAL) {
                    a.A = h->A.p + a_off;
                    g.dA = h->tdA.p + a_off;
                    a_off += (size_t)n * sh.np * (sh.lmax + 1) * (sh.lmax + 1);
                }
                a.gfp = nullptr;
                a.accumulate = 0;
                a.warps = 4;
                a.nz_p = nullptr;
                a.nz_w = nullptr;
                a.fwd_alpha = nullptr;
                a.nl2 = sh.nl2;
                a.sl = sh.nl2 + sh.ninv;
                a.Gx = nullptr;
                g.j.bF = dbF;
                g.j.bW = dbW;
                g.j.sid = h->sid.p;
                g.j.u = nullptr;
                g.j.dA = nullptr;
                g.gfp = h->tgfp.p;
                g.dfp = h->tdfp.p;
                g.partial = h->twpart.p;
                g.G = G;
                g.M1x = nullptr;
                g.M2x = nullptr;
                if (sh.ninv && n > 0) {  // the invariant columns' parts of M1 and M2
                    InvArgs ia = inv_args(h, r, k, n, a.A, sh);
                    ia.dA = g.dA;
                    ia.gfp = h->tgfp.p;
                    ia.dfp = h->tdfp.p;
                    ia.M1x = h->tM1x.p + (a.A - h->A.p);
                    ia.M2x = h->tM2x.p + (a.A - h->A.p);
                    CK(launch_invariants_wgrad(ia, st));
                    ++h->launches;
                    g.M1x = ia.M1x;
                    g.M2x = ia.M2x;
                }
                CK(cudaMemsetAsync(h->twpart.p, 0, sizeof(float) * (size_t)G * per, st));
                if (n > 0) {
                    CK(launch_wgrad(sh.kind, sh.lmax, sh.np, sh.n1, g, st));
                    ++h->launches;
                }
                CK(launch_wgrad_final(h->twpart.p, G, (int)per, h->twgrad.p + w_off, st));
                ++h->launches;
                w_off += per;
            }
        }
    }
    CK(cudaGetLastError());
}

// Scatter the per-run blocks of h->twgrad (already on the host as w) into the caller's
// layout: per species its sub-bases' matrices [tn][np][n].  A mirror or shared basis
// uses its source's parameters (nnap_main.hpp:410-420: the gradient goes to the source
// species), a mirror with the neighbour species t and source exchanged.
void scatter_wgrad(const nnap_handle* h, const std::vector<double>& w, double* grad_fp) {
    const Model& m = h->model;
    const int T = m.ntypes();
    std::vector<size_t> off(T + 1, 0);
    for (int t = 0; t < T; ++t) {
        size_t f = 0;
        for (auto& b : m.sp[t].subs) f += b.W.size();
        off[t + 1] = off[t] + f;
    }
    std::fill(grad_fp, grad_fp + off[T], 0.0);
    size_t w_off = 0;
    for (auto& r : h->runs) {
        for (size_t k = 0; k < r.subs.size(); ++k) {
            const SubShape& sh = r.subs[k];
            const size_t blk = (size_t)sh.np * sh.n1;
            for (int tc = r.t0; tc < r.t1; ++tc) {
                const Species& sp = m.sp[tc];
                const int o = sp.basis_src ? sp.basis_src - 1 : tc;
                if (!m.sp[o].subs[k].fused) continue;
                size_t sub_off = 0;
                for (size_t q = 0; q < k; ++q) sub_off += m.sp[o].subs[q].W.size();
                for (int tn = 0; tn < T; ++tn) {
                    int tt = tn;
                    if (sp.basis_mirror) tt = tn == o ? tc : (tn == tc ? o : tn);
                    const double* src = w.data() + w_off + ((size_t)(tc - r.t0) * T + tn) * blk;
                    double* dst = grad_fp + off[o] + sub_off + (size_t)tt * blk;
                    for (size_t e = 0; e < blk; ++e) dst[e] += src[e];
                }
            }
            w_off += (size_t)(r.t1 - r.t0) * T * blk;
        }
    }
}

}  // namespace
}  // namespace nnapgb

using namespace nnapgb;

extern "C" {

int nnap_param_sizes(const nnap_handle* h, int type, int* fp_size, int* nn_size) {
    if (!h || !fp_size || !nn_size) return NNAP_ERR_ARG;
    if (h->dead) return NNAP_ERR_DEAD;
    if (type < 1 || type > h->model.ntypes()) return NNAP_ERR_BAD_TYPE;
    *fp_size = fp_params(h->model.sp[type - 1]);
    *nn_size = net_params(h->model.sp[type - 1]);
    return NNAP_OK;
}

int nnap_train_grad_batch(nnap_handle* h, int nstruct, const int* natoms, const double* x, const int* type,
                          const int* box_kind, const double* boxes, const double* bgrad_energies,
                          const double* bgrad_forces, const double* bgrad_virial, double* grad_fp,
                          double* grad_nn) {
    return guarded(h, [&]() -> int {
        if (nstruct < 1 || !natoms || !box_kind || !boxes) throw ApiFail(NNAP_ERR_ARG, "invalid batch description");
        if (!grad_nn) throw ApiFail(NNAP_ERR_ARG, "grad_nn is NULL");
        const Model& m = h->model;
        if (m.radial_fn || m.act) throw ApiFail(NNAP_ERR_UNSUPPORTED, "training gradients are computed for NNAP models only");
        for (auto& r : h->runs)
            for (auto& sh : r.subs)
                if (!desc_compiled(sh.kind, sh.basis, sh.lmax, sh.np, sh.n1))
                    throw ApiFail(NNAP_ERR_UNSUPPORTED, "training gradients are compiled for the shapes of "
                                                        "NNAP_RADIAL_SHAPES / NNAP_SPH_SHAPES only");
        for (auto& sp : m.sp)
            if (sp.hidden.size() > 4) throw ApiFail(NNAP_ERR_UNSUPPORTED, "training gradients take at most 4 hidden layers");
        const int T = m.ntypes();
        const bool want_w = grad_fp && any_fused(m);
        h->launches = 0;
        const Batch& B = plan_batch(h, nstruct, natoms, box_kind, boxes);
        if (B.natoms && (!x || !type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        upload_inputs(h, B.natoms, x, type);
        struct Fp32Desc {  // FP32 descriptors for the gradients, restored on every exit
            nnap_handle* h;
            ~Fp32Desc() { h->fp32_desc = false; }
        } fp32_guard{h};
        h->fp32_desc = true;
        evaluate(h, B, h->x.p, h->type.p, true);
        train_enqueue(h, B, bgrad_energies, bgrad_forces, bgrad_virial, want_w);
        int Ptot = 0;
        for (int t = 0; t < T; ++t) Ptot += net_params(m.sp[t]);
        if (Ptot) CK(cudaMemcpyAsync(grad_nn, h->tgrad.p, sizeof(double) * Ptot, cudaMemcpyDeviceToHost, h->stream));
        std::vector<double> w;
        if (want_w) {
            size_t wtot = 0;
            for (auto& r : h->runs)
                for (auto& sh : r.subs) wtot += (size_t)(r.t1 - r.t0) * T * sh.np * sh.n1;
            w.resize(wtot);
            CK(cudaMemcpyAsync(w.data(), h->twgrad.p, sizeof(double) * wtot, cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
        if (grad_fp) {
            if (want_w) {
                scatter_wgrad(h, w, grad_fp);
            } else {
                size_t F = 0;
                for (int t = 0; t < T; ++t) F += fp_params(m.sp[t]);
                std::memset(grad_fp, 0, sizeof(double) * F);
            }
        }
        return NNAP_OK;
    });
}

}  // extern "C"
