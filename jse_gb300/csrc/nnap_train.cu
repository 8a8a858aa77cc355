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

constexpr int kTrainChunk = 1024;  // slots per partial sum

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

void train_enqueue(nnap_handle* h, const Batch& B, const double* bE, const double* bF, const double* bW) {
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
            ja.bF = dbF;
            ja.bW = dbW;
            ja.sid = h->sid.p;
            ja.u = h->tu.p;
            if (n > 0 && (dbF || dbW)) {
                CK(launch_jvp(s.kind, s.lmax, s.np, s.n1, ja, st));
                ++h->launches;
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
        for (int l = 0; l < 4; ++l) a.H[l] = l < nd.nlayer ? nd.H[l] : 0;
        a.w = nd.w32.p;
        a.sigma_e = (float)nd.sigma_e;
        a.bE = dbE;
        a.rec = h->trec.p;
        a.V = Vmax;
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
    CK(cudaGetLastError());
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
        const int T = m.ntypes();
        if (grad_fp)
            for (auto& sp : m.sp)
                for (auto& b : sp.subs)
                    if (b.fused)
                        throw ApiFail(NNAP_ERR_UNSUPPORTED,
                                      "gradients of fused radial weights (wtype fuse/rfuse/exfuse) are not computed");
        h->launches = 0;
        Batch B = plan_batch(h, nstruct, natoms, box_kind, boxes);
        if (B.natoms && (!x || !type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        upload_inputs(h, B.natoms, x, type);
        evaluate(h, B, h->x.p, h->type.p, true);
        train_enqueue(h, B, bgrad_energies, bgrad_forces, bgrad_virial);
        int Ptot = 0;
        for (int t = 0; t < T; ++t) Ptot += net_params(m.sp[t]);
        if (Ptot) CK(cudaMemcpyAsync(grad_nn, h->tgrad.p, sizeof(double) * Ptot, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (grad_fp) {
            size_t F = 0;
            for (int t = 0; t < T; ++t) F += fp_params(m.sp[t]);
            std::memset(grad_fp, 0, sizeof(double) * F);
        }
        return NNAP_OK;
    });
}

}  // extern "C"
