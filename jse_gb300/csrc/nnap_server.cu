// Serving: structures kept resident on the device across successive evaluations and
// evaluated together by continuous batching (no counterpart in the reference, whose
// NNAP evaluates one structure per call and rebuilds its neighbour list every time).
//
// A server owns one handle.  Each admitted structure (a "slot") holds, in device
// memory drawn from the server's own stream-ordered memory pool, its species, its
// neighbour rows at rc + skin (Verlet rows) and the wrap counts of its last rebuild.
// One step evaluates any set of slots in one batched launch sequence:
//   k_tick_atoms -> k_wrap_resident -> [rebuild of the slots that need it:
//   k_wrap_bin .. k_neighbors at rc + skin -> k_verlet_store] -> k_filter at rc ->
//   species sort, mirror index, descriptors, networks, gradients, gather, reductions
// with one host synchronisation at the end.  A slot is rebuilt when it is new or when
// one of its atoms moved more than skin/2 since its last rebuild, so the kept pairs
// are exactly the full search's pairs (NeighborListGetter.java:1018-1050).
//
// Admission is bounded by a device-memory budget covering the resident arrays and the
// per-atom work buffers of a step over every resident atom, and by a slot count.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "api_internal.hpp"
#include "resident.cuh"

namespace nnapgb {
__global__ void k_tick_atoms(const SlotDev*, int*, int*);
__global__ void k_wrap_resident(const StructDev*, const int*, const double*, const int*, int, int, double*, float4*,
                                float4*, int4*, int*);
__global__ void k_verlet_store(const SlotDev*, const int*, PairBufs, int, const int4*);
__global__ void k_filter(const StructDev*, const SlotDev*, const int*, const double*, const float4*, const float4*,
                         const int4*, int, int, PairBufs, int*, int*);
}  // namespace nnapgb

using namespace nnapgb;

namespace {

constexpr int kFilterWarps = 4;  // must match k_resident.cu

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct ServerSlot {
    bool used = false;
    int n = 0;
    int kind = 0;
    double box[9];
    StructDev grid;              // rebuild grid at rc + skin (cell counts, search reach)
    StructDev evs;               // the box at rc with the rebuild grid's cells (a0 set per step)
    long long gen = 0;           // bumped whenever the slot's device arrays are (re)allocated
    std::vector<int> type;       // host copy of the species
    std::vector<double> xb;      // positions at the last rebuild (caller's frame)
    bool need_build = true;
    void* mem = nullptr;         // one pool allocation holding the arrays below
    size_t bytes = 0;
    SlotDev dev{};               // device pointers (a0 set per step)
    int last_a0 = -1;            // atom offset in the last step that evaluated it
    long long last_step = -1;   // last successful step that evaluated it
    long long last_stamp = -1;  // last step call that listed it
};

}  // namespace

struct nnap_server {
    nnap_handle* h = nullptr;
    double skin = 0.5, rc = 0.0, rcv = 0.0;
    size_t budget = 0;
    int max_structs = 0;
    cudaMemPool_t pool = nullptr;
    int Mv = 0;  // Verlet row capacity shared by all slots
    std::vector<ServerSlot> slots;
    std::vector<int> free_ids;
    size_t resident_bytes = 0;
    long long resident_atoms = 0;
    int nresident = 0;
    long long steps = 0, builds = 0, stamp = 0;
    // per-step device arrays owned by the server
    DevBuf<StructDev> sdev_build;
    DevBuf<SlotDev> dslots;
    DevBuf<int4> kw;
    DevBuf<int> type_b;
    DevBuf<double> x;
    Pinned stage_in, stage_out;
    // last step: structures in batch order (for neighbour-list queries)
    int last_natoms = 0;
    long long gens = 0;  // generation counter of slot allocations
    // the step in flight between nnap_server_submit and nnap_server_collect
    struct Pending {
        bool active = false;
        int nslots = 0, N = 0, nbs = 0, flags = 0;
        std::vector<int> ids, order, a0, n;  // caller's slots; batch position -> caller index; per batch position
        std::vector<long long> gen;           // slot generations at submission
        std::vector<size_t> in_off;           // caller-order atom offsets
        double* hx = nullptr;                 // staged positions, batch order (pinned)
        double *oe = nullptr, *ov = nullptr, *oea = nullptr, *of = nullptr, *ova = nullptr;  // pinned outputs
    } pend;
};

namespace {

int fail_s(nnap_server* s, int status, const std::string& m) {
    if (s && s->h) s->h->err = m;
    return status;
}

// Device bytes of the per-atom work buffers of one step (pair rows at capacity Mv,
// descriptors, gradients, coefficient rows, positions, outputs).
size_t work_bytes_per_atom(const nnap_server* s) {
    const nnap_handle* h = s->h;
    size_t b = (size_t)s->Mv * (8 + 16 + 4 + 16 + 2);
    b += (size_t)h->fp_stride * 4 * 2;
    size_t a = 0;
    bool inv = false;
    for (auto& r : h->runs)
        for (auto& sb : r.subs) {
            if (sb.kind == KIND_SPHERICAL) a += (size_t)sb.np * (sb.lmax + 1) * (sb.lmax + 1);
            inv = inv || sb.ninv > 0;
        }
    b += a * 4 * (inv ? 2 : 1);  // A, and its invariant-column gradient when present
    b += 24 + 24 + 32 + 16 + 4 * 8 + 8 + 24 + 72;
    return b;
}

// Resident bytes of one slot of n atoms at Verlet capacity Mv.
size_t slot_bytes(int n, int Mv) {
    return align256((size_t)n * Mv * 8) + align256((size_t)n * Mv * 2) + align256((size_t)n * 4) +
           align256((size_t)n * 16) + align256((size_t)n * 4);
}

size_t resident_total(const nnap_server* s, int Mv) {
    size_t t = 0;
    for (auto& sl : s->slots)
        if (sl.used) t += slot_bytes(sl.n, Mv);
    return t;
}

// Verlet capacity for a structure of n atoms in volume vol at cutoff rcv.
int verlet_capacity(int n, double vol, double rcv) {
    const double mean = 4.18879020478639 * rcv * rcv * rcv * (n / vol);
    const int M = (int)std::ceil(1.3 * mean + 24.0);
    return std::max(32, (M + 7) & ~7);
}

void slot_alloc(nnap_server* s, ServerSlot& sl) {
    nnap_handle* h = s->h;
    const size_t n = sl.n, Mv = s->Mv;
    sl.bytes = slot_bytes(sl.n, s->Mv);
    void* p = nullptr;
    CK(cudaMallocFromPoolAsync(&p, sl.bytes, s->pool, h->stream));
    sl.mem = p;
    char* c = static_cast<char*>(p);
    sl.dev.vkey = reinterpret_cast<uint64_t*>(c);
    c += align256(n * Mv * 8);
    sl.dev.vgrp = reinterpret_cast<uint16_t*>(c);
    c += align256(n * Mv * 2);
    sl.dev.vcnt = reinterpret_cast<int*>(c);
    c += align256(n * 4);
    sl.dev.kb = reinterpret_cast<int4*>(c);
    c += align256(n * 16);
    int* t = reinterpret_cast<int*>(c);
    sl.dev.type = t;
    sl.dev.n = sl.n;
    sl.dev.a0 = 0;
    CK(cudaMemcpyAsync(t, sl.type.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
    sl.need_build = true;
    sl.gen = ++s->gens;
    s->resident_bytes += sl.bytes;
}

void slot_free(nnap_server* s, ServerSlot& sl) {
    if (sl.mem) cudaFreeAsync(sl.mem, s->h->stream);
    sl.mem = nullptr;
    s->resident_bytes -= sl.bytes;
    sl.bytes = 0;
}

// Grow the shared Verlet capacity: every slot gets new arrays and is rebuilt.
void set_capacity(nnap_server* s, int Mv) {
    for (auto& sl : s->slots)
        if (sl.used) slot_free(s, sl);
    s->Mv = Mv;
    for (auto& sl : s->slots)
        if (sl.used) slot_alloc(s, sl);
}

}  // namespace

namespace {

template <class T>
T* carve(char*& c, size_t count) {
    T* p = reinterpret_cast<T*>(c);
    c += align256(count * sizeof(T));
    return p;
}

// Run f(lo, hi) over [0, n) on up to 8 host threads (one when n is small).
template <class F>
void host_parallel(size_t n, size_t grain, F&& f) {
    const size_t nt = std::min<size_t>(8, std::max<size_t>(1, n / std::max<size_t>(grain, 1)));
    if (nt <= 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    const size_t per = (n + nt - 1) / nt;
    for (size_t k = 1; k < nt; ++k) {
        const size_t lo = k * per, hi = std::min(n, lo + per);
        if (lo < hi) th.emplace_back([&f, lo, hi]() { f(lo, hi); });
    }
    f(0, std::min(n, per));
    for (auto& t : th) t.join();
}

// Queue one step over the listed slots (positions xs[q] of slot ids[q]) without waiting:
// inputs are staged (the caller's arrays may change once this returns), every kernel and
// the copies of the outputs into pinned staging are on the handle's stream.
// rebuild_all: every listed slot is rebuilt (the retry after a capacity overflow).
void submit_impl(nnap_server* s, int nslots, const int* ids, const double* const* xs, int flags, bool rebuild_all) {
    nnap_handle* h = s->h;
    const int T = h->model.ntypes();
    cudaStream_t st = h->stream;
    std::vector<size_t> in_off(nslots + 1, 0);
    const long long stamp = ++s->stamp;
    for (int q = 0; q < nslots; ++q) {
        const int id = ids[q];
        if (id < 0 || id >= (int)s->slots.size() || !s->slots[id].used) throw ApiFail(NNAP_ERR_ARG, "slot is not admitted");
        if (s->slots[id].last_stamp == stamp) throw ApiFail(NNAP_ERR_ARG, "slot listed twice in one step");
        if (!xs[q]) throw ApiFail(NNAP_ERR_ARG, "positions of a slot are NULL");
        s->slots[id].last_stamp = stamp;
        in_off[q + 1] = in_off[q] + (size_t)s->slots[id].n;
    }
    const int N = (int)in_off[nslots];
    // which slots are rebuilt: new ones, and those with an atom displaced by more than skin/2
    const double lim = 0.5 * s->skin * (1.0 - 1e-9);
    const double lim2 = lim * lim;
    std::vector<char> rb(nslots, rebuild_all ? 1 : 0);
    if (!rebuild_all)
        host_parallel((size_t)nslots, 64, [&](size_t lo, size_t hi) {
            for (size_t q = lo; q < hi; ++q) {
                const ServerSlot& sl = s->slots[ids[q]];
                bool need = sl.need_build;
                const double* xq = xs[q];
                for (int i = 0; !need && i < sl.n; ++i) {
                    const double dx = xq[3 * i] - sl.xb[3 * i], dy = xq[3 * i + 1] - sl.xb[3 * i + 1],
                                 dz = xq[3 * i + 2] - sl.xb[3 * i + 2];
                    need = !(dx * dx + dy * dy + dz * dz <= lim2);
                }
                rb[q] = need;
            }
        });
    // batch order: rebuilt slots first, so the rebuild works on a prefix of the atoms
    std::vector<int> order;
    for (int q = 0; q < nslots; ++q)
        if (rb[q]) order.push_back(q);
    const int nbs = (int)order.size();
    for (int q = 0; q < nslots; ++q)
        if (!rb[q]) order.push_back(q);
    Batch B;
    B.nstruct = nslots;
    B.natoms = N;
    B.sc.push_back(0);
    std::vector<StructDev> gsd;
    std::vector<SlotDev> sdv;
    int a0 = 0, c0 = 0, nb_atoms = 0;
    for (int t = 0; t < nslots; ++t) {
        ServerSlot& sl = s->slots[ids[order[t]]];
        StructDev d = sl.evs;
        d.a0 = a0;
        B.sd.push_back(d);
        if (t < nbs) {
            StructDev g = sl.grid;
            g.a0 = a0;
            g.n = sl.n;
            g.c0 = c0;
            c0 += g.nc[0] * g.nc[1] * g.nc[2];
            gsd.push_back(g);
            nb_atoms += sl.n;
        }
        SlotDev sv = sl.dev;
        sv.a0 = a0;
        sv.n = sl.n;
        sdv.push_back(sv);
        for (int b = 0; b < sl.n; b += kRedChunk) {
            B.cb.push_back(a0 + b);
            B.ce.push_back(a0 + std::min(sl.n, b + kRedChunk));
        }
        B.sc.push_back((int)B.cb.size());
        a0 += sl.n;
    }
    B.ncells = std::max(c0, 1);
    const int nchunks = (int)B.cb.size();
    // buffers: the handle's work arrays at row capacity Mv, then the server's own
    h->M = s->Mv;
    h->GS = 0;  // filtered rows keep no group starts: the mirror search bisects
    ensure_work(h, N, nslots, B.ncells, nchunks);
    drop_graph(h);
    h->layout_ok = false;
    s->kw.ensure(std::max(N, 1));
    s->type_b.ensure(std::max(N, 1));
    s->x.ensure(3 * (size_t)std::max(N, 1));
    s->dslots.ensure(nslots);
    s->sdev_build.ensure(std::max(nbs, 1));
    // pinned staging of everything uploaded, in batch order
    const size_t in_bytes = align256(sizeof(double) * 3 * (size_t)N) + align256(sizeof(StructDev) * nslots) +
                            align256(sizeof(StructDev) * std::max(nbs, 1)) + align256(sizeof(SlotDev) * nslots) +
                            3 * align256(sizeof(int) * (size_t)(nchunks + nslots + 1));
    char* c = static_cast<char*>(s->stage_in.ensure(in_bytes));
    double* hx = carve<double>(c, 3 * (size_t)N);
    StructDev* hsd = carve<StructDev>(c, nslots);
    StructDev* hgd = carve<StructDev>(c, std::max(nbs, 1));
    SlotDev* hsl = carve<SlotDev>(c, nslots);
    int* hcb = carve<int>(c, nchunks + nslots + 1);
    int* hce = carve<int>(c, nchunks + nslots + 1);
    int* hsc = carve<int>(c, nchunks + nslots + 1);
    host_parallel((size_t)nslots, 64, [&](size_t lo, size_t hi) {
        for (size_t t = lo; t < hi; ++t) {
            const int q = order[t];
            std::memcpy(hx + 3 * (size_t)B.sd[t].a0, xs[q], sizeof(double) * 3 * (in_off[q + 1] - in_off[q]));
        }
    });
    std::memcpy(hsd, B.sd.data(), sizeof(StructDev) * nslots);
    if (nbs) std::memcpy(hgd, gsd.data(), sizeof(StructDev) * nbs);
    std::memcpy(hsl, sdv.data(), sizeof(SlotDev) * nslots);
    if (nchunks) {
        std::memcpy(hcb, B.cb.data(), sizeof(int) * nchunks);
        std::memcpy(hce, B.ce.data(), sizeof(int) * nchunks);
    }
    std::memcpy(hsc, B.sc.data(), sizeof(int) * (nslots + 1));
    if (N) CK(cudaMemcpyAsync(s->x.p, hx, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->sdev.p, hsd, sizeof(StructDev) * nslots, cudaMemcpyHostToDevice, st));
    if (nbs) CK(cudaMemcpyAsync(s->sdev_build.p, hgd, sizeof(StructDev) * nbs, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->dslots.p, hsl, sizeof(SlotDev) * nslots, cudaMemcpyHostToDevice, st));
    if (nchunks) {
        CK(cudaMemcpyAsync(h->chunk_b.p, hcb, sizeof(int) * nchunks, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(h->chunk_e.p, hce, sizeof(int) * nchunks, cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(h->struct_chunks.p, hsc, sizeof(int) * (nslots + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(h->status.p, 0, sizeof(int) * 2, st));
    // launches
    h->launches = 0;
    h->mark(0);
    int* sid = h->sid.p;
    int* tb = s->type_b.p;
    k_tick_atoms<<<nslots, 256, 0, st>>>(s->dslots.p, sid, tb);
    ++h->launches;
    if (N > 0) {
        k_wrap_resident<<<(N + 255) / 256, 256, 0, st>>>(h->sdev.p, sid, s->x.p, tb, N, T, h->xw.p, h->xf.p,
                                                         h->xlo.p, s->kw.p, h->status.p);
        ++h->launches;
    }
    if (nb_atoms > 0) {  // rebuild the Verlet rows of the prefix at rc + skin
        CK(cudaMemsetAsync(h->cell_count.p, 0, sizeof(int) * B.ncells, st));
        CK(cudaMemsetAsync(h->cell_fill.p, 0, sizeof(int) * B.ncells, st));
        k_wrap_bin<<<(nb_atoms + 255) / 256, 256, 0, st>>>(s->sdev_build.p, sid, s->x.p, tb, nb_atoms, T, h->xw.p,
                                                           h->xf.p, h->xlo.p, h->cell_of.p, h->cell_count.p,
                                                           h->status.p);
        k_scan_excl<<<1, 1024, 0, st>>>(h->cell_count.p, B.ncells, h->cell_start.p);
        k_fill_cells<<<(nb_atoms + 255) / 256, 256, 0, st>>>(h->cell_of.p, nb_atoms, h->cell_start.p,
                                                             h->cell_fill.p, h->cell_atoms.p);
        k_sort_cells<<<(B.ncells * 32 + 255) / 256, 256, 0, st>>>(h->cell_start.p, B.ncells, h->cell_atoms.p);
        k_cell_order<<<(nb_atoms + 255) / 256, 256, 0, st>>>(h->cell_atoms.p, nb_atoms, h->xf.p, h->xlo.p, h->xfc.p,
                                                             h->xloc.p);
        const int nw = h->tune.nb_warps;
        k_neighbors<<<(nb_atoms + nw - 1) / nw, 32 * nw, 0, st>>>(
            s->sdev_build.p, sid, h->xw.p, h->xf.p, h->xlo.p, h->xfc.p, h->xloc.p, h->cell_of.p, h->cell_start.p,
            h->cell_atoms.p, nb_atoms, pair_bufs(h), h->status.p, h->status.p + 1);
        k_verlet_store<<<(unsigned)(((size_t)nb_atoms * 32 + 127) / 128), 128, 0, st>>>(s->dslots.p, sid,
                                                                                       pair_bufs(h), nb_atoms,
                                                                                       s->kw.p);
        h->launches += 7;
    }
    if (N > 0) {
        k_filter<<<(N + kFilterWarps - 1) / kFilterWarps, 32 * kFilterWarps, 0, st>>>(
            h->sdev.p, s->dslots.p, sid, h->xw.p, h->xf.p, h->xlo.p, s->kw.p, N, s->Mv, pair_bufs(h), h->status.p,
            h->status.p + 1);
        ++h->launches;
    }
    enqueue_species_mirror(h, B, tb);
    h->mark(1);
    enqueue_eval(h, B, tb, false, true);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_status, h->status.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
    // outputs in batch order into pinned staging
    const size_t out_bytes = align256(sizeof(double) * nslots) + align256(sizeof(double) * 9 * nslots) +
                             align256(sizeof(double) * (size_t)N) + align256(sizeof(double) * 3 * (size_t)N) +
                             align256(sizeof(double) * 9 * (size_t)N);
    char* oc = static_cast<char*>(s->stage_out.ensure(out_bytes));
    auto& P = s->pend;
    P.oe = carve<double>(oc, nslots);
    P.ov = carve<double>(oc, 9 * (size_t)nslots);
    P.oea = carve<double>(oc, N);
    P.of = carve<double>(oc, 3 * (size_t)N);
    P.ova = carve<double>(oc, 9 * (size_t)N);
    if (flags & NNAP_WANT_ENERGY)
        CK(cudaMemcpyAsync(P.oe, h->energy.p, sizeof(double) * nslots, cudaMemcpyDeviceToHost, st));
    if (flags & NNAP_WANT_VIRIAL)
        CK(cudaMemcpyAsync(P.ov, h->virial.p, sizeof(double) * 9 * nslots, cudaMemcpyDeviceToHost, st));
    if ((flags & NNAP_WANT_ENERGIES) && N)
        CK(cudaMemcpyAsync(P.oea, h->e_atom.p, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    if ((flags & NNAP_WANT_FORCES) && N)
        CK(cudaMemcpyAsync(P.of, h->forces.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, st));
    if ((flags & NNAP_WANT_VIRIALS) && N)
        CK(cudaMemcpyAsync(P.ova, h->virials.p, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, st));
    P.active = true;
    P.nslots = nslots;
    P.N = N;
    P.nbs = nbs;
    P.flags = flags;
    P.ids.assign(ids, ids + nslots);
    P.order = order;
    P.in_off = in_off;
    P.hx = hx;
    P.a0.resize(nslots);
    P.n.resize(nslots);
    P.gen.resize(nslots);
    for (int t = 0; t < nslots; ++t) {
        P.a0[t] = B.sd[t].a0;
        P.n[t] = B.sd[t].n;
        P.gen[t] = s->slots[ids[order[t]]].gen;
    }
}

// Wait for the step in flight and copy its outputs (caller order).  A Verlet row that
// overflowed the shared capacity grows it and reruns the step with every slot rebuilt,
// from the staged positions.
void collect_impl(nnap_server* s, const Outputs& o) {
    nnap_handle* h = s->h;
    auto& P = s->pend;
    if (!P.active) throw ApiFail(NNAP_ERR_ARG, "no step in flight");
    for (int attempt = 0;; ++attempt) {
        const cudaError_t se = cudaStreamSynchronize(h->stream);
        if (se != cudaSuccess) {
            P.active = false;
            throw CudaFail(se, "cudaStreamSynchronize");
        }
        const int bits = h->h_status[0];
        const int maxc = h->h_status[1];
        if (bits & (ERRBIT_BAD_TYPE | ERRBIT_TIMEOUT | ERRBIT_CELLS | ERRBIT_NO_MIRROR)) {
            P.active = false;
            if (bits & ERRBIT_BAD_TYPE) throw ApiFail(NNAP_ERR_BAD_TYPE, "species outside 1..ntypes");
            if (bits & ERRBIT_TIMEOUT) throw ApiFail(NNAP_ERR_TIMEOUT, "a bounded tensor-core wait gave up");
            if (bits & ERRBIT_CELLS) throw ApiFail(NNAP_ERR_ARG, "an atom moved too many boxes since its rebuild");
            throw ApiFail(NNAP_ERR_CAPACITY, "neighbour list is not symmetric");
        }
        if ((bits & ERRBIT_CAPACITY) || maxc > s->Mv) {
            if (attempt >= 2) {
                P.active = false;
                throw ApiFail(NNAP_ERR_CAPACITY, "Verlet capacity could not be established");
            }
            // positions in caller order from the staged copy, then the step again
            std::vector<double> xc(3 * (size_t)P.N);
            std::vector<const double*> xs(P.nslots);
            for (int t = 0; t < P.nslots; ++t) {
                const int q = P.order[t];
                std::memcpy(xc.data() + 3 * P.in_off[q], P.hx + 3 * (size_t)P.a0[t], sizeof(double) * 3 * P.n[t]);
            }
            for (int q = 0; q < P.nslots; ++q) xs[q] = xc.data() + 3 * P.in_off[q];
            set_capacity(s, ((int)std::ceil(maxc * 1.15) + 8 + 7) & ~7);
            const std::vector<int> ids = P.ids;
            P.active = false;
            submit_impl(s, (int)ids.size(), ids.data(), xs.data(), P.flags, true);
            continue;
        }
        break;
    }
    const int flags = P.flags;
    for (int t = 0; t < P.nslots; ++t) {
        const int q = P.order[t];
        ServerSlot& sl = s->slots[P.ids[q]];
        const bool same = sl.used && sl.gen == P.gen[t];  // not reallocated since submission
        if (same) {
            sl.last_a0 = P.a0[t];
            sl.last_step = s->steps;
            if (t < P.nbs) {
                sl.xb.assign(P.hx + 3 * (size_t)P.a0[t], P.hx + 3 * ((size_t)P.a0[t] + sl.n));
                sl.need_build = false;
                ++s->builds;
            }
        }
        const size_t n = P.n[t], a = P.a0[t], off = P.in_off[q];
        if ((flags & NNAP_WANT_ENERGY) && o.energy) o.energy[q] = P.oe[t];
        if ((flags & NNAP_WANT_VIRIAL) && o.virial) std::memcpy(o.virial + 9 * q, P.ov + 9 * t, sizeof(double) * 9);
        if ((flags & NNAP_WANT_ENERGIES) && o.energies) std::memcpy(o.energies + off, P.oea + a, sizeof(double) * n);
        if ((flags & NNAP_WANT_FORCES) && o.forces) std::memcpy(o.forces + 3 * off, P.of + 3 * a, sizeof(double) * 3 * n);
        if ((flags & NNAP_WANT_VIRIALS) && o.virials)
            std::memcpy(o.virials + 9 * off, P.ova + 9 * a, sizeof(double) * 9 * n);
    }
    s->last_natoms = P.N;
    ++s->steps;
    P.active = false;
}

}  // namespace

// =================================================================== C ABI
extern "C" {

int nnap_server_create(nnap_handle* h, double skin, size_t memory_budget, int max_structs, nnap_server** out) {
    if (!out) return NNAP_ERR_ARG;
    *out = nullptr;
    return guarded(h, [&]() -> int {
        if (!(skin >= 0.0) || !std::isfinite(skin)) throw ApiFail(NNAP_ERR_ARG, "skin must be >= 0");
        if (memory_budget == 0) throw ApiFail(NNAP_ERR_ARG, "memory budget must be positive");
        std::unique_ptr<nnap_server> s(new nnap_server());
        s->h = h;
        s->skin = skin;
        s->rc = h->model.rcut_max;
        s->rcv = s->rc + skin;
        s->budget = memory_budget;
        s->max_structs = max_structs > 0 ? max_structs : 4096;
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = h->device;
        CK(cudaMemPoolCreate(&s->pool, &props));
        uint64_t keep = memory_budget;  // freed slot memory stays in the pool for the next admission
        CK(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        *out = s.release();
        return NNAP_OK;
    });
}

int nnap_server_destroy(nnap_server* s) {
    if (!s) return NNAP_ERR_ARG;
    nnap_handle* h = s->h;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    for (auto& sl : s->slots)
        if (sl.used) slot_free(s, sl);
    cudaStreamSynchronize(h->stream);
    s->sdev_build.release();
    s->dslots.release();
    s->kw.release();
    s->type_b.release();
    s->x.release();
    s->stage_in.release();
    s->stage_out.release();
    if (s->pool) cudaMemPoolDestroy(s->pool);
    h->layout_ok = false;
    delete s;
    return NNAP_OK;
}

int nnap_server_admit(nnap_server* s, int natoms, const int* type, int box_kind, const double* box, int* slot) {
    if (!s || !slot) return NNAP_ERR_ARG;
    *slot = -1;
    nnap_handle* h = s->h;
    return guarded(h, [&]() -> int {
        if (natoms < 1 || !type || !box) throw ApiFail(NNAP_ERR_ARG, "admission needs atoms, species and a box");
        const int T = h->model.ntypes();
        for (int i = 0; i < natoms; ++i)
            if (type[i] < 1 || type[i] > T) throw ApiFail(NNAP_ERR_BAD_TYPE, "species outside 1..ntypes");
        const StructDev grid = make_struct(box_kind, box, s->rcv, 0, natoms, 0);
        const int Mv = std::max(s->Mv, verlet_capacity(natoms, grid.vol, s->rcv));
        // budget: every resident slot (at the capacity after admission) plus this one, and
        // the work buffers of a step over all resident atoms
        const size_t res = resident_total(s, Mv) + slot_bytes(natoms, Mv);
        const int Mv_saved = s->Mv;
        s->Mv = Mv;
        const size_t work = work_bytes_per_atom(s) * (size_t)(s->resident_atoms + natoms);
        s->Mv = Mv_saved;
        if (res + work > s->budget) {
            if (s->nresident == 0) throw ApiFail(NNAP_ERR_CAPACITY, "structure does not fit the memory budget");
            return fail_s(s, NNAP_ERR_BUSY, "memory budget in use; retry after a release");
        }
        if (s->nresident >= s->max_structs) return fail_s(s, NNAP_ERR_BUSY, "all slots in use; retry after a release");
        if (Mv > s->Mv) set_capacity(s, Mv);
        int id;
        if (!s->free_ids.empty()) {
            id = s->free_ids.back();
            s->free_ids.pop_back();
        } else {
            id = (int)s->slots.size();
            s->slots.emplace_back();
        }
        ServerSlot& sl = s->slots[id];
        sl = ServerSlot();
        sl.used = true;
        sl.n = natoms;
        sl.kind = box_kind;
        std::memcpy(sl.box, box, sizeof sl.box);
        sl.grid = grid;
        {  // the box at rc, searched with the rebuild grid's cells (one per slot, reused every step)
            StructDev d = make_struct(box_kind, box, s->rc, 0, natoms, 0);
            int Rm = 0;
            for (int k = 0; k < 3; ++k) {
                d.nc[k] = grid.nc[k];
                d.R[k] = grid.R[k];
                Rm = std::max(Rm, d.R[k]);
            }
            d.rc2_hi = screen_bound(d, s->rc, Rm + 1);
            sl.evs = d;
        }
        sl.type.assign(type, type + natoms);
        try {
            slot_alloc(s, sl);
        } catch (...) {
            sl.used = false;
            s->free_ids.push_back(id);
            throw;
        }
        ++s->nresident;
        s->resident_atoms += natoms;
        *slot = id;
        return NNAP_OK;
    });
}

int nnap_server_release(nnap_server* s, int slot) {
    if (!s) return NNAP_ERR_ARG;
    return guarded(s->h, [&]() -> int {
        if (slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot].used)
            throw ApiFail(NNAP_ERR_ARG, "slot is not admitted");
        if (s->pend.active && std::find(s->pend.ids.begin(), s->pend.ids.end(), slot) != s->pend.ids.end())
            throw ApiFail(NNAP_ERR_ARG, "slot is part of the step in flight; collect it first");
        ServerSlot& sl = s->slots[slot];
        slot_free(s, sl);
        s->resident_atoms -= sl.n;
        --s->nresident;
        sl = ServerSlot();
        s->free_ids.push_back(slot);
        return NNAP_OK;
    });
}

int nnap_server_step(nnap_server* s, int nslots, const int* slots, const double* x, int flags, double* energy,
                     double* energies, double* forces, double* virial, double* virials) {
    if (!s) return NNAP_ERR_ARG;
    return guarded(s->h, [&]() -> int {
        if (nslots < 1 || !slots || !x) throw ApiFail(NNAP_ERR_ARG, "a step needs slots and positions");
        if (s->pend.active) throw ApiFail(NNAP_ERR_BUSY, "a submitted step is in flight; collect it first");
        Outputs o{energy, energies, forces, virial, virials};
        check_outputs(flags, o);
        std::vector<const double*> xs(nslots);
        size_t off = 0;
        for (int q = 0; q < nslots; ++q) {
            if (slots[q] < 0 || slots[q] >= (int)s->slots.size() || !s->slots[slots[q]].used)
                throw ApiFail(NNAP_ERR_ARG, "slot is not admitted");
            xs[q] = x + 3 * off;
            off += (size_t)s->slots[slots[q]].n;
        }
        submit_impl(s, nslots, slots, xs.data(), flags, false);
        collect_impl(s, o);
        return NNAP_OK;
    });
}

int nnap_server_submit(nnap_server* s, int nslots, const int* slots, const double* const* xs, int flags) {
    if (!s) return NNAP_ERR_ARG;
    return guarded(s->h, [&]() -> int {
        if (nslots < 1 || !slots || !xs) throw ApiFail(NNAP_ERR_ARG, "a step needs slots and positions");
        if (s->pend.active) throw ApiFail(NNAP_ERR_BUSY, "a submitted step is in flight; collect it first");
        const int known = NNAP_WANT_ENERGY | NNAP_WANT_ENERGIES | NNAP_WANT_FORCES | NNAP_WANT_VIRIAL | NNAP_WANT_VIRIALS;
        if (flags & ~known) throw ApiFail(NNAP_ERR_ARG, "unknown output flags");
        submit_impl(s, nslots, slots, xs, flags, false);
        return NNAP_OK;
    });
}

int nnap_server_collect(nnap_server* s, double* energy, double* energies, double* forces, double* virial,
                        double* virials) {
    if (!s) return NNAP_ERR_ARG;
    return guarded(s->h, [&]() -> int {
        if (!s->pend.active) throw ApiFail(NNAP_ERR_ARG, "no step in flight");
        Outputs o{energy, energies, forces, virial, virials};
        check_outputs(s->pend.flags, o);
        collect_impl(s, o);
        return NNAP_OK;
    });
}

int nnap_server_neighbor_list(nnap_server* s, int slot, int* counts, long long cap, int* j, int* img,
                              long long* total) {
    if (!s) return NNAP_ERR_ARG;
    nnap_handle* h = s->h;
    return guarded(h, [&]() -> int {
        if (!counts || !total) throw ApiFail(NNAP_ERR_ARG, "NULL argument");
        if (s->pend.active) throw ApiFail(NNAP_ERR_BUSY, "a submitted step is in flight; collect it first");
        if (slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot].used)
            throw ApiFail(NNAP_ERR_ARG, "slot is not admitted");
        const ServerSlot& sl = s->slots[slot];
        if (sl.last_step != s->steps - 1 || sl.last_a0 < 0)
            throw ApiFail(NNAP_ERR_ARG, "slot was not evaluated by the last step");
        const int n = sl.n, a0 = sl.last_a0, M = h->M;
        std::vector<int> cnt(n);
        std::vector<uint64_t> keys((size_t)n * M);
        CK(cudaMemcpyAsync(cnt.data(), h->pcount.p + a0, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(keys.data(), h->pkey.p + (size_t)a0 * M, sizeof(uint64_t) * keys.size(),
                           cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        long long t = 0;
        for (int i = 0; i < n; ++i) {
            counts[i] = cnt[i];
            for (int k = 0; k < cnt[i]; ++k, ++t) {
                if (!j) continue;
                if (t >= cap) throw ApiFail(NNAP_ERR_CAPACITY, "neighbour output capacity too small");
                const uint64_t key = keys[(size_t)i * M + k];
                j[t] = (int)(key >> 32) - a0;
                int na, nb, nc;
                unpack_img((uint32_t)key, na, nb, nc);
                img[3 * t] = na; img[3 * t + 1] = nb; img[3 * t + 2] = nc;
            }
        }
        *total = t;
        return NNAP_OK;
    });
}

int nnap_server_stats(const nnap_server* s, long long* out8) {
    if (!s || !out8) return NNAP_ERR_ARG;
    out8[0] = s->nresident;
    out8[1] = s->resident_atoms;
    out8[2] = (long long)s->resident_bytes;
    out8[3] = (long long)(work_bytes_per_atom(s) * (size_t)s->resident_atoms);
    out8[4] = s->steps;
    out8[5] = s->builds;
    out8[6] = s->Mv;
    out8[7] = (long long)s->budget;
    return NNAP_OK;
}

}  // extern "C"
