// Host-side internals shared by the C ABI translation units: error types, device
// arrays, the handle (model upload, work buffers, launch-sequence cache) and the
// stages of the evaluation pipeline.  Not part of the public interface.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nnap_gb300.h"
#include "common.cuh"
#include "desc.cuh"
#include "model.hpp"
#include "net_tc.cuh"
#include "train.cuh"

namespace nnapgb {

// k_struct.cu
__global__ void k_wrap_bin(const StructDev*, const int*, const double*, const int*, int, int, double*, float4*,
                           float4*, int*, int*, int*);
__global__ void k_scan_excl(const int*, int, int*);
__global__ void k_fill_cells(const int*, int, const int*, int*, int*);
__global__ void k_sort_cells(const int*, int, int*);
__global__ void k_cell_order(const int*, int, const float4*, const float4*, float4*, float4*);
__global__ void k_renumber(int*, int, const float4*, const float4*, const double*, const int*, const int*, float4*,
                           float4*, double*, int*, int*, int*);
__global__ void k_unpermute(const double*, const int*, int, double*);
__global__ void k_neighbors(const StructDev*, const int*, const double*, const float4*, const float4*, const float4*,
                            const float4*, const int*, const int*, const int*, int, PairBufs, int*, int*);
__global__ void k_mirror(const StructDev*, const int*, PairBufs, int, int*);
__global__ void k_type_hist(const int*, int, int, int*);
__global__ void k_type_offsets(int*, int, int, int*);
__global__ void k_type_scatter(const int*, int, int, const int*, int*);
__global__ void k_gather(PairBufs, int, const int*, double*, double*);
__global__ void k_reduce_chunks(const int*, const int*, const double*, const double*, double*);
__global__ void k_reduce_structs(const int*, int, const double*, double*, double*);

// Launch shapes chosen per atom-count bucket by the autotuner (defaults below).
struct Tuning {
    int desc_fwd_warps = 4;  // warps per CTA of the descriptor forward kernels
    int desc_bwd_warps = 4;  // warps per CTA of the descriptor backward kernels
    int nb_warps = 4;        // warps per CTA of the neighbour kernel
    int gather_block = 128;  // threads per CTA of the force / virial gather
    int net_split = 4;       // threads per tile row of the tensor-core network (2 or 4)
};
constexpr int kTuneParams = 5;
constexpr int kSortBlock = 256;   // must match k_struct.cu
constexpr int kRedBlock = 256;    // must match k_struct.cu
constexpr int kRedChunk = 1024;   // atoms per reduction chunk

struct CudaFail : std::runtime_error {
    cudaError_t code;
    CudaFail(cudaError_t c, const char* what)
        : std::runtime_error(std::string(what) + ": " + cudaGetErrorString(c)), code(c) {}
};
struct ApiFail : std::runtime_error {
    int status;
    ApiFail(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define CK(call)                                            \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) throw ::nnapgb::CudaFail(e_, #call);   \
    } while (0)

// Grow-only device array.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    void ensure(size_t n) {
        if (n <= cap) return;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(n, 1);
        CK(cudaMalloc(&p, want * sizeof(T)));
        cap = want;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// Pinned host staging grown on demand.
struct Pinned {
    void* p = nullptr;
    size_t cap = 0;
    void* ensure(size_t n) {
        if (n <= cap) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        CK(cudaMallocHost(&p, std::max<size_t>(n, 256)));
        cap = std::max<size_t>(n, 256);
        return p;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

struct SubShape {
    int kind, lmax, np, n1;
    double rcut;
    int nl2, l3, l4, ninv;  // power-spectrum columns, l3max, l4max, invariant columns
    int basis;              // radial functions: kRbNNAP or kRbNEP
    bool operator==(const SubShape& o) const {
        return kind == o.kind && lmax == o.lmax && np == o.np && n1 == o.n1 && rcut == o.rcut && nl2 == o.nl2 &&
               l3 == o.l3 && l4 == o.l4 && basis == o.basis;
    }
};

// Species t0..t1-1 sharing the sub-basis shapes (and descriptor length).
struct Run {
    int t0, t1;
    std::vector<SubShape> subs;
    std::vector<int> fp_off;
    std::vector<DevBuf<float>> W;  // per sub: [T][T][NP][N1]
    // per sub: sparse form of W ([T][T][N1][kNz] rows and weights), empty when a column
    // has more than kNz nonzero rows or N1 >= NP (the backward then stays in NP space)
    std::vector<DevBuf<int>> nzp;
    std::vector<DevBuf<float>> nzw;
    // per sub: alpha[tc][tn][p] of the radial-space forward ([T][kFwdTypes][NP]), empty
    // unless every row p of W has its only nonzero in column p mod N1, N1 < NP, T <= kFwdTypes
    std::vector<DevBuf<float>> falpha;
    // per sub: the forward may run on the tensor cores (falpha present, every |alpha| at
    // most kTcAlphaMax); used in mixed precision
    std::vector<char> tc_fwd;
    // per sub: invariant-column terms (indices into A, -1 past the order; coefficients)
    // and each column's first term, [ninv + 1]
    std::vector<DevBuf<int4>> inv_idx;
    std::vector<DevBuf<float>> inv_coef;
    std::vector<DevBuf<int>> inv_start;
    // per sub: the spherical kernels scan the compact rows of the handle's sub_rc cutoff
    std::vector<char> use_sub;
    // per sub: NEP type-wise cutoffs, [T][T] (rc, 1/rc), empty when the pairs share rcut
    std::vector<DevBuf<float2>> prc;
};

struct NetDev {
    int D, nlayer;
    int H[kNetMaxLayers];
    DevBuf<float> w32;
    double mu_e, sigma_e;
    NetTC tc;  // tensor-core parameters (mixed precision)
    int act;   // kActSiLU or kActTanh
};

// One planned evaluation: the structures and the reduction chunks (chunk c covers atoms
// [cb[c], ce[c]); structure s owns chunks [sc[s], sc[s+1])).
struct Batch {
    int nstruct = 0, natoms = 0, ncells = 0;
    std::vector<StructDev> sd;
    std::vector<int> cb, ce, sc;
};

struct Outputs {
    double *energy = nullptr, *energies = nullptr, *forces = nullptr, *virial = nullptr, *virials = nullptr;
};

}  // namespace nnapgb

struct nnap_handle {
    nnapgb::Model model;
    int precision = NNAP_PREC_FP32;
    // descriptors on the FP32 pipe even in mixed precision (set while training gradients,
    // which are FP32 whatever the handle's precision)
    bool fp32_desc = false;
    // the last batch layout and the counts, kinds and boxes it was planned from
    nnapgb::Batch plan;
    std::vector<int> plan_nat, plan_kind;
    std::vector<double> plan_box;
    bool plan_valid = false;
    bool net_tc = false;  // networks on the tensor cores (mixed precision, SiLU networks)
    std::string net_notes;  // species whose network runs the FP32 kernel on a mixed handle, and why
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    bool dead = false;
    int launches = 0;
    int fp_stride = 0;
    std::vector<nnapgb::Run> runs;
    std::vector<nnapgb::NetDev> nets;
    // work buffers
    nnapgb::DevBuf<double> x, xw, e_atom, forces, virials, energy, virial, partial;
    nnapgb::DevBuf<int> type, sid, cell_of, cell_count, cell_fill, cell_start, cell_atoms, perm, block_counts,
        type_start;
    nnapgb::DevBuf<int> chunk_b, chunk_e, struct_chunks, status;
    nnapgb::DevBuf<float4> xf, xlo, xfc, xloc;  // positions as float + low parts; copies in cell order
    // the evaluation in cell order (k_renumber): wrapped positions, cell and species of each
    // cell-order position, the atom at each, and per-atom energies back in atom order
    nnapgb::DevBuf<double> xw2, e_out;
    nnapgb::DevBuf<int> cell_of2, type2, orig;
    bool renumbered = false;  // the last enqueue ran in cell order
    nnapgb::DevBuf<uint16_t> pgrp;
    nnapgb::DevBuf<nnapgb::StructDev> sdev;
    nnapgb::DevBuf<uint64_t> pkey;
    nnapgb::DevBuf<float4> pdx, pg, pdxlo;  // pdxlo: low parts of the displacements (ZBL models)
    nnapgb::DevBuf<int> prev, pcount;
    nnapgb::DevBuf<float> fp, gfp, A, Gx;  // Gx: invariant-column part of dE/dA (when present)
    nnapgb::DevBuf<double> zbl_z, zbl_zp, zbl_para, zbl_rc;  // NEP ZBL: per species Z, Z^0.23; flexible parameters
    // compact rows of the entries within sub_rc (0: none) for spherical sub-bases whose
    // cutoff is well inside the neighbour cutoff: dx and row position [n][M], count [n]
    double sub_rc = 0.0;
    nnapgb::DevBuf<float4> sdx;
    nnapgb::DevBuf<int> spos, scount;
    int M = 0;
    // LAMMPS-style boundary: caller's atoms (local + ghost), list, targets of the scatter
    nnapgb::DevBuf<double> lmp_x, lmp_forces, lmp_virials;
    nnapgb::Pinned lmp_pin_in, lmp_pin_out;  // per-call layout arrays in, results out
    // the list on the device from the last LAMMPS call (reused with nlflag = 0)
    bool lmp_cached = false;
    int lmp_inum = 0, lmp_nall = 0, lmp_deg = 0;
    size_t lmp_total = 0;
    nnapgb::DevBuf<int> lmp_type, lmp_ilist, lmp_off, lmp_idx, lmp_rowtype, lmp_rowof, lmp_tcount, lmp_tstart,
        lmp_tfill, lmp_tlist;
    // force-training gradients: directional derivatives, upstream gradients, per-slot
    // network records, chunk partials and the FP64 result
    nnapgb::DevBuf<float> tu, trec, tpart, tbW, tdA, tgfp, tdfp, twpart, tM1x, tM2x;
    nnapgb::DevBuf<float4> tbF;
    nnapgb::DevBuf<double> tbFd, tbE, tgrad, twgrad;
    nnapgb::DevBuf<nnapgb::GradTile> ttiles;
    int GS = 0;                  // cell-offset groups per atom + 1 kept by k_neighbors (0: none)
    nnapgb::DevBuf<int> gstart;  // [n][GS] group starts of each neighbour row
    int* h_status = nullptr;  // pinned: [0]=err bits [1]=max count [2..]=type_start
    bool profiling = false;
    cudaEvent_t order_ev = nullptr;
    // launch-sequence cache (CUDA graph) and the layout it was sized for
    bool use_graphs = true;
    bool layout_ok = false;
    int layout_runs = 0;
    std::vector<long long> last_layout, gkey;
    cudaGraphExec_t gexec = nullptr;
    int glaunches = 0;  // kernel launches of the captured sequence
    nnapgb::StructDev* h_sdev = nullptr;  // pinned staging of the structure descriptors
    size_t h_sdev_cap = 0;
    int sm_count = 148;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // launch shapes: the ones in use, and the autotuner's choice per atom-count bucket
    nnapgb::Tuning tune;
    bool autotune = false;
    std::map<int, nnapgb::Tuning> tuned;
    bool capturing = false;
    void mark(int k) {
        // inside stream capture an ordinary record is only a dependency marker; an external
        // event node records the event when the graph runs
        if (profiling) CK(cudaEventRecordWithFlags(ev[k], stream, capturing ? cudaEventRecordExternal : 0));
    }
};

namespace nnapgb {

int fail(nnap_handle* h, int status, const std::string& m);

// Run f() with the handle's device current and turn exceptions into status codes.
template <class F>
int guarded(nnap_handle* h, F&& f) {
    if (!h) return NNAP_ERR_ARG;
    if (h->dead) return fail(h, NNAP_ERR_DEAD, "this NNAP is dead");
    h->err.clear();
    try {
        CK(cudaSetDevice(h->device));
        return f();
    } catch (const ApiFail& e) {
        return fail(h, e.status, e.what());
    } catch (const CudaFail& e) {
        cudaGetLastError();  // leave no error behind for the caller's next CUDA call
        return fail(h, NNAP_ERR_CUDA, e.what());
    } catch (const std::bad_alloc&) {
        return fail(h, NNAP_ERR_CAPACITY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(h, NNAP_ERR_ARG, e.what());
    }
}

// Box geometry of one structure of n atoms for cutoff rc: box rows, cell grid, float
// screen bound (a0 and c0 left at zero).  Shared by every entry point; never throws:
// returns NNAP_OK, or NNAP_ERR_ARG with *why (may be NULL) set for a bad box kind, a
// box that is not right-handed with finite positive volume, a non-finite or
// non-positive cutoff, or a box too thin for the cutoff.
int struct_geometry(int kind, const double* box, double rc, int n, StructDev& s, const char** why);
// Structure descriptor for cutoff rc (struct_geometry, throwing ApiFail on failure).
StructDev make_struct(int kind, const double* box, double rc, int a0, int n, int c0);
// Float screen bound for cutoff rc when image shifts reach Rm cells.
float screen_bound(const StructDev& s, double rc, int Rm);
// Neighbour capacity per atom for the densest structure of a batch at cutoff rc.
int initial_capacity(const Batch& B, double rc);
// Set the row capacity and size the pair buffers for n atoms.
void grow_pairs(nnap_handle* h, int n, int M);
PairBufs pair_bufs(nnap_handle* h);
// Size every per-atom work buffer for n atoms, nstruct structures, ncells cells and
// nchunks reduction chunks (no copies, no synchronisation).
void ensure_work(nnap_handle* h, int n, int nstruct, int ncells, int nchunks);
// Queue the species sort of n rows (slots ordered by species, stable).
void enqueue_species(nnap_handle* h, int n, const int* d_type);
// Queue the species sort of the batch's atoms and the mirror index of the pair rows.
void enqueue_species_mirror(nnap_handle* h, const Batch& B, const int* d_type);
// Queue descriptors, networks and descriptor gradients; with gather, also the
// force / virial gather over mirrored rows and the per-structure reductions.
// orig: the atom of each row when the rows are in cell order (forces and virials are
// written at it), or NULL when rows are atoms.
void enqueue_eval(nnap_handle* h, const Batch& B, const int* d_type, bool fp_only, bool gather,
                  const int* orig = nullptr);
// Run the whole launch sequence of a batch (neighbours, species order, descriptors and,
// unless fp_only, networks, pair gradients and reductions), growing the neighbour
// capacity and repeating as needed; returns after the stream has drained.
void evaluate(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type, bool fp_only);
// Plan a batch: structure descriptors, cell grids and reduction chunks.
const Batch& plan_batch(nnap_handle* h, int nstruct, const int* natoms, const int* kinds, const double* boxes);
// Copy host positions and species into the handle's device buffers.
void upload_inputs(nnap_handle* h, int n, const double* x, const int* type);
// Bytes of the spherical expansion-coefficient arena for n atom slots.
size_t a_arena_size(nnap_handle* h, int n);
void check_outputs(int flags, const Outputs& o);
// Forget the captured launch sequence of the handle.
void drop_graph(nnap_handle* h);

}  // namespace nnapgb
