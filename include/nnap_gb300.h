/*
 * nnap_gb300.h -- C ABI of the GB300-native NNAP energy/force/virial evaluator.
 *
 * The library replaces the per-structure evaluation path of jse's NNAP potential
 * (jsex.nnap.NNAP).  It reads the same JSON and YAML model files and returns the same
 * energies, forces and virials, computed on one GPU.  Plain pointers and sizes only;
 * every call returns an nnap_status (0 = success) and never throws.
 *
 * Conventions (identical to the reference):
 *   - species are 1-based integers indexing the model's "models" list;
 *   - positions are Cartesian, in the frame whose origin is the box origin; they are
 *     wrapped into the box in FP64 exactly as IBox.wrapPBC does (IBox.java:145-151);
 *   - box is 9 doubles, rows a, b, c.  box_kind selects how it is read:
 *       NNAP_BOX_ORTHO  diagonal only (jse.atom.Box / LmpBox),
 *       NNAP_BOX_LMP    a=(lx,0,0) b=(xy,ly,0) c=(xz,yz,lz) (jse.lmp.LmpBoxPrism),
 *       NNAP_BOX_PRISM  three general vectors (jse.atom.BoxPrism);
 *   - neighbours are all periodic images j' with |x_j' - x_i|^2 < rcut^2 (strict, FP64),
 *     including images of atom i itself (NeighborListGetter.java:1018-1050);
 *   - forces F_i = -dE/dx_i; virials use the per-atom convention of
 *     IPairPotential.calEnergyForceVirials (IPairPotential.java:811-1022): the pair term
 *     dx_ij (x) g_ij is assigned to the neighbour j; components are ordered
 *     xx, yy, zz, xy, xz, yz, yx, zx, zy; the total virial is their sum.
 *
 * Thread safety: one handle serves one host thread at a time (NNAP.java:38); distinct
 * handles are independent.  Each handle owns one CUDA stream and grow-only device
 * buffers; no allocation happens in steady-state calls once the buffers have grown.
 */
#ifndef NNAP_GB300_H
#define NNAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nnap_handle nnap_handle;

/* Status codes.  Nonzero returns correspond to the reference's IllegalStateException /
 * IllegalArgumentException / CudaException paths (NNAP.java:131-176, 507, 756;
 * CudaCore.java:110). */
typedef enum {
    NNAP_OK = 0,
    NNAP_ERR_BAD_MODEL = 1,    /* model text invalid or inconsistent                */
    NNAP_ERR_BAD_TYPE = 2,     /* species outside 1..ntypes (NNAP.java:507)           */
    NNAP_ERR_CAPACITY = 3,     /* internal capacity exceeded and could not grow       */
    NNAP_ERR_CUDA = 4,         /* a CUDA runtime call failed; see nnap_last_error     */
    NNAP_ERR_UNSUPPORTED = 5,  /* model shape beyond the kernels' shared memory       */
    NNAP_ERR_ARG = 6,          /* invalid argument (null pointer, bad size, bad box)  */
    NNAP_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up                  */
    NNAP_ERR_DEAD = 8,         /* handle already destroyed                            */
    NNAP_ERR_BUSY = 9          /* server budget or slots in use; retry after a release */
} nnap_status;

/* Precision modes.  NNAP_PREC_FP32 is the plain drop-in (FP32 descriptors and FP32
 * network); NNAP_PREC_MIXED evaluates the network as BF16 tensor-core GEMMs with FP32
 * accumulation and FP32 output layer.  Both use FP64 wrapping, FP64 displacements
 * and FP64 energy/force/virial reductions. */
typedef enum { NNAP_PREC_FP32 = 0, NNAP_PREC_MIXED = 1 } nnap_precision;

typedef enum { NNAP_BOX_ORTHO = 0, NNAP_BOX_LMP = 1, NNAP_BOX_PRISM = 2 } nnap_box_kind;

/* Output selection flags for the compute calls. */
enum {
    NNAP_WANT_ENERGY = 1,     /* total energy (1 double)                    */
    NNAP_WANT_ENERGIES = 2,   /* per-atom energies (n doubles)              */
    NNAP_WANT_FORCES = 4,     /* forces (3n doubles, xyz interleaved)       */
    NNAP_WANT_VIRIAL = 8,     /* total virial (9 doubles)                   */
    NNAP_WANT_VIRIALS = 16    /* per-atom virials (9n doubles)              */
};

/* Create a handle from model text in the format read by NNAP(Map) / NNAP(String path)
 * (NNAP.java:402-426): JSON, or YAML (the form IO.yaml2map reads for .yaml / .yml files,
 * NNAP.java:407-411) for text that does not start with '{'.  device is the CUDA ordinal.
 * Replaces the NNAP constructor + JIT compile (NNAP.java:129-401, 446-470).  Every shape
 * the format allows is evaluated (nmax <= 20, lmax <= 12, any weight type, any hidden
 * widths); NNAP_ERR_UNSUPPORTED only for shapes beyond shared memory. */
int nnap_create(const char* model_json, size_t len, int precision, int device, nnap_handle** out);
/* Same, reading the JSON or YAML text from a file (NNAP(String), NNAP.java:407-411). */
int nnap_create_from_file(const char* path, int precision, int device, nnap_handle** out);
/* Parse and validate model text (JSON or YAML) without a GPU, as nnap_create does before
 * any device work: NNAP_OK with the species count and a 64-bit digest of every value the
 * kernels consume (equal digests: equal models), or NNAP_ERR_BAD_MODEL with the reason in
 * err (errlen bytes, may be NULL).  No counterpart in the reference, whose loader runs
 * inside the NNAP constructor (NNAP.java:129-307). */
int nnap_model_check(const char* model_text, size_t len, int* ntypes, uint64_t* digest, char* err, size_t errlen);
/* Create a handle from NEP potential text (nep.txt, the file read by NEP(String),
 * NEP.java:98-100 and 786-1010): potential models nep3, nep4 and nep5, with or without
 * ZBL (nepV_zbl, fixed or flexible) and with or without type-wise cutoffs; other
 * variants (dipole, polarizability) return NNAP_ERR_UNSUPPORTED.  Species are
 * 1-based like every other call (NEP's 0-based species + 1).  The handle serves every
 * evaluation entry point (compute, batch, device, LAMMPS, server); NNAP_PREC_MIXED is
 * accepted and evaluates exactly like NNAP_PREC_FP32 (the tanh network runs in FP32);
 * nnap_train_grad_batch returns NNAP_ERR_UNSUPPORTED.  Replaces the NEP constructor +
 * JIT compile and NEP.calEnergyForceVirial (NEP.java:171-212). */
int nnap_create_nep(const char* nep_txt, size_t len, int precision, int device, nnap_handle** out);
/* Same, reading the nep.txt text from a file. */
int nnap_create_nep_from_file(const char* path, int precision, int device, nnap_handle** out);
/* Release the handle and its device memory (NNAP.close, NNAP.java:472-486). */
int nnap_destroy(nnap_handle* h);

/* Model queries: NNAP.ntypes / rcutMax / symbol / units (NNAP.java:86-90, 489-491). */
int nnap_ntypes(const nnap_handle* h, int* ntypes);
int nnap_rcut_max(const nnap_handle* h, double* rcut);
int nnap_symbol(const nnap_handle* h, int type, char* buf, size_t buflen);
int nnap_descriptor_size(const nnap_handle* h, int type, int* size);
/* Message of the last failing call on this handle (empty when none). */
const char* nnap_last_error(const nnap_handle* h);

/* Energy / forces / virials of one periodic structure, host buffers.
 * Replaces IPairPotential.calEnergyForceVirials(APC, ...) for an NNAP
 * (IPairPotential.java:811-1022 -> NNAP.calEnergyForceVirial, NNAP.java:553-594).
 * x: 3n doubles; type: n ints (1-based); box: 9 doubles.  Outputs selected by flags;
 * unselected output pointers may be NULL.  Synchronous. */
int nnap_compute(nnap_handle* h, int natoms, const double* x, const int* type, int box_kind, const double* box,
                 int flags, double* energy, double* energies, double* forces, double* virial, double* virials);

/* Same computation on device-resident buffers; x, type, and every output are device
 * pointers, box stays a host array.  Work is ordered after `stream` (a cudaStream_t; NULL
 * is CUDA's default stream) and `stream` is made to wait for the results.  The whole
 * evaluation is queued without intermediate host synchronisation; the call then waits
 * for it once, to read the error and neighbour-capacity word (an overflowing capacity
 * is grown and the evaluation repeated). */
int nnap_compute_device(nnap_handle* h, int natoms, const double* d_x, const int* d_type, int box_kind,
                        const double* box, int flags, double* d_energy, double* d_energies, double* d_forces,
                        double* d_virial, double* d_virials, void* stream);

/* Many independent structures in one launch sequence (the batched form; each structure
 * gives the same result as nnap_compute on it alone, within floating-point rounding).
 * natoms[s] atoms per structure; x/type are concatenated over structures; box_kind[s]
 * and boxes[9*s] per structure.  energy[s] and virial[9*s] are per structure; energies,
 * forces, virials are concatenated per atom.  Host buffers, synchronous. */
int nnap_compute_batch(nnap_handle* h, int nstruct, const int* natoms, const double* x, const int* type,
                       const int* box_kind, const double* boxes, int flags, double* energy, double* energies,
                       double* forces, double* virial, double* virials);

/* The batched form on device-resident buffers: d_x / d_type hold the concatenated
 * structures; natoms, box_kind and boxes stay host arrays; every output is a device
 * pointer with the layout of nnap_compute_batch.  Ordering as nnap_compute_device. */
int nnap_compute_batch_device(nnap_handle* h, int nstruct, const int* natoms, const double* d_x, const int* d_type,
                              const int* box_kind, const double* boxes, int flags, double* d_energy,
                              double* d_energies, double* d_forces, double* d_virial, double* d_virials,
                              void* stream);

/* Descriptor vectors of every atom (NNAP.calFp, NNAP.java:596-632 -> jse_nnap_calFp,
 * nnap_interface.cpp:11-25).  fp is n x stride doubles, stride >= the largest
 * descriptor size; entries beyond an atom's own size are zero.  Host buffers. */
int nnap_compute_fp(nnap_handle* h, int natoms, const double* x, const int* type, int box_kind, const double* box,
                    double* fp, int stride);

/* Full neighbour list of one structure with the model's largest cutoff, for parity
 * checks against NeighborListGetter (NeighborListGetter.java:1018-1050).  counts: n
 * ints; if j is non-NULL, j/img (cap and 3*cap ints) receive, atom by atom, the
 * neighbour index and its image (n_a, n_b, n_c) along a, b, c.  *total receives the
 * number of pairs.  Host buffers. */
int nnap_neighbor_list(nnap_handle* h, int natoms, const double* x, const int* type, int box_kind,
                       const double* box, int* counts, long long cap, int* j, int* img, long long* total);

/* LAMMPS-style evaluation: one call per force evaluation of a LAMMPS pair style.  It
 * replaces the reference's jse_nnap_lammps2cuda + jse_nnap_computeLammpsCuda +
 * jse_nnap_cuda2lammps sequence (nnap_interface_cuda.cu:319-483, driven by
 * NNAP.java:919-1030 for PairNNAP_gpu).  Inputs are LAMMPS's own arrays:
 *   inum local atoms ilist[inum] with full neighbour lists numneigh[i] / firstneigh[i]
 *   (indices into 0..nall-1; special-bond bits above 0x1FFFFFFF are masked off);
 *   x: nall x 3 doubles (local then ghost atoms, ghosts already at their image
 *   positions); type: nall LAMMPS types, mapped through type_map[type] to 1-based NNAP
 *   species (type_map NULL: identity; it must cover every type value present).
 * A pair is kept when |x_j - x_i|^2 < rcut^2 (FP64).  Results are ADDED to LAMMPS's
 * accumulators, as cuda2lammps does: f (nall x 3, ghosts included, for LAMMPS's reverse
 * communication), *eng_vdwl (eflag), eatom[i] (eflag_atom), virial[6] (vflag: xx, yy,
 * zz, xy, xz, yz), vatom (nall x 6, vflag_atom) and cvatom (nall x 9, cvflag_atom:
 * xx, yy, zz, xy, xz, yz, yx, zx, zy), the pair term dx (x) g assigned to the neighbour.
 * The scatter is atomic-free and deterministic.  Host buffers, synchronous. */
int nnap_compute_lammps(nnap_handle* h, int inum, int nall, const int* ilist, const int* numneigh,
                        const int* const* firstneigh, const double* x, const int* type, const int* type_map,
                        int eflag, int vflag, int eflag_atom, int vflag_atom, int cvflag_atom, double* f,
                        double* eng_vdwl, double* eatom, double* virial, double* vatom, double* cvatom);
/* Same, with the reference's nlflag (jse_nnap_lammps2cuda, NNAP.java:948-1000: nlflag =
 * neighbor->ago == 0).  nlflag = 0 reuses the device copy of the list sent by the last
 * call on this handle that had nlflag = 1 (nnap_compute_lammps counts as one): ilist,
 * numneigh and firstneigh must be unchanged and are not read; inum and nall must match
 * (NNAP_ERR_ARG otherwise, or when no such call precedes).  Positions and types are sent
 * every call; pairs are re-filtered by the cutoff every call. */
int nnap_compute_lammps_nl(nnap_handle* h, int nlflag, int inum, int nall, const int* ilist, const int* numneigh,
                           const int* const* firstneigh, const double* x, const int* type, const int* type_map,
                           int eflag, int vflag, int eflag_atom, int vflag_atom, int cvflag_atom, double* f,
                           double* eng_vdwl, double* eatom, double* virial, double* vatom, double* cvatom);

/* Parameter counts of species `type` (1-based): *fp_size entries of its basis's C-level
 * parameters (the internal radial-fuse matrices of its sub-bases, [t_nei][np][n] each,
 * WTypeBasis.cptrParameterSize, WTypeBasis.java:609-611) and *nn_size of its network
 * (hidden W [out][in] per layer | output W | hidden b per layer | output b,
 * FeedForward.mountCptrParameter, FeedForward.java:310-316). */
int nnap_param_sizes(const nnap_handle* h, int type, int* fp_size, int* nn_size);

/* Force-training gradients: dL/dparameters of
 *   L = sum_i bE_i E_i + sum_i bF_i . F_i + sum_s sum_ab bW_sab W_sab
 * over a batch of structures (E per-atom energies, F forces, W_s the total virial of
 * structure s, components xx, yy, zz, xy, xz, yz, yx, zx, zy).  Replaces the per-atom
 * training pair jse_nnap_forwardEnergyForce + jse_nnap_backwardEnergyForce
 * (nnap_interface.cpp:142-232) as TrainerNNAP drives it (TrainerNNAP.java:1006-1175:
 * every pair (i, j) receives bF_j - bF_i plus the stress terms as the upstream gradient
 * of its g_ij, and bE_i as that of E_i).  Batch layout as nnap_compute_batch.
 * bgrad_energies (n), bgrad_forces (3n) and bgrad_virial (9 per structure) may each be
 * NULL (zero).  grad_nn receives, concatenated over species, the network gradients in
 * the layout of nnap_param_sizes; grad_fp (may be NULL) the basis gradients in the same
 * way: for sub-bases with trainable radial weights (wtype fuse, rfuse, exfuse, and
 * post-fused ones) the gradient of the internal radial-fuse matrix, added to the species
 * that owns the parameters (a mirror or shared basis's gradient goes to its source, as
 * in nnap_main.hpp:398-445); zero for the other weight types, for which the reference
 * computes none.  Arithmetic is FP32 with FP64 sums over fixed partitions of the atoms,
 * whatever the handle's precision, so repeated calls return identical results.  Host
 * buffers, synchronous. */
int nnap_train_grad_batch(nnap_handle* h, int nstruct, const int* natoms, const double* x, const int* type,
                          const int* box_kind, const double* boxes, const double* bgrad_energies,
                          const double* bgrad_forces, const double* bgrad_virial, double* grad_fp,
                          double* grad_nn);

/* Number of this library's kernels launched by the last compute call on the handle. */
int nnap_last_launch_count(const nnap_handle* h, int* count);

/* Stage timing (no counterpart in the reference; used by the benchmark).  When on,
 * compute calls record CUDA events on the handle's stream around five stages:
 * [0] wrap, cells, neighbour rows, mirror index and species sort; [1] descriptors
 * forward; [2] network; [3] descriptors backward; [4] force/virial gather and FP64
 * reductions.  nnap_stage_times waits for the last call and returns milliseconds. */
int nnap_set_profiling(nnap_handle* h, int on);
/* CUDA-graph replay of repeated evaluations (on by default; no counterpart in the
 * reference).  The first call of a layout (atom counts, box kinds, cell grids, buffer
 * addresses) runs eagerly, the second is captured, later ones replay the graph. */
int nnap_set_graphs(nnap_handle* h, int on);
/* Launch-shape autotuning (no counterpart in the reference).  Evaluations are grouped
 * into atom-count buckets, natoms in [2^b, 2^(b+1)).  With autotuning on, the first
 * evaluation of a bucket that has no shapes yet times the candidates of each stage on
 * the caller's own batch (warps per CTA 2/4/8 of the descriptor forward, descriptor
 * backward and neighbour kernels; 64/128/256 threads per CTA of the gather; 2 or 4
 * threads per row of the tensor-core network) and keeps the fastest; later evaluations
 * of the bucket reuse them.  Off by default; untuned buckets use 4, 4, 4, 128, 4. */
int nnap_set_autotune(nnap_handle* h, int on);
/* Shapes used for natoms atoms: [descriptor forward warps, descriptor backward warps,
 * neighbour warps, gather threads, network threads per row]; *tuned = 1 when the
 * bucket has tuned (or installed) shapes, 0 for the defaults.  tuned may be NULL. */
int nnap_get_tuning(nnap_handle* h, int natoms, int* shapes5, int* tuned);
/* Install shapes for the bucket of natoms (e.g. saved from an earlier run). */
int nnap_set_tuning(nnap_handle* h, int natoms, const int* shapes5);
int nnap_stage_times(nnap_handle* h, double* ms5);

/* Per-atom neighbour counts of one structure without allocating any memory.  This entry
 * point has no counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc when they need the answer: an engine (or a framework's caching allocator)
 * that reserves all device memory for its own pool up front, so a later cudaMalloc
 * fails, or code in a latency-critical loop where cudaMalloc/cudaFree would synchronise
 * the device.  No handle is needed; rcut is the cutoff.  d_x (3n doubles), d_type
 * (n ints) and d_counts (n ints) are device pointers; box is a host array.  The box
 * and cutoff pass the same checks as every other entry point (NNAP_ERR_ARG otherwise).
 * Its scratch is one fixed 2 MiB device array compiled into the library (held by every
 * GPU that loads it): at most 16384 atoms and 16384 cells of the cell list, larger
 * inputs return NNAP_ERR_CAPACITY before any device work.  The first call on each
 * device looks up that array's address and should come before any stream capture.
 * All calls share the array, so calls whose work overlaps on the GPU race.  Work is
 * queued on `stream` (NULL: CUDA's default stream) and the call waits for it. */
int nnap_neighbor_counts_noalloc(int natoms, const double* d_x, const int* d_type, int box_kind, const double* box,
                                 double rcut, int* d_counts, void* stream);

/* ---------------------------------------------------------------- serving
 * Resident structures evaluated by continuous batching (no counterpart in the
 * reference, which evaluates one structure per call and rebuilds its neighbour list
 * each time).  A server owns one handle until nnap_server_destroy: make no other call
 * on that handle meanwhile, and destroy the server before the handle.
 *
 * nnap_server_admit makes a structure resident (its species, box and neighbour rows at
 * rcut + skin stay on the device) and returns its slot.  nnap_server_step evaluates any
 * set of slots together in one batched launch sequence; slots admitted since the last
 * step join it, released ones leave it.  A slot's neighbour rows are rebuilt when it is
 * new or when one of its atoms moved more than skin/2 (in the caller's coordinates)
 * since its last rebuild; otherwise the stored rows are filtered at rcut, which gives
 * exactly the full search's neighbour set.  Admission is refused with NNAP_ERR_BUSY
 * while memory_budget bytes (the resident arrays plus the work buffers of a step over
 * every resident atom) or max_structs slots (0: 4096) are in use, and with
 * NNAP_ERR_CAPACITY for a structure that would not fit an empty server. */
typedef struct nnap_server nnap_server;
int nnap_server_create(nnap_handle* h, double skin, size_t memory_budget, int max_structs, nnap_server** out);
int nnap_server_destroy(nnap_server* s);
/* Admit one structure: natoms atoms, species type[natoms], box as in nnap_compute. */
int nnap_server_admit(nnap_server* s, int natoms, const int* type, int box_kind, const double* box, int* slot);
int nnap_server_release(nnap_server* s, int slot);
/* Evaluate the listed slots (each at most once) at positions x, the slots' atoms
 * concatenated in the order of `slots`.  Outputs as nnap_compute_batch, in the same
 * order (energy[q], virial[9*q] per listed slot).  Host buffers, synchronous. */
int nnap_server_step(nnap_server* s, int nslots, const int* slots, const double* x, int flags, double* energy,
                     double* energies, double* forces, double* virial, double* virials);
/* The same step in two halves, so the caller's host work overlaps the device: submit
 * stages the positions (xs[q]: the 3 n_q positions of slots[q]; the arrays may change as
 * soon as it returns) and queues the whole evaluation without waiting; collect waits for
 * it and writes the outputs selected by the submitted flags, in the order of `slots`
 * (layout of nnap_server_step).  One step at a time: a second submit, a step call or a
 * neighbour-list query before the collect returns NNAP_ERR_BUSY, the release of a slot of
 * the step in flight NNAP_ERR_ARG; admissions are allowed meanwhile. */
int nnap_server_submit(nnap_server* s, int nslots, const int* slots, const double* const* xs, int flags);
int nnap_server_collect(nnap_server* s, double* energy, double* energies, double* forces, double* virial,
                        double* virials);
/* Neighbour list that the last step used for `slot` (layout of nnap_neighbor_list;
 * neighbour indices local to the slot). */
int nnap_server_neighbor_list(nnap_server* s, int slot, int* counts, long long cap, int* j, int* img,
                              long long* total);
/* out8: resident slots, resident atoms, resident bytes, work bytes, steps, slot
 * rebuilds, neighbour-row capacity, memory budget. */
int nnap_server_stats(const nnap_server* s, long long* out8);

#ifdef __cplusplus
}
#endif

#endif /* NNAP_GB300_H */
