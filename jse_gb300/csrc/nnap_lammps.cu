// LAMMPS-style boundary: one call per force evaluation of a LAMMPS pair style, with
// LAMMPS's own data (local atoms, ghost atoms, full neighbour list).  It stands where
// the reference's GPU pair style calls jse_nnap_lammps2cuda, jse_nnap_computeLammpsCuda
// and jse_nnap_cuda2lammps in turn (nnap_interface_cuda.cu:319-483, NNAP.java:919-1030):
// the same inputs, the same accumulation into LAMMPS's arrays, one synchronous call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "api_internal.hpp"

namespace nnapgb {
__global__ void k_lmp_rows(int, int, const int*, const int*, const int*, const double*, const int*, int, double,
                           PairBufs, int*, int*, int*);
__global__ void k_lmp_count(PairBufs, int, int*);
__global__ void k_lmp_fill(PairBufs, int, const int*, int*, int*);
__global__ void k_lmp_gather(PairBufs, int, const int*, const int*, const int*, double*, double*);
__global__ void k_lmp_virial_sum(const double*, int, double*);
}  // namespace nnapgb

using namespace nnapgb;

namespace {
constexpr int kLmpNeighMask = 0x1FFFFFFF;  // LAMMPS keeps special-bond bits above this mask
constexpr size_t kLmpThreadedEntries = 1 << 18;  // list entries from which the copy is threaded
constexpr unsigned kLmpMaxThreads = 8;
}

namespace {

// nlflag = 0: the list (inum, nall, ilist, numneigh, firstneigh) is the one of the last
// call with nlflag = 1 on this handle; its device copy is reused and only positions and
// types are sent (NNAP.computeLammpsCuda passes nlflag = neighbor->ago == 0 to
// jse_nnap_lammps2cuda, NNAP.java:948-1000).
int compute_lammps(nnap_handle* h, int nlflag, int inum, int nall, const int* ilist, const int* numneigh,
                   const int* const* firstneigh, const double* x, const int* type, const int* type_map, int eflag,
                   int vflag, int eflag_atom, int vflag_atom, int cvflag_atom, double* f, double* eng_vdwl,
                   double* eatom, double* virial, double* vatom, double* cvatom) {
    return guarded(h, [&]() -> int {
        if (inum < 0 || nall < inum) throw ApiFail(NNAP_ERR_ARG, "need 0 <= inum <= nall");
        if (inum > 0 && (!ilist || !numneigh || !firstneigh)) throw ApiFail(NNAP_ERR_ARG, "neighbour list is NULL");
        if (nall > 0 && (!x || !type || !f)) throw ApiFail(NNAP_ERR_ARG, "positions, types or forces are NULL");
        if (eflag && !eng_vdwl) throw ApiFail(NNAP_ERR_ARG, "energy accumulator is NULL");
        if (eflag_atom && !eatom) throw ApiFail(NNAP_ERR_ARG, "per-atom energies are NULL");
        if (vflag && !virial) throw ApiFail(NNAP_ERR_ARG, "virial accumulator is NULL");
        if (vflag_atom && !vatom) throw ApiFail(NNAP_ERR_ARG, "per-atom virials are NULL");
        if (cvflag_atom && !cvatom) throw ApiFail(NNAP_ERR_ARG, "centroid per-atom virials are NULL");
        h->launches = 0;
        if (nall == 0) return NNAP_OK;
        const bool reuse = !nlflag;
        if (reuse && !(h->lmp_cached && h->lmp_inum == inum && h->lmp_nall == nall))
            throw ApiFail(NNAP_ERR_ARG, "nlflag = 0 needs the list of an earlier call with the same inum and nall");
        h->lmp_cached = false;  // set again once this call's list is on the device
        // host-side layout, written straight into pinned staging: species through the type
        // map, the row of each local atom, the list in ilist order
        size_t total = reuse ? h->lmp_total : 0;
        int deg_max = reuse ? h->lmp_deg : 0;
        for (int ii = 0; ii < inum && !reuse; ++ii) {
            const int i = ilist[ii];
            if (i < 0 || i >= nall) throw ApiFail(NNAP_ERR_ARG, "ilist entries must be distinct atoms");
            if (numneigh[i] < 0) throw ApiFail(NNAP_ERR_ARG, "negative neighbour count");
            total += (size_t)numneigh[i];
            deg_max = std::max(deg_max, numneigh[i]);
        }
        if (total > (size_t)INT32_MAX) throw ApiFail(NNAP_ERR_CAPACITY, "more than 2^31 neighbour entries");
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        const size_t in_bytes = 2 * al(sizeof(int) * nall) + al(sizeof(int) * ((size_t)inum + 1)) +
                                al(sizeof(int) * std::max<size_t>(total, 1));
        char* pin = static_cast<char*>(h->lmp_pin_in.ensure(in_bytes));
        int* ty = reinterpret_cast<int*>(pin);
        int* row_of = reinterpret_cast<int*>(pin + al(sizeof(int) * nall));
        int* off = reinterpret_cast<int*>(pin + 2 * al(sizeof(int) * nall));
        int* nidx = reinterpret_cast<int*>(pin + 2 * al(sizeof(int) * nall) + al(sizeof(int) * ((size_t)inum + 1)));
        for (int a = 0; a < nall; ++a) ty[a] = type_map ? type_map[type[a]] : type[a];
        for (int a = 0; a < nall && !reuse; ++a) row_of[a] = -1;
        off[0] = 0;
        if (!reuse) {
        for (int ii = 0; ii < inum; ++ii) {
            const int i = ilist[ii];
            if (row_of[i] >= 0) throw ApiFail(NNAP_ERR_ARG, "ilist entries must be distinct atoms");
            row_of[i] = ii;
            off[ii + 1] = off[ii] + numneigh[i];
        }
        // the list copy (the bulk of the host work) in contiguous ranges of ilist, one per thread
        auto copy_rows = [&](int a, int b) {
            for (int ii = a; ii < b; ++ii) {
                const int i = ilist[ii];
                const int* src = firstneigh[i];
                int* dst = nidx + off[ii];
                for (int jj = 0, c = numneigh[i]; jj < c; ++jj) dst[jj] = src[jj] & kLmpNeighMask;
            }
        };
        const int nth = total >= kLmpThreadedEntries
                            ? (int)std::min<unsigned>(kLmpMaxThreads, std::max(1u, std::thread::hardware_concurrency()))
                            : 1;
        if (nth > 1) {
            std::vector<std::thread> th;
            for (int k = 1; k < nth; ++k)
                th.emplace_back(copy_rows, (int)((long long)inum * k / nth), (int)((long long)inum * (k + 1) / nth));
            copy_rows(0, inum / nth);
            for (auto& t : th) t.join();
        } else {
            copy_rows(0, inum);
        }
        }
        // device buffers: rows for the local atoms at capacity = longest list
        const int n1 = std::max(inum, 1);
        h->M = std::max(8, (deg_max + 7) & ~7);
        h->GS = 0;
        ensure_work(h, n1, 1, 1, 1);
        drop_graph(h);
        h->layout_ok = false;
        h->lmp_x.ensure(3 * (size_t)nall);
        h->lmp_type.ensure(nall);
        h->lmp_ilist.ensure(n1);
        h->lmp_off.ensure((size_t)inum + 1);
        h->lmp_idx.ensure(std::max<size_t>(total, 1));
        h->lmp_rowtype.ensure(n1);
        h->lmp_rowof.ensure(nall);
        h->lmp_tcount.ensure(nall);
        h->lmp_tstart.ensure((size_t)nall + 1);
        h->lmp_tfill.ensure(nall);
        h->lmp_tlist.ensure(std::max<size_t>(total, 1));
        h->lmp_forces.ensure(3 * (size_t)nall);
        h->lmp_virials.ensure(9 * (size_t)nall);
        cudaStream_t st = h->stream;
        const int T = h->model.ntypes();
        CK(cudaMemcpyAsync(h->lmp_x.p, x, sizeof(double) * 3 * nall, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(h->lmp_type.p, ty, sizeof(int) * nall, cudaMemcpyHostToDevice, st));
        if (!reuse) {
            CK(cudaMemcpyAsync(h->lmp_rowof.p, row_of, sizeof(int) * nall, cudaMemcpyHostToDevice, st));
            if (inum) {
                CK(cudaMemcpyAsync(h->lmp_ilist.p, ilist, sizeof(int) * inum, cudaMemcpyHostToDevice, st));
                CK(cudaMemcpyAsync(h->lmp_off.p, off, sizeof(int) * (inum + 1), cudaMemcpyHostToDevice, st));
            }
            if (total) CK(cudaMemcpyAsync(h->lmp_idx.p, nidx, sizeof(int) * total, cudaMemcpyHostToDevice, st));
        }
        CK(cudaMemsetAsync(h->status.p, 0, sizeof(int) * 2, st));
        CK(cudaMemsetAsync(h->lmp_tcount.p, 0, sizeof(int) * nall, st));
        CK(cudaMemsetAsync(h->lmp_tfill.p, 0, sizeof(int) * nall, st));
        // rows, species order, descriptors / network / gradients, then the scatter
        Batch B;
        B.nstruct = 1;
        B.natoms = inum;
        const double rc = h->model.rcut_max;
        if (inum) {
            k_lmp_rows<<<(unsigned)(((size_t)inum * 32 + 255) / 256), 256, 0, st>>>(
                inum, nall, h->lmp_ilist.p, h->lmp_off.p, h->lmp_idx.p, h->lmp_x.p, h->lmp_type.p, T, rc * rc,
                pair_bufs(h), h->lmp_rowtype.p, h->status.p, h->status.p + 1);
            ++h->launches;
            enqueue_species(h, inum, h->lmp_rowtype.p);
            enqueue_eval(h, B, h->lmp_rowtype.p, false, false);
            const size_t slots = (size_t)inum * h->M;
            k_lmp_count<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(pair_bufs(h), inum, h->lmp_tcount.p);
            h->launches += 1;
        }
        k_scan_excl<<<1, 1024, 0, st>>>(h->lmp_tcount.p, nall, h->lmp_tstart.p);
        if (inum) {
            const size_t slots = (size_t)inum * h->M;
            k_lmp_fill<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(pair_bufs(h), inum, h->lmp_tstart.p,
                                                                       h->lmp_tfill.p, h->lmp_tlist.p);
            ++h->launches;
        }
        k_sort_cells<<<(unsigned)(((size_t)nall * 32 + 255) / 256), 256, 0, st>>>(h->lmp_tstart.p, nall,
                                                                                  h->lmp_tlist.p);
        k_lmp_gather<<<(nall + 127) / 128, 128, 0, st>>>(pair_bufs(h), nall, h->lmp_rowof.p, h->lmp_tstart.p,
                                                         h->lmp_tlist.p, h->lmp_forces.p, h->lmp_virials.p);
        h->launches += 3;
        CK(cudaGetLastError());
        // results back (pinned) and into LAMMPS's accumulators; a global virial alone is
        // summed on the device in a fixed order
        const bool per_atom_v = vflag_atom || cvflag_atom;
        if (vflag && !per_atom_v) {
            k_lmp_virial_sum<<<1, kLmpSumThreads, 0, st>>>(h->lmp_virials.p, nall, h->virial.p);
            ++h->launches;
            CK(cudaGetLastError());
        }
        const size_t out_bytes = al(sizeof(double) * 3 * nall) + al(sizeof(double) * n1) +
                                 al(sizeof(double) * (per_atom_v ? 9 * (size_t)nall : 9));
        char* pout = static_cast<char*>(h->lmp_pin_out.ensure(out_bytes));
        double* fo = reinterpret_cast<double*>(pout);
        double* eo = reinterpret_cast<double*>(pout + al(sizeof(double) * 3 * nall));
        double* vo = reinterpret_cast<double*>(pout + al(sizeof(double) * 3 * nall) + al(sizeof(double) * n1));
        CK(cudaMemcpyAsync(h->h_status, h->status.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(fo, h->lmp_forces.p, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, st));
        if ((eflag || eflag_atom) && inum)
            CK(cudaMemcpyAsync(eo, h->e_atom.p, sizeof(double) * inum, cudaMemcpyDeviceToHost, st));
        if (per_atom_v)
            CK(cudaMemcpyAsync(vo, h->lmp_virials.p, sizeof(double) * 9 * nall, cudaMemcpyDeviceToHost, st));
        else if (vflag)
            CK(cudaMemcpyAsync(vo, h->virial.p, sizeof(double) * 6, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        const int bits = h->h_status[0];
        if (bits & ERRBIT_BAD_TYPE) throw ApiFail(NNAP_ERR_BAD_TYPE, "species outside 1..ntypes");
        if (bits & ERRBIT_CELLS) throw ApiFail(NNAP_ERR_ARG, "neighbour or ilist index outside 0..nall-1");
        if (bits & ERRBIT_TIMEOUT) throw ApiFail(NNAP_ERR_TIMEOUT, "a bounded tensor-core wait gave up");
        if (bits & ERRBIT_CAPACITY) throw ApiFail(NNAP_ERR_CAPACITY, "neighbour rows overflowed");
        for (size_t q = 0; q < 3 * (size_t)nall; ++q) f[q] += fo[q];
        if (eflag)
            for (int ii = 0; ii < inum; ++ii) *eng_vdwl += eo[ii];
        if (eflag_atom)
            for (int ii = 0; ii < inum; ++ii) eatom[ilist[ii]] += eo[ii];
        if (per_atom_v) {
            for (int a = 0; a < nall; ++a) {
                const double* w = vo + 9 * (size_t)a;
                if (vflag)
                    for (int c = 0; c < 6; ++c) virial[c] += w[c];
                if (vflag_atom)
                    for (int c = 0; c < 6; ++c) vatom[6 * (size_t)a + c] += w[c];
                if (cvflag_atom)
                    for (int c = 0; c < 9; ++c) cvatom[9 * (size_t)a + c] += w[c];
            }
        } else if (vflag) {
            for (int c = 0; c < 6; ++c) virial[c] += vo[c];
        }
        h->lmp_cached = true;
        h->lmp_inum = inum;
        h->lmp_nall = nall;
        h->lmp_total = total;
        h->lmp_deg = deg_max;
        return NNAP_OK;
    });
}

}  // namespace

extern "C" int nnap_compute_lammps(nnap_handle* h, int inum, int nall, const int* ilist, const int* numneigh,
                                   const int* const* firstneigh, const double* x, const int* type,
                                   const int* type_map, int eflag, int vflag, int eflag_atom, int vflag_atom,
                                   int cvflag_atom, double* f, double* eng_vdwl, double* eatom, double* virial,
                                   double* vatom, double* cvatom) {
    return compute_lammps(h, 1, inum, nall, ilist, numneigh, firstneigh, x, type, type_map, eflag, vflag, eflag_atom,
                          vflag_atom, cvflag_atom, f, eng_vdwl, eatom, virial, vatom, cvatom);
}

extern "C" int nnap_compute_lammps_nl(nnap_handle* h, int nlflag, int inum, int nall, const int* ilist,
                                      const int* numneigh, const int* const* firstneigh, const double* x,
                                      const int* type, const int* type_map, int eflag, int vflag, int eflag_atom,
                                      int vflag_atom, int cvflag_atom, double* f, double* eng_vdwl, double* eatom,
                                      double* virial, double* vatom, double* cvatom) {
    return compute_lammps(h, nlflag, inum, nall, ilist, numneigh, firstneigh, x, type, type_map, eflag, vflag,
                          eflag_atom, vflag_atom, cvflag_atom, f, eng_vdwl, eatom, virial, vatom, cvatom);
}
