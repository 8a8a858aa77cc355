// Driver around the reference's own per-atom NNAP arithmetic.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build.py together with the
// reference's nnap_interface.cpp after oracle/nnapgen.py has expanded it (and the
// headers it includes) into oracle/_ref/<shape>/src.  The expanded reference files
// are build output and are never committed.
//
// The driver restates the orchestration that surrounds the reference's exported
// per-atom function jse_nnap_calEnergyForce (nnap_interface.cpp:48-89):
//   * the per-atom loop of NNAP.calEnergyForceVirial (NNAP.java:553-594),
//   * the static round-robin thread split of ParforThreadPool (ParforThreadPool.java:87-110)
//     with per-thread neighbour buffers (NNAP.java:188-224) and per-thread output
//     arrays summed at the end (IPairPotential.java:895-906, 1008-1020),
//   * the energy / force / virial accumulators (IPairPotential.java:919-1006), with the
//     per-atom virial assigned to the neighbour index (GPUMD convention, NNAP.java:589-590).
// The neighbour list itself is supplied by the caller (the oracle's restatement of
// NeighborListGetter), because the reference's Java neighbour search cannot run here.

#include <cstring>
#include <thread>
#include <vector>

extern "C" int jse_nnap_calEnergyForce(double* aNlDx, double* aNlDy, double* aNlDz, int* aNlType, int aNeiNum, int ctype,
                                       double** aFpHyperParam, double** aFpParam, double** aNnParam, double* aNormParam,
                                       double* rOutEng, double* rGradNlDx, double* rGradNlDy, double* rGradNlDz,
                                       double* rFpForwardCache);
extern "C" int jse_nnap_forwardEnergyForce(double* aNlDx, double* aNlDy, double* aNlDz, int* aNlType, int aNeiNum,
                                           int ctype, double** aFpHyperParam, double** aFpParam, double** aNnParam,
                                           double* aNormParam, double* rOutEng, double* rGradNlDx, double* rGradNlDy,
                                           double* rGradNlDz, double* rFpForwardCache, double* rNnForwardCache,
                                           double* rFpBackwardCache, double* rNnBackwardCache);
extern "C" int jse_nnap_backwardEnergyForce(double* aNlDx, double* aNlDy, double* aNlDz, int* aNlType, int aNeiNum,
                                            int ctype, double** aFpHyperParam, double** aFpParam, double** aNnParam,
                                            double* aNormParam, double aBGradEng, double* aBGradAGradNlDx,
                                            double* aBGradAGradNlDy, double* aBGradAGradNlDz, double** rBGradFpParam,
                                            double** rBGradNnParam, double* aFpForwardCache, double* aNnForwardCache,
                                            double* aFpBackwardCache, double* aNnBackwardCache,
                                            double* rFpBackwardBackwardCache);
extern "C" int jse_nnap_calFp(double* aNlDx, double* aNlDy, double* aNlDz, int* aNlType, int aNeiNum, int ctype,
                              double** aFpHyperParam, double** aFpParam, double* rFp);

namespace {

struct ThreadBuf {
    std::vector<double> dx, dy, dz, gx, gy, gz, cache;
    std::vector<int> ty;
    std::vector<double> e, f, v;
    int status = 0;
};

void run_atoms(int tid, int nthreads, int n_eval, const int* type, const long* nei_off, const int* nei_j,
               const double* nei_dx, double** hp, double** fpp, double** nnp, double** normp,
               long cache_per_nei, long cache_const, bool want_e, bool want_f, bool want_v, ThreadBuf& B) {
    for (int i = tid; i < n_eval; i += nthreads) {
        const long o = nei_off[i];
        const int nn = (int)(nei_off[i + 1] - o);
        B.dx.resize(nn + 1); B.dy.resize(nn + 1); B.dz.resize(nn + 1);
        B.gx.resize(nn + 1); B.gy.resize(nn + 1); B.gz.resize(nn + 1);
        B.ty.resize(nn + 1);
        B.cache.resize(cache_per_nei * (nn + 1) + cache_const);
        for (int j = 0; j < nn; ++j) {
            B.dx[j] = nei_dx[3 * (o + j)];
            B.dy[j] = nei_dx[3 * (o + j) + 1];
            B.dz[j] = nei_dx[3 * (o + j) + 2];
            B.ty[j] = type[nei_j[o + j]];
        }
        double e = 0.0;
        const int ct = type[i];
        int code = jse_nnap_calEnergyForce(B.dx.data(), B.dy.data(), B.dz.data(), B.ty.data(), nn, ct,
                                           hp, fpp, nnp, normp[ct - 1], &e, B.gx.data(), B.gy.data(), B.gz.data(),
                                           B.cache.data());
        if (code != 0) { B.status = code; return; }
        if (want_e) B.e[i] += e;
        for (int j = 0; j < nn; ++j) {
            const int jj = nei_j[o + j];
            const double fx = B.gx[j], fy = B.gy[j], fz = B.gz[j];
            if (want_f) {
                B.f[3 * i] -= fx; B.f[3 * i + 1] -= fy; B.f[3 * i + 2] -= fz;
                B.f[3 * jj] += fx; B.f[3 * jj + 1] += fy; B.f[3 * jj + 2] += fz;
            }
            if (want_v) {
                const double dx = B.dx[j], dy = B.dy[j], dz = B.dz[j];
                double* v = B.v.data() + 9 * (size_t)jj;
                v[0] += dx * fx; v[1] += dy * fy; v[2] += dz * fz;
                v[3] += dx * fy; v[4] += dx * fz; v[5] += dy * fz;
                v[6] += dy * fx; v[7] += dz * fx; v[8] += dz * fy;
            }
        }
    }
}

}  // namespace

extern "C" {

// Energies, forces and per-atom virials of one structure through the reference's
// per-atom arithmetic.  Atoms [0, n_eval) are evaluated (n_eval <= n; a prefix is used
// to time a bounded sample); output arrays hold n atoms.  Any of e_atom/force/virial
// may be NULL.  Returns the first nonzero code of the reference function, or 0.
int ref_compute(int T, double** hp, double** fpp, double** nnp, double** normp, int n, int n_eval, const int* type,
                const long* nei_off, const int* nei_j, const double* nei_dx, long cache_per_nei, long cache_const,
                int nthreads, double* e_atom, double* force, double* virial) {
    (void)T;
    if (nthreads < 1) nthreads = 1;
    std::vector<ThreadBuf> bufs(nthreads);
    for (auto& B : bufs) {
        if (e_atom) B.e.assign(n, 0.0);
        if (force) B.f.assign(3 * (size_t)n, 0.0);
        if (virial) B.v.assign(9 * (size_t)n, 0.0);
    }
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t)
        th.emplace_back(run_atoms, t, nthreads, n_eval, type, nei_off, nei_j, nei_dx, hp, fpp, nnp, normp,
                        cache_per_nei, cache_const, e_atom != nullptr, force != nullptr, virial != nullptr,
                        std::ref(bufs[t]));
    run_atoms(0, nthreads, n_eval, type, nei_off, nei_j, nei_dx, hp, fpp, nnp, normp, cache_per_nei, cache_const,
              e_atom != nullptr, force != nullptr, virial != nullptr, bufs[0]);
    for (auto& t : th) t.join();
    for (auto& B : bufs) if (B.status) return B.status;
    if (e_atom) { std::memset(e_atom, 0, sizeof(double) * n); for (auto& B : bufs) for (int i = 0; i < n; ++i) e_atom[i] += B.e[i]; }
    if (force) { std::memset(force, 0, sizeof(double) * 3 * n); for (auto& B : bufs) for (size_t i = 0; i < 3 * (size_t)n; ++i) force[i] += B.f[i]; }
    if (virial) { std::memset(virial, 0, sizeof(double) * 9 * n); for (auto& B : bufs) for (size_t i = 0; i < 9 * (size_t)n; ++i) virial[i] += B.v[i]; }
    return 0;
}

// Descriptor vectors through the reference's jse_nnap_calFp (nnap_interface.cpp:11-25).
int ref_fp(double** hp, double** fpp, int n, const int* type, const long* nei_off, const int* nei_j,
           const double* nei_dx, double* fp, int fp_stride) {
    std::vector<double> dx, dy, dz;
    std::vector<int> ty;
    for (int i = 0; i < n; ++i) {
        const long o = nei_off[i];
        const int nn = (int)(nei_off[i + 1] - o);
        dx.resize(nn + 1); dy.resize(nn + 1); dz.resize(nn + 1); ty.resize(nn + 1);
        for (int j = 0; j < nn; ++j) {
            dx[j] = nei_dx[3 * (o + j)]; dy[j] = nei_dx[3 * (o + j) + 1]; dz[j] = nei_dx[3 * (o + j) + 2];
            ty[j] = type[nei_j[o + j]];
        }
        int code = jse_nnap_calFp(dx.data(), dy.data(), dz.data(), ty.data(), nn, type[i], hp, fpp, fp + (size_t)i * fp_stride);
        if (code) return code;
    }
    return 0;
}

// Parameter gradients of a force-and-energy loss through the reference's per-atom
// training pair jse_nnap_forwardEnergyForce / jse_nnap_backwardEnergyForce
// (nnap_interface.cpp:142-232), driven like the force branch of TrainerNNAP
// (TrainerNNAP.java:1006-1175):
//   the loss is L = sum_i bE_i E_i + sum_i bF_i . F_i + sum_ab bW_ab W_ab (W the total virial,
//   components xx, yy, zz, xy, xz, yz, yx, zx, zy);
//   each pair (i, j) with displacement dx = x_j - x_i receives the upstream gradient of
//   its g_ij = -dE_i/d(dx):  bF_j - bF_i + (sum_a bW_ax dx_a, sum_a bW_ay dx_a, sum_a bW_az dx_a)
//   (TrainerNNAP.java:1142-1160 with the stress terms written for all nine components).
// bgrad_e (n), bgrad_f (3n) and bgrad_w (9) may each be NULL (zero).  grad_fp and grad_nn
// receive the concatenation over species of the reference's C-level parameter gradients
// (fp_size[t] and nn_size[t] doubles per species); per-thread gradient arrays are summed
// in thread order as NNAP.backwardParameter sums them (NNAP.java:659-668).
int ref_train_grad(int T, double** hp, double** fpp, double** nnp, double** normp, int n, const int* type,
                   const long* nei_off, const int* nei_j, const double* nei_dx, long cache_per_nei, long cache_const,
                   int nthreads, const double* bgrad_e, const double* bgrad_f, const double* bgrad_w,
                   const long* fp_size, const long* nn_size, double* grad_fp, double* grad_nn) {
    if (nthreads < 1) nthreads = 1;
    long fp_tot = 0, nn_tot = 0;
    for (int t = 0; t < T; ++t) { fp_tot += fp_size[t]; nn_tot += nn_size[t]; }
    struct Acc {
        std::vector<double> gfp, gnn;
        std::vector<double*> pfp, pnn;
        int status = 0;
    };
    std::vector<Acc> acc(nthreads);
    for (auto& A : acc) {
        A.gfp.assign(fp_tot + 1, 0.0);
        A.gnn.assign(nn_tot + 1, 0.0);
        long of = 0, on = 0;
        for (int t = 0; t < T; ++t) {
            A.pfp.push_back(A.gfp.data() + of);
            A.pnn.push_back(A.gnn.data() + on);
            of += fp_size[t];
            on += nn_size[t];
        }
    }
    auto work = [&](int tid) {
        Acc& A = acc[tid];
        std::vector<double> dx, dy, dz, gx, gy, gz, bx, by, bz, c0, c1, c2, c3, c4;
        std::vector<int> ty;
        for (int i = tid; i < n; i += nthreads) {
            const long o = nei_off[i];
            const int nn = (int)(nei_off[i + 1] - o);
            const size_t csz = (size_t)cache_per_nei * (nn + 1) + cache_const;
            dx.resize(nn + 1); dy.resize(nn + 1); dz.resize(nn + 1); ty.resize(nn + 1);
            gx.assign(nn + 1, 0.0); gy.assign(nn + 1, 0.0); gz.assign(nn + 1, 0.0);
            bx.assign(nn + 1, 0.0); by.assign(nn + 1, 0.0); bz.assign(nn + 1, 0.0);
            c0.assign(csz, 0.0); c1.assign(csz, 0.0); c2.assign(csz, 0.0); c3.assign(csz, 0.0); c4.assign(csz, 0.0);
            for (int j = 0; j < nn; ++j) {
                dx[j] = nei_dx[3 * (o + j)];
                dy[j] = nei_dx[3 * (o + j) + 1];
                dz[j] = nei_dx[3 * (o + j) + 2];
                ty[j] = type[nei_j[o + j]];
            }
            const int ct = type[i];
            double e = 0.0;
            int code = jse_nnap_forwardEnergyForce(dx.data(), dy.data(), dz.data(), ty.data(), nn, ct, hp, fpp, nnp,
                                                   normp[ct - 1], &e, gx.data(), gy.data(), gz.data(), c0.data(),
                                                   c1.data(), c2.data(), c3.data());
            if (code) { A.status = code; return; }
            for (int j = 0; j < nn; ++j) {
                const int jj = nei_j[o + j];
                double sx = 0.0, sy = 0.0, sz = 0.0;
                if (bgrad_f) {
                    sx += bgrad_f[3 * (size_t)jj] - bgrad_f[3 * (size_t)i];
                    sy += bgrad_f[3 * (size_t)jj + 1] - bgrad_f[3 * (size_t)i + 1];
                    sz += bgrad_f[3 * (size_t)jj + 2] - bgrad_f[3 * (size_t)i + 2];
                }
                if (bgrad_w) {
                    const double* w = bgrad_w;
                    sx += w[0] * dx[j] + w[6] * dy[j] + w[7] * dz[j];
                    sy += w[3] * dx[j] + w[1] * dy[j] + w[8] * dz[j];
                    sz += w[4] * dx[j] + w[5] * dy[j] + w[2] * dz[j];
                }
                bx[j] = sx; by[j] = sy; bz[j] = sz;
            }
            const double be = bgrad_e ? bgrad_e[i] : 0.0;
            code = jse_nnap_backwardEnergyForce(dx.data(), dy.data(), dz.data(), ty.data(), nn, ct, hp, fpp, nnp,
                                                normp[ct - 1], be, bx.data(), by.data(), bz.data(), A.pfp.data(),
                                                A.pnn.data(), c0.data(), c1.data(), c2.data(), c3.data(), c4.data());
            if (code) { A.status = code; return; }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& t : th) t.join();
    for (auto& A : acc) if (A.status) return A.status;
    if (grad_fp) {
        std::memset(grad_fp, 0, sizeof(double) * fp_tot);
        for (auto& A : acc) for (long k = 0; k < fp_tot; ++k) grad_fp[k] += A.gfp[k];
    }
    if (grad_nn) {
        std::memset(grad_nn, 0, sizeof(double) * nn_tot);
        for (auto& A : acc) for (long k = 0; k < nn_tot; ++k) grad_nn[k] += A.gnn[k];
    }
    return 0;
}

}  // extern "C"
