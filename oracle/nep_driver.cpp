// Driver around the reference's own per-atom NEP arithmetic.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/nep_ref.py together with the reference's
// nep_interface.cpp after oracle/nepgen.py has expanded it for one model into
// oracle/_ref/<shape>/src (build output, never committed).  It restates the per-atom loop
// of NEP.calEnergyForceVirial (NEP.java:160-212): jse_nep_calEnergyForce
// (nep_interface.cpp:106-188) per atom over the caller's neighbour list (threads over
// atoms like ParforThreadPool, each with private accumulators), pair terms
// scattered as F_i -= f_ij, F_j += f_ij and the per-atom virial dx (x) f_ij assigned to
// the neighbour (the accumulators of IPairPotential.java:919-1006).  Species are 0-based
// here, as the reference's arithmetic expects.
#include <cstring>
#include <thread>
#include <vector>

extern "C" int jse_nep_calEnergyForce(const double* nl_dx, const double* nl_dy, const double* nl_dz,
                                      const int* nl_type, int num_neigh, int ctype, const int* atomic_numbers,
                                      const double* q_scaler, const double** ann_w0, const double** ann_b0,
                                      const double** ann_w1, const double* ann_b1, const double* ann_c,
                                      const double* zbl_para, const double* gn_radial, const double* gn_angular,
                                      const double* gnp_radial, const double* gnp_angular, double* eng, double* nl_fx,
                                      double* nl_fy, double* nl_fz, double* fp, double* sum_fxyz);

namespace {

struct Args {
    const int* atomic_numbers;
    const double* zbl_para;
    const double* q_scaler;
    const double** w0;
    const double** b0;
    const double** w1;
    const double* b1;
    const double* c;
    int dim, sum_size, n_eval;
    const int* type;
    const long* nei_off;
    const int* nei_j;
    const double* nei_dx;
};

// Atoms tid, tid + nthreads, ... of [0, n_eval) (static round-robin, ParforThreadPool
// style); every thread scatters into its own full-size accumulators.
int run_atoms(const Args& a, int tid, int nthreads, double* e_atom, double* force, double* virial) {
    std::vector<double> dx, dy, dz, fx, fy, fz, fp(a.dim + 8), sf(a.sum_size + 8);
    std::vector<int> ty;
    for (int i = tid; i < a.n_eval; i += nthreads) {
        const long o = a.nei_off[i];
        const int nn = (int)(a.nei_off[i + 1] - o);
        dx.resize(nn + 1); dy.resize(nn + 1); dz.resize(nn + 1);
        fx.resize(nn + 1); fy.resize(nn + 1); fz.resize(nn + 1); ty.resize(nn + 1);
        for (int j = 0; j < nn; ++j) {
            dx[j] = a.nei_dx[3 * (o + j)];
            dy[j] = a.nei_dx[3 * (o + j) + 1];
            dz[j] = a.nei_dx[3 * (o + j) + 2];
            ty[j] = a.type[a.nei_j[o + j]];
        }
        double e = 0.0;
        const int code = jse_nep_calEnergyForce(dx.data(), dy.data(), dz.data(), ty.data(), nn, a.type[i],
                                                a.atomic_numbers, a.q_scaler, a.w0, a.b0, a.w1, a.b1, a.c, a.zbl_para,
                                                nullptr, nullptr, nullptr, nullptr, &e, fx.data(), fy.data(),
                                                fz.data(), fp.data(), sf.data());
        if (code) return code;
        e_atom[i] += e;
        for (int j = 0; j < nn; ++j) {
            const int jj = a.nei_j[o + j];
            force[3 * i] -= fx[j]; force[3 * i + 1] -= fy[j]; force[3 * i + 2] -= fz[j];
            force[3 * jj] += fx[j]; force[3 * jj + 1] += fy[j]; force[3 * jj + 2] += fz[j];
            double* v = virial + 9 * (size_t)jj;
            v[0] += dx[j] * fx[j]; v[1] += dy[j] * fy[j]; v[2] += dz[j] * fz[j];
            v[3] += dx[j] * fy[j]; v[4] += dx[j] * fz[j]; v[5] += dy[j] * fz[j];
            v[6] += dy[j] * fx[j]; v[7] += dz[j] * fx[j]; v[8] += dz[j] * fy[j];
        }
    }
    return 0;
}

}  // namespace

// Evaluates atoms [0, n_eval) over the caller's full neighbour rows with nthreads threads;
// outputs cover all n atoms (a neighbour's force and virial shares included).
extern "C" int nep_ref_compute(int T, const int* atomic_numbers, const double* zbl_para, const double* q_scaler,
                               const double** w0,
                               const double** b0, const double** w1, const double* b1, const double* c, int dim,
                               int sum_size, int n, int n_eval, int nthreads, const int* type, const long* nei_off,
                               const int* nei_j, const double* nei_dx, double* e_atom, double* force,
                               double* virial) {
    (void)T;
    if (nthreads < 1) nthreads = 1;
    const Args a{atomic_numbers, zbl_para, q_scaler, w0, b0, w1, b1, c, dim, sum_size, n_eval, type, nei_off, nei_j,
                 nei_dx};
    std::vector<std::vector<double>> acc(nthreads);
    std::vector<int> codes(nthreads, 0);
    for (auto& v : acc) v.assign((size_t)13 * n, 0.0);
    auto work = [&](int t) {
        double* b = acc[t].data();
        codes[t] = run_atoms(a, t, nthreads, b, b + n, b + 4 * (size_t)n);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
    for (int t = 0; t < nthreads; ++t)
        if (codes[t]) return codes[t];
    // fixed-order reduction over threads: results do not depend on scheduling
    std::memset(e_atom, 0, sizeof(double) * n);
    std::memset(force, 0, sizeof(double) * 3 * n);
    std::memset(virial, 0, sizeof(double) * 9 * n);
    for (int t = 0; t < nthreads; ++t) {
        const double* b = acc[t].data();
        for (size_t q = 0; q < (size_t)n; ++q) e_atom[q] += b[q];
        for (size_t q = 0; q < (size_t)3 * n; ++q) force[q] += b[n + q];
        for (size_t q = 0; q < (size_t)9 * n; ++q) virial[q] += b[4 * (size_t)n + q];
    }
    return 0;
}
