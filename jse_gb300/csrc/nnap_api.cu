// C ABI of the NNAP GB300 evaluator: handle lifetime, device buffers and the
// evaluation pipeline (see include/nnap_gb300.h for the contract).
//
// Pipeline of one evaluation over a batch of structures (a single structure is a
// batch of one):
//   k_wrap_bin -> k_scan_excl -> k_fill_cells -> k_sort_cells
//   -> k_renumber (energy/force evaluations: atoms in cell order from here on; descriptor-
//      only calls take k_cell_order and keep atom order) -> k_neighbors
//   -> species sort (k_type_hist, k_type_offsets, k_type_scatter) -> k_mirror
//   -> descriptor forward (per run of species sharing a basis shape, per sub-basis)
//   -> network per species -> descriptor backward -> k_gather -> k_reduce_chunks
//   -> k_reduce_structs, then one host synchronisation (neighbour capacity, error bits).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "api_internal.hpp"
#include "zbl.cuh"
#include "pdl.cuh"

using namespace nnapgb;

namespace nnapgb {

int fail(nnap_handle* h, int status, const std::string& m) {
    if (h) h->err = m;
    return status;
}

// ------------------------------------------------------------------ model upload
void upload_model(nnap_handle* h) {
    const Model& m = h->model;
    const int T = m.ntypes();
    if (T > kMaxTypes) throw ApiFail(NNAP_ERR_UNSUPPORTED, "more than 16 species");
    int dmax = 0;
    for (auto& sp : m.sp) dmax = std::max(dmax, sp.D);
    h->fp_stride = (dmax + 3) & ~3;
    // runs of consecutive species with identical sub-basis shapes
    for (int t = 0; t < T;) {
        Run r;
        r.t0 = t;
        auto shape = [&m](const SubBasis& b) {
            return SubShape{b.kind, b.lmax, b.np, b.nmax + 1, b.rcut, b.nl2, b.l3max, b.l4max, (int)b.inv.size(),
                            m.radial_fn ? kRbNEP : kRbNNAP};
        };
        for (auto& b : m.sp[t].subs) {
            r.subs.push_back(shape(b));
            r.fp_off.push_back(b.fp_off);
        }
        int u = t + 1;
        while (u < T) {
            const auto& su = m.sp[u].subs;
            bool same = su.size() == r.subs.size() && m.sp[u].D == m.sp[t].D;
            for (size_t k = 0; same && k < su.size(); ++k)
                same = r.subs[k] == shape(su[k]);
            if (!same) break;
            ++u;
        }
        r.t1 = u;
        for (size_t k = 0; k < r.subs.size(); ++k) {
            const SubShape& s = r.subs[k];
            if (!desc_supported(s.kind, s.basis, s.lmax, s.np, s.n1)) {
                char buf[160];
                std::snprintf(buf, sizeof buf, "descriptor shape beyond shared memory: %s kind=%d lmax=%d np=%d nmax=%d",
                              s.basis == kRbNEP ? "NEP" : "NNAP", s.kind, s.lmax, s.np, s.n1 - 1);
                throw ApiFail(NNAP_ERR_UNSUPPORTED, buf);
            }
            std::vector<float> W((size_t)T * T * s.np * s.n1, 0.f);
            for (int tc = r.t0; tc < r.t1; ++tc) {
                const std::vector<double>& src = m.sp[tc].subs[k].W;  // [tn][np][n1]
                for (size_t q = 0; q < src.size(); ++q) W[(size_t)tc * T * s.np * s.n1 + q] = (float)src[q];
            }
            r.W.emplace_back();
            r.W.back().ensure(W.size());
            CK(cudaMemcpy(r.W.back().p, W.data(), W.size() * sizeof(float), cudaMemcpyHostToDevice));
            // sparse columns for the radial-space backward
            std::vector<int> zp((size_t)T * T * s.n1 * kNz, -1);
            std::vector<float> zw(zp.size(), 0.f);
            bool sparse = s.kind == KIND_SPHERICAL && s.n1 < s.np && s.basis == kRbNNAP;
            for (int tc = r.t0; tc < r.t1 && sparse; ++tc)
                for (int tn = 0; tn < T && sparse; ++tn)
                    for (int n = 0; n < s.n1 && sparse; ++n) {
                        int z = 0;
                        for (int p = 0; p < s.np; ++p) {
                            const float v = W[(((size_t)tc * T + tn) * s.np + p) * s.n1 + n];
                            if (v == 0.f) continue;
                            if (z == kNz) { sparse = false; break; }
                            const size_t q = (((size_t)tc * T + tn) * s.n1 + n) * kNz + z++;
                            zp[q] = p;
                            zw[q] = v;
                        }
                    }
            // invariant-column terms (the same for every species of the run)
            r.inv_idx.emplace_back();
            r.inv_coef.emplace_back();
            r.inv_start.emplace_back();
            if (s.ninv) {
                const auto& cols = m.sp[r.t0].subs[k].inv;
                std::vector<int4> ti;
                std::vector<float> tc;
                std::vector<int> cs{0};
                for (auto& col : cols) {
                    for (auto& q : col) {
                        ti.push_back(make_int4(q.idx[0], q.idx[1], q.idx[2], q.idx[3]));
                        tc.push_back((float)q.coeff);
                    }
                    cs.push_back((int)ti.size());
                }
                r.inv_idx.back().ensure(ti.size());
                r.inv_coef.back().ensure(tc.size());
                r.inv_start.back().ensure(cs.size());
                CK(cudaMemcpy(r.inv_idx.back().p, ti.data(), ti.size() * sizeof(int4), cudaMemcpyHostToDevice));
                CK(cudaMemcpy(r.inv_coef.back().p, tc.data(), tc.size() * sizeof(float), cudaMemcpyHostToDevice));
                CK(cudaMemcpy(r.inv_start.back().p, cs.data(), cs.size() * sizeof(int), cudaMemcpyHostToDevice));
            }
            // per-row scales for the radial-space forward
            {
                std::vector<float> al((size_t)T * kFwdTypes * s.np, 0.f);
                bool diag = s.kind == KIND_SPHERICAL && s.n1 < s.np && T <= kFwdTypes && s.basis == kRbNNAP;
                for (int tc = r.t0; tc < r.t1 && diag; ++tc)
                    for (int tn = 0; tn < T && diag; ++tn)
                        for (int p = 0; p < s.np && diag; ++p)
                            for (int nn = 0; nn < s.n1; ++nn) {
                                const float v = W[(((size_t)tc * T + tn) * s.np + p) * s.n1 + nn];
                                if (nn == p % s.n1) al[((size_t)tc * kFwdTypes + tn) * s.np + p] = v;
                                else if (v != 0.f) { diag = false; break; }
                            }
                r.falpha.emplace_back();
                bool tc = diag;
                if (diag) {
                    r.falpha.back().ensure(al.size());
                    CK(cudaMemcpy(r.falpha.back().p, al.data(), al.size() * sizeof(float), cudaMemcpyHostToDevice));
                    for (float v : al) tc = tc && std::fabs(v) <= kTcAlphaMax;
                }
                r.tc_fwd.push_back(tc);
            }
            // a spherical sub-basis after the first, on the channel-space kernels, with a cutoff
            // well inside the neighbour cutoff scans compact rows (one such cutoff per model)
            {
                const bool pspace = !sparse && !r.falpha.back().p;
                bool use = s.kind == KIND_SPHERICAL && k > 0 && pspace && s.rcut <= 0.85 * m.rcut_max;
                if (use && h->sub_rc == 0.0) h->sub_rc = s.rcut;
                r.use_sub.push_back(use && s.rcut == h->sub_rc);
            }
            // NEP type-wise cutoffs of the run's species pairs
            r.prc.emplace_back();
            if (!m.sp[r.t0].subs[k].pair_rc.empty()) {
                std::vector<float2> q((size_t)T * T, make_float2((float)s.rcut, (float)(1.0 / s.rcut)));
                for (int tc = r.t0; tc < r.t1; ++tc)
                    for (int tn = 0; tn < T; ++tn) {
                        const double rc = m.sp[tc].subs[k].pair_rc[tn];
                        q[(size_t)tc * T + tn] = make_float2((float)rc, (float)(1.0 / rc));
                    }
                r.prc.back().ensure(q.size());
                CK(cudaMemcpy(r.prc.back().p, q.data(), q.size() * sizeof(float2), cudaMemcpyHostToDevice));
            }
            r.nzp.emplace_back();
            r.nzw.emplace_back();
            if (sparse) {
                r.nzp.back().ensure(zp.size());
                r.nzw.back().ensure(zw.size());
                CK(cudaMemcpy(r.nzp.back().p, zp.data(), zp.size() * sizeof(int), cudaMemcpyHostToDevice));
                CK(cudaMemcpy(r.nzw.back().p, zw.data(), zw.size() * sizeof(float), cudaMemcpyHostToDevice));
            }
        }
        h->runs.push_back(std::move(r));
        t = u;
    }
    // NEP's ZBL term
    if (m.zbl.on) {
        std::vector<double> z(T), zp(T), par(m.zbl.para.begin(), m.zbl.para.end());
        for (int t = 0; t < T; ++t) {
            z[t] = (double)m.zbl.z[t];
            zp[t] = std::pow((double)m.zbl.z[t], 0.23);
        }
        h->zbl_z.ensure(T);
        h->zbl_zp.ensure(T);
        h->zbl_para.ensure(std::max<size_t>(par.size(), 1));
        CK(cudaMemcpy(h->zbl_z.p, z.data(), sizeof(double) * T, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->zbl_zp.p, zp.data(), sizeof(double) * T, cudaMemcpyHostToDevice));
        if (!par.empty())
            CK(cudaMemcpy(h->zbl_para.p, par.data(), sizeof(double) * par.size(), cudaMemcpyHostToDevice));
        if (!m.zbl.pair_rc.empty()) {
            const std::vector<double>& rcp = m.zbl.pair_rc;
            h->zbl_rc.ensure(rcp.size());
            CK(cudaMemcpy(h->zbl_rc.p, rcp.data(), sizeof(double) * rcp.size(), cudaMemcpyHostToDevice));
        }
    }
    // networks
    h->nets.resize(T);
    for (int t = 0; t < T; ++t) {
        const Species& sp = m.sp[t];
        NetDev& nd = h->nets[t];
        if (sp.hidden.size() > (size_t)kNetMaxLayers) throw ApiFail(NNAP_ERR_UNSUPPORTED, "more than 16 hidden layers");
        nd.D = sp.D;
        nd.nlayer = (int)sp.hidden.size();
        for (int l = 0; l < nd.nlayer; ++l) nd.H[l] = sp.hidden[l];
        if (!net_fp32_fits(nd.D, nd.nlayer, nd.H))
            throw ApiFail(NNAP_ERR_UNSUPPORTED, "network too wide for shared memory ((2 + layers) x widest layer "
                                                "above 7264)");
        nd.mu_e = sp.mu_e;
        nd.sigma_e = sp.sigma_e;
        nd.act = m.act ? kActTanh : kActSiLU;
        std::vector<float> w;
        for (int i = 0; i < sp.D; ++i) w.push_back((float)sp.mu[i]);
        for (int i = 0; i < sp.D; ++i) w.push_back((float)(1.0 / sp.sigma[i]));
        int in = sp.D;
        for (int l = 0; l < nd.nlayer; ++l) {
            const int H = sp.hidden[l];
            for (int i = 0; i < in; ++i)
                for (int o = 0; o < H; ++o) w.push_back((float)sp.Wh[l][(size_t)o * in + i]);
            for (size_t q = 0; q < sp.Wh[l].size(); ++q) w.push_back((float)sp.Wh[l][q]);
            for (int o = 0; o < H; ++o) w.push_back((float)sp.bh[l][o]);
            in = H;
        }
        for (int o = 0; o < in; ++o) w.push_back((float)sp.wo[o]);
        w.push_back((float)sp.bo);
        nd.w32.ensure(w.size());
        CK(cudaMemcpy(nd.w32.p, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
        if (h->net_tc) {
            // a network outside the tensor-core kernel's limits (widths above 256, more than
            // 8 layers, operands beyond shared memory or TMEM) runs the FP32 kernel
            std::string why;
            if (!net_tc_prepare(sp, nd.tc, why)) {
                net_tc_release(nd.tc);
                h->net_notes += sp.symbol + ": " + why + "; ";
            }
        }
    }
}

// ------------------------------------------------------------------ structure setup (host)
void cross3(const double* u, const double* v, double* r) {
    r[0] = u[1] * v[2] - v[1] * u[2];
    r[1] = u[2] * v[0] - v[2] * u[0];
    r[2] = u[0] * v[1] - v[0] * u[1];
}

// Smallest eigenvalue of G = H H^T for the box matrix H (rows a, b, c): the squared
// smallest singular value, so |u H| >= sqrt of it times |u| for any direct-coordinate
// vector u.  The closed form of a symmetric 3 x 3 matrix's eigenvalues (trace, the
// deviatoric part's norm and determinant, one arccosine), less a margin of 1e-12 of the
// largest eigenvalue for its rounding: the result stays a lower bound, which is all the
// cell pruning needs.
double smallest_sq_singular(const StructDev& s) {
    const double* r[3] = {s.a, s.b, s.c};
    double G[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) G[i][j] = r[i][0] * r[j][0] + r[i][1] * r[j][1] + r[i][2] * r[j][2];
    const double off = G[0][1] * G[0][1] + G[0][2] * G[0][2] + G[1][2] * G[1][2];
    if (off == 0.0) return std::max(0.0, std::min(G[0][0], std::min(G[1][1], G[2][2])));
    const double q = (G[0][0] + G[1][1] + G[2][2]) / 3.0;
    const double d0 = G[0][0] - q, d1 = G[1][1] - q, d2 = G[2][2] - q;
    const double p = std::sqrt((d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * off) / 6.0);
    if (!(p > 0.0)) return std::max(0.0, q);
    // B = (G - q I) / p; r = det(B) / 2 in [-1, 1]
    const double b00 = d0 / p, b11 = d1 / p, b22 = d2 / p, b01 = G[0][1] / p, b02 = G[0][2] / p, b12 = G[1][2] / p;
    const double det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
    const double rr = std::min(1.0, std::max(-1.0, 0.5 * det));
    const double phi = std::acos(rr) / 3.0;
    const double lmax = q + 2.0 * p * std::cos(phi);
    const double lmin = q + 2.0 * p * std::cos(phi + 2.0943951023931957);  // + 2 pi / 3
    return std::max(0.0, lmin - 1e-12 * std::fabs(lmax));
}

// Float bound for the candidate screen: rc^2 plus the worst rounding of the FP32
// difference (x_j + shift) - x_i for image shifts up to Rm + 2 box lengths.
float screen_bound(const StructDev& s, double rc, int Rm) {
    double ext = 0.0;
    for (int d = 0; d < 3; ++d) ext += std::fabs(s.a[d]) + std::fabs(s.b[d]) + std::fabs(s.c[d]);
    const double eps = 16.0 * (ext * (2 + Rm)) * std::ldexp(1.0, -24);
    const double margin = 2.0 * std::sqrt(3.0) * rc * eps + 3.0 * eps * eps + 16.0 * rc * rc * std::ldexp(1.0, -24);
    return (float)(rc * rc + margin) * (1.0f + 1e-6f);
}

constexpr double kHalfCellAtoms = 20.0;  // atoms per rc^3 from which cells are rc/2 wide

int struct_geometry(int kind, const double* box, double rc, int n, StructDev& s, const char** why) {
    std::memset(&s, 0, sizeof s);
    const char* dummy = nullptr;
    const char*& msg = why ? *why : dummy;
    if (kind < 0 || kind > 2) {
        msg = "box_kind must be 0, 1 or 2";
        return NNAP_ERR_ARG;
    }
    if (!box) {
        msg = "box is NULL";
        return NNAP_ERR_ARG;
    }
    if (!(rc > 0.0) || !std::isfinite(rc)) {
        msg = "the cutoff must be positive and finite";
        return NNAP_ERR_ARG;
    }
    s.kind = kind;
    for (int d = 0; d < 3; ++d) { s.a[d] = box[d]; s.b[d] = box[3 + d]; s.c[d] = box[6 + d]; }
    if (kind == 0) {
        s.a[1] = s.a[2] = s.b[0] = s.b[2] = s.c[0] = s.c[1] = 0.0;
    } else if (kind == 1) {
        s.a[1] = s.a[2] = s.b[2] = 0.0;
    }
    cross3(s.b, s.c, s.bc);
    cross3(s.c, s.a, s.ca);
    cross3(s.a, s.b, s.ab);
    s.vol = (s.a[1] * s.b[2] - s.b[1] * s.a[2]) * s.c[0] + (s.a[2] * s.b[0] - s.b[2] * s.a[0]) * s.c[1] +
            (s.a[0] * s.b[1] - s.b[0] * s.a[1]) * s.c[2];
    if (!(s.vol > 0.0) || !std::isfinite(s.vol)) {
        msg = "box must be right-handed with positive volume";
        return NNAP_ERR_ARG;
    }
    auto nrm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    const double h[3] = {s.vol / nrm(s.bc), s.vol / nrm(s.ca), s.vol / nrm(s.ab)};
    // cells at least rc wide, or rc/2 wide where an rc^3 volume holds many atoms: the
    // 5^3-cell stencil, trimmed by each cell's distance bound, visits about half the
    // candidates of the 3^3 stencil
    const int div = (double)n / s.vol * rc * rc * rc >= kHalfCellAtoms ? 2 : 1;
    for (int d = 0; d < 3; ++d) {
        if (!std::isfinite(h[d]) || !(h[d] > 0.0)) {
            msg = "box must be right-handed with positive volume";
            return NNAP_ERR_ARG;
        }
        // bounded in double before any conversion to int
        const double ncd = std::min(1024.0, std::max(1.0, std::floor(h[d] * div / rc)));
        s.nc[d] = (int)ncd;
        const double Rd = std::floor(rc * ncd / h[d] + 1e-6) + 1.0;
        if (!(Rd <= 64.0)) {
            msg = "box too thin for the cutoff";
            return NNAP_ERR_ARG;
        }
        s.R[d] = (int)Rd;
    }
    if ((2 * s.R[0] + 1) * (2 * s.R[1] + 1) * (2 * s.R[2] + 1) > 65535) {
        msg = "box too thin for the cutoff";
        return NNAP_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d) {
        s.fa[d] = (float)s.a[d]; s.fb[d] = (float)s.b[d]; s.fc[d] = (float)s.c[d];
        s.la[d] = (float)(s.a[d] - (double)s.fa[d]);
        s.lb[d] = (float)(s.b[d] - (double)s.fb[d]);
        s.lc[d] = (float)(s.c[d] - (double)s.fc[d]);
    }
    s.rc2 = rc * rc;
    s.rc2_hi = screen_bound(s, rc, std::max(s.R[0], std::max(s.R[1], s.R[2])));
    for (int d = 0; d < 3; ++d) {
        s.iv[0][d] = (float)(s.bc[d] / s.vol);
        s.iv[1][d] = (float)(s.ca[d] / s.vol);
        s.iv[2][d] = (float)(s.ab[d] / s.vol);
    }
    s.smin2 = (float)(smallest_sq_singular(s) * (1.0 - 1e-5));
    s.n = n;
    return NNAP_OK;
}

StructDev make_struct(int kind, const double* box, double rc, int a0, int n, int c0) {
    StructDev s;
    const char* why = "";
    const int st = struct_geometry(kind, box, rc, n, s, &why);
    if (st != NNAP_OK) throw ApiFail(st, why);
    s.a0 = a0;
    s.c0 = c0;
    return s;
}

// ------------------------------------------------------------------ pipeline
// The batch layout of a call.  The last one is kept with the counts, kinds and boxes it was
// made from, and returned again while they are unchanged (repeated evaluations of the same
// structures skip the per-structure geometry).
const Batch& plan_batch(nnap_handle* h, int nstruct, const int* natoms, const int* kinds, const double* boxes) {
    if (h->plan_valid && h->plan.nstruct == nstruct && nstruct > 0 &&
        std::memcmp(h->plan_nat.data(), natoms, sizeof(int) * nstruct) == 0 &&
        std::memcmp(h->plan_kind.data(), kinds, sizeof(int) * nstruct) == 0 &&
        std::memcmp(h->plan_box.data(), boxes, sizeof(double) * 9 * nstruct) == 0)
        return h->plan;
    h->plan_valid = false;
    Batch B;
    B.nstruct = nstruct;
    const double rc = h->model.rcut_max;
    int a0 = 0, c0 = 0;
    B.sc.push_back(0);
    for (int s = 0; s < nstruct; ++s) {
        if (natoms[s] < 0) throw ApiFail(NNAP_ERR_ARG, "negative atom count");
        StructDev d = make_struct(kinds[s], boxes + 9 * s, rc, a0, natoms[s], c0);
        B.sd.push_back(d);
        for (int b = 0; b < natoms[s]; b += kRedChunk) {
            B.cb.push_back(a0 + b);
            B.ce.push_back(a0 + std::min(natoms[s], b + kRedChunk));
        }
        B.sc.push_back((int)B.cb.size());
        c0 += d.nc[0] * d.nc[1] * d.nc[2];
        a0 += natoms[s];
    }
    B.natoms = a0;
    B.ncells = c0;
    h->plan = std::move(B);
    h->plan_nat.assign(natoms, natoms + nstruct);
    h->plan_kind.assign(kinds, kinds + nstruct);
    h->plan_box.assign(boxes, boxes + 9 * (size_t)nstruct);
    h->plan_valid = true;
    return h->plan;
}

void grow_pairs(nnap_handle* h, int n, int M) {
    h->M = M;
    const size_t np = (size_t)std::max(n, 1) * M;
    h->pkey.ensure(np);
    h->pdx.ensure(np);
    h->pg.ensure(np);
    h->prev.ensure(np);
    h->pgrp.ensure(np);
    if (h->model.zbl.on) h->pdxlo.ensure(np);
    if (h->sub_rc > 0.0) {
        h->sdx.ensure(np);
        h->spos.ensure(np);
        h->scount.ensure(std::max(n, 1));
    }
}

PairBufs pair_bufs(nnap_handle* h) {
    PairBufs P;
    P.M = h->M;
    P.key = h->pkey.p;
    P.dx = h->pdx.p;
    P.dxlo = h->model.zbl.on ? h->pdxlo.p : nullptr;
    P.rev = h->prev.p;
    P.g = h->pg.p;
    P.grp = h->pgrp.p;
    P.count = h->pcount.p;
    P.gstart = h->GS ? h->gstart.p : nullptr;
    P.GS = h->GS;
    return P;
}

int initial_capacity(const Batch& B, double rc) {
    double dens = 0.0;
    for (auto& s : B.sd)
        if (s.n > 0) dens = std::max(dens, s.n / s.vol);
    const double mean = 4.18879020478639 * rc * rc * rc * dens;
    int M = (int)std::ceil(1.3 * mean + 24.0);
    return std::max(32, (M + 7) & ~7);
}

// A-arena rows: every (run, spherical sub-basis) owns n rows of P*K floats, indexed by
// the slot offset inside its run, so no host knowledge of species counts is needed.
size_t a_arena_size(nnap_handle* h, int n) {
    size_t tot = 0;
    for (auto& r : h->runs)
        for (auto& s : r.subs)
            if (s.kind == KIND_SPHERICAL) tot += (size_t)n * s.np * (s.lmax + 1) * (s.lmax + 1);
    return tot;
}

void ensure_work(nnap_handle* h, int n, int nstruct, int ncells, int nchunks) {
    const int T = h->model.ntypes();
    const int n1 = std::max(n, 1);
    h->sdev.ensure(std::max(nstruct, 1));
    h->sid.ensure(n1);
    h->xw.ensure(3 * (size_t)n1);
    h->xf.ensure(n1);
    h->xlo.ensure(n1);
    h->xfc.ensure(n1);
    h->xloc.ensure(n1);
    h->xw2.ensure(3 * (size_t)n1);
    h->e_out.ensure(n1);
    h->cell_of2.ensure(n1);
    h->type2.ensure(n1);
    h->orig.ensure(n1);
    h->cell_of.ensure(n1);
    h->cell_count.ensure(std::max(ncells, 1));
    h->cell_fill.ensure(std::max(ncells, 1));
    h->cell_start.ensure(ncells + 1);
    h->cell_atoms.ensure(n1);
    h->pcount.ensure(n1);
    h->perm.ensure(n1);
    const int nb = (n + kSortBlock - 1) / kSortBlock;
    h->block_counts.ensure((size_t)std::max(nb, 1) * T);
    h->type_start.ensure(T + 1);
    h->status.ensure(2);
    grow_pairs(h, n, h->M);
    h->fp.ensure((size_t)n1 * h->fp_stride);
    h->gfp.ensure((size_t)n1 * h->fp_stride);
    h->A.ensure(std::max<size_t>(a_arena_size(h, n), 1));
    bool inv = false;
    for (auto& r : h->runs)
        for (auto& sh : r.subs) inv = inv || sh.ninv > 0;
    if (inv) h->Gx.ensure(std::max<size_t>(a_arena_size(h, n), 1));
    h->e_atom.ensure(n1);
    h->forces.ensure(3 * (size_t)n1);
    h->virials.ensure(9 * (size_t)n1);
    h->chunk_b.ensure(std::max(nchunks, 1));
    h->chunk_e.ensure(std::max(nchunks, 1));
    h->struct_chunks.ensure(nstruct + 1);
    h->partial.ensure(10 * (size_t)std::max(nchunks, 1));
    h->energy.ensure(std::max(nstruct, 1));
    h->virial.ensure(9 * (size_t)std::max(nstruct, 1));
}

// Size every buffer for the batch and upload the layout arrays that depend only on the
// atom counts (structure of each atom, reduction chunks).  Runs outside graph capture.
void prepare_layout(nnap_handle* h, const Batch& B) {
    const int n = B.natoms;
    const int nchunks = (int)B.cb.size();
    if (h->M == 0) h->M = initial_capacity(B, h->model.rcut_max);
    ensure_work(h, n, B.nstruct, B.ncells, nchunks);
    // group starts of the neighbour rows, for the mirror search (kept up to 127 offset groups)
    int gs = 0;
    for (auto& d : B.sd) gs = std::max(gs, (2 * d.R[0] + 1) * (2 * d.R[1] + 1) * (2 * d.R[2] + 1) + 1);
    h->GS = gs <= 128 ? gs : 0;
    if (h->GS) h->gstart.ensure((size_t)std::max(n, 1) * h->GS);
    if (h->h_sdev_cap < (size_t)B.nstruct) {
        if (h->h_sdev) cudaFreeHost(h->h_sdev);
        h->h_sdev = nullptr;
        CK(cudaMallocHost(&h->h_sdev, sizeof(StructDev) * B.nstruct));
        h->h_sdev_cap = B.nstruct;
    }
    cudaStream_t st = h->stream;
    if (n) {  // structure of every atom: built only when the layout changes
        std::vector<int> sid((size_t)n);
        for (int q = 0; q < B.nstruct; ++q) std::fill(sid.begin() + B.sd[q].a0, sid.begin() + B.sd[q].a0 + B.sd[q].n, q);
        CK(cudaMemcpyAsync(h->sid.p, sid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
    }
    if (nchunks) {
        CK(cudaMemcpyAsync(h->chunk_b.p, B.cb.data(), sizeof(int) * nchunks, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(h->chunk_e.p, B.ce.data(), sizeof(int) * nchunks, cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(h->struct_chunks.p, B.sc.data(), sizeof(int) * (B.nstruct + 1), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
}

// Cell list and neighbour rows of every atom of the batch (cutoff and cell grid from
// the structure descriptors already on the device).
void enqueue_neighbors(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type, bool renumber) {
    const int n = B.natoms;
    const int T = h->model.ntypes();
    cudaStream_t st = h->stream;
    CK(cudaMemsetAsync(h->cell_count.p, 0, sizeof(int) * B.ncells, st));
    CK(cudaMemsetAsync(h->cell_fill.p, 0, sizeof(int) * B.ncells, st));
    if (n > 0) {
        CK(launch_pdl(k_wrap_bin, dim3((n + 255) / 256), dim3(256), 0, st, h->sdev.p, h->sid.p, d_x, d_type, n, T, h->xw.p, h->xf.p,
                                                    h->xlo.p, h->cell_of.p, h->cell_count.p, h->status.p));
        ++h->launches;
    }
    CK(launch_pdl(k_scan_excl, dim3(1), dim3(1024), 0, st, h->cell_count.p, B.ncells, h->cell_start.p));
    ++h->launches;
    if (n > 0) {
        CK(launch_pdl(k_fill_cells, dim3((n + 255) / 256), dim3(256), 0, st, h->cell_of.p, n, h->cell_start.p, h->cell_fill.p, h->cell_atoms.p));
        CK(launch_pdl(k_sort_cells, dim3((B.ncells * 32 + 255) / 256), dim3(256), 0, st, h->cell_start.p, B.ncells, h->cell_atoms.p));
        const int nw = h->tune.nb_warps;
        if (renumber) {  // the rest of the evaluation numbers atoms in cell order
            CK(launch_pdl(k_renumber, dim3((n + 255) / 256), dim3(256), 0, st, h->cell_atoms.p, n, h->xf.p, h->xlo.p,
                          h->xw.p, h->cell_of.p, d_type, h->xfc.p, h->xloc.p, h->xw2.p, h->cell_of2.p, h->type2.p,
                          h->orig.p));
            CK(launch_pdl(k_neighbors, dim3((n + nw - 1) / nw), dim3(32 * nw), 0, st, h->sdev.p, h->sid.p, h->xw2.p,
                          h->xfc.p, h->xloc.p, h->xfc.p, h->xloc.p, h->cell_of2.p, h->cell_start.p, h->cell_atoms.p,
                          n, pair_bufs(h), h->status.p, h->status.p + 1));
        } else {
            CK(launch_pdl(k_cell_order, dim3((n + 255) / 256), dim3(256), 0, st, h->cell_atoms.p, n, h->xf.p, h->xlo.p,
                          h->xfc.p, h->xloc.p));
            CK(launch_pdl(k_neighbors, dim3((n + nw - 1) / nw), dim3(32 * nw), 0, st, h->sdev.p, h->sid.p, h->xw.p,
                          h->xf.p, h->xlo.p, h->xfc.p, h->xloc.p, h->cell_of.p, h->cell_start.p, h->cell_atoms.p, n,
                          pair_bufs(h), h->status.p, h->status.p + 1));
        }
        h->launches += 4;
    }
}

void enqueue_species(nnap_handle* h, int n, const int* d_type) {
    if (n <= 0) return;
    const int T = h->model.ntypes();
    cudaStream_t st = h->stream;
    const int nb = (n + kSortBlock - 1) / kSortBlock;
    CK(launch_pdl(k_type_hist, dim3(nb), dim3(kSortBlock), 0, st, d_type, n, T, h->block_counts.p));
    CK(launch_pdl(k_type_offsets, dim3(1), dim3(1024), 0, st, h->block_counts.p, nb, T, h->type_start.p));
    CK(launch_pdl(k_type_scatter, dim3(nb), dim3(kSortBlock), 0, st, d_type, n, T, h->block_counts.p, h->perm.p));
    h->launches += 3;
}

void enqueue_species_mirror(nnap_handle* h, const Batch& B, const int* d_type) {
    const int n = B.natoms;
    if (n <= 0) return;
    enqueue_species(h, n, d_type);
    CK(launch_pdl(k_mirror, dim3((unsigned)(((size_t)n * 32 + 255) / 256)), dim3(256), 0, h->stream, 
        h->sdev.p, h->sid.p, pair_bufs(h), n, h->status.p));
    ++h->launches;
}

void enqueue_eval(nnap_handle* h, const Batch& B, const int* d_type, bool fp_only, bool gather, const int* orig) {
    const int n = B.natoms;
    const int T = h->model.ntypes();
    cudaStream_t st = h->stream;
    if (n > 0) CK(cudaMemsetAsync(h->fp.p, 0, sizeof(float) * (size_t)n * h->fp_stride, st));
    // descriptors, per run of species sharing a basis shape and per sub-basis
    // compact rows for the sub-bases that scan them (once per evaluation)
    bool sub_built = false;
    auto descriptors = [&](bool fwd) {
        size_t a_off = 0;
        for (auto& r : h->runs) {
            for (size_t k = 0; k < r.subs.size(); ++k) {
                const SubShape& s = r.subs[k];
                DescArgs a;
                a.perm = h->perm.p;
                a.range = h->type_start.p;
                a.t0 = r.t0;
                a.t1 = r.t1;
                a.nmax = n;
                a.type = d_type;
                a.P = pair_bufs(h);
                a.W = r.W[k].p;
                a.T = T;
                a.rcut = (float)s.rcut;
                a.fp = h->fp.p;
                a.fp_stride = h->fp_stride;
                a.fp_off = r.fp_off[k];
                a.pair_rc = r.prc[k].p;
                a.A = nullptr;
                a.Gx = nullptr;
                size_t this_off = a_off;
                if (s.kind == KIND_SPHERICAL) {
                    a.A = h->A.p + a_off;
                    a_off += (size_t)n * s.np * (s.lmax + 1) * (s.lmax + 1);
                }
                a.gfp = h->gfp.p;
                a.accumulate = k > 0;
                a.warps = fwd ? h->tune.desc_fwd_warps : h->tune.desc_bwd_warps;
                a.nz_p = r.nzp[k].p;
                a.nz_w = r.nzw[k].p;
                a.fwd_alpha = r.falpha[k].p;
                a.tc_sms = (fwd && h->precision == NNAP_PREC_MIXED && !h->fp32_desc && r.tc_fwd[k]) ? h->sm_count : 0;
                a.err = h->status.p;
                a.nl2 = s.nl2;
                a.sl = s.nl2 + s.ninv;
                a.sub_dx = nullptr;
                a.sub_pos = nullptr;
                a.sub_count = nullptr;
                if (r.use_sub[k] && n > 0) {
                    if (!sub_built) {
                        CK(launch_subrows(a.P, n, (float)h->sub_rc, h->sdx.p, h->spos.p, h->scount.p, st));
                        ++h->launches;
                        sub_built = true;
                    }
                    a.sub_dx = h->sdx.p;
                    a.sub_pos = h->spos.p;
                    a.sub_count = h->scount.p;
                }
                // invariant columns: forward after the expansion, their dE/dA before the backward
                InvArgs ia;
                std::memset(&ia, 0, sizeof ia);
                if (s.ninv && n > 0) {
                    ia.perm = h->perm.p;
                    ia.range = h->type_start.p;
                    ia.t0 = r.t0;
                    ia.t1 = r.t1;
                    ia.nmax = n;
                    ia.A = a.A;
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
                    ia.sl = a.sl;
                    ia.Gx = h->Gx.p + this_off;
                    if (!fwd) {
                        CK(launch_invariants(ia, false, st));
                        ++h->launches;
                        a.Gx = ia.Gx;
                    }
                }
                if (n > 0) {
                    CK(launch_descriptor(s.kind, s.basis, s.lmax, s.np, s.n1, a, fwd, st));
                    ++h->launches;
                    if (fwd && s.ninv) {
                        CK(launch_invariants(ia, true, st));
                        ++h->launches;
                    }
                }
            }
        }
    };
    descriptors(true);
    h->mark(2);
    if (!fp_only && n > 0) {
        std::vector<NetArgs> args(T);
        for (int t = 0; t < T; ++t) {
            const NetDev& nd = h->nets[t];
            NetArgs& a = args[t];
            a.perm = h->perm.p;
            a.range = h->type_start.p;
            a.t = t;
            a.nmax = n;
            a.fp = h->fp.p;
            a.fp_stride = h->fp_stride;
            a.D = nd.D;
            a.nlayer = nd.nlayer;
            for (int l = 0; l < kNetMaxLayers; ++l) a.H[l] = l < nd.nlayer ? nd.H[l] : 0;
            a.w = nd.w32.p;
            a.mu_e = nd.mu_e;
            a.sigma_e = nd.sigma_e;
            a.e_atom = h->e_atom.p;
            a.gfp = h->gfp.p;
            a.act = nd.act;
            if (!(h->net_tc && nd.tc.ready)) {
                CK(launch_net_fp32(a, st));
                ++h->launches;
            }
        }
        if (h->net_tc) {
            // one launch per run of consecutive tensor-core species with the same network layout
            for (int t = 0; t < T;) {
                const NetTC& a0 = h->nets[t].tc;
                if (!a0.ready) { ++t; continue; }
                int u = t + 1;
                while (u < T && h->nets[u].tc.ready && h->nets[u].tc.D == a0.D && h->nets[u].tc.L.same(a0.L)) ++u;
                const NetTC* tcs[kMaxTypes];
                for (int k = t; k < u; ++k) tcs[k - t] = &h->nets[k].tc;
                CK(launch_net_tc(&args[t], tcs, u - t, h->status.p, h->sm_count, h->tune.net_split, st));
                ++h->launches;
                t = u;
            }
        }
    }
    h->mark(3);
    if (!fp_only) descriptors(false);
    if (!fp_only && n > 0 && h->model.zbl.on) {  // NEP's ZBL term: energies and pair gradients
        const ZblModel& zm = h->model.zbl;
        ZblArgs za;
        za.flexible = zm.flexible ? 1 : 0;
        za.T = T;
        za.rc_inner = zm.rc_inner;
        za.rc_outer = zm.rc_outer;
        za.z = h->zbl_z.p;
        za.zp = h->zbl_zp.p;
        za.para = h->zbl_para.p;
        za.rc_pair = h->zbl_rc.p;
        CK(launch_nep_zbl(pair_bufs(h), n, d_type, za, h->e_atom.p, st));
        ++h->launches;
    }
    h->mark(4);
    if (!fp_only && gather) {
        if (n > 0) {
            const int gb = h->tune.gather_block;  // threads per CTA, four per atom
            CK(launch_pdl(k_gather, dim3((unsigned)(((size_t)n * 4 + gb - 1) / gb)), dim3(gb), 0, st, pair_bufs(h), n,
                          orig, h->forces.p, h->virials.p));
            ++h->launches;
        }
        const int nchunks = (int)B.cb.size();
        if (nchunks) {
            CK(launch_pdl(k_reduce_chunks, dim3(nchunks), dim3(kRedBlock), 0, st, h->chunk_b.p, h->chunk_e.p, h->e_atom.p, h->virials.p,
                                                            h->partial.p));
            ++h->launches;
        }
        CK(launch_pdl(k_reduce_structs, dim3((B.nstruct * 32 + 127) / 128), dim3(128), 0, st, h->struct_chunks.p, B.nstruct, h->partial.p,
                                                                        h->energy.p, h->virial.p));
        ++h->launches;
    }
    h->mark(5);
}

// Queue the whole evaluation on the handle's stream without any host synchronisation
// (capturable into a CUDA graph).  The structure descriptors are copied from the pinned
// staging array, so a replay picks up new boxes.
void enqueue(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type, bool fp_only) {
    cudaStream_t st = h->stream;
    h->launches = 0;
    h->mark(0);
    CK(cudaMemcpyAsync(h->sdev.p, h->h_sdev, sizeof(StructDev) * B.nstruct, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(h->status.p, 0, sizeof(int) * 2, st));
    // energy / force evaluations run in cell order (descriptor-only calls, which return
    // per-slot rows or neighbour rows, keep atom order)
    const bool renumber = !fp_only && B.natoms > 0;
    h->renumbered = renumber;
    enqueue_neighbors(h, B, d_x, d_type, renumber);
    const int* dt = renumber ? h->type2.p : d_type;
    enqueue_species_mirror(h, B, dt);
    h->mark(1);
    enqueue_eval(h, B, dt, fp_only, true, renumber ? h->orig.p : nullptr);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_status, h->status.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
}

// Identity of a launch sequence: what the captured graph depends on.
std::vector<long long> layout_key(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type, bool fp_only) {
    std::vector<long long> k = {B.nstruct, B.natoms, B.ncells, h->M, (long long)(intptr_t)d_x,
                                (long long)(intptr_t)d_type, fp_only ? 1 : 0, h->profiling ? 1 : 0,
                                h->tune.desc_fwd_warps, h->tune.desc_bwd_warps, h->tune.nb_warps,
                                h->tune.gather_block, h->tune.net_split, h->fp32_desc ? 1 : 0};
    for (auto& s : B.sd) {
        k.push_back(s.n);
        k.push_back(s.kind);
        for (int d = 0; d < 3; ++d) { k.push_back(s.nc[d]); k.push_back(s.R[d]); }
    }
    return k;
}

void drop_graph(nnap_handle* h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->gkey.clear();
}

// Atom-count bucket of the autotuner: natoms in [2^b, 2^(b+1)).
int size_bucket(int natoms) {
    int b = 0;
    while (b < 30 && (2 << b) <= natoms) ++b;
    return b;
}

bool valid_tuning(const Tuning& t) {
    auto in = [](int v, std::initializer_list<int> c) { return std::find(c.begin(), c.end(), v) != c.end(); };
    return in(t.desc_fwd_warps, {2, 4, 8}) && in(t.desc_bwd_warps, {2, 4, 8}) && in(t.nb_warps, {2, 4, 8}) &&
           in(t.gather_block, {64, 128, 256}) && in(t.net_split, {2, 4});
}

// Device milliseconds of the five stages of one eager evaluation with the current shapes.
void stage_ms(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type, double* ms) {
    enqueue(h, B, d_x, d_type, false);
    CK(cudaStreamSynchronize(h->stream));
    const int bits = h->h_status[0];
    if (bits & ERRBIT_BAD_TYPE) throw ApiFail(NNAP_ERR_BAD_TYPE, "species outside 1..ntypes");
    if (bits & ERRBIT_TIMEOUT) throw ApiFail(NNAP_ERR_TIMEOUT, "a bounded tensor-core wait gave up");
    for (int k = 0; k < 5; ++k) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, h->ev[k], h->ev[k + 1]));
        ms[k] = t;
    }
}

// Stage-by-stage search over the launch shapes: for each parameter in turn, every
// candidate is timed (one warm-up, best of two) on the stage it governs with the other
// parameters at their best values so far.  The inputs are the caller's own batch.
Tuning tune_launches(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type) {
    for (auto& e : h->ev)
        if (!e) CK(cudaEventCreate(&e));
    const bool prof = h->profiling;
    h->profiling = true;
    drop_graph(h);
    Tuning best = h->tune;
    auto score = [&](const Tuning& t, int stage) {
        h->tune = t;
        double ms[5], lo = 1e300;
        stage_ms(h, B, d_x, d_type, ms);
        for (int r = 0; r < 2; ++r) {
            stage_ms(h, B, d_x, d_type, ms);
            lo = std::min(lo, ms[stage]);
        }
        return lo;
    };
    struct Param {
        int Tuning::*field;
        int stage;
        std::vector<int> cand;
    };
    std::vector<Param> params = {{&Tuning::nb_warps, 0, {2, 4, 8}},
                                 {&Tuning::desc_fwd_warps, 1, {2, 4, 8}},
                                 {&Tuning::desc_bwd_warps, 3, {2, 4, 8}},
                                 {&Tuning::gather_block, 4, {64, 128, 256}}};
    if (h->net_tc) params.push_back({&Tuning::net_split, 2, {2, 4}});
    try {
        for (auto& p : params) {
            int bv = best.*(p.field);
            double bt = 1e300;
            for (int v : p.cand) {
                Tuning t = best;
                t.*(p.field) = v;
                const double x = score(t, p.stage);
                if (x < bt) {
                    bt = x;
                    bv = v;
                }
            }
            best.*(p.field) = bv;
        }
    } catch (...) {
        h->profiling = prof;
        throw;
    }
    h->profiling = prof;
    h->tune = best;
    return best;
}

// Evaluate a planned batch whose inputs are on the device.  The first call of a layout
// runs eagerly and validates the neighbour capacity; the second captures the launch
// sequence into a CUDA graph; later calls replay it.  Synchronises before returning.
void evaluate(nnap_handle* h, const Batch& B, const double* d_x, const int* d_type, bool fp_only) {
    // launch shapes of this atom-count bucket (tuned now if autotuning is on and the bucket is new)
    int tune_bucket = -1;
    {
        const int b = size_bucket(B.natoms);
        auto it = h->tuned.find(b);
        if (it != h->tuned.end()) h->tune = it->second;
        else if (h->autotune && !fp_only && B.natoms > 0) tune_bucket = b;
        else h->tune = Tuning();
    }
    const bool same_layout = h->layout_ok && h->last_layout == layout_key(h, B, nullptr, nullptr, fp_only);
    if (!same_layout) {
        drop_graph(h);
        prepare_layout(h, B);
        h->layout_ok = true;
        h->last_layout = layout_key(h, B, nullptr, nullptr, fp_only);
        h->layout_runs = 0;
    }
    std::memcpy(h->h_sdev, B.sd.data(), sizeof(StructDev) * B.nstruct);
    for (int attempt = 0; attempt < 4; ++attempt) {
        const std::vector<long long> key = layout_key(h, B, d_x, d_type, fp_only);
        if (h->gexec && h->gkey == key) {
            CK(cudaGraphLaunch(h->gexec, h->stream));
            h->launches = h->glaunches;
        } else if (h->use_graphs && h->layout_runs >= 1) {
            drop_graph(h);
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            h->capturing = true;
            try {
                enqueue(h, B, d_x, d_type, fp_only);
            } catch (...) {
                h->capturing = false;
                cudaStreamEndCapture(h->stream, &g);
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                throw;
            }
            h->capturing = false;
            CK(cudaStreamEndCapture(h->stream, &g));
            cudaError_t e = cudaGraphInstantiate(&h->gexec, g, 0);
            cudaGraphDestroy(g);
            CK(e);
            h->gkey = key;
            h->glaunches = h->launches;
            CK(cudaGraphLaunch(h->gexec, h->stream));
        } else {
            enqueue(h, B, d_x, d_type, fp_only);
        }
        CK(cudaStreamSynchronize(h->stream));
        ++h->layout_runs;
        const int bits = h->h_status[0];
        if (bits & ERRBIT_BAD_TYPE) throw ApiFail(NNAP_ERR_BAD_TYPE, "species outside 1..ntypes");
        if (bits & ERRBIT_TIMEOUT) throw ApiFail(NNAP_ERR_TIMEOUT, "a bounded tensor-core wait gave up");
        const int maxc = h->h_status[1];
        if (maxc <= h->M) {
            if (bits & ERRBIT_NO_MIRROR) throw ApiFail(NNAP_ERR_CAPACITY, "neighbour list is not symmetric");
            if (tune_bucket >= 0) {
                h->tuned[tune_bucket] = tune_launches(h, B, d_x, d_type);
                // the outputs of this call come from the chosen shapes
                enqueue(h, B, d_x, d_type, fp_only);
                CK(cudaStreamSynchronize(h->stream));
                h->last_layout = layout_key(h, B, nullptr, nullptr, fp_only);
                h->layout_runs = 1;
            }
            return;
        }
        // neighbour rows overflowed: grow the capacity and evaluate again
        drop_graph(h);
        grow_pairs(h, B.natoms, ((int)std::ceil(maxc * 1.15) + 8 + 7) & ~7);
        h->last_layout = layout_key(h, B, nullptr, nullptr, fp_only);
        h->layout_runs = 0;
    }
    throw ApiFail(NNAP_ERR_CAPACITY, "neighbour capacity could not be established");
}

void copy_out(nnap_handle* h, const Batch& B, int flags, const Outputs& o, cudaMemcpyKind kind) {
    cudaStream_t st = h->stream;
    const size_t n = B.natoms;
    if ((flags & NNAP_WANT_ENERGY) && o.energy)
        CK(cudaMemcpyAsync(o.energy, h->energy.p, sizeof(double) * B.nstruct, kind, st));
    if ((flags & NNAP_WANT_ENERGIES) && o.energies && n) {
        const double* e = h->e_atom.p;
        if (h->renumbered) {  // per-atom energies of a cell-ordered evaluation, back in atom order
            k_unpermute<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(h->e_atom.p, h->orig.p, (int)n, h->e_out.p);
            CK(cudaGetLastError());
            e = h->e_out.p;
        }
        CK(cudaMemcpyAsync(o.energies, e, sizeof(double) * n, kind, st));
    }
    if ((flags & NNAP_WANT_FORCES) && o.forces && n)
        CK(cudaMemcpyAsync(o.forces, h->forces.p, sizeof(double) * 3 * n, kind, st));
    if ((flags & NNAP_WANT_VIRIAL) && o.virial)
        CK(cudaMemcpyAsync(o.virial, h->virial.p, sizeof(double) * 9 * B.nstruct, kind, st));
    if ((flags & NNAP_WANT_VIRIALS) && o.virials && n)
        CK(cudaMemcpyAsync(o.virials, h->virials.p, sizeof(double) * 9 * n, kind, st));
}

void check_outputs(int flags, const Outputs& o) {
    if ((flags & NNAP_WANT_ENERGY) && !o.energy) throw ApiFail(NNAP_ERR_ARG, "energy output is NULL");
    if ((flags & NNAP_WANT_ENERGIES) && !o.energies) throw ApiFail(NNAP_ERR_ARG, "energies output is NULL");
    if ((flags & NNAP_WANT_FORCES) && !o.forces) throw ApiFail(NNAP_ERR_ARG, "forces output is NULL");
    if ((flags & NNAP_WANT_VIRIAL) && !o.virial) throw ApiFail(NNAP_ERR_ARG, "virial output is NULL");
    if ((flags & NNAP_WANT_VIRIALS) && !o.virials) throw ApiFail(NNAP_ERR_ARG, "virials output is NULL");
}

void upload_inputs(nnap_handle* h, int n, const double* x, const int* type) {
    h->x.ensure(3 * (size_t)std::max(n, 1));
    h->type.ensure(std::max(n, 1));
    if (n) {
        CK(cudaMemcpyAsync(h->x.p, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->type.p, type, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
    }
}

}  // namespace nnapgb

// =================================================================== C ABI
// Handle creation shared by the NNAP and NEP loaders.  NEP's tanh networks always run
// on the FP32 network kernel; NNAP_PREC_MIXED then changes nothing for them.
static int create_handle(Model&& model, int precision, int device, nnap_handle** out) {
    std::unique_ptr<nnap_handle> h(new (std::nothrow) nnap_handle());
    if (!h) return NNAP_ERR_CAPACITY;
    h->model = std::move(model);
    h->precision = precision;
    h->net_tc = precision == NNAP_PREC_MIXED && h->model.act == 0;
    h->device = device;
    try {
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        CK(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
        CK(cudaMallocHost(&h->h_status, sizeof(int) * (3 + kMaxTypes)));
        CK(upload_sh_constants());
        CK(upload_sh_constants_train());
        CK(upload_sh_constants_gen());
        upload_model(h.get());
    } catch (const ApiFail& e) {
        std::fprintf(stderr, "nnap_create: %s\n", e.what());
        nnap_destroy(h.release());
        return e.status;
    } catch (const CudaFail& e) {
        std::fprintf(stderr, "nnap_create: %s\n", e.what());
        nnap_destroy(h.release());
        return NNAP_ERR_CUDA;
    }
    *out = h.release();
    return NNAP_OK;
}

static bool read_file(const char* path, std::string& s) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    s = ss.str();
    return true;
}

extern "C" {

int nnap_create(const char* model_json, size_t len, int precision, int device, nnap_handle** out) {
    if (!model_json || !out) return NNAP_ERR_ARG;
    *out = nullptr;
    if (precision != NNAP_PREC_FP32 && precision != NNAP_PREC_MIXED) return NNAP_ERR_ARG;
    Model m;
    try {
        m = load_model(model_json, len);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "nnap_create: %s\n", e.what());
        return NNAP_ERR_BAD_MODEL;
    }
    return create_handle(std::move(m), precision, device, out);
}

int nnap_model_check(const char* model_text, size_t len, int* ntypes, uint64_t* digest, char* err, size_t errlen) {
    if (!model_text) return NNAP_ERR_ARG;
    if (err && errlen) err[0] = 0;
    try {
        const Model m = load_model(model_text, len);
        if (ntypes) *ntypes = m.ntypes();
        if (digest) *digest = model_digest(m);
        return NNAP_OK;
    } catch (const std::exception& e) {
        if (err && errlen) {
            std::strncpy(err, e.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return NNAP_ERR_BAD_MODEL;
    }
}

int nnap_create_from_file(const char* path, int precision, int device, nnap_handle** out) {
    std::string s;
    if (!path || !out || !read_file(path, s)) return NNAP_ERR_ARG;
    return nnap_create(s.data(), s.size(), precision, device, out);
}

int nnap_create_nep(const char* nep_txt, size_t len, int precision, int device, nnap_handle** out) {
    if (!nep_txt || !out) return NNAP_ERR_ARG;
    *out = nullptr;
    if (precision != NNAP_PREC_FP32 && precision != NNAP_PREC_MIXED) return NNAP_ERR_ARG;
    Model m;
    try {
        m = load_nep_model(nep_txt, len);
    } catch (const NepUnsupported& e) {
        std::fprintf(stderr, "nnap_create_nep: %s\n", e.what());
        return NNAP_ERR_UNSUPPORTED;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "nnap_create_nep: %s\n", e.what());
        return NNAP_ERR_BAD_MODEL;
    }
    return create_handle(std::move(m), precision, device, out);
}

int nnap_create_nep_from_file(const char* path, int precision, int device, nnap_handle** out) {
    std::string s;
    if (!path || !out || !read_file(path, s)) return NNAP_ERR_ARG;
    return nnap_create_nep(s.data(), s.size(), precision, device, out);
}

int nnap_destroy(nnap_handle* h) {
    if (!h) return NNAP_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->dead = true;
    for (auto& r : h->runs) {
        for (auto& w : r.W) w.release();
        for (auto& b : r.nzp) b.release();
        for (auto& b : r.nzw) b.release();
        for (auto& b : r.falpha) b.release();
        for (auto& b : r.inv_idx) b.release();
        for (auto& b : r.inv_coef) b.release();
        for (auto& b : r.inv_start) b.release();
    }
    for (auto& nd : h->nets) { nd.w32.release(); net_tc_release(nd.tc); }
    for (auto* b : {&h->tu, &h->trec, &h->tpart, &h->tbW, &h->tdA, &h->tgfp, &h->tdfp, &h->twpart, &h->tM1x, &h->tM2x})
        b->release();
    for (auto* b : {&h->tbFd, &h->tbE, &h->tgrad, &h->twgrad}) b->release();
    h->tbF.release();
    h->ttiles.release();
    h->x.release(); h->xw.release(); h->e_atom.release(); h->forces.release(); h->virials.release();
    h->energy.release(); h->virial.release(); h->partial.release();
    h->type.release(); h->sid.release(); h->cell_of.release(); h->cell_count.release(); h->cell_fill.release();
    h->cell_start.release(); h->cell_atoms.release(); h->perm.release(); h->block_counts.release();
    h->type_start.release(); h->chunk_b.release(); h->chunk_e.release(); h->struct_chunks.release();
    h->status.release(); h->xf.release(); h->xlo.release(); h->pgrp.release(); h->sdev.release(); h->pkey.release(); h->pdx.release(); h->pg.release();
    h->prev.release(); h->pcount.release(); h->fp.release(); h->gfp.release(); h->A.release(); h->Gx.release(); h->gstart.release();
    h->sdx.release(); h->spos.release(); h->scount.release();
    h->zbl_z.release(); h->zbl_zp.release(); h->zbl_para.release(); h->zbl_rc.release();
    for (auto* b : {&h->lmp_x, &h->lmp_forces, &h->lmp_virials}) b->release();
    h->lmp_pin_in.release();
    h->lmp_pin_out.release();
    for (auto* b : {&h->lmp_type, &h->lmp_ilist, &h->lmp_off, &h->lmp_idx, &h->lmp_rowtype, &h->lmp_rowof,
                    &h->lmp_tcount, &h->lmp_tstart, &h->lmp_tfill, &h->lmp_tlist})
        b->release();
    for (auto& e : h->ev) if (e) cudaEventDestroy(e);
    if (h->order_ev) cudaEventDestroy(h->order_ev);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->h_sdev) cudaFreeHost(h->h_sdev);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return NNAP_OK;
}

int nnap_ntypes(const nnap_handle* h, int* ntypes) {
    if (!h || !ntypes) return NNAP_ERR_ARG;
    *ntypes = h->model.ntypes();
    return NNAP_OK;
}

int nnap_rcut_max(const nnap_handle* h, double* rcut) {
    if (!h || !rcut) return NNAP_ERR_ARG;
    *rcut = h->model.rcut_max;
    return NNAP_OK;
}

int nnap_symbol(const nnap_handle* h, int type, char* buf, size_t buflen) {
    if (!h || !buf || buflen == 0) return NNAP_ERR_ARG;
    if (type < 1 || type > h->model.ntypes()) return NNAP_ERR_BAD_TYPE;
    std::snprintf(buf, buflen, "%s", h->model.sp[type - 1].symbol.c_str());
    return NNAP_OK;
}

int nnap_descriptor_size(const nnap_handle* h, int type, int* size) {
    if (!h || !size) return NNAP_ERR_ARG;
    if (type < 1 || type > h->model.ntypes()) return NNAP_ERR_BAD_TYPE;
    *size = h->model.sp[type - 1].D;
    return NNAP_OK;
}

const char* nnap_last_error(const nnap_handle* h) { return h ? h->err.c_str() : "null handle"; }

int nnap_last_launch_count(const nnap_handle* h, int* count) {
    if (!h || !count) return NNAP_ERR_ARG;
    *count = h->launches;
    return NNAP_OK;
}

int nnap_set_profiling(nnap_handle* h, int on) {
    return guarded(h, [&]() -> int {
        for (auto& e : h->ev)
            if (!e) CK(cudaEventCreate(&e));
        h->profiling = on != 0;
        return NNAP_OK;
    });
}

int nnap_stage_times(nnap_handle* h, double* ms5) {
    if (!ms5) return NNAP_ERR_ARG;
    return guarded(h, [&]() -> int {
        if (!h->ev[5]) throw ApiFail(NNAP_ERR_ARG, "profiling was never enabled");
        CK(cudaEventSynchronize(h->ev[5]));
        for (int k = 0; k < 5; ++k) {
            float t = 0.f;
            CK(cudaEventElapsedTime(&t, h->ev[k], h->ev[k + 1]));
            ms5[k] = t;
        }
        return NNAP_OK;
    });
}

int nnap_compute(nnap_handle* h, int natoms, const double* x, const int* type, int box_kind, const double* box,
                 int flags, double* energy, double* energies, double* forces, double* virial, double* virials) {
    return nnap_compute_batch(h, 1, &natoms, x, type, &box_kind, box, flags, energy, energies, forces, virial,
                              virials);
}

int nnap_compute_batch(nnap_handle* h, int nstruct, const int* natoms, const double* x, const int* type,
                       const int* box_kind, const double* boxes, int flags, double* energy, double* energies,
                       double* forces, double* virial, double* virials) {
    return guarded(h, [&]() -> int {
        if (nstruct < 1 || !natoms || !box_kind || !boxes) throw ApiFail(NNAP_ERR_ARG, "invalid batch description");
        Outputs o{energy, energies, forces, virial, virials};
        check_outputs(flags, o);
        h->launches = 0;
        const Batch& B = plan_batch(h, nstruct, natoms, box_kind, boxes);
        if (B.natoms && (!x || !type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        upload_inputs(h, B.natoms, x, type);
        evaluate(h, B, h->x.p, h->type.p, false);
        copy_out(h, B, flags, o, cudaMemcpyDeviceToHost);
        CK(cudaStreamSynchronize(h->stream));
        return NNAP_OK;
    });
}

int nnap_compute_device(nnap_handle* h, int natoms, const double* d_x, const int* d_type, int box_kind,
                        const double* box, int flags, double* d_energy, double* d_energies, double* d_forces,
                        double* d_virial, double* d_virials, void* stream) {
    return guarded(h, [&]() -> int {
        if (!box) throw ApiFail(NNAP_ERR_ARG, "box is NULL");
        Outputs o{d_energy, d_energies, d_forces, d_virial, d_virials};
        check_outputs(flags, o);
        const Batch& B = plan_batch(h, 1, &natoms, &box_kind, box);
        if (natoms && (!d_x || !d_type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        // NULL is CUDA's default stream; the handle's stream is ordered after the caller's
        // work and the caller's stream waits for the results.
        cudaStream_t user = (cudaStream_t)stream;
        if (!h->order_ev) CK(cudaEventCreateWithFlags(&h->order_ev, cudaEventDisableTiming));
        CK(cudaEventRecord(h->order_ev, user));
        CK(cudaStreamWaitEvent(h->stream, h->order_ev, 0));
        evaluate(h, B, d_x, d_type, false);
        copy_out(h, B, flags, o, cudaMemcpyDeviceToDevice);
        CK(cudaEventRecord(h->order_ev, h->stream));
        CK(cudaStreamWaitEvent(user, h->order_ev, 0));
        return NNAP_OK;
    });
}

int nnap_compute_batch_device(nnap_handle* h, int nstruct, const int* natoms, const double* d_x, const int* d_type,
                              const int* box_kind, const double* boxes, int flags, double* d_energy,
                              double* d_energies, double* d_forces, double* d_virial, double* d_virials,
                              void* stream) {
    return guarded(h, [&]() -> int {
        if (nstruct < 1 || !natoms || !box_kind || !boxes) throw ApiFail(NNAP_ERR_ARG, "invalid batch description");
        Outputs o{d_energy, d_energies, d_forces, d_virial, d_virials};
        check_outputs(flags, o);
        const Batch& B = plan_batch(h, nstruct, natoms, box_kind, boxes);
        if (B.natoms && (!d_x || !d_type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        cudaStream_t user = (cudaStream_t)stream;
        if (!h->order_ev) CK(cudaEventCreateWithFlags(&h->order_ev, cudaEventDisableTiming));
        CK(cudaEventRecord(h->order_ev, user));
        CK(cudaStreamWaitEvent(h->stream, h->order_ev, 0));
        evaluate(h, B, d_x, d_type, false);
        copy_out(h, B, flags, o, cudaMemcpyDeviceToDevice);
        CK(cudaEventRecord(h->order_ev, h->stream));
        CK(cudaStreamWaitEvent(user, h->order_ev, 0));
        return NNAP_OK;
    });
}

int nnap_set_autotune(nnap_handle* h, int on) {
    return guarded(h, [&]() -> int {
        h->autotune = on != 0;
        return NNAP_OK;
    });
}

int nnap_get_tuning(nnap_handle* h, int natoms, int* shapes5, int* tuned) {
    if (!shapes5) return NNAP_ERR_ARG;
    return guarded(h, [&]() -> int {
        auto it = h->tuned.find(size_bucket(natoms));
        const Tuning t = it != h->tuned.end() ? it->second : Tuning();
        shapes5[0] = t.desc_fwd_warps;
        shapes5[1] = t.desc_bwd_warps;
        shapes5[2] = t.nb_warps;
        shapes5[3] = t.gather_block;
        shapes5[4] = t.net_split;
        if (tuned) *tuned = it != h->tuned.end() ? 1 : 0;
        return NNAP_OK;
    });
}

int nnap_set_tuning(nnap_handle* h, int natoms, const int* shapes5) {
    if (!shapes5) return NNAP_ERR_ARG;
    return guarded(h, [&]() -> int {
        Tuning t;
        t.desc_fwd_warps = shapes5[0];
        t.desc_bwd_warps = shapes5[1];
        t.nb_warps = shapes5[2];
        t.gather_block = shapes5[3];
        t.net_split = shapes5[4];
        if (!valid_tuning(t)) throw ApiFail(NNAP_ERR_ARG, "launch shapes outside the tuned candidates");
        h->tuned[size_bucket(natoms)] = t;
        drop_graph(h);
        h->layout_ok = false;
        return NNAP_OK;
    });
}

int nnap_set_graphs(nnap_handle* h, int on) {
    return guarded(h, [&]() -> int {
        h->use_graphs = on != 0;
        if (!h->use_graphs) drop_graph(h);
        return NNAP_OK;
    });
}

int nnap_compute_fp(nnap_handle* h, int natoms, const double* x, const int* type, int box_kind, const double* box,
                    double* fp, int stride) {
    return guarded(h, [&]() -> int {
        if (!box || !fp) throw ApiFail(NNAP_ERR_ARG, "NULL argument");
        int dmax = 0;
        for (auto& sp : h->model.sp) dmax = std::max(dmax, sp.D);
        if (stride < dmax) throw ApiFail(NNAP_ERR_ARG, "stride smaller than the descriptor size");
        h->launches = 0;
        const Batch& B = plan_batch(h, 1, &natoms, &box_kind, box);
        if (natoms && (!x || !type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        upload_inputs(h, natoms, x, type);
        evaluate(h, B, h->x.p, h->type.p, true);
        std::vector<float> f((size_t)natoms * h->fp_stride);
        std::vector<int> perm(natoms);
        if (natoms) {
            CK(cudaMemcpyAsync(f.data(), h->fp.p, sizeof(float) * f.size(), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(perm.data(), h->perm.p, sizeof(int) * natoms, cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
        for (int s = 0; s < natoms; ++s) {
            const int a = perm[s];
            const int D = h->model.sp[type[a] - 1].D;
            for (int q = 0; q < stride; ++q) fp[(size_t)a * stride + q] = q < D ? f[(size_t)s * h->fp_stride + q] : 0.0;
        }
        return NNAP_OK;
    });
}

int nnap_neighbor_list(nnap_handle* h, int natoms, const double* x, const int* type, int box_kind, const double* box,
                       int* counts, long long cap, int* j, int* img, long long* total) {
    return guarded(h, [&]() -> int {
        if (!box || !counts || !total) throw ApiFail(NNAP_ERR_ARG, "NULL argument");
        h->launches = 0;
        const Batch& B = plan_batch(h, 1, &natoms, &box_kind, box);
        if (natoms && (!x || !type)) throw ApiFail(NNAP_ERR_ARG, "positions or types are NULL");
        upload_inputs(h, natoms, x, type);
        evaluate(h, B, h->x.p, h->type.p, true);
        std::vector<int> cnt(natoms);
        std::vector<uint64_t> keys((size_t)natoms * h->M);
        if (natoms) {
            CK(cudaMemcpyAsync(cnt.data(), h->pcount.p, sizeof(int) * natoms, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(keys.data(), h->pkey.p, sizeof(uint64_t) * keys.size(), cudaMemcpyDeviceToHost,
                               h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
        long long t = 0;
        for (int i = 0; i < natoms; ++i) {
            counts[i] = cnt[i];
            for (int k = 0; k < cnt[i]; ++k, ++t) {
                if (!j) continue;
                if (t >= cap) throw ApiFail(NNAP_ERR_CAPACITY, "neighbour output capacity too small");
                const uint64_t key = keys[(size_t)i * h->M + k];
                j[t] = (int)(key >> 32);
                int na, nb, nc;
                unpack_img((uint32_t)key, na, nb, nc);
                img[3 * t] = na; img[3 * t + 1] = nb; img[3 * t + 2] = nc;
            }
        }
        *total = t;
        return NNAP_OK;
    });
}

}  // extern "C"
