// FP64 CPU oracle for the NNAP energy/force/virial path.
//
// TEST INFRASTRUCTURE ONLY.  Loaded through ctypes by tests/, by
// __graft_entry__.smoke() and by the CPU-baseline leg of bench.py.  The product
// library (jse_gb300/csrc) never links or calls this file.
//
// This is an independent restatement of the reference's arithmetic, written from
// the mathematics (not a translation of the reference's template code):
//   * IBox.wrapPBC / toDirect / toCartesian           IBox.java:145-222, BoxPrism.java:162-175
//   * full neighbour list, strict d^2 < rc^2 on wrapped positions, periodic
//     images including images of the atom itself      NeighborListGetter.java:260-372, 704-918, 1018-1050
//   * radial Chebyshev basis                           nnap_util.hpp:226-280, basis_Chebyshev.hpp:82-231
//   * real spherical harmonics and their theta/phi
//     derivatives                                      basis_SphericalUtil.hpp:12-231
//   * spherical-Chebyshev power spectrum fwd/bwd       basis_SphericalChebyshev.hpp:264-525,
//                                                      basis_SphericalUtil.hpp:378-394, 469-484
//   * normalised SiLU feed-forward network fwd/bwd     nnap_main.hpp:267-323, nn_FeedForward.hpp:8-261
//   * per-atom scatter of pair gradients to forces and
//     to per-atom virials on the neighbour            NNAP.java:553-594, IPairPotential.java:919-1006
//
// Every weight type (default/none/full/exfull/fuse/rfuse/exfuse) is evaluated
// through the per-species internal radial-fuse matrix W[t_nei][np][n] that the
// reference's loader builds (WTypeBasis.java:202-304); the reference evaluates the
// non-fused types with explicit weighted sums, which is the same arithmetic up to
// FP64 rounding.
//
// Bispectrum columns (l3max/l4max > 0) are not restated here; the loader rejects them.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

constexpr double kPi4 = 12.566370614359172;  // 4*pi
constexpr double kSnap = 1.0e-10;            // MathEX.Code.DBL_EPSILON, MathEX.java:1213

struct Box {
    int kind;          // 0 orthogonal, 1 LAMMPS lower-triangular, 2 general prism
    double a[3], b[3], c[3];
    double bc[3], ca[3], ab[3], vol;
};

inline void cross(const double* u, const double* v, double* r) {
    // IXYZ.cross (IXYZ.java:84-89): (uy*vz - vy*uz, uz*vx - vz*ux, ux*vy - vx*uy)
    r[0] = u[1] * v[2] - v[1] * u[2];
    r[1] = u[2] * v[0] - v[2] * u[0];
    r[2] = u[0] * v[1] - v[0] * u[1];
}
inline double dot3(const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; }
inline double mixed(const double* u, const double* v, const double* w) {
    // IXYZ.mixed (IXYZ.java:96-101): cross(u, v) . w
    return (u[1] * v[2] - v[1] * u[2]) * w[0] + (u[2] * v[0] - v[2] * u[0]) * w[1] + (u[0] * v[1] - v[0] * u[1]) * w[2];
}

Box make_box(int kind, const double* m) {
    Box B;
    B.kind = kind;
    for (int d = 0; d < 3; ++d) { B.a[d] = m[d]; B.b[d] = m[3 + d]; B.c[d] = m[6 + d]; }
    if (kind == 0) {  // only the diagonal matters
        B.a[1] = B.a[2] = B.b[0] = B.b[2] = B.c[0] = B.c[1] = 0.0;
    } else if (kind == 1) {
        B.a[1] = B.a[2] = B.b[2] = 0.0;
    }
    cross(B.b, B.c, B.bc);
    cross(B.c, B.a, B.ca);
    cross(B.a, B.b, B.ab);
    B.vol = mixed(B.a, B.b, B.c);
    return B;
}

inline void snap(double& v) {
    double r = std::nearbyint(v);  // round-half-even; only |v - r| < 1e-10 matters
    if (std::fabs(v - r) < kSnap) v = r;
}

void to_direct(const Box& B, double* p) {
    double x = p[0], y = p[1], z = p[2];
    if (B.kind == 0) {
        p[0] = x / B.a[0]; p[1] = y / B.b[1]; p[2] = z / B.c[2];
    } else if (B.kind == 1) {
        const double X = B.a[0], Y = B.b[1], Z = B.c[2], XY = B.b[0], XZ = B.c[0], YZ = B.c[1];
        p[0] = x / X - XY * y / (X * Y) + (XY * YZ - XZ * Y) * z / (X * Y * Z);
        p[1] = y / Y - YZ * z / (Y * Z);
        p[2] = z / Z;
    } else {
        double r[3] = {x, y, z};
        p[0] = dot3(B.bc, r) / B.vol;
        p[1] = dot3(B.ca, r) / B.vol;
        p[2] = dot3(B.ab, r) / B.vol;
    }
    snap(p[0]); snap(p[1]); snap(p[2]);
}

void to_cartesian(const Box& B, double* s) {
    double u = s[0], v = s[1], w = s[2];
    if (B.kind == 0) {
        s[0] = u * B.a[0]; s[1] = v * B.b[1]; s[2] = w * B.c[2];
    } else if (B.kind == 1) {
        const double X = B.a[0], Y = B.b[1], Z = B.c[2], XY = B.b[0], XZ = B.c[0], YZ = B.c[1];
        s[0] = X * u + XY * v + XZ * w;
        s[1] = Y * v + YZ * w;
        s[2] = Z * w;
    } else {
        s[0] = B.a[0] * u + B.b[0] * v + B.c[0] * w;
        s[1] = B.a[1] * u + B.b[1] * v + B.c[1] * w;
        s[2] = B.a[2] * u + B.b[2] * v + B.c[2] * w;
    }
}

// Perpendicular distance between the two faces spanned by the other two vectors.
void plane_distances(const Box& B, double* h) {
    auto nrm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    h[0] = std::fabs(B.vol) / nrm(B.bc);
    h[1] = std::fabs(B.vol) / nrm(B.ca);
    h[2] = std::fabs(B.vol) / nrm(B.ab);
}

// Image shift n_a*A + n_b*B + n_c*C, summed in that order.
inline void image_shift(const Box& B, int na, int nb, int nc, double* s) {
    for (int d = 0; d < 3; ++d) s[d] = (na * B.a[d] + nb * B.b[d]) + nc * B.c[d];
}

// ---------------------------------------------------------------- spherical harmonics
// Normalised associated Legendre functions P[l][m] (Condon-Shortley phase included),
// Y_{l,0} = P_l0, Y_{l,m} = sqrt2 P_lm cos(m phi), Y_{l,-m} = sqrt2 P_lm sin(m phi),
// stored at index l*l + l + m, as in basis_SphericalUtil.hpp:12-101.
struct SphWork {
    int L;
    std::vector<double> P, dP;  // (L+1)*(L+1) laid out l*(l+1)/2+m ... use full square for clarity
};

void legendre(int L, double ct, double st, double* P /*[(L+1)^2] index l*(L+1)+m*/, int stride) {
    P[0] = 0.28209479177387814347;  // 1/sqrt(4 pi)
    for (int m = 1; m <= L; ++m)
        P[m * stride + m] = -std::sqrt(1.0 + 0.5 / m) * st * P[(m - 1) * stride + (m - 1)];
    for (int m = 0; m < L; ++m)
        P[(m + 1) * stride + m] = std::sqrt(2.0 * m + 3.0) * ct * P[m * stride + m];
    for (int m = 0; m <= L; ++m) {
        for (int l = m + 2; l <= L; ++l) {
            double A = std::sqrt((4.0 * l * l - 1.0) / (double(l) * l - double(m) * m));
            double Bc = -std::sqrt((double(l - 1) * (l - 1) - double(m) * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
            P[l * stride + m] = A * (ct * P[(l - 1) * stride + m] + Bc * P[(l - 2) * stride + m]);
        }
    }
}

// Y, dY/dtheta, dY/dphi for a displacement (dx,dy,dz) of length r.
// Returns the trig factors used to build the Cartesian chain rule.
struct Angles { double ct, st, cp, sp, dxy; bool pole; };

Angles sph_eval(int L, double dx, double dy, double dz, double r, double* Y, double* Yt, double* Yp) {
    Angles an;
    an.dxy = std::hypot(dx, dy);
    an.ct = dz / r;
    an.st = an.dxy / r;
    // numericEqual(dxy, 0): |dxy| below 8 * DBL_MIN_NORMAL (nnap_util.hpp:148-153)
    an.pole = std::fabs(an.dxy) < 8.0 * 2.2250738585072014E-308;
    if (an.pole) { an.cp = 1.0; an.sp = 0.0; } else { an.cp = dx / an.dxy; an.sp = dy / an.dxy; }
    const int S = L + 2;
    std::vector<double> P((L + 2) * S, 0.0);
    legendre(L, an.ct, an.st, P.data(), S);
    // cos(m phi), sin(m phi) by the Chebyshev recurrence on cos(phi)
    std::vector<double> cm(L + 1), sm(L + 1);
    cm[0] = 1.0; sm[0] = 0.0;
    if (L >= 1) { cm[1] = an.cp; sm[1] = an.sp; }
    for (int m = 2; m <= L; ++m) {
        cm[m] = 2.0 * an.cp * cm[m - 1] - cm[m - 2];
        sm[m] = 2.0 * an.cp * sm[m - 1] - sm[m - 2];
    }
    const double r2 = 1.4142135623730951;
    for (int l = 0; l <= L; ++l) {
        const int c0 = l * l + l;
        for (int m = 0; m <= l; ++m) {
            // dP_lm/dtheta = 1/2 [ sqrt((l-m)(l+m+1)) P_{l,m+1} - sqrt((l+m)(l-m+1)) P_{l,m-1} ],
            // with P_{l,-1} = -P_{l,1}.
            double up = (m + 1 <= l) ? std::sqrt(double(l - m) * (l + m + 1)) * P[l * S + m + 1] : 0.0;
            double pm1 = (m >= 1) ? P[l * S + m - 1] : -P[l * S + 1];
            double dn = (l >= 1) ? std::sqrt(double(l + m) * (l - m + 1)) * pm1 : 0.0;
            double dPt = 0.5 * (up - dn);
            double Plm = P[l * S + m];
            if (m == 0) {
                Y[c0] = Plm; Yt[c0] = dPt; Yp[c0] = 0.0;
            } else {
                Y[c0 + m] = r2 * Plm * cm[m];
                Y[c0 - m] = r2 * Plm * sm[m];
                Yt[c0 + m] = r2 * dPt * cm[m];
                Yt[c0 - m] = r2 * dPt * sm[m];
                Yp[c0 + m] = -m * Y[c0 - m];
                Yp[c0 - m] = m * Y[c0 + m];
            }
        }
    }
    if (an.pole) std::fill(Yp, Yp + (L + 1) * (L + 1), 0.0);
    return an;
}

// ---------------------------------------------------------------- radial functions
inline void cheby(int N, double x, double* T) {
    T[0] = 1.0;
    if (N >= 1) T[1] = x;
    for (int n = 2; n <= N; ++n) T[n] = 2.0 * x * T[n - 1] - T[n - 2];
}
// -(1/r) d/dr of T_n(1 - 2r/rc):  (2/(r rc)) n U_{n-1}(x)
inline void cheby_grad(int N, double r, double rc, double* G) {
    double x = 1.0 - 2.0 * r / rc;
    double mul = 2.0 / (r * rc);
    G[0] = 0.0;
    if (N < 1) return;
    double um2 = 0.0, um1 = mul;  // U_{-1}=0, U_0=1 (scaled)
    G[1] = 1.0 * um1;
    if (N >= 2) {
        double u = 2.0 * mul * x;
        G[2] = 2.0 * u;
        um2 = um1; um1 = u;
        for (int n = 3; n <= N; ++n) {
            double un = 2.0 * x * um1 - um2;
            G[n] = n * un;
            um2 = um1; um1 = un;
        }
    }
}
inline double cutoff(double r, double rc) { double u = 1.0 - (r / rc) * (r / rc); return u * u * u * u; }
inline double cutoff_grad(double r, double rc) { double u = 1.0 - (r / rc) * (r / rc); return 8.0 * u * u * u / (rc * rc); }

// ---------------------------------------------------------------- model description
// spec (ints) per species t, concatenated:
//   [nsub, D, nlayer, h_1..h_nlayer, nn_off, norm_off,
//    then per sub: kind(0 radial,1 sph), nmax, L, np, param_off, fp_off, nl2, ninv, inv_off]
// L is the largest l of the expansion (max of lmax, l3max, l4max); nl2 = lmax + 1
// power-spectrum columns and ninv invariant columns per channel follow each other
// (calSphL2/L3/L4 of basis_SphericalChebyshev.hpp:321-351).  The invariant columns are
// polynomials in A stored at params[inv_off]: per column [nterms, then per term
// (order, i1, i2, i3, i4, coefficient)], i4 unused for order 3.
// params (doubles): all parameter blocks; rcut per sub in rcut[] (flattened per species).
struct Sub { int kind, nmax, lmax, np, param_off, fp_off, nl2, ninv, inv_off; double rcut; };
struct Species {
    int D, mirror, nlayer, nn_off, norm_off;  // mirror: 1-based species whose basis is mirrored (0: none)
    std::vector<int> hidden;
    std::vector<Sub> subs;
};

std::vector<Species> parse_spec(int T, const int* spec, const double* rcuts) {
    std::vector<Species> sp(T);
    int k = 0, ri = 0;
    for (int t = 0; t < T; ++t) {
        int nsub = spec[k++];
        sp[t].D = spec[k++];
        sp[t].mirror = spec[k++];
        sp[t].nlayer = spec[k++];
        for (int i = 0; i < sp[t].nlayer; ++i) sp[t].hidden.push_back(spec[k++]);
        sp[t].nn_off = spec[k++];
        sp[t].norm_off = spec[k++];
        for (int s = 0; s < nsub; ++s) {
            Sub b;
            b.kind = spec[k++]; b.nmax = spec[k++]; b.lmax = spec[k++]; b.np = spec[k++];
            b.param_off = spec[k++]; b.fp_off = spec[k++];
            b.nl2 = spec[k++]; b.ninv = spec[k++]; b.inv_off = spec[k++];
            b.rcut = rcuts[ri++];
            sp[t].subs.push_back(b);
        }
    }
    return sp;
}

inline double silu(double z, double* grad) {
    double s = 1.0 / (1.0 + std::exp(-z));
    *grad = s * (1.0 + z * (1.0 - s));
    return z * s;
}

// Descriptor forward for one atom; A (per sph sub) kept for the backward pass.
void descriptor_forward(const Species& S, int T, const double* params, int nn, const int* ntype,
                        const double* ndx, double* fp, std::vector<std::vector<double>>& Astore) {
    std::fill(fp, fp + S.D, 0.0);
    Astore.assign(S.subs.size(), {});
    for (size_t si = 0; si < S.subs.size(); ++si) {
        const Sub& b = S.subs[si];
        const int N1 = b.nmax + 1, NP = b.np;
        const double* W = params + b.param_off;
        std::vector<double> Rn(N1), Rnp(NP);
        if (b.kind == 0) {
            for (int j = 0; j < nn; ++j) {
                const double* d = ndx + 3 * j;
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (r >= b.rcut) continue;
                cheby(b.nmax, 1.0 - 2.0 * r / b.rcut, Rn.data());
                double fc = cutoff(r, b.rcut);
                const double* Wt = W + (size_t)(ntype[j] - 1) * NP * N1;
                for (int p = 0; p < NP; ++p) {
                    double acc = 0.0;
                    for (int n = 0; n < N1; ++n) acc += Wt[p * N1 + n] * Rn[n];
                    fp[b.fp_off + p] += fc * acc;
                }
            }
        } else {
            const int L = b.lmax, K = (L + 1) * (L + 1);
            std::vector<double>& A = Astore[si];
            A.assign((size_t)NP * K, 0.0);
            std::vector<double> Y(K), Yt(K), Yp(K);
            for (int j = 0; j < nn; ++j) {
                const double* d = ndx + 3 * j;
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (r >= b.rcut) continue;
                sph_eval(L, d[0], d[1], d[2], r, Y.data(), Yt.data(), Yp.data());
                cheby(b.nmax, 1.0 - 2.0 * r / b.rcut, Rn.data());
                double fc = cutoff(r, b.rcut);
                const double* Wt = W + (size_t)(ntype[j] - 1) * NP * N1;
                for (int p = 0; p < NP; ++p) {
                    double acc = 0.0;
                    for (int n = 0; n < N1; ++n) acc += Wt[p * N1 + n] * Rn[n];
                    double c = fc * acc;
                    for (int k = 0; k < K; ++k) A[(size_t)p * K + k] += c * Y[k];
                }
            }
            const int SL = b.nl2 + b.ninv;
            for (int p = 0; p < NP; ++p) {
                for (int l = 0; l < b.nl2; ++l) {
                    double s = 0.0;
                    for (int m = -l; m <= l; ++m) { double a = A[(size_t)p * K + l * l + l + m]; s += a * a; }
                    fp[b.fp_off + p * SL + l] = kPi4 / (2.0 * l + 1.0) * s;
                }
                // three- and four-body invariants: sum of coefficient x product of A entries
                const double* tab = params + b.inv_off;
                const double* Ap = A.data() + (size_t)p * K;
                for (int c = 0; c < b.ninv; ++c) {
                    const int nt = (int)*tab++;
                    double s = 0.0;
                    for (int q = 0; q < nt; ++q, tab += 6) {
                        double prod = tab[5] * Ap[(int)tab[1]] * Ap[(int)tab[2]] * Ap[(int)tab[3]];
                        if ((int)tab[0] == 4) prod *= Ap[(int)tab[4]];
                        s += prod;
                    }
                    fp[b.fp_off + p * SL + b.nl2 + c] = s;
                }
            }
        }
    }
}

// Network forward + input gradient.  Returns E_i; fills gfp = dE_i/dfp.
double network(const Species& S, const double* params, const double* fp, double* gfp) {
    const double* norm = params + S.norm_off;
    const double mu_e = norm[0], sig_e = norm[1];
    const double* mu = norm + 2;
    const double* sg = norm + 2 + S.D;
    const double* w = params + S.nn_off;
    int hw = 0, hb = 0, fan = S.D;
    for (int l = 0; l < S.nlayer; ++l) { hw += S.hidden[l] * fan; hb += S.hidden[l]; fan = S.hidden[l]; }
    const double* ow = w + hw;
    const double* bias = ow + fan;
    const double ob = bias[hb];
    std::vector<std::vector<double>> act(S.nlayer + 1), dact(S.nlayer);
    act[0].resize(S.D);
    for (int i = 0; i < S.D; ++i) act[0][i] = (fp[i] - mu[i]) / sg[i];
    const double* Wl = w;
    const double* bl = bias;
    fan = S.D;
    for (int l = 0; l < S.nlayer; ++l) {
        int H = S.hidden[l];
        act[l + 1].resize(H);
        dact[l].resize(H);
        for (int o = 0; o < H; ++o) {
            double z = 0.0;
            for (int i = 0; i < fan; ++i) z += Wl[(size_t)o * fan + i] * act[l][i];
            z += bl[o];
            act[l + 1][o] = silu(z, &dact[l][o]);
        }
        Wl += (size_t)H * fan; bl += H; fan = H;
    }
    double out = ob;
    for (int i = 0; i < fan; ++i) out += ow[i] * act[S.nlayer][i];
    // backward
    std::vector<double> g(fan);
    for (int i = 0; i < fan; ++i) g[i] = sig_e * ow[i];
    for (int l = S.nlayer - 1; l >= 0; --l) {
        int H = S.hidden[l];
        int in = (l == 0) ? S.D : S.hidden[l - 1];
        Wl -= (size_t)H * in;
        std::vector<double> gi(in, 0.0);
        for (int o = 0; o < H; ++o) {
            double dz = g[o] * dact[l][o];
            for (int i = 0; i < in; ++i) gi[i] += dz * Wl[(size_t)o * in + i];
        }
        g.swap(gi);
    }
    for (int i = 0; i < S.D; ++i) gfp[i] = g[i] / sg[i];
    return out * sig_e + mu_e;
}

// Descriptor backward: pair gradients g_j = -dE_i/d(x_j - x_i), accumulated into gout.
void descriptor_backward(const Species& S, const double* params, int nn, const int* ntype, const double* ndx,
                         const double* gfp, const std::vector<std::vector<double>>& Astore, double* gout) {
    for (size_t si = 0; si < S.subs.size(); ++si) {
        const Sub& b = S.subs[si];
        const int N1 = b.nmax + 1, NP = b.np;
        const double* W = params + b.param_off;
        std::vector<double> Rn(N1), Rg(N1), Rnp(NP), dRn(N1), dc(NP);
        if (b.kind == 0) {
            const double* gf = gfp + b.fp_off;
            for (int j = 0; j < nn; ++j) {
                const double* d = ndx + 3 * j;
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (r >= b.rcut) continue;
                cheby(b.nmax, 1.0 - 2.0 * r / b.rcut, Rn.data());
                cheby_grad(b.nmax, r, b.rcut, Rg.data());
                double fc = cutoff(r, b.rcut), fcg = cutoff_grad(r, b.rcut);
                const double* Wt = W + (size_t)(ntype[j] - 1) * NP * N1;
                double dfc = 0.0;
                std::fill(dRn.begin(), dRn.end(), 0.0);
                for (int p = 0; p < NP; ++p) {
                    double rnp = 0.0;
                    for (int n = 0; n < N1; ++n) rnp += Wt[p * N1 + n] * Rn[n];
                    dfc += gf[p] * rnp;
                    for (int n = 0; n < N1; ++n) dRn[n] += gf[p] * fc * Wt[p * N1 + n];
                }
                double gr = dfc * fcg;
                for (int n = 0; n < N1; ++n) gr += dRn[n] * Rg[n];
                gout[3 * j + 0] += gr * d[0];
                gout[3 * j + 1] += gr * d[1];
                gout[3 * j + 2] += gr * d[2];
            }
        } else {
            const int L = b.lmax, K = (L + 1) * (L + 1);
            const std::vector<double>& A = Astore[si];
            std::vector<double> G((size_t)NP * K, 0.0);
            const int SL = b.nl2 + b.ninv;
            for (int p = 0; p < NP; ++p) {
                for (int l = 0; l < b.nl2; ++l) {
                    double coef = 2.0 * kPi4 / (2.0 * l + 1.0) * gfp[b.fp_off + p * SL + l];
                    for (int m = -l; m <= l; ++m) {
                        int k = l * l + l + m;
                        G[(size_t)p * K + k] = coef * A[(size_t)p * K + k];
                    }
                }
                // d(invariant)/dA: each factor of a product in turn
                const double* tab = params + b.inv_off;
                const double* Ap = A.data() + (size_t)p * K;
                double* Gp = G.data() + (size_t)p * K;
                for (int c = 0; c < b.ninv; ++c) {
                    const int nt = (int)*tab++;
                    const double g = gfp[b.fp_off + p * SL + b.nl2 + c];
                    for (int q = 0; q < nt; ++q, tab += 6) {
                        const int ord = (int)tab[0];
                        for (int f = 0; f < ord; ++f) {
                            double prod = g * tab[5];
                            for (int o = 0; o < ord; ++o)
                                if (o != f) prod *= Ap[(int)tab[1 + o]];
                            Gp[(int)tab[1 + f]] += prod;
                        }
                    }
                }
            }
            std::vector<double> Y(K), Yt(K), Yp(K), dY(K);
            for (int j = 0; j < nn; ++j) {
                const double* d = ndx + 3 * j;
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (r >= b.rcut) continue;
                Angles an = sph_eval(L, d[0], d[1], d[2], r, Y.data(), Yt.data(), Yp.data());
                cheby(b.nmax, 1.0 - 2.0 * r / b.rcut, Rn.data());
                cheby_grad(b.nmax, r, b.rcut, Rg.data());
                double fc = cutoff(r, b.rcut), fcg = cutoff_grad(r, b.rcut);
                const double* Wt = W + (size_t)(ntype[j] - 1) * NP * N1;
                std::fill(dY.begin(), dY.end(), 0.0);
                std::fill(dRn.begin(), dRn.end(), 0.0);
                double dfc = 0.0;
                for (int p = 0; p < NP; ++p) {
                    double rnp = 0.0;
                    for (int n = 0; n < N1; ++n) rnp += Wt[p * N1 + n] * Rn[n];
                    double c = fc * rnp;
                    double dcp = 0.0;
                    for (int k = 0; k < K; ++k) {
                        double gk = G[(size_t)p * K + k];
                        dY[k] += gk * c;
                        dcp += gk * Y[k];
                    }
                    dfc += dcp * rnp;
                    for (int n = 0; n < N1; ++n) dRn[n] += dcp * fc * Wt[p * N1 + n];
                }
                double gr = dfc * fcg, gt = 0.0, gp = 0.0;
                for (int n = 0; n < N1; ++n) gr += dRn[n] * Rg[n];
                for (int k = 0; k < K; ++k) { gt += dY[k] * Yt[k]; gp += dY[k] * Yp[k]; }
                // (-d theta/dx, ...) and (-d phi/dx, ...), as in calYPthetaPphi
                double tpx = -an.ct * an.cp / r, tpy = -an.ct * an.sp / r, tpz = an.st / r;
                double ppx = an.pole ? 0.0 : an.sp / an.dxy, ppy = an.pole ? 0.0 : -an.cp / an.dxy;
                gout[3 * j + 0] += gr * d[0] + gt * tpx + gp * ppx;
                gout[3 * j + 1] += gr * d[1] + gt * tpy + gp * ppy;
                gout[3 * j + 2] += gr * d[2] + gt * tpz;
            }
        }
    }
}

}  // namespace

extern "C" {

// IBox.wrapPBC applied to every atom (AtomicParameterCalculator.java:141-147, 214-221).
int oracle_wrap(int n, const double* x, int box_kind, const double* box, double* xw) {
    Box B = make_box(box_kind, box);
    for (int i = 0; i < n; ++i) {
        double p[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
        to_direct(B, p);
        for (int d = 0; d < 3; ++d)
            if (p[d] < 0.0 || p[d] >= 1.0) p[d] -= std::floor(p[d]);
        to_cartesian(B, p);
        xw[3 * i] = p[0]; xw[3 * i + 1] = p[1]; xw[3 * i + 2] = p[2];
    }
    return 0;
}

// Full neighbour list on wrapped positions.  Pass nbr_j == NULL to only count.
// Entries per atom are (j, image na/nb/nc, dx/dy/dz); cap bounds the total.
// Returns the total number of pairs, or -1 if cap is exceeded.
long oracle_neighbors(int n, const double* xw, int box_kind, const double* box, double rcut,
                      int* counts, long cap, int* nbr_j, int* nbr_img, double* nbr_dx) {
    Box B = make_box(box_kind, box);
    double h[3];
    plane_distances(B, h);
    int nc[3], R[3];
    for (int d = 0; d < 3; ++d) {
        nc[d] = std::max(1, (int)std::floor(h[d] / rcut));
        if (nc[d] > 1024) nc[d] = 1024;
        R[d] = (int)std::ceil(rcut * nc[d] / h[d]) + 1;
    }
    const long ncell = (long)nc[0] * nc[1] * nc[2];
    std::vector<int> cell_of(n);
    std::vector<std::vector<int>> cells(ncell);
    for (int i = 0; i < n; ++i) {
        double s[3] = {xw[3 * i], xw[3 * i + 1], xw[3 * i + 2]};
        to_direct(B, s);
        int c[3];
        for (int d = 0; d < 3; ++d) {
            c[d] = (int)std::floor(s[d] * nc[d]);
            c[d] = std::min(std::max(c[d], 0), nc[d] - 1);
        }
        long id = c[0] + (long)nc[0] * (c[1] + (long)nc[1] * c[2]);
        cell_of[i] = (int)id;
        cells[id].push_back(i);
    }
    const double rc2 = rcut * rcut;
    long total = 0;
    for (int i = 0; i < n; ++i) {
        long id = cell_of[i];
        int ci[3] = {(int)(id % nc[0]), (int)((id / nc[0]) % nc[1]), (int)(id / ((long)nc[0] * nc[1]))};
        int cnt = 0;
        for (int oc = -R[2]; oc <= R[2]; ++oc)
        for (int ob = -R[1]; ob <= R[1]; ++ob)
        for (int oa = -R[0]; oa <= R[0]; ++oa) {
            int q[3] = {ci[0] + oa, ci[1] + ob, ci[2] + oc}, img[3], cc[3];
            for (int d = 0; d < 3; ++d) {
                img[d] = (int)std::floor((double)q[d] / nc[d]);
                cc[d] = q[d] - img[d] * nc[d];
            }
            double sh[3];
            image_shift(B, img[0], img[1], img[2], sh);
            const std::vector<int>& cl = cells[cc[0] + (long)nc[0] * (cc[1] + (long)nc[1] * cc[2])];
            for (int j : cl) {
                if (j == i && img[0] == 0 && img[1] == 0 && img[2] == 0) continue;
                double dx = (xw[3 * j] + sh[0]) - xw[3 * i];
                double dy = (xw[3 * j + 1] + sh[1]) - xw[3 * i + 1];
                double dz = (xw[3 * j + 2] + sh[2]) - xw[3 * i + 2];
                double d2 = dx * dx + dy * dy + dz * dz;
                if (!(d2 < rc2)) continue;
                if (nbr_j) {
                    if (total >= cap) return -1;
                    nbr_j[total] = j;
                    nbr_img[3 * total] = img[0]; nbr_img[3 * total + 1] = img[1]; nbr_img[3 * total + 2] = img[2];
                    nbr_dx[3 * total] = dx; nbr_dx[3 * total + 1] = dy; nbr_dx[3 * total + 2] = dz;
                }
                ++cnt;
                ++total;
            }
        }
        counts[i] = cnt;
    }
    return total;
}

// Brute-force enumeration over all pairs and all images |n| <= R; for small test cases.
long oracle_neighbors_brute(int n, const double* xw, int box_kind, const double* box, double rcut,
                            int* counts, long cap, int* nbr_j, int* nbr_img) {
    Box B = make_box(box_kind, box);
    double h[3];
    plane_distances(B, h);
    int R[3];
    for (int d = 0; d < 3; ++d) R[d] = (int)std::ceil(rcut / h[d]) + 1;
    const double rc2 = rcut * rcut;
    long total = 0;
    for (int i = 0; i < n; ++i) {
        int cnt = 0;
        for (int j = 0; j < n; ++j)
            for (int a = -R[0]; a <= R[0]; ++a)
            for (int b = -R[1]; b <= R[1]; ++b)
            for (int c = -R[2]; c <= R[2]; ++c) {
                if (j == i && a == 0 && b == 0 && c == 0) continue;
                double sh[3];
                image_shift(B, a, b, c, sh);
                double dx = (xw[3 * j] + sh[0]) - xw[3 * i];
                double dy = (xw[3 * j + 1] + sh[1]) - xw[3 * i + 1];
                double dz = (xw[3 * j + 2] + sh[2]) - xw[3 * i + 2];
                double d2 = dx * dx + dy * dy + dz * dz;
                if (!(d2 < rc2)) continue;
                if (nbr_j) {
                    if (total >= cap) return -1;
                    nbr_j[total] = j;
                    nbr_img[3 * total] = a; nbr_img[3 * total + 1] = b; nbr_img[3 * total + 2] = c;
                }
                ++cnt; ++total;
            }
        counts[i] = cnt;
    }
    return total;
}

// Energies, forces and per-atom virials for one structure given its neighbour CSR.
//   type[i] is 1-based; nei_off has n+1 entries; nei_dx holds x_j(+image) - x_i.
//   e_atom[n], force[3n], virial[9n] (xx,yy,zz,xy,xz,yz,yx,zx,zy), fp_out[n*fp_stride] (optional),
//   pair_g[3*npairs] (optional) receive the results.  Returns 0 on success.
//   Atoms [0, n_eval) are evaluated (n_eval <= n, a prefix is used to time a bounded sample).
int oracle_compute(int T, const int* spec, const double* rcuts, const double* params,
                   int n, int n_eval, const int* type, const long* nei_off, const int* nei_j, const double* nei_dx,
                   double* e_atom, double* force, double* virial, double* fp_out, int fp_stride, double* pair_g) {
    std::vector<Species> sp = parse_spec(T, spec, rcuts);
    std::vector<int> ntype;
    std::vector<double> g, fp, gfp;
    std::vector<std::vector<double>> Astore;
    if (force) std::fill(force, force + 3 * (size_t)n, 0.0);
    if (virial) std::fill(virial, virial + 9 * (size_t)n, 0.0);
    for (int i = 0; i < n_eval; ++i) {
        int ti = type[i];
        if (ti < 1 || ti > T) return 2;
        const Species& S = sp[ti - 1];
        long o = nei_off[i];
        int nn = (int)(nei_off[i + 1] - o);
        ntype.resize(nn);
        for (int j = 0; j < nn; ++j) {
            int tj = type[nei_j[o + j]];
            if (tj < 1 || tj > T) return 2;
            // a mirror basis sees its own species and the mirrored one swapped
            // (nnap_main.hpp:40-48, MirrorBasis.java)
            if (S.mirror) tj = tj == S.mirror ? ti : (tj == ti ? S.mirror : tj);
            ntype[j] = tj;
        }
        const double* ndx = nei_dx + 3 * o;
        fp.assign(S.D, 0.0);
        gfp.assign(S.D, 0.0);
        descriptor_forward(S, T, params, nn, ntype.data(), ndx, fp.data(), Astore);
        if (fp_out) std::copy(fp.begin(), fp.end(), fp_out + (size_t)i * fp_stride);
        double e = network(S, params, fp.data(), gfp.data());
        if (e_atom) e_atom[i] = e;
        g.assign(3 * (size_t)nn, 0.0);
        descriptor_backward(S, params, nn, ntype.data(), ndx, gfp.data(), Astore, g.data());
        if (pair_g) std::copy(g.begin(), g.end(), pair_g + 3 * o);
        for (int j = 0; j < nn; ++j) {
            int jj = nei_j[o + j];
            const double fx = g[3 * j], fy = g[3 * j + 1], fz = g[3 * j + 2];
            const double dx = ndx[3 * j], dy = ndx[3 * j + 1], dz = ndx[3 * j + 2];
            if (force) {
                force[3 * i] -= fx; force[3 * i + 1] -= fy; force[3 * i + 2] -= fz;
                force[3 * jj] += fx; force[3 * jj + 1] += fy; force[3 * jj + 2] += fz;
            }
            if (virial) {
                double* v = virial + 9 * (size_t)jj;
                v[0] += dx * fx; v[1] += dy * fy; v[2] += dz * fz;
                v[3] += dx * fy; v[4] += dx * fz; v[5] += dy * fz;
                v[6] += dy * fx; v[7] += dz * fx; v[8] += dz * fy;
            }
        }
    }
    return 0;
}

}  // extern "C"
