// NEP potential files (nep.txt) mapped onto the NNAP descriptor pipeline.
//
// The loader follows NEP(String) (NEP.java:786-1010): a header of whitespace-separated
// lines, then one number per line (the network parameters, the descriptor coefficients
// c and the dim descriptor scales q_scaler).  Potential models nep3, nep4 and nep5,
// with or without ZBL (fixed or flexible) and type-wise cutoffs, are mapped; the other
// variants (dipole, polarizability) throw NepUnsupported.
//
// NEP's per-atom arithmetic (nep_core.hpp, find_q / find_q_with_4body / _5body and
// apply_ann_one_layer) is, in the quantities of the NNAP pipeline:
//   radial sub-basis      q_n = sum_j g_n(r_ij), g_n = sum_k c_R[t_i][t_j][n][k] f_k(r_ij; rc_R)
//   spherical sub-basis   A[n][lm] = sum_j g_n(r_ij) Y_lm,   g_n from c_A and rc_A
//                         q_nl = sum_m A[n][lm]^2          (l = 1 .. l_max)
//                         4-body column = L3(2 2 2), 5-body column = L4(1 1 1 1) of A[n]
//   network               E_i = sum_h w1[h] tanh(sum_d w0[h][d] q_d s_d - b0[h]) - b1 [- w1_T]
// with f_k = (T_k(2(r/rc - 1)^2 - 1) + 1)/2 (cos(pi r/rc) + 1)/2 (kernel radial basis
// kRbNEP) and c_X[t_i][t_j][n][k] = c[off_X + (n (b_X + 1) + k) T^2 + t_i T + t_j].
// The spherical sub-basis computes every power-spectrum column 4 pi/(2l+1) sum_m A^2 for
// l = 0 .. l_max and the invariant columns of l3max = 2 (222, 112) and l4max = 1 (1111);
// the network reads the columns NEP uses through 1/sigma = s_d (2l+1)/(4 pi) (power
// spectrum) or s_d (the rest) and gives the l = 0 and 112 columns zero weights.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

#include "model.hpp"

namespace nnapgb {
namespace {

constexpr double kPi = 3.14159265358979323846;

// Element symbols in periodic-table order (H .. Pu); a species' atomic number is its index + 1
constexpr int kNumElements = 94;
const char* const kElements[kNumElements] = {
    "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",
    "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge",
    "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd",
    "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd",
    "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg",
    "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Np", "Pu"};

// Covalent radii (A) by periodic-table index, the table NEP's type-wise cutoffs scale
// (COVALENT_RADIUS, nep_core.hpp:247-258)
const double kCovalentRadius[kNumElements] = {
    0.426667, 0.613333, 1.6, 1.25333, 1.02667, 1.0, 0.946667, 0.84,
    0.853333, 0.893333, 1.86667, 1.66667, 1.50667, 1.38667, 1.46667, 1.36,
    1.32, 1.28, 2.34667, 2.05333, 1.77333, 1.62667, 1.61333, 1.46667,
    1.42667, 1.38667, 1.33333, 1.32, 1.34667, 1.45333, 1.49333, 1.45333,
    1.53333, 1.46667, 1.52, 1.56, 2.52, 2.22667, 1.96, 1.85333,
    1.76, 1.65333, 1.53333, 1.50667, 1.50667, 1.44, 1.53333, 1.64,
    1.70667, 1.68, 1.68, 1.64, 1.76, 1.74667, 2.78667, 2.34667,
    2.16, 1.96, 2.10667, 2.09333, 2.08, 2.06667, 2.01333, 2.02667,
    2.01333, 2.0, 1.98667, 1.98667, 1.97333, 2.04, 1.94667, 1.82667,
    1.74667, 1.64, 1.57333, 1.54667, 1.48, 1.49333, 1.50667, 1.76,
    1.73333, 1.73333, 1.81333, 1.74667, 1.84, 1.89333, 2.68, 2.41333,
    2.22667, 2.10667, 2.02667, 2.04, 2.05333, 2.06667};

void bad(const std::string& m) { throw std::runtime_error("nep.txt: " + m); }

int to_int(const std::string& s) {
    char* e = nullptr;
    const long v = std::strtol(s.c_str(), &e, 10);
    if (!e || *e) bad("expected an integer, found '" + s + "'");
    return (int)v;
}

double to_double(const std::string& s) {
    char* e = nullptr;
    const double v = std::strtod(s.c_str(), &e);
    if (!e || *e) bad("expected a number, found '" + s + "'");
    return v;
}

}  // namespace

Model load_nep_model(const char* text, size_t len) {
    std::vector<std::vector<std::string>> lines;
    {
        std::istringstream in(std::string(text, len));
        std::string ln;
        while (std::getline(in, ln)) {
            std::istringstream ls(ln);
            std::vector<std::string> tok;
            std::string t;
            while (ls >> t) tok.push_back(t);
            if (!tok.empty()) lines.push_back(tok);
        }
    }
    size_t at = 0;
    auto next = [&](size_t n_expect, const char* what) -> const std::vector<std::string>& {
        if (at >= lines.size()) bad(std::string("file ends before: ") + what);
        const auto& t = lines[at++];
        if (n_expect && t.size() != n_expect) bad(std::string("this line should be ") + what);
        return t;
    };
    // nep4 2 Si O
    const auto& head = next(0, "the model line");
    if (head.size() < 3) bad("the first line should have at least 3 items");
    int version = 0;
    const bool zbl = head[0].size() > 4 && head[0].compare(head[0].size() - 4, 4, "_zbl") == 0;
    const std::string kind = zbl ? head[0].substr(0, head[0].size() - 4) : head[0];
    if (kind == "nep3") version = 3;
    else if (kind == "nep4") version = 4;
    else if (kind == "nep5") version = 5;
    else if (head[0].rfind("nep", 0) == 0)
        throw NepUnsupported("NEP variant " + head[0] + " is not supported (potential models nep3, nep4, nep5, with or without ZBL)");
    else bad("unknown model type " + head[0]);
    const int T = to_int(head[1]);
    if (T < 1 || (int)head.size() != 2 + T) bad("the first line should list the atom symbols");
    // zbl rc_inner rc_outer (both zero: flexible per-pair parameters after the scales)
    double zin = 0.0, zout = 0.0;
    if (zbl) {
        const auto& z = next(3, "zbl rc_inner rc_outer");
        if (z[0] != "zbl") bad("this line should be zbl rc_inner rc_outer");
        zin = to_double(z[1]);
        zout = to_double(z[2]);
    }
    const bool zflex = zbl && zin == 0.0 && zout == 0.0;
    // cutoff rc_R rc_A MN_R MN_A [factors]
    const auto& cut = next(0, "cutoff");
    if (cut.size() != 5 && cut.size() != 8) bad("this line should be cutoff rc_radial rc_angular MN_radial MN_angular");
    const double rcR = to_double(cut[1]), rcA = to_double(cut[2]);
    // type-wise cutoff factors (radial, angular, ZBL): a radial factor > 0 gives every
    // species pair of the descriptors its own cutoffs, a ZBL factor > 0 the fixed-form ZBL
    // its own radii (NEP.java:905-916)
    const double fR = cut.size() == 8 ? to_double(cut[5]) : 0.0;
    const double fA = cut.size() == 8 ? to_double(cut[6]) : 0.0;
    const double fZ = cut.size() == 8 ? to_double(cut[7]) : 0.0;
    const bool tw = fR > 0.0, twz = fZ > 0.0;
    if (!(rcR > 0.0) || !(rcA > 0.0)) bad("cutoffs must be positive");
    const auto& nm = next(3, "n_max n_max_radial n_max_angular");
    const int nR = to_int(nm[1]), nA = to_int(nm[2]);
    const auto& bs = next(3, "basis_size basis_size_radial basis_size_angular");
    const int bR = to_int(bs[1]), bA = to_int(bs[2]);
    const auto& lm = next(4, "l_max l_max_3body l_max_4body l_max_5body");
    const int L = to_int(lm[1]);
    // the flags only count columns; the reference keys the terms on the count (find_q,
    // nep_core.hpp:943-955): the 4-body column when there is one extra, the 5-body column
    // when there are two
    const int nextra = (to_int(lm[2]) == 2 ? 1 : 0) + (to_int(lm[3]) == 1 ? 1 : 0);
    const bool b4 = nextra >= 1, b5 = nextra >= 2;
    const auto& ann = next(3, "ANN num_neurons 0");
    const int H = to_int(ann[1]);
    if (nR < 0 || nA < 0 || bR < 0 || bA < 0 || L < 1 || H < 1) bad("invalid sizes");
    const int numL = L + nextra;
    const int dim = (nR + 1) + (nA + 1) * numL;
    const int per = (dim + 2) * H + (version == 5 ? 1 : 0);
    const int npa = version == 3 ? (dim + 2) * H + 1 : per * T + 1;
    const int ncR = T * T * (nR + 1) * (bR + 1);
    const int npd = ncR + T * T * (nA + 1) * (bA + 1);
    std::vector<double> v;
    while (at < lines.size()) v.push_back(to_double(lines[at++][0]));
    const int nz = zflex ? 10 * T * (T + 1) / 2 : 0;
    if ((int)v.size() != npa + npd + dim + nz) bad("wrong number of parameters");
    const double* c = v.data() + npa;
    const double* qs = v.data() + npa + npd;
    const double b1 = v[npa - 1];

    // periodic-table index of each species, 0 (hydrogen) when the symbol is not an element
    std::vector<int> anum(T, 0);
    for (int t = 0; t < T; ++t)
        for (int e = 0; e < kNumElements; ++e)
            if (head[2 + t] == kElements[e]) {
                anum[t] = e;
                break;
            }
    // a pair's type-wise cutoff: min(rc, (R_cov,i + R_cov,j) factor) (nep_core.hpp:1078, 1121, 1371)
    auto pair_cut = [&](double rc, double f, int ti, int tj) {
        return std::min(rc, (kCovalentRadius[anum[ti]] + kCovalentRadius[anum[tj]]) * f);
    };

    Model m;
    m.units = "metal";
    m.rcut_max = std::max(rcR, rcA);
    m.radial_fn = 1;
    m.act = 1;
    if (zbl) {
        m.zbl.on = true;
        m.zbl.flexible = zflex;
        m.zbl.rc_inner = zin;
        m.zbl.rc_outer = zout;
        for (int t = 0; t < T; ++t) m.zbl.z.push_back(anum[t] + 1);
        m.zbl.para.assign(v.begin() + npa + npd + dim, v.end());
        if (twz && !zflex)  // rc_outer shrunk to the pair's covalent size, rc_inner its half
            for (int ti = 0; ti < T; ++ti)
                for (int tj = 0; tj < T; ++tj) {
                    const double ro = pair_cut(zout, fZ, ti, tj);
                    m.zbl.pair_rc.push_back(0.5 * ro);
                    m.zbl.pair_rc.push_back(ro);
                }
    }
    const int l3 = b4 ? 2 : 0, l4 = b5 ? 1 : 0;
    const auto inv = invariant_columns(l3, l4);
    const int nl2 = L + 1, sl = nl2 + (int)inv.size();
    const int D = (nR + 1) + (nA + 1) * sl;
    // NEP descriptor column d -> (our column, 1/sigma factor of s_d)
    std::vector<int> col(dim);
    std::vector<double> kap(dim, 1.0);
    for (int n = 0; n <= nR; ++n) col[n] = n;
    for (int l = 1; l <= L; ++l)
        for (int n = 0; n <= nA; ++n) {
            const int d = (nR + 1) + (l - 1) * (nA + 1) + n;
            col[d] = (nR + 1) + n * sl + l;
            kap[d] = (2.0 * l + 1.0) / (4.0 * kPi);
        }
    int d0 = (nR + 1) + L * (nA + 1);
    if (b4) {
        for (int n = 0; n <= nA; ++n) col[d0 + n] = (nR + 1) + n * sl + nl2;              // L3(2 2 2)
        d0 += nA + 1;
    }
    if (b5)
        for (int n = 0; n <= nA; ++n) col[d0 + n] = (nR + 1) + n * sl + nl2 + (b4 ? 2 : 0);  // L4(1 1 1 1)
    for (int t = 0; t < T; ++t) {
        Species sp;
        sp.symbol = head[2 + t];
        SubBasis r;
        r.kind = KIND_RADIAL;
        r.nmax = bR;
        r.np = nR + 1;
        r.fp_off = 0;
        r.size = r.np;
        r.rcut = rcR;
        r.W.assign((size_t)T * r.np * (bR + 1), 0.0);
        for (int tn = 0; tn < T; ++tn)
            for (int n = 0; n <= nR; ++n)
                for (int k = 0; k <= bR; ++k)
                    r.W[((size_t)tn * r.np + n) * (bR + 1) + k] = c[(n * (bR + 1) + k) * T * T + t * T + tn];
        SubBasis s;
        s.kind = KIND_SPHERICAL;
        s.nmax = bA;
        s.np = nA + 1;
        s.lmax = std::max(L, std::max(l3, l4));
        s.nl2 = nl2;
        s.l3max = l3;
        s.l4max = l4;
        s.inv = inv;
        s.fp_off = r.size;
        s.size = s.np * sl;
        s.rcut = rcA;
        s.W.assign((size_t)T * s.np * (bA + 1), 0.0);
        for (int tn = 0; tn < T; ++tn)
            for (int n = 0; n <= nA; ++n)
                for (int k = 0; k <= bA; ++k)
                    s.W[((size_t)tn * s.np + n) * (bA + 1) + k] = c[ncR + (n * (bA + 1) + k) * T * T + t * T + tn];
        if (tw)
            for (int tn = 0; tn < T; ++tn) {
                r.pair_rc.push_back(pair_cut(rcR, fR, t, tn));
                s.pair_rc.push_back(pair_cut(rcA, fA, t, tn));
            }
        sp.subs = {r, s};
        sp.D = D;
        // network: one tanh layer of H units
        const double* w = v.data() + (version == 3 ? 0 : (size_t)t * per);
        sp.hidden = {H};
        sp.Wh.assign(1, std::vector<double>((size_t)H * D, 0.0));
        sp.bh.assign(1, std::vector<double>(H, 0.0));
        for (int h = 0; h < H; ++h) {
            for (int d = 0; d < dim; ++d) sp.Wh[0][(size_t)h * D + col[d]] = w[(size_t)h * dim + d];
            sp.bh[0][h] = -w[(size_t)H * dim + h];
        }
        sp.wo.assign(w + (size_t)H * dim + H, w + (size_t)H * dim + 2 * H);
        sp.bo = -b1 - (version == 5 ? w[(size_t)H * dim + 2 * H] : 0.0);
        sp.mu.assign(D, 0.0);
        sp.sigma.assign(D, 1.0);
        for (int d = 0; d < dim; ++d) {
            const double f = qs[d] * kap[d];
            if (!(f != 0.0) || !std::isfinite(f)) bad("descriptor scales must be finite and nonzero");
            sp.sigma[col[d]] = 1.0 / f;
        }
        sp.mu_e = 0.0;
        sp.sigma_e = 1.0;
        m.sp.push_back(std::move(sp));
    }
    return m;
}

}  // namespace nnapgb
