// Model-file loader: the reference's JSON model format -> packed per-species blocks.
//
// Keys, defaults and checks follow the reference loader:
//   NNAP.java:129-176 (version <= 6, models[].symbol, default basis spherical_chebyshev,
//   torch key rejected), Basis.java:22-68 (basis types and aliases),
//   Chebyshev.java:33-69 / SphericalChebyshev.java:60-103 (nmax, lmax, l3max, l4max,
//   rcut defaults and limits), MergedBasis.java:193-229 (merged sub-bases),
//   WTypeBasis.java:306-426 (wtype, fuse/rfuse/post_fuse weights, weight
//   standardisation), FeedForward.java:131-221 (network), NNAP.java:270-307
//   (normalisation, ref_eng, norm_mu_eng/norm_sigma_eng taken from the first model
//   that carries them).
#include "model.hpp"

#include <algorithm>

#include <cmath>
#include <stdexcept>

#include "json.hpp"
#include "yaml.hpp"

namespace nnapgb {
namespace {

enum { WT_DEFAULT = 0, WT_NONE = -1, WT_FULL = 2, WT_EXFULL = 3, WT_FUSE = 4, WT_RFUSE = 5, WT_EXFUSE = 6 };

[[noreturn]] void bad(const std::string& m) { throw std::runtime_error(m); }

std::vector<double> num_list(const JValue& v, const char* what) {
    if (v.kind != JValue::ARR) bad(std::string(what) + " must be a list");
    std::vector<double> out;
    out.reserve(v.arr.size());
    for (auto& e : v.arr) {
        if (e.kind == JValue::ARR) {  // row-major nested lists are flattened
            auto sub = num_list(e, what);
            out.insert(out.end(), sub.begin(), sub.end());
        } else {
            out.push_back(e.as_num());
        }
    }
    return out;
}

int size_n(int wt, int T, int nmax, int fuse_size) {
    switch (wt) {
        case WT_EXFULL: return T > 1 ? (T + 1) * (nmax + 1) : nmax + 1;
        case WT_FULL: case WT_RFUSE: return T * (nmax + 1);
        case WT_NONE: return nmax + 1;
        case WT_DEFAULT: return T > 1 ? 2 * nmax + 2 : nmax + 1;
        case WT_FUSE: return fuse_size * (nmax + 1);
        case WT_EXFUSE: return (fuse_size + 1) * (nmax + 1);
    }
    bad("invalid wtype");
}

int parse_wtype(const JValue* v) {
    if (!v) return WT_DEFAULT;
    if (v->kind == JValue::NUM) return (int)v->num;
    const std::string& s = v->as_str();
    if (s == "default") return WT_DEFAULT;
    if (s == "none") return WT_NONE;
    if (s == "full") return WT_FULL;
    if (s == "exfull") return WT_EXFULL;
    if (s == "fuse") return WT_FUSE;
    if (s == "rfuse") return WT_RFUSE;
    if (s == "exfuse") return WT_EXFUSE;
    bad("wtype must be one of default, none, full, exfull, fuse, rfuse, exfuse");
}

double num_or(const JValue& m, const char* k, double d) {
    const JValue* v = m.get(k);
    return v ? v->as_num() : d;
}
bool bool_or(const JValue& m, std::initializer_list<const char*> ks, bool d) {
    const JValue* v = m.get_any(ks);
    if (!v) return d;
    if (v->kind != JValue::BOOL) bad("expected a boolean");
    return v->b;
}

// Typed weight type: with a single species every "plain" type degenerates to none.
int typed_wtype(int wt, int T) {
    if (T == 1 && (wt == WT_EXFULL || wt == WT_FULL || wt == WT_NONE || wt == WT_DEFAULT)) return WT_NONE;
    return wt;
}

// Post-fuse -> rfuse conversion (WTypeBasis.postFuse2RFuse_, WTypeBasis.java:412-526).
std::vector<double> post_fuse_to_rfuse(const std::vector<double>& pw, int wt, int T, int nmax, int sn,
                                       const std::vector<double>& fw, int fuse_size) {
    const int NP = (int)pw.size() / sn, N1 = nmax + 1;
    std::vector<double> out((size_t)T * NP * N1, 0.0);
    const int tw = typed_wtype(wt, T);
    for (int t = 1; t <= T; ++t)
        for (int p = 0; p < NP; ++p) {
            double* L = &out[((size_t)(t - 1) * NP + p) * N1];
            const double* R = &pw[(size_t)p * sn];
            auto addv = [&](const double* src, double w) { for (int n = 0; n < N1; ++n) L[n] += w * src[n]; };
            auto setv = [&](const double* src) { for (int n = 0; n < N1; ++n) L[n] = src[n]; };
            switch (tw) {
                case WT_FUSE: for (int k = 0; k < fuse_size; ++k) addv(R + k * N1, fw[(t - 1) * fuse_size + k]); break;
                case WT_EXFUSE: setv(R); for (int k = 0; k < fuse_size; ++k) addv(R + (k + 1) * N1, fw[(t - 1) * fuse_size + k]); break;
                case WT_FULL: setv(R + (t - 1) * N1); break;
                case WT_EXFULL: setv(R); addv(R + t * N1, 1.0); break;
                case WT_NONE: setv(R); break;
                case WT_DEFAULT: setv(R); addv(R + N1, (t & 1) ? (double)t : -(double)t); break;
                default: bad("invalid wtype for post_fuse");
            }
        }
    return out;
}

SubBasis load_sub(int kind, int T, const JValue& m) {
    SubBasis b;
    b.kind = kind;
    b.nmax = (int)num_or(m, "nmax", 5);
    b.rcut = num_or(m, "rcut", 6.0);
    int l3 = 0, l4 = 0;
    if (kind == KIND_SPHERICAL) {
        b.lmax = (int)num_or(m, "lmax", 6);
        l3 = (int)num_or(m, "l3max", 0);
        l4 = (int)num_or(m, "l4max", 0);
        if (b.lmax < 0 || b.lmax > 12) bad("lmax must be in [0, 12]");
        if (l3 < 0 || l3 > 6) bad("l3max must be in [0, 6]");
        if (l4 < 0 || l4 > 3) bad("l4max must be in [0, 3]");
        if (bool_or(m, {"noradial"}, false)) bad("noradial is invalid");
        if (!bool_or(m, {"l3cross"}, true) || !bool_or(m, {"l4cross"}, true)) bad("no l3cross/l4cross is invalid");
    }
    if (b.nmax < 0 || b.nmax > 20) bad("nmax must be in [0, 20]");
    if (const JValue* fs = m.get("fuse_style"))
        if (fs->as_str() != "limited") bad("no limited fuse_style is invalid");
    if (m.get("rfunc_scales") || m.get("system_scales")) bad("rfunc_scales/system_scales are invalid");
    int wt = parse_wtype(m.get("wtype"));
    const bool ws = bool_or(m, {"weight_standardization", "ws"}, false);
    std::vector<double> fw;
    int fuse_size = 0;
    if (wt == WT_FUSE || wt == WT_EXFUSE) {
        const JValue* fwv = m.get("fuse_weight");
        const JValue* fsv = m.get("fuse_size");
        if (fwv) {
            if (!fsv) {  // legacy column-wise layout
                const auto& cols = fwv->arr;
                if (cols.empty()) bad("empty fuse_weight");
                size_t nr = cols[0].arr.size();
                for (size_t r = 0; r < nr; ++r)
                    for (auto& c : cols) fw.push_back(c.arr.at(r).as_num());
            } else {
                fw = num_list(*fwv, "fuse_weight");
            }
        } else {
            if (!fsv) bad("fuse_weight or fuse_size required for fuse wtype");
            fw.assign((size_t)T * fsv->as_int(), 0.0);
        }
        if (fw.size() % T) bad("size of fuse weight mismatch");
        fuse_size = (int)fw.size() / T;
    }
    int sn = size_n(wt, T, b.nmax, fuse_size);
    std::vector<double> rw;
    double scale = 1.0;
    bool have_rw = false;
    if (wt == WT_RFUSE) {
        if (m.get("post_fuse_size") || m.get("post_fuse_weight")) bad("post_fuse keys are invalid for rfuse");
        if (const JValue* v = m.get("rfuse_weight")) rw = num_list(*v, "rfuse_weight");
        else if (const JValue* s = m.get("rfuse_size")) rw.assign((size_t)s->as_int() * sn, 0.0);
        else bad("rfuse_weight or rfuse_size required for rfuse");
        if (const JValue* s = m.get("rfuse_size"))
            if ((size_t)s->as_int() * sn != rw.size()) bad("size of rfuse weight mismatch");
        scale = num_or(m, "rfuse_scale", 1.0);
        have_rw = true;
    } else {
        const JValue* flag = m.get("post_fuse");
        bool disabled = flag && flag->kind == JValue::BOOL && !flag->b;
        const JValue* pwv = m.get("post_fuse_weight");
        if (!disabled && (flag || m.get("post_fuse_size") || pwv)) {
            if (!pwv) bad("post_fuse_weight is required for post_fuse");
            std::vector<double> pw = num_list(*pwv, "post_fuse_weight");
            scale = num_or(m, "post_fuse_scale", 1.0);
            rw = post_fuse_to_rfuse(pw, wt, T, b.nmax, sn, fw, fuse_size);
            wt = WT_RFUSE;
            fw.clear();
            have_rw = true;
            sn = size_n(WT_RFUSE, T, b.nmax, 0);
        }
    }
    if (have_rw && rw.size() % sn) bad("size of rfuse weight mismatch");
    const int tw = typed_wtype(wt, T);
    const int N1 = b.nmax + 1;
    b.np = have_rw ? (int)(rw.size() / sn) : sn;
    const int NP = b.np;
    b.W.assign((size_t)T * NP * N1, 0.0);
    auto put = [&](int t, int row, int n, double v) { b.W[((size_t)(t - 1) * NP + row) * N1 + n] = v; };
    // Internal radial-fuse matrix (WTypeBasis.updateParameters_, WTypeBasis.java:202-304).
    switch (tw) {
        case WT_RFUSE: {
            if (!ws) {
                b.W = rw;
            } else {
                for (int p = 0; p < NP; ++p) {
                    double norm = 1e-5;
                    for (int t = 1; t <= T; ++t)
                        for (int n = 0; n < N1; ++n) norm += std::fabs(rw[((size_t)(t - 1) * NP + p) * N1 + n]);
                    norm /= sn;
                    for (int t = 1; t <= T; ++t)
                        for (int n = 0; n < N1; ++n) {
                            size_t i = ((size_t)(t - 1) * NP + p) * N1 + n;
                            b.W[i] = rw[i] / norm;
                        }
                }
            }
            for (double& w : b.W) w *= scale;
            break;
        }
        case WT_FUSE:
            for (int t = 1; t <= T; ++t)
                for (int k = 0; k < fuse_size; ++k)
                    for (int n = 0; n < N1; ++n) put(t, k * N1 + n, n, fw[(t - 1) * fuse_size + k]);
            break;
        case WT_EXFUSE:
            for (int t = 1; t <= T; ++t) {
                for (int n = 0; n < N1; ++n) put(t, n, n, 1.0);
                for (int k = 0; k < fuse_size; ++k)
                    for (int n = 0; n < N1; ++n) put(t, (k + 1) * N1 + n, n, fw[(t - 1) * fuse_size + k]);
            }
            break;
        case WT_FULL:
            for (int t = 1; t <= T; ++t)
                for (int n = 0; n < N1; ++n) put(t, (t - 1) * N1 + n, n, 1.0);
            break;
        case WT_EXFULL:
            for (int t = 1; t <= T; ++t)
                for (int n = 0; n < N1; ++n) { put(t, n, n, 1.0); put(t, t * N1 + n, n, 1.0); }
            break;
        case WT_NONE:
            for (int t = 1; t <= T; ++t)
                for (int n = 0; n < N1; ++n) put(t, n, n, 1.0);
            break;
        case WT_DEFAULT:
            for (int t = 1; t <= T; ++t) {
                const double wtv = (t & 1) ? (double)t : -(double)t;
                for (int n = 0; n < N1; ++n) { put(t, n, n, 1.0); put(t, N1 + n, n, wtv); }
            }
            break;
        default: bad("invalid wtype");
    }
    if (kind == KIND_SPHERICAL) {
        // the expansion runs to the largest l any column needs (SphericalChebyshev.java:39-44)
        b.nl2 = b.lmax + 1;
        b.l3max = l3;
        b.l4max = l4;
        b.inv = invariant_columns(l3, l4);
        b.lmax = std::max(b.lmax, std::max(l3, l4));
    }
    b.size = kind == KIND_RADIAL ? NP : NP * (b.nl2 + (int)b.inv.size());
    b.fused = tw == WT_RFUSE || tw == WT_FUSE || tw == WT_EXFUSE;
    return b;
}

int kind_of(const std::string& s) {
    if (s == "spherical_chebyshev" || s == "sph_cheby") return KIND_SPHERICAL;
    if (s == "chebyshev" || s == "cheby") return KIND_RADIAL;
    return -1;
}

// SharedFeedForward.load + updateParameters_ (SharedFeedForward.java:162-339): the base
// network with, in each hidden layer, its first H - S rows and biases replaced by the
// species' own values (zeros when absent); the output layer is the base's when the last
// shared dimension is 1, else the species' own.
void load_shared_network(Species& sp, const Species& base, const JValue& m) {
    if (m.get("shared_flags")) bad("shared in layer nn is invalid now");
    if (const JValue* in = m.get("input_dim"))
        if (in->as_int() != sp.D) bad("input dimension mismatch");
    if (sp.D != base.D) bad("input dimensions mismatch for shared nn");
    const JValue* shv = m.get_any({"shared_hidden_dims", "shared_nnarch"});
    if (!shv) bad("key shared_hidden_dims required for shared_feed_forward");
    std::vector<int> sh;
    for (auto& e : shv->arr) sh.push_back(e.as_int());
    const size_t L = base.hidden.size();
    if (sh.size() == L) sh.push_back(0);
    if (sh.size() != L + 1) bad("the number of hidden layers mismatch");
    const JValue* hw = m.get("hidden_weights");
    const JValue* hb = m.get("hidden_biases");
    if (hw && hw->arr.size() != L) bad("the number of hidden weights mismatch");
    if (hb && hb->arr.size() != L) bad("the number of hidden biases mismatch");
    sp.hidden = base.hidden;
    sp.Wh = base.Wh;
    sp.bh = base.bh;
    int fan = sp.D;
    for (size_t l = 0; l < L; ++l) {
        const int H = base.hidden[l];
        if (sh[l] < 0 || sh[l] > H) bad("invalid shared dimension");
        const int U = H - sh[l];
        for (int o = 0; o < U; ++o) {
            for (int i = 0; i < fan; ++i) sp.Wh[l][(size_t)o * fan + i] = 0.0;
            sp.bh[l][o] = 0.0;
        }
        if (hw) {
            const JValue& rows = hw->arr[l];
            if ((int)rows.arr.size() != U) bad("nrows of hidden weight mismatch");
            for (int o = 0; o < U; ++o) {
                if ((int)rows.arr[o].arr.size() != fan) bad("ncols of hidden weight mismatch");
                for (int i = 0; i < fan; ++i) sp.Wh[l][(size_t)o * fan + i] = rows.arr[o].arr[i].as_num();
            }
        }
        if (hb) {
            std::vector<double> v = num_list(hb->arr[l], "hidden_biases");
            if ((int)v.size() != U) bad("size of hidden bias mismatch");
            for (int o = 0; o < U; ++o) sp.bh[l][o] = v[o];
        }
        fan = H;
    }
    if (sh[L] != 0 && sh[L] != 1) bad("invalid shared output dimension");
    if (sh[L] == 1) {
        sp.wo = base.wo;
        sp.bo = base.bo;
    } else {
        sp.wo.assign(fan, 0.0);
        sp.bo = 0.0;
        if (const JValue* ow = m.get("output_weight")) {
            sp.wo = num_list(*ow, "output_weight");
            if ((int)sp.wo.size() != fan) bad("size of output weight mismatch");
        }
        if (const JValue* ob = m.get("output_bias")) sp.bo = ob->as_num();
    }
}

void load_network(Species& sp, const JValue* nnv) {
    static const JValue empty_obj = [] { JValue v; v.kind = JValue::OBJ; return v; }();
    const JValue& m = nnv ? *nnv : empty_obj;
    if (const JValue* t = m.get("type"))
        if (t->as_str() != "feed_forward") bad("unsupported nn type: " + t->as_str());
    if (const JValue* in = m.get("input_dim"))
        if (in->as_int() != sp.D) bad("input dimension mismatch");
    if (const JValue* h = m.get_any({"hidden_dims", "nnarch"})) {
        for (auto& e : h->arr) sp.hidden.push_back(e.as_int());
    } else {
        sp.hidden = {32, 32};
    }
    if (sp.hidden.empty()) bad("at least one hidden layer is required");
    const JValue* hw = m.get("hidden_weights");
    const JValue* hb = m.get("hidden_biases");
    if (hw && hw->arr.size() != sp.hidden.size()) bad("the number of hidden weights mismatch");
    if (hb && hb->arr.size() != sp.hidden.size()) bad("the number of hidden biases mismatch");
    int fan = sp.D;
    for (size_t l = 0; l < sp.hidden.size(); ++l) {
        const int H = sp.hidden[l];
        std::vector<double> w((size_t)H * fan, 0.0), b(H, 0.0);
        if (hw) {
            const JValue& rows = hw->arr[l];
            if ((int)rows.arr.size() != H) bad("nrows of hidden weight mismatch");
            for (int o = 0; o < H; ++o) {
                if ((int)rows.arr[o].arr.size() != fan) bad("ncols of hidden weight mismatch");
                for (int i = 0; i < fan; ++i) w[(size_t)o * fan + i] = rows.arr[o].arr[i].as_num();
            }
        }
        if (hb) {
            std::vector<double> v = num_list(hb->arr[l], "hidden_biases");
            if ((int)v.size() != H) bad("size of hidden bias mismatch");
            b = v;
        }
        sp.Wh.push_back(std::move(w));
        sp.bh.push_back(std::move(b));
        fan = H;
    }
    sp.wo.assign(fan, 0.0);
    if (const JValue* ow = m.get("output_weight")) {
        sp.wo = num_list(*ow, "output_weight");
        if ((int)sp.wo.size() != fan) bad("size of output weight mismatch");
    }
    if (const JValue* ob = m.get("output_bias")) sp.bo = ob->as_num();
}

// JSON text starts with '{' (a model file is an object); anything else is read as YAML
// (NNAP.java:407-411 reads .yaml / .yml files with IO.yaml2map, IO.java:853).
JValue parse_model_text(const char* text, size_t len) {
    size_t k = 0;
    while (k < len && (text[k] == ' ' || text[k] == '\t' || text[k] == '\n' || text[k] == '\r')) ++k;
    if (k < len && text[k] == '{') {
        try {
            return JParser(text, len).parse();
        } catch (const std::runtime_error& json_error) {
            try {  // a YAML flow mapping (unquoted keys, comments) is not JSON
                return YParser(text, len).parse();
            } catch (const std::runtime_error&) {
                throw json_error;
            }
        }
    }
    return YParser(text, len).parse();
}

}  // namespace

Model load_model(const char* text, size_t len) {
    JValue root = parse_model_text(text, len);
    if (root.kind != JValue::OBJ) bad("model must be a JSON or YAML mapping");
    if (const JValue* v = root.get("version"))
        if (v->as_int() > 6) bad("unsupported model version");
    const JValue* models = root.get("models");
    if (!models || models->kind != JValue::ARR || models->arr.empty()) bad("no models in model file");
    Model M;
    if (const JValue* u = root.get("units")) M.units = u->kind == JValue::STR ? u->str : "";
    const int T = (int)models->arr.size();
    M.sp.resize(T);
    double mu_e = 0.0, sig_e = 1.0;
    bool have_mu = false, have_sig = false;
    // bases: concrete ones first; mirror and shared ones refer to them (Basis.java:22-66)
    enum { PLAIN = 0, MIRROR = 1, SHARE = 2 };
    std::vector<int> bkind(T, PLAIN), bsrc(T, 0), nn_plain(T, 0);
    for (int t = 0; t < T; ++t) {
        const JValue& mm = models->arr[t];
        Species& sp = M.sp[t];
        const JValue* sym = mm.get("symbol");
        if (!sym) bad("no symbol in model");
        sp.symbol = sym->kind == JValue::STR ? sym->str : std::to_string(sym->as_int());
        if (mm.get("torch")) bad("torch model is invalid");
        const JValue* bm = mm.get("basis");
        std::string bt = "spherical_chebyshev";
        if (bm && bm->get("type")) bt = bm->get("type")->as_str();
        static const JValue empty = [] { JValue v; v.kind = JValue::OBJ; return v; }();
        if (bt == "merge" || bt == "merged_basis") {
            const JValue* list = bm->get("basis");
            if (!list || list->arr.empty()) bad("key basis required for merge");
            for (auto& sm : list->arr) {
                std::string st = sm.get("type") ? sm.get("type")->as_str() : "spherical_chebyshev";
                int k = kind_of(st);
                if (k < 0) bad("unsupported basis type: " + st);
                sp.subs.push_back(load_sub(k, T, sm));
            }
        } else if (bt == "mirror" || bt == "mirror_basis" || bt == "share" || bt == "shared_basis") {
            const bool mirror = bt == "mirror" || bt == "mirror_basis";
            const JValue* src = bm->get(mirror ? "mirror" : "share");
            if (!src) bad(mirror ? "key mirror required for mirror_basis" : "key share required for shared_basis");
            bkind[t] = mirror ? MIRROR : SHARE;
            bsrc[t] = src->as_int();
        } else {
            int k = kind_of(bt);
            if (k < 0) bad("unsupported basis type: " + bt);
            sp.subs.push_back(load_sub(k, T, bm ? *bm : empty));
        }
        if (!have_sig) if (const JValue* v = mm.get("norm_sigma_eng")) { sig_e = v->as_num(); have_sig = true; }
        if (!have_mu) if (const JValue* v = mm.get("norm_mu_eng")) { mu_e = v->as_num(); have_mu = true; }
    }
    for (int t = 0; t < T; ++t) {
        if (bkind[t] == PLAIN) continue;
        const int s = bsrc[t];
        // a mirror or shared basis of a mirror or shared basis reads an empty parameter
        // block in the reference's generated code, so only concrete sources are accepted
        if (s < 1 || s > T || bkind[s - 1] != PLAIN) bad("the source of a mirror or shared basis must be a plain basis");
        M.sp[t].subs = M.sp[s - 1].subs;
        M.sp[t].basis_src = s;
        M.sp[t].basis_mirror = bkind[t] == MIRROR;
        if (bkind[t] == MIRROR) {
            // neighbours of the centre's own species and of the mirrored one swap roles
            // (nnap_main.hpp:40-48): W_t[tn] = W_s[sigma(tn)], sigma exchanging t+1 and s
            for (auto& b : M.sp[t].subs) {
                const size_t blk = (size_t)b.np * (b.nmax + 1);
                const std::vector<double> W0 = b.W;
                for (int tn = 1; tn <= T; ++tn) {
                    const int from = tn == s ? t + 1 : (tn == t + 1 ? s : tn);
                    std::copy(W0.begin() + (size_t)(from - 1) * blk, W0.begin() + (size_t)from * blk,
                              b.W.begin() + (size_t)(tn - 1) * blk);
                }
            }
        }
    }
    for (int t = 0; t < T; ++t) {
        Species& sp = M.sp[t];
        int off = 0;
        for (auto& b : sp.subs) { b.fp_off = off; off += b.size; M.rcut_max = std::max(M.rcut_max, b.rcut); }
        sp.D = off;
    }
    // networks: plain feed-forward ones first; a mirror species takes its source's network
    // unchanged, a shared one merges its own rows into its base's (NeuralNetwork.java:24-65)
    for (int t = 0; t < T; ++t) {
        const JValue* nnv = models->arr[t].get("nn");
        if (bkind[t] == MIRROR) {
            if (nnv) bad("nn data of a mirror basis must be empty");
            continue;
        }
        if (nnv && nnv->get("type") && nnv->get("type")->as_str() == "shared_feed_forward") continue;
        load_network(M.sp[t], nnv);
        nn_plain[t] = 1;
    }
    for (int t = 0; t < T; ++t) {
        if (nn_plain[t]) continue;
        Species& sp = M.sp[t];
        const JValue* nnv = models->arr[t].get("nn");
        const int s = bkind[t] == MIRROR ? bsrc[t] : (nnv->get("share") ? nnv->get("share")->as_int() : 0);
        if (s < 1 || s > T || !nn_plain[s - 1]) bad("a shared network needs a plain feed_forward source");
        const Species& base = M.sp[s - 1];
        if (bkind[t] == MIRROR) {
            sp.hidden = base.hidden;
            sp.Wh = base.Wh;
            sp.bh = base.bh;
            sp.wo = base.wo;
            sp.bo = base.bo;
        } else {
            load_shared_network(sp, base, *nnv);
        }
    }
    for (int t = 0; t < T; ++t) {
        const JValue* mmp = &models->arr[t];
        Species& sp = M.sp[t];
        if (bkind[t] == MIRROR) {  // normalisation of the mirrored species (NNAP.java:281-289)
            if (mmp->get("ref_eng")) bad("ref_eng of a mirror basis must be empty");
            if (mmp->get_any({"norm_vec", "norm_sigma", "norm_mu"})) bad("normalisation of a mirror basis must be empty");
            mmp = &models->arr[bsrc[t] - 1];
        }
        const JValue& mm = *mmp;
        const double ref = mm.get("ref_eng") ? mm.get("ref_eng")->as_num() : 0.0;
        sp.mu_e = mu_e + ref;
        sp.sigma_e = sig_e;
        sp.mu.assign(sp.D, 0.0);
        sp.sigma.assign(sp.D, 1.0);
        if (const JValue* v = mm.get("norm_mu")) {
            sp.mu = num_list(*v, "norm_mu");
            if ((int)sp.mu.size() != sp.D) bad("size of norm_mu mismatch");
        }
        if (const JValue* v = mm.get_any({"norm_sigma", "norm_vec"})) {
            sp.sigma = num_list(*v, "norm_sigma");
            if ((int)sp.sigma.size() != sp.D) bad("size of norm_sigma mismatch");
        }
    }
    return M;
}

// 64-bit FNV-1a over every value the kernels consume (basis shapes and matrices, network
// weights, normalisation, cutoffs), in a fixed order: equal digests mean equal models.
uint64_t model_digest(const Model& M) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        for (size_t k = 0; k < n; ++k) { h ^= c[k]; h *= 1099511628211ull; }
    };
    auto num = [&mix](double v) { mix(&v, sizeof v); };
    auto vec = [&](const std::vector<double>& v) { num((double)v.size()); for (double x : v) num(x); };
    num((double)M.ntypes());
    num(M.rcut_max);
    for (const Species& sp : M.sp) {
        mix(sp.symbol.data(), sp.symbol.size());
        num((double)sp.D);
        for (const SubBasis& b : sp.subs) {
            for (int v : {b.kind, b.nmax, b.lmax, b.np, b.nl2, b.l3max, b.l4max, b.fp_off, b.size}) num((double)v);
            num(b.rcut);
            vec(b.W);
            vec(b.pair_rc);
        }
        for (int H : sp.hidden) num((double)H);
        for (auto& w : sp.Wh) vec(w);
        for (auto& b : sp.bh) vec(b);
        vec(sp.wo);
        num(sp.bo);
        vec(sp.mu);
        vec(sp.sigma);
        num(sp.mu_e);
        num(sp.sigma_e);
    }
    return h;
}

}  // namespace nnapgb
