// Host-side NNAP model: parsed from the reference's JSON model format and packed
// into the per-species blocks the GPU kernels consume.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "invariants.hpp"

namespace nnapgb {

enum { KIND_RADIAL = 0, KIND_SPHERICAL = 1 };

// One (possibly merged) sub-basis of a species.  W is the internal radial-fuse
// matrix W[t_nei-1][np][n] (WTypeBasis.java:202-304); the descriptor entries of this
// sub-basis start at fp_off within the species' descriptor.
struct SubBasis {
    int kind = KIND_SPHERICAL;
    // lmax: largest l of the expansion A (the largest of the file's lmax, l3max, l4max);
    // nl2: power-spectrum columns per channel (the file's lmax + 1), followed by the
    // invariant columns inv (l3max / l4max) of the same channel
    int nmax = 5, lmax = 0, np = 0, nl2 = 1, l3max = 0, l4max = 0;
    std::vector<std::vector<InvTerm>> inv;
    int fp_off = 0, size = 0;
    double rcut = 6.0;
    std::vector<double> pair_rc;  // NEP type-wise cutoffs: per neighbour species (<= rcut), or empty
    bool fused = false;     // wtype fuse / rfuse / exfuse: the matrix is a trainable parameter
    std::vector<double> W;  // T * np * (nmax+1)
};

struct Species {
    std::string symbol;
    std::vector<SubBasis> subs;
    int D = 0;                               // descriptor length
    std::vector<int> hidden;                 // hidden widths
    std::vector<std::vector<double>> Wh;     // per layer, row-major [out][in]
    std::vector<std::vector<double>> bh;     // per layer
    std::vector<double> wo;                  // output weights
    double bo = 0.0;                         // output bias
    std::vector<double> mu, sigma;           // descriptor normalisation
    double mu_e = 0.0, sigma_e = 1.0;        // energy denormalisation (mu includes ref_eng)
    int basis_src = 0;                       // mirror / shared basis: 1-based source species (0: own)
    bool basis_mirror = false;               // the basis is a mirror of basis_src's
};

// NEP's ZBL short-range term (nepV_zbl): per pair r < 2.5 A, the screened Coulomb
// repulsion with the universal screening function and a cosine switch from rc_inner to
// rc_outer (fixed form), or ten per-species-pair parameters [rc_inner, rc_outer, a1, b1,
// .., a4, b4] (flexible form); see k_zbl.cu.
struct ZblModel {
    bool on = false, flexible = false;
    double rc_inner = 0.0, rc_outer = 0.0;
    std::vector<int> z;        // atomic number of each species
    std::vector<double> para;  // flexible: 10 per pair (t1 <= t2, row-major upper triangle)
    std::vector<double> pair_rc;  // fixed form, type-wise radii: [T][T][2] (rc_inner, rc_outer), or empty
};

struct Model {
    std::vector<Species> sp;
    std::string units;
    double rcut_max = 0.0;
    ZblModel zbl;
    int radial_fn = 0;  // radial functions of every sub-basis: 0 NNAP Chebyshev, 1 NEP
    int act = 0;        // hidden activation of every network: 0 SiLU, 1 tanh (NEP)
    int ntypes() const { return (int)sp.size(); }
};

// Parse (JSON, or YAML for text that does not start with '{') and pack; throws
// std::runtime_error with a message on invalid input.
Model load_model(const char* text, size_t len);
// FNV-1a digest of everything the kernels consume from a model.
uint64_t model_digest(const Model& M);

// A valid NEP file of a variant the GPU path does not evaluate (dipole, polarizability).
struct NepUnsupported : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Parse a NEP potential file (nep.txt) into the equivalent NNAP-pipeline model (see
// nep_model.cpp); throws std::runtime_error on invalid input and NepUnsupported.
Model load_nep_model(const char* text, size_t len);

}  // namespace nnapgb
