// hfx_scf.hpp -- SCF driver interface (host C++).
#pragma once

#include <functional>
#include <vector>

#include "hfx_internal.hpp"

namespace hfx {

// G builder: P -> G = J[P] - 1/2 K[P]; `final` marks the final-check build.
using GBuilder = std::function<void(const double* P, double* G, bool final)>;
// UHF builder: (Pa, Pb) -> J[Pa+Pb], K[Pa], K[Pb].
using JKBuilder = std::function<void(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb, bool final)>;

struct ScfOutput {
    double E_tot = 0, E_ele = 0, E_nuc = 0, E_prev = 0, last_rmsd = 0;
    int iterations = 0;
    bool converged = false;
    int K = 0, n_electrons = 0;
    int fock_builds = 0;
    double seconds = 0;
    std::vector<double> P, P2, C, e, e2;
};

// Per-molecule setup of the SCF (S, H = T + V, X = S^-1/2, E_nuc), computed
// once and reusable across SCFs of the same geometry.
struct ScfSetup {
    int K = 0;
    std::vector<double> S, H, X;
    double E_nuc = 0.0;
};
ScfSetup scf_setup(const Basis& b);

ScfOutput rhf_diis(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt, const double* P0,
                   const GBuilder& g);
ScfOutput uhf_diis(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt, int na, int nb,
                   const double* Pa0, const double* Pb0, const JKBuilder& jk);

ScfOutput rhf_diis(const Basis& b, const hfx_scf_options& opt, const double* P0, const GBuilder& g);
ScfOutput uhf_diis(const Basis& b, const hfx_scf_options& opt, int na, int nb, const double* Pa0, const double* Pb0,
                   const JKBuilder& jk);

}  // namespace hfx
