// hfx_scf.hpp -- SCF driver interface (host C++).
#pragma once

#include <functional>
#include <vector>

#include "hfx_internal.hpp"

namespace hfx {

// Build modes requested by the drivers.
enum BuildMode {
    BUILD_DEFAULT = 0,      // the job's own precision plan (FP64, or mixed FP32/FP64)
    BUILD_FP64 = 1,         // every quartet in FP64
    BUILD_FP64_DELTA = 2    // FP64 build of a density difference, density-weighted screening
};
// G builder: P -> G = J[P] - 1/2 K[P] (linear in P).
using GBuilder = std::function<void(const double* P, double* G, int mode)>;
// UHF builder: (Pa, Pb) -> J[Pa+Pb], K[Pa], K[Pb].
using JKBuilder = std::function<void(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb, int mode)>;

// When the mixed-precision SCF leaves its FP32 phase.  The FP32 quartets put
// a floor under the commutator error ||FPS - SPF|| that the convergence test
// cannot pass, so the last cycles run in FP64 (one full build, then FP64
// builds of the density change).  The switch comes once the error norm is
// below kSwitchFactor * epsilon -- early enough that the FP32 error (~1e-7 in
// F) is small against the remaining error, so the DIIS history built in FP32
// still serves the FP64 cycles and the iteration count stays that of an FP64
// SCF -- or when the error norm stops falling (no new low by at least 10% in
// four iterations) after it has come below kStallFloor, where an FP32 error
// floor holds the SCF back.  (Above that floor the reference's DIIS can
// itself pause for a few iterations with an unchanged density, in FP64 too.)
class MixedPhaseSwitch {
public:
    explicit MixedPhaseSwitch(double epsilon) : tol_(kSwitchFactor * epsilon) {}
    // true once the FP32 phase should end; call once per iteration
    bool update(double rmsd, double err_norm)
    {
        ++n_;
        if (n_ < kFirstTracked) return false;   // zero-density start, damped iterations
        (void)rmsd;
        if (err_norm < tol_) return true;
        if (err_norm < 0.9 * best_) {
            best_ = err_norm;
            since_ = 0;
        } else {
            ++since_;
        }
        return best_ < kStallFloor && since_ >= kStallIterations;
    }
    static constexpr double kSwitchFactor = 1000.0;
    static constexpr double kStallFloor = 1e-3;   // ||FPS - SPF|| (Eh)
    static constexpr int kStallIterations = 4;
    static constexpr int kFirstTracked = 4;        // the first DIIS iteration

private:
    double tol_;
    double best_ = 1e300;
    int n_ = 0, since_ = 0;
};

struct ScfOutput {
    double E_tot = 0, E_ele = 0, E_nuc = 0, E_prev = 0, last_rmsd = 0;
    int iterations = 0;
    bool converged = false;
    int K = 0, n_electrons = 0;
    int fock_builds = 0;
    int mixed_builds = 0, fp64_builds = 0, delta_builds = 0;
    int projections = 0, projection_fallbacks = 0;
    double seconds = 0;
    double fock_ms = 0;
    std::vector<double> P, P2, C, e, e2;
};

// Per-molecule setup of the SCF (S, H = T + V, X = S^-1/2, E_nuc), computed
// once and reusable across SCFs of the same geometry.
struct ScfSetup {
    int K = 0;
    std::vector<double> S, H, X;
    double E_nuc = 0.0;
};
// gpu: S, T, V on the current CUDA device instead of the host
ScfSetup scf_setup(const Basis& b, bool gpu = false);

ScfOutput rhf_diis(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt, const double* P0,
                   const GBuilder& g);
ScfOutput uhf_diis(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt, int na, int nb,
                   const double* Pa0, const double* Pb0, const JKBuilder& jk);

ScfOutput rhf_diis(const Basis& b, const hfx_scf_options& opt, const double* P0, const GBuilder& g);
ScfOutput uhf_diis(const Basis& b, const hfx_scf_options& opt, int na, int nb, const double* Pa0, const double* Pb0,
                   const JKBuilder& jk);

}  // namespace hfx
