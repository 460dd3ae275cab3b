// hfx_batch.hpp -- lockstep SCFs of several molecules on one packed job
// (hfx_batch.cpp), used by hfx_batch_scf and by the request server's packed
// mode.
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "hfx_dscf.hpp"
#include "hfx_engine.hpp"

namespace hfx {

struct PackedMember {
    hfx_scf_options scf{};
    int n_alpha = 0, n_beta = 0;    // UHF occupations
    const ScfControl* ctl = nullptr;
    // index of the molecule whose final density this one starts from (the
    // reference's scan warm start, run.hpp:353-368), or -1 for the zero
    // density; only the directly preceding molecule (index - 1) is allowed,
    // so that warm-started molecules form chains solved one after another
    int warm_from = -1;
};

struct PackedRunStats {
    double setup_s = 0.0;           // packed job (pair data, Schwarz, plans)
    int builds = 0;                 // packed Fock builds run
    double build_ms = 0.0;          // their device time
    double quartets = 0.0;          // surviving shell quartets of one build, all molecules
    double flops_fp64 = 0.0;
};

// Called from the molecule's own thread when its SCF ends: out is null when
// it failed (status and message say why).
using PackedDone = std::function<void(int index, ScfOutput* out, hfx_status status, const std::string& message)>;

// Runs the SCFs of `bases` (one method: nspin 1 = RHF, 2 = UHF) in lockstep
// on one packed job built with options jo.  Molecules linked by warm_from
// form chains (a chain's molecules run one after another, each from the
// previous one's final density); at most max_parallel chains iterate at once
// (0: all, capped at 256).  Throws only when the packed job
// itself cannot be built; every molecule's own failure goes to done.
PackedRunStats run_packed(const std::vector<Basis>& bases, const hfx_options& jo, int nspin,
                          const std::vector<PackedMember>& members, int max_parallel, const PackedDone& done);

}  // namespace hfx
