"""The lockstep batched SCF (one packed Fock build per cycle over every
molecule still iterating) gives each molecule the energy and iteration count
of its own SCF: energies within 1 uHa, iterations within +-1, for mixed
sizes and basis sets, RHF and UHF, and with fewer parallel slots than
molecules (molecules joining and leaving the packed job)."""
import numpy as np
import pytest

import hartree_fock_cpp_gb300 as H
from hartree_fock_cpp_gb300 import workloads as W

pytestmark = pytest.mark.gpu
E_TOL = 1e-6


def _rhf_mix():
    mols = [(cfg, "cc-pVTZ") for cfg in W.nacl_scan(8)[::3]]          # f functions, K=78
    mols += [(cfg, "6-31G*") for cfg in W.water_scan(6)[::2]]          # K=19
    mols += [(W.water(), "STO-3G"), (W.benzene(), "cc-pVDZ")]
    return mols


@pytest.mark.parametrize("max_parallel", [0, 3])
def test_batch_rhf_matches_single_runs(max_parallel):
    mols = _rhf_mix()
    res, st = H.batch_scf(mols, max_parallel=max_parallel)
    assert st["molecules"] == len(mols) and st["cycles"] > 0
    for (cfg, bs), r in zip(mols, res):
        a = H.rhf_diis(cfg, bs)
        assert r["converged"] and a["converged"]
        assert abs(r["E_tot"] - a["E_tot"]) < E_TOL, (bs, r["E_tot"], a["E_tot"])
        assert abs(r["iterations"] - a["iterations"]) <= 1


def test_batch_uhf_matches_single_runs():
    oh = [[("O", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, r))] for r in (1.7, 1.83, 2.0)]
    nh2 = [("N", (0.0, 0.0, 0.0)), ("H", (0.0, 1.5, 1.1)), ("H", (0.0, -1.5, 1.1))]
    mols = [(c, "6-31G*") for c in oh] + [(nh2, "cc-pVDZ")]
    spins = [(5, 4)] * 3 + [(5, 4)]
    res, st = H.batch_scf(mols, method="UHF", spins=spins)
    for (cfg, bs), sp, r in zip(mols, spins, res):
        a = H.uhf_diis(cfg, bs, spin_occ=sp)
        assert r["converged"] and a["converged"]
        assert abs(r["E_tot"] - a["E_tot"]) < E_TOL
        assert abs(r["iterations"] - a["iterations"]) <= 1


def test_batch_mixed_precision_within_1uha_of_fp64():
    mols = [(cfg, "cc-pVDZ") for cfg in W.water_scan(4)] + [(W.benzene(), "cc-pVDZ")]
    kw = dict(epsilon=1e-7, energy_threshold=1e-8)
    r64, _ = H.batch_scf(mols, **kw)
    rmx, _ = H.batch_scf(mols, precision=H.HFX_PREC_MIXED, fp32_threshold=1e-1, **kw)
    for a, b in zip(r64, rmx):
        assert a["converged"] and b["converged"]
        assert abs(a["E_tot"] - b["E_tot"]) < E_TOL
    assert sum(b["mixed_builds"] for b in rmx) > 0


def test_batch_warm_chains_match_sequential_warm_started_scan():
    """warm_chain = 3: chains of three consecutive scan points, each point
    starting from the previous point's final density while the chains iterate
    together; every point matches the sequential scan that starts each point
    from the previous one (run_bl_scan, run.hpp:353-368) in energy (1 uHa)
    and iteration count (+-1)."""
    pts = W.water_scan(6)
    mols = [(cfg, "cc-pVDZ") for cfg in pts]
    res, st = H.batch_scf(mols, warm_chain=3)
    assert st["molecules"] == 6
    for chain in (range(0, 3), range(3, 6)):
        P = None
        for i in chain:
            a = H.rhf_diis(pts[i], "cc-pVDZ", set_initial_density=P is not None, P0=P)
            P = a["density"]
            r = res[i]
            assert r["converged"] and a["converged"]
            assert abs(r["E_tot"] - a["E_tot"]) < E_TOL
            assert abs(r["iterations"] - a["iterations"]) <= 1, (i, r["iterations"], a["iterations"])
    # warm-started points need fewer iterations than the chain heads
    assert res[1]["iterations"] < res[0]["iterations"]


def test_batch_warm_chain_matches_reference_loop_fixture():
    """Two consecutive water/cc-pVTZ scan points in one chain: the second
    point's iteration count is the reference loop's warm-started count
    (tests/golden/scf_golden.json, from the reference's own tensor)."""
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scf_golden.json")))
    head, warm = g["water_ccpvtz_20"], g["water_ccpvtz_21_warm"]
    cfg = lambda c: [(s, tuple(x)) for s, x in c["config"]]
    res, _ = H.batch_scf([(cfg(head), "cc-pVTZ"), (cfg(warm), "cc-pVTZ")], warm_chain=2)
    for r, c in ((res[0], head), (res[1], warm)):
        # the reference loop over the accurate-Boys tensor where the fixture has it
        E, it = c.get("E_tot_stable", c["E_tot"]), c.get("iterations_stable", c["iterations"])
        assert abs(r["E_tot"] - E) < E_TOL
        assert abs(r["iterations"] - it) <= 1, (r["iterations"], it)
