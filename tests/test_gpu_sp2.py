"""The device SCF's density step: the SP2 projector (hfx_sp2.cu) against
cuSOLVER syevd.  The reference diagonalises the Fock matrix every iteration
(scf.hpp:205-419, 423-682); the projector gives the same occupied-space
projector, so the SCF must take the same iterations to the same energy, and
the MO energies returned at the end (one syevd of the last Fock matrix) must
be the same.  Without a HOMO-LUMO gap the projector does not converge and the
iteration falls back to syevd."""
import numpy as np
import pytest

import hartree_fock_cpp_gb300 as H
from hartree_fock_cpp_gb300 import workloads as W

pytestmark = pytest.mark.gpu

E_TOL = 1e-9
WATER = [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 1.43, 1.11)), ("H", (0.0, -1.43, 1.11))]


def _pair(run, *args, **kw):
    a = run(*args, eigensolver=H.HFX_EIG_AUTO, **kw)
    b = run(*args, eigensolver=H.HFX_EIG_SYEVD, **kw)
    return a, b


@pytest.mark.parametrize("config,basis", [(WATER, "cc-pVTZ"), (W.benzene(), "cc-pVDZ")])
def test_rhf_projector_matches_syevd(config, basis):
    a, b = _pair(H.rhf_diis, config, basis, epsilon=1e-7, energy_threshold=1e-8)
    assert a["converged"] and b["converged"]
    # a DIIS-extrapolated Fock matrix of the early iterations may have no gap:
    # those iterations take syevd
    assert a["projections"] + a["projection_fallbacks"] == a["iterations"]
    assert a["projections"] >= a["iterations"] - 3
    assert b["projections"] == 0 and b["projection_fallbacks"] == 0
    assert a["iterations"] == b["iterations"]
    assert abs(a["E_tot"] - b["E_tot"]) < E_TOL
    assert np.abs(a["density"] - b["density"]).max() < 1e-8
    assert np.abs(a["mo_energy"] - b["mo_energy"]).max() < 1e-8


def test_uhf_projector_matches_syevd():
    """NH2 radical (C2v, no degenerate levels), 5 alpha and 4 beta electrons."""
    nh2 = [("N", (0.0, 0.0, 0.0)), ("H", (0.0, 1.514, 1.204)), ("H", (0.0, -1.514, 1.204))]
    a, b = _pair(H.uhf_diis, nh2, "6-31G*", spin_occ=(5, 4), epsilon=1e-7)
    assert a["converged"] and b["converged"]
    assert a["projections"] + a["projection_fallbacks"] == 2 * a["iterations"]
    assert a["projections"] >= 2 * a["iterations"] - 3
    assert a["iterations"] == b["iterations"]
    assert abs(a["E_tot"] - b["E_tot"]) < E_TOL


def test_uhf_degenerate_beta_level_matches_syevd():
    """OH radical: the beta electrons fill one of the two degenerate pi
    orbitals, so the iterations with no gap take syevd; the SCF still follows
    the syevd run."""
    oh = [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.83))]
    a, b = _pair(H.uhf_diis, oh, "6-31G*", spin_occ=(5, 4), epsilon=1e-7)
    assert a["converged"] and b["converged"]
    assert a["projection_fallbacks"] >= 1
    assert a["projections"] + a["projection_fallbacks"] == 2 * a["iterations"]
    assert a["iterations"] == b["iterations"]
    assert abs(a["E_tot"] - b["E_tot"]) < E_TOL


def test_batched_scan_projector_matches_syevd():
    mols = [(c, "6-31G") for c in W.water_scan(64)[::16]]
    ra, _ = H.batch_scf(mols, epsilon=1e-7, warm_chain=2, eigensolver=H.HFX_EIG_AUTO)
    rb, _ = H.batch_scf(mols, epsilon=1e-7, warm_chain=2, eigensolver=H.HFX_EIG_SYEVD)
    for a, b in zip(ra, rb):
        assert a["converged"] and b["converged"]
        assert a["projections"] > 0 and b["projections"] == 0
        assert a["iterations"] == b["iterations"]
        assert abs(a["E_tot"] - b["E_tot"]) < E_TOL


def test_degenerate_fermi_level_falls_back_to_syevd():
    """RHF carbon atom: three electron pairs over 1s, 2s and a threefold
    degenerate 2p shell, so the starting Fock matrix has no gap at the Fermi
    level and the projector must hand that iteration to syevd."""
    r = H.rhf_diis([("C", (0.0, 0.0, 0.0))], "6-31G", max_it=6, epsilon=1e-7)
    assert r["projection_fallbacks"] >= 1
    assert r["projections"] + r["projection_fallbacks"] == r["iterations"]
    assert np.isfinite(r["E_tot"])
