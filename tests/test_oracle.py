"""The oracle (C restatement of the reference's integrals.hpp / linalg.hpp
plus the numpy SCF restatement) pinned against the reference's own outputs:
golden fixtures made from the reference compiled unchanged, and the
reference's published STO-3G energy curves."""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return json.load(open(os.path.join(GOLD, name)))


def test_water_sto3g_tensor_matches_reference_exactly():
    g = _load("water_sto3g.json")
    orc = O.Oracle([tuple(a) for a in g["config"]], g["basis"])
    assert orc.K == g["K"] == 7
    eri = orc.repulsion_tensor(g["threshold"])
    ref = np.array(g["eri"])
    assert eri.shape == ref.shape == (406,)
    assert np.abs(eri - ref).max() == 0.0
    # (O1s O1s|O1s O1s)
    assert abs(eri[0] - 4.785065752279990) < 1e-14


def test_water_sto3g_schwarz_and_one_electron():
    g = _load("water_sto3g.json")
    orc = O.Oracle([tuple(a) for a in g["config"]], g["basis"])
    assert np.abs(orc.schwarz_bounds() - np.array(g["schwarz"])).max() == 0.0
    S, T, V = orc.one_electron()
    for M, key in ((S, "S"), (T, "T"), (V, "V")):
        assert np.abs(M.ravel() - np.array(g[key])).max() < 1e-13


@pytest.mark.parametrize("idx", range(5))
def test_eri_samples_match_reference(idx):
    s = _load("eri_samples.json")[idx]
    orc = O.Oracle([tuple(a) for a in s["config"]], s["basis"])
    assert orc.K == s["K"]
    n = 40 if s["K"] > 100 else len(s["quartets"])
    vals = orc.eri_list(s["quartets"][:n])
    ref = np.array(s["eri"][:n])
    assert np.abs(vals - ref).max() <= 1e-14 * max(1.0, np.abs(ref).max())


def test_boys_reference_vs_stable():
    # the reference's upward recursion agrees with an accurate F_m where it is
    # well conditioned and loses digits for moderate T and high m
    L = O.lib()
    for m in range(0, 4):
        for T in (0.5, 2.0, 10.0, 30.0):
            a, b = L.orc_boys_reference(m, T), L.orc_boys_stable(m, T)
            assert abs(a - b) <= 1e-13 * max(1.0, abs(b))
    assert abs(L.orc_boys_reference(8, 0.1) - L.orc_boys_stable(8, 0.1)) > 1e-9 * L.orc_boys_stable(8, 0.1)


def test_contraction_symmetry_and_consistency():
    g = _load("water_sto3g.json")
    K = 7
    eri = np.array(g["eri"])
    rng = np.random.default_rng(3)
    P = rng.normal(size=(K, K))
    P = P + P.T
    G = O.repulsion_matrix(P, eri)
    J = O.coulomb_matrix(P, np.zeros_like(P), eri)
    X = O.exchange_matrix(P, eri)
    assert np.abs(G - (J - 0.5 * X)).max() < 1e-12
    full = O.full_eri(eri, K)
    assert np.abs(J - np.einsum("ijkl,kl->ij", full, P)).max() < 1e-12
    assert np.abs(X - np.einsum("ikjl,kl->ij", full, P)).max() < 1e-12


@pytest.mark.parametrize("case", [0, 2, 5, 9, 11, 16])
def test_scf_oracle_reproduces_reference_curves(case):
    e = _load("reference_energies.json")[case]
    res = O.rhf_diis([tuple(a) for a in e["config"]], e["basis"], charge=e["charge"])
    assert res["converged"]
    assert abs(res["E_tot"] - e["E"]) < 1e-6


def test_reference_library_if_present():
    path = os.path.join(O.HERE, "_ref", "libhfref.so")
    if not os.path.exists(path):
        pytest.skip("reference checkout not available here")
    r = O.RefLib()
    cfg = [("O", (0.0, 0.0, 0.2217)), ("H", (0.0, 1.4309, -0.8867)), ("H", (0.0, -1.4309, -0.8867))]
    r.build(cfg, "6-31G*", O.BASIS_PATH)
    orc = O.Oracle(cfg, "6-31G*")
    rng = np.random.default_rng(1)
    for _ in range(20):
        i, j, k, l = (int(x) for x in rng.integers(0, orc.K, 4))
        assert orc.eri(i, j, k, l) == r.eri(i, j, k, l)


def _grid_golden():
    import json
    return json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grid_golden.json")))


def _grid_matrices(K):
    # the closed-form matrices of tests/golden/make_grid_golden.py
    i, j = np.meshgrid(np.arange(K), np.arange(K), indexing="ij")
    return np.cos(0.37 * i + 0.53 * j) + np.cos(0.37 * j + 0.53 * i), np.sin(0.11 * i * j + 0.7 * i)


def test_grid_restatement_matches_reference_golden():
    """The oracle's restatement of function_eval / electron_density /
    orbital_wf / box_points (cube.hpp:9-168) against the reference's own code
    (tests/golden/grid_golden.json, cube.hpp compiled unchanged)."""
    for c in _grid_golden():
        fb = O.FlatBasis([(s, tuple(x)) for s, x in c["config"]], c["basis"])
        assert fb.K == c["K"]
        P, C = _grid_matrices(fb.K)
        box = O.box_points(c["center"], c["L"], c["res"])
        assert np.array_equal(box, np.array(c["box"]))
        for pts, rho, psi in ((box, c["rho_box"], c["psi_box"]), (np.array(c["points"]), c["rho_points"],
                                                                  c["psi_points"])):
            rho, psi = np.array(rho), np.array(psi)
            assert np.abs(O.electron_density(fb, P, pts) - rho).max() < 1e-13 * np.abs(rho).max()
            assert np.abs(O.orbital_wf(fb, C, c["column"], pts) - psi).max() < 1e-13 * max(1.0, np.abs(psi).max())
