"""Electron density and orbitals on grids (GPU) against the oracle's
restatement of the reference's function_eval / electron_density /
orbital_wf (cube.hpp:9-135) on the reference's box_points grid."""
import os

import numpy as np
import pytest

import oracle as O
import hartree_fock_cpp_gb300 as H
from hartree_fock_cpp_gb300 import cube, workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,basis", [(W.water(), "cc-pVDZ"), (W.nacl_scan(8)[3], "cc-pVTZ")])
def test_density_and_orbitals_on_a_box_match_oracle(cfg, basis):
    b = H.basis_construction(cfg, basis)
    fb = O.FlatBasis(cfg, basis)
    rng = np.random.default_rng(3)
    P = rng.normal(size=(b.K, b.K)) * 0.1
    P = P + P.T
    C = rng.normal(size=(b.K, b.K))
    center, L, res = (0.1, -0.2, 0.3), 9.0, 11
    pts = O.box_points(center, L, res)
    rho = cube.density3d(b, P, center, L, res)
    ref = O.electron_density(fb, P, pts)
    assert np.abs(rho["field"] - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    psi = cube.orbital3d(b, C, 5, center, L, res)
    ref = O.orbital_wf(fb, C, 5, pts)
    assert np.abs(psi["field"] - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    assert rho["res"] == res and abs(rho["dx"] - L / (res - 1)) < 1e-15


def test_points_and_density_of_a_converged_scf_integrates_to_n_electrons(tmp_path):
    cfg = W.water()
    r = H.rhf_diis(cfg, "6-31G*")
    b = H.basis_construction(cfg, "6-31G*")
    # explicit points: a plane through the molecule
    xy = np.stack(np.meshgrid(np.linspace(-3, 3, 7), np.linspace(-3, 3, 7), indexing="ij"), -1).reshape(-1, 2)
    pts = np.concatenate([xy, np.zeros((xy.shape[0], 1))], axis=1)
    fb = O.FlatBasis(cfg, "6-31G*")
    v = cube.points_eval(b, r["density"], pts)
    assert np.abs(v - O.electron_density(fb, r["density"], pts)).max() < 1e-12
    # integral of rho over a large box ~ number of electrons (the plain sum
    # at dx = 0.15 bohr under-samples the oxygen 1s cusp by about 0.6%)
    res, L = 96, 14.0
    rho = cube.density3d(b, r["density"], (0.0, 0.0, 0.0), L, res)
    n = rho["field"].sum() * rho["dx"] ** 3
    assert abs(n - 10.0) < 0.1
    f = os.path.join(tmp_path, "density.cube")
    cube.write_cube_file(f, cube.density3d(b, r["density"], (0, 0, 0), 6.0, 4), cfg)
    lines = open(f).read().splitlines()
    assert lines[2].split()[0] == "3" and lines[3].split()[0] == "4"
    assert len(lines[6 + 3].split()) == 6


def test_grid_kernels_match_reference_golden():
    """Box grids and explicit points on the GPU against the reference's own
    cube.hpp evaluation (tests/golden/grid_golden.json): 1e-12 relative to the
    field's largest value."""
    import json
    g = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grid_golden.json")))
    for c in g:
        cfg = [(s, tuple(x)) for s, x in c["config"]]
        b = H.basis_construction(cfg, c["basis"])
        K = b.K
        i, j = np.meshgrid(np.arange(K), np.arange(K), indexing="ij")
        P = np.cos(0.37 * i + 0.53 * j) + np.cos(0.37 * j + 0.53 * i)
        C = np.sin(0.11 * i * j + 0.7 * i)
        rho = cube.density3d(b, P, tuple(c["center"]), c["L"], c["res"])["field"].ravel()
        psi = cube.orbital3d(b, C, c["column"], tuple(c["center"]), c["L"], c["res"])["field"].ravel()
        for got, ref in ((rho, c["rho_box"]), (psi, c["psi_box"])):
            ref = np.array(ref)
            assert np.abs(got - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
        pts = np.array(c["points"])
        for got, ref in ((cube.points_eval(b, P, pts), c["rho_points"]),
                         (cube.points_eval(b, C, pts, index=c["column"]), c["psi_points"])):
            ref = np.array(ref)
            assert np.abs(got - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
