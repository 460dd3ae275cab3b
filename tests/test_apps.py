"""The JSON apps (single_run / bl_scan / dissociation): option parsing and
validation as include/run.hpp (CPU), and end-to-end runs on the GPU engine
against the reference's published STO-3G curves."""
import json
import math
import os

import numpy as np
import pytest

from hartree_fock_cpp_gb300 import apps, BASIS_PATH

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _write(tmp_path, d, name="in.json"):
    p = tmp_path / name
    p.write_text(json.dumps(d))
    return str(p)


def test_read_scf_options_defaults_and_polar(tmp_path):
    p = _write(tmp_path, {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G",
                          "atoms": [{"symbol": "H", "position": [0, 0, 0]},
                                    {"symbol": "H", "coordinate_type": "polar", "position": [1.4, 90.0, 0.0]}]})
    o = apps.read_scf_options(p)
    assert o["method"] == "RHF" and o["folder_name"] == "test" and o["charge"] == 0
    assert o["eri_device"] == "CPU" and o["max_it"] == 10000 and o["epsilon"] == 1e-6
    assert o["damping"] == 0.3 and o["screening_threshold"] == 1e-8
    x, y, z = o["config"][1][1]
    assert abs(x - 1.4) < 1e-12 and abs(y) < 1e-12 and abs(z) < 1e-12


@pytest.mark.parametrize("missing", ["basis_path", "save_path", "basis", "atoms"])
def test_read_scf_options_required_keys(tmp_path, missing):
    d = {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G",
         "atoms": [{"symbol": "H", "position": [0, 0, 0]}]}
    del d[missing]
    with pytest.raises(RuntimeError, match="Missing required JSON field: " + missing):
        apps.read_scf_options(_write(tmp_path, d))


def test_uhf_needs_spin_occupancy_and_coordinate_type_checked(tmp_path):
    d = {"method": "UHF", "basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G",
         "atoms": [{"symbol": "H", "position": [0, 0, 0]}]}
    with pytest.raises(RuntimeError, match="spin_occupancy"):
        apps.read_scf_options(_write(tmp_path, d))
    d = {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G",
         "atoms": [{"symbol": "H", "coordinate_type": "spherical", "position": [0, 0, 0]}]}
    with pytest.raises(RuntimeError, match="Unknown coordinate_type"):
        apps.read_scf_options(_write(tmp_path, d))


def test_blscan_options_and_distance_segments(tmp_path):
    d = {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G", "central_atom": "H",
         "atoms": [{"symbol": "H", "angular_position": [0.0, 0.0]}],
         "distances": [[0.5, 1.1, 4], [1.1, 1.7, 3]]}
    o = apps.read_blscan_options(_write(tmp_path, d))
    dist = apps.scan_distances(o["distances"])
    assert np.allclose(dist, [0.5, 0.7, 0.9, 1.1, 1.4, 1.7])
    bad = dict(d, distances=[[1.0, 0.5, 3]])
    with pytest.raises(RuntimeError, match="stop must be larger"):
        apps.read_blscan_options(_write(tmp_path, bad))
    bad = dict(d, distances=[[0.5, 1.0, 1]])
    with pytest.raises(RuntimeError, match="at least 2"):
        apps.read_blscan_options(_write(tmp_path, bad))
    g = apps.scan_geometry(o, 1.4)
    assert g[0] == ("H", (0.0, 0.0, 0.0)) and abs(g[1][1][2] - 1.4) < 1e-12


def test_cpu_eri_device_is_rejected():
    import hartree_fock_cpp_gb300 as H
    with pytest.raises(H.HfxError):
        H.rhf_diis([("H", (0, 0, 0)), ("H", (1.4, 0, 0))], "STO-3G", eri_device="CPU")


@pytest.mark.gpu
def test_single_run_water(tmp_path):
    d = {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G", "eri_hardware": "GPU",
         "folder_name": "w", "atoms": [{"symbol": s, "position": list(p)} for s, p in
                                       [("O", (0, 0, 0.2217)), ("H", (0, 1.4309, -0.8867)),
                                        ("H", (0, -1.4309, -0.8867))]]}
    r = apps.run_scf_from_options(apps.read_scf_options(_write(tmp_path, d)))
    meta = json.load(open(tmp_path / "w" / "metadata.json"))
    assert meta["converged"] and abs(meta["total_energy"] - r["E_tot"]) < 1e-12
    assert meta["n_basis"] == 7


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_bl_scan_h2_against_reference_curve(tmp_path, batched):
    gold = [e for e in json.load(open(os.path.join(GOLD, "reference_energies.json"))) if e["curve"] == "H2_vr"]
    Rs = sorted(g["R"] for g in gold)[:3]
    d = {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G", "central_atom": "H",
         "eri_hardware": "GPU", "atoms": [{"symbol": "H", "angular_position": [90.0, 0.0]}],
         "distances": [[Rs[0], Rs[1], 2], [Rs[1], Rs[2], 2]]}
    r = apps.run_bl_scan(apps.read_blscan_options(_write(tmp_path, d)), batched=batched)
    ref = {g["R"]: g["E"] for g in gold}
    for R, E in zip(r["distances"], r["energies"]):
        assert abs(E - ref[min(ref, key=lambda x: abs(x - R))]) < 1e-6
    assert (tmp_path / "test" / "scan_data.csv").exists()


@pytest.mark.gpu
def test_dissociation_h2(tmp_path):
    d = {"basis_path": BASIS_PATH, "save_path": str(tmp_path), "basis": "STO-3G", "eri_hardware": "GPU",
         "atoms": [{"symbol": "H", "position": [0, 0, 0]}, {"symbol": "H", "position": [1.4, 0, 0]}]}
    r = apps.run_dissociation(apps.read_scf_options(_write(tmp_path, d)))
    # H atom (STO-3G, UHF) and H2 at 1.4 bohr
    assert abs(r["atom_energies"]["H"] - (-0.466581849557)) < 1e-6
    assert r["dissociation_energy"] > 0.1
