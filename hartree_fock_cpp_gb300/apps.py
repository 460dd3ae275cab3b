"""The reference's JSON-driven apps on the GPU engine:

  python -m hartree_fock_cpp_gb300.apps single_run   input.json
  python -m hartree_fock_cpp_gb300.apps bl_scan      input.json [--batched [--warm-chain N]]
  python -m hartree_fock_cpp_gb300.apps dissociation input.json

Input keys, defaults and validation follow include/run.hpp (read_scf_options
:55-125, read_blscan_options :212-296); the SCFs are rhf_diis / uhf_diis with
the direct GPU Fock build.  Outputs keep the reference's file names and keys
(metadata.json, scan_data.csv + scan_info.json, include/save.hpp) for the
quantities this engine produces; density/coefficient CSVs are written as
plain K x K tables.

eri_hardware "GPU" runs the engine; "CPU" names the reference's own
stored-tensor path, which this library does not contain, and is rejected.
bl_scan --batched solves the scan geometries together on one packed job
(batch_scf: one Fock build per SCF cycle over all points still iterating), in
chains of --warm-chain consecutive points that start from the previous
point's density; without it the scan runs point after point with the
previous density as the initial guess, as run_bl_scan does
(run.hpp:329-368).  dissociation solves the free atoms as one UHF batch.
"""
import argparse
import collections
import json
import math
import os
import time

import numpy as np

from . import batch_scf, rhf_diis, uhf_diis, HFX_PREC_FP64, HFX_PREC_MIXED, HfxError

ANGLE = math.pi / 180.0

# run.hpp:457-494
ATOM_SPIN = {"H": (1, 0), "He": (1, 1), "Li": (2, 1), "Be": (2, 2), "B": (3, 2), "C": (4, 2), "N": (4, 3),
             "O": (5, 3), "F": (5, 4), "Ne": (5, 5), "Na": (6, 5), "Mg": (6, 6), "Al": (7, 6), "Si": (8, 6),
             "P": (8, 7), "S": (9, 7), "Cl": (9, 8), "Ar": (9, 9)}


def _require(d, key):
    if key not in d:
        raise RuntimeError("Missing required JSON field: " + key)          # run.hpp:12-18


def polar3d(r, theta, phi):                                                 # types.hpp:207-215
    return (r * math.sin(theta) * math.cos(phi), r * math.sin(theta) * math.sin(phi), r * math.cos(theta))


def _common(d, opt):
    opt["folder_name"] = d.get("folder_name", "test")
    opt["charge"] = d.get("charge", 0)
    opt["eri_device"] = d.get("eri_hardware", "CPU")
    opt["max_it"] = d.get("max_iterations", 10000)
    opt["epsilon"] = d.get("epsilon", 1e-6)
    opt["damping"] = d.get("damping", 0.3)
    opt["screening_threshold"] = d.get("screening_threshold", 1e-8)
    # engine extensions (absent from the reference's files; defaults keep its behaviour)
    opt["precision"] = {"fp64": HFX_PREC_FP64, "mixed": HFX_PREC_MIXED}[d.get("precision", "fp64")]
    opt["fp32_threshold"] = d.get("fp32_schwarz_threshold", 0.0)


def read_scf_options(path):
    """run.hpp:55-125"""
    with open(path) as f:
        d = json.load(f)
    for k in ("basis_path", "save_path", "basis", "atoms"):
        _require(d, k)
    opt = {"method": d.get("method", "RHF"), "basis": d["basis"], "basis_path": d["basis_path"],
           "save_path": d["save_path"]}
    _common(d, opt)
    if opt["method"] == "UHF":
        _require(d, "spin_occupancy")
        opt["n_alpha"] = d["spin_occupancy"]["alpha"]
        opt["n_beta"] = d["spin_occupancy"]["beta"]
    cfg = []
    for a in d["atoms"]:
        ct = a.get("coordinate_type", "cartesian")
        r = a["position"]
        if ct == "cartesian":
            pos = (float(r[0]), float(r[1]), float(r[2]))
        elif ct == "polar":
            pos = polar3d(float(r[0]), float(r[1]) * ANGLE, float(r[2]) * ANGLE)
        else:
            raise RuntimeError("Unknown coordinate_type: " + ct)
        cfg.append((a["symbol"], pos))
    opt["config"] = cfg
    return opt


def _scf_kw(opt):
    return dict(charge=opt["charge"], eri_device=opt["eri_device"], max_it=opt["max_it"], epsilon=opt["epsilon"],
                damping=opt["damping"], screening_threshold=opt["screening_threshold"],
                precision=opt["precision"], fp32_threshold=opt["fp32_threshold"])


def _system_string(symbols):
    c = collections.OrderedDict()
    for s in symbols:
        c[s] = c.get(s, 0) + 1
    return "".join(s + (str(n) if n > 1 else "") for s, n in c.items())


def _save(folder, meta, mats):
    os.makedirs(folder, exist_ok=True)
    with open(os.path.join(folder, "metadata.json"), "w") as f:
        json.dump(meta, f, indent=4)
    for name, m in mats.items():
        np.savetxt(os.path.join(folder, name + ".csv"), np.atleast_2d(m), delimiter=",")


def run_scf_from_options(opt):
    """run.hpp:129-172"""
    t0 = time.time()
    if opt["method"] == "RHF":
        r = rhf_diis(opt["config"], opt["basis"], opt["basis_path"], **_scf_kw(opt))
        mats = {"density": r["density"], "coefficient": r["coefficient"], "orbital_energies": r["mo_energy"]}
    elif opt["method"] == "UHF":
        r = uhf_diis(opt["config"], opt["basis"], opt["basis_path"], spin_occ=(opt["n_alpha"], opt["n_beta"]),
                     **_scf_kw(opt))
        mats = {"density_alpha": r["Pa"], "density_beta": r["Pb"], "orbital_energies_alpha": r["Ea"],
                "orbital_energies_beta": r["Eb"]}
    else:
        raise RuntimeError("Unknown SCF method: " + opt["method"])
    meta = collections.OrderedDict(
        method=opt["method"], basis=opt["basis"], n_basis=r["K"], unit="Hartree", n_iterations=r["iterations"],
        converged=r["converged"], ERI_hardware=opt["eri_device"],
        system=_system_string([s for s, _ in opt["config"]]), charge_e=opt["charge"],
        total_energy=r["E_tot"], electronic_energy=r["E_ele"], nuclear_energy=r["E_nuc"],
        duration_s=time.time() - t0)
    _save(os.path.join(opt["save_path"], opt["folder_name"]), meta, mats)
    return r


def read_blscan_options(path):
    """run.hpp:212-296"""
    with open(path) as f:
        d = json.load(f)
    for k in ("basis_path", "save_path", "basis", "atoms", "central_atom", "distances"):
        _require(d, k)
    opt = {"basis": d["basis"], "basis_path": d["basis_path"], "save_path": d["save_path"],
           "central_atom": d["central_atom"], "method": "RHF"}
    _common(d, opt)
    opt["config"] = []
    for a in d["atoms"]:
        _require(a, "angular_position")
        r = a["angular_position"]
        if not isinstance(r, list) or len(r) != 2:
            raise RuntimeError("angular_position must be [theta, phi]")
        opt["config"].append((a["symbol"], (float(r[0]), float(r[1]))))
    opt["distances"] = []
    for seg in d["distances"]:
        if not isinstance(seg, list) or len(seg) != 3:
            raise RuntimeError("each distance range must be [start, stop, n_points]")
        start, stop, n = float(seg[0]), float(seg[1]), int(seg[2])
        if n < 2:
            raise RuntimeError("distance range n_points must be at least 2")
        if stop <= start:
            raise RuntimeError("distance range stop must be larger than start")
        opt["distances"].append((start, stop, n))
    return opt


def scan_distances(segments):
    """run.hpp:304-322: concatenated linspaces, dropping each segment's first
    point after the first segment."""
    out = []
    for start, stop, n in segments:
        seg = list(np.linspace(start, stop, n))
        if out and seg:
            seg = seg[1:]
        out.extend(seg)
    return out


def scan_geometry(opt, r):
    cfg = [(opt["central_atom"], (0.0, 0.0, 0.0))]
    for sym, (th, ph) in opt["config"]:
        cfg.append((sym, polar3d(r, th * ANGLE, ph * ANGLE)))
    return cfg


def run_bl_scan(opt, batched=False, max_parallel=0, warm_chain=8):
    """run.hpp:300-423.  batched=True solves the points together on one
    packed job (batch_scf: one Fock build per SCF cycle over all points still
    iterating) in chains of warm_chain consecutive points, each point of a
    chain starting from the previous point's density as in the sequential
    scan (warm_chain <= 1: every point from the zero density); homo/lumo are
    then not reported (NaN)."""
    t0 = time.time()
    dist = scan_distances(opt["distances"])
    E, homo, lumo, its = [], [], [], []
    K = None
    if batched:
        kw = _scf_kw(opt)
        kw.pop("eri_device")
        res, _ = batch_scf([(scan_geometry(opt, r), opt["basis"]) for r in dist], max_parallel=max_parallel,
                           param_path=opt["basis_path"], warm_chain=warm_chain, **kw)
        for r in res:
            E.append(r["E_tot"])
            its.append(r["iterations"])
            homo.append(float("nan"))
            lumo.append(float("nan"))
            K = r["K"]
    else:
        P = None
        for r in dist:
            res = rhf_diis(scan_geometry(opt, r), opt["basis"], opt["basis_path"],
                           set_initial_density=P is not None, P0=P, **_scf_kw(opt))
            P = res["density"]
            ne = res["Ne"]
            E.append(res["E_tot"])
            homo.append(float(res["mo_energy"][ne // 2 - 1]))
            lumo.append(float(res["mo_energy"][ne // 2]))
            its.append(res["iterations"])
            K = res["K"]
    out = os.path.join(opt["save_path"], opt["folder_name"])
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(out, "scan_data.csv"), "w") as f:
        f.write("distance,total_energy,homo_energy,lumo_energy,iterations\n")
        for row in zip(dist, E, homo, lumo, its):
            f.write(",".join(repr(float(x)) for x in row) + "\n")
    info = collections.OrderedDict(
        system=_system_string([opt["central_atom"]] + [s for s, _ in opt["config"]]), method="RHF",
        basis=opt["basis"], basis_size=K, n_points=len(dist), min_distance=dist[0], max_distance=dist[-1],
        duration_seconds=time.time() - t0, files={"scan_data": "scan_data.csv"})
    with open(os.path.join(out, "scan_info.json"), "w") as f:
        json.dump(info, f, indent=4)
    return dict(distances=dist, energies=E, homo=homo, lumo=lumo, iterations=its, K=K)


def run_dissociation(opt):
    """run.hpp:498-577: RHF molecule, UHF atoms with atom_spin_occupancy."""
    t0 = time.time()
    if opt["method"] != "RHF":
        raise RuntimeError("dissociation energy only support RHF molecules")
    mol = rhf_diis(opt["config"], opt["basis"], opt["basis_path"], **_scf_kw(opt))
    counts = collections.Counter(s for s, _ in opt["config"])
    for sym in sorted(counts):
        if sym not in ATOM_SPIN:
            raise RuntimeError("Spin occupancy not implemented for atom: " + sym)
    # the free atoms as one UHF batch on a packed job
    kw = _scf_kw(opt)
    kw.pop("eri_device")
    kw["charge"] = 0
    atoms = sorted(counts)
    res, _ = batch_scf([([(sym, (0.0, 0.0, 0.0))], opt["basis"]) for sym in atoms], method="UHF",
                       spins=[ATOM_SPIN[sym] for sym in atoms], param_path=opt["basis_path"], **kw)
    atom_E = {sym: r["E_tot"] for sym, r in zip(atoms, res)}
    Ed = sum(counts[s] * atom_E[s] for s in counts) - mol["E_tot"]
    meta = collections.OrderedDict(
        method="RHF", basis=opt["basis"], n_basis=mol["K"], system=_system_string([s for s, _ in opt["config"]]),
        energy=mol["E_tot"], dissociation_energy=Ed, atoms=sorted(counts),
        atom_numbers=[counts[s] for s in sorted(counts)], atom_energies=[atom_E[s] for s in sorted(counts)],
        duration_s=time.time() - t0)
    _save(os.path.join(opt["save_path"], opt["folder_name"]), meta, {"density": mol["density"]})
    return dict(energy=mol["E_tot"], dissociation_energy=Ed, atom_energies=atom_E)


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m hartree_fock_cpp_gb300.apps")
    ap.add_argument("app", choices=["single_run", "bl_scan", "dissociation"])
    ap.add_argument("input")
    ap.add_argument("--batched", action="store_true", help="bl_scan: the points together on one packed job")
    ap.add_argument("--warm-chain", type=int, default=8,
                    help="bl_scan --batched: consecutive points per warm-started chain (<= 1: all cold)")
    a = ap.parse_args(argv)
    if a.app == "single_run":
        r = run_scf_from_options(read_scf_options(a.input))
        print("E_tot = %.10f  iterations = %d  converged = %s" % (r["E_tot"], r["iterations"], r["converged"]))
    elif a.app == "bl_scan":
        r = run_bl_scan(read_blscan_options(a.input), batched=a.batched, warm_chain=a.warm_chain)
        for d, e in zip(r["distances"], r["energies"]):
            print("%.6f %.10f" % (d, e))
    else:
        r = run_dissociation(read_scf_options(a.input))
        print("dissociation energy = %.10f" % r["dissociation_energy"])


if __name__ == "__main__":
    main()
