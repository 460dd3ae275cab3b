"""Generate the golden fixtures under tests/golden/ from the reference itself.

Sources (read here only; nothing at test time reads the reference):
  * oracle/_ref/libhfref.so -- the reference's include/integrals.hpp and
    basis.hpp compiled unchanged (oracle/Makefile `ref` target): ERIs,
    Schwarz bounds and one-electron matrices;
  * the reference's published SCF results results/STO-3G/*_vr.csv (R, E
    curves of its own RHF code): a few points per curve.
Run from the repository root:
  HF_REFERENCE=<reference checkout> python tests/golden/make_golden.py
"""
import csv
import json
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, REPO)
import oracle as O  # noqa: E402
from hartree_fock_cpp_gb300 import workloads as W  # noqa: E402

REF = O.reference_checkout()     # HF_REFERENCE: a checkout of the reference
OUT = os.path.dirname(os.path.abspath(__file__))


def water_sto3g():
    r = O.RefLib()
    K = r.build(W.water(), "STO-3G", O.BASIS_PATH)
    eri = r.repulsion_tensor(1e-8)
    Q = r.schwarz_bounds()
    S, T, V = r.one_electron()
    return dict(config=W.water(), basis="STO-3G", K=K, threshold=1e-8, eri=eri.tolist(), schwarz=Q.tolist(),
                S=S.ravel().tolist(), T=T.ravel().tolist(), V=V.ravel().tolist())


def eri_samples(name, config, basis, n=160, seed=7):
    r = O.RefLib()
    K = r.build(config, basis, O.BASIS_PATH)
    rng = np.random.default_rng(seed)
    quartets = []
    while len(quartets) < n:
        i, j, k, l = (int(x) for x in rng.integers(0, K, 4))
        if i < j:
            i, j = j, i
        if k < l:
            k, l = l, k
        if i * (i + 1) // 2 + j < k * (k + 1) // 2 + l:
            i, j, k, l = k, l, i, j
        quartets.append((i, j, k, l))
    vals = [r.eri(*q) for q in quartets]
    # diagonal quartets for the Schwarz products of the sampled pairs
    qd = {}
    for (i, j, k, l) in quartets:
        for a, b in ((i, j), (k, l)):
            if (a, b) not in qd:
                v = r.eri(a, b, a, b)
                qd[(a, b)] = float(np.sqrt(max(v, 0.0)))
    return dict(name=name, config=config, basis=basis, K=K, quartets=quartets, eri=vals,
                q_ij=[qd[(q[0], q[1])] for q in quartets], q_kl=[qd[(q[2], q[3])] for q in quartets])


CURVES = [
    ("H2_vr", "H", "H", 0, [1000, 2000, 3333, 6000, 9999]),
    ("HeHp_vr", "He", "H", 1, [500, 2000, 3333, 6000]),
    ("HF_vr", "H", "F", 0, [500, 1000, 1666]),
    ("LiH_vr_1", "Li", "H", 0, [100, 333, 600]),
    ("LiH_vr_2", "Li", "H", 0, [100, 333]),
    ("BeH2_vr_1", "Be", "H", 0, [100, 333]),
    ("BeH2_vr_2", "Be", "H", 0, [500, 1000]),
]


def energies():
    out = []
    for name, a, b, charge, rows in CURVES:
        data = list(csv.DictReader(open(os.path.join(REF, "results", "STO-3G", name + ".csv"))))
        for idx in rows:
            R, E = float(data[idx]["R"]), float(data[idx]["E"])
            if name.startswith("BeH2"):
                config = [(a, (0.0, 0.0, 0.0)), (b, (R, 0.0, 0.0)), (b, (-R, 0.0, 0.0))]
            else:
                config = [(a, (0.0, 0.0, 0.0)), (b, (R, 0.0, 0.0))]
            # keep only points that a cold-start SCF reproduces (the curves were
            # made as warm-started scans)
            res = O.rhf_diis(config, "STO-3G", charge=charge, max_it=500)
            if not res["converged"] or abs(res["E_tot"] - E) > 5e-7:
                continue
            out.append(dict(curve=name, row=idx, R=R, E=E, charge=charge, config=config, basis="STO-3G",
                            oracle_iterations=res["iterations"]))
    return out


def main():
    if REF is None:
        sys.exit("set HF_REFERENCE to a checkout of the reference")
    O.build_oracle()
    json.dump(water_sto3g(), open(os.path.join(OUT, "water_sto3g.json"), "w"))
    samples = [eri_samples("water_631gs", W.water(), "6-31G*"),
               eri_samples("water_ccpvtz", W.water(), "cc-pVTZ", n=80),
               eri_samples("benzene_ccpvdz", W.benzene(), "cc-pVDZ"),
               eri_samples("decane_631gs", W.n_decane(), "6-31G*"),
               eri_samples("nacl_ccpvtz", [("Na", (0.0, 0.0, 0.0)), ("Cl", (0.0, 0.0, 4.46))], "cc-pVTZ", n=60)]
    json.dump(samples, open(os.path.join(OUT, "eri_samples.json"), "w"))
    json.dump(energies(), open(os.path.join(OUT, "reference_energies.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
