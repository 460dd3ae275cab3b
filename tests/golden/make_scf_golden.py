"""Generate the SCF and Fock-matrix fixtures of the benchmark configurations.

TEST INFRASTRUCTURE.  Sources (read here only; nothing at test time reads the
reference):
  * the reference's own include/integrals.hpp compiled unchanged into
    oracle/_ref/libhfref.so (``make -C oracle ref REF=<checkout>``): the full
    screened unique-ERI tensor of each molecule (repulsion_tensor,
    integrals.hpp:754-787, its loop spread over host threads);
  * the oracle's C restatement (oracle/hf_oracle.c, pinned to the reference by
    tests/golden/water_sto3g.json and eri_samples.json) with the accurate Boys
    function, for the Fock-matrix fixtures that are compared element by
    element at 1e-10 (the reference's upward Boys recursion moves single ERIs
    by up to ~1e-8, see hf_oracle.c);
  * the numpy restatement of rhf_diis (scf.hpp:205-419) in oracle/oracle.py,
    with the reference's repulsion_matrix contraction (linalg.hpp:100-129) over
    the stored tensor, for energies and iteration counts.

Fixtures written (small: energies, iteration counts, and K x K matrices, never
tensors):
  scf_golden.json  per case: molecule, basis, SCF settings, E_tot, iterations,
                   converged; warm-started scan points carry the case whose
                   converged density they start from
  fock_golden.npz  per matrix case: the input densities P, Pa, Pb and the
                   outputs G = repulsion_matrix(P), J = coulomb_matrix(Pa, Pb),
                   Ka/Kb = exchange_matrix(Pa/Pb), from the stable-Boys tensor,
                   plus G from the reference's own tensor (G_ref)

Usage (from the repository root; the reference checkout is given by
HF_REFERENCE):
  HF_REFERENCE=<checkout> python tests/golden/make_scf_golden.py [case ...]
Cases: water_tz, nacl_tz, benzene, decane, then water_tz_stable and
nacl_tz_stable (the same scan points over the stable-Boys tensor; they add
E_tot_stable / iterations_stable to the existing entries).  Default: all.
Each case merges its entries into the existing fixture files.  With
HF_TENSOR_CACHE=<directory> the tensors are kept there between runs (the
stable-Boys stages reuse the tensors of the earlier ones).
"""
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402

_spec = importlib.util.spec_from_file_location("hfx_workloads",
                                               os.path.join(REPO, "hartree_fock_cpp_gb300", "workloads.py"))
W = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(W)

JSON = os.path.join(HERE, "scf_golden.json")
NPZ = os.path.join(HERE, "fock_golden.npz")

# SCF settings.  BENCH: the benchmark's stated convergence (DIIS 8, |dE| < 1e-8
# and RMS dD < 1e-7); SCAN: the reference's defaults (scf.hpp:205-213).
BENCH = dict(epsilon=1e-7, energy_threshold=1e-8)
SCAN = dict(epsilon=1e-6, energy_threshold=0.0)
NACL_POINTS = (20, 21)        # of nacl_scan(64): R = 4.611, 4.667 bohr
WATER_POINTS = (0, 20, 21)    # of water_scan(64): r = 1.400, 1.908, 1.933 bohr


def log(msg):
    print("[%s] %s" % (time.strftime("%H:%M:%S"), msg), flush=True)


CACHE = os.environ.get("HF_TENSOR_CACHE")   # optional directory: tensors kept between runs


def _cached(kind, config, basis, make):
    if not CACHE:
        return make()
    import hashlib
    key = hashlib.sha1(json.dumps([kind, basis, config]).encode()).hexdigest()[:16]
    path = os.path.join(CACHE, "%s_%s.npy" % (kind, key))
    if os.path.exists(path):
        return np.load(path)
    eri = make()
    os.makedirs(CACHE, exist_ok=True)
    np.save(path, eri)
    return eri


def ref_tensor(config, basis):
    def make():
        r = O.RefLib()
        K = r.build(config, basis, O.BASIS_PATH)
        t = time.perf_counter()
        eri = r.repulsion_tensor_mt(1e-8)
        log("reference tensor %s K=%d: %d unique ERIs in %.0f s" % (basis, K, eri.size, time.perf_counter() - t))
        return eri
    return _cached("ref", config, basis, make)


def stable_tensor(config, basis):
    def make():
        orc = O.Oracle(config, basis, stable_boys=True)
        t = time.perf_counter()
        eri = orc.repulsion_tensor_mt(1e-8)
        log("stable-Boys tensor %s K=%d in %.0f s" % (basis, orc.K, time.perf_counter() - t))
        return eri
    return _cached("stable", config, basis, make)


def rhf(config, basis, eri, settings, P0=None):
    t = time.perf_counter()
    res = O.rhf_diis(config, basis, fock_builder=lambda P: O.contract_mt("G", P, eri), P0=P0, **settings)
    log("  rhf: E = %.10f, %d iterations, converged %s (%.0f s)"
        % (res["E_tot"], res["iterations"], res["converged"], time.perf_counter() - t))
    return res


def entry(config, basis, settings, res, **extra):
    e = dict(config=config, basis=basis, method="RHF", settings=settings, E_tot=res["E_tot"],
             iterations=res["iterations"], converged=bool(res["converged"]), K=res["K"])
    e.update(extra)
    return e


def matrices(prefix, config, basis, P, eri_ref, seed):
    """G, J, Ka, Kb of the stable-Boys tensor at the converged density P and a
    spin split of it, plus G of the reference's own tensor."""
    eri = stable_tensor(config, basis)
    K = P.shape[0]
    rng = np.random.default_rng(seed)
    X = rng.normal(scale=0.02, size=(K, K))
    X = X + X.T
    Pa, Pb = 0.5 * P + X, 0.5 * P - X
    out = {prefix + "P": P, prefix + "Pa": Pa, prefix + "Pb": Pb,
           prefix + "G": O.contract_mt("G", P, eri),
           prefix + "J": O.contract_mt("J", Pa, eri, Pb),
           prefix + "Ka": O.contract_mt("K", Pa, eri),
           prefix + "Kb": O.contract_mt("K", Pb, eri),
           prefix + "G_ref": O.contract_mt("G", P, eri_ref)}
    log("  %s: max|G - G_ref| = %.2e" % (prefix, np.abs(out[prefix + "G"] - out[prefix + "G_ref"]).max()))
    return out


def case_scan(name, configs, points, basis, mat_point):
    cases, mats = {}, {}
    dens = {}
    for idx in points:
        cfg = configs[idx]
        eri = ref_tensor(cfg, basis)
        res = rhf(cfg, basis, eri, SCAN)
        key = "%s_%d" % (name, idx)
        cases[key] = entry(cfg, basis, SCAN, res, scan_index=idx)
        dens[idx] = res["density"]
        if idx - 1 in dens:
            w = rhf(cfg, basis, eri, SCAN, P0=dens[idx - 1])
            cases[key + "_warm"] = entry(cfg, basis, SCAN, w, scan_index=idx, warm_start_from="%s_%d" % (name, idx - 1))
        if idx == mat_point:
            mats.update(matrices(key + ".", cfg, basis, res["density"], eri, seed=idx))
    return cases, mats


def case_water_tz():
    return case_scan("water_ccpvtz", W.water_scan(64), WATER_POINTS, "cc-pVTZ", 20)


def case_nacl_tz():
    return case_scan("nacl_ccpvtz", W.nacl_scan(64), NACL_POINTS, "cc-pVTZ", 20)


def case_benzene():
    cfg = W.benzene()
    eri = ref_tensor(cfg, "cc-pVDZ")
    res = rhf(cfg, "cc-pVDZ", eri, BENCH)
    return {"benzene_ccpvdz": entry(cfg, "cc-pVDZ", BENCH, res)}, {}


def case_decane():
    cfg = W.n_decane()
    eri = ref_tensor(cfg, "6-31G*")
    res = rhf(cfg, "6-31G*", eri, BENCH)
    return {"decane_631gs": entry(cfg, "6-31G*", BENCH, res)}, {}


def stable_scan(name, configs, points, basis):
    """The scan points' SCF over the stable-Boys tensor (the reference's
    algorithm with an accurate F_m(T)): E_tot_stable / iterations_stable
    beside the reference's own numbers.  Where the reference's upward Boys
    recursion moves the ERIs far enough to shift the energy by more than
    1 uHa, the engine (accurate Boys) is held to these."""
    data = json.load(open(JSON))
    dens = {}
    for idx in points:
        cfg = configs[idx]
        eri = stable_tensor(cfg, basis)
        key = "%s_%d" % (name, idx)
        res = rhf(cfg, basis, eri, SCAN)
        data[key].update(E_tot_stable=res["E_tot"], iterations_stable=res["iterations"])
        dens[idx] = res["density"]
        if key + "_warm" in data and idx - 1 in dens:
            w = rhf(cfg, basis, eri, SCAN, P0=dens[idx - 1])
            data[key + "_warm"].update(E_tot_stable=w["E_tot"], iterations_stable=w["iterations"])
    return data


def case_nacl_tz_stable():
    return stable_scan("nacl_ccpvtz", W.nacl_scan(64), NACL_POINTS, "cc-pVTZ"), {}


def case_water_tz_stable():
    return stable_scan("water_ccpvtz", W.water_scan(64), WATER_POINTS, "cc-pVTZ"), {}


CASES = {"water_tz": case_water_tz, "nacl_tz": case_nacl_tz, "benzene": case_benzene, "decane": case_decane,
         "water_tz_stable": case_water_tz_stable, "nacl_tz_stable": case_nacl_tz_stable}


def main(names):
    if O.reference_checkout() is None:
        sys.exit("set HF_REFERENCE to a checkout of the reference")
    O.build_oracle()
    for n in names:
        log("case " + n)
        cases, mats = CASES[n]()
        data = json.load(open(JSON)) if os.path.exists(JSON) else {}
        data.update(cases)
        with open(JSON, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        if mats:
            old = dict(np.load(NPZ)) if os.path.exists(NPZ) else {}
            old.update(mats)
            np.savez_compressed(NPZ, **old)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
