"""Synthetic molecular inputs (seeded; no external dataset is involved).

Geometries are lists of (symbol, (x, y, z)) in bohr, the reference's
``config`` format (run.hpp:28-51).  Configurations:
  water          O (0,0,0.2217), H (0,+-1.4309,-0.8867)             STO-3G, K=7
  benzene        D6h ring in the xy plane, C r=2.6379, H r=4.6800     cc-pVDZ, K=120
  n_decane       all-trans zigzag C10H22, C-C 2.91, C-H 2.06, tetrahedral
                 angles, per-atom Gaussian noise sigma=0.05 (seed 20261203)   6-31G*, K=194
  nacl_scan      Na at origin, Cl on z at linspace(3.5, 7.0, n)          cc-pVTZ
  water_scan     O at origin, symmetric O-H r = linspace(1.4, 3.0, n), HOH 104.5 deg   cc-pVTZ
  random_molecule  acyclic single-bonded trees of heavy atoms {C,N,O,S}, H-capped
                 (the served request stream)
"""
import math

import numpy as np

SEED = 20261203
TETRA = math.radians(109.4712)


def water():
    return [("O", (0.0, 0.0, 0.2217)), ("H", (0.0, 1.4309, -0.8867)), ("H", (0.0, -1.4309, -0.8867))]


def benzene():
    at = []
    for k in range(6):
        a = math.radians(60.0 * k)
        at.append(("C", (2.6379 * math.cos(a), 2.6379 * math.sin(a), 0.0)))
    for k in range(6):
        a = math.radians(60.0 * k)
        at.append(("H", (4.6800 * math.cos(a), 4.6800 * math.sin(a), 0.0)))
    return at


def _unit(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v)


def n_decane(noise=0.05, seed=SEED, n_carbon=10):
    """All-trans zigzag alkane CnH(2n+2) in the xy plane."""
    cc, ch = 2.91, 2.06
    dx, dy = cc * math.sin(TETRA / 2), cc * math.cos(TETRA / 2)
    C = [np.array([i * dx, (i % 2) * dy, 0.0]) for i in range(n_carbon)]
    atoms = [("C", c) for c in C]
    z = np.array([0.0, 0.0, 1.0])
    half = TETRA / 2
    for i in range(n_carbon):
        nbr = [C[j] for j in (i - 1, i + 1) if 0 <= j < n_carbon]
        if len(nbr) == 2:
            u1, u2 = _unit(nbr[0] - C[i]), _unit(nbr[1] - C[i])
            b = -_unit(u1 + u2)
            for s in (1.0, -1.0):
                atoms.append(("H", C[i] + ch * (math.cos(half) * b + s * math.sin(half) * z)))
        else:
            u = _unit(nbr[0] - C[i])
            e1 = _unit(np.cross(z, u))
            for k in range(3):
                ph = 2 * math.pi * k / 3
                d = -u / 3.0 + math.sqrt(8.0) / 3.0 * (math.cos(ph) * e1 + math.sin(ph) * z)
                atoms.append(("H", C[i] + ch * d))
    rng = np.random.default_rng(seed)
    xyz = np.array([p for _, p in atoms]) + rng.normal(0.0, noise, size=(len(atoms), 3))
    return [(s, tuple(float(x) for x in xyz[k])) for k, (s, _) in enumerate(atoms)]


def nacl_scan(n=64):
    return [[("Na", (0.0, 0.0, 0.0)), ("Cl", (0.0, 0.0, float(r)))] for r in np.linspace(3.5, 7.0, n)]


def water_scan(n=64, angle_deg=104.5):
    h = math.radians(angle_deg) / 2
    out = []
    for r in np.linspace(1.4, 3.0, n):
        out.append([("O", (0.0, 0.0, 0.0)), ("H", (0.0, float(r * math.sin(h)), float(r * math.cos(h)))),
                    ("H", (0.0, float(-r * math.sin(h)), float(r * math.cos(h))))])
    return out


BOND = {frozenset(("C", "C")): 2.91, frozenset(("C", "N")): 2.78, frozenset(("C", "O")): 2.70,
        frozenset(("C", "S")): 3.44, frozenset(("N", "N")): 2.78, frozenset(("N", "O")): 2.70,
        frozenset(("O", "O")): 2.70, frozenset(("N", "S")): 3.30, frozenset(("O", "S")): 3.20,
        frozenset(("S", "S")): 3.90}
VALENCE = {"C": 4, "N": 3, "O": 2, "S": 2}
Z = {"H": 1, "C": 6, "N": 7, "O": 8, "S": 16}


def random_molecule(rng, n_heavy, max_tries=200):
    """Acyclic single-bonded tree of n_heavy atoms from {C,N,O,S}, grown atom
    by atom at tetrahedral angles, rejecting any placement closer than 2.0
    bohr to an existing atom, then H-capped (X-H in U[1.9, 2.5]).  Returns the
    config, or None if growth failed."""
    kinds = ["C", "N", "O", "S"]
    probs = [0.55, 0.2, 0.15, 0.1]
    atoms = [("C", np.zeros(3))]
    bonds = {0: []}
    for _ in range(n_heavy - 1):
        placed = False
        for _try in range(max_tries):
            parent = int(rng.integers(0, len(atoms)))
            ps = atoms[parent][0]
            if len(bonds[parent]) >= VALENCE[ps]:
                continue
            kind = kinds[int(rng.choice(4, p=probs))]
            d = BOND[frozenset((ps, kind))]
            pos = _tetra_direction(atoms, bonds, parent, rng)
            cand = atoms[parent][1] + d * pos
            if min(np.linalg.norm(cand - a[1]) for a in atoms) < 2.0:
                continue
            idx = len(atoms)
            atoms.append((kind, cand))
            bonds[idx] = [parent]
            bonds[parent].append(idx)
            placed = True
            break
        if not placed:
            return None
    heavy = list(atoms)
    out = [(s, p) for s, p in heavy]
    for i, (s, p) in enumerate(heavy):
        free = VALENCE[s] - len(bonds[i])
        for _ in range(free):
            ok = False
            for _try in range(max_tries):
                dirn = _tetra_direction(heavy + [(q, r) for q, r in out[len(heavy):]], bonds, i, rng)
                cand = p + float(rng.uniform(1.9, 2.5)) * dirn
                if min(np.linalg.norm(cand - a[1]) for a in out) < 2.0 - 1e-9 and not _is_cap_ok(cand, out, p):
                    continue
                out.append(("H", cand))
                ok = True
                break
            if not ok:
                return None
    return [(s, tuple(float(x) for x in p)) for s, p in out]


def _is_cap_ok(cand, out, parent_pos):
    # the parent itself is always closer than 2.0 to nothing (X-H >= 1.9 is allowed for the bond itself)
    for s, p in out:
        if np.allclose(p, parent_pos):
            continue
        if np.linalg.norm(cand - p) < 2.0:
            return False
    return True


def _tetra_direction(atoms, bonds, i, rng):
    """A direction from atom i at roughly tetrahedral angles to its bonds."""
    p = atoms[i][1]
    nb = [atoms[j][1] for j in bonds.get(i, []) if j < len(atoms)]
    if not nb:
        v = rng.normal(size=3)
        return _unit(v)
    us = [_unit(q - p) for q in nb]
    for _ in range(64):
        v = _unit(rng.normal(size=3))
        if all(abs(math.acos(max(-1.0, min(1.0, float(np.dot(v, u))))) - TETRA) < 0.25 for u in us):
            return v
    # fall back: opposite of the mean bond direction
    return -_unit(sum(us)) if np.linalg.norm(sum(us)) > 1e-8 else _unit(rng.normal(size=3))


def n_electrons(config, charge=0):
    return sum(Z.get(s, 0) if s in Z else _z(s) for s, _ in config) - charge


def _z(sym):
    els = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]
    return els.index(sym) + 1


def served_stream(n_jobs=2000, seed=SEED, max_heavy=24):
    """The served request stream: n_jobs molecules with 2..max_heavy heavy
    atoms; 80% closed-shell RHF, 20% UHF doublets (one H removed,
    n_alpha = n_beta + 1); basis STO-3G / 6-31G* / cc-pVDZ at 0.3/0.4/0.3."""
    rng = np.random.default_rng(seed)
    jobs = []
    while len(jobs) < n_jobs:
        nh = int(rng.integers(2, max_heavy + 1))
        mol = random_molecule(rng, nh)
        if mol is None:
            continue
        basis = ["STO-3G", "6-31G*", "cc-pVDZ"][int(rng.choice(3, p=[0.3, 0.4, 0.3]))]
        uhf = rng.random() < 0.2
        if uhf:
            hs = [k for k, (s, _) in enumerate(mol) if s == "H"]
            del mol[hs[int(rng.integers(0, len(hs)))]]
            ne = n_electrons(mol)
            jobs.append(dict(config=mol, basis=basis, method="UHF", spin=((ne + 1) // 2, ne // 2)))
        else:
            jobs.append(dict(config=mol, basis=basis, method="RHF"))
    return jobs
