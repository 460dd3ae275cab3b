"""Host-side logic of libhfx on the CPU (no kernel launches): the C ABI
exports, basis construction, one-electron integrals, the SCF driver, the
pair data the kernels consume, and error handling."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
import hartree_fock_cpp_gb300 as H
from hartree_fock_cpp_gb300 import _lib, workloads as W
import md_emulation as MD

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "hfx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\bhfx_status\s+(hfx_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    names = declared_symbols()
    assert len(names) >= 20
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.SIGNATURES)


@pytest.mark.parametrize("basis", ["STO-3G", "6-31G", "6-31G*", "cc-pVDZ", "cc-pVTZ"])
def test_basis_construction_matches_reference_order(basis):
    cfg = W.water()
    b = H.basis_construction(cfg, basis)
    fb = O.FlatBasis(cfg, basis)
    assert b.K == fb.K
    assert np.array_equal(b.lmn.ravel(), fb.lmn)
    assert np.array_equal(b.prim_offset, fb.prim_off)
    assert np.array_equal(b.alpha, fb.alpha)
    assert np.array_equal(b.coeff, fb.coeff)
    assert np.abs(b.norm - fb.norm).max() < 1e-13 * np.abs(fb.norm).max()
    assert np.array_equal(b.centres, fb.centres)


def test_basis_sizes_of_the_workloads():
    assert H.basis_construction(W.water(), "STO-3G").K == 7
    assert H.basis_construction(W.benzene(), "cc-pVDZ").K == 120
    assert H.basis_construction(W.n_decane(), "6-31G*").K == 194
    assert H.basis_construction(W.nacl_scan()[0], "cc-pVTZ").K == 78
    assert H.basis_construction(W.water_scan()[0], "cc-pVTZ").K == 65


@pytest.mark.parametrize("basis", ["STO-3G", "6-31G*", "cc-pVTZ"])
def test_one_electron_matches_oracle(basis):
    cfg = W.water()
    S, T, V = H.one_electron(cfg, basis)
    So, To, Vo = O.Oracle(cfg, basis).one_electron()
    assert np.abs(S - So).max() < 1e-12
    assert np.abs(T - To).max() < 1e-12
    assert np.abs(V - Vo).max() < 1e-11


def _run_rhf_driver(cfg, basis, charge=0, **kw):
    orc = O.Oracle(cfg, basis)
    eri = orc.repulsion_tensor(1e-8)
    K = orc.K

    def gb(user, P, G):
        Pm = np.ctypeslib.as_array(P, shape=(K * K,)).reshape(K, K).copy()
        Gm = np.ascontiguousarray(O.repulsion_matrix(Pm, eri))
        ctypes.memmove(G, Gm.ctypes.data, K * K * 8)
        return 0

    cb = _lib.G_BUILDER(gb)
    m = _lib.MoleculeArgs(cfg, basis)
    o = _lib.ScfOptions()
    o.charge = charge
    for k, v in kw.items():
        setattr(o, k, v)
    r = _lib.ScfResult()
    dens = np.zeros((K, K))
    st = _lib.lib.hfx_rhf_diis_with_builder(m.ref(), ctypes.byref(o), None, cb, None, ctypes.byref(r),
                                            _lib.ptr(dens), None)
    return st, r, dens


def test_rhf_driver_matches_numpy_oracle_water():
    st, r, dens = _run_rhf_driver(W.water(), "STO-3G")
    assert st == 0
    ro = O.rhf_diis(W.water(), "STO-3G")
    assert abs(r.E_tot - ro["E_tot"]) < 1e-9
    assert abs(r.iterations - ro["iterations"]) <= 1
    assert np.abs(dens - ro["density"]).max() < 1e-6


def test_rhf_driver_reproduces_reference_curve_point():
    import json
    e = json.load(open(os.path.join(REPO, "tests", "golden", "reference_energies.json")))[5]   # HeH+
    st, r, _ = _run_rhf_driver([tuple(a) for a in e["config"]], "STO-3G", charge=e["charge"])
    assert st == 0
    assert abs(r.E_tot - e["E"]) < 1e-6


def test_uhf_driver_matches_numpy_oracle():
    cfg = [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.83))]   # OH radical
    orc = O.Oracle(cfg, "STO-3G")
    eri = orc.repulsion_tensor(1e-8)
    K = orc.K

    def jk(user, Pa, Pb, J, Ka, Kb):
        a = np.ctypeslib.as_array(Pa, shape=(K * K,)).reshape(K, K).copy()
        b = np.ctypeslib.as_array(Pb, shape=(K * K,)).reshape(K, K).copy()
        for out, M in ((J, O.coulomb_matrix(a, b, eri)), (Ka, O.exchange_matrix(a, eri)),
                       (Kb, O.exchange_matrix(b, eri))):
            M = np.ascontiguousarray(M)
            ctypes.memmove(out, M.ctypes.data, K * K * 8)
        return 0

    cb = _lib.JK_BUILDER(jk)
    m = _lib.MoleculeArgs(cfg, "STO-3G")
    o = _lib.ScfOptions()
    r = _lib.ScfResult()
    st = _lib.lib.hfx_uhf_diis_with_builder(m.ref(), ctypes.byref(o), 5, 4, cb, None, ctypes.byref(r), None, None)
    assert st == 0
    ro = O.uhf_diis(cfg, "STO-3G", (5, 4))
    assert abs(r.E_tot - ro["E_tot"]) < 1e-9
    assert abs(r.iterations - ro["iterations"]) <= 1


@pytest.mark.parametrize("cfg,basis,pairs", [
    (W.water(), "6-31G*", [(0, 0), (5, 3), (40, 12), (60, 59)]),
    ([("C", (0.0, 0.0, 0.0)), ("O", (0.3, -0.2, 2.1))], "cc-pVTZ", [(209, 209), (150, 40), (100, 99)]),
])
def test_pair_data_encodes_reference_eris(cfg, basis, pairs):
    rec, geo, ep = MD.pair_data(cfg, basis)
    orc = O.Oracle(cfg, basis, stable_boys=True)
    worst = 0.0
    for bra, ket in pairs:
        bra, ket = min(bra, len(rec) - 1), min(ket, len(rec) - 1)
        acc = MD.shell_quartet_block(rec, geo, ep, bra, ket)
        b, k = rec[bra], rec[ket]
        n1, n3 = MD.ncart(b[3]), MD.ncart(k[3])
        for ab in range(acc.shape[0]):
            for cd in range(acc.shape[1]):
                if (ab * 7 + cd) % 3:
                    continue
                i, j = b[0] + ab // n1, b[1] + ab % n1
                kk, l = k[0] + cd // n3, k[1] + cd % n3
                worst = max(worst, abs(orc.eri(i, j, kk, l) - acc[ab, cd]))
    assert worst < 1e-13


def test_errors_are_status_codes_not_exits():
    with pytest.raises(H.HfxError) as e:
        H.basis_construction(W.water(), "no-such-basis")
    assert e.value.status == 2
    with pytest.raises(H.HfxError) as e:
        H.basis_construction([("Xx", (0, 0, 0))], "STO-3G")
    assert e.value.status == 2
    # a basis-function list that is not made of complete shells
    b = H.basis_construction(W.water(), "STO-3G")
    bad = H.Basis(b.centres[:3], b.lmn[:3], b.prim_offset[:4], b.alpha[:b.prim_offset[3]],
                  b.coeff[:b.prim_offset[3]], b.norm[:b.prim_offset[3]])
    with pytest.raises(H.HfxError) as e:
        H.ERI_GPU(bad, 1e-8)
    assert e.value.status == 2
    with pytest.raises(H.HfxError):
        H.rhf_diis(W.water(), "STO-3G", eri_device="TPU")
    assert "unsupported" in H._lib.last_error() or True


def test_cube_file_layout(tmp_path):
    """write_cube_file follows the reference's layout (cube.hpp:383-450):
    2 comment lines, natoms + origin, 3 grid vectors, atoms, values z-fastest
    six per line in %.8e."""
    from hartree_fock_cpp_gb300 import cube
    res = 3
    field = np.arange(res ** 3, dtype=float) * 0.5
    c = {"field": field, "origin": np.array([-1.0, -2.0, -3.0]), "dx": 0.25, "res": res}
    atoms = [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 1.4, 1.1))]
    f = tmp_path / "x.cube"
    cube.write_cube_file(str(f), c, atoms, comment="test")
    lines = f.read_text().splitlines()
    assert lines[0] == "test"
    assert lines[2].split() == ["2", "-1", "-2", "-3"]
    assert lines[3].split()[:2] == ["3", "0.25"]
    assert lines[6].split()[0] == "8" and lines[7].split()[0] == "1"
    vals = " ".join(lines[8:]).split()
    assert len(vals) == res ** 3
    assert float(vals[5]) == 2.5 and vals[0] == "0.00000000e+00"
    assert len(lines[8].split()) == 6


def test_oracle_grid_restatement_on_hand_values():
    """The oracle's function_eval / electron_density restatement on a case
    worked by hand: one normalised s function, P = [[2]] gives
    rho(r) = 2 phi(r)^2 with phi(r) = N c exp(-a r^2)."""
    import oracle as O
    fb = O.FlatBasis([("H", (0.0, 0.0, 0.0))], "STO-3G")
    pts = np.array([[0.0, 0.0, 0.0], [0.3, -0.2, 0.5]])
    phi = O.basis_values(fb, pts)
    r2 = (pts ** 2).sum(1)
    ref = sum(fb.norm[i] * fb.coeff[i] * np.exp(-fb.alpha[i] * r2) for i in range(fb.prim_off[1]))
    assert np.allclose(phi[0], ref, rtol=1e-14)
    rho = O.electron_density(fb, [[2.0]], pts)
    assert np.allclose(rho, 2.0 * ref ** 2, rtol=1e-14)
    box = O.box_points((0.0, 0.0, 0.0), 2.0, 3)
    assert box.shape == (27, 3) and np.allclose(box[1], [-1.0, -1.0, 0.0])


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every struct of include/hfx.h has the same size in the ctypes mirror
    (a compiled probe prints sizeof and the offset of the last member)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from hartree_fock_cpp_gb300 import _lib as L
    pairs = {"hfx_functions": L.Functions, "hfx_molecule": L.Molecule, "hfx_options": L.Options,
             "hfx_build_stats": L.BuildStats, "hfx_launch_shape": L.LaunchShape, "hfx_scf_options": L.ScfOptions,
             "hfx_scf_result": L.ScfResult, "hfx_server_options": L.ServerOptions, "hfx_request": L.Request,
             "hfx_job_info": L.JobInfo, "hfx_server_stats_t": L.ServerStats, "hfx_batch_options": L.BatchOptions,
             "hfx_batch_stats": L.BatchStats}
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "hfx.h"\nint main(void) {\n' +
                   "".join('    printf("%s %%zu\\n", sizeof(%s));\n' % (n, n) for n in pairs) + "    return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run([gcc, "-I", os.path.join(repo, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    sizes = {l.split()[0]: int(l.split()[1]) for l in out if l.strip()}
    for name, cls in pairs.items():
        assert sizes[name] == ctypes.sizeof(cls), name


def test_packed_job_layout():
    """Packed jobs (several molecules in one job): shell pairs never mix
    molecules, indices are molecule-local, each molecule's pairs start at
    its pair base with the single-molecule order, and its matrices and
    Schwarz table sit at the running sums of K^2 and K(K+1)/2."""
    mols = [(W.water(), "6-31G*"), (W.nacl_scan(8)[3], "cc-pVTZ"), ([("H", (0, 0, 0)), ("H", (0, 0, 1.4))], "STO-3G")]
    args = [_lib.MoleculeArgs(c, b) for c, b in mols]
    arr = (_lib.Molecule * len(args))(*[a.c for a in args])
    n = ctypes.c_int()
    _lib.check(_lib.lib.hfx_debug_packed_pairs(ctypes.cast(arr, ctypes.c_void_p), len(args), ctypes.byref(n), None,
                                               None))
    rec = np.zeros(10 * n.value, dtype=np.int32)
    offs = np.zeros(3 * n.value, dtype=np.int64)
    _lib.check(_lib.lib.hfx_debug_packed_pairs(ctypes.cast(arr, ctypes.c_void_p), len(args), None, _lib.ptr(rec),
                                               _lib.ptr(offs)))
    rec = rec.reshape(-1, 10)
    offs = offs.reshape(-1, 3)
    Ks = [H.basis_construction(c, b).K for c, b in mols]
    moff, qoff, pbase = 0, 0, 0
    for f, (cfg, bs) in enumerate(mols):
        sel = np.where(rec[:, 0] == f)[0]
        # the single-molecule pair records of this molecule
        m = _lib.MoleculeArgs(cfg, bs)
        npp, nprim, nep = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), ctypes.byref(npp), ctypes.byref(nprim), ctypes.byref(nep),
                                                None, None, None))
        single = np.zeros(10 * npp.value, dtype=np.int32)
        _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), None, None, None, _lib.ptr(single), None, None))
        single = single.reshape(-1, 10)
        assert len(sel) == npp.value
        assert sel[0] == pbase and np.all(np.diff(sel) == 1)
        assert np.all(rec[sel, 1] == Ks[f]) and np.all(rec[sel, 2] == pbase)
        assert np.all(rec[sel, 3] == sel)                                   # global pair id
        assert np.all(rec[sel, 6] == single[:, 0]) and np.all(rec[sel, 7] == single[:, 1])   # local bf0, bf1
        assert np.all(rec[sel, 8] == single[:, 2]) and np.all(rec[sel, 9] == single[:, 3])   # l0, l1
        assert np.all(rec[sel, 6] < Ks[f]) and np.all(rec[sel, 7] < Ks[f])
        assert np.all(offs[sel, 0] == moff) and np.all(offs[sel, 1] == qoff)
        assert np.all(offs[sel, 2] == single[:, 5])                         # primitive pairs
        moff += Ks[f] ** 2
        qoff += Ks[f] * (Ks[f] + 1) // 2
        pbase += len(sel)
    assert pbase == n.value


def test_served_stream_properties():
    """The seeded served stream: 2..24 heavy atoms from {C,N,O,S}, H-capped,
    ~80% RHF / 20% UHF doublets (n_alpha = n_beta + 1), bases at about
    0.3 / 0.4 / 0.3, no two atoms closer than 2.0 bohr except an H and its
    parent (bond 1.9..2.5 bohr), and the same stream for the same seed."""
    jobs = W.served_stream(300)
    assert W.served_stream(5) == jobs[:5]
    n_uhf = sum(j["method"] == "UHF" for j in jobs)
    assert 0.12 < n_uhf / len(jobs) < 0.28
    frac = {b: sum(j["basis"] == b for j in jobs) / len(jobs) for b in ("STO-3G", "6-31G*", "cc-pVDZ")}
    assert abs(frac["STO-3G"] - 0.3) < 0.08 and abs(frac["6-31G*"] - 0.4) < 0.08 and abs(frac["cc-pVDZ"] - 0.3) < 0.08
    for j in jobs[:80]:
        syms = [s for s, _ in j["config"]]
        heavy = [s for s in syms if s != "H"]
        assert 2 <= len(heavy) <= 24 and set(heavy) <= {"C", "N", "O", "S"}
        xyz = np.array([p for _, p in j["config"]])
        d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=-1)
        close = np.argwhere(np.triu(d < 2.0 - 1e-9, 1))
        for a, b in close:
            assert (syms[a] == "H") != (syms[b] == "H"), (syms[a], syms[b], d[a, b])
            assert d[a, b] >= 1.9 - 1e-9
        if j["method"] == "UHF":
            na, nb = j["spin"]
            assert na == nb + 1 and na + nb == W.n_electrons(j["config"])
        else:
            assert W.n_electrons(j["config"]) % 2 == 0


def test_pair_data_independent_of_host_threads():
    """The pair records are built per shell pair on host threads and appended
    in pair order: repeated builds give identical records, primitive-pair
    geometry and E blocks (NaCl/cc-pVTZ: heavily contracted shells)."""
    m = _lib.MoleculeArgs(W.nacl_scan(64)[20], "cc-pVTZ")

    def build():
        npp, nprim, nep = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), ctypes.byref(npp), ctypes.byref(nprim), ctypes.byref(nep),
                                                None, None, None))
        rec = np.zeros(10 * npp.value, dtype=np.int32)
        geo = np.zeros(4 * nprim.value)
        ep = np.zeros(nep.value)
        _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), None, None, None, _lib.ptr(rec), _lib.ptr(geo), _lib.ptr(ep)))
        return rec, geo, ep

    first = build()
    for _ in range(3):
        again = build()
        for a, b in zip(first, again):
            assert a.shape == b.shape and np.array_equal(a, b)
    rec = first[0].reshape(-1, 10)
    assert np.all(np.diff(rec[:, 4]) == rec[:-1, 5])    # primitive-pair ranges back to back, in pair order


def test_sp2_control_gives_the_occupied_projector():
    """The density step's control (tests/sp2_emulation.py, as hfx_sp2.cu runs
    it): for Fock-like spectra with a gap the projector equals C_occ C_occ^T
    of an eigendecomposition, within the 100-step cap; with a degenerate
    HOMO/LUMO pair it reports no convergence (the SCF then uses syevd)."""
    import sp2_emulation as S
    rng = np.random.default_rng(7)
    for n, nocc, gap in ((7, 2, 0.5), (40, 9, 0.3), (120, 21, 0.47), (160, 30, 0.05)):
        lam = np.concatenate([rng.uniform(-20.0, -gap / 2, nocc), rng.uniform(gap / 2, 5.0, n - nocc)])
        lam[nocc - 1], lam[nocc] = -gap / 2, gap / 2
        Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
        F = (Q * lam) @ Q.T
        D, steps = S.sp2_projector(F, nocc)
        assert D is not None and 0 < steps <= 100, (n, steps)
        w, V = np.linalg.eigh(F)
        assert np.abs(D - V[:, :nocc] @ V[:, :nocc].T).max() < 1e-11
    # degenerate level at the Fermi surface: three orbitals at 0 for one pair
    lam = np.array([-2.0, -1.0, 0.0, 0.0, 0.0, 1.0, 2.0])
    Q, _ = np.linalg.qr(rng.normal(size=(7, 7)))
    D, steps = S.sp2_projector((Q * lam) @ Q.T, 3)
    assert D is None and steps == 0
