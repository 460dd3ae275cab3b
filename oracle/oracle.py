"""Python face of the oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The engine (``hartree_fock_cpp_gb300``) never does.

Contents
  * basis construction restated from the reference's include/basis.hpp
    (cart_norm :28-49, angmom_partition :52-64, build_shell :67-113,
    basis_construction :157-262), producing flat arrays for hf_oracle.c;
  * ctypes bindings to oracle/_build/libhforacle.so (the C restatement of
    include/integrals.hpp and include/linalg.hpp, see hf_oracle.c);
  * optional bindings to oracle/_ref/libhfref.so (the reference's own
    integrals.hpp compiled unchanged; only where a reference checkout exists);
  * a numpy restatement of the reference's SCF drivers rhf_diis
    (include/scf.hpp:205-419) and uhf_diis (include/scf.hpp:423-682), with
    numpy.linalg.eigh standing in for Eigen's SelfAdjointEigenSolver and a
    complete-pivoting LU solve restating Eigen's fullPivLu rank handling
    (Eigen is not available here).
"""
import csv
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
BASIS_PATH = os.path.join(REPO, "hartree_fock_cpp_gb300", "basis")

ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na",
            "Mg", "Al", "Si", "P", "S", "Cl", "Ar", "K", "Ca", "Sc", "Ti",
            "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge",
            "As", "Se", "Br", "Kr"]          # atoms.hpp:10-14
ANGMOM = ["S", "P", "D", "F", "G", "H"]     # basis.hpp:178


def nameZ(sym):
    return ELEMENTS.index(sym) + 1


def double_factorial(n):                    # basis.hpp:14-25
    r = 1
    while n > 0:
        r *= n
        n -= 2
    return r


def cart_norm(alpha, lx, ly, lz):           # basis.hpp:28-49
    L = lx + ly + lz
    num = (4.0 * alpha) ** L
    den = double_factorial(2 * lx - 1) * double_factorial(2 * ly - 1) * double_factorial(2 * lz - 1)
    return (2.0 * alpha / math.pi) ** 0.75 * math.sqrt(num / den)


def angmom_partition(l):                    # basis.hpp:52-64
    return [(a, b, l - a - b) for a in range(l + 1) for b in range(l - a + 1)]


def read_shells(basis_set, element, basis_path=BASIS_PATH):
    """Shells of one element in CSV order: list of (L, exponents, coefficients).
    Mirrors the slicing and checks of basis.hpp:180-231."""
    fn = os.path.join(basis_path, basis_set, element + ".csv")
    if not os.path.isfile(fn):
        raise RuntimeError("Critical Error: File does not exist or is invalid at path: " + fn)
    rows = list(csv.DictReader(open(fn)))
    shells = []
    cur_id = None
    for r in rows:
        sid = int(r["shell_id"])
        if sid != cur_id:
            shells.append([sid, r["L"].strip(), [], [], []])
            cur_id = sid
        shells[-1][2].append(float(r["exponent"]))
        shells[-1][3].append(float(r["coefficient"]))
        shells[-1][4].append(int(r["primitive_id"]))
    out = []
    for j, (sid, L, ex, co, pid) in enumerate(shells):
        if max(pid) + 1 != len(ex):
            raise RuntimeError("wrong primitive number")
        if sid != j:
            raise RuntimeError("building shells in the wrong order")
        out.append((ANGMOM.index(L), ex, co))
    return out


class FlatBasis:
    """Basis functions in the reference's order, flattened for hf_oracle.c."""

    def __init__(self, config, basis_set, basis_path=BASIS_PATH):
        centres, lmn, prim_off, alpha, coeff, norm = [], [], [0], [], [], []
        for sym, R in config:                      # basis.hpp:180-247
            for (L, ex, co) in read_shells(basis_set, sym, basis_path):
                for (lx, ly, lz) in angmom_partition(L):
                    centres.append(R)
                    lmn.append((lx, ly, lz))
                    for a, c in zip(ex, co):
                        alpha.append(a)
                        coeff.append(c)
                        norm.append(cart_norm(a, lx, ly, lz))
                    prim_off.append(len(alpha))
        self.K = len(lmn)
        self.centres = np.ascontiguousarray(np.array(centres, dtype=np.float64).reshape(-1, 3))
        self.cx = np.ascontiguousarray(self.centres[:, 0])
        self.cy = np.ascontiguousarray(self.centres[:, 1])
        self.cz = np.ascontiguousarray(self.centres[:, 2])
        self.lmn = np.ascontiguousarray(np.array(lmn, dtype=np.int32).reshape(-1))
        self.prim_off = np.array(prim_off, dtype=np.int32)
        self.alpha = np.array(alpha, dtype=np.float64)
        self.coeff = np.array(coeff, dtype=np.float64)
        self.norm = np.array(norm, dtype=np.float64)
        self.atoms_Z = np.array([nameZ(s) for s, _ in config], dtype=np.int32)
        self.atoms_xyz = np.ascontiguousarray(np.array([R for _, R in config], dtype=np.float64).reshape(-1))


class _CBasis(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int),
                ("cx", ctypes.c_void_p), ("cy", ctypes.c_void_p), ("cz", ctypes.c_void_p),
                ("lmn", ctypes.c_void_p), ("prim_off", ctypes.c_void_p),
                ("alpha", ctypes.c_void_p), ("coeff", ctypes.c_void_p), ("norm", ctypes.c_void_p)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def reference_checkout():
    """Directory of a reference checkout, from the HF_REFERENCE environment
    variable; None when it is unset or does not hold the reference."""
    ref = os.environ.get("HF_REFERENCE")
    if ref and os.path.isdir(os.path.join(ref, "include")):
        return ref
    return None


def build_oracle():
    """Compile hf_oracle.c (and the reference shim where a checkout is given)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref = reference_checkout()
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "libhforacle.so")
        if not os.path.exists(path):
            build_oracle()
        L = ctypes.CDLL(path)
        L.orc_boys.restype = ctypes.c_double
        L.orc_boys.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_boys_reference.restype = ctypes.c_double
        L.orc_boys_reference.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_boys_stable.restype = ctypes.c_double
        L.orc_boys_stable.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_basis_repulsion.restype = ctypes.c_double
        L.orc_basis_repulsion.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4
        L.orc_set_stable_boys.argtypes = [ctypes.c_int]
        L.orc_schwarz_bounds.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_repulsion_tensor.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.orc_eri_list.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                   ctypes.c_size_t, ctypes.c_void_p]
        L.orc_eri_list_mt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int]
        L.orc_overlap_kinetic.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_attraction.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]
        L.orc_repulsion_matrix.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_repulsion_tensor_mt.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
        L.orc_contract_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_coulomb_matrix.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]
        L.orc_exchange_matrix.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


class Oracle:
    """Integrals of one molecule/basis through the C restatement."""

    def __init__(self, config, basis_set, basis_path=BASIS_PATH, stable_boys=False):
        self.fb = FlatBasis(config, basis_set, basis_path)
        self.K = self.fb.K
        self.stable_boys = stable_boys
        fb = self.fb
        self._c = _CBasis(fb.K, _ptr(fb.cx).value, _ptr(fb.cy).value, _ptr(fb.cz).value,
                          _ptr(fb.lmn).value, _ptr(fb.prim_off).value, _ptr(fb.alpha).value,
                          _ptr(fb.coeff).value, _ptr(fb.norm).value)

    def _mode(self):
        lib().orc_set_stable_boys(1 if self.stable_boys else 0)

    def eri(self, i, j, k, l):
        self._mode()
        return lib().orc_basis_repulsion(ctypes.byref(self._c), i, j, k, l)

    def schwarz_bounds(self):
        self._mode()
        out = np.zeros(self.K * (self.K + 1) // 2)
        lib().orc_schwarz_bounds(ctypes.byref(self._c), _ptr(out))
        return out

    def repulsion_tensor(self, threshold=1e-8):
        self._mode()
        npair = self.K * (self.K + 1) // 2
        out = np.zeros(npair * (npair + 1) // 2)
        lib().orc_repulsion_tensor(ctypes.byref(self._c), threshold, _ptr(out))
        return out

    def repulsion_tensor_mt(self, threshold=1e-8, nthreads=None):
        """repulsion_tensor spread over host threads (bit-identical result)."""
        self._mode()
        npair = self.K * (self.K + 1) // 2
        out = np.zeros(npair * (npair + 1) // 2)
        lib().orc_repulsion_tensor_mt(ctypes.byref(self._c), threshold, _ptr(out), nthreads or os.cpu_count())
        return out

    def eri_list(self, ijkl, bounds=None, threshold=1e-8, nthreads=1):
        self._mode()
        ijkl = np.ascontiguousarray(np.asarray(ijkl, dtype=np.int32).reshape(-1, 4))
        out = np.zeros(len(ijkl))
        b = _ptr(np.ascontiguousarray(bounds)) if bounds is not None else None
        if nthreads > 1:
            lib().orc_eri_list_mt(ctypes.byref(self._c), b, threshold, _ptr(ijkl), len(ijkl), _ptr(out),
                                  nthreads)
        else:
            lib().orc_eri_list(ctypes.byref(self._c), b, threshold, _ptr(ijkl), len(ijkl), _ptr(out))
        return out

    def one_electron(self):
        self._mode()
        K = self.K
        S, T, V = np.zeros((K, K)), np.zeros((K, K)), np.zeros((K, K))
        lib().orc_overlap_kinetic(ctypes.byref(self._c), _ptr(S), _ptr(T))
        lib().orc_attraction(ctypes.byref(self._c), len(self.fb.atoms_Z), _ptr(self.fb.atoms_Z),
                             _ptr(self.fb.atoms_xyz), _ptr(V))
        return S, T, V


# ---------------- grid evaluation (cube.hpp:9-168) ----------------

def linspace(start, stop, n):               # visual.hpp:42-51
    step = (stop - start) / (n - 1)
    return [start + i * step for i in range(n)]


def box_points(center, L, res):             # cube.hpp:137-168, index3d order (indexing.hpp:10-12)
    x = linspace(center[0] - L / 2, center[0] + L / 2, res)
    y = linspace(center[1] - L / 2, center[1] + L / 2, res)
    z = linspace(center[2] - L / 2, center[2] + L / 2, res)
    X, Y, Z = np.meshgrid(np.array(x), np.array(y), np.array(z), indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def basis_values(fb, r):
    """phi_mu(r) for every basis function and point, function_eval
    (cube.hpp:9-41): sum_i N_i c_i (x-Ax)^l (y-Ay)^m (z-Az)^n exp(-a_i d^2)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    phi = np.zeros((fb.K, r.shape[0]))
    lmn = fb.lmn.reshape(-1, 3)
    for mu in range(fb.K):
        A = fb.centres[mu]
        dx, dy, dz = r[:, 0] - A[0], r[:, 1] - A[1], r[:, 2] - A[2]
        d2 = dx * dx + dy * dy + dz * dz
        l, m, n = (int(v) for v in lmn[mu])
        val = np.zeros(r.shape[0])
        for i in range(fb.prim_off[mu], fb.prim_off[mu + 1]):
            val += fb.norm[i] * fb.coeff[i] * dx ** l * dy ** m * dz ** n * np.exp(-fb.alpha[i] * d2)
        phi[mu] = val
    return phi


def electron_density(fb, P, r):             # cube.hpp:44-93: sum over pairs, 2x off-diagonal
    phi = basis_values(fb, r)
    P = np.asarray(P).reshape(fb.K, fb.K)
    iu = np.triu_indices(fb.K)
    w = np.where(iu[0] == iu[1], 1.0, 2.0) * P[iu]
    return np.einsum("p,pn,pn->n", w, phi[iu[0]], phi[iu[1]])


def orbital_wf(fb, C, idx, r):              # cube.hpp:96-135
    phi = basis_values(fb, r)
    C = np.asarray(C).reshape(fb.K, fb.K)
    return C[:, idx] @ phi


def repulsion_matrix(P, eri):               # linalg.hpp:100-129
    K = P.shape[0]
    P = np.ascontiguousarray(P, dtype=np.float64)
    G = np.zeros((K, K))
    lib().orc_repulsion_matrix(K, _ptr(P), _ptr(eri), _ptr(G))
    return G


def coulomb_matrix(P1, P2, eri):            # linalg.hpp:215-257
    K = P1.shape[0]
    P1 = np.ascontiguousarray(P1, dtype=np.float64)
    P2 = np.ascontiguousarray(P2, dtype=np.float64)
    J = np.zeros((K, K))
    lib().orc_coulomb_matrix(K, _ptr(P1), _ptr(P2), _ptr(eri), _ptr(J))
    return J


def exchange_matrix(P, eri):                # linalg.hpp:260-296
    K = P.shape[0]
    P = np.ascontiguousarray(P, dtype=np.float64)
    Kx = np.zeros((K, K))
    lib().orc_exchange_matrix(K, _ptr(P), _ptr(eri), _ptr(Kx))
    return Kx


def contract_mt(kind, P1, eri, P2=None, nthreads=None):
    """repulsion_matrix ("G"), coulomb_matrix ("J", P1 + P2) or
    exchange_matrix ("K") spread over host threads; each element is the
    serial function's sum in the same order."""
    K = P1.shape[0]
    P1 = np.ascontiguousarray(P1, dtype=np.float64)
    P2 = np.ascontiguousarray(P2 if P2 is not None else np.zeros((K, K)), dtype=np.float64)
    out = np.zeros((K, K))
    lib().orc_contract_mt({"G": 1, "J": 2, "K": 3}[kind], K, _ptr(P1), _ptr(P2), _ptr(eri), _ptr(out),
                          nthreads or os.cpu_count())
    return out


def eri_index(i, j, k, l):                  # indexing.hpp:42-53
    ij = max(i, j) * (max(i, j) + 1) // 2 + min(i, j)
    kl = max(k, l) * (max(k, l) + 1) // 2 + min(k, l)
    if ij < kl:
        ij, kl = kl, ij
    return ij * (ij + 1) // 2 + kl


def full_eri(unique, K):
    """Expand the packed unique-ERI array into a dense (K,K,K,K) tensor."""
    i, j, k, l = np.meshgrid(*([np.arange(K)] * 4), indexing="ij")
    ij = np.maximum(i, j) * (np.maximum(i, j) + 1) // 2 + np.minimum(i, j)
    kl = np.maximum(k, l) * (np.maximum(k, l) + 1) // 2 + np.minimum(k, l)
    a, b = np.maximum(ij, kl), np.minimum(ij, kl)
    return unique[a * (a + 1) // 2 + b]


# ------------------------- SCF restatement (scf.hpp) -------------------------

def repulsion_energy(config):               # scf.hpp:64-78
    E = 0.0
    for a in range(len(config)):
        for b in range(a + 1, len(config)):
            Ra, Rb = np.array(config[a][1]), np.array(config[b][1])
            E += nameZ(config[a][0]) * nameZ(config[b][0]) / np.linalg.norm(Ra - Rb)
    return E


def xmatrix(S):                             # linalg.hpp:132-147
    s, U = np.linalg.eigh(S)
    return U @ np.diag(1.0 / np.sqrt(s)) @ U.T


def eig_problem(F, X):                      # linalg.hpp:150-170
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    return X @ Cp, e


def fock_diis(fock_hist, err_hist):         # linalg.hpp:405-510
    n = len(err_hist)
    B = np.zeros((n + 1, n + 1))
    for i in range(n):
        for j in range(n):
            B[i, j] = float(np.dot(err_hist[i].ravel(), err_hist[j].ravel()))
    B[:n, n] = -1.0
    B[n, :n] = 1.0
    rhs = np.zeros(n + 1)
    rhs[n] = 1.0
    c = full_piv_lu_solve(B, rhs)
    return sum(c[i] * fock_hist[i] for i in range(n))


def full_piv_lu_solve(A, b):
    """Gaussian elimination with complete pivoting, rank decided like Eigen's
    FullPivLU (pivots below eps*min(rows,cols)*|largest pivot| count as zero;
    the free unknowns of a rank-deficient system are set to zero) -- the
    reference's diis_coefficients uses A.fullPivLu().solve(rhs)
    (linalg.hpp:430-447)."""
    A = np.array(A, dtype=np.float64)
    r = np.array(b, dtype=np.float64)
    n = A.shape[0]
    colp = list(range(n))
    maxpiv = 0.0
    rank = n
    for k in range(n):
        sub = np.abs(A[k:, k:])
        pi, pj = np.unravel_index(np.argmax(sub), sub.shape)
        pi += k
        pj += k
        piv = abs(A[pi, pj])
        if k == 0:
            maxpiv = piv
        if piv <= np.finfo(float).eps * n * maxpiv or piv == 0.0:
            rank = k
            break
        if pi != k:
            A[[pi, k], :] = A[[k, pi], :]
            r[[pi, k]] = r[[k, pi]]
        if pj != k:
            A[:, [pj, k]] = A[:, [k, pj]]
            colp[pj], colp[k] = colp[k], colp[pj]
        for i in range(k + 1, n):
            f = A[i, k] / A[k, k]
            if f != 0.0:
                A[i, k:] -= f * A[k, k:]
                r[i] -= f * r[k]
    y = np.zeros(n)
    for i in range(rank - 1, -1, -1):
        y[i] = (r[i] - A[i, i + 1:rank] @ y[i + 1:rank]) / A[i, i]
    x = np.zeros(n)
    for j in range(n):
        x[colp[j]] = y[j]
    return x


def _energy(P, F, H):                       # scf.hpp:28-39
    return 0.5 * float(np.sum(P * (H + F)))


def rhf_diis(config, basis_set, charge=0, fock_builder=None, P0=None, max_it=10000, epsilon=1e-6,
             damping=0.3, screening_threshold=1e-8, energy_threshold=0.0, basis_path=BASIS_PATH,
             stable_boys=False):
    """numpy restatement of rhf_diis (scf.hpp:205-419).

    fock_builder(P) -> G overrides the stored-tensor contraction (used to run
    the same loop on another G builder).  energy_threshold > 0 adds the
    |E_n - E_{n-1}| criterion to the reference's RMSD/error criteria."""
    orc = Oracle(config, basis_set, basis_path, stable_boys)
    K = orc.K
    n_e = sum(nameZ(s) for s, _ in config) - charge
    S, T, V = orc.one_electron()
    H = T + V
    E_nuc = repulsion_energy(config)
    X = xmatrix(S)
    if fock_builder is None:
        eri = orc.repulsion_tensor(screening_threshold)
        fock_builder = lambda P: repulsion_matrix(P, eri)
    P = np.zeros((K, K)) if P0 is None else np.array(P0, dtype=np.float64).reshape(K, K)
    fock_hist, err_hist = [], []
    n_it, success, E_tot, E_prev = 0, False, 0.0, None
    C = e = None
    for i in range(max_it):
        n_it += 1
        G = fock_builder(P)
        F = H + G
        err = F @ P @ S - S @ P @ F
        fock_hist.append(F); err_hist.append(err)
        if len(fock_hist) > 8:
            fock_hist.pop(0); err_hist.pop(0)
        E_cur = _energy(P, F, H)
        if n_it >= 4:
            F = fock_diis(fock_hist, err_hist)
        C, e = eig_problem(F, X)
        nocc = n_e // 2
        P_new = 2.0 * C[:, :nocc] @ C[:, :nocc].T
        P_diff = math.sqrt(float(np.mean((P_new - P) ** 2)))
        err_norm = float(np.linalg.norm(err))
        dE_ok = energy_threshold <= 0 or (E_prev is not None and abs(E_cur - E_prev) < energy_threshold)
        E_prev = E_cur
        if P_diff < epsilon and err_norm < epsilon and dE_ok:
            Gf = fock_builder(P_new)                     # rhf_final_check scf.hpp:107-137
            Ff = H + Gf
            fe = float(np.linalg.norm(Ff @ P_new @ S - S @ P_new @ Ff))
            if fe < epsilon:
                success = True
                P = P_new
                E_tot = E_nuc + _energy(P_new, Ff, H)
                break
        P = P_new if n_it >= 4 else damping * P_new + (1 - damping) * P
        if i == max_it - 1:
            Gf = fock_builder(P)
            E_tot = E_nuc + _energy(P, H + Gf, H)
    return dict(E_tot=E_tot, E_nuc=E_nuc, iterations=n_it, converged=success, density=P,
                coefficient=C, mo_energy=e, K=K, Ne=n_e)


def uhf_diis(config, basis_set, spin_occ, charge=0, jk_builder=None, Pa0=None, Pb0=None, max_it=10000,
             epsilon=1e-6, damping=0.3, screening_threshold=1e-8, energy_threshold=0.0,
             basis_path=BASIS_PATH, stable_boys=False):
    """numpy restatement of uhf_diis (scf.hpp:423-682).  jk_builder(Pa, Pb) ->
    (J, Ka, Kb) overrides the stored-tensor contractions."""
    orc = Oracle(config, basis_set, basis_path, stable_boys)
    K = orc.K
    n_e = sum(nameZ(s) for s, _ in config) - charge
    na, nb = spin_occ
    if n_e != na + nb:
        raise RuntimeError("inconsistency in electron number")
    S, T, V = orc.one_electron()
    H = T + V
    E_nuc = repulsion_energy(config)
    X = xmatrix(S)
    if jk_builder is None:
        eri = orc.repulsion_tensor(screening_threshold)
        jk_builder = lambda Pa, Pb: (coulomb_matrix(Pa, Pb, eri), exchange_matrix(Pa, eri),
                                     exchange_matrix(Pb, eri))
    Pa = np.zeros((K, K)) if Pa0 is None else np.array(Pa0).reshape(K, K)
    Pb = np.zeros((K, K)) if Pb0 is None else np.array(Pb0).reshape(K, K)
    fock_hist, err_hist = [], []
    n_it, success, E_tot, E_prev = 0, False, 0.0, None
    for i in range(max_it):
        n_it += 1
        J, Ka, Kb = jk_builder(Pa, Pb)
        Fa, Fb = H + J - Ka, H + J - Kb
        Ra = Fa @ Pa @ S - S @ Pa @ Fa
        Rb = Fb @ Pb @ S - S @ Pb @ Fb
        E_cur = _energy(Pa, Fa, H) + _energy(Pb, Fb, H)
        fock_hist.append(np.concatenate([Fa.ravel(), Fb.ravel()]))
        err_hist.append(np.concatenate([Ra.ravel(), Rb.ravel()]))
        if len(fock_hist) > 8:
            fock_hist.pop(0); err_hist.pop(0)
        if n_it >= 4:
            Fd = fock_diis(fock_hist, err_hist)
            Fa, Fb = Fd[:K * K].reshape(K, K), Fd[K * K:].reshape(K, K)
        Ca, Ea = eig_problem(Fa, X)
        Cb, Eb = eig_problem(Fb, X)
        Pa_new = Ca[:, :na] @ Ca[:, :na].T
        Pb_new = Cb[:, :nb] @ Cb[:, :nb].T
        da = math.sqrt(float(np.mean((Pa - Pa_new) ** 2)))
        db = math.sqrt(float(np.mean((Pb - Pb_new) ** 2)))
        en = float(np.linalg.norm(np.concatenate([Ra.ravel(), Rb.ravel()])))
        dE_ok = energy_threshold <= 0 or (E_prev is not None and abs(E_cur - E_prev) < energy_threshold)
        E_prev = E_cur
        if da < epsilon and db < epsilon and en < epsilon and dE_ok:
            J, Ka, Kb = jk_builder(Pa_new, Pb_new)           # uhf_final_check scf.hpp:140-185
            Fa_f, Fb_f = H + J - Ka, H + J - Kb
            ea = np.linalg.norm(Fa_f @ Pa_new @ S - S @ Pa_new @ Fa_f)
            eb = np.linalg.norm(Fb_f @ Pb_new @ S - S @ Pb_new @ Fb_f)
            if math.sqrt(ea * ea + eb * eb) < epsilon:
                success = True
                Pa, Pb = Pa_new, Pb_new
                E_tot = E_nuc + _energy(Pa, Fa_f, H) + _energy(Pb, Fb_f, H)
                break
        if n_it >= 4:
            Pa, Pb = Pa_new, Pb_new
        else:
            Pa = damping * Pa_new + (1 - damping) * Pa
            Pb = damping * Pb_new + (1 - damping) * Pb
        if i == max_it - 1:
            J, Ka, Kb = jk_builder(Pa, Pb)
            E_tot = E_nuc + _energy(Pa, H + J - Ka, H) + _energy(Pb, H + J - Kb, H)
    return dict(E_tot=E_tot, E_nuc=E_nuc, iterations=n_it, converged=success, Pa=Pa, Pb=Pb, K=K,
                Ea=Ea, Eb=Eb)


# ------------------- reference compiled unchanged (optional) ------------------

class RefLib:
    """The reference's own integrals.hpp via oracle/_ref/libhfref.so (exists
    only where a checkout of the reference was available at build time)."""

    def __init__(self):
        path = os.path.join(HERE, "_ref", "libhfref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        L.ref_build_basis.restype = ctypes.c_int
        L.ref_build_basis.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                      ctypes.c_char_p]
        L.ref_boys.restype = ctypes.c_double
        L.ref_boys.argtypes = [ctypes.c_int, ctypes.c_double]
        L.ref_basis_repulsion.restype = ctypes.c_double
        L.ref_basis_repulsion.argtypes = [ctypes.c_int] * 4
        L.ref_schwarz_bounds.argtypes = [ctypes.c_void_p]
        L.ref_repulsion_tensor.argtypes = [ctypes.c_double, ctypes.c_void_p]
        L.ref_repulsion_tensor_mt.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
        L.ref_one_electron.argtypes = [ctypes.c_void_p] * 3
        L.ref_nprims_total.restype = ctypes.c_int
        L.ref_export_basis.argtypes = [ctypes.c_void_p] * 6
        self.L = L
        self.K = 0

    def build(self, config, basis_set, basis_path=BASIS_PATH):
        syms = (ctypes.c_char_p * len(config))(*[s.encode() for s, _ in config])
        xyz = np.ascontiguousarray(np.array([R for _, R in config], dtype=np.float64).reshape(-1))
        K = self.L.ref_build_basis(len(config), ctypes.cast(syms, ctypes.c_void_p), _ptr(xyz),
                                   basis_set.encode(), basis_path.encode())
        if K < 0:
            raise RuntimeError("reference basis_construction failed")
        self.K = K
        return K

    def export_basis(self):
        K, n = self.K, self.L.ref_nprims_total()
        c, lmn, off = np.zeros(3 * K), np.zeros(3 * K, np.int32), np.zeros(K + 1, np.int32)
        a, co, no = np.zeros(n), np.zeros(n), np.zeros(n)
        self.L.ref_export_basis(_ptr(c), _ptr(lmn), _ptr(off), _ptr(a), _ptr(co), _ptr(no))
        return c.reshape(K, 3), lmn.reshape(K, 3), off, a, co, no

    def schwarz_bounds(self):
        out = np.zeros(self.K * (self.K + 1) // 2)
        self.L.ref_schwarz_bounds(_ptr(out))
        return out

    def repulsion_tensor(self, threshold=1e-8):
        npair = self.K * (self.K + 1) // 2
        out = np.zeros(npair * (npair + 1) // 2)
        self.L.ref_repulsion_tensor(threshold, _ptr(out))
        return out

    def repulsion_tensor_mt(self, threshold=1e-8, nthreads=None):
        npair = self.K * (self.K + 1) // 2
        out = np.zeros(npair * (npair + 1) // 2)
        self.L.ref_repulsion_tensor_mt(threshold, _ptr(out), nthreads or os.cpu_count())
        return out

    def eri(self, i, j, k, l):
        return self.L.ref_basis_repulsion(i, j, k, l)

    def one_electron(self):
        K = self.K
        S, T, V = np.zeros((K, K)), np.zeros((K, K)), np.zeros((K, K))
        self.L.ref_one_electron(_ptr(S), _ptr(T), _ptr(V))
        return S, T, V


class RefGridLib:
    """The reference's own cube.hpp grid evaluation via
    oracle/_ref/libhfref_grid.so (only where a checkout of the reference was
    available at build time)."""

    def __init__(self):
        path = os.path.join(HERE, "_ref", "libhfref_grid.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        L.refg_build_basis.restype = ctypes.c_int
        L.refg_build_basis.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                       ctypes.c_char_p]
        L.refg_points.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.refg_box_points.argtypes = [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.c_void_p]
        self.L = L
        self.K = 0

    def build(self, config, basis_set, basis_path=BASIS_PATH):
        syms = (ctypes.c_char_p * len(config))(*[s.encode() for s, _ in config])
        xyz = np.ascontiguousarray(np.array([R for _, R in config], dtype=np.float64).reshape(-1))
        K = self.L.refg_build_basis(len(config), ctypes.cast(syms, ctypes.c_void_p), _ptr(xyz),
                                    basis_set.encode(), basis_path.encode())
        if K < 0:
            raise RuntimeError("reference basis_construction failed")
        self.K = K
        return K

    def points(self, M, column, xyz):
        M = np.ascontiguousarray(M, dtype=np.float64)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz))
        self.L.refg_points(_ptr(M), int(column), _ptr(xyz), len(xyz), _ptr(out))
        return out

    def box_points(self, center, L, res):
        out = np.zeros((res ** 3, 3))
        self.L.refg_box_points(float(center[0]), float(center[1]), float(center[2]), float(L), int(res), _ptr(out))
        return out
