"""hartree_fock_cpp_gb300 -- GB300-native direct-SCF Fock-build engine behind
the ERI/Fock call of KLYYCYNN/hartree_fock_cpp.

Host-side mirror of the reference's interface for this path, over the C ABI
of libhfx.so (include/hfx.h):

  basis_construction(config, basis_set, param_path)   basis.hpp:157-262
  schwarz_bounds(basis)                                integrals.hpp:732-752
  ERI_GPU(basis, threshold)                            eri.cu:20-89 (packed eri_index layout)
  FockBuilder(...).repulsion_matrix(P)                 linalg.hpp:100-129 (direct, no stored tensor)
  FockBuilder(...).coulomb_exchange(Pa, Pb)            linalg.hpp:215-296
  rhf_diis(config, basis_set, param_path, ...)          scf.hpp:205-419
  uhf_diis(config, basis_set, param_path, spin_occ, ...) scf.hpp:423-682

``config`` is the reference's list of (symbol, (x, y, z)) pairs in bohr.
Errors raise HfxError carrying the engine's status code; the engine has no
CPU fallback (eri_device "CPU" is the reference's own stored-tensor path and
is not part of this library).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import BASIS_PATH, HFX_EIG_AUTO, HFX_EIG_SYEVD, HFX_PREC_FP64, HFX_PREC_MIXED, HfxError, check, lib, ptr

__all__ = ["Basis", "basis_construction", "schwarz_bounds", "ERI_GPU", "FockBuilder", "rhf_diis", "uhf_diis",
           "one_electron", "measure_peaks", "measure_dmma_peak", "HfxError", "HFX_PREC_FP64", "HFX_PREC_MIXED",
           "HFX_EIG_AUTO", "HFX_EIG_SYEVD", "BASIS_PATH",
           "eri_index", "pair_index", "batch_scf"]


def pair_index(a, b):                     # indexing.hpp:33-40
    if a < b:
        a, b = b, a
    return a * (a + 1) // 2 + b


def eri_index(i, j, k, l):                # indexing.hpp:42-53
    ij, kl = pair_index(i, j), pair_index(k, l)
    if ij < kl:
        ij, kl = kl, ij
    return ij * (ij + 1) // 2 + kl


class Basis:
    """Flat basis-function list (the reference's std::vector<basis_function>)."""

    def __init__(self, centres, lmn, prim_offset, alpha, coeff, norm):
        self.centres = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1, 3)
        self.lmn = np.ascontiguousarray(lmn, dtype=np.int32).reshape(-1, 3)
        self.prim_offset = np.ascontiguousarray(prim_offset, dtype=np.int32)
        self.alpha = np.ascontiguousarray(alpha, dtype=np.float64)
        self.coeff = np.ascontiguousarray(coeff, dtype=np.float64)
        self.norm = np.ascontiguousarray(norm, dtype=np.float64)
        self.K = self.lmn.shape[0]
        self.c = _lib.Functions(self.K, self.centres.ctypes.data, self.lmn.ctypes.data, self.prim_offset.ctypes.data,
                                self.alpha.ctypes.data, self.coeff.ctypes.data, self.norm.ctypes.data)

    def ref(self):
        return ctypes.byref(self.c)

    def __len__(self):
        return self.K


def basis_construction(config, basis_set, param_path=None):
    """basis.hpp:157-262 -- atoms in order, CSV shells in order, Cartesian
    components in angmom_partition order, cart_norm per component."""
    m = _lib.MoleculeArgs(config, basis_set, param_path)
    K, n = ctypes.c_int(), ctypes.c_int()
    check(lib.hfx_build_functions(m.ref(), ctypes.byref(K), ctypes.byref(n), None, None, None, None, None, None))
    K, n = K.value, n.value
    c, lmn, off = np.zeros(3 * K), np.zeros(3 * K, np.int32), np.zeros(K + 1, np.int32)
    a, co, no = np.zeros(n), np.zeros(n), np.zeros(n)
    check(lib.hfx_build_functions(m.ref(), None, None, ptr(c), ptr(lmn), ptr(off), ptr(a), ptr(co), ptr(no)))
    return Basis(c, lmn, off, a, co, no)


def _options(screening_threshold=1e-8, precision=HFX_PREC_FP64, fp32_threshold=0.0, device=0):
    o = _lib.Options()
    o.screening_threshold = screening_threshold
    o.precision = precision
    o.fp32_threshold = fp32_threshold
    o.device = device
    return o


class FockBuilder:
    """One device-resident job (basis, pair data, Schwarz table, quartet work
    lists) reused for every Fock build of an SCF."""

    def __init__(self, basis=None, *, config=None, basis_set=None, param_path=None, screening_threshold=1e-8,
                 precision=HFX_PREC_FP64, fp32_threshold=0.0, device=0):
        self._opt = _options(screening_threshold, precision, fp32_threshold, device)
        self._job = ctypes.c_void_p()
        if basis is not None:
            self._basis = basis
            check(lib.hfx_create(basis.ref(), ctypes.byref(self._opt), ctypes.byref(self._job)))
        else:
            self._mol = _lib.MoleculeArgs(config, basis_set, param_path)
            check(lib.hfx_create_molecule(self._mol.ref(), ctypes.byref(self._opt), ctypes.byref(self._job)))
        k = ctypes.c_int()
        check(lib.hfx_nbasis(self._job, ctypes.byref(k)))
        self.K = k.value

    def close(self):
        if self._job:
            check(lib.hfx_destroy(self._job))
            self._job = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _mat(self, P):
        P = np.ascontiguousarray(P, dtype=np.float64)
        if P.shape != (self.K, self.K):
            raise HfxError(1, "density must be %d x %d" % (self.K, self.K))
        return P

    def schwarz_bounds(self):
        Q = np.zeros(self.K * (self.K + 1) // 2)
        check(lib.hfx_schwarz(self._job, ptr(Q)))
        return Q

    def repulsion_matrix(self, P):
        """G = J[P] - 1/2 K[P] (linalg.hpp:100-129)."""
        P = self._mat(P)
        G = np.zeros_like(P)
        check(lib.hfx_fock_rhf(self._job, ptr(P), ptr(G)))
        return G

    def coulomb_exchange(self, Pa, Pb):
        """(J[Pa+Pb], K[Pa], K[Pb]) (linalg.hpp:215-296)."""
        Pa, Pb = self._mat(Pa), self._mat(Pb)
        J, Ka, Kb = np.zeros_like(Pa), np.zeros_like(Pa), np.zeros_like(Pa)
        check(lib.hfx_fock_uhf(self._job, ptr(Pa), ptr(Pb), ptr(J), ptr(Ka), ptr(Kb)))
        return J, Ka, Kb

    def repulsion_matrix_device(self, dP_ptr, dG_ptr):
        """Device-pointer variant (pointers as ints, K*K doubles each)."""
        check(lib.hfx_fock_rhf_device(self._job, ctypes.c_void_p(dP_ptr), ctypes.c_void_p(dG_ptr)))

    def coulomb_exchange_device(self, dPa, dPb, dJ, dKa, dKb):
        check(lib.hfx_fock_uhf_device(self._job, *[ctypes.c_void_p(x) for x in (dPa, dPb, dJ, dKa, dKb)]))

    def eri_unique(self, threshold=1e-8):
        npair = self.K * (self.K + 1) // 2
        out = np.zeros(npair * (npair + 1) // 2)
        check(lib.hfx_eri_unique(self._job, threshold, ptr(out)))
        return out

    def autotune_fp32_threshold(self, P, target_dE=2.5e-7):
        """Largest FP32 Schwarz cut keeping |dE| at density P within target_dE;
        switches this job to mixed precision at it.  Returns (tau, dE,
        ms_fp64, ms_mixed)."""
        P = self._mat(P)
        t, d, a, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib.hfx_autotune_fp32_threshold(self._job, ptr(P), target_dE, ctypes.byref(t), ctypes.byref(d),
                                              ctypes.byref(a), ctypes.byref(b)))
        return t.value, d.value, a.value, b.value

    def launch_shape(self):
        s = _lib.LaunchShape()
        check(lib.hfx_get_launch_shape(self._job, ctypes.byref(s)))
        return dict(small_chunk=s.small_chunk, warp_chunk=s.warp_chunk, warp_max_warps=s.warp_max_warps,
                    lane_min_npp=s.lane_min_npp)

    def set_launch_shape(self, small_chunk=256, warp_chunk=4096, warp_max_warps=8, lane_min_npp=6):
        s = _lib.LaunchShape(small_chunk, warp_chunk, warp_max_warps, lane_min_npp)
        check(lib.hfx_set_launch_shape(self._job, ctypes.byref(s)))

    def autotune_launch_shape(self, P, builds=2):
        """Coordinate search over the launch shape at density P; the job keeps
        the fastest.  Returns (shape dict, best build ms)."""
        P = self._mat(P)
        s = _lib.LaunchShape()
        ms = ctypes.c_double()
        check(lib.hfx_autotune_launch_shape(self._job, ptr(P), int(builds), ctypes.byref(s), ctypes.byref(ms)))
        return dict(small_chunk=s.small_chunk, warp_chunk=s.warp_chunk, warp_max_warps=s.warp_max_warps,
                    lane_min_npp=s.lane_min_npp), ms.value

    def plan(self, mixed=None):
        """Launch groups of the job's Fock-build plan (the mixed plan of a mixed
        job unless mixed=False): one dict per group."""
        m = 1 if mixed is None or mixed else 0
        n = ctypes.c_int()
        check(lib.hfx_debug_plan(self._job, m, ctypes.byref(n), None))
        rows = np.zeros((n.value, 10))
        check(lib.hfx_debug_plan(self._job, m, ctypes.byref(n), ptr(rows)))
        keys = ("kind", "pcb", "pck", "fp32", "tasks", "flops", "prims", "grid", "slice", "warps_per_cta")
        return [{k: (float(v) if k in ("flops", "prims") else int(v)) for k, v in zip(keys, r)} for r in rows]

    def stats(self):
        s = _lib.BuildStats()
        check(lib.hfx_last_build_stats(self._job, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _lib.BuildStats._fields_ if k != "reserved"}


def schwarz_bounds(basis):
    """integrals.hpp:732-752 on the device."""
    with FockBuilder(basis, screening_threshold=-1.0) as fb:
        return fb.schwarz_bounds()


def ERI_GPU(basis, threshold=1e-8):
    """Literal replacement of ERI_GPU (eri.cu:20-89): all unique ERIs in
    eri_index order, zero where Q_ij*Q_kl < threshold."""
    npair = basis.K * (basis.K + 1) // 2
    out = np.zeros(npair * (npair + 1) // 2)
    check(lib.hfx_eri_gpu(basis.ref(), threshold, ptr(out)))
    return out


def _scf_options(charge, max_it, epsilon, damping, screening_threshold, energy_threshold, precision,
                 fp32_threshold, eigensolver=0):
    o = _lib.ScfOptions()
    o.eigensolver = eigensolver
    o.max_iterations = max_it
    o.epsilon = epsilon
    o.damping = damping
    o.screening_threshold = screening_threshold
    o.energy_threshold = energy_threshold
    o.charge = charge
    o.precision = precision
    o.fp32_threshold = fp32_threshold
    return o


def _check_device(eri_device):
    if eri_device not in ("CPU", "GPU"):
        raise HfxError(1, "unsupported ERI computing platform")      # scf.hpp:223-225
    if eri_device == "CPU":
        raise HfxError(5, "eri_device 'CPU' is the reference's stored-tensor path; this engine is the GPU path")


def rhf_diis(config, basis_set, param_path=None, charge=0, eri_device="GPU", set_initial_density=False, P0=None,
             max_it=10000, epsilon=1e-6, damping=0.3, screening_threshold=1e-8, energy_threshold=0.0,
             precision=HFX_PREC_FP64, fp32_threshold=0.0, raise_on_nonconvergence=False, eigensolver=HFX_EIG_AUTO,
             verbose=False):
    """scf.hpp:205-419 with the direct GPU Fock build.  Returns a dict shaped
    like the reference's rhf_data (types.hpp:50-73).  eigensolver: the density
    step, HFX_EIG_AUTO (SP2 projector, syevd fallback) or HFX_EIG_SYEVD;
    verbose: one line per iteration on stderr."""
    _check_device(eri_device)
    m = _lib.MoleculeArgs(config, basis_set, param_path)
    o = _scf_options(charge, max_it, epsilon, damping, screening_threshold, energy_threshold, precision,
                     fp32_threshold, eigensolver)
    o.verbose = int(bool(verbose))
    K = ctypes.c_int()
    check(lib.hfx_one_electron(m.ref(), None, None, None, ctypes.byref(K)))
    K = K.value
    P0a = None
    if set_initial_density:
        P0a = np.ascontiguousarray(P0, dtype=np.float64).reshape(-1)
        if P0a.size != K * K:
            raise HfxError(1, "initial density matrix dimension inconsistent with basis size")
    r = _lib.ScfResult()
    dens, coef, mo = np.zeros((K, K)), np.zeros((K, K)), np.zeros(K)
    st = lib.hfx_rhf_diis(m.ref(), ctypes.byref(o), ptr(P0a), ctypes.byref(r), ptr(dens), ptr(coef), ptr(mo))
    if st != 0 and not (st == 6 and not raise_on_nonconvergence):
        check(st)
    return dict(E_tot=r.E_tot, E_ele=r.E_ele, E_nuc=r.E_nuc, iterations=r.iterations, converged=bool(r.converged),
                K=r.K, Ne=r.n_electrons, density=dens, coefficient=coef, mo_energy=mo, duration=r.seconds,
                fock_ms=r.fock_ms, fock_builds=r.fock_builds, mixed_builds=r.mixed_builds, fp64_builds=r.fp64_builds,
                delta_builds=r.delta_builds, projections=r.projections,
                projection_fallbacks=r.projection_fallbacks, hardware=eri_device, BasisSet=basis_set, charge=charge)


def uhf_diis(config, basis_set, param_path=None, spin_occ=(1, 0), charge=0, eri_device="GPU",
             set_initial_density=False, Pa0=None, Pb0=None, max_it=10000, epsilon=1e-6, damping=0.3,
             screening_threshold=1e-8, energy_threshold=0.0, precision=HFX_PREC_FP64, fp32_threshold=0.0,
             raise_on_nonconvergence=False, eigensolver=HFX_EIG_AUTO):
    """scf.hpp:423-682 with the direct GPU J/Ka/Kb build."""
    _check_device(eri_device)
    m = _lib.MoleculeArgs(config, basis_set, param_path)
    o = _scf_options(charge, max_it, epsilon, damping, screening_threshold, energy_threshold, precision,
                     fp32_threshold, eigensolver)
    K = ctypes.c_int()
    check(lib.hfx_one_electron(m.ref(), None, None, None, ctypes.byref(K)))
    K = K.value
    a0 = b0 = None
    if set_initial_density:
        a0 = np.ascontiguousarray(Pa0, dtype=np.float64).reshape(-1)
        b0 = np.ascontiguousarray(Pb0, dtype=np.float64).reshape(-1)
        if a0.size != K * K or b0.size != K * K:
            raise HfxError(1, "initial density matrix dimension inconsistent with basis size")
    r = _lib.ScfResult()
    Pa, Pb, ea, eb = np.zeros((K, K)), np.zeros((K, K)), np.zeros(K), np.zeros(K)
    st = lib.hfx_uhf_diis(m.ref(), ctypes.byref(o), int(spin_occ[0]), int(spin_occ[1]), ptr(a0), ptr(b0),
                          ctypes.byref(r), ptr(Pa), ptr(Pb), ptr(ea), ptr(eb))
    if st != 0 and not (st == 6 and not raise_on_nonconvergence):
        check(st)
    return dict(E_tot=r.E_tot, E_ele=r.E_ele, E_nuc=r.E_nuc, iterations=r.iterations, converged=bool(r.converged),
                K=r.K, Pa=Pa, Pb=Pb, Ea=ea, Eb=eb, duration=r.seconds, fock_ms=r.fock_ms,
                fock_builds=r.fock_builds, mixed_builds=r.mixed_builds, fp64_builds=r.fp64_builds,
                delta_builds=r.delta_builds, projections=r.projections,
                projection_fallbacks=r.projection_fallbacks, Na=int(spin_occ[0]), Nb=int(spin_occ[1]), hardware=eri_device,
                BasisSet=basis_set, charge=charge)


def batch_scf(molecules, method="RHF", spins=None, charge=0, max_it=10000, epsilon=1e-6, damping=0.3,
              screening_threshold=1e-8, energy_threshold=0.0, precision=HFX_PREC_FP64, fp32_threshold=0.0,
              max_parallel=0, param_path=None, warm_chain=0, eigensolver=HFX_EIG_AUTO):
    """Lockstep batched SCF (hfx_batch_scf): `molecules` is a list of
    (config, basis_set); all of them iterate together on one packed job, one
    Fock build per SCF cycle over every molecule still iterating.  The
    batched counterpart of the reference's sequential scan drivers
    (run.hpp:300-423, 498-577).  warm_chain = c > 1: chains of c consecutive
    molecules, each starting from the previous one's final density (the
    reference scan's warm start, run.hpp:353-368), the chains iterating
    together; otherwise every molecule starts from the zero density.
    UHF takes spins = [(n_alpha, n_beta), ...].  Returns (results, stats):
    one dict per molecule (E_tot, iterations, converged, ...) and the batch's
    timing."""
    n = len(molecules)
    if n == 0:
        return [], {}
    uhf = method.upper() == "UHF"
    if uhf and (spins is None or len(spins) != n):
        raise HfxError(1, "batch UHF needs one (n_alpha, n_beta) per molecule")
    args = [_lib.MoleculeArgs(cfg, bs, param_path) for cfg, bs in molecules]
    mols = (_lib.Molecule * n)(*[a.c for a in args])
    na = nb = None
    if uhf:
        na = np.ascontiguousarray([int(s[0]) for s in spins], dtype=np.int32)
        nb = np.ascontiguousarray([int(s[1]) for s in spins], dtype=np.int32)
    o = _scf_options(charge, max_it, epsilon, damping, screening_threshold, energy_threshold, precision,
                     fp32_threshold, eigensolver)
    bo = _lib.BatchOptions()
    bo.method = 1 if uhf else 0
    bo.max_parallel = int(max_parallel)
    bo.warm_chain = int(warm_chain)
    res = (_lib.ScfResult * n)()
    st = _lib.BatchStats()
    status = lib.hfx_batch_scf(ctypes.cast(mols, ctypes.c_void_p), n, ptr(na), ptr(nb), ctypes.byref(o),
                               ctypes.byref(bo), ctypes.cast(res, ctypes.c_void_p), ctypes.byref(st))
    if status not in (0, 6):
        check(status)
    out = [dict(E_tot=r.E_tot, E_ele=r.E_ele, E_nuc=r.E_nuc, iterations=r.iterations, converged=bool(r.converged),
                K=r.K, duration=r.seconds, fock_ms=r.fock_ms, fock_builds=r.fock_builds,
                mixed_builds=r.mixed_builds, fp64_builds=r.fp64_builds, delta_builds=r.delta_builds, projections=r.projections,
                projection_fallbacks=r.projection_fallbacks)
           for r in res]
    stats = dict(seconds=st.seconds, setup_seconds=st.setup_seconds, cycles=st.cycles, molecules=st.molecules,
                 build_ms=st.build_ms, quartets=st.quartets, flops_fp64=st.flops_fp64)
    return out, stats


def one_electron(config, basis_set, param_path=None, gpu=False, device=0):
    """(S, T, V) of the molecule (integrals.hpp:10-536), on the host or, with
    gpu=True, on CUDA device `device`."""
    m = _lib.MoleculeArgs(config, basis_set, param_path)
    K = ctypes.c_int()
    check(lib.hfx_one_electron(m.ref(), None, None, None, ctypes.byref(K)))
    K = K.value
    S, T, Vm = np.zeros((K, K)), np.zeros((K, K)), np.zeros((K, K))
    if gpu:
        check(lib.hfx_one_electron_gpu(m.ref(), int(device), ptr(S), ptr(T), ptr(Vm), None))
    else:
        check(lib.hfx_one_electron(m.ref(), ptr(S), ptr(T), ptr(Vm), None))
    return S, T, Vm


def measure_peaks(device=0):
    """FP64 and FP32 FMA-loop GFLOP/s of the device."""
    a, b = ctypes.c_double(), ctypes.c_double()
    check(lib.hfx_measure_peaks(device, ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def measure_dmma_peak(device=0):
    """FP64 tensor-core (mma.sync m8n8k4 f64) loop GFLOP/s of the device."""
    a = ctypes.c_double()
    check(lib.hfx_measure_dmma_peak(device, ctypes.byref(a)))
    return a.value
