"""ctypes binding of libhfx.so (include/hfx.h).

The engine has no CPU fallback: if the shared library is missing this module
raises at import, and every compute call goes through the CUDA library.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhfx.so")
BASIS_PATH = os.path.join(HERE, "basis")

HFX_OK = 0
STATUS_NAMES = {0: "HFX_OK", 1: "HFX_ERR_INVALID", 2: "HFX_ERR_BASIS", 3: "HFX_ERR_CUDA", 4: "HFX_ERR_OOM",
                5: "HFX_ERR_UNSUPPORTED", 6: "HFX_ERR_NOT_CONVERGED", 7: "HFX_ERR_CANCELLED", 8: "HFX_ERR_TIMEOUT",
                9: "HFX_ERR_NUMERIC"}
HFX_PREC_FP64 = 0
HFX_PREC_MIXED = 1
HFX_EIG_AUTO = 0
HFX_EIG_SYEVD = 1


class HfxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class Functions(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int), ("centres", ctypes.c_void_p), ("lmn", ctypes.c_void_p),
                ("prim_offset", ctypes.c_void_p), ("alpha", ctypes.c_void_p), ("coeff", ctypes.c_void_p),
                ("norm", ctypes.c_void_p)]


class Molecule(ctypes.Structure):
    _fields_ = [("natom", ctypes.c_int), ("symbols", ctypes.c_void_p), ("xyz", ctypes.c_void_p),
                ("basis_set", ctypes.c_char_p), ("basis_path", ctypes.c_char_p)]


class Options(ctypes.Structure):
    _fields_ = [("screening_threshold", ctypes.c_double), ("precision", ctypes.c_int),
                ("fp32_threshold", ctypes.c_double), ("device", ctypes.c_int), ("reserved", ctypes.c_int * 8)]


class BuildStats(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double), ("kernel_ms", ctypes.c_double), ("quartets", ctypes.c_double), ("quartets_fp32", ctypes.c_double),
                ("prim_quartets", ctypes.c_double), ("flops_fp64", ctypes.c_double),
                ("flops_fp32", ctypes.c_double), ("launches", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


class LaunchShape(ctypes.Structure):
    _fields_ = [("small_chunk", ctypes.c_int), ("warp_chunk", ctypes.c_int), ("warp_max_warps", ctypes.c_int),
                ("lane_min_npp", ctypes.c_int), ("reserved", ctypes.c_int * 4)]


class ScfOptions(ctypes.Structure):
    _fields_ = [("max_iterations", ctypes.c_int), ("epsilon", ctypes.c_double), ("damping", ctypes.c_double),
                ("screening_threshold", ctypes.c_double), ("energy_threshold", ctypes.c_double),
                ("charge", ctypes.c_int), ("precision", ctypes.c_int), ("fp32_threshold", ctypes.c_double),
                ("fp64_final_cycles", ctypes.c_int), ("start_diis", ctypes.c_int), ("max_history", ctypes.c_int),
                ("verbose", ctypes.c_int), ("eigensolver", ctypes.c_int), ("reserved", ctypes.c_int * 5)]


class ScfResult(ctypes.Structure):
    _fields_ = [("E_tot", ctypes.c_double), ("E_ele", ctypes.c_double), ("E_nuc", ctypes.c_double),
                ("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("K", ctypes.c_int),
                ("n_electrons", ctypes.c_int), ("seconds", ctypes.c_double), ("fock_ms", ctypes.c_double),
                ("fock_builds", ctypes.c_int), ("mixed_builds", ctypes.c_int), ("fp64_builds", ctypes.c_int),
                ("delta_builds", ctypes.c_int), ("projections", ctypes.c_int),
                ("projection_fallbacks", ctypes.c_int), ("reserved", ctypes.c_int * 2)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("max_active", ctypes.c_int), ("hbm_budget_gb", ctypes.c_double), ("device", ctypes.c_int),
                ("precision", ctypes.c_int), ("fp32_threshold", ctypes.c_double), ("pack_max", ctypes.c_int),
                ("reserved", ctypes.c_int * 7)]


class Request(ctypes.Structure):
    _fields_ = [("mol", Molecule), ("method", ctypes.c_int), ("n_alpha", ctypes.c_int), ("n_beta", ctypes.c_int),
                ("scf", ScfOptions), ("precision", ctypes.c_int), ("fp32_threshold", ctypes.c_double),
                ("timeout_s", ctypes.c_double), ("inject_fault", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


class JobInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("status", ctypes.c_int), ("E_tot", ctypes.c_double),
                ("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("K", ctypes.c_int),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_end", ctypes.c_double),
                ("fock_ms", ctypes.c_double), ("fock_builds", ctypes.c_int), ("message", ctypes.c_char * 256)]


class ServerStats(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_int), ("running", ctypes.c_int), ("done", ctypes.c_int), ("failed", ctypes.c_int),
                ("max_concurrent", ctypes.c_int), ("budget_bytes", ctypes.c_double),
                ("in_use_bytes", ctypes.c_double), ("max_session_members", ctypes.c_int),
                ("sessions_created", ctypes.c_int), ("reserved", ctypes.c_int * 4)]


class BatchOptions(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("max_parallel", ctypes.c_int), ("warm_chain", ctypes.c_int),
                ("reserved", ctypes.c_int * 5)]


class BatchStats(ctypes.Structure):
    _fields_ = [("seconds", ctypes.c_double), ("setup_seconds", ctypes.c_double), ("cycles", ctypes.c_int),
                ("molecules", ctypes.c_int), ("build_ms", ctypes.c_double), ("quartets", ctypes.c_double),
                ("flops_fp64", ctypes.c_double), ("reserved", ctypes.c_double * 5)]


G_BUILDER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double))
JK_BUILDER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))

V = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
P = ctypes.POINTER

# symbol -> (restype, argtypes); every symbol include/hfx.h declares
SIGNATURES = {
    "hfx_create": (I, [V, V, P(V)]),
    "hfx_create_molecule": (I, [V, V, P(V)]),
    "hfx_destroy": (I, [V]),
    "hfx_nbasis": (I, [V, P(I)]),
    "hfx_export_functions": (I, [V, V, V, V, V, V, V, P(I)]),
    "hfx_schwarz": (I, [V, V]),
    "hfx_fock_rhf": (I, [V, V, V]),
    "hfx_fock_uhf": (I, [V, V, V, V, V, V]),
    "hfx_fock_rhf_device": (I, [V, V, V]),
    "hfx_fock_uhf_device": (I, [V, V, V, V, V, V]),
    "hfx_fock_rhf_device_noalloc": (I, [V, V, V]),
    "hfx_eri_unique": (I, [V, D, V]),
    "hfx_eri_gpu": (I, [V, D, V]),
    "hfx_job_rhf": (I, [V, V, V, V, V, V, V]),
    "hfx_job_uhf": (I, [V, V, I, I, V, V, V, V, V]),
    "hfx_last_build_stats": (I, [V, V]),
    "hfx_get_launch_shape": (I, [V, V]),
    "hfx_set_launch_shape": (I, [V, V]),
    "hfx_autotune_launch_shape": (I, [V, V, I, V, P(D)]),
    "hfx_autotune_fp32_threshold": (I, [V, V, D, P(D), P(D), P(D), P(D)]),
    "hfx_rhf_diis": (I, [V, V, V, V, V, V, V]),
    "hfx_uhf_diis": (I, [V, V, I, I, V, V, V, V, V, V, V]),
    "hfx_rhf_diis_with_builder": (I, [V, V, V, G_BUILDER, V, V, V, V]),
    "hfx_uhf_diis_with_builder": (I, [V, V, I, I, JK_BUILDER, V, V, V, V]),
    "hfx_build_functions": (I, [V, P(I), P(I), V, V, V, V, V, V]),
    "hfx_debug_pair_data": (I, [V, P(I), P(I), P(ctypes.c_longlong), V, V, V]),
    "hfx_debug_packed_pairs": (I, [V, I, P(I), V, V]),
    "hfx_debug_plan": (I, [V, I, P(I), V]),
    "hfx_one_electron": (I, [V, V, V, V, P(I)]),
    "hfx_one_electron_gpu": (I, [V, I, V, V, V, P(I)]),
    "hfx_grid_density": (I, [V, I, V, V, D, I, V]),
    "hfx_grid_orbital": (I, [V, I, V, I, V, D, I, V]),
    "hfx_points_eval": (I, [V, I, V, I, V, ctypes.c_longlong, V]),
    "hfx_last_error": (I, [ctypes.c_char_p, ctypes.c_size_t]),
    "hfx_measure_peaks": (I, [I, P(D), P(D)]),
    "hfx_measure_dmma_peak": (I, [I, P(D)]),
    "hfx_server_create": (I, [V, P(V)]),
    "hfx_server_submit": (I, [V, V, P(ctypes.c_longlong)]),
    "hfx_server_poll": (I, [V, ctypes.c_longlong, V]),
    "hfx_server_wait": (I, [V, ctypes.c_longlong, D, V]),
    "hfx_server_cancel": (I, [V, ctypes.c_longlong]),
    "hfx_server_drain": (I, [V, D]),
    "hfx_server_density": (I, [V, ctypes.c_longlong, V, V]),
    "hfx_server_stats": (I, [V, V]),
    "hfx_server_destroy": (I, [V]),
    "hfx_batch_scf": (I, [V, I, V, V, V, V, V, V]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libhfx.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`"
                          % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib.hfx_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status):
    if status != HFX_OK:
        raise HfxError(status, last_error())
    return status


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class MoleculeArgs:
    """Keeps the ctypes views of one molecule alive."""

    def __init__(self, config, basis_set, basis_path=None):
        self.symbols = [s for s, _ in config]
        self._sym = (ctypes.c_char_p * len(config))(*[s.encode() for s in self.symbols])
        self.xyz = np.ascontiguousarray(np.array([list(r) for _, r in config], dtype=np.float64).reshape(-1))
        self._bs = basis_set.encode()
        self._bp = (basis_path or BASIS_PATH).encode()
        self.c = Molecule(len(config), ctypes.cast(self._sym, ctypes.c_void_p), self.xyz.ctypes.data, self._bs,
                          self._bp)

    def ref(self):
        return ctypes.byref(self.c)
