"""Python face of the request server (include/hfx.h, hfx_server_*): RHF/UHF
jobs submitted as they arrive, admitted by worker slot and device-memory
footprint, run concurrently on one GPU (continuous batching)."""
import ctypes

import numpy as np

from . import _lib
from ._lib import HFX_PREC_FP64, check, lib

JOB_STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}
FAULTS = {"none": 0, "setup": 1, "oom": 2, "alloc": 3, "iteration": 4}


class Server:
    def __init__(self, max_active=8, hbm_budget_gb=0.0, device=0, precision=HFX_PREC_FP64, fp32_threshold=0.0,
                 pack_max=0):
        """pack_max > 1: packed mode.  Each running request joins a Fock session
        shared with up to pack_max - 1 other requests of the same method,
        options and size class; every SCF cycle is one build over all of them
        (one launch per quartet class), and requests that arrive while a
        session iterates join it at their next cycle."""
        o = _lib.ServerOptions()
        o.max_active = max_active
        o.pack_max = pack_max
        o.hbm_budget_gb = hbm_budget_gb
        o.device = device
        o.precision = precision
        o.fp32_threshold = fp32_threshold
        self._s = ctypes.c_void_p()
        check(lib.hfx_server_create(ctypes.byref(o), ctypes.byref(self._s)))
        self._keep = {}

    def submit(self, config, basis_set, method="RHF", spin=None, charge=0, epsilon=1e-6, energy_threshold=0.0,
               max_it=10000, precision=-1, fp32_threshold=0.0, timeout_s=0.0, inject_fault="none",
               basis_path=None, screening_threshold=1e-8):
        m = _lib.MoleculeArgs(config, basis_set, basis_path)
        r = _lib.Request()
        r.mol = m.c
        r.method = 1 if method == "UHF" else 0
        if method == "UHF":
            r.n_alpha, r.n_beta = int(spin[0]), int(spin[1])
        r.scf.max_iterations = max_it
        r.scf.epsilon = epsilon
        r.scf.energy_threshold = energy_threshold
        r.scf.charge = charge
        r.scf.screening_threshold = screening_threshold
        r.precision = precision
        r.fp32_threshold = fp32_threshold
        r.timeout_s = timeout_s
        r.inject_fault = FAULTS[inject_fault] if isinstance(inject_fault, str) else int(inject_fault)
        jid = ctypes.c_longlong()
        check(lib.hfx_server_submit(self._s, ctypes.byref(r), ctypes.byref(jid)))
        return jid.value

    @staticmethod
    def _info(i):
        return dict(state=JOB_STATES[i.state], status=i.status, E_tot=i.E_tot, iterations=i.iterations,
                    converged=bool(i.converged), K=i.K, t_submit=i.t_submit, t_admit=i.t_admit, t_end=i.t_end,
                    fock_ms=i.fock_ms, fock_builds=i.fock_builds, message=i.message.decode(errors="replace"))

    def poll(self, jid):
        i = _lib.JobInfo()
        check(lib.hfx_server_poll(self._s, jid, ctypes.byref(i)))
        return self._info(i)

    def wait(self, jid, timeout_s=0.0):
        i = _lib.JobInfo()
        check(lib.hfx_server_wait(self._s, jid, timeout_s, ctypes.byref(i)))
        return self._info(i)

    def cancel(self, jid):
        check(lib.hfx_server_cancel(self._s, jid))

    def drain(self, timeout_s=0.0):
        check(lib.hfx_server_drain(self._s, timeout_s))

    def density(self, jid, K, uhf=False):
        Pa = np.zeros((K, K))
        Pb = np.zeros((K, K)) if uhf else None
        check(lib.hfx_server_density(self._s, jid, _lib.ptr(Pa), _lib.ptr(Pb)))
        return (Pa, Pb) if uhf else Pa

    def stats(self):
        st = _lib.ServerStats()
        check(lib.hfx_server_stats(self._s, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_ if k != "reserved"}

    def close(self):
        if self._s:
            check(lib.hfx_server_destroy(self._s))
            self._s = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
