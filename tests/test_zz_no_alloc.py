"""The allocation-free RHF build (hfx_fock_rhf_device_noalloc) against the
regular device build (hfx_fock_rhf_device), through the C ABI.

The no-allocation entry point exists for callers that cannot let the library
call cudaMalloc at build time (an application whose allocator owns the
device memory, or a loop that must not be stalled by cudaMalloc's device
synchronisation).  It keeps its scratch in one static device array that every
call reuses, so this test makes two calls in a row: the second must not see
stale accumulators from the first.  Tolerance: 1e-10 per matrix element, the
Fock-matrix tolerance of the other GPU parity tests.

This file sorts last so that a run stopping at the first failure has already
run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MAT_TOL = 1e-10


def test_noalloc_build_matches_regular_build_twice():
    torch = pytest.importorskip("torch")
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import _lib, workloads as W

    with H.FockBuilder(config=W.benzene(), basis_set="cc-pVDZ") as fb:
        K = fb.K
        rng = np.random.default_rng(11)
        mats = []
        for _ in range(2):
            P = rng.normal(size=(K, K)) * 0.1
            mats.append(P + P.T)
        for P in mats:
            dP = torch.tensor(P, device="cuda", dtype=torch.float64)
            g_ref = torch.zeros_like(dP)
            g_new = torch.full_like(dP, float("nan"))
            torch.cuda.synchronize()
            _lib.check(_lib.lib.hfx_fock_rhf_device(fb._job, ctypes.c_void_p(dP.data_ptr()),
                                                    ctypes.c_void_p(g_ref.data_ptr())))
            _lib.check(_lib.lib.hfx_fock_rhf_device_noalloc(fb._job, ctypes.c_void_p(dP.data_ptr()),
                                                            ctypes.c_void_p(g_new.data_ptr())))
            torch.cuda.synchronize()
            a, b = g_ref.cpu().numpy(), g_new.cpu().numpy()
            assert np.isfinite(b).all()
            assert np.abs(a - b).max() < MAT_TOL
