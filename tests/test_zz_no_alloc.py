"""The allocation-free RHF build (hfx_fock_rhf_device_noalloc) against the
regular device build (hfx_fock_rhf_device), through the C ABI.

The no-allocation entry point exists for callers that cannot let the library
call cudaMalloc at build time (an application whose allocator owns the
device memory, or a loop that must not be stalled by cudaMalloc's device
synchronisation).  It keeps its scratch in one static device array that every
call reuses, so each case makes two calls in a row: the second must not see
stale accumulators from the first.  Tolerance: 1e-10 per matrix element, the
Fock-matrix tolerance of the other GPU parity tests.

This file sorts last so that a run stopping at the first failure has already
run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MAT_TOL = 1e-10
HFX_ERR_UNSUPPORTED = 5


def _compare_twice(fb, seed):
    torch = pytest.importorskip("torch")
    from hartree_fock_cpp_gb300 import _lib

    K = fb.K
    rng = np.random.default_rng(seed)
    for _ in range(2):
        P = rng.normal(size=(K, K)) * 0.1
        P = P + P.T
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


def test_noalloc_build_matches_regular_build_twice():
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import workloads as W

    with H.FockBuilder(config=W.benzene(), basis_set="cc-pVDZ") as fb:
        _compare_twice(fb, 11)


def test_noalloc_mixed_precision_job_matches_regular_build_twice():
    """A mixed-precision job: its FP32 quartets read the float density copies
    that the job allocated when it was created."""
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import workloads as W

    with H.FockBuilder(config=W.water(), basis_set="6-31G*", precision=H.HFX_PREC_MIXED,
                       fp32_threshold=1e-2) as fb:
        _compare_twice(fb, 12)
        assert fb.stats()["quartets_fp32"] > 0


def test_noalloc_rejects_jobs_above_its_static_limit():
    """K = 610 (C24H50/cc-pVDZ) is above the 512-function limit of the static
    scratch: HFX_ERR_UNSUPPORTED, and the output buffer is left untouched."""
    torch = pytest.importorskip("torch")
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import _lib, workloads as W

    with H.FockBuilder(config=W.n_decane(n_carbon=24), basis_set="cc-pVDZ") as fb:
        assert fb.K > 512
        dP = torch.zeros((fb.K, fb.K), device="cuda", dtype=torch.float64)
        dG = torch.full_like(dP, 7.0)
        st = _lib.lib.hfx_fock_rhf_device_noalloc(fb._job, ctypes.c_void_p(dP.data_ptr()),
                                                  ctypes.c_void_p(dG.data_ptr()))
        torch.cuda.synchronize()
        assert st == HFX_ERR_UNSUPPORTED
        assert bool((dG == 7.0).all())
