"""The request server: concurrent jobs give the same results as the same jobs
run alone (energies within 1 uHa, iteration counts within +-1), and host-side
faults fail only their own job with a status code."""
import pytest

import hartree_fock_cpp_gb300 as H
from hartree_fock_cpp_gb300 import workloads as W
from hartree_fock_cpp_gb300.server import Server

pytestmark = pytest.mark.gpu
E_TOL = 1e-6

OH = [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.83))]
MIX = [
    dict(config=W.water(), basis_set="STO-3G", method="RHF"),
    dict(config=W.water(), basis_set="cc-pVDZ", method="RHF"),
    dict(config=W.benzene(), basis_set="cc-pVDZ", method="RHF"),
    dict(config=OH, basis_set="6-31G*", method="UHF", spin=(5, 4)),
    dict(config=W.n_decane(), basis_set="6-31G*", method="RHF"),
    dict(config=W.nacl_scan(8)[3], basis_set="cc-pVTZ", method="RHF"),
]


def _alone(job):
    if job["method"] == "UHF":
        return H.uhf_diis(job["config"], job["basis_set"], spin_occ=job["spin"])
    return H.rhf_diis(job["config"], job["basis_set"])


def test_results_same_alone_and_in_the_mix():
    alone = [_alone(j) for j in MIX]
    with Server(max_active=6) as srv:
        ids = [srv.submit(**j) for j in MIX]
        srv.drain(600)
        infos = [srv.poll(i) for i in ids]
        st = srv.stats()
    assert st["max_concurrent"] >= 2
    for j, a, inf in zip(MIX, alone, infos):
        assert inf["state"] == "done", inf
        assert inf["converged"]
        assert abs(inf["E_tot"] - a["E_tot"]) < E_TOL, (j["basis_set"], inf["E_tot"], a["E_tot"])
        assert abs(inf["iterations"] - a["iterations"]) <= 1


def test_faults_fail_only_their_own_job():
    with Server(max_active=4) as srv:
        good = srv.submit(W.water(), "STO-3G")
        bad_basis = srv.submit(W.water(), "no-such-basis")
        bad_elem = srv.submit([("Xx", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.4))], "STO-3G")
        oom = srv.submit(W.water(), "STO-3G", inject_fault="oom")
        alloc = srv.submit(W.water(), "STO-3G", inject_fault="alloc")
        it = srv.submit(W.water(), "STO-3G", inject_fault="iteration")
        slow = srv.submit(W.benzene(), "cc-pVDZ", timeout_s=1e-3)
        srv.drain(300)
        g = srv.poll(good)
        assert g["state"] == "done" and g["converged"]
        assert srv.poll(bad_basis)["status"] == 2          # HFX_ERR_BASIS
        assert srv.poll(bad_elem)["status"] == 2
        assert srv.poll(oom)["status"] == 4                # HFX_ERR_OOM
        assert srv.poll(alloc)["status"] == 4
        assert srv.poll(it)["status"] == 9                 # HFX_ERR_NUMERIC (injected)
        assert srv.poll(slow)["status"] == 8               # HFX_ERR_TIMEOUT
        # the server keeps serving after the failures
        after = srv.submit(W.water(), "STO-3G")
        assert srv.wait(after, 120)["converged"]
        st = srv.stats()
        assert st["failed"] == 6 and st["running"] == 0


def test_cancel_queued_job():
    with Server(max_active=1) as srv:
        first = srv.submit(W.benzene(), "cc-pVDZ")
        second = srv.submit(W.water(), "STO-3G")
        srv.cancel(second)
        srv.drain(300)
        assert srv.poll(first)["converged"]
        assert srv.poll(second)["status"] == 7             # HFX_ERR_CANCELLED


def test_packed_mode_results_same_alone_and_in_the_pack():
    """pack_max > 1: running requests of one method share Fock sessions (one
    build per SCF cycle over all members of a size class, one launch per
    class); each result equals the job run alone, and a faulty request in a
    session fails alone."""
    rhf = [j for j in MIX if j["method"] == "RHF"]
    alone = [_alone(j) for j in rhf]
    with Server(max_active=8, pack_max=8) as srv:
        ids = [srv.submit(**j) for j in rhf]
        bad = srv.submit(config=W.water(), basis_set="6-31G*", inject_fault="iteration")
        uhf = srv.submit(config=OH, basis_set="6-31G*", method="UHF", spin=(5, 4))
        srv.drain(600)
        infos = [srv.poll(i) for i in ids]
        ib, iu = srv.poll(bad), srv.poll(uhf)
        st = srv.stats()
    for j, a, inf in zip(rhf, alone, infos):
        assert inf["state"] == "done", inf
        assert inf["converged"]
        assert abs(inf["E_tot"] - a["E_tot"]) < E_TOL
        assert abs(inf["iterations"] - a["iterations"]) <= 1
    assert ib["state"] == "failed"
    assert iu["state"] == "done" and iu["converged"]
    assert st["max_session_members"] >= 2


def test_request_arriving_mid_scf_joins_the_running_session():
    """A request submitted while another of its size class iterates joins
    that session at its next cycle (continuous batching inside one build);
    both results equal the jobs run alone.  Mixed precision, where a cycle can
    hold mixed and FP64 (incremental) builds as separate variants."""
    import time
    jobs = [dict(config=W.n_decane(), basis_set="6-31G*"), dict(config=W.benzene(), basis_set="cc-pVDZ")]
    kw = dict(precision=H.HFX_PREC_MIXED, fp32_threshold=0.03)
    alone = [H.rhf_diis(j["config"], j["basis_set"], **kw) for j in jobs]
    with Server(max_active=4, pack_max=4, precision=H.HFX_PREC_MIXED, fp32_threshold=0.03) as srv:
        first = srv.submit(**jobs[0])
        # the second request arrives once the first is admitted (setting up or
        # iterating: a whole n-decane SCF now takes well under a second)
        t0 = time.time()
        while srv.poll(first)["state"] == "queued" and time.time() - t0 < 60:
            time.sleep(0.005)
        second = srv.submit(**jobs[1])
        srv.drain(600)
        infos = [srv.poll(first), srv.poll(second)]
        st = srv.stats()
    for a, inf in zip(alone, infos):
        assert inf["state"] == "done" and inf["converged"], inf
        assert abs(inf["E_tot"] - a["E_tot"]) < E_TOL
        assert abs(inf["iterations"] - a["iterations"]) <= 1
    assert infos[1]["t_admit"] < infos[0]["t_end"]       # admitted while the first was iterating
    assert st["max_session_members"] == 2 and st["sessions_created"] == 1


def test_packed_members_keep_their_own_screening_threshold():
    """Requests with different Schwarz thresholds never share a Fock session:
    each result equals the same request run alone."""
    thr = (1e-8, 1e-3)
    alone = [H.rhf_diis(W.water(), "cc-pVDZ", screening_threshold=t) for t in thr]
    assert abs(alone[0]["E_tot"] - alone[1]["E_tot"]) > 10 * E_TOL   # the thresholds matter
    with Server(max_active=2, pack_max=4) as srv:
        ids = [srv.submit(W.water(), "cc-pVDZ", screening_threshold=t) for t in thr]
        srv.drain(300)
        infos = [srv.poll(i) for i in ids]
        st = srv.stats()
    for a, inf in zip(alone, infos):
        assert inf["state"] == "done" and inf["converged"], inf
        assert abs(inf["E_tot"] - a["E_tot"]) < E_TOL
    assert st["sessions_created"] == 2


def test_packed_admission_within_a_small_memory_budget():
    """The budget fits one request but not two: the second waits for memory
    outside any session (a session never waits on a request that has not
    joined it), and both finish."""
    with Server(max_active=2, pack_max=4, hbm_budget_gb=0.1) as srv:
        ids = [srv.submit(W.water(), "STO-3G") for _ in range(3)]
        srv.drain(120)
        infos = [srv.poll(i) for i in ids]
        st = srv.stats()
    for inf in infos:
        assert inf["state"] == "done" and inf["converged"], inf
    assert st["in_use_bytes"] == 0


@pytest.mark.parametrize("pack_max", [0, 8])
def test_mixed_precision_requests_same_alone_and_served(pack_max):
    """Mixed-precision requests (RHF and UHF) follow the mixed-precision SCF
    protocol in the server as they do alone (FP32 builds, then FP64 final
    cycles): the same energies and iteration counts, per-job and packed."""
    jobs = [dict(config=W.water(), basis_set="cc-pVDZ", method="RHF"),
            dict(config=OH, basis_set="6-31G*", method="UHF", spin=(5, 4)),
            dict(config=W.benzene(), basis_set="cc-pVDZ", method="RHF")]
    kw = dict(precision=H.HFX_PREC_MIXED, fp32_threshold=0.03)
    alone = [H.uhf_diis(j["config"], j["basis_set"], spin_occ=j["spin"], **kw) if j["method"] == "UHF"
             else H.rhf_diis(j["config"], j["basis_set"], **kw) for j in jobs]
    assert sum(a["mixed_builds"] for a in alone) > 0
    with Server(max_active=4, pack_max=pack_max, precision=H.HFX_PREC_MIXED, fp32_threshold=0.03) as srv:
        ids = [srv.submit(**j) for j in jobs]
        srv.drain(600)
        infos = [srv.poll(i) for i in ids]
    for a, inf in zip(alone, infos):
        assert inf["state"] == "done" and inf["converged"], inf
        assert abs(inf["E_tot"] - a["E_tot"]) < E_TOL
        assert abs(inf["iterations"] - a["iterations"]) <= 1
