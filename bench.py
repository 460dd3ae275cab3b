"""Benchmark of the direct-SCF Fock-build engine (one JSON line on rank 0).

Workload (N=1): benzene RHF/cc-pVDZ (K=120, 21 doubly occupied), the FP64 GPU
drop-in for the reference's ERI/Fock call, reference SCF settings with the
stated convergence (DIIS 8, |dE| < 1e-8 Eh and RMS dD < 1e-7).  One step = one
SCF solve from a zero density.

  value  RHF solves/s with the job resident in HBM (basis, pair data, Schwarz
         table and quartet lists uploaded before the timed region; each SCF
         iteration moves only the K x K density / G through the C ABI)
  e2e    RHF solves/s through hfx_rhf_diis (molecule in host memory: basis
         construction, job setup, uploads, every SCF iteration, downloads)
  extra  FP64 Fock builds/s of the device-pointer build, p50/p99 solve
         latency, the roofline of the shell-quartet kernel against the
         measured FP64 FMA-loop peak, and the reference-algorithm CPU baseline
         timed on this host's cores on a bounded sample.

--impl reference times the reference's CPU algorithm for the same workload
(oracle port of integrals.hpp repulsion_tensor + linalg.hpp repulsion_matrix,
all host threads, bounded sample per step, extrapolated to solves/s).
Multi-GPU: replicas only (one independent solve stream per rank), launched
with torchrun; value = solves of all ranks / max time.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "RHF solves/s"
UNIT = "solves/s"
WORKLOAD = "benzene RHF/cc-pVDZ, FP64 direct J/K (K=120, 21 occ), DIIS(8), |dE|<1e-8 & RMS dD<1e-7"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws):
    """The largest per-rank value over all ranks (the slowest rank's time);
    NCCL reduces on the GPU, gloo on the CPU."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, t_max, ws):
    """Units all ranks processed (each rank the same count) over the slowest rank's time."""
    return ws * units_per_rank / t_max


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except Exception:
                continue
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(torch, buf):
    buf.zero_()


def cpu_baseline(config, basis, iterations, sample_quartets, nthreads, seed=20261203):
    """Reference algorithm (oracle port of integrals.hpp:754-787 + linalg.hpp:100-129)
    on a bounded sample: time per unique BF quartet over the host threads and one
    O(K^4) repulsion_matrix contraction; extrapolated to one SCF solve."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    orc = O.Oracle(config, basis)
    K = orc.K
    npair = K * (K + 1) // 2
    nq = npair * (npair + 1) // 2
    t0 = time.perf_counter()
    Q = orc.schwarz_bounds()
    t_schwarz = time.perf_counter() - t0
    rng = np.random.default_rng(seed)
    qid = rng.integers(0, nq, size=sample_quartets)
    # quartet id -> (i,j,k,l) as indexing.hpp:55-85
    p1 = ((np.sqrt(8.0 * qid + 1.0) - 1.0) / 2.0).astype(np.int64)
    p1 -= (p1 * (p1 + 1) // 2 > qid)
    p1 += ((p1 + 1) * (p1 + 2) // 2 <= qid)
    p2 = qid - p1 * (p1 + 1) // 2
    def unpair(p):
        a = ((np.sqrt(8.0 * p + 1.0) - 1.0) / 2.0).astype(np.int64)
        a -= (a * (a + 1) // 2 > p)
        a += ((a + 1) * (a + 2) // 2 <= p)
        return a, p - a * (a + 1) // 2
    i, j = unpair(p1)
    k, l = unpair(p2)
    ijkl = np.stack([i, j, k, l], 1).astype(np.int32)
    surv = Q[p1] * Q[p2] >= 1e-8
    t0 = time.perf_counter()
    orc.eri_list(ijkl, bounds=Q, threshold=1e-8, nthreads=nthreads)
    t_sample = time.perf_counter() - t0
    frac = float(surv.mean())
    t_tensor = t_schwarz + t_sample / sample_quartets * nq
    P = np.eye(K)
    eri_dummy = np.zeros(nq)
    t0 = time.perf_counter()
    O.repulsion_matrix(P, eri_dummy)
    t_contract = time.perf_counter() - t0
    t_solve = t_tensor + iterations * t_contract
    return dict(value=1.0 / t_solve, unit=UNIT, cores=nthreads, kind="port", K=K,
                sample="%d random unique BF quartets of %d (%.1f%% survive 1e-8 screening) on %d threads, "
                       "plus one O(K^4) repulsion_matrix; extrapolated: tensor %.1f s + %d x %.2f s contraction"
                       % (sample_quartets, nq, 100 * frac, nthreads, t_tensor, iterations, t_contract),
                seconds_per_solve=t_solve, sample_seconds=t_sample + t_contract + t_schwarz)


def load_workloads():
    """The synthetic workload generators, loaded from their file (numpy only):
    importing the package would load the engine's library into the process."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("hfx_workloads",
                                                  os.path.join(REPO, "hartree_fock_cpp_gb300", "workloads.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def reference_iterations():
    """SCF iterations of the headline workload in the reference's own loop:
    the oracle's rhf_diis (scf.hpp:205-419) over the tensor of the reference's
    integrals.hpp compiled unchanged (tests/golden/scf_golden.json)."""
    with open(os.path.join(REPO, "tests", "golden", "scf_golden.json")) as f:
        return int(json.load(f)["benzene_ccpvdz"]["iterations"])


def workload_config(K, ws):
    """The config dict of the headline workload, the same in both arms."""
    return {"workload": WORKLOAD, "molecule": "benzene D6h (C r=2.6379, H r=4.68 bohr)", "basis": "cc-pVDZ",
            "K": K, "parallelism": "replicas" if ws > 1 else "single",
            "l2": "GPU arm: flushed between steps (512 MB write)"}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    W = load_workloads()
    nthreads = os.cpu_count() or 1
    cfg = W.benzene()
    iters = reference_iterations()
    vals = []
    base = None
    for s in range(args.warmup + args.steps):
        b = cpu_baseline(cfg, "cc-pVDZ", iters, sample_quartets=2000 * nthreads, nthreads=nthreads,
                         seed=20261203 + s)
        if s >= args.warmup:
            vals.append(b["seconds_per_solve"])
            base = b
    t = float(np.mean(vals))
    v = 1.0 / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(base["K"], ws),
            "reference_impl": "reference CPU algorithm (oracle port of integrals.hpp repulsion_tensor + "
                              "linalg.hpp repulsion_matrix), host threads, %d SCF iterations of the reference "
                              "loop" % iters,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": base["kind"],
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_engine(args):
    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import _lib, workloads as W

    fp64_peak, fp32_peak = H.measure_peaks(local)
    try:
        dmma_peak = H.measure_dmma_peak(local)
    except Exception:  # noqa: BLE001 - reported as unmeasured
        dmma_peak = None
    cfg = W.benzene()
    basis = "cc-pVDZ"
    scf_kw = dict(epsilon=1e-7, energy_threshold=1e-8)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # ---- value: device-resident job, solves/s -------------------------------
    fb = H.FockBuilder(config=cfg, basis_set=basis, device=local)
    K = fb.K
    mol = fb._mol
    o = _lib.ScfOptions()
    o.epsilon = scf_kw["epsilon"]
    o.energy_threshold = scf_kw["energy_threshold"]
    res = _lib.ScfResult()
    dens = np.zeros((K, K))

    def solve_resident():
        st = _lib.lib.hfx_job_rhf(fb._job, ctypes.byref(o), None, ctypes.byref(res), _lib.ptr(dens), None, None)
        _lib.check(st)
        return res.iterations, res.fock_builds, res.E_tot

    for _ in range(args.warmup):
        solve_resident()
    # launch shape (chunk sizes, warps per CTA) from the autotuner, at the
    # converged density of the warm-up solves; untimed setup
    shape, _ = fb.autotune_launch_shape(dens, builds=2)
    solve_resident()
    lat = []
    iters = builds = 0
    E_val = None
    clocks = Clocks(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(args.steps):
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        it, nb, E_val = solve_resident()
        e1.record()
        torch.cuda.synchronize()
        lat.append(e0.elapsed_time(e1))
        iters, builds = it, nb
    clk = clocks.stop()
    torch.cuda.synchronize()
    t_total = max_over_ranks(sum(lat) / 1e3, ws)
    value = whole_job_rate(args.steps, t_total, ws)

    # ---- Fock builds/s (device-pointer build) and the kernel roofline --------
    rng = np.random.default_rng(0)
    P = torch.tensor(dens if np.abs(dens).sum() > 0 else rng.normal(size=(K, K)), device="cuda",
                     dtype=torch.float64)
    G = torch.zeros_like(P)
    for _ in range(2):
        fb.repulsion_matrix_device(P.data_ptr(), G.data_ptr())
    kms, bms = [], []
    for _ in range(max(3, args.steps)):
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        fb.repulsion_matrix_device(P.data_ptr(), G.data_ptr())
        s = fb.stats()
        kms.append(s["kernel_ms"])
        bms.append(s["ms"])
    s = fb.stats()
    kernel_ms = float(np.mean(kms))
    build_ms = float(np.mean(bms))
    flops = s["flops_fp64"]
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    peak = fp64_peak / 1e3

    # ---- mixed vs FP64 Fock builds on n-decane/6-31G* ------------------------
    mixed = None if args.no_mixed else section(mixed_section, H, W, torch, flush, args, local, scf_kw,
                                                          (fp64_peak, fp32_peak))

    # ---- served request stream: continuous batching vs one-at-a-time FP64 ----
    served = section(serve_section, H, W, args.serve_jobs, local, rate_list(args.serve_rates)) \
        if args.serve_jobs > 0 else None

    # ---- batched radial scans: packed lockstep SCF vs one-at-a-time FP64 -----
    scans = section(scan_section, H, W, args.scan_points) if args.scan_points > 0 else None

    # ---- e2e: through hfx_rhf_diis with host buffers -------------------------
    e2e_lat = []
    r = None
    for k in range(1 + args.steps):
        t0 = time.perf_counter()
        r = H.rhf_diis(cfg, basis, **scf_kw)
        dt = time.perf_counter() - t0
        if k > 0:
            e2e_lat.append(dt)
    e2e_t = max_over_ranks(float(np.mean(e2e_lat)), ws)
    m = H._lib.MoleculeArgs(cfg, basis)
    npp = ctypes.c_int()
    npr = ctypes.c_int()
    nep = ctypes.c_longlong()
    _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), ctypes.byref(npp), ctypes.byref(npr), ctypes.byref(nep), None,
                                            None, None))
    setup_bytes = nep.value * 8 + npr.value * 32 + npp.value * 48 + s["quartets"] * 8
    h2d = int(setup_bytes + r["fock_builds"] * K * K * 8)
    d2h = int(r["fock_builds"] * K * K * 8 + K * (K + 1) // 2 * 8 + npp.value * 8)

    if rank != 0:
        if ws > 1:
            torch.distributed.barrier()
        return
    cpu = None
    ref_iters = None
    try:
        ref_iters = reference_iterations()
    except Exception:  # noqa: BLE001 - fixture absent: the engine's own count
        pass
    if ws == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        b = cpu_baseline(cfg, basis, ref_iters or iters, sample_quartets=2000 * nthreads, nthreads=nthreads)
        cpu = {k: b[k] for k in ("value", "unit", "cores", "kind", "sample")}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(K, ws),
        "launch_shape": shape,
        "served_stream": served,
        "batched_scans": scans,
        "mixed_precision": mixed,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "scf": {"iterations": iters, "fock_builds": builds, "E_tot": E_val, "reference_iterations": ref_iters,
                "density_step": {"sp2_projections": res.projections, "syevd_fallbacks": res.projection_fallbacks}},
        "fock_builds_per_s": {"fp64": 1e3 / build_ms},
        "eri_rate": {"shell_quartets_per_s": s["quartets"] / (kernel_ms * 1e-3),
                     "primitive_quartets_per_s": s["prim_quartets"] / (kernel_ms * 1e-3),
                     "shell_quartets_per_build": s["quartets"], "note": "surviving (Schwarz-screened) quartets of one FP64 build"},
        "roofline": {"bound": "fp64_pipe", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "peak_source": "measured FP64 FMA-loop peak of this GPU (hfx_measure_peaks, same run)",
                     "flops_per_launch": flops, "kernel_ms": kernel_ms, "fp32_peak_tflops": fp32_peak / 1e3,
                     "dmma_peak_tflops": dmma_peak / 1e3 if dmma_peak else None},
        "e2e": {"value": whole_job_rate(1, e2e_t, ws), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "solves": len(e2e_lat)},
        "gpu_launches": int(args.steps * builds * s["launches"]),
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    line["summary"] = summary(line)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.barrier()


def summary(line):
    """Compact digest of the secondary sections, printed as the line's last key."""
    out = {"roofline_frac_fp64": round(line["roofline"]["frac"], 4)}
    mx = line.get("mixed_precision") or {}
    if "speedup" in mx:
        out["mixed"] = {k: (float("%.4g" % mx[k]) if isinstance(mx[k], float) else mx[k]) for k in
                        ("speedup", "fp32_threshold", "fp32_quartet_fraction", "max_dF_vs_fp64", "scf_dE_vs_fp64",
                         "fock_builds_per_s_fp64", "fock_builds_per_s_mixed")}
        out["mixed"]["roofline_frac"] = round(mx["roofline"]["frac"], 4)
    elif mx:
        out["mixed"] = mx
    sv = line.get("served_stream") or {}
    if "rates" in sv:
        rows = []
        for e in sv["rates"]:
            row = {"x": e["arrival_rate_x"]}
            for key in ("one_at_a_time_fp64", "served_mixed", "served_mixed_packed"):
                if key in e:
                    row[key] = [round(e[key]["solves_per_s"], 3), round(e[key]["p99_s"], 2)]
            rows.append(row)
        out["served_solves_per_s_p99_s"] = rows
    elif sv:
        out["served"] = sv
    sc = line.get("batched_scans") or {}
    if "speedup" in sc:
        out["scans"] = {"batched_solves_per_s": round(sc["batched"]["solves_per_s"], 3),
                        "one_at_a_time_warm_solves_per_s": round(sc["one_at_a_time_fp64_warm"]["solves_per_s"], 3),
                        "speedup": round(sc["speedup"], 3),
                        "max_iteration_diff_warm_points": sc["max_iteration_diff_warm_points"]}
    elif sc:
        out["scans"] = sc
    return out


def section(fn, *a):
    """A secondary section of the bench line: its dict, or its error (the
    headline metric is still printed)."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 - any failure is reported in the line
        return {"error": "%s: %s" % (type(e).__name__, e)}


def mixed_section(H, W, torch, flush, args, local, scf_kw, peaks):
    """n-decane/6-31G*: FP64 vs mixed Fock builds at the autotuned FP32 cut,
    max|dF| against the FP64 build, and the mixed SCF's |dE| against FP64."""
    cfg_d = W.n_decane()
    r64 = H.rhf_diis(cfg_d, "6-31G*", **scf_kw)
    Pd = r64["density"]
    Kd = Pd.shape[0]
    fbm = H.FockBuilder(config=cfg_d, basis_set="6-31G*", device=local)
    # FP32 cut: the largest tau whose build changes the energy at the converged
    # density by at most half of the 1 uHa target
    tau, dE_proxy, _, _ = fbm.autotune_fp32_threshold(Pd, 5e-7)
    shape_mx, _ = fbm.autotune_launch_shape(Pd, builds=2)
    fb64 = H.FockBuilder(config=cfg_d, basis_set="6-31G*", device=local)
    shape_64, _ = fb64.autotune_launch_shape(Pd, builds=2)
    dPd = torch.tensor(Pd, device="cuda", dtype=torch.float64)
    dG64 = torch.zeros_like(dPd)
    dGmx = torch.zeros_like(dPd)
    tms, kms = {}, {}
    for name, f, out in (("fp64", fb64, dG64), ("mixed", fbm, dGmx)):
        f.repulsion_matrix_device(dPd.data_ptr(), out.data_ptr())
        ts, ks = [], []
        for _ in range(max(3, args.steps)):
            flush_l2(torch, flush)
            torch.cuda.synchronize()
            f.repulsion_matrix_device(dPd.data_ptr(), out.data_ptr())
            ts.append(f.stats()["ms"])
            ks.append(f.stats()["kernel_ms"])
        tms[name] = float(np.mean(ts))
        kms[name] = float(np.mean(ks))
    smx = fbm.stats()
    kms_mx = kms["mixed"]
    max_dF = float((dGmx - dG64).abs().max().item())
    rmx = H.rhf_diis(cfg_d, "6-31G*", precision=H.HFX_PREC_MIXED, fp32_threshold=tau, **scf_kw)
    mixed = {"workload": "n-decane C10H22 RHF/6-31G* (K=%d), seed 20261203 noise 0.05 bohr" % Kd,
             "fp32_threshold": tau, "autotune_target_dE": 5e-7, "autotune_dE": dE_proxy,
             "launch_shape_fp64": shape_64, "launch_shape_mixed": shape_mx,
             "fock_builds_per_s_fp64": 1e3 / tms["fp64"], "fock_builds_per_s_mixed": 1e3 / tms["mixed"],
             "speedup": tms["fp64"] / tms["mixed"], "fp32_quartet_fraction": smx["quartets_fp32"] / smx["quartets"],
             "max_dF_vs_fp64": max_dF, "scf_dE_vs_fp64": rmx["E_tot"] - r64["E_tot"],
             "scf_iterations_fp64": r64["iterations"], "scf_iterations_mixed": rmx["iterations"],
             "scf_fock_ms_fp64": r64["fock_ms"], "scf_fock_ms_mixed": rmx["fock_ms"],
             "scf_builds_mixed_fp64_delta": [rmx["mixed_builds"], rmx["fp64_builds"], rmx["delta_builds"]],
             # pipe-time fraction of the mixed build's quartet kernels:
             # (F64 / peak64 + F32 / peak32) / elapsed
             "roofline": {"bound": "fp64+fp32 pipes", "flops_fp64": smx["flops_fp64"], "flops_fp32": smx["flops_fp32"],
                          "kernel_ms": kms_mx, "peak_fp64_tflops": peaks[0] / 1e3, "peak_fp32_tflops": peaks[1] / 1e3,
                          "frac": (smx["flops_fp64"] / (peaks[0] * 1e9) + smx["flops_fp32"] / (peaks[1] * 1e9))
                          / (kms_mx * 1e-3)}}
    fbm.close()
    fb64.close()
    return mixed


def serve_section(H, W, n_jobs, device, rate_factors=(1.0, 2.0, 4.0), tau=0.03, max_it=60, seed=20261203):
    """First n_jobs requests of the seeded served stream (random C/N/O/S trees,
    80% RHF / 20% UHF doublets, STO-3G / 6-31G* / cc-pVDZ).  Baseline: the
    plain FP64 GPU path one job at a time.  Served: Poisson arrivals at each
    rate factor x the baseline throughput into the request server (mixed
    precision, continuous batching); solves/s over the span from the first
    arrival to the last result, and p50/p99 time from arrival to converged
    energy.  SCFs are capped at max_it iterations (non-converged jobs count as
    finished, not solved).  The baseline's latency under the same arrivals is
    computed from its measured per-job times (a single queue)."""
    from hartree_fock_cpp_gb300.server import Server
    jobs = W.served_stream(n_jobs, seed=seed)
    Ks = [H.basis_construction(j["config"], j["basis"]).K for j in jobs]
    seq_lat, seq_E, seq_ok = [], [], 0
    t0 = time.perf_counter()
    for j in jobs:
        t = time.perf_counter()
        kw = dict(max_it=max_it)
        r = (H.uhf_diis(j["config"], j["basis"], spin_occ=j["spin"], **kw) if j["method"] == "UHF"
             else H.rhf_diis(j["config"], j["basis"], **kw))
        seq_lat.append(time.perf_counter() - t)
        seq_E.append(r["E_tot"] if r["converged"] else None)
        seq_ok += int(r["converged"])
    T_seq = time.perf_counter() - t0
    mu = n_jobs / T_seq
    out = {"sample": "first %d requests of the seeded stream (seed %d), K %d..%d, max %d SCF iterations"
                     % (n_jobs, seed, min(Ks), max(Ks), max_it),
           "one_at_a_time_fp64": {"solves_per_s": seq_ok / T_seq, "jobs_per_s": mu, "converged": seq_ok},
           "rates": []}
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0, size=n_jobs)
    for rf in rate_factors:
        lam = rf * mu
        arrivals = np.cumsum(gaps / lam)
        arrivals -= arrivals[0]
        free_at, seq_resp = 0.0, []
        for a, d in zip(arrivals, seq_lat):
            start = max(a, free_at)
            free_at = start + d
            seq_resp.append(free_at - a)
        def serve(pack_max):
            with Server(max_active=16, device=device, precision=H.HFX_PREC_MIXED, fp32_threshold=tau,
                        pack_max=pack_max) as srv:
                ids = []
                t0 = time.perf_counter()
                for a, j in zip(arrivals, jobs):
                    dt = a - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                    ids.append(srv.submit(j["config"], j["basis"], method=j["method"], spin=j.get("spin"),
                                          max_it=max_it))
                srv.drain(3600)
                T_srv = time.perf_counter() - t0
                infos = [srv.poll(i) for i in ids]
                st = srv.stats()
            lat = [i["t_end"] - i["t_submit"] for i in infos]
            extra = {"max_session_members": st["max_session_members"]} if pack_max > 1 else {}
            ok = sum(1 for i in infos if i["converged"])
            dE = [abs(i["E_tot"] - e) for i, e in zip(infos, seq_E) if e is not None and i["converged"]]
            return {"solves_per_s": ok / T_srv, "jobs_per_s": n_jobs / T_srv,
                    "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                    "converged": ok, "max_concurrent": st["max_concurrent"], "fp32_threshold": tau,
                    "max_abs_dE_vs_fp64": float(max(dE)) if dE else None, **extra}
        entry = {
            "arrival_rate_x": rf, "arrival_span_s": float(arrivals[-1]),
            "one_at_a_time_fp64": {"solves_per_s": seq_ok / free_at,
                                   "p50_s": float(np.percentile(seq_resp, 50)),
                                   "p99_s": float(np.percentile(seq_resp, 99))},
            "served_mixed": serve(0)}
        if rf >= 2.0:
            # packed mode: running requests share Fock sessions (up to 8 members per
            # method, options and size class; one launch per class per cycle)
            entry["served_mixed_packed"] = serve(8)
        out["rates"].append(entry)
    return out


def scan_section(H, W, n_each, chain=8):
    """NaCl (Na-Cl 3.5..7.0 bohr) and water symmetric-stretch (O-H 1.4..3.0
    bohr, 104.5 deg) scans, cc-pVTZ, FP64, n_each points of each 64-point
    scan.  Batched: the lockstep batched SCF (one packed Fock build per cycle
    over every point still iterating) with warm-started chains of `chain`
    consecutive points, each point starting from the previous point's final
    density.  Baseline: the plain FP64 GPU path one point at a time, each
    point warm-started from the previous one, as the reference's run_bl_scan
    does (run.hpp:353-368).  Warm-started points of the batch start from the
    same density as in the baseline, so their energies and iteration counts
    are compared (chain heads start from the zero density)."""
    step = max(1, 64 // n_each)
    scans = [W.nacl_scan(64)[::step][:n_each], W.water_scan(64)[::step][:n_each]]
    mols = [(c, "cc-pVTZ") for sc in scans for c in sc]
    # batched: chains never cross from one scan into the other
    t0 = time.perf_counter()
    res = []
    cycles = 0
    build_ms = 0.0
    setup_s = 0.0
    res, st = H.batch_scf(mols, max_it=200, warm_chain=chain)
    T_b = time.perf_counter() - t0
    cycles, build_ms, setup_s = st["cycles"], st["build_ms"], st["setup_seconds"]
    ok = sum(1 for r in res if r["converged"])
    # one at a time, warm-started point to point
    seq = []
    t0 = time.perf_counter()
    for sc in scans:
        P = None
        for c in sc:
            r = H.rhf_diis(c, "cc-pVTZ", max_it=200, set_initial_density=P is not None, P0=P)
            P = r["density"]
            seq.append(r)
    T_s = time.perf_counter() - t0
    seq_ok = sum(1 for r in seq if r["converged"])
    warm = [i for i in range(len(mols)) if i % chain != 0]
    dE = [abs(seq[i]["E_tot"] - res[i]["E_tot"]) for i in range(len(mols))]
    dI = [abs(seq[i]["iterations"] - res[i]["iterations"]) for i in warm]
    return {"workload": "%d NaCl + %d water cc-pVTZ scan points (every %d-th of 64 each), RHF FP64, K=78/65"
                        % (len(scans[0]), len(scans[1]), step),
            "batched": {"solves_per_s": ok / T_b, "seconds": T_b, "setup_s": setup_s, "cycles": cycles,
                        "packed_build_ms_mean": build_ms / max(1, cycles), "converged": ok,
                        "molecules": len(mols), "warm_chain": chain,
                        "iterations": sum(r["iterations"] for r in res)},
            "one_at_a_time_fp64_warm": {"solves_per_s": seq_ok / T_s, "seconds": T_s, "converged": seq_ok,
                                        "iterations": sum(r["iterations"] for r in seq)},
            "speedup": (ok / T_b) / (seq_ok / T_s),
            "max_abs_dE_vs_single": float(max(dE)), "max_iteration_diff_warm_points": int(max(dI)) if dI else 0}


def rate_list(text):
    return tuple(float(x) for x in text.split(",") if x.strip())


def run_serve_only(args):
    """The served-stream section alone (a longer prefix of the stream, other
    rates): one JSON object."""
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import workloads as W
    print(json.dumps(serve_section(H, W, args.serve_jobs, 0, rate_list(args.serve_rates))), flush=True)


def run_fock_only(args):
    """Small fixed case for profilers: one job, a few device Fock builds."""
    import torch
    import hartree_fock_cpp_gb300 as H
    from hartree_fock_cpp_gb300 import workloads as W
    cfg = getattr(W, args.molecule)()
    prec = H.HFX_PREC_MIXED if args.precision == "mixed" else H.HFX_PREC_FP64
    fb = H.FockBuilder(config=cfg, basis_set=args.basis, precision=prec, fp32_threshold=args.tau)
    K = fb.K
    rng = np.random.default_rng(0)
    P = rng.normal(size=(K, K)) * 0.1
    P = torch.tensor(P + P.T, device="cuda", dtype=torch.float64)
    G = torch.zeros_like(P)
    for _ in range(args.builds):
        fb.repulsion_matrix_device(P.data_ptr(), G.data_ptr())
    s = fb.stats()
    print(json.dumps({"molecule": args.molecule, "basis": args.basis, "K": K, "builds": args.builds,
                      "last_build_ms": s["ms"], "kernel_ms": s["kernel_ms"], "flops": s["flops_fp64"],
                      "quartets": s["quartets"]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision section")
    ap.add_argument("--serve-jobs", type=int, default=12, help="served-stream sample size (0: skip)")
    ap.add_argument("--serve-rates", default="1,2,4",
                    help="served stream: arrival rates as multiples of the one-at-a-time FP64 throughput")
    ap.add_argument("--serve-only", action="store_true", help="run the served-stream section alone")
    ap.add_argument("--scan-points", type=int, default=64,
                    help="batched-scan section: points of each 64-point scan (64: the full 64+64; 0: skip)")
    ap.add_argument("--fock-only", action="store_true",
                    help="profiling case: job setup + --builds device Fock builds of --molecule/--basis")
    ap.add_argument("--molecule", default="benzene", choices=["water", "benzene", "n_decane"])
    ap.add_argument("--basis", default="cc-pVDZ")
    ap.add_argument("--builds", type=int, default=2)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--tau", type=float, default=0.03, help="fock-only: FP32 Schwarz cut (mixed)")
    args = ap.parse_args()
    if args.fock_only:
        run_fock_only(args)
    elif args.serve_only:
        run_serve_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
