#!/usr/bin/env python
"""Frequency-point solves/s at 1e-10 relative residual on one GB300.

Workload: the coupled vibroacoustic sweep -- a 60 x 40 DSG4 aluminium plate
(0.6 x 0.4 m, t = 2 mm, eta = 0.02, simply supported) on a 60 x 40 x 30 Fluid8
air cavity (depth 0.3 m), 2,400 InterfaceMindlin quads, unit force at a
seeded plate node, f = 1..500 Hz (n = 85,034 DOFs). Synthetic, seeded
(no public dataset exists for this path).

A step solves one batch of `--batch` (default 48) frequencies of the sweep
through the mixed path (FP32 fronts + FP64 refinement to ||f - A u|| / ||f|| <= 1e-10);
the plain FP64 path is timed beside it. `value` is whole-job solves/s with
inputs resident in HBM; `e2e` is the same metric through elp_solve with host
buffers (the right-hand side copied in and every solution copied out each step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "freq-point solves/s at 1e-10 rel residual (mixed FP32-front LU + FP64 refinement)"
UNIT = "solves/s"
TOL = 1e-10


def load_pkg():
    name = "elpaso_core_gb300"
    if name in sys.modules:
        return sys.modules[name]
    path = os.path.join(ROOT, "elpaso-core_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location(name, path, submodule_search_locations=[os.path.dirname(path)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def workload(meshes, args):
    if args.workload == "plate_cavity":
        return meshes.plate_cavity()
    if args.workload == "plate_cavity_small":
        return meshes.plate_cavity(20, 14, 10, 0.6, 0.4, 0.3)
    raise SystemExit(f"unknown workload {args.workload}")


def workload_label(d):
    return (f"{d.name}: DSG4 plate + Fluid8 cavity coupled by InterfaceMindlin quads, "
            "1-500 Hz sweep (1 Hz step, seeded order), unit force")


SWEEP = 1.0 + np.random.default_rng(20260101).permutation(500)
N_ORACLE = 6  # frequencies of the sweep solved by the oracle (CPU baseline and error check)


def sweep(rank, world, step, batch):
    """Frequencies (Hz) of one step on one rank: consecutive blocks of a seeded
    permutation of the 1..500 Hz (1 Hz step) sweep, so every step mixes the
    ill-conditioned low end with the rest of the band."""
    base = (step * world + rank) * batch
    return SWEEP[np.arange(base, base + batch) % 500]


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self, device=0):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(device):
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def cpu_baseline(meshes, args, n_freq=6, keep=0):
    """The oracle (CPU restatement of the reference path) timed on this host.
    Per frequency: the reference's per-w element loop (C, one thread) and an
    FP64 multifrontal LU with nested dissection (oracle/mf.py, the MUMPS
    algorithm restated; dense fronts in LAPACK/BLAS on every host core).
    The symbolic analysis is done once, outside the timed sample, as MUMPS
    reuses it across frequencies; Dirichlet columns are lifted to the
    right-hand side as on the GPU. The first frequency is a warm-up; the
    value is the median over the next n_freq - 1 (at least 5 when the time
    budget allows). Returns (baseline dict, oracle solutions of the first
    `keep` frequencies of the sweep)."""
    from oracle import oracle as orc
    d = workload(meshes, args)
    s = orc.System(d)
    mf = orc.multifrontal(s)
    times, worst, sols = [], 0.0, []
    t_all = time.perf_counter()
    for k in range(max(n_freq, keep)):
        om = 2 * np.pi * SWEEP[k % 500]
        t0 = time.perf_counter()
        A, rhs = s.lifted(om)
        mf.factor(A)
        x = mf.solve(rhs)
        times.append(time.perf_counter() - t0)
        worst = max(worst, float(np.linalg.norm(rhs - A @ x) / np.linalg.norm(s.f)))
        if k < keep:
            sols.append(x)
        if k + 1 >= max(2, keep) and time.perf_counter() - t_all > args.cpu_budget_s:
            break
    timed = times[1:] if len(times) > 1 else times
    med = statistics.median(timed)
    return ({"value": 1.0 / med, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
             "sample": f"{len(timed)} frequency(ies) of the {d.name} sweep after 1 warm-up, median "
                       f"{med:.2f} s each (min {min(timed):.2f}, max {max(timed):.2f}): C element loop + FP64 "
                       f"multifrontal LU (LAPACK/BLAS on {os.cpu_count()} threads); max rel residual {worst:.1e}; "
                       "SciPy SuperLU (COLAMD, one thread) on the same lifted system, measured separately: 160 s "
                       "for one frequency on 8 x86 cores (too slow for a bounded sample)"},
            sols)


def oracle_errors(meshes, args, x_by_prec, sols):
    """||x - x_ref||_1 / ||x_ref||_1 of the GPU solutions against the oracle's
    FP64 direct solves of the same frequencies (the first of the sweep), and
    the relative residual of both, with the oracle's matrix."""
    from oracle import oracle as orc
    d = workload(meshes, args)
    s = orc.System(d)
    out = {}
    for name, x in x_by_prec.items():
        errs, res = [], []
        for k, xr in enumerate(sols):
            om = 2 * np.pi * SWEEP[k]
            A, f = s.matrix(om), s.rhs(om)
            errs.append(float(np.linalg.norm(x[k] - xr, 1) / np.linalg.norm(xr, 1)))
            res.append(float(np.linalg.norm(f - A @ x[k]) / np.linalg.norm(f)))
        out[name] = {"max_err_vs_oracle": max(errs), "max_rel_residual_oracle_matrix": max(res),
                     "frequencies_hz": [float(SWEEP[k]) for k in range(len(sols))]}
    return out


def assembly_measurement(elp, meshes, n_cube=100, repeats=5, fp64_peak=None):
    """K1 on the 100^3 Brick8 cube (1M elements, 3.09M dofs, 245M nonzeros,
    interior nodes perturbed, 4 random materials): device time of the one
    persistent assembly launch, against HBM and FP64 roofs.

    Algorithmic bytes per assembly (the minimum traffic of the result):
    K and M values written once (2 nnz x 8 B), col_idx read once (nnz x 4 B),
    row_ptr (n + 1) x 4, coordinates 24 B per node, connectivity 32 B and a
    material id 2 B per element. Algorithmic work: ~9.5k flop per element
    in the closed form used (J, J^-1, the gradients g and w g at 8 Gauss
    points: 2.8k; 36 node-pair blocks of 9 FMA + the mass FMA per Gauss point:
    5.8k; the 36 K blocks: 0.9k). Timed twice: FP64 throughout (the default,
    the drop-in), then with the double-float contractions
    (ELP_ASSEMBLY_DOUBLE_FLOAT: the gradients and Gauss-point sums in FP32
    pairs, J and J^-1 in FP64)."""
    d = meshes.solid_cube(n_cube)
    m = elp.Model(d).assemble()
    info = m.info()
    mean_ms, best_ms = m.time_assembly(repeats)
    nnz, n, ne, nn = info["nnz"], info["n_dofs"], info["n_elements"], d.n_nodes
    byts = 2 * nnz * 8 + nnz * 4 + (n + 1) * 4 + nn * 24 + ne * (32 + 2)
    flops = 9.5e3 * ne
    hbm, _, src = peaks()
    gbs = byts / (mean_ms / 1e3) / 1e9
    out = {"workload": f"solid_cube_{n_cube}: {ne} Brick8, {n} dofs, nnz {nnz}", "kernel_ms_mean": mean_ms,
           "kernel_ms_best": best_ms, "elements_per_s": ne / (mean_ms / 1e3),
           "algorithmic_bytes": byts, "achieved_gbs": gbs, "hbm_peak_gbs": hbm, "hbm_frac": gbs / hbm,
           "fp64_gflops": flops / (mean_ms / 1e3) / 1e9,
           "fp64_peak_tflops_measured": fp64_peak,
           "fp64_frac": (flops / (mean_ms / 1e3) / 1e12 / fp64_peak) if fp64_peak else None,
           "note": f"HBM peak {src}; FP64 peak measured by elp_peak_fp64 (FMA chains on every SM); "
                   "FP64 is the binding roof of this kernel on GB300"}
    m.set_assembly(elp.ASSEMBLY_DOUBLE_FLOAT)  # assembles again
    df_mean, df_best = m.time_assembly(repeats)
    df_gbs = byts / (df_mean / 1e3) / 1e9
    out["double_float"] = {"kernel_ms_mean": df_mean, "kernel_ms_best": df_best,
                           "elements_per_s": ne / (df_mean / 1e3), "achieved_gbs": df_gbs,
                           "hbm_frac": df_gbs / hbm, "speedup_vs_fp64": mean_ms / df_mean}
    m.close()
    return out


def _server_stream(elp, srv, reqs, rate=None, timeout_s=600.0):
    """Submits `reqs` [(model id, n dofs, omegas)] all at once (rate None) or
    as a Poisson stream of `rate` requests/s, and collects every result.
    Returns (per-request results, wall seconds from the first submission)."""
    import threading
    rng = np.random.default_rng(20260101 + 17)
    gaps = rng.exponential(1.0 / rate, len(reqs)) if rate else np.zeros(len(reqs))
    results, outs = [], []
    done = threading.Event()

    def collect():
        for _ in range(len(reqs)):
            results.append(srv.wait(timeout_s * 1e3))
        done.set()

    t0 = time.perf_counter()
    th = threading.Thread(target=collect, daemon=True)
    th.start()
    t_next = t0
    by_id = {}
    for (mid, n, oms), gap in zip(reqs, gaps):
        t_next += gap
        delay = t_next - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        x = np.zeros((len(oms), n), np.complex128)
        outs.append(x)
        by_id[srv.submit(mid, oms, x)] = (mid, oms)
    done.wait(timeout_s)
    th.join(1.0)
    for r in results:  # which model and frequencies each result belongs to
        r["model"], r["omegas"] = by_id.get(r["request_id"], (None, None))
    return results, time.perf_counter() - t0


def _status_counts(res):
    """{status: count} over request results (0 = every frequency at the target)."""
    out = {}
    for r in res:
        out[str(r["status"])] = out.get(str(r["status"]), 0) + 1
    return out


def serving_measurement(elp, meshes, n_stream=300, n_probe=40):
    """Latency under load through the C-ABI serving loop (elp_server_*), the
    serving workload's shape: 8 resident models with DOF counts log-uniform
    in 5k-500k (seeded, stratified), alternately DSG4 shell plates and Brick8
    steel slabs, each request 1-64 frequencies from U(1, 500) Hz on a
    uniformly chosen model. Capacity = requests/s of a saturating burst of
    `n_probe` requests; then a Poisson stream of `n_stream` requests at 80%
    of that capacity (the serving workload names 10,000; 300 keep the bench
    within minutes). Latency = arrival -> last frequency returned (server
    clock)."""
    descs = meshes.serving_models()
    models = [elp.Model(d) for d in descs]
    ns = [m.n for m in models]
    srv = elp.Server(hbm_budget_bytes=200 << 30, max_inflight=4, precision=elp.MIXED, tol=TOL, omega_batch=16)
    mids = [srv.add_model(m) for m in models]
    rng = np.random.default_rng(20260101 + 5)

    def make(k):
        out = []
        for _ in range(k):
            i = int(rng.integers(len(mids)))
            oms = 2 * np.pi * rng.uniform(1.0, 500.0, int(rng.integers(1, 65)))
            out.append((mids[i], ns[i], oms))
        return out

    # warm-up: every model prepared (assembly, symbolic upload, workspaces)
    _server_stream(elp, srv, [(mids[i], ns[i], 2 * np.pi * np.array([50.0, 300.0])) for i in range(len(mids))])
    probe = make(n_probe)
    res_p, t_p = _server_stream(elp, srv, probe)
    cap = n_probe / t_p
    stream = make(n_stream)
    res, t_s = _server_stream(elp, srv, stream, rate=0.8 * cap)
    lat = np.array([r["latency_ms"] for r in res])
    per_omega = np.array([r["latency_ms"] / r["n_omega"] for r in res])
    solves = sum(len(q[2]) for q in stream)
    srv.close()
    for m in models:
        m.close()
    p50, p99 = float(np.percentile(lat, 50)), float(np.percentile(lat, 99))
    return {"models": [d.name for d in descs], "models_dofs": ns, "requests": len(res),
            "omegas_per_request": "U{1..64}", "capacity_req_s": cap,
            "capacity_solves_s": sum(len(q[2]) for q in probe) / t_p, "offered_req_s": 0.8 * cap,
            "achieved_solves_s": solves / t_s,
            "latency_ms": {"p50": p50, "p99": p99, "max": float(lat.max()), "mean": float(lat.mean()),
                           "p99_over_p50": p99 / p50},
            "latency_per_frequency_ms": {"p50": float(np.percentile(per_omega, 50)),
                                         "p99": float(np.percentile(per_omega, 99))},
            "request_status": _status_counts(res + res_p),
            "max_rel_residual": max(r["max_rel_residual"] for r in res + res_p),
            # requests short of the target: model, frequency count and the residual reached
            "not_at_target": [{"model": descs[mids.index(r["model"])].name if r["model"] in mids else None,
                               "status": r["status"], "max_rel_residual": r["max_rel_residual"],
                               "n_omega": r["n_omega"]}
                              for r in res + res_p if r["status"] != 0][:24],
            "server": "max_inflight 4, omega_batch 16, 2 workspace lanes per model, HBM budget 200 GiB, mixed"}


def large_models_measurement(elp, meshes, n_omega=8):
    """The largest models of the serving range: a 54^3 Brick8 cube (499,125
    DOFs; its top separator alone is a 9k-pivot dense front) and a 407 x 407
    DSG4 plate (499,392 DOFs), each solved at `n_omega` frequencies through
    elp_solve (mixed). elp_solve sizes its batches to half the free device
    memory and picks the front store (whole fronts, or the compact factor
    store when they do not fit); the device memory its workspaces hold
    afterwards is reported beside the per-frequency workspace of both stores."""
    import torch
    out = {}
    for d in (meshes.cube(54), meshes.plate(407, 407, 1.0, 1.0, 0.003)):
        m = elp.Model(d)
        t0 = time.perf_counter()
        m.assemble().analyse()
        t_setup = time.perf_counter() - t0
        info = m.info()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        oms = 2 * np.pi * np.linspace(20.0, 480.0, n_omega)
        t0 = time.perf_counter()
        x, infos = m.solve(oms, precision=elp.MIXED, raise_on_noconv=False)
        t = time.perf_counter() - t0
        free1 = torch.cuda.mem_get_info()[0]
        out[d.name] = {"n_dofs": info["n_dofs"], "max_front": info["max_front"],
                       "factor_tflop_per_frequency": info["factor_flops"] / 1e12,
                       "whole_fronts_gb_per_frequency": info["factor_entries"] * 8 / 1e9,
                       "compact_store_gb_per_frequency": (info["factor_stored"] + info["front_pool"]) * 8 / 1e9,
                       "frequencies": n_omega, "seconds": t, "solves_s": n_omega / t, "setup_s": t_setup,
                       "max_rel_residual": max(i["rel_residual"] for i in infos),
                       "converged": sum(i["converged"] for i in infos),
                       "workspace_gb_held": (free0 - free1) / 1e9}
        m.close()
        del x
    return out


def grouped_plates_measurement(elp, meshes, count=256, n_omega=32, repeats=2):
    """The batched-plates workload through ONE group (elp_group_*): the 256
    plates are one system whose tree levels are factorised by launches over
    the fronts of all plates, every element integrated in one pass, each
    plate at its own 32 frequencies from U(10, 400) Hz. Group creation and
    the first solve (assembly, symbolic upload, workspaces) are outside the
    timed region; the timed region solves all 8,192 (plate, frequency) pairs
    `repeats` times (new frequencies each time), host buffers in and out."""
    descs = meshes.batched_plates(count)
    models = [elp.Model(d) for d in descs]
    t0 = time.perf_counter()
    g = elp.Group(models)
    t_create = time.perf_counter() - t0
    rng = np.random.default_rng(20260101 + 4)
    oms = [2 * np.pi * rng.uniform(10.0, 400.0, (count, n_omega)) for _ in range(repeats + 1)]
    # the autotuner on a 32-plate subgroup (size class: DSG4 plates of 363-19,683 DOFs), then that
    # tuning for the whole group
    sub = elp.Group(models[:32])
    tuned, tuned_s, trials = sub.autotune(oms[0][:32, :16], precision=elp.MIXED)
    sub.close()
    g.set_tuning(**tuned)
    info = g.info()
    t0 = time.perf_counter()
    g.solve(oms[0], precision=elp.MIXED, raise_on_noconv=False)  # assembly, symbolic upload, workspaces
    t_first = time.perf_counter() - t0
    worst, notconv = 0.0, 0
    t0 = time.perf_counter()
    for r in range(repeats):
        _, infos = g.solve(oms[r + 1], precision=elp.MIXED, raise_on_noconv=False)
        for row in infos:
            for i in row:
                worst = max(worst, i["rel_residual"])
                notconv += i["converged"] == 0
    t = time.perf_counter() - t0
    g.close()
    for m in models:
        m.close()
    return {"models": count, "dofs_total": info["n_dofs"], "fronts": info["n_fronts"], "levels": info["n_levels"],
            "solves": count * n_omega * repeats, "seconds": t, "solves_s": count * n_omega * repeats / t,
            "max_rel_residual": worst, "not_converged": notconv, "group_create_s": t_create,
            "first_solve_s": t_first, "factor_gflop_per_slot": info["factor_flops"] / 1e9,
            "autotune": {"size_class": "32 DSG4 plates, 16 frequencies each", "chosen": tuned,
                         "trials": trials},
            "note": "status of a frequency short of 1e-10 is reported, not hidden (its FP64 floor "
                    "eps |||A| |x||| / ||f|| can exceed 1e-10); timed through elp_group_solve with host buffers"}


def batched_plates_measurement(elp, meshes, count=256, n_omega=32):
    """The batched-plates workload: `count` simply supported DSG4 plates m x m,
    m ~ U{10..80} (363-19,683 DOFs), t ~ U(1, 5) mm, each with n_omega
    frequencies from U(10, 400) Hz, all submitted at once to the serving loop.
    Models are created, assembled and analysed before the timed region."""
    descs = meshes.batched_plates(count)
    models = [elp.Model(d).assemble().analyse() for d in descs]
    srv = elp.Server(hbm_budget_bytes=160 << 30, max_inflight=4, precision=elp.MIXED, tol=TOL, omega_batch=n_omega)
    mids = [srv.add_model(m) for m in models]
    rng = np.random.default_rng(20260101 + 4)
    reqs = [(mid, m.n, 2 * np.pi * rng.uniform(10.0, 400.0, n_omega)) for mid, m in zip(mids, models)]
    _server_stream(elp, srv, reqs[:4])  # first-touch workspaces of the server threads
    res, t = _server_stream(elp, srv, reqs)
    out = {"models": count, "dofs_range": [min(m.n for m in models), max(m.n for m in models)],
           "solves": count * n_omega, "seconds": t, "solves_s": count * n_omega / t,
           "request_status": _status_counts(res),
           "max_rel_residual": max(r["max_rel_residual"] for r in res),
           "note": "status 6 = a frequency whose FP64 rounding floor eps |||A| |x||| / ||f|| exceeds 1e-10 "
                   "(no FP64 solution reaches the target there); its residual is reported as reached",
           "latency_ms": {"p50": float(np.percentile([r["latency_ms"] for r in res], 50)),
                          "p99": float(np.percentile([r["latency_ms"] for r in res], 99))}}
    srv.close()
    for m in models:
        m.close()
    return out


# ncu: DRAM read + write of the tensor-core class (k_gemm_tc, k_schur_tc,
# k_pack_schur) in one factorisation of the plate-cavity model, per frequency
TC_CLASS_DRAM_BYTES_PER_FREQUENCY = (20.174e9 + 3.642e9) / 2


def run_ours(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    elp = load_pkg()
    meshes = importlib.import_module("elpaso_core_gb300.meshes")
    fp64_peak = elp.peak_fp64()
    d = workload(meshes, args)
    t0 = time.perf_counter()
    m = elp.Model(d)
    t_create = time.perf_counter() - t0
    m.assemble()
    asm_ms, asm_best = m.time_assembly(3)
    t0 = time.perf_counter()
    m.analyse()
    t_sym = time.perf_counter() - t0
    # the project's autotuner (timed solves of the sweep's first batch; set-up, outside the timed region),
    # or the tuning given with --tuning (a profiling run that must reproduce a benched configuration
    # without the autotuner's many launches before the timed step)
    t0 = time.perf_counter()
    if args.tuning:
        m.set_tuning(**dict((k, int(v)) for k, v in (kv.split("=") for kv in args.tuning.split(","))))
        autotune = {"chosen": m.tuning(), "given": args.tuning}
    else:
        tuned, tuned_s, tune_trials = m.autotune(2 * np.pi * sweep(rank, world, 30_000, args.batch),
                                                 precision=elp.MIXED)
        autotune = {"chosen": tuned, "seconds_per_step_chosen": tuned_s, "trials": tune_trials,
                    "wall_s": time.perf_counter() - t0}
    info = m.info()
    n = info["n_dofs"]
    S = args.batch
    stream = torch.cuda.current_stream()
    sh = C.c_void_p(stream.cuda_stream)
    lib = elp.load_library()
    rhs = torch.from_numpy(m.rhs().view(np.float64).copy()).cuda()
    f_dev = rhs.view(1, n * 2).repeat(S, 1).contiguous()
    x_dev = torch.zeros((S, n * 2), dtype=torch.float64, device="cuda")
    infos = (elp.SolveInfo * S)()

    def solve_step(step, prec, stats=None):
        oms = np.ascontiguousarray(2 * np.pi * sweep(rank, world, step, S))
        rc = lib.elp_solve_device(m.handle, oms.ctypes.data_as(C.c_void_p), S, prec, C.c_void_p(f_dev.data_ptr()),
                                  C.c_void_p(x_dev.data_ptr()), C.cast(infos, C.c_void_p), TOL, sh)
        if rc != 0:
            raise RuntimeError(lib.elp_last_error().decode())
        if stats is not None:
            for i in range(S):
                stats.append(infos[i].rel_residual)
                stats_it.append(infos[i].iterations)

    launches_before = {}

    def timed(prec, steps, warmup):
        for w in range(warmup):
            solve_step(10_000 + w, prec)
        res = []
        global stats_it
        torch.cuda.synchronize()
        launches_before[prec] = sum(v["launches"] for v in elp.profile_read().values())
        elp.profile(False)  # resets the launch counters: they count the timed steps only
        if dist:
            dist.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(steps):
            solve_step(k, prec, res)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1)
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, res

    global stats_it
    stats_it = []
    clocks = Clocks()
    # library launches since the process started (set-up), for ncu's launch skip
    launches_setup = sum(v["launches"] for v in elp.profile_read().values())
    elp.profile(False)
    clocks.start()
    ms_mixed, res_mixed = timed(elp.MIXED, args.steps, args.warmup)
    clk = clocks.stop(local)
    timed_launches = sum(v["launches"] for v in elp.profile_read().values())
    it_mixed = list(stats_it)
    stats_it = []
    # end to end through elp_solve with pinned host buffers
    f_host = torch.empty((S, n), dtype=torch.complex128, pin_memory=True).numpy()
    f_host[:] = m.rhs()
    x_host = torch.empty((S, n), dtype=torch.complex128, pin_memory=True).numpy()
    e2e_steps = max(1, args.steps // 2)
    m.solve(2 * np.pi * sweep(rank, world, 20_000, S), precision=elp.MIXED, f=f_host, out=x_host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        m.solve(2 * np.pi * sweep(rank, world, k, S), precision=elp.MIXED, f=f_host, out=x_host)
    e2e_s = time.perf_counter() - t0
    e2e = e2e_steps * S * world / e2e_s

    value = args.steps * S * world / (ms_mixed / 1e3)

    # live per-kernel-class timing for the roofline (one profiled step)
    elp.profile(True)
    solve_step(0, elp.MIXED)
    torch.cuda.synchronize()
    prof = elp.profile_read()
    elp.profile(False)
    # the tensor-core front updates (Crout and Schur from the fronts, packed
    # Schur, its pack pass) are one class of work: the factorisation's GEMMs
    groups = {k: v for k, v in prof.items() if k not in ("gemm_tc", "schur_tc", "pack")}
    groups["gemm_tc"] = {"ms": sum(prof[k]["ms"] for k in ("gemm_tc", "schur_tc", "pack")),
                         "launches": sum(prof[k]["launches"] for k in ("gemm_tc", "schur_tc", "pack"))}
    top = max(groups.items(), key=lambda kv: kv[1]["ms"])
    hbm, bf16, src = peaks()
    roof = None
    if top[0] == "gemm" or top[0] == "gemm_tc":
        flops = info["gemm_flops"] * S
        ach = flops / (top[1]["ms"] / 1e3) / 1e12
        roof = {"kernel": top[0], "bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                "frac": ach / bf16,
                # DRAM bytes of the class per step: the per-frequency traffic of one factorisation
                # from ncu x the frequencies of the step (each frequency repeats the same launches)
                "traffic": TC_CLASS_DRAM_BYTES_PER_FREQUENCY * S if d.name.startswith("plate_cavity_60x40x30")
                else None,
                "traffic_ref": "ncu, profiles/tensor_core_class_traffic_plate_cavity_60x40x30_batch2.md: "
                               "20.17 GB read + 3.64 GB written by the class's 292 launches of one "
                               "factorisation at 2 frequencies (11.9 GB per frequency), x frequencies "
                               "per step",
                "note": f"algorithmic = Schur-update flops of one factorisation x {S} frequencies; "
                        f"peak = dense bf16 ({src})"}
    else:
        if top[0] in ("forward", "backward"):
            byts = info["factor_bytes"] * S / 2 * prof[top[0]]["launches"] / max(1, info["n_levels"])
        else:
            byts = None
        ach = byts / (top[1]["ms"] / 1e3) / 1e9 if byts else None
        roof = {"kernel": top[0], "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": (ach / hbm) if ach else None, "traffic": None, "note": f"peak = copy bandwidth ({src})"}
    roof["breakdown_ms_per_step"] = {k: round(v["ms"], 3) for k, v in prof.items() if v["launches"]}
    roof["breakdown_launches_per_step"] = {k: v["launches"] for k, v in prof.items() if v["launches"]}

    # plain FP64 last: its workspaces stay allocated, and the mixed measurements
    # above all run with the same memory free
    plain_steps = args.plain_steps
    plain = None
    if plain_steps > 0:  # 0: skip the plain FP64 measurement (small profiling runs)
        ms_plain, res_plain = timed(elp.FP64_PLAIN, plain_steps, 1)
        it_plain = list(stats_it)
        plain = plain_steps * S * world / (ms_plain / 1e3)
    # solutions of the first frequencies of the sweep, for the error against the
    # oracle's FP64 direct solve (untimed; the oracle solves them in cpu_baseline)
    x_oracle_check = {}
    if rank == 0 and world == 1 and not args.no_cpu:
        om_chk = 2 * np.pi * SWEEP[:N_ORACLE]
        x_oracle_check["mixed"] = m.solve(om_chk, precision=elp.MIXED)[0]
        x_oracle_check["plain_fp64"] = m.solve(om_chk, precision=elp.FP64_PLAIN)[0]
    m.close()  # release the sweep model's workspaces before the other measurements allocate theirs

    asm100 = None
    if rank == 0 and not args.no_assembly:
        asm100 = assembly_measurement(elp, meshes, n_cube=args.assembly_n, fp64_peak=fp64_peak)
    serving = plates = large = None
    if rank == 0 and not args.no_serving:
        serving = serving_measurement(elp, meshes, n_stream=args.serving_requests)
        plates = {"grouped": grouped_plates_measurement(elp, meshes),
                  "serving_loop": batched_plates_measurement(elp, meshes)}
        large = large_models_measurement(elp, meshes)
    cpu = None
    err_vs_oracle = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, sols = cpu_baseline(meshes, args, keep=N_ORACLE)
        err_vs_oracle = oracle_errors(meshes, args, x_oracle_check, sols)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mixed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 fronts + f64 refinement", "data": "synthetic",
            "config": {"workload": workload_label(d),
                       "n_dofs": n, "nnz": info["nnz"], "frequencies_per_step": S, "parallelism": f"freq-shard x{world}",
                       "l2": "inputs larger than L2 (front arena "
                             f"{info['factor_entries'] * 8 * S / 1e9:.1f} GB per step)",
                       "fronts": info["n_fronts"], "max_front": info["max_front"], "levels": info["n_levels"],
                       "factor_gflop": info["factor_flops"] / 1e9},
            "plain_fp64": None if plain is None else {
                "value": plain, "unit": UNIT, "ms_per_step": ms_plain / plain_steps,
                "factor_fp64_tflops": plain * info["factor_flops"] / 1e12,
                "factor_fp64_frac_of_measured_peak": plain * info["factor_flops"] / 1e12 / fp64_peak,
                "fp64_peak_tflops_measured": fp64_peak,
                "max_rel_residual": max(res_plain), "iterations": [min(it_plain), max(it_plain)]},
            "speedup_mixed_vs_plain": None if plain is None else value / plain,
            "max_rel_residual": max(res_mixed), "refine_iterations": [min(it_mixed), max(it_mixed)],
            "err_vs_oracle": err_vs_oracle,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": S * n * 16, "d2h_bytes_per_step": S * n * 16},
            "gpu_launches": int(timed_launches),
            # library kernels (demangled names elp::k_*, elp::assemble_*) launched before the
            # timed region of the mixed path: set-up, then the warm-up steps
            "launches_before_timed": int(launches_setup + launches_before[elp.MIXED]),
            "roofline": roof,
            "assembly": {"kernel_ms": asm_best, "elements": info["n_elements"], "host_create_s": t_create,
                         "symbolic_s": t_sym},
            "autotune": autotune,
            "assembly_solid_cube": asm100,
            "serving": serving,
            "batched_plates": plates,
            "large_models": large,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    load_pkg()
    meshes_mod = importlib.import_module("elpaso_core_gb300.meshes")
    b, _ = cpu_baseline(meshes_mod, args, n_freq=max(6, args.steps))
    d = workload(meshes_mod, args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    # n_gpus: the N this arm was launched with; the work runs on rank 0's host cores only
    line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * args.batch / b["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "impl": "reference", "data": "synthetic",
            "config": {"workload": workload_label(d), "frequencies_per_step": args.batch, "host_cores_only": True,
                       "note": "the reference (PETSc/MUMPS) cannot be built here; its CPU path is timed "
                               "as the oracle restatement (element loop + multifrontal LU)"},
            "cpu_baseline": b,
            "e2e": {"value": b["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plate_cavity")
    ap.add_argument("--batch", type=int, default=48)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-assembly", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--assembly-n", type=int, default=100, help="edge of the Brick8 cube of the assembly measurement")
    ap.add_argument("--cpu-budget-s", type=float, default=90.0)
    ap.add_argument("--serving-requests", type=int, default=300,
                    help="requests of the Poisson stream of the serving measurement")
    ap.add_argument("--tuning", default="",
                    help="leaf=..,schur_tile=..,pack_count=..,pack_min_border=..,lanes=.. instead of the autotuner")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
