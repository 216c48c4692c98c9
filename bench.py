#!/usr/bin/env python3
"""Benchmark: systems solved per second at normwise backward error <= 1e-12.

Workload (one step): one SMR91 implicit substep over the production batch --
S=5 coupled equations on Ny=192 order-8 B-spline collocation points
(N=960, KL=KU=34), Nx=256 x Nz=192 wavenumbers -> 24,768 complex128
systems: explicit operator y = P (M + phi_e L) u, complex64 band LU with FP64
iterative refinement (spec zcgbsvx,aiter=5,siter=25,diter=5,tolsc=145) and
complex128 fallback, permutation back to natural order.  Inputs are seeded
synthetic data of the reference's shapes (no dataset exists for this path),
resident in HBM and larger than L2.

--impl reference times the reference algorithm on the host cores (the
oracle's restatement of the bsmbsm/zcgbsvx driver over SciPy's OpenBLAS
LAPACK) on the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "systems solved/s at rel-resid <=1e-12 (mixed c64 LU + FP64 refinement)"
UNIT = "systems/s"
SPEC = dict(aiter=5, siter=25, diter=5, tolsc=145.0)


def rank_config(cfg, rank: int, world: int):
    """Weak scaling over replicas: rank r solves its own wavenumber block of
    the same shape (the configuration's seed offset by the rank); no data
    crosses ranks."""
    from suzerain_gb300 import synth
    if world <= 1:
        return cfg
    return synth.Config(**{**cfg.__dict__, "seed": cfg.seed + 1000 * rank})


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time (the job's time) when world > 1."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "of measured"
    return 6800.0, "of fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(cfg, cs, kx, kz, u, phi_e, phi_i, nsample: int, nthreads: int,
                 mixed: bool = True, idx=None):
    """The reference algorithm on host threads over a bounded sample (evenly
    spaced systems of the batch, or the given indices).  Returns the
    baseline record and the oracle's per-system results."""
    from oracle import oracle as O
    if idx is None:
        idx = np.linspace(0, len(kx) - 1, nsample).round().astype(int)
    nsample = len(idx)
    ob = O.openblas_path() is not None
    r = O.batch_solve(cs, kx[idx], kz[idx], u[idx], phi_exp=phi_e, phi_imp=phi_i, mixed=mixed,
                      aiter=SPEC["aiter"], siter=SPEC["siter"], diter=SPEC["diter"],
                      tolsc=cfg.tolsc, nthreads=nthreads, openblas=ob)
    lat = r["latency"]
    rec = dict(value=nsample / r["wall"], unit=UNIT, cores=nthreads, kind="port",
               sample=(f"{nsample} of {len(kx)} systems of the same batch, evenly spaced; "
                       f"{'zcgbsvx' if mixed else 'zgbsv'} driver restated in C over "
                       f"{'SciPy OpenBLAS' if ob else 'restated zgbtf2'} LAPACK, one system "
                       f"per thread, {nthreads} threads"),
               p50_ms=float(np.percentile(lat, 50) * 1e3),
               p99_ms=float(np.percentile(lat, 99) * 1e3),
               wall_s=r["wall"], info_nonzero=int((r["info"] != 0).sum()))
    if mixed:
        rec["fact_double"] = r["fact"].count("D")
        rec["siter_mean"] = float(r["siter"].mean())
    return rec, r, idx


EDGES = [0.0] + [10.0 ** e for e in range(-17, -5)] + [float("inf")]
EDGE_NAMES = ["0"] + [f"1e{e}" for e in range(-17, -5)] + ["inf"]


def rel_err_hist(x, ref) -> dict:
    """Per-system ||x - ref||_inf / ||ref||_inf as a histogram over decades."""
    err = np.max(np.abs(x - ref), axis=1) / np.max(np.abs(ref), axis=1)
    counts = [int(((err >= lo) & (err < hi)).sum()) for lo, hi in zip(EDGES[:-1], EDGES[1:])]
    return {"systems": int(len(err)), "max": float(err.max()), "median": float(np.median(err)),
            "edges": EDGE_NAMES, "counts": counts}


def oracle_parity(cs, kx, kz, u, phi_e, phi_i, idx, x_mixed, x_plain, fact_gpu, nthreads,
                  mixed_ref=None) -> dict:
    """GPU results against the FP64 oracle (the zgbsv restatement pinned to
    the reference build) on the same systems: per-system forward error of
    the mixed and complex128 solutions, and the mixed path's complex128
    decisions against the oracle's zcgbsvx."""
    from oracle import oracle as O
    ob = O.openblas_path() is not None
    o = O.batch_solve(cs, kx[idx], kz[idx], u[idx], phi_exp=phi_e, phi_imp=phi_i,
                      nthreads=nthreads, openblas=ob)
    out = {"oracle": f"zgbsv restated in C over {'SciPy OpenBLAS' if ob else 'restated zgbtf2'}",
           "mixed_vs_fp64_oracle": rel_err_hist(x_mixed, o["x"])}
    if x_plain is not None:
        out["plain_vs_fp64_oracle"] = rel_err_hist(x_plain, o["x"])
    if mixed_ref is not None:
        f_o = mixed_ref["fact"]
        out["fact_agree"] = float(np.mean([a == b for a, b in zip(fact_gpu, f_o)]))
        out["fact_double_gpu"] = fact_gpu.count("D")
        out["fact_double_oracle"] = f_o.count("D")
    return out


def run_reference(args):
    """The reference algorithm (the oracle's C restatement of the bsmbsm +
    zcgbsvx driver over SciPy's OpenBLAS) on the host cores, over the whole
    batch by default, with inputs from the host-only generator: this process
    never loads the GPU library."""
    rank, local, world = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    from suzerain_gb300 import _native as nat
    nat.bind_generator(O.SYNTH_PATH)
    from suzerain_gb300 import synth
    cfg = synth.CONFIGS[args.config]
    cs, kx, kz, u = cfg.batch()
    phi_e, phi_i = synth.smr91_phis(cfg.phi)
    nthreads = os.cpu_count() or 1
    nsample = args.ref_sample if args.ref_sample > 0 else len(kx)
    times = []
    r = None
    for step in range(args.warmup + args.steps):
        r, _, _ = cpu_baseline(cfg, cs, kx, kz, u, phi_e, phi_i, nsample, nthreads)
        if step >= args.warmup:
            times.append(nsample / r["value"])
    t = sum(times)
    value = nsample * args.steps / t
    same = nsample == len(kx)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64+f64",
        "data": "synthetic (seeded generator of the reference's shapes)",
        "config": {"workload": workload_name(args.config, cfg, cs,
                                             len(kx) if same else nsample, len(kx)),
                   "operator": synth.describe_operator(cfg),
                   "global_batch": nsample, "seq_len": cs.N, "parallelism": "host threads",
                   "same_config": same},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": r["sample"], "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_libraries": loaded_libraries(),
    }
    print(json.dumps(line))
    return 0


def loaded_libraries() -> list:
    """The repository's shared libraries mapped into this process."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for ln in f:
                path = ln.split()[-1] if ln.strip() else ""
                if path.startswith(ROOT) and path.endswith(".so"):
                    out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def workload_name(config, cfg, cs, nsys, nbatch) -> str:
    return (f"SMR91 substep, configuration {config}: S={cs.S} Ny={cs.n} k={cfg.k} N={cs.N} "
            f"KL=KU={cs.KL}, {nsys} of {nbatch} systems per step")


def timed(fn, steps: int, stream) -> float:
    """ms for `steps` calls of fn, CUDA events on stream, synchronized both sides."""
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_variant(key, args, nthreads) -> dict:
    """A bounded run of another operator of the production shape (the
    literal wall mask or the stiff variant): mixed and complex128
    systems/s over the whole batch, decisions, backward error, forward
    error against the FP64 oracle and the host-core reference on a sample."""
    import torch
    from suzerain_gb300 import plan as P, synth
    cfg = synth.CONFIGS[key]
    cs, kx, kz, u = cfg.batch()
    nsys = len(kx)
    phi_e, phi_i = synth.smr91_phis(cfg.phi)
    spec = P.RefineSpec(**{**SPEC, "tolsc": cfg.tolsc})
    stream = torch.cuda.current_stream()
    du = torch.from_numpy(u).cuda()
    dout = torch.empty_like(du)
    # every system may fall back to complex128 (the literal mask sends most)
    bp = P.BatchPlan(cs, kx, kz, parts=args.parts, max_double_slots=nsys, method="M")
    bp.substep("M", phi_e, phi_i, du, dout, spec)
    ms = timed(lambda: bp.substep("M", phi_e, phi_i, du, dout, spec), args.variant_steps, stream)
    rep = bp.report()
    berr = bp.backward_error()
    unserved = bp.unserved()
    x_mixed = dout.cpu().numpy()
    bp.close()
    bz = P.BatchPlan(cs, kx, kz, parts=args.parts, method="Z")
    bz.substep("Z", phi_e, phi_i, du, dout, spec)
    zms = timed(lambda: bz.substep("Z", phi_e, phi_i, du, dout, spec), 1, stream)
    zberr = bz.backward_error()
    x_plain = dout.cpu().numpy()
    bz.close()
    del du, dout
    torch.cuda.empty_cache()
    cpu, om, idx = cpu_baseline(cfg, cs, kx, kz, u, phi_e, phi_i, args.variant_sample, nthreads)
    par = oracle_parity(cs, kx, kz, u, phi_e, phi_i, idx, x_mixed[idx], x_plain[idx],
                        "".join(rep["fact"][i] for i in idx), nthreads, mixed_ref=om)
    return {
        "workload": workload_name(key, cfg, cs, nsys, nsys),
        "operator": synth.describe_operator(cfg),
        "value": nsys * args.variant_steps / (ms / 1e3), "unit": UNIT,
        "ms_per_step": ms / args.variant_steps, "steps": args.variant_steps,
        "rel_resid_max": float(berr.max()), "fact_double": rep["fact"].count("D"),
        "siter_mean": float(rep["siter"].mean()), "siter_max": int(rep["siter"].max()),
        "unserved": int(unserved),
        "plain_c128": {"value": nsys / (zms / 1e3), "ms_per_step": zms,
                       "rel_resid_max": float(zberr.max())},
        "parity": par, "cpu_baseline": cpu,
    }


def run_packed(cfg, cs, kx, kz, u, phi_i, args, peak) -> dict:
    """The caller-packed form: every system's P A P^T as a packed complex128
    band in HBM (packc, LD x N), solved by sgb_zcgbsvx_batched, the
    batched counterpart of bsmbsm_solver_zcgbsvx's solve
    (suzerain/bsmbsm_solver.cpp:377-414).  Here the algorithmic bytes
    16 N (LD + 2) per system are what the kernels really read."""
    import ctypes as C
    import torch
    from suzerain_gb300 import _native as nat, plan as P
    L = nat.load()
    nsys, N = u.shape
    LD = cs.LD
    stream = torch.cuda.current_stream()
    pl = P.Plan(cs, kx, kz)
    ab = torch.empty((nsys, N * LD), dtype=torch.complex128, device="cuda")
    pl.assemble_packed(phi_i, ab, LD, 0, stream=stream.cuda_stream)
    pl.close()
    q = np.array([(i % cs.S) * cs.n + i // cs.S for i in range(N)])
    b = torch.from_numpy(u).cuda()[:, torch.from_numpy(q).cuda()].contiguous()
    x = torch.empty_like(b)
    rep = {k: torch.zeros(nsys, dtype=t, device="cuda") for k, t in
           (("info", torch.int32), ("siter", torch.int32), ("diter", torch.int32),
            ("res", torch.float64), ("tolsc", torch.float64), ("fact", torch.uint8))}
    R = nat.RefineReport(*(rep[k].data_ptr() for k in ("info", "siter", "diter", "res",
                                                         "tolsc", "fact")))
    S = nat.RefineSpec(SPEC["aiter"], SPEC["siter"], SPEC["diter"], cfg.tolsc)

    def step():
        nat.check(L.sgb_zcgbsvx_batched(nsys, N, cs.KL, cs.KU, b"N", ab.data_ptr(), LD,
                                        LD * N, b.data_ptr(), x.data_ptr(), C.byref(S),
                                        C.byref(R), stream.cuda_stream), "sgb_zcgbsvx_batched")
    step()
    ms = timed(step, args.packed_steps, stream) / args.packed_steps
    fact = rep["fact"].cpu().numpy().tobytes().decode()
    tolsc = rep["tolsc"].cpu().numpy()
    bytes_per_sys = 16 * N * (LD + 2)
    achieved = nsys * bytes_per_sys / (ms / 1e3) / 1e9
    del ab, b, x
    torch.cuda.empty_cache()
    return {"value": nsys / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "steps": args.packed_steps,
            "entry": "sgb_zcgbsvx_batched over packc bands (LD x N complex128 per system)",
            "band_bytes": int(nsys * LD * N * 16),
            "fact_double": fact.count("D"), "converged": bool((tolsc <= 1.0).all()),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "note": "whole solve, B_sys = 16 N (LD+2)"}}


def run_ours(args):
    import torch
    rank, local, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from suzerain_gb300 import build as B
    B.build()
    from suzerain_gb300 import _native as nat, plan as P, synth
    L = nat.load()
    if L.sgb_device_ok() != 0:
        raise RuntimeError(nat.last_error())
    nthreads = os.cpu_count() or 1
    cfg = synth.CONFIGS[args.config]
    cfg = rank_config(cfg, rank, world)
    cs, kx, kz, u = cfg.batch()
    if args.nsys:          # first nsys systems of the same batch (profiling runs)
        kx, kz, u = kx[:args.nsys], kz[:args.nsys], u[:args.nsys]
    nsys, N = u.shape
    phi_e, phi_i = synth.smr91_phis(cfg.phi)
    spec = P.RefineSpec(**{**SPEC, "tolsc": cfg.tolsc})
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    du = torch.from_numpy(u).cuda()
    dout = torch.empty_like(du)
    # The timed substeps run the batch as `parts` resident plans on as many
    # streams (capturable substeps: no host synchronization inside), so that
    # one part's FP64 kernels overlap another's complex64 factor.
    parts = max(1, min(args.parts, nsys))
    runner = P.BatchPlan(cs, kx, kz, parts=parts, max_double_slots=args.double_slots,
                         method=args.method)

    def step():
        runner.substep(args.method, phi_e, phi_i, du, dout, spec, stream=sptr)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- timed region: K substeps, inputs resident in HBM ----------------
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    l0 = L.sgb_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = L.sgb_launch_count() - l0
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    value = nsys * world * args.steps / (ms / 1e3)
    async_faults = L.sgb_async_faults()

    if args.profile_step:
        # profiling runs: the warm-up and timed substeps only, then exit, so
        # that a launch list of this command holds exactly those launches
        if rank == 0:
            print(json.dumps({"profile_step": True, "steps": args.steps, "warmup": args.warmup,
                              "launches_before_timed": int(l0),
                              "gpu_launches": int(launches), "ms_per_step": ms / args.steps,
                              "launches_per_step": int(launches) // max(1, args.steps)}))
        runner.close()
        return 0

    # ---- accuracy of the last step (untimed) ------------------------------
    rep = runner.report()
    berr = runner.backward_error()
    ok = bool(berr.max() <= 1e-12 and (rep["info"] == 0).all()) and runner.unserved() == 0
    x_mixed = dout.cpu().numpy()
    dev_bytes = runner.device_bytes()

    # ---- end to end through the public API, host buffers -----------------
    # every step copies the whole batch in from pinned host memory and the
    # result out, part by part on the parts' streams (sgb_batch_substep_host)
    hu = torch.from_numpy(u).pin_memory()
    ho = torch.empty_like(hu).pin_memory()
    hun, hon = hu.numpy(), ho.numpy()
    for _ in range(3):
        runner.substep_host(args.method, phi_e, phi_i, hun, hon, spec, stream=sptr)
    torch.cuda.synchronize()
    # host-timed: keep the interpreter's garbage collector out of the loop
    gc.collect()
    gc.disable()
    e2e_step_ms = []
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        t1 = time.perf_counter()
        runner.substep_host(args.method, phi_e, phi_i, hun, hon, spec, stream=sptr)
        e2e_step_ms.append((time.perf_counter() - t1) * 1e3)
    e2e_s = time.perf_counter() - t0
    gc.enable()
    e2e = nsys * args.e2e_steps / e2e_s
    e2e_same = bool(np.array_equal(hon, x_mixed))
    runner.close()
    del hu, ho

    # ---- per-phase attribution (one plan, separate pass with events) ------
    plan = P.Plan(cs, kx, kz, max_double_slots=args.double_slots)
    plan.substep(args.method, phi_e, phi_i, du, dout, spec, stream=sptr)
    plan.set_timing(True)
    for _ in range(max(1, min(args.steps, 3))):
        plan.substep(args.method, phi_e, phi_i, du, dout, spec, stream=sptr)
    torch.cuda.synchronize()
    phases = plan.timings()
    plan.set_timing(False)

    # ---- complex128 plain path for the mixed-vs-FP64 ratio ---------------
    fp64 = None
    x_plain = None
    if args.fp64_steps > 0:
        plan.substep("Z", phi_e, phi_i, du, dout, spec, stream=sptr)
        fms = timed(lambda: plan.substep("Z", phi_e, phi_i, du, dout, spec, stream=sptr),
                    args.fp64_steps, stream) / args.fp64_steps
        berr64 = plan.backward_error(stream=sptr)
        x_plain = dout.cpu().numpy()
        fp64 = {"systems_per_s": nsys / (fms / 1e3), "ms_per_step": fms,
                "rel_resid_max": float(berr64.max()),
                "mixed_speedup": (nsys / (ms / args.steps / 1e3)) / (nsys / (fms / 1e3))}
    plan.close()
    del du, dout
    torch.cuda.empty_cache()

    # ---- roofline of the dominant kernel ----------------------------------
    peak, peak_src = read_peaks()
    ld = cs.LD
    bytes_per_sys = 16 * N * (ld + 2)       # read packed c128 A once + b + x
    dom = max(phases.items(), key=lambda kv: kv[1][0]) if phases else None
    roof = None
    if dom:
        name, (tot_ms, calls) = dom
        per_launch_ms = tot_ms / calls
        achieved = nsys * bytes_per_sys / (per_launch_ms / 1e3) / 1e9
        traffic = None
        tf = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tf):
            traffic = json.load(open(tf)).get(name)
        roof = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                "traffic": traffic, "algorithmic_bytes_per_system": bytes_per_sys,
                "launch_ms": per_launch_ms}
    step_ms = ms / args.steps
    whole = nsys * bytes_per_sys / (step_ms / 1e3) / 1e9

    cpu = parity = None
    if rank == 0 and not args.no_cpu:
        cpu, om, idx = cpu_baseline(cfg, cs, kx, kz, u, phi_e, phi_i, args.cpu_sample, nthreads)
        parity = oracle_parity(cs, kx, kz, u, phi_e, phi_i, idx, x_mixed[idx],
                               None if x_plain is None else x_plain[idx],
                               "".join(rep["fact"][i] for i in idx), nthreads, mixed_ref=om)

    extras = {}
    if rank == 0 and not args.no_extras:
        for key in ("2literal", "2stiff"):
            try:
                extras[key] = run_variant(key, args, nthreads)
            except Exception as exc:      # recorded, the headline stands
                extras[key] = {"error": repr(exc)}
        try:
            extras["packed_path"] = run_packed(cfg, cs, kx, kz, u, phi_i, args, peak)
        except Exception as exc:
            extras["packed_path"] = {"error": repr(exc)}
        # bounded configuration-3 and configuration-4 runs (their own modes,
        # --config 3 / --config 4, run them at full size)
        if args.extra_cases > 0:
            try:
                extras["batching"] = batching_run(args.extra_cases, 2, 1, 256, local)
            except Exception as exc:
                extras["batching"] = {"error": repr(exc)}
        if args.extra_requests > 0:
            try:
                extras["serving"] = serving_run(args.extra_requests, (0.5, 0.9), ("M",))
            except Exception as exc:
                extras["serving"] = {"error": repr(exc)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 factor + f64 refinement",
            "data": "synthetic (seeded generator of the reference's shapes)",
            "config": {"workload": workload_name(args.config, cfg, cs, nsys, nsys)
                                   + f", method {args.method}",
                       "operator": synth.describe_operator(cfg),
                       "global_batch": nsys * world, "seq_len": N,
                       "parallelism": f"wavenumber blocks x{world}",
                       "parts": parts,
                       "l2": "inputs larger than L2 (u 380 MB, factors 20 GB)"},
            "rel_resid_max": float(berr.max()), "all_converged": ok and async_faults == 0,
            "async_faults": async_faults,
            "fact_double": rep["fact"].count("D"),
            "siter_mean": float(rep["siter"].mean()),
            "gpu_launches": int(launches),
            "clocks": clocks,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(nsys * N * 16),
                    "d2h_bytes_per_step": int(nsys * N * 16), "steps": args.e2e_steps,
                    "step_ms_min": min(e2e_step_ms),
                    "step_ms_median": statistics.median(e2e_step_ms),
                    "step_ms_max": max(e2e_step_ms),
                    "step_ms": [round(t, 3) for t in e2e_step_ms],
                    "entry": "sgb_batch_substep_host (pinned host buffers, per-part copies "
                             "overlapped with the other parts' substeps)",
                    "same_result_as_device_entry": e2e_same},
            "roofline": roof,
            "path_hbm_fraction": {"achieved_GBs": whole, "frac": whole / peak,
                                  "note": "whole substep, algorithmic bytes 16*N*(LD+2) per system"},
            "phases_ms": {k: v[0] / v[1] for k, v in phases.items()},
            "fp64_plain": fp64,
            "parity": parity,
            "cpu_baseline": cpu,
            "device_bytes": dev_bytes,
            **extras,
            "native_libraries": loaded_libraries(),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def batching_run(cases: int, steps: int, warmup: int, tune_nsys: int, local: int,
                 ragged: bool = True) -> dict:
    """Configuration 3's step over `cases` cases: every case resident (one
    plan each), factor shapes tuned per geometry when tune_nsys > 0, one step
    = the three SMR91 substeps of every case recorded into one CUDA graph
    over 8 streams and replayed.  ragged: one persistent complex64 factor
    launch per substep over every case instead of one per case.  value =
    system solves per second (each system solved once per substep)."""
    import torch
    from suzerain_gb300 import multicase, plan as P, synth
    cfgs = synth.config3_cases(cases)
    t0 = time.perf_counter()
    mc = multicase.MultiCase(cfgs, nstreams=8, max_double_slots=128, ragged=ragged)
    tuned = mc.tune("C", nsys=tune_nsys, reps=1) if tune_nsys > 0 else {}
    spec = P.RefineSpec(**SPEC)
    mc.capture("M", spec)
    setup_s = time.perf_counter() - t0
    for _ in range(warmup):
        mc.replay()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    sampler = ClockSampler(local)
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        mc.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    nsys = mc.nsys
    solves = nsys * mc.nsubsteps * steps
    berr = mc.backward_error()
    out = {
        "value": solves / (ms / 1e3), "unit": "systems/s", "steps": steps, "warmup": warmup,
        "ms_per_step": ms / steps,
        "workload": f"config 3: {len(cfgs)} cases, S in {{5,7}}, k in {{6,8}}, Ny in 32..256, "
                    f"{nsys} systems, {len(mc.geometries())} geometries; step = 3 SMR91 "
                    f"substeps of every case, one CUDA graph over 8 streams"
                    + (", ragged factor" if ragged else ""),
        "cases": len(cfgs), "systems": nsys, "geometries": len(mc.geometries()),
        "rel_resid_max": float(berr.max()), "unserved": mc.unserved(),
        "gpu_launches": int(mc.graph_kernels) * steps,
        "tuned_shapes": {f"{k[0]} N={k[1]} KL={k[2]}": list(v) for k, v in tuned.items()},
        "setup_s": setup_s, "clocks": clocks, "device_bytes": mc.device_bytes(),
    }
    mc.close()
    del mc
    torch.cuda.empty_cache()
    return out


def serving_run(requests: int, levels, methods) -> dict:
    """Configuration 4: a Poisson stream of substep-solve requests with case
    shapes drawn as in configuration 3 and lifetimes of 3..30 substeps,
    served by the continuous-batching loop under a 120 GB HBM budget.  The
    capacity (system solves/s with every request present at t = 0) is
    measured first; then the arrival rate runs at the given fractions of it.
    p50/p99 per-substep latency and throughput per level and method."""
    import torch
    from suzerain_gb300 import plan as P, serve, synth
    spec = P.RefineSpec(**SPEC)
    pool = synth.config3_cases(64, seed=synth.SEED_BASE + 4)
    mean_sys = sum(c.nsys for c in pool) / len(pool)
    out = {}
    for method in methods:
        nreq = requests if method == "M" else max(4, requests // 5)
        srv = serve.Server(budget_bytes=120e9, method=method, spec=spec, nstreams=8)
        # warm-up (kernel attributes, first-touch) and capacity
        srv.run(serve.poisson_trace(4, 1e9, seed=99, configs=pool, life=(3, 3)))
        tr = serve.poisson_trace(nreq, 1e9, seed=100, configs=pool)
        srv.prebuild(tr)
        cap = srv.run(tr)
        cap_sps = cap["throughput"]
        lv = []
        for lvl in levels:
            rate = lvl * cap_sps / (mean_sys * 16.5)      # cases/s
            tr = serve.poisson_trace(nreq, rate, seed=int(lvl * 1000), configs=pool)
            srv.prebuild(tr)
            st = srv.run(tr)
            lv.append({"load": lvl, "rate_cases_per_s": rate, **st})
        out[method] = {"requests_per_level": nreq, "capacity_system_solves_per_s": cap_sps,
                       "levels": lv}
    torch.cuda.empty_cache()
    return out


def run_config3(args) -> int:
    """Configuration 3 as its own bench line (all 64 cases by default)."""
    import torch
    rank, local, world = dist_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    from suzerain_gb300 import build as B
    B.build()
    from suzerain_gb300 import _native as nat
    L = nat.load()
    if L.sgb_device_ok() != 0:
        raise RuntimeError(nat.last_error())
    r = batching_run(args.cases, args.steps, args.warmup, 512, local,
                     ragged=not args.per_case_factor)
    line = {
        "metric": "system solves/s at rel-resid <=1e-12 (mixed c64 LU + FP64 refinement)",
        "value": r["value"], "unit": "systems/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 factor + f64 refinement",
        "data": "synthetic (seeded generator of the reference's shapes)",
        "config": {"workload": r["workload"], "l2": "inputs larger than L2"},
        "rel_resid_max": r["rel_resid_max"], "unserved": r["unserved"],
        "gpu_launches": r["gpu_launches"], "tuned_shapes": r["tuned_shapes"],
        "clocks": r["clocks"], "e2e": None, "device_bytes": r["device_bytes"],
    }
    print(json.dumps(line))
    return 0


def run_config4(args) -> int:
    """Configuration 4 as its own bench line.  Requests per level are bounded
    (--requests) so the run ends in minutes; --levels picks the loads."""
    import torch
    rank, local, world = dist_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    from suzerain_gb300 import build as B
    B.build()
    from suzerain_gb300 import _native as nat
    L = nat.load()
    if L.sgb_device_ok() != 0:
        raise RuntimeError(nat.last_error())
    levels = [float(x) for x in args.levels.split(",")]
    methods = ("M", "Z") if args.fp64_steps > 0 else ("M",)
    out = serving_run(args.requests, levels, methods)
    best = out["M"]["levels"][-1]
    line = {
        "metric": "system solves/s under Poisson load (serving), p50/p99 per-substep latency",
        "value": best["throughput"], "unit": "systems/s", "n_gpus": 1,
        "steps": best["substeps"], "warmup": 1, "ms_per_step": best["p50_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor + f64 refinement",
        "data": "synthetic (seeded generator of the reference's shapes)",
        "config": {"workload": f"config 4: Poisson requests, case shapes of config 3, "
                               f"lifetimes 3..30 substeps, 120 GB budget, {args.requests} "
                               f"requests per level (mixed), loads {args.levels}"},
        "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"],
        "serving": out,
        "e2e": None,
    }
    print(json.dumps(line))
    return 0


def run_profile_factor(args) -> int:
    """Profiling run of the complex64 factor on the first --nsys systems
    (default 4096) of configuration 2, rows assembled from the model: one
    mixed substep with two warps per system, then one with three (the
    shapes of the bandwidth-specialized instance), each with one factor
    launch; prints one JSON line of the factor's CUDA-event times and
    exits."""
    import torch
    rank, local, world = dist_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    from suzerain_gb300 import build as B
    B.build()
    from suzerain_gb300 import _native as nat, plan as P, synth, tune as T
    L = nat.load()
    if L.sgb_device_ok() != 0:
        raise RuntimeError(nat.last_error())
    nsys = args.nsys or 4096
    cfg = synth.CONFIGS[2]
    cs, kx, kz, u = cfg.batch()
    kx, kz, u = kx[:nsys], kz[:nsys], u[:nsys]
    phi_e, phi_i = synth.smr91_phis(cfg.phi)
    pl = P.Plan(cs, kx, kz, max_double_slots=64)
    du = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    out = torch.empty_like(du)
    spec = P.RefineSpec(**SPEC)
    saved = T.get_shape("C", cs.N, cs.KL, cs.KU)
    times = {}
    try:
        pl.set_timing(True)
        for nw in (2, 3):
            T.set_shape("C", cs.N, cs.KL, cs.KU, 4, nw)
            pl.substep("M", phi_e, phi_i, du, out, spec)
            torch.cuda.synchronize()
            t, n = pl.timings()["factor_c64"]
            times[f"nw{nw}"] = t / n
            pl.set_timing(False)
            pl.set_timing(True)
    finally:
        T.set_shape("C", cs.N, cs.KL, cs.KU, *saved)
        pl.close()
    print(json.dumps({"profile_factor": True, "systems": nsys, "factor_ms": times}))
    return 0


def run_profile_kernels(args) -> int:
    """Profiling runs of the kernels beside the headline substep, on the
    first --nsys systems (default 4096) of configuration 2: the packed-band
    assembly (sgb_plan_assemble_packed), the caller-packed mixed solve
    (sgb_zcgbsvx_batched: factor from the packed band, packed FP64
    residual), the FP64 backward-error check, and the production operator
    (rholut_imexop, k = 8, Ny = 192, N = 960) packed and applied for as many
    wavenumber pairs.  Each runs twice; prints one JSON line of CUDA-event
    times and exits."""
    import ctypes as C
    import torch
    rank, local, world = dist_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    from suzerain_gb300 import build as B
    B.build()
    from suzerain_gb300 import _native as nat, plan as P, rholut, synth
    L = nat.load()
    if L.sgb_device_ok() != 0:
        raise RuntimeError(nat.last_error())
    nsys = args.nsys or 4096
    cfg = synth.CONFIGS[2]
    cs, kx, kz, u = cfg.batch()
    kx, kz, u = kx[:nsys], kz[:nsys], u[:nsys]
    phi_e, phi_i = synth.smr91_phis(cfg.phi)
    N, LD = cs.N, cs.LD
    stream = torch.cuda.current_stream()
    out = {}

    def ev(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        return timed(fn, reps, stream) / reps

    pl = P.Plan(cs, kx, kz, max_double_slots=256)
    ab = torch.empty((nsys, N * LD), dtype=torch.complex128, device="cuda")
    out["assemble_packed_ms"] = ev(lambda: pl.assemble_packed(phi_i, ab, LD, 0, stream=stream.cuda_stream))
    q = np.array([(i % cs.S) * cs.n + i // cs.S for i in range(N)])
    b = torch.from_numpy(u).cuda()[:, torch.from_numpy(q).cuda()].contiguous()
    x = torch.empty_like(b)
    rep = {k: torch.zeros(nsys, dtype=t, device="cuda") for k, t in
           (("info", torch.int32), ("siter", torch.int32), ("diter", torch.int32),
            ("res", torch.float64), ("tolsc", torch.float64), ("fact", torch.uint8))}
    R = nat.RefineReport(*(rep[k].data_ptr() for k in ("info", "siter", "diter", "res",
                                                         "tolsc", "fact")))
    S = nat.RefineSpec(SPEC["aiter"], SPEC["siter"], SPEC["diter"], cfg.tolsc)
    out["packed_zcgbsvx_ms"] = ev(lambda: nat.check(L.sgb_zcgbsvx_batched(
        nsys, N, cs.KL, cs.KU, b"N", ab.data_ptr(), LD, LD * N, b.data_ptr(), x.data_ptr(),
        C.byref(S), C.byref(R), stream.cuda_stream), "sgb_zcgbsvx_batched"))
    del ab, b, x
    du = torch.from_numpy(u).cuda()
    dout = torch.empty_like(du)
    pl.substep("M", phi_e, phi_i, du, dout, P.RefineSpec(**{**SPEC, "tolsc": cfg.tolsc}),
               stream=stream.cuda_stream)
    out["backward_error_ms"] = ev(lambda: pl.backward_error(stream=stream.cuda_stream))
    pl.close()
    del du, dout
    torch.cuda.empty_cache()
    # production operator on the configuration-2 wall-normal geometry
    Ny, k = 192, 8
    x01 = np.linspace(0, 1, Ny - k + 2)
    bp = np.array([2 * L.suzerain_htstretch2(2.0, 1.0, float(t)) for t in x01])
    w = L.sgb_bsplineop_alloc_breakpoints(k, len(bp), bp.ctypes.data, 2)
    y = np.linspace(0, 2, Ny)
    prof = {nm: 0.2 * (1 + 0.3 * np.sin((i + 1) * y)) for i, nm in enumerate(rholut.PROFILES)}
    prof["nu"] = 1 + 0.1 * np.cos(y)
    op = rholut.Operator(dict(Re=3000.0, Pr=0.7, Ma=1.5, alpha=3.0, gamma=1.4), prof, w)
    g = op.geometry
    km = torch.from_numpy(np.asarray(kx, dtype=np.float64)).cuda()
    kn = torch.from_numpy(np.asarray(kz, dtype=np.float64)).cuda()
    pab = torch.empty((nsys, g.N * g.LD), dtype=torch.complex128, device="cuda")
    out["rholut_pack_ms"] = ev(lambda: op.pack(complex(phi_i, 0), km, kn, pab, stream=stream.cuda_stream))
    xt = torch.from_numpy(u).cuda()
    yt = torch.empty_like(xt)
    out["rholut_accumulate_ms"] = ev(lambda: op.accumulate(complex(phi_e, 0), km, kn, xt, 0, yt,
                                                           stream=stream.cuda_stream))
    op.close()
    L.suzerain_bsplineop_free(w)
    print(json.dumps({"profile_kernels": True, "nsys": nsys, "N": N, **out}))
    return 0


def run_peaks(args) -> int:
    """Pipe-throughput microbenchmarks of this GPU (FP64 FMA, FP32 FMA, packed
    FP32 FMA, shared-memory loads) with the clocks seen meanwhile: the
    denominators of the compute-pipe fractions quoted for the factor and the
    FP64 kernels.  One JSON line."""
    import ctypes as C
    import torch
    rank, local, world = dist_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    from suzerain_gb300 import build as B
    B.build()
    from suzerain_gb300 import _native as nat
    L = nat.load()
    if L.sgb_device_ok() != 0:
        raise RuntimeError(nat.last_error())
    out = (C.c_double * 7)()
    sampler = ClockSampler(local)
    sampler.start()
    runs = []
    for _ in range(max(1, args.steps)):
        nat.check(L.sgb_measure_peaks(out, None), "sgb_measure_peaks")
        runs.append(list(out))
    clocks = sampler.stop()
    best = [max(r[i] for r in runs) for i in range(4)]
    sm = clocks.get("sm_mhz") or out[5]
    line = {"peaks": {"fp64_fma_tflops": best[0], "fp32_fma_tflops": best[1],
                      "fp32_ffma2_tflops": best[2], "smem_load_tbs": best[3],
                      "smem_bytes_per_clk_per_sm": best[3] * 1e12 / out[6] / (sm * 1e6),
                      "sm_count": int(out[6]), "sm_clock_mhz_used": sm},
            "method": "8 independent chains per thread, 64 warps per SM, CUDA events; "
                      "best of the runs; smem: conflict-free 64-bit loads",
            "runs": len(runs), "clocks": clocks}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default=2,
                    type=lambda s: s if s in ("2stiff", "2literal") else int(s))
    ap.add_argument("--method", default="M", choices=["M", "Z"])
    ap.add_argument("--double-slots", type=int, default=2048)
    ap.add_argument("--parts", type=int, default=4,
                    help="resident plans (one stream each) the timed batch is split into")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="reference arm: systems per step (0: the whole batch)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the literal-mask, stiff, packed-band, batching and serving runs")
    ap.add_argument("--variant-steps", type=int, default=2)
    ap.add_argument("--variant-sample", type=int, default=1024)
    ap.add_argument("--packed-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cases", type=int, default=64, help="configuration 3: number of cases")
    ap.add_argument("--per-case-factor", action="store_true",
                    help="configuration 3: one complex64 factor launch per case instead of "
                         "the ragged launch over all cases")
    ap.add_argument("--requests", type=int, default=40,
                    help="configuration 4: requests per load level (mixed)")
    ap.add_argument("--levels", default="0.1,0.3,0.5,0.7,0.9",
                    help="configuration 4: loads, fractions of the measured capacity")
    ap.add_argument("--extra-cases", type=int, default=16,
                    help="default line: configuration-3 cases of the `batching` key (0: skip)")
    ap.add_argument("--extra-requests", type=int, default=16,
                    help="default line: requests per level of the `serving` key (0: skip)")
    ap.add_argument("--nsys", type=int, default=0,
                    help="use only the first NSYS systems of the batch (profiling)")
    ap.add_argument("--profile-step", action="store_true",
                    help="run the warm-up and timed substeps only (launch lists)")
    ap.add_argument("--peaks", action="store_true",
                    help="print this GPU's pipe-throughput microbenchmarks and exit")
    ap.add_argument("--profile-kernels", action="store_true",
                    help="run the kernels beside the headline substep once each (profiling)")
    ap.add_argument("--profile-factor", action="store_true",
                    help="one mixed substep per complex64 factor shape, two then three warps "
                         "(profiling)")
    args = ap.parse_args()
    if args.peaks:
        return run_peaks(args)
    if args.profile_factor:
        return run_profile_factor(args)
    if args.profile_kernels:
        return run_profile_kernels(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 3:
        return run_config3(args)
    if args.config == 4:
        return run_config4(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
