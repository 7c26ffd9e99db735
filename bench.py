"""Benchmark: IS-SPA MD throughput (atom-steps/s, ns/day) on one GB300.

Workload: the plain drop-in path on the 1100-atom system (50 chains of 22
atoms, nMC = 50, 60 A box, all-pairs FP32 nonbond + IS-SPA, Andersen at
298 K), synthetic inputs of the benchmark's shapes (no public dataset).
One step = one full MD step: bonded, IS-SPA field + force, nonbond,
leapfrog (graph-replayed).

  python bench.py [--steps K] [--warmup W] [--impl gb300|reference] [--no-batched] [--no-extra]

The gb300 arm prints one JSON line with device-timed throughput, the end-to-end
figure through the C ABI with host buffers, the roofline of the dominant
kernel and two CPU baselines timed on this host: the reference's own OpenMP
path (src/isspa_force.omp.c, compiled unmodified) and the FP64 CPU oracle
(same physics as the engine).  Further sections: the 44-atom system, the
reference's published ADI2 umbrella run through the drop-in executable, 64
umbrella windows in one engine, the 16 384-atom precision workload and the
adjoint.  The reference arm times the reference's OpenMP path with all host
threads on the same workload (the FP64 oracle where that file cannot be
built).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "isspa-force-cuda_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "oracle", "ref_omp")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "atom-steps/s (IS-SPA MD, plain single window, FP32)"
UNIT = "atom-steps/s"
DT_PS = 0.002
L2_FLUSH = 256 << 20  # twice the 129 MB L2
# algorithmic work per pair / point, FMA = 2 flops (fixed convention)
FLOP_FIELD_PAIR, FLOP_FORCE_PAIR, FLOP_POINT, FLOP_NB_PAIR = 38, 88, 30, 32


def ns_per_day(steps_per_s: float) -> float:
    return steps_per_s * DT_PS * 1e-3 * 86400.0


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self):
        if not self.lines:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(kernel)


def force_errors(f, ref, floor=0.10):
    """Normwise max |dF| / max |F| and the per-atom |dF_i| / |F_i| (median,
    max) over atoms with |F_i| >= floor x the largest |F|."""
    f = np.asarray(f, np.float64)[:, :3]
    ref = np.asarray(ref, np.float64)[:, :3]
    mag = np.linalg.norm(ref, axis=1)
    sel = mag >= floor * mag.max()
    rel = np.linalg.norm(f - ref, axis=1)[sel] / mag[sel]
    return {"normwise": float(np.abs(f - ref).max() / np.abs(ref).max()),
            "per_atom_median": float(np.median(rel)), "per_atom_max": float(rel.max()),
            "per_atom_floor": floor, "atoms_checked": int(sel.sum())}


def cpu_oracle_rate(system, budget_s: float, min_steps: int = 1, max_steps: int = 1000000, gpu_force=None,
                    warmup: int = 0):
    """Full force evaluations + leapfrog of the FP64 oracle on all host cores.
    With `gpu_force` (the engine's total force of step 0 on the same state)
    the first oracle step also checks it (force_errors)."""
    import oracle

    oracle.build()
    cores = host_cores()
    o = oracle.Oracle(system, threads=cores)
    err = None
    for k in range(warmup):
        o.total_force(seed=system.seed, step=k)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        f, _, _ = o.total_force(seed=system.seed, step=n)
        if n == 0 and gpu_force is not None:
            err = force_errors(gpu_force, f)
        o.leapfrog(f, seed=system.seed, step=n)
        n += 1
        if n >= min_steps and time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return system.n_atoms * n / dt, n, dt, cores, err


def ref_omp():
    """The reference's OpenMP path bound to the 1100-atom system, or the reason it is unavailable."""
    try:
        import isspa_gb300.synth as synth
        from time_ref_omp import RefOmp

        return RefOmp(synth.config_plain(seed=2)), None
    except Exception as exc:  # no checkout and no staged copy, or no compiler
        return None, f"{type(exc).__name__}: {exc}"


def best_threads(r, cores: int):
    """Thread count at which the reference's OpenMP path runs fastest on this
    host (its glibc rand() calls serialise threads, so all cores is not
    always fastest): three calls at each of 1, 2, 4, ... and all cores."""
    counts = sorted({1, cores} | {t for t in (2, 4, 8, 16, 32, 64) if t < cores})
    scan = {}
    for t in counts:
        r.call(t)
        t0 = time.perf_counter()
        for _ in range(3):
            r.call(t)
        scan[t] = r.n * 3 / (time.perf_counter() - t0)
    return max(scan, key=scan.get), {str(k): round(v, 1) for k, v in scan.items()}


def cpu_reference_omp(budget_s: float):
    """cpu_baseline of kind "reference": the reference's own OpenMP CPU path on
    all host cores (and on one), one call per step."""
    from time_ref_omp import CAVEAT, cpu_model

    r, why = ref_omp()
    if r is None:
        return None, why
    cores = host_cores()
    best, scan = best_threads(r, cores)
    v, n, dt = r.rate(best, budget_s, min_calls=3)
    return {"value": round(v, 1), "unit": UNIT, "cores": best, "kind": "reference",
            "sample": f"{n} calls of cpu_ispa_force (src/isspa_force.omp.c:11-105, compiled unmodified) on the "
                      f"same 1100-atom system, nMC 50, {best} OpenMP threads, the fastest count on this host "
                      f"({dt:.1f} s)",
            "threads_scan_atom_steps_per_s": scan, "host_cores": cores,
            "cpu": cpu_model(), "caveat": CAVEAT, "source_sha256": r.source_sha256}, None


def workload_config():
    """The workload both arms report (identical dicts)."""
    return {"workload": "plain drop-in path: 1100 atoms (50 x 22-atom chains), nMC=50, 60 A box, "
                        "all-pairs nonbond + IS-SPA, leapfrog/Andersen 298 K, dt 2 fs",
            "n_atoms": 1100, "n_mc": 50, "mc_points": 55000, "box_A": 60.0,
            "l2": "256 MB written between timed steps (outside the timed intervals)"}


def run_gb300(args):
    import build as engine_build
    import isspa_gb300 as ig

    engine_build.build()
    sysm = ig.synth.config_plain(seed=2)
    N, M = sysm.n_atoms, sysm.n_mc
    P = N * M
    eng = ig.Engine(sysm)
    f_step0 = eng.compute_forces()  # step-0 forces, checked against the oracle in the CPU leg
    eng.zero_forces()
    shapes = eng.shapes() if args.no_autotune else eng.autotune()
    shapes["autotuned"] = not args.no_autotune
    eng.step(args.warmup)
    eng.time_steps_detailed(max(args.warmup, 3), L2_FLUSH)
    # about half a second of further untimed steps, so that the SM clock has
    # left its idle state before the timed region starts
    per_step_ms = eng.time_steps(20) / 20
    warm_steps = int(min(20000, max(0, 500.0 / max(per_step_ms, 1e-3))))
    eng.step(warm_steps)
    eng.synchronize()
    with ClockSampler(0) as clk:
        # the step as it runs (one single-step graph per timed interval), then
        # the same step captured with an event pair around every kernel for the
        # per-kernel durations (those event nodes lengthen the step itself)
        total_ms = eng.time_steps(args.steps, L2_FLUSH)
        instr_ms, kern = eng.time_steps_detailed(args.steps, L2_FLUSH)
    eng.synchronize()
    status = eng.device_status()
    ms_step = total_ms / args.steps
    value = N * args.steps / (total_ms * 1e-3)

    # end to end through the C ABI (isspa_step_host, called as a C caller would:
    # buffer addresses computed once) with host buffers from isspa_host_alloc;
    # every step moves positions and velocities in and positions, velocities
    # and forces out, inside the timed region
    L = ig.abi.lib()
    nbytes = 16 * N
    arrs = [ig.host_array((N, 4)) for _ in range(5)]
    addr = [a.ctypes.data for a in arrs]
    arrs[0][:] = eng.positions()
    arrs[1][:] = eng.velocities()
    step_host = L.isspa_step_host
    for _ in range(3):
        ig.abi.check(step_host(eng._h, addr[0], addr[1], addr[2], addr[3], addr[4]), "step_host")
    t0 = time.perf_counter()
    for k in range(args.steps):
        src, dst = (0, 2) if k % 2 == 0 else (2, 0)
        rc = step_host(eng._h, addr[src], addr[src + 1], addr[dst], addr[dst + 1], addr[4])
        if rc:
            ig.abi.check(rc, "step_host")
    e2e_s = time.perf_counter() - t0
    e2e = N * args.steps / e2e_s
    del arrs

    # roofline of the dominant kernel (FP32 CUDA-core bound: the pair sums are
    # not contractions); peak = live FMA probe on this GPU
    flops = {"field": FLOP_FIELD_PAIR * N * P + FLOP_POINT * P, "force": FLOP_FORCE_PAIR * N * P,
             "nonbond": FLOP_NB_PAIR * N * (N - 1)}
    avg = {k: (v[0] / v[1]) for k, v in kern.items() if v[1] > 0}
    dom = max(avg, key=avg.get)
    peak_fp32 = ig.measure_fp32_peak()
    kname = {"field": "field_kernel", "force": "force_kernel", "nonbond": "nonbond_kernel"}.get(dom, dom)
    if dom in flops:
        achieved = flops[dom] / (avg[dom] * 1e-3) / 1e12
        roof = {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(peak_fp32, 3),
                "unit": "TFLOP/s", "frac": round(achieved / peak_fp32, 4),
                "traffic": ncu_traffic(kname), "kernel": kname,
                "peak_source": "measured FP32 FMA probe on this GPU (MEASURED_PEAKS.json has HBM and bf16 only)"}
    else:
        roof = {"bound": "fp32", "achieved": None, "peak": round(peak_fp32, 3), "unit": "TFLOP/s",
                "frac": None, "traffic": None, "kernel": kname}
    step_flops = sum(flops.values())
    roof["step_achieved_tflops"] = round(step_flops / (ms_step * 1e-3) / 1e12, 3)
    roof["step_frac"] = round(roof["step_achieved_tflops"] / peak_fp32, 4)
    pk = measured_peaks()
    hbm_bytes = 16 * N * 4 + 64 * P * 2  # pos/vel/force read+write, point records written and read once
    roof["hbm"] = {"achieved_gbs": round(hbm_bytes / (ms_step * 1e-3) / 1e9, 2),
                   "peak_gbs": pk.get("hbm_gbs") if pk else 6800.0,
                   "peak_source": "MEASURED_PEAKS.json" if pk else "fallback"}
    launches = int(sum(v[1] for v in kern.values()))

    cpu_value, cpu_steps, cpu_s, cores, f_err = cpu_oracle_rate(sysm, budget_s=args.cpu_budget, gpu_force=f_step0)
    port = {"value": round(cpu_value, 1), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{cpu_steps} full MD steps of the same 1100-atom system ({cpu_s:.1f} s), FP64 CPU oracle "
                      "(the engine's physics: bonded, IS-SPA, nonbond, leapfrog), OpenMP"}
    ref_line, ref_why = cpu_reference_omp(budget_s=args.cpu_budget / 2)
    cfg = workload_config()
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "ns_per_day": round(ns_per_day(args.steps / (total_ms * 1e-3)), 1),
        "config": cfg,
        "run": {"timing": "value: K single-step graph replays, CUDA events around each; kernel durations: "
                          "K more replays of the step captured with events around every kernel",
                "graph": True, "instrumented_ms_per_step": round(instr_ms / args.steps, 5),
                "warmup_extra_steps": warm_steps, "launch_shapes": shapes},
        "e2e": {"value": round(e2e, 1), "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes,
                "d2h_bytes_per_step": 3 * nbytes,
                "path": "isspa_step_host per step (host wall clock, synchronous call) with isspa_host_alloc "
                        "buffers, which the GPU reads and writes directly"},
        "gpu_launches": launches,
        "kernel_ms_per_launch": {k: round(v, 5) for k, v in avg.items()},
        "roofline": roof,
        "cpu_baseline": ref_line if ref_line is not None else port,
        "cpu_baseline_port": port,
        "device_status": status,
        "force_error": dict(f_err or {}, target=1e-5,
                            what="total force of step 0 (bonded, IS-SPA, nonbond) against the FP64 oracle on the "
                                 "same Philox MC points"),
    }
    if ref_line is None:
        line["cpu_baseline_reference_unavailable"] = ref_why
    clocks = clk.summary()
    line["clocks"] = clocks
    if not args.no_extra:
        line["small_44"] = run_small(ig, args)
        line["adi2_published"] = run_adi2_published(args)
    if not args.no_batched:
        line["batched"] = run_batched(ig, args, value)
    if not args.no_extra:
        line["precision"] = run_precision(ig, args, peak_fp32)
        line["adjoint"] = run_adjoint(ig)
    print(json.dumps(line))


def run_small(ig, args):
    """The 44-atom system (2 chains of 22, nMC 20, 40 A box): single-step
    graph replays timed with events (L2 flushed between them, as the headline),
    and a production-style run of back-to-back 8-step graphs timed on the host
    clock, the way the reference's run logs measure ns/day."""
    import oracle

    s = ig.synth.config_small(seed=1)
    eng = ig.Engine(s)
    f0 = eng.compute_forces()
    eng.zero_forces()
    shapes = eng.autotune()
    ref, _, _ = oracle.Oracle(s).total_force(seed=s.seed, step=0)
    eng.step(200)
    steps = max(200, args.steps)
    ms = eng.time_steps(steps, L2_FLUSH)
    _, kern = eng.time_steps_detailed(steps, L2_FLUSH)
    n_run = 40000
    eng.synchronize()
    t0 = time.perf_counter()
    eng.step(n_run)
    eng.synchronize()
    dt = time.perf_counter() - t0
    status = eng.device_status()
    eng.close()
    return {"workload": "44 atoms (2 x 22-atom chains), nMC=20, 40 A box, leapfrog/Andersen 298 K, dt 2 fs",
            "steps": steps, "value": round(s.n_atoms * steps / (ms * 1e-3), 1), "unit": UNIT,
            "ms_per_step": round(ms / steps, 5), "ns_per_day": round(ns_per_day(steps / (ms * 1e-3)), 1),
            "run": {"steps": n_run, "seconds": round(dt, 4), "value": round(s.n_atoms * n_run / dt, 1),
                    "ns_per_day": round(ns_per_day(n_run / dt), 1),
                    "timing": "isspa_step over back-to-back 8-step graphs, host wall clock"},
            "kernel_ms_per_launch": {k: round(v[0] / max(v[1], 1), 5) for k, v in kern.items()},
            "launch_shapes": shapes, "device_status": status, "force_error": force_errors(f0, ref)}


ADI2_PUBLISHED_NS_DAY = 1272.74  # timing_tests/ADI2_US/window_10.0/ADI2.run0.log:66, GeForce GTX 1080


def run_adi2_published(args, n_steps: int = 50000):
    """The reference's published ADI2 umbrella run (44 atoms, nMC 100, 200 A
    box, US k = 20 at x0 = 10 A, seed 34669, trajectory output every 1000
    steps) through the drop-in executable on the reference's own input files,
    with its own ns/day report (wall clock of the step loop, as the
    reference's timing_class)."""
    import re
    import shutil
    import tempfile

    golden = os.path.join(ROOT, "tests", "golden")
    exe = os.path.join(ROOT, "isspa-force-cuda_gb300", "total_force_gb300")
    with tempfile.TemporaryDirectory() as d:
        for f in ("ADI2.prmtop", "ADI2.isspatop", "ADI2.rst7"):
            shutil.copy(os.path.join(golden, f), os.path.join(d, f))
        with open(os.path.join(golden, "ADI2.us")) as f:
            us = f.read().replace("XXX", "10.0")
        with open(os.path.join(d, "us_params.dat"), "w") as f:
            f.write(us)
        cfg = "\n".join([
            "velRst = 0", "inputVel = notread.rst", "prmtop = ADI2.prmtop", "inputCoord = ADI2.rst7",
            "isspaPrmtop = ADI2.isspatop", "forFile = forces.xyz", "posFile = positions.xyz",
            "velFile = velocities.xyz", "posRstFile = positions.rst", "velRstFile = velocities.rst",
            "nMC = 100", f"nSteps = {n_steps}", "deltaWrite = 1000", "temperature = 298.00", "seed = 34669",
            "cutoff = 12.0", "dielectric = 1.0", "boxLength = 200.0", "US = 1", "usCfgFile = us_params.dat",
            "pnu = 0.02", ""])
        with open(os.path.join(d, "config.txt"), "w") as f:
            f.write(cfg)
        r = subprocess.run([exe, "config.txt"], cwd=d, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            return {"error": f"drop-in executable exited {r.returncode}: {r.stderr.strip()[-300:]}"}
        m = re.search(r"Average ns/day =\s*([0-9.]+)", r.stdout)
        t = re.search(r"Elapsed CPU/GPU time =\s*([0-9.]+) ms", r.stdout)
        shapes = re.search(r"launch shapes: (.*)", r.stdout)
    nsd = float(m.group(1))
    ms = float(t.group(1))
    return {"workload": "ADI2 dimer (44 atoms), the reference's published umbrella run settings: nMC 100, "
                        "200 A box, US k=20 x0=10 A, seed 34669, output every 1000 steps, reference input files; "
                        "Andersen pnu 0.02 set explicitly (the published config leaves pnu uninitialised, and "
                        "without a thermostat the stochastic IS-SPA force heats the system without bound)",
            "steps": n_steps, "ns_per_day": nsd, "seconds": round(ms * 1e-3, 3),
            "value": round(44 * n_steps / (ms * 1e-3), 1), "unit": UNIT,
            "published_ns_per_day": ADI2_PUBLISHED_NS_DAY, "published_hardware": "GeForce GTX 1080",
            "ratio_vs_published": round(nsd / ADI2_PUBLISHED_NS_DAY, 2),
            "launch_shapes": shapes.group(1) if shapes else None,
            "timing": "total_force_gb300 step loop, host wall clock (timing_class.cpp:57-58)"}


def run_batched(ig, args, plain_value):
    """64 umbrella windows (44..1100 atoms) in one engine against the plain
    single-window path run window by window on the same GPU (the way the
    reference runs one window per process), both timed as single-step graph
    replays with 256 MB written between steps."""
    wins = ig.synth.config_batched(n_windows=64, seed=4)
    eng = ig.Engine(wins)
    shapes = eng.shapes() if args.no_autotune else eng.autotune()
    nat = sum(w.n_atoms for w in wins)
    steps = max(200, args.steps)
    eng.step(3)
    ms = eng.time_steps(steps, L2_FLUSH)
    _, kern = eng.time_steps_detailed(min(steps, 50), L2_FLUSH)
    status = eng.device_status()
    batched = nat * steps / (ms * 1e-3)
    eng.close()
    plain_ms, plain_steps = 0.0, 20
    for w in wins:
        e1 = ig.Engine(w)
        e1.step(3)
        plain_ms += e1.time_steps(plain_steps, L2_FLUSH) / plain_steps
        e1.close()
    plain = nat / (plain_ms * 1e-3)
    return {"windows": len(wins), "atoms_total": nat, "steps": steps, "seconds_timed": round(ms * 1e-3, 3),
            "value": round(batched, 1), "unit": UNIT, "ms_per_step": round(ms / steps, 4),
            "aggregate_ns_per_day": round(len(wins) * ns_per_day(steps / (ms * 1e-3)), 1),
            "plain_per_window_value": round(plain, 1), "plain_steps_per_window": plain_steps,
            "speedup_vs_plain": round(batched / plain, 2),
            "l2": "256 MB written between timed steps on both sides",
            "launch_shapes": shapes, "device_status": status,
            "kernel_ms_per_step": {k: round(v[0] / max(v[1], 1), 4) for k, v in kern.items()}}


def run_precision(ig, args, peak_fp32):
    """16 384-atom precision workload (256 x 64-atom chains, nMC 100, 1.64 M MC
    points): device-timed graph steps and the force kernel's FP32 rate."""
    s = ig.synth.config_precision(seed=3)
    N, P = s.n_atoms, s.n_atoms * s.n_mc
    eng = ig.Engine(s)
    shapes = eng.shapes() if args.no_autotune else eng.autotune(reps=1)
    eng.step(2)
    steps = 5
    ms = eng.time_steps(steps, L2_FLUSH)
    _, kern = eng.time_steps_detailed(steps, L2_FLUSH)
    # each pass alone on the GPU (per-call entry points, CUDA events around the
    # launch): in the step graph the bonded / nonbond branch shares the SMs
    # with the field pass, so its event interval there is not its own time
    alone = {}
    bonded = lambda timed: eng.bond_force(timed) + eng.angle_force(timed) + eng.dih_force(timed)
    for name, call in (("nonbond", eng.nonbond_force), ("bonded (bond + angle + dihedral calls)", bonded)):
        eng.zero_forces()
        call(True)
        alone[name] = round(min(call(True) for _ in range(3)), 4)
    eng.zero_forces()
    status = eng.device_status()
    eng.close()
    # the optional cutoff mode of the nonbond pass (12 A, skin 2 A) on the same
    # configuration: the first call builds the neighbour list, later calls find
    # no atom moved and run the displacement check and the pairs only
    ec = ig.Engine(s, nonbond_cutoff=12.0)
    ec.zero_forces()
    first = ec.nonbond_force(True)
    steady = min(ec.nonbond_force(True) for _ in range(5))
    cut = {"cutoff_A": 12.0, "skin_A": 2.0, "ms_first_call_with_build": round(first, 4),
           "ms_per_call_without_build": round(steady, 4), "list": ec.nonbond_list_stats(),
           "rows": ec.shapes()["nonbond_list_rows"], "cells": ec.shapes()["nonbond_list_cells"],
           "device_status": ec.device_status()}
    ec.close()
    avg = {k: v[0] / v[1] for k, v in kern.items() if v[1] > 0}
    force_tf = FLOP_FORCE_PAIR * N * P / (avg["force"] * 1e-3) / 1e12
    field_tf = (FLOP_FIELD_PAIR * N * P + FLOP_POINT * P) / (avg["field"] * 1e-3) / 1e12
    return {"workload": "256 x 64-atom chains (16384 atoms), nMC=100 (1.64 M points), 120 A box, charges +-0.8 e",
            "steps": steps, "value": round(N * steps / (ms * 1e-3), 1), "unit": UNIT,
            "ms_per_step": round(ms / steps, 3),
            "ns_per_day": round(ns_per_day(steps / (ms * 1e-3)), 2),
            "kernel_ms_per_launch": {k: round(v, 3) for k, v in avg.items()},
            "kernel_ms_alone": alone,
            "nonbond_alone_tflops": round(FLOP_NB_PAIR * N * (N - 1) / (alone["nonbond"] * 1e-3) / 1e12, 2),
            "nonbond_alone_frac": round(FLOP_NB_PAIR * N * (N - 1) / (alone["nonbond"] * 1e-3) / 1e12 / peak_fp32, 4),
            "nonbond_cutoff_mode": cut,
            "force_kernel_tflops": round(force_tf, 2), "force_kernel_frac": round(force_tf / peak_fp32, 4),
            "field_kernel_tflops": round(field_tf, 2), "field_kernel_frac": round(field_tf / peak_fp32, 4),
            "launch_shapes": shapes, "device_status": status,
            "force_error": "sampled against the FP64 oracle in tests/test_gpu_precision.py"}


def run_adjoint(ig):
    """Differentiation workload: 16 umbrella windows of 550 atoms (nMC 50), the
    adjoint of the window mean forces for one frame (MC points regenerated),
    wall time per call including its host-side set-up."""
    wins = ig.synth.config_adjoint()
    eng = ig.Engine(wins)
    eng.step(3)
    eng.adjoint_mean_force([3])
    reps = 5
    t0 = time.perf_counter()
    for k in range(reps):
        eng.adjoint_mean_force([4 + k])
    dt = (time.perf_counter() - t0) / reps
    status = eng.device_status()
    eng.close()
    return {"workload": "16 windows x 550 atoms (25 x 22-atom chains), nMC=50, 50 A box, r0 5..12 A",
            "ms_per_frame": round(dt * 1e3, 3), "frames_per_s": round(1.0 / dt, 1), "timing": "host wall clock",
            "device_status": status,
            "accuracy": "dJ/dtheta within 4.4e-7 of FP64 central differences (tests/test_gpu_adjoint.py)"}


def run_reference(args):
    """The reference's own CPU path on the host cores: cpu_ispa_force of
    src/isspa_force.omp.c (compiled unmodified) on the 1100-atom system, one
    call per step, at the thread count (up to all host cores) where it runs
    fastest here, W untimed and K timed calls.  Where that file cannot be
    built, the FP64 CPU oracle (a restatement of the reference's CUDA kernels)
    takes its place."""
    import isspa_gb300.synth as synth

    cores = host_cores()
    r, why = ref_omp()
    if r is not None:
        from time_ref_omp import CAVEAT, cpu_model

        best, scan = best_threads(r, cores)
        for _ in range(args.warmup):
            r.call(best)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r.call(best)
        dt = time.perf_counter() - t0
        value = r.n * args.steps / dt
        base = {"value": round(value, 1), "unit": UNIT, "cores": best, "kind": "reference",
                "sample": f"{args.steps} calls of cpu_ispa_force (src/isspa_force.omp.c:11-105, compiled "
                          f"unmodified), 1100 atoms, nMC 50, {best} OpenMP threads: the fastest of a scan over "
                          f"1..{cores} threads on this host ({dt:.2f} s)",
                "threads_scan_atom_steps_per_s": scan, "host_cores": cores,
                "cpu": cpu_model(), "caveat": CAVEAT, "source_sha256": r.source_sha256}
        dtype = "f32"
    else:
        sysm = synth.config_plain(seed=2)
        value, n, dt, cores, _ = cpu_oracle_rate(sysm, budget_s=1e9, min_steps=args.steps, max_steps=args.steps,
                                                 warmup=args.warmup)
        base = {"value": round(value, 1), "unit": UNIT, "cores": cores, "kind": "port",
                "sample": f"{n} full MD steps ({dt:.1f} s) of the FP64 CPU oracle; the reference's OpenMP file "
                          f"is unavailable here ({why})"}
        dtype = "f64"
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": workload_config(), "cpu_baseline": base,
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_variants(args):
    """A/B of the engine's result-preserving variants on each workload, with
    every other launch shape at the autotuner's choice: the three step modes
    (1 branched graph of separate kernels, 2 fused cooperative integrator,
    3 single-kernel cooperative step, the last with split-4 field tiles and
    per-pair loops as it runs them), modes 1 and 2 with the kernel chain
    launched as programmatic dependents, and the field pass's atom staging
    (thread loads against 1-D bulk copies).  Step times are single-step graph
    replays (CUDA events, 256 MB written between steps); back-to-back runs of
    8-step graphs by the host clock; kernel times from the event-instrumented
    step."""
    import build as engine_build
    import isspa_gb300 as ig

    engine_build.build()

    def adi2():
        w = ig.System.from_config(os.path.join(ROOT, "tests", "golden", "adi2_config.txt"))
        w.n_mc = 100
        w.pnu = 0.02
        return w

    cases = [("44 atoms, nMC 20", lambda: ig.synth.config_small(seed=1), 400),
             ("ADI2 44 atoms, nMC 100, 200 A box", adi2, 400),
             ("1100 atoms, nMC 50", lambda: ig.synth.config_plain(seed=2), 400),
             ("64 windows, 41 206 atoms", lambda: ig.synth.config_batched(n_windows=64, seed=4), 60)]
    out = {}
    for name, make, steps in cases:
        system = make()
        e = ig.Engine(system)
        tuned = e.autotune()
        e.close()
        base = {k: int(tuned[k]) for k in ("field_split", "force_chunk", "force_tail_chunk",
                                            "force_atoms_per_thread", "field_vote", "force_vote")}
        base["nonbond_chunk"] = int(tuned["nonbond_partners_per_item"])
        res = {"autotuned": tuned}
        # step_pdl 2: ordinary launches; 1: the field -> force -> leapfrog
        # chain as programmatic dependents (the pair timed twice, interleaved)
        # isspa_fused 1: field and force passes as one launch (field split 4, 8
        # or 16 only; the engine reports 0 where it falls back)
        # force_overlap 1: force items start on stamped field tiles
        runs = [("mode1", 1, 0, 2, 2, 2), ("mode1_pdl", 1, 0, 1, 2, 2), ("mode1_pdl_overlap", 1, 0, 1, 2, 1),
                ("mode1_pdl_fused", 1, 0, 1, 1, 2), ("mode2", 2, 0, 2, 2, 2), ("mode2_pdl", 2, 0, 1, 2, 2),
                ("mode3", 3, 0, 2, 2, 2), ("mode1_field_tma", 1, 1, 2, 2, 2), ("mode1_again", 1, 0, 2, 2, 2),
                ("mode1_pdl_again", 1, 0, 1, 2, 2), ("mode1_pdl_overlap_again", 1, 0, 1, 2, 1),
                ("mode1_pdl_fused_again", 1, 0, 1, 1, 2)]
        for label, mode, tma, pdl, fused, ov in runs:
            o = dict(base, integrator=mode, field_tma=tma, step_pdl=pdl, isspa_fused=fused, force_overlap=ov)
            if mode == 3:
                o.update(field_split=4, field_vote=0, force_vote=0)
            e = ig.Engine(system, **o)
            e.step(20)
            ms = e.time_steps(steps, L2_FLUSH) / steps
            n = 4000 if ms < 0.1 else 200
            e.synchronize()
            t0 = time.perf_counter()
            e.step(n)
            e.synchronize()
            run_ms = (time.perf_counter() - t0) / n * 1e3
            _, kern = e.time_steps_detailed(min(steps, 50), L2_FLUSH)
            res[label] = {"integrator": e.shapes()["integrator"], "field_tma": e.shapes()["field_tma"],
                          "step_pdl": e.shapes()["step_pdl"], "isspa_fused": e.shapes()["isspa_fused"],
                          "force_overlap": e.shapes()["force_overlap"],
                          "step_ms": round(ms, 5), "run_ms_per_step": round(run_ms, 5),
                          "kernel_ms": {k: round(v[0] / v[1], 5) for k, v in kern.items() if v[1]},
                          "device_status": e.device_status()}
            e.close()
        out[name] = res
    print(json.dumps({"variants": out, "timing": "step_ms: single-step graph replays, CUDA events, 256 MB "
                      "written between steps; run_ms_per_step: back-to-back 8-step graphs, host clock"}))


def _cu_profiler(on: bool):
    """cuProfilerStart/Stop of the driver API: with `ncu --profile-from-start
    off` only the launches in between are profiled."""
    import ctypes as C

    drv = C.CDLL("libcuda.so.1")
    rc = drv.cuProfilerStart() if on else drv.cuProfilerStop()
    if rc != 0:
        raise RuntimeError(f"cuProfiler{'Start' if on else 'Stop'} returned {rc}")


def run_profile_case(args):
    """Graph steps of a workload for ncu launch lists and captures: the same
    engine and autotuned launch shapes as the benchmark, then `profile_steps`
    steps inside a cuProfilerStart/Stop range (run ncu with
    --profile-from-start off to skip the autotuner's trial launches)."""
    import build as engine_build
    import isspa_gb300 as ig

    engine_build.build()
    if args.workload == "batched":
        system = ig.synth.config_batched(n_windows=64, seed=4)
    elif args.workload == "precision":
        system = ig.synth.config_precision(seed=3)
    elif args.workload == "small":
        system = ig.synth.config_small(seed=1)
    else:
        system = ig.synth.config_plain(seed=2)
    fixed = None
    if args.shapes_file and os.path.exists(args.shapes_file):
        with open(args.shapes_file) as f:
            fixed = json.load(f)
    if fixed is not None:
        # the shapes an earlier run of this command chose: an ncu run replays them
        # instead of autotuning under the profiler, whose serialised launches
        # would favour other shapes
        eng = ig.Engine(system, field_split=fixed["field_split"], force_chunk=fixed["force_chunk"],
                        force_atoms_per_thread=fixed["force_atoms_per_thread"],
                        force_tail_chunk=fixed["force_tail_chunk"], field_vote=fixed["field_vote"],
                        force_vote=fixed["force_vote"], integrator=fixed["integrator"],
                        nonbond_chunk=fixed["nonbond_partners_per_item"], field_tma=fixed["field_tma"],
                        step_pdl=1 if fixed.setdefault("step_pdl", 0) else 2,
                        isspa_fused=1 if fixed.setdefault("isspa_fused", 0) else 2,
                        force_overlap=1 if fixed.setdefault("force_overlap", 0) else 2)
        shapes = eng.shapes()
        if shapes != fixed:
            raise RuntimeError(f"shapes from {args.shapes_file} not reproduced: {shapes} != {fixed}")
    else:
        eng = ig.Engine(system)
        shapes = eng.shapes() if args.no_autotune else eng.autotune()
        if args.shapes_file:
            with open(args.shapes_file, "w") as f:
                json.dump(shapes, f)
    eng.step(2)
    eng.synchronize()
    _cu_profiler(True)
    eng.step(args.profile_steps)
    eng.synchronize()
    _cu_profiler(False)
    print(json.dumps({"profile_case": args.workload, "steps": args.profile_steps, "atoms": eng.n_atoms,
                      "points": eng.n_points, "launch_shapes": shapes}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="run this many untimed graph steps and exit (profiling case)")
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "precision", "small"])
    ap.add_argument("--shapes-file", default="",
                    help="profiling case: launch shapes to use; written by the autotuner when absent")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the precision-workload and adjoint sections")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--variants", action="store_true",
                    help="A/B the step modes and the field pass's staging on four workloads and exit")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return  # replicas only: the engine runs on one GPU; other ranks do no work
    if args.profile_steps > 0:
        run_profile_case(args)
    elif args.variants:
        run_variants(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
