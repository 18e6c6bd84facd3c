"""Benchmark: EAM atom-steps/s of the GB300 step (mixed precision and plain FP64) on one GPU.

Workload (default): BCC Fe-1.5Cu-1.0Ni, 200^3 unit cells = 16,000,000 atoms, 600 K Maxwell start,
dt = 1 fs, synthetic 3-element setfl table (seeded). A step is one velocity-Verlet loop body of the
reference (firststep, decide, exchanges, computeEam, secondstep) over the whole box.

  value  resident throughput: inputs already in HBM, CUDA events on the library's stream
  e2e    the drop-in path: each step uploads the host slot array (pinned) and downloads it back,
         through mg_step_host
  roofline  the dominant kernel (the force pass) against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (the reference's algorithm restated) on the host cores

--impl reference times the CPU restatement of the reference's path on all host cores instead.
For --gpus N > 1 every rank runs an independent replica (the path's domain decomposition is not
built for several GPUs); value is the sum over ranks, timed as the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EAM atom-steps/s on 1 GB300: mixed-precision & batched vs plain FP64"
UNIT = "atom-steps/s"
# algorithmic bytes per atom-step (whole step: sweep 1 reads x, type, writes df = 33 B; sweep 2
# reads x, type, df, v and writes x, v = 105 B)
BYTES_PER_ATOM_STEP = 138
BYTES_PER_ATOM_FORCE_SWEEP = 105


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="fecuni_200c")
    p.add_argument("--fp64-steps", type=int, default=10)
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cells", type=int, default=0, help="override the workload's unit cells per edge")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--resident-only", action="store_true",
                   help="time only the resident step (no accuracy, FP64, drift, e2e or CPU legs)")
    return p.parse_args()


def dist_init(n):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("MG_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
        return rank, world, dist
    return 0, 1, None


def reduce_max(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, device=None):
    if dist is not None:
        import torch
        if device is not None:
            dist.barrier(device_ids=[device.index]) if device.type == "cuda" else dist.barrier()
        else:
            dist.barrier()


# ------------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
# CPU side: the oracle (the reference's algorithm restated) timed on the host cores
# ------------------------------------------------------------------------------------------------
def _cpu_worker(args):
    cells, n_ele, seed, pot_path, budget_s, cu, ni = args
    from oracle import oracle
    import __graft_entry__ as ge
    wl = ge._package().workloads
    a0, rcf = 2.855, 5.6 / 2.855
    atoms = wl.build_state(cells, a0, rcf, temperature=600.0, seed=seed, cu_frac=cu, ni_frac=ni)
    s = oracle.OracleSim(cells, a0, rcf, pot_path)
    s.set_atoms(atoms)
    s.prepare()
    s.simulate(1)
    steps, elapsed = 0, 0.0
    while elapsed < budget_s:
        elapsed += s.time_simulate(1)
        steps += 1
    return steps * 2 * cells[0] * cells[1] * cells[2], elapsed


def cpu_baseline(workload, pot_path, seconds):
    """P single-threaded oracle processes (P = host cores), each stepping its own replica of a
    bounded sub-box of the workload: the one-rank-per-core arrangement of the reference's MPI runs."""
    from oracle import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    sub = (30, 30, 30)
    ctx = mp.get_context("spawn")
    args = [(sub, workload.n_ele, 100 + r, pot_path, seconds, workload.cu_frac, workload.ni_frac)
            for r in range(cores)]
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, args)
    wall = time.perf_counter() - t0
    atom_steps = sum(r[0] for r in res)
    per_proc = [r[0] / r[1] for r in res]
    value = sum(per_proc)  # every process runs concurrently for ~seconds
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{cores} oracle processes x {sub[0]}^3-cell sub-box ({2 * sub[0]**3} atoms) of the "
                      f"{workload.name} composition, ~{seconds:.0f} s of steps each, FP64, one thread each",
            "wall_s": wall, "atom_steps": atom_steps}


# ------------------------------------------------------------------------------------------------
def run_reference(args):
    rank, world, dist = dist_init(args.gpus)
    if rank != 0:
        return
    import __graft_entry__ as ge
    pkg = ge._package()
    w = pkg.workloads.WORKLOADS[args.workload]
    with tempfile.TemporaryDirectory() as tmp:
        pot = pkg.workloads.workload_potential(w, tmp)
        per_step_s = max(1.0, args.cpu_seconds / max(1, args.steps + args.warmup))
        cb = cpu_baseline(w, pot, max(args.cpu_seconds, per_step_s))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{w.name}: {w.n_atoms} atoms (CPU sample: {cb['sample']})"},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    rank, world, dist = dist_init(args.gpus)
    import torch
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    device = torch.device("cuda", local_rank)
    import __graft_entry__ as ge
    pkg = ge._package()
    pkg.load_library()
    wl = pkg.workloads
    w = wl.WORKLOADS[args.workload]
    if args.cells:
        import dataclasses
        w = dataclasses.replace(w, cells=(args.cells,) * 3, name=f"{w.name}@{args.cells}c")
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    tmp = tempfile.mkdtemp()
    pot = wl.workload_potential(w, tmp)
    t0 = time.perf_counter()
    atoms = wl.workload_state(w, seed=w.seed + rank)
    gen_s = time.perf_counter() - t0
    n_atoms = w.n_atoms

    tuning = {}

    def make_ctx(prec):
        c = pkg.Context(w.cells, w.lattice_const, w.cutoff_radius_factor, precision=prec, device=local_rank)
        c.pot_init_setfl(pot)
        c.set_timestep(w.dt)
        c.upload(atoms)
        c.prepare()
        tuning[prec] = c.autotune(reps=2)  # cached per (box, precision) after the first call
        return c

    # ---- resident ----
    ctx = make_ctx(args.precision)
    ctx.simulate(args.warmup, sync=True)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
    ctx.enable_timing(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.4)
    barrier(dist, device)
    torch.cuda.synchronize()
    ev0.record(stream)
    ctx.simulate(args.steps, sync=False)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier(dist, device)
    clocks = sampler.stop()
    ms_total = ev0.elapsed_time(ev1)
    ms_total = reduce_max(dist, ms_total, device)
    ms_per_step = ms_total / args.steps
    kt = ctx.kernel_times()
    ctx.enable_timing(False)
    thermo = ctx.thermo()
    launches = ctx.launches_per_step() * args.steps
    value = world * n_atoms * args.steps / (ms_total / 1e3)

    force_ms = kt.get("lat_force", float("nan"))
    achieved = BYTES_PER_ATOM_FORCE_SWEEP * n_atoms / (force_ms / 1e3) / 1e9
    step_achieved = BYTES_PER_ATOM_STEP * n_atoms / (ms_per_step / 1e3) / 1e9
    if args.resident_only:
        ctx.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "ms_per_step": ms_per_step, "precision": args.precision, "workload": w.name,
                              "kernel_ms_per_step": kt, "roofline_achieved_gbs": achieved, "clocks": clocks,
                              "tuning": tuning}))
        return

    # ---- accuracy of the mixed form against the FP64 form on the same state ----
    ctx64 = make_ctx("fp64")
    a64, _ = ctx64.download()
    ctxm = make_ctx("mixed")
    am, _ = ctxm.download()
    ctxm.close()
    loc = wl.local_slot_indices(w.cells, w.cutoff_radius_factor)
    d = am["f"][loc] - a64["f"][loc]
    f_rms = float(np.sqrt((d ** 2).mean()))
    f_max = float(np.abs(d).max())
    del a64, am, d

    # ---- plain FP64, resident ----
    ctx64.simulate(2, sync=True)
    s64 = torch.cuda.ExternalStream(ctx64.stream(), device=device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s64)
    ctx64.simulate(args.fp64_steps, sync=False)
    e1.record(s64)
    e1.synchronize()
    ms64 = reduce_max(dist, e0.elapsed_time(e1), device) / args.fp64_steps
    value64 = world * n_atoms / (ms64 / 1e3)
    ctx64.close()

    # ---- energy drift of the mixed form (outside the timed region) ----
    drift = None
    try:
        ctxd = make_ctx("mixed")
        series = []
        for k in range(6):
            th = ctxd.thermo(with_energy=True)
            series.append((k * 20 * w.dt, (th["potential_energy"] + th["kinetic_energy"] * wl.MVV2E) / n_atoms))
            ctxd.simulate(20, sync=True)
        t = np.array([s[0] for s in series])
        e = np.array([s[1] for s in series])
        slope = float(np.polyfit(t, e, 1)[0])
        drift = {"ev_per_atom_per_ps": slope, "span_ps": float(t[-1]), "points": len(t)}
        ctxd.close()
    except Exception as exc:  # keep the bench line even if the drift pass fails
        drift = {"error": str(exc)}

    # ---- end to end through the drop-in call (host slot array, pinned) ----
    host = atoms.copy()
    inter = np.zeros(ctx.n_slots // 100 + 1024, dtype=pkg.ATOM_DTYPE)
    pkg.host_register(host)
    e2e_ctx = make_ctx("mixed")
    n_inter = 0
    e2e_ctx.step_host(host, inter, n_inter, 1)  # warm
    barrier(dist, device)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        n_inter = e2e_ctx.step_host(host, inter, n_inter, 1)
    e2e_s = reduce_max(dist, time.perf_counter() - t0, device)
    pkg.host_unregister(host)
    e2e_ctx.close()
    e2e_value = world * n_atoms * args.e2e_steps / e2e_s
    bytes_io = host.nbytes + n_inter * pkg.ATOM_DTYPE.itemsize

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(w, pot, args.cpu_seconds)

    ctx.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pair/spline terms, compensated f32 sums, f64 state", "data": "synthetic",
        "config": {"workload": f"{w.name}: BCC Fe-1.5at%Cu-1.0at%Ni, {w.cells[0]}^3 unit cells = {n_atoms} atoms, "
                               f"{w.temperature:.0f} K Maxwell start, dt {w.dt * 1000:.0f} fs, synthetic 3-element setfl "
                               f"(nr = nrho = 5000, rc 5.6 A)",
                   "precision": "mixed", "l2": "working set ~1.9 GB > 129 MB L2 (no flush needed)",
                   "parallelism": f"{world} independent replica(s), one per GPU"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                "path": "mg_step_host: pinned host slot array in, one loop body, slot array out"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None,
                     "kernel": "lat_force (mixed)", "kernel_ms": force_ms,
                     "bytes_per_atom": BYTES_PER_ATOM_FORCE_SWEEP, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "step_achieved_gbs": step_achieved, "step_frac": step_achieved / hbm_peak},
        "kernel_ms_per_step": kt,
        "fp64": {"value": value64, "ms_per_step": ms64, "steps": args.fp64_steps},
        "mixed_over_fp64": value / value64,
        "accuracy": {"force_rms_ev_per_A": f_rms, "force_max_ev_per_A": f_max, "reference": "FP64 GPU form",
                     "nve_drift": drift},
        "gpu_launches": launches,
        "tuning": tuning,
        "clocks": clocks,
        "state": {"n_inter": thermo["n_inter"], "device_errors": thermo["device_errors"], "gen_s": gen_s},
    }
    if cb is not None:
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
