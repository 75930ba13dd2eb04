#!/usr/bin/env python
"""Benchmark of the SuLi per-time-step hot path on GB300.

Workload (default): the batched ensemble -- 256 independent sloshing /
dam-break cases, grid dims drawn per axis from U{32..96} (seed 0), advanced
in lockstep by the same launches, mixed precision (FP32 storage and
stencils, FP32 inner passes -- CG preconditioned by a multigrid V-cycle by
default, --precond jacobi for the reference's Jacobi-scaled CG -- inside
FP64 iterative refinement, FP64 sums).  A "step" is one full time step of
every case (1_principal.f90:69-124).

Printed JSON line (rank 0): value = cell-steps/s of the mixed form with all
fields resident in HBM; the plain FP64 form of the same workload is timed
beside it ("fp64"), the e2e figure goes through the C ABI with host
buffers (state uploaded from pinned host memory and read back every step),
the roofline entry is the dominant kernel timed alone over every case
(CUDA events on the library's stream), "accuracy" is the mixed form against
the FP64 form on the 64x32x32 dam break after 200 steps, "output" times
the field records (PRTSCR) of 16 cases and a restart save + load outside
the timed region, "surface_tension" the capillary column with and without
t_tens, "models" the open channel under each visco model (none, Smagorinsky,
k-equation LES, DES), the still-water tank under the projection and the
IPA and the sloshing tank with and without a sponge layer, and cpu_baseline
is the oracle (a port of the reference,
OpenMP where the reference has it) on a bounded sample.

--impl reference times the reference's CPU implementation (the oracle port:
no Fortran compiler exists on either machine) on the same workload: each
step is one time step of one case of the workload (a bounded sample), and
the line reports the same metric, unit and config as this arm.

--gpus N without torchrun starts N ranks itself (torch.distributed.run).
The ensemble is partitioned: an ensemble of 256 x N cases drawn from seed 0,
rank r advancing cases r, r + N, r + 2N, ... (256 per rank) with no
data-path collective; value = all ranks' cell-steps over the slowest rank's
time (weak scaling: the per-GPU work is fixed as N grows).
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
# the headline metric, printed identically by both arms
METRIC = "cell-steps/s, mixed vs FP64 on one GB300 at \u22641e-6 rel L2; CG HBM GB/s"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ensemble",
                    choices=["ensemble", "wave_tank", "dam_break", "k_channel", "open_channel"])
    ap.add_argument("--ncases", type=int, default=256)
    ap.add_argument("--precond", default="multigrid", choices=["multigrid", "jacobi"],
                    help="inner FP32 passes of the mixed form")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-jacobi", action="store_true",
                    help="skip the mixed form with Jacobi-scaled FP32 passes (the precision-only ratio)")
    ap.add_argument("--side-steps", type=int, default=5,
                    help="timed steps of the FP64 and Jacobi legs (at most --steps)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the single-grid configurations (the 512x128x128 open channel with IBM and "
                         "LES, the 1024x256x256 wave tank) timed in both forms")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--profile-kernel", type=int, default=-1,
                    help="profiling mode: after the warm-up steps of the mixed form, one launch of kernel K "
                         "(0 CG matrix-vector, 1 smoother half-sweep, 2 CG update, 3 one-pass smoother sweep) between "
                         "cudaProfilerStart/Stop, for ncu --profile-from-start off; prints its time")
    ap.add_argument("--mms-steps", type=int, default=100,
                    help="steps of the manufactured-solution runs at 32^3, 64^3, 128^3 (0: skip)")
    ap.add_argument("--no-output", action="store_true",
                    help="skip the field-output and restart measurement")
    ap.add_argument("--accuracy-steps", type=int, default=200,
                    help="steps of the dam-break mixed-vs-FP64 accuracy run (0: skip)")
    return ap.parse_args(argv)


# ---------------------------------------------------------------------------
def make_cases(args, precision, rank=0, world=1, precond=None):
    """The cases rank `rank` of `world` advances.  The ensemble is one draw
    of ncases x world cases (seed 0) partitioned round-robin across the
    ranks; the single-grid workloads run as replicas, one per rank."""
    from suli_gb300 import cases
    if args.workload == "ensemble":
        n = args.ncases * world
        cs = ensemble_share(n, rank, world, precision)
        name = "ensemble_%d_U32-96_seed0" % n
    elif args.workload == "wave_tank":
        cs = [cases.wave_tank(precision=precision)]
        name = "wave_tank_1024x256x256"
    elif args.workload == "k_channel":
        cs = [cases.k_channel(256, 64, 128, m_turb=2, precision=precision)]
        name = "k_channel_les_256x64x128"
    elif args.workload == "open_channel":
        cs = [cases.open_channel(512, 128, 128, precision=precision, balanced=True)]
        name = "open_channel_ibm_les_512x128x128"
    else:
        cs = [cases.dam_break(precision=precision)]
        name = "dam_break_64x32x32"
    pc = args.precond if precond is None else precond
    for c in cs:
        c.params.mixed_precond = 1 if pc == "multigrid" else 0
    return name, cs


def ensemble_share(n, rank, world, precision, lo=32, hi=96):
    """Rank `rank`'s share of an n-case ensemble (dims U{lo..hi}, seed 0):
    cases rank, rank + world, rank + 2 world, ... (round-robin, so every rank
    gets the same mix of sizes)."""
    from suli_gb300 import cases
    dims, hcol, amp = cases.ensemble_dims(n, seed=0, lo=lo, hi=hi)
    return [cases.ensemble_case(i, dims, hcol, amp, precision=precision) for i in range(rank, n, world)]


def config_of(args, name, world):
    """The config object both arms print (the two arms' lines compare over it)."""
    return {"workload": name, "cases_per_gpu": args.ncases if args.workload == "ensemble" else 1,
            "l2": "inputs larger than L2 (working set of GBs per GPU)"}


class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
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
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                if isinstance(v, dict):
                    v = v.get("burst", v.get("value"))
                return float(v), "measured"
    except Exception:
        pass
    return FALLBACK_HBM_GBS, "fallback"


def start_gpu(cs):
    from suli_gb300.solver import SuliGPU
    g = SuliGPU([c.params for c in cs])
    g.start([c.fields for c in cs])
    return g


def _nvtx(torch):
    """(push, pop) of torch's NVTX ranges, or no-ops where they are missing."""
    try:
        push, pop = torch.cuda.nvtx.range_push, torch.cuda.nvtx.range_pop
        push("probe")
        pop()
        return push, pop
    except Exception:
        return (lambda name: None), (lambda: None)


def timed_steps(g, k, torch):
    """Time k steps with CUDA events on the library's stream (synchronized on
    both sides), inside an NVTX range "timed_steps" (so a profiler can keep
    to the timed launches: ncu --nvtx --nvtx-include "timed_steps/").  The
    interpreter's cyclic garbage collector runs before, not during, the
    timed steps (each step is a host call: a collection of the bench's
    earlier arrays inside the region would idle the GPU)."""
    s = torch.cuda.ExternalStream(g.stream_handle())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    g.synchronize()
    gc.collect()
    gc.disable()
    try:
        nvtx = _nvtx(torch)
        nvtx[0]("timed_steps")
        e0.record(s)
        g.step(k)
        e1.record(s)
        nvtx[1]()
        g.synchronize()
        e1.synchronize()
    finally:
        gc.enable()
    return e0.elapsed_time(e1)


def job_totals(cells, ms, dist=None, torch=None):
    """Whole-job totals of a weak-scaling run: each rank advanced its own
    ensemble (seed = rank) with no data-path collective, so the job's work is
    the sum of the ranks' cells and its time the slowest rank's."""
    if dist is None:
        return float(cells), float(ms)
    t = torch.tensor([float(cells), float(ms)], dtype=torch.float64)
    c = t[0:1].clone()
    m = t[1:2].clone()
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(c.item()), float(m.item())


def run_form(args, cs, torch, sampler=None, dist=None, steps=None, warmup=None):
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    g = start_gpu(cs)
    g.step(warmup)
    g.synchronize()
    if dist is not None:
        dist.barrier()
    g.profile(True)
    if sampler:
        sampler.start()
    ms = timed_steps(g, steps, torch)
    clocks = sampler.stop() if sampler else None
    prof = g.profile_read()
    cells = sum(c.cells for c in cs)
    job_cells, ms = job_totals(cells, ms, dist, torch)
    g.job_cells = job_cells
    return g, ms, prof, clocks


def rel_l2(a, b):
    n = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / n) if n > 0 else float(np.linalg.norm(a.ravel()))


def compare_forms(gm, g64, ncheck):
    errs = {"velocity": 0.0, "PRD1": 0.0, "LS": 0.0}
    for c in range(ncheck):
        vm = np.concatenate([gm.download(n, c).ravel() for n in ("U", "V", "W")])
        v6 = np.concatenate([g64.download(n, c).ravel() for n in ("U", "V", "W")])
        errs["velocity"] = max(errs["velocity"], rel_l2(vm, v6))
        for n in ("PRD1", "LS"):
            a = gm.download(n, c)[1:-1, 1:-1, 1:-1] if n == "PRD1" else gm.download(n, c)
            b = g64.download(n, c)[1:-1, 1:-1, 1:-1] if n == "PRD1" else g64.download(n, c)
            if n == "PRD1":
                a = a - a.mean()
                b = b - b.mean()
            errs[n] = max(errs[n], rel_l2(a, b))
    return errs


def accuracy_run(args):
    """The mixed form against the plain FP64 form (which matches the oracle
    to 1e-10) on the dam-break configuration: 64x32x32, 200 steps, outside
    any timed region.  Relative L2 after the last step."""
    from suli_gb300 import cases
    from suli_gb300._abi import PREC_FP64, PREC_MIXED
    out = {"workload": "dam_break_64x32x32", "steps": args.accuracy_steps}
    gs = {}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        c = cases.dam_break(64, 32, 32, precision=prec)
        c.params.mixed_precond = 1 if args.precond == "multigrid" else 0
        g = start_gpu([c])
        g.step(args.accuracy_steps)
        g.synchronize()
        gs[name] = g
    errs = compare_forms(gs["mixed"], gs["fp64"], 1)
    for g in gs.values():
        g.close()
    out.update({"rel_l2_" + k: v for k, v in errs.items()})
    return out


def output_run(gm, ncases):
    """The output path outside any timed region: PRTSCR records (t_plot = 1)
    of the first `ncases` cases of the mixed handle (device kernel, one copy
    to pinned memory, file write), and a restart save + load of a 4-case
    mixed batch, into a temporary directory.  Wall time, bytes, GB/s."""
    import shutil
    import tempfile
    from suli_gb300 import cases
    from suli_gb300._abi import PREC_MIXED
    from suli_gb300 import solver
    d = tempfile.mkdtemp(prefix="suli_out_")
    try:
        out = {}
        gm.synchronize()
        t0 = time.perf_counter()
        nbytes = 0
        for c in range(ncases):
            path = os.path.join(d, "campos_%05d" % (10 + c))
            gm.write_fields(path, c, 1)
            nbytes += os.path.getsize(path)
        dt_w = time.perf_counter() - t0
        out["fields"] = {"cases": ncases, "t_plot": 1, "bytes": nbytes, "s": dt_w, "GB_s": nbytes / dt_w / 1e9}
        dims, hcol, amp = cases.ensemble_dims(4, seed=0)
        cs = [cases.ensemble_case(i, dims, hcol, amp, precision=PREC_MIXED) for i in range(4)]
        g = solver.SuliGPU([c.params for c in cs])
        g.start([c.fields for c in cs])
        g.step(1)
        path = os.path.join(d, "restart.bin")
        t0 = time.perf_counter()
        g.restart_save(path)
        dt_s = time.perf_counter() - t0
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        g.restart_load(path)
        dt_l = time.perf_counter() - t0
        g.close()
        out["restart"] = {"cases": 4, "bytes": size, "save_s": dt_s, "load_s": dt_l,
                          "save_GB_s": size / dt_s / 1e9, "load_GB_s": size / dt_l / 1e9}
        out["dir"] = "temporary directory (tmpfs or local disk of the host)"
        return out
    finally:
        shutil.rmtree(d, ignore_errors=True)


def tension_run(torch, steps=10, warmup=3):
    """Surface tension's cost outside the timed region: the capillary column
    (64^3, mixed form) with t_tens = 1 and with t_tens = 0, cell-steps/s."""
    from suli_gb300 import cases
    from suli_gb300._abi import PREC_MIXED
    out = {"workload": "capillary_column_64x64x64", "steps": steps}
    for tens in (1, 0):
        c = cases.capillary_column(64, 64, 0.25, precision=PREC_MIXED)
        c.params.t_tens = tens
        g = start_gpu([c])
        g.step(warmup)
        ms = timed_steps(g, steps, torch)
        g.close()
        out["t_tens_%d" % tens] = {"value": c.cells * steps / (ms / 1e3), "ms_per_step": ms / steps}
    out["overhead"] = out["t_tens_0"]["value"] / out["t_tens_1"]["value"] - 1.0
    return out


def models_run(torch, steps=10, warmup=3):
    """The k-equation model, the implicit pressure algorithm and the sponge
    layer outside the timed region, mixed form, cell-steps/s: the open
    channel (256 x 64 x 128) with m_turb = 0 (none), 1 (Smagorinsky), 2
    (k-equation LES), 3 (DES); the tilted still-water tank (256 x 64 x 128)
    with t_press = 1 (projection, three graddin + posdin per step) and 2
    (IPA: exp_press, one graddin); the sloshing tank (256 x 32 x 128) with
    esp_type = 0, 1, 2."""
    from suli_gb300 import cases
    from suli_gb300._abi import PREC_MIXED
    out = {"k_equation": {"workload": "k_channel_256x64x128", "steps": steps},
           "ipa": {"workload": "ipa_tank_256x64x128", "steps": steps},
           "sponge": {"workload": "sponge_tank_256x32x128", "steps": steps}}
    for m in (0, 1, 2, 3):
        c = cases.k_channel(256, 64, 128, m_turb=max(m, 2), precision=PREC_MIXED)
        c.params.m_turb = m
        if m < 2:
            del c.fields["KA"]
        g = start_gpu([c])
        g.step(warmup)
        ms = timed_steps(g, steps, torch)
        g.close()
        out["k_equation"]["m_turb_%d" % m] = {"value": c.cells * steps / (ms / 1e3), "ms_per_step": ms / steps}
    for tp in (1, 2):
        c = cases.ipa_tank(256, 64, 128, precision=PREC_MIXED)
        c.params.t_press = tp
        if tp == 1:
            del c.fields["PRD0"]
        g = start_gpu([c])
        g.step(warmup)
        ms = timed_steps(g, steps, torch)
        d = g.diag()
        g.close()
        out["ipa"]["t_press_%d" % tp] = {"value": c.cells * steps / (ms / 1e3), "ms_per_step": ms / steps,
                                         "cg_iters_last_step": list(d.cg_iters)}
    for esp in (0, 1, 2):
        c = cases.sponge_tank(256, 32, 128, esp_type=esp, precision=PREC_MIXED)
        g = start_gpu([c])
        g.step(warmup)
        ms = timed_steps(g, steps, torch)
        d = g.diag()
        t0 = time.perf_counter()
        g.complementos()                      # the sponge kernel and the momentum sources alone
        g.synchronize()
        g.close()
        out["sponge"]["esp_type_%d" % esp] = {"value": c.cells * steps / (ms / 1e3), "ms_per_step": ms / steps,
                                              "cg_iters_last_step": list(d.cg_iters),
                                              "complementos_ms_host": (time.perf_counter() - t0) * 1e3}
    return out


def configs_run(args, torch):
    """The two single-grid configurations outside the timed region, each in
    the mixed form and the plain FP64 form on the same initial state (3
    warm-up and a few timed steps each): cell-steps/s of both, their ratio,
    the pressure iterations, and the mixed form's relative L2 difference from
    the FP64 form after the last step (the FP64 form is the one held to the
    oracle at 1e-10 on reduced grids).
      open channel 512 x 128 x 128, 4 x 1 x 1 m, depth 0.6 m, inflow 0.5 m/s
        with a seeded 5 % perturbation, balanced free outflow, IBM cylinder
        D = 0.1 m at x = 1.0, Smagorinsky Cs = 0.1, CG tol 1e-8 relative;
      wave tank 1024 x 256 x 256 (67 M cells), 8 x 2 x 2 m, depth 1.0 m,
        surface 0.05 sin(pi x), still water, Smagorinsky LES, CG tol 1e-8
        relative."""
    from suli_gb300 import cases
    from suli_gb300._abi import PREC_FP64, PREC_MIXED
    builders = {
        "open_channel_ibm_les_512x128x128": (lambda prec: cases.open_channel(512, 128, 128, precision=prec,
                                                                             balanced=True), 5),
        "wave_tank_les_1024x256x256": (lambda prec: cases.wave_tank(precision=prec), 3),
    }
    out = {}
    for name, (make, k) in builders.items():
        row = {"steps": k, "warmup": 3}
        gs = {}
        try:
            for form, prec in (("mixed", PREC_MIXED), ("fp64", PREC_FP64)):
                c = make(prec)
                c.params.mixed_precond = 1 if args.precond == "multigrid" else 0
                g = start_gpu([c])
                g.step(3)
                ms = timed_steps(g, k, torch)
                d = g.diag()
                row[form] = {"value": c.cells * k / (ms / 1e3), "ms_per_step": ms / k,
                             "cg_iters_last_step": list(d.cg_iters), "cg_outer_last_step": list(d.cg_outer)}
                gs[form] = g
            row["mixed_over_fp64"] = row["mixed"]["value"] / row["fp64"]["value"]
            row["mixed_vs_fp64_rel_l2"] = compare_forms(gs["mixed"], gs["fp64"], 1)
        except Exception as e:  # reported, not hidden
            row["error"] = repr(e)
        for g in gs.values():
            g.close()
        out[name] = row
    return out


def mms_run(args):
    """The manufactured solution (13_mms.f90, steady) at 32^3, 64^3, 128^3 in
    both forms, args.mms_steps steps each, outside any timed region: RMS
    error of u, v, w against the analytic fields and the observed order."""
    from suli_gb300 import cases
    from suli_gb300._abi import PREC_FP64, PREC_MIXED
    out = {"steps": args.mms_steps, "errors_uvw": {}}
    for n in (32, 64, 128):
        row = {}
        for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
            c = cases.mms_case(n, precision=prec)
            c.params.mixed_precond = 1 if args.precond == "multigrid" else 0
            g = start_gpu([c])
            g.step(args.mms_steps)
            row[name] = g.mms_error()[:3]
            g.close()
        out["errors_uvw"][str(n)] = row
    e = out["errors_uvw"]
    out["observed_order_u"] = {form: [math.log(e[a][form][0] / e[b][form][0], 2) for a, b in (("32", "64"), ("64", "128"))]
                               for form in ("fp64", "mixed")}
    return out


def e2e_run(args, cs, torch, parts=2):
    """Per step: pinned host state -> device, one step, device -> host, for
    every case.  The cases are dealt round-robin to `parts` handles, each
    driven by its own host thread on its own stream (the library's transfer
    and step calls block only their own handle's stream), so one part's
    transfers run while another part steps (part p starts when part p-1 has
    uploaded its first inputs).  After 3 untimed warm-up steps,
    as the device-timed legs (the autotuner and the step graph are built by
    then)."""
    import threading
    groups = [cs[i::parts] for i in range(parts)]
    gs = [start_gpu(grp) for grp in groups]
    for g in gs:
        g.step(3)
    names = ("U", "V", "W", "LS", "PRD1")
    h2d = 0
    lists = []
    keep = []
    for g, grp in zip(gs, groups):
        items = []
        for c in range(len(grp)):
            for n in names:
                a = g.download(n, c)
                t = torch.empty(a.shape[::-1], dtype=torch.float64).pin_memory()
                pinned = t.numpy().T
                pinned[...] = a
                keep.append(t)
                items.append((n, c, pinned))
                h2d += a.nbytes
        lists.append(items)
        g.synchronize()
    ksteps = max(3, args.steps)
    start = threading.Barrier(parts + 1)
    # part p starts once part p-1 has its first inputs on the device, so the
    # parts' transfers fall in the others' steps from the first step on
    uploaded = [threading.Event() for _ in range(parts)]
    errors = []

    def drive(q, g, items):
        try:
            start.wait()
            if q > 0:
                uploaded[q - 1].wait()
            for s_ in range(ksteps):
                g.upload_many(items)       # every field of every case of the part, one call
                if s_ == 0:
                    uploaded[q].set()
                g.step(1)
                g.download_many(items)
            g.synchronize()
        except Exception as e:             # re-raised by the caller
            errors.append(e)
            uploaded[q].set()

    threads = [threading.Thread(target=drive, args=(q, g, items)) for q, (g, items) in enumerate(zip(gs, lists))]
    for th in threads:
        th.start()
    gc.collect()        # the cyclic collector runs before the timed steps, not in them
    gc.disable()
    try:
        start.wait()
        t0 = time.perf_counter()
        for th in threads:
            th.join()
        dt = time.perf_counter() - t0
    finally:
        gc.enable()
    for g in gs:
        g.close()
    if errors:
        raise errors[0]
    cells = sum(c.cells for c in cs)
    return {"value": cells * ksteps / dt, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": h2d, "steps": ksteps,
            "path": "suli_upload_fields/suli_step/suli_download_fields (C ABI), pinned host buffers; "
                    "the cases in %d handles of their own streams, one host thread each, so one part's "
                    "transfers overlap another's step" % parts}


def _oracle_case(c):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    p = c.params.copy()
    p.precision = 0
    o = pyoracle.Oracle(p)
    for k, v in c.fields.items():
        o.set_field(k, v)
    o.heaviside_init()
    if p.ibm_t == 2 and c.obstacle:
        ob = c.obstacle
        o.obstaculo_cylinder(ob["xc"], ob["yc"], ob["radius"])
        o.ibm_setup()
    for n in (1, 2, 3):
        o.contorno(n)
    return o, p


def cpu_baseline(args, cs, steps=None, warmup=1):
    """The oracle (port of the reference, OpenMP where the reference has it)
    on a bounded sample of the workload: its first case, `warmup` untimed
    steps, then either exactly `steps` timed steps or, when steps is None,
    steps until ~cpu_seconds of work have been done.  Wall time per step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    pyoracle.Oracle.set_threads(cores)
    c = cs[0]
    o, p = _oracle_case(c)
    o.step(max(1, warmup))
    n = 0
    t0 = time.perf_counter()
    while True:
        o.step(1)
        n += 1
        if steps is not None:
            if n >= steps:
                break
        elif time.perf_counter() - t0 > args.cpu_seconds or n >= 50:
            break
    dt = time.perf_counter() - t0
    return {"value": c.cells * n / dt, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": "%s: %d steps of one %dx%dx%d case after %d untimed, FP64 oracle, OpenMP in CG/interp "
                      "as upstream" % (c.name, n, p.nx, p.ny, p.nz, max(1, warmup)),
            "steps": n, "ms_per_step": dt * 1e3 / n}


def side_legs(args, torch, dist, rank, world, value):
    """The plain FP64 form and the mixed form with Jacobi-scaled FP32 passes
    (the reference's own CG in FP32 inside FP64 refinement) on the same
    workload: the FP64 form's speed, mixed over FP64 (multigrid passes: the
    precision change plus the preconditioner) and mixed-Jacobi over FP64
    (the precision change alone)."""
    from suli_gb300._abi import PREC_FP64, PREC_MIXED
    out = {}
    k = max(1, min(args.side_steps, args.steps))
    legs = []
    if not args.no_fp64:
        legs.append(("fp64", PREC_FP64, args.precond))
    if not args.no_jacobi and args.precond == "multigrid":
        legs.append(("mixed_jacobi", PREC_MIXED, "jacobi"))
    for key, prec, pc in legs:
        try:
            _, cs = make_cases(args, prec, rank, world, precond=pc)
            g, ms, prof, _ = run_form(args, cs, torch, None, dist, steps=k, warmup=3)
            v = g.job_cells * k / (ms / 1e3)
            leg = {"value": v, "ms_per_step": ms / k, "steps": k, "gpu_launches": int(prof.launches),
                   "cg_iters_case0": list(g.diag(0).cg_iters)}
            if key == "fp64":
                leg["cg_GBs_algorithmic"] = (7 * 8.0 * prof.cg_cell_iters / (prof.cg_ms / 1e3) / 1e9
                                             if prof.cg_ms > 0 else None)
            out[key] = (leg, g)
        except Exception as e:  # reported, not hidden
            out[key] = ({"error": repr(e)}, None)
    return out


# ---------------------------------------------------------------------------
def relaunch_distributed(args):
    """--gpus N > 1 without torchrun: start N ranks (one per GPU) through
    torch.distributed.run on 127.0.0.1 and return its exit code."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def reference_arm(args, rank, world):
    """--impl reference: the oracle port on this host's cores, on the same
    metric, unit and config as this arm; each step one time step of the
    workload's first case (rank 0 only)."""
    from suli_gb300._abi import PREC_FP64
    if rank != 0:
        return
    name, cs = make_cases(args, PREC_FP64, 0, world)
    res = cpu_baseline(args, cs, steps=args.steps, warmup=args.warmup)
    line = {"metric": METRIC, "value": res["value"], "unit": "cell-steps/s", "n_gpus": world,
            "steps": res["steps"], "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": config_of(args, name, world),
            "e2e": {"value": res["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "cpu_baseline": {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "note": "the reference Fortran cannot be built (no Fortran compiler on either machine): its "
                    "line-faithful C restatement runs instead (bit-identical to the reference's own "
                    "routines on the golden cases of tests/golden/), compiled -O3 with OpenMP where the "
                    "reference has it; a step is one time step of one case of the workload, so "
                    "ms_per_step is per case-step"}
    print(json.dumps(line))


def main():
    args = parse()
    assert args.warmup >= 3 or args.impl == "reference", "at least 3 warm-up steps"
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_distributed(args))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    from suli_gb300._abi import PREC_MIXED

    if args.impl == "reference":
        reference_arm(args, rank, world)
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    from suli_gb300 import build
    build.build()
    from suli_gb300 import solver
    sms, devname = solver.device_info()

    name, cs_m = make_cases(args, PREC_MIXED, rank, world)
    cells = sum(c.cells for c in cs_m)
    if args.profile_kernel >= 0:
        g = start_gpu(cs_m)
        g.step(args.warmup)
        g.time_kernel(args.profile_kernel, 2)      # untimed: tables and caches warm
        g.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
        g.time_kernel(args.profile_kernel, 1)
        torch.cuda.cudart().cudaProfilerStop()
        ms, by = g.time_kernel(args.profile_kernel, 20)
        g.close()
        print(json.dumps({"profile_kernel": args.profile_kernel, "workload": name, "cells": cells,
                          "ms_per_launch": ms, "algorithmic_bytes_per_launch": by,
                          "GBs": by / (ms / 1e3) / 1e9, "timing": "20 launches between CUDA events"}))
        return
    sampler = ClockSampler(local) if rank == 0 else None
    gm, ms_m, prof_m, clocks = run_form(args, cs_m, torch, sampler, dist)
    value = gm.job_cells * args.steps / (ms_m / 1e3)
    peak, peak_src = measured_peak_hbm()
    line = {
        "metric": METRIC,
        "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_m / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": config_of(args, name, world),
        "e2e": None, "roofline": None, "cpu_baseline": None,
        "fp64": None, "mixed_over_fp64": None, "mixed_jacobi": None, "mixed_jacobi_over_fp64": None,
        "gpu_launches": int(prof_m.launches),
        "clocks": clocks,
        "run": {"cases": len(cs_m), "cells_per_gpu": cells, "precision": "mixed",
                "mixed_passes": "FP32 CG preconditioned by a multigrid V-cycle" if args.precond == "multigrid"
                else "FP32 Jacobi-scaled CG",
                "working_set_GB": cells * 4 * 46 / 1e9, "device": devname, "sms": sms,
                "partition": "cases r, r+N, ... of one ensemble on rank r" if args.workload == "ensemble"
                else "replicas"},
    }
    # roofline of the dominant kernel, timed alone over every case of the
    # workload with CUDA events on the library's stream (burst peak)
    if args.precond == "multigrid":
        kern = 1 if os.environ.get("SULI_MG_FUSED") == "0" else 3
    else:
        kern = 0
    kname = {0: "k_cgi_A (CG matrix-vector product + p.Ap)",
             1: "k_mg_smooth on the case grid (one red-black half-sweep)",
             3: "k_mg_sweep on the case grid (one whole red-black sweep in one pass)"}[kern]
    ms_k, bytes_k = gm.time_kernel(kern, 20)
    ach = bytes_k / (ms_k / 1e3) / 1e9
    # DRAM bytes per cell of one launch (dram__bytes_read.sum +
    # dram__bytes_write.sum over cells) from an ncu capture of the same
    # kernel on the first 24 cases of this ensemble; times this workload's cells
    traffic_per_cell = {0: 166.6e6 / 6914626, 1: 233.2e6 / 6914626, 3: 218.0e6 / 6914626}[kern]
    line["roofline"] = {"bound": "hbm", "kernel": kname, "achieved": ach, "peak": peak, "unit": "GB/s",
                        "frac": ach / peak,
                        "traffic": traffic_per_cell * cells if traffic_per_cell is not None else None,
                        "traffic_source": "ncu capture on the 24-case ensemble, bytes per cell x cells",
                        "peak_source": peak_src,
                        "algorithmic_bytes_per_launch": bytes_k, "ms_per_launch": ms_k,
                        "timing": "kernel alone, 20 launches between CUDA events, all cases of the workload"}
    ms_a, bytes_a = gm.time_kernel(0, 20)
    line["roofline_cg_matvec"] = {"kernel": "k_cgi_A", "achieved": bytes_a / (ms_a / 1e3) / 1e9,
                                  "ms_per_launch": ms_a, "algorithmic_bytes_per_launch": bytes_a}
    line["cg_loop"] = {"cell_iters": prof_m.cg_cell_iters, "ms": prof_m.cg_ms}
    tun = gm.tuning()
    tun["gain"] = tun["default_ms"] / tun["tuned_ms"] if tun["tuned_ms"] > 0 else None
    tun["timed"] = "one convdiff, one V-cycle and one level-0 sweep over every case, defaults vs chosen shapes"
    line["autotune"] = tun
    diag = gm.diag(0)
    line["cg_iters_case0"] = list(diag.cg_iters)
    line["cg_outer_case0"] = list(diag.cg_outer)
    legs = side_legs(args, torch, dist, rank, world, value)
    g64 = None
    if "fp64" in legs:
        line["fp64"], g64 = legs["fp64"]
        if g64 is not None:
            line["mixed_over_fp64"] = value / line["fp64"]["value"]
            line["mixed_vs_fp64_rel_l2"] = compare_forms(gm, g64, min(4, len(cs_m)))
    if "mixed_jacobi" in legs:
        line["mixed_jacobi"], gj = legs["mixed_jacobi"]
        if gj is not None:
            if g64 is not None:
                line["mixed_jacobi_over_fp64"] = line["mixed_jacobi"]["value"] / line["fp64"]["value"]
                line["mixed_jacobi_vs_fp64_rel_l2"] = compare_forms(gj, g64, min(4, len(cs_m)))
            gj.close()
    if g64 is not None:
        g64.close()
    if rank == 0 and not args.no_output:
        try:
            line["output"] = output_run(gm, min(16, len(cs_m)))
        except Exception as e:
            line["output"] = {"error": repr(e)}
        try:
            line["surface_tension"] = tension_run(torch)
        except Exception as e:
            line["surface_tension"] = {"error": repr(e)}
        try:
            line["models"] = models_run(torch)
        except Exception as e:
            line["models"] = {"error": repr(e)}
    gm.close()
    if rank == 0 and not args.no_configs:
        try:
            line["configs"] = configs_run(args, torch)
        except Exception as e:
            line["configs"] = {"error": repr(e)}
    if args.accuracy_steps > 0 and rank == 0:
        try:
            line["accuracy"] = accuracy_run(args)
        except Exception as e:
            line["accuracy"] = {"error": repr(e)}
    if args.mms_steps > 0 and rank == 0:
        try:
            line["mms"] = mms_run(args)
        except Exception as e:
            line["mms"] = {"error": repr(e)}
    if not args.no_e2e:
        try:
            line["e2e"] = e2e_run(args, cs_m, torch)
        except Exception as e:
            line["e2e"] = {"error": repr(e)}
    if rank == 0 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(args, cs_m)
        except Exception as e:
            line["cpu_baseline"] = {"error": repr(e)}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
