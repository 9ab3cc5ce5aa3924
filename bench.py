"""Throughput benchmark of the per-level advance on GB300.

One step = one advance of the whole level (all cells), with the next step's
CFL bound fused in; K timed steps follow W untimed warm-up steps.  Workload:
a seeded 8192 x 8192 FP64 fractal-terrain circular dam break (hydrostatic-Roe,
MUSCL van Leer, 20% NODATA, walls).  The inputs (4.3 GB) exceed the 129 MB L2,
so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: one process per GPU under torchrun, each advancing its own replica
(the level does not shard across GPUs here: replicas only, weak scaling);
value = all cells updated by all ranks / max over ranks of the timed region.

--impl reference times the reference's arithmetic on the host cores: the
reference itself cannot be built on this machine (it needs AMReX, MPI and
HDF5), so the oracle's OpenMP restatement of the same per-box arithmetic runs
instead, on a bounded sample of the workload per step.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "FP64 Mcell-updates/s (plain vs batched, 1 GB300, %HBM roofline); adjoint/fwd cost"
UNIT = "Mcell-updates/s"
PEAKS = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
HBM_GBS = float(PEAKS.get("hbm_gbs", 6800.0))
HBM_SRC = "measured" if "hbm_gbs" in PEAKS else "fallback"
# FP64 issue roof: the DFMA rate is measured on the GPU at the start of the run
# (hx_measure_fp64_rate); this GB300 figure (0.597 T inst/s) is the fallback.
FP64_DFMA_PER_S = 0.597e12
FP64_SRC = "GB300 figure measured earlier (fallback)"
BYTES_PER_CELL = {"f64": 64, "f32": 32}  # read h hu hv z n, write h hu hv
NX = NY = 8192


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_case(nx, ny):
    from hydroexa_gb300 import workloads
    return workloads.fractal_dam_break(nx, ny, seed=3)


class CpuLevel:
    """The oracle's OpenMP time loop (all host threads) on the whole level:
    library, level descriptor and state copies are prepared here, outside any
    timed region; ``steps(k)`` then advances the state in place (per step the
    CFL reduction and one advance, as the reference's time loop does)."""

    def __init__(self, case, method):
        import numpy as np
        import oracle
        oracle.build()
        self.oracle = oracle
        self.case = case
        self.method = method
        g = case.geom
        self.L = oracle.Level(g.nx, g.ny, g.dx, g.dy, g.bc_lo, g.bc_hi)
        self.st = [np.array(a, dtype=np.float64, order="C", copy=True) for a in (case.h, case.hu, case.hv)]
        self.z = np.ascontiguousarray(case.z, dtype=np.float64)
        self.n = np.ascontiguousarray(case.n, dtype=np.float64)
        self.threads = oracle.max_threads()
        self.cells = g.nx * g.ny

    def steps(self, k):
        r = self.oracle.run(self.L, self.method, *self.st, self.z, self.n, k, self.case.cfl, copy=False)
        assert r[5] == 0, "oracle time loop stopped (dt collapse)"


def cpu_sample(case, method=1, budget_s=12.0):
    """A bounded sample of the CPU time loop on the whole level: one untimed
    step, then as many steps as fit in ~budget_s (2 to 20)."""
    cpu = CpuLevel(case, method)
    t0 = time.perf_counter()
    cpu.steps(1)
    t1 = time.perf_counter() - t0
    k = max(2, min(20, int(budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    cpu.steps(k)
    el = time.perf_counter() - t0
    g = case.geom
    return {"value": cpu.cells * k / el / 1e6, "unit": UNIT, "cores": cpu.threads, "kind": "port",
            "sample": f"oracle OpenMP restatement (not the reference binary): {k} steps of the whole "
                      f"{g.nx}x{g.ny} level, {el:.1f} s"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    case = make_case(NX, NY)
    cpu = CpuLevel(case, 1)  # set-up (build, copies, level descriptor) outside the timed region
    cpu.steps(args.warmup)
    t0 = time.perf_counter()
    cpu.steps(args.steps)
    el = time.perf_counter() - t0
    value = cpu.cells * args.steps / el / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu.threads, "kind": "port",
                         "sample": "%d steps (after %d untimed) of the whole %dx%d level: per step the CFL reduction "
                                   "and one hydrostatic-Roe advance; oracle OpenMP restatement of the reference's "
                                   "per-box arithmetic (the reference needs AMReX/MPI/HDF5 and cannot be built "
                                   "here)" % (args.steps, args.warmup, NX, NY)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def config_dict():
    return {"workload": "fractal-terrain circular dam break 8192x8192 FP64, hydrostatic-Roe MUSCL van Leer, "
                        "20% NODATA, reflective walls",
            "nx": NX, "ny": NY, "method": "HydrostaticRoe", "precision": "FP64",
            "l2": "no flush: 4.3 GB of inputs per step > 129 MB L2", "seed": 3}


def main():
    global NX, NY
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"])
    ap.add_argument("--size", type=int, default=NX, help="level side (default 8192)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"])
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--ensemble-count", type=int, default=256, help="ensemble members (default 256)")
    ap.add_argument("--adjoint-steps", type=int, default=2000, help="adjoint run length (default 2000)")
    ap.add_argument("--method", default="hydrostatic", choices=["hydrostatic", "roe"])
    ap.add_argument("--details", default=str(ROOT / "_build" / "bench_details.json"),
                    help="file for the full ensemble and adjoint tables (the JSON line carries their summaries)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    NX = NY = args.size
    if args.impl == "reference":
        return run_reference(args)

    import ctypes
    import numpy as np
    import torch

    import hydroexa_gb300
    from hydroexa_gb300 import capi, ranks
    from hydroexa_gb300.level import DtAccum, Level

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    hydroexa_gb300.build()
    global FP64_DFMA_PER_S, FP64_SRC
    FP64_DFMA_PER_S = capi.fp64_rates()[0]
    FP64_SRC = "measured in this run (hx_measure_fp64_rate)"
    arith = capi.HX_ARITH_FAST if args.arith == "fast" else capi.HX_ARITH_EXACT
    case = make_case(NX, NY)
    cells = NX * NY
    dtype = torch.float64 if args.precision == "f64" else torch.float32
    if args.method == "roe":
        # the classic solver has no NODATA wall: time it on the same terrain without the NODATA mask
        from hydroexa_gb300 import workloads
        case = workloads.fractal_dam_break(NX, NY, seed=3, nodata_frac=0.0)
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, dtype=dtype, device=dev)
    stream = torch.cuda.current_stream(dev)
    method = capi.HX_METHOD_HYDROSTATIC_ROE if args.method == "hydrostatic" else capi.HX_METHOD_ROE

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # ---- warm-up
    assert lev.run(method, args.warmup, case.cfl, arith=arith) == 0
    # ---- timed: K steps, one advance kernel each (+ the initial CFL pass)
    barrier()
    n0 = capi.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        lev.run(method, args.steps, case.cfl, arith=arith, check_status=False)
        e1.record(stream)
        e1.synchronize()
    barrier()
    launches = capi.launch_count() - n0
    status = lev.status.read()
    assert status == 0, f"device status {status}"
    ms = ranks.reduce_real_max([e0.elapsed_time(e1)])[0]  # the slowest rank's time
    value = ws * cells * args.steps / (ms * 1e-3) / 1e6

    # ---- dominant kernel: per-launch duration with events on its stream
    acc_out = torch.empty_like(lev.state)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * 5)]
    dt = 0.5 * lev.compute_dt()[0] * case.cfl
    nxt = DtAccum(dev)  # the loop's kernel: the next step's CFL bound folded in
    for k in range(5):
        ev[2 * k].record(stream)
        lev.advance(method, dt, out=acc_out, next_dt=nxt, arith=arith)
        ev[2 * k + 1].record(stream)
    torch.cuda.synchronize(dev)
    kms = statistics.mean(ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(5))
    achieved_gbs = BYTES_PER_CELL[args.precision] * cells / (kms * 1e-3) / 1e9
    profile = load_profile_summary()
    epi = None
    if args.method == "hydrostatic":
        epi = epilogue_measure(lev, dt, acc_out, arith, stream)

    # ---- end to end through the host-buffer C-ABI call (pinned host memory)
    e2e = None
    if args.precision == "f64":  # every rank times its own replica end to end (the host-buffer call is FP64)
        pin = [torch.from_numpy(a.copy()).pin_memory() for a in (case.h, case.hu, case.hv, case.z, case.n)]
        P = [ctypes.c_void_p(t.data_ptr()) for t in pin]
        lo = (ctypes.c_int32 * 2)(*case.geom.bc_lo)
        hi = (ctypes.c_int32 * 2)(*case.geom.bc_hi)
        tout = ctypes.c_double()
        sh = ctypes.c_void_p(stream.cuda_stream)
        L = capi.lib()

        def e2e_step():
            rc = L.hx_level_run_host_f64(method, NX, NY, case.geom.dx, case.geom.dy, lo, hi, P[0], P[1], P[2], P[3],
                                         P[4], 1, case.cfl, arith, ctypes.byref(tout), sh)
            assert rc == 0, rc
        for _ in range(2):
            e2e_step()
        # enough calls (~1 s) that one call slowed by the host does not set the figure; no collection of
        # Python garbage between the calls (the host thread issues each call's work)
        ke = max(3, min(2 * args.steps, 40))
        barrier()
        marks = [torch.cuda.Event(enable_timing=True) for _ in range(ke + 1)]
        gc.disable()
        marks[0].record(stream)
        for k in range(ke):
            e2e_step()
            marks[k + 1].record(stream)
        marks[-1].synchronize()
        gc.enable()
        ems = ranks.reduce_real_max([marks[0].elapsed_time(marks[-1])])[0]
        calls = sorted(marks[k].elapsed_time(marks[k + 1]) for k in range(ke))
        L.hx_host_cache_release()
        e2e = {"value": ws * cells * ke / (ems * 1e-3) / 1e6, "unit": UNIT, "h2d_bytes_per_step": 40 * cells,
               "d2h_bytes_per_step": 24 * cells + 12, "steps": ke,
               "call": "hx_level_run_host_f64 (host buffers in/out, one step per call)",
               # the spread of the calls (each includes its host copies, whose rate varies with the host)
               "ms_per_call": {"min": calls[0], "median": calls[len(calls) // 2], "max": calls[-1]}}

    # the exact arithmetic form on the same level (bit-equal to the oracle and to the reference's drivers),
    # a few steps: its rate beside the fast form's headline
    exact = None
    if args.arith == "fast":
        xs = 5
        assert lev.run(method, 1, case.cfl, arith=capi.HX_ARITH_EXACT) == 0  # warm-up
        barrier()
        x0 = torch.cuda.Event(enable_timing=True)
        x1 = torch.cuda.Event(enable_timing=True)
        x0.record(stream)
        lev.run(method, xs, case.cfl, arith=capi.HX_ARITH_EXACT, check_status=False)
        x1.record(stream)
        x1.synchronize()
        xms = ranks.reduce_real_max([x0.elapsed_time(x1)])[0]
        exact = {"value": ws * cells * xs / (xms * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": xms / xs, "steps": xs,
                 "what": "HX_ARITH_EXACT: the reference's operation order, no multiply-add contraction"}

    ens = None
    if args.precision == "f64" and args.method == "hydrostatic" and not args.no_ensemble:
        del lev
        torch.cuda.empty_cache()
        ens = ensemble_measure(dev, count=args.ensemble_count)

    adj = None
    if args.precision == "f64" and args.method == "hydrostatic" and not args.no_adjoint:
        torch.cuda.empty_cache()
        adj = adjoint_measure(dev, nsteps=args.adjoint_steps)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(case, method=method)

    if rank == 0:
        pipe = (fp64_pipe(profile, kms) if (args.precision, args.method, args.arith) == ("f64", "hydrostatic", "fast")
                and cells >= 1 << 22 else None)
        if ens is not None or adj is not None:
            Path(args.details).parent.mkdir(parents=True, exist_ok=True)
            Path(args.details).write_text(json.dumps({"ensemble": ens, "adjoint": adj}, indent=1))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": args.precision, "data": "synthetic (seeded fractal terrain; no dataset)",
            "fp64_pipe_frac": pipe["frac"] if pipe else None,
            "ensemble": ensemble_summary(ens),
            "adjoint": adjoint_summary(adj),
            "epilogue": epi,
            "exact_form": exact,
            "details_file": args.details if (ens is not None or adj is not None) else None,
            "config": dict(config_dict(), arith=args.arith, nx=NX, ny=NY, precision=args.precision.upper(),
                           method={"hydrostatic": "HydrostaticRoe", "roe": "Roe (no NODATA)"}[args.method]),
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {
                "bound": "hbm", "achieved": achieved_gbs, "peak": HBM_GBS, "unit": "GB/s",
                "frac": achieved_gbs / HBM_GBS, "traffic": profiled_traffic(profile, cells, args),
                "peak_source": HBM_SRC,
                "kernel": dominant_kernel(args, arith, cells),
                "kernel_ms": kms, "algorithmic_bytes_per_launch": BYTES_PER_CELL[args.precision] * cells,
                "note": "FP64-issue bound on GB300: see fp64_pipe",
                "fp64_pipe": pipe,
            },
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def epilogue_measure(lev, dt, out, arith, stream, reps=5):
    """The step with its epilogue (eta = h + z and the conservation diagnostics
    written by the update) against the plain step followed by the separate eta
    and diagnostics passes, one launch sequence at a time with events on the
    launching stream.  Inputs larger than L2 (8192^2 x 5 planes)."""
    import ctypes

    import torch

    from hydroexa_gb300 import capi
    from hydroexa_gb300.level import array4, box
    L = capi.lib()
    g = lev.geom
    b = box((0, 0), (g.nx - 1, g.ny - 1))
    eta = torch.empty_like(lev.state[0])
    diag = torch.empty(5, dtype=torch.float64, device=lev.state.device)
    work = torch.empty(int(L.hx_diagnostics_work_bytes(b)), dtype=torch.uint8, device=lev.state.device)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    sfx = lev.sfx
    d_out = lev._desc(out)
    T, O, E = array4(lev.terrain), array4(out), array4(eta)
    sh = ctypes.c_void_p(stream.cuda_stream)

    def fused():
        lev.advance_epilogue(dt, out=out, arith=arith, stream=stream)

    def separate():
        lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, out=out, arith=arith, stream=stream)
        capi.check(getattr(L, "hx_derive_eta_box_" + sfx)(ctypes.byref(O), ctypes.byref(T), ctypes.byref(E), b, sh))
        if sfx == "f64":
            capi.check(L.hx_level_diagnostics_f64(ctypes.byref(d_out), vp(diag), vp(work), sh))
        else:
            Rt = ctypes.c_float
            capi.check(L.hx_diagnostics_box_f32(ctypes.byref(O), ctypes.byref(T), b, Rt(g.dx), Rt(g.dy), vp(diag),
                                                vp(work), sh))

    def timed(fn):
        fn()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps)]
        for k in range(reps):
            ev[2 * k].record(stream)
            fn()
            ev[2 * k + 1].record(stream)
        torch.cuda.synchronize(lev.state.device)
        return statistics.mean(ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(reps))

    def plain():
        lev.advance(capi.HX_METHOD_HYDROSTATIC_ROE, dt, out=out, arith=arith, stream=stream)

    p_ms, f_ms, s_ms = timed(plain), timed(fused), timed(separate)
    return {"fused_ms": f_ms, "separate_ms": s_ms, "plain_step_ms": p_ms,
            "fused_over_plain": f_ms / p_ms - 1.0, "separate_over_plain": s_ms / p_ms - 1.0,
            "what": "step + eta (DeriveEtaFrom) + mass/momentum/KE/min-h diagnostics: fused into the update "
                    "(hx_level_advance_epilogue) vs the plain step then the two separate passes"}


def ensemble_measure(dev, steps=24, warmup=6, plain_steps=6, count=256):
    """256 independent dam breaks, sides log-uniform in
    [64, 1024].  Batched (one persistent launch per step, CUDA graph, tile shape
    per size class from the autotuner) against the members advanced one after
    another, (a) with the per-level device time loop and (b) with the
    reference's per-step host read of the CFL bound.  A bounded sample of the
    500-step runs: `steps` (multiple of 6) timed steps after `warmup`."""
    import torch

    from hydroexa_gb300 import capi, workloads
    from hydroexa_gb300.ensemble import SHAPE_NAMES, Ensemble, autotune

    cases = workloads.ensemble(count=count, seed=4)
    cells = sum(c.cells for c in cases)
    cfl = cases[0].cfl
    per_class, report = autotune(cases, device=dev, steps=6)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3

    ens = Ensemble(cases, device=dev)
    ens.set_shapes_by_class(per_class)
    assert all(x == 0 for x in ens.run(warmup, cfl))
    n0 = capi.launch_count()
    t_b = timed(lambda: ens.run(steps, cfl, check_status=False))
    launches = capi.launch_count() - n0
    assert all(x == 0 for x in ens.status.cpu().tolist())
    del ens
    ref = Ensemble(cases, device=dev)
    ref.member_loop(1, cfl)
    t_m = timed(lambda: ref.member_loop(steps, cfl))
    ref.plain_loop(1, cfl)
    t_p = timed(lambda: ref.plain_loop(plain_steps, cfl))
    del ref
    v_b = cells * steps / t_b / 1e6
    v_m = cells * steps / t_m / 1e6
    v_p = cells * plain_steps / t_p / 1e6
    return {"workload": "%d independent FP64 dam breaks (hydrostatic-Roe), sides log-uniform in [64,1024] (seed 4), "
                        "%d cells, %d timed steps per member (sample of the 500-step runs)" % (count, cells, steps),
            "batched": v_b, "member_loop": v_m, "plain_loop_host_dt": v_p, "unit": UNIT,
            "speedup_vs_member_loop": v_b / v_m, "speedup_vs_plain_loop": v_b / v_p,
            "batched_launches": launches,
            "tile_shape_per_class": [SHAPE_NAMES[x] for x in per_class],
            "class_edges": [128, 384]}


def adjoint_measure(dev, nsteps=2000, every=45, fd_eps=1e-6):
    """Gauge-misfit gradient of a 512x512 FP64 hydrostatic-Roe run of 2000
    steps (smooth bed of 32 Gaussians, 0.2 m hump, 64 gauges, reference series
    from a run on a perturbed bed), checkpoints every 45 steps.  Reports the
    forward+reverse cost against the plain forward time loop of the same steps,
    the working set with and without checkpoints, the gradient against the
    N-step tangent-linear model (exact arithmetic, same trajectory), and
    central-difference directional checks (steps 1e-6 and 1e-7) of this run
    and of a smooth, non-quiescent variant over growing horizons."""
    import numpy as np
    import torch

    from hydroexa_gb300 import capi, workloads
    from hydroexa_gb300.adjoint import GaugeProblem, tangent_misfit
    from hydroexa_gb300.level import Level

    case, gauges = workloads.adjoint_case(nsteps=nsteps)
    g = case.geom
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    z, h0, zero = T(case.z), T(case.h), torch.zeros((g.ny, g.nx), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3, out

    lev = Level.from_numpy(g, case.h, case.hu, case.hv, case.z, case.n, device=dev)
    lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, 20, case.cfl, arith=capi.HX_ARITH_FAST)
    lev = Level.from_numpy(g, case.h, case.hu, case.hv, case.z, case.n, device=dev)
    t_plain, _ = timed(lambda: lev.run(capi.HX_METHOD_HYDROSTATIC_ROE, nsteps, case.cfl, arith=capi.HX_ARITH_FAST,
                                       check_status=False))
    assert lev.status.read() == 0
    del lev
    prob = GaugeProblem(g, zero.clone(), gauges, nsteps, case.cfl, checkpoint_every=every)
    dz = T(workloads.smooth_field(g.nx, g.ny, seed=6, amplitude=0.02))
    href = prob.forward(z + dz, h0, zero, zero).clone()
    prob.forward(z, h0, zero, zero)  # warm-up
    prob.reverse(href)
    t_fwd, series = timed(lambda: prob.forward(z, h0, zero, zero))
    n0 = capi.launch_count()
    t_rev, grads = timed(lambda: prob.reverse(href))
    rev_launches = capi.launch_count() - n0
    prob_bytes = prob.work_bytes
    J0 = float(((series - href) ** 2).sum())

    def fd_check(prob, base, href, grads, seeds, nx, ny, steps=(fd_eps, fd_eps / 10)):
        out = {}
        for name, k, seed in seeds:
            d = T(workloads.smooth_field(nx, ny, seed=seed, amplitude=1.0))
            ad = float((grads[k] * d).sum())
            rec = {"adjoint": ad}
            for eps in steps:
                plus, minus = list(base), list(base)
                plus[k] = base[k] + eps * d
                minus[k] = base[k] - eps * d
                jp = float(((prob.forward(*plus) - href) ** 2).sum())
                jm = float(((prob.forward(*minus) - href) ** 2).sum())
                fdv = (jp - jm) / (2 * eps)
                rec["step_%g" % eps] = {"central_difference": fdv, "rel_err": abs(ad - fdv) / max(abs(fdv), 1e-300)}
            rec["best_rel_err"] = min(v["rel_err"] for key, v in rec.items() if key.startswith("step_"))
            out[name] = rec
        return out

    fd = fd_check(prob, [z, h0, zero, zero], href, grads, (("z", 0, 7), ("h0", 1, 8)), g.nx, g.ny)
    face_records = bool(prob.options & capi.HX_ADJ_FACE_RECORDS)

    def max_rel_diff(ga, gb):
        """Largest |a - b| / max|b| over the four gradient planes (the record
        path differs from recomputation in the last bits only)."""
        return max(float((a - b).abs().max()) / max(float(b.abs().max()), 1e-300) for a, b in zip(ga, gb))
    store_all = capi.lib().hx_adjoint_work_bytes_f64(g.nx, g.ny, g.nx, nsteps, 0, 0)
    del prob
    # binomial checkpointing with 20 snapshot slots: the same gradient in a fifth of the memory
    slots = 20
    pb = GaugeProblem(g, zero.clone(), gauges, nsteps, case.cfl, checkpoint_every=-slots)
    pb.forward(z, h0, zero, zero)
    t_rev_b, gb = timed(lambda: pb.reverse(href))
    binomial = {"slots": slots, "work_bytes": pb.work_bytes, "reverse_s": t_rev_b,
                "cost_vs_forward": (t_fwd + t_rev_b) / t_plain,
                "recompute_steps": int(capi.lib().hx_adjoint_recompute_steps(nsteps, -slots)),
                "max_rel_diff_vs_checkpointed": max_rel_diff(gb, grads)}
    del pb
    # every state kept (12.6 GB at 512^2 x 2000 steps fits HBM): no recompute, the memory/time other end
    pa = GaugeProblem(g, zero.clone(), gauges, nsteps, case.cfl, checkpoint_every=0)
    t_fwd_a, _ = timed(lambda: pa.forward(z, h0, zero, zero))
    t_rev_a, ga = timed(lambda: pa.reverse(href))
    store_all_run = {"work_bytes": pa.work_bytes, "forward_s": t_fwd_a, "reverse_s": t_rev_a,
                     "cost_vs_forward": (t_fwd_a + t_rev_a) / t_plain,
                     "max_rel_diff_vs_checkpointed": max_rel_diff(ga, grads)}
    del pa
    # the exact arithmetic form: the reverse sweep against the N-step tangent-linear model of the same trajectory
    pe = GaugeProblem(g, zero.clone(), gauges, nsteps, case.cfl, checkpoint_every=every, arith=capi.HX_ARITH_EXACT)
    pe.forward(z, h0, zero, zero)
    t_rev_exact, ge = timed(lambda: pe.reverse(href))
    dirs = [T(workloads.smooth_field(g.nx, g.ny, seed=sd, amplitude=1.0)) for sd in (7, 8)] + [zero, zero]
    t0 = time.perf_counter()
    tan = tangent_misfit(pe, [z, h0, zero, zero], dirs, href)
    t_tan = time.perf_counter() - t0
    ad_e = sum(float((gk * dk).sum()) for gk, dk in zip(ge, dirs))
    tangent = {"arith": "exact", "direction": "smooth fields (seeds 7, 8) in z and h0", "adjoint": ad_e,
               "tangent_linear": tan, "rel_err": abs(ad_e - tan) / max(abs(tan), 1e-300),
               "reverse_exact_s": t_rev_exact, "tangent_s": t_tan}
    del pe
    # the same bed and gauges from a state with no quiescent region, over growing horizons
    scan = []
    for hsteps in [h for h in (30, 100, 300) if h <= nsteps]:
        sc, sg = workloads.adjoint_smooth_case(nsteps=hsteps)
        base = [T(sc.z), T(sc.h), T(sc.hu), T(sc.hv)]
        sp = GaugeProblem(g, zero.clone(), sg, hsteps, sc.cfl, checkpoint_every=every)
        sref = sp.forward(base[0] + dz, *base[1:]).clone()
        sp.forward(*base)
        sgr = sp.reverse(sref)
        # a central difference is exact to O(eps^2) only while no limiter or bed kink lies within eps; the
        # usual step scan (1e-5 .. 1e-8) shows the V of truncation against kinks and rounding
        scan.append({"steps": hsteps, "fd": fd_check(sp, base, sref, sgr, (("z", 0, 7), ("h0", 1, 8), ("hu0", 2, 9)),
                                                     g.nx, g.ny, steps=(1e-5, 1e-6, 1e-7, 1e-8))})
        del sp
    # a state with no kink in the gauges' domain of dependence: the configured FD step, 1e-6
    mono = {}
    for hsteps in [h for h in (100, 300) if h <= nsteps]:
        mc, mg = workloads.adjoint_monotone_case(nsteps=hsteps)
        base = [T(mc.z), T(mc.h), T(mc.hu), T(mc.hv)]
        mp = GaugeProblem(mc.geom, zero.clone(), mg, hsteps, mc.cfl, checkpoint_every=every)
        mref = mp.forward(base[0] + dz, *base[1:]).clone()
        mp.forward(*base)
        mgr = mp.reverse(mref)
        mono["steps_%d" % hsteps] = fd_check(mp, base, mref, mgr, (("z", 0, 7), ("h0", 1, 8), ("hu0", 2, 9)),
                                             g.nx, g.ny, steps=(1e-6,))
        del mp
    return {"workload": "512x512 FP64 hydrostatic-Roe, %d steps, smooth bed (32 Gaussians, 0.3 m), 0.2 m hump, "
                        "64 gauges, reference series from a perturbed bed (seed 6, 0.02 m)" % nsteps,
            "loss": J0, "checkpoint_every": every, "face_records": face_records,
            "plain_forward_s": t_plain, "adjoint_forward_s": t_fwd, "reverse_s": t_rev,
            "cost_vs_forward": (t_fwd + t_rev) / t_plain, "reverse_vs_forward": t_rev / t_plain,
            "reverse_launches": rev_launches,
            "work_bytes_checkpointed": prob_bytes, "work_bytes_store_all": int(store_all),
            "binomial": binomial,
            "store_all": store_all_run,
            "tangent_check": tangent,
            "fd_check": fd,
            "fd_check_note": "the initial state is a lake at rest outside the hump: limiters there sit on their "
                             "flat-data branch (|dp| <= 1e-12), a kink that a 1e-6 step leaves, and the exact "
                             "linearisation of single-stage MUSCL + forward Euler grows by up to 1.064 per step",
            "fd_kink_free": {"workload": "512x512, planar bed 0.2x + 0.1y, free surface and currents increasing "
                                         "strictly in x and y, open boundaries, 64 gauges in the central "
                                         "[0.3, 0.7]^2: no limiter, bed-maximum, sonic or CFL arg-max switch "
                                         "within the gauges' domain of dependence", "runs": mono},
            "fd_horizon_scan": {"workload": "same bed and gauges, free surface 1.0 + 0.05 m undulation + 0.2 m hump, "
                                            "smooth currents up to 0.2 m/s (no quiescent region)",
                                "runs": scan}}


def ensemble_summary(ens):
    """The ensemble figures the JSON line carries (the full record goes to the details file)."""
    if ens is None:
        return None
    return {"batched": ens["batched"], "member_loop": ens["member_loop"],
            "host_dt_loop": ens["plain_loop_host_dt"], "ratio": ens["speedup_vs_plain_loop"],
            "ratio_vs_member_loop": ens["speedup_vs_member_loop"], "unit": UNIT,
            "tile_shape_per_class": ens["tile_shape_per_class"]}


def adjoint_summary(adj):
    """The adjoint figures the JSON line carries: cost against the forward run,
    the gradient against the N-step tangent-linear model, and the central
    differences with the configured step 1e-6 (configured run; kink-free state)."""
    if adj is None:
        return None
    fd = adj["fd_check"]
    kink_free = [v["best_rel_err"] for run in adj["fd_kink_free"]["runs"].values() for v in run.values()]
    return {"cost_vs_forward": adj["cost_vs_forward"], "reverse_vs_forward": adj["reverse_vs_forward"],
            "tangent_rel_err": adj["tangent_check"]["rel_err"],
            "fd_configured_rel_err": {k: v["step_1e-06"]["rel_err"] for k, v in fd.items()},
            "fd_configured_note": "not a derivative check: within a 1e-6 step the configured 2000-step run crosses "
                                  "limiter and bed-maximum kinks, and its exact linearisation grows up to 1.064 per "
                                  "step; tangent_rel_err checks that run, fd_kink_free checks the central "
                                  "differences",
            "fd_kink_free_max_rel_err": max(kink_free) if kink_free else None,
            "binomial_cost_vs_forward": adj["binomial"]["cost_vs_forward"],
            "store_all_cost_vs_forward": adj["store_all"]["cost_vs_forward"],
            "work_bytes_checkpointed": adj["work_bytes_checkpointed"]}


def dominant_kernel(args, arith, cells):
    """The kernel that advances the level in the timed loop: the persistent
    32 x 32 kernel for FP64 hydrostatic levels of 2048^2 cells and more, else
    the tile kernel of the method and precision."""
    form = "true" if arith else "false"
    if (args.method, args.precision) == ("hydrostatic", "f64") and cells >= 1 << 22:
        return "k_hydro_persist<%s>" % form
    return "%s<%s,%s,LevelSrc>" % ("k_hydro_tile" if args.method == "hydrostatic" else "k_classic_tile",
                                   "double" if args.precision == "f64" else "float", form)


def load_profile_summary():
    """Per-launch DRAM traffic and FP64 instruction counts of the dominant
    kernel from the committed ncu summary (profiles/), when present."""
    p = ROOT / "profiles" / "k_hydro_persist_metrics.txt"  # JSON figures from the ncu summary
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return {}
    return {}


def profiled_traffic(profile, cells, args):
    """DRAM bytes per launch of the dominant kernel: the captured bytes per
    cell (each cell is read and written once, so traffic scales with the
    cell count) times this run's cells.  The capture is of the FP64 fast-form
    hydrostatic persistent kernel; other variants report null."""
    per_cell = profile.get("traffic_bytes_per_cell")
    if per_cell is None or (args.method, args.precision, args.arith) != ("hydrostatic", "f64", "fast") or \
            cells < 1 << 22:  # the capture is of the 32 x 32 tile that levels of 2048^2 cells and more take
        return None
    return per_cell * cells


def fp64_pipe(profile, kms):
    """Achieved FP64 instruction rate of the dominant kernel against the
    measured DFMA issue rate (the binding roof of the FP64 advance)."""
    inst = profile.get("fp64_inst_per_cell")
    if not inst:
        return {"peak_dfma_per_s": FP64_DFMA_PER_S, "peak_source": FP64_SRC, "achieved": None, "frac": None}
    cells = NX * NY
    rate = inst * cells / (kms * 1e-3)
    return {"peak_dfma_per_s": FP64_DFMA_PER_S, "peak_source": FP64_SRC, "achieved_inst_per_s": rate,
            "frac": rate / FP64_DFMA_PER_S, "inst_per_cell": inst,
            "source": "FP64 instructions per cell from the ncu capture in profiles/"}


if __name__ == "__main__":
    sys.exit(main())
