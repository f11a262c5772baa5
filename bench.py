"""Benchmark of the eqcycle time-stepping hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the 480x240-element damage-zone model (1.85M GLL nodes, 961 fault nodes;
preset ``dz480``), seeded synthetic initial state (V = Vpl, theta with 1 % seeded noise).
A step is one time step of the simulation loop (src/main.jl:220-452).  The timed window
is the interseismic regime: the state starts at t = 0 with dt set to the step dtevol!
gives for steady sliding at the plate rate (about 42 days), W untimed steps follow, then
exactly K timed steps.  value = simulated years advanced in the K steps per hour of
device time (CUDA events on the library stream).

Methods: the headline runs the mixed-precision solver (FP32 stiffness apply and multigrid
inside an FP64 reliable-update CG, FP64 friction and state); the plain FP64 method runs the
same window and is reported beside it.  Both stop CG at ||r|| <= 1e-8 ||b||.

Beside the headline the default line carries, untimed: `mixed_error`, the mixed method's
per-step error against the plain FP64 method (lockstep runs from the same start, quasi-static
window and Newmark steps from a fast start), and `whole_cycle`, both methods over the first 20
simulated years of the workload from the seeded start (interseismic steps, the nucleation, the
first event's rupture and dynamic phase, afterslip), with the event statistics compared.

--impl reference times the reference's algorithm on the host cores: the CPU oracle in
reference mode (Ruge-Stueben AMG with Gauss-Seidel V-cycle inside CG, FP64 friction), the
restatement of the Julia code (Julia is not installed here, so `julia run.jl` itself cannot
run).  Its steps are whole QS steps from the seeded start, at least 3, more within a time
budget; the default line's `cpu_baseline` is the same sample (at least 2 steps), taken in a
spawned process while the GPU runs the untimed legs.

N > 1 GPUs (launched by torchrun, one rank per GPU; --gpus must equal WORLD_SIZE): the
single-model path does not shard (replicas only); every rank advances its own replica and
value sums the ranks' simulated years over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

YR = 365 * 24 * 3600.0


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    dist.init_process_group(backend="gloo")
    return rank, ws, dist


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _allreduce(dist, v, op):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=op)
    return float(t.item())


# FP32 apply kernels by eqc_options.apply_variant
APPLY_KERNELS = {0: "k_apply_rows<6,3>", 4: "k_apply_rows<4,3>", 5: "k_apply_rows<8,2>", 6: "k_apply_rows<12,1>",
                 7: "k_apply_rows<6,2>", 8: "k_apply_walk"}


class Clocks:
    """SM clock and clock-event (throttle) reasons sampled every 2 ms during the timed region,
    read through NVML (libnvidia-ml, read-only queries); nvidia-smi at 200 ms if NVML cannot
    be loaded."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device: int):
        import threading
        self.samples, self.smax, self.mask = [], 0.0, 0
        self.p = None
        self.stop_ev = threading.Event()
        self.th = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit")
            cnt = ctypes.c_uint(0)
            nv.nvmlDeviceGetCount_v2(ctypes.byref(cnt))
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            idx = device
            if cnt.value == 1:
                idx = 0
            elif vis and all(x.strip().isdigit() for x in vis.split(",")):
                idx = int(vis.split(",")[device])
            h = ctypes.c_void_p()
            if nv.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) != 0:
                raise OSError("nvmlDeviceGetHandleByIndex")
            mx = ctypes.c_uint(0)
            nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))   # NVML_CLOCK_SM
            self.smax = float(mx.value)

            def run():
                clk, rs = ctypes.c_uint(0), ctypes.c_ulonglong(0)
                while not self.stop_ev.is_set():
                    if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0:
                        self.samples.append(float(clk.value))
                    if nv.nvmlDeviceGetCurrentClocksEventReasons(h, ctypes.byref(rs)) == 0:
                        self.mask |= int(rs.value)
                    time.sleep(0.002)
            self.th = threading.Thread(target=run, daemon=True)
            self.th.start()
            return
        except Exception:
            self.th = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"eqc_clocks_{os.getpid()}.csv")
        Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.th is not None:
            self.stop_ev.set()
            self.th.join(timeout=5)
            if not self.samples:
                return None
            return {"sm_mhz": float(np.median(self.samples)), "sm_max_mhz": self.smax,
                    "reasons": sorted(n for b, n in self.REASONS.items() if self.mask & b),
                    "samples": len(self.samples), "source": "nvml, 2 ms"}
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        with open(self.path) as f:
            return parse_clock_csv(f)


def parse_clock_csv(lines):
    """Clock record from nvidia-smi's CSV lines (the query of Clocks, noheader, nounits): median SM
    clock, maximum SM clock, and the throttle reasons seen active in any sample; None without a
    valid sample.  Lines that do not parse (a partial last line, "[N/A]") are skipped."""
    sm, smax, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in lines:
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9:
            continue
        try:
            sm.append(float(parts[1]))
            smax = max(smax, float(parts[2]))
        except ValueError:
            continue
        for n, v in zip(names, parts[5:9]):
            if v.lower().startswith("active"):
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
            "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def steady_dt(solver, P):
    """The step dtevol! takes for the initial steady sliding (rate-limited by XiLf/V)."""
    Vf = 2 * solver.state("v")[P.iarray.iFlt - 1] + P.float_.Vpl
    return solver.dtevol(1e30, P.float_.dt0, Vf, 1)


L2_BYTES = 129 * 2 ** 20   # GB300's L2


def stream_copies(nbytes: int) -> int:
    """Working-set replicas whose total is at least twice L2 (each launch then reads from HBM)."""
    return int(min(64, max(2, -(-2 * L2_BYTES // max(nbytes, 1)))))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_window(P, precision, W, K, device, params=None, **kw):
    from eqcycle_gb300 import Solver
    s = Solver(P, precision=precision, cg_tol=1e-8, device=device, **kw)
    if params is not None:
        s.set_guess_params(params)
    s.init(P.cfg.V_init)
    s.set_scalar("dt", steady_dt(s, P))
    if W:
        s.run(W)
    t0 = s.scalar("t")
    l0 = s.launches()
    st = s.run(K)
    launches = s.launches() - l0
    sim_years = (st["t"] - t0) / YR
    return s, st, sim_years, launches


def cpu_baseline_sample(P, budget_s=240.0, min_steps=1, nthreads=None, name="dz480"):
    """The oracle in reference mode on the host cores: whole QS steps from the same start, at
    least min_steps of them, more while the time spent stays within half the budget."""
    from oracle import pyoracle
    nthreads = nthreads or os.cpu_count() or 1
    pyoracle.set_threads(nthreads)
    o = pyoracle.Oracle(P.cfg)
    # same start as the GPU window: t = 0, dt = the steady dtevol! step
    Vf = 2 * o.state("v")[o.get("iFlt") - 1] + P.float_.Vpl
    import ctypes as C
    dt_s = pyoracle.lib().orc_dtevol(o.h, 1e30, P.float_.dt0, Vf.ctypes.data_as(C.POINTER(C.c_double)), 1)
    o.set_state("dt", dt_s)
    t_setup = time.time()
    o.qs_solve(np.zeros(o.Nf), np.zeros(o.nglob), tol=1e-8, mode=0, maxit=1)  # builds the AMG hierarchy
    setup_s = time.time() - t_setup
    steps, wall, t0, per_step = 0, 0.0, o.scalar("t"), []
    while True:
        t1 = time.time()
        n = o.run(1, qs_mode=0, qs_tol=1e-8)
        per_step.append(time.time() - t1)
        wall += per_step[-1]
        steps += n
        if n == 0 or (steps >= min_steps and wall + wall / steps > budget_s):
            break
    sim_years = (o.scalar("t") - t0) / YR
    cg = o.get("cg_iters")
    return {"value": sim_years / (wall / 3600.0), "unit": "sim-years/hr", "cores": nthreads, "kind": "port",
            "sample": f"the first {steps} interseismic QS steps of {name} from the seeded start (dt "
                      f"{dt_s:.3g} s), the oracle in reference mode (RS-AMG + symmetric Gauss-Seidel V-cycle in CG "
                      f"to 1e-8, FP64 friction), {int(cg.sum())} CG iterations, {wall:.1f} s wall "
                      f"(per step {', '.join(f'{x:.0f}' for x in per_step)} s); value = simulated years of these "
                      f"steps over their wall time, no extrapolation; AMG setup {setup_s:.1f} s excluded",
            "steps": steps, "wall_s": wall, "sim_years": sim_years, "per_step_s": per_step,
            "cg_iters_per_solve": float(cg.sum()) / max(1, 2 * steps)}


def _cpu_baseline_child(workload, budget_s, min_steps, nthreads, q):
    """cpu_baseline_sample in a spawned process (the oracle only: no CUDA in this process), so
    that the host-core sample runs while the GPU legs run in the parent."""
    try:
        from eqcycle_gb300 import preset, set_parameters
        P = set_parameters(preset(workload))
        q.put(cpu_baseline_sample(P, budget_s=budget_s, min_steps=min_steps, nthreads=nthreads, name=workload))
    except Exception as e:  # reported in the JSON line instead of the sample
        q.put({"error": repr(e)})


def start_cpu_baseline(workload, budget_s, min_steps, nthreads):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_cpu_baseline_child, args=(workload, budget_s, min_steps, nthreads, q), daemon=True)
    p.start()
    return p, q


def finish_cpu_baseline(job, timeout_s):
    p, q = job
    try:
        res = q.get(timeout=timeout_s)
    except Exception:
        res = {"error": "CPU sample did not finish in time"}
    p.join(timeout=10)
    if p.is_alive():
        p.kill()
    return res


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def mixed_error_leg(P, device, W, K, dyn_steps=300):
    """Per-step error of the mixed-precision method against the plain FP64 method on the
    workload, both from the same start and stepped in lockstep (one step per call, outside any
    timed region): after each of W + K interseismic quasi-static steps from the steady-sliding
    start, and after each of dyn_steps Newmark steps from a fast start (the fault sliding at
    5 cm/s, the dynamic regime).  Errors are max-norm relative to the FP64 field: the whole
    displacement field d, the fault slip (2 d + Vpl t on the fault), the fault slip rate
    (2 v + Vpl) and the state psi; the maximum over the steps is reported."""
    from eqcycle_gb300 import EQC_FP64, EQC_GUESS_EXTRAPOLATE, EQC_MIXED, Solver
    iF = P.iarray.iFlt - 1
    Vpl = P.float_.Vpl
    out = {}
    for phase in ("quasi_static", "dynamic"):
        a = Solver(P, precision=EQC_FP64, cg_tol=1e-8, device=device)
        b = Solver(P, precision=EQC_MIXED, cg_tol=1e-8, device=device, guess=EQC_GUESS_EXTRAPOLATE)
        n = W + K if phase == "quasi_static" else dyn_steps
        err = {"d": 0.0, "slip": 0.0, "slip_rate": 0.0, "psi": 0.0}
        for s in (a, b):
            if phase == "quasi_static":
                s.init(P.cfg.V_init)
                s.set_scalar("dt", steady_dt(s, P))
            else:
                s.init(5e-2)
        regimes = set()
        for k in range(n):
            sa, sb = a.run(1), b.run(1)
            regimes.add(int(sa["dyn_steps"]) * 2 + int(sa["qs_steps"]))
            t = a.scalar("t")
            full = phase == "quasi_static" or k % 25 == 24 or k == n - 1
            da = a.state("d") if full else None
            db = b.state("d") if full else None
            va, vb = a.state("v")[iF], b.state("v")[iF]
            if full:
                err["d"] = max(err["d"], _rel(db, da))
                err["slip"] = max(err["slip"], _rel(2 * db[iF] + Vpl * t, 2 * da[iF] + Vpl * t))
            err["slip_rate"] = max(err["slip_rate"], _rel(2 * vb + Vpl, 2 * va + Vpl))
            err["psi"] = max(err["psi"], _rel(b.state("psi"), a.state("psi")))
        out[phase] = {"steps": n, "regime": "dynamic" if regimes == {2} else "quasi-static" if regimes == {1}
                      else "mixed", **{f"max_rel_err_{k}": v for k, v in err.items()}}
        a.close()
        b.close()
    out["note"] = ("mixed (FP32 apply and multigrid in an FP64 reliable-update CG to 1e-8; FP64 friction, state "
                   "and Newmark accumulation) against plain FP64 (CG to 1e-8), same start, compared after every "
                   "step; displacement field every step in the quasi-static phase, every 25 steps in the "
                   "dynamic one")
    return out


def cycle_leg(P, device, years=20.0, budget_s=400.0):
    """Whole earthquake cycle on the workload: the plain FP64 method and the mixed method
    (extrapolated guess, smoother autotuned after its first 20 quasi-static steps) each run the
    simulation from the seeded start to t = `years` (the dz480 model nucleates at about 1.5 yr
    and its first event ends near 7 yr: the window holds the interseismic start, the nucleation,
    the rupture and its dynamic phase, the afterslip and the return to interseismic steps), or
    until budget_s seconds of wall time.  value = simulated years per hour of device time (CUDA
    events); event statistics of the two runs are compared (first event start, coseismic slip,
    hypocentre depth, Mw)."""
    from eqcycle_gb300 import EQC_FP64, EQC_GUESS_EXTRAPOLATE, EQC_GUESS_PREVIOUS, EQC_MIXED, Solver
    from eqcycle_gb300.events import catalogue, compare
    mu = P.cfg.rho1 * P.cfg.vs1 ** 2
    out, cats = {}, {}
    t_stop = years * YR
    for name, prec, guess in (("plain_fp64", EQC_FP64, EQC_GUESS_PREVIOUS), ("mixed", EQC_MIXED, EQC_GUESS_EXTRAPOLATE)):
        with Solver(P, precision=prec, cg_tol=1e-8, guess=guess, device=device) as s:
            s.init(P.cfg.V_init)
            gpu_ms, qs, dyn, cg, solves, wall0, tuned = 0.0, 0, 0, 0, 0, time.time(), None
            while s.scalar("t") < t_stop and time.time() - wall0 < budget_s:
                st = s.run(5000, t_stop)
                gpu_ms += st["gpu_ms"]
                qs += st["qs_steps"]
                dyn += st["dyn_steps"]
                cg += st["cg_iters"]
                solves += st["qs_solves"]
                if prec == EQC_MIXED and tuned is None and qs >= 20:
                    tuned = s.autotune(reps=2)
            years_run = s.scalar("t") / YR
            res = s.results()
        cats[name] = catalogue(res, P.farray.FltX, mu)
        out[name] = {"sim_years": years_run, "value": years_run / (gpu_ms / 3.6e6) if gpu_ms else None,
                     "gpu_s": gpu_ms / 1e3, "wall_s": time.time() - wall0, "qs_steps": qs, "dyn_steps": dyn,
                     "cg_iters_per_solve": cg / max(solves, 1), "autotune": tuned, **cats[name].summary()}
    a, b = cats["plain_fp64"], cats["mixed"]
    cmp = compare(a, b)
    if len(a.tStart) and len(b.tStart):
        cmp["first_event_start"] = float(abs(b.tStart[0] - a.tStart[0]) / a.tStart[0])
    if len(a.Mw) and len(b.Mw):
        cmp["Mw_abs"] = float(np.max(np.abs(b.Mw[:len(a.Mw)] - a.Mw[:len(b.Mw)])))
    out["event_statistics_mixed_vs_fp64"] = cmp
    pv, mv = out["plain_fp64"]["value"], out["mixed"]["value"]
    out["speedup_mixed_vs_plain_fp64"] = mv / pv if pv and mv else None
    out["window"] = (f"t = 0 to {years:g} yr from the seeded start, both methods (first event "
                     f"{a.tStart[0] / YR if len(a.tStart) else float('nan'):.2f} to "
                     f"{a.tEnd[0] / YR if len(a.tEnd) else float('nan'):.2f} yr in the FP64 run)")
    return out


def bench_ours(args):
    from eqcycle_gb300 import set_parameters, preset, EQC_FP64, EQC_MIXED
    rank, ws, dist = _dist()
    device = int(os.environ.get("LOCAL_RANK", "0"))
    P = set_parameters(preset(args.workload))
    nglob, Nel, Nf = P.int_.nglob, P.int_.Nel, P.int_.FltNglob
    out = {}
    # ---- plain FP64 method on the window
    s64, st64, sy64, _ = run_window(P, EQC_FP64, args.warmup, args.steps, device)
    s64.close()

    def leg(st_, sy_, s_=None):
        d = {"value": sy_ / (st_["gpu_ms"] / 3.6e6) if st_["gpu_ms"] else None,
             "qs_step_ms": st_["gpu_ms"] / max(st_["qs_steps"], 1),
             "cg_iters_per_solve": st_["cg_iters"] / max(st_["qs_solves"], 1)}
        if s_ is not None:
            d["guess_kept"], d["guess_tried"] = s_.scalar("guess_kept"), s_.scalar("guess_tried")
        return d
    # ---- headline: mixed precision with the extrapolated guess and the autotuned smoother;
    # state at the window start kept for the e2e leg
    from eqcycle_gb300 import Solver, EQC_GUESS_EXTRAPOLATE
    s = Solver(P, precision=EQC_MIXED, cg_tol=1e-8, device=device, guess=EQC_GUESS_EXTRAPOLATE,
               use_graphs=0 if args.no_graphs else 1)
    s.init(P.cfg.V_init)
    s.set_scalar("dt", steady_dt(s, P))
    if args.warmup:
        s.run(args.warmup)
    t_tune = time.time()
    tuned = s.autotune(reps=3)   # after the warm-up: trial solves of a representative step
    tuned["wall_s"] = time.time() - t_tune
    start = {k: s.state(k) for k in ("d", "v", "a", "psi", "tau")}
    t_start, dt_start, iso_start = s.scalar("t"), s.scalar("dt"), s.scalar("isolver")
    clocks = Clocks(device)
    _barrier(dist)
    l0 = s.launches()
    st = s.run(args.steps)
    _barrier(dist)
    launches = s.launches() - l0
    clk = clocks.stop()
    sim_years = (st["t"] - t_start) / YR
    dev_s = st["gpu_ms"] / 1e3
    dev_s_max = _allreduce(dist, dev_s, _max_op())
    tot_years = _allreduce(dist, sim_years, _sum_op())
    value = tot_years / (dev_s_max / 3600.0)
    # ---- e2e: the same window through the C ABI with host buffers (state in, run, state out),
    # the state in pinned host memory as a caller that streams states would keep it
    keep = []

    def pinned(n):
        import torch
        if not torch.cuda.is_available():
            return np.empty(n)
        torch.cuda.set_device(device)
        t = torch.empty(n, dtype=torch.float64, pin_memory=True)
        keep.append(t)
        return t.numpy()
    start_p = {k: pinned(v.size) for k, v in start.items()}
    for k, v in start.items():
        start_p[k][:] = v
    end = {k: pinned(v.size) for k, v in start.items()}
    h2d = sum(start_p[k].nbytes for k in start_p) + 3 * 8
    t1 = time.perf_counter()
    for k, v in start_p.items():
        s.set_state(k, v)
    s.set_scalar("t", t_start)
    s.set_scalar("dt", dt_start)
    s.set_scalar("isolver", iso_start)
    st_e = s.run(args.steps)
    for k in end:
        s.state(k, out=end[k])
    e2e_s = time.perf_counter() - t1
    d2h = sum(end[k].nbytes for k in end) + args.steps * 96
    e2e_years = (st_e["t"] - t_start) / YR
    e2e_s_max = _allreduce(dist, e2e_s, _max_op())
    e2e_value = _allreduce(dist, e2e_years, _sum_op()) / (e2e_s_max / 3600.0)
    # ---- roofline of the dominant kernel (FP32 stiffness apply, L2 flushed between launches)
    peak, peak_kind = measured_peaks()
    ms32_cold = s.time_apply(1, 50, True)
    bytes32 = 4 * (2 * nglob + 25 * Nel)
    nc32 = stream_copies(bytes32)
    ms32 = s.time_apply_stream(1, 12 * nc32, nc32)
    ms64 = s.time_apply(0, 20, True)
    msdf = s.time_apply(2, 20, True)
    bytes64 = 8 * (2 * nglob + 25 * Nel)
    # DRAM bytes per launch of the kernel the autotuner chose, from one ncu capture
    kname = APPLY_KERNELS.get(tuned.get("apply_variant", 0), "k_apply_rows<6,3>")
    traffic = None
    tp = os.path.join(ROOT, "profiles", f"kapply_{args.workload}_traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get("fp32_bytes_per_launch", {}).get(kname)
    s.close()
    # ---- the same window with the previous-step guess (the reference's), and with the learned
    # guess trained on pairs the plain solver logs on 8 other seeds of the workload
    from eqcycle_gb300 import EQC_GUESS_LEARNED, EQC_GUESS_PREVIOUS
    deg = dict(mg_degree=tuned["mg_degree"], mg_degree_coarse=tuned["mg_degree_coarse"])
    sp, stp, syp, _ = run_window(P, EQC_MIXED, args.warmup, args.steps, device, guess=EQC_GUESS_PREVIOUS, **deg)
    sp.close()
    learned = None
    if args.learned_pairs > 0:
        t_l = time.time()
        per_seed = max(1, args.learned_pairs // 8)
        xs, ys = [], []
        for seed in range(1, 9):
            Ps = set_parameters(preset(args.workload, seed=seed))
            with Solver(Ps, precision=EQC_MIXED, cg_tol=1e-8, device=device, **deg) as sl:
                sl.guess_log(per_seed)
                sl.init(Ps.cfg.V_init)
                sl.set_scalar("dt", steady_dt(sl, Ps))
                sl.run(per_seed)
                x, y = sl.guess_pairs()
            xs.append(x)
            ys.append(y)
        with Solver(P, precision=EQC_MIXED, device=device) as st_:
            st_.guess_init(0)
            st_.guess_train(np.concatenate(xs), np.concatenate(ys), epochs=20, lr=1e-3, batch=256, seed=0)
            params = st_.guess_params()
        sl_, stl, syl, _ = run_window(P, EQC_MIXED, args.warmup, args.steps, device, params=params,
                                      guess=EQC_GUESS_LEARNED, **deg)
        learned = leg(stl, syl, sl_)
        learned["pairs"] = int(sum(len(x) for x in xs))
        learned["train_and_log_s"] = time.time() - t_l
        sl_.close()
    # ---- the host-core sample of the reference's algorithm runs in a spawned process (no CUDA
    # there) while the untimed legs below use the GPU; one core is left to drive the GPU
    cpu_job = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu_job = start_cpu_baseline(args.workload, args.cpu_budget, args.cpu_min_steps,
                                     max(1, (os.cpu_count() or 2) - 1))
    mixed_error = mixed_error_leg(P, device, args.warmup, args.steps) if not args.no_cycle else None
    whole_cycle = cycle_leg(P, device, years=args.cycle_leg_years, budget_s=args.cycle_leg_budget) \
        if not args.no_cycle else None
    if rank != 0:
        return
    line = {
        "metric": "sim-years/hr", "value": value, "unit": "sim-years/hr", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / max(st["steps"], 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic: seeded initial state of the damage-zone model (no dataset)",
        "config": {"workload": f"{args.workload}: {'damage-zone' if P.cfg.damage else 'homogeneous'} model of "
                               f"NelX x NelY = {P.cfg.NelX} x {P.cfg.NelY} elements, {nglob:,} nodes, {Nf:,} fault "
                               f"nodes; interseismic window after {args.warmup} warm-up steps from the steady-sliding "
                               f"start; mixed-precision multigrid-PCG (tol 1e-8), extrapolated initial guess, "
                               f"autotuned smoother",
                   "nodes": nglob, "fault_nodes": Nf, "parallelism": f"replicas x{ws}",
                   "l2": "stiffness-apply roofline: launches rotate over working-set replicas larger than L2"},
        "qs_step_ms": 1e3 * dev_s / max(st["qs_steps"], 1), "cg_iters_per_solve": st["cg_iters"] / max(st["qs_solves"], 1),
        "sim_years_in_window": sim_years,
        "plain_fp64": leg(st64, sy64),
        "mixed_previous_guess": leg(stp, syp),
        "learned_mixed": learned,
        "autotune": tuned,
        "e2e": {"value": e2e_value, "unit": "sim-years/hr", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps},
        "roofline": {"bound": "hbm", "achieved": bytes32 / (ms32 * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": bytes32 / (ms32 * 1e-3) / 1e9 / peak, "traffic": traffic,
                     "kernel": f"{kname} (FP32 stiffness apply, one element per lane; chosen by the autotuner)",
                     "peak_kind": peak_kind,
                     "launch_us": ms32 * 1e3, "algorithmic_bytes": bytes32,
                     "timing": f"{12 * nc32} back-to-back launches rotating over {nc32} replicas of the working set "
                               f"({nc32 * bytes32 / 2 ** 20:.0f} MiB > L2), CUDA events around the batch",
                     "single_launch_l2_flushed_us": ms32_cold * 1e3,
                     "single_launch_frac": bytes32 / (ms32_cold * 1e-3) / 1e9 / peak},
        "fp64_apply": {"launch_us": ms64 * 1e3, "algorithmic_bytes": bytes64,
                       "achieved_gbs": bytes64 / (ms64 * 1e-3) / 1e9,
                       "double_float_launch_us": msdf * 1e3},
        "gpu_launches": launches,
    }
    line["speedup_vs_plain_fp64"] = value / line["plain_fp64"]["value"] if line["plain_fp64"]["value"] else None
    if clk:
        line["clocks"] = clk
    line["mixed_error"] = mixed_error
    line["whole_cycle"] = whole_cycle
    if cpu_job is not None:
        cb = finish_cpu_baseline(cpu_job, timeout_s=3 * args.cpu_budget + 600)
        if "error" not in cb:
            cb["concurrent"] = "ran on the host cores while the GPU ran the untimed legs (mixed_error, whole_cycle)"
        line["cpu_baseline"] = cb
    print(json.dumps(line), flush=True)


def _max_op():
    try:
        import torch.distributed as dist
        return dist.ReduceOp.MAX
    except Exception:
        return None


def _sum_op():
    try:
        import torch.distributed as dist
        return dist.ReduceOp.SUM
    except Exception:
        return None


def bench_reference(args):
    rank, ws, dist = _dist()
    if rank != 0:
        return
    from eqcycle_gb300 import set_parameters, preset
    P = set_parameters(preset(args.workload))
    # whole QS steps of the reference algorithm: at least 3 (about 100 s each on 16 Arm cores: the
    # symmetric Gauss-Seidel smoother of the reference's AMG is sequential), more within the budget
    cb = cpu_baseline_sample(P, budget_s=max(args.cpu_budget, 360.0), min_steps=max(3, args.cpu_min_steps),
                             name=args.workload)
    line = {"impl": "reference", "metric": "sim-years/hr", "value": cb["value"], "unit": "sim-years/hr",
            "n_gpus": ws, "steps": cb["steps"], "warmup": 0, "ms_per_step": 1e3 * cb["wall_s"] / max(cb["steps"], 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded initial state of the damage-zone model (no dataset)",
            "config": {"workload": f"{args.workload}: interseismic QS steps from the steady-sliding start, "
                                   "reference algorithm (RS-AMG + Gauss-Seidel in CG, tol 1e-8) on the host cores"},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "sim-years/hr", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_profile_steps(args):
    """The headline method on the workload, host-driven (every kernel a separate launch, for an
    ncu launch list), with its solver settings given on the command line instead of autotuned
    (an autotuner timed under a profiler chooses differently): W warm-up steps, then K steps;
    prints how many kernels the K steps launched (the tail of the launch list)."""
    from eqcycle_gb300 import EQC_GUESS_EXTRAPOLATE, EQC_MIXED, Solver, preset, set_parameters
    P = set_parameters(preset(args.workload))
    s = Solver(P, precision=EQC_MIXED, cg_tol=1e-8, guess=EQC_GUESS_EXTRAPOLATE, use_graphs=1 if args.graphs else 0,
               apply_variant=args.apply_variant, mg_degree=args.mg_degree, mg_degree_coarse=args.mg_degree_coarse,
               reliable_delta=args.reliable_delta)
    if args.dynamic:   # Newmark steps: the fault sliding at 5 cm/s, above the regime threshold
        s.init(5e-2)
    else:
        s.init(P.cfg.V_init)
        s.set_scalar("dt", steady_dt(s, P))
    s.run(args.warmup)
    l0 = s.launches()
    st = s.run(args.steps)
    print(json.dumps({"workload": args.workload, "launches_in_steps": s.launches() - l0, "steps": st}), flush=True)
    s.close()


def bench_setup(args):
    """Model setup time on the workload mesh: the host setup (set_parameters over the whole mesh,
    then eqc_create uploading iglob/W/M) against the setup on the device (structured_parameters
    over the mesh edges, then eqc_create_structured building W, M, 1/M and diag K with kernels),
    with eqc_create's phases; the multigrid hierarchy is built on the host in both."""
    from eqcycle_gb300 import EQC_MIXED, Solver, preset, set_parameters, structured_parameters
    cfg = preset(args.workload)
    out = {"workload": args.workload}
    for name, fn in (("host", set_parameters), ("device", structured_parameters)):
        t0 = time.perf_counter()
        P = fn(cfg)
        t1 = time.perf_counter()
        s = Solver(P, precision=EQC_MIXED)
        t2 = time.perf_counter()
        out[name] = {"parameters_s": t1 - t0, "create_s": t2 - t1, "total_s": t2 - t0,
                     **{k: s.scalar(f"setup_ms_{k}") for k in ("numbering", "elements", "nodes", "other",
                                                                 "hierarchy")}}
        s.close()
    print(json.dumps(out), flush=True)


def bench_kernel(args):
    """Stiffness apply alone on the workload mesh, L2 flushed between launches."""
    from eqcycle_gb300 import EQC_PC_JACOBI, Solver, preset, set_parameters
    P = set_parameters(preset(args.workload))
    nglob, Nel = P.int_.nglob, P.int_.Nel
    peak, kind = measured_peaks()
    with Solver(P, precond=EQC_PC_JACOBI, apply_variant=args.apply_variant) as s:
        out = {"workload": args.workload, "nodes": nglob, "elements": Nel, "peak_gbs": peak, "peak_kind": kind,
               "apply_variant": args.apply_variant}
        for name, dt, es in (("f32", 1, 4), ("f64", 0, 8)):
            if args.dtype not in ("both", name):
                continue
            ms = s.time_apply(dt, args.nrep, True)
            B = es * (2 * nglob + 25 * Nel)
            nc = stream_copies(B)
            mss = s.time_apply_stream(dt, max(args.nrep, 4 * nc), nc)
            out[name] = {"launch_us": ms * 1e3, "algorithmic_bytes": B, "achieved_gbs": B / ms / 1e6,
                         "frac": B / ms / 1e6 / peak,
                         "stream": {"launch_us": mss * 1e3, "copies": nc, "achieved_gbs": B / mss / 1e6,
                                    "frac": B / mss / 1e6 / peak}}
    print(json.dumps(out), flush=True)


def bench_learned(args):
    """Learned initial guess on the damage-zone model: pairs logged by the plain solver on
    8 training seeds, Adam on the GPU, evaluated on 2 held-out seeds against the previous-step
    and the extrapolated guess (same 1e-8 CG tolerance for all)."""
    from eqcycle_gb300 import (EQC_GUESS_EXTRAPOLATE, EQC_GUESS_LEARNED, EQC_GUESS_PREVIOUS, EQC_MIXED, Solver,
                               preset, set_parameters)
    per_seed = max(1, args.pairs // 8)
    t0 = time.time()
    xs, ys = [], []
    for seed in range(1, 9):
        P = set_parameters(preset(args.workload, seed=seed))
        with Solver(P, precision=EQC_MIXED, cg_tol=1e-8, guess=EQC_GUESS_PREVIOUS) as s:
            s.guess_log(per_seed)
            s.init(P.cfg.V_init)
            s.set_scalar("dt", steady_dt(s, P))
            s.run(per_seed)
            x, y = s.guess_pairs()
        xs.append(x)
        ys.append(y)
    xin, tgt = np.concatenate(xs), np.concatenate(ys)
    t_log = time.time() - t0
    held = []
    params = None
    report = {"metric": "learned initial guess", "workload": args.workload, "pairs": int(len(xin)),
              "train_seeds": list(range(1, 9)), "heldout_seeds": [9, 10], "log_s": t_log}
    for seed in (9, 10):
        P = set_parameters(preset(args.workload, seed=seed))
        res = {}
        for name, mode in (("previous", EQC_GUESS_PREVIOUS), ("extrapolate", EQC_GUESS_EXTRAPOLATE),
                           ("learned", EQC_GUESS_LEARNED)):
            with Solver(P, precision=EQC_MIXED, cg_tol=1e-8, guess=mode) as s:
                if mode == EQC_GUESS_LEARNED:
                    if params is None:
                        s.guess_init(0)
                        t1 = time.time()
                        losses = s.guess_train(xin, tgt, epochs=args.epochs, lr=1e-3, batch=256, seed=0)
                        report["train_s"] = time.time() - t1
                        report["train_loss"] = [float(v) for v in losses]
                        params = s.guess_params()
                    else:
                        s.set_guess_params(params)
                if mode == EQC_GUESS_PREVIOUS:
                    s.guess_log(args.steps + args.warmup)
                s.init(P.cfg.V_init)
                s.set_scalar("dt", steady_dt(s, P))
                s.run(args.warmup)
                tw = s.scalar("t")
                st = s.run(args.steps)
                if mode == EQC_GUESS_PREVIOUS:
                    hx, hy = s.guess_pairs()
                    held.append((hx, hy))
                res[name] = {"guess_kept": s.scalar("guess_kept"), "guess_tried": s.scalar("guess_tried"),
                             "qs_step_ms": st["gpu_ms"] / max(st["qs_steps"], 1),
                             "cg_iters_per_solve": st["cg_iters"] / max(st["qs_solves"], 1),
                             "sim_years_per_hr": (st["t"] - tw) / YR / (st["gpu_ms"] / 3.6e6) if st["gpu_ms"] else None}
        report[f"seed{seed}"] = res
    # held-out error of the network against the previous-step guess (which predicts 0)
    P = set_parameters(preset(args.workload, seed=9))
    hx = np.concatenate([h[0] for h in held])
    hy = np.concatenate([h[1] for h in held])
    with Solver(P, precision=EQC_MIXED) as s:
        s.set_guess_params(params)
        report["heldout_mse_network"] = s.guess_eval(hx, hy)
    report["heldout_mse_previous"] = float(np.mean(hy.astype(np.float64) ** 2))
    print(json.dumps(report), flush=True)


def bench_ensemble(args):
    """The batched ensemble: 64 uneven damage-zone models (120x60 to 480x240 elements, seeded
    parameters) advanced by one CUDA-graph launch per step, mixed precision with the extrapolated
    guess, or (--ensemble-guess learned) with the learned guess: every member first steps
    --learn-steps quasi-static steps on its own logging (features, increment) pairs, trains its own
    network on them on the GPU and then runs with it, the on-device check keeping an increment only
    where it lowers the residual; compared with the same members stepped one after another with
    their own graphs.  Under torchrun the members are split across the ranks (shard_members; no
    exchange), each rank runs its share as one ensemble, and the whole-job value is all ranks'
    simulated years over the slowest rank's device time (a fixed total of members: strong
    scaling)."""
    from eqcycle_gb300 import (EQC_GUESS_EXTRAPOLATE, EQC_GUESS_LEARNED, EQC_MIXED, Ensemble, Solver,
                               ensemble_members, structured_parameters)
    from eqcycle_gb300.config import shard_members
    rank, ws, dist = _dist()
    device = int(os.environ.get("LOCAL_RANK", "0"))
    learned = args.ensemble_guess == "learned"
    t0 = time.time()
    cfgs_all = ensemble_members(args.members)
    cfgs = [cfgs_all[k] for k in shard_members(cfgs_all, rank, ws)]
    solvers, nodes, train_s, pairs = [], 0, 0.0, 0
    for k, c in enumerate(cfgs):
        P = structured_parameters(c)   # element and node data built on the device
        s = Solver(P, precision=EQC_MIXED, cg_tol=1e-8, device=device,
                   guess=EQC_GUESS_LEARNED if learned else EQC_GUESS_EXTRAPOLATE)
        s.init(c.V_init)
        s.set_scalar("dt", steady_dt(s, P))
        if learned:   # the member's own pairs, its own network (no network until it is trained)
            s.guess_init(k + 1)
            s.guess_log(args.learn_steps)
            s.run(args.learn_steps)
            xin, tgt = s.guess_pairs()
            t1 = time.time()
            s.guess_train(xin, tgt, epochs=args.epochs, lr=1e-3, batch=min(256, max(1, len(xin))), seed=k)
            train_s += time.time() - t1
            pairs += len(xin)
        solvers.append(s)
        nodes += P.int_.nglob
    setup_s = time.time() - t0
    E = Ensemble(solvers)
    E.run(args.warmup)
    t_start = [s.scalar("t") for s in solvers]
    gk = lambda key: sum(s.scalar(key) for s in solvers)
    g0 = (gk("guess_kept"), gk("guess_tried"))
    _barrier(dist)
    stats, ms = E.run(args.steps)
    _barrier(dist)
    g1 = (gk("guess_kept"), gk("guess_tried"))
    ms_max = _allreduce(dist, ms, _max_op())
    years = _allreduce(dist, sum((st["t"] - t0_) / YR for st, t0_ in zip(stats, t_start)), _sum_op())
    value = years / (ms_max / 3.6e6)
    # the same number of steps, member after member (each with its own step graph)
    t_seq = [s.scalar("t") for s in solvers]
    seq_ms = 0.0
    for s in solvers:
        seq_ms += s.run(args.steps)["gpu_ms"]
    seq_ms_max = _allreduce(dist, seq_ms, _max_op())
    seq_years = _allreduce(dist, sum((s.scalar("t") - t) / YR for s, t in zip(solvers, t_seq)), _sum_op())
    cnt = lambda key: int(_allreduce(dist, sum(st[key] for st in stats), _sum_op()))
    qs, dyn, cg, solves = cnt("qs_steps"), cnt("dyn_steps"), cnt("cg_iters"), cnt("qs_solves")
    line = {"metric": "ensemble sim-years/hr", "value": value, "unit": "sim-years/hr", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / max(args.steps, 1),
            "higher_is_better": True, "scaling": "strong", "members": len(cfgs_all),
            "members_rank0": len(solvers), "nodes_total": int(_allreduce(dist, nodes, _sum_op())),
            "qs_steps": qs, "dyn_steps": dyn, "cg_iters_per_solve": cg / max(1, solves),
            "sequential": {"value": seq_years / (seq_ms_max / 3.6e6), "ms_per_step": seq_ms_max / max(args.steps, 1)},
            "setup_s": setup_s,
            "config": {"workload": f"{len(solvers)} damage-zone models, 120x60 to 480x240 elements, seeded "
                                   f"parameters; one graph launch per ensemble step; mixed precision, "
                                   + ("learned guess (each member's own network, trained on its first "
                                      f"{args.learn_steps} quasi-static steps)" if learned else "extrapolated guess")}}
    if learned:
        line["learned"] = {"pairs_rank0": pairs, "train_s_rank0": train_s,   # the timed steps' guesses
                           "guess_kept": int(_allreduce(dist, g1[0] - g0[0], _sum_op())),
                           "guess_tried": int(_allreduce(dist, g1[1] - g0[1], _sum_op()))}
    E.close()
    for s in solvers:
        s.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_cycle(args):
    """Whole earthquake cycles, quasi-static and dynamic phases: the plain FP64 method and the mixed
    method (extrapolated guess, autotuned smoother) each run the model for --years simulated years
    (or until --cycle-budget seconds of wall time), then their event catalogues are compared
    (recurrence interval, coseismic slip, hypocentre depth)."""
    from eqcycle_gb300 import EQC_FP64, EQC_GUESS_EXTRAPOLATE, EQC_GUESS_PREVIOUS, EQC_MIXED, Solver, preset, \
        set_parameters
    from eqcycle_gb300.events import catalogue, compare
    wl = args.workload or "homog48"
    cfg = preset(wl)
    P = set_parameters(cfg)
    t_end = (args.years or cfg.total_years) * YR
    mu = cfg.rho1 * cfg.vs1 ** 2
    out, cats = {}, {}
    for name, prec, guess in (("plain_fp64", EQC_FP64, EQC_GUESS_PREVIOUS), ("mixed", EQC_MIXED, EQC_GUESS_EXTRAPOLATE)):
        with Solver(P, precision=prec, cg_tol=1e-8, guess=guess) as s:
            s.init(cfg.V_init)
            gpu_ms, qs, dyn, cg, solves, wall0 = 0.0, 0, 0, 0, 0, time.time()
            tuned = None
            while s.scalar("t") < t_end and time.time() - wall0 < args.cycle_budget:
                st = s.run(2000, t_end)
                gpu_ms += st["gpu_ms"]
                qs += st["qs_steps"]
                dyn += st["dyn_steps"]
                cg += st["cg_iters"]
                solves += st["qs_solves"]
                if prec == EQC_MIXED and tuned is None and qs >= 20:
                    tuned = s.autotune(reps=2)
            years = s.scalar("t") / YR
            res = s.results()
        cat = catalogue(res, P.farray.FltX, mu)
        cats[name] = cat
        out[name] = {"sim_years": years_run, "value": years_run / (gpu_ms / 3.6e6) if gpu_ms else None,
                     "gpu_s": gpu_ms / 1e3, "wall_s": time.time() - wall0, "qs_steps": qs, "dyn_steps": dyn,
                     "cg_iters_per_solve": cg / max(solves, 1), "autotune": tuned, **cat.summary()}
    line = {"metric": "sim-years/hr over whole cycles", "workload": wl, "years_target": t_end / YR,
            "plain_fp64": out["plain_fp64"], "mixed": out["mixed"],
            "event_statistics_mixed_vs_fp64": compare(cats["plain_fp64"], cats["mixed"])}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=None, help="dz480 (default), dz960, homog48 (--cycle default), ...")
    ap.add_argument("--cpu-budget", type=float, default=240.0,
                    help="host-core sample of the reference algorithm: wall seconds (whole QS steps)")
    ap.add_argument("--cpu-min-steps", type=int, default=2, help="... and at least this many steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cycle", action="store_true",
                    help="default run without the whole-cycle and mixed-error legs")
    ap.add_argument("--cycle-leg-budget", type=float, default=300.0,
                    help="default run: wall seconds per method of the whole-cycle leg")
    ap.add_argument("--cycle-leg-years", type=float, default=20.0,
                    help="default run: simulated years of the whole-cycle leg (from the seeded start)")
    ap.add_argument("--kernel-only", action="store_true", help="time the stiffness apply alone")
    ap.add_argument("--setup", action="store_true", help="time the model setup, host against device")
    ap.add_argument("--profile-steps", action="store_true",
                    help="host-driven headline steps with the solver settings below, for an ncu launch list")
    ap.add_argument("--dynamic", action="store_true", help="with --profile-steps: dynamic (Newmark) steps")
    ap.add_argument("--graphs", action="store_true", help="with --profile-steps: graph-replayed (batched) steps")
    ap.add_argument("--mg-degree", type=int, default=0, help="with --profile-steps: SEM-level Chebyshev degree")
    ap.add_argument("--mg-degree-coarse", type=int, default=0, help="with --profile-steps: vertex-level degree")
    ap.add_argument("--reliable-delta", type=float, default=0.0, help="with --profile-steps: update factor")
    ap.add_argument("--dtype", default="both", choices=["both", "f32", "f64"])
    ap.add_argument("--nrep", type=int, default=20)
    ap.add_argument("--learned", action="store_true", help="learned initial guess: train and evaluate")
    ap.add_argument("--ensemble", action="store_true", help="batched ensemble of uneven fault models")
    ap.add_argument("--cycle", action="store_true", help="whole cycles: sim-years/hr and event statistics")
    ap.add_argument("--years", type=float, default=0.0, help="--cycle: simulated years (default: the workload's)")
    ap.add_argument("--cycle-budget", type=float, default=600.0, help="--cycle: wall seconds per method")
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--ensemble-guess", default="extrapolate", choices=["extrapolate", "learned"],
                    help="--ensemble: the members' initial guess")
    ap.add_argument("--learn-steps", type=int, default=60,
                    help="--ensemble --ensemble-guess learned: logged quasi-static steps per member before training")
    ap.add_argument("--no-graphs", action="store_true",
                    help="headline leg without CUDA graphs (host-driven steps; for per-kernel profiling)")
    ap.add_argument("--pairs", type=int, default=2400, help="--learned: training pairs over 8 seeds")
    ap.add_argument("--learned-pairs", type=int, default=480,
                    help="training pairs (8 seeds) for the learned-guess leg of the default run (0: skip)")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--apply-variant", type=int, default=0,
                    help="stiffness apply kernel: 0 default, 1 one tile per CTA (TMA), 2 plain tile loads, "
                         "3 persistent TMA pipeline, 4-7 element per lane with 4/8/12/6 rows per CTA, 8 TMA walk")
    args = ap.parse_args()
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != ws:
        # one process per GPU: N > 1 ranks come from torchrun, which sets WORLD_SIZE
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={ws}; for N > 1 launch one rank per GPU with "
                 f"python -m torch.distributed.run --nnodes=1 --nproc-per-node {args.gpus} "
                 f"--master-addr 127.0.0.1 --master-port <port> bench.py --gpus {args.gpus} ...")
    if args.workload is None and not args.cycle:
        args.workload = "dz480"
    if args.kernel_only:
        bench_kernel(args)
    elif args.setup:
        bench_setup(args)
    elif args.profile_steps:
        bench_profile_steps(args)
    elif args.learned:
        bench_learned(args)
    elif args.ensemble:
        bench_ensemble(args)
    elif args.cycle:
        bench_cycle(args)
    elif args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
