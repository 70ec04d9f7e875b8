"""Benchmark of the orbit-integration hot path (one JSON line on rank 0).

Default workload (the headline configuration): MilkyWayPotential, 262,144
orbits, radii log-uniform 0.5-100 kpc, Dopri5 with the PID controller (rtol 1e-8,
atol 1e-10, max_steps 2**16), per-orbit durations log-uniform 0.1-5 Gyr and
10-1000 saves per orbit, all in one persistent launch. One "step" is one pass
of the integrator over the whole batch. Metric: orbit-steps/s = accepted RK
steps (counted by the kernel) per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload uneven|plain|grad] [--orbits N]

--impl reference times the reference path's CPU implementation on the host
cores: galax itself needs JAX, which is absent, so this is the C++ FP64
restatement of the same arithmetic (oracle/), with every host thread.
Multi-GPU: orbits shard across ranks with no collective (weak scaling).
"""

from __future__ import annotations

import argparse
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

WORKLOADS = {
    "uneven": "batched uneven plain: MilkyWayPotential, Dopri5 PID rtol=1e-8 atol=1e-10 max_steps=2**16, "
              "radii log-uniform 0.5-100 kpc, durations log-uniform 0.1-5 Gyr, 10-1000 saves/orbit, "
              "one persistent launch",
    "plain": "plain small: MilkyWayPotential, Dopri8 fixed dt=1 Myr over 1 Gyr, 100 uniform saves",
    "train": "surrogate training alone: MLP 3-256-256-256-256-1 SiLU fitted to the subhalo remainder beyond "
             "12 kpc (potential and gradient, exact second-order loss gradient, Adam), batch 8192, "
             "one CUDA graph per step, tensor-core products (bf16, split bf16x3 where FP32 accuracy is needed)",
    "subhalos": "plain FP64 direct sum: MilkyWayPotential + 512 Plummer subhalos (the learned surrogate's tables), "
                "Dopri5 fixed dt=1 Myr over 1 Gyr, disk-like orbits at 4-20 kpc, final state saved",
    "grad": "differentiation: MilkyWayPotential, Dopri8 fixed dt=0.5 Myr over 2 Gyr, squared-distance loss, "
            "adjoint with checkpoints every 256 steps",
    "surrogate": "learned surrogate: MilkyWayPotential + 512 Plummer subhalos (m log-uniform 1e6-1e8 Msun, "
                 "r_s U(0.1,1) kpc, centres at U(5,50) kpc); MLP 3-256-256-256-256-1 SiLU on the subhalo part "
                 "beyond a C2 taper of radius 12 kpc (the part inside summed directly from cell lists: FP64 offsets "
                 "and accumulation, FP32 terms), "
                 "BF16 weights, FP32 accumulation, trained on 4M FP64 samples; Dopri5 dt=1 Myr over 1 Gyr",
    "stream": "stream-like batched gradient: Plummer progenitor (1e5 Msun, b=0.02 kpc) at 20 kpc apocentre in "
              "MilkyWayPotential, integrated back 3 Gyr; 3,000 release times (King tidal radius), 2 particles each "
              "with seeded Gaussian offsets (0.1 r_t, 0.1 v_circ); 6,000 particles to the present in MW + moving "
              "progenitor, Dopri8 dt=1 Myr; adjoint of a summed squared track residual w.r.t. all 12 MW parameters "
              "(halo m and r_s among them), through particles, release map and progenitor orbit",
    "mlp": "surrogate MLP inference alone: forward + input gradient of 3-256-256-256-256-1 SiLU at n points "
           "(random weights), fused tensor-core kernel",
}
DEFAULT_ORBITS = {"uneven": 262_144, "plain": 1024, "subhalos": 65_536, "grad": 65_536, "surrogate": 1_048_576,
                  "mlp": 1_048_576, "stream": 3000, "train": 0}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:  # noqa: BLE001
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:  # noqa: BLE001
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
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
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak() -> dict:
    """Measured FP64 FMA throughput of this GPU (MEASURED_PEAKS.json has no FP64 entry)."""
    import ctypes as C

    import torch

    from galax_gb300 import _lib

    L = _lib.load()
    ms, fl = C.c_double(), C.c_double()
    best = 0.0
    for _ in range(3):
        _lib.check(L.gal_fp64_peak_probe(20000, C.byref(ms), C.byref(fl), torch.cuda.current_stream().cuda_stream),
                   "gal_fp64_peak_probe")
        best = max(best, fl.value / (ms.value * 1e-3))
    import torch

    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    mhz = measured_peaks().get("sm_max_mhz") or 2070.0
    # issue ceiling: one FP64 FMA (2 flops) per SM sub-partition every other clock
    ceiling = props.multi_processor_count * 4 * mhz * 1e6 / 1e12
    return {"tflops": best / 1e12, "issue_ceiling_tflops": ceiling,
            "how": "dependent-chain DFMA probe, 8 chains/thread, full-device grid, best of 3; issue ceiling = "
                   "SMs x 4 flop/clk x max SM clock"}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:  # noqa: BLE001
        return {}


def flops_per_step(method: int) -> int:
    from galax_gb300.flops import STEP_FLOPS_MW

    return STEP_FLOPS_MW[method]


# ------------------------------------------------------------------ workloads
def make_uneven(n: int, seed: int):
    import galax_gb300 as gx
    from galax_gb300 import workloads as W

    mw = gx.MilkyWayPotential()
    return mw, W.uneven_ics(lambda x: mw.gradient(x), n, seed=seed)


def run_ours(args) -> dict | None:
    import torch

    import galax_gb300 as gx
    from galax_gb300 import _lib
    from galax_gb300.dynamics import Workspace, integrate

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    n = args.orbits or DEFAULT_ORBITS[args.workload]
    if args.workload == "grad":
        return run_grad(args, n, rank, world, dist)
    if args.workload == "plain":
        return run_plain(args, n, rank, world, dist)
    if args.workload == "subhalos":
        return run_subhalos(args, n, rank, world, dist)
    if args.workload == "train":
        return run_train(args, rank, world, dist)
    if args.workload == "surrogate":
        return run_surrogate(args, n, rank, world, dist)
    if args.workload == "mlp":
        return run_mlp(args, n, rank, world, dist)
    if args.workload == "stream":
        return run_stream(args, n, rank, world, dist)
    mw, b = make_uneven(n, seed=1 + rank)  # weak scaling: every rank its own shard
    solver = gx.Dopri8() if args.method == 8 else gx.Dopri5()
    cfg = gx.Integrator(solver=solver, stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                        max_steps=2**16).config()
    dev = "cuda"
    y0 = torch.as_tensor(b.y0, device=dev).t().contiguous()
    t0 = torch.as_tensor(b.t0, device=dev)
    t1 = torch.as_tensor(b.t1, device=dev)
    offs = torch.as_tensor(b.save_offsets, device=dev)
    sts = torch.as_tensor(b.save_ts, device=dev)
    total_saves = int(b.save_offsets[-1])
    ws = Workspace()
    stream = torch.cuda.current_stream()

    def longest_first(y0_, t0_, t1_):
        # hand-out order for the first pass: cost estimate = duration x local
        # orbital frequency sqrt(|grad Phi| / r), longest first (part of every
        # timed step: one gradient kernel and a device sort)
        r = torch.linalg.vector_norm(y0_[:3], dim=0)
        a = torch.linalg.vector_norm(mw.gradient(y0_[:3].t()), dim=1)
        return torch.argsort((t1_ - t0_).abs() * torch.sqrt(a / r), descending=True).to(torch.int32)

    def step():
        order = longest_first(y0, t0, t1)
        return integrate(mw, y0, t0, t1, sts, cfg, save_offsets=offs, order=order, soa=True, workspace=ws)

    out, status, steps = step()  # first call: lazy set-up outside any measurement
    torch.cuda.synchronize()
    tuning = None
    if not args.no_autotune:
        from galax_gb300.autotune import tune

        tuning = tune(step, 5, True)
    for _ in range(args.warmup):
        out, status, steps = step()
    torch.cuda.synchronize()
    accepted = int(steps.sum())
    n_bad = int((status != 0).sum())
    del out
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    team_blocks = (tuning or {}).get("best", {}).get("team_blocks", 32)  # the library's default is 32
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        out, status, steps = step()
        launches += 1
    e1.record(stream)
    torch.cuda.synchronize()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms = ms_total / args.steps
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
        acc_t = torch.tensor([accepted], device=dev, dtype=torch.float64)
        dist.all_reduce(acc_t)
        accepted_all = float(acc_t)
    else:
        accepted_all = accepted
    value = accepted_all / (ms * 1e-3)

    # ---- end to end through the public call with pinned host buffers
    h_y0 = torch.as_tensor(b.y0.T.copy()).pin_memory()
    h_t0 = torch.as_tensor(b.t0).pin_memory()
    h_t1 = torch.as_tensor(b.t1).pin_memory()
    h_offs = torch.as_tensor(b.save_offsets).pin_memory()
    h_ts = torch.as_tensor(b.save_ts).pin_memory()
    h_out = torch.empty((6, total_saves), dtype=torch.float64).pin_memory()
    h_status = torch.empty(n, dtype=torch.int32).pin_memory()
    h2d = sum(x.numel() * x.element_size() for x in (h_y0, h_t0, h_t1, h_offs, h_ts))
    d2h = h_out.numel() * 8 + h_status.numel() * 4

    def e2e_step():
        # the initial states and spans are copied in; the save grid (1 GB) is
        # read by the kernels in place from pinned host memory, and saves and
        # statuses are written straight into pinned host buffers (device-visible
        # host memory), so both large transfers overlap the integration
        dy0 = h_y0.to(dev, non_blocking=True)
        dt0 = h_t0.to(dev, non_blocking=True)
        dt1 = h_t1.to(dev, non_blocking=True)
        order = longest_first(dy0, dt0, dt1)
        return integrate(mw, dy0, dt0, dt1, h_ts, cfg, save_offsets=h_offs, order=order, soa=True, workspace=ws,
                         out=h_out, status=h_status)[2]

    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_start = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e_acc = e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t_start) * 1e3 / e2e_steps
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t)
    e2e_value = accepted_all / (e2e_ms * 1e-3)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return None
    peak = fp64_peak()
    f_step = flops_per_step(args.method)
    achieved = accepted * f_step / (ms * 1e-3) / 1e12
    traffic = traffic_from_profiles()
    save_bytes = total_saves * 6 * 8
    line = {
        "metric": "orbit-steps/s", "value": value, "unit": "orbit-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy, galactic units)",
        "config": {"workload": WORKLOADS["uneven"].replace("Dopri5", f"Dopri{args.method}"), "orbits_per_gpu": n,
                   "accepted_steps_per_gpu": accepted,
                   "orbits_not_finished": n_bad, "saves_per_gpu": total_saves,
                   "save_bytes_per_step": save_bytes,
                   "l2": "inputs larger than L2: 1.0 GB save-time grid read and 6.3 GB of saves written per step",
                   "parallelism": f"orbit shards x{world}, no collective",
                   "schedule": "two passes, longest remaining work first", "launch_autotune": tuning},
        "e2e": {"value": e2e_value, "unit": "orbit-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "path": "pinned host -> gal_integrate -> pinned host (initial states "
                                                "copied in; save grid read and saves written by the kernels in "
                                                "device-visible pinned memory)"},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak["tflops"], "unit": "TFLOP/s",
                     "issue_ceiling": peak["issue_ceiling_tflops"],
                     "frac_of_issue_ceiling": achieved / peak["issue_ceiling_tflops"],
                     "frac": achieved / peak["tflops"], "traffic": traffic,
                     "flops_per_accepted_step": f_step,
                     "note": "FP64 pipe bound; achieved counts accepted steps only (rejected attempts, saves and "
                             "initial-step selection are extra work, so frac is a lower bound); peak measured live "
                             "(" + peak["how"] + ")",
                     "hbm": {"achieved_gbs": save_bytes / (ms * 1e-3) / 1e9,
                             "peak_gbs": measured_peaks().get("hbm_gbs"),
                             "note": "save writes only; of measured"}},
        "clocks": clk,
        # per step: the gradient kernel of the hand-out order, the first pass,
        # three ordering kernels and the second pass (one launch, or two when
        # the longest orbits go to four-warp teams)
        "gpu_launches": launches * (1 + ((6 if team_blocks > 0 else 5) if cfg.schedule else 1)),
    }
    # the CPU baseline, full-size parity and the other workloads go with the headline (Dopri5) line
    if world == 1 and not args.no_cpu_baseline and args.method == 5:
        line["cpu_baseline"], sample = cpu_baseline(b, target_s=args.cpu_seconds)
        line["parity"] = parity_at_full_size(b, sample, h_out.numpy(), h_status.numpy(), e2e_acc.cpu().numpy())
    if world == 1 and args.extras and args.method == 5:
        line["extra"] = run_extras(args)
    if dist:
        dist.destroy_process_group()
    return line


def parity_at_full_size(b, sample, out_gpu, status_gpu, acc_gpu, rtol: float = 1e-8) -> dict:
    """The CPU-baseline leg's oracle orbits against the GPU saves of the same
    orbits from the end-to-end run of the full batch: per orbit, the largest
    relative position and velocity error over its saves (|dq|/|q|, |dv|/|v|),
    and whether the accepted-step counts are equal."""
    idx, saves_o, st_o, acc_o = sample
    offs = b.save_offsets
    lens = offs[idx + 1] - offs[idx]
    pos = np.repeat(offs[idx] - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens) + np.arange(int(lens.sum()))
    g = out_gpu[:, pos].T  # (saves, 6), the oracle's order
    err = np.zeros(len(g))
    for sl in (slice(0, 3), slice(3, 6)):
        d = np.linalg.norm(g[:, sl] - saves_o[:, sl], axis=1)
        err = np.maximum(err, d / np.maximum(np.linalg.norm(saves_o[:, sl], axis=1), 1e-300))
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    per_orbit = np.maximum.reduceat(err, starts) if len(err) else np.zeros(0)
    same = acc_gpu[idx] == acc_o
    worst = int(np.argmax(per_orbit))
    sensitivity = _sensitivity(b, idx, per_orbit, saves_o, starts, lens, 10 * rtol)
    return {
        "orbits_compared": int(len(idx)), "saves_compared": int(len(g)),
        "max_rel": float(per_orbit.max()), "median_rel": float(np.median(per_orbit)),
        "p999_rel": float(np.quantile(per_orbit, 0.999)),
        "within_10x_rtol": float(np.mean(per_orbit <= 10 * rtol)),
        "identical_step_sequences": float(np.mean(same)),
        "max_rel_where_step_counts_equal": float(per_orbit[same].max()) if same.any() else None,
        "status_equal": bool(np.array_equal(status_gpu[idx], st_o)),
        "worst_orbit": {"accepted_steps": int(acc_o[worst]), "rel": float(per_orbit[worst])},
        "longest_orbit_compared": {"accepted_steps": int(acc_o.max()),
                                   "rel": float(per_orbit[int(np.argmax(acc_o))])},
        "orbits_over_40k_steps": int(np.sum(acc_o > 40_000)),
        "sensitivity_control": sensitivity,
        "note": "oracle = C++ FP64 restatement (per-orbit PID controllers); GPU saves from the end-to-end run; "
                "identical_step_sequences = equal accepted-step counts; tolerance 10 x rtol = 1e-7",
    }


def _sensitivity(b, idx, per_orbit, saves_o, starts, lens, tol, n_control: int = 2000) -> dict:
    """Whether the orbits beyond tolerance are ones whose saves the oracle itself
    cannot pin: each is integrated again on the oracle from its initial state
    with every coordinate moved by one unit in the last place (a relative
    2**-52), and compared with the oracle's unperturbed run. An orbit whose
    saves move by more than the tolerance under that perturbation amplifies
    rounding (chaotic, or close encounters with the nucleus), so no FP64
    implementation with a different rounding sequence can match it to the
    tolerance. A random sample of the orbits within tolerance is the control."""
    from oracle import oracle as O

    cfg = O.solver_cfg(5, True, rtol=1e-8, atol=1e-10, max_steps=2**16)
    bad = np.nonzero(per_orbit > tol)[0]
    good = np.nonzero(per_orbit <= tol)[0]
    rng = np.random.default_rng(7)
    ctrl = rng.choice(good, min(n_control, len(good)), replace=False) if len(good) else good

    def moved(sel):
        if len(sel) == 0:
            return np.zeros(0)
        o = idx[sel]
        y0 = b.y0[o] * (1.0 + 2.0**-52)
        grids = [b.save_ts[b.save_offsets[i]:b.save_offsets[i + 1]] for i in o]
        sv, *_ = O.integrate(O.milky_way(), y0, b.t0[o], b.t1[o], grids, cfg, nthreads=os.cpu_count() or 1,
                             flat=True)
        ref = np.concatenate([saves_o[starts[j]:starts[j] + lens[j]] for j in sel])
        err = np.zeros(len(ref))
        for sl in (slice(0, 3), slice(3, 6)):
            d = np.linalg.norm(sv[:, sl] - ref[:, sl], axis=1)
            err = np.maximum(err, d / np.maximum(np.linalg.norm(ref[:, sl], axis=1), 1e-300))
        st = np.concatenate([[0], np.cumsum(lens[sel])[:-1]])
        return np.maximum.reduceat(err, st)

    mb, mc = moved(bad), moved(ctrl)
    return {
        "orbits_beyond_tolerance": int(len(bad)),
        "of_which_oracle_moves_beyond_tolerance_under_1ulp": float(np.mean(mb > tol)) if len(mb) else None,
        "median_oracle_1ulp_divergence_of_those": float(np.median(mb)) if len(mb) else None,
        "control_orbits": int(len(ctrl)),
        "control_oracle_moves_beyond_tolerance_under_1ulp": float(np.mean(mc > tol)) if len(mc) else None,
    }


def run_uneven_dopri8(steps: int = 2, warmup: int = 1) -> dict:
    """The headline batch (262,144 uneven orbits, PID rtol 1e-8 atol 1e-10) with
    Dopri8, galax's default method, with the longest orbits on four-warp teams
    (team SM count and split fraction picked by the autotuner, launch shape the
    library's) and, once, without them."""
    import torch

    import galax_gb300 as gx
    from galax_gb300 import _lib
    from galax_gb300.dynamics import Workspace, integrate
    from galax_gb300.flops import STEP_FLOPS_MW

    mw, b = make_uneven(DEFAULT_ORBITS["uneven"], seed=1)
    cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                        max_steps=2**16).config()
    dev = "cuda"
    y0 = torch.as_tensor(b.y0, device=dev).t().contiguous()
    t0, t1 = torch.as_tensor(b.t0, device=dev), torch.as_tensor(b.t1, device=dev)
    offs, sts = torch.as_tensor(b.save_offsets, device=dev), torch.as_tensor(b.save_ts, device=dev)
    ws = Workspace()
    stream = torch.cuda.current_stream()

    def step():
        r = torch.linalg.vector_norm(y0[:3], dim=0)
        a = torch.linalg.vector_norm(mw.gradient(y0[:3].t()), dim=1)
        order = torch.argsort((t1 - t0).abs() * torch.sqrt(a / r), descending=True).to(torch.int32)
        return integrate(mw, y0, t0, t1, sts, cfg, save_offsets=offs, order=order, soa=True, workspace=ws)

    from galax_gb300.autotune import tune

    L = _lib.load()
    step()  # first call: lazy set-up outside any measurement
    torch.cuda.synchronize()
    tuning = tune(step, 8, True, candidates=())
    team = tuning["best"]["team_blocks"]
    res = {}
    for blocks in (team, 0):
        _lib.check(L.gal_set_team(blocks), "gal_set_team")
        for _ in range(warmup):
            _, st, acc = step()
        ms = _timed(step, steps if blocks else 1, stream)
        res[blocks] = (ms, int(acc.sum()), int((st != 0).sum()))
    _lib.check(L.gal_set_team(32), "gal_set_team")  # the library's defaults again
    _lib.check(L.gal_set_split_fraction(0.1), "gal_set_split_fraction")
    ms, accepted, bad = res[team]
    peak = fp64_peak()
    achieved = accepted * STEP_FLOPS_MW[8] / (ms * 1e-3) / 1e12
    return {"metric": "orbit-steps/s", "value": accepted / (ms * 1e-3), "unit": "orbit-steps/s",
            "ms_per_step": ms, "steps": steps, "warmup": warmup,
            "config": {"workload": WORKLOADS["uneven"].replace("Dopri5", "Dopri8"), "accepted_steps": accepted,
                       "orbits_not_finished": bad, "autotune": tuning},
            "without_teams": {"ms_per_step": res[0][0], "value": res[0][1] / (res[0][0] * 1e-3)},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak["tflops"], "unit": "TFLOP/s",
                     "issue_ceiling": peak["issue_ceiling_tflops"],
                     "frac_of_issue_ceiling": achieved / peak["issue_ceiling_tflops"],
                         "frac": achieved / peak["tflops"], "flops_per_accepted_step": STEP_FLOPS_MW[8]}}


def run_extras(args) -> dict:
    """The other two parts of the metric on the same GPU, after the headline:
    gradients/s of the differentiation workload at full size, and the learned
    surrogate against the plain FP64 direct sum; and the headline batch with
    Dopri8."""
    import argparse as _ap

    out = {"uneven_dopri8": run_uneven_dopri8()}
    g = run_grad(_ap.Namespace(**{**vars(args), "steps": 2, "warmup": 3, "t1": 0.0}), DEFAULT_ORBITS["grad"], 0, 1,
                 None)
    out["grad"] = {k: g[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "config", "e2e",
                                     "roofline", "gpu_launches")}
    sg = run_surrogate(_ap.Namespace(**{**vars(args), "steps": 2, "warmup": 3}), DEFAULT_ORBITS["surrogate"], 0, 1,
                       None)
    out["surrogate"] = {k: sg[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "config",
                                           "plain_fp64_direct_sum", "speedup_vs_plain", "median_rel_pos_err_1gyr",
                                           "roofline", "gpu_launches")}
    return out


def _timed(fn, steps, stream):
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _max_over_ranks(x, dist):
    import torch

    if not dist:
        return x
    t = torch.tensor([x], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def run_grad(args, n, rank, world, dist) -> dict | None:
    """Differentiation workload: MW, Dopri8 dt=0.5 Myr over 2 Gyr, loss = sum of
    squared distances of the final points to perturbed targets, gradients with
    respect to the 6 initial conditions of every orbit and the component
    parameters, checkpoints every 256 steps. Metric: gradients (orbits) per second."""
    import torch

    import galax_gb300 as gx
    from galax_gb300 import workloads as W
    from galax_gb300.adjoint import _run as adjoint_run
    from galax_gb300.dynamics import integrate

    mw = gx.MilkyWayPotential()
    y0h = W.disk_like_ics(lambda x: mw.gradient(x), n, seed=2 + rank)
    dt, t1 = 0.5, float(args.t1 or 2000.0)
    cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=dt).config()
    y0 = torch.as_tensor(y0h, device="cuda").t().contiguous()
    out, _, _ = integrate(mw, y0, 0.0, t1, torch.tensor([t1]), cfg, soa=True)
    rng = np.random.default_rng(20 + rank)
    pert = np.concatenate([rng.normal(0, 0.1, (n, 3)), rng.normal(0, 2 * 0.001022712165045695, (n, 3))], axis=1)
    target = (out[:, 0, :] + torch.as_tensor(pert.T, device="cuda")).contiguous()
    stream = torch.cuda.current_stream()

    def step():
        return adjoint_run(mw, y0, 0.0, t1, dt, 8, 256, target_soa=target)

    for _ in range(args.warmup):
        step()
    if dist:
        dist.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms = _max_over_ranks(_timed(step, args.steps, stream), dist)
    clk = clocks.stop()
    yT, gy, gp = step()
    value = n * world / (ms * 1e-3)
    # end to end: pinned host inputs, gradients back to pinned host
    h_y0 = torch.as_tensor(y0h.T.copy()).pin_memory()
    h_tg = target.cpu().pin_memory()
    h_gy = torch.empty((6, n), dtype=torch.float64).pin_memory()
    h_gp = torch.empty((4, 3), dtype=torch.float64).pin_memory()

    def e2e():
        dy = h_y0.to("cuda", non_blocking=True)
        dtg = h_tg.to("cuda", non_blocking=True)
        _, g1, g2 = adjoint_run(mw, dy, 0.0, t1, dt, 8, 256, target_soa=dtg)
        h_gy.copy_(g1, non_blocking=True)
        h_gp.copy_(g2, non_blocking=True)

    e2e()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e()
    torch.cuda.synchronize()
    e2e_ms = _max_over_ranks((time.perf_counter() - t) * 1e3 / args.steps, dist)
    if rank != 0:
        return None
    from galax_gb300.flops import STEP_FLOPS_MW

    nsteps = int(round(t1 / dt))
    flops = n * nsteps * STEP_FLOPS_MW[8] * 4  # forward, segment recompute, stage recompute, reverse sweep
    peak = fp64_peak()
    achieved = flops / (ms * 1e-3) / 1e12
    return {
        "metric": "grads/s", "value": value, "unit": "grads/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded numpy, galactic units)",
        "config": {"workload": WORKLOADS["grad"], "orbits_per_gpu": n, "steps_per_orbit": nsteps,
                   "gradient": "6 initial conditions per orbit + (m, l1, l2) of the 4 components",
                   "l2": "checkpoints (n x 16 x 48 B) and segment buffer (n x 256 x 48 B = 0.8 GB) exceed L2"},
        "e2e": {"value": n * world / (e2e_ms * 1e-3), "unit": "grads/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 2 * 6 * n * 8, "d2h_bytes_per_step": 6 * n * 8 + 12 * 8},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak["tflops"], "unit": "TFLOP/s",
                     "issue_ceiling": peak["issue_ceiling_tflops"],
                     "frac_of_issue_ceiling": achieved / peak["issue_ceiling_tflops"],
                     "frac": achieved / peak["tflops"], "traffic": None,
                     "note": "algorithmic flops = 4 x Dopri8 forward step flops per step; peak measured live"},
        "clocks": clk, "gpu_launches": 2 * args.steps,
    }


def run_plain(args, n, rank, world, dist) -> dict | None:
    """Plain small workload: MW, 1,024 orbits, Dopri8 dt=1 Myr over 1 Gyr, 100 saves."""
    import torch

    import galax_gb300 as gx
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate

    mw = gx.MilkyWayPotential()
    y0h = W.disk_like_ics(lambda x: mw.gradient(x), n, seed=0 + rank)
    cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
    y0 = torch.as_tensor(y0h, device="cuda").t().contiguous()
    ts = torch.linspace(0, 1000, 100, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        return integrate(mw, y0, 0.0, 1000.0, ts, cfg, soa=True)

    for _ in range(args.warmup):
        step()
    ms = _max_over_ranks(_timed(step, args.steps, stream), dist)
    if rank != 0:
        return None
    value = n * world * 1000 / (ms * 1e-3)
    from galax_gb300.flops import STEP_FLOPS_MW

    peak = fp64_peak()
    achieved = n * 1000 * STEP_FLOPS_MW[8] / (ms * 1e-3) / 1e12
    return {"metric": "orbit-steps/s", "value": value, "unit": "orbit-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS["plain"], "orbits_per_gpu": n},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak["tflops"], "unit": "TFLOP/s",
                     "issue_ceiling": peak["issue_ceiling_tflops"],
                     "frac_of_issue_ceiling": achieved / peak["issue_ceiling_tflops"],
                         "frac": achieved / peak["tflops"],
                         "note": "1,024 orbits occupy 8 of 152 SMs: latency-bound by construction"},
            "gpu_launches": args.steps}


def subhalo_tables():
    """The Milky Way, the 512 Plummer subhalos, and both as one 516-component table."""
    import galax_gb300 as gx
    from galax_gb300 import workloads as W
    from galax_gb300.potential import from_component_array

    mw = gx.MilkyWayPotential()
    m, b, c = W.subhalo_table(3, 512)
    sub_arr = np.zeros(512, mw.component_array().dtype)
    sub_arr["kind"] = 4
    sub_arr["m"], sub_arr["l1"], sub_arr["origin"] = m, b, c
    return mw, from_component_array(sub_arr), from_component_array(np.concatenate([mw.component_array(), sub_arr]))


def run_subhalos(args, n, rank, world, dist) -> dict | None:
    """The plain FP64 direct sum over the 516-component table (the learned
    surrogate's denominator) on its own, with its FP64 roofline."""
    import torch

    import galax_gb300 as gx
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate
    from galax_gb300.flops import STEP_FLOPS_MW_SUBHALOS

    mw, _, full = subhalo_tables()
    y0 = torch.as_tensor(W.disk_like_ics(lambda x: mw.gradient(x), n, seed=31 + rank), device="cuda")
    dt, t1 = 1.0, args.t1 if args.t1 > 0 else 1000.0
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.ConstantStepSize(), dt0=dt).config()
    ys = y0.t().contiguous()
    ts = torch.tensor([t1], dtype=torch.float64)
    stream = torch.cuda.current_stream()

    def step():
        return integrate(full, ys, 0.0, t1, ts, cfg, soa=True)

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms = _max_over_ranks(_timed(step, args.steps, stream), dist)
    clk = clocks.stop()
    _, st, _ = step()
    if rank != 0:
        return None
    nsteps = int(round(t1 / dt))
    value = n * world * nsteps / (ms * 1e-3)
    peak = fp64_peak()
    achieved = n * nsteps * STEP_FLOPS_MW_SUBHALOS[5] / (ms * 1e-3) / 1e12
    return {"metric": "orbit-steps/s", "value": value, "unit": "orbit-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS["subhalos"].replace("1 Gyr", f"{t1:g} Myr"), "orbits_per_gpu": n,
                       "steps_per_orbit": nsteps, "orbits_not_finished": int((st != 0).sum())},
            "roofline": {"bound": "fp64", "kernel": "k_integrate_table", "achieved": achieved,
                         "peak": peak["tflops"], "unit": "TFLOP/s", "issue_ceiling": peak["issue_ceiling_tflops"],
                         "frac_of_issue_ceiling": achieved / peak["issue_ceiling_tflops"],
                         "frac": achieved / peak["tflops"], "flops_per_step": STEP_FLOPS_MW_SUBHALOS[5]},
            "clocks": clk, "gpu_launches": args.steps}


# algorithmic flops of one training step (batch b): 18 products of 2 b 256^2
# (forward 3, input gradient 3, second-order pass 6, weight gradients 6 terms)
# plus the 3-wide and 1-wide first/last-layer products
def train_step_flops(b: int) -> float:
    return b * (18 * 2 * 256 * 256 + 6 * 2 * 3 * 256 + 4 * 2 * 256)


def run_train(args, rank, world, dist) -> dict | None:
    """Surrogate training alone: training steps/s of the device-driven loop
    (gal_mlp_train, one CUDA graph per step) on the surrogate workload's data."""
    import torch

    from galax_gb300 import surrogate as S
    from galax_gb300 import workloads as W

    _, sub, _ = subhalo_tables()
    npts, batch = args.train_points, 8192
    xt = torch.as_tensor(W.training_points(npts, seed=30), device="cuda")
    phi_t, g_t = sub.potential(xt), sub.gradient(xt)
    near = S.ShortRange(sub, args.split_radius) if args.split_radius > 0 else None
    if near is not None:
        ps, gs = near.evaluate(xt)
        phi_t, g_t = phi_t - ps, g_t - gs
    stream = torch.cuda.current_stream()

    def step():
        return S.train(xt, phi_t, g_t, length_scale=50.0, epochs=args.train_epochs, batch=batch, lr=2e-3)

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms = _max_over_ranks(_timed(step, args.steps, stream), dist)
    clk = clocks.stop()
    _, rep = step()
    if rank != 0:
        return None
    nsteps = (npts // batch) * args.train_epochs
    per_step_ms = ms / nsteps
    peaks = measured_peaks()
    achieved = train_step_flops(batch) / (per_step_ms * 1e-3) / 1e12
    return {"metric": "training steps/s", "value": world * nsteps / (ms * 1e-3), "unit": "steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 / bf16x3, f32 accumulate",
            "data": "synthetic", "ms_per_training_step": per_step_ms,
            "seconds_for_400_epochs_on_4M_points": per_step_ms * 1e-3 * (4_194_304 // batch) * 400,
            "config": {"workload": WORKLOADS["train"], "train_points": npts, "train_epochs": args.train_epochs,
                       "batch": batch, "training_steps_per_bench_step": nsteps,
                       "loss_first_last": [rep.loss[0], rep.loss[-1]]},
            "roofline": {"bound": "latency (kernel chain)", "achieved": achieved, "peak": peaks.get("bf16_tflops"),
                         "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                         "flops_per_training_step": train_step_flops(batch),
                         "note": "algorithmic flops; the 8192-row products are too small to fill the tensor cores, so "
                                 "the step is set by its chain of ~25 dependent kernels"},
            # per training step: gather, 9 forward/input-gradient kernels (first layer with the weight
            # images, 6 products, 2 row sums), 22 of the second-order pass (9 products, 3 two-term
            # weight-gradient products and their 3 split-K sums, 7 column-sum and loss kernels), Adam
            # and the step counter
            "clocks": clk, "gpu_launches": args.steps * nsteps * 34}


def run_surrogate(args, n, rank, world, dist) -> dict | None:
    """Learned-surrogate workload: orbit-steps/s of the surrogate path (analytic Milky
    Way in FP64 + MLP subhalo term on the tensor cores) against the plain FP64
    direct sum over all 516 components, and the surrogate's median relative
    position error after 1 Gyr (measured against the plain path)."""
    import torch

    import galax_gb300 as gx
    from galax_gb300 import surrogate as S
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate
    from galax_gb300.flops import STEP_FLOPS_MW_SUBHALOS

    mw, sub, full = subhalo_tables()
    # training set: positions log-uniform in radius, FP64 targets from the direct sum;
    # with a split radius the MLP learns only the long-range remainder and the
    # short-range part is summed exactly along the orbits
    npts = args.train_points
    xt = torch.as_tensor(W.training_points(npts, seed=30), device="cuda")
    phi_t, g_t = sub.potential(xt), sub.gradient(xt)
    near = S.ShortRange(sub, args.split_radius) if args.split_radius > 0 else None
    if near is not None:
        ps, gs = near.evaluate(xt)
        phi_t, g_t = phi_t - ps, g_t - gs
    torch.cuda.synchronize()
    t = time.perf_counter()
    mlp, rep = S.train(xt, phi_t, g_t, length_scale=50.0, epochs=args.train_epochs, batch=8192, lr=2e-3)
    train_s = time.perf_counter() - t
    # initial conditions as the small plain workload, radii 4-20 kpc
    y0 = torch.as_tensor(W.disk_like_ics(lambda x: mw.gradient(x), n, seed=31 + rank), device="cuda")
    dt, t1 = 1.0, 1000.0
    stream = torch.cuda.current_stream()

    def surrogate_step():
        return S.integrate(mw, mlp, y0, 0.0, t1, dt, near=near)

    for _ in range(args.warmup):
        surrogate_step()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms = _max_over_ranks(_timed(surrogate_step, args.steps, stream), dist)
    clk = clocks.stop()
    yT_sur = surrogate_step()
    nsteps = int(round(t1 / dt))
    value = n * world * nsteps / (ms * 1e-3)
    # MLP kernel alone on 1M points (one stage evaluation)
    xq = y0[:, :3].t().contiguous()
    mlp.evaluate(xq.t())
    mlp_ms = _timed(lambda: mlp.evaluate(xq.t()), 10, stream)
    mlp_flops = 2.0 * (3 * 256 * 2 + 6 * 256 * 256 + 256)  # forward + input gradient per point
    # plain FP64 direct sum over all 516 components, on a subsample
    ns = min(n, args.plain_orbits)
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.ConstantStepSize(), dt0=dt).config()
    ys = y0[:ns].t().contiguous()

    def plain_step():
        return integrate(full, ys, 0.0, t1, torch.tensor([t1]), cfg, soa=True)

    plain_step()
    plain_ms = _timed(plain_step, 1, stream)
    out, st, _ = plain_step()
    yT_plain = out[:, 0, :].t()
    yT_mw = S.integrate(mw, None, y0[:ns], 0.0, t1, dt)
    err = lambda a: (torch.linalg.vector_norm(a[:, :3] - yT_plain[:, :3], dim=1)  # noqa: E731
                     / torch.linalg.vector_norm(yT_plain[:, :3], dim=1))
    e_sur = err(yT_sur[:ns])
    e_mw = err(yT_mw)
    plain_value = ns * nsteps / (plain_ms * 1e-3)
    if rank != 0:
        return None
    peaks = measured_peaks()
    achieved_tf = n * mlp_flops / (mlp_ms * 1e-3) / 1e12
    return {
        "metric": "orbit-steps/s (surrogate)", "value": value, "unit": "orbit-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 state, bf16 MLP", "data": "synthetic",
        "config": {"workload": WORKLOADS["surrogate"], "orbits_per_gpu": n, "steps_per_orbit": nsteps,
                   "train_points": npts, "train_epochs": args.train_epochs, "train_seconds": round(train_s, 2),
                   "split_radius_kpc": args.split_radius,
                   "train_loss_first_last": [rep.loss[0], rep.loss[-1]]},
        "plain_fp64_direct_sum": {"value": plain_value, "unit": "orbit-steps/s", "orbits": ns, "ms": plain_ms,
                                  "fp64_tflops": plain_value * STEP_FLOPS_MW_SUBHALOS[5] / 1e12,
                                  "frac_of_fp64_probe": plain_value * STEP_FLOPS_MW_SUBHALOS[5] / 1e12
                                  / fp64_peak()["tflops"]},
        "speedup_vs_plain": value / plain_value,
        "median_rel_pos_err_1gyr": {"surrogate": float(e_sur.median()), "analytic_mw_only": float(e_mw.median()),
                                    "surrogate_p90": float(torch.quantile(e_sur, 0.9)),
                                    "measured_on_orbits": ns},
        "roofline": {"bound": "tensor", "kernel": "k_mlp_infer", "achieved": achieved_tf,
                     "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                     "frac": achieved_tf / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                     "traffic": None, "ms_per_1M_points": mlp_ms,
                     "note": "MLP forward + input gradient on 1,048,576 points, algorithmic flops; peak = measured "
                             "burst BF16 (cuBLAS) from MEASURED_PEAKS.json"},
        # per run: the first slope (stage kernel + MLP), then per step six stage kernels and six MLP launches
        "clocks": clk, "gpu_launches": args.steps * (2 + 2 * 6 * nsteps),
    }


def run_mlp(args, n, rank, world, dist) -> dict | None:
    """The tensor-core MLP kernel alone (one stage evaluation of the surrogate)."""
    import torch

    from galax_gb300 import surrogate as S

    mlp = S.MLPSurrogate(S.init_params(0), 50.0, 1e-3)
    rng = np.random.default_rng(1)
    x = torch.as_tensor(rng.normal(size=(n, 3)) * 20.0, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        mlp.evaluate(x)
    ms = _max_over_ranks(_timed(lambda: mlp.evaluate(x), args.steps, stream), dist)
    if rank != 0:
        return None
    flops = 2.0 * (3 * 256 * 2 + 6 * 256 * 256 + 256)
    achieved = n * flops / (ms * 1e-3) / 1e12
    peaks = measured_peaks()
    return {"metric": "MLP evaluations/s", "value": n * world / (ms * 1e-3), "unit": "points/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": WORKLOADS["mlp"], "points": n},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                         "frac": achieved / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None},
            "gpu_launches": args.steps}


def run_stream(args, n_rel, rank, world, dist) -> dict | None:
    """Stream-like batched gradient. One step = the whole pipeline: progenitor
    orbit (back, then forward), release map, 2 n_rel particles to the present,
    and the adjoint through all of it. Metric: stream gradients per second
    (each a full gradient of the track loss)."""
    import torch

    import galax_gb300 as gx
    from galax_gb300 import stream as ST
    from galax_gb300 import workloads as W
    from galax_gb300.flops import STEP_FLOPS_MW, STEP_FLOPS_MW_PLUMMER

    mw = gx.MilkyWayPotential()
    s = W.stream_setup(lambda x: mw.gradient(x), n_release=n_rel, seed=4 + rank)
    cfg = ST.config(n_release=n_rel, dt=s.dt, w_now=s.w_now, prog_m=s.prog_m, prog_b=s.prog_b, method=8,
                    k_ckpt=args.stream_ckpt)
    noise = torch.as_tensor(s.noise, device="cuda")
    base = ST.simulate(mw, cfg, noise)
    target = (base.final + torch.as_tensor(s.pert, device="cuda")).contiguous()
    stream = torch.cuda.current_stream()

    def step():
        return ST.gradient(mw, cfg, noise, target)

    def fwd():
        return ST.simulate(mw, cfg, noise)

    for _ in range(args.warmup):
        step()
    if dist:
        dist.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms = _max_over_ranks(_timed(step, args.steps, stream), dist)
    clk = clocks.stop()
    fwd_ms = _timed(fwd, max(1, args.steps), stream)
    g = step()
    # end to end: host noise and targets in, gradient and loss out
    h_noise = torch.as_tensor(s.noise).pin_memory()
    h_target = target.cpu().pin_memory()
    h_grad = torch.empty((4, 3), dtype=torch.float64).pin_memory()

    def e2e():
        r = ST.gradient(mw, cfg, h_noise.to("cuda", non_blocking=True), h_target.to("cuda", non_blocking=True))
        h_grad.copy_(r.grad_params, non_blocking=True)

    e2e()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e()
    torch.cuda.synchronize()
    e2e_ms = _max_over_ranks((time.perf_counter() - t) * 1e3 / args.steps, dist)
    if rank != 0:
        return None
    particle_steps = sum(2 * (n_rel - r) for r in range(n_rel))
    fwd_flops = particle_steps * STEP_FLOPS_MW_PLUMMER[8] + 2 * n_rel * STEP_FLOPS_MW[8]
    flops = 4 * fwd_flops  # forward, segment recompute, stage recompute, reverse sweep
    peak = fp64_peak()
    achieved = flops / (ms * 1e-3) / 1e12
    line = {
        "metric": "stream gradients/s", "value": world / (ms * 1e-3), "unit": "gradients/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy, galactic units)",
        "config": {"workload": WORKLOADS["stream"], "releases": n_rel, "particles": 2 * n_rel,
                   "particle_steps": particle_steps, "forward_ms": fwd_ms,
                   "forward_particle_steps_per_s": particle_steps / (fwd_ms * 1e-3),
                   "halo_grad_m_rs": [float(g.grad_params[1][0]), float(g.grad_params[1][1])],
                   "adjoint_storage": "every particle stage stored (k_ckpt=0)" if args.stream_ckpt == 0 else
                   f"checkpoints every {args.stream_ckpt} steps",
                   "l2": "each step recomputes everything from the inputs; stored stages (17 GB) and mu partials "
                         "(176 MB) exceed L2"},
        "e2e": {"value": world / (e2e_ms * 1e-3), "unit": "gradients/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(s.noise.size * 8 + target.numel() * 8), "d2h_bytes_per_step": 12 * 8},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak["tflops"], "unit": "TFLOP/s",
                     "issue_ceiling": peak["issue_ceiling_tflops"],
                     "frac_of_issue_ceiling": achieved / peak["issue_ceiling_tflops"],
                     "frac": achieved / peak["tflops"], "traffic": None,
                     "note": "algorithmic flops = 4 x forward (particle steps x 2,562 + progenitor 2 x n_rel x 2,276), "
                             "the checkpointed adjoint's count, kept as the unit of work for both storage modes; "
                             "6,000 particles fill 188 warps, and the progenitor is one serial orbit, so the "
                             "pipeline is bound by FP64 latency along its longest chains, not by the FP64 pipe"},
        # per gradient: progenitor, release map and particles forward; the particle adjoint (Hessians,
        # sweep and parameter terms when every stage is stored, one kernel when checkpointed); the
        # progenitor-cotangent reduction, release-map adjoint, progenitor Hessians, sweep and
        # parameter terms; the final reduction
        "clocks": clk, "gpu_launches": (3 + (3 if args.stream_ckpt == 0 else 1) + 5 + 1) * args.steps,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = stream_cpu_baseline(s)
    return line


def stream_cpu_baseline(s) -> dict:
    """The oracle's stream pipeline on every host core: one forward plus central
    differences in the halo mass and scale radius (4 more forwards)."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    comps = O.milky_way()
    t = time.perf_counter()
    base = O.stream_forward(comps, s, nthreads=cores)["final"]
    target = base + s.pert
    for ci, fld in ((1, "m"), (1, "l1")):
        for sgn in (1.0, -1.0):
            c2 = comps.copy()
            c2[ci][fld] *= 1.0 + sgn * 1e-5
            O.stream_loss(c2, s, target, nthreads=cores)
    dt = time.perf_counter() - t
    return {"value": 1.0 / dt, "unit": "gradients/s", "cores": cores, "kind": "port",
            "sample": f"one full stream gradient (forward + 4 forwards of central differences), {dt:.1f} s wall"}


def traffic_from_profiles():
    """DRAM bytes per launch of the integrate kernel, from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "integrate_dopri5_uneven.md")
    try:
        for ln in open(p):
            if ln.startswith("traffic_bytes_per_full_launch:"):
                return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def cpu_baseline(b, target_s: float = 15.0) -> dict:
    """The oracle (C++ FP64, OpenMP over orbits, all host threads) on a bounded
    sample of the same orbits; value = accepted steps per second."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    cfg = O.solver_cfg(5, True, rtol=1e-8, atol=1e-10, max_steps=2**16)
    comps = O.milky_way()
    rng = np.random.default_rng(99)
    idx_all = rng.permutation(len(b.t1))

    def run(idx):
        grids = [b.save_ts[b.save_offsets[i]:b.save_offsets[i + 1]] for i in idx]
        t = time.perf_counter()
        saves, st, acc, _ = O.integrate(comps, b.y0[idx], b.t0[idx], b.t1[idx], grids, cfg, nthreads=cores,
                                        flat=True)
        return time.perf_counter() - t, int(acc.sum()), (idx, saves, st, acc)

    m = max(64, 4 * cores)
    dt, acc, res = run(idx_all[:m])
    while dt < 1.0 and m < len(idx_all):
        m = min(len(idx_all), m * 4)
        dt, acc, res = run(idx_all[:m])
    m2 = int(min(len(idx_all), max(m, m * target_s / max(dt, 1e-3))))
    if m2 > m:
        dt, acc, res = run(idx_all[:m2])
        m = m2
    return ({"value": acc / dt, "unit": "orbit-steps/s", "cores": cores, "kind": "port",
             "sample": f"{m} randomly chosen orbits of the same workload ({acc} accepted steps, {dt:.1f} s wall)"},
            res)


def run_reference(args) -> dict | None:
    """CPU implementation of the path on the host cores (the oracle port; galax needs JAX, absent here)."""
    rank, _, world = dist_env()
    if rank != 0:
        return None
    from oracle import oracle as O
    from galax_gb300 import workloads as W

    n = args.orbits or DEFAULT_ORBITS["uneven"]
    b = W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), n, seed=1)
    cores = os.cpu_count() or 1
    cfg = O.solver_cfg(5, True, rtol=1e-8, atol=1e-10, max_steps=2**16)
    comps = O.milky_way()
    rng = np.random.default_rng(99)
    per_step = args.ref_orbits
    times, accs = [], []
    for i in range(args.warmup + args.steps):
        idx = rng.choice(n, per_step, replace=False)
        grids = [b.save_ts[b.save_offsets[j]:b.save_offsets[j + 1]] for j in idx]
        t = time.perf_counter()
        _, st, acc, _ = O.integrate(comps, b.y0[idx], b.t0[idx], b.t1[idx], grids, cfg, nthreads=cores)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            times.append(dt)
            accs.append(int(acc.sum()))
    value = sum(accs) / sum(times)
    sample = f"{per_step} random orbits of the workload per step, {cores} threads"
    return {"impl": "reference", "metric": "orbit-steps/s", "value": value, "unit": "orbit-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy, galactic units)",
            "config": {"workload": WORKLOADS["uneven"], "orbits_per_step": per_step},
            "cpu_baseline": {"value": value, "unit": "orbit-steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "orbit-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "galax (JAX) is not installed on this machine; this is the C++ FP64 restatement of its "
                    "orbit arithmetic (oracle/) on every host thread"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=tuple(WORKLOADS), default="uneven")
    ap.add_argument("--orbits", type=int, default=0)
    ap.add_argument("--method", type=int, choices=(5, 8), default=5,
                    help="uneven workload: Dopri5 (the headline) or Dopri8 (galax's default method)")
    ap.add_argument("--ref-orbits", type=int, default=8192)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--extras", action=argparse.BooleanOptionalAction, default=True,
                    help="uneven workload at one GPU: also measure the gradient and surrogate workloads")
    ap.add_argument("--t1", type=float, default=0.0, help="grad workload: end time in Myr (default 2000)")
    ap.add_argument("--train-points", type=int, default=4_194_304, help="surrogate workload: training samples")
    ap.add_argument("--train-epochs", type=int, default=400, help="surrogate workload: training epochs")
    ap.add_argument("--plain-orbits", type=int, default=65_536, help="surrogate workload: orbits for the plain path")
    ap.add_argument("--stream-ckpt", type=int, default=0,
                    help="stream workload: particle checkpoint interval (0 = store every stage, no recompute)")
    ap.add_argument("--split-radius", type=float, default=12.0,
                    help="surrogate workload: short-range split radius in kpc (0 = the MLP learns the whole sum)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
