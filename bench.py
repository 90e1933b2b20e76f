"""Benchmark of the Poisson solve loop on GB300 (one JSON line on stdout).

Metric: time to ||r||/||b|| <= 1e-10 at 512^3 (plain FP64 vs mixed precision),
with HBM GB/s of the dominant kernel.  Workload: 512^3 unknowns, Dirichlet 0, b = -f
with f a seeded unit-RMS Gaussian random field, P(k) ~ k^-2 (seed 2), solved by
BiCGSTAB + Chebyshev(11) (the reference CPU preset) from x = 0.

One step = one full solve.  `value` is the device time per solve of the fastest
form, mixed+learned: FP64 iterative refinement around FP32 flexible CG whose
preconditioner is Chebyshev smoothing plus a U-Net coarse-grid correction (the
network trained here, outside the timed region, by the library's own kernels).
`e2e` is the same solve through pps_solve() on pinned host buffers, copies
included (b uploads first; x's upload and its copy out overlap the solve, and the
returned x is checked bit for bit against the device-resident solve's): its value
is the median over the steps (the host memory the copies read
and write is shared with the machine's other jobs, and a contended copy can run at
a fraction of its usual rate; the mean and every sample are listed beside it).  The
reference method (BiCGSTAB + Chebyshev) is timed beside it in mixed
precision and in plain FP64.  Every field is 0.5-1.1 GB, far larger than the 129 MB L2, so no L2 flush
is needed between steps.  Outside the timed region the line also carries: the
headline's V-cycle with its coarsest level solved without the network (what the
network earns), the compositions at 256^3, the batched solves, the learned
preconditioner at 128^3, and the 1024^3 charges solve (mixed+learned and plain FP64).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--size M] [--impl reference]
  python bench.py --profile-case ...     (one capped solve for an ncu capture, no bench line)

--impl reference times the reference's CPU implementation of the path on the host
cores: one complete solve by the oracle's C restatement (bit-identical to the
reference solver), all host threads on the element-wise passes, sums serial as in
the reference, its K steps consecutive chunks of that one solve's iterations.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to ||r||/||b|| <= 1e-10 at 512^3 (mixed+learned vs plain FP64), 1 GB300"
NET_GRID = 16   # the U-Net runs as the coarsest-level solver on a 16^3 grid
# multigrid V-cycle of the learned preconditioner: Chebyshev smoother degree on the
# solver's grid, on the intermediate levels, and the smoothing interval ratio
VCYCLE = (5, 4, 8.0)
TOL = 1e-10
DEGREE = 11
# Iterations the reference BiCGSTAB+Chebyshev(11) needs on this workload, measured by
# running the oracle's C restatement (bit-identical to the reference solver) to
# convergence at 512^3 on the GB300 host (16 threads: 172 s, true ||r||/||b|| 9.3e-11).
# The CPU leg multiplies its timed per-iteration cost by it.
REFERENCE_ITERATIONS = {512: 166}
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "cheb_sweep_fp32_traffic.txt")
PROFILE_TRAFFIC_FCG = os.path.join(ROOT, "profiles", "fcg_kernels_traffic.txt")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Replica coordination under torchrun: barrier and max over ranks (gloo, host)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()   # let the sampler start before the timed region does
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        busy = [v for v in sm if mx and v > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_ratio(path=PROFILE_TRAFFIC):
    """dram bytes / algorithmic bytes of the kernel a committed ncu summary covers
    (default: one FP32 sweep launch)."""
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_over_algorithmic:"):
            return float(line.split(":")[1])
    return None


def make_inputs(m: int):
    from parallelpoissonsolver_gb300 import workloads
    b = workloads.random_field(m, seed=2, slope=-2.0)
    x = np.zeros_like(b)
    return x, b


def train_network(args, dev: int, coarsen: int):
    """The learned preconditioner's U-Net: linear 3-level 16/32/64 network trained on
    16^3 (f, u) pairs (half k^-2 random fields, half Gaussian blobs) with the library's
    own kernels; u solves the operator of the multigrid cycle's coarsest level after
    `coarsen` coarsenings (its upper wall 2^-coarsen spacings above the last unknown),
    exactly.  The network is that level's solver inside flexible CG."""
    import torch

    import parallelpoissonsolver_gb300 as pps
    from parallelpoissonsolver_gb300 import learned

    t0 = time.perf_counter()
    train = learned.make_dataset_batch(NET_GRID, 10000, args.train_samples, coarsen, device=dev)
    held = learned.make_dataset_batch(NET_GRID, 30000, args.held_out_pairs, coarsen, device=dev)
    t_data = time.perf_counter() - t0
    scale = learned.fit_scale(train)
    net = pps.UNet((16, 32, 64), seed=1, device=dev, linear=True)
    t1 = time.perf_counter()
    losses = learned.train(net, train, scale, args.train_steps, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    errs = learned.evaluate(net, held, scale)
    info = {"grid": f"{NET_GRID}^3", "channels": [16, 32, 64], "activation": "identity (linear U-Net)",
            "precision": "BF16 weights/activations, FP32 accumulation (tensor cores)",
            "train_pairs": len(train), "held_out_pairs": len(held), "steps": args.train_steps,
            "final_loss": float(np.mean(losses[-100:])),
            "held_out_rel_err_median": float(np.median(errs)), "held_out_rel_err_max": float(np.max(errs)),
            "data_s": t_data, "train_s": t_train, "scale": scale, "coarsen": coarsen}
    return net, scale, info


def learned_gain(m: int, scale: float):
    """(coarsening levels, output gain) to use the NET_GRID^3 network on an m^3 grid."""
    import math
    k = int(round(math.log2(m / NET_GRID)))
    return k, scale * ((2 ** k / (m + 1)) / (1.0 / (NET_GRID + 1))) ** 2


def run_gpu(args, dist: Dist):
    import torch

    import parallelpoissonsolver_gb300 as pps

    dev = dist.local
    torch.cuda.set_device(dev)
    m = args.size
    grid = pps.BlockGrid.cube(m)
    x_h, b_h = make_inputs(m)
    b_d = torch.from_numpy(b_h).to(f"cuda:{dev}")
    x_d = torch.zeros_like(b_d)
    G = b_h.size
    prec = pps.ChebyshevIteration(DEGREE)

    net, scale, net_info = train_network(args, dev, learned_gain(m, 1.0)[0])
    k, gain = learned_gain(m, scale)
    flags = pps.LEARNED_PRECONDITIONER
    head = pps.FlexibleCG(grid, prec, tolerance=TOL, max_iteration=20000, form="mixed", use_graph=True,
                          inner_tol=args.learned_inner_tol, device=dev)
    head.set_learned(net, k, gain, flags)
    head.set_learned_cycle(*VCYCLE)
    mixed = pps.BiCGSTAB(grid, prec, tolerance=TOL, max_iteration=20000, form="mixed", use_graph=False,
                         inner_tol=args.inner_tol, device=dev)
    plain = pps.BiCGSTAB(grid, prec, tolerance=TOL, max_iteration=20000, form="fp64", use_graph=False,
                         device=dev)
    tuned = {"mixed+learned": head.autotune(), "mixed": mixed.autotune(), "fp64": plain.autotune()}

    def solve(s):
        x_d.zero_()
        torch.cuda.current_stream().synchronize()   # the solver runs on its own stream
        st = s.solve_device(x_d.data_ptr(), b_d.data_ptr())
        if st != pps.OK:
            raise RuntimeError(f"solve failed: {pps.status_string(st)} {pps.last_error()}")
        return s.stats()

    for _ in range(args.warmup):
        solve(head)
    torch.cuda.synchronize()

    # ---- timed region: K mixed+learned solves, fields resident in HBM ----
    dist.barrier()
    torch.cuda.synchronize()
    stats = []
    with ClockSampler(dev) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            stats.append(solve(head))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dist.barrier()
    dev_times = [s["seconds_solve"] for s in stats]
    t_step = dist.max(sum(dev_times) / len(dev_times))
    head_x = x_d.clone()

    # ---- what the network earns: the same V-cycle with its coarsest-level solver
    # swapped (no fallback, so each cycle's own convergence shows) ----
    coarse = coarse_solver_comparison(args, grid, prec, net, k, gain, dev, solve)

    # ---- the reference method in mixed precision, and in plain FP64 ----
    mixed_stats = [solve(mixed) for _ in range(max(1, args.plain_steps))]
    t_mixed = sum(s["seconds_solve"] for s in mixed_stats) / len(mixed_stats)
    plain_stats = [solve(plain) for _ in range(max(1, args.plain_steps))]
    t_plain = sum(s["seconds_solve"] for s in plain_stats) / len(plain_stats)
    plain_x = x_d.clone()
    rel_diff = float(torch.linalg.norm(head_x - plain_x) / torch.linalg.norm(plain_x))

    # ---- e2e: the C ABI on pinned host buffers, copies inside the timed region ----
    xp = torch.zeros(b_h.shape, dtype=torch.float64).pin_memory()
    bp = torch.from_numpy(b_h).pin_memory()
    xn, bn = xp.numpy(), bp.numpy()
    e2e, e2e_parts = [], []
    for kk in range(args.steps + 1):
        xn[...] = 0.0
        t = time.perf_counter()
        st = head(xn, bn)
        el = time.perf_counter() - t
        if st != pps.OK:
            raise RuntimeError(f"e2e solve failed: {pps.status_string(st)}")
        if kk > 0:
            e2e.append(el)
            d = head.stats()
            e2e_parts.append((d["seconds_h2d"], d["seconds_solve"], d["seconds_d2h"], d["seconds_total"], el))
    e2e_overlap = head.stats()["copy_overlap"]
    e2e_same_x = bool(np.array_equal(xn.view(np.uint64), head_x.cpu().numpy().view(np.uint64)))
    t_e2e = dist.max(statistics.median(e2e))
    t_e2e_mean = dist.max(sum(e2e) / len(e2e))
    e2e_split = {k: statistics.median(p[i] for p in e2e_parts)
                 for i, k in enumerate(("h2d_s", "solve_s", "d2h_s", "call_s", "python_s"))}

    # ---- roofline of the headline's dominant kernels: flexible CG's direction + stencil
    # (k_fcg_p_stencil_v4) and x, r update (k_fcg_update_xr_flat), the two largest of its
    # solve.  The headline replays CUDA graphs, which carry no events, so the same solver
    # settings run once more uncaptured with the two kernels bracketed by events ----
    probe = pps.FlexibleCG(grid, prec, tolerance=TOL, max_iteration=20000, form="mixed", use_graph=False,
                           inner_tol=args.learned_inner_tol, device=dev)
    probe.set_learned(net, k, gain, flags)
    probe.set_learned_cycle(*VCYCLE)
    probe.set_tuning(head.tuning())
    solve(probe)
    kstats = [solve(probe) for _ in range(2)]
    probe.close()
    kry_s = sum(s["krylov_seconds"] for s in kstats)
    kry_b = sum(s["krylov_bytes"] for s in kstats)
    kry_n = sum(s["krylov_launches"] for s in kstats)

    # ---- roofline of the FP32 Chebyshev sweep (the reference method's dominant kernel),
    # event-timed in the mixed BiCGSTAB solves (degree 11: all 16 B sweeps) ----
    sweep_s = sum(s["sweep_seconds"] for s in mixed_stats)
    sweep_n = sum(s["sweep_launches"] for s in mixed_stats)
    sweep_b = sum(s["sweep_bytes"] for s in mixed_stats)
    peak, peak_src = measured_peaks()
    achieved = (sweep_b / sweep_s) / 1e9 if sweep_s > 0 else None
    ratio = traffic_ratio()
    per_launch_alg = sweep_b / sweep_n if sweep_n else None

    def summary(s, t):
        return {"value": t, "unit": "s", "iterations": s["iterations"], "refinements": s["refinements"],
                "err_true": s["err_true"],
                "sweep_gbs": (s["sweep_bytes"] / s["sweep_seconds"]) / 1e9 if s["sweep_seconds"] > 0 else None}

    out = {
        "metric": METRIC,
        "value": t_step,
        "unit": "s",
        "n_gpus": dist.ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_step * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 stencil/smoother/Krylov fields, bf16 U-Net (fp32 accum), f64 residual/dots/refinement",
        "data": "synthetic: seeded k^-2 Gaussian random field (numpy PCG64 seed 2), unit RMS",
        "config": {
            "workload": f"{m}^3 interior unknowns, h=1/{m + 1}, Dirichlet 0, -lap u = f, f ~ P(k) k^-2 field; "
                        f"stop at FP64 ||r||/||b_adj|| <= {TOL:g}",
            "form": "mixed+learned: FP64 iterative refinement around FP32 flexible CG (inner tolerance "
                    f"{args.learned_inner_tol:g}); preconditioner = multigrid V-cycle over {k + 1} levels: "
                    f"Chebyshev({VCYCLE[0]}) smoothing on the {m}^3 grid (interval [lmax/{VCYCLE[2]:g}, lmax]), "
                    f"Jacobi-scaled Chebyshev({VCYCLE[1]}) pre- and post-smoothing on each intermediate level "
                    f"(interval [2/{VCYCLE[2]:g}, 2] of D^-1 A_l, A_l with the upper wall one fine spacing above "
                    f"the last unknown), the U-Net trained for that operator as the {NET_GRID}^3 coarse solver",
            "l2": "no flush: every field (0.5-1.1 GB) exceeds the 129 MB L2",
            "parallelism": f"replicas x{dist.ws}" if dist.ws > 1 else "single GPU, single domain",
            "iterations": stats[-1]["iterations"],
            "refinements": stats[-1]["refinements"],
            "learned_applications": stats[-1]["learned_applications"],
            "fallback_iteration": stats[-1]["fallback_iteration"],
            "err_true": stats[-1]["err_true"],
            "network": net_info,
            "tiles": tuned,
        },
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": 2 * G * 8, "d2h_bytes_per_step": G * 8,
                "statistic": "median over the steps", "mean_s": t_e2e_mean,
                "median_split": e2e_split, "samples_s": [round(v, 5) for v in e2e],
                "copy_overlap": e2e_overlap, "x_bitwise_equal_to_device_solve": e2e_same_x,
                "samples_ms_h2d_solve_d2h_call": [[round(1e3 * v, 2) for v in p[:4]] for p in e2e_parts]},
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "forms": {
            "mixed+learned (FCG)": summary(stats[-1], t_step),
            "mixed (reference BiCGSTAB + Chebyshev)": summary(mixed_stats[-1], t_mixed),
            "plain_fp64 (reference BiCGSTAB + Chebyshev)": summary(plain_stats[-1], t_plain),
        },
        "plain_fp64": summary(plain_stats[-1], t_plain),
        "speedup_vs_plain_fp64": t_plain / t_step,
        "speedup_mixed_only_vs_plain_fp64": t_plain / t_mixed,
        "vs_plain_fp64_rel_l2": rel_diff,
        "hbm_gbs_solve": stats[-1]["hbm_bytes"] / stats[-1]["seconds_solve"] / 1e9,
        "roofline": {
            "bound": "hbm",
            "kernel": "k_fcg_p_stencil_v4 + k_fcg_update_xr_flat (the headline solve's two largest kernels: "
                      "flexible CG's direction + stencil, 16 B per unknown, and x, r update, 24 B per unknown; "
                      "event-timed in uncaptured solves with the headline's settings)",
            "achieved": (kry_b / kry_s) / 1e9 if kry_s > 0 else None,
            "peak": peak,
            "unit": "GB/s",
            "frac": ((kry_b / kry_s) / 1e9 / peak) if kry_s > 0 else None,
            "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else peak_src,
            "traffic": (traffic_ratio(PROFILE_TRAFFIC_FCG) * kry_b / kry_n * 2)
                       if (traffic_ratio(PROFILE_TRAFFIC_FCG) and kry_n) else None,
            "traffic_unit": "bytes per launch pair (direction + update)",
            "algorithmic_bytes_per_launch_pair": kry_b / kry_n * 2 if kry_n else None,
            "launches_timed": kry_n,
        },
        "roofline_sweep": {
            "bound": "hbm",
            "kernel": "k_cheb_v4<1>, k_cheb_v4<2> (the FP32 Chebyshev sweeps, one float4 per thread: Y with its "
                      "6 neighbours, B, [Z] in, W out; 12 / 16 B per unknown; timed in the mixed BiCGSTAB solves, "
                      "the smoother kernels of the headline too)",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else peak_src,
            "traffic": (ratio * per_launch_alg) if (ratio and per_launch_alg) else None,
            "algorithmic_bytes_per_launch": per_launch_alg,
            "launches_timed": sweep_n,
        },
        "clocks": clocks.summary(),
        "wall_s_timed_region": wall,
        "coarse_solvers": coarse,
    }
    if not args.no_learned_128:
        out["learned_128"] = run_learned_128(args, dev)
    head.close()
    mixed.close()
    plain.close()
    return out, plain_stats[-1]["iterations"]


def coarse_solver_comparison(args, grid, prec, net, k: int, gain: float, dev: int, solve):
    """The headline's flexible CG + V-cycle with the coarsest level (16^3)
    solved four ways: the trained network, no correction, the coarse levels' Jacobi-
    scaled Chebyshev smoother, and the level operator's exact inverse (tensor-product
    eigen-solve).  Same workload, tolerance, inner tolerance and graph replay as the
    headline, with the fallback switched off.  Per variant: iterations, refinements,
    device time per solve (median of 3 after one warm-up) and the true residual."""
    import parallelpoissonsolver_gb300 as pps
    kinds = [("network", pps.COARSE_NETWORK), ("zero", pps.COARSE_ZERO), ("smooth", pps.COARSE_SMOOTH),
             ("exact", pps.COARSE_EXACT)]
    s = pps.FlexibleCG(grid, prec, tolerance=TOL, max_iteration=20000, form="mixed", use_graph=True,
                       inner_tol=args.learned_inner_tol, device=dev)
    s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER | pps.LEARNED_NO_FALLBACK)
    s.set_learned_cycle(*VCYCLE)
    s.autotune()
    out = {"coarse_grid": f"{NET_GRID}^3", "fallback": "off", "timing": "median of 3 solves after 1 warm-up"}
    for name, kind in kinds:
        s.set_coarse_solver(kind)
        solve(s)
        runs = [solve(s) for _ in range(3)]
        r = runs[-1]
        out[name] = {"seconds": statistics.median(x["seconds_solve"] for x in runs), "iterations": r["iterations"],
                     "refinements": r["refinements"], "err_true": r["err_true"]}
    s.close()
    return out


def run_learned_128(args, dev: int):
    """Learned initial guess and preconditioner at 128^3 on held-out seeds (half k^-2
    fields, half blobs): flexible CG with the network (two-grid cycle and multigrid
    V-cycle; the network trained for two coarsenings) against the reference method
    (BiCGSTAB + Chebyshev) and against flexible CG without it, all FP64 to 1e-10."""
    import torch

    import parallelpoissonsolver_gb300 as pps
    from parallelpoissonsolver_gb300 import learned

    m = 128
    grid = pps.BlockGrid.cube(m)
    net, scale, _ = train_network(args, dev, learned_gain(m, 1.0)[0])
    k, gain = learned_gain(m, scale)
    forms = {
        "bicgstab": pps.BiCGSTAB(grid, pps.ChebyshevIteration(DEGREE), tolerance=TOL, form="fp64", device=dev),
        "fcg": pps.FlexibleCG(grid, pps.ChebyshevIteration(DEGREE), tolerance=TOL, form="fp64", device=dev),
        "fcg+learned": pps.FlexibleCG(grid, pps.ChebyshevIteration(DEGREE), tolerance=TOL, form="fp64",
                                      use_graph=False, device=dev),
        "fcg+learned-vcycle": pps.FlexibleCG(grid, pps.ChebyshevIteration(DEGREE), tolerance=TOL, form="fp64",
                                             use_graph=True, device=dev),
    }
    forms["fcg+learned"].set_learned(net, k, gain, pps.LEARNED_INITIAL_GUESS | pps.LEARNED_PRECONDITIONER |
                                     pps.LEARNED_POST_SMOOTH)
    forms["fcg+learned-vcycle"].set_learned(net, k, gain, pps.LEARNED_INITIAL_GUESS | pps.LEARNED_PRECONDITIONER)
    forms["fcg+learned-vcycle"].set_learned_cycle(*VCYCLE)
    res = {n: {"iterations": [], "seconds": [], "err_true": []} for n in forms}
    for i in range(args.held_out):
        seed = 30000 + i
        b = learned.rhs(m, seed, "field" if seed % 2 == 0 else "blobs")
        bd = torch.from_numpy(b).cuda(dev)
        for n, s in forms.items():
            xd = torch.zeros_like(bd)
            torch.cuda.synchronize()
            st = s.solve_device(xd.data_ptr(), bd.data_ptr())
            d = s.stats()
            res[n]["iterations"].append(d["iterations"] if st == pps.OK else -1)
            res[n]["seconds"].append(d["seconds_solve"])
            res[n]["err_true"].append(d["err_true"])
    for s in forms.values():
        s.close()
    net.close()
    out = {"workload": f"{m}^3, Dirichlet 0, {args.held_out} held-out seeds (30000+), FP64 to {TOL:g}"}
    for n, r in res.items():
        out[n] = {"mean_iterations": float(np.mean(r["iterations"])), "mean_seconds": float(np.mean(r["seconds"])),
                  "max_err_true": float(np.max(r["err_true"]))}
    out["iteration_gain_vs_fcg"] = out["fcg"]["mean_iterations"] / out["fcg+learned-vcycle"]["mean_iterations"]
    out["time_gain_vs_bicgstab"] = out["bicgstab"]["mean_seconds"] / out["fcg+learned-vcycle"]["mean_seconds"]
    return out


def run_large(args, dev: int):
    """The 1024^3 charges solve (default on; --no-large skips it): one Dirichlet solve of 64
    Gaussian charges on a k^-3 background, the mixed + learned V-cycle (network on the
    16^3 level, six coarsenings; two timed solves after a warm-up) against the plain
    FP64 BiCGSTAB + Chebyshev path (one solve), both to 1e-10."""
    import math

    import torch

    import parallelpoissonsolver_gb300 as pps
    from parallelpoissonsolver_gb300 import workloads

    m = 1024
    grid = pps.BlockGrid.cube(m)
    b_d = workloads.charges_device(m, device=f"cuda:{dev}")
    x_d = torch.zeros_like(b_d)
    k = int(round(math.log2(m / NET_GRID)))
    net, scale, info = train_network(args, dev, k)
    _, gain = learned_gain(m, scale)

    def solve(s):
        x_d.zero_()
        torch.cuda.synchronize()
        st = s.solve_device(x_d.data_ptr(), b_d.data_ptr())
        return pps.status_string(st), s.stats()

    head = pps.FlexibleCG(grid, pps.ChebyshevIteration(DEGREE), tolerance=TOL, max_iteration=20000, form="mixed",
                          use_graph=True, inner_tol=args.learned_inner_tol, device=dev)
    head.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER)
    head.set_learned_cycle(*VCYCLE)
    head.autotune()
    solve(head)   # warm-up
    runs = [solve(head) for _ in range(2)]
    head_x = x_d.clone()
    head.close()
    plain = pps.BiCGSTAB(grid, pps.ChebyshevIteration(DEGREE), tolerance=TOL, max_iteration=20000, form="fp64",
                         use_graph=True, device=dev)
    st_p, d_p = solve(plain)
    plain.close()
    rel = float(torch.linalg.norm(head_x - x_d) / torch.linalg.norm(x_d))
    net.close()
    t_head = sum(d["seconds_solve"] for _, d in runs) / len(runs)
    return {
        "workload": f"{m}^3 interior unknowns, Dirichlet 0, 64 Gaussian charges (width 2h, amplitude +-1) on a "
                    f"k^-3 random-field background at 0.1 RMS; stop at FP64 ||r||/||b_adj|| <= {TOL:g}",
        "mixed+learned": {"status": runs[-1][0], "value": t_head, "unit": "s",
                          "iterations": runs[-1][1]["iterations"], "refinements": runs[-1][1]["refinements"],
                          "err_true": runs[-1][1]["err_true"], "network_coarsen": k,
                          "network_held_out_rel_err_median": info["held_out_rel_err_median"]},
        "plain_fp64": {"status": st_p, "value": d_p["seconds_solve"], "unit": "s", "iterations": d_p["iterations"],
                       "err_true": d_p["err_true"]},
        "speedup_vs_plain_fp64": d_p["seconds_solve"] / t_head,
        "vs_plain_fp64_rel_l2": rel,
    }


def composition_cpu_sample(m: int, cfg: dict, outer_its: int, inner_its: int, threads: int):
    """Bounded sample of the oracle port (bit-identical to the reference CPU solver)
    for a composition with an inner solver: set-up alone (maxit 0), then one outer
    iteration with 2 and with 4 inner iterations per application (2 applications
    per BiCGSTAB iteration), extrapolated to the GPU run's iteration counts."""
    from oracle import oracle as O
    g = O.cube(m)
    x0, b0 = make_inputs(m)

    def t(**kw):
        c = O.Config(**{**cfg, **kw, "threads": threads})
        tt = time.perf_counter()
        O.solve(g, c, x0.copy(), b0.copy())
        return time.perf_counter() - tt

    t(maxit=1, prec_maxit=1)   # warm the thread pool, page in the fields
    t0, t2, t4 = t(maxit=0), t(maxit=1, prec_maxit=2), t(maxit=1, prec_maxit=4)
    t_inner = max(t4 - t2, 0.0) / 4.0
    t_outer = max(t2 - t0 - 4.0 * t_inner, 0.0)
    return {"value": t0 + outer_its * t_outer + inner_its * t_inner, "unit": "s", "cores": threads, "kind": "port",
            "sample": f"{m}^3: set-up, then one outer iteration with 2 and 4 inner iterations per application; "
                      f"{t_inner * 1e3:.1f} ms per inner iteration, {t_outer * 1e3:.1f} ms per outer iteration "
                      f"outside them, extrapolated to {outer_its} outer / {inner_its} inner iterations"}


def chebyshev_cpu_sample(m: int, degree: int, threads: int):
    """The oracle's Chebyshev main solver at degrees 4 and 12; the difference gives the
    cost of a sweep, extrapolated to `degree`."""
    from oracle import oracle as O
    g = O.cube(m)
    x0, b0 = make_inputs(m)

    def t(n):
        c = O.Config(krylov=O.CHEBYSHEV_MAIN, cheb_degree=n, cheb_eps=0.0, rescale_min=1.0, rescale_max=1.0,
                     threads=threads)
        tt = time.perf_counter()
        O.solve(g, c, x0.copy(), b0.copy())
        return time.perf_counter() - tt

    t(2)
    t4, t12 = t(4), t(12)
    sweep = max(t12 - t4, 0.0) / 8.0
    return {"value": t4 + (degree - 4) * sweep, "unit": "s", "cores": threads, "kind": "port",
            "sample": f"{m}^3 at degrees 4 and 12: {sweep * 1e3:.1f} ms per sweep, extrapolated to degree {degree}"}


def run_compositions(args, dev: int, threads: int):
    """The other compositions of inputParam.hpp on the benchmark's field at
    --comp-size^3 (k^-2 random field, Dirichlet 0, stop at 1e-10): BiCGSTAB
    preconditioned by an inner BiCGSTAB solve (CPU/include/inputParam.hpp:30, the CPU
    preset 1e-6 / 150 iterations) and by an inner CG solve with the Chebyshev
    polynomial (inputParam.hpp:29), and the Chebyshev iteration as the main solver
    (ALP/include/inputParam.hpp:37) with its eigenvalue bounds unscaled.  Each: device
    time of a solve, iterations, the algorithmic HBM bytes of all its kernels over that
    time against the measured copy bandwidth, and the oracle's CPU time extrapolated
    from a bounded sample."""
    import math

    import torch

    import parallelpoissonsolver_gb300 as pps

    m = args.comp_size
    grid = pps.BlockGrid.cube(m)
    x_h, b_h = make_inputs(m)
    b_d = torch.from_numpy(b_h).to(f"cuda:{dev}")
    x_d = torch.zeros_like(b_d)
    peak, peak_kind = measured_peaks()
    # degree of the Chebyshev main solver: the polynomial's error bound
    # 2 ((sqrt(k) - 1) / (sqrt(k) + 1))^n below 1e-12 for the condition number k
    lmin = 3 * 4 * math.sin(math.pi / 2 / (m + 1)) ** 2
    lmax = 3 * 4 * math.sin(m * math.pi / 2 / (m + 1)) ** 2
    q = (math.sqrt(lmax / lmin) - 1) / (math.sqrt(lmax / lmin) + 1)
    deg_fp64 = int(math.ceil(math.log(1e-12 / 2) / math.log(q)))
    deg_mixed = int(math.ceil(math.log(1e-5 / 2) / math.log(q)))
    cheb_main = pps.ChebyshevIteration(deg_fp64, 0.0, 1.0, 1.0)
    solvers = {
        "bicgstab+inner_bicgstab": {f: pps.BiCGSTAB(grid, pps.BiCGSTABPreconditioner(1e4 * 1e-10, 150),
                                                    tolerance=TOL, max_iteration=5000, form=f, device=dev)
                                    for f in ("fp64", "mixed")},
        "bicgstab+inner_cg_chebyshev": {f: pps.BiCGSTAB(grid, pps.BaseCGPreconditioner(1e4 * 1e-10, 150,
                                                                                       pps.ChebyshevIteration(DEGREE)),
                                                        tolerance=TOL, max_iteration=5000, form=f, device=dev)
                                        for f in ("fp64", "mixed")},
        "chebyshev_main": {
            "fp64": pps.ChebyshevSolver(grid, cheb_main, tolerance=TOL, form="fp64", use_graph=False, device=dev),
            "mixed": pps.ChebyshevSolver(grid, pps.ChebyshevIteration(deg_mixed, 0.0, 1.0, 1.0), tolerance=TOL,
                                         form="mixed", use_graph=False, device=dev)},
    }
    out = {"workload": f"{m}^3, Dirichlet 0, k^-2 random field (seed 2), stop at ||r||/||b_adj|| <= {TOL:g}; "
                       f"Chebyshev main solver on [lambda_min, lambda_max] (rescale 1, epsilon 0) of degree "
                       f"{deg_fp64} (FP64, one application) or {deg_mixed} (MIXED, per refinement pass)",
           "peak_gbs": peak, "peak_kind": peak_kind}
    for name, forms in solvers.items():
        out[name] = {}
        for f, s in forms.items():
            s.autotune()
            runs = []
            for _ in range(3):   # the first run is the warm-up
                x_d.zero_()
                torch.cuda.synchronize()
                st = s.solve_device(x_d.data_ptr(), b_d.data_ptr(), raise_on_error=False)
                runs.append((st, s.stats()))
            t = statistics.mean(d["seconds_solve"] for _, d in runs[1:])
            st, d = runs[-1]
            rel_err = d["err_true"] / d["norm_b"] if name == "chebyshev_main" else d["err_true"]
            achieved = d["hbm_bytes"] / t / 1e9
            out[name][f] = {"status": pps.status_string(st), "seconds": t, "iterations": d["iterations"],
                            "inner_iterations": d["precond_iterations"], "refinements": d["refinements"],
                            "true_rel_residual": rel_err, "algorithmic_gbs": achieved,
                            "frac_of_peak": achieved / peak, "kernel_launches": d["kernel_launches"]}
            if name == "chebyshev_main" and d["sweep_seconds"] > 0:
                out[name][f]["sweep_gbs"] = d["sweep_bytes"] / d["sweep_seconds"] / 1e9
            s.close()
    if not args.no_cpu_baseline:
        base = dict(tol=TOL, maxit=5000, prec_tol=1e4 * 1e-10, prec_maxit=150)
        for name, cfg in (("bicgstab+inner_bicgstab", dict(precond=2, prec_inner=0)),
                          ("bicgstab+inner_cg_chebyshev", dict(precond=3, prec_inner=1, cheb_degree=DEGREE))):
            r = out[name]["fp64"]
            cpu = composition_cpu_sample(m, {**base, **cfg}, r["iterations"], r["inner_iterations"], threads)
            out[name]["cpu_baseline"] = cpu
            out[name]["fp64_speedup_vs_cpu"] = cpu["value"] / r["seconds"]
            out[name]["mixed_speedup_vs_cpu"] = cpu["value"] / out[name]["mixed"]["seconds"]
        cpu = chebyshev_cpu_sample(m, deg_fp64, threads)
        out["chebyshev_main"]["cpu_baseline"] = cpu
        out["chebyshev_main"]["fp64_speedup_vs_cpu"] = cpu["value"] / out["chebyshev_main"]["fp64"]["seconds"]
    return out


def batch_coarsenings(m: int) -> int:
    """Coarsenings of the persistent batch's V-cycle for edge m: halve while above 16."""
    k = 0
    while m > 16 and m % 2 == 0:
        m //= 2
        k += 1
    return k


def run_batched(args, dist: Dist):
    """256 independent Dirichlet problems, edges uniform on {32,48,64,96,128}, each f a
    seeded sum of 1-8 Gaussian blobs, MIXED form to 1e-10.  The value: the persistent
    batch -- flexible CG with a multigrid V-cycle per problem (exact coarsest solve),
    the whole batch ONE cooperative launch replayed as a CUDA graph.  Beside it: the
    same method run problem after problem by the single-grid solver, and the
    per-phase batch of the reference method (BiCGSTAB + Chebyshev, one launch per
    phase over all problems, autotuned tiles per grid size)."""
    import torch

    import parallelpoissonsolver_gb300 as pps
    from parallelpoissonsolver_gb300 import workloads

    edges = workloads.batch_edges(args.batch_problems, seed=3)
    grids = [pps.BlockGrid.cube(m) for m in edges]
    rhs = [workloads.blobs(m, 3 + i) for i, m in enumerate(edges)]

    def timed(bt, steps):
        times, stats = [], None
        for k in range(1 + steps):
            for i, b in enumerate(rhs):
                bt.set(i, np.zeros_like(b), b)
            torch.cuda.synchronize()
            st = bt.solve()
            if st != pps.OK:
                raise RuntimeError(f"batched solve: {pps.status_string(st)} {pps.last_error()}")
            stats = bt.stats()
            if k > 0:
                times.append(stats["seconds_solve"])
        return sum(times) / len(times), stats

    bt = pps.Batch(grids, tolerance=TOL, inner_tol=args.learned_inner_tol, device=dist.local, method="vcycle")
    t_batch, stats = timed(bt, args.batch_steps)
    errs = [bt.get(i)[1]["err_true"] for i in range(len(edges))]

    # the same method problem after problem: flexible CG + V-cycle with the exact coarsest solve
    net = pps.UNet((16, 32, 64), seed=1, linear=True, device=dist.local)   # holds the cycle's settings only
    solvers = {}
    for m in sorted(set(edges)):
        s = pps.FlexibleCG(pps.BlockGrid.cube(m), pps.ChebyshevIteration(DEGREE), tolerance=TOL,
                           max_iteration=20000, form="mixed", inner_tol=args.learned_inner_tol, device=dist.local)
        s.set_learned(net, batch_coarsenings(m), 1.0, pps.LEARNED_PRECONDITIONER | pps.LEARNED_NO_FALLBACK)
        s.set_learned_cycle(*VCYCLE)
        s.set_coarse_solver(pps.COARSE_EXACT)
        s.autotune()
        solvers[m] = s

    def sequential():
        for i, b in enumerate(rhs):
            bt.set(i, np.zeros_like(b), b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its = 0
        for i, m in enumerate(edges):
            xd, bd = bt.field_device(i)
            st = solvers[m].solve_device(xd, bd)
            if st != pps.OK:
                raise RuntimeError(f"single solve {i}: {pps.status_string(st)}")
            its = max(its, solvers[m].get_num_iteration_final())
        torch.cuda.synchronize()
        return time.perf_counter() - t0, its

    sequential()   # warm-up (graphs captured)
    t_seq, seq_iters = sequential()
    for s in solvers.values():
        s.close()
    net.close()
    bt.close()

    # the reference method as a per-phase batch (one measured solve after a warm-up)
    ref = pps.Batch(grids, pps.ChebyshevIteration(DEGREE), tolerance=TOL, inner_maxit=5000, device=dist.local)
    for i, b in enumerate(rhs):
        ref.set(i, np.zeros_like(b), b)
    ref.autotune()
    t_ref, ref_stats = timed(ref, 1)
    ref.close()
    return {
        "workload": f"{len(edges)} Dirichlet problems, edges uniform on {{32,48,64,96,128}} (seed 3), f = sum of "
                    f"1-8 Gaussian blobs (seeds 3+p); MIXED to {TOL:g}",
        "method": "flexible CG + multigrid V-cycle per problem (Chebyshev(5) fine smoothing, Jacobi-Chebyshev(4) "
                  "on the coarse levels, exact coarsest solve at <= 16^3), FP64 refinement; ONE persistent "
                  "cooperative launch replayed as a CUDA graph",
        "value": t_batch, "unit": "s", "steps": args.batch_steps,
        "unknowns": stats["unknowns"], "converged": stats["converged"], "max_err_true": stats["max_err_true"],
        "max_inner_iterations": stats["max_iterations"], "max_refinements": stats["max_refinements"],
        "kernel_launches": stats["kernel_launches"], "graph_replays": stats["graph_replays"],
        "median_err_true": float(np.median(errs)),
        "sequential_same_method_s": t_seq, "sequential_max_iterations": seq_iters,
        "speedup_vs_sequential": t_seq / t_batch,
        "per_phase_bicgstab_batch_s": t_ref, "per_phase_bicgstab_kernel_launches": ref_stats["kernel_launches"],
        "per_phase_bicgstab_max_inner_iterations": ref_stats["max_iterations"],
        "speedup_vs_per_phase_bicgstab": t_ref / t_batch,
    }


def cpu_sample(m: int, iterations_needed: int | None, threads: int):
    """Bounded sample of the reference CPU solve on this workload: set-up plus a few
    BiCGSTAB iterations of the oracle port (bit-identical to the reference)."""
    from oracle import oracle as O
    O.build(ref=False)
    g = O.cube(m)
    x0, b0 = make_inputs(m)
    # warm the thread pool and page in the fields, then time set-up + 3 iterations
    O.solve(g, O.Config(tol=TOL, maxit=1, threads=threads), x0.copy(), b0.copy())
    x, b = x0.copy(), b0.copy()
    t = time.perf_counter()
    r = O.solve(g, O.Config(tol=TOL, maxit=3, threads=threads), x, b)
    total = time.perf_counter() - t
    t_iter = r.seconds_loop / max(r.iterations, 1)
    t_setup = max(total - r.seconds_loop, 0.0)
    n_it = iterations_needed if iterations_needed else 1
    return {
        "value": t_setup + n_it * t_iter,
        "unit": "s",
        "cores": threads,
        "kind": "port",
        "sample": f"{m}^3, set-up + 3 BiCGSTAB iterations of the oracle port (bit-identical to the "
                  f"reference CPU solver; {threads} threads on element-wise passes, serial sums); "
                  f"extrapolated to {n_it} iterations: {t_iter:.3f} s/iteration, {t_setup:.3f} s set-up",
        "seconds_per_iteration": t_iter,
        "seconds_setup": t_setup,
    }


def reference_arm(m: int, steps: int, warmup: int, threads: int, n_gpus: int):
    """The reference arm: ONE complete solve of the workload to 1e-10 by the oracle
    port (bit-identical to the reference CPU solver), timed in `steps` chunks of
    consecutive BiCGSTAB iterations.  Chunk boundaries are the port's own wall-clock
    stamps at the end of iterations round(i n / steps); the first chunk includes the
    set-up (normalisation, first residual), the last the final true residual.  So
    ms_per_step x steps is the measured time to solution, not an extrapolation.
    Warm-up steps: set-up plus one iteration each, on copies of the same input."""
    from oracle import oracle as O
    O.build(ref=False)
    g = O.cube(m)
    x0, b0 = make_inputs(m)
    for _ in range(max(warmup, 0)):
        O.solve(g, O.Config(tol=TOL, maxit=1, threads=threads), x0.copy(), b0.copy())
    x, b = x0.copy(), b0.copy()
    r, st = O.solve_stamped(g, O.Config(tol=TOL, maxit=20000, threads=threads), x, b)
    n = r.iterations
    k = max(1, steps)
    cuts = [st[0]] + [st[min(max(round(i * n / k), 1), n)] for i in range(1, k)] + [st[n + 1]]
    chunks = [b_ - a_ for a_, b_ in zip(cuts[:-1], cuts[1:])]
    total = float(st[n + 1] - st[0])
    sample = (f"one complete {m}^3 solve to ||r||/||b|| <= {TOL:g} by the oracle port (bit-identical to the "
              f"reference CPU solver; {threads} threads on element-wise passes, serial sums as in the reference): "
              f"{n} BiCGSTAB iterations in {total:.1f} s, timed in {k} chunks of consecutive iterations")
    return {
        "impl": "reference", "metric": METRIC, "value": total, "unit": "s", "n_gpus": n_gpus,
        "steps": k, "warmup": warmup, "ms_per_step": total * 1e3 / k, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (same workload)",
        "config": {"workload": f"{m}^3, Dirichlet 0, k^-2 random field, BiCGSTAB+Chebyshev(11), tol {TOL:g}",
                   "step": "a chunk of consecutive iterations of one complete solve (the steps sum to it)",
                   "iterations": n, "err_iter": r.err_iter, "err_true": r.err_true,
                   "seconds_per_iteration": float((st[n] - st[1]) / max(n - 1, 1)),
                   "chunk_seconds": [round(c, 3) for c in chunks]},
        "cpu_baseline": {"kind": "port", "cores": threads, "sample": sample, "value": total, "unit": "s"},
        "e2e": {"value": total, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def profile_case(argv):
    """One capped solve of the benchmark workload, sized for an ncu capture (not a
    bench line): `--repeat` solves of the k^-2 random field at `--size`^3 with the
    iteration cap `--maxit`, so that a capture sees a handful of launches of every
    kernel of the loop on fields larger than L2; exits 0 whether or not the cap stops
    the solve.  --learned: flexible CG with a saved U-Net as the coarse-grid
    correction (the headline form); --cycle F,C,RATIO: the multigrid V-cycle.

        python bench.py --profile-case --size 320 --form mixed --maxit 2
        python bench.py --profile-case --size 320 --krylov fcg --maxit 3
        python bench.py --profile-case --save-net net.npz
        python bench.py --profile-case --size 512 --learned net.npz --cycle 5,4,8 --maxit 20000 \\
            --refinements 12 --inner-tol 1e-5
    """
    import math

    import parallelpoissonsolver_gb300 as pps
    from parallelpoissonsolver_gb300 import workloads

    ap = argparse.ArgumentParser(prog="bench.py --profile-case")
    ap.add_argument("--size", type=int, default=320)
    ap.add_argument("--form", default="mixed", choices=list(pps.FORMS))
    ap.add_argument("--maxit", type=int, default=2)
    ap.add_argument("--degree", type=int, default=11)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--save-net", default=None, help="train the linear U-Net and save it here, then exit")
    ap.add_argument("--net-grid", type=int, default=16, help="edge of the network's grid")
    ap.add_argument("--coarsen", type=int, default=5, help="coarsenings whose coarsest-level operator --save-net learns")
    ap.add_argument("--learned", default=None, help="saved U-Net to use as the coarse-grid correction")
    ap.add_argument("--cycle", default=None, help="fine,coarse,ratio of the multigrid V-cycle (with --learned)")
    ap.add_argument("--inner-tol", type=float, default=3e-3)
    ap.add_argument("--post-smooth", action="store_true", help="Chebyshev post-smoothing on the solver's grid")
    ap.add_argument("--refinements", type=int, default=1)
    ap.add_argument("--krylov", default="bicgstab", choices=("bicgstab", "fcg"),
                    help="Krylov loop without --learned (fcg: flexible CG with the Chebyshev preconditioner)")
    ap.add_argument("--batch-problems", type=int, default=0,
                    help="instead: one persistent V-cycle batch of this many problems of the batched workload")
    ap.add_argument("--fcg-staged", action="store_true",
                    help="flexible CG's direction kernel with its inputs staged by TMA (tuning fcg_staged)")
    a = ap.parse_args(argv)
    if a.batch_problems > 0:
        edges = workloads.batch_edges(a.batch_problems, seed=3)
        bt = pps.Batch([pps.BlockGrid.cube(m) for m in edges], tolerance=1e-10, inner_tol=1e-5, method="vcycle")
        for i, m in enumerate(edges):
            b = workloads.blobs(m, 3 + i)
            bt.set(i, np.zeros_like(b), b)
        for _ in range(a.repeat):
            for i, m in enumerate(edges):
                b = workloads.blobs(m, 3 + i)
                bt.set(i, np.zeros_like(b), b)
            st = bt.solve()
            d = bt.stats()
            print(f"status {pps.status_string(st)}: {d['converged']}/{len(edges)} converged, "
                  f"{d['seconds_solve'] * 1e3:.2f} ms, max inner iterations {d['max_iterations']}")
        bt.close()
        return
    if a.save_net:
        from parallelpoissonsolver_gb300 import learned
        train = learned.make_dataset(a.net_grid, range(10000, 10256), coarsen=a.coarsen)
        scale = learned.fit_scale(train)
        net = pps.UNet((16, 32, 64), seed=1, linear=True)
        learned.train(net, train, scale, 4000, lr=1e-3)
        net.save(a.save_net)
        with np.load(a.save_net) as d:
            np.savez(a.save_net, scale=np.array(scale), net_grid=np.array(a.net_grid), **{k: d[k] for k in d.files})
        print(f"saved {a.save_net}: scale {scale:.6g}")
        return
    grid = pps.BlockGrid.cube(a.size)
    b = workloads.random_field(a.size, seed=2)
    if a.learned:
        net = pps.UNet.load_file(a.learned)
        saved = np.load(a.learned)
        scale = float(saved["scale"])
        ng = int(saved["net_grid"]) if "net_grid" in saved.files else 32
        k = int(round(math.log2(a.size / ng)))
        gain = scale * ((2 ** k / (a.size + 1)) / (1.0 / (ng + 1))) ** 2
        s = pps.FlexibleCG(grid, pps.ChebyshevIteration(a.degree), tolerance=1e-10, max_iteration=a.maxit,
                           form=a.form, inner_maxit=a.maxit, max_refinements=a.refinements, use_graph=False,
                           inner_tol=a.inner_tol)
        flags = pps.LEARNED_PRECONDITIONER | pps.LEARNED_NO_FALLBACK
        if not a.cycle:
            flags |= pps.LEARNED_INITIAL_GUESS
        if a.post_smooth or not a.cycle:
            flags |= pps.LEARNED_POST_SMOOTH
        s.set_learned(net, k, gain, flags)
        if a.cycle:
            fd, cd, ratio = a.cycle.split(",")
            s.set_learned_cycle(int(fd), int(cd), float(ratio))
    else:
        cls = pps.FlexibleCG if a.krylov == "fcg" else pps.BiCGSTAB
        s = cls(grid, pps.ChebyshevIteration(a.degree), tolerance=1e-10, max_iteration=a.maxit,
                form=a.form, inner_maxit=a.maxit, max_refinements=1, use_graph=a.graph)
        if a.fcg_staged:
            s.set_tuning({**s.tuning(), "fcg_staged": 1})
    for _ in range(a.repeat):
        x = grid.new_field()
        st = s(x, b.copy(), raise_on_error=True)
        d = s.stats()
        print(f"status {pps.status_string(st)}: {d['iterations']} iterations, {d['kernel_launches']} launches, "
              f"{d['seconds_solve'] * 1e3:.2f} ms, sweep {d['sweep_bytes'] / max(d['sweep_seconds'], 1e-12) / 1e9:.0f} GB/s")
    s.close()



def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--profile-case":
        profile_case(sys.argv[2:])
        return
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--inner-tol", type=float, default=3e-3)
    ap.add_argument("--learned-inner-tol", type=float, default=1e-5)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-compositions", action="store_true")
    ap.add_argument("--comp-size", type=int, default=256)
    ap.add_argument("--no-large", action="store_true", help="skip the 1024^3 charges solve (~3 min)")
    ap.add_argument("--no-learned-128", action="store_true")
    ap.add_argument("--held-out", type=int, default=64, help="held-out right-hand sides of the 128^3 solves")
    ap.add_argument("--held-out-pairs", type=int, default=1000, help="held-out pairs the network is scored on")
    ap.add_argument("--train-samples", type=int, default=20000)
    ap.add_argument("--train-steps", type=int, default=20000)
    ap.add_argument("--batch-problems", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-threads", type=int, default=0)
    args = ap.parse_args()
    threads = args.cpu_threads or os.cpu_count() or 1

    dist = Dist()
    if args.impl == "reference":
        if dist.rank == 0:
            print(json.dumps(reference_arm(args.size, args.steps, args.warmup, threads, dist.ws)), flush=True)
        dist.close()
        return

    out, iters_fp64 = run_gpu(args, dist)
    if not args.no_batched:
        out["batched"] = run_batched(args, dist)
    if not args.no_compositions and dist.rank == 0:
        out["compositions"] = run_compositions(args, dist.local, threads)
    if not args.no_large and dist.rank == 0:
        out["large_1024"] = run_large(args, dist.local)
    if dist.rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_sample(args.size, REFERENCE_ITERATIONS.get(args.size) or iters_fp64, threads)
        print(json.dumps(out), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
