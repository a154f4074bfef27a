#!/usr/bin/env python
"""Benchmark of the q-LSKUM primal iteration on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision mixed|fp64] [--workload transonic|subsonic]

Workload (default "transonic"): a seeded NACA 0012 point cloud, 1024 wall
points x 1000 rings = 1,024,000 points (first spacing 2e-3 chord, far field
20 chords, 10% jitter, 10 neighbours), M 0.85, AoA 1, CFL 0.2, VL_CONST 50,
limiter on, 3 inner iterations.  A step is one pseudo-time iteration of the
whole cloud (4 SSPRK stages).  Metric: point-iterations per second.

Our arm prints one JSON line with the mixed-precision solve as `value` (or
FP64 with --precision fp64) and, beside it, the FP64 drop-in's rate and the
Cl / Cd difference between the two forms after the same iterations, the
end-to-end rate through the C ABI with host buffers, the roofline of the
dominant kernel and the CPU baseline (the C restatement oracle on the host
cores).  `--impl reference` times the reference algorithm on the host cores
(the oracle restatement: the reference's own sources are not on this
machine) and prints the same metric.

Multi-GPU: the path does not shard (one cloud per solve); with --gpus N every
rank runs an independent replica and `value` is the sum over ranks
("replicas only", weak scaling).
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

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(REPO, "c-_serial_gb300"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOADS = {
    # te_spread: the cosine law's trailing-edge wall spacing of the 160-point
    # ring (3.9e-4 chord) instead of 1e-5 (cloudgen.naca4_surface)
    "transonic": dict(cloud=dict(n_wall=1024, n_layers=1000, first_spacing=2e-3, radius=20.0, seed=2,
                                 te_spread=0.064),
                      solver=dict(mach=0.85, aoa=1.0, cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=3)),
    "subsonic": dict(cloud=dict(n_wall=160, n_layers=60, first_spacing=2e-3, radius=20.0, seed=1),
                     solver=dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=0)),
    # main element + 30%-chord flap at 20 deg, 1.5%-chord slot, ~16M points (two_element_cloud
    # defaults); M 0.2, AoA 8; CFL / VL_CONST / inner iterations as config 1 (the recipe gives none)
    "two_element": dict(cloud=dict(), solver=dict(mach=0.2, aoa=8.0, cfl=0.2, vl_const=50.0, power=0.0,
                                                  inner_iterations=0)),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 20 ms while running
    (nvidia-smi's own loop, one child process, stopped by its own PID)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_ms: int = 20):
        self.gpu = gpu_index
        self.period = period_ms
        self.rows = []
        self._p = None
        self._t = None

    def _read(self):
        for line in self._p.stdout:
            f = [v.strip() for v in line.split(",")]
            if len(f) >= 9:
                self.rows.append(f)

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                        "--format=csv,noheader,nounits", f"-lms={self.period}"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            time.sleep(2.5 * self.period / 1000.0)      # first samples before the timed work
        except Exception:
            self._p = None
        return self

    def __exit__(self, *a):
        if self._p is not None:
            time.sleep(self.period / 1000.0)
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
            if self._t:
                self._t.join(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in self.rows for j in range(4) if len(r) > 5 + j and r[5 + j] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.rows)}


def max_over_ranks(value: float, dist=None, device="cpu") -> float:
    """The slowest rank's time (the whole job's time under weak scaling)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_cloud(workload):
    from qlskum import cloudgen
    if workload == "two_element":
        return cloudgen.two_element_cloud(**WORKLOADS[workload]["cloud"])
    return cloudgen.make_cloud(**WORKLOADS[workload]["cloud"])


def flux_update_bytes(cloud, precision: str, unit_weights: bool = True) -> float:
    """Compulsory bytes one fused flux + update launch moves (each array once).

    Per point: own q / dq / qm, normal, limiter eps^2, delta, flag, nbhs, (FP64:
    the 4 LSQ moment sets, 128 B), prim in, prim out, q out, prim_old on 1
    stage of 4 and the wave speed on 1 of 4 (averaged), slice base; per edge:
    neighbour index, edge vector (mixed, power 0: {delx, dely} FP32; else
    {delx, dely, w delx, w dely}), the folded solve weights of its x and y
    half-ranges (mixed: FP32 pair; FP64: rotated weights {dels w, deln w}),
    membership byte.  Neighbour gathers are served from cache (counted once,
    as the point's own rows).
    """
    n = cloud.n
    e = int(cloud.nbhs.sum())
    if precision == "mixed":
        per_pt = 16 + 32 + 32 + 16 + 4 + 4 + 1 + 4 + 32 + 32 + 16 + 32 / 4 + 4 / 4 + 8 / 32
        per_edge = 4 + 8 + 8 + 1 if unit_weights else 4 + 16 + 8 + 1
    else:
        per_pt = 32 + 64 + 64 + 16 + 8 + 8 + 1 + 4 + 128 + 32 + 32 + 32 + 32 / 4 + 8 / 4 + 8 / 32
        per_edge = 4 + 32 + 16 + 1
    return n * per_pt + e * per_edge


def point_pass_bytes(cloud, precision: str, unit_weights: bool = True) -> dict:
    """Compulsory bytes of one launch of each per-stage kernel, counted like
    flux_update_bytes (each per-point array once per launch that needs it,
    neighbour gathers served from cache, the streamed per-edge data once).

    Mixed form (q, dq, qm FP32):
    * gradient + max / min: own q 16, dq0 32 and qm 32 written, nbhs 4, slice
      base 8/32; per edge neighbour index 4, folded gradient weights 8; the
      first stage of four also the time step (wave speed 4 per point, delta 4
      written, edge length 4 per edge), averaged over the stages;
    * inner step: dq0 32, own dq 32, dq out 32, nbhs and slice base; per edge
      index 4, edge vector 8 (16 with weights), folded weights 8;
    * flux + update: flux_update_bytes.
    FP64 form: the same arrays at 8-byte widths (moments 32 B per point, edge
    vector and weights 32 B per edge in the gradient and inner kernels)."""
    n = cloud.n
    e = int(cloud.nbhs.sum())
    if precision == "mixed":
        grad = n * (16 + 32 + 32 + 4 + 8 / 32 + (4 + 4) / 4) + e * (4 + 8 + 4 / 4)
        inner = n * (32 + 32 + 32 + 4 + 8 / 32) + e * (4 + (8 if unit_weights else 16) + 8)
    else:
        grad = n * (32 + 64 + 64 + 32 + 4 + 8 / 32 + (8 + 8) / 4) + e * (4 + 32 + 8 / 4)
        inner = n * (32 + 64 + 64 + 32 + 4 + 8 / 32) + e * (4 + 32)
    return {"gradient": grad, "inner": inner, "flux_update": flux_update_bytes(cloud, precision, unit_weights)}


def bytes_per_point_iteration(cloud, precision: str, inner: int, unit_weights: bool = True) -> dict:
    """Algorithmic bytes per point-iteration: 4 stages x (gradient + inner x
    inner step + flux + update), from point_pass_bytes, divided by the points.
    FP64 also by the survey's formula 4 (252 + 404 + 220 inner) + 100 (the
    reference's arrays at 10 neighbours)."""
    pb = point_pass_bytes(cloud, precision, unit_weights)
    per = 4 * (pb["gradient"] + inner * pb["inner"] + pb["flux_update"]) / cloud.n
    k = float(cloud.nbhs.mean())
    out = {"bytes": per, "neighbours_per_point": k}
    if precision == "mixed":
        out["formula"] = ("4*((86.25+13K) + inner*(100.25+20K) + (198.25+21K)) with K neighbours per point "
                          "(unit weights; FP32 q/dq/qm, FP64 prim, FP32 folded weights)")
    else:
        out["formula"] = "4*(252 + 404 + 220*inner) + 100 (FP64 arrays, K = 10)"
        out["survey_bytes"] = 4 * (252 + 404 + 220 * inner) + 100
    return out


def measured_profile(workload, precision, kernel, key="traffic"):
    """A per-launch figure of `kernel` from the committed ncu summary of this
    workload, or (None, None): 'traffic' = dram__bytes_read.sum +
    dram__bytes_write.sum, 'inst' = smsp__inst_executed.sum (warp
    instructions).  The summaries carry lines '<key> <precision> <kernel> <value>'."""
    import glob
    family = None
    for path in sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                                              f"*_{workload}_1M.md"))):
        try:
            for line in open(path):
                f = line.strip().strip("`").split()
                if len(f) == 4 and f[0] == key and f[1] == precision:
                    if f[2] == kernel:
                        return float(f[3]), f[2]
                    if f[2].split("<")[0] == kernel.split("<")[0]:
                        family = (float(f[3]), f[2])   # same code and data, another launch shape
        except OSError:
            pass
    return family if family else (None, None)


def flux_kernel_form(variant: int) -> str:
    """Kernel name of a mixed flux_variant (as qlskum_set_launch_config numbers
    them): 4..7 staged gathers, 10..13 register prefetch, 14..18 register
    prefetch with the owner's data in shared memory, else per-edge gathers."""
    if 4 <= variant <= 7:
        return "k_flux_update_st"
    if 10 <= variant <= 13:
        return "k_flux_update_rp"
    if 14 <= variant <= 18:
        return "k_flux_update_rps"
    return "k_flux_update"


def measured_traffic(workload, precision, kernel):
    return measured_profile(workload, precision, kernel, "traffic")


def time_solver(qlskum, torch, solver, steps):
    """Device time of `steps` iterations on the solver's own stream (CUDA events)."""
    stream = torch.cuda.ExternalStream(solver.stream)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    solver.synchronize()
    l0 = solver.launches
    start.record(stream)
    solver.q_lskum(steps)
    end.record(stream)
    end.synchronize()
    solver.synchronize()
    return start.elapsed_time(end) / 1e3, solver.launches - l0


def e2e_rate(qlskum, solver, n, steps, warmup=2):
    """Point-iter/s through the C ABI with host buffers: per step, upload prim
    from pinned host memory, one fpi_solver iteration, read back prim and the
    residual.  `warmup` untimed steps of the same loop come first."""
    import torch
    host = torch.empty((n, 4), dtype=torch.float64).pin_memory()
    host.copy_(torch.from_numpy(solver.prim))
    out = torch.empty((n, 4), dtype=torch.float64).pin_memory()
    arr_in = host.numpy()
    arr_out = out.numpy()
    import ctypes as C
    it = solver.iteration

    def step(arr_in, it):
        solver.set_prim(arr_in)
        solver.fpi_solver(it)
        solver._ck(solver._L.qlskum_get_prim(solver._h, arr_out.ctypes.data_as(C.POINTER(C.c_double))))
        return solver.residual_history()[-1]

    for _ in range(warmup):
        it += 1
        step(arr_in, it)
        arr_in = arr_out
    solver.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        it += 1
        res = step(arr_in, it)
        arr_in = arr_out
    dt = time.perf_counter() - t0
    _ = res
    return n * steps / dt, 32 * n, 32 * n + 24 * it


def cpu_baseline(workload, cloud, threads, iters):
    import qlskum_oracle
    qlskum_oracle.build()
    kw = WORKLOADS[workload]["solver"]
    o = qlskum_oracle.Oracle(cloud, mach=kw["mach"], aoa=kw["aoa"], cfl=kw["cfl"], vl_const=kw["vl_const"],
                             power=kw["power"], inner_iterations=kw["inner_iterations"], threads=threads)
    t0 = time.perf_counter()
    o.run(iters)
    dt = time.perf_counter() - t0
    return cloud.n * iters / dt, dt


def batch_workload(seed=3, n_clouds=32, n_cases=64, size_range=(20_000, 500_000)):
    """Seeded NACA 4-digit clouds (thickness 8-16%, camber 0-4%, camber
    position 0.3-0.5) of 20k-500k points, and flight conditions M 0.5-0.85,
    AoA -2..4 deg; case j solves cloud j mod n_clouds."""
    from qlskum import cloudgen
    rng = np.random.default_rng(seed)
    clouds = []
    for k in range(n_clouds):
        size = int(rng.uniform(*size_range))
        n_wall = max(64, int(round(np.sqrt(size) / 8)) * 8)
        n_layers = max(12, size // n_wall)
        t = rng.uniform(0.08, 0.16)
        m = rng.uniform(0.0, 0.04)
        pc = rng.uniform(0.3, 0.5)
        clouds.append(cloudgen.make_cloud(n_wall=n_wall, n_layers=n_layers, first_spacing=2e-3, radius=20.0,
                                          seed=100 + k, m=m, p=pc, t=t))
    cases = [(j % n_clouds, rng.uniform(0.5, 0.85), rng.uniform(-2.0, 4.0)) for j in range(n_cases)]
    return clouds, cases


def run_adjoint_check(args):
    """The discrete adjoint on the 1.02 M-point NACA 0012 cloud at M 0.63,
    AoA 2: FP64 handle, dCl and dCd w.r.t. Mach, AoA and the normal
    displacement of every wall point through K iterations from the free
    stream (each iteration's state checkpointed), timed against the same K
    primal iterations; checked against central differences of the FP64
    solver (which matches the reference's serial path to 1e-10) on 16 seeded
    wall points (away from the trailing edge) and both scalars.  Wall clock,
    host-synchronous calls."""
    import qlskum
    qlskum.load()
    cloud = make_cloud("transonic")
    kw = dict(WORKLOADS["transonic"]["solver"], mach=0.63, aoa=2.0)
    k, stride = max(1, args.adjoint_iters), args.adjoint_stride
    s = qlskum.Solver(cloud, precision=qlskum.FP64, **kw)
    s.adjoint_gradient("cl", iters=k, wall=True, stride=stride)       # allocation of the K stage sets
    grads, t_adj = {}, {}
    for obj in ("cl", "cd"):
        t0 = time.perf_counter()
        grads[obj] = s.adjoint_gradient(obj, iters=k, wall=True, stride=stride)
        t_adj[obj] = time.perf_counter() - t0
    t0 = time.perf_counter()
    s.q_lskum(k)
    s.synchronize()
    t_pr = time.perf_counter() - t0
    nrm = s.field(qlskum.FIELD_NORMALS)
    shape = s.shape_points
    s.close()

    def objective(mach=kw["mach"], aoa=kw["aoa"], c=cloud):
        t = qlskum.Solver(c, precision=qlskum.FP64, **dict(kw, mach=mach, aoa=aoa))
        t.q_lskum(k)
        cl, cd = t.objective()[:2]
        t.close()
        return {"cl": cl, "cd": cd}

    def moved(m, d):
        from qlskum.cloudgen import Cloud
        x, y = cloud.x.copy(), cloud.y.copy()
        x[m] += d * nrm[m][0]
        y[m] += d * nrm[m][1]
        return Cloud(x, y, cloud.left, cloud.right, cloud.flag_1, cloud.flag_2, cloud.min_dist, cloud.nbhs, cloud.conn)

    t_fd = time.perf_counter()
    hm, ha, hws = 1e-6, 1e-5, (1e-8, 3e-8)
    fd = {"dmach": {}, "daoa": {}}
    a, b = objective(mach=kw["mach"] + hm), objective(mach=kw["mach"] - hm)
    fd["dmach"] = {o: (a[o] - b[o]) / (2 * hm) for o in ("cl", "cd")}
    a, b = objective(aoa=kw["aoa"] + ha), objective(aoa=kw["aoa"] - ha)
    fd["daoa"] = {o: (a[o] - b[o]) / (2 * ha) for o in ("cl", "cd")}
    te = {0, int(cloud.left[0]) - 1, int(cloud.right[0]) - 1}
    rng = np.random.default_rng(16)
    pts = rng.choice(sorted(set(range(shape)) - te), size=16, replace=False)
    err = {o: {"dmach": abs(grads[o]["dmach"] - fd["dmach"][o]) / max(abs(fd["dmach"][o]), 1e-12),
               "daoa": abs(grads[o]["daoa"] - fd["daoa"][o]) / max(abs(fd["daoa"][o]), 1e-12)} for o in ("cl", "cd")}
    # each wall point at two steps: a difference quotient that moves with the
    # step straddles a discontinuity of the map (the limiter's |dn| <= 1e-5
    # cut, a switch of the time step's minimum), which the adjoint, the
    # derivative of the branch taken, does not see
    wall = {o: [] for o in ("cl", "cd")}
    for m in pts:
        q = {o: [] for o in ("cl", "cd")}
        for hw in hws:
            a, b = objective(c=moved(m, hw)), objective(c=moved(m, -hw))
            for o in ("cl", "cd"):
                q[o].append((a[o] - b[o]) / (2 * hw))
        for o in ("cl", "cd"):
            wall[o].append({"point": int(m), "adjoint": float(grads[o]["dwall"][m]), "fd": q[o]})
    for o in ("cl", "cd"):
        scale = float(np.abs(grads[o]["dwall"]).max())
        rel = lambda ad, f: abs(ad - f) / max(abs(f), 1e-2 * scale)
        err[o]["dwall_step_small"] = max(rel(w["adjoint"], w["fd"][0]) for w in wall[o])
        err[o]["dwall_step_large"] = max(rel(w["adjoint"], w["fd"][1]) for w in wall[o])
        # points whose two quotients agree to 1e-3 (no discontinuity within the steps)
        smooth = [w for w in wall[o] if abs(w["fd"][0] - w["fd"][1]) <= 1e-3 * max(abs(w["fd"][0]), 1e-2 * scale)]
        err[o]["dwall_smooth_points"] = len(smooth)
        err[o]["dwall_smooth_max"] = max((rel(w["adjoint"], w["fd"][0]) for w in smooth), default=None)
    t_fd = time.perf_counter() - t_fd
    ratio = max(t_adj.values()) / t_pr
    line = {
        "metric": "adjoint_over_primal", "value": ratio, "unit": "x", "n_gpus": 1, "steps": k, "warmup": 1,
        "ms_per_step": 1e3 * max(t_adj.values()) / k, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "naca0012_1024x1000_adjoint", "points": cloud.n, "mach": kw["mach"], "aoa": kw["aoa"],
                   "inner_iterations": kw["inner_iterations"], "iterations_differentiated": k,
                   "checkpoint_stride": stride, "wall_points": shape, "precision": "fp64",
                   "parallelism": "single"},
        "adjoint": {o: {"seconds": t_adj[o], "dmach": grads[o]["dmach"], "daoa_per_deg": grads[o]["daoa"],
                        "dwall_max_abs": float(np.abs(grads[o]["dwall"]).max())} for o in ("cl", "cd")},
        "primal_seconds": t_pr,
        "fd_check": {"steps": {"mach": hm, "aoa_deg": ha, "wall": list(hws)}, "wall": wall,
                     "max_rel_err": err, "seconds": t_fd,
                     "note": "central differences of the FP64 solver, K iterations from the free stream"},
    }
    print(json.dumps(line), flush=True)


def run_long(args):
    """The mixed and FP64 forms on the same cloud for --long-iters iterations
    from the free stream (the 1.02 M-point transonic recipe runs 5000):
    Cl, Cd, the residual norm and the total entropy of both every
    --long-every iterations, the primitive state's difference at the end.
    Stops at the first non-finite state of either form and says which."""
    import qlskum
    qlskum.load()
    cloud = make_cloud(args.workload)
    kw = WORKLOADS[args.workload]["solver"]
    forms = {"mixed": qlskum.Solver(cloud, precision=qlskum.MIXED, **kw),
             "fp64": qlskum.Solver(cloud, precision=qlskum.FP64, **kw)}
    seconds = {k: 0.0 for k in forms}
    rows, done, failed = [], 0, None
    while done < args.long_iters and failed is None:
        k = min(args.long_every, args.long_iters - done)
        for name, s in forms.items():
            t0 = time.perf_counter()
            try:
                s.q_lskum(k)
                s.synchronize()
            except qlskum.QlskumError as e:
                failed = {"form": name, "before_iteration": done + k, "error": str(e)}
                break
            seconds[name] += time.perf_counter() - t0
        if failed:
            break
        done += k
        obj = {n: s.objective() for n, s in forms.items()}
        res = {n: float(s.residual_history()[-1][0]) for n, s in forms.items()}
        row = {"iteration": done, "cl": obj["fp64"][0], "cd": obj["fp64"][1], "res_fp64": res["fp64"],
               "res_mixed": res["mixed"], "abs_dcl": abs(obj["mixed"][0] - obj["fp64"][0]),
               "abs_dcd": abs(obj["mixed"][1] - obj["fp64"][1]),
               "rel_dentropy": abs(obj["mixed"][3] - obj["fp64"][3]) / abs(obj["fp64"][3])}
        rows.append(row)
        log(json.dumps(row))
    out = {"workload": args.workload, "points": cloud.n,
           "iterations": done, "failed": failed, "seconds": seconds, "history": rows}
    if failed is None:
        pm, pd = forms["mixed"].prim, forms["fp64"].prim
        out["prim_rel_err"] = float((np.abs(pm - pd) / np.abs(pd).max(axis=0)).max())
    print(json.dumps(out), flush=True)


def run_batch(args):
    """Batched launch: 64 flight conditions over 32 uneven clouds, mixed precision."""
    import torch
    import qlskum
    qlskum.load()
    t0 = time.perf_counter()
    clouds, cases = batch_workload()
    log(f"batch: {len(clouds)} clouds, {sum(c.n for c in clouds)} cloud points, generated in "
        f"{time.perf_counter() - t0:.1f}s")
    kw = dict(cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=3)
    # at most 20 timed iterations: some of the 64 transonic cases drift to a
    # non-finite state within ~100 iterations on these synthetic clouds
    args.steps = min(args.steps, 20)
    b = qlskum.Batch(clouds, cases, **kw)
    b.run(args.warmup)
    stream = torch.cuda.ExternalStream(b.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = b.launches
    with ClockSampler(0) as clocks:
        e0.record(stream)
        b.run(args.steps)
        e1.record(stream)
        e1.synchronize()
    dt = e0.elapsed_time(e1) / 1e3
    value = b.total_points * args.steps / dt
    cl, cd, _, _ = b.objective()
    # per-case Cl / Cd against the FP64 form of the same case and iterations (first 4 cases)
    errs = []
    for k in range(min(4, len(cases))):
        ci, mach, aoa = cases[k]
        s = qlskum.Solver(clouds[ci], mach=mach, aoa=aoa, precision=qlskum.FP64, **kw)
        s.q_lskum(args.warmup + args.steps)
        c64 = s.objective()
        errs.append({"case": k, "points": clouds[ci].n, "mach": mach, "aoa": aoa, "cl": cl[k],
                     "abs_dcl": abs(cl[k] - c64[0]), "abs_dcd": abs(cd[k] - c64[1])})
        del s
    line = {"metric": "point-iter/s", "value": value, "unit": "point-iter/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "batch_64_conditions_32_clouds", "cases": len(cases),
                       "points": b.total_points, "cloud_sizes": [c.n for c in clouds], **kw,
                       "precision": "mixed"},
            "clocks": clocks.summary(), "gpu_launches": b.launches - l0, "tuning": b.tuning(),
            "cl_vs_fp64": errs}
    print(json.dumps(line), flush=True)


def batch_leg(torch, qlskum, warmup=3, steps=10):
    """The batched launch on a reduced config-3 workload for the default
    line: 8 seeded NACA 4-digit clouds of 20k-100k points, 16 flight
    conditions (M 0.5-0.85, AoA -2..4 deg), mixed precision, 3 inner
    iterations, autotuned; aggregate point-iter/s over all cases (CUDA
    events on the batch's stream)."""
    t0 = time.perf_counter()
    clouds, cases = batch_workload(seed=4, n_clouds=8, n_cases=16, size_range=(20_000, 100_000))
    t_gen = time.perf_counter() - t0
    kw = dict(cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=3)
    b = qlskum.Batch(clouds, cases, **kw)
    b.run(warmup)
    stream = torch.cuda.ExternalStream(b.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = b.launches
    e0.record(stream)
    b.run(steps)
    e1.record(stream)
    e1.synchronize()
    dt = e0.elapsed_time(e1) / 1e3
    cl, cd, _, _ = b.objective()
    out = {"workload": "batch_16_conditions_8_clouds_20k_100k", "value": b.total_points * steps / dt,
           "unit": "point-iter/s", "steps": steps, "warmup": warmup, "ms_per_step": dt / steps * 1e3,
           "cases": len(cases), "points": b.total_points, "cloud_sizes": [c.n for c in clouds],
           "gpu_launches": b.launches - l0, "tuning": b.tuning(), "finite": bool(np.isfinite(cl).all()),
           "cloud_generation_s": t_gen, **kw}
    b.close()
    return out


def two_element_leg(torch, qlskum, warmup=3, steps=10, fp64_steps=3, adjoint_iters=4, adjoint_stride=1):
    """Config 5 at a reduced size for the default line: the two-element cloud
    (NACA 0012 main element + 30%-chord flap at 20 deg, 1.5%-chord slot,
    4096 + 1024 wall points) with a coarser background (h0 4e-4, growth
    0.04: ~450k points instead of ~16M), M 0.2, AoA 8, inner 0.  Mixed
    point-iter/s (CUDA events on the library's stream), the FP64 form on the
    same cloud and iteration count for the ratio and the Cl / Cd gap, and
    the mixed adjoint of Cl (every iteration's stage data kept, as in the
    1.02 M legs) against the same primal iterations."""
    t0 = time.perf_counter()
    cloud = cloudgen_mod().two_element_cloud(h0=4e-4, growth=0.04)
    t_gen = time.perf_counter() - t0
    kw = WORKLOADS["two_element"]["solver"]
    s = qlskum.Solver(cloud, precision=qlskum.MIXED, **kw)
    s.q_lskum(warmup)
    dt, launches = time_solver(qlskum, torch, s, steps)
    cl, cd, _, _ = s.objective()
    f = qlskum.Solver(cloud, precision=qlskum.FP64, **kw)
    f.q_lskum(warmup)
    dt64, _ = time_solver(qlskum, torch, f, fp64_steps)
    f.q_lskum(steps - fp64_steps)
    cl64, cd64, _, _ = f.objective()
    f.close()
    adj = measure_adjoint(s, "mixed", adjoint_iters, adjoint_stride, cloud.n)
    s.close()
    return {"workload": "two_element_450k", "points": cloud.n, "value": cloud.n * steps / dt,
            "unit": "point-iter/s", "steps": steps, "warmup": warmup, "ms_per_step": dt / steps * 1e3,
            "gpu_launches": launches, "fp64_point_iter_s": cloud.n * fp64_steps / dt64,
            "after_iterations": warmup + steps, "cl": cl, "cd": cd, "abs_dcl": abs(cl - cl64),
            "abs_dcd": abs(cd - cd64), "adjoint_mixed": adj, "cloud_generation_s": t_gen,
            "cloud": {"h0": 4e-4, "growth": 0.04, "n_main": 4096, "n_flap": 1024}, **kw}


def cloudgen_mod():
    from qlskum import cloudgen
    return cloudgen


def run_reference(args, rank, world):
    if rank != 0:
        return
    workload = args.workload
    if workload not in WORKLOADS:
        # the batch and adjoint measurements have no single-cloud CPU counterpart
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU reference run for the {workload} workload"}),
              flush=True)
        return
    import qlskum_oracle
    qlskum_oracle.build()
    threads = os.cpu_count() or 1
    # the same cloud as our arm; the timed iterations bounded to about two
    # minutes of host time (the rate is per point-iteration, so a shorter
    # sample of the same workload measures the same quantity)
    cloud = make_cloud(workload)
    kw = WORKLOADS[workload]["solver"]
    o = qlskum_oracle.Oracle(cloud, mach=kw["mach"], aoa=kw["aoa"], cfl=kw["cfl"], vl_const=kw["vl_const"],
                             power=kw["power"], inner_iterations=kw["inner_iterations"], threads=threads)
    t0 = time.perf_counter()
    o.run(1)
    t_first = time.perf_counter() - t0
    warm = max(0, min(args.warmup, int(20.0 / max(t_first, 1e-9))) - 1)
    if warm:
        o.run(warm)
    steps = max(1, min(args.steps, int(120.0 / max(t_first, 1e-9))))
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    v = cloud.n * steps / dt
    line = {
        "impl": "reference", "metric": "point-iter/s", "value": v, "unit": "point-iter/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(workload, cloud),
        "cpu_baseline": {"value": v, "unit": "point-iter/s", "cores": threads, "kind": "port",
                         "sample": f"the same {cloud.n}-point cloud, {steps} timed iterations after {1 + warm} "
                                   f"warm-up, C restatement of the reference's serial FP64 path with OpenMP "
                                   f"over points"},
        "e2e": {"value": v, "unit": "point-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(workload, cloud=None):
    w = WORKLOADS[workload]
    if workload == "two_element":
        c = dict(workload="naca0012_plus_30pct_flap_20deg_slot1.5pct", **w["solver"])
        c["points"] = cloud.n if cloud is not None else None
        c["l2"] = "inputs larger than L2; no flush"
        return c
    c = dict(workload=f"naca0012_{w['cloud']['n_wall']}x{w['cloud']['n_layers']}", **w["solver"])
    c["points"] = w["cloud"]["n_wall"] * w["cloud"]["n_layers"]
    c["l2"] = "inputs larger than L2 (edge arrays alone > 129 MB); no flush" if workload == "transonic" else \
        "inputs smaller than L2"
    return c


def measure_adjoint(sf, precision, k, stride, n):
    """Wall-clock cost of one adjoint gradient (K kept iterations reversed)
    and of one fixed-point adjoint iteration, each over the same handle's
    primal iteration."""
    # untimed: the first call allocates; the primal's state buffers rotate
    # through three phases with one captured graph each, so three calls of K
    # iterations start in every phase before the timed one
    for _ in range(3):
        sf.adjoint_gradient("cl", iters=k, stride=stride)
    t0 = time.perf_counter()
    g = sf.adjoint_gradient("cl", iters=k, stride=stride)
    t_adj = time.perf_counter() - t0
    t0 = time.perf_counter()
    sf.q_lskum(k)
    sf.synchronize()
    t_pr = time.perf_counter() - t0
    # steady-state form: adjoint iterations at the current state, per iteration
    sf.adjoint_fixed_point("cl", adj_iters=k)
    sf.adjoint_fixed_point("cl", adj_iters=2 * k)
    t0 = time.perf_counter()
    sf.adjoint_fixed_point("cl", adj_iters=k)
    t_a = time.perf_counter() - t0
    t0 = time.perf_counter()
    sf.adjoint_fixed_point("cl", adj_iters=2 * k)
    t_b = time.perf_counter() - t0
    fp_it = max(t_b - t_a, 1e-9) / k
    return {"objective": "cl", "iterations": k, "points": n, "checkpoint_stride": stride,
            "primal_precision": precision,
            "reverse": "mixed iteration (FP32 edge work, FP64 update)" if precision == "mixed" else "FP64 iteration",
            "checkpointed": {"seconds": t_adj, "primal_seconds": t_pr, "adjoint_over_primal": t_adj / t_pr,
                             "note": "K primal iterations from the free stream, kept, then reversed"},
            "fixed_point": {"seconds_per_adjoint_iteration": fp_it,
                            "seconds_per_primal_iteration": t_pr / k,
                            "adjoint_over_primal": fp_it / (t_pr / k)},
            "dcl_dmach": g["dmach"], "dcl_daoa_per_deg": g["daoa"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="transonic", choices=sorted(WORKLOADS) + ["batch", "adjoint"],
                    help="adjoint: the FP64 adjoint on the 1.02 M cloud at M 0.63, AoA 2, with its FD check")
    ap.add_argument("--adjoint-stride", type=int, default=1,
                    help="adjoint checkpoint stride in iterations (2 = every 8 SSPRK steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--cpu-iters", type=int, default=3,
                    help="iterations of the CPU baseline (one core and all cores)")
    ap.add_argument("--no-batch-leg", dest="batch_leg", action="store_false",
                    help="skip the reduced batched-launch and two-element legs of the default line")
    ap.add_argument("--adjoint-iters", type=int, default=3,
                    help="iterations differentiated by the adjoint timings (FP64 and mixed handles; 0: skip)")
    ap.add_argument("--long-iters", type=int, default=0,
                    help="instead of the benchmark: the mixed and FP64 forms side by side for this many "
                         "iterations (Cl, Cd, residual, entropy every --long-every)")
    ap.add_argument("--long-every", type=int, default=500)
    ap.add_argument("--launch", default="auto",
                    help="mixed launch shape 'flux_variant,point_block,staged' (e.g. 6,64,0) instead of autotuning")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "batch":
        if rank == 0:
            run_batch(args)
        return
    if args.workload == "adjoint":
        if rank == 0:
            run_adjoint_check(args)
        return
    if args.long_iters:
        if rank == 0:
            run_long(args)
        return

    import torch
    import qlskum
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    qlskum.load()
    t_gen = time.perf_counter()
    cloud = make_cloud(args.workload)
    log(f"cloud {cloud.n} points generated in {time.perf_counter() - t_gen:.1f}s")
    kw = WORKLOADS[args.workload]["solver"]
    prec = qlskum.MIXED if args.precision == "mixed" else qlskum.FP64
    solver = qlskum.Solver(cloud, precision=prec, **kw)
    if args.launch != "auto" and prec == qlskum.MIXED:
        solver.set_launch_config(*[int(v) for v in args.launch.split(",")])
    solver.q_lskum(args.warmup)
    solver.synchronize()

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(local) as clocks:
        dt, launches = time_solver(qlskum, torch, solver, args.steps)
    barrier()
    dt = max_over_ranks(dt, pg, "cuda")
    value = cloud.n * args.steps * world / dt
    cl, cd, cm, ent = solver.objective()

    # per-kernel device time of the dominant kernel (events around each launch)
    solver.set_kernel_timing(True)
    solver.q_lskum(2)
    kt = solver.kernel_timing()
    solver.set_kernel_timing(False)
    fl_ms, fl_n = kt["flux_update"]
    total_ms = sum(v[0] for v in kt.values())
    peak, peak_kind = measured_peaks()
    unit_w = kw["power"] == 0.0
    pbytes = point_pass_bytes(cloud, args.precision, unit_w)
    nbytes = pbytes["flux_update"]
    achieved = nbytes / (fl_ms / fl_n / 1e3) / 1e9
    lc = solver.launch_config()
    kname = (f"{flux_kernel_form(lc['flux_variant'])}<{lc['flux_block']},{lc['flux_min_blocks']}>"
             if prec == qlskum.MIXED else "k_flux_update<128>")
    traffic, traffic_kernel = measured_traffic(args.workload, args.precision, kname)
    # every per-stage kernel against HBM (event-timed launches, compulsory
    # bytes), with its ncu DRAM traffic per launch where a committed summary has it
    names = {"gradient": "k_q_derivatives", "inner": "k_q_inner", "flux_update": kname}
    kernels = {}
    for kk in ("gradient", "inner", "flux_update"):
        ms, nl = kt[kk]
        if nl:
            a = pbytes[kk] / (ms / nl / 1e3) / 1e9
            tr, tr_k = measured_traffic(args.workload, args.precision, names[kk])
            kernels[kk] = {"kernel": names[kk], "algorithmic_bytes_per_launch": pbytes[kk],
                           "avg_launch_ms": ms / nl, "launches": nl, "achieved_gbs": a, "frac": a / peak,
                           "share": ms / total_ms, "traffic": tr, "traffic_captured_on": tr_k}
    # the flux kernel's instruction-issue roofline: its warp instructions
    # per launch (ncu, committed summary) over 152 SMs x 4 schedulers x the
    # SM clock sampled in the timed region
    inst, inst_kernel = measured_profile(args.workload, args.precision, kname, "inst")
    sm_mhz = clocks.summary().get("sm_mhz") or 2070.0
    issue = None
    bound = "hbm"
    if inst:
        n_sm = torch.cuda.get_device_properties(0).multi_processor_count
        t_issue = inst / (n_sm * 4 * sm_mhz * 1e6)
        issue = {"warp_instructions_per_launch": inst, "captured_on": inst_kernel, "sms": n_sm,
                 "sm_mhz": sm_mhz, "issue_limited_ms": t_issue * 1e3,
                 "frac": t_issue / (fl_ms / fl_n / 1e3),
                 "note": "1.0 = one warp instruction per scheduler per cycle for the whole launch"}
        bound = "issue" if issue["frac"] > achieved / peak else "hbm"
    if "flux_update" in kernels:
        kernels["flux_update"].update(bound=bound, issue=issue)
    # the line's roofline is the dominant kernel's: the largest share of the
    # iteration's device time (all three stay in `kernels`)
    dom = max(kernels, key=lambda k: kernels[k]["share"]) if kernels else "flux_update"
    if dom == "flux_update" or dom not in kernels:
        roofline = {"bound": bound, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": traffic, "traffic_captured_on": traffic_kernel,
                    "kernel": f"{kname} ({args.precision})", "algorithmic_bytes_per_launch": nbytes,
                    "avg_launch_ms": fl_ms / fl_n, "kernel_share": fl_ms / total_ms}
    else:
        kd = kernels[dom]
        roofline = {"bound": "hbm", "achieved": kd["achieved_gbs"], "peak": peak, "unit": "GB/s",
                    "frac": kd["frac"], "traffic": kd["traffic"], "traffic_captured_on": kd["traffic_captured_on"],
                    "kernel": f"{kd['kernel']} ({args.precision})",
                    "algorithmic_bytes_per_launch": kd["algorithmic_bytes_per_launch"],
                    "avg_launch_ms": kd["avg_launch_ms"], "kernel_share": kd["share"]}
    roofline.update({"peak_source": f"{peak_kind} hbm_gbs", "dominant": dom, "issue": issue, "kernels": kernels,
                     "note": "achieved = algorithmic bytes per launch / event-timed launch; the dominant kernel "
                             "has the largest share of the iteration; issue = the flux kernel's issue roofline"})
    bpi = bytes_per_point_iteration(cloud, args.precision, kw["inner_iterations"], unit_w)
    whole = bpi["bytes"] * cloud.n / (dt / args.steps) / 1e9
    roofline["iteration"] = dict(bpi, achieved_gbs=whole, frac=whole / peak,
                                 note="bytes per point-iteration x points / ms_per_step")

    # the other form on the same cloud and iteration count, for the ratio and the Cl / Cd gap
    other = qlskum.FP64 if prec == qlskum.MIXED else qlskum.MIXED
    s2 = qlskum.Solver(cloud, precision=other, **kw)
    s2.q_lskum(args.warmup)
    dt2, _ = time_solver(qlskum, torch, s2, args.fp64_steps if other == qlskum.FP64 else args.steps)
    n2 = args.fp64_steps if other == qlskum.FP64 else args.steps
    v2 = cloud.n * n2 * world / dt2
    s2.q_lskum(args.steps - n2) if args.steps > n2 else None
    cl2, cd2, cm2, ent2 = s2.objective()
    fp64_value, mixed_value = (v2, value) if other == qlskum.FP64 else (value, v2)
    r1 = float(solver.residual_history()[-1][0])
    r2 = float(s2.residual_history()[-1][0])
    ent64 = ent2 if other == qlskum.FP64 else ent
    compare = {"fp64_point_iter_s": fp64_value, "mixed_point_iter_s": mixed_value,
               "mixed_over_fp64": mixed_value / fp64_value, "fp64_timed_iterations": n2,
               "after_iterations": args.warmup + args.steps,
               "cl": cl, "cd": cd, "abs_dcl": abs(cl - cl2), "abs_dcd": abs(cd - cd2),
               "total_entropy_fp64": ent64, "abs_dentropy": abs(ent - ent2),
               "rel_dentropy": abs(ent - ent2) / max(abs(ent64), 1e-300),
               "res_new_mixed": r1 if prec == qlskum.MIXED else r2,
               "res_new_fp64": r2 if prec == qlskum.MIXED else r1,
               "rel_dres": abs(r1 - r2) / max(abs(r2 if prec == qlskum.MIXED else r1), 1e-300)}

    # discrete adjoint: dCl/dMach, dCl/dAoA through K iterations from the
    # free stream (checkpointed primal + reverse sweep), against the same K
    # primal iterations on the same handle; host-synchronous calls, wall
    # clock.  The FP64 handle (the drop-in form) and the mixed handle (the
    # reverse of the mixed iteration); the two-element workload only the
    # mixed one.
    adjoint = adjoint_mixed = None
    if args.adjoint_iters > 0:
        mixed_h = solver if prec == qlskum.MIXED else s2
        fp64_h = s2 if prec == qlskum.MIXED else solver
        adjoint_mixed = measure_adjoint(mixed_h, "mixed", args.adjoint_iters, args.adjoint_stride, cloud.n)
        if args.workload != "two_element":
            adjoint = measure_adjoint(fp64_h, "fp64", args.adjoint_iters, args.adjoint_stride, cloud.n)
    del s2

    # end to end through the C ABI with host buffers
    e2e_steps = max(3, min(args.steps, 10))
    e2e_v, h2d, d2h = e2e_rate(qlskum, solver, cloud.n, e2e_steps)
    e2e_v *= world

    batch = two_el = None
    if rank == 0 and world == 1 and args.batch_leg and args.workload == "transonic":
        batch = batch_leg(torch, qlskum)
        two_el = two_element_leg(torch, qlskum)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the reference's serial path on one host core (the benchmark spec's
        # baseline), and the same code on every host core beside it
        ci = args.cpu_iters
        cv, cdt = cpu_baseline(args.workload, cloud, 1, ci)
        thr = os.cpu_count() or 1
        cv_all, cdt_all = cpu_baseline(args.workload, cloud, thr, ci)
        cpu = {"value": cv, "unit": "point-iter/s", "cores": 1, "kind": "port",
               "sample": f"{ci} iterations of the same {cloud.n}-point cloud from the free stream ({cdt:.1f}s), "
                         f"C restatement of the reference's serial FP64 path (bit-identical to it on x86-64), "
                         f"one core",
               "all_cores": {"value": cv_all, "cores": thr, "seconds": cdt_all, "iterations": ci}}

    if rank == 0:
        line = {
            "metric": "point-iter/s", "value": value, "unit": "point-iter/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": dict(workload_config(args.workload, cloud), precision=args.precision,
                           parallelism="replicas" if world > 1 else "single"),
            "clocks": clocks.summary(), "gpu_launches": launches,
            "e2e": {"value": e2e_v, "unit": "point-iter/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": roofline, "cpu_baseline": cpu, "fp64_vs_mixed": compare, "adjoint": adjoint,
            "adjoint_mixed": adjoint_mixed, "batch": batch, "two_element": two_el,
            "kernel_ms_per_iteration": {k: v[0] / max(1, 2) for k, v in kt.items()},
            "launch_config": solver.launch_config(),
        }
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
