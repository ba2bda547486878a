#!/usr/bin/env python3
"""Throughput of the DFSPH step in particle-steps/s on the 1M-fluid dam break.

Workload (one "step" = one frame of mps::System::OnUpdate over the whole scene): 100^3 fluid
particles (r = 0.005, spacing 0.01, seeded jitter +-0.001) in a 3 x 1.5 x 2 m tank with ~210k
single-layer wall particles, y up, open top, cubic spline kernel, rho0 1000, viscosity 0.01,
surface tension 0.05, dt 5e-4, 0.1 % density / divergence tolerances (synthetic data of the
stated shape; the reference ships no dataset).

value: fluid particles x timed steps / device time (CUDA events on the launching stream, max
over ranks), inputs resident in HBM.  e2e: the same through the host-buffer C-ABI call
(mps_step_host: pinned H2D of the state, step, D2H of the state, every step).  roofline: the
dominant kernel's algorithmic bytes per launch / its mean launch time (CUDA events), against the
measured HBM copy bandwidth.  cpu_baseline: the FP64 OpenMP oracle on the host cores.
--impl reference: the reference's own CUDA step (moonsh5009/MPS_CUDA, FP64, rebuilt headless for
sm_103a) on the same workload; under torchrun only rank 0 runs it.
With --gpus N > 1 every rank runs its own replica (the step does not shard without a halo
exchange), so total work grows with N (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s (DFSPH, 1M fluid)"
UNIT = "particle-steps/s"
# algorithmic bytes per fluid particle of each kernel (compulsory SoA FP32 traffic) and per
# boundary particle of a boundary-reading pass
ALGO_BYTES = {"pressure_A": 44, "pressure_B": 52, "cg_ap": 72, "cg_vector": 112}
BOUNDARY_BYTES = 16


def overrides(args) -> dict:
    """Library config fields set on the command line."""
    out = {}
    if args.cg_form is not None:
        out["cg_form"] = args.cg_form
    if args.block_size is not None:
        out["block_size"] = args.block_size
    if getattr(args, "stage", None) is not None:
        out["stage"] = args.stage
    return out


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def radix_passes(sim) -> int:
    return int(sim.stats()["sort_passes"])


def workload_config(scene, world: int = 1) -> dict:
    """The `config` object of both arms' JSON lines (same keys and values for the same workload)."""
    cfg = scene.config
    return {"workload": scene.name, "fluid_particles": scene.n, "boundary_particles": scene.nb,
            "kernel": "cubic spline" if cfg.get("kernel", 1) == 1 else "poly6 / spiky",
            "dt": scene.physics["dt"],
            "tolerances": "density %g, divergence %g, CG r.r %g" % (cfg.get("cd_tol", 1e-3), cfg.get("df_tol", 1e-3),
                                                                 cfg.get("cg_tol", 1e-2)),
            "l2": "inputs larger than L2: state + neighbour lists + CG vectors ~%.0f MB > 129 MB"
                  % ((scene.n * (32 + 4 * 40 + 80)) / 1e6),
            "parallelism": "replicas" if world > 1 else "single"}


def cpu_baseline(scene, pos4, vel4, gpu_iters, budget_s: float = 12.0, max_steps: int = 6):
    """FP64 OpenMP oracle on the host cores, on the GPU's timed window: it starts from the GPU's
    state at the start of that window (pos4 / vel4 in particle-ID order) and runs whole steps
    until `budget_s` of CPU time has passed (at least one step)."""
    import numpy as np
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    o = O.from_scene(scene, threads=threads)
    o.set_fluid(pos4[:, :3].astype(np.float64), vel4[:, :3].astype(np.float64), vel4[:, 3].astype(np.float64),
                pos4[:, 3].astype(np.float64))
    steps, iters = 0, []
    t0 = time.perf_counter()
    while steps < max_steps and (steps == 0 or time.perf_counter() - t0 < budget_s):
        o.step(1)
        st = o.stats()
        iters.append([st["df_iters"], st["cg_iters"], st["cd_iters"]])
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": scene.n * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the first {steps} step(s) of the GPU's timed window of {scene.name} ({scene.n} fluid, "
                      f"{scene.nb} boundary), from the GPU's state at the window's start; FP64 OpenMP restatement "
                      f"of the reference step on {threads} host threads, {dt:.1f} s",
            "iterations_per_step": iters, "gpu_iterations_per_step_mean": gpu_iters}


def run_ours(args, scene, rank, world, local_rank):
    import torch
    from mps_cuda_gb300 import Simulation, build
    from mps_cuda_gb300._lib import K_BUILD_NBRS, K_CG_AP, K_CG_VECTOR, K_DENSITY_ALPHA, K_PRESSURE_A, K_PRESSURE_B

    build.build()
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    sim = Simulation.from_scene(scene, device=local_rank, use_graph=0 if args.eager else 1, **overrides(args))

    def barrier():
        if dist:
            import torch.distributed as td
            td.barrier()

    sim.step(args.warmup, stream)
    torch.cuda.synchronize(dev)
    st0 = sim.stats()
    snap_p, snap_v = sim.get_fluid(stream)  # e2e replays the same steps from this state
    barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    repeat_ms = []
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        sim.step(args.steps, stream)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize(dev)
        barrier()
        ms = e0.elapsed_time(e1)
        st1 = sim.stats()
        # further windows of the same length continuing the run (spread of the figure, and more
        # clock samples under load); `value` is the first window's
        # (the windows differ in work: the scene evolves, and so do the solvers' iteration counts)
        win_iters = []
        prev = st1
        for _ in range(args.repeats):
            r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            r0.record(stream)
            sim.step(args.steps, stream)
            r1.record(stream)
            r1.synchronize()
            repeat_ms.append(r0.elapsed_time(r1) / args.steps)
            cur = sim.stats()
            win_iters.append([(cur["iters_total"][k] - prev["iters_total"][k]) / args.steps for k in range(3)])
            prev = cur
    torch.cuda.synchronize(dev)
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if dist:
        import torch.distributed as td
        td.all_reduce(t, op=td.ReduceOp.MAX)
    ms_max = float(t.item())
    value = scene.n * args.steps * world / (ms_max / 1e3)
    runs = [st1["runs_total"][k] - st0["runs_total"][k] for k in range(3)]
    passes = [st1["passes_total"][k] - st0["passes_total"][k] for k in range(3)]
    iters = [st1["iters_total"][k] - st0["iters_total"][k] for k in range(3)]
    P = radix_passes(sim)
    static = sim.launches_per_step((0, 0, 0), P)
    launches = args.steps * static + sim.launches_per_step(tuple(passes), P) - static

    # ---- e2e through the host-buffer C-ABI call (pinned H2D + step + D2H every step), replaying
    # the timed steps from the same starting state
    pin_p = torch.empty((scene.n, 4), dtype=torch.float32, pin_memory=True)
    pin_v = torch.empty((scene.n, 4), dtype=torch.float32, pin_memory=True)
    e2e_steps = args.steps
    pin_p.numpy()[:] = snap_p
    pin_v.numpy()[:] = snap_v
    torch.cuda.synchronize(dev)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.step_host(pin_p.numpy(), pin_v.numpy(), 1, stream)
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if dist:
        import torch.distributed as td
        td.all_reduce(t, op=td.ReduceOp.MAX)
    e2e_s = float(t.item())
    e2e = {"value": scene.n * e2e_steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 32 * scene.n,
           "d2h_bytes_per_step": 32 * scene.n, "steps": e2e_steps}

    # ---- roofline of the dominant kernel (CUDA events on the same stream, after the timed work)
    reps = 20
    t_a = sim.profile_kernel(K_PRESSURE_A, reps, stream)
    t_b = sim.profile_kernel(K_PRESSURE_B, reps, stream)
    t_ap = sim.profile_kernel(K_CG_AP, reps, stream)
    shares = {"pressure_A": t_a * (runs[0] + runs[2]), "pressure_B": t_b * (runs[0] + runs[2]), "cg_ap": t_ap * runs[1]}
    per = {"pressure_A": t_a, "pressure_B": t_b, "cg_ap": t_ap}
    if not args.cg_form:  # three-pass CG (default): its update + direction passes
        per["cg_vector"] = sim.profile_kernel(K_CG_VECTOR, reps, stream)
        shares["cg_vector"] = per["cg_vector"] * runs[1]
    # once-a-step passes (not roofline candidates: no per-launch byte count is claimed for them)
    once = {"build_nbrs": sim.profile_kernel(K_BUILD_NBRS, 5, stream),
            "density_alpha": sim.profile_kernel(K_DENSITY_ALPHA, 5, stream)}
    dom = max(shares, key=shares.get)
    bnd = scene.nb if dom.startswith("pressure") else 0
    algo = ALGO_BYTES[dom] * scene.n + BOUNDARY_BYTES * bnd
    peak, src = measured_peaks()
    achieved = algo / (per[dom] / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "dram_traffic.json"
    if tf.exists():
        d = json.loads(tf.read_text()).get(dom)
        if d:
            traffic = d.get("bytes_per_launch_full_workload")
    step_algo = (432 + 96 * (runs[0] + runs[2]) / args.steps + 184 * runs[1] / args.steps) * scene.n + \
        16 * scene.nb * (1 + 2 * (runs[0] + runs[2]) / args.steps)
    metric = METRIC if scene.name == "dam_break_1m" else f"particle-steps/s (DFSPH, {scene.name})"
    line = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": workload_config(scene, world),
        "iterations_per_step": {"df": iters[0] / args.steps, "cg": iters[1] / args.steps, "cd": iters[2] / args.steps},
        "windows": {"ms_per_step": [ms_max / args.steps] + repeat_ms,
                    "median_ms_per_step": statistics.median([ms_max / args.steps] + repeat_ms),
                    "iterations_per_step_df_cg_cd": [[iters[k] / args.steps for k in range(3)]] + win_iters,
                    "note": "the timed window, then %d more windows of %d steps continuing the run" %
                            (len(repeat_ms), args.steps)},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": src, "traffic": traffic, "traffic_source": "profiles/dram_traffic.json (ncu capture at 512k particles scaled to 1M)" if traffic else None,
                     "algorithmic_bytes_per_launch": algo, "ms_per_launch": per[dom],
                     "ms_per_launch_all": per, "ms_per_launch_once_a_step": once,
                     "solver_loop_kernels_ms_per_step": sum(shares.values()) / args.steps},
        "step_roofline": {"algorithmic_bytes_per_step": step_algo,
                          "achieved_gbs": step_algo / (ms_max / args.steps / 1e3) / 1e9},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scene, snap_p, snap_v,
                                            [iters[k] / args.steps for k in range(3)])
    if dist:
        import torch.distributed as td
        td.destroy_process_group()
    return line


def run_batched(args, scenes_list, rank, world, local_rank):
    """256 independent scenes: one set of launches per pass over all scenes (CUDA graph, device
    loops that run until every scene has converged) vs. the same scenes stepped one by one."""
    import torch
    from mps_cuda_gb300 import BatchedSimulation, Simulation, build
    from mps_cuda_gb300.sharding import partition_scenes
    build.build()
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    mine = partition_scenes([s.n for s in scenes_list], world)[rank]
    local = [scenes_list[i] for i in mine]
    n_local = sum(s.n for s in local)
    from mps_cuda_gb300.autotune import autotune
    best, tuned = autotune(lambda **c: BatchedSimulation(local, device=local_rank, **c))
    sim = BatchedSimulation(local, device=local_rank, **best)
    sim.step(args.warmup, stream)
    torch.cuda.synchronize(dev)
    st0 = sim.stats()
    if dist:
        import torch.distributed as td
        td.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        sim.step(args.steps, stream)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    st1 = sim.stats()
    passes = [st1["passes_total"][k] - st0["passes_total"][k] for k in range(3)]
    P = radix_passes(sim)
    static = sim.launches_per_step((0, 0, 0), P)
    launches = args.steps * static + sim.launches_per_step(tuple(passes), P) - static
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    tot = torch.tensor([n_local], dtype=torch.float64, device=dev)
    if dist:
        import torch.distributed as td
        td.all_reduce(t, op=td.ReduceOp.MAX)
        td.all_reduce(tot)
    ms_max = float(t.item())
    value = float(tot.item()) * args.steps / (ms_max / 1e3)
    its = sim.scene_iters()
    sim.close()
    # the same scenes, one plain step each, launched one scene after the other
    sims = [Simulation.from_scene(s, device=local_rank) for s in local]
    for s in sims:
        s.step(args.warmup, stream)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for s in sims:
        s.step(1, stream)
    e1.record(stream)
    e1.synchronize()
    per_ms = e0.elapsed_time(e1)
    per_value = n_local / (per_ms / 1e3)
    for s in sims:
        s.close()
    line = {
        "metric": "particle-steps/s (DFSPH, 256 batched scenes)", "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched_256", "scenes": len(scenes_list), "fluid_particles": sum(s.n for s in scenes_list),
                   "boundary_particles": sum(s.nb for s in scenes_list), "parallelism": "scenes split over ranks"},
        "per_scene_launches": {"value": per_value, "unit": UNIT, "ms_for_all_scenes_one_step": per_ms},
        "batched_over_per_scene": value / per_value,
        "autotuned": {"best": best, "ms_per_step": {f"bs{c['block_size']}_d{c['sort_digit_bits']}_u{c.get('cg_unroll', 4)}": round(ms, 3)
                                                    for ms, c in tuned}},
        "max_iterations": {"df": int(its[:, 0].max()), "cg": int(its[:, 1].max()), "cd": int(its[:, 2].max())},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if dist:
        import torch.distributed as td
        td.destroy_process_group()
    return line


def adjoint_launches(sim, K: int, nsteps: int, every: int, radix: int, dpasses) -> int:
    """Kernel launches of one forward + reverse: graph steps (forward and segment recompute), the
    recorded eager step and the reverse kernels of every step.  dpasses: the solver passes the
    steps launched (DF, Jacobi, CD; the stats' passes_total over the run)."""
    static = sim.launches_per_step((0, 0, 0), radix)
    nseg = (nsteps + every - 1) // every
    nrun = nsteps + (nsteps - nseg) + nsteps       # forward, segment recompute, recorded steps
    loops = sim.launches_per_step(tuple(dpasses), radix) - static
    eager_extra = 2               # recorded step: solver init/finish around the Jacobi sweeps
    reverse = 10 + 5 * K          # gather, index, collision, 2K CD, K Jacobi, set-up, ST factor, 2K DF, density x2, scatter, sums
    return nrun * static + loops + nsteps * (eager_extra + reverse)


def host_gradient_baseline(scene, steps: int = 1):
    """FP64 torch reverse-mode of the same step on the host cores (the checker's restatement)."""
    import numpy as np
    import torch
    from oracle import adjoint_ref as A
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    R = A.RefScene(scene.pos4, scene.vel4, scene.bpos4, scene.material, scene.physics, True,
                   int(scene.config["fixed_iters"]))
    rng = np.random.default_rng(0)
    gx, gv = rng.normal(size=(scene.n, 3)), rng.normal(size=(scene.n, 3))
    t0 = time.perf_counter()
    A.gradient(R, steps, gx, gv)
    dt = time.perf_counter() - t0
    return {"value": scene.n * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} step(s) forward + reverse of one {scene.name} scene ({scene.n} fluid), FP64 torch "
                      f"autograd of the restated step on the host cores, {dt:.1f} s"}


def fd_check(scene, horizon: int, every: int, device: int):
    """GPU gradient of the centre-of-mass loss against FP64 central differences of the C++ oracle
    (eps = 1e-4 relative) for one scene over `horizon` steps: directional derivatives of v0 along
    the gradient and along a seeded random direction, d/dviscosity, d/dsurface_tension."""
    import numpy as np
    import torch
    from mps_cuda_gb300 import Simulation
    from mps_cuda_gb300.adjoint import AdjointRollout, com_loss
    from oracle import oracle as O
    target = np.array(scene.meta["target"], np.float64)
    m = scene.vel4[:, 3].astype(np.float64)

    def loss_np(x, v):
        com = (m[:, None] * x).sum(0) / m.sum()
        return float(((com - target) ** 2).sum() + 1e-3 * (v * v).sum(1).mean())

    sim = Simulation.from_scene(scene, device=device)
    roll = AdjointRollout(sim, horizon, every)
    pT, vT = roll.forward()
    xT = torch.tensor(pT[:, :3], dtype=torch.float64, requires_grad=True)
    vTt = torch.tensor(vT[:, :3], dtype=torch.float64, requires_grad=True)
    com_loss(xT, vTt, torch.tensor(m), [0, scene.n], torch.tensor(target[None, :])).sum().backward()
    g4x = np.zeros((scene.n, 4), np.float32)
    g4v = np.zeros((scene.n, 4), np.float32)
    g4x[:, :3] = xT.grad.numpy()
    g4v[:, :3] = vTt.grad.numpy()
    _, ov, par = roll.backward(g4x, g4v)
    sim.close()
    cfg = dict(scene.config, visc_solver=1)
    threads = os.cpu_count() or 1
    v0 = scene.vel4[:, :3].astype(np.float64)
    u = np.random.default_rng(1234).normal(size=v0.shape)

    def oracle_loss(vel=None, **mat):
        sc_mat = dict(scene.material, **mat)
        o = O.Oracle(O.params(sc_mat, scene.physics, cfg, hash_size=tuple(
            int(2 ** np.ceil(np.log2(max(4, e / sc_mat["radius"] * 2 + 4))))
            for e in np.asarray(scene.physics["max"]) - np.asarray(scene.physics["min"])), threads=threads))
        o.set_boundary(scene.bpos4[:, :3].astype(np.float64), scene.bpos4[:, 3].astype(np.float64))
        o.set_fluid(scene.pos4[:, :3].astype(np.float64), v0 if vel is None else vel, m,
                    scene.pos4[:, 3].astype(np.float64))
        o.step(horizon)
        return loss_np(o.get("pos"), o.get("vel"))

    out = {"horizon": horizon, "scene": scene.name, "eps_relative": 1e-4}
    g = ov[:, :3].astype(np.float64)
    gn = float(np.linalg.norm(g))
    eps = 1e-4 * np.abs(v0).max()
    # along the gradient itself (projection = |grad|, no cancellation) ...
    ug = g / gn
    fd = (oracle_loss(vel=v0 + eps * ug) - oracle_loss(vel=v0 - eps * ug)) / (2 * eps)
    out["v0_gradient_direction"] = {"fd": fd, "adjoint": gn, "rel_err": abs(gn - fd) / abs(fd)}
    # ... and along a seeded random unit direction (error relative to |grad|: a random projection
    # of a gradient can cancel to near zero)
    u = u / np.linalg.norm(u)
    fd = (oracle_loss(vel=v0 + eps * u) - oracle_loss(vel=v0 - eps * u)) / (2 * eps)
    ad = float((g * u).sum())
    out["v0_random_direction"] = {"fd": fd, "adjoint": ad, "err_over_grad_norm": abs(ad - fd) / gn}
    for k, name in ((0, "viscosity"), (1, "surface_tension")):
        val = float(scene.material[name])
        e = 1e-4 * val
        fd = (oracle_loss(**{name: val + e}) - oracle_loss(**{name: val - e})) / (2 * e)
        out[name] = {"fd": fd, "adjoint": float(par[0, k]), "rel_err": abs(float(par[0, k]) - fd) / abs(fd)}
    return out


def run_adjoint(args, rank, world, local_rank):
    """Forward + reverse of the 200-step rollout of 32 seeded 16k-particle scenes (one batched
    handle), gradients of the centre-of-mass loss w.r.t. v0, viscosity and surface tension."""
    import numpy as np
    import torch
    from mps_cuda_gb300 import BatchedSimulation, build, scenes
    from mps_cuda_gb300.adjoint import AdjointRollout, com_loss, rollout
    build.build()
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    scs = scenes.adjoint_scenes(32, seed=rank)   # every rank its own 32 scenes (weak scaling)
    horizon = args.steps
    every = 20
    K = int(scs[0].config["fixed_iters"])
    sim = BatchedSimulation(scs, device=local_rank)
    n = sim.n
    mass = torch.tensor(np.concatenate([s.vel4[:, 3] for s in scs]), dtype=torch.float64)
    targets = torch.tensor([s.meta["target"] for s in scs], dtype=torch.float64)
    p0, v0 = sim.get_fluid()

    def cotangents(pT, vT):
        xT = torch.tensor(pT[:, :3], dtype=torch.float64, requires_grad=True)
        vTt = torch.tensor(vT[:, :3], dtype=torch.float64, requires_grad=True)
        L = com_loss(xT, vTt, mass, sim.offsets, targets)
        L.sum().backward()
        g4x = np.zeros((n, 4), np.float32)
        g4v = np.zeros((n, 4), np.float32)
        g4x[:, :3] = xT.grad.numpy()
        g4v[:, :3] = vTt.grad.numpy()
        return L.detach().numpy(), g4x, g4v

    # warm-up: a short rollout forward + reverse (graph capture, buffers)
    warm = AdjointRollout(sim, args.warmup, min(every, args.warmup))
    pT, vT = warm.forward(p0, v0)
    warm.backward(*cotangents(pT, vT)[1:])
    roll = AdjointRollout(sim, horizon, every)
    roll.reserve()
    torch.cuda.synchronize(dev)
    if dist:
        td.barrier()
    e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    sa = sim.stats(check=False)
    with ClockSampler(local_rank) as clk:
        sim.set_fluid(p0, v0)
        e0.record(stream)
        L_check = roll.lib.mps_adjoint_forward(sim.h, horizon, every, None)
        e1.record(stream)
        e1.synchronize()
        pT, vT = sim.get_fluid()
        loss, g4x, g4v = cotangents(pT, vT)
        e2.record(stream)
        op, ov, par = roll.backward(g4x, g4v)
        e3.record(stream)
        e3.synchronize()
    assert L_check == 0
    sb = sim.stats(check=False)
    dpasses = [sb["passes_total"][k] - sa["passes_total"][k] for k in range(3)]
    fwd_ms, bwd_ms = e0.elapsed_time(e1), e2.elapsed_time(e3)
    if dist:   # the slowest rank's times; the value counts every rank's particles
        t = torch.tensor([fwd_ms, bwd_ms], dtype=torch.float64, device=dev)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        fwd_ms, bwd_ms = float(t[0]), float(t[1])
    total_ms = fwd_ms + bwd_ms
    value = n * world * horizon / (total_ms / 1e3)
    # e2e: the torch.autograd harness with host tensors (state H2D, rollout, D2H, loss, reverse)
    x0 = torch.tensor(p0[:, :3], dtype=torch.float64, requires_grad=True)
    v0t = torch.tensor(v0[:, :3], dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(scs[0].material["viscosity"], dtype=torch.float64, requires_grad=True)
    sg = torch.tensor(scs[0].material["surface_tension"], dtype=torch.float64, requires_grad=True)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    xT, vTt = rollout(roll, x0, v0t, mu, sg)
    com_loss(xT, vTt, mass, sim.offsets, targets).sum().backward()
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        e2e_s = float(t.item())
    same = bool(np.allclose(v0t.grad.numpy(), ov[:, :3], rtol=0, atol=0))
    line = {
        "metric": "particle-steps/s (DFSPH adjoint: forward + reverse, 32 x 16k scenes)", "value": value,
        "unit": UNIT, "n_gpus": world, "steps": horizon, "warmup": args.warmup,
        "ms_per_step": total_ms / horizon, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "adjoint_16k", "scenes": len(scs), "fluid_particles": n, "boundary_particles": sim.nb,
                   "fixed_iters": K, "visc_solver": "jacobi", "checkpoint_every": every, "horizon": horizon,
                   "loss": "|COM_T - target|^2 + 1e-3 mean |v_T|^2 per scene",
                   "l2": "inputs larger than L2: per-step tape ~%.0f MB > 129 MB" % (roll.memory_bytes() / 1e6)},
        "forward": {"ms": fwd_ms, "particle_steps_per_s": n * horizon / (fwd_ms / 1e3)},
        "reverse": {"ms": bwd_ms, "particle_steps_per_s": n * horizon / (bwd_ms / 1e3)},
        "adjoint_memory_bytes": roll.memory_bytes(),
        "loss_mean": float(np.mean(loss)),
        "grad": {"v0_norm": float(np.linalg.norm(ov[:, :3])), "d_viscosity_mean": float(par[:, 0].mean()),
                 "d_surface_tension_mean": float(par[:, 1].mean()), "finite": bool(np.isfinite(ov).all() and np.isfinite(par).all())},
        "roofline": None,
        "roofline_note": "per-kernel HBM roofline is reported by the plain-step line (dam_break_1m)",
        "e2e": {"value": n * world * horizon / e2e_s, "unit": UNIT, "h2d_bytes_per_step": (32 * n + 32 * n) / horizon,
                "d2h_bytes_per_step": (32 * n + 32 * n + 32 * n) / horizon,
                "note": "torch.autograd.Function over the C ABI: initial state in, final state out, cotangents in, "
                        "gradients out, host loss; bytes amortised over the horizon", "same_gradient": same},
        "gpu_launches": adjoint_launches(sim, K, horizon, every, radix_passes(sim), dpasses),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = host_gradient_baseline(scs[0], 1)
    if args.check:
        line["gradient_check"] = [fd_check(scs[k], args.check_steps, min(every, args.check_steps), local_rank)
                                  for k in range(args.check_scenes)]
    sim.close()
    if dist:
        td.destroy_process_group()
    return line


def _step_vs_oracle(sim, o, scene, mps, orc, sim1=None, o1=None):
    """One step from an identical state on both sides, phase by phase; per-quantity errors.  Each
    solver phase starts from the GPU's velocities on both sides.  With sim1 / o1 (fixed_iters = 1)
    the stiffness of each pressure solve's first iteration is compared from the same state."""
    import numpy as np
    p, v = sim.get_fluid()

    def to_oracle(oo):
        oo.set_fluid(p[:, :3].astype(np.float64), v[:, :3].astype(np.float64), v[:, 3].astype(np.float64),
                     p[:, 3].astype(np.float64))

    def rel(a, b):
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))

    out = {}
    if sim1 is not None:
        sim1.set_fluid(p, v)
        to_oracle(o1)
        for ph in (mps.PHASE_SORT, mps.PHASE_NEIGHBORS, mps.PHASE_BVOLUME, mps.PHASE_DENSITY_ALPHA):
            sim1.phase(ph)
        for ph in (orc.ZSORT, orc.NEIGHBORS, orc.BVOLUME, orc.DENSITY, orc.ALPHA, orc.GRAVITY):
            o1.phase(ph)
        for gph, oph, name in ((mps.PHASE_DF, orc.DF, "df"), (mps.PHASE_VISCST, orc.VISCST, None),
                               (mps.PHASE_CD, orc.CD, "cd")):
            o1.put("vel", sim1.get_field("vel")[:, :3].astype(np.float64))
            sim1.phase(gph)
            o1.phase(oph)
            if name:
                out[f"pressure_{name}_first_iteration_max_rel"] = rel(sim1.get_field("pressure").astype(np.float64),
                                                                      o1.get("pressure"))
        sim1.phase(mps.PHASE_ADVECT)
    to_oracle(o)
    for ph in (mps.PHASE_SORT, mps.PHASE_NEIGHBORS, mps.PHASE_BVOLUME, mps.PHASE_DENSITY_ALPHA):
        sim.phase(ph)
    for ph in (orc.ZSORT, orc.NEIGHBORS, orc.BVOLUME, orc.DENSITY, orc.ALPHA, orc.GRAVITY):
        o.phase(ph)
    rho0 = scene.material["density"]
    rg, ro = sim.get_field("density").astype(np.float64), o.get("density")
    ag, ao = sim.get_field("alpha").astype(np.float64), o.get("alpha")
    out.update({"density_max_rel": float(np.abs(rg - ro).max() / rho0),
                "density_rms_rel": float(np.sqrt(np.mean((rg - ro) ** 2)) / rho0),
                "alpha_max_rel": float(np.abs(ag - ao).max() / np.abs(ao).max())})
    for gph, oph, name in ((mps.PHASE_DF, orc.DF, "df"), (mps.PHASE_VISCST, orc.VISCST, "cg"), (mps.PHASE_CD, orc.CD, "cd")):
        v_in = sim.get_field("vel")[:, :3].astype(np.float64)
        o.put("vel", v_in)   # each solve from the same state
        sim.phase(gph)
        o.phase(oph)
        vg, vo = sim.get_field("vel")[:, :3].astype(np.float64), o.get("vel")
        out[f"velocity_after_{name}_max_rel"] = float(np.abs(vg - vo).max() / np.abs(vo).max())
        if name == "cg":
            ig, io = sim.stats()["cg_iters"], o.stats()["cg_iters"]
            cg_iters_oracle = io
            out["cg_rr_final_gpu_oracle_tol"] = [sim.stats()["cg_rr"], o.stats()["cg_rr"], float(sim.cfg.cg_tol)]
            if ig != io and ig > 1:
                # the adaptive stop (r.r < tol) fell on different iterations: the same solve on the
                # oracle with the GPU's number of updates (the loop counter minus one), from the same state
                o.put("vel", v_in)
                o.set_fixed_iters(ig - 1)
                o.phase(oph)
                o.set_fixed_iters(0)
                vo2 = o.get("vel")
                out["velocity_after_cg_same_updates_max_rel"] = float(np.abs(vg - vo2).max() / np.abs(vo2).max())
                o.put("vel", vo)
    st, so = sim.stats(), o.stats()
    out["iters_gpu"] = [st["df_iters"], st["cg_iters"], st["cd_iters"]]
    out["iters_oracle"] = [so["df_iters"], cg_iters_oracle, so["cd_iters"]]   # (the adaptive CG's count)
    kg, ko = sim.get_field("pressure").astype(np.float64), o.get("pressure")
    out["pressure_max_rel"] = float(np.abs(kg - ko).max() / max(np.abs(ko).max(), 1e-30))
    out["pressure_rms_rel"] = float(np.sqrt(np.mean((kg - ko) ** 2)) / max(np.sqrt(np.mean(ko ** 2)), 1e-30))
    vg, vo = sim.get_field("vel")[:, :3].astype(np.float64), o.get("vel")
    out["velocity_max_rel"] = float(np.abs(vg - vo).max() / np.abs(vo).max())
    out["velocity_rms_rel"] = float(np.sqrt(np.mean((vg - vo) ** 2)) / np.sqrt(np.mean(vo ** 2)))
    sim.phase(mps.PHASE_ADVECT)
    return out


def run_precision(args, rank, world, local_rank):
    """Precision study: the 4M colliding-blocks scene for `steps` steps (default 500); every
    `every` steps one step is taken phase by phase on the GPU and on the FP64 oracle from the
    same (the GPU's current) state and the per-step errors are recorded."""
    import numpy as np
    import torch
    import mps_cuda_gb300 as mps
    from mps_cuda_gb300 import Simulation, build, scenes
    from oracle import oracle as orc
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    sc = scenes.colliding_4m(seed=rank, scale=args.scale)
    sim = Simulation.from_scene(sc, device=local_rank, **overrides(args))
    sim1 = Simulation.from_scene(sc, device=local_rank, fixed_iters=1, **overrides(args))
    threads = os.cpu_count() or 1
    o = orc.from_scene(sc, threads=threads)
    o1 = orc.from_scene(sc, config=dict(fixed_iters=1), threads=threads)
    every = args.sample_every
    samples, gpu_ms, gpu_steps = [], 0.0, 0
    t_oracle = 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t = 0
    while t < args.steps:
        if t % every == 0:
            t0 = time.perf_counter()
            rec = _step_vs_oracle(sim, o, sc, mps, orc, sim1, o1)
            t_oracle += time.perf_counter() - t0
            rec["step"] = t
            samples.append(rec)
            t += 1
            continue
        k = min(every - t % every, args.steps - t)
        e0.record(stream)
        sim.step(k, stream)
        e1.record(stream)
        e1.synchronize()
        gpu_ms += e0.elapsed_time(e1)
        gpu_steps += k
        t += k
    keys = ["density_max_rel", "density_rms_rel", "alpha_max_rel", "pressure_df_first_iteration_max_rel",
            "pressure_cd_first_iteration_max_rel", "velocity_after_df_max_rel", "velocity_after_cg_max_rel",
            "velocity_after_cd_max_rel", "pressure_max_rel", "pressure_rms_rel", "velocity_max_rel", "velocity_rms_rel"]
    same = [r for r in samples if r["iters_gpu"] == r["iters_oracle"]]
    line = {
        "metric": "particle-steps/s (DFSPH, 4M colliding blocks) + per-step error vs FP64",
        "value": sc.n * gpu_steps / (gpu_ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": 0, "ms_per_step": gpu_ms / max(gpu_steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": sc.name, "fluid_particles": sc.n, "boundary_particles": sc.nb,
                   "sampled_every": every, "samples": len(samples), "oracle_threads": threads,
                   "note": "timed steps are the graph steps between samples; sampled steps run phase by phase, "
                           "each solve from the GPU's velocities on both sides; *_first_iteration: the "
                           "stiffness of a solve's first iteration from the same state (fixed_iters = 1); "
                           "pressure_max_rel: the stiffness after the last iteration of the adaptive solve"},
        "max_over_samples": {k: max(r[k] for r in samples) for k in keys},
        "max_over_samples_equal_iterations": {k: max(r[k] for r in same) for k in keys} if same else None,
        "samples_with_equal_iterations": len(same),
        "samples": samples,
        "oracle_seconds": t_oracle,
    }
    return line


def run_longrun(args, rank, world, local_rank):
    """Long-run agreement: the 32k dam break for `steps` steps (default 1000) on the GPU and on the
    FP64 oracle from the same initial state; mean density error, kinetic energy and free-surface
    height (99th percentile of y) compared every `sample_every` steps."""
    import numpy as np
    import torch
    from mps_cuda_gb300 import Simulation, build, scenes
    from oracle import oracle as orc
    build.build()
    torch.cuda.set_device(local_rank)
    sc = scenes.dam_break_32k(seed=rank)
    sim = Simulation.from_scene(sc, device=local_rank, **overrides(args))
    o = orc.from_scene(sc, threads=os.cpu_count() or 1)
    rho0 = sc.material["density"]
    m = sc.vel4[:, 3].astype(np.float64)

    def stats(x, v, rho):
        return {"mean_density_error": float(np.mean(np.maximum(rho / rho0 - 1.0, 0.0))),
                "kinetic_energy": float(0.5 * (m * (v * v).sum(1)).sum()),
                "surface_height": float(np.percentile(x[:, 1], 99))}

    rows = []
    done = 0
    t0 = time.perf_counter()
    while done < args.steps:
        k = min(args.sample_every, args.steps - done)
        sim.step(k)
        o.step(k)
        done += k
        p, v = sim.get_fluid()
        g = stats(p[:, :3].astype(np.float64), v[:, :3].astype(np.float64), sim.get_field("density").astype(np.float64))
        r = stats(o.get("pos"), o.get("vel"), o.get("density"))
        rows.append({"step": done, "gpu": g, "oracle": r,
                     "rel_diff": {k2: abs(g[k2] - r[k2]) / max(abs(r[k2]), 1e-30) for k2 in g}})
    wall = time.perf_counter() - t0
    final = rows[-1]["rel_diff"]
    return {
        "metric": "long-run agreement with FP64 (32k dam break)", "value": max(final.values()), "unit": "max relative difference at the last sample",
        "n_gpus": 1, "steps": args.steps, "warmup": 0, "ms_per_step": None, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": sc.name, "fluid_particles": sc.n, "boundary_particles": sc.nb,
                   "sample_every": args.sample_every, "surface_height": "99th percentile of fluid y",
                   "mean_density_error": "mean of max(rho/rho0 - 1, 0)"},
        "final_rel_diff": final, "max_rel_diff_over_samples": {k2: max(r["rel_diff"][k2] for r in rows) for k2 in final},
        "samples": rows, "wall_seconds": wall,
    }


def run_reference(args, scene, rank, world, local_rank):
    """The reference's own CUDA step (FP64) on rank 0."""
    if rank != 0:
        return None
    from oracle import refstep
    import ctypes
    cudart = ctypes.CDLL("libcudart.so")
    cudart.cudaSetDevice(local_rank)
    try:
        ref = refstep.RefStep(scene, variant="config")
    except Exception as e:  # noqa: BLE001
        return {"impl": "reference", "unavailable": f"reference step could not be set up: {e}"}
    ref.step(args.warmup)
    with ClockSampler(local_rank) as clk:
        t0 = time.perf_counter()
        ref.step(args.steps)
        dt = time.perf_counter() - t0
    value = scene.n * args.steps / dt
    loops = ref.loops()
    line = {
        "impl": "reference", "metric": METRIC if scene.name == "dam_break_1m" else f"particle-steps/s (DFSPH, {scene.name})", "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(scene, world),
        "implementation": "moonsh5009/MPS_CUDA step, FP64, rebuilt headless for sm_103a (USE_CUBIC_KERNEL 1, "
                          "tolerance literals set to the configuration's 1e-3 / 1e-3)",
        "last_step_loops": {"df": loops[0], "cg": loops[1], "cd": loops[2]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "reference",
                         "sample": f"{args.steps} steps of the reference's own CUDA step on the GPU, driven by one "
                                   f"host thread (the reference has no CPU implementation of the step); host wall "
                                   f"clock around its synchronous step calls"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "clocks": clk.summary(),
    }
    ref.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (adjoint_16k: the rollout horizon, 200)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="dam_break_1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--eager", action="store_true",
                    help="host-driven solver loops instead of the CUDA graph (same kernels; for ncu, which "
                         "cannot profile kernels of graphs with conditional nodes)")
    ap.add_argument("--check", action="store_true",
                    help="adjoint_16k: also check the gradient against FP64 central differences of the oracle")
    ap.add_argument("--check-steps", type=int, default=20)
    ap.add_argument("--check-scenes", type=int, default=1)
    ap.add_argument("--sample-every", type=int, default=50, help="precision_4m / longrun_32k: steps between samples")
    ap.add_argument("--scale", type=float, default=1.0, help="precision_4m: block size scale (1 = 2 x 2M)")
    ap.add_argument("--cg-form", type=int, default=None, choices=[0, 1],
                    help="CG arrangement: 0 three-pass (the reference's, library default), 1 two-pass")
    ap.add_argument("--block-size", type=int, default=None, choices=[64, 128, 256],
                    help="threads per block of the neighbour-sum kernels (library default 128)")
    ap.add_argument("--stage", type=int, default=None, choices=[0, 1],
                    help="neighbour passes: 1 = gathers from shared-memory neighbourhood tiles")
    ap.add_argument("--repeats", type=int, default=4,
                    help="further timed windows after the first (reported beside value)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.steps is None:
        args.steps = {"adjoint_16k": 200, "precision_4m": 500, "longrun_32k": 1000}.get(args.config, 10)
    rank, world, local_rank = env_rank()
    from mps_cuda_gb300 import scenes
    special = {"precision_4m": run_precision, "longrun_32k": run_longrun}
    if args.config in special and args.impl == "ours":
        line = special[args.config](args, rank, world, local_rank) if rank == 0 else None
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.config == "adjoint_16k" and args.impl == "ours":
        line = run_adjoint(args, rank, world, local_rank)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    if args.config == "batched_256":
        line = run_batched(args, scenes.batched_scenes(256, seed=0), rank, world, local_rank)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    scene = scenes.CONFIGS[args.config](seed=rank) if args.config != "reference_surface_tension" else \
        scenes.reference_surface_tension()
    if args.impl == "reference":
        line = run_reference(args, scene, rank, world, local_rank)
    else:
        line = run_ours(args, scene, rank, world, local_rank)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
