"""Benchmark of the implicit corotational tet-FEM step on GB300.

Default workload (N=1): the single large cantilever beam, 64x64x257 nodes
(1,052,672 nodes, 5,080,320 tetrahedra), spacing 0.5, interior jitter
0.05*spacing, 5-tet split, E=5000, nu=0.45, method=polar, total mass 1,
gravity -9.81 y, z=0 fixed, dt=0.01, Rayleigh 0.1/0.1, CG 50 iterations,
tolerance 1e-7, threshold 1e-9 (the reference default threshold 1e-5 is
replaced by 1e-9, as the workload's CG tolerance is 1e-7). The inputs are
seeded synthetic meshes; no dataset is involved.

A "step" is one EulerImplicitSolver step of that beam. `value` is
tet-steps/s of the mixed-precision path (FP32 element math and solver
vectors, FP64 dots and state) with the mesh and state resident in HBM,
timed with CUDA events on the scene's stream. `e2e` is the same metric
through the C ABI with the state uploaded from pinned host memory and the
positions read back every step. The plain FP64 path, the position error of
mixed vs FP64 after 100 steps, the addDForce roofline and a CPU baseline
(the CPU oracle, multi-threaded, bounded sample) are reported beside it.

--impl reference times the reference's CPU algorithm (the oracle port; the
reference itself cannot be built here) on the same workload.
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

from sofa_gb300 import workloads as wl  # noqa: E402

CONFIG = wl.SINGLE_BEAM


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", default=None, help="override node grid, e.g. 32,32,129")
    ap.add_argument("--error-steps", type=int, default=100)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-single-thread", action="store_true", help="skip the single-thread CPU baseline step")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: build the mixed scene, run warm-up + steps, print a short line")
    ap.add_argument("--profile-batched", action="store_true",
                    help="profiling run of the batched workload alone: admission, warm-up + steps, a short line")
    ap.add_argument("--profile-pcg", action="store_true",
                    help="profiling run of mixed Jacobi-PCG on the stiff-inclusion block: warm-up + steps of "
                         "--pcg-iterations iterations, a short line")
    ap.add_argument("--pcg-iterations", type=int, default=100)
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-beam batched workload")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving workload")
    ap.add_argument("--no-ill-conditioned", action="store_true", help="skip the stiff-inclusion workload")
    ap.add_argument("--ill-steps", type=int, default=50)
    ap.add_argument("--beams", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=50, help="timed steps of the batched workload")
    ap.add_argument("--requests", type=int, default=1000, help="requests per arrival rate in the serving sample")
    ap.add_argument("--serve-window", type=float, default=12.0,
                    help="seconds of arrivals per rate in the serving sample (the stream stops at whichever ends "
                         "first)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # the timed region starts once sampling runs (nvidia-smi takes a
            # moment to start; at most 5 s)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_mesh(cfg):
    return wl.single_beam_mesh(cfg)


def make_scene(capi, mesh, cfg, precision, **extra):
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"], precision)
    return capi.Scene(fem, **wl.single_beam_solver(cfg, mesh), **extra)


def replica_barrier(torch, world):
    """Barrier across replicas (no-op for one process)."""
    if world > 1:
        torch.distributed.barrier()


def replica_max(torch, t_local, world, device):
    """Max over ranks of a per-rank duration: replicas exchange no data, the
    job's time is the slowest rank's."""
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, n_tets, steps, t_max):
    """Whole-job tet-steps/s: every rank advances its own copy of the workload."""
    return world * n_tets * steps / t_max


def time_steps(torch, scene, steps, warmup, world=1):
    """CUDA-event time of `steps` steps on the scene's stream after `warmup`
    untimed steps, with a barrier and a device synchronisation on both sides."""
    stream = torch.cuda.ExternalStream(scene.stream)
    scene.step(warmup)
    scene.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    replica_barrier(torch, world)
    e0.record(stream)
    scene.step(steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    replica_barrier(torch, world)
    return e0.elapsed_time(e1) / 1e3


def time_add_dforce(torch, capi, scene, mesh, reps=20):
    """Average duration of one addDForce call (element + gather kernels) on
    the scene's stream, from CUDA events."""
    fem = scene.fem
    dt = torch.float32 if fem.precision == "mixed" else torch.float64
    g = torch.Generator(device="cuda").manual_seed(0)
    dx = torch.randn((mesh.n_nodes, 3), dtype=dt, device="cuda", generator=g) * 1e-3
    df = torch.zeros((mesh.n_nodes, 3), dtype=dt, device="cuda")
    stream = torch.cuda.ExternalStream(scene.stream)
    torch.cuda.synchronize()
    for _ in range(3):
        fem.add_dforce(dx.data_ptr(), df.data_ptr(), -1e-3, stream=scene.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fem.add_dforce(dx.data_ptr(), df.data_ptr(), -1e-3, stream=scene.stream)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def adddforce_bytes(n_tets, n_nodes, p_e, p_v):
    """Algorithmic bytes of one addDForce call: per element 16 B indices,
    9 p_e rotation, 15 p_e (12 J + 3 K), 16 B of gather slots; per node
    3 p_v read (dx) and 3 p_v written (df); 4 (N+1) B row pointers."""
    return n_tets * (16 + 9 * p_e + 15 * p_e + 16) + n_nodes * (6 * p_v) + 4 * (n_nodes + 1)


def e2e_steps(torch, capi, scene, mesh, steps):
    """Through the C ABI with host buffers: each step uploads the state
    (positions and velocities) from pinned host memory, steps once and reads
    the resulting positions back into pinned host memory."""
    n3 = (mesh.n_nodes, 3)
    xh = torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy()
    vh = torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy()
    xo = torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy()
    scene.state_into(xh, vh)
    scene.set_state(xh, vh)
    scene.step(1)
    scene.state_into(xo)
    t0 = time.perf_counter()
    for _ in range(steps):
        scene.set_state(xh, vh)
        scene.step(1)
        scene.state_into(xo)
    t1 = time.perf_counter()
    return t1 - t0, xh.nbytes + vh.nbytes, xo.nbytes


def beam_population(n, seed, members=None):
    return wl.beam_population(n, seed, members)


def run_batched(torch, capi, args, plain_best):
    """The batched workload: 256 beams of the population in one batch, mixed
    precision, warm-up steps then BATCH_STEPS timed steps (CUDA events on the
    batch stream). Every beam's positions after all those steps are compared
    with the same beams batched in FP64 (FMA)."""
    beams = beam_population(args.beams, seed=3)
    tets = sum(m.n_tets for m, _ in beams)
    nodes = sum(m.n_nodes for m, _ in beams)
    threads = min(16, host_threads())
    b = capi.Batch("mixed", budget_bytes=int(60e9), max_meshes=args.beams + 8, max_cg_iterations=25)
    # elements per patch picked by timing a sample of the population (every
    # 16th beam) before admission
    t0 = time.perf_counter()
    pe, pe_ms = b.tune_patch_size([(m.positions, m.tetrahedra, kw) for m, kw in beams[::16]], steps_per_trial=2)
    pe_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    slots = b.add_meshes([(m.positions, m.tetrahedra, kw) for m, kw in beams], threads=threads)
    admit_s = time.perf_counter() - t0
    # launch tiles picked by timing this mix (state restored; results unchanged)
    t0 = time.perf_counter()
    b.tune(steps_per_trial=2, use_cache=False)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.stream)
    b.step(args.warmup)
    b.sync()
    k = args.batch_steps
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(k)
    e1.record(stream)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    info = b.info()
    tuning = b.tuning()
    xm = [b.state(s_)[0] for s_ in slots]
    its_m = [b.stats(s_)[0] for s_ in slots]
    b.close()
    value = tets * k / t
    # every beam against the FP64 (FMA) batch after the same number of steps
    bb = capi.Batch("fp64_fma", budget_bytes=int(60e9), max_meshes=args.beams + 8, max_cg_iterations=25)
    slots64 = bb.add_meshes([(m.positions, m.tetrahedra, kw) for m, kw in beams], threads=threads)
    bb.step(args.warmup + k)
    x64 = [bb.state(s_)[0] for s_ in slots64]
    its_64 = [bb.stats(s_)[0] for s_ in slots64]
    bb.close()
    errs, derrs = [], []
    for (m, _), a, r in zip(beams, xm, x64):
        errs.append(float(np.linalg.norm(a - r) / np.linalg.norm(r)))
        d = np.linalg.norm(r - m.positions)
        derrs.append(float(np.linalg.norm(a - r) / d) if d > 0 else 0.0)
    return {"workload": f"{len(beams)} beams, {nodes} nodes, {tets} tets, mixed precision, one launch per phase, "
                        "CUDA-graph steps", "tet_steps_per_s": value, "ms_per_step": t / k * 1e3, "steps": k,
            "admission_s": admit_s, "budget_used_bytes": info["budget_used"],
            "tiles": dict(tuning, tuning_s=tune_s,
                          patch_size_sample_ms_per_step={str(k): v for k, v in pe_ms.items()},
                          patch_size_tuning_s=pe_s),
            "speedup_vs_plain_fp64_single_mesh": value / plain_best,
            "position_error": {"steps": args.warmup + k, "beams_checked": len(beams),
                               "rel_l2_position_max": max(errs), "rel_l2_position_median": float(np.median(errs)),
                               "rel_l2_displacement_max": max(derrs),
                               "rel_l2_displacement_median": float(np.median(derrs)),
                               "beams_with_other_cg_iteration_count_last_step":
                                   int(sum(a != c for a, c in zip(its_m, its_64))),
                               "reference": "the same beams batched in FP64 (FMA)"}}


def run_serving(torch, capi, args, plain_best):
    """Poisson arrivals of simulate-K-steps requests (K uniform in [1, 200])
    on beams drawn from the batched workload's distribution, HBM budget
    150 GB, mixed precision. Per arrival rate the stream is args.requests
    requests or args.serve_window seconds of arrivals, whichever ends first
    (the count is reported); then it drains."""
    pool = beam_population(32, seed=5)
    rng = np.random.default_rng(11)
    results = {}
    for lam in (50, 200, 1000):
        srv = capi.Server("mixed", budget_bytes=int(150e9), max_meshes=512, max_cg_iterations=25,
                          prep_threads=min(8, host_threads()), max_steps_per_launch=8)
        picks = rng.integers(0, len(pool), args.requests)
        ks = rng.integers(1, 201, args.requests)
        gaps = rng.exponential(1.0 / lam, args.requests)
        t_start = time.perf_counter()
        t_next = t_start
        n_sub = 0
        for i in range(args.requests):
            t_next += gaps[i]
            if t_next - t_start > args.serve_window:
                break
            dt = t_next - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            mesh, kw = pool[picks[i]]
            srv.submit(mesh.positions, mesh.tetrahedra, int(ks[i]), **kw)
            n_sub += 1
        srv.wait_idle(1800)
        st = srv.stats()
        done = srv.poll(n_sub + 16)
        srv.close()
        ok = [c for c in done if c["status"] == 0]
        offered = float(np.mean([pool[p][0].n_tets * k for p, k in zip(picks[:n_sub], ks[:n_sub])])) * lam
        results[str(lam)] = {"requests": n_sub, "completed": st["completed"], "failed": st["failed"],
                             "tet_steps_per_s": st["tet_steps"] / st["wall_s"], "p50_ms": st["p50_ms"],
                             "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                             "step_p50_ms": st["step_p50_ms"], "step_p99_ms": st["step_p99_ms"],
                             "launches": st["launches"],
                             "mean_queue_ms": float(np.mean([c["queue_ms"] for c in ok])) if ok else None,
                             "offered_tet_steps_per_s": offered, "gpu_busy_fraction": st["busy_s"] / st["wall_s"],
                             "wall_s": st["wall_s"]}
    # plain path: one request at a time through the FP64 single-mesh scene;
    # scene creation (host preparation, uploads, element init) timed apart
    # from the steps and the read-back of the positions
    n_fp = 32
    t_steps = t_create = 0.0
    ts = 0
    for i in range(n_fp):
        mesh, kw = pool[int(rng.integers(0, len(pool)))]
        k = int(rng.integers(1, 201))
        t0 = time.perf_counter()
        fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, kw["young"], kw["poisson"], kw["method"],
                                  "fp64_fma")
        sc = capi.Scene(fem, dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=25,
                        cg_tolerance=1e-5, cg_threshold=1e-5, total_mass=1.0, fixed=mesh.fixed)
        sc.sync()
        t1 = time.perf_counter()
        sc.step(k)
        sc.state()
        t2 = time.perf_counter()
        sc.close()
        t_create += t1 - t0
        t_steps += t2 - t1
        ts += mesh.n_tets * k
    plain_serial = ts / t_steps
    best = max(v["tet_steps_per_s"] for v in results.values())
    return {"arrival_rates": results,
            "sample": f"up to {args.requests} requests or {args.serve_window:g} s of Poisson arrivals per rate "
                      "(a bounded sample of the 10,000-request stream), 32 distinct beams",
            "admission": "arrival order with head-of-line blocking: the oldest waiting request is admitted when a "
                         "mesh slot and a contiguous block of the HBM budget fit it; each launch advances every "
                         "admitted mesh by up to 8 steps, never past the nearest finishing request",
            "plain_fp64_one_at_a_time_tet_steps_per_s": plain_serial,
            "plain_fp64_one_at_a_time": {"requests": n_fp, "steps_s": t_steps, "creation_s": t_create,
                                         "tet_steps_per_s_with_creation": ts / (t_steps + t_create)},
            "speedup_vs_plain_fp64_one_at_a_time": best / plain_serial,
            "speedup_vs_plain_fp64_single_mesh": best / plain_best}


ILL = wl.INCLUSION


def run_ill_conditioned(torch, capi, args):
    """Stiff spherical inclusion (E 1e6 in a 1e3 beam, nu 0.49), gravity and a
    seeded tip traction, CG 200 / 1e-10: the FP32 solve with an FP64 residual
    every 20 iterations and the plain FP32 solve against a pure FP64 run."""
    from sofa_gb300 import topology as topo

    ib = topo.inclusion_beam(ILL["n"], seed=ILL["seed"], young_out=ILL["young_out"], young_in=ILL["young_in"])
    m = ib.mesh
    steps = max(1, args.ill_steps)

    def run(precision, replace):
        fem = capi.TetrahedronFEM(m.positions, m.tetrahedra, ib.young, ILL["poisson"], ILL["method"], precision)
        sc = capi.Scene(fem, dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=ILL["cg_iterations"],
                        cg_tolerance=ILL["cg_tolerance"], cg_threshold=1e-20, gravity=(0.0, -9.81, 0.0),
                        vertex_mass=1.0 / m.n_nodes, fixed=m.fixed, residual_replacement=replace)
        sc.set_external_force(ib.tip_force)
        stream = torch.cuda.ExternalStream(sc.stream)
        sc.step(1)
        sc.sync()
        sc.set_state(m.positions, np.zeros_like(m.positions))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        sc.step(steps)
        e1.record(stream)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        its, res = sc.sync()
        x, _ = sc.state()
        sc.close()
        return x, t, its, res

    x64, t64, i64, r64 = run("fp64_fma", 0)
    xr, tr, ir, rr = run("mixed", ILL["replace_every"])
    xm, tm, im, rm = run("mixed", 0)
    d = float(np.linalg.norm(x64 - m.positions))
    nx = float(np.linalg.norm(x64))

    def arm(x, t, its, res):
        return {"tet_steps_per_s": m.n_tets * steps / t, "ms_per_step": t / steps * 1e3,
                "cg_iterations_last_step": its, "cg_residual_last_step": res,
                "rel_l2_position": float(np.linalg.norm(x - x64) / nx),
                "rel_l2_displacement": float(np.linalg.norm(x - x64) / d) if d > 0 else None}

    return {"workload": f"{ILL['n'][0]}x{ILL['n'][1]}x{ILL['n'][2]} beam, {m.n_tets} tets, spherical inclusion "
                        f"radius 0.25 width, E {ILL['young_in']:g} in {ILL['young_out']:g}, nu {ILL['poisson']}, "
                        f"tip traction {ib.traction:.3f} along -y, CG {ILL['cg_iterations']}/{ILL['cg_tolerance']:g}",
            "steps": steps, "reference": "pure FP64 (FMA) run of the same scene",
            "fp64": {"tet_steps_per_s": m.n_tets * steps / t64, "ms_per_step": t64 / steps * 1e3,
                     "cg_iterations_last_step": i64, "cg_residual_last_step": r64},
            "mixed_residual_replacement": dict(arm(xr, tr, ir, rr), every=ILL["replace_every"]),
            "mixed_plain": arm(xm, tm, im, rm)}


def oracle_scene(pyoracle, fem, mesh, cfg):
    return pyoracle.OracleScene(fem, vertex_mass=cfg["total_mass"] / mesh.n_nodes, gravity=cfg["gravity"],
                                fixed=mesh.fixed, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"],
                                rayleigh_mass=cfg["rm"], cg_iterations=cfg["cg_iterations"],
                                cg_tolerance=cfg["cg_tolerance"], cg_threshold=cfg["cg_threshold"])


def cpu_baseline_leg(capi, mesh, cfg, threads, parity_steps=3, single_thread=True):
    """The CPU baseline: the oracle (an FP64 restatement of the reference's
    CPU path) timed on the host cores, one full step with `threads` threads
    (thread-local force buffers, as the MultiThreading plugin) and one with a
    single thread (the reference's serial loops). The same oracle, run
    `parity_steps` steps in its exact parallel mode (bit-identical to one
    thread), is the checker of the GPU arms on this workload: FP64 reference
    rounding with serial dots must be bit-identical; FP64-FMA and mixed are
    reported on both norms."""
    from oracle import pyoracle

    pyoracle.build()
    ofem = pyoracle.OracleFEM(mesh.positions, mesh.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"])
    pyoracle.set_threads(threads, exact=True)
    sc = oracle_scene(pyoracle, ofem, mesh, cfg)
    t0 = time.perf_counter()
    sc.step(parity_steps)
    t_exact = time.perf_counter() - t0
    xr, vr = sc.state()
    it_ref = sc.last_iterations
    del sc
    pyoracle.set_threads(threads)
    sc = oracle_scene(pyoracle, ofem, mesh, cfg)
    t0 = time.perf_counter()
    sc.step(1)
    t_mt = time.perf_counter() - t0
    del sc
    t_1 = None
    if single_thread:
        pyoracle.set_threads(1)
        sc = oracle_scene(pyoracle, ofem, mesh, cfg)
        t0 = time.perf_counter()
        sc.step(1)
        t_1 = time.perf_counter() - t0
        del sc
    pyoracle.set_threads(1)
    del ofem
    E = mesh.n_tets
    base = {"value": E / t_mt, "unit": "tet-steps/s", "cores": threads, "kind": "port",
            "sample": f"1 full step of the workload ({E} tets, CG {cfg['cg_iterations']}), FP64 CPU oracle with "
                      f"{threads} threads and thread-local force buffers, {t_mt:.1f} s"}
    if t_1 is not None:
        base["single_thread"] = {"value": E / t_1, "unit": "tet-steps/s", "cores": 1,
                                 "sample": f"1 full step, one thread (the reference's serial loops), {t_1:.1f} s"}
    # the GPU arms against the oracle's trajectory
    d = np.linalg.norm(xr - mesh.positions)
    parity = {"steps": parity_steps, "checker": f"CPU oracle, exact parallel mode on {threads} threads "
                                                f"({t_exact:.1f} s), bit-identical to one thread"}
    for prec, extra in (("fp64", dict(serial_dots=True)), ("fp64_fma", {}), ("mixed", {})):
        g = make_scene(capi, mesh, cfg, prec, **extra)
        g.step(parity_steps)
        it, _ = g.sync()
        x, v = g.state()
        g.close()
        arm = {"rel_l2_position": float(np.linalg.norm(x - xr) / np.linalg.norm(xr)),
               "rel_l2_displacement": float(np.linalg.norm(x - xr) / d) if d > 0 else None,
               "cg_iterations_equal": bool(it == it_ref)}
        if prec == "fp64":
            arm["bit_identical"] = bool(np.array_equal(x, xr) and np.array_equal(v, vr))
            parity["fp64_reference_rounding_serial_dots"] = arm
        else:
            parity[prec] = arm
    return base, parity


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_reference(args, cfg, rank):
    if rank != 0:
        return 0
    mesh = make_mesh(cfg)
    threads = host_threads()
    from oracle import pyoracle

    pyoracle.build()
    pyoracle.set_threads(threads)
    fem = pyoracle.OracleFEM(mesh.positions, mesh.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"])
    sc = pyoracle.OracleScene(fem, vertex_mass=cfg["total_mass"] / mesh.n_nodes, gravity=cfg["gravity"],
                              fixed=mesh.fixed, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"],
                              rayleigh_mass=cfg["rm"], cg_iterations=cfg["cg_iterations"],
                              cg_tolerance=cfg["cg_tolerance"], cg_threshold=cfg["cg_threshold"])
    sc.step(args.warmup)
    t0 = time.perf_counter()
    sc.step(args.steps)
    dt = time.perf_counter() - t0
    value = mesh.n_tets * args.steps / dt
    line = {
        "metric": "tet-steps/s", "value": value, "unit": "tet-steps/s", "impl": "reference", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(cfg, mesh),
        "cpu_baseline": {"value": value, "unit": "tet-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps of the workload after {args.warmup} warm-up steps, "
                                   "FP64 CPU oracle (restatement of the reference CPU path) with thread-local "
                                   "force buffers"},
        "e2e": {"value": value, "unit": "tet-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(cfg, mesh):
    return {"workload": f"single cantilever beam {cfg['n'][0]}x{cfg['n'][1]}x{cfg['n'][2]} nodes, "
                        f"{mesh.n_tets} tets, method={cfg['method']}, CG {cfg['cg_iterations']}/"
                        f"{cfg['cg_tolerance']:g}",
            "n_nodes": mesh.n_nodes, "n_tets": mesh.n_tets, "method": cfg["method"],
            "cg_iterations": cfg["cg_iterations"], "cg_tolerance": cfg["cg_tolerance"], "dt": cfg["dt"],
            "l2": "inputs larger than L2 (element data ~0.6 GB FP32, 1.2 GB FP64 vs 129 MB L2)",
            "parallelism": "replicas"}


def main():
    args = parse()
    cfg = dict(CONFIG)
    if args.n:
        cfg["n"] = tuple(int(v) for v in args.n.split(","))
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, cfg, rank)

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    if args.profile_batched:
        beams = beam_population(args.beams, seed=3)
        b = capi.Batch("mixed", budget_bytes=int(60e9), max_meshes=args.beams + 8, max_cg_iterations=25)
        b.add_meshes([(m.positions, m.tetrahedra, kw) for m, kw in beams], threads=min(16, host_threads()))
        b.step(args.warmup + args.steps)
        b.sync()
        print(json.dumps({"profile_run": True, "batched": b.info()}))
        return 0
    if args.profile_pcg:
        from sofa_gb300 import topology as topo

        ib = topo.inclusion_beam(ILL["n"], seed=ILL["seed"], young_out=ILL["young_out"], young_in=ILL["young_in"])
        m = ib.mesh
        fem = capi.TetrahedronFEM(m.positions, m.tetrahedra, ib.young, ILL["poisson"], ILL["method"], "mixed")
        sc = capi.Scene(fem, dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=args.pcg_iterations,
                        cg_tolerance=1e-20, cg_threshold=1e-20, gravity=(0.0, -9.81, 0.0),
                        vertex_mass=1.0 / m.n_nodes, fixed=m.fixed, linear_solver="pcg", preconditioner="jacobi")
        sc.set_external_force(ib.tip_force)
        sc.step(args.warmup + args.steps)
        it, res = sc.sync()
        print(json.dumps({"profile_run": True, "pcg": {"n_tets": m.n_tets, "iterations": it, "r.z/b.b": res}}))
        return 0
    mesh = make_mesh(cfg)
    E, N = mesh.n_tets, mesh.n_nodes
    hbm_peak, peak_kind = peaks()

    mixed = make_scene(capi, mesh, cfg, "mixed")
    mixed.step(1)
    mixed.sync()
    if args.profile:
        t = time_steps(torch, mixed, args.steps, args.warmup)
        # then three addDForce calls through the C ABI (the roofline unit)
        t_df = time_add_dforce(torch, capi, mixed, mesh, reps=3)
        print(json.dumps({"profile_run": True, "n_tets": E, "ms_per_step": t / max(args.steps, 1) * 1e3,
                          "adddforce_ms": t_df * 1e3}))
        return 0
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_mixed = time_steps(torch, mixed, args.steps, args.warmup, world)
    iters_mixed, res_mixed = mixed.sync()
    t_max = replica_max(torch, t_mixed, world, "cuda")
    value = replica_value(world, E, args.steps, t_max)

    # addDForce roofline on the mixed path
    t_df = time_add_dforce(torch, capi, mixed, mesh)
    alg = adddforce_bytes(E, N, 4, 4)
    achieved = alg / t_df / 1e9

    # end to end through the C ABI with host buffers
    e2e_t, h2d, d2h = e2e_steps(torch, capi, mixed, mesh, max(2, min(args.steps, 10)))
    e2e_steps_n = max(2, min(args.steps, 10))
    e2e_value = world * E * e2e_steps_n / e2e_t

    # plain FP64 path (reference rounding and FMA variants)
    plain = {}
    for prec in ("fp64_fma", "fp64"):
        sc = make_scene(capi, mesh, cfg, prec)
        sc.step(1)
        sc.sync()
        k = max(2, min(args.steps, 5))
        t = time_steps(torch, sc, k, 1)
        plain[prec] = {"tet_steps_per_s": E * k / t, "ms_per_step": t / k * 1e3}
        sc.close()

    # position error of mixed vs FP64 after error-steps steps, and along the
    # way: the GPU FP64 reference-rounding run is the reference, the FP64-FMA
    # run against it shows how far two FP64 roundings drift on this workload
    err = None
    if not args.no_error and rank == 0:
        marks = sorted({1, 20, args.error_steps})
        runs = {}
        for prec in ("fp64", "fp64_fma", "mixed"):
            sc_ = make_scene(capi, mesh, cfg, prec)
            done, xs_ = 0, {}
            for mk in marks:
                sc_.step(mk - done)
                done = mk
                xs_[mk] = sc_.state()[0]
            sc_.close()
            runs[prec] = xs_

        def norms(a, b):
            d_ = np.linalg.norm(b - mesh.positions)
            return {"rel_l2_position": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                    "rel_l2_displacement": float(np.linalg.norm(a - b) / d_) if d_ > 0 else None}

        last = args.error_steps
        err = dict(steps=last, **norms(runs["mixed"][last], runs["fp64"][last]), target_uses="rel_l2_position",
                   reference="GPU FP64 run of the same workload in the reference's rounding (no FMA)")
        err["by_step"] = {str(mk): {"mixed_vs_fp64": norms(runs["mixed"][mk], runs["fp64"][mk]),
                                    "fp64_fma_vs_fp64": norms(runs["fp64_fma"][mk], runs["fp64"][mk])}
                          for mk in marks}
        del runs

    cpu = None
    oracle_parity = None
    if not args.no_cpu_baseline and rank == 0:
        cpu, oracle_parity = cpu_baseline_leg(capi, mesh, cfg, host_threads(),
                                              single_thread=not args.no_single_thread)

    plain_best = max(p["tet_steps_per_s"] for p in plain.values())
    batched = None
    if not args.no_batched and rank == 0:
        batched = run_batched(torch, capi, args, plain_best)
    serving = None
    if not args.no_serving and rank == 0:
        serving = run_serving(torch, capi, args, plain_best)

    ill = None
    if not args.no_ill_conditioned and rank == 0:
        ill = run_ill_conditioned(torch, capi, args)

    # DRAM bytes of one addDForce launch from an ncu capture of the same
    # kernel (profiles/), scaled to this workload's element count
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            t = json.load(open(prof))
            traffic = t["dram_bytes_per_launch"] * E / t["n_tets"]
        except (OSError, ValueError, KeyError, ZeroDivisionError):
            traffic = None

    # per step: the force and right-hand side patch pass (element pass with
    # SGB_PATCH_RHS=0) and node pass (four kernels with SGB_FUSED_RHS=0), CG
    # iterations x (matvec + update), Euler update
    fused_rhs = os.environ.get("SGB_FUSED_RHS", "1") != "0"
    launches_per_step = (3 if fused_rhs else 5) + 2 * cfg["cg_iterations"]
    line = {
        "metric": "tet-steps/s", "value": value, "unit": "tet-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 dots and state)", "data": "synthetic",
        "config": workload_config(cfg, mesh),
        "cg_iterations_last_step": iters_mixed, "cg_residual_last_step": res_mixed,
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": value / plain_best,
        "batched": batched,
        "serving": serving,
        "position_error": err,
        "oracle_parity": oracle_parity,
        "ill_conditioned": ill,
        "roofline": {"kernel": "addDForce (element + gather kernels, mixed)", "bound": "hbm",
                     "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "peak_kind": peak_kind, "traffic": traffic, "algorithmic_bytes": alg,
                     "avg_launch_ms": t_df * 1e3},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "tet-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
