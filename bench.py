"""Benchmark of the ADER-DG element update (ADER + local + neighbour) on one GB300.

Workload (the configuration the metric is quoted on): elastic, convergence order 6
(56 basis functions x 9 quantities), 400,000 tetrahedra = 40 x 40 x 50 cubes of 5 tets,
periodic, cube edge 100 m, rho/vp/vs = 2700/6000/3464 each perturbed +-10% per cell
(seeded), DOFs seeded U[-1, 1], CFL time step (cfl 0.5).  Synthetic data throughout.

A bench "step" is one global time step of proxy kernel 'all' over all cells.
  value : cell-updates/s with DOFs resident in HBM, device time (CUDA events on the
          library's stream) over exactly K steps, max over ranks.
  e2e   : the same metric through the public C ABI with host buffers: every step is
          sei_run_host(all, 1 step) = pinned-host -> device copy of the DOFs, the step,
          device -> host copy of the result.
The DOF, time-integrated DOF and operator arrays (about 3 GB) exceed L2 (129 MB), so no
L2 flush is needed between steps.

--impl reference times the oracle port of the reference's CPU path (FP64 C, all host
threads) on a bounded sample of the same workload (a smaller periodic cube of the same
shape parameters), one time step per bench step.

Multiple GPUs (torchrun): the path does not shard; each rank runs an independent replica
and value = total cell updates of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ADER-DG cell-updates/s on 1 GB300: mixed-prec vs plain FP32 at stated L2 err"
UNIT = "cell-updates/s"
ORDER = 6
DIMS = (40, 40, 50)
PERTURB = 0.1
SEED = 2024
CPU_SAMPLE_DIMS = (8, 8, 10)
FALLBACK_HBM_GBS = 6800.0


def bytes_per_cell(order, kernel):
    """Algorithmic HBM bytes per cell and launch (float32, each array touched once)."""
    b = order * (order + 1) * (order + 2) // 6
    dof = 4 * 9 * ((b + 3) // 4 * 4)
    if kernel == "local":  # fused ADER + local: read Q, write Q, write I, star non-zeros, A+ x4, face types
        return 3 * dof + 4 * 72 + 4 * 324 + 4
    if kernel == "ader":  # read Q, write I, star non-zeros
        return 2 * dof + 4 * 72
    if kernel == "lint":  # read Q, write Q, read I, star non-zeros, A+ x4, face types
        return 3 * dof + 4 * 72 + 4 * 324 + 4
    if kernel == "neighbor":  # read Q, write Q, read neighbour I (once per cell), A- x4, relations
        return 3 * dof + 4 * 324 + 16 + 4 + 4
    f = order * (order + 1) // 2
    trace = 4 * 4 * 9 * ((f + 3) // 4 * 4)  # face traces of one cell, [4][9][FP] float32
    if kernel in ("lint_trace", "lint_tc"):  # local integral that also writes the face traces
        return 3 * dof + 4 * 72 + 4 * 324 + 4 + trace
    if kernel == "neighbor_tc":  # read Q, write Q, read the four neighbour traces, A- x4, relations
        return 2 * dof + trace + 4 * 324 + 16 + 4 + 4
    if kernel == "neighbor_fused":  # the same plus the cell's own four traces and A+ x4 (local flux)
        return 2 * dof + 2 * trace + 8 * 324 + 16 + 4 + 4
    if kernel == "lintv":  # read I, Q += volume (read and write in L2), star non-zeros, write the traces
        return 3 * dof + 4 * 72 + trace
    if kernel == "localv":  # read Q, Q += volume, star non-zeros, write the traces (I stays on chip)
        return 2 * dof + 4 * 72 + trace
    if kernel == "model":  # compulsory traffic of one fused cell update (reference data model)
        return 4 * dof + 4 * 72 + 4 * 324 + 4 * 324 + 16 + 4
    raise ValueError(kernel)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample():
    """The CPU sample of the workload, set up entirely by the oracle (no product code)."""
    import numpy as np

    from oracle import cube_mesh, dg_setup

    topo, coords = cube_mesh.periodic_cube(*CPU_SAMPLE_DIMS)
    n = topo.shape[0]
    rng = np.random.default_rng(SEED)
    f = rng.uniform(1 - PERTURB, 1 + PERTURB, (n, 3))
    rho, vp, vs = 2700.0 * f[:, 0], 6000.0 * f[:, 1], 3464.0 * f[:, 2]
    mu = rho * vs * vs
    mat = np.stack([rho, mu, rho * vp * vp - 2 * mu], axis=1)
    nb, side, orient = dg_setup.face_relations(topo)
    ops = dg_setup.cell_operators(coords, mat, nb)
    dt = dg_setup.cfl_timestep(coords, vp, ORDER, 0.5).min()
    q = rng.uniform(-1, 1, (n, 9, dg_setup.nbasis3(ORDER)))
    args = (ops["star"], ops["AplusT"], ops["AminusT"], nb, side, orient)
    return n, q, args, dt, np.zeros((n, 4), np.int8)


def cpu_baseline(k_steps=None, budget_s=12.0, sample=None):
    """Oracle port (FP64 C, OpenMP on all host threads) on a bounded sample of the workload."""
    from oracle import oracle_py

    n, q, args, dt, ft = sample or cpu_sample()
    o = oracle_py.Oracle(ORDER)
    t0 = time.perf_counter()
    q = o.steps(q, *args, dt, 1, ft)
    one = time.perf_counter() - t0
    steps = k_steps if k_steps else max(1, min(200, int(budget_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    q = o.steps(q, *args, dt, steps, ft)
    el = time.perf_counter() - t0
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": n * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"order {ORDER} elastic, {n} tets ({CPU_SAMPLE_DIMS[0]}x{CPU_SAMPLE_DIMS[1]}x{CPU_SAMPLE_DIMS[2]} "
                      f"cubes, same material/seed distribution), {steps} steps of kernel 'all', FP64",
            "seconds": el, "steps": steps, "cells": n}


ACC_STEPS = 50


def accuracy_vs_oracle(local, paths, sample):
    """Relative L2 error per quantity of each arithmetic path after ACC_STEPS steps of kernel 'all'
    against the FP64 oracle, on the CPU sample's seeded inputs (mesh, operators, DOFs, dt); part
    of the CPU leg, the oracle being the checker."""
    import numpy as np

    from oracle import oracle_py
    from seissol_gb300 import Context

    n, q, args, dt, ft = sample
    ref = oracle_py.Oracle(ORDER).steps(q, *args, dt, ACC_STEPS, ft)
    star, aplus, aminus, nb, side, orient = args
    out = {}
    for path in paths:
        prec, tc_local = PATHS[path]
        ctx = Context(ORDER, device=local, precision=prec)
        if tc_local:
            ctx.set_option(3, 1)
        ctx.set_cells(star, aplus, aminus, nb, side, orient, ft)
        ctx.set_dofs(q.astype(np.float32))
        ctx.run("all", dt, ACC_STEPS)
        ctx.sync()
        got = ctx.get_dofs().astype(np.float64)
        ctx.close()
        errs = [float(np.linalg.norm(got[:, k] - ref[:, k]) / np.linalg.norm(ref[:, k])) for k in range(9)]
        out[path] = {"rel_l2_max": max(errs), "rel_l2_per_quantity": errs}
    return {"vs": "FP64 oracle (CPU)", "steps": ACC_STEPS, "cells": n,
            "sample": f"{CPU_SAMPLE_DIMS[0]}x{CPU_SAMPLE_DIMS[1]}x{CPU_SAMPLE_DIMS[2]} cubes x 5 tets, same material "
                      "and DOF distributions as the workload", "paths": out}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier_max(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from oracle import oracle_py
    sample = cpu_sample()
    base = cpu_baseline(k_steps=1, sample=sample)
    # warm-up and K timed steps, each one time step of the sample
    n, q, a, dt, ft = sample
    o = oracle_py.Oracle(ORDER)
    for _ in range(args.warmup):
        q = o.steps(q, *a, dt, 1, ft)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        q = o.steps(q, *a, dt, 1, ft)
    el = time.perf_counter() - t0
    value = n * args.steps / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"elastic order {ORDER}, bounded sample of {n} tets of the 400,000-tet periodic cube "
                                   "(same material and DOF distributions), kernel all", "cells": n, "order": ORDER},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": base["cores"], "kind": "port",
                             "sample": base["sample"].replace("1 steps", f"{args.steps} timed steps (one per bench step)")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


DR_DIMS = (6, 100, 100)  # 60,000 cubes = 300,000 tets; fault plane x = 3 h: 100 x 100 cube faces = 20,000 faces
DR_SEED = 77


LTS_DIMS = (34, 34, 34)  # 39,304 cubes = 196,520 tets


def lts_measurement(local, cycles, visco=True):
    """Rate-2 local time stepping on a graded cube: order 5, viscoelastic with 3 mechanisms (35 x 27;
    Qp 100, Qs 50, fc 0.5 Hz, ratio 100) or elastic (35 x 9), 196,520 tets, the LTS profile of the
    mesh generator (x edges in four bands of 50 to 735 m on 60/25/10/5 % of the intervals, y and z
    edges 1,600 m), material +-10 %, CFL 0.5; at most four clusters.
    One cycle advances every cluster by the coarsest step.  Reported: cell updates per second
    (a cell update = one step of one cell in its own cluster), the simulated time per wall second
    against global time stepping at the finest step (same kernels, same simulated time), with the
    cycles launched directly and replayed from one recorded CUDA graph."""
    import numpy as np

    from seissol_gb300 import Context

    out = {}
    for mode in ("direct", "graph"):
        ctx = Context(5, device=local)
        n = ctx.build_periodic_cube(*LTS_DIMS, h=50.0, perturb=PERTURB, seed=SEED, grading=8.0, lts_profile=1)
        if visco:
            ctx.visco_setup(100.0, 50.0, 0.5, 100.0)
        ncl = ctx.lts_setup(0.5, 4)
        start, dts = ctx.lts_clusters()
        counts = np.diff(start)
        ctx.set_option(2, 1 if mode == "graph" else 0)  # SEI_OPT_LTS_GRAPH
        ctx.lts_run(2)
        ctx.sync()
        ctx.lts_run(cycles)
        ctx.sync()
        ms = ctx.last_run_ms()
        updates = float((counts * (2.0 ** (ncl - 1 - np.arange(ncl)))).sum()) * cycles
        sim = cycles * dts[-1]
        out[mode] = {"ms_per_cycle": ms / cycles, "cell_updates_per_s": updates / (ms / 1e3),
                     "simulated_s_per_wall_s": sim / (ms / 1e3)}
        if mode == "direct":
            steps = cycles << (ncl - 1)
            ctx.run("all", dts[0], 2)
            ctx.sync()
            ctx.run("all", dts[0], steps)
            ctx.sync()
            gms = ctx.last_run_ms()
            out["global_stepping"] = {"dt": dts[0], "steps": steps, "ms": gms,
                                      "cell_updates_per_s": n * steps / (gms / 1e3),
                                      "simulated_s_per_wall_s": steps * dts[0] / (gms / 1e3)}
        ctx.close()
    eq = ("viscoelastic order 5 (35x27, 3 mechanisms, Qp 100, Qs 50, fc 0.5 Hz, ratio 100)" if visco
          else "elastic order 5 (35x9)")
    return {"workload": f"{eq}, 196,520-tet graded periodic cube 34^3 cubes x 5 tets, LTS profile (x edges in four "
                        "bands 50 / 137 / 299 / 735 m on 60/25/10/5 % of the x intervals, y and z edges 1,600 m), "
                        "material +-10%, CFL 0.5, at most 4 rate-2 clusters",
            "cells": n, "clusters": int(ncl), "cells_per_cluster": [int(x) for x in counts],
            "cluster_split_percent": [round(100.0 * int(x) / n, 1) for x in counts],
            "cluster_dt": [float(x) for x in dts], "cycles": cycles, "direct": out["direct"], "graph": out["graph"],
            "global_stepping": out["global_stepping"],
            "lts_speedup_simulated_time": out["graph"]["simulated_s_per_wall_s"]
            / out["global_stepping"]["simulated_s_per_wall_s"]}


def config1_measurement(local, steps=100):
    """The plain proxy workload: elastic order 4 (20 x 9), 10,000 tets (10 x 10 x 20 cubes of
    edge 100 m), homogeneous material (rho 2700, vp 6000, vs 3464), DOFs U[-1, 1], kernel 'all',
    `steps` global steps.  Both GPU paths against the FP64 oracle on the same DOFs (relative L2
    per quantity after the run), and the oracle's own single-thread CPU throughput."""
    import numpy as np

    from oracle import oracle_py
    from seissol_gb300 import Context

    dims = (10, 10, 20)
    out, q32 = {}, None
    for path in ("fp32", "f16x3"):
        ctx = Context(4, device=local, precision=PATHS[path][0])
        n = ctx.build_periodic_cube(*dims, h=100.0, rho=2700.0, vp=6000.0, vs=3464.0, perturb=0.0, seed=SEED)
        if q32 is None:
            q32 = np.random.default_rng(SEED).uniform(-1, 1, (n, 9, 20)).astype(np.float32)
            cells, dt = ctx.get_cells(), ctx.cfl_timestep(0.5)
        ctx.set_dofs(q32)
        ctx.run("all", dt, 3)  # warm-up
        ctx.set_dofs(q32)
        ctx.run("all", dt, steps)
        ctx.sync()
        ms = ctx.last_run_ms()
        out[path] = {"ms_per_step": ms / steps, "cell_updates_per_s": n * steps / (ms / 1e3), "dofs": ctx.get_dofs()}
        ctx.close()
    t0 = time.perf_counter()
    ref = oracle_py.Oracle(4).steps(q32.astype(np.float64), cells["star"].astype(np.float64),
                                    cells["AplusT"].astype(np.float64), cells["AminusT"].astype(np.float64),
                                    cells["neighbor"], cells["side"], cells["orient"], dt, steps, cells["face_type"])
    cpu_s = time.perf_counter() - t0
    for path, r in out.items():
        got = r.pop("dofs").astype(np.float64)
        errs = [float(np.linalg.norm(got[:, k] - ref[:, k]) / np.linalg.norm(ref[:, k])) for k in range(9)]
        r["rel_l2_vs_fp64_max"] = max(errs)
        r["rel_l2_vs_fp64_per_quantity"] = errs
    return {"workload": f"elastic order 4, {n:,}-tet periodic cube 10x10x20 cubes x 5 tets (edge 100 m), homogeneous "
                        f"material, DOFs U[-1,1], kernel all, {steps} global steps, CFL 0.5",
            "paths": out, "fp64_oracle": {"seconds": cpu_s, "cell_updates_per_s": n * steps / cpu_s, "cores": 1},
            "note": "10,000 cells fill a fraction of the GPU: the GPU step time is launch-bound here"}


def output_measurement(local, steps, nrecv=1000):
    """Cost of the receiver output on the headline workload: elastic order 6, 400,000 tets, mixed
    path, kernel all.  `steps` steps are timed without receivers, then with `nrecv` receivers at
    seeded random points sampled every dt / 4 (time, nine quantities, rotation and strain: 19 columns),
    then the drain of the staged samples to host memory.  CUDA events time the GPU side, a wall
    clock the whole call."""
    import numpy as np

    from seissol_gb300 import Context

    ctx = Context(ORDER, device=local, precision=PATHS["f16x3"][0])
    n = ctx.build_periodic_cube(*DIMS, perturb=PERTURB, seed=SEED)
    dt = ctx.cfl_timestep(0.5)
    coords, _, _ = ctx.get_geometry()
    lo, hi = coords.reshape(-1, 3).min(axis=0), coords.reshape(-1, 3).max(axis=0)
    rng = np.random.default_rng(SEED + 5)
    pts = lo + (hi - lo) * rng.uniform(0.01, 0.99, (nrecv, 3))

    def timed():
        ctx.run("all", dt, 3)
        ctx.sync()
        t0 = time.perf_counter()
        ctx.run("all", dt, steps)
        ctx.sync()
        return ctx.last_run_ms() / steps, (time.perf_counter() - t0) * 1e3 / steps

    plain_ms, plain_wall = timed()
    t0 = time.perf_counter()
    ctx.receivers_setup(pts, dt / 4, rotation=True, strain=True)
    setup_ms = (time.perf_counter() - t0) * 1e3
    ctx.receivers_read()  # samples of the setup time
    recv_ms, recv_wall = timed()
    t0 = time.perf_counter()
    samples = ctx.receivers_read()
    read_ms = (time.perf_counter() - t0) * 1e3
    ctx.close()
    return {"workload": f"elastic order {ORDER}, {n:,}-tet periodic cube {DIMS[0]}x{DIMS[1]}x{DIMS[2]} cubes, mixed "
                        f"path, kernel all, {steps} steps after 3 warm-up steps; {nrecv} receivers at seeded random "
                        "points, sampled every dt/4, 9 quantities + rotation + strain",
            "receivers": nrecv, "steps": steps, "ms_per_step_without": plain_ms, "ms_per_step_with": recv_ms,
            "overhead_ms_per_step": recv_ms - plain_ms, "overhead_frac": recv_ms / plain_ms - 1.0,
            "wall_ms_per_step_without": plain_wall, "wall_ms_per_step_with": recv_wall,
            "setup_ms": setup_ms, "samples_read": int(samples.shape[0]), "columns": int(samples.shape[2]),
            "read_ms": read_ms, "read_bytes": int(samples.nbytes)}


def plasticity_measurement(local, steps):
    """Off-fault plasticity on the headline workload (elastic order 6, 400,000 tets, mixed path,
    kernel all): `steps` steps timed without and with plasticity on every cell (bulk friction
    0.6, c cos(phi) ~ U[0.7, 1.5] x 87 MPa, initial stress U[-1, 1] MPa, T_v 0.05 s, the default
    lattice nodes); the difference is the plasticity kernel's time, against its algorithmic bytes
    (stresses, initial loading, cohesion and friction at the nodes read; for yielding cells the
    stresses written and the plastic strain read and written)."""
    import numpy as np

    from seissol_gb300 import Context

    hbm, _ = peaks()
    ctx = Context(ORDER, device=local, precision=PATHS["f16x3"][0])
    n = ctx.build_periodic_cube(*DIMS, perturb=PERTURB, seed=SEED)
    dt = ctx.cfl_timestep(0.5)
    B = ctx.B
    q0 = ctx.get_dofs()

    def timed():
        ctx.set_dofs(q0)
        ctx.run("all", dt, 3)
        ctx.sync()
        ctx.run("all", dt, steps)
        ctx.sync()
        return ctx.last_run_ms() / steps

    plain = timed()
    rng = np.random.default_rng(SEED + 7)
    ctx.plasticity_setup(np.full(n, 0.6), rng.uniform(0.7, 1.5, n) * 8.7e7 / np.cos(np.arctan(0.6)),
                         rng.uniform(-1e6, 1e6, (n, 6)), tv=0.05)
    with_pl = timed()
    yields = ctx.plasticity_yield_count() / (steps + 3)
    ctx.close()
    share = yields / n
    per_cell = 4 * (6 * 56 + 6 * B + 2 * B + 1) + share * 4 * (6 * 56 + 2 * 7 * B)
    kern_ms = with_pl - plain
    return {"workload": f"elastic order {ORDER}, {n:,}-tet periodic cube {DIMS[0]}x{DIMS[1]}x{DIMS[2]} cubes, mixed "
                        f"path, kernel all, {steps} steps after 3 warm-up steps, with and without plasticity on "
                        "every cell (bulk friction 0.6, c cos(phi) ~ U[0.7, 1.5] x 87 MPa, T_v 0.05 s, default "
                        "lattice nodes)",
            "steps": steps, "ms_per_step_without": plain, "ms_per_step_with": with_pl,
            "plasticity_ms_per_step": kern_ms, "yielding_cell_share": share,
            "algorithmic_bytes_per_cell": per_cell,
            "algorithmic_gbs": per_cell * n / (kern_ms / 1e3) / 1e9 if kern_ms > 0 else None,
            "frac_of_measured_hbm": per_cell * n / (kern_ms / 1e3) / 1e9 / hbm if kern_ms > 0 else None}


def ingest_measurement(local):
    """sei_set_mesh at benchmark size: the 400,000-tet cube of the headline workload given as PUML
    arrays (1.6 M geometric vertices, connectivity, identify-vertex topology, material), ingested
    into a device context (face relations, operators, upload), beside the built-in cube generator
    on the same device; the two contexts' cell arrays must agree bit for bit."""
    import numpy as np

    from seissol_gb300 import Context

    host = Context(ORDER, device=-1)
    n = host.build_periodic_cube(*DIMS, perturb=PERTURB, seed=SEED)
    coords, material, topo = host.get_geometry()
    geo = coords.reshape(-1, 3)
    con = np.arange(4 * n, dtype=np.int64).reshape(n, 4)
    identify = np.empty(4 * n, np.int64)
    identify[con.reshape(-1)] = topo.reshape(-1)
    a = Context(ORDER, device=local)
    t0 = time.perf_counter()
    a.build_periodic_cube(*DIMS, perturb=PERTURB, seed=SEED)
    cube_s = time.perf_counter() - t0
    b = Context(ORDER, device=local)
    t0 = time.perf_counter()
    nb, nf = b.set_mesh(geo, con, material, identify=identify)
    ingest_s = time.perf_counter() - t0
    ca, cb = a.get_cells(), b.get_cells()
    same = nb == n and all(np.array_equal(ca[k], cb[k]) for k in ca)
    for c in (host, a, b):
        c.close()
    return {"workload": f"{n:,}-tet periodic cube {DIMS[0]}x{DIMS[1]}x{DIMS[2]} cubes as PUML arrays "
                        f"({len(geo):,} vertices + identify), order {ORDER}, device context",
            "cells": n, "set_mesh_s": ingest_s, "cells_per_s": n / ingest_s, "builtin_cube_s": cube_s,
            "identical_to_builtin": bool(same)}


def lts_accuracy(local, visco, cycles):
    """Accuracy of the local-time-stepping paths on a small case of the same structure: order 5
    viscoelastic (FP32 kernels) or order 6 elastic mixed precision with the fault (FVW, the fault
    configuration's distributions, float32 pre-solve on), on the LTS mesh profile (h 50 m,
    material +-10 %; 4 x 4 x 8 cubes = 640 tets viscoelastic, whose dense FP64 oracle is slow,
    8 x 8 x 8 = 2,560 tets elastic), `cycles` LTS cycles from U[-1, 1] DOFs against the FP64
    oracle: relative L2 per quantity, and for the fault the slip rate and state."""
    import numpy as np

    from oracle import dg_setup, oracle_py
    from oracle import visco as V
    from seissol_gb300 import Context, RSParams

    order = 5 if visco else 6
    ctx = Context(order, device=local, precision=0 if visco else PATHS["f16x3"][0])
    dims = (4, 4, 8) if visco else (8, 8, 8)
    n = ctx.build_periodic_cube(*dims, h=50.0, perturb=PERTURB, seed=SEED, grading=8.0, lts_profile=1,
                                fault_plane=-1 if visco else 4)
    dr = None
    if visco:
        ctx.visco_setup(100.0, 50.0, 0.5, 100.0)
    else:
        rs = RSParams.fault_config(seed=DR_SEED)
        ctx.dr_setup(rs)
        ctx.set_option(6, 1)  # SEI_OPT_DR_REFINE32
    ncl = ctx.lts_setup(0.5, 4)
    start, dts = ctx.lts_clusters()
    cl = np.repeat(np.arange(ncl), np.diff(start))
    coords, material, _ = ctx.get_geometry()
    cells = ctx.get_cells()
    nq = 27 if visco else 9
    q0 = np.random.default_rng(SEED).uniform(-1, 1, (n, nq, ctx.B)).astype(np.float32)
    ctx.set_dofs(q0)
    if visco:
        mats, thetas = [], []
        for rho, mu, lam in material:
            mu_u, lam_u, omega, theta = V.fit_attenuation(rho, mu, lam, 100.0, 50.0, 0.5, 100.0)
            mats.append([rho, mu_u, lam_u])
            thetas.append(theta)
        ops = V.cell_operators(coords, np.array(mats), omega, np.array(thetas), cells["neighbor"])
        ocells = {"star": np.concatenate([ops["star"], ops["ET"][:, None]], axis=1), "AplusT": ops["AplusT"],
                  "AminusT": ops["AminusT"], "neighbor": cells["neighbor"], "side": cells["side"],
                  "orient": cells["orient"], "face_type": cells["face_type"]}
        oracle = V.ViscoLts(order)
    else:
        ocells, oracle = cells, oracle_py.Oracle(order)
        fields = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
                      trac1="traction1", trac2="traction2")
        state = {k: ctx.dr_state(v) for k, v in fields.items()}
        params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                              "max_newton", "max_outer")}
        dr = {"faces": ctx.dr_faces(), "params": params, "state": state, "a": ctx.dr_state("a"),
              "init": np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)}
    ctx.lts_run(cycles)
    ctx.sync()
    got = ctx.get_dofs().astype(np.float64)
    t0 = time.perf_counter()
    ref = oracle_py.lts_cycles(oracle, q0.astype(np.float64), ocells, cl, dts[0], cycles, dr=dr)
    cpu_s = time.perf_counter() - t0
    errs = [float(np.linalg.norm(got[:, k] - ref[:, k]) / np.linalg.norm(ref[:, k])) for k in range(nq)]
    res = {"workload": (f"{'viscoelastic order 5 (27 quantities), FP32 kernels' if visco else 'elastic order 6, mixed precision, planar fault (FVW), float32 pre-solve'}"
                        f", {n:,} tets of the LTS mesh profile ({dims[0]}x{dims[1]}x{dims[2]} cubes), {ncl} clusters "
                        f"{[int(x) for x in np.diff(start)]}, {cycles} cycles = {cycles << (ncl - 1)} finest steps"),
           "vs": "FP64 oracle (CPU)", "rel_l2_max": max(errs), "rel_l2_per_quantity": errs, "oracle_seconds": cpu_s}
    if dr is not None:
        vg = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
        vr = np.hypot(dr["state"]["v1"], dr["state"]["v2"])
        res["slip_rate_max_rel"] = float((np.abs(vg - vr) / np.maximum(vr, 1e-30)).max())
        res["slip_rate_rel_l2"] = float(np.linalg.norm(vg - vr) / np.linalg.norm(vr))
        res["psi_max_abs"] = float(np.abs(ctx.dr_state("psi") - dr["state"]["psi"]).max())
    ctx.close()
    return res


def visco_bytes_per_cell(kind):
    """Algorithmic bytes per cell of the viscoelastic O5 launches (float32, 27 x 36 per DOF block)."""
    dof = 4 * 27 * 36
    el = 4 * 9 * 36
    small = 4 * (72 + 9 + 9)  # star non-zeros, gradients, theta
    if kind == "ader":  # read Q, write I
        return 2 * dof + small
    if kind == "lint":  # read Q, write Q, read I, A+ and W+ of 4 faces, face types
        return 3 * dof + small + 4 * 4 * (81 + 54) + 4
    if kind == "neighbor":  # read Q, write Q, elastic columns of the neighbours' I, A- and W-
        return 2 * dof + el + 4 * 4 * (81 + 54) + 16 + 4 + 4
    raise ValueError(kind)


def visco_measurement(local, steps):
    """Viscoelastic equations (3 mechanisms, 27 quantities), order 5, 196,520 tets (34^3 cubes of 5
    tets, edge 100 m, material +-10 %), Qp 100, Qs 50, central frequency 0.5 Hz, ratio 100, kernel
    all, CFL 0.5 (the equations and order of the viscoelastic configuration, on global time steps)."""
    from seissol_gb300 import Context

    hbm, _ = peaks()
    ctx = Context(5, device=local)
    n = ctx.build_periodic_cube(34, 34, 34, perturb=PERTURB, seed=SEED)
    ctx.visco_setup(100.0, 50.0, 0.5, 100.0)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 3)
    ctx.sync()
    ctx.run("all", dt, steps)
    ctx.sync()
    ms = ctx.last_run_ms()
    ctx.set_profiling(True)
    ctx.run("all", dt, steps)
    ctx.sync()
    by_kind = ctx.kernel_times_by_kind()
    ctx.set_profiling(False)
    ctx.close()
    kern = {k: v[0] / v[1] for k, v in by_kind.items() if k in ("ader", "lint", "neighbor") and v[1] > 0}
    roof = {k: {"ms": t, "algorithmic_gbs": visco_bytes_per_cell(k) * n / (t / 1e3) / 1e9,
                "frac_of_measured_hbm": visco_bytes_per_cell(k) * n / (t / 1e3) / 1e9 / hbm} for k, t in kern.items()}
    return {"workload": "viscoelastic order 5 (35x27, 3 mechanisms), 196,520-tet periodic cube 34^3 cubes x 5 tets, "
                        "material +-10%, Qp 100, Qs 50, fc 0.5 Hz, ratio 100, kernel all, GTS, CFL 0.5",
            "cells": n, "steps": steps, "ms_per_step": ms / steps, "cell_updates_per_s": n * steps / (ms / 1e3),
            "kernels": roof,
            "step_model_bytes_per_cell": 23744,
            "step_model_frac": n * steps / (ms / 1e3) * 23744 / (hbm * 1e9)}


def dr_measurement(local, steps, order=4, dims=None, plane=3, warm_precision=0, perturb=0.0):
    """Dynamic rupture on the fault workload: elastic order 4, 300,000 tets, a planar fault of
    20,000 faces (25 points each), fast-velocity-weakening friction with a ~ U[0.008, 0.02],
    sn ~ U[-120, -40] MPa, tau ~ U[20, 75] MPa, V_init = 1e-16 m/s, kernel all_dr.

    A training run (its own seed) records samples of the plain Newton solve at ten points of a
    run of the same length and trains the warm-start network on the GPU; then two contexts with the same (other) seed run
    `steps` steps from the same initial state, plain and warm-started, timed with CUDA events.
    Reported: cell- and face-updates/s of each, Newton iterations per point and step (all
    solves and the first solve of each time point), and the largest slip-rate difference."""
    import numpy as np

    from seissol_gb300 import Context, RSParams

    dims = dims or DR_DIMS
    nb3 = order * (order + 1) * (order + 2) // 6

    def make(seed, precision=0):
        ctx = Context(order, device=local, precision=precision)
        n = ctx.build_periodic_cube(*dims, perturb=perturb, seed=seed, fault_plane=plane)
        nf = ctx.dr_setup(RSParams.fault_config(seed=seed + 2))
        rng = np.random.default_rng(seed)
        ctx.set_dofs(rng.uniform(-1, 1, (n, 9, nb3)).astype(np.float32))
        return ctx, n, nf

    # training samples from the plain solve along a whole run of the training fault: 40,000
    # samples at the start of each tenth of the run
    t0 = time.perf_counter()
    tr, _, _ = make(DR_SEED)
    dt = tr.cfl_timestep(0.5)
    chunks, nchunk = [], 10
    for k in range(nchunk):
        tr.dr_record_samples(400000 // nchunk)
        tr.run("all_dr", dt, 1)
        tr.sync()
        chunks.append(tr.dr_samples())
        tr.dr_record_samples(0)
        tr.run("all_dr", dt, max(steps // nchunk - 1, 0))
    samples = np.concatenate(chunks)
    nsamp = len(samples)
    loss0, loss1 = tr.mlp_train(samples=samples, steps=1500, lr=3e-3, seed=1)
    params, norm = tr.mlp_get()
    tr.close()
    train_s = time.perf_counter() - t0
    out = {}
    states, early = {}, {}
    k_early = min(20, steps)
    # arms: the reference's float64 Newton from the previous slip rate (plain); the network's first
    # guess alone (warm); the float32 pre-solve alone (refine32); both (warm_refine32).  With a
    # mixed-precision arm, the FP32-kernel arms isolate the solver's effect from the arithmetic's.
    arms = {"plain": (False, False, 0), "warm": (True, False, 0), "refine32": (False, True, 0),
            "warm_refine32": (True, True, 0)}
    if warm_precision:
        arms["warm_refine32_mixed"] = (True, True, warm_precision)
    for mode, (net, r32, prec) in arms.items():
        ctx, n, nf = make(DR_SEED + 1, prec)
        if net:
            ctx.mlp_set(params, norm)
            ctx.dr_warm_start(True)
        ctx.set_option(6, int(r32))  # SEI_OPT_DR_REFINE32
        ctx.dr_reset_counters()
        ctx.run("all_dr", dt, k_early)
        ctx.sync()
        ms = ctx.last_run_ms()
        early[mode] = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
        if steps > k_early:
            ctx.run("all_dr", dt, steps - k_early)
            ctx.sync()
            ms += ctx.last_run_ms()
        tot, npts, first = ctx.dr_newton_iterations(first=True)
        it32 = ctx.dr_newton_iterations32()
        states[mode] = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
        ctx.set_profiling(True)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        by_kind = ctx.kernel_times_by_kind()
        fault_ms = by_kind["fault"][0]
        step_kernels = {k: v[0] for k, v in by_kind.items() if v[1] > 0}
        ctx.close()
        out[mode] = {"ms_per_step": ms / steps, "cell_updates_per_s": n * steps / (ms / 1e3),
                     "face_updates_per_s": nf * steps / (ms / 1e3), "fault_kernel_ms": fault_ms,
                     "kernel_ms_one_step": step_kernels, "network_guess": net, "float32_presolve": r32,
                     "newton_iters_per_point_step": tot / (npts * steps),
                     "first_solve_iters_per_point_step": first / (npts * steps),
                     "float32_iters_per_point_step": it32 / (npts * steps)}
    head = "warm_refine32"
    vp, vw = states["plain"], states[head]

    def ratio(a, b, key):
        return out[a][key] / max(out[b][key], 1e-30)

    res = {"workload": f"elastic order {order}, {n:,}-tet periodic cube {dims[0]}x{dims[1]}x{dims[2]} cubes "
                       f"(material +-{round(100 * perturb)}%), planar fault of {nf:,} faces x {(order + 1) ** 2} "
                       "points, FVW rate-and-state (a ~ U[0.008,0.02], sn ~ U[-120,-40] MPa, tau ~ U[20,75] MPa, "
                       f"V_init 1e-16), kernel all_dr, {steps} steps from the initial state",
           "cells": n, "faces": nf, "steps": steps, "arms": out,
           "plain": out["plain"], "warm_start": out[head],
           "warm_start_arm": "network first guess + float32 pre-solve, float64 Newton polish (FP32 kernels)",
           "newton_iters_note": "newton_iters are the float64 Newton iterations of the reference's solver "
                                "(tolerance unchanged); float32_iters are the pre-solve's iterations on ln V",
           "float64_iteration_ratio": ratio("plain", head, "newton_iters_per_point_step"),
           "first_solve_float64_iteration_ratio": ratio("plain", head, "first_solve_iters_per_point_step"),
           "network_alone_iteration_ratio": ratio("plain", "warm", "newton_iters_per_point_step"),
           "network_first_solve_iteration_ratio": ratio("plain", "warm", "first_solve_iters_per_point_step"),
           "network_float32_iteration_ratio": ratio("refine32", head, "float32_iters_per_point_step"),
           "wall_speedup_vs_plain": ratio("plain", head, "ms_per_step"),
           "wall_speedup_network_alone": ratio("plain", "warm", "ms_per_step"),
           "wall_speedup_refine32_alone": ratio("plain", "refine32", "ms_per_step"),
           "max_abs_dV": float(np.abs(vp - vw).max()),
           "max_rel_dV": float((np.abs(vp - vw) / np.maximum(vp, 1e-30)).max()),
           f"max_rel_dV_after_{k_early}_steps": float((np.abs(early["plain"] - early[head])
                                                        / np.maximum(early["plain"], 1e-30)).max()),
           "dV_between": f"plain and {head} (same arithmetic)",
           "dV_note": "plain and warm-started runs are separate trajectories: every solve converges to the "
                      "Newton tolerance, and the tolerance-level differences feed back through the wave field "
                      "over the run; tests/test_gpu_mlp.py pins the per-solve identity from one shared state",
           "training": {"samples": nsamp, "adam_steps": 1500, "loss_first": loss0, "loss_last": loss1,
                        "seconds_incl_recording": train_s}}
    if warm_precision:
        res["mixed_warm_vs_plain_speedup"] = ratio("plain", "warm_refine32_mixed", "ms_per_step")
        res["max_rel_dV_mixed_warm_vs_plain"] = float((np.abs(vp - states["warm_refine32_mixed"])
                                                       / np.maximum(vp, 1e-30)).max())
    return res


def lsw_measurement(local, steps, order=4, dims=None, plane=3):
    """The fault workload with linear slip weakening instead of rate and state: elastic order 4,
    300,000 tets, a planar fault of 20,000 faces x 25 points, mu_s 0.677, mu_d 0.525, d_c 0.01 m,
    sn0 ~ U[-125, -115] MPa, tau1_0 ~ U[62, 78] MPa, forced rupture at t = 0 on the faces of the
    first tenth of the fault (a strip), kernel all_dr, `steps` steps timed with CUDA events; one
    more profiled step gives the fault kernel's time.  Reported beside the rate-and-state numbers:
    the law's own cost, the share of points that ruptured, and the accumulated slip."""
    import numpy as np

    from seissol_gb300 import Context, LSWParams

    dims = dims or DR_DIMS
    nb3 = order * (order + 1) * (order + 2) // 6
    ctx = Context(order, device=local)
    n = ctx.build_periodic_cube(*dims, perturb=0.0, seed=DR_SEED + 1, fault_plane=plane)
    nf = ctx.dr_setup_lsw(LSWParams.fault_config(law=1, seed=DR_SEED + 3))
    npts = (order + 1) ** 2
    tf = np.full((nf, npts), 1e300)
    tf[: nf // 10] = 0.0
    ctx.dr_set_state("forced_rupture_time", tf)
    rng = np.random.default_rng(DR_SEED + 1)
    ctx.set_dofs(rng.uniform(-1, 1, (n, 9, nb3)).astype(np.float32))
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all_dr", dt, 3)  # warm-up
    ctx.sync()
    ctx.run("all_dr", dt, steps)
    ctx.sync()
    ms = ctx.last_run_ms()
    ctx.set_profiling(True)
    ctx.run("all_dr", dt, 1)
    ctx.sync()
    by_kind = ctx.kernel_times_by_kind()
    trup = ctx.dr_state("rupture_time")
    slip = ctx.dr_state("slip")
    res = {"workload": f"elastic order {order}, {n:,}-tet periodic cube {dims[0]}x{dims[1]}x{dims[2]} cubes, planar "
                       f"fault of {nf:,} faces x {npts} points, linear slip weakening (mu_s 0.677, mu_d 0.525, "
                       "d_c 0.01 m, sn0 ~ U[-125,-115] MPa, tau1_0 ~ U[62,78] MPa), forced rupture at t = 0 on "
                       f"the first tenth of the faces, kernel all_dr, {steps} steps after 3 warm-up steps",
           "cells": n, "faces": nf, "steps": steps, "ms_per_step": ms / steps,
           "cell_updates_per_s": n * steps / (ms / 1e3), "face_updates_per_s": nf * steps / (ms / 1e3),
           "fault_kernel_ms": by_kind["fault"][0],
           "kernel_ms_one_step": {k: v[0] for k, v in by_kind.items() if v[1] > 0},
           "ruptured_point_share": float((trup >= 0).mean()), "mean_slip_m": float(np.abs(slip).mean()),
           "fault_time_s": ctx.dr_time()}
    ctx.close()
    return res


def lts_fault_measurement(local, cycles):
    """The combined configuration with local time stepping: elastic order 6, 1,000,000 tets of a
    graded periodic cube (8 x 100 x 250 cubes, the LTS mesh profile along z: edges in four bands
    of 50 to 735 m on 60/25/10/5 % of the z intervals, x and y edges 1,600 m; material +-10%), a
    planar fault of 50,000 faces x 49 points (FVW, the fault configuration's distributions), at
    most 4 rate-2 clusters; both cells of a fault face share a cluster and the fault step runs in
    its cluster's correction.  Arms over `cycles` LTS cycles (graph replay): FP32 kernels with
    the plain Newton (the plain GPU path); mixed precision (tensor-core local + neighbour flux
    from the pool blocks' face traces) with the plain Newton; mixed with the learned Newton start
    (trained on samples of a plain run of another fault seed); and mixed with the learned start
    and the float32 pre-solve."""
    import numpy as np

    from seissol_gb300 import Context, RSParams

    def make(seed, precision=0):
        ctx = Context(6, device=local, precision=precision)
        n = ctx.build_periodic_cube(8, 100, 250, h=50.0, perturb=PERTURB, seed=SEED, fault_plane=4, grading=8.0,
                                    lts_profile=1)
        nf = ctx.dr_setup(RSParams.fault_config(seed=seed + 2))
        rng = np.random.default_rng(seed)
        ctx.set_dofs(rng.uniform(-1, 1, (n, 9, 56)).astype(np.float32))
        ncl = ctx.lts_setup(0.5, 4)
        ctx.set_option(2, 1)  # SEI_OPT_LTS_GRAPH
        return ctx, n, nf, ncl

    t0 = time.perf_counter()
    tr, _, _, _ = make(DR_SEED)
    chunks = []
    for _ in range(max(cycles, 1)):
        tr.dr_record_samples(400000 // max(cycles, 1))
        tr.lts_run(1)
        tr.sync()
        chunks.append(tr.dr_samples())
    tr.dr_record_samples(0)
    samples = np.concatenate(chunks)
    loss0, loss1 = tr.mlp_train(samples=samples, steps=1500, lr=3e-3, seed=1)
    params, norm = tr.mlp_get()
    tr.close()
    train_s = time.perf_counter() - t0
    out, states = {}, {}
    arms = {"plain": (0, False, False), "mixed": (1, False, False), "mixed_warm": (1, True, False),
            "mixed_warm_refine32": (1, True, True)}
    for mode, (prec, net, r32) in arms.items():
        ctx, n, nf, ncl = make(DR_SEED + 1, prec)
        if net:
            ctx.mlp_set(params, norm)
            ctx.dr_warm_start(True)
        ctx.set_option(6, int(r32))  # SEI_OPT_DR_REFINE32
        start, dts = ctx.lts_clusters()
        sizes = np.diff(start)
        faces = ctx.dr_faces()
        cl_of = np.repeat(np.arange(ncl), sizes)
        fcl = np.bincount(cl_of[faces["cells"][:, 0]], minlength=ncl)
        ctx.lts_run(1)  # records the cycle graph
        ctx.sync()
        ctx.dr_reset_counters()
        ctx.lts_run(cycles)
        ctx.sync()
        ms = ctx.last_run_ms()
        tot, npts, first = ctx.dr_newton_iterations(first=True)
        it32 = ctx.dr_newton_iterations32()
        states[mode] = (np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2")), ctx.get_dofs())
        ctx.close()
        upd = int(sum(int(sz) * (1 << (ncl - 1 - k)) for k, sz in enumerate(sizes)))  # cell updates per cycle
        dr_steps = int(sum(int(f) * (1 << (ncl - 1 - k)) for k, f in enumerate(fcl)))  # face steps per cycle
        per = max(npts / nf * dr_steps * cycles, 1)
        out[mode] = {"ms_per_cycle": ms / cycles, "cell_updates_per_s": upd * cycles / (ms / 1e3),
                     "face_updates_per_s": dr_steps * cycles / (ms / 1e3),
                     "simulated_s_per_wall_s": float(dts[-1]) * cycles / (ms / 1e3),
                     "newton_iters_per_point_face_step": tot / per, "first_solve_iters_per_point_face_step": first / per,
                     "float32_iters_per_point_face_step": it32 / per, "precision": "f16x3" if prec else "fp32",
                     "network_guess": net, "float32_presolve": r32}
    head = "mixed_warm"
    vp, qp = states["plain"]
    vm, qm = states["mixed"]
    vw, qw = states[head]

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    return {"workload": f"elastic order 6, {n:,}-tet graded periodic cube 8x100x250 cubes (LTS mesh profile along z, "
                        f"material +-10%), planar fault of {nf:,} faces x 49 points (FVW), {ncl} rate-2 clusters, "
                        f"{cycles} LTS cycles, graph replay",
            "cells": n, "faces": nf, "clusters": ncl, "cells_per_cluster": [int(v) for v in sizes],
            "cluster_split_percent": [round(100.0 * int(v) / n, 1) for v in sizes],
            "faces_per_cluster": [int(v) for v in fcl], "cluster_dt": [float(v) for v in dts], "cycles": cycles,
            "arms": out, "plain": out["plain"], "warm_start": out[head],
            "warm_start_arm": "mixed precision + network first guess",
            "speedup_vs_plain_fp32": out["plain"]["ms_per_cycle"] / out[head]["ms_per_cycle"],
            "mixed_vs_fp32_speedup_plain_newton": out["plain"]["ms_per_cycle"] / out["mixed"]["ms_per_cycle"],
            "float64_iteration_ratio": out["mixed"]["newton_iters_per_point_face_step"]
            / max(out[head]["newton_iters_per_point_face_step"], 1e-30),
            "first_solve_float64_iteration_ratio": out["mixed"]["first_solve_iters_per_point_face_step"]
            / max(out[head]["first_solve_iters_per_point_face_step"], 1e-30),
            "dofs_rel_l2_mixed_vs_fp32": rel(qm, qp), "dofs_rel_l2_mixed_warm_vs_fp32": rel(qw, qp),
            "slip_rate_rel_l2_mixed_vs_fp32": rel(vm, vp), "slip_rate_rel_l2_warm_vs_mixed": rel(vw, vm),
            "training": {"samples": int(len(samples)), "loss_first": loss0, "loss_last": loss1,
                         "seconds_incl_recording": train_s}}


PATHS = {"fp32": (0, 0), "f16x3": (1, 0), "f16x3_tc_local": (1, 1)}
PATH_DESC = {"fp32": "FP32 CUDA cores (sparse, non-zero flops)",
             "f16x3": "mixed: neighbour and local flux on tcgen05 tensor cores (split FP16 x3) from stored face "
                      "traces, ADER and volume integral FP32 CUDA cores",
             "f16x3_tc_local": "mixed: local integral and neighbour flux on tcgen05 tensor cores (split FP16 x3), "
                               "ADER FP32 CUDA cores"}


def kname(kind, path, tune=None):
    """Name of the CUDA kernel behind a launch kind of the step ('ader', 'local' for the one-launch
    cell-local kernel, 'lint', 'neighbor'; tune: the autotuner's choice, else the defaults)."""
    t = tune or {}
    tc_local = t.get("tc_local", PATHS.get(path, (0, 0))[1])
    nb_form = t.get("nb_form", 2)
    if path == "fp32":
        return f"sei_{kind}_o{ORDER}"
    if kind == "neighbor":
        return f"sei_nbt<{ORDER}>" if nb_form else f"sei_nb_tc<{ORDER}>"
    if kind == "lint" and tc_local:
        return f"sei_lintt<{ORDER}>" if tc_local == 1 else f"sei_lint_tc<{ORDER}>"
    if kind == "lint":
        return f"sei_lintv_o{ORDER}" if nb_form == 2 else f"sei_lint_trace_o{ORDER}"
    if kind == "local":
        return f"sei_localv_o{ORDER}"
    return f"sei_{kind}_o{ORDER}"


# algorithmic byte model of each kernel (bytes_per_cell kinds)
BYTES_KIND = {"sei_ader": "ader", "sei_local": "local", "sei_lint": "lint", "sei_neighbor": "neighbor",
              "sei_lint_trace": "lint_trace", "sei_lintt": "lint_tc", "sei_lint_tc": "lint_tc", "sei_nb_tc": "neighbor_tc",
              "sei_lintv": "lintv", "sei_localv": "localv"}


def bytes_kind(kind, path, tune=None):
    name = kname(kind, path, tune)
    if name.startswith("sei_nbt"):
        t = tune or {}
        fused = t.get("nb_form", 2) == 2 and not t.get("tc_local", PATHS.get(path, (0, 0))[1])
        return "neighbor_fused" if fused else "neighbor_tc"
    return BYTES_KIND[name.split("<")[0].rsplit("_o", 1)[0] if "<" not in name else name.split("<")[0]]


def measure_path(args, world, local, path, hbm, peak_kind, e2e_steps=0):
    """Kernel 'all' on the workload in one arithmetic path: throughput, per-kernel launch times,
    roofline of the dominant launch and (optionally) the end-to-end host-buffer figure."""
    import torch

    from seissol_gb300 import Context

    prec, tc_local = PATHS[path]
    rank = int(os.environ.get("RANK", "0"))
    ctx = Context(ORDER, device=local, precision=prec)
    if args.fused_local:
        ctx.set_option(1, 1)  # SEI_OPT_FUSED_LOCAL
    if tc_local:
        ctx.set_option(3, int(tc_local))  # SEI_OPT_TC_LOCAL: 1 transposed tensor-core kernel
    n = ctx.build_periodic_cube(*DIMS, perturb=PERTURB, seed=SEED + rank)
    dt = ctx.cfl_timestep(0.5)
    tune = None
    fused = bool(args.fused_local)
    if args.autotune:
        # the variants of this path timed on this mesh; the fastest stays set (DOFs unchanged)
        tune = ctx.autotune(dt, 3)
        fused = bool(tune["fused_local"])
        tc_local = int(tune["tc_local"])
        if path != "fp32":
            path = "f16x3_tc_local" if tc_local else "f16x3"
    ctx.run("all", dt, args.warmup)
    ctx.sync()
    torch.cuda.synchronize(local)
    barrier(world)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(local)
        barrier(world)
        ctx.run("all", dt, args.steps)
        ctx.sync()
        torch.cuda.synchronize(local)
        ms = ctx.last_run_ms()
        barrier(world)
    ms = barrier_max(world, ms)
    value = world * n * args.steps / (ms / 1e3)

    # per-launch durations inside a profiled run of the same workload
    ctx.set_profiling(True)
    ctx.run("all", dt, args.steps)
    ctx.sync()
    by_kind = ctx.kernel_times_by_kind()
    ctx.set_profiling(False)
    names = {"ader": "local" if fused else "ader", "lint": "lint", "neighbor": "neighbor"}
    kernels = {names[k]: v[0] / v[1] for k, v in by_kind.items() if k in names and v[1] > 0}
    launches = sum(v[1] for v in by_kind.values())
    dom = max(kernels, key=kernels.get)
    algo = bytes_per_cell(ORDER, bytes_kind(dom, path, tune)) * n
    achieved = algo / (kernels[dom] / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "dram_traffic_per_cell.txt")
    if os.path.exists(tf):
        for line in open(tf):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kname(dom, path, tune):
                traffic = float(parts[1]) * n
    roof = {"bound": "hbm", "kernel": kname(dom, path, tune), "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": f"{peak_kind} hbm_gbs", "traffic": traffic,
            "algorithmic_bytes_per_launch": algo, "launch_ms": kernels[dom],
            "step_model_frac": value / world * bytes_per_cell(ORDER, "model") / (hbm * 1e9)}
    try:
        from seissol_gb300.codegen.gen_kernels import nnz_flops
        f = nnz_flops(ORDER)
        roof["nonzero_tflops"] = value / world * (f["ader"] + f["local"] + f["neighbor"]) / 1e12
    except Exception:
        pass

    # end to end through the C ABI with pinned host buffers, one step per call
    e2e = None
    if e2e_steps > 0:
        B = 56
        hin = torch.empty((n, 9, B), dtype=torch.float32, pin_memory=True)
        hout = torch.empty((n, 9, B), dtype=torch.float32, pin_memory=True)
        hin.copy_(torch.from_numpy(ctx.get_dofs()))
        import ctypes
        pin, pout = ctypes.c_void_p(hin.data_ptr()), ctypes.c_void_p(hout.data_ptr())
        for _ in range(2):
            ctx._check(ctx.lib.sei_run_host(ctx.h, 0, dt, 1, pin, pout), "sei_run_host")
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx._check(ctx.lib.sei_run_host(ctx.h, 0, dt, 1, pin, pout), "sei_run_host")
            hin, hout = hout, hin
            pin, pout = pout, pin
        el = barrier_max(world, time.perf_counter() - t0)
        nbytes = n * 9 * B * 4
        e2e = {"value": world * n * e2e_steps / el, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": e2e_steps, "path": path,
               "call": "sei_run_host(SEI_KERNEL_ALL, dt, 1, dofs_in, dofs_out) with pinned host DOFs"}
        # the copy ceiling: one cudaMemcpyAsync of the same bytes each way, pinned, CUDA events
        dev = torch.empty((n, 9, B), dtype=torch.float32, device=f"cuda:{local}")
        s = torch.cuda.Stream(device=local)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        with torch.cuda.stream(s):
            dev.copy_(hin, non_blocking=True)  # warm-up
            hout.copy_(dev, non_blocking=True)
            ev[0].record(s)
            dev.copy_(hin, non_blocking=True)
            ev[1].record(s)
            ev[2].record(s)
            hout.copy_(dev, non_blocking=True)
            ev[3].record(s)
        s.synchronize()
        h2d_ms, d2h_ms = ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])
        e2e["copy_ceiling"] = {"h2d_gbs": nbytes / (h2d_ms / 1e3) / 1e9, "d2h_gbs": nbytes / (d2h_ms / 1e3) / 1e9,
                               "ms_both_ways": h2d_ms + d2h_ms,
                               "cell_updates_per_s_if_copies_alone": world * n / ((h2d_ms + d2h_ms) / 1e3),
                               "how": "one cudaMemcpyAsync of the step's DOFs each way, pinned host memory, "
                                      "CUDA events on a side stream"}
        del dev
    ctx.close()
    return {"value": value, "ms": ms, "n": n, "kernels": kernels, "launches": launches, "roofline": roof,
            "clocks": clk.summary(), "e2e": e2e, "description": PATH_DESC[path], "autotune": tune}


def run_ours(args, world, rank, local):
    hbm, peak_kind = peaks()
    paths = ["fp32", "f16x3"] if args.precision == "both" else [args.precision]
    if args.tc_local and "f16x3" in paths:
        paths[paths.index("f16x3")] = "f16x3_tc_local"
    res = {p: measure_path(args, world, local, p, hbm, peak_kind) for p in paths}
    best = max(res, key=lambda p: res[p]["value"])
    if args.e2e_steps > 0:
        res[best]["e2e"] = measure_path(args, world, local, best, hbm, peak_kind, args.e2e_steps)["e2e"]
    head = res[best]
    n, ms, value = head["n"], head["ms"], head["value"]
    roof, clocks, kernels, launches, e2e = head["roofline"], head["clocks"], head["kernels"], head["launches"], head["e2e"]
    paths_out = {p: {"value": r["value"], "ms_per_step": r["ms"] / args.steps, "kernel_ms_per_step": r["kernels"],
                     "roofline_kernel": r["roofline"]["kernel"], "roofline_frac": r["roofline"]["frac"],
                     "description": r["description"], "autotune": r["autotune"]} for p, r in res.items()}
    mixed = [p for p in res if p != "fp32"]
    ratio = res[mixed[0]]["value"] / res["fp32"]["value"] if mixed and "fp32" in res else None

    dr = None
    if rank == 0 and args.dr_steps > 0:
        dr = dr_measurement(local, args.dr_steps)
        dr["linear_slip_weakening"] = lsw_measurement(local, args.dr_steps)
    lts = None
    if rank == 0 and args.lts_cycles > 0:
        lts = lts_measurement(local, args.lts_cycles)
    vis = None
    if rank == 0 and args.visco_steps > 0:
        vis = visco_measurement(local, args.visco_steps)
    comb = None
    if rank == 0 and args.combined_steps > 0:
        # order 6, 1,000,000 tets, 50,000-face fault: plain = FP32 + plain Newton, warm = mixed
        # path + learned Newton start; global time stepping (the LTS form is the next measurement)
        comb = dr_measurement(local, args.combined_steps, order=6, dims=(8, 100, 250), plane=4, warm_precision=1,
                              perturb=PERTURB)
    comb_lts = None
    if rank == 0 and args.combined_lts_cycles > 0:
        comb_lts = lts_fault_measurement(local, args.combined_lts_cycles)
        comb_lts["accuracy_small_case"] = lts_accuracy(local, visco=False, cycles=13)
    if lts is not None:
        lts["accuracy_small_case"] = lts_accuracy(local, visco=True, cycles=1)
    cfg1 = None
    if rank == 0 and args.config1_steps > 0:
        cfg1 = config1_measurement(local, args.config1_steps)
    out = ing = pl = None
    if rank == 0 and args.output_steps > 0:
        out = output_measurement(local, args.output_steps)
        ing = ingest_measurement(local)
        pl = plasticity_measurement(local, args.output_steps)

    base = acc = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sample = cpu_sample()
        base = cpu_baseline(sample=sample)
        acc = accuracy_vs_oracle(local, list(res), sample)
        for p, a in acc["paths"].items():
            paths_out[p]["rel_l2_vs_fp64"] = a["rel_l2_max"]
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "elastic order 6 (56x9), 400,000-tet periodic cube 40x40x50 cubes x 5 tets, "
                                       "material +-10% per cell, kernel all (ADER+local+neighbour), GTS, CFL 0.5",
                           "cells_per_gpu": n, "order": ORDER, "path": best, "precision": PATH_DESC[best],
                           "l2": "inputs larger than L2 (~3 GB resident per GPU), no flush",
                           "parallelism": f"replicas x{world}"},
                "roofline": roof, "cpu_baseline": base, "e2e": e2e, "clocks": clocks,
                "gpu_launches": launches, "kernel_ms_per_step": kernels, "paths": paths_out,
                "mixed_vs_fp32": ratio, "accuracy": acc, "dynamic_rupture": dr, "combined_o6_fault": comb,
                "combined_o6_fault_lts": comb_lts, "proxy_o4_10k": cfg1,
                "local_time_stepping": lts, "viscoelastic": vis, "receiver_output": out, "mesh_ingestion": ing,
                "plasticity": pl}
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fused-local", action="store_true", help="ADER and local integral in one launch")
    ap.add_argument("--precision", choices=("both", "fp32", "f16x3"), default="both",
                    help="arithmetic path(s) timed; 'both' reports the faster as value and the other beside it")
    ap.add_argument("--tc-local", action="store_true", help="f16x3: local integral on the tensor cores too")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="time the default variant of each path instead of the autotuned one")
    ap.add_argument("--dr-steps", type=int, default=200,
                    help="steps of the dynamic-rupture measurement (plain and warm-started); 0 skips it")
    ap.add_argument("--config1-steps", type=int, default=100,
                    help="steps of the order-4, 10,000-tet proxy workload against the FP64 oracle; 0 skips it")
    ap.add_argument("--output-steps", type=int, default=50,
                    help="steps of the receiver-output and plasticity measurements (then the mesh-ingestion "
                         "timing); 0 skips them")
    ap.add_argument("--combined-steps", type=int, default=10,
                    help="steps of the combined order-6 measurement (1M tets, 50,000-face fault); 0 skips it")
    ap.add_argument("--combined-lts-cycles", type=int, default=3,
                    help="LTS cycles of the combined order-6 measurement with 4 clusters; 0 skips it")
    ap.add_argument("--visco-steps", type=int, default=20,
                    help="steps of the viscoelastic measurement; 0 skips it")
    ap.add_argument("--lts-cycles", type=int, default=10,
                    help="cycles of the local-time-stepping measurement; 0 skips it")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_ours(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
