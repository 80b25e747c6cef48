"""Benchmark: particle-updates/s of the WCSPH time step on the 3-D dam break
(524,288 fluid + 430,572 wall particles, h = 1.3 dx, Tait, alpha = 0.01).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload dambreak3d|peristalsis|poiseuille|batched]

Own arm: the CUDA solver through its C ABI.  `value` is fluid particles x steps /
device seconds with the state resident in HBM (the step is replayed as a CUDA
graph; the working set exceeds the 126 MB L2, so no flush is needed); `e2e` is
the same metric through the public API with host buffers: every step uploads
position/velocity/leap-frog velocity from pinned host memory, runs update() and
reads the three arrays back.  The dominant kernel's roofline uses its algorithmic
bytes per launch over its CUDA-event duration inside timed steps.

Reference arm (--impl reference): the reference's CPU restatement (oracle port;
the reference itself is CUDA-only and its host code needs OpenGL) on all host
cores, same workload and metric.

N > 1 (torchrun): independent replicas, one per GPU (the step has no exchange),
barrier + max-over-ranks timing, value summed over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "particle-updates/s"

# Algorithmic bytes per particle and stage (float4 arrays read or written once,
# neighbour re-reads counted once; cell-table terms left out).  hash: position in,
# hash, rank and the cell count; sort (counting sort): hash + rank in, hash + index
# out, then hash + index in, index out, with the gather of position and leap-frog
# velocity into the sorted copies (64) in the same pass.
STAGE_BYTES = {
    "hash": 28, "sort": 92, "reorder": 0, "density": 32,
    "force": {0: 68, 1: 68, 2: 120}, "integrate": {0: 112, 1: 112, 2: 128},
}


# Algorithmic flops of the neighbour loops: 10 per candidate (distance test) and
# per interacting pair 15 (density) or 45 (force).
FLOPS_CANDIDATE, FLOPS_DENSITY_PAIR, FLOPS_FORCE_PAIR = 10, 15, 45


def pair_counts(p, pos, sample=2048, seed=0):
    """Mean candidates visited (the kernels' trimmed row walk) and mean interacting
    neighbours (|r| < 2h, other than itself) per fluid particle, from a seeded sample."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    fluid_w = 4.0 if p.system == 0 else 0.0
    xyz = pos[:, :3].astype(np.float64)
    fl = np.flatnonzero(pos[:, 3] == fluid_w)
    pick = fl[rng.choice(fl.size, min(sample, fl.size), replace=False)]
    h = float(p.smoothing_radius)
    tree = cKDTree(xyz)
    inter = np.array([len(v) - 1 for v in tree.query_ball_point(xyz[pick], 2.0 * h)], np.float64)
    g = np.array([int(v) for v in p.grid_size])
    o = np.array([float(v) for v in p.world_origin])
    if p.system == 0:
        cs = np.array([float(v) for v in p.cell_size])
        cell = np.floor((xyz - o) / cs).astype(np.int64)
    else:
        cs = np.full(3, 2.0 * float(p.particle_radius))
        cell = np.floor((xyz - o) * 0.5 / float(p.particle_radius)).astype(np.int64)
    cell %= g
    counts = np.zeros((g[2], g[1], g[0]), np.int64)
    np.add.at(counts, (cell[:, 2], cell[:, 1], cell[:, 0]), 1)
    c = int(p.cell_count)
    s2 = (2.0 * h / cs[0]) ** 2
    trim = not (p.system == 0 and not p.lj_cutoff)
    planar = int(p.dims) == 2
    cand = np.zeros(pick.size)
    for k, i in enumerate(pick):
        f = (xyz[i] - o) / cs
        gi = np.floor(f).astype(np.int64)
        tot = 0
        for dz in ([0] if planar else range(-c, c + 1)):
            for dy in range(-c, c + 1):
                xa, xb = gi[0] - c, gi[0] + c
                if trim:
                    yu, zu = gi[1] + dy, gi[2] + dz
                    dym = (yu - f[1]) if dy > 0 else ((f[1] - (yu + 1)) if dy < 0 else 0.0)
                    dzm = (zu - f[2]) if dz > 0 else ((f[2] - (zu + 1)) if dz < 0 else 0.0)
                    dym, dzm = max(dym - 1e-3, 0.0), max(dzm - 1e-3, 0.0)
                    r2 = s2 - dym * dym - dzm * dzm
                    if r2 <= 0:
                        continue
                    R = np.sqrt(r2) + 1e-3
                    xa, xb = max(xa, int(np.floor(f[0] - R))), min(xb, int(np.floor(f[0] + R)))
                    if xa > xb:
                        continue
                xs = np.arange(xa, xb + 1) % g[0]
                tot += int(counts[(gi[2] + dz) % g[2], (gi[1] + dy) % g[1], xs].sum())
        cand[k] = tot
    return float(cand.mean()), float(inter.mean())


def load_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id=None):
        self.proc = None
        self.lines = []
        cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "100"]
        if gpu_id is not None:
            cmd[1:1] = ["-i", str(gpu_id)]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def gpu_selector():
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        return vis.split(",")[int(os.environ.get("LOCAL_RANK", "0")) % len(vis.split(","))]
    try:
        import torch
        props = torch.cuda.get_device_properties(int(os.environ.get("LOCAL_RANK", "0")))
        return "GPU-" + str(props.uuid)
    except Exception:
        return None


DATA = "synthetic (seeded lattices + jitter, seed 1973)"

# C2: the 64x128x64 column in a 256x192x64-cell tank with 3 wall layers
DAMBREAK3D_TANK, DAMBREAK3D_LAYERS = (256, 192, 64), 3


def working_set_note(n, cells):
    """Working set of the step (seven float4 particle arrays, four uint32 ones,
    two uint32 cell tables): above the 126 MB L2, so no flush between steps."""
    mb = (n * (7 * 16 + 4 * 4) + 8 * cells) / 1e6
    return "inputs larger than L2 (working set %.0f MB)" % mb


def workload_config(name, p, n):
    """The `config` object of a single-scene workload, from its parameter block
    (both arms print the same one)."""
    grid = [int(v) for v in p.grid_size]
    cells = grid[0] * grid[1] * grid[2]
    if name == "dambreak3d":
        cfg = {"workload": "dambreak3d", "fluid": [int(v) for v in p.fluid_size],
               "tank_cells": list(DAMBREAK3D_TANK), "wall_layers": DAMBREAK3D_LAYERS, "particles": n,
               "h_over_dx": 1.3, "kernel": "wendland-3d", "eos": "tait gamma 7, c0 = 10 sqrt(2gH)",
               "alpha": round(float(p.av_alpha), 6), "dt": float(p.delta_time), "grid": grid}
    elif name == "peristalsis":
        cfg = {"workload": "peristalsis2d", "fluid": [int(p.fluid_size[0]), int(p.fluid_size[1])],
               "particles": n, "waves": int(p.wave_count), "amplitude_over_R": 0.3, "reynolds": 10,
               "dt": float(p.delta_time), "grid": grid}
        cells = grid[0] * grid[1]  # planar: one z layer
    else:
        cfg = {"workload": "poiseuille2d", "fluid": [64, 64], "particles": n, "wall_rows": 3,
               "physics": "cubic spline h = 1.3 dx, Tait gamma 7, c0 = 10 u_max, nu = 1e-6",
               "dt": float(p.delta_time), "grid": grid}
        cells = grid[0] * grid[1]
    cfg["parallelism"] = "replicas1"
    cfg["l2"] = working_set_note(n, cells)
    return cfg


def batched_config(P, N, F, D, scenes_total=256):
    table = sum(int(p.grid_size[0]) * int(p.grid_size[1]) for p in P)
    n = int(sum(N))
    return {"workload": "batched256", "scenes": scenes_total, "scenes_this_rank": len(P),
            "families": {"poiseuille": sum(d[0] == "poiseuille" for d in D),
                         "dambreak": sum(d[0] == "dambreak" for d in D)},
            "fluid_counts": "log-uniform [4096, 262144] (seed 1973)",
            "nu": "log-uniform [1e-6, 1e-4]; Poiseuille body force scaled with nu, dam-break "
                  "artificial viscosity 0.38 sqrt(nu / 1e-5)",
            "particles": n, "fluid": int(sum(F)), "table_cells": table, "steps_per_graph": 10,
            "kernel": "wendland-2d", "parallelism": "replicas1", "l2": working_set_note(n, table)}


def make_workload(name):
    import cmag_gb300 as cm
    from cmag_gb300 import presets
    if name == "dambreak3d":
        p, n, tank, L = presets.dambreak3d()
        s = cm.DamBreakSystem(params=p, num_particles=n)
        s.scene3d(tank, L, 0.01, 1973)
        fluid = int(np.prod(p.fluid_size))
    elif name == "peristalsis":
        p = presets.peristalsis_c3()
        s = cm.PeristalsisSystem(params=p)
        s.reset()
        n = s.getNumParticles()
        fluid = int(p.fluid_size[0]) * int(p.fluid_size[1])
    else:
        p = presets.poiseuille_c1(reference_physics=False)
        s = cm.PoiseuilleFlowSystem(params=p)
        s.reset()
        n = s.getNumParticles()
        fluid = 64 * 64
    return s, p, n, fluid, workload_config(name, p, n)


class BatchedRun:
    """The batched-scenes workload behind the calls main() makes on a solver.
    With N ranks, rank r takes the scenes k with k % N == r (no exchange)."""

    def __init__(self, rank=0, world=1):
        from cmag_gb300 import presets
        from cmag_gb300.batch import Batch
        P, N, F, D = presets.batched_scenes()
        mine = [k for k in range(len(P)) if k % world == rank]
        self.P = [P[k] for k in mine]
        self.N = [N[k] for k in mine]
        self.F = [F[k] for k in mine]
        self.D = [D[k] for k in mine]
        self.b = Batch(self.P, self.N)
        for k, p in enumerate(self.P):
            self.b.reset(k)
            if p.system == 0:  # release the dam (the reference harnesses' removeRightBoundary)
                self.b.dambreak_remove_right_boundary(k)
        self.b.set_graphs(True, 10)
        self.n = self.b.num_particles
        self.ranges = [self.b.scene_range(k) for k in range(len(self.P))]
        self.table_cells = sum(int(p.grid_size[0]) * int(p.grid_size[1]) for p in self.P)

    def update_n(self, k):
        self.b.update_n(k)

    def update(self):
        self.b.update()

    def autotune(self, reps):
        self.b.autotune(reps)
        return [[g["density_lanes"], g["force_lanes"]] for g in self.b.groups()]

    def timed_update(self, k):
        return self.b.timed_update(k)

    def synchronize(self):
        self.b.synchronize()

    def set_stage_timing(self, on):
        self.b.set_stage_timing(on)

    def stage_times(self):
        return self.b.stage_times()

    def upload(self, array, host):
        """Every scene's rows in one call (scenes one after another)."""
        self.b.set_array_all(array, host)

    def download(self, array, host):
        self.b.get_array_all(array, out=host)

    def close(self):
        self.b.close()


def make_batched(rank, world):
    run = BatchedRun(rank, world)
    groups = run.b.groups()
    cfg = batched_config(run.P, run.N, run.F, run.D)
    cfg["launch_groups"] = len(groups)
    meta = {"force_b": 68, "integrate_b": 112, "groups": groups}
    return run, run.n, int(sum(run.F)), cfg, meta


def merged_runs(groups, key):
    """Neighbour-loop launches per stage: consecutive launch groups with the same
    kernel variant (family, search shape, lists, lanes `key`) share one launch."""
    runs, prev = 0, None
    for g in groups:
        v = (g["system"], g["planar"], g["trim"], g["lists"], g[key])
        if v != prev:
            runs += 1
        prev = v
    return runs


def cpu_run(name, steps, threads):
    """Oracle port on `threads` host threads: particle-updates/s and seconds for
    `steps` full steps of the workload (derived on the oracle alone)."""
    from oracle import workloads as W
    _, n, fluid, st = W.workload(name)
    st.step(threads=threads)  # warm (page-in, allocation)
    t0 = time.perf_counter()
    for _ in range(steps):
        st.step(threads=threads)
    dt = time.perf_counter() - t0
    return fluid * steps / dt, dt


def front_of(s, column_width):
    """Surge front over the initial column width: the largest fluid x
    (XFrontTest.h:64-86, a device reduction) plus the particle radius, i.e. the
    free surface, so that runs at different spacings compare."""
    lo, hi = s.fluid_extent()
    return (float(hi[0]) + float(s.params.particle_radius)) / column_width


def run_to_t1(s, p, kept, t_end=1.0, sample_dt=0.01, column_width=0.5):
    """The 3-D dam break from its initial state to t_end: device seconds of the
    steps (CUDA events around chunks of sample_dt), steps, list rebuilds and the
    surge front at every sample (read between the timed chunks)."""
    s.scene3d(DAMBREAK3D_TANK, DAMBREAK3D_LAYERS, 0.01, 1973)
    if kept:
        s.set_verlet(kept)
    dt = float(p.delta_time)
    per = int(round(sample_dt / dt))
    total = int(round(t_end / dt))
    s.update_n(1)  # graph capture, outside the timing
    s.synchronize()
    r0 = s.verlet()[1] if kept else 0
    done, ms = 1, 0.0
    times, fronts = [dt], [front_of(s, column_width)]
    while done < total:
        k = min(per, total - done)
        ms += s.timed_update(k)
        done += k
        times.append(done * dt)
        fronts.append(front_of(s, column_width))
    s.synchronize()
    return {"device_s": ms / 1e3, "steps": total, "rebuilds": (s.verlet()[1] - r0) if kept else None,
            "ms_per_step": ms / (total - 1), "t_end": t_end, "times": times, "fronts": fronts}


def reference_gpu_bar(steps=20, warmup=5):
    """The reference's own DamBreak kernels on this GPU (DamBreak.Core/fluid_kernel.cu
    built for sm_103a into oracle/_ref, driven in the order of DamBreakSystem::update
    with thrust::sort_by_key), timed beside the library:
      * the reference's 2-D dam break at the 3-D workload's fluid count (a 512 x 1024
        column in a 2048 x 1024 x 4 grid, reference physics in both): the same
        arithmetic, so the ratio is a like-for-like speed-up;
      * the 3-D workload's 954,860 particles on a power-of-two 512 x 256 x 128 grid
        (the reference masks its hash): the reference kernels' own 3-D loops (7^3
        cells per particle, its 2-D kernel normalisation, alpha 0.38 and uncut wall
        force: the arithmetic of its 2-D physics on 3-D data), for the cost of the
        reference's search at this size.
    Device time per step from CUDA events; stage times from events around stages."""
    import cmag_gb300 as cm
    from cmag_gb300 import presets
    from oracle import ref_gpu as RG
    if not RG.available():
        return {"unavailable": "the reference's kernels were not built on this host (the cubin is compiled from "
                               "the reference sources, which only the build host has)"}
    out = {}
    names = ["hash", "sort", "reorder", "density", "force", "integrate"]
    # (a) like for like: the reference's 2-D dam break, 524,288 fluid particles;
    # its particle mass (fluidSystem.cpp:49) and dt belong to its 128-column, so
    # they scale with the particle area and the spacing (same rest density and
    # CFL number as the reference's own scene)
    kw = presets.dambreak_xfront(512)
    p = presets.dambreak_params(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    p.particle_mass = np.float32(float(p.particle_mass) * (128.0 / 512) ** 2)
    p.delta_time = np.float32(1e-4 * 128 / 512)
    s = cm.DamBreakSystem(params=p)
    s.reset()
    s.removeRightBoundary()
    ref = RG.RefGpu(s.params, s.getArray(cm.POSITION))
    ref.steps(warmup)
    ref_ms = ref.timed_steps(steps)
    ref_stage = ref.stage_ms(steps)
    ref.close()
    s.update_n(warmup)
    own_ms = s.timed_update(steps)
    s.set_stage_timing(True)
    s.update_n(steps)
    own_stage, tsteps = s.stage_times()
    s.set_stage_timing(False)
    n, fluid = s.getNumParticles(), 512 * 1024
    s.close()
    out["dambreak2d_512x1024_reference_physics"] = {
        "particles": n, "fluid": fluid, "grid": list(kw["grid_size"]), "steps": steps,
        "reference_ms_per_step": ref_ms / steps, "own_ms_per_step": own_ms / steps,
        "reference_updates_per_s": fluid * steps / (ref_ms / 1e3),
        "own_updates_per_s": fluid * steps / (own_ms / 1e3),
        "speedup": ref_ms / own_ms,
        "reference_stage_ms": {k: round(v / steps, 5) for k, v in zip(names, ref_stage)},
        "own_stage_ms": {k: round(v / max(tsteps, 1), 5) for k, v in zip(names, own_stage)}}
    # (b) the 3-D workload's particles through the reference's own loops
    p3, n3, tank, L = presets.dambreak3d()
    pr = p3.copy()
    pr.grid_size[0], pr.grid_size[1], pr.grid_size[2] = 512, 256, 128
    pos = np.zeros((n3, 4), np.float32)
    s3 = cm.DamBreakSystem(params=p3, num_particles=n3)
    s3.scene3d(tank, L, 0.01, 1973)
    pos[:] = s3.getArray(cm.POSITION)
    s3.close()
    # timed from the lattice: with its 2-D normalisation on 3-D data the
    # reference's pressures are far off, so later steps would time a scattering
    # column instead of the search
    k3 = 3
    ref = RG.RefGpu(pr, pos)
    ms3 = ref.timed_steps(k3)
    ref.close()
    ref = RG.RefGpu(pr, pos)
    st3 = ref.stage_ms(k3)
    ref.close()
    out["dambreak3d_954860_reference_loops"] = {
        "particles": n3, "fluid": 524288, "grid": [512, 256, 128], "steps": k3,
        "note": "the first steps from the initial lattice",
        "reference_ms_per_step": ms3 / k3, "reference_updates_per_s": 524288 * k3 / (ms3 / 1e3),
        "reference_stage_ms": {k: round(v / k3, 5) for k, v in zip(names, st3)}}
    return out


def front_errors(fronts, fine, tank_over_column):
    """Max and mean relative front error against the fine run while the fine front
    is short of the far wall (95 % of the tank length)."""
    fronts, fine = np.asarray(fronts), np.asarray(fine)
    m = min(len(fronts), len(fine))
    fronts, fine = fronts[:m], fine[:m]
    judged = fine < 0.95 * tank_over_column
    err = np.abs(fronts - fine) / fine
    return float(err[judged].max()), float(err[judged].mean())


def learned_to_t1(fine, t_end=1.0, seed=1973):
    """The learned coarse form (32x64x32 fluid, dt 1e-4, the closure trained by
    cmag_gb300/train_closure.py on other seeds) and the plain coarse run, from the
    block means of the fine initial state of `seed`, to t_end: device seconds and
    surge-front errors against the plain fine run (`fine`: run_to_t1's result for
    the same seed, fronts every 0.01 s)."""
    from cmag_gb300 import train_closure as TC
    from cmag_gb300.closure import Pair, rollout
    if not os.path.exists(TC.DEFAULT_OUT):
        return {"unavailable": "no trained closure (%s)" % os.path.relpath(TC.DEFAULT_OUT, HERE)}
    c, rec = TC.load()
    pair = Pair()
    tank_over_column = pair.tank_f[0] / pair.fluid_f[0]
    out = {"strength": rec["strength"], "train_seeds": len(rec["train_seeds"]),
           "validation_seed": rec["validation_seed"], "held_out_seed": seed,
           "validation_front_err": rec["validation_front_err"], "window_coarse_steps": rec["window_coarse_steps"]}
    for name in ("coarse", "coarse_closure"):
        pair.coarse.set_closure(c if name == "coarse_closure" and rec["strength"] > 0 else None)
        pair.start(seed)
        pair.coarse.update_n(1)  # graph capture, outside the timing
        pair.start(seed)
        secs, times, fronts = rollout(pair.coarse, t_end, 0.01, TC.COLUMN_WIDTH)
        emax, emean = front_errors(fronts, fine["fronts"], tank_over_column)
        m = min(len(fronts), len(fine["fronts"]))
        err = np.abs(np.asarray(fronts[:m]) - np.asarray(fine["fronts"][:m])) / np.asarray(fine["fronts"][:m])
        judged = np.asarray(fine["fronts"][:m]) < 0.95 * tank_over_column
        out[name] = {"device_s": secs, "steps": int(round(t_end / float(pair.pc.delta_time))),
                     "front_err_max": emax, "front_err_mean": emean,
                     "t_of_max_err": float(np.asarray(times[:m])[judged][np.argmax(err[judged])]),
                     "speedup_vs_fine": fine["device_s"] / secs,
                     "meets_2pct_front": emax <= 0.02,
                     "fronts_every_0.05s": [round(float(f), 4) for f in fronts[::5]]}
    pair.coarse.set_closure(None)
    pair.close()
    c.close()
    return out


def batched_to_t1(steps=10):
    """The batch's 128 dam-break scenes to t = 1 s (per-scene dt), batched against
    one scene at a time (each alone, at its autotuned best): device seconds
    extrapolated from `steps` measured steps of each configuration (the batch
    steps every scene until the last reaches t = 1 s; alone, each scene stops at
    its own).  A scene's batched trajectory is its lone trajectory bit for bit,
    so the surge-front error of batching is zero."""
    import cmag_gb300 as cm
    from cmag_gb300 import presets
    from cmag_gb300.batch import Batch
    P, N, F, D = presets.batched_scenes()
    ks = [k for k in range(len(P)) if D[k][0] == "dambreak"]
    Pd, Nd = [P[k] for k in ks], [N[k] for k in ks]
    b = Batch(Pd, Nd)
    for k in range(len(Pd)):
        b.reset(k)
        b.dambreak_remove_right_boundary(k)
    b.set_graphs(True, 10)
    b.update_n(10)
    b.autotune(2)
    b.update_n(10)
    ms_b = b.timed_update(steps) / steps
    b.close()
    t_single = []
    for k in ks:
        s = cm.DamBreakSystem(params=P[k], num_particles=N[k])
        s.reset()
        s.removeRightBoundary()
        s.update_n(3)
        s.autotune(2)
        s.update_n(3)
        t_single.append(s.timed_update(steps) / steps)
        s.close()
    to_t1 = [int(np.ceil(1.0 / float(P[k].delta_time))) for k in ks]
    plain_s = sum(n * t for n, t in zip(to_t1, t_single)) / 1e3
    batched_s = max(to_t1) * ms_b / 1e3
    return {"scenes": len(ks), "particles": int(sum(Nd)), "fluid": int(sum(F[k] for k in ks)),
            "steps_to_t1": [min(to_t1), max(to_t1)], "measured_steps": steps,
            "batch_ms_per_step": ms_b, "sum_of_single_ms_per_step": float(sum(t_single)),
            "plain_device_s_to_t1": plain_s, "batched_device_s_to_t1": batched_s,
            "speedup": plain_s / batched_s, "front_err_vs_plain": 0.0,
            "note": "device seconds extrapolated from measured per-step times; batched trajectories are "
                    "bit-identical to the lone runs (tests/test_gpu_batch.py)"}


def dist_init(n_gpus):
    if n_gpus <= 1 and "RANK" not in os.environ:
        return None
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return dist


def barrier_max(dist, value):
    from cmag_gb300.replicas import aggregate
    return aggregate(dist, value, 0.0, device="cuda")[0]


def barrier_sum(dist, value):
    from cmag_gb300.replicas import aggregate
    return aggregate(dist, 0.0, value, device="cuda")[1]


def run_reference(args):
    """The reference's CPU arm: the oracle's restatement of the reference kernels
    (the reference itself has no CPU implementation of the step) on all host
    cores, on a bounded sample of the workload.  Only the oracle is loaded: the
    workload's parameters and scene come from oracle/workloads.py."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    from oracle import workloads as W
    O.build()
    threads = os.cpu_count() or 1
    if args.workload == "batched":
        P, N, F, D = W.batched_scenes()
        value, secs, sample = cpu_run_batched(P, N, F, D, threads, budget_s=60.0)
        steps = 1
        cfg = batched_config(P, N, F, D)
    else:
        p, n, fluid, st = W.workload(args.workload)
        cfg = workload_config(args.workload, p, n)
        t0 = time.perf_counter()
        for _ in range(args.warmup):
            st.step(threads=threads)
        per_step = (time.perf_counter() - t0) / max(args.warmup, 1)
        # bounded sample: at most ~60 s of timed CPU work
        steps = max(1, min(args.steps, int(60.0 / max(per_step, 1e-6))))
        t0 = time.perf_counter()
        for _ in range(steps):
            st.step(threads=threads)
        secs = time.perf_counter() - t0
        value = fluid * steps / secs
        sample = ("%d full steps of the %d-particle scene (of %d requested), after %d warm-up steps; "
                  "oracle restatement of the reference kernels in their floating-point order"
                  % (steps, n, args.steps, args.warmup))
    line = {"metric": METRIC, "value": value, "unit": "particle-updates/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": DATA, "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "particle-updates/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "particle-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_run_batched(P, N, F, D, threads, budget_s=20.0):
    """Oracle port on a bounded sample of the batch: the smallest, median and
    largest scene of each family, one step each after a warm step, repeated
    while within the time budget.  Returns particle-updates/s, seconds and the
    sample."""
    from oracle import oracle as O
    picks = []
    for fam in ("poiseuille", "dambreak"):
        ks = sorted([k for k, d in enumerate(D) if d[0] == fam], key=lambda k: F[k])
        if ks:
            picks += sorted({ks[0], ks[len(ks) // 2], ks[-1]})
    states = []
    for k in picks:
        st = O.OracleState(P[k], N[k]).reset_reference()
        st.step(threads=threads)
        states.append((k, st))
    fluid = 0
    t0 = time.perf_counter()
    rounds = 0
    while True:
        for k, st in states:
            st.step(threads=threads)
            fluid += F[k]
        rounds += 1
        if time.perf_counter() - t0 > budget_s or rounds >= 5:
            break
    dt = time.perf_counter() - t0
    return fluid / dt, dt, "%d round(s) of one step of scenes %s (min/median/max fluid count per family)" % (
        rounds, picks)


def run_learned(args):
    """Learned closure (3-D dam break at 2x the spacing of the fine 64x128x64
    column, 65,536 fluid particles): build training data from fine runs, train on
    the GPU, choose the correction's strength on a validation seed against its
    fine run, then time fine, coarse and coarse + closure runs of a held-out seed
    to t_end and compare their surge fronts."""
    import torch
    import cmag_gb300 as cm  # noqa: F401
    from cmag_gb300.closure import (Closure, Pair, choose_strength, collect, normalization_from,
                                    output_limit_from, rollout, train)
    from oracle import closure_oracle as CO
    t_end, width = args.t_end, 0.5
    pair = Pair()
    fine_dt = float(pair.pf.delta_time)
    every = 2 * int(round(args.sample_every / (2 * fine_dt)))
    snaps = int(round(args.t_train / args.sample_every))
    seeds = list(range(2001, 2001 + args.train_seeds))
    t0 = time.perf_counter()
    feat, tgt = collect(pair, seeds, snaps, every)
    t_data = time.perf_counter() - t0
    c = Closure(CO.init_params(0))
    mean, inv, scale = normalization_from(feat, tgt)
    c.set_normalization(mean, inv, scale)
    c.set_output_limit(output_limit_from(tgt, scale))
    train_rows = int(feat.shape[0])
    t0 = time.perf_counter()
    losses = train(c, feat, tgt, steps=args.train_steps, batch=65536, lr=2e-3, lr_final=1e-4,
                   log_every=max(1, args.train_steps // 5))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del feat, tgt
    # each solver at its best for the timed runs: lanes per particle and interaction
    # lists chosen on a developed flow (t = 0.1 s of the held-out seed)
    lanes = {}
    for name, sysm, steps in (("fine", pair.fine, 2000), ("coarse", pair.coarse, 1000)):
        pair.start(999)
        sysm.update_n(steps)
        lanes[name] = list(sysm.autotune(3))
    # the fine run judges the closure on a validation seed: strength of the
    # correction (0 = plain coarse) with the smallest front error there
    valid = 998
    t0 = time.perf_counter()
    strength, verr = choose_strength(pair, c, valid, t_end, width)
    t_valid = time.perf_counter() - t0

    held = 999
    runs = {}
    for name in ("fine", "coarse", "coarse_closure"):
        sysm = pair.fine if name == "fine" else pair.coarse
        pair.coarse.set_closure(c if name == "coarse_closure" and strength > 0.0 else None)
        pair.start(held)
        sysm.update_n(3)  # warm-up and graph capture (restarted below)
        pair.start(held)
        secs, times, fronts = rollout(sysm, t_end, 0.01, width)
        runs[name] = {"device_s_to_t_end": secs, "steps": int(round(t_end / float(sysm.params.delta_time))),
                      "fronts": fronts, "times": times}
    pair.coarse.set_closure(None)
    ff = runs["fine"]["fronts"]
    tank_len = pair.tank_f[0] / pair.fluid_f[0]  # tank length over column width
    judged = ff < 0.95 * tank_len   # before the surge meets the far wall
    out = {}
    for name in ("coarse", "coarse_closure"):
        err = np.abs(runs[name]["fronts"] - ff) / ff
        out[name] = {"front_err_max": float(err[judged].max()), "front_err_mean": float(err[judged].mean()),
                     "device_s_to_t_end": runs[name]["device_s_to_t_end"],
                     "speedup_vs_fine": runs["fine"]["device_s_to_t_end"] / runs[name]["device_s_to_t_end"]}
    nfc = pair.nfluid_c
    cl = runs["coarse_closure"]
    value = nfc * cl["steps"] / cl["device_s_to_t_end"]
    line = {"metric": METRIC, "value": value, "unit": "particle-updates/s", "n_gpus": 1,
            "steps": cl["steps"], "warmup": 3, "ms_per_step": 1e3 * cl["device_s_to_t_end"] / cl["steps"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16",
            "data": "synthetic (seeded lattices + jitter)",
            "config": {"workload": "learned_closure", "fine_fluid": list(pair.fluid_f),
                       "coarse_fluid": list(pair.fluid_c), "t_end": t_end,
                       "train_seeds": len(seeds), "snapshots_per_seed": snaps,
                       "train_rows": train_rows, "train_steps": args.train_steps,
                       "validation_seed": valid, "held_out_seed": held,
                       "network": "16-64-64-64-3 SiLU, bf16 params/activations"},
            "learned": {"fine_device_s_to_t_end": runs["fine"]["device_s_to_t_end"],
                        "coarse": out["coarse"], "coarse_closure": out["coarse_closure"],
                        "meets_2pct_front": out["coarse_closure"]["front_err_max"] <= 0.02,
                        "strength": strength, "lanes_density_force_lists": lanes,
                        "validation_front_err": {str(f): [round(a, 4), round(b, 4)] for f, (a, b) in verr.items()},
                        "data_s": t_data, "train_s": t_train, "validation_s": t_valid, "losses": losses,
                        "fronts": {k: [round(float(v), 4) for v in r["fronts"][::10]] for k, r in runs.items()}}}
    pair.close()
    c.close()
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--workload", default="dambreak3d",
                    choices=["dambreak3d", "peristalsis", "poiseuille", "batched", "learned"])
    ap.add_argument("--t-end", type=float, default=1.0, help="learned: simulated time of the timed runs")
    ap.add_argument("--t-train", type=float, default=1.0, help="learned: time span of the training runs")
    ap.add_argument("--sample-every", type=float, default=0.025, help="learned: seconds between samples")
    ap.add_argument("--train-seeds", type=int, default=3)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--neighbor-lists", choices=["auto", "on", "off"], default="auto",
                    help="single-scene workloads: the autotuner's choice, or force interaction lists on/off")
    ap.add_argument("--cpu-steps", type=int, default=20,
                    help="full steps of the CPU baseline sample (about 10 s on 16 cores for the dam break)")
    ap.add_argument("--verlet", type=float, default=0.0,
                    help="single scenes: neighbour lists kept over steps with this skin (particle spacings); "
                         "0: the reference's per-step sort and cell walk")
    ap.add_argument("--t-start", type=float, default=0.125,
                    help="dam break: simulated seconds run (untimed, part of the setup) before warm-up; "
                         "0.125 s is the middle of the configured 5000-step run")
    ap.add_argument("--no-t1", action="store_true", help="skip the plain run to t = 1 s")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip timing the reference's kernels on the GPU")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned coarse run to t = 1 s")
    ap.add_argument("--no-batched-t1", action="store_true", help="skip the batched dam breaks to t = 1 s")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args)
        return

    from cmag_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    if args.workload == "learned":
        run_learned(args)
        return
    dist = dist_init(args.gpus)
    rank = int(os.environ.get("RANK", "0"))
    world = dist.get_world_size() if dist else 1
    import torch
    torch.cuda.init()
    import cmag_gb300 as cm

    batched = args.workload == "batched"
    if batched:
        s, n, fluid, cfg, meta = make_batched(rank, world)
        p = None
        cfg["parallelism"] = "scenes sharded over %d rank(s)" % world
    else:
        s, p, n, fluid, cfg = make_workload(args.workload)
        cfg["parallelism"] = "replicas%d" % world
        meta = {"force_b": STAGE_BYTES["force"][p.system],
                "integrate_b": STAGE_BYTES["integrate"][p.system],
                # hash, 3 scan, 2 sort (with the sorted gather), density, force,
                # integrate (+ the phase block for Peristalsis, whose wall
                # configuration runs in the hash pass)
                "launches": {0: 9, 1: 9, 2: 10}[p.system]}

    kept = (not batched) and args.verlet > 0 and args.neighbor_lists == "auto"
    if not batched and args.workload == "dambreak3d" and args.t_start > 0:
        # the timed steps start from a developed flow (the surge under way), not
        # from the column at rest
        s.update_n(int(round(args.t_start / float(p.delta_time))))
        cfg["t_start"] = args.t_start
    if kept:
        s.set_verlet(args.verlet)
    # warm-up (graph capture happens on the first step), then pick the lanes per
    # particle of the neighbour loops on this workload
    s.update_n(args.warmup)
    # the autotuner's choice, unless the neighbour loops are pinned (profiles: ncu
    # serialises launches and would skew its timings)
    tuning = {"lanes_density_force_lists": list(s.autotune(3)) if args.neighbor_lists == "auto" else []}
    if batched:
        groups = s.b.groups()
        meta["launches"] = 1 + 3 + 2 + merged_runs(groups, "density_lanes") + merged_runs(groups, "force_lanes") + 1
        tuning["launch_groups"] = len(groups)
        tuning["neighbour_launches_per_step"] = meta["launches"] - 7
    if kept:
        tuning = {"kept_lists_skin": args.verlet}
    if args.neighbor_lists != "auto" and not batched:
        # a fixed choice (e.g. for profiles, where ncu's serialised launches skew
        # the autotuner's timings): one lane per particle with or without lists
        s.set_groups(1, 1)
        s.set_neighbor_lists(args.neighbor_lists == "on")
        tuning["lanes_density_force_lists"] = [1, 1, args.neighbor_lists == "on"]
    s.update_n(2)
    s.synchronize()
    rebuilds0 = s.verlet()[1] if kept else 0

    # ---- device-resident timed region ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu_selector())
    time.sleep(0.3)
    ms = s.timed_update(args.steps)
    time.sleep(0.3)
    clocks = sampler.stop()
    torch.cuda.synchronize()
    ms = barrier_max(dist, ms)
    secs = ms / 1e3
    total_fluid = fluid if not dist else int(barrier_sum(dist, fluid))
    value = total_fluid * args.steps / secs if batched else fluid * args.steps * world / secs
    s.synchronize()
    if kept:
        tuning["rebuilds_in_timed_steps"] = s.verlet()[1] - rebuilds0

    # ---- per-stage times (plain launches, events around each stage) ----
    s.set_stage_timing(True)
    s.update_n(args.steps)
    stage_ms, tsteps = s.stage_times()
    s.set_stage_timing(False)
    names = ["hash", "sort", "reorder", "density", "force", "integrate"]
    per_stage = {nm: stage_ms[k] / max(tsteps, 1) for k, nm in enumerate(names)}
    dom = max(per_stage, key=per_stage.get)
    bytes_pp = {"hash": STAGE_BYTES["hash"], "sort": STAGE_BYTES["sort"],
                "reorder": STAGE_BYTES["reorder"], "density": STAGE_BYTES["density"],
                "force": meta["force_b"], "integrate": meta["integrate_b"]}
    peak, peak_kind = load_peaks()
    achieved = bytes_pp[dom] * n / (per_stage[dom] / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(HERE, "profiles", "traffic_%s.json" % cfg["workload"])
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(dom)

    # ---- the neighbour loops against the FP32 issue roofline ----
    fp32 = None
    if not batched:
        try:
            cand, inter = pair_counts(p, s.getArray(cm.POSITION))
            mhz = (clocks or {}).get("sm_mhz") or 2070.0
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            peak_tf = sms * 128 * 2 * mhz * 1e6 / 1e12
            fp32 = {"candidates_per_particle": round(cand, 1), "neighbours_per_particle": round(inter, 1),
                    "peak_tflops": round(peak_tf, 1),
                    "peak_kind": "nominal: %d SMs x 128 FP32 lanes x 2 flop x sampled SM clock" % sms}
            lists = bool(tuning.get("lanes_density_force_lists", [1, 1, True])[2])
            fp32["force_path"] = "interaction lists" if lists else "cell walk"
            for k, per_pair in (("density", FLOPS_DENSITY_PAIR), ("force", FLOPS_FORCE_PAIR)):
                # the list-driven force visits interacting pairs only; the DamBreak
                # force runs for fluid particles only
                visits = 0.0 if (k == "force" and lists) else cand
                fl = FLOPS_CANDIDATE * visits + per_pair * inter
                parts = fluid if (k == "force" and p.system == 0) else n
                tf = fl * parts / (per_stage[k] / 1e3) / 1e12
                fp32[k] = {"flops_per_particle": round(fl, 1), "achieved_tflops": round(tf, 3),
                           "frac": round(tf / peak_tf, 4)}
        except Exception as e:  # scipy missing: report the HBM roofline alone
            fp32 = {"unavailable": str(e)[:120]}

    # ---- end-to-end through the public API with host buffers ----
    arrays = [cm.POSITION, cm.VELOCITY, cm.VELOCITYLEAPFROG]
    host = {a: torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy() for a in arrays}
    if batched:
        put = lambda a: s.upload(a, host[a])  # noqa: E731
        get = lambda a: s.download(a, host[a])  # noqa: E731
    if batched:
        put_all = lambda: [put(a) for a in arrays]  # noqa: E731
        get_all = lambda: [get(a) for a in arrays]  # noqa: E731
    else:
        # the three arrays in one call each way (one synchronisation per call)
        put_all = lambda: s.setArrays({a: host[a] for a in arrays})  # noqa: E731
        get_all = lambda: s.getArrays({a: host[a] for a in arrays})  # noqa: E731
    get_all()
    e2e_steps = max(1, min(args.steps, 20 if batched else 50))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        put_all()
        s.update()
        get_all()
    e2e_secs = barrier_max(dist, time.perf_counter() - t0)
    e2e_value = (total_fluid if batched else fluid * world) * e2e_steps / e2e_secs
    io_bytes = 3 * 16 * n

    line = {
        "metric": METRIC, "value": value, "unit": "particle-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "strong" if batched else "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded lattices%s, seed 1973)" % ("" if batched else " + jitter"),
        "config": cfg,
        "e2e": {"value": e2e_value, "unit": "particle-updates/s", "h2d_bytes_per_step": io_bytes,
                "d2h_bytes_per_step": io_bytes, "steps": e2e_steps},
        "gpu_launches": meta["launches"] * args.steps,
        "tuning": tuning,
        "stage_ms": {k: round(v, 5) for k, v in per_stage.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "bytes_per_particle": bytes_pp[dom], "fp32": fp32},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        from oracle import oracle as O
        O.build()
        if batched:
            v, dt, sample = cpu_run_batched(s.P, s.N, s.F, s.D, threads)
        else:
            v, dt = cpu_run(args.workload, args.cpu_steps, threads)
            sample = ("%d full step(s) of the same %d-particle scene from its initial state (oracle "
                      "restatement of the reference kernels, all host threads)" % (args.cpu_steps, n))
        line["cpu_baseline"] = {"value": v, "unit": "particle-updates/s", "cores": threads,
                                "kind": "port", "seconds": dt, "sample": sample}
        if not batched:
            v1, dt1 = cpu_run(args.workload, 1, 1)
            line["cpu_baseline"]["one_core"] = {"value": v1, "seconds": dt1, "sample": "1 full step, 1 thread"}
    if not batched and args.workload == "dambreak3d" and rank == 0 and world == 1 and not args.no_ref_gpu:
        line["reference_gpu"] = reference_gpu_bar()
        bar = line["reference_gpu"].get("dambreak3d_954860_reference_loops")
        if bar:
            line["reference_gpu"]["own_vs_reference_loops"] = value / bar["reference_updates_per_s"]
    if not batched and args.workload == "dambreak3d" and not args.no_t1 and world == 1:
        # the metric's second half: wall-time to t = 1 s at <= 2 % front error,
        # plain fine vs learned coarse vs batched
        t1 = run_to_t1(s, p, args.verlet if kept else 0.0)
        line["to_t1"] = {"plain_fine": {k: (round(v, 5) if isinstance(v, float) else v) for k, v in t1.items()
                                        if k not in ("times", "fronts")},
                         "fronts_every_0.05s": [round(f, 4) for f in t1["fronts"][::5]]}
        s.close()
        s = None
        if not args.no_learned:
            line["to_t1"]["learned_coarse"] = learned_to_t1(t1)
        if not args.no_batched_t1:
            line["to_t1"]["batched_dambreak128"] = batched_to_t1()
    if s is not None:
        s.close()
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
