"""Benchmark of the GB300 MR advection step (one JSON line on stdout).

Workload (the max_level-12 2D configuration): linear advection
u_t + a.grad(u) = 0 on [0,1]^2, a = (1, 0.5), MRMesh min level 4, max level 12
(4096^2 finest-equivalent), max_stencil_size 2 with the minimal ghost width
disabled (as demos/FiniteVolume/advection_2d.cpp), Dirichlet 0, FP64.  The
initial condition is a seeded sum of 16 indicator squares and 16 Gaussians.
One step = make_MRAdapt(eps=1e-4, regularity=2) + update_ghost_mr + the
upwind step, dt = 0.5 dx(max_level).  The metric is active cell-updates/s:
leaf cells advanced per second, adaptation and ghost work included.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU implementation of the same path (the oracle
port of samurai's algorithm: the reference itself cannot be built here) on
the host cores, on the same workload, metric and unit.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from advection_cases import ball_3d, shapes_2d  # noqa: E402
from samurai_gb300.replicas import reduce_over_ranks, shard_instances  # noqa: E402

CFG = dict(dim=2, min_level=4, max_level=12, a=(1.0, 0.5), eps=1e-4, regularity=2.0, seed=2026, cfl=0.5)
# the 3D workload (--workload advection3d): ball + 8 Gaussians, a = (1,1,1), L3..9
CFG_3D = dict(dim=3, min_level=3, max_level=9, a=(1.0, 1.0, 1.0), eps=1e-3, regularity=1.0, seed=2026, cfl=0.3)
METRIC = "active cell-updates/s"
UNIT = "cell-updates/s"
L2_BYTES = 129 * 1024 * 1024
UPWIND_DRAM_BYTES_PER_CELL = 8572672.0 / 511813.0


def workload_config(extra=None):
    if CFG["dim"] == 3:
        desc = ("3D MR linear advection, min_level 3, max_level %d, a=(1,1,1), eps 1e-3, regularity 1, "
                "ball + 8 Gaussians (seed %d), Dirichlet 0, dt=0.3*dx_min, upwind" % (CFG["max_level"], CFG["seed"]))
    else:
        desc = ("2D MR linear advection, min_level 4, max_level %d, a=(1,0.5), eps 1e-4, regularity 2, "
                "16 squares + 16 Gaussians (seed %d), Dirichlet 0, dt=0.5*dx_min, upwind" % (CFG["max_level"], CFG["seed"]))
    c = {
        "workload": desc,
        "min_level": CFG["min_level"],
        "max_level": CFG["max_level"],
        "max_stencil_radius": 1,
        "prediction_radius": 1,
        "l2": "flushed (256 MiB write) before every timed step",
    }
    if extra:
        c.update(extra)
    return c


def uniform_mesh(mesh, dim, level):
    """make the leaf cells of `mesh` the uniform mesh of `level`"""
    idx = np.arange(1 << level, dtype=np.int32)
    if dim == 2:
        y, x = np.meshgrid(idx, idx, indexing="ij")
        coords = np.stack([x.ravel(), y.ravel()], axis=1)
    else:
        z, y, x = np.meshgrid(idx, idx, idx, indexing="ij")
        coords = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    mesh.set_cells(np.full(coords.shape[0], level, np.int32), coords)


def initial_values(level, coords):
    if CFG["dim"] == 3:
        return ball_3d(CFG["seed"])(level, coords)
    return shapes_2d(CFG["seed"])(level, coords)


# ------------------------------------------------------------------ helpers
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_info():
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "processor\t")) and ":" in line and "model name" in line.lower():
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    return model or os.uname().machine


def clock_dir():
    """where the raw nvidia-smi samples go: $SG_CLOCK_LOG_DIR, else the temporary directory"""
    d = os.environ.get("SG_CLOCK_LOG_DIR") or tempfile.gettempdir()
    os.makedirs(d, exist_ok=True)
    return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, path):
        self.path = path
        self.proc = None
        try:
            self.f = open(path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


UPWIND_ISSUED = {2: 10 * 2 + 3 + 2, 3: 10 * 3 + 5 + 2}
# DRAM bytes per launch of the kernels named dominant, by (dim, max_level, kernel), from ncu captures (profiles/):
# (bytes, how they were measured)
DOMINANT_TRAFFIC = {
    (2, 12, "ghost_level"): (959558.0, "ncu dram__bytes_read.sum + dram__bytes_write.sum averaged over the 22 k_ghost_level launches of one "
                              "2D max_level-12 step (levels 12..2, twice; caches emptied by ncu before each launch)"),
}


def left_shared(level, coords):
    """leaves whose left x-neighbour is a leaf of the same level"""
    key_bits = 21
    dim = coords.shape[1]
    total = 0
    for l in np.unique(level):
        c = coords[level == l].astype(np.int64) + 64
        k = c[:, 0] | (c[:, 1] << key_bits)
        if dim == 3:
            k = k | (c[:, 2] << (2 * key_bits))
        total += int(np.isin(k - 1, k).sum())
    return total


def halo_count(level, coords):
    """Distinct same-level non-leaf neighbours (+-1 along each axis) of the
    leaf cells: the ghost values the upwind stencil reads."""
    key_bits = 21
    dim = coords.shape[1]
    total = 0
    for l in np.unique(level):
        c = coords[level == l].astype(np.int64) + 64

        def key(x):
            k = x[:, 0] | (x[:, 1] << key_bits)
            if dim == 3:
                k = k | (x[:, 2] << (2 * key_bits))
            return k

        keys = key(c)
        nb = []
        for d in range(dim):
            for s_ in (1, -1):
                cc = c.copy()
                cc[:, d] += s_
                nb.append(key(cc))
        nb = np.unique(np.concatenate(nb))
        total += int(np.setdiff1d(nb, np.unique(keys), assume_unique=True).size)
    return total


# ------------------------------------------------- per-kernel step table
PX, PY = 32, 8  # padding of the level boxes (samurai_gb300/csrc/sg_core.cuh)


def level_words(dim, maxl):
    """32-bit words per level of the dense bitmaps (sg::make_geom)"""
    out = []
    for l in range(maxl + 1):
        n = 1 << l
        W = (n + 31) // 32 + 2
        R = n + 2 * PY
        out.append(W * (R if dim == 2 else R * R))
    return out


def mesh_id_counts(sim, maxl):
    """cells of each MRMesh id over all levels, from the exported intervals"""
    out = {}
    for mid in ("cells", "proj_cells", "union_cells", "reference"):
        tot = 0
        for lev in range(maxl + 1):
            iv = sim.mesh.intervals(mid, lev)
            tot += int(np.sum(iv[:, 1].astype(np.int64) - iv[:, 0]))
        out[mid] = tot
    return out


# bitmaps a word kernel reads or writes, per word of the levels it covers
# (4 bytes each): the algorithmic traffic of the integer mesh kernels
WORD_KERNEL_BITMAPS = {
    "hc_cag": 3, "hc2_cag_on": 4, "hc2_cag_z": 4, "cag_on": 2, "union": 3, "ref0": 4, "ref0_xy": 4, "ref0_z": 4, "ref_children": 4,
    "proj": 3, "scan_sums": 2, "scan_write": 5, "tag_flags": 3, "new_cells": 4, "grad_coarsen": 2, "grad_expand": 2, "grad_expand_xy": 2,
    "grad_expand_z": 2, "grad_down": 5, "grad_apply": 3, "compare": 2,
}


def kernel_bytes(name, dim, counts, halo, words_all, words_ref, passes):
    """Algorithmic bytes of one step's launches of kernel `name` (each array
    element counted once per kernel): passes = (fronts, backs) of the step's
    Harten passes.  FP64 kernels from the mesh-id counts, word kernels from the
    words of the levels they cover."""
    nc, nr, npj = counts["cells"], counts["reference"], counts["proj_cells"]
    ch = 1 << dim
    fronts, backs = passes
    ghosts = max(nr - nc - npj, 0)
    per_front = {
        "tag_init": 9 * nr,
        "ghost_level": 8 * (ch + 1) * npj,           # projection: 2^d children read, 1 written
        "ghost_levels_small": 0,
        "ghost_corner_projection": 0,
        "predict": 8 * ghosts + 8 * ghosts // ch,    # ghost written + its coarse parent read
        "predict_small": 0,
        "detail": 8 * (1 + 2 * ch) * npj,            # parent + children read, children's details written
        "criteria": (8 * (ch + 1) + ch) * npj,       # details read, tags written
        "maximum": 2 * (ch + 1) * npj,               # tags read and written
        "maximum_small": 0,
        "keep_boundary": 0,
    }
    if name == "upwind" or name == "convection":
        return 16 * nc + 8 * halo
    if name in per_front:
        return per_front[name] * fronts
    if name == "update_fields":
        return 16 * nr * backs
    if name in WORD_KERNEL_BITMAPS:
        words = words_all if name in ("tag_flags", "new_cells", "compare", "scan_sums", "scan_write") else words_ref
        # the scan and mesh construction run once per back half, the others once per front half
        n = backs if name in ("hc_cag", "hc2_cag_on", "hc2_cag_z", "cag_on", "union", "ref0", "ref0_xy", "ref0_z", "ref_children", "proj",
                              "scan_sums", "scan_write") else fronts
        return 4 * WORD_KERNEL_BITMAPS[name] * words * n
    return 0


def step_kernel_table(sim, step, dim, maxl, minl, halo, peak):
    """One traced step: per kernel its launches, device time (from the
    per-launch trace events, inside the captured graphs), algorithmic bytes and
    achieved GB/s against the measured HBM peak."""
    sim.mesh.kernel_trace(True)  # capture the traced launch sequences once
    step()
    sim.mesh.kernel_trace(False)
    counts = mesh_id_counts(sim, maxl)
    sim.mesh.synchronize()
    sim.mesh.kernel_trace(True)
    passes = step()
    rows, valid = sim.mesh.kernel_trace(False)
    words = level_words(dim, maxl)
    lmin = max(minl - 2, 0)
    words_ref, words_all = sum(words[lmin:]), sum(words)
    fronts = passes
    backs = passes - 1 if passes < maxl - minl else passes
    table = []
    total_b = 0
    total_ms = 0.0
    for name, n, ms in sorted(rows, key=lambda r: -r[2]):
        b = kernel_bytes(name, dim, counts, halo, words_all, words_ref, (fronts, backs))
        total_b += b
        total_ms += ms
        gbs = b / (ms * 1e-3) / 1e9 if ms > 0 else None
        table.append({"kernel": name, "launches": n, "us": round(1e3 * ms, 2), "algorithmic_bytes": int(b),
                      "GB_s": round(gbs, 2) if gbs is not None else None, "frac_of_hbm": round(gbs / peak, 5) if gbs is not None else None})
    return {"valid": valid, "harten_passes": passes, "launches": sum(r[1] for r in rows), "traced_ms": total_ms,
            "algorithmic_bytes": int(total_b), "kernels": table,
            "mesh_counts": counts,
            "note": "one step traced inside its captured graphs: each launch's time runs from the previous launch's end event (or the "
                    "head event of its graph: host round trips between graphs are charged to no kernel) to its own (kernel time plus "
                    "the gap before it); bytes: each array element once per kernel (FP64 kernels from the mesh-id counts, word kernels "
                    "4 B per bitmap word of the levels they cover)"}


# --------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from samurai_gb300 import build as gpu_build

    gpu_build.build()
    import samurai_gb300 as sg

    dim, minl, maxl = CFG["dim"], CFG["min_level"], CFG["max_level"]
    a = list(CFG["a"])
    dt = CFG["cfl"] / (1 << maxl)
    sim = sg.AdvectionSim(dim, minl, maxl, 1, 1)
    if args.init_level is not None and args.init_level < maxl:
        # the initial condition sampled on a coarser uniform mesh (the adaptation refines where the details ask)
        uniform_mesh(sim.mesh, dim, args.init_level)
    lv, co, _ = sim.cells()
    sim.set_cell_values(initial_values(lv, co))
    sim.adapt(CFG["eps"], CFG["regularity"])  # initial adaptation, as the demo does before its loop
    stream_ptr = sim.mesh.stream()
    stream = torch.cuda.ExternalStream(stream_ptr)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")

    def step():
        # MRadaptation, update_ghost_mr, upwind, swap: sg_step, one captured graph per step
        return sim.step(CFG["eps"], CFG["regularity"], a, dt)

    # the launch-shape autotuner on this problem (the timed steps below use its choice)
    tune = None
    if not args.no_tune:
        d_ms, t_ms, shape = sim.autotune(CFG["eps"], CFG["regularity"], a, dt, steps=10)
        tune = {"default_ms_per_step": d_ms, "tuned_ms_per_step": t_ms, "shape": shape,
                "how": "sg_autotune: coordinate descent over threads per block, grid limit and one-block chain limits, "
                       "10 steps from the same state per candidate, best of two"}
    for _ in range(args.warmup):
        step()
    sim.mesh.synchronize()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident timed region
    sampler = ClockSampler(local, os.path.join(clock_dir(), "clocks_rank%d.csv" % rank)) if rank == 0 else None
    barrier()
    total_ms = 0.0
    cell_updates = 0
    sim.mesh.launch_count(reset=True)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        n_cells = sim.nb_cells()
        with torch.cuda.stream(stream):
            ev0.record(stream)
        step()
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
        cell_updates += n_cells
    launches = sim.mesh.launch_count()
    barrier()
    clocks = sampler.stop() if sampler else None
    ms = total_ms / args.steps
    total_ms_max, cell_updates_all = reduce_over_ranks(total_ms, cell_updates, world, device="cuda")
    value = cell_updates_all / (total_ms_max / 1e3)
    if args.quick:
        # profiling runs: the timed steps only
        if rank == 0:
            free, total = torch.cuda.mem_get_info()
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": total_ms_max / args.steps, "quick": True,
                              "config": workload_config({"cells_final": sim.nb_cells(), "initial_mesh_level": args.init_level or maxl}),
                              "device_memory_used_gb": (total - free) / 1e9}))
        return

    # ---- end-to-end through the C ABI with host buffers
    cap = sim.mesh.nb_cells("reference") * 4 + 1024
    host = torch.empty(cap, dtype=torch.float64, pin_memory=True)
    hbuf = host.numpy()
    e2e_steps = max(1, min(args.steps, 50))
    h2d = d2h = 0
    e2e_updates = 0
    n_ref = sim.nb_ref()
    hbuf[:n_ref] = sim.u.array()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        n_ref = sim.nb_ref()
        if n_ref > cap:
            raise RuntimeError("pinned buffer too small")
        sim.u.set_array(hbuf[:n_ref])
        h2d += 8 * n_ref
        e2e_updates += sim.nb_cells()
        step()
        n_ref = sim.nb_ref()
        out = hbuf[:n_ref]


        sg._check(sg.lib().sg_field_download(sim.u.h, out.ctypes.data_as(ctypes.c_void_p), n_ref), "download")
        d2h += 8 * n_ref
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_updates * world / e2e_s

    # ---- roofline of the upwind kernel, timed alone on its launch stream
    nc, _ = sim.mesh.counts()
    lv, co, _ = sim.cells()
    lv_all, co_all = lv, co
    halo = halo_count(lv, co)
    alg_bytes = 16 * nc + 8 * halo
    reps = 20
    upw_ms = 0.0
    for _ in range(reps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            ev0.record(stream)
        sim.unp1.assign_upwind(sim.u, a, dt)
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        upw_ms += ev0.elapsed_time(ev1)
    upw_ms /= reps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = alg_bytes / (upw_ms / 1e3) / 1e9
    # FP64 roof: the upwind formula of the reference costs 5 FP64 operations
    # per face flux plus 5 (2D) to assemble the update: 26 per cell in 2D
    # the reference's formula: 5 FP64 operations per face flux (2 dim fluxes),
    # 2 dim - 1 to combine them, 3 to scale and update: 26 in 2D, 38 in 3D
    fp64_ref_ops = (10 * dim + 2 * dim - 1 + 3) * nc
    # FP64 instructions issued by k_upwind: 5 per face flux (2 dim faces), 2 dim - 1
    # additions to combine them and 2 for u - dt * s (the 2^l scaling moves the
    # exponent); the left x-flux is taken from the previous lane when that lane
    # holds the left neighbour (5 fewer)
    fp64_ops = UPWIND_ISSUED[dim] * nc - 5 * left_shared(lv_all, co_all)
    try:
        fp64_peak = sg.device_fp64_rate()
    except Exception:
        fp64_peak = None
    # DRAM bytes of one k_upwind launch of this workload, from an ncu capture
    # (8 572 672 B read + 768 B written on a mesh of about 511 813 leaf cells:
    # the sixth step of a run of this benchmark), scaled to this launch's leaf
    # cells: the traffic grows with the cells read and written
    traffic = UPWIND_DRAM_BYTES_PER_CELL * nc

    # ---- samurai's named timers over a few extra steps (per-phase GPU time)
    phase_steps = 10
    sim.mesh.timers(enable=True, reset=True)
    for _ in range(phase_steps):
        step()
    phases = {k: round(v[0] / phase_steps, 4) for k, v in sim.mesh.timers(enable=False).items()}

    # ---- one step traced launch by launch: per-kernel time, bytes, GB/s; the
    # step's algorithmic bytes over the device-timed step
    lv, co, _ = sim.cells()
    ktab = step_kernel_table(sim, step, dim, maxl, minl, halo_count(lv, co), peak)
    step_ms = total_ms_max / args.steps
    # the dominant kernel: the largest share of the traced step
    dom = ktab["kernels"][0]
    dom_launch_ms = dom["us"] / 1e3 / max(dom["launches"], 1)
    dom_bytes = dom["algorithmic_bytes"] / max(dom["launches"], 1)
    roofline = {"bound": "hbm", "kernel": dom["kernel"], "achieved": dom_bytes / (dom_launch_ms * 1e-3) / 1e9 if dom_launch_ms > 0 else None,
                "peak": peak, "peak_source": peak_src, "unit": "GB/s", "traffic": DOMINANT_TRAFFIC.get((dim, maxl, dom["kernel"]), (None, None))[0],
                "traffic_source": DOMINANT_TRAFFIC.get((dim, maxl, dom["kernel"]), (None, None))[1],
                "algorithmic_bytes_per_launch": int(dom_bytes), "launch_ms": dom_launch_ms, "launches_per_step": dom["launches"],
                "share_of_step": dom["us"] / 1e3 / ktab["traced_ms"] if ktab["traced_ms"] > 0 else None,
                "timing": "per-launch trace events inside the captured graphs, one step"}
    roofline["frac"] = roofline["achieved"] / peak if roofline["achieved"] else None
    roofline_step = {"algorithmic_bytes": ktab["algorithmic_bytes"], "ms_per_step": step_ms,
                     "achieved": ktab["algorithmic_bytes"] / (step_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s"}
    roofline_step["frac"] = roofline_step["achieved"] / peak

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        extras["adjoint"] = adjoint_record(args, fd_directions=8, steps=256)
        extras["batch"] = batch_record(args, steps=10, warmup=3, serial_steps=3)

    cpu = cpu_baseline(sim, a, dt) if (rank == 0 and not args.no_cpu_baseline) else None

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": total_ms_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic: seeded squares + Gaussians (no dataset involved)",
            "config": workload_config({"parallelism": "replicas" if world > 1 else "single GPU",
                                       "cells_final": int(nc), "reference_cells_final": int(sim.nb_ref())}),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d / e2e_steps), "d2h_bytes_per_step": int(d2h / e2e_steps),
                    "steps": e2e_steps, "api": "sg_field_upload + sg_step (MRadaptation, update_ghost_mr, upwind, swap) + sg_field_download"},
            "roofline": roofline,
            "roofline_step": roofline_step,
            "kernels_step": ktab,
            "upwind_roofline": {"bound": "hbm", "kernel": "k_upwind", "achieved": achieved, "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                                "frac": achieved / peak, "traffic": traffic,
                                "traffic_source": "ncu dram__bytes of a 536 428-cell launch, scaled by leaf cells",
                                "algorithmic_bytes": int(alg_bytes), "launch_ms": upw_ms, "timing": "k_upwind alone, L2 flushed, 20 launches",
                                "cells": int(nc), "halo": int(halo),
                                "fp64": {"achieved_gflops": fp64_ops / (upw_ms / 1e3) / 1e9, "peak_gflops": fp64_peak,
                                         "peak_source": "measured in this run (sg_device_fp64_rate probe)",
                                         "frac": (fp64_ops / (upw_ms / 1e3) / 1e9 / fp64_peak) if fp64_peak else None,
                                         "ops_per_launch": int(fp64_ops), "reference_formula_ops": int(fp64_ref_ops),
                                         "note": "FP64 instructions the kernel issues: %d per leaf cell, %d fewer when the left x-face flux "
                                                 "comes from the previous lane (counted for every leaf whose left neighbour is a leaf of the same "
                                                 "level: an upper bound on the sharing); the reference's formula counts %d"
                                                 % (UPWIND_ISSUED[dim], 5, 10 * dim + 2 * dim - 1 + 3)}},
            "gpu_launches": int(launches),
            "launches_per_step": launches / args.steps,
            "phases_ms_per_step": phases,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "autotune": tune,
            "adjoint": extras.get("adjoint"),
            "batch": extras.get("batch"),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(sim, a, dt, budget_s=15.0):
    """The CPU oracle advanced from the GPU's current state (same mesh, same
    leaf values) for about budget_s seconds of steps, 1 thread."""
    from oracle.pyoracle import OracleSim

    lv, co, _ = sim.cells()
    vals = sim.cell_values()
    o = OracleSim(CFG["dim"], CFG["min_level"], CFG["max_level"], 1, 1)
    o.set_cells(lv, co)
    o.set_cell_values(vals)
    t0 = time.perf_counter()
    n = 0
    updates = 0
    while True:
        updates += o.nb_cells()
        o.adapt(CFG["eps"], CFG["regularity"])
        o.update_ghost()
        o.upwind(list(a), dt, 0)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": updates / el, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_info(),
            "sample": "%d steps of the same workload from the GPU run's final mesh and values (%.1f s)" % (n, el)}


def batch_cpu_baseline(probs, sims, budget_s=15.0):
    """The CPU oracle stepping the batched instances one after the other (as a
    samurai user would), each from the GPU run's current mesh and values, for
    about budget_s seconds; 1 thread."""
    from oracle.pyoracle import OracleSim

    t_run = 0.0
    updates = 0
    n = 0
    for p, sim in zip(probs, sims):
        lv, co, _ = sim.cells()
        o = OracleSim(2, p["min_level"], p["max_level"], 1, 1)
        o.set_cells(lv, co)
        o.set_cell_values(sim.cell_values())
        t0 = time.perf_counter()
        updates += o.nb_cells()
        o.adapt(p["eps"], p["regularity"])
        o.update_ghost()
        o.upwind(list(p["a"]), p["dt"], 0)
        t_run += time.perf_counter() - t0
        n += 1
        if t_run > budget_s:
            break
    return {"value": updates / t_run, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_info(),
            "sample": "one time step of each of the first %d instances, from the GPU run's meshes and values (%.1f s)" % (n, t_run)}


# --------------------------------------------------------- reference arm
def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle.pyoracle import OracleSim

    dim, minl, maxl = CFG["dim"], CFG["min_level"], CFG["max_level"]
    dt = CFG["cfl"] / (1 << maxl)
    t_setup = time.perf_counter()
    o = OracleSim(dim, minl, maxl, 1, 1)
    lv, co, _ = o.cells()
    o.set_cell_values(initial_values(lv, co))
    o.adapt(CFG["eps"], CFG["regularity"])
    for _ in range(args.warmup):
        o.adapt(CFG["eps"], CFG["regularity"])
        o.update_ghost()
        o.upwind(list(CFG["a"]), dt, 0)
    setup = time.perf_counter() - t_setup
    budget = 90.0
    t0 = time.perf_counter()
    n = 0
    updates = 0
    while n < args.steps:
        updates += o.nb_cells()
        o.adapt(CFG["eps"], CFG["regularity"])
        o.update_ghost()
        o.upwind(list(CFG["a"]), dt, 0)
        n += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = updates / el
    sample = "%d of %d requested steps after the initial adaptation (setup %.0f s), 1 thread" % (n, args.steps, setup)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": n,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * el / n,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: seeded squares + Gaussians (no dataset involved)",
        "config": workload_config({"parallelism": "sequential CPU (the reference MR path has no threading)"}),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_info(), "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_batch(args):
    """The batched workload as its own benchmark line (--workload batch)."""
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")  # one hardware queue per busy stream
    line = batch_record(args, args.steps, args.warmup, max(1, min(args.steps, 10)), full=True)
    if line is not None:
        print(json.dumps(line))


def batch_record(args, steps, warmup, serial_steps, full=False):
    """256 independent 2D problems (max_level U{7..11}, min_level 2, a U[-1,1]^2,
    1-8 shapes, eps 1e-3 or 1e-4) stepped together through sg_batch_step, and
    the same problems stepped one after the other through the serial calls.
    Returns the record (rank 0) or None."""
    import torch

    from samurai_gb300 import build as gpu_build

    gpu_build.build()
    import samurai_gb300 as sg
    from advection_cases import batch_instances

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    all_probs = batch_instances(2027, args.instances)
    # N GPUs: each rank advances its shard of the instances (no exchange)
    mine = shard_instances([4.0 ** p["max_level"] for p in all_probs], rank, world)
    probs = [all_probs[i] for i in mine]
    sims = []
    for p in probs:
        s = sg.AdvectionSim(2, p["min_level"], p["max_level"])
        lv, co, _ = s.cells()
        s.set_cell_values(p["u0"](lv, co))
        sims.append(s)
    batch = sg.Batch(sims, n_threads=args.batch_threads)
    eps = [p["eps"] for p in probs]
    reg = [p["regularity"] for p in probs]
    a = [p["a"] for p in probs]
    dt = [p["dt"] for p in probs]
    batch.adapt(eps, reg)
    # the batch's launch-shape autotuner (sg_batch_autotune; the timed steps use its choice)
    tune = None
    if not args.no_tune:
        d_ms, t_ms, shape = batch.autotune(eps, reg, a, dt, steps=3)
        tune = {"default_ms_per_step": d_ms, "tuned_ms_per_step": t_ms, "shape": shape,
                "how": "sg_batch_autotune: one-block chain limit shared by the instances, then threads per block; "
                       "3 batched steps from the same state per candidate"}
    for _ in range(warmup):
        batch.step(eps, reg, a, dt)
    batch.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(fn, steps):
        total, updates = 0.0, 0
        for _ in range(steps):
            n = sum(s.nb_cells() for s in sims)
            flush.fill_(1)
            barrier()
            t0 = time.perf_counter()
            fn()
            barrier()
            total += time.perf_counter() - t0
            updates += n
        return total, updates

    sampler = ClockSampler(local, os.path.join(clock_dir(), "clocks_batch.csv")) if (rank == 0 and full) else None
    b_s, b_updates = timed(lambda: (batch.step(eps, reg, a, dt), batch.synchronize()), steps)
    clocks = sampler.stop() if sampler else None
    b_ms, b_updates = reduce_over_ranks(1e3 * b_s, b_updates, world, device="cuda")
    b_s = b_ms / 1e3

    def serial_step():
        for p, s in zip(probs, sims):
            s.adapt(p["eps"], p["regularity"])
            s.update_ghost()
            s.upwind(p["a"], p["dt"])

    # the serial calls with the instances' own launch shapes (the batch sets its own)
    batch.close()
    s_s, s_updates = timed(serial_step, serial_steps)
    s_ms, s_updates = reduce_over_ranks(1e3 * s_s, s_updates, world, device="cuda")
    s_s = s_ms / 1e3
    cells = [s.nb_cells() for s in sims]
    if rank != 0:
        return None
    cpu = None if (args.no_cpu_baseline or not full) else batch_cpu_baseline(probs, sims)
    line = {
        "metric": METRIC,
        "value": b_updates / b_s,
        "unit": UNIT,
        "n_gpus": world,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": 1e3 * b_s / steps,
        "higher_is_better": True,
        "scaling": "strong",  # a fixed set of instances shared by the ranks
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: seeded shapes per instance (no dataset involved)",
        "config": {"workload": "%d independent 2D MR advection problems: max_level U{7..11}, min_level 2, a U[-1,1]^2, 1-8 shapes, "
                               "eps 1e-3 or 1e-4, regularity 2, dt=0.5*dx_min (seed 2027)" % len(all_probs),
                   "parallelism": "instances sharded over %d GPU(s), no exchange" % world,
                   "host_threads": args.batch_threads, "cells_final_total_rank0": int(sum(cells)),
                   "cells_final_max": int(max(cells)), "cells_final_min": int(min(cells)),
                   "timing": "wall clock between device synchronisations, L2 flushed (256 MiB write) before every step"},
        "serial": {"value": s_updates / s_s, "unit": UNIT, "steps": serial_steps, "ms_per_step": 1e3 * s_s / serial_steps,
                   "api": "sg_adapt + sg_update_ghost_mr + sg_upwind + sg_field_swap per instance, one after the other"},
        "speedup_vs_serial": (b_updates / b_s) / (s_updates / s_s),
        "autotune": tune,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    batch.close()
    del sims
    return line


def run_adjoint(args):
    """The adjoint workload as its own benchmark line (--workload adjoint)."""
    print(json.dumps(adjoint_record(args, args.fd_directions, args.adjoint_steps)))


def adjoint_record(args, fd_directions, steps):
    """The adjoint workload: 2D, min_level 3, max_level 10, a = (1, 0.7), 256
    steps, J = sum vol (u_T - u_tgt)^2 with a seeded Gaussian target,
    checkpoints every 16 steps.  Times a plain forward (the loop through the
    serial calls), the recorded forward and the backward pass, and checks the
    gradient: dot-product test and central finite differences on the recorded
    meshes along seeded directions in u0 and along each velocity component."""
    import torch

    from samurai_gb300 import build as gpu_build

    gpu_build.build()
    import samurai_gb300 as sg
    from advection_cases import cell_volumes, gaussian_target

    torch.cuda.set_device(0)
    minl, maxl, eps, reg, K = 3, 10, 1e-4, 2.0, 16
    a = (1.0, 0.7)
    dt = 0.5 / (1 << maxl)
    s = sg.AdvectionSim(2, minl, maxl)
    lv, co, _ = s.cells()
    s.set_cell_values(shapes_2d(2028, 8, 8)(lv, co))
    s.adapt(eps, reg)
    adj = sg.Adjoint(s.u, checkpoint_every=K)
    u0 = s.cell_values()
    tgt_f = gaussian_target(2029)

    def objective(uT):
        lvT, coT = adj.cells("final")
        vol = cell_volumes(lvT)
        tgt = tgt_f(lvT, coT)
        return float(np.sum(vol * (uT - tgt) ** 2)), 2.0 * vol * (uT - tgt)

    adj.record(u0, steps, eps, reg, a, dt)  # warm-up (graphs, allocations)
    _, gT = objective(adj.final())
    adj.backward(gT)
    # the plain forward: the same loop from the same state through the serial
    # calls, no recording (warmed up, then reset to the initial mesh and u0)
    plain = sg.AdvectionSim(2, minl, maxl)
    lv0, co0 = adj.cells("initial")

    def plain_loop(n):
        plain.mesh.set_cells(lv0, co0)
        plain.set_cell_values(u0)
        plain.mesh.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            plain.adapt(eps, reg)
            plain.update_ghost()
            plain.upwind(a, dt)
        plain.mesh.synchronize()
        return time.perf_counter() - t0

    plain_loop(16)  # warm-up (graph captures)
    t_plain = plain_loop(steps)
    plain_uT = plain.cell_values()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    uT = adj.record(u0, steps, eps, reg, a, dt)
    t_fwd = time.perf_counter() - t0
    assert np.array_equal(plain_uT, uT), "the recorded forward differs from the plain loop"
    J, gT = objective(uT)
    t0 = time.perf_counter()
    g0, ga = adj.backward(gT)
    t_bwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    adj.replay(u0, a)
    t_rep = time.perf_counter() - t0

    rng = np.random.default_rng(2030)
    n0, nT, _ = adj.counts()
    v, w = rng.standard_normal(n0), rng.standard_normal(nT)
    Lv = adj.replay(v, a)
    LTw, _ = adj.backward(w)
    dot_err = abs(float(Lv @ w) - float(v @ LTw)) / max(abs(float(Lv @ w)), 1e-300)
    fd_u = []
    for _ in range(fd_directions):
        d = rng.standard_normal(n0)
        h = 1e-3
        jp, _ = objective(adj.replay(u0 + h * d, a))
        jm, _ = objective(adj.replay(u0 - h * d, a))
        fd = (jp - jm) / (2 * h)
        fd_u.append(abs(fd - float(g0 @ d)) / max(abs(fd), 1e-300))
    fd_a = []
    for k in range(2):
        h = 1e-6
        ap, am = list(a), list(a)
        ap[k] += h
        am[k] -= h
        jp, _ = objective(adj.replay(u0, ap))
        jm, _ = objective(adj.replay(u0, am))
        fd = (jp - jm) / (2 * h)
        fd_a.append(abs(fd - ga[k]) / max(abs(fd), 1e-300))
    line = {
        "metric": "adjoint time steps/s",
        "value": steps / t_bwd,
        "unit": "steps/s",
        "n_gpus": 1,
        "steps": steps,
        "higher_is_better": True,
        "dtype": "f64",
        "data": "synthetic: seeded squares + Gaussians, seeded Gaussian target (no dataset involved)",
        "config": {"workload": "adjoint of the 2D MR advection loop: min_level 3, max_level 10, a=(1,0.7), eps 1e-4, regularity 2, "
                               "%d steps, checkpoints every %d steps, J = sum vol (u_T - u_tgt)^2" % (steps, K),
                   "cells_initial": int(n0), "cells_final": int(nT), "timing": "wall clock between device synchronisations"},
        "plain_forward_ms_per_step": 1e3 * t_plain / steps,
        "forward_record_ms_per_step": 1e3 * t_fwd / steps,
        "replay_ms_per_step": 1e3 * t_rep / steps,
        "backward_ms_per_step": 1e3 * t_bwd / steps,
        "backward_over_forward": t_bwd / t_fwd,
        "gradient_over_plain_forward": (t_fwd + t_bwd) / t_plain,
        "J": J,
        "dJ_da": [float(x) for x in ga],
        "checks": {"dot_product_rel_err": dot_err, "fd_u0_directions": len(fd_u), "fd_u0_max_rel_err": max(fd_u) if fd_u else None,
                   "fd_a_rel_err": fd_a, "fd_note": "central differences on the recorded meshes, h = 1e-3 (u0, exact for quadratic J), 1e-6 (a)"},
    }
    adj.close()
    return line


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="skip the adjoint and batch sub-records of the default run")
    p.add_argument("--no-tune", action="store_true", help="time the default launch shape (no sg_autotune)")
    p.add_argument("--quick", action="store_true", help="profiling runs: warm-up and timed steps only, a short line")
    p.add_argument("--workload", default="advection2d", choices=["advection2d", "advection3d", "batch", "adjoint"],
                   help="advection2d: the max_level-12 2D problem (default); batch: independent problems through sg_batch_step; "
                        "adjoint: the discrete adjoint of a max_level-10 loop")
    p.add_argument("--max-level", type=int, default=None, help="another max_level for the advection workloads")
    p.add_argument("--init-level", type=int, default=None,
                   help="advection workloads: sample the initial condition on the uniform mesh of this level (default: max_level)")
    p.add_argument("--adjoint-steps", type=int, default=256)
    p.add_argument("--fd-directions", type=int, default=64)
    p.add_argument("--instances", type=int, default=256)
    p.add_argument("--batch-threads", type=int, default=8)
    args = p.parse_args()
    # one hardware queue per busy stream for the batched instances (set before CUDA starts)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "advection3d":
        CFG.clear()
        CFG.update(CFG_3D)
    if args.max_level is not None:
        CFG["max_level"] = args.max_level
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
