#!/usr/bin/env python
"""Benchmark: exact GPU export of a seeded 256-primitive CSG tree on a 512^3 grid.

One step = one complete export of the tree on the GPU -- FP32 distances at every one of
the 515^3 lattice samples through the export octree's clipped programs, naive surface
nets (vertices + faces), gradient normals and material colours per vertex -- with the
compiled tree already resident in HBM.  `value` is samples/s over all ranks; `e2e` is
the same metric through the C ABI call a user makes (tg_export_tree: tree handle in,
mesh in host memory out, octree build and all host<->device copies inside the timing).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times Tangerine's CPU export of the same workload on the host cores
instead: its own code (the AsyncParallelSurfaceNets thunks on its Pool() threadpool, then
per-vertex Gradient + GetMaterial) where the reference library built from its sources loads,
otherwise -- on the GPU host, which has neither the sources nor a way to run x86 builds --
the C restatement in oracle/port run in the reference's cost mode (8 corner evaluations per
cell, 6 per face check).  Its K timed steps are K z-slabs that together make one complete
export; `kind` in the line says which code ran.  `--workload cpu-compare` (x86 host with the
reference sources) times both CPU codes on the same whole export.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "samples/s & 512^3 meshes/s: exact GPU vs surrogate-culled (same mesh) vs CPU"
SEED = 1
PRIMS = 256
RES = 512
WORKLOAD = (f"exact export (bricks without surface skipped, same mesh): seeded {PRIMS}-primitive CSG tree (seed {SEED}; 60% union, 20% diff, 10% inter, "
            f"10% smooth-union; depth <= 12), FP32 on a {RES}^3 grid over [-2,2]^3 "
            f"({RES + 3}^3 lattice samples), surface nets + gradient normals + material colours")
# The config both arms print (the GPU arm and `--impl reference`).
CONFIG = {"workload": WORKLOAD, "samples_per_mesh": (RES + 3) ** 3,
          "l2": "GPU arm: L2 flushed between steps (512 MB write outside the per-step events); per-step working set "
                "0.55 GB lattice > L2",
          "parallelism": "GPU arm: one GPU (replicas for N > 1); reference arm: all host cores of rank 0"}

# FP32 operations per program op (mul/add/sub/div/sqrt/min/max/abs = 1 each), from the
# formulas in tangerine/sdf_evaluator.cpp:165-295 and the interpreter's transforms.
OP_FLOPS = {1: 7, 2: 24, 3: 19, 4: 10, 5: 17, 6: 38, 7: 36, 8: 5,        # brushes
            9: 1, 10: 1, 11: 2, 12: 9, 13: 9, 14: 10, 15: 1,           # set ops, flate
            16: 3, 17: 18, 18: 1}                                       # offset, matrix, scale field
OP_SKIP = {1: 1, 2: 3, 3: 3, 4: 2, 5: 2, 6: 2, 7: 3, 8: 3, 9: 0, 10: 0, 11: 0, 12: 1, 13: 1, 14: 1,
           15: 1, 16: 3, 17: 16, 18: 1}


def program_flops(words: np.ndarray) -> int:
    pc, total = 0, 0
    n = words.size
    while pc < n:
        op = int(words[pc])
        pc += 1
        if op == 0:
            break
        total += OP_FLOPS[op]
        pc += OP_SKIP[op]
    return total


def algorithmic_flops(cells, children, words, grid) -> tuple[int, int]:
    """Sum over lattice samples of the flops of the program SDFOctree::Eval runs there,
    counted exactly by assigning index boxes of the lattice to octree cells."""
    f = np.float32
    axes = [f(o) + np.arange(n, dtype=np.int64).astype(f) * f(grid.step)
            for o, n in ((grid.x0, grid.sx + 1), (grid.y0, grid.sy + 1), (grid.z0, grid.sz + 1))]
    flops_of = [program_flops(words[int(c[11]): int(c[11]) + int(c[12])]) for c in cells]
    total_flops = 0
    total_samples = 0
    stack = [(0, (0, axes[0].size), (0, axes[1].size), (0, axes[2].size))]
    while stack:
        node, bx, by, bz = stack.pop()
        size = (bx[1] - bx[0]) * (by[1] - by[0]) * (bz[1] - bz[0])
        if size <= 0:
            continue
        own = size
        if cells[node][9] == 0:
            piv = cells[node][:3]
            splits = [int(np.searchsorted(axes[a], f(piv[a]), side="right")) for a in range(3)]
            for octant in range(8):
                child = int(children[node][octant])
                if child < 0:
                    continue
                box = []
                for a, b in enumerate((bx, by, bz)):
                    hi_side = (octant >> a) & 1
                    lo, hi = (max(b[0], splits[a]), b[1]) if hi_side else (b[0], min(b[1], splits[a]))
                    box.append((lo, hi))
                csize = max(0, box[0][1] - box[0][0]) * max(0, box[1][1] - box[1][0]) * max(0, box[2][1] - box[2][0])
                own -= csize
                stack.append((child, box[0], box[1], box[2]))
        total_flops += own * flops_of[node]
        total_samples += own
    return total_flops, total_samples


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id: str | None):
        self.proc = None
        self.lines: list[str] = []
        self.device_id = device_id

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.device_id:
            cmd += ["-i", self.device_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except json.JSONDecodeError:
            return {}
    return {}


def committed_traffic(kernel: str):
    """Per-launch DRAM bytes (read + write) of a kernel from the committed ncu summaries:
    lines `traffic <kernel>: <bytes> bytes per launch`."""
    import re
    for p in sorted((ROOT / "profiles").glob("*.md")):
        for line in p.read_text().splitlines():
            m = re.match(r"^traffic (\w+): (\d+) bytes per launch", line.strip())
            if m and m.group(1) == kernel:
                return {"bytes_per_launch": int(m.group(2)), "source": f"profiles/{p.name}"}
    return None


def cost_lattice(cells, children, words, grid):
    """int32 lattice (z, y, x) of the flops of the program SDFOctree::Eval runs at each
    lattice point: each octree cell's program over its index box, children overriding."""
    f = np.float32
    axes = [f(o) + np.arange(n, dtype=np.int64).astype(f) * f(grid.step)
            for o, n in ((grid.x0, grid.sx + 1), (grid.y0, grid.sy + 1), (grid.z0, grid.sz + 1))]
    flops_of = [program_flops(words[int(c[11]): int(c[11]) + int(c[12])]) for c in cells]
    cost = np.zeros((axes[2].size, axes[1].size, axes[0].size), np.int32)
    stack = [(0, (0, axes[0].size), (0, axes[1].size), (0, axes[2].size))]
    while stack:
        node, bx, by, bz = stack.pop()
        if bx[1] <= bx[0] or by[1] <= by[0] or bz[1] <= bz[0]:
            continue
        cost[bz[0]:bz[1], by[0]:by[1], bx[0]:bx[1]] = flops_of[node]
        if cells[node][9] != 0:
            continue
        piv = cells[node][:3]
        splits = [int(np.searchsorted(axes[a], f(piv[a]), side="right")) for a in range(3)]
        for octant in range(8):
            child = int(children[node][octant])
            if child < 0:
                continue
            box = []
            for a, b in enumerate((bx, by, bz)):
                lo, hi = (max(b[0], splits[a]), b[1]) if (octant >> a) & 1 else (b[0], min(b[1], splits[a]))
                box.append((lo, hi))
            stack.append((child, box[0], box[1], box[2]))
    return cost


def brick_flops(cost, grid, bricks, B):
    """(flops, lattice points) over the union of the kept bricks' lattice boxes."""
    nx, ny, nz = grid.sx + 1, grid.sy + 1, grid.sz + 1
    nbx, nby = (grid.sx + B - 1) // B, (grid.sy + B - 1) // B
    mask = np.zeros((nz, ny, nx), bool)
    for b in bricks.tolist():
        bx, by, bz = b % nbx, (b // nbx) % nby, b // (nbx * nby)
        i0, j0, k0 = bx * B, by * B, bz * B
        mask[k0:min(k0 + B, nz - 1) + 1, j0:min(j0 + B, ny - 1) + 1, i0:min(i0 + B, nx - 1) + 1] = True
    return int(cost[mask].sum(dtype=np.int64)), int(mask.sum())


def cpu_checker(prefer_reference=True):
    """(library, kind): Tangerine's own CPU code built from its sources (oracle/_ref) where
    it loads -- the x86 container that holds the sources -- else the C restatement in
    oracle/port, which builds on any host (the GPU host has no reference sources, and x86
    binaries do not run on its Arm cores)."""
    from oracle import oracle as O
    if prefer_reference:
        try:
            ref = O.reference() if O.REF_SO.exists() else None
            if ref is not None:
                return ref, "reference"
        except OSError:
            pass
    return O.port(), "port"


def slab_bounds(sz: int, parts: int):
    """`parts` contiguous z-ranges of cells [k0, k1) that partition the lattice's sz cells."""
    edges = [round(i * sz / parts) for i in range(parts + 1)]
    return [(edges[i], edges[i + 1]) for i in range(parts) if edges[i + 1] > edges[i]]


def cpu_export_slab(cpu, kind, o, grid, k0, k1, threads):
    """Tangerine's CPU export of cells with k0 <= k < k1 (all x, y) on all host threads:
    the surface-nets cell and face passes as the reference runs them (8 corner evaluations
    per cell, 6 per face check, through SDFOctree::Eval) and per-vertex Gradient +
    GetMaterial.  Returns (seconds, lattice samples the slab owns, vertices)."""
    from tangerine_gb300 import workloads as W
    z0 = float(np.float32(grid.z0) + np.float32(k0) * np.float32(grid.step))
    g = W.ExportGrid(grid.x0, grid.y0, z0, grid.step, grid.sx, grid.sy, k1 - k0)
    t = time.perf_counter()
    if kind == "reference":
        m = cpu.surface_nets(o, g, threads=0)
        cpu.vertex_attributes(o, m.vertices, threads=0)
    else:
        m = cpu.surface_nets(o, g, threads=threads, faithful=True)
        cpu.vertex_attributes(o, m.vertices, threads=threads)
    dt = time.perf_counter() - t
    owned = (grid.sx + 1) * (grid.sy + 1) * ((k1 - k0) + (1 if k1 == grid.sz else 0))
    return dt, owned, m.vertices.shape[0]


def cpu_full_export(spec, grid, parts=20, prefer_reference=True, max_seconds=None):
    """The whole export on the host cores, slab after slab: every one of the lattice's
    samples is owned by exactly one slab.  The face pass skips each slab's first cell layer
    (its neighbours below lie in the slab before), about 1/26 of the face checks at 20
    slabs: the CPU side is timed slightly in its favour.  With max_seconds, slabs spread
    over the whole z range (bit-reversed order) run until that much time is spent, and the
    rate is that of the slabs run (labelled in `sample`)."""
    cpu, kind = cpu_checker(prefer_reference)
    threads = cpu.hardware_threads()
    h = cpu.build(spec)
    o = cpu.octree(h)
    try:
        slabs = slab_bounds(grid.sz, parts)
        bits = max(1, (len(slabs) - 1).bit_length())
        order = sorted(range(len(slabs)), key=lambda i: int(format(i, f"0{bits}b")[::-1], 2))
        secs, samples, done = 0.0, 0, 0
        for i in order:
            k0, k1 = slabs[i]
            dt, owned, _ = cpu_export_slab(cpu, kind, o, grid, k0, k1, threads)
            secs += dt
            samples += owned
            done += 1
            if max_seconds is not None and secs >= max_seconds:
                break
        whole = done == len(slabs)
        what = (f"the whole {grid.sx - 2}^3 export ({samples} lattice samples) in {parts} z-slabs" if whole else
                f"{done} of {len(slabs)} z-slabs spread over the {grid.sx - 2}^3 export ({samples} lattice samples)")
        return {"value": samples / secs, "unit": "samples/s", "cores": threads, "kind": kind, "seconds": secs,
                "sample": f"{what}, {secs:.1f} s: " + CPU_KIND_TEXT[kind]}
    finally:
        cpu.octree_free(o)
        cpu.free(h)


CPU_KIND_TEXT = {
    "reference": "Tangerine's own AsyncParallelSurfaceNets thunks on its Pool() threadpool over the SDFOctree "
                 "(surface_nets.cpp:864-1121, threadpool.cpp:27-40), then per-vertex Gradient + GetMaterial on Pool(), "
                 "built from the reference sources",
    "port": "C restatement of the reference export on all host threads (8 corner evaluations per cell and 6 per face "
            "check as the reference's thunks make, then per-vertex gradient + colour); the reference itself cannot run "
            "on this host (its sources are not here, and x86 builds do not run on Arm)",
}


def cpu_baseline(spec, grid, max_seconds=30.0):
    """The cpu_baseline object: the export on the host cores -- whole at 512^3 (about 10 s
    on 16 Grace cores), spread slabs for about max_seconds on larger lattices."""
    return cpu_full_export(spec, grid, parts=max(20, grid.sz // 26), max_seconds=max_seconds)


def reference_arm(args, rank):
    """`--impl reference`: Tangerine's CPU export of the same workload.  The K timed steps
    are the K z-slabs of one partition of the lattice, so together they are one complete
    export, measured slab by slab (nothing extrapolated); the W warm-up steps run slabs of
    a W-way partition first.  value = the lattice's samples / the K steps' summed time."""
    if rank != 0:
        return
    from tangerine_gb300 import workloads as W
    spec = W.random_tree(SEED, PRIMS)
    grid = W.export_grid(resolution=RES)
    cpu, kind = cpu_checker(not args.port)
    threads = cpu.hardware_threads()
    h = cpu.build(spec)
    o = cpu.octree(h)
    try:
        for k0, k1 in slab_bounds(grid.sz, max(args.warmup, 1))[: max(args.warmup, 1)]:
            cpu_export_slab(cpu, kind, o, grid, k0, min(k1, k0 + 8), threads)
        t0 = time.perf_counter()
        step_s, samples, vertices = [], 0, 0
        for k0, k1 in slab_bounds(grid.sz, args.steps):
            dt, owned, nv = cpu_export_slab(cpu, kind, o, grid, k0, k1, threads)
            step_s.append(dt)
            samples += owned
            vertices += nv
        wall = time.perf_counter() - t0
    finally:
        cpu.octree_free(o)
        cpu.free(h)
    assert samples == grid.corners, (samples, grid.corners)
    total = float(np.sum(step_s))
    value = samples / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": args.gpus,
        "steps": len(step_s), "warmup": args.warmup, "ms_per_step": 1e3 * total / len(step_s),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": CONFIG,
        "meshes_per_s": 1.0 / total,
        "vertices": vertices,
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": kind,
                         "sample": f"one whole {RES}^3 export ({samples} lattice samples) as {len(step_s)} z-slab steps, "
                                   f"{total:.1f} s: " + CPU_KIND_TEXT[kind]},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)


def cpu_compare(args):
    """x86 leg (where the reference sources are present): the reference's own CPU export
    and the C restatement over the same whole 512^3 export on the same host threads."""
    from tangerine_gb300 import workloads as W
    spec = W.random_tree(SEED, PRIMS)
    grid = W.export_grid(resolution=args.compare_res)
    ref = cpu_full_export(spec, grid, parts=args.steps, prefer_reference=True)
    if ref["kind"] != "reference":
        print(json.dumps({"workload": "cpu-compare", "unavailable": "the reference library (oracle/_ref) is not built here"}))
        return
    port = cpu_full_export(spec, grid, parts=args.steps, prefer_reference=False)
    print(json.dumps({"workload": "cpu-compare", "resolution": args.compare_res, "threads": ref["cores"],
                      "reference_samples_per_s": ref["value"], "port_samples_per_s": port["value"],
                      "port_over_reference": port["value"] / ref["value"],
                      "reference_seconds": ref["seconds"], "port_seconds": port["seconds"]}), flush=True)


def mesh_difference(a, b):
    """(identical, symmetric Hausdorff distance between the vertex sets)."""
    same = (a.vertices.shape == b.vertices.shape and np.array_equal(a.vertices, b.vertices)
            and np.array_equal(a.faces, b.faces))
    if same:
        return True, 0.0
    from scipy.spatial import cKDTree
    if len(a.vertices) == 0 or len(b.vertices) == 0:
        return False, float("inf")
    d1 = cKDTree(b.vertices).query(a.vertices)[0].max()
    d2 = cKDTree(a.vertices).query(b.vertices)[0].max()
    return False, float(max(d1, d2))


def surrogate_leg(prog, grid, samples, args, stream, sp, flush, exact_ms, dense_ms, world, brick=0, fitted=None,
                  exact_same_ms=None):
    """Trains the network on the program (unless `fitted` is one already trained on it),
    then times the culled export with it deciding which bricks to skip: alone, and with the
    exact test on the bricks it keeps.  exact_ms: the exact-culled export at its best brick
    size; exact_same_ms: the exact-culled export at this leg's brick size, where it differs."""
    import torch
    from tangerine_gb300 import _lib, sdf
    sur = fitted or sdf.Surrogate()
    info = sur.fit(prog) if fitted is None else sur.info()
    exact_mesh = prog.export_mesh(grid, brick=brick)
    out = {"train_seconds": info.train_seconds, "data_seconds": info.data_seconds, "samples": int(info.samples),
           "steps": int(info.steps), "max_error": info.max_error, "p99_error": info.p99_error,
           "mean_error": info.mean_error, "final_loss": info.final_loss, "modes": {}}
    bsize = brick or 7
    out["margin"] = sur.margin(0.8660254 * bsize * grid.step)
    for mode, only in (("network alone", True), ("network + exact test", False)):
        m = sur.export_mesh(prog, grid, brick=brick, only=only)
        same, hausdorff = mesh_difference(m, exact_mesh)
        bricks, kept = sdf.last_export_stats()
        for _ in range(2):
            sur.export_mesh_device(prog, grid, brick=brick, only=only, stream=sp)
        st = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            st[i].record(stream)
            sur.export_mesh_device(prog, grid, brick=brick, only=only, stream=sp)
            en[i].record(stream)
        torch.cuda.synchronize()
        ms = float(np.sum([a.elapsed_time(b) for a, b in zip(st, en)]))
        out["modes"][mode] = {"value": world * samples * args.steps / (ms * 1e-3), "unit": "samples/s",
                              "ms_per_step": ms / args.steps, "bricks_evaluated": kept, "bricks": bricks,
                              "same_mesh_as_exact": same, "hausdorff": hausdorff,
                              "hausdorff_over_bbox_diagonal": hausdorff / (4.0 * 3 ** 0.5),
                              "vs_exact_culled": exact_ms / ms, "vs_dense": dense_ms / ms}
        if exact_same_ms is not None:
            out["modes"][mode]["vs_exact_culled_same_bricks"] = exact_same_ms / ms
    best_mode = max(out["modes"], key=lambda k: out["modes"][k]["value"])
    out["value"] = out["modes"][best_mode]["value"]
    out["unit"] = "samples/s"
    # End to end through the C ABI: tg_export_mesh_surrogate fills a tg_mesh in host memory,
    # which the caller releases with tg_mesh_free.
    only = best_mode == "network alone"
    lib = _lib.load()
    g = sdf._grid(grid)
    flags = sdf._flags(True, False, brick, 0, only)

    def c_export():
        hm = _lib.HostMesh()
        _lib.check(lib.tg_export_mesh_surrogate(prog.ptr, sur.ptr, _lib.C.byref(g), flags, _lib.C.byref(hm),
                                                _lib.C.c_void_p(sp)), "tg_export_mesh_surrogate")
        nv, nf = int(hm.vertex_count), int(hm.face_count)
        nbytes = nv * (12 + 12 + 4 + (3 if hm.colors else 0)) + nf * 12
        lib.tg_mesh_free(_lib.C.byref(hm))
        return nbytes

    reps = max(3, min(args.steps, 10))
    c_export()     # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        d2h = c_export()
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    out["e2e"] = {"value": world * samples * reps / secs, "unit": "samples/s", "h2d_bytes_per_step": 0,
                  "d2h_bytes_per_step": int(d2h), "call": f"tg_export_mesh_surrogate ({best_mode}), host mesh out"}
    if fitted is None:
        sur.close()
    return out


def surrogate_1024_leg(prog, args, stream, sp, flush, world):
    """The surrogate-culled workload inside the default line: the same tree on the 1024^3
    grid -- dense, exact-culled (7^3-cell bricks, its best size, and 32^3) and network-culled
    (network + exact test, and the network alone) in 32^3 bricks, where the network gains
    most over the exact test at the same brick size, and in 7^3 bricks; same mesh required,
    one network trained on the tree.  vs_exact_culled compares with the exact export at its
    best brick size."""
    import torch
    from tangerine_gb300 import sdf
    from tangerine_gb300 import workloads as W
    grid = W.export_grid(resolution=1024)
    samples = grid.corners
    steps = max(2, min(args.steps, 5))

    def timed(fn):
        for _ in range(2):
            fn()
        st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        torch.cuda.synchronize()
        for i in range(steps):
            flush.zero_()
            st[i].record(stream)
            fn()
            en[i].record(stream)
        torch.cuda.synchronize()
        return float(np.sum([a.elapsed_time(b) for a, b in zip(st, en)]))

    dense_ms = timed(lambda: prog.export_mesh_device(grid, dense=True, stream=sp))
    exact_ms = timed(lambda: prog.export_mesh_device(grid, stream=sp))
    _, exact_kept = sdf.last_export_stats()
    exact32_ms = timed(lambda: prog.export_mesh_device(grid, brick=32, stream=sp))
    _, exact32_kept = sdf.last_export_stats()
    sub = argparse.Namespace(steps=steps, warmup=2)
    net = sdf.Surrogate()
    net.fit(prog)
    sur = surrogate_leg(prog, grid, samples, sub, stream, sp, flush, exact_ms, dense_ms, world, brick=32, fitted=net,
                        exact_same_ms=exact32_ms)
    sur["bricks_7"] = surrogate_leg(prog, grid, samples, sub, stream, sp, flush, exact_ms, dense_ms, world, brick=7,
                                    fitted=net)["modes"]
    net.close()
    sur["workload"] = (f"the same tree on a 1024^3 grid over [-2,2]^3 ({samples} lattice samples); network: 16-level "
                       f"hash grid + 3x64 BF16 layers trained on 2^22 exact samples; modes in 32^3-cell bricks, "
                       f"bricks_7 in 7^3-cell bricks")
    sur["exact_culled"] = {"value": world * samples * steps / (exact_ms * 1e-3), "ms_per_step": exact_ms / steps,
                           "bricks_evaluated": exact_kept, "brick_cells": 7}
    sur["exact_culled_32"] = {"value": world * samples * steps / (exact32_ms * 1e-3), "ms_per_step": exact32_ms / steps,
                              "bricks_evaluated": exact32_kept, "brick_cells": 32}
    sur["dense"] = {"value": world * samples * steps / (dense_ms * 1e-3), "ms_per_step": dense_ms / steps}
    sur["steps"] = steps
    return sur


def our_arm(args, rank, world, local_rank):
    import torch
    from tangerine_gb300 import build as B
    B.build()
    from tangerine_gb300 import _lib, sdf
    from tangerine_gb300 import workloads as W

    torch.cuda.set_device(local_rank)
    from tangerine_gb300.replicas import Replicas
    group = Replicas(world, rank)

    def barrier():
        group.barrier()

    spec = W.random_tree(SEED, PRIMS)
    grid = W.export_grid(resolution=RES)
    samples = grid.corners
    tree = sdf.from_spec(spec)
    prog = sdf.compile(tree)
    info = prog.info()
    # One non-default stream for everything: the L2 flush, the CUDA events and the
    # library's work (a null stream would send the library to its own stream, where the
    # flush and the events would not be ordered with the work they bracket).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    lib = _lib.load()

    # Warm-up (allocates the engine's buffers).
    dm = None
    for _ in range(args.warmup):
        dm = prog.export_mesh_device(grid, stream=sp)
        prog.export_mesh_device(grid, dense=True, stream=sp)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # Timed region: K exports, L2 flushed between them outside the per-step events.
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sdf.profile_reset()
    sdf.profile_enable(True)
    dev_uuid = None
    try:
        dev_uuid = str(torch.cuda.get_device_properties(local_rank).uuid)
        dev_uuid = dev_uuid if dev_uuid.startswith("GPU-") else "GPU-" + dev_uuid
    except Exception:
        dev_uuid = None
    torch.cuda.synchronize()
    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(dev_uuid) as clocks:
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            dm = prog.export_mesh_device(grid, stream=sp)
            ends[i].record(stream)
        torch.cuda.synchronize()
        barrier()
    wall = time.perf_counter() - wall0
    sdf.profile_enable(False)
    bricks, active_bricks = sdf.last_export_stats()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(np.sum(step_ms))
    total_ms = group.max(total_ms)
    kernels = {}
    for name in ("classify_bricks", "list_bricks", "eval_bricks", "cell_flags", "scan", "cell_vertices", "faces", "attributes"):
        ms, n = sdf.profile_read(name)
        kernels[name] = {"ms_per_step": ms / args.steps, "launches": n}
    vertex_count, face_count = int(dm.vertex_count), int(dm.face_count)

    # The dense form (every lattice point evaluated, as the reference does), same mesh.
    sdf.profile_reset()
    sdf.profile_enable(True)
    dstarts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    dends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        dstarts[i].record(stream)
        prog.export_mesh_device(grid, dense=True, stream=sp)
        dends[i].record(stream)
    torch.cuda.synchronize()
    sdf.profile_enable(False)
    dense_ms = float(np.sum([s.elapsed_time(e) for s, e in zip(dstarts, dends)]))
    eval_grid_ms = sdf.profile_read("eval_grid")[0] / args.steps

    value = world * samples * args.steps / (total_ms * 1e-3)
    # Launches of our kernels per step: classify, brick list (scan 3 + compaction), brick
    # evaluation with the cell pass, scan (3), vertices, scan (3), faces, normals, colours.
    launches_per_step = 16

    # The surrogate-culled form: the network trained on this tree decides which bricks to
    # skip (alone, or followed by the exact test); same mesh required.
    surrogate = None if args.skip_surrogate else surrogate_leg(prog, grid, samples, args, stream, sp, flush, total_ms, dense_ms,
                                                                world)
    surrogate_1024 = None if args.skip_surrogate else surrogate_1024_leg(prog, args, stream, sp, flush, world)

    # End to end through the C ABI: tree handle in, host mesh out, every step.
    # About 2 ms a call: 50 calls keep one slow call (the host is shared) from moving the mean much.
    e2e_steps = 0 if args.skip_e2e else max(3, min(5 * args.steps, 50))
    e2e = None
    if e2e_steps:
        lo = np.array([-2, -2, -2], np.float32)
        hi = np.array([2, 2, 2], np.float32)
        # The C ABI call itself: tg_export_tree fills a tg_mesh in host memory, which the
        # caller releases with tg_mesh_free.
        def c_export():
            hm = _lib.HostMesh()
            _lib.check(lib.tg_export_tree(tree.handle, _lib.as_ptr(lo), _lib.as_ptr(hi), float(4.0 / RES),
                                          _lib.C.byref(hm), _lib.C.c_void_p(sp)), "tg_export_tree")
            counts = (int(hm.vertex_count), int(hm.face_count), bool(hm.colors))
            lib.tg_mesh_free(_lib.C.byref(hm))
            return counts
        for _ in range(3):
            c_export()     # warm
        torch.cuda.synchronize()
        barrier()
        calls = []
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            tc = time.perf_counter()
            nv, nf, has_colors = c_export()
            calls.append(time.perf_counter() - tc)
        torch.cuda.synchronize()
        barrier()
        e2e_s = time.perf_counter() - t0
        calls.sort()
        e2e_s = group.max(e2e_s)
        prog_bytes = info.octree_cells * 64 + info.code_quads * 16 + info.materials * 4
        d2h = nv * (12 + 12 + 4 + (3 if has_colors else 0)) + nf * 12
        phases = sdf.last_export_timing()
        oct_s, comp_s = _lib.C.c_double(), _lib.C.c_double()
        lib.tg_debug_compile_seconds(tree.handle, 0, _lib.C.byref(oct_s), _lib.C.byref(comp_s))
        e2e = {"value": world * samples * e2e_steps / e2e_s, "unit": "samples/s",
               "last_call_phases_s": {"octree_compile": phases[0], "upload": phases[1], "gpu_export": phases[2],
                                      "copy_to_host": phases[3]},
               "host_compile_split_s": {"octree": oct_s.value, "programs": comp_s.value - oct_s.value},
               "h2d_bytes_per_step": int(prog_bytes), "d2h_bytes_per_step": int(d2h),
               "meshes_per_s": world * e2e_steps / e2e_s,
               "calls": e2e_steps, "median_call_ms": calls[len(calls) // 2] * 1e3, "slowest_call_ms": calls[-1] * 1e3,
               "call": "tg_export_tree (octree build + compile, the GPU testing bricks on the root cell's program meanwhile; upload + rest of the GPU export + copy to host)"}

    # Roofline of the dominant kernel of the timed export (the distance interpreter on the
    # kept bricks): exact algorithmic flops over the lattice points of those bricks.
    cells, children, words = tree.debug_octree()
    flops, counted = algorithmic_flops(cells, children, words, grid)
    assert counted == samples, (counted, samples)
    prog.export_mesh_device(grid, stream=sp)
    kept_list, bsize = sdf.last_export_bricks()
    cost = cost_lattice(cells, children, words, grid)
    assert int(cost.sum(dtype=np.int64)) == flops
    brick_fl, brick_points = brick_flops(cost, grid, kept_list, bsize)
    del cost
    eval_bricks_ms = kernels["eval_bricks"]["ms_per_step"]
    fp32 = _lib.C.c_double()
    _lib.check(lib.tg_measure_fp32_peak(_lib.C.byref(fp32), sp), "fp32 peak")
    achieved = brick_fl / (eval_bricks_ms * 1e-3) / 1e12
    traffic = committed_traffic("EvalBricksCellsKernel")
    dense_achieved = flops / (eval_grid_ms * 1e-3) / 1e12
    roofline = {"bound": "fp32", "achieved": achieved, "peak": fp32.value, "unit": "TFLOP/s",
                "frac": achieved / fp32.value, "traffic": traffic["bytes_per_launch"] if traffic else None,
                "traffic_source": traffic["source"] if traffic else None,
                "kernel": "EvalBricksCellsKernel (distance interpreter on the kept bricks of the timed export, with the "
                          "cell pass on each brick's values in shared memory folded in; its time counts both)",
                "flops_per_launch": brick_fl, "lattice_points_per_launch": brick_points,
                "algorithmic_bytes_per_launch": 4 * brick_points,
                "peak_source": "measured in this run: FFMA throughput probe (tg_measure_fp32_peak), of measured",
                "note": "kernels are built with -fmad=false for bit-exact parity, so every mul and add issues "
                        "separately: half the FFMA flop rate is the arithmetic ceiling",
                "hbm": {"achieved_gbs": 4 * brick_points / (eval_bricks_ms * 1e-3) / 1e9,
                        "peak_gbs": measured_peaks().get("hbm_gbs", 6800.0)},
                "dense_interpreter": {"kernel": "EvalGridKernel (every lattice point, dense export)",
                                      "flops_per_launch": flops, "ms": eval_grid_ms, "achieved_tflops": dense_achieved,
                                      "frac": dense_achieved / fp32.value}}

    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cb = cpu_baseline(spec, grid)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": CONFIG,
            "mesh": {"vertices": vertex_count, "faces": face_count, "octree_cells": info.octree_cells},
            "meshes_per_s": world * args.steps / (total_ms * 1e-3),
            "bricks": {"size_cells": 7, "total": bricks, "evaluated": active_bricks,
                       "evaluated_fraction": active_bricks / max(1, bricks)},
            "surrogate_culled": surrogate,
            "surrogate_culled_1024": surrogate_1024,
            "dense_export": {"value": world * samples * args.steps / (dense_ms * 1e-3), "unit": "samples/s",
                             "ms_per_step": dense_ms / args.steps, "eval_grid_ms": eval_grid_ms,
                             "note": "every lattice point evaluated (the reference's work); identical mesh"},
            "kernels_ms_per_step": {k: v["ms_per_step"] for k, v in kernels.items()},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks.summary(),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    prog.close()
    group.close()


def render_arm(args, rank, world, local_rank):
    """Sphere-traced depth + normal + colour, 64 seeded poses at radius 4 around a
    1024-primitive tree, 1920x1080, 256 steps, epsilon 1e-4, 60 degree vertical FOV."""
    import torch
    from tangerine_gb300 import build as B
    B.build()
    from tangerine_gb300 import _lib, sdf
    from tangerine_gb300 import workloads as W
    torch.cuda.set_device(local_rank)
    width, height, poses_n, steps, eps = 1920, 1080, 64, 256, 1e-4
    spec = W.random_tree(5, 1024)
    tree = sdf.from_spec(spec)
    prog = sdf.compile(tree)
    poses = W.camera_poses(5, poses_n, radius=4.0)
    cams = sdf.cameras(poses, fov_y_degrees=60.0)
    lib = _lib.load()
    # One non-default stream for everything: the L2 flush, the CUDA events and the
    # library's work (a null stream would send the library to its own stream, where the
    # flush and the events would not be ordered with the work they bracket).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    px = width * height
    depth = torch.empty(poses_n * px, dtype=torch.float32, device="cuda")
    normals = torch.empty(poses_n * px * 3, dtype=torch.float32, device="cuda")
    colors = torch.empty(poses_n * px * 3, dtype=torch.uint8, device="cuda")

    def render(count, exact, cam_array):
        _lib.check(lib.tg_render(prog.ptr, cam_array, count, width, height, steps, eps, 1 if exact else 0,
                                 _lib.C.c_void_p(depth.data_ptr()), _lib.C.c_void_p(normals.data_ptr()),
                                 _lib.C.c_void_p(colors.data_ptr()), 1, _lib.C.c_void_p(sp)), "tg_render")

    for _ in range(args.warmup):
        render(4, False, cams)
    sdf.profile_reset()
    sdf.profile_enable(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        render(poses_n, False, cams)
    ev1.record(stream)
    torch.cuda.synchronize()
    sdf.profile_enable(False)
    ms = ev0.elapsed_time(ev1) / args.steps
    hits = float(torch.isfinite(depth).float().mean().item())
    rays = poses_n * px
    # Exact (reference step sequence on the whole tree) on two poses.
    exact_cams = sdf.cameras(poses[:2], fov_y_degrees=60.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    render(2, True, exact_cams)
    e1.record(stream)
    torch.cuda.synchronize()
    exact_rays_s = 2 * px / (e0.elapsed_time(e1) * 1e-3)
    exact_depth = depth[:2 * px].clone()
    # Network steps with exact final steps, all poses; agreement with the exact tracer on the
    # first two.
    network = None
    if not args.skip_surrogate:
        sur = sdf.Surrogate()
        t0 = time.perf_counter()
        sinfo = sur.fit(prog)
        fit_s = time.perf_counter() - t0

        def render_net(n, cam_array):
            _lib.check(lib.tg_render_surrogate(prog.ptr, sur.ptr, cam_array, n, width, height, steps, eps,
                                               _lib.C.c_void_p(depth.data_ptr()), _lib.C.c_void_p(normals.data_ptr()),
                                               _lib.C.c_void_p(colors.data_ptr()), 1, _lib.C.c_void_p(sp)), "tg_render_surrogate")

        render_net(2, exact_cams)
        torch.cuda.synchronize()
        net_depth = depth[:2 * px]
        he, hn = torch.isfinite(exact_depth), torch.isfinite(net_depth)
        both = he & hn
        agree = float((he == hn).float().mean().item())
        dd = (exact_depth[both] - net_depth[both]).abs()
        max_dd = float(dd.max().item()) if bool(both.any()) else 0.0
        far = int((dd > 2e-3).sum().item())
        n0, n1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0.record(stream)
        render_net(poses_n, cams)
        n1.record(stream)
        torch.cuda.synchronize()
        net_ms = n0.elapsed_time(n1)
        ns, es = sdf.last_render_steps()
        network = {"rays_per_s": rays / (net_ms * 1e-3), "ms_all_poses": net_ms, "fit_seconds": fit_s,
                   "held_out_max_error": sinfo.max_error, "step_margin": sinfo.margin,
                   "network_iterations_per_ray": ns / rays, "exact_steps_per_ray": es / rays,
                   "vs_exact_only": (rays / (net_ms * 1e-3)) / exact_rays_s,
                   "hit_agreement_with_exact": agree, "max_depth_difference": max_dd,
                   "rays_both_hit_depth_over_2e-3": far, "rays_compared": 2 * px,
                   "note": "network step bounds (tcgen05 network per lockstep iteration) then exact whole-tree steps; "
                           "every hit is the exact program's"}
        sur.close()
    # End to end: host buffers, all poses.
    hd = np.empty(rays, np.float32)
    hn = np.empty(rays * 3, np.float32)
    hc = np.empty(rays * 3, np.uint8)
    t = time.perf_counter()
    _lib.check(lib.tg_render(prog.ptr, cams, poses_n, width, height, steps, eps, 0, _lib.as_ptr(hd), _lib.as_ptr(hn),
                             _lib.as_ptr(hc), 0, _lib.C.c_void_p(sp)), "tg_render")
    e2e_s = time.perf_counter() - t
    cpu = None
    if not args.skip_cpu:
        from oracle import oracle as O
        port = O.port()
        h = port.build(spec)
        try:
            stride = 41
            o, d = W.camera_rays(poses[0], width, height, cams[0].tan_half_fov)
            idx = np.arange(px)[::stride]
            o, d = np.ascontiguousarray(o[idx]), np.ascontiguousarray(d[idx])
            t = time.perf_counter()
            hit, travel, pos = port.raymarch(h, o, d, steps, eps, threads=0)
            if hit.any():
                port.gradient(h, pos[hit])
                port.color(h, pos[hit])
            secs = time.perf_counter() - t
            cpu = {"value": len(idx) / secs, "unit": "rays/s", "cores": port.hardware_threads(), "kind": "port",
                   "sample": f"every {stride}th pixel of pose 0 ({len(idx)} rays, {secs:.1f} s): SDFNode::RayMarch + "
                             f"Gradient + GetMaterial on the whole tree, C restatement"}
        finally:
            port.free(h)
    line = {"metric": "rays/s: sphere-traced depth+normal+colour (1024-primitive tree, 64 poses, 1920x1080)",
            "value": rays / (ms * 1e-3), "unit": "rays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "render: seeded 1024-primitive tree (seed 5), 64 seeded poses on a radius-4 sphere, "
                                   "1920x1080, 60 deg vertical FOV, 256 steps, epsilon 1e-4, octree-bounded steps",
                       "hit_fraction": hits},
            "exact_rays_per_s": exact_rays_s,
            "network_steps": network,
            "e2e": {"value": rays / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": rays * 19},
            "cpu_baseline": cpu, "gpu_launches": args.steps}
    if rank == 0:
        print(json.dumps(line), flush=True)
    prog.close()


def batch_arm(args, rank, world, local_rank):
    """512 seeded trees (primitives log-uniform in [4, 1024], grids uniform over
    {64, 128, 192, 256, 384}^3) exported together by one persistent launch replayed from a
    CUDA graph, per-class brick size and lanes from the autotuner; samples/s and meshes/s."""
    import concurrent.futures as cf
    import torch
    from tangerine_gb300 import build as B
    B.build()
    from tangerine_gb300 import sdf
    from tangerine_gb300 import workloads as W
    torch.cuda.set_device(local_rank)
    count = args.batch_models
    models = W.batch_workload(SEED, count, valid=lambda spec: sdf.has_export_octree(sdf.from_spec(spec)))

    def make(item):
        seed, prims, res = item
        return sdf.compile(sdf.from_spec(W.random_tree(seed, prims))), W.export_grid(resolution=res)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 8) as ex:
        built = list(ex.map(make, models))
    compile_s = time.perf_counter() - t0
    progs = [p for p, _ in built]
    grids = [g for _, g in built]
    samples = int(sum(g.corners for g in grids))
    # One non-default stream for everything: the L2 flush, the CUDA events and the
    # library's work (a null stream would send the library to its own stream, where the
    # flush and the events would not be ordered with the work they bracket).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    batch = sdf.Batch(progs, grids)
    t0 = time.perf_counter()
    batch.autotune(stream=sp)
    tune_s = time.perf_counter() - t0
    bricks, lanes = batch.tuning()
    for _ in range(max(1, args.warmup)):
        batch.run(stream=sp)

    def timed(fn, steps):
        st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        torch.cuda.synchronize()
        for i in range(steps):
            flush.zero_()
            st[i].record(stream)
            fn()
            en[i].record(stream)
        torch.cuda.synchronize()
        return float(np.sum([a.elapsed_time(b) for a, b in zip(st, en)]))

    with ClockSampler(None) as clocks:
        ms = timed(lambda: batch.run(stream=sp), args.steps)
    info = batch.info()
    # The same models one export call each (the single-model pipeline, same tuning).
    def sequential():
        for p, g, b, l in zip(progs, grids, bricks, lanes):
            p.export_mesh_device(g, brick=int(b), lanes=int(l), stream=sp)
    seq_ms = timed(sequential, 1)
    # End to end: the batch run plus every mesh copied to host memory.
    t0 = time.perf_counter()
    e2e_steps = 2
    d2h = 0
    for _ in range(e2e_steps):
        batch.run(stream=sp)
        d2h = 0
        for m in range(count):
            mesh = batch.mesh(m, stream=sp)
            d2h += mesh.vertices.nbytes + mesh.normals.nbytes + mesh.faces.nbytes + mesh.cubes.nbytes + \
                (mesh.colors.nbytes if mesh.colors is not None else 0)
    e2e_s = time.perf_counter() - t0
    # The surrogate form: a learned bound per large model culls its bricks inside the same
    # graph, the kept bricks also take the exact test; every mesh must stay the exact one.
    surrogate = None
    if not args.skip_surrogate:
        large = [m for m in range(count) if models[m][1] >= 256 and models[m][2] >= 256]
        exact_meshes = {m: batch.mesh(m, stream=sp) for m in large}
        t0 = time.perf_counter()
        nets = [None] * count
        for m in large:
            nets[m] = sdf.Surrogate(samples=1 << 20, steps=600, batch=1 << 16, validation=1 << 18)
            nets[m].fit(progs[m])
        fit_s = time.perf_counter() - t0
        batch.set_surrogates(nets, only=False)
        for _ in range(max(1, args.warmup)):
            batch.run(stream=sp)
        sur_ms = timed(lambda: batch.run(stream=sp), args.steps)
        sinfo = batch.info()
        same = all(np.array_equal(batch.mesh(m, stream=sp).vertices, exact_meshes[m].vertices) and
                   np.array_equal(batch.mesh(m, stream=sp).faces, exact_meshes[m].faces) for m in large)
        surrogate = {"value": samples * args.steps / (sur_ms * 1e-3), "ms_per_step": sur_ms / args.steps,
                     "vs_exact_batch": ms / sur_ms, "models_with_network": len(large), "fit_seconds_total": fit_s,
                     "bricks_evaluated": sinfo.bricks_evaluated, "same_meshes_as_exact": bool(same),
                     "note": "a 16-level hash grid + 3x64 BF16 network per model with >= 256 primitives on a >= 256^3 grid "
                             "(600 Adam steps each), network bits written before the persistent launch, kept bricks "
                             "re-tested exactly"}
        batch.set_surrogates([None] * count)
        for n in nets:
            if n is not None:
                n.close()
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        big = max(range(count), key=lambda m: models[m][1] * models[m][2] ** 2)
        cb = cpu_baseline(W.random_tree(models[big][0], models[big][1]), grids[big])
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        cpu["sample"] = f"model {big} ({models[big][1]} primitives, {models[big][2]}^3): " + cpu["sample"]
    hist = {}
    for b, l in zip(bricks, lanes):
        hist[f"{b}x{l}"] = hist.get(f"{b}x{l}", 0) + 1
    line = {"metric": f"samples/s & meshes/s: {count} trees exported in one persistent launch",
            "value": samples * args.steps / (ms * 1e-3), "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{count} seeded CSG trees (seed {SEED}; a tree left empty by its set operations is "
                                   f"replaced by its sequence's next seed), primitives log-uniform in [4, 1024], grids "
                                   f"uniform over {{64,128,192,256,384}}^3 over [-2,2]^3; exact export with normals + colours; "
                                   f"one cooperative launch per step replayed from a CUDA graph",
                       "samples_per_step": samples, "l2": "flushed between steps"},
            "meshes_per_s": count * args.steps / (ms * 1e-3),
            "batch": {"bricks": info.bricks, "bricks_evaluated": info.bricks_evaluated, "vertices": info.vertices,
                      "faces": info.faces, "graph": info.graph, "blocks": info.blocks, "reruns": info.reruns,
                      "device_gb": info.device_bytes / 1e9, "autotune_seconds": tune_s, "compile_seconds": compile_s,
                      "tuning_histogram_brick_x_lanes": hist},
            "sequential_exports": {"ms_per_step": seq_ms, "value": samples / (seq_ms * 1e-3),
                                   "note": "same models, one tg_export_mesh_device call each"},
            "surrogate_form": surrogate,
            "cpu_baseline": cpu,
            "e2e": {"value": samples * e2e_steps / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(d2h), "call": "tg_batch_run + tg_batch_mesh for every model"},
            "gpu_launches": args.steps, "clocks": clocks.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    batch.close()
    for p in progs:
        p.close()


def surrogate_arm(args, rank, world, local_rank):
    """The 256-primitive tree on a 1024^3 grid in 32^3 bricks: dense exact, exact-culled (at
    its best brick size, 7^3 cells, and at 32^3) and surrogate-culled exports (same mesh),
    samples/s."""
    import torch
    from tangerine_gb300 import build as B
    B.build()
    from tangerine_gb300 import sdf
    from tangerine_gb300 import workloads as W
    torch.cuda.set_device(local_rank)
    res, brick = 1024, 32
    spec = W.random_tree(SEED, PRIMS)
    grid = W.export_grid(resolution=res)
    samples = grid.corners
    prog = sdf.compile(sdf.from_spec(spec))
    # One non-default stream for everything: the L2 flush, the CUDA events and the
    # library's work (a null stream would send the library to its own stream, where the
    # flush and the events would not be ordered with the work they bracket).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        st = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            st[i].record(stream)
            fn()
            en[i].record(stream)
        torch.cuda.synchronize()
        return float(np.sum([a.elapsed_time(b) for a, b in zip(st, en)]))

    dense_ms = timed(lambda: prog.export_mesh_device(grid, dense=True, stream=sp))
    # The exact export at its best brick size (7^3 cells) is what the network must beat;
    # the same-brick exact export is reported beside it.
    best_exact_ms = timed(lambda: prog.export_mesh_device(grid, stream=sp))
    _, best_exact_kept = sdf.last_export_stats()
    exact_ms = timed(lambda: prog.export_mesh_device(grid, brick=brick, stream=sp))
    _, exact_kept = sdf.last_export_stats()
    with ClockSampler(None) as clocks:
        sur = surrogate_leg(prog, grid, samples, args, stream, sp, flush, best_exact_ms, dense_ms, world, brick=brick,
                            exact_same_ms=exact_ms)
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cb = cpu_baseline(spec, grid)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    best_mode = max(sur["modes"], key=lambda k: sur["modes"][k]["value"])
    best = sur["modes"][best_mode]
    ms = best["ms_per_step"]
    line = {"metric": f"samples/s: surrogate-culled export, {PRIMS}-primitive tree, {res}^3 grid in {brick}^3 bricks (same mesh)",
            "value": best["value"], "unit": "samples/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"seeded {PRIMS}-primitive tree (seed {SEED}), {res}^3 grid over [-2,2]^3 "
                                   f"({res + 3}^3 lattice samples) in {brick}^3-cell bricks; network: 16-level hash grid "
                                   f"+ 3x64 BF16 layers trained on 2^22 exact samples (half uniform, half |d|<0.05); "
                                   f"mode: {best_mode}",
                       "l2": "flushed between steps"},
            "meshes_per_s": 1e3 / ms,
            "exact_culled": {"value": world * samples * args.steps / (best_exact_ms * 1e-3),
                             "ms_per_step": best_exact_ms / args.steps, "bricks_evaluated": best_exact_kept, "brick_cells": 7},
            "exact_culled_same_bricks": {"value": world * samples * args.steps / (exact_ms * 1e-3),
                                         "ms_per_step": exact_ms / args.steps, "bricks_evaluated": exact_kept,
                                         "brick_cells": brick},
            "dense_exact": {"value": world * samples * args.steps / (dense_ms * 1e-3), "ms_per_step": dense_ms / args.steps},
            "surrogate": sur, "cpu_baseline": cpu,
            "e2e": sur["e2e"], "gpu_launches": (16 if best_mode == "network alone" else 21) * args.steps,
            "clocks": clocks.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    prog.close()


def exports_arm(args, rank, world, local_rank):
    """The exports beside the mesh export on the 256-primitive tree: Sodapop's meshing job
    at its density 20, the point-cloud export at 0.01-unit voxels with 5 refinement steps,
    and the MagicaVoxel export at 64 voxels per unit; each against the C restatement."""
    import torch
    from tangerine_gb300 import build as B
    B.build()
    from tangerine_gb300 import sdf
    from tangerine_gb300 import workloads as W
    torch.cuda.set_device(local_rank)
    spec = W.random_tree(SEED, PRIMS)
    tree = sdf.from_spec(spec)
    prog = sdf.compile(tree)
    info = prog.info()
    lo = np.array(info.bounds_min[:], np.float32)
    hi = np.array(info.bounds_max[:], np.float32)
    density, cloud_step, refine, vox_grid = 20.0, 0.01, 5, 64.0
    kernels = {"soda": ("soda_lattice", "soda_cache", "soda_flags", "scan", "soda_vertices", "soda_faces", "soda_attributes"),
               "cloud": ("cloud_flags", "list_cells", "cloud_refine", "attributes"),
               "vox": ("vox_flags", "list_cells")}

    def timed(fn, names):
        for _ in range(max(1, args.warmup)):
            fn()
        sdf.profile_reset()
        sdf.profile_enable(True)
        t = time.perf_counter()
        for _ in range(args.steps):
            out = fn()
        wall = (time.perf_counter() - t) / args.steps
        sdf.profile_enable(False)
        kms = {k: sdf.profile_read(k)[0] / args.steps for k in names}
        return out, wall, kms

    with ClockSampler(None) as clocks:
        d, soda_wall, soda_k = timed(lambda: tree.sodapop_mesh(density), kernels["soda"])
        cloud, cloud_wall, cloud_k = timed(lambda: prog.export_point_cloud(lo, hi, cloud_step, refine), kernels["cloud"])
        vox, vox_wall, vox_k = timed(lambda: prog.export_voxels(vox_grid, 1), kernels["vox"])
    soda_cells = int(np.prod(d.grid[6:9].astype(np.int64)))
    n_cloud = int(np.prod(np.ceil((hi - lo) / np.float32(cloud_step)).astype(np.int64)))
    vsize = vox[1]
    n_vox = int(vsize[0]) * int(vsize[1]) * int(vsize[2])
    cloud_gpu_ms = sum(cloud_k.values())
    vox_gpu_ms = sum(vox_k.values())
    soda_gpu_ms = sum(soda_k.values())
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        from oracle import oracle as O
        port = O.port()
        h = port.build(spec)
        try:
            t = time.perf_counter()
            port.sodapop(h, density)
            soda_cpu = time.perf_counter() - t
            # Middle z-slabs of the same lattices (8 voxel layers each), one core.
            mid = np.float32(0.5) * (lo[2] + hi[2])
            slab_lo = np.array([lo[0], lo[1], mid], np.float32)
            slab_hi = np.array([hi[0], hi[1], mid + np.float32(8 * cloud_step)], np.float32)
            o = port.octree(h)
            t = time.perf_counter()
            pts, _ = port.point_cloud(o, slab_lo, slab_hi, cloud_step, refine)
            port.vertex_attributes(o, pts, threads=1)
            cloud_cpu = time.perf_counter() - t
            port.octree_free(o)
            slab_voxels = int(np.prod(np.ceil((slab_hi - slab_lo) / np.float32(cloud_step)).astype(np.int64)))
            t = time.perf_counter()
            vox_small, vs_small, _ = port.vox(h, 8.0, 1)
            vox_cpu = time.perf_counter() - t
            cpu = {"sodapop_meshes_per_s": 1.0 / soda_cpu,
                   "point_cloud_voxels_per_s": slab_voxels / cloud_cpu,
                   "vox_voxels_per_s": int(np.prod(vs_small)) / vox_cpu,
                   "cores": 1, "kind": "port",
                   "sample": f"C restatement, one core: the whole Sodapop job ({soda_cpu:.2f} s); the point cloud on "
                             f"an 8-layer middle z-slab ({slab_voxels} voxels, {cloud_cpu:.2f} s); VoxExport's test at "
                             f"8 voxels per unit ({int(np.prod(vs_small))} voxels, {vox_cpu:.2f} s; full-tree eval per "
                             f"voxel, the same per-voxel work as at 64)"}
        finally:
            port.free(h)
    line = {"metric": "voxels/s: point-cloud export (with Sodapop meshing and MagicaVoxel export beside it)",
            "value": world * n_cloud / cloud_wall, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": cloud_wall * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"seeded {PRIMS}-primitive tree (seed {SEED}): point cloud at {cloud_step}-unit voxels "
                                   f"over the tree bounds ({n_cloud} voxels), {refine} refinement steps, normals + colours; "
                                   f"Sodapop meshing at density {density:g}; MagicaVoxel at {vox_grid:g} voxels per unit",
                       "l2": "inputs resident; results copied to host every step"},
            "point_cloud": {"voxels": n_cloud, "points": int(cloud.vertices.shape[0]), "ms_per_call": cloud_wall * 1e3,
                            "gpu_kernel_ms": cloud_k, "voxels_per_s_gpu": n_cloud / (cloud_gpu_ms * 1e-3)},
            "sodapop": {"cells": soda_cells, "vertices": int(d.positions.shape[0]), "faces": int(d.faces.shape[0]),
                        "ms_per_call": soda_wall * 1e3, "meshes_per_s": 1.0 / soda_wall,
                        "host_octree_and_compile_ms": d.compile_seconds * 1e3, "gpu_kernel_ms": soda_k,
                        "gpu_kernels_total_ms": soda_gpu_ms},
            "vox": {"voxels": n_vox, "kept": int(vox[0].shape[0]), "ms_per_call": vox_wall * 1e3, "gpu_kernel_ms": vox_k,
                    "voxels_per_s": n_vox / vox_wall, "voxels_per_s_gpu": n_vox / (vox_gpu_ms * 1e-3)},
            "e2e": {"value": world * n_cloud / cloud_wall, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(cloud.vertices.shape[0]) * 31},
            "cpu_baseline": cpu, "gpu_launches": 7, "clocks": clocks.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    prog.close()


def main():
    global RES, WORKLOAD, CONFIG
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--skip-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--batch-models", type=int, default=512, help="trees in the batch workload")
    ap.add_argument("--port", action="store_true", help="reference arm: time the C restatement even where the "
                                                        "reference library loads")
    ap.add_argument("--compare-res", type=int, default=512, help="cpu-compare: grid resolution")
    ap.add_argument("--workload", default="export",
                    choices=["export", "render", "surrogate", "batch", "exports", "cpu-compare"],
                    help="export: the 512^3 mesh export (the benchmark); render: the sphere-tracing workload; "
                         "surrogate: the 1024^3 export in 32^3 bricks with the learned bound; batch: 512 trees in one "
                         "launch; exports: Sodapop meshing, point cloud and MagicaVoxel; cpu-compare: the reference's "
                         "CPU export against the C restatement (x86 host with the reference sources)")
    ap.add_argument("--skip-surrogate", action="store_true", help="skip the surrogate-culled leg of the export")
    ap.add_argument("--resolution", type=int, default=RES,
                    help="grid resolution (512 is the benchmark; smaller values are profiling cases)")
    args = ap.parse_args()
    if args.resolution != RES:
        WORKLOAD = WORKLOAD.replace(f"{RES}^3", f"{args.resolution}^3").replace(f"({RES + 3}^3", f"({args.resolution + 3}^3")
        RES = args.resolution
        CONFIG = dict(CONFIG, workload=WORKLOAD, samples_per_mesh=(RES + 3) ** 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "cpu-compare":
        cpu_compare(args)
    elif args.impl == "reference":
        reference_arm(args, rank)
    elif args.workload == "render":
        render_arm(args, rank, world, local_rank)
    elif args.workload == "surrogate":
        surrogate_arm(args, rank, world, local_rank)
    elif args.workload == "batch":
        batch_arm(args, rank, world, local_rank)
    elif args.workload == "exports":
        exports_arm(args, rank, world, local_rank)
    else:
        our_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
