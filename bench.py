"""Benchmark: Gvoxels/s of SDF -> mesh dual contouring at 1024^3 on one GB300.

Workload (one "step"): the CSG SDF -- a rounded box (half-size 0.7, radius
0.05) minus a smooth union (k = 0.02) of 64 seeded spheres, unioned with a
torus (0.5, 0.1) -- meshed at 1024^3 cells over [-1, 1]^3: grid evaluation,
sign changes, crossings, mass-point vertices with normals, quads -> triangle
indices, all on the device.  A voxel is a cell; value = N^3 * steps / time.
The lattice evaluation is tile-pruned when the autotuner finds that faster:
per tile, the operands of min / max / smooth operators that an interval
pass proves cannot change any point's binary32 value are skipped, and the
mesh is bit-identical to the full evaluation (a GPU test).

  value        device time per step (CUDA events on the launching stream),
               mesh buffers resident, L2 flushed between steps (outside the
               events)
  e2e          the C-ABI call a user makes per job: s2m_mesh_create (device
               buffers, pipeline, count readback) + the mesh copied to pinned
               host memory + s2m_mesh_free
  roofline     the phase that takes the most device time (CUDA events around
               every launch of the timed steps): its algorithmic bytes (or, for
               the evaluation, the SDF operations it executed) per launch over
               its event time per launch
  full_evaluation  the same job with tile pruning off (every SDF operation at
               every lattice point), timed the same way
  cpu_baseline the CPU oracle (restatement of the reference rule) on a bounded
               window of slices of the same job, on all host cores and on one

The same line also carries compact results of the other configurations, each
measured in this run:
  mandelbulb_2048  the power-8 Mandelbulb (8 iterations, bounds 2.5) at
               2048^3, reference rule and precision mode
  batch256     256 seeded random CSG trees in one persistent launch, beside
               the plain per-job pipeline on the same jobs (modules compiled
               beforehand)
  serve        a Poisson request stream at several rates through the
               continuous-batching server, beside the plain per-job pipeline
               with the same compiled modules

--impl reference times the CPU implementation alone (the reference itself
is Rust + wgpu and cannot run here) and prints the same line.
N > 1 GPUs (torchrun): independent replicas, one job per rank, no collective
on the data path ("replicas only").
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FULL = 1024
BOUNDS = 2.0
METRIC = "Gvoxels/s at 1024^3"
UNIT = "Gvoxels/s"
CPU_SAMPLE_SLICES = 16     # cpu_baseline: cell slices [504, 520) of the 1024^3 job
CPU_SAMPLE_SLICES_1T = 2   # ... on one host thread: [504, 506)
REF_STEP_SLICES = 4        # --impl reference: cell slices per step
CPU_Z0 = 504


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--resolution", type=int, default=None)
    ap.add_argument("--workload", default="csg64_1024", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-full-eval", action="store_true", help="skip the run without tile pruning")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the mandelbulb_2048 / batch256 / serve sub-results of the headline line")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# name -> (resolution, bounds, precision mode, description)
WORKLOADS = {
    "batch256": (0, 2.0, False, "256 seeded random CSG trees (sphere/box/torus/capsule; union/subtract/intersect/"
                                "smooth-min), resolutions log-uniform over {64,96,128,192,256,384}"),
    "serve": (0, 2.0, False, "Poisson arrivals (seeded), 90% random CSG trees + 10% Mandelbulbs, resolution "
                             "round(exp U(ln 64, ln 1024)), 120 GB admission budget"),
    "csg64_1024": (1024, 2.0, False, "rounded box - smooth union (k=0.02) of 64 spheres (splitmix64 seed 0) + torus"),
    "mandelbulb_2048": (2048, 2.5, True, "Mandelbulb power 8, 8 iterations, bailout 2 (GLSL), precision mode: "
                                         "QEF vertex, FP32 compensated sums, FP64 solve"),
}
_ACTIVE = {"name": "csg64_1024"}
MANDEL_DESC = "Mandelbulb power 8, 8 iterations, bailout 2, offset 0.003 (GLSL), bounds 2.5"


def reduce_max(value: float, device=None) -> float:
    """Max over ranks (replicas: the job-wide time is the slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(items, rank: int, world: int):
    """Jobs of one rank: round-robin, disjoint, together complete (no data-path collective)."""
    return items[rank::world]


def workload():
    from sdf2mesh_gb300 import workloads
    if _ACTIVE["name"] == "mandelbulb_2048":
        return workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    return workloads.csg64(seed=0)


def oracle_kind():
    import oracle
    return oracle.MANDELBULB if _ACTIVE["name"] == "mandelbulb_2048" else oracle.CSG


def cpu_sample(n_slices, z0, resolution, threads=0):
    """The oracle (reference rule, binary32) on cell slices [z0, z0 + n) of the job."""
    import oracle
    _, prm = workload()
    t = time.perf_counter()
    _, bounds, qef, _ = WORKLOADS[_ACTIVE["name"]]
    m = oracle.mesh(oracle_kind(), prm, resolution, bounds, z_begin=z0, z_end=z0 + n_slices, threads=threads, qef=qef)
    dt = time.perf_counter() - t
    return dt, m


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_arm(a):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    N = a.resolution
    z0 = max(0, min(CPU_Z0, N - REF_STEP_SLICES))
    cells = REF_STEP_SLICES * N * N
    for _ in range(a.warmup):
        cpu_sample(REF_STEP_SLICES, z0, N)
    times = []
    for _ in range(a.steps):
        dt, _ = cpu_sample(REF_STEP_SLICES, z0, N)
        times.append(dt)
    tot = sum(times)
    v = cells * a.steps / tot / 1e9
    sample = (f"cell slices [{z0}, {z0 + REF_STEP_SLICES}) of the {N}^3 job per step "
              f"({cells} voxels), quads included")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": tot / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": _ACTIVE["name"], "resolution": N, "bounds": WORKLOADS[_ACTIVE["name"]][1],
                   "sdf": WORKLOADS[_ACTIVE["name"]][3],
                   "implementation": "CPU oracle: C++ restatement of the reference rule, OpenMP"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": host_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference (Rust + wgpu) is unavailable on this box: no Rust toolchain, no graphics stack",
    }), flush=True)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        hi = max(sm)
        load = [x for x in sm if x >= 0.5 * hi] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return {"hbm_gbs": 6800.0}, "fallback (6.8 TB/s, no MEASURED_PEAKS.json)"


PHASE_PROFILE = "phases_csg64_1024.md"


def phase_traffic():
    """DRAM bytes per 1024^3 CSG job of each pipeline phase, from the committed
    ncu summary of one job (profiles/phases_csg64_1024.md: lines
    `traffic_<phase> = <bytes>`)."""
    out = {}
    try:
        for line in open(os.path.join(ROOT, "profiles", PHASE_PROFILE)):
            if line.startswith("traffic_") and "=" in line:
                k, v = line.split("=", 1)
                out[k.strip()[len("traffic_"):]] = float(v)
    except OSError:
        pass
    return out


def phase_bytes(phase, N, C, V, T, pruned, resident=False):
    """Algorithmic DRAM bytes of one job's phase (what it must read and write at
    least): 2 point bits (sign, near-zero) per lattice point for classification
    (plus the 4-byte values when the lattice is materialised), 8-byte keys and
    32 bytes of corner values per candidate (read and written by classification
    unless the lattice stays resident for the vertex kernel, which then reads
    them), 28 bytes per vertex (position, normal, cell key), 12 bytes per
    triangle."""
    P3 = float(N + 1) ** 3
    if phase == "cells":
        return 2.0 * P3 / 8.0 + (0.0 if pruned else 4.0 * P3) + C * 8 + (0.0 if resident else C * (32 + 32))
    if phase == "vertices":
        return C * (8 + 32) + C * (8 + 24)
    if phase == "vcompact":
        return C * 8 + V * (24 + 28)
    if phase == "rowscan":
        return 8.0 * N * N
    if phase == "quads":
        return V * 8 + T * 12
    return 0.0


def time_job(s2m, L, sdf, state, stream, flush, steps, warmup, barrier, clocks=None, e2e_steps=None):
    """Device time of `steps` runs of one job (CUDA events on its stream, L2
    flushed before each outside the events, per-kernel events on), then the
    same job end to end through the C ABI: s2m_mesh_create + the reference's
    TriangleMesh (positions, normals, triangle indices) copied to pinned host
    memory + s2m_mesh_free."""
    import torch
    sp = stream.cuda_stream
    mesh = s2m.mesh_device(sdf, state, sp)
    info = mesh.info()
    nverts, ntris = int(info.nverts), int(info.ntris)
    for _ in range(warmup):
        mesh.run_async(sp)
        mesh.sync(sp)
    mesh.set_profiling(True)
    mesh.reset_profile()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    barrier()
    if clocks:
        clocks.start()
    w0 = time.perf_counter()
    for i in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            evs[i][0].record(stream)
        mesh.run_async(sp)
        with torch.cuda.stream(stream):
            evs[i][1].record(stream)
        mesh.sync(sp)
    barrier()
    wall = time.perf_counter() - w0
    clk = clocks.stop() if clocks else None
    mesh.set_profiling(False)
    dev_ms = sum(s.elapsed_time(e) for s, e in evs)
    prof = mesh.profile()
    ops = mesh.eval_ops()
    launches = int(info.kernel_launches)
    out = {"mesh": mesh, "info": info, "nverts": nverts, "ntris": ntris, "dev_ms": dev_ms, "prof": prof,
           "eval_ops": ops, "wall": wall, "clocks": clk, "launches_per_step": launches}
    # ---- end to end through the C ABI: create -> pinned host copy -> free ----
    host_pos = torch.empty(3 * nverts + 3, dtype=torch.float32, pin_memory=True)
    host_nrm = torch.empty(3 * nverts + 3, dtype=torch.float32, pin_memory=True)
    host_tri = torch.empty(3 * ntris + 3, dtype=torch.int32, pin_memory=True)
    p = state.params()
    err = ctypes.create_string_buffer(4096)
    e2e_ms = []
    parts = {"create_ms": 0.0, "copy_to_host_ms": 0.0, "free_ms": 0.0, "create_setup_ms": 0.0,
             "create_launch_ms": 0.0, "create_wait_ms": 0.0, "create_runs": 0.0}
    # untimed warm-up of the same calls: the first create beside the timed mesh
    # grows the stream-ordered pool (a one-time cost per process, like loading
    # the module); later creates reuse the blocks the previous free returned
    for _ in range(max(1, min(warmup, 3))):
        h = ctypes.c_void_p()
        rc = L.s2m_mesh_create(sdf.handle, ctypes.byref(p), ctypes.c_void_p(sp), ctypes.byref(h), err, len(err))
        if rc != 0:
            raise RuntimeError(err.value.decode())
        L.s2m_mesh_copy_to_host(h, host_pos.data_ptr(), host_nrm.data_ptr(), None, host_tri.data_ptr(),
                                ctypes.c_void_p(sp))
        L.s2m_mesh_free(h)
    barrier()
    for i in range(e2e_steps or steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        torch.cuda.synchronize()
        t = time.perf_counter()
        h = ctypes.c_void_p()
        rc = L.s2m_mesh_create(sdf.handle, ctypes.byref(p), ctypes.c_void_p(sp), ctypes.byref(h), err, len(err))
        if rc != 0:
            raise RuntimeError(err.value.decode())
        mi = s2m.MeshInfo()
        L.s2m_mesh_get_info(h, ctypes.byref(mi))
        if mi.nverts != nverts or mi.ntris != ntris:
            raise RuntimeError("e2e mesh differs from the timed mesh")
        t1 = time.perf_counter()
        rc = L.s2m_mesh_copy_to_host(h, host_pos.data_ptr(), host_nrm.data_ptr(), None,
                                     host_tri.data_ptr(), ctypes.c_void_p(sp))
        t2 = time.perf_counter()
        L.s2m_mesh_free(h)
        t3 = time.perf_counter()
        e2e_ms.append((t3 - t) * 1e3)
        parts["create_ms"] += (t1 - t) * 1e3
        parts["copy_to_host_ms"] += (t2 - t1) * 1e3
        parts["free_ms"] += (t3 - t2) * 1e3
        parts["create_setup_ms"] += mi.host_setup_ms
        parts["create_launch_ms"] += mi.host_launch_ms
        parts["create_wait_ms"] += mi.host_wait_ms
        parts["create_runs"] += mi.runs
        if rc != 0:
            raise RuntimeError("copy to host failed")
    barrier()
    out["create_copy_ms"] = sum(e2e_ms)
    out["create_copy_steps"] = len(e2e_ms)
    out["create_copy_parts_ms"] = {k: v / len(e2e_ms) for k, v in parts.items()}
    # ---- the one-call path: s2m_mesh_generate (z parts whose host copies
    # overlap the next part's kernels) + s2m_host_mesh_free ----
    hm = s2m.HostMesh()
    gen_ms, gen_parts = [], 0
    for i in range(max(1, min(warmup, 3)) + (e2e_steps or steps)):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = L.s2m_mesh_generate(sdf.handle, ctypes.byref(p), 0, ctypes.c_void_p(sp), ctypes.byref(hm), err, len(err))
        if rc != 0:
            raise RuntimeError(err.value.decode())
        if hm.nverts != nverts or hm.ntris != ntris:
            raise RuntimeError("generate's mesh differs from the timed mesh")
        gen_parts = int(hm.parts)
        L.s2m_host_mesh_free(ctypes.byref(hm))
        if i >= max(1, min(warmup, 3)):
            gen_ms.append((time.perf_counter() - t) * 1e3)
    barrier()
    # the same call with the number of z parts fixed, for the record
    by_parts = {}
    for k in (1, 2, 3, 4):
        ts = []
        for i in range(3):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
            torch.cuda.synchronize()
            t = time.perf_counter()
            rc = L.s2m_mesh_generate(sdf.handle, ctypes.byref(p), k, ctypes.c_void_p(sp), ctypes.byref(hm), err,
                                     len(err))
            if rc != 0:
                raise RuntimeError(err.value.decode())
            kk = int(hm.parts)
            L.s2m_host_mesh_free(ctypes.byref(hm))
            ts.append((time.perf_counter() - t) * 1e3)
        by_parts[str(kk)] = round(min(ts[1:]), 4)
    out["e2e_ms"] = sum(gen_ms)
    out["e2e_steps"] = len(gen_ms)
    out["e2e_parts"] = gen_parts
    out["e2e_ms_by_parts"] = by_parts
    out["e2e_parts_ms"] = {k: v / len(e2e_ms) for k, v in parts.items()}
    out["d2h"] = nverts * (12 + 12) + ntris * 12
    return out


def kernels_table(prof, steps):
    ms = prof["ms"]
    tot = max(1e-9, sum(ms.values()))
    return {k: {"launches_per_step": prof["launches"][k] // steps, "ms_per_step": ms[k] / steps,
                "share": ms[k] / tot} for k in ms}


def eval_roofline(s2m, sp, sdf, r, steps):
    """Roofline of the evaluation phase: the SDF operations it executed (with tile
    pruning: counted per tile by the tile pass; else the frontend's count per
    point as written) against the measured FP32 or SFU issue rate."""
    prof, ops = r["prof"], r["eval_ops"]
    ms = prof["ms"]["eval_planes"]
    n_eval = max(1, prof["launches"]["eval_planes"])
    pts = max(1.0, ops["points"])
    fp32_pp, sfu_pp = ops["fp32_ops"] / pts, ops["sfu_ops"] / pts
    fp32_peak = s2m.measure_fp32_peak(sp)
    sfu_peak = s2m.measure_sfu_peak(sp)
    fp32_gops = fp32_pp * prof["eval_points"] / (ms * 1e-3) / 1e9
    sfu_gops = sfu_pp * prof["eval_points"] / (ms * 1e-3) / 1e9
    sfu_bound = sfu_pp / max(1e-9, sfu_peak) > fp32_pp / max(1e-9, fp32_peak)
    return {"bound": "sfu" if sfu_bound else "fp32", "kernel": "s2m_tiles + s2m_evalpl_*" if ops["pruned"]
            else "s2m_eval_*", "achieved": sfu_gops if sfu_bound else fp32_gops,
            "peak": sfu_peak if sfu_bound else fp32_peak, "unit": "Gop/s",
            "frac": (sfu_gops / sfu_peak) if sfu_bound else (fp32_gops / fp32_peak),
            "fp32_frac": fp32_gops / fp32_peak, "sfu_frac": sfu_gops / sfu_peak,
            "ms_per_launch": ms / n_eval,
            "algorithmic": f"{fp32_pp:g} FP32 + {sfu_pp:g} SFU ops per lattice point x "
                           f"{prof['eval_points'] / n_eval:.0f} points per launch",
            "ops_source": ("tile pass: active segments' operations x points of each tile" if ops["pruned"]
                           else "frontend op count per point as written (loops at their full trip count: an upper "
                                "bound of what points that bail out early execute)"),
            "peak_source": "measured in this run: s2m_fp32_probe (FP32 add/mul issue rate) and s2m_sfu_probe "
                           "(MUFU rsqrt issue rate)",
            "traffic": None}


def dominant_roofline(s2m, sp, sdf, r, N, steps, pk, pk_kind, traffic_per_job=None):
    """The phase with the most device time: evaluation against its op roofline,
    any other phase against HBM with its algorithmic bytes."""
    prof = r["prof"]
    ms = prof["ms"]
    dom = max(ms, key=lambda k: ms[k])
    C, V, T = float(r["info"].candidate_cells), float(r["nverts"]), float(r["ntris"])
    pruned = bool(r["eval_ops"]["pruned"])
    # one slab with the listed evaluation: the lattice stays resident for the vertex kernel
    resident = pruned and "evalpl" in sdf.eval_variant()[0] and int(r["info"].slab_depth) >= N - 1
    if dom == "eval_planes":
        roof = eval_roofline(s2m, sp, sdf, r, steps)
    else:
        nl = max(1, prof["launches"][dom])
        per_launch_ms = ms[dom] / nl
        launches_per_job = nl / steps
        b = phase_bytes(dom, N, C, V, T, pruned, resident) / launches_per_job
        achieved = b / (per_launch_ms * 1e-3) / 1e9
        tr = (traffic_per_job or {}).get(dom)
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "peak_source": pk_kind,
                "algorithmic_bytes_per_launch": b, "ms_per_launch": per_launch_ms,
                "algorithmic": "point bits 2 per lattice point, candidates 8 B key + 32 B corners written and "
                               "corners read, vertices 28 B, triangles 12 B (per phase as it must move them)",
                "traffic": tr / launches_per_job if tr else None,
                "traffic_source": f"ncu dram__bytes_read.sum + dram__bytes_write.sum of the phase's launches in "
                                  f"one job (profiles/{PHASE_PROFILE})" if tr else None}
    roof["dominant_by_time"] = dom
    # contouring as a whole (every phase after the evaluation), per 8(d)
    cont_ms = sum(ms[k] for k in ms if k != "eval_planes") / steps
    cont_b = sum(phase_bytes(k, N, C, V, T, pruned, resident) for k in ("cells", "vertices", "vcompact", "rowscan", "quads"))
    return roof, {"bound": "hbm", "ms_per_job": cont_ms, "bytes_per_job": cont_b,
                  "achieved": cont_b / (cont_ms * 1e-3) / 1e9 if cont_ms > 0 else None, "peak": pk["hbm_gbs"],
                  "unit": "GB/s", "frac": (cont_b / (cont_ms * 1e-3) / 1e9) / pk["hbm_gbs"] if cont_ms > 0 else None,
                  "peak_source": pk_kind}


def ours(a):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    import sdf2mesh_gb300 as s2m
    from sdf2mesh_gb300 import build as b
    b.build()
    L = s2m.load_library()

    N = a.resolution
    src, _ = workload()
    t0 = time.perf_counter()
    _, bounds, qef, desc = WORKLOADS[a.workload]
    lang = s2m.LANG_GLSL if a.workload.startswith("mandelbulb") else s2m.LANG_WGSL
    # compile cold (an empty module cache) and warm (the same source again, from the cache)
    cache_env = os.environ.get("S2M_CACHE_DIR")
    os.environ["S2M_CACHE_DIR"] = tempfile.mkdtemp(prefix="s2m_cache_")
    shader = s2m.Sdf3DShader.from_source(src, lang, "sdf")
    sdf = shader.compile()
    compile_s = time.perf_counter() - t0
    cold_info = sdf.compile_info()
    t0 = time.perf_counter()
    sdf_warm = shader.compile()
    compile_warm_s = time.perf_counter() - t0
    warm_info = sdf_warm.compile_info()
    sdf_warm.close()
    if cache_env is None:
        del os.environ["S2M_CACHE_DIR"]
    else:
        os.environ["S2M_CACHE_DIR"] = cache_env
    fp32_ops, sfu_ops = sdf.op_counts()
    prune_comb, _ = sdf.prune_info()

    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    state = s2m.AppState(resolution=N, bounds=bounds, qef=qef)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)  # 256 MiB > 126 MB L2

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed steps, then end to end -------------------------------
    r = time_job(s2m, L, sdf, state, stream, flush, a.steps, a.warmup, barrier, Clocks(local))
    mesh, info, nverts, ntris = r["mesh"], r["info"], r["nverts"], r["ntris"]
    tot_ms = reduce_max(r["dev_ms"], dev)
    voxels_step = float(N) ** 3
    value = voxels_step * a.steps * ws / (tot_ms * 1e-3) / 1e9
    e2e_tot = reduce_max(r["e2e_ms"], dev)
    e2e_value = voxels_step * r["e2e_steps"] * ws / (e2e_tot * 1e-3) / 1e9

    # ---- the same job without tile pruning (every operation at every point) --
    full_eval = None
    if prune_comb > 0 and not a.no_full_eval:
        plain = shader.compile(prune=False)
        fmesh = s2m.mesh_device(plain, state, sp)
        for _ in range(2):
            fmesh.run_async(sp)
            fmesh.sync(sp)
        fmesh.set_profiling(True)
        barrier()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
        for i in range(3):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                evs[i][0].record(stream)
            fmesh.run_async(sp)
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
            fmesh.sync(sp)
        f_ms = reduce_max(sum(s.elapsed_time(e) for s, e in evs), dev)
        f_prof = fmesh.profile()
        f_mi = fmesh.info()
        if int(f_mi.nverts) != nverts or int(f_mi.ntris) != ntris:
            raise RuntimeError("the full evaluation's mesh differs from the pruned one")
        full_eval = {"value": voxels_step * 3 * ws / (f_ms * 1e-3) / 1e9, "unit": UNIT, "steps": 3,
                     "ms_per_step": f_ms / 3, "eval_variant": plain.eval_variant()[0],
                     "eval_ms_per_step": f_prof["ms"]["eval_planes"] / 3,
                     "mesh": "same vertex and triangle counts (bit-identity is a GPU test)"}
        fmesh.close()
        plain.close()

    if rank != 0:
        mesh.close()
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    pk, pk_kind = peaks()
    roof, contour = dominant_roofline(s2m, sp, sdf, r, N, a.steps, pk, pk_kind,
                                      phase_traffic() if (a.workload == "csg64_1024" and N == 1024) else None)
    eval_view = eval_roofline(s2m, sp, sdf, r, a.steps)

    cpu = None
    if not a.no_cpu_baseline:
        n = min(CPU_SAMPLE_SLICES if a.workload == "csg64_1024" else 4, N)
        z0 = max(0, min(CPU_Z0, N - n))
        dt, _ = cpu_sample(n, z0, N)
        n1 = min(CPU_SAMPLE_SLICES_1T, N)
        dt1, _ = cpu_sample(n1, z0, N, threads=1)
        cpu = {"value": n * N * N / dt / 1e9, "unit": UNIT, "cores": host_threads(), "kind": "port",
               "sample": f"CPU oracle (reference rule, binary32, OpenMP) on cell slices [{z0}, {z0 + n}) "
                         f"of the {N}^3 job: {n * N * N} voxels in {dt:.2f} s",
               "one_thread": {"value": n1 * N * N / dt1 / 1e9, "unit": UNIT, "cores": 1,
                              "sample": f"cell slices [{z0}, {z0 + n1}): {n1 * N * N} voxels in {dt1:.2f} s"}}

    eval_ops = r["eval_ops"]
    pts_run = max(1.0, eval_ops["points"])
    metric = METRIC if a.workload == "csg64_1024" and N == 1024 else f"Gvoxels/s at {N}^3 ({a.workload})"
    line = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": tot_ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": a.workload, "resolution": N, "bounds": bounds, "sdf": desc,
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "flushed between steps (256 MiB write, outside the timed events)",
                   "precision": ("precision mode: lattice corners, QEF vertex, FP32 compensated sums, FP64 solve"
                                 if qef else "reference rule in binary32, no FMA contraction, IEEE div/sqrt"),
                   "evaluation": ("tile-pruned (exact: bit-identical to every operation at every point)"
                                  if eval_ops["pruned"] else "every SDF operation at every lattice point")},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": r["d2h"],
                "ms_per_step": e2e_tot / r["e2e_steps"], "z_parts": r["e2e_parts"],
                "ms_by_z_parts": r["e2e_ms_by_parts"],
                "path": "s2m_mesh_generate + s2m_host_mesh_free: the reference's TriangleMesh (positions, normals, "
                        "triangle indices) in pinned host memory, the job in z parts whose device-to-host copies "
                        "overlap the next part's kernels; inputs are the compiled SDF module and a 48-byte "
                        "parameter block passed as kernel arguments",
                "create_copy_free": {"value": float(N) ** 3 * r["create_copy_steps"] / (r["create_copy_ms"] * 1e-3)
                                     / 1e9, "ms_per_step": r["create_copy_ms"] / r["create_copy_steps"],
                                     "parts_ms": r["create_copy_parts_ms"],
                                     "path": "s2m_mesh_create + s2m_mesh_copy_to_host (pinned) + s2m_mesh_free"}},
        "roofline": roof,
        "roofline_contouring": contour,
        "roofline_evaluation": eval_view,
        "kernels": kernels_table(r["prof"], a.steps),
        "full_evaluation": full_eval,
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
        "gpu_launches": r["launches_per_step"] * a.steps,
        "mesh": {"vertices": nverts, "triangles": ntris, "invalid_quads": int(info.invalid_quads),
                 "candidate_cells": int(info.candidate_cells), "slab_depth": int(info.slab_depth)},
        "compile_s": {"cold": compile_s, "warm": compile_warm_s, "nvrtc_programs": cold_info["programs"],
                      "cold_cache_hits": cold_info["cache_hits"], "warm_cache_hits": warm_info["cache_hits"],
                      "note": "frontend + NVRTC (parallel programs) + module load; warm = the same source "
                              "again, served by the on-disk module cache"},
        "eval_variant": sdf.eval_variant()[0],
        "tile_pruning": {"combinators": prune_comb, "used": eval_ops["pruned"],
                         "fp32_ops_per_point": eval_ops["fp32_ops"] / pts_run,
                         "sfu_ops_per_point": eval_ops["sfu_ops"] / pts_run,
                         "fp32_ops_per_point_as_written": fp32_ops},
        "eval_variants": [{"name": n, "ns_per_point": t, "registers": rg, "local_bytes": lb}
                          for n, t, rg, lb in sdf.eval_variants()],
        "triangles_per_s": ntris * a.steps * ws / (tot_ms * 1e-3),
        "wall_s_timed": r["wall"],
    }
    mesh.close()
    if ws == 1 and not a.no_extras and a.workload == "csg64_1024":
        line["mandelbulb_2048"] = sub_mandelbulb(s2m, L, stream, flush, barrier, pk, pk_kind)
        line["batch256"] = sub_batch(s2m)
        line["serve"] = sub_serve(s2m)
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# The other configurations, as compact sub-results of the headline line.


def sub_mandelbulb(s2m, L, stream, flush, barrier, pk, pk_kind, N=2048, B=2.5, steps=3, warmup=3):
    """Mandelbulb 2048^3 (bounds 2.5): the reference rule and precision mode, each
    device-timed and end to end, with the evaluation's SFU / FP32 fractions."""
    from sdf2mesh_gb300 import workloads
    src, _ = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    t = time.perf_counter()
    sdf = s2m.Sdf3DShader.from_source(src, s2m.LANG_GLSL, "sdf").compile()
    out = {"sdf": MANDEL_DESC, "resolution": N, "unit": UNIT, "steps": steps, "warmup": warmup,
           "compile_s": time.perf_counter() - t}
    sp = stream.cuda_stream
    for mode, qef in (("reference_rule", False), ("precision", True)):
        clk = Clocks(0)
        r = time_job(s2m, L, sdf, s2m.AppState(resolution=N, bounds=B, qef=qef), stream, flush, steps, warmup,
                     barrier, clk, e2e_steps=2)
        roof, _ = dominant_roofline(s2m, sp, sdf, r, N, steps, pk, pk_kind)
        ev = eval_roofline(s2m, sp, sdf, r, steps)
        out[mode] = {
            "value": float(N) ** 3 * steps / (r["dev_ms"] * 1e-3) / 1e9, "ms_per_step": r["dev_ms"] / steps,
            "e2e": {"value": float(N) ** 3 * r["e2e_steps"] / (r["e2e_ms"] * 1e-3) / 1e9,
                    "ms_per_step": r["e2e_ms"] / r["e2e_steps"], "parts_ms": r["e2e_parts_ms"],
                    "d2h_bytes_per_step": r["d2h"], "h2d_bytes_per_step": 0},
            "roofline": {k: roof[k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac",
                                              "dominant_by_time") if k in roof},
            "evaluation": {"sfu_frac": ev["sfu_frac"], "fp32_frac": ev["fp32_frac"], "bound": ev["bound"],
                           "ops_source": ev["ops_source"]},
            "kernels": {k: round(v["ms_per_step"], 3) for k, v in kernels_table(r["prof"], steps).items()},
            "launches_per_step": r["launches_per_step"],
            "mesh": {"vertices": r["nverts"], "triangles": r["ntris"],
                     "invalid_quads": int(r["info"].invalid_quads), "slab_depth": int(r["info"].slab_depth)},
            "clocks": r["clocks"]}
        if mode == "reference_rule":
            out[mode]["stl_binary_write"] = time_binary_stl(r["mesh"])
        r["mesh"].close()
    sdf.close()
    return out


def time_binary_stl(dmesh):
    """Write the mesh as binary STL from all host threads (s2m_write_stl_binary):
    GB/s of file bytes, on a RAM-backed file system when there is one, so that
    the figure is the writer's rather than the disk's."""
    host = dmesh.to_host()
    d = "/dev/shm" if os.path.isdir("/dev/shm") else tempfile.gettempdir()
    path = os.path.join(d, f"s2m_bench_{os.getpid()}.stl")
    try:
        t = time.perf_counter()
        host.write_stl_binary_to_file(path)
        dt = time.perf_counter() - t
        size = os.path.getsize(path)
        return {"bytes": size, "seconds": dt, "gb_per_s": size / dt / 1e9, "threads": host_threads(),
                "path": d, "triangles": int(host.triangle_indices.shape[0])}
    except Exception as e:  # no room for the file: report, do not fail the bench
        return {"error": str(e)[:200], "path": d}
    finally:
        if os.path.exists(path):
            os.unlink(path)


def batch_jobs(n=256, seed=4):
    from sdf2mesh_gb300 import workloads
    rng = workloads.SplitMix64(seed)
    jobs = []
    for i in range(n):
        src, prog = workloads.random_tree(i)
        N = workloads.log_uniform_resolution(rng)
        jobs.append((src, prog, N))
    return jobs


def compile_all(s2m, sources):
    """Compile distinct sources on all host threads (NVRTC releases the GIL)."""
    uniq = list(dict.fromkeys(sources))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(16, host_threads()))) as ex:
        mods = dict(zip(uniq, ex.map(lambda s: s2m.Sdf3DShader.from_source(*s).compile(), uniq)))
    return mods


def plain_per_job(jobs, precompiled=None):
    """The plain pipeline, one job at a time: compile the .sdf3d source (NVRTC) and mesh it
    (s2m_mesh_create), or with `precompiled` modules only mesh it.  Returns seconds per job."""
    import sdf2mesh_gb300 as s2m
    t = time.perf_counter()
    for k, (src, _, N) in enumerate(jobs):
        sdf = precompiled[k] if precompiled else s2m.Sdf3DShader.from_source(src).compile()
        m = s2m.mesh_device(sdf, s2m.AppState(resolution=N, bounds=2.0))
        m.close()
        if not precompiled:
            sdf.close()
    return (time.perf_counter() - t) / len(jobs)


def sub_batch(s2m, steps=3, warmup=3):
    """256 random CSG trees in one persistent launch, beside the plain per-job
    pipeline on the same jobs with every module compiled (and tuned) beforehand."""
    import torch
    jobs = batch_jobs()
    voxels = float(sum(N ** 3 for _, _, N in jobs))

    def one():
        bt = s2m.Batch()
        for _, prog, N in jobs:
            bt.add_csg(prog, s2m.AppState(resolution=N, bounds=2.0))
        t = time.perf_counter()
        bt.run()
        dt = time.perf_counter() - t
        ms, launches, _ = bt.stats()
        prof = bt.stage_profile()
        bt.close()
        return dt, ms, launches, prof

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    res = [one() for _ in range(steps)]
    clk = clocks.stop()
    wall = sum(x[0] for x in res)
    mps = len(jobs) * steps / wall
    mods = compile_all(s2m, [(src, s2m.LANG_WGSL, "sdf") for src, _, _ in jobs])
    pre = [mods[(src, s2m.LANG_WGSL, "sdf")] for src, _, _ in jobs]
    plain_per_job(jobs, pre)  # warm: autotuner, pools
    plain_s = plain_per_job(jobs, pre)
    for m in mods.values():
        m.close()
    return {"metric": "meshes/s (256 CSG jobs per step, one persistent launch)", "value": mps, "unit": "meshes/s",
            "steps": steps, "warmup": warmup, "ms_per_step": wall / steps * 1e3,
            "gvoxels_per_s": voxels * steps / wall / 1e9, "device_ms_per_step": sum(x[1] for x in res) / steps,
            "launches_per_step": res[0][2],
            "stage_block_ms": {k: round(v, 3) for k, v in res[-1][3].items()},
            "plain_per_job_precompiled": {"meshes_per_s": 1.0 / plain_s, "gvoxels_per_s": voxels / len(jobs) / plain_s
                                          / 1e9, "path": "s2m_mesh_create + s2m_mesh_free per job, same 256 jobs, "
                                                         "modules compiled and tuned beforehand"},
            "speedup_vs_precompiled_same_mix": mps * plain_s, "clocks": clk}


def serve_requests(n, seed=2000):
    """Request contents: 90% random CSG trees, 10% Mandelbulbs, resolution
    round(exp U(ln 64, ln 1024)); arrival gaps Exp(1) (scaled by 1/rate)."""
    from sdf2mesh_gb300 import workloads
    rng = workloads.SplitMix64(seed)
    reqs = []
    t = 0.0
    for _ in range(n):
        t += -math.log(1.0 - rng.u01())
        N = int(round(math.exp(rng.uniform(math.log(64), math.log(1024)))))
        if rng.u01() < 0.1:
            reqs.append((t, "mandelbulb", None, N))
        else:
            src, _ = workloads.random_tree(int(rng.next() % 100000))
            reqs.append((t, "csg", src, N))
    return reqs


def run_serve_sweep(s2m, rates, nreq, reqs=None):
    """Each rate: the same seeded requests, arrivals at `rate` req/s, through
    (1) the continuous-batching server (requests as .sdf3d / GLSL text) and (2)
    the plain per-job pipeline, one request at a time in arrival order, with
    every module compiled beforehand (the same cache the server holds)."""
    from sdf2mesh_gb300 import workloads
    mb_src, _ = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    reqs = reqs or serve_requests(nreq)

    def state(kind, N):
        return s2m.AppState(resolution=N, bounds=2.5 if kind == "mandelbulb" else 2.0)

    def key(kind, src):
        return (mb_src, s2m.LANG_GLSL, "sdf") if kind == "mandelbulb" else (src, s2m.LANG_WGSL, "sdf")

    mods = compile_all(s2m, [key(k, s) for _, k, s, _ in reqs])
    pre = [mods[key(k, s)] for _, k, s, _ in reqs]
    # warm both paths once: autotuner per module, pools, the server's source
    # cache (its background compiles of the CSG sources are served by the
    # on-disk module cache that compile_all filled)
    server = s2m.Server(memory_budget_bytes=120 << 30, max_inflight=2, max_batch_jobs=64, keep_results=False,
                        sdf_workers=4)
    for (_, kind, src, N) in reqs:
        k = key(kind, src)
        server.submit_source(k[0], state(kind, N), k[1], k[2])
    server.drain(3600)
    t_wait = time.perf_counter()
    while server.stats()["compiles_pending"] and time.perf_counter() - t_wait < 600:
        time.sleep(0.05)
    for (_, kind, src, N) in reqs:  # again, now on the compiled modules (their first jobs tune them)
        k = key(kind, src)
        server.submit_source(k[0], state(kind, N), k[1], k[2])
    server.drain(3600)
    for k, (_, kind, src, N) in enumerate(reqs):
        s2m.mesh_device(pre[k], state(kind, N)).close()

    def paced(t0, rate):
        for r in reqs:
            d = t0 + r[0] / rate - time.perf_counter()
            if d > 0:
                time.sleep(d)
            yield r

    table = []
    for rate in rates:
        server.reset_stats()
        t0 = time.perf_counter()
        for (_, kind, src, N) in paced(t0, rate):
            k = key(kind, src)
            server.submit_source(k[0], state(kind, N), k[1], k[2])
        server.drain(3600)
        sst = server.stats()
        lat = []
        t0 = time.perf_counter()
        for i, (t, kind, src, N) in enumerate(paced(t0, rate)):
            s2m.mesh_device(pre[i], state(kind, N)).close()
            lat.append((time.perf_counter() - t0 - t / rate) * 1e3)
        span = time.perf_counter() - t0
        lat.sort()
        plain = {"meshes_per_s": len(reqs) / span, "p50_ms": lat[len(lat) // 2],
                 "p99_ms": lat[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))]}
        table.append({"rate": rate, "served": {"meshes_per_s": sst["meshes_per_s"], "p50_ms": sst["p50_ms"],
                                               "p99_ms": sst["p99_ms"], "launches": sst["batches"],
                                               "gvoxels_per_s": sst["gvoxels_per_s"],
                                               "peak_gb": sst["peak_bytes"] / 1e9,
                                               "ran_compiled": sst["ran_compiled"],
                                               "ran_interpreted": sst["ran_interpreted"]},
                      "plain_per_job_precompiled": plain,
                      "speedup_vs_precompiled": sst["meshes_per_s"] / plain["meshes_per_s"]})
    server.close()
    for m in mods.values():
        m.close()
    return table


def sub_serve(s2m, rates=(10, 30, 100, 300, 1000, 2000), nreq=48):
    table = run_serve_sweep(s2m, list(rates), nreq)
    return {"metric": "served meshes/s and latency vs the plain per-job pipeline (same compiled modules)",
            "requests_per_rate": nreq, "sdf": WORKLOADS["serve"][3],
            "sweep": [{"rate": t["rate"], "meshes_per_s": t["served"]["meshes_per_s"],
                       "p50_ms": t["served"]["p50_ms"], "p99_ms": t["served"]["p99_ms"],
                       "plain_meshes_per_s": t["plain_per_job_precompiled"]["meshes_per_s"],
                       "plain_p50_ms": t["plain_per_job_precompiled"]["p50_ms"],
                       "plain_p99_ms": t["plain_per_job_precompiled"]["p99_ms"],
                       "speedup_vs_precompiled": t["speedup_vs_precompiled"]} for t in table]}


# ---------------------------------------------------------------------------
# Stand-alone lines of the other configurations (--workload batch256 / serve).


def batch_arm(a):
    import torch
    torch.cuda.set_device(0)
    import sdf2mesh_gb300 as s2m
    from sdf2mesh_gb300 import build as b
    b.build()
    r = sub_batch(s2m, steps=a.steps, warmup=a.warmup)
    line = {"metric": r["metric"], "value": r["value"], "unit": "meshes/s", "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch256", "jobs": 256, "sdf": WORKLOADS["batch256"][3], "bounds": 2.0,
                       "path": "s2m_batch_run: one persistent launch over a device work queue, CSG interpreter"},
            "gpu_launches": r["launches_per_step"] * a.steps,
            "e2e": {"value": r["value"], "unit": "meshes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            **{k: r[k] for k in ("gvoxels_per_s", "device_ms_per_step", "plain_per_job_precompiled",
                                 "speedup_vs_precompiled_same_mix", "stage_block_ms", "clocks")}}
    print(json.dumps(line), flush=True)


def serve_arm(a):
    import torch
    torch.cuda.set_device(0)
    import sdf2mesh_gb300 as s2m
    from sdf2mesh_gb300 import build as b
    b.build()
    rates = [10, 30, 100, 300, 1000, 2000]
    table = run_serve_sweep(s2m, rates, 48)
    for t in table:
        print(json.dumps(t), file=sys.stderr, flush=True)
    top = table[-1]
    line = {
        "metric": "served meshes/s (Poisson stream, 2000 req/s offered)", "value": top["served"]["meshes_per_s"],
        "unit": "meshes/s", "n_gpus": 1, "steps": len(rates), "warmup": 1,
        "ms_per_step": 1e3 / max(1e-9, top["served"]["meshes_per_s"]), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serve", "requests_per_rate": 48, "rates": rates, "sdf": WORKLOADS["serve"][3],
                   "served": "s2m_server_submit_source: requests are .sdf3d / GLSL text",
                   "plain_per_job": "one request at a time in arrival order: s2m_mesh_create with the modules "
                                    "compiled beforehand"},
        "p50_ms": top["served"]["p50_ms"], "p99_ms": top["served"]["p99_ms"],
        "sweep": table,
        "e2e": {"value": top["served"]["meshes_per_s"], "unit": "meshes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "ours" and a.workload == "batch256":
        return batch_arm(a)
    if a.impl == "ours" and a.workload == "serve":
        return serve_arm(a)
    _ACTIVE["name"] = a.workload
    if a.resolution is None:
        a.resolution = WORKLOADS[a.workload][0]
    if a.impl == "reference":
        reference_arm(a)
    else:
        ours(a)


if __name__ == "__main__":
    main()
