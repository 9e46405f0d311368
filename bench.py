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
  roofline     the dominant kernel, from CUDA events around every launch of
               the timed steps; for the evaluation, the SDF operations it
               executed (with tile pruning: counted per tile by the tile pass)
  full_evaluation  the same job with tile pruning off (every SDF operation at
               every lattice point), timed the same way
  cpu_baseline the CPU oracle (restatement of the reference rule, OpenMP on all
               host cores) on a bounded window of slices of the same job

--impl reference times that CPU implementation alone (the reference itself
is Rust + wgpu and cannot run here) and prints the same line.
N > 1 GPUs (torchrun): independent replicas, one job per rank, no collective
on the data path ("replicas only").
"""
from __future__ import annotations

import argparse
import ctypes
import json
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


EVAL_PROFILE = {False: "s2m_eval_csg64_512.md", True: "job_csg64_1024.md"}


def eval_traffic_per_point(pruned=False):
    """DRAM bytes per lattice point of the evaluation (pruned: tile pass + pruned
    kernel), from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", EVAL_PROFILE[pruned])
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_point"):
                return float(line.split("=")[1])
    except OSError:
        pass
    return None


JOB_PROFILE = "job_csg64_1024.md"


def job_profile():
    """Warp instructions and DRAM bytes per job of the pruned evaluation phase
    (CSG at 1024^3), from the committed ncu summary of one job."""
    out = {}
    try:
        for line in open(os.path.join(ROOT, "profiles", JOB_PROFILE)):
            for key in ("eval_inst_per_job", "eval_dram_bytes_per_job"):
                if line.startswith(key):
                    out[key] = float(line.split("=")[1])
    except OSError:
        pass
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


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
    shader = s2m.Sdf3DShader.from_source(src, lang, "sdf")
    sdf = shader.compile()
    compile_s = time.perf_counter() - t0
    fp32_ops, sfu_ops = sdf.op_counts()
    prune_comb, _ = sdf.prune_info()

    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    state = s2m.AppState(resolution=N, bounds=bounds, qef=qef)
    mesh = s2m.mesh_device(sdf, state, sp)
    info = mesh.info()
    nverts, ntris = int(info.nverts), int(info.ntris)
    launches_per_step = int(info.kernel_launches)

    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)  # 256 MiB > 126 MB L2

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def timed(m, steps, warmup, clocks=None):
        """Device time of `steps` runs of mesh m (CUDA events on its stream,
        L2 flushed before each, outside the events), with per-kernel events."""
        for _ in range(warmup):
            m.run_async(sp)
            m.sync(sp)
        m.set_profiling(True)
        m.reset_profile()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        if clocks:
            clocks.start()
        w0 = time.perf_counter()
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                evs[i][0].record(stream)
            m.run_async(sp)
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
            m.sync(sp)
        barrier()
        w = time.perf_counter() - w0
        clk = clocks.stop() if clocks else None
        m.set_profiling(False)
        return sum(s.elapsed_time(e) for s, e in evs), m.profile(), w, clk

    # ---- device-timed steps -------------------------------------------------
    tot_ms, prof, wall, clk = timed(mesh, a.steps, a.warmup, Clocks(local))
    eval_ops = mesh.eval_ops()  # SDF operations the last run executed
    tot_ms = reduce_max(tot_ms, dev)
    voxels_step = float(N) ** 3
    value = voxels_step * a.steps * ws / (tot_ms * 1e-3) / 1e9

    # ---- the same job without tile pruning (every operation at every point) --
    full_eval = None
    if prune_comb > 0 and not a.no_full_eval:
        plain = shader.compile(prune=False)
        fmesh = s2m.mesh_device(plain, state, sp)
        f_ms, f_prof, _, _ = timed(fmesh, a.steps, max(1, min(a.warmup, 2)))
        f_ms = reduce_max(f_ms, dev)
        f_mi = fmesh.info()
        if int(f_mi.nverts) != nverts or int(f_mi.ntris) != ntris:
            raise RuntimeError("the full evaluation's mesh differs from the pruned one")
        f_ops = fmesh.eval_ops()
        full_eval = {"value": voxels_step * a.steps * ws / (f_ms * 1e-3) / 1e9, "unit": UNIT,
                     "ms_per_step": f_ms / a.steps, "eval_variant": plain.eval_variant()[0],
                     "eval_ms_per_step": f_prof["ms"]["eval_planes"] / a.steps,
                     "fp32_ops_per_step": f_ops["fp32_ops"], "sfu_ops_per_step": f_ops["sfu_ops"],
                     "mesh": "same vertex and triangle counts (bit-identity is a GPU test)"}
        fmesh.close()
        plain.close()

    # ---- end to end through the C ABI: create -> pinned host copy -> free ----
    host_pos = torch.empty(3 * nverts + 3, dtype=torch.float32, pin_memory=True)
    host_nrm = torch.empty(3 * nverts + 3, dtype=torch.float32, pin_memory=True)
    host_tri = torch.empty(3 * ntris + 3, dtype=torch.int32, pin_memory=True)
    p = state.params()
    err = ctypes.create_string_buffer(4096)
    e2e_ms = []
    d2h = 0
    barrier()
    for i in range(a.steps):
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
        # the reference's TriangleMesh: vertices (position, normal) and triangle indices
        rc = L.s2m_mesh_copy_to_host(h, host_pos.data_ptr(), host_nrm.data_ptr(), None,
                                     host_tri.data_ptr(), ctypes.c_void_p(sp))
        L.s2m_mesh_free(h)
        e2e_ms.append((time.perf_counter() - t) * 1e3)
        if rc != 0:
            raise RuntimeError("copy to host failed")
        d2h = nverts * (12 + 12) + ntris * 12
    barrier()
    e2e_tot = sum(e2e_ms)
    e2e_tot = reduce_max(e2e_tot, dev)
    e2e_value = voxels_step * a.steps * ws / (e2e_tot * 1e-3) / 1e9

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel -------------------------------------
    ms = prof["ms"]
    dom = max(ms, key=lambda k: ms[k])
    fp32_peak = s2m.measure_fp32_peak(sp)  # Gop/s, one FP32 add or mul per lane per cycle
    pk, pk_kind = peaks()
    n_eval = max(1, prof["launches"]["eval_planes"])
    roof = {}
    kernels = {}
    for k in ms:
        nl = prof["launches"][k]
        kernels[k] = {"launches_per_step": nl // a.steps, "ms_per_step": ms[k] / a.steps,
                      "share": ms[k] / max(1e-9, sum(ms.values()))}
    # ops the evaluation executes per point: the SDF as written; with a run-of-4 variant its run
    # form (the x/y-only part once per 4 points); with tile pruning the operations of the segments
    # the tile pass left active, counted per tile (eval_ops of the last run)
    variant = sdf.eval_variant()[0]
    per_point_scalar = (fp32_ops, sfu_ops)
    pts_run = max(1.0, eval_ops["points"])
    fp32_ops, sfu_ops = eval_ops["fp32_ops"] / pts_run, eval_ops["sfu_ops"] / pts_run
    eval_gops = fp32_ops * prof["eval_points"] / (ms["eval_planes"] * 1e-3) / 1e9
    eval_sfu = sfu_ops * prof["eval_points"] / (ms["eval_planes"] * 1e-3) / 1e9
    scalar_equiv_gops = per_point_scalar[0] * prof["eval_points"] / (ms["eval_planes"] * 1e-3) / 1e9
    # contouring passes: bytes they must move per job (state them in one place)
    V, T = nverts, ntris
    contour_bytes = (V * (32 + 32)            # vcompact: candidate read + vertex write (pos, nrm, key)
                     + 8.0 * N * N            # rowcnt + rowstart
                     + V * 8 + T * 12)        # quads: key read + triangle indices
    contour_ms = (ms["vcompact"] + ms["rowscan"] + ms["quads"]) / a.steps
    contour_gbs = contour_bytes / (contour_ms * 1e-3) / 1e9 if contour_ms > 0 else None
    if dom in ("eval_planes", "cells", "vertices"):
        # evaluation: bound by FP32 issue or by the SFU, whichever the SDF's op mix hits first
        sfu_peak = s2m.measure_sfu_peak(sp)
        per_launch_ms = ms["eval_planes"] / n_eval
        t_fp32 = fp32_ops / fp32_peak
        t_sfu = sfu_ops / sfu_peak if sfu_peak > 0 else 0.0
        tpp = eval_traffic_per_point(eval_ops["pruned"]) if a.workload == "csg64_1024" else None
        traffic = tpp * prof["eval_points"] / n_eval if tpp else None
        common = {"kernel": "s2m_tiles + s2m_evalp_*" if eval_ops["pruned"] else "s2m_eval_*",
                  "traffic": traffic, "traffic_source": (
                      "ncu dram__bytes_read.sum + dram__bytes_write.sum per lattice point from "
                      f"profiles/{EVAL_PROFILE[eval_ops['pruned']]}, scaled by points per launch")
                  if traffic else None,
                  "tile_pruning": eval_ops["pruned"],
                  "ms_per_launch": per_launch_ms,
                  "algorithmic": f"{fp32_ops:g} FP32 + {sfu_ops:g} SFU ops per lattice point x "
                                 f"{prof['eval_points'] / n_eval:.0f} points per launch",
                  "fp32_gops": eval_gops, "fp32_peak_gops": fp32_peak, "sfu_gops": eval_sfu,
                  "variant": variant, "per_point_ops_as_written": {"fp32": per_point_scalar[0], "sfu": per_point_scalar[1]},
                  "per_point_ops_executed": {"fp32": fp32_ops, "sfu": sfu_ops},
                  "executed_ops_source": ("tile pass: active segments' operations x points of each tile"
                                          if eval_ops["pruned"] else "frontend op count x points"),
                  "fp32_gops_as_written": scalar_equiv_gops,
                  "sfu_peak_gops": sfu_peak, "dominant_by_time": dom,
                  "peak_source": "measured in this run: s2m_fp32_probe (FP32 add/mul issue rate) and "
                                 "s2m_sfu_probe (MUFU rsqrt issue rate); MEASURED_PEAKS.json has neither"}
        jp = job_profile() if (eval_ops["pruned"] and a.workload == "csg64_1024" and N == 1024) else {}
        if t_sfu > t_fp32:
            roof = {"bound": "sfu", "achieved": eval_sfu, "peak": sfu_peak, "unit": "Gop/s",
                    "frac": eval_sfu / sfu_peak, **common}
        else:
            roof = {"bound": "fp32", "achieved": eval_gops, "peak": fp32_peak, "unit": "Gop/s",
                    "frac": eval_gops / fp32_peak, **common}
        if jp.get("eval_inst_per_job"):
            # Tile pruning leaves under one FP32 operation per lattice point: the phase is
            # bound by instruction issue (interval code, tests of the activity bits, IEEE
            # division and square-root sequences, point-bit stores), so its roofline is the
            # issue rate: warp instructions per second against 4 per SM and clock.
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
            t_job = ms["eval_planes"] / a.steps * 1e-3
            if mhz and t_job > 0:
                issue_peak = sms * 4 * mhz * 1e6 / 1e9
                achieved = jp["eval_inst_per_job"] / t_job / 1e9
                fp32_view = {"bound": roof["bound"], "achieved": roof["achieved"], "peak": roof["peak"],
                             "unit": roof["unit"], "frac": roof["frac"]}
                roof = {**common, "bound": "issue", "achieved": achieved, "peak": issue_peak,
                        "unit": "G warp-instructions/s", "frac": achieved / issue_peak,
                        "kernel": "s2m_tiles_coarse + s2m_tiles + s2m_fill_decided + s2m_evalpl_* (one job)",
                        "traffic": jp.get("eval_dram_bytes_per_job"),
                        "traffic_source": f"ncu dram__bytes_read.sum + dram__bytes_write.sum of the phase's "
                                          f"launches in one job (profiles/{JOB_PROFILE})",
                        "instructions_per_job": jp["eval_inst_per_job"],
                        "instructions_source": f"ncu smsp__inst_executed.sum of the phase's launches in one "
                                               f"job (profiles/{JOB_PROFILE})",
                        "achieved_unit_time": "CUDA events of the phase per step",
                        "peak_source": f"{sms} SMs x 4 warp schedulers x {mhz:.0f} MHz (median SM clock "
                                       "sampled during the timed steps)",
                        "fp32_view": fp32_view}
    else:
        roof = {"bound": "hbm", "kernel": dom, "achieved": contour_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": (contour_gbs or 0) / pk["hbm_gbs"], "peak_source": pk_kind, "traffic": None}
    contour = {"bound": "hbm", "achieved": contour_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
               "frac": (contour_gbs or 0) / pk["hbm_gbs"], "peak_source": f"{pk_kind} (MEASURED_PEAKS hbm_gbs)",
               "bytes_per_job": contour_bytes}

    cpu = None
    if not a.no_cpu_baseline:
        n = min(CPU_SAMPLE_SLICES if a.workload == "csg64_1024" else 4, N)
        z0 = max(0, min(CPU_Z0, N - n))
        dt, _ = cpu_sample(n, z0, N)
        cpu = {"value": n * N * N / dt / 1e9, "unit": UNIT, "cores": host_threads(), "kind": "port",
               "sample": f"CPU oracle (reference rule, binary32, OpenMP) on cell slices [{z0}, {z0 + n}) "
                         f"of the {N}^3 job: {n * N * N} voxels in {dt:.2f} s"}

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
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_tot / a.steps,
                "path": "s2m_mesh_create + s2m_mesh_copy_to_host (pinned: positions, normals, triangle indices, "
                        "the reference's TriangleMesh) + s2m_mesh_free; inputs are the "
                        "compiled SDF module and a 48-byte parameter block passed as kernel arguments"},
        "full_evaluation": full_eval,
        "roofline": roof,
        "roofline_contouring": contour,
        "kernels": kernels,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": launches_per_step * a.steps,
        "mesh": {"vertices": nverts, "triangles": ntris, "invalid_quads": int(info.invalid_quads),
                 "candidate_cells": int(info.candidate_cells), "slab_depth": int(info.slab_depth)},
        "compile_s": compile_s,
        "eval_variant": sdf.eval_variant()[0],
        "tile_pruning": {"combinators": prune_comb, "used": eval_ops["pruned"],
                         "fp32_ops_per_point": fp32_ops, "sfu_ops_per_point": sfu_ops,
                         "fp32_ops_per_point_as_written": per_point_scalar[0]},
        "eval_variants": [{"name": n, "ns_per_point": t, "registers": r, "local_bytes": l}
                          for n, t, r, l in sdf.eval_variants()],
        "triangles_per_s": ntris * a.steps * ws / (tot_ms * 1e-3),
        "wall_s_timed": wall,
    }
    print(json.dumps(line), flush=True)
    mesh.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Batching and serving workloads (spec changes (2) and (3)).


def batch_jobs(n=256, seed=4):
    from sdf2mesh_gb300 import workloads
    rng = workloads.SplitMix64(seed)
    jobs = []
    for i in range(n):
        src, prog = workloads.random_tree(i)
        N = workloads.log_uniform_resolution(rng)
        jobs.append((src, prog, N))
    return jobs


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


def batch_arm(a):
    import torch
    torch.cuda.set_device(0)
    import sdf2mesh_gb300 as s2m
    from sdf2mesh_gb300 import build as b
    b.build()
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
        bt.close()
        return dt, ms, launches

    for _ in range(a.warmup):
        one()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    res = [one() for _ in range(a.steps)]
    clk = clocks.stop()
    wall = sum(r[0] for r in res)
    dev_ms = sum(r[1] for r in res)
    launches = res[0][2]
    # plain per-job pipeline on a bounded sample of the same jobs (first 32)
    sample = jobs[:32]
    plain_compile = plain_per_job(sample)
    pre = [s2m.Sdf3DShader.from_source(src).compile() for src, _, _ in sample]
    plain_per_job(sample[:4], pre[:4])  # warm (autotune, pools)
    plain_mesh = plain_per_job(sample, pre)
    sample_vox = float(sum(N ** 3 for _, _, N in sample)) / len(sample)
    mps = len(jobs) * a.steps / wall
    line = {
        "metric": "meshes/s (batch of 256 CSG jobs)", "value": mps, "unit": "meshes/s", "n_gpus": 1,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": wall / a.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch256", "jobs": len(jobs), "sdf": WORKLOADS["batch256"][3], "bounds": 2.0,
                   "path": "s2m_batch_run: one persistent launch over a device work queue, CSG interpreter"},
        "gvoxels_per_s": voxels * a.steps / wall / 1e9,
        "device_ms_per_step": dev_ms / a.steps,
        "gpu_launches": launches * a.steps,
        "plain_per_job": {"meshes_per_s_with_compile": 1.0 / plain_compile, "meshes_per_s_precompiled": 1.0 / plain_mesh,
                          "sample": "first 32 jobs of the same list, mean voxels per job %.3g vs %.3g in the batch"
                                    % (sample_vox, voxels / len(jobs)),
                          "speedup_vs_with_compile": mps / (1.0 / plain_compile),
                          "speedup_vs_precompiled_same_mix": (voxels / len(jobs) / sample_vox) * mps / (1.0 / plain_mesh)},
        "e2e": {"value": mps, "unit": "meshes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def serve_requests(rate, n, seed):
    """Poisson arrivals at `rate` req/s: 90% random CSG trees, 10% Mandelbulbs."""
    import math
    from sdf2mesh_gb300 import workloads
    rng = workloads.SplitMix64(seed)
    t = 0.0
    reqs = []
    for i in range(n):
        t += -math.log(1.0 - rng.u01()) / rate
        N = int(round(math.exp(rng.uniform(math.log(64), math.log(1024)))))
        if rng.u01() < 0.1:
            reqs.append((t, "mandelbulb", None, None, N))
        else:
            src, prog = workloads.random_tree(int(rng.next() % 100000))
            reqs.append((t, "csg", src, prog, N))
    return reqs


def serve_arm(a):
    import torch
    torch.cuda.set_device(0)
    import sdf2mesh_gb300 as s2m
    from sdf2mesh_gb300 import build as b
    from sdf2mesh_gb300 import workloads
    b.build()
    mb_src, _ = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    rates = [10, 30, 100, 300, 1000, 2000]
    nreq = 48
    table = []

    def paced(reqs, t0):
        for r in reqs:
            d = t0 + r[0] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            yield r

    def state(kind, N):
        return s2m.AppState(resolution=N, bounds=2.5 if kind == "mandelbulb" else 2.0)

    for rate in rates:
        reqs = serve_requests(rate, nreq, seed=rate)
        # served: requests are source text (the plugin surface); CSG-shaped sources run on the
        # batch interpreter, the Mandelbulb GLSL compiles once and is cached
        server = s2m.Server(memory_budget_bytes=120 << 30, max_inflight=2, max_batch_jobs=64, keep_results=False)
        t0 = time.perf_counter()
        for (t, kind, src, prog, N) in paced(reqs, t0):
            if kind == "csg":
                server.submit_source(src, state(kind, N))
            else:
                server.submit_source(mb_src, state(kind, N), s2m.LANG_GLSL, "sdf")
        server.drain(3600)
        sst = server.stats()
        server.close()

        def plain(precompiled):
            lat = []
            t0 = time.perf_counter()
            for k, (t, kind, src, prog, N) in enumerate(paced(reqs, t0)):
                if precompiled is not None:
                    sdf = precompiled[k]
                elif kind == "csg":
                    sdf = s2m.Sdf3DShader.from_source(src).compile()
                else:
                    sdf = s2m.Sdf3DShader.from_source(mb_src, s2m.LANG_GLSL, "sdf").compile()
                m = s2m.mesh_device(sdf, state(kind, N))
                m.close()
                if precompiled is None:
                    sdf.close()
                lat.append((time.perf_counter() - t0 - t) * 1e3)
            span = time.perf_counter() - t0
            lat.sort()
            return {"meshes_per_s": len(reqs) / span, "p50_ms": lat[len(lat) // 2],
                    "p99_ms": lat[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))]}

        # plain per-job pipeline: one request at a time in arrival order, compiling its source
        p_compile = plain(None)
        # the same with every module compiled before the clock starts
        mods = {}
        pre = []
        for (t, kind, src, prog, N) in reqs:
            key = mb_src if kind == "mandelbulb" else src
            if key not in mods:
                mods[key] = (s2m.Sdf3DShader.from_source(mb_src, s2m.LANG_GLSL, "sdf") if kind == "mandelbulb"
                             else s2m.Sdf3DShader.from_source(src)).compile()
            pre.append(mods[key])
        p_pre = plain(pre)
        for m in mods.values():
            m.close()
        table.append({"rate": rate, "served": {"meshes_per_s": sst["meshes_per_s"], "p50_ms": sst["p50_ms"],
                                               "p99_ms": sst["p99_ms"], "launches": sst["batches"],
                                               "gvoxels_per_s": sst["gvoxels_per_s"],
                                               "peak_gb": sst["peak_bytes"] / 1e9},
                      "plain_per_job": p_compile, "plain_per_job_precompiled": p_pre,
                      "speedup": sst["meshes_per_s"] / p_compile["meshes_per_s"],
                      "speedup_vs_precompiled": sst["meshes_per_s"] / p_pre["meshes_per_s"]})
        print(json.dumps(table[-1]), file=sys.stderr, flush=True)
    top = table[-1]
    line = {
        "metric": "served meshes/s (Poisson stream, 2000 req/s offered)", "value": top["served"]["meshes_per_s"],
        "unit": "meshes/s", "n_gpus": 1, "steps": len(rates), "warmup": 0,
        "ms_per_step": 1e3 / max(1e-9, top["served"]["meshes_per_s"]), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serve", "requests_per_rate": nreq, "rates": rates, "sdf": WORKLOADS["serve"][3],
                   "served": "s2m_server_submit_source: requests are .sdf3d / GLSL text",
                   "plain_per_job": "one request at a time in arrival order: NVRTC compile of its source + "
                                    "s2m_mesh_create (and, beside it, the same with modules compiled beforehand)"},
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
