#!/usr/bin/env python3
"""Benchmark of the GB300 tessellation chain (one JSON line on stdout).

Workload (N=1): the batched scene — 256 instances of four procedural meshes of
uneven size (icosphere 5,120 / torus 12,288 / planar grid 32,768 / subdivided
cube 1,536 triangles; 3.31M base triangles, 51,840 clusters of <= 64
triangles), seeded transforms in a 40^3 box, 512^2 fp32 value-noise maps at
scale 0.03, camera orbiting at radius 30 over 60 frames, 1920x1080, 4 px per
segment (the reference's default tessRatePixels), frustum culling on. One step
= one frame of the chain (frame reset .. BLAS list insertion) recorded as a
CUDA graph of one persistent launch per stage.

  value : tessellated triangles per second (Readback.numTotalTriangles / frame
          time), frame inputs resident in HBM, CUDA events on the launching
          stream, L2 flushed (256 MiB write) between timed frames
  e2e   : same metric through the C ABI with host buffers
          (tc_frame_build_graph_host): per frame the FrameConstants pair and
          the RenderInstance array are read from pinned host memory and the
          Readback written back to it by kernels of the frame graph, inside
          the events (memcpy_variant: the same traffic by cudaMemcpyAsync
          around tc_frame_build_graph)
  roofline : the frame's dominant kernel, algorithmic bytes (metrics.py) over
          its CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline : the CPU oracle (C++ restatement of the reference shaders,
          all host cores) on a time-bounded sample of the same frames

--impl reference times that CPU restatement alone (the reference itself only
exists as Vulkan GLSL, which cannot run here).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NUM_ORBIT_FRAMES = 60
WORKLOAD = ("batched scene: 256 instances of 4 procedural meshes (icosphere 5120, torus 12288, grid 32768, "
            "cube 1536 tris; 3.31M base tris, 51840 clusters <=64 tris), 512^2 fp32 value-noise maps scale 0.03, "
            "orbit camera r=30 over 60 frames, 1920x1080, 4 px/segment, frustum culling on, split factor 8")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-extras", action="store_true", help="skip the plain-path and terrain measurements")
    p.add_argument("--no-tune", action="store_true", help="keep the default launch schedule (no autotuning)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--profile-case", choices=["batched", "batched_host", "terrain", "terrain_stages", "transient", "raster"],
                   default=None,
                   help="run only `warmup` + `steps` graph frames of one case (for ncu captures) and exit")
    return p.parse_args()


def replica_totals(seconds: float, tris: float, device):
    """Whole-job figures of N independent replicas (the path does not shard:
    every rank builds its own frames): the slowest rank's time and the sum of
    all ranks' tessellated triangles. Only these two numbers are exchanged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return seconds, tris
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([tris], dtype=torch.float64, device=device)
    dist.all_reduce(n)
    return float(t.item()), float(n.item())


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def _free_port() -> int:
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def spawn_replicas(cmd: list, n: int) -> int:
    """`bench.py --gpus N` started without torchrun: run `cmd` as N ranks, one
    per GPU (RANK / LOCAL_RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT set as
    torchrun would). The path does not shard, so the ranks are independent
    replicas that meet only for the barrier and the max / sum of the timing.
    Rank 0's output passes through; returns the worst exit code."""
    port = _free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen(cmd, env=env, stdout=None if r == 0 else subprocess.DEVNULL))
    return max(p.wait() for p in procs)


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9 and parts[1].isdigit():
                        rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        mhz = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": int(rows[0][2]), "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU oracle leg (reference arm and cpu_baseline)
# ---------------------------------------------------------------------------

def cpu_oracle_rate(seconds: float, threads: int | None = None):
    from oracle.binding import Oracle
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import scene as S
    threads = threads or os.cpu_count()
    ora = Oracle()
    scene = S.scene_batched(256)
    caps = L.default_caps()
    st = ora.new_state(scene, caps, L.FLAG_CULLING)
    fcs = [S.frame_constants(S.camera_orbit(f)) for f in range(NUM_ORBIT_FRAMES)]
    tris, frames = 0, 0
    t0 = time.perf_counter()
    while True:
        f = frames % NUM_ORBIT_FRAMES
        st, _ = ora.frame(scene, fcs[f], caps, L.FLAG_CULLING, threads=threads,
                          camera_last=fcs[(f - 1) % NUM_ORBIT_FRAMES], state=st)
        tris += int(st.readback.read(L.Readback, 1)[0]["numTotalTriangles"])
        frames += 1
        el = time.perf_counter() - t0
        if el >= seconds and frames >= 3:
            break
    return tris / el, el, frames, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    steps = []
    for _ in range(args.warmup):
        cpu_oracle_rate(0.0)
    tris_total, el_total, frames_total, threads = 0.0, 0.0, 0, os.cpu_count()
    for _ in range(args.steps):
        rate, el, frames, threads = cpu_oracle_rate(max(1.0, args.cpu_seconds / max(args.steps, 1)))
        steps.append(el / frames * 1e3)
        tris_total += rate * el
        el_total += el
        frames_total += frames
    value = tris_total / el_total
    line = {
        "metric": "tessellated tris/s", "value": value, "unit": "tris/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(steps), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural meshes and value-noise maps)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "step": "one frame on the CPU"},
        "cpu_baseline": {"value": value, "unit": "tris/s", "cores": threads, "kind": "port",
                         "sample": f"{frames_total} frames of the batched scene in {el_total:.1f} s; the reference "
                                   "has no CPU path and its GLSL needs Vulkan, so this is the C++ restatement"},
        "e2e": {"value": value, "unit": "tris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def recorded_traffic(key: str):
    """DRAM bytes (read + write) per launch of a stage, from the ncu capture
    summarised in profiles/traffic.txt (lines `<case>/<stage> <bytes>`), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 2 and parts[0] == key:
                return int(parts[1])
    return None


# What ncu shows limits each measured stage (profiles/: classify_batched.md,
# instantiate_parts_terrain.md); the roofline stays HBM bandwidth.
LIMITERS = {
    "batched/cluster_classify": "instruction issue and latency, not DRAM: the 256 instances share 4 meshes, so "
                                "the working set is L2-resident (DRAM 0.3-1.1 %); k_classify_count issue-bound "
                                "(67 % issue active), k_classify_full_vertices long-scoreboard-bound",
    "terrain/triangle_instantiate": "L1 data pipe and instruction issue in k_instantiate_parts (61 % issue "
                                    "active, LSU data pipe 73 %, DRAM 30 %), DRAM traffic below the "
                                    "algorithmic bytes",
}


def recorded_position_errors():
    """|GPU - FP64 twin| of the generated vertices per configuration, as the
    GPU parity tests measured them (profiles/position_error.txt, lines
    `<config> <max> <rms> <scene diagonal>`), or None."""
    path = os.path.join(ROOT, "profiles", "position_error.txt")
    if not os.path.exists(path):
        return None
    out = {}
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 4 and not line.startswith("#"):
                mx, rms, diag = (float(x) for x in parts[1:])
                out[parts[0]] = {"max": mx, "rms": rms, "scene_diagonal": diag, "max_over_diagonal": mx / diag}
    out["source"] = "tests/test_gpu_fullsize.py, tests/test_gpu_parity.py on a GB300 (profiles/position_error.txt)"
    return out


def stage_sequence(pipe, n_inst):
    from vk_tessellated_clusters_gb300 import layouts as L
    seq = [("frame_begin", ()), ("instances_classify", ()), ("clusters_cull", (0, n_inst)),
           ("build_setup", (L.BUILD_SETUP_CLASSIFY,)), ("cluster_classify", (0, n_inst)),
           ("build_setup", (L.BUILD_SETUP_SPLIT,))]
    passes = pipe.split_passes()
    for p in range(passes):
        seq.append(("triangle_split", (0, n_inst)))
        if p + 1 < passes:
            seq.append(("build_setup", (L.BUILD_SETUP_SPLIT_PASS,)))
    seq += [("build_setup", (L.BUILD_SETUP_INSTANTIATE_TESS,)), ("triangle_instantiate", (0, 0xFFFFFFFF)),
            ("build_setup", (L.BUILD_SETUP_BUILD_BLAS,)), ("blas_setup_insertion", ()), ("blas_clusters_insert", ())]
    return seq


def profile_stages(pipe, torch, frames, set_frame, flush, reps=1, read_outputs=True):
    """Per-stage CUDA-event durations (ms) over the given frames (and each
    frame's outputs, unless read_outputs is false)."""
    n_inst = pipe.args.numInstances
    seq = stage_sequence(pipe, n_inst)
    acc = {}
    outs = []
    for f in frames:
        set_frame(f)
        flush()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(seq) + 1)]
        evs[0].record()
        for i, (name, extra) in enumerate(seq):
            pipe.stage(name, *extra)
            evs[i + 1].record()
        torch.cuda.synchronize()
        for i, (name, _) in enumerate(seq):
            key = name if name not in ("build_setup", "triangle_split") else name
            acc.setdefault(key, []).append(evs[i].elapsed_time(evs[i + 1]))
        if read_outputs:
            outs.append(pipe.outputs())
    return acc, outs


def split_timings(pipe, torch, frames, set_frame, flush):
    """The split stage both ways on the same frames (CUDA events on the
    launching stream): every pass its own launch with the SPLIT_PASS set-up
    between (the reference's multipass dispatches) against all passes in one
    launch (tc_triangle_split_all, what the frame graph uses)."""
    from vk_tessellated_clusters_gb300 import layouts as L
    n = pipe.args.numInstances
    passes = pipe.split_passes()
    res = {"passes": passes, "per_pass_launches_ms": [], "one_launch_ms": []}
    for f in frames:
        for form in ("per_pass_launches_ms", "one_launch_ms"):
            set_frame(f)
            for name, extra in stage_sequence(pipe, n)[:6]:  # frame_begin .. BUILD_SETUP_SPLIT
                pipe.stage(name, *extra)
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            if form == "one_launch_ms":
                pipe.stage("triangle_split_all")
            else:
                for p in range(passes):
                    pipe.stage("triangle_split", 0, n)
                    if p + 1 < passes:
                        pipe.stage("build_setup", L.BUILD_SETUP_SPLIT_PASS)
            e1.record()
            torch.cuda.synchronize()
            res[form].append(e0.elapsed_time(e1))
    res["per_pass_launches_samples"] = list(res["per_pass_launches_ms"])
    res["one_launch_samples"] = list(res["one_launch_ms"])
    res["per_pass_launches_ms"] = statistics.median(res["per_pass_launches_ms"])
    res["one_launch_ms"] = statistics.median(res["one_launch_ms"])
    b = pipe.state.build.read(L.SceneBuilding, 1)[0]
    res["split_items"] = int(b["splitWriteCounter"])
    return res


def run_ours(args):
    import torch
    from vk_tessellated_clusters_gb300 import build_lib, native
    if not os.path.exists(native.LIB_PATH):
        build_lib.build()
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import metrics as M
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    scene = S.scene_batched(256)
    caps = L.default_caps()
    flags = L.FLAG_CULLING
    pipe = TessellationPipeline(scene, caps, flags, device=local)

    # all orbit frames' constants resident on the device; a step copies its pair in
    fcs = [S.frame_constants(S.camera_orbit(f)) for f in range(NUM_ORBIT_FRAMES)]
    import numpy as np
    fc_bytes = np.stack([np.frombuffer(fc.tobytes(), np.uint8) for fc in fcs])
    fc_dev = torch.from_numpy(fc_bytes).to(dev)
    view_t = pipe.state.view.handle
    last_t = pipe.state.view_last.handle
    FC = L.FrameConstants.itemsize

    def set_frame(f):
        view_t[:FC].copy_(fc_dev[f % NUM_ORBIT_FRAMES])
        last_t[:FC].copy_(fc_dev[(f - 1) % NUM_ORBIT_FRAMES])

    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def flush():
        flush_buf.fill_(1)

    rb_host = torch.empty(L.Readback.itemsize, dtype=torch.uint8, pin_memory=True)

    def read_tris():
        rb_host.copy_(pipe.state.readback.handle[:L.Readback.itemsize])
        return int(rb_host.numpy().view(L.Readback)[0]["numTotalTriangles"])

    # ---- launch schedule: autotuned on six orbit frames (outside the timing) ---
    tune_report = None
    if not args.no_tune:
        from vk_tessellated_clusters_gb300.autotune import autotune
        _, tune_report = autotune(pipe, list(range(0, NUM_ORBIT_FRAMES, NUM_ORBIT_FRAMES // 6)), set_frame, flush)

    # ---- warm-up --------------------------------------------------------------
    for s in range(args.warmup):
        set_frame(s)
        pipe.build("graph")
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    # ---- timed region: K frames, graph replay, L2 flushed between frames -------
    launches0 = pipe.launch_count()
    times, tris = [], []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for s in range(args.steps):
            set_frame(args.warmup + s)
            # the L2 flush runs right before the frame, so the GPU is busy while
            # the host submits the start event and the graph: the events see
            # the frame's device time, not the host's submission latency
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            pipe.build("graph")
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
            tris.append(read_tris())
        torch.cuda.synchronize()
    gpu_launches = pipe.launch_count() - launches0
    if world > 1:
        torch.distributed.barrier()
    t_total = sum(times) / 1e3
    tris_total = float(sum(tris))
    t_total, tris_total = replica_totals(t_total, tris_total, dev)
    value = tris_total / t_total
    errs = pipe.device_errors()

    # ---- e2e through the C ABI with host buffers ------------------------------
    # A frame's inputs (its FrameConstants, the previous frame's, the instance
    # records) sit side by side in one block: the application's per-frame data
    # (pageable) is written into one pinned staging block, which the frame
    # moves into one device block that the frame arguments point into.
    inst_rec = pipe.state.res.instance_records.view(np.uint8).reshape(-1)
    blk = 2 * FC + inst_rec.size
    host_np = np.empty((NUM_ORBIT_FRAMES, blk), np.uint8)
    for f in range(NUM_ORBIT_FRAMES):
        host_np[f, :FC] = fc_bytes[f]
        host_np[f, FC:2 * FC] = fc_bytes[(f - 1) % NUM_ORBIT_FRAMES]
        host_np[f, 2 * FC:] = inst_rec
    stage = torch.empty(blk, dtype=torch.uint8, pin_memory=True)
    stage_np = stage.numpy()
    dev_block = torch.empty(blk + 256, dtype=torch.uint8, device=dev)
    base = (dev_block.data_ptr() + 255) // 256 * 256  # RenderInstance records 16-byte aligned (FC is a multiple of 16)
    off = base - dev_block.data_ptr()
    fa = pipe.state.args
    saved_ptrs = (fa.view, fa.viewLast, fa.instances)
    fa.view, fa.viewLast, fa.instances = base, base + FC, base + 2 * FC
    h2d = blk

    def e2e_run(step):
        times_, tris_ = [], []
        for s in range(args.warmup + args.steps):
            f = s % NUM_ORBIT_FRAMES
            flush()  # before the step, as in the device-resident loop
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            stage_np[:] = host_np[f]
            step()
            e1.record()
            e1.synchronize()
            if s >= args.warmup:
                times_.append(e0.elapsed_time(e1))
                tris_.append(int(rb_host.numpy().view(L.Readback)[0]["numTotalTriangles"]))
        return times_, tris_

    # the public call: the frame graph reads the input block from pinned host
    # memory and writes the Readback to pinned host memory itself
    e2e_times, e2e_tris = e2e_run(lambda: pipe.build_host(stage.data_ptr(), base, blk, rb_host.data_ptr()))
    e2e_value = sum(e2e_tris) / (sum(e2e_times) / 1e3)

    # the same traffic through the copy engines (cudaMemcpyAsync each way) around tc_frame_build_graph
    def memcpy_step():
        dev_block[off:off + blk].copy_(stage, non_blocking=True)
        pipe.build("graph")
        rb_host.copy_(pipe.state.readback.handle[:L.Readback.itemsize], non_blocking=True)

    mc_times, mc_tris = e2e_run(memcpy_step)
    fa.view, fa.viewLast, fa.instances = saved_ptrs

    # ---- per-stage profile and roofline of the dominant kernel ---------------------
    prof_frames = list(range(0, NUM_ORBIT_FRAMES, max(1, NUM_ORBIT_FRAMES // 6)))[:6]
    stage_ms, outs = profile_stages(pipe, torch, prof_frames, set_frame, flush)
    means = {k: statistics.mean(v) for k, v in stage_ms.items()}
    main_stages = {k: v for k, v in means.items() if k not in ("build_setup", "frame_begin")}
    dominant = max(main_stages, key=main_stages.get)
    byte_fn = {"cluster_classify": lambda o: M.classify_bytes(o, scene),
               "triangle_instantiate": lambda o: M.instantiate_bytes(o, pipe.entries, scene)}
    peak, peak_kind = measured_peak_hbm()
    roof = None
    if dominant in byte_fn:
        alg = statistics.mean(byte_fn[dominant](o) for o in outs)
        achieved = alg / (means[dominant] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes_per_launch": alg,
                "launch_ms": means[dominant], "traffic": recorded_traffic(f"batched/{dominant}"),
                "limiter": LIMITERS.get(f"batched/{dominant}")}
    inst_alg = statistics.mean(M.instantiate_bytes(o, pipe.entries, scene) for o in outs)
    stage_gbs = {"cluster_classify": statistics.mean(M.classify_bytes(o, scene) for o in outs)
                 / (means["cluster_classify"] / 1e3) / 1e9,
                 "triangle_instantiate": inst_alg / (means["triangle_instantiate"] / 1e3) / 1e9}

    result = {
        "metric": "tessellated tris/s", "value": value, "unit": "tris/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural meshes and value-noise maps)",
        "config": {"workload": WORKLOAD, "instances": 256, "base_triangles": scene.total_triangles,
                   "clusters": scene.total_clusters, "tessellated_tris_per_frame": statistics.mean(tris),
                   "l2": "flushed between timed frames (256 MiB write)", "mode": "CUDA graph, batched persistent stages",
                   "schedule": pipe.schedule(), "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": "tris/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": L.Readback.itemsize, "ms_per_step": statistics.mean(e2e_times),
                "call": "tc_frame_build_graph_host",
                "memcpy_variant": {"value": sum(mc_tris) / (sum(mc_times) / 1e3),
                                   "ms_per_step": statistics.mean(mc_times)}},
        "gpu_launches": gpu_launches,
        "clocks": clk.summary(),
        "roofline": roof,
        "stages_ms": means,
        "stage_gbs": stage_gbs,
        "device_errors": errs,
        "position_error_vs_fp64": recorded_position_errors(),
        "autotune": tune_report,
    }

    if not args.no_extras:
        result["batched_vs_plain"] = batched_vs_plain(pipe, torch, set_frame, flush)
        pipe.close()
        del pipe
        torch.cuda.empty_cache()
        result["terrain"] = terrain_bandwidth(torch, dev, local, peak, tune=not args.no_tune)
        t = result["terrain"]
        # the instantiate stage of the bandwidth configuration, beside the headline's dominant kernel
        inst = {"kernel": "triangle_instantiate", "workload": t["workload"],
                "bound": "hbm", "achieved": t["instantiate_gbs"], "peak": peak, "unit": "GB/s",
                "frac": t["instantiate_frac_of_peak"], "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": t["instantiate_algorithmic_bytes"],
                "launch_ms": t["stages_ms"]["triangle_instantiate"], "schedule": t["instantiate_schedule"],
                "traffic": recorded_traffic("terrain/triangle_instantiate"),
                "limiter": LIMITERS.get("terrain/triangle_instantiate")}
        if result["roofline"] is not None:
            result["roofline"]["instantiate_terrain"] = inst
        torch.cuda.empty_cache()
        result["backward_forward"] = backward_forward(torch, dev, local)
        torch.cuda.empty_cache()
        result["hit_decode"] = hit_decode(torch, local, peak)
        torch.cuda.empty_cache()
        result["frame_variants"] = frame_variants(torch, local, result["config"]["schedule"])
        torch.cuda.empty_cache()
        result["raster_batches"] = raster_batches(torch, local, peak)
        torch.cuda.empty_cache()
        result["animation"] = animation_fwd_bwd(torch, dev, local, result["config"]["schedule"])
    if rank == 0:
        result["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(result))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def batched_vs_plain(pipe, torch, set_frame, flush, frames=(3, 17, 31)):
    out = {}
    for mode in ("graph", "batched", "plain"):
        ts = []
        for f in frames:
            set_frame(f)
            pipe.build(mode)  # warm
            torch.cuda.synchronize()
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = pipe.launch_count()
            e0.record()
            pipe.build(mode)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
            out[f"{mode}_launches"] = pipe.launch_count() - l0
        out[f"{mode}_ms"] = statistics.mean(ts)
    out["plain_over_graph"] = out["plain_ms"] / out["graph_ms"]
    out["outputs_identical"] = "checked by tests/test_gpu_parity.py (batched, graph, plain byte-identical)"
    return out


def terrain_bandwidth(torch, dev, local, peak, tune=True):
    """Large bandwidth case: HBM GB/s of the instantiate stage on the terrain,
    with its own autotuned launch schedule (its split passes and vertex counts
    differ from the batched scene's)."""
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import metrics as M
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    scene = S.scene_terrain()
    caps = terrain_caps()
    pipe = TessellationPipeline(scene, caps, L.FLAG_CULLING, device=local)
    pipe.set_cameras(S.camera_terrain())
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    pipe.build("graph")
    torch.cuda.synchronize()
    tune_report = None
    flush = lambda: flush_buf.fill_(1)  # noqa: E731
    if tune:
        from vk_tessellated_clusters_gb300.autotune import autotune
        _, tune_report = autotune(pipe, [0, 0, 0], lambda f: None, flush)
    frame_sched = pipe.schedule()
    # the instantiate stage's own launch shape (the frame's tuning weighs it
    # against the concurrent split passes): its grid and register fields
    stage_sched, stage_search = frame_sched, None
    if tune:
        stage_sched, stage_search = tune_instantiate_stage(pipe, torch, flush, frame_sched)
    pipe.set_schedule(stage_sched)
    stage_ms, outs = profile_stages(pipe, torch, [0, 0, 0], lambda f: None, flush)
    pipe.set_schedule(frame_sched)
    means = {k: statistics.mean(v) for k, v in stage_ms.items()}
    o = outs[-1]
    alg = M.instantiate_bytes(o, pipe.entries, scene)
    gbs = alg / (means["triangle_instantiate"] / 1e3) / 1e9
    res = {"workload": "terrain 1024x1024 quads (2,097,152 tris), 4096^2 fp16 fBm 8 octaves, scale 0.1 extent, "
                       "camera 10 deg grazing at height 2, 3840x2160, 4 px/segment",
           "tessellated_tris": int(o["readback"]["numTotalTriangles"]),
           "part_triangles": int(o["readback"]["numPartTriangles"]),
           "classify_part_triangles": M.classify_parts_written(o),
           "split_triangles": int(o["readback"]["numSplitTriangles"]),
           "generated_vertices": int(o["readback"]["numGenVertices"]),
           "stages_ms": means, "instantiate_algorithmic_bytes": alg, "instantiate_gbs": gbs,
           "instantiate_frac_of_peak": gbs / peak,
           "schedule": frame_sched, "autotune": tune_report,
           "instantiate_schedule": stage_sched, "instantiate_search": stage_search,
           "frame_ms_graph": None}
    frame_ms = []
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush_buf.fill_(1)
        e0.record()
        pipe.build("graph")
        e1.record()
        torch.cuda.synchronize()
        frame_ms.append(e0.elapsed_time(e1))
    res["frame_ms_graph"] = statistics.median(frame_ms)
    res["tris_per_s"] = res["tessellated_tris"] / (res["frame_ms_graph"] / 1e3)
    res["split"] = split_timings(pipe, torch, [0, 0, 0], lambda f: None, lambda: flush_buf.fill_(1))
    res["device_errors"] = pipe.device_errors()
    pipe.close()
    return res


INSTANTIATE_SPACE = {"vertexBlocksPerSM": (4, 5, 6), "vertexGridPerSM": (0, 8, 16), "scanBlocksPerSM": (4, 8, 16)}


def tune_instantiate_stage(pipe, torch, flush, base):
    """Grid search of the fields the instantiate stage's launches read, on the
    per-stage entry points (mean of three frames each, L2 flushed): the
    best schedule and the search's record."""
    import itertools
    best, best_ms, trials = dict(base), None, 0
    keys = sorted(INSTANTIATE_SPACE)
    for vals in itertools.product(*(INSTANTIATE_SPACE[k] for k in keys)):
        sched = dict(base, **dict(zip(keys, vals)))
        pipe.set_schedule(sched)
        ms, _ = profile_stages(pipe, torch, [0, 0, 0], lambda f: None, flush, read_outputs=False)
        t = statistics.mean(ms["triangle_instantiate"])
        trials += 1
        if best_ms is None or t < best_ms:
            best, best_ms = sched, t
    pipe.set_schedule(base)
    return best, {"space": INSTANTIATE_SPACE, "trials": trials, "best_ms": best_ms}


def hit_decode(torch, local, peak, n=1 << 20, reps=20):
    """Hit-time decode (tc_decode_hits) of 2^20 seeded hits on a batched-scene
    frame (orbit frame 0), hits and results resident on the device: hits/s and
    the algorithmic GB/s (24 B hit read, 40 B result written, per part hit its
    24 B part record, per hit the 16 B cluster header and 3 index bytes)."""
    import numpy as np
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.hits import sample_hits
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    scene = S.scene_batched(256)
    pipe = TessellationPipeline(scene, L.default_caps(), L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS, device=local)
    pipe.set_cameras(S.camera_orbit(0))
    pipe.build("graph")
    out = pipe.outputs()
    hits = sample_hits(out, scene, pipe.entries, n, seed=3)
    dev = f"cuda:{pipe.device}"
    d_hits = torch.from_numpy(hits.view(np.uint8).reshape(-1).copy()).to(dev)
    d_out = torch.empty(n * L.BaseHit.itemsize, dtype=torch.uint8, device=dev)
    for _ in range(3):
        pipe.decode_hits_device(d_hits, d_out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        pipe.decode_hits_device(d_hits, d_out)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    parts = int(np.count_nonzero((hits["clusterID"] >> 30) == L.RT_CLUSTER_MODE_SINGLE_TESSELLATED))
    alg = n * (24 + 40 + 16 + 3) + parts * 24
    ok = int(np.count_nonzero(d_out.cpu().numpy().view(L.BaseHit)["status"] == L.HIT_OK))
    pipe.close()
    return {"hits": n, "part_hits": parts, "ms": ms, "hits_per_s": n / (ms / 1e3),
            "algorithmic_gbs": alg / (ms / 1e3) / 1e9, "frac_of_peak": alg / (ms / 1e3) / 1e9 / peak,
            "decoded_ok": ok, "l2": "hits and results (67 MB) stay in L2 across the timed launches",
            "parity": "tests/test_gpu_parity.py::test_hit_decode_matches_oracle (field-exact vs oracle)"}


def raster_batches(torch, local, peak, reps=20):
    """tc_raster_batches on a batched-scene frame (256 instances, orbit frame
    0): parts batched per second and the algorithmic GB/s (per part its 24 B
    record, base attributes (3 x 32 B) and per vertex 28 B written (world +
    clip), per triangle 7 B written), outputs resident on the device."""
    import ctypes
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import native
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    pipe = TessellationPipeline(S.scene_batched(256), L.default_caps(), L.FLAG_CULLING, device=local)
    pipe.set_cameras(S.camera_orbit(0))
    pipe.build("graph")
    res = pipe.raster_batches()
    ro, _ = pipe.state.raster_outputs()

    def launch():
        native.check(pipe.lib.tc_raster_batches(pipe.ctx, ctypes.byref(pipe.args), ctypes.byref(ro), pipe.stream()),
                     "tc_raster_batches")

    for _ in range(3):
        launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.current_stream())
    for _ in range(reps):
        launch()
    e1.record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nb, nv, nt = res["counts"]
    parts = int(res["batches"]["partCount"].sum()) if nb else 0
    alg = parts * (24 + 96) + nv * 28 + nt * 7
    errs = pipe.device_errors()
    pipe.close()
    return {"parts": parts, "batches": nb, "vertices": nv, "triangles": nt, "ms": ms,
            "parts_per_s": parts / (ms / 1e3), "algorithmic_gbs": alg / (ms / 1e3) / 1e9,
            "frac_of_peak": alg / (ms / 1e3) / 1e9 / peak, "device_errors": errs,
            "parity": "tests/test_gpu_parity.py::test_raster_batches_match_oracle"}


def frame_variants(torch, local, schedule, frames=(3, 17, 31)):
    """The batched scene's frame (256 instances, graph replay, L2 flushed)
    with the reference's optional shader paths on: PN-triangle displacement
    with the ripple animation (amplitude 0.02, frequency 8, speed 1.5), 1X and
    2X transient builds, and all of them (the reference's ray-tracing
    defaults), against the same frames without: ms per frame and triangles per
    second of each."""
    import statistics as st
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    scene = S.scene_batched(256)
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    trans = L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X
    out = {}
    for name, extra in (("plain_flags", 0), ("pn_ripple", L.FLAG_PN | L.FLAG_RIPPLE), ("transient", trans),
                        ("pn_ripple_transient", L.FLAG_PN | L.FLAG_RIPPLE | trans)):
        pipe = TessellationPipeline(scene, L.default_caps(), L.FLAG_CULLING | extra, device=local)
        pipe.set_schedule(schedule)
        ts, tris, builds = [], [], []
        for f in frames:
            fc = S.frame_constants(S.camera_orbit(f))
            fc["animationRippleAmplitude"], fc["animationRippleFrequency"] = 0.02, 8.0
            fc["animationRippleSpeed"], fc["animationState"] = 1.5, 0.1 * f
            pipe.set_cameras(fc, S.camera_orbit(f - 1))
            for _ in range(3):
                pipe.build("graph")
            torch.cuda.synchronize()
            flush_buf.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            pipe.build("graph")
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
            rb = pipe.outputs()["readback"]
            tris.append(int(rb["numTotalTriangles"]))
            builds.append(int(rb["numTransBuilds"]))
        assert pipe.device_errors() == 0
        pipe.close()
        ms = st.mean(ts)
        out[name] = {"ms": ms, "tris_per_s": st.mean(tris) / (ms / 1e3), "transient_builds": st.mean(builds)}
    for name in ("pn_ripple", "transient", "pn_ripple_transient"):
        out[name]["over_plain_flags"] = out[name]["ms"] / out["plain_flags"]["ms"]
    out["parity"] = ("tests/test_gpu_parity.py::test_pn_and_ripple_bit_exact, ::test_transient_builds_bit_exact "
                     "(integers bit-exact, positions within tolerance)")
    return out


def backward_forward(torch, dev, local, reps=10):
    """Differentiation case: the icosphere frame (20,480 triangles, 1024^2 fp32
    4-octave value noise, scale 0.05, camera at distance 3, 8 px/segment) with
    its tessellation decisions frozen; L = sum |v - t|^2 with t from a map of
    another seed. Times the frozen forward (vertex generation), the backward
    (gradient scatter into positions, normals and all texels) and the full
    frame build, with CUDA events."""
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.autograd import FrozenFrame, tessellate
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    scene = S.scene_icosphere()
    caps = L.default_caps(visible_bits=12, part_bits=18, split_bits=14, vertex_bits=21, megs=256)
    pipe = TessellationPipeline(scene, caps, L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS, device=local)
    pipe.set_cameras(S.camera_icosphere())
    pipe.build("graph")
    frozen = FrozenFrame(pipe)
    tex = frozen.texels[0]
    orig = tex.detach().clone()
    with torch.no_grad():
        tex.copy_(torch.from_numpy(S.value_noise(1024, 4, seed=1)).to(dev))
    target = frozen.generate()
    with torch.no_grad():
        tex.copy_(orig)
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(fn):
        ts = []
        for i in range(reps + 2):
            flush_buf.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            if i >= 2:
                ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    def timed_back_to_back(fn, n=20):
        """Device time per call with `n` calls enqueued back to back (the host
        runs ahead, so launch latency is hidden as in a training loop)."""
        ts = []
        for i in range(reps // 2 + 2):
            flush_buf.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(n):
                fn()
            e1.record()
            torch.cuda.synchronize()
            if i >= 2:
                ts.append(e0.elapsed_time(e1) / n)
        return statistics.median(ts)

    grad_v = 2 * (frozen.generate() - target)
    fwd_ms = timed(lambda: pipe.stage("generate_vertices"))
    _, table = frozen.gradient_buffers(dev)
    bwd_kernel_ms = timed(lambda: frozen.launch_backward(grad_v, table))
    bwd_ms = timed(lambda: frozen.scatter_gradients(grad_v))
    fwd_b2b = timed_back_to_back(lambda: frozen.generate())
    bwd_b2b = timed_back_to_back(lambda: frozen.scatter_gradients(grad_v))
    frame_ms = timed(lambda: pipe.build("graph"))
    # one autograd step end to end for the record
    v = tessellate(frozen)
    loss = ((v - target) ** 2).sum()
    loss.backward()
    res = {"workload": "icosphere 20,480 tris, 1024^2 fp32 value-noise map, decisions frozen, L = sum |v - t|^2",
           "vertices": frozen.num_vertices, "forward_ms": fwd_ms, "backward_kernel_ms": bwd_kernel_ms,
           "backward_ms": bwd_ms, "frame_build_ms": frame_ms,
           "backward_kernel_over_forward": bwd_kernel_ms / fwd_ms, "backward_over_forward": bwd_ms / fwd_ms,
           "forward_autograd_back_to_back_ms": fwd_b2b, "backward_autograd_back_to_back_ms": bwd_b2b,
           "backward_over_forward_back_to_back": bwd_b2b / fwd_b2b,
           "backward_over_frame_build": bwd_ms / frame_ms,
           "loss": float(loss.item()), "device_errors": pipe.device_errors(),
           "gradient_check": "tests/test_gpu_backward.py: rel. error vs FP64 adjoint <= 1e-4, 64-parameter central differences"}
    pipe.close()
    return res


def animation_fwd_bwd(torch, dev, local, schedule, frames=300, plain_frames=6):
    """Batched differentiable animation: 1,024 instances of the four batched
    meshes with seeded rigid motion (omega U[0,1] rad/s, speed U[0,2] units/s)
    at 60 frames/s over `frames` frames, orbit camera, frustum culling. A
    frame = this frame's instance records and camera copied in (device to
    device), then one CUDA graph replay of the whole forward frame plus the
    zeroing of the four 512^2 fp32 map gradients and the backward with
    dL/dv = v (L = 0.5 * sum |v|^2). Latency per frame with CUDA events, L2
    flushed between frames; the same frames through per-instance launches for
    `plain_frames` frames."""
    import numpy as np
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    scene = S.scene_batched(1024)
    caps = L.default_caps()
    pipe = TessellationPipeline(scene, caps, L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS, device=local)
    if schedule:
        pipe.set_schedule(schedule)
    motion = S.animation_motion(len(scene.instances))
    base_recs = pipe.state.res.instance_records
    recs = np.repeat(base_recs[None], frames, axis=0)
    for f in range(frames):
        W = S.animated_worlds(scene, motion, f / 60.0)
        recs[f]["worldMatrix"] = np.transpose(W, (0, 2, 1)).reshape(len(W), 16).astype(np.float32)
    rec_bytes = base_recs.nbytes
    recs_dev = torch.from_numpy(recs.view(np.uint8).reshape(frames, rec_bytes)).to(dev)
    fcs = np.stack([np.frombuffer(S.frame_constants(S.camera_orbit(f % NUM_ORBIT_FRAMES)).tobytes(), np.uint8)
                    for f in range(NUM_ORBIT_FRAMES)])
    fc_dev = torch.from_numpy(fcs).to(dev)
    FC = L.FrameConstants.itemsize
    inst_t, view_t, last_t = pipe.state.res.instances.handle, pipe.state.view.handle, pipe.state.view_last.handle

    def set_frame(f):
        inst_t[:rec_bytes].copy_(recs_dev[f])
        view_t[:FC].copy_(fc_dev[f % NUM_ORBIT_FRAMES])
        last_t[:FC].copy_(fc_dev[(f - 1) % NUM_ORBIT_FRAMES])

    map_floats = [t.texels.size for t in scene.textures]
    grads = torch.zeros(sum(map_floats), dtype=torch.float32, device=dev)
    starts = np.concatenate([[0], np.cumsum(map_floats)[:-1]])
    tex_ptrs = torch.tensor([grads.data_ptr() + 4 * int(o) for o in starts], dtype=torch.int64, device=dev)
    targets = torch.zeros(2 * len(scene.instances), dtype=torch.int64, device=dev)  # no position/normal grads
    gv = pipe.state.gen_vertices.addr

    def fwd_bwd(mode):
        pipe.build(mode)
        grads.zero_()
        pipe.backward(gv, targets.data_ptr(), tex_ptrs.data_ptr())

    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    rb = pipe.state.readback

    # capture forward + gradient zeroing + backward as one graph
    set_frame(0)
    fwd_bwd("batched")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fwd_bwd("batched")
    torch.cuda.synchronize()

    def timed_frames(run, frame_ids):
        lat, tris = [], []
        for f in frame_ids:
            flush_buf.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            set_frame(f)
            run()
            e1.record()
            torch.cuda.synchronize()
            lat.append(e0.elapsed_time(e1))
            tris.append(int(rb.read(L.Readback, 1)[0]["numTotalTriangles"]))
        return lat, tris

    for f in range(3):  # warm-up
        set_frame(f)
        g.replay()
    torch.cuda.synchronize()
    lat, tris = timed_frames(g.replay, range(frames))
    errs = pipe.device_errors()
    plain_ids = list(range(0, frames, frames // plain_frames))[:plain_frames]
    plat, ptris = timed_frames(lambda: fwd_bwd("plain"), plain_ids)
    same = [tris[f] for f in plain_ids] == ptris
    grad_norm = float(grads.norm().item())
    pipe.close()
    q = lambda v, p: float(np.percentile(np.asarray(v), p))
    return {"workload": "1,024 instances of the 4 batched meshes (13.2M base tris), seeded rigid motion "
                        "(omega U[0,1] rad/s, speed U[0,2] units/s, 60 frames/s), orbit camera 1920x1080, "
                        "culling on; forward frame + backward into 4 x 512^2 fp32 maps, L = 0.5 sum |v|^2",
            "frames": frames, "graph_p50_ms": q(lat, 50), "graph_p99_ms": q(lat, 99),
            "graph_tris_per_s": sum(tris) / (sum(lat) / 1e3),
            "tessellated_tris_per_frame": {"min": min(tris), "max": max(tris)},
            "plain_frames": len(plat), "plain_p50_ms": q(plat, 50), "plain_p99_ms": q(plat, 99),
            "plain_tris_per_s": sum(ptris) / (sum(plat) / 1e3),
            "plain_over_graph_p50": q(plat, 50) / q([lat[f] for f in plain_ids], 50),
            "plain_same_triangle_counts": same, "texel_grad_norm": grad_norm, "device_errors": errs,
            "l2": "flushed between frames (256 MiB write)"}


def cpu_baseline(args):
    rate, el, frames, threads = cpu_oracle_rate(args.cpu_seconds)
    return {"value": rate, "unit": "tris/s", "cores": threads, "kind": "port",
            "sample": f"{frames} frames of the batched scene ({el:.1f} s, {threads} threads)"}


def terrain_caps():
    from vk_tessellated_clusters_gb300 import layouts as L
    return L.default_caps(visible_bits=16, part_bits=21, split_bits=18, vertex_bits=25, megs=2048)


def run_profile_case(args):
    """A short, fixed sequence of frames of one case: the command ncu captures."""
    import numpy as np
    import torch
    from vk_tessellated_clusters_gb300 import layouts as L
    from vk_tessellated_clusters_gb300 import scene as S
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    flags = L.FLAG_CULLING
    if args.profile_case in ("batched", "batched_host", "transient", "raster"):
        scene, caps = S.scene_batched(256), L.default_caps()
        cams = [S.camera_orbit(f) for f in range(args.warmup + args.steps)]
        if args.profile_case == "transient":
            flags |= L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X
    else:
        scene, caps = S.scene_terrain(), terrain_caps()
        cams = [S.camera_terrain()] * (args.warmup + args.steps)
    pipe = TessellationPipeline(scene, caps, flags)
    host_io = args.profile_case == "batched_host"
    if host_io:
        # the e2e form: frame constants and instance records from one pinned
        # staging block, the Readback to pinned host memory (tc_frame_build_graph_host)
        FC = L.FrameConstants.itemsize
        rec = pipe.state.res.instance_records.view(np.uint8).reshape(-1)
        blk = 2 * FC + rec.size
        stage = torch.empty(blk, dtype=torch.uint8, pin_memory=True)
        stage_np = stage.numpy()
        stage_np[2 * FC:] = rec
        dev_block = torch.empty(blk + 256, dtype=torch.uint8, device="cuda")
        base = (dev_block.data_ptr() + 255) // 256 * 256
        rb_host = torch.empty(L.Readback.itemsize, dtype=torch.uint8, pin_memory=True)
        fa = pipe.args
        fa.view, fa.viewLast, fa.instances = base, base + FC, base + 2 * FC
    for i, cam in enumerate(cams):
        if host_io:
            torch.cuda.synchronize()  # the previous frame has read the staging block
            stage_np[:FC] = np.frombuffer(S.frame_constants(cam).tobytes(), np.uint8)
            stage_np[FC:2 * FC] = np.frombuffer(S.frame_constants(cams[i - 1] if i else cam).tobytes(), np.uint8)
            pipe.build_host(stage.data_ptr(), base, blk, rb_host.data_ptr())
            continue
        pipe.set_cameras(cam, cams[i - 1] if i else cam)
        if args.profile_case == "terrain_stages":  # the per-stage entry points, as the bench's stage timings run them
            for name, extra in stage_sequence(pipe, pipe.args.numInstances):
                pipe.stage(name, *extra)
        else:
            pipe.build("graph")
        if args.profile_case == "raster":
            pipe.raster_batches()
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": args.profile_case, "frames": len(cams), "device_errors": pipe.device_errors(),
                      "readback_tris": int(pipe.state.readback.read(L.Readback, 1)[0]["numTotalTriangles"]),
                      "host_readback_tris": int(rb_host.numpy().view(L.Readback)[0]["numTotalTriangles"]) if host_io
                      else None}))
    pipe.close()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ and not args.profile_case:
        return spawn_replicas([sys.executable, os.path.abspath(__file__)] + sys.argv[1:], args.gpus)
    if args.profile_case:
        return run_profile_case(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
