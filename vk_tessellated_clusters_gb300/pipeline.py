"""GPU tessellation pipeline on the C ABI: the host-side mirror of the
reference renderer's compute part (RendererRayTraceClustersTess::init/render,
src/renderer_raytrace_clusters_tess.cpp:166-692 without the CLAS/BLAS builds).

    pipe = TessellationPipeline(scene, caps)
    pipe.set_cameras(camera)
    pipe.build()            # batched: one persistent launch per stage
    pipe.build("graph")     # same, recorded once as a CUDA graph and replayed
    pipe.build("plain")     # every stage launched once per instance
    out = pipe.outputs()
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import layouts as L
from . import native
from .frame import DeviceMemory, FrameState
from .scene import Camera, Scene, frame_constants
from .table import load_raw_table, lookup_entries, synthetic_templates


class TessellationPipeline:
    def __init__(self, scene: Scene, caps: dict | None = None, flags: int = L.FLAG_CULLING, device: int = 0,
                 schedule: dict | None = None):
        import torch
        self.torch = torch
        if not torch.cuda.is_available():
            raise RuntimeError("TessellationPipeline needs a CUDA device (sm_103a)")
        self.lib = native.lib()
        self.device = device
        self.scene = scene
        self.caps = dict(caps or L.default_caps())
        self.flags = flags
        self.mem = DeviceMemory(device)
        self.state = FrameState(scene, self.mem, self.caps, flags)
        desc = L.ContextDesc()
        desc.maxInstances = len(scene.instances)
        desc.maxTotalClusters = scene.total_clusters
        desc.caps = L.caps_from(self.caps)
        desc.device = device
        ctx = ctypes.c_void_p()
        native.check(self.lib.tc_context_create(ctypes.byref(desc), ctypes.byref(ctx)), "tc_context_create")
        self.ctx = ctx
        raw = load_raw_table()
        self.raw_table = raw
        self.entries = lookup_entries(raw)
        info = L.TableInfoC()
        native.check(self.lib.tc_table_init(ctx, raw.vertices.ctypes.data, raw.vertices.size, raw.triangles.ctypes.data,
                                            raw.triangles.size, raw.configs.ctypes.data, raw.num_configs,
                                            raw.max_edge_segments, ctypes.byref(info)), "tc_table_init")
        self.table_info = info
        addr, size = synthetic_templates(self.entries)
        self._tmpl = (addr, size)
        native.check(self.lib.tc_table_set_templates(ctx, addr.ctypes.data, size.ctypes.data, self.stream()),
                     "tc_table_set_templates")
        if schedule:
            self.set_schedule(schedule)

    # ---- plumbing -------------------------------------------------------------

    def stream(self) -> int:
        return self.torch.cuda.current_stream(self.device).cuda_stream

    @property
    def args(self) -> L.FrameArgs:
        return self.state.args

    def set_schedule(self, sched: dict) -> None:
        s = L.Schedule()
        cur = self.schedule()
        for k in L.SCHEDULE_FIELDS:
            setattr(s, k, int(sched.get(k, cur[k])))
        native.check(self.lib.tc_set_schedule(self.ctx, ctypes.byref(s)), "tc_set_schedule")

    def schedule(self) -> dict:
        s = L.Schedule()
        native.check(self.lib.tc_get_schedule(self.ctx, ctypes.byref(s)), "tc_get_schedule")
        return {k: getattr(s, k) for k in L.SCHEDULE_FIELDS}

    def set_cameras(self, now: Camera | np.ndarray, last: Camera | np.ndarray | None = None) -> None:
        fc = now if isinstance(now, np.ndarray) else frame_constants(now)
        fl = fc if last is None else (last if isinstance(last, np.ndarray) else frame_constants(last))
        self.state.set_cameras(fc, fl)

    # ---- frame -----------------------------------------------------------------

    def build(self, mode: str = "batched") -> None:
        fn = {"batched": self.lib.tc_frame_build, "graph": self.lib.tc_frame_build_graph,
              "plain": self.lib.tc_frame_build_plain}[mode]
        native.check(fn(self.ctx, ctypes.byref(self.args), self.stream()), f"tc_frame_build ({mode})")

    def build_host(self, host_inputs: int, device_inputs: int, nbytes: int, host_readback: int) -> None:
        """The graph frame with its host traffic inside the graph
        (tc_frame_build_graph_host): `nbytes` from the pinned host block at
        `host_inputs` to the device block at `device_inputs` before the frame
        (the frame args may point into it), the Readback to the pinned host
        buffer at `host_readback` after it."""
        native.check(self.lib.tc_frame_build_graph_host(self.ctx, ctypes.byref(self.args), host_inputs, device_inputs,
                                                        nbytes, host_readback, self.stream()),
                     "tc_frame_build_graph_host")

    def stage(self, name: str, *extra) -> None:
        f = getattr(self.lib, "tc_" + name)
        native.check(f(self.ctx, ctypes.byref(self.args), *extra, self.stream()), name)

    def split_passes(self) -> int:
        return int(self.lib.tc_split_pass_count(self.caps["splitFactor"]))

    def launch_count(self) -> int:
        return int(self.lib.tc_launch_count(self.ctx))

    def device_errors(self) -> int:
        bits = ctypes.c_uint32()
        native.check(self.lib.tc_read_device_errors(self.ctx, ctypes.byref(bits), self.stream()), "tc_read_device_errors")
        return bits.value

    def lookback_probe(self, published: bool) -> int:
        """tc_lookback_probe: one bounded look-back wait for a predecessor that
        is published (returns its prefix, 7) or never is (the wait runs out
        after the schedule's lookbackSpinLimit polls and returns 0)."""
        out = ctypes.c_uint64()
        native.check(self.lib.tc_lookback_probe(self.ctx, 1 if published else 0, ctypes.byref(out), self.stream()),
                     "tc_lookback_probe")
        return out.value

    def outputs(self) -> dict:
        self.torch.cuda.synchronize(self.device)
        return self.state.outputs(self.entries)

    def gen_vertices_tensor(self, count: int):
        """Device view of the first `count` generated vertices (float32, N x 3)."""
        t = self.state.gen_vertices.handle[:12 * count]
        return t.view(self.torch.float32).view(-1, 3)

    def decode_hits_device(self, hits, out) -> None:
        """tc_decode_hits on device tensors: `hits` uint8 (n x 24 B), `out` uint8 (n x 40 B)."""
        n = hits.numel() // L.Hit.itemsize
        native.check(self.lib.tc_decode_hits(self.ctx, ctypes.byref(self.args), hits.data_ptr(), n, out.data_ptr(),
                                             self.stream()), "tc_decode_hits")

    def decode_hits(self, hits: np.ndarray) -> np.ndarray:
        """Decode cluster-ray-tracing hits (L.Hit records) against the last built
        frame into base-mesh hits (L.BaseHit records)."""
        torch = self.torch
        hits = np.ascontiguousarray(hits, dtype=L.Hit)
        d_hits = torch.from_numpy(hits.view(np.uint8).reshape(-1).copy()).to(f"cuda:{self.device}")
        d_out = torch.empty(len(hits) * L.BaseHit.itemsize, dtype=torch.uint8, device=f"cuda:{self.device}")
        self.decode_hits_device(d_hits, d_out)
        return d_out.cpu().numpy().view(L.BaseHit)

    def raster_batches(self) -> dict:
        """tc_raster_batches on the last built frame: batch records, vertices in
        world and clip space, batch-local indices and primitive IDs."""
        ro, _ = self.state.raster_outputs()
        native.check(self.lib.tc_raster_batches(self.ctx, ctypes.byref(self.args), ctypes.byref(ro), self.stream()),
                     "tc_raster_batches")
        self.torch.cuda.synchronize(self.device)
        return self.state.raster_results()

    def backward(self, grad_vertices, grad_targets_addr: int, grad_texels_addr: int) -> None:
        native.check(self.lib.tc_instantiate_backward(self.ctx, ctypes.byref(self.args), int(grad_vertices),
                                                      int(grad_targets_addr), int(grad_texels_addr), self.stream()),
                     "tc_instantiate_backward")

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.torch.cuda.synchronize(self.device)
            self.lib.tc_context_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
