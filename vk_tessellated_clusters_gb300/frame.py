"""Frame buffers in the reference's buffer protocol, in host or device memory.

``FrameState`` carves the buffers a frame of the tessellation chain reads and
writes (the reference's BufferRanges carving, src/renderer_raytrace_clusters_tess.cpp:200-310),
fills a SceneBuilding with their addresses and assembles the tc_frame_args.
The same code builds the host-memory variant handed to the CPU oracle (every
address a host pointer) and the device-memory variant handed to the CUDA
library, so both see identical inputs.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import layouts as L
from .scene import Scene, instance_records

# Base address of the CLAS destination memory. The chain only computes
# addresses inside it (tempClusterAddresses = genClusterData + offset); the
# memory itself is written by the CLAS build, which is out of scope.
GEN_CLUSTER_DATA_BASE = 0x6000_0000_0000


class Buf:
    """One allocation: ``addr`` is what goes into the protocol structs."""

    def __init__(self, mem, nbytes, handle, addr):
        self.mem, self.nbytes, self.handle, self.addr = mem, nbytes, handle, addr

    def read(self, dtype, count=None, offset=0) -> np.ndarray:
        dtype = np.dtype(dtype)
        if count is None:
            count = (self.nbytes - offset) // dtype.itemsize
        return self.mem.read(self, offset, count * dtype.itemsize).view(dtype)

    def write(self, arr, offset=0) -> None:
        self.mem.write(self, np.ascontiguousarray(arr).view(np.uint8).reshape(-1), offset)


class HostMemory:
    """numpy-backed buffers (addresses are host pointers)."""

    def alloc(self, nbytes: int, fill: int = 0) -> Buf:
        a = np.full(max(int(nbytes), 16) + 256, fill, np.uint8)
        off = (-a.ctypes.data) % 256
        v = a[off:off + max(int(nbytes), 16)]
        return Buf(self, int(nbytes), v, v.ctypes.data)

    def upload(self, arr: np.ndarray) -> Buf:
        raw = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
        b = self.alloc(raw.size)
        b.handle[:raw.size] = raw
        return b

    def read(self, buf: Buf, offset: int, nbytes: int) -> np.ndarray:
        return buf.handle[offset:offset + nbytes].copy()

    def write(self, buf: Buf, raw: np.ndarray, offset: int) -> None:
        buf.handle[offset:offset + raw.size] = raw


class DeviceMemory:
    """torch CUDA tensors (uint8) as plain device memory."""

    def __init__(self, device=0):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", device) if isinstance(device, int) else torch.device(device)

    def alloc(self, nbytes: int, fill: int = 0) -> Buf:
        t = self.torch.full((max(int(nbytes), 16),), fill, dtype=self.torch.uint8, device=self.device)
        return Buf(self, int(nbytes), t, t.data_ptr())

    def upload(self, arr: np.ndarray) -> Buf:
        raw = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
        b = self.alloc(raw.size)
        if raw.size:
            b.handle[:raw.size].copy_(self.torch.from_numpy(raw.copy()))
        return b

    def read(self, buf: Buf, offset: int, nbytes: int) -> np.ndarray:
        return buf.handle[offset:offset + nbytes].cpu().numpy()

    def write(self, buf: Buf, raw: np.ndarray, offset: int) -> None:
        if raw.size:
            buf.handle[offset:offset + raw.size].copy_(self.torch.from_numpy(raw.copy()))


class SceneResources:
    """Geometry, displacement maps and the RenderInstance array in one memory space."""

    def __init__(self, scene: Scene, mem):
        self.scene = scene
        self.geo = []
        addrs = []
        for g in scene.geometries:
            bufs = dict(positions=mem.upload(g.positions), normals=mem.upload(g.normals),
                        texcoords=mem.upload(g.texcoords), clusters=mem.upload(g.clusters),
                        clusterLocalTriangles=mem.upload(g.local_triangles), clusterBboxes=mem.upload(g.bboxes),
                        clusterTemplateAdresses=mem.upload(g.template_addresses),
                        clusterTemplateInstantiatonSizes=mem.upload(g.template_sizes))
            self.geo.append(bufs)
            addrs.append({k: v.addr for k, v in bufs.items()})
        self.tex = [mem.upload(t.texels) for t in scene.textures]
        trec = np.zeros(max(len(scene.textures), 1), L.DisplacementTexture)
        for i, t in enumerate(scene.textures):
            trec[i] = (self.tex[i].addr, t.texels.shape[1], t.texels.shape[0], t.format, 0)
        self.textures = mem.upload(trec)
        self.instance_records = instance_records(scene, addrs)
        self.instances = mem.upload(self.instance_records)

    def set_world_matrices(self, worlds) -> None:
        """Per-frame instance transforms (row-major 4x4 each)."""
        from .scene import mat_colmajor
        for i, w in enumerate(worlds):
            self.instance_records[i]["worldMatrix"] = mat_colmajor(w)
        self.instances.write(self.instance_records)


class FrameState:
    """All per-frame buffers plus the SceneBuilding and tc_frame_args."""

    def __init__(self, scene: Scene, mem, caps: dict, flags: int = L.FLAG_CULLING):
        self.mem, self.caps, self.flags = mem, dict(caps), int(flags)
        self.res = SceneResources(scene, mem)
        n = len(scene.instances)
        k = self.caps
        self.view = mem.alloc(L.FrameConstants.itemsize)
        self.view_last = mem.alloc(L.FrameConstants.itemsize)
        self.readback = mem.alloc(L.Readback.itemsize)
        self.instance_states = mem.alloc(4 * n)
        self.visible_clusters = mem.alloc(L.ClusterInfo.itemsize * k["maxVisibleClusters"])
        self.full_clusters = mem.alloc(L.ClusterInfo.itemsize * k["maxGeneratedClusters"])
        self.split_triangles = mem.alloc(L.TessTriangleInfo.itemsize * k["maxSplitTriangles"])
        self.part_triangles = mem.alloc(L.TessTriangleInfo.itemsize * k["maxPartTriangles"])
        self.gen_vertices = mem.alloc(12 * k["maxGeneratedVertices"])
        self.temp_instance_ids = mem.alloc(4 * k["maxGeneratedClusters"])
        self.temp_instantiations = mem.alloc(L.TemplateInstantiateInfo.itemsize * k["maxGeneratedClusters"])
        self.temp_cluster_addresses = mem.alloc(8 * k["maxGeneratedClusters"])
        self.temp_cluster_sizes = mem.alloc(4 * k["maxGeneratedClusters"])
        self.blas_build_infos = mem.alloc(L.BlasBuildInfo.itemsize * n)
        self.blas_build_sizes = mem.alloc(4 * n)
        self.blas_cluster_addresses = mem.alloc(8 * k["maxGeneratedClusters"])
        sb = np.zeros((), L.SceneBuilding)
        sb["numRenderInstances"] = n
        sb["instanceStates"] = self.instance_states.addr
        sb["visibleClusters"] = self.visible_clusters.addr
        sb["fullClusters"] = self.full_clusters.addr
        sb["splitTriangles"] = self.split_triangles.addr
        sb["partTriangles"] = self.part_triangles.addr
        sb["genClusterData"] = GEN_CLUSTER_DATA_BASE
        sb["genVertices"] = self.gen_vertices.addr
        sb["tempInstanceIDs"] = self.temp_instance_ids.addr
        sb["tempInstantiations"] = self.temp_instantiations.addr
        sb["tempClusterAddresses"] = self.temp_cluster_addresses.addr
        sb["tempClusterSizes"] = self.temp_cluster_sizes.addr
        sb["blasBuildInfos"] = self.blas_build_infos.addr
        sb["blasBuildSizes"] = self.blas_build_sizes.addr
        sb["blasClusterAddresses"] = self.blas_cluster_addresses.addr
        self.transient = bool(self.flags & (L.FLAG_TRANSIENT_1X | L.FLAG_TRANSIENT_2X))
        if self.transient:
            from .scene import basic_cluster_sizes
            g = k["maxGeneratedClusters"]
            self.trans_instance_ids = mem.alloc(4 * g)
            self.trans_builds = mem.alloc(L.ClasBuildInfo.itemsize * g)
            self.trans_cluster_addresses = mem.alloc(8 * g)
            self.trans_cluster_sizes = mem.alloc(4 * g)
            self.basic_cluster_sizes = mem.upload(basic_cluster_sizes())
            sb["transInstanceIDs"] = self.trans_instance_ids.addr
            sb["transBuilds"] = self.trans_builds.addr
            sb["transClusterAddresses"] = self.trans_cluster_addresses.addr
            sb["transClusterSizes"] = self.trans_cluster_sizes.addr
            sb["basicClusterSizes"] = self.basic_cluster_sizes.addr
            # the index and map bytes alias the vertex and part arrays (shaderio_building.h:240-246)
            sb["transTriMappings"] = self.part_triangles.addr
            sb["transTriIndices"] = self.gen_vertices.addr
        self.scene_building_host = sb
        self.build = mem.upload(sb)
        self.args = L.FrameArgs()
        self.args.view = self.view.addr
        self.args.viewLast = self.view_last.addr
        self.args.instances = self.res.instances.addr
        self.args.build = self.build.addr
        self.args.readback = self.readback.addr
        self.args.textures = self.res.textures.addr if scene.textures else 0
        self.args.numInstances = n
        self.args.numTextures = len(scene.textures)
        self.args.totalClusters = scene.total_clusters
        self.args.flags = self.flags
        self.args.caps = L.caps_from(self.caps)

    def raster_outputs(self, parts: int | None = None):
        """Output buffers for tc_raster_batches, sized for `parts` part
        triangles (default: the built frame's; at most one batch per part, 78
        vertices and 121 triangles each)."""
        if parts is None:
            parts = min(int(self.scene_building()["partTriangleCounter"]), self.caps["maxPartTriangles"])
        n = max(1, int(parts))
        if getattr(self, "_raster", None) is None or self._raster_parts < n:
            self._raster_parts = n
            mv, mt = 78 * n, L.RASTER_BATCH_TRIANGLES * n
            bufs = {"batches": self.mem.alloc(L.RasterBatch.itemsize * n), "counts": self.mem.alloc(16),
                    "clipPositions": self.mem.alloc(16 * mv), "worldPositions": self.mem.alloc(12 * mv),
                    "indices": self.mem.alloc(3 * mt), "primitiveIDs": self.mem.alloc(4 * mt)}
            ro = L.RasterOutputs()
            for k, b in bufs.items():
                setattr(ro, k, b.addr)
            ro.maxBatches, ro.maxVertices, ro.maxTriangles = n, mv, mt
            self._raster = (ro, bufs)
        return self._raster

    def raster_results(self) -> dict:
        """The last tc_raster_batches results, cut to the written counts."""
        _, bufs = self._raster
        nb, nv, nt = (int(x) for x in bufs["counts"].read(np.uint32, 3))
        return {"counts": (nb, nv, nt), "batches": bufs["batches"].read(L.RasterBatch, nb),
                "clipPositions": bufs["clipPositions"].read(np.float32, 4 * nv).reshape(-1, 4),
                "worldPositions": bufs["worldPositions"].read(np.float32, 3 * nv).reshape(-1, 3),
                "indices": bufs["indices"].read(np.uint8, 3 * nt).reshape(-1, 3),
                "primitiveIDs": bufs["primitiveIDs"].read(np.uint32, nt)}

    def set_cameras(self, fc_now: np.ndarray, fc_last: np.ndarray | None = None) -> None:
        self.view.write(fc_now)
        self.view_last.write(fc_now if fc_last is None else fc_last)

    # ---- readout ---------------------------------------------------------------

    def scene_building(self) -> np.ndarray:
        return self.build.read(L.SceneBuilding, 1)[0]

    def outputs(self, entries: np.ndarray | None = None) -> dict:
        """Compacted frame outputs; addresses rebased to offsets so host and
        device runs compare directly."""
        sb = self.scene_building()
        n = len(self.res.scene.instances)
        k = self.caps
        out = {"build": sb, "readback": self.readback.read(L.Readback, 1)[0],
               "instanceStates": self.instance_states.read(np.uint32, n)}
        nvis = min(int(sb["visibleClusterCounter"]), k["maxVisibleClusters"])
        out["visibleClusters"] = self.visible_clusters.read(L.ClusterInfo, nvis)
        out["splitTriangles"] = self.split_triangles.read(L.TessTriangleInfo, k["maxSplitTriangles"])
        nparts = min(int(sb["partTriangleCounter"]), k["maxPartTriangles"])
        out["partTriangles"] = self.part_triangles.read(L.TessTriangleInfo, nparts)
        ntemp = min(int(sb["tempInstantiateCounter"]), k["maxGeneratedClusters"])
        ti = self.temp_instantiations.read(L.TemplateInstantiateInfo, ntemp).copy()
        ti["vertexBufferAddress"] -= np.uint64(self.gen_vertices.addr)
        out["tempInstantiations"] = ti
        out["tempInstanceIDs"] = self.temp_instance_ids.read(np.uint32, ntemp)
        out["tempClusterAddresses"] = self.temp_cluster_addresses.read(np.uint64, ntemp)
        if self.flags & L.FLAG_WRITE_FULLCLUSTERS:
            nfull = int(np.count_nonzero((ti["clusterIdOffset"] >> 30) == 0))
            out["fullClusters"] = self.full_clusters.read(L.ClusterInfo, nfull)
        bi = self.blas_build_infos.read(L.BlasBuildInfo, n).copy()
        bi["clusterReferences"] -= np.uint64(self.blas_cluster_addresses.addr)
        out["blasBuildInfos"] = bi
        out["blasClusterAddresses"] = self.blas_cluster_addresses.read(np.uint64, int(sb["blasClusterCounter"]))
        # generated vertices of the accepted instantiations (accepted items form a prefix)
        nverts = 0
        if ntemp:
            last = ti[ntemp - 1]
            base = int(last["vertexBufferAddress"]) // 12
            if (int(last["clusterIdOffset"]) >> 30) == 0:
                # full cluster: its vertex count is the cluster's
                nverts = base + self._full_cluster_vertices(out, ntemp - 1)
            else:
                if entries is None:
                    from .table import load_raw_table, lookup_entries
                    entries = lookup_entries(load_raw_table())
                part = out["partTriangles"][int(last["clusterIdOffset"]) & 0x3FFFFFFF]
                nverts = base + int(entries[(int(part["triangleID_config"]) >> 16) & 0x7FFF]["numVertices"])
        if not self.transient:
            out["genVertices"] = self.gen_vertices.read(np.float32, 3 * nverts).reshape(-1, 3)
            return out
        # transient builds: their records, the back slots of partTriangles and
        # the index bytes after their vertices (in build order); genVertices
        # keeps only vertex slots (a batch's unused slots are zeros), every
        # other byte (index bytes, rejected allocations) reads as zero
        ntr = min(int(sb["transBuildCounter"]), k["maxGeneratedClusters"])
        tb = self.trans_builds.read(L.ClasBuildInfo, ntr).copy()
        tb["vertexBuffer"] -= np.uint64(self.gen_vertices.addr)
        tb["indexBuffer"] -= np.uint64(self.gen_vertices.addr)
        out["transBuilds"] = tb
        out["transInstanceIDs"] = self.trans_instance_ids.read(np.uint32, ntr)
        out["transClusterAddresses"] = self.trans_cluster_addresses.read(np.uint64, ntr)
        ranges = []  # (first vertex, vertex count)
        for j in range(ntemp):
            base = int(ti[j]["vertexBufferAddress"]) // 12
            if (int(ti[j]["clusterIdOffset"]) >> 30) == 0:
                ranges.append((base, self._full_cluster_vertices(out, j)))
            else:
                if entries is None:
                    from .table import load_raw_table, lookup_entries
                    entries = lookup_entries(load_raw_table())
                part = out["partTriangles"][int(ti[j]["clusterIdOffset"]) & 0x3FFFFFFF]
                ranges.append((base, int(entries[(int(part["triangleID_config"]) >> 16) & 0x7FFF]["numVertices"])))
        parts_raw = self.part_triangles.read(np.uint8, L.TessTriangleInfo.itemsize * k["maxPartTriangles"])
        tparts, tidx = [], []
        for r in tb:
            mode, poff = int(r["clusterID"]) >> 30, int(r["clusterID"]) & 0x3FFFFFFF
            ntri, nv = int(r["packed"]) & 0x1FF, (int(r["packed"]) >> 9) & 0x1FF
            slots = 3 if mode == L.RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED else (8 + ntri + 23) // 24
            tparts.append(parts_raw[24 * poff:24 * (poff + slots)])
            ibytes = 96 if mode == L.RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED else (ntri * 3 + 11) // 12 * 12
            tidx.append((int(r["indexBuffer"]), ibytes))
            ranges.append((int(r["vertexBuffer"]) // 12, nv))
        out["transParts"] = np.concatenate(tparts) if tparts else np.zeros(0, np.uint8)
        end = max([a + n for a, n in ranges] + [(o + n + 11) // 12 for o, n in tidx] + [0])
        raw = self.gen_vertices.read(np.uint8, 12 * end)
        out["transIndices"] = (np.concatenate([raw[o:o + n] for o, n in tidx]) if tidx else np.zeros(0, np.uint8))
        keep = np.zeros(end, bool)
        for a, n in ranges:
            keep[a:a + n] = True
        gv = raw.view(np.float32).reshape(-1, 3).copy()
        gv[~keep] = 0
        out["genVertices"] = gv
        return out

    def _full_cluster_vertices(self, out, j) -> int:
        scene = self.res.scene
        inst = int(out["tempInstanceIDs"][j])
        g = scene.geometries[scene.instances[inst].geometry]
        addr = int(out["tempInstantiations"][j]["clusterTemplateAddress"])
        # template addresses are unique per cluster of a geometry (scene._finish)
        cid = int(np.flatnonzero(g.template_addresses == np.uint64(addr))[0])
        return int(g.clusters[cid]["numVertices"])


def args_ptr(args: L.FrameArgs):
    return ctypes.byref(args)
