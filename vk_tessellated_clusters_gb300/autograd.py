"""Differentiable displaced-vertex generation through torch.autograd.

The tessellation decisions of a built frame (segment counts, configs, split
tree, instantiation order) are piecewise constant in the inputs, so they are
held fixed: the differentiable function maps base positions, base normals and
displacement texels to the frame's generated vertices

    part triangle : v = P(w) + normalize(N(w)) * (bilinear(tex, uv(w)) * s + o)
    full cluster  : v = p + normalize(n) * (bilinear(tex, uv) * s + o)

(triangle_tess_template_instantiate.comp.glsl:343-371,
cluster_classify.comp.glsl:457-482), with forward tc_generate_vertices and
backward tc_instantiate_backward (CUDA kernels). The parameters are views of
the pipeline's own device buffers, so in-place updates (an optimiser step) are
seen by the next frame.

    frozen = FrozenFrame(pipe)               # after pipe.build(...) with FLAG_WRITE_FULLCLUSTERS
    v = tessellate(frozen)                    # (num_vertices, 3) float32
    loss = ((v - target) ** 2).sum(); loss.backward()
    frozen.positions[0].grad, frozen.normals[0].grad, frozen.texels[0].grad
"""
from __future__ import annotations

import numpy as np

from . import layouts as L


class FrozenFrame:
    def __init__(self, pipe):
        import torch
        self.torch = torch
        if not (pipe.state.flags & L.FLAG_WRITE_FULLCLUSTERS):
            raise ValueError("the frame must be built with FLAG_WRITE_FULLCLUSTERS")
        self.pipe = pipe
        torch.cuda.synchronize(pipe.device)
        out = pipe.state
        self.num_vertices = self._accepted_vertex_count()
        scene = pipe.scene
        res = out.res
        self.positions = [self._view(b["positions"], g.positions.shape) for b, g in zip(res.geo, scene.geometries)]
        self.normals = [self._view(b["normals"], g.normals.shape) for b, g in zip(res.geo, scene.geometries)]
        self.texels = []
        for buf, t in zip(res.tex, scene.textures):
            if t.format != L.TEXEL_F32:
                self.texels.append(None)  # only fp32 maps are differentiable parameters
            else:
                self.texels.append(buf.handle[:t.texels.nbytes].view(torch.float32).view(t.texels.shape))
        for p in self.parameters():
            p.requires_grad_(True)
        self._inst_geo = np.array([i.geometry for i in scene.instances], np.int64)
        self._layout_gradients(scene)

    def _layout_gradients(self, scene) -> None:
        """All gradients of one backward live in one flat float32 buffer; the
        kernel's pointer tables (per instance dPositions/dNormals, per map
        texels) point into it once and for all, so a backward is a zero fill,
        the kernel and one copy out, with no host-to-device transfer."""
        torch = self.torch
        sizes = [p.numel() for p in self.positions] + [n.numel() for n in self.normals]
        sizes += [t.numel() if t is not None else 0 for t in self.texels]
        starts = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self._grad_floats = int(starts[-1])
        self._grad_starts = starts
        ng = len(self.positions)
        rel = np.zeros((len(self._inst_geo), 2), np.int64)
        rel[:, 0] = 4 * starts[self._inst_geo]
        rel[:, 1] = 4 * starts[ng + self._inst_geo]
        tex = np.array([4 * starts[2 * ng + i] if t is not None else -1 for i, t in enumerate(self.texels)] or [-1],
                       np.int64)
        self._num_targets = rel.size
        # one persistent gradient buffer and its pointer table (built once);
        # every backward zeroes it, accumulates into it and hands out a copy
        self._flat = torch.zeros(self._grad_floats, dtype=torch.float32, device=self.pipe.device)
        base = self._flat.data_ptr()
        table = np.concatenate([rel.reshape(-1), tex])
        table = np.where(table >= 0, table + base, 0).astype(np.int64)
        self._table = torch.from_numpy(table).to(self.pipe.device)

    def _view(self, buf, shape):
        n = int(np.prod(shape))
        return buf.handle[:4 * n].view(self.torch.float32).view(*shape)

    def _accepted_vertex_count(self) -> int:
        out = self.pipe.outputs()
        return len(out["genVertices"])

    def parameters(self) -> list:
        return [p for p in self.positions + self.normals + self.texels if p is not None]

    # ---- forward / backward on the C ABI ------------------------------------------------

    def generate(self):
        """Vertices of the frozen frame from the current parameters (a copy)."""
        self.pipe.stage("generate_vertices")
        return self.pipe.gen_vertices_tensor(self.num_vertices).clone()

    def gradient_buffers(self, device=None):
        """The persistent flat float32 gradient buffer, zeroed (enqueued on the
        current stream), and the kernel's pointer table into it."""
        self._flat.zero_()
        return self._flat, self._table

    def launch_backward(self, grad_vertices, table) -> None:
        """tc_instantiate_backward: accumulates dL/dv into the buffer `table` points at."""
        self.pipe.backward(grad_vertices.data_ptr(), table.data_ptr(), table.data_ptr() + 8 * self._num_targets)

    def scatter_gradients(self, grad_vertices):
        """dL/dv -> (dPositions, dNormals, dTexels), lists parallel to the
        parameters; all enqueued on the current stream, no synchronisation."""
        buf, table = self.gradient_buffers()
        self.launch_backward(grad_vertices.contiguous().float(), table)
        flat = buf.clone()
        st = self._grad_starts
        ng = len(self.positions)
        views = [flat[st[i]:st[i + 1]] for i in range(len(st) - 1)]
        dP = [views[i].view(p.shape) for i, p in enumerate(self.positions)]
        dN = [views[ng + i].view(n.shape) for i, n in enumerate(self.normals)]
        dT = [views[2 * ng + i].view(t.shape) if t is not None else None for i, t in enumerate(self.texels)]
        return dP, dN, dT


class _Tessellate:
    """torch.autograd.Function, built lazily so importing this module needs no torch."""
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            import torch

            class TessellateFunction(torch.autograd.Function):
                @staticmethod
                def forward(ctx, frozen, *params):
                    ctx.frozen = frozen
                    return frozen.generate()

                @staticmethod
                def backward(ctx, grad):
                    f = ctx.frozen
                    dP, dN, dT = f.scatter_gradients(grad)
                    grads = []
                    for p, g in zip(f.positions, dP):
                        grads.append(g)
                    for n, g in zip(f.normals, dN):
                        grads.append(g)
                    for t, g in zip(f.texels, dT):
                        if t is not None:
                            grads.append(g)
                    return (None, *grads)

            cls.fn = TessellateFunction
        return cls.fn


def tessellate(frozen: FrozenFrame):
    return _Tessellate.get().apply(frozen, *frozen.parameters())
