"""Synthetic, seeded scenes in the reference's cluster format.

The reference loads glTF meshes and clusterizes them with meshoptimizer
(src/scene.cpp:393-552), neither of which is part of the tessellation path.
Here procedural meshes stand in for the glTF scenes and a small clusterizer of
our own (spatially sorted greedy packing, <= 64 triangles / <= 64 vertices per
cluster, per-cluster vertex duplication as in src/scene.cpp:519-552) produces
the same data layout: cluster headers, 8-bit cluster-local triangle indices,
per-cluster vertex ranges and bounding boxes. Displacement maps are seeded,
tileable value noise / fBm in [0, 1].

Everything here is deterministic for a given seed and uses only elementwise
IEEE arithmetic, so the same inputs are produced on any host.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import layouts as L


def _libm(fn, *xs) -> np.ndarray:
    """Elementwise libm function. numpy's SIMD kernels for some
    transcendental functions (arctan2, arccos, arcsin) round differently on
    hosts with and without AVX-512, which would make the generated scenes,
    and every output digest over them, depend on the machine."""
    return np.vectorize(fn, otypes=[np.float64])(*xs)


# The small linear algebra below is written out with a fixed operation order
# (separate IEEE multiplies and adds) instead of BLAS / LAPACK, whose kernels
# use FMA or other summation orders depending on the host CPU.
def _norm3(v) -> float:
    x, y, z = (float(t) for t in v)
    return math.sqrt(x * x + y * y + z * z)


def _dot3(a, b) -> float:
    return float(a[0]) * float(b[0]) + float(a[1]) * float(b[1]) + float(a[2]) * float(b[2])


def _row_norms(v: np.ndarray) -> np.ndarray:
    """Euclidean norms of the rows of an (n, 3) array, in the array's dtype."""
    sq = v * v
    return np.sqrt(sq[:, 0] + sq[:, 1] + sq[:, 2])


def _mm(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Matrix product over the last two axes (batched), terms summed in k order."""
    out = a[..., :, 0, None] * b[..., 0, None, :]
    for k in range(1, a.shape[-1]):
        out = out + a[..., :, k, None] * b[..., k, None, :]
    return out


def _inv4(m: np.ndarray) -> np.ndarray:
    """4x4 inverse by cofactors (adjugate / determinant), in Python floats."""
    a = [[float(m[i, j]) for j in range(4)] for i in range(4)]

    def minor(r, c):
        rows = [i for i in range(4) if i != r]
        cols = [j for j in range(4) if j != c]
        (p, q, t), (u, v, w), (x, y, z) = ([a[i][j] for j in cols] for i in rows)
        return p * (v * z - w * y) - q * (u * z - w * x) + t * (u * y - v * x)

    cof = [[(-1.0 if (i + j) & 1 else 1.0) * minor(i, j) for j in range(4)] for i in range(4)]
    det = a[0][0] * cof[0][0] + a[0][1] * cof[0][1] + a[0][2] * cof[0][2] + a[0][3] * cof[0][3]
    return np.array([[cof[j][i] / det for j in range(4)] for i in range(4)])

MAX_CLUSTER_TRIANGLES = 64
MAX_CLUSTER_VERTICES = 64


# ---------------------------------------------------------------------------
# meshes (indexed triangle lists, float64 during construction)
# ---------------------------------------------------------------------------

@dataclass
class Mesh:
    positions: np.ndarray  # (V, 3)
    normals: np.ndarray  # (V, 3)
    texcoords: np.ndarray  # (V, 2)
    triangles: np.ndarray  # (T, 3) int
    grid: tuple | None = None  # (nx, ny) for regular grids: enables tile clusterization


def icosphere(subdivisions: int, radius: float = 1.0) -> Mesh:
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / _norm3(p) for p in v]
    faces = [tuple(x) for x in f]
    for _ in range(subdivisions):
        cache: dict = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / _norm3(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    P = np.array(verts) * radius
    N = np.array(verts)
    # spherical mapping
    u = _libm(math.atan2, N[:, 2], N[:, 0]) / (2 * np.pi) + 0.5
    vv = _libm(math.acos, np.clip(N[:, 1], -1, 1)) / np.pi
    return Mesh(P, N, np.stack([u, vv], 1), np.array(faces, dtype=np.int64))


def torus(R: float = 1.0, r: float = 0.3, nu: int = 128, nv: int = 48) -> Mesh:
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = 2 * np.pi * i / nu
    b = 2 * np.pi * j / nv
    cx, cz = _libm(math.cos, a), _libm(math.sin, a)
    cb, sb = _libm(math.cos, b), _libm(math.sin, b)
    P = np.stack([(R + r * cb) * cx, r * sb, (R + r * cb) * cz], -1).reshape(-1, 3)
    N = np.stack([cb * cx, sb, cb * cz], -1).reshape(-1, 3)
    UV = np.stack([i / nu, j / nv], -1).reshape(-1, 2).astype(np.float64)
    idx = lambda a_, b_: (a_ % nu) * nv + (b_ % nv)
    q00, q10, q01, q11 = idx(i, j), idx(i + 1, j), idx(i, j + 1), idx(i + 1, j + 1)
    T = np.concatenate([np.stack([q00, q01, q10], -1).reshape(-1, 3), np.stack([q10, q01, q11], -1).reshape(-1, 3)])
    # interleave the two triangles of each quad
    T = T.reshape(2, -1, 3).transpose(1, 0, 2).reshape(-1, 3)
    return Mesh(P, N, UV, T)


def grid(nx: int, ny: int, extent_x: float = 1.0, extent_y: float = 1.0) -> Mesh:
    """Planar grid in the xz plane (y up), nx * ny quads, two triangles each."""
    xs = np.arange(nx + 1) / nx * extent_x - extent_x / 2
    zs = np.arange(ny + 1) / ny * extent_y - extent_y / 2
    X, Z = np.meshgrid(xs, zs, indexing="xy")  # (ny+1, nx+1)
    P = np.stack([X, np.zeros_like(X), Z], -1).reshape(-1, 3)
    N = np.tile(np.array([0.0, 1.0, 0.0]), (P.shape[0], 1))
    U, V = np.meshgrid(np.arange(nx + 1) / nx, np.arange(ny + 1) / ny, indexing="xy")
    UV = np.stack([U, V], -1).reshape(-1, 2)
    r, c = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    v00 = r * (nx + 1) + c
    v10 = v00 + 1
    v01 = v00 + (nx + 1)
    v11 = v01 + 1
    T = np.stack([np.stack([v00, v01, v10], -1), np.stack([v10, v01, v11], -1)], 2).reshape(-1, 3)
    return Mesh(P, N, UV, T, grid=(nx, ny))


def subdivided_cube(na: int = 16, nb: int = 8, half: float = 0.5) -> Mesh:
    """6 faces of na x nb quads (2 triangles each): 6 * na * nb * 2 triangles."""
    Ps, Ns, UVs, Ts = [], [], [], []
    base = 0
    axes = [(0, 1, 2, 1.0), (0, 1, 2, -1.0), (1, 2, 0, 1.0), (1, 2, 0, -1.0), (2, 0, 1, 1.0), (2, 0, 1, -1.0)]
    for ua, va, na_, sgn in axes:
        us = np.arange(na + 1) / na
        vs = np.arange(nb + 1) / nb
        Ug, Vg = np.meshgrid(us, vs, indexing="xy")
        p = np.zeros(Ug.shape + (3,))
        p[..., ua] = (Ug * 2 - 1) * half
        p[..., va] = (Vg * 2 - 1) * half * sgn
        p[..., na_] = half * sgn
        n = np.zeros_like(p)
        n[..., na_] = sgn
        Ps.append(p.reshape(-1, 3))
        Ns.append(n.reshape(-1, 3))
        UVs.append(np.stack([Ug, Vg], -1).reshape(-1, 2))
        r, c = np.meshgrid(np.arange(nb), np.arange(na), indexing="ij")
        v00 = base + r * (na + 1) + c
        v10, v01 = v00 + 1, v00 + (na + 1)
        v11 = v01 + 1
        Ts.append(np.stack([np.stack([v00, v10, v01], -1), np.stack([v10, v11, v01], -1)], 2).reshape(-1, 3))
        base += (na + 1) * (nb + 1)
    return Mesh(np.concatenate(Ps), np.concatenate(Ns), np.concatenate(UVs), np.concatenate(Ts))


# ---------------------------------------------------------------------------
# clusterization
# ---------------------------------------------------------------------------

@dataclass
class Geometry:
    """One mesh in the reference's cluster layout (shaderio_scene.h:101-156)."""
    positions: np.ndarray  # (V, 3) float32, per-cluster duplicated
    normals: np.ndarray  # (V, 3) float32
    texcoords: np.ndarray  # (V, 2) float32
    clusters: np.ndarray  # Cluster records
    local_triangles: np.ndarray  # uint8, 3 per triangle
    bboxes: np.ndarray  # BBox records
    template_addresses: np.ndarray  # uint64 per cluster (synthetic: CLAS templates are built elsewhere)
    template_sizes: np.ndarray  # uint32 per cluster
    lo: np.ndarray
    hi: np.ndarray
    num_triangles: int = 0

    @property
    def num_clusters(self) -> int:
        return len(self.clusters)


def _morton3(q: np.ndarray) -> np.ndarray:
    def spread(x):
        x = x.astype(np.uint64) & np.uint64(0x3FF)
        x = (x | (x << np.uint64(16))) & np.uint64(0x030000FF)
        x = (x | (x << np.uint64(8))) & np.uint64(0x0300F00F)
        x = (x | (x << np.uint64(4))) & np.uint64(0x030C30C3)
        x = (x | (x << np.uint64(2))) & np.uint64(0x09249249)
        return x
    return spread(q[:, 0]) | (spread(q[:, 1]) << np.uint64(1)) | (spread(q[:, 2]) << np.uint64(2))


def _greedy_clusters(mesh: Mesh) -> list[np.ndarray]:
    """Spatially sorted greedy packing: triangles in Morton order of their
    centroids, a cluster closes when the next triangle would exceed 64
    triangles or 64 unique vertices."""
    T = mesh.triangles
    cen = mesh.positions[T].mean(1)
    lo, hi = cen.min(0), cen.max(0)
    q = np.floor((cen - lo) / np.maximum(hi - lo, 1e-12) * 1023.0).astype(np.int64)
    order = np.argsort(_morton3(q), kind="stable")
    clusters, cur, verts = [], [], set()
    for t in order:
        tv = T[t]
        new = [v for v in tv if v not in verts]
        if cur and (len(cur) + 1 > MAX_CLUSTER_TRIANGLES or len(verts) + len(set(new)) > MAX_CLUSTER_VERTICES):
            clusters.append(np.array(cur))
            cur, verts = [], set()
        cur.append(t)
        verts.update(tv.tolist())
    if cur:
        clusters.append(np.array(cur))
    return clusters


def _grid_tile_clusters(mesh: Mesh, tx: int = 8, ty: int = 4) -> list[np.ndarray]:
    nx, ny = mesh.grid
    r, c = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    quad = r * nx + c
    tile = (r // ty) * ((nx + tx - 1) // tx) + (c // tx)
    tri_tile = np.repeat(tile.reshape(-1), 2)
    tri_idx = np.stack([quad * 2, quad * 2 + 1], -1).reshape(-1)
    order = np.lexsort((tri_idx, tri_tile))
    tiles_sorted = tri_tile[order]
    bounds = np.flatnonzero(np.diff(tiles_sorted)) + 1
    return np.split(tri_idx[order], bounds)


def clusterize(mesh: Mesh, geometry_id: int = 0) -> Geometry:
    if mesh.grid is not None and mesh.grid[0] % 8 == 0 and mesh.grid[1] % 4 == 0:
        return _clusterize_grid(mesh, geometry_id)
    groups = _greedy_clusters(mesh)
    pos, nrm, uv, lt, cl = [], [], [], [], []
    first_vertex = first_local_tri = first_tri = 0
    for g in groups:
        tv = mesh.triangles[g]
        uniq, inv = np.unique(tv.reshape(-1), return_inverse=True)
        # local order: first use
        first_use = np.full(len(uniq), 1 << 30)
        np.minimum.at(first_use, inv, np.arange(inv.size))
        rank = np.empty(len(uniq), np.int64)
        rank[np.argsort(first_use, kind="stable")] = np.arange(len(uniq))
        local = rank[inv]
        ordered = uniq[np.argsort(first_use, kind="stable")]
        pos.append(mesh.positions[ordered])
        nrm.append(mesh.normals[ordered])
        uv.append(mesh.texcoords[ordered])
        lt.append(local.astype(np.uint8))
        cl.append((len(ordered), len(g), first_tri, first_vertex, first_local_tri))
        first_vertex += len(ordered)
        first_local_tri += len(g) * 3
        first_tri += len(g)
    return _finish(np.concatenate(pos), np.concatenate(nrm), np.concatenate(uv), np.concatenate(lt), cl,
                   mesh.triangles.shape[0], geometry_id)


def _clusterize_grid(mesh: Mesh, geometry_id: int, tx: int = 8, ty: int = 4) -> Geometry:
    """Vectorised tiling of a regular grid into tx x ty quad tiles
    (2 * tx * ty <= 64 triangles, (tx + 1) * (ty + 1) <= 64 vertices)."""
    nx, ny = mesh.grid
    nt_x, nt_y = nx // tx, ny // ty
    ntiles = nt_x * nt_y
    # local vertex grid of a tile
    lr, lc = np.meshgrid(np.arange(ty + 1), np.arange(tx + 1), indexing="ij")
    tr, tc = np.meshgrid(np.arange(nt_y), np.arange(nt_x), indexing="ij")
    gv = ((tr.reshape(-1, 1, 1) * ty + lr[None]) * (nx + 1) + (tc.reshape(-1, 1, 1) * tx + lc[None])).reshape(ntiles, -1)
    nv_tile = (tx + 1) * (ty + 1)
    # local triangles of a tile (same as the mesh's quad split)
    qr, qc = np.meshgrid(np.arange(ty), np.arange(tx), indexing="ij")
    l00 = qr * (tx + 1) + qc
    l10, l01 = l00 + 1, l00 + (tx + 1)
    l11 = l01 + 1
    ltri = np.stack([np.stack([l00, l01, l10], -1), np.stack([l10, l01, l11], -1)], 2).reshape(-1, 3)
    nt_tile = ltri.shape[0]
    flat = gv.reshape(-1)
    cl = np.zeros(ntiles, L.Cluster)
    cl["numVertices"] = nv_tile
    cl["numTriangles"] = nt_tile
    cl["firstTriangle"] = np.arange(ntiles) * nt_tile
    cl["firstLocalVertex"] = np.arange(ntiles) * nv_tile
    cl["firstLocalTriangle"] = np.arange(ntiles) * nt_tile * 3
    lt = np.tile(ltri.reshape(-1).astype(np.uint8), ntiles)
    return _finish(mesh.positions[flat], mesh.normals[flat], mesh.texcoords[flat], lt, cl, mesh.triangles.shape[0],
                   geometry_id)


def _finish(pos, nrm, uv, lt, cl, num_tris, geometry_id) -> Geometry:
    if not isinstance(cl, np.ndarray):
        arr = np.zeros(len(cl), L.Cluster)
        for i, c in enumerate(cl):
            arr[i] = c
        cl = arr
    pos = pos.astype(np.float32)
    nrm = nrm.astype(np.float32)
    uv = uv.astype(np.float32)
    nc = len(cl)
    # per-cluster bounding boxes (src/scene.cpp:463-517)
    idx = np.repeat(np.arange(nc), cl["numVertices"].astype(np.int64))
    lo = np.full((nc, 3), np.inf, np.float32)
    hi = np.full((nc, 3), -np.inf, np.float32)
    np.minimum.at(lo, idx, pos)
    np.maximum.at(hi, idx, pos)
    bb = np.zeros(nc, L.BBox)
    bb["lo"] = lo
    bb["hi"] = hi
    tri_cluster = np.repeat(np.arange(nc), cl["numTriangles"].astype(np.int64))
    gidx = lt.reshape(-1, 3).astype(np.int64) + cl["firstLocalVertex"][tri_cluster].astype(np.int64)[:, None]
    e = np.stack([_row_norms(pos[gidx[:, k]] - pos[gidx[:, (k + 1) % 3]]) for k in range(3)], 1)
    emin = np.full(nc, np.inf, np.float32)
    emax = np.zeros(nc, np.float32)
    np.minimum.at(emin, tri_cluster, e.min(1).astype(np.float32))
    np.maximum.at(emax, tri_cluster, e.max(1).astype(np.float32))
    bb["shortestEdge"] = emin
    bb["longestEdge"] = emax
    # synthetic CLAS template data (produced by the CLAS template build, out of scope):
    # unique addresses and a size that grows with the triangle count
    taddr = (np.uint64(0x7F00_0000_0000) + np.uint64(geometry_id) * np.uint64(1 << 32)
             + np.arange(nc, dtype=np.uint64) * np.uint64(256))
    tsize = (128 + 48 * cl["numTriangles"].astype(np.uint32)).astype(np.uint32)
    return Geometry(pos, nrm, uv, cl, lt.astype(np.uint8), bb, taddr, tsize, pos.min(0), pos.max(0), int(num_tris))


# ---------------------------------------------------------------------------
# displacement maps
# ---------------------------------------------------------------------------

def value_noise(size: int, octaves: int, seed: int, base_freq: int = 4, persistence: float = 0.5,
                dtype=np.float32) -> np.ndarray:
    """Tileable value noise / fBm in [0, 1]: per octave a random lattice of
    base_freq * 2^o cells, smoothstep-interpolated, amplitudes persistence^o,
    normalised to exactly [0, 1]."""
    rng = np.random.default_rng(seed)
    out = np.zeros((size, size), np.float32)
    amp, total = 1.0, 0.0
    coord_base = (np.arange(size, dtype=np.float64) + 0.5) / size
    for o in range(octaves):
        f = base_freq << o
        lattice = rng.random((f, f), dtype=np.float32)
        c = coord_base * f
        i0 = np.floor(c).astype(np.int64)
        t = (c - i0).astype(np.float32)
        s = t * t * (np.float32(3) - np.float32(2) * t)
        i0 %= f
        i1 = (i0 + 1) % f
        rows = lattice[:, i0] * (1 - s)[None, :] + lattice[:, i1] * s[None, :]  # (f, size)
        img = rows[i0, :] * (1 - s)[:, None] + rows[i1, :] * s[:, None]
        out += np.float32(amp) * img
        total += amp
        amp *= persistence
    out /= np.float32(total)
    mn, mx = out.min(), out.max()
    out = (out - mn) / (mx - mn)
    return out.astype(dtype)


# ---------------------------------------------------------------------------
# transforms and camera (glm conventions: column-major, RH, depth [0, 1])
# ---------------------------------------------------------------------------

def mat_colmajor(M: np.ndarray) -> np.ndarray:
    """Row-major 4x4 (math convention) -> 16 floats column-major (glm)."""
    return np.asarray(M, np.float64).T.reshape(-1).astype(np.float32)


def translate_rotate_scale(t, q, s) -> np.ndarray:
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * s
    M[:3, 3] = t
    return M


def random_unit_quaternion(rng) -> np.ndarray:
    u1, u2, u3 = rng.random(3)
    u1, u2, u3 = float(u1), float(u2), float(u3)
    return np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                     math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3)])[[3, 0, 1, 2]]


def look_at(eye, center, up) -> np.ndarray:
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= _norm3(f)
    s = np.cross(f, up)
    s /= _norm3(s)
    u = np.cross(s, f)
    M = np.eye(4)
    M[0, :3], M[1, :3], M[2, :3] = s, u, -f
    M[0, 3], M[1, 3], M[2, 3] = -_dot3(s, eye), -_dot3(u, eye), _dot3(f, eye)
    return M


def perspective_rh_zo(fovy_rad, aspect, near, far) -> np.ndarray:
    th = math.tan(fovy_rad / 2)
    P = np.zeros((4, 4))
    P[0, 0] = 1 / (aspect * th)
    P[1, 1] = 1 / th
    P[2, 2] = far / (near - far)
    P[3, 2] = -1
    P[2, 3] = -(far * near) / (far - near)
    return P


@dataclass
class Camera:
    eye: tuple
    center: tuple
    up: tuple = (0.0, 1.0, 0.0)
    fovy_deg: float = 45.0
    width: int = 1920
    height: int = 1080
    near: float = 0.01
    far: float = 1000.0
    tess_rate_pixels: float = 8.0
    displacement_scale: float = 1.0
    displacement_offset: float = 0.0


def frame_constants(cam: Camera) -> np.ndarray:
    """FrameConstants as filled by src/tessellatedclusters.cpp:562-607."""
    fc = np.zeros((), L.FrameConstants)
    P = perspective_rh_zo(math.radians(cam.fovy_deg), cam.width / cam.height, cam.near, cam.far)
    P[1, 1] *= -1  # projection[1][1] *= -1
    V = look_at(cam.eye, cam.center, cam.up)
    VP = _mm(P, V)
    Vi = _inv4(V)
    fc["projMatrix"] = mat_colmajor(P)
    fc["projMatrixI"] = mat_colmajor(_inv4(P))
    fc["viewProjMatrix"] = mat_colmajor(VP)
    fc["viewProjMatrixI"] = mat_colmajor(_inv4(VP))
    fc["viewMatrix"] = mat_colmajor(V)
    fc["viewMatrixI"] = mat_colmajor(Vi)
    fc["viewPos"] = np.append(Vi[:3, 3], 1.0).astype(np.float32)
    fc["viewDir"] = np.append(-Vi[:3, 2], 0.0).astype(np.float32)
    fc["viewPlane"] = fc["viewDir"]
    fc["viewport"] = (cam.width, cam.height)
    fc["viewportf"] = (cam.width, cam.height)
    fc["tessRate"] = np.float32(1.0 / cam.tess_rate_pixels) if cam.tess_rate_pixels else np.float32(0)
    fc["displacementScale"] = cam.displacement_scale
    fc["displacementOffset"] = cam.displacement_offset
    fc["nearPlane"] = cam.near
    fc["farPlane"] = cam.far
    fc["wUpDir"] = cam.up
    fc["hizSizeFactors"] = (1, 1, 1, 1)
    fc["hizSizeMax"] = 1
    fc["visFilterInstanceID"] = 0xFFFFFFFF
    fc["visFilterClusterID"] = 0xFFFFFFFF
    return fc


# ---------------------------------------------------------------------------
# scenes
# ---------------------------------------------------------------------------

@dataclass
class Instance:
    geometry: int
    world: np.ndarray  # 4x4 row-major
    displacement_index: int = -1
    displacement_scale: float = 0.0
    displacement_offset: float = 0.0


@dataclass
class Texture:
    texels: np.ndarray  # (H, W) float32 / float16 / uint16
    format: int


@dataclass
class Scene:
    name: str
    geometries: list
    instances: list
    textures: list = field(default_factory=list)

    @property
    def total_clusters(self) -> int:
        return sum(self.geometries[i.geometry].num_clusters for i in self.instances)

    @property
    def total_triangles(self) -> int:
        return sum(self.geometries[i.geometry].num_triangles for i in self.instances)


def instance_records(scene: Scene, addresses: list[dict]) -> np.ndarray:
    """RenderInstance array; `addresses[g]` maps geometry buffer names to addresses."""
    recs = np.zeros(len(scene.instances), L.RenderInstance)
    for i, inst in enumerate(scene.instances):
        g = scene.geometries[inst.geometry]
        a = addresses[inst.geometry]
        r = recs[i]
        r["worldMatrix"] = mat_colmajor(inst.world)
        r["geometryID"] = inst.geometry
        r["numTriangles"] = g.num_triangles
        r["numVertices"] = g.positions.shape[0]
        r["numClusters"] = g.num_clusters
        r["displacementIndex"] = inst.displacement_index
        r["displacementScale"] = inst.displacement_scale
        r["displacementOffset"] = inst.displacement_offset
        r["geoLo"] = np.append(g.lo, 1.0)
        r["geoHi"] = np.append(g.hi, 1.0)
        for k in ("positions", "normals", "texcoords", "clusters", "clusterLocalTriangles", "clusterBboxes",
                  "clusterTemplateAdresses", "clusterTemplateInstantiatonSizes"):
            r[k] = a[k]
        recs[i] = r
    return recs


def basic_cluster_sizes() -> np.ndarray:
    """Worst-case CLAS sizes by triangle count (0..64) for transient builds, a
    synthetic stand-in for the driver's size query the reference uploads
    (raytracing_cluster_data.cpp:363-386); above the template sizes (128 + 48
    per triangle) because they cannot use the cluster's topology."""
    return (192 + 64 * np.arange(65, dtype=np.uint32)).astype(np.uint32)


def scene_icosphere(subdivisions: int = 5, map_size: int = 1024, octaves: int = 4, seed: int = 0,
                    displacement_scale: float = 0.05) -> Scene:
    """One icosphere (radius 1) with a value-noise displacement map (plain small config)."""
    g = clusterize(icosphere(subdivisions), 0)
    tex = Texture(value_noise(map_size, octaves, seed), L.TEXEL_F32)
    return Scene("icosphere", [g], [Instance(0, np.eye(4), 0, displacement_scale, 0.0)], [tex])


def camera_icosphere() -> Camera:
    return Camera(eye=(0.0, 0.0, 3.0), center=(0.0, 0.0, 0.0), fovy_deg=45.0, width=1920, height=1080, near=0.01,
                  far=100.0, tess_rate_pixels=8.0)


def scene_batched(num_instances: int = 256, seed: int = 1, map_size: int = 512, octaves: int = 4,
                  displacement_scale: float = 0.03, box: float = 40.0) -> Scene:
    """Four meshes of uneven size instanced with seeded transforms (batched config)."""
    meshes = [icosphere(4), torus(1.0, 0.3, 128, 48), grid(128, 128, 2.0, 2.0), subdivided_cube(16, 8)]
    geos = [clusterize(m, i) for i, m in enumerate(meshes)]
    texs = [Texture(value_noise(map_size, octaves, seed * 100 + i), L.TEXEL_F32) for i in range(4)]
    rng = np.random.default_rng(seed)
    insts = []
    for i in range(num_instances):
        gi = i % 4
        t = rng.random(3) * box
        q = random_unit_quaternion(rng)
        s = 0.5 + 1.5 * rng.random()
        insts.append(Instance(gi, translate_rotate_scale(t, q, s), gi, displacement_scale, 0.0))
    return Scene("batched", geos, insts, texs)


def animation_motion(num_instances: int, seed: int = 3):
    """Seeded rigid motion per instance: a random rotation axis with angular
    speed U[0, 1] rad/s, and a random direction with speed U[0, 2] units/s."""
    rng = np.random.default_rng(seed)
    axes = rng.normal(size=(num_instances, 3))
    axes /= _row_norms(axes)[:, None]
    omega = rng.random(num_instances)
    dirs = rng.normal(size=(num_instances, 3))
    dirs /= _row_norms(dirs)[:, None]
    velocity = dirs * (2.0 * rng.random(num_instances))[:, None]
    return axes, omega, velocity


def animated_worlds(scene: "Scene", motion, t: float) -> np.ndarray:
    """World matrices (n, 4, 4) at time t: each instance spins about its own
    origin (axis, omega * t) and translates by velocity * t."""
    axes, omega, velocity = motion
    base = np.stack([i.world for i in scene.instances])
    ang = omega * t
    c, s_, k = _libm(math.cos, ang)[:, None, None], _libm(math.sin, ang)[:, None, None], axes
    K = np.zeros((len(k), 3, 3))
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 0] = -k[:, 2], k[:, 1], k[:, 2]
    K[:, 1, 2], K[:, 2, 0], K[:, 2, 1] = -k[:, 0], -k[:, 1], k[:, 0]
    R = np.eye(3)[None] + s_ * K + (1 - c) * _mm(K, K)  # Rodrigues
    W = base.copy()
    W[:, :3, :3] = _mm(R, base[:, :3, :3])
    W[:, :3, 3] = base[:, :3, 3] + velocity * t
    return W


def camera_orbit(frame: int, num_frames: int = 60, radius: float = 30.0, center=(20.0, 20.0, 20.0),
                 height: float = 10.0, tess_rate_pixels: float = 4.0) -> Camera:
    a = 2 * math.pi * frame / num_frames
    eye = (center[0] + radius * math.cos(a), center[1] + height, center[2] + radius * math.sin(a))
    return Camera(eye=eye, center=center, fovy_deg=45.0, width=1920, height=1080, near=0.01, far=1000.0,
                  tess_rate_pixels=tess_rate_pixels)


def scene_terrain(n: int = 1024, extent: float = 1024.0, map_size: int = 4096, octaves: int = 8, seed: int = 2,
                  relative_scale: float = 0.1) -> Scene:
    """Terrain grid of n x n quads with an fp16 fBm map (bandwidth config)."""
    g = clusterize(grid(n, n, extent, extent), 0)
    tex = Texture(value_noise(map_size, octaves, seed, dtype=np.float16), L.TEXEL_F16)
    return Scene("terrain", [g], [Instance(0, np.eye(4), 0, relative_scale * extent, 0.0)], [tex])


def camera_terrain(extent: float = 1024.0, height: float = 2.0, pitch_deg: float = 10.0) -> Camera:
    eye = np.array([0.0, height, 0.0])
    p = math.radians(pitch_deg)
    d = np.array([math.cos(p) * 0.0, -math.sin(p), math.cos(p)])
    return Camera(eye=tuple(eye), center=tuple(eye + d * 10.0), fovy_deg=45.0, width=3840, height=2160, near=0.01,
                  far=4 * extent, tess_rate_pixels=4.0)
