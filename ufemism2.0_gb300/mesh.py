"""Triangular meshes in UFEMISM's connectivity conventions.

The velocity solver consumes a mesh exactly as UFEMISM's ``type_mesh`` holds it
(src/UPSY/types/mesh_types.f90:57-97), with 1-based indices and 0 meaning "none":

* ``V(nV,2)``      vertex coordinates [m]
* ``nC, C``        vertex neighbours, counter-clockwise; for border vertices ordered
                   "from edge to edge" (mesh_types.f90:59)
* ``niTri, iTri``  triangles around a vertex, counter-clockwise (mesh_types.f90:61);
                   here ``iTri(vi,k)`` is the triangle between ``C(vi,k)`` and ``C(vi,k+1)``
* ``VBI``          vertex border index 0 free, 1 N, 2 NE, 3 E, 4 SE, 5 S, 6 SW, 7 W, 8 NW
                   (mesh_types.f90:62)
* ``Tri(nTri,3)``  vertices counter-clockwise (mesh_types.f90:65)
* ``TriC(nTri,3)`` neighbour triangle across from the 1st, 2nd, 3rd vertex (mesh_types.f90:67)
* ``TriBI``        triangle border index, by the border walk of ``calc_TriBI``
                   (src/UPSY/mesh/mesh_secondary.f90:72-135)
* ``TriGC(nTri,2)`` geometric centres (p+q+r)/3 (mesh_secondary.f90:432-469,
                   src/UPSY/basic/math_utilities/plane_geometry.f90:311-320)

2-D arrays are stored column-major (Fortran order), as the Fortran caller holds them.

Point placement is this project's own: a quadtree refined by a resolution function plus
adaptive points along the domain border, triangulated by Qhull's Delaunay (scipy). The
reference builds its meshes by Ruppert refinement (src/UPSY/mesh/mesh_refinement_basic.f90),
which this generator does not reproduce; only the connectivity conventions matter to the
velocity solve.
"""
from __future__ import annotations

import numpy as np

NC_MEM = 32  # mesh_types.f90:39


class Mesh:
    """A mesh in UFEMISM conventions (1-based indices, Fortran-ordered 2-D arrays)."""

    def __init__(self, V, Tri0, TriC0, xmin, xmax, ymin, ymax, nz=12, zeta=None):
        self.xmin, self.xmax, self.ymin, self.ymax = float(xmin), float(xmax), float(ymin), float(ymax)
        self.nV = int(V.shape[0])
        self.nTri = int(Tri0.shape[0])
        self.nC_mem = NC_MEM
        self.V = np.asfortranarray(V, dtype=np.float64)
        self.Tri = np.asfortranarray(Tri0 + 1, dtype=np.int32)
        self.TriC = np.asfortranarray(np.where(TriC0 >= 0, TriC0 + 1, 0), dtype=np.int32)
        self._build_vertex_connectivity(Tri0)
        self._build_border_indices()
        self._build_TriGC()
        self.set_zeta(nz, zeta)

    @classmethod
    def from_arrays(cls, V, nC, C, niTri, iTri, VBI, Tri, TriC, TriBI, TriGC, zeta, box):
        """A mesh from stored UFEMISM-convention arrays (1-based), e.g. a test fixture."""
        self = cls.__new__(cls)
        self.xmin, self.xmax, self.ymin, self.ymax = (float(b) for b in box)
        self.V = np.asfortranarray(V, dtype=np.float64)
        self.nV = int(self.V.shape[0])
        self.Tri = np.asfortranarray(Tri, dtype=np.int32)
        self.nTri = int(self.Tri.shape[0])
        self.TriC = np.asfortranarray(TriC, dtype=np.int32)
        self.nC = np.ascontiguousarray(nC, dtype=np.int32)
        self.C = np.asfortranarray(C, dtype=np.int32)
        self.nC_mem = int(self.C.shape[1])
        self.niTri = np.ascontiguousarray(niTri, dtype=np.int32)
        self.iTri = np.asfortranarray(iTri, dtype=np.int32)
        self.VBI = np.ascontiguousarray(VBI, dtype=np.int32)
        self.TriBI = np.ascontiguousarray(TriBI, dtype=np.int32)
        self.TriGC = np.asfortranarray(TriGC, dtype=np.float64)
        self.set_zeta(len(zeta), zeta)
        return self

    # -- vertical grid ---------------------------------------------------------------
    def set_zeta(self, nz, zeta=None):
        """Regular zeta grid by default (src/UPSY/mesh/mesh_zeta.f90:60-80)."""
        if zeta is None:
            zeta = np.array([(k - 1) / (nz - 1) for k in range(1, nz + 1)], dtype=np.float64)
        zeta = np.ascontiguousarray(zeta, dtype=np.float64)
        assert zeta.shape == (nz,)
        self.nz = int(nz)
        self.zeta = zeta

    # -- connectivity ----------------------------------------------------------------
    def _build_vertex_connectivity(self, tri):
        V = self.V
        nV, nTri = self.nV, self.nTri
        a = tri.reshape(-1)
        b = tri[:, [1, 2, 0]].reshape(-1)
        c = tri[:, [2, 0, 1]].reshape(-1)
        t = np.repeat(np.arange(nTri), 3)
        ang = np.arctan2(V[b, 1] - V[a, 1], V[b, 0] - V[a, 0])
        order = np.lexsort((ang, a))
        a, b, c, t = a[order], b[order], c[order], t[order]
        counts = np.bincount(a, minlength=nV)
        if counts.min() < 1:
            raise ValueError("mesh has a vertex that belongs to no triangle")
        start = np.zeros(nV + 1, dtype=np.int64)
        start[1:] = np.cumsum(counts)

        nC = counts.copy()
        niTri = counts.copy()
        C = np.zeros((nV, NC_MEM), dtype=np.int32, order="F")
        iTri = np.zeros((nV, NC_MEM), dtype=np.int32, order="F")
        if counts.max() + 1 > NC_MEM:
            raise ValueError("vertex with more than nC_mem neighbours")

        # A vertex is on the mesh boundary when one of its incident triangles has no
        # counter-clockwise successor: the b of that incidence is not the c of another.
        pos = np.arange(a.size) - start[a]
        # interior default: angular order
        C[a, pos] = b + 1
        iTri[a, pos] = t + 1

        # successor check: for interior vertices every b appears as some c
        key_b = a.astype(np.int64) * nV + b
        key_c = a.astype(np.int64) * nV + c
        has_pred = np.isin(key_b, key_c)
        border_v = np.unique(a[~has_pred])
        for vi in border_v:
            s, e = start[vi], start[vi + 1]
            bs, cs, ts = b[s:e], c[s:e], t[s:e]
            # first incidence: its b is nobody's c
            j0 = int(np.nonzero(~np.isin(bs, cs))[0][0])
            # walk counter-clockwise: next incidence has b == current c
            nb_map = {int(bb): k for k, bb in enumerate(bs)}
            seqC, seqT = [], []
            k = j0
            for _ in range(e - s):
                seqC.append(int(bs[k]))
                seqT.append(int(ts[k]))
                nxt = int(cs[k])
                if nxt in nb_map:
                    k = nb_map[nxt]
                else:
                    last = nxt
                    break
            else:  # pragma: no cover - a border vertex always ends on a border edge
                raise ValueError("border walk did not terminate")
            seqC.append(last)
            if len(seqT) != e - s:
                raise ValueError("non-manifold vertex neighbourhood")
            n = len(seqC)
            C[vi, :] = 0
            iTri[vi, :] = 0
            C[vi, :n] = np.array(seqC) + 1
            iTri[vi, : n - 1] = np.array(seqT) + 1
            nC[vi] = n
            niTri[vi] = n - 1
        self.nC = nC.astype(np.int32)
        self.niTri = niTri.astype(np.int32)
        self.C = C
        self.iTri = iTri
        self._is_border_vertex = np.zeros(nV, dtype=bool)
        self._is_border_vertex[border_v] = True

    def _build_border_indices(self):
        x, y = self.V[:, 0], self.V[:, 1]
        on_w, on_e = x == self.xmin, x == self.xmax
        on_s, on_n = y == self.ymin, y == self.ymax
        VBI = np.zeros(self.nV, dtype=np.int32)
        VBI[on_n] = 1
        VBI[on_e] = 3
        VBI[on_s] = 5
        VBI[on_w] = 7
        VBI[on_n & on_e] = 2
        VBI[on_s & on_e] = 4
        VBI[on_s & on_w] = 6
        VBI[on_n & on_w] = 8
        if np.any(self._is_border_vertex != (VBI > 0)):
            raise ValueError("mesh boundary does not coincide with the rectangular domain border")
        self.VBI = VBI
        self.TriBI = calc_TriBI(self.nV, self.nC, self.C, self.niTri, self.iTri, VBI, self.nTri)

    def _build_TriGC(self):
        Tri0 = self.Tri - 1
        p, q, r = self.V[Tri0[:, 0]], self.V[Tri0[:, 1]], self.V[Tri0[:, 2]]
        self.TriGC = np.asfortranarray(((p + q) + r) / 3.0)

    # -- helpers ---------------------------------------------------------------------
    def tri_area(self):
        Tri0 = self.Tri - 1
        p, q, r = self.V[Tri0[:, 0]], self.V[Tri0[:, 1]], self.V[Tri0[:, 2]]
        return 0.5 * ((q[:, 0] - p[:, 0]) * (r[:, 1] - p[:, 1]) - (q[:, 1] - p[:, 1]) * (r[:, 0] - p[:, 0]))

    def min_angle_deg(self):
        Tri0 = self.Tri - 1
        P = [self.V[Tri0[:, k]] for k in range(3)]
        angs = []
        for k in range(3):
            u = P[(k + 1) % 3] - P[k]
            w = P[(k + 2) % 3] - P[k]
            cosang = (u * w).sum(1) / np.sqrt((u * u).sum(1) * (w * w).sum(1))
            angs.append(np.degrees(np.arccos(np.clip(cosang, -1, 1))))
        return float(np.min(angs))

    def arrays(self):
        """The mesh arrays by name, as the C-ABI expects them."""
        return dict(V=self.V, nC=self.nC, C=self.C, niTri=self.niTri, iTri=self.iTri, VBI=self.VBI,
                    Tri=self.Tri, TriC=self.TriC, TriBI=self.TriBI, TriGC=self.TriGC, zeta=self.zeta)


def calc_TriBI(nV, nC, C, niTri, iTri, VBI, nTri):
    """Triangle border indices by walking the domain border from the south-west corner.

    Follows src/UPSY/mesh/mesh_secondary.f90:72-135: every triangle touching a border
    vertex takes that vertex's VBI, the walk steps to ``C(vi, nC(vi))``, and a corner
    vertex with a single triangle stamps its corner index on it.
    """
    TriBI = np.zeros(nTri, dtype=np.int32)
    sw = np.nonzero(VBI == 6)[0]
    if sw.size == 0:
        raise ValueError("no south-west corner vertex")
    vi = int(sw[0])
    vi_sw = vi
    vi_se = vi_ne = vi_nw = -1
    n_cycles = 0
    while True:
        n_cycles += 1
        if n_cycles > nV:
            raise ValueError("got stuck tracing the domain border")
        for k in range(niTri[vi]):
            TriBI[iTri[vi, k] - 1] = VBI[vi]
        vi = int(C[vi, nC[vi] - 1]) - 1
        if VBI[vi] == 4:
            vi_se = vi
        if VBI[vi] == 2:
            vi_ne = vi
        if VBI[vi] == 8:
            vi_nw = vi
        if vi == vi_sw:
            break
    for vc, code in ((vi_sw, 6), (vi_se, 4), (vi_ne, 2), (vi_nw, 8)):
        if vc < 0:
            raise ValueError("corner vertex not found on the border walk")
        if niTri[vc] == 1:
            TriBI[iTri[vc, 0] - 1] = code
    return TriBI


# --------------------------------------------------------------------------------------
# point placement
# --------------------------------------------------------------------------------------

def _border_points(p0, p1, res_fn):
    """Points along the segment p0->p1 (excluding p1) spaced by the local resolution."""
    p0, p1 = np.asarray(p0, float), np.asarray(p1, float)
    L = float(np.hypot(*(p1 - p0)))
    d = (p1 - p0) / L
    ts = [0.0]
    t = 0.0
    while True:
        p = p0 + t * d
        step = float(res_fn(np.array([p[0]]), np.array([p[1]]))[0])
        t += step
        if t > L - 0.5 * step:
            break
        ts.append(t)
    ts = np.array(ts)
    pts = p0[None, :] + ts[:, None] * d[None, :]
    return pts


def generate_points(xmin, xmax, ymin, ymax, res_fn, seed=0, jitter=0.18):
    """Quadtree point cloud following the resolution function ``res_fn(x, y) -> m``."""
    rng = np.random.default_rng(seed)
    W, H = xmax - xmin, ymax - ymin
    s0 = min(W, H)
    nx, ny = max(1, int(round(W / s0))), max(1, int(round(H / s0)))
    sx, sy = W / nx, H / ny
    gx, gy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    cx = xmin + (gx.ravel() + 0.5) * sx
    cy = ymin + (gy.ravel() + 0.5) * sy
    hx = np.full(cx.shape, sx)
    hy = np.full(cy.shape, sy)
    leaves_x, leaves_y, leaves_h = [], [], []
    for _ in range(40):
        if cx.size == 0:
            break
        # resolution: min over centre and corners so refinement reaches neighbours
        r = res_fn(cx, cy)
        for ox in (-0.5, 0.5):
            for oy in (-0.5, 0.5):
                r = np.minimum(r, res_fn(cx + ox * hx, cy + oy * hy))
        split = np.maximum(hx, hy) > r
        leaves_x.append(cx[~split]); leaves_y.append(cy[~split]); leaves_h.append(np.maximum(hx, hy)[~split])
        cx, cy, hx, hy = cx[split], cy[split], hx[split], hy[split]
        ncx, ncy = [], []
        for ox in (-0.25, 0.25):
            for oy in (-0.25, 0.25):
                ncx.append(cx + ox * hx)
                ncy.append(cy + oy * hy)
        cx, cy = np.concatenate(ncx), np.concatenate(ncy)
        hx, hy = np.tile(hx / 2, 4), np.tile(hy / 2, 4)
    px = np.concatenate(leaves_x)
    py = np.concatenate(leaves_y)
    ph = np.concatenate(leaves_h)
    px = px + rng.uniform(-jitter, jitter, px.shape) * ph
    py = py + rng.uniform(-jitter, jitter, py.shape) * ph
    # keep interior points away from the border
    rb = res_fn(px, py)
    keep = (px > xmin + 0.5 * rb) & (px < xmax - 0.5 * rb) & (py > ymin + 0.5 * rb) & (py < ymax - 0.5 * rb)
    interior = np.stack([px[keep], py[keep]], 1)
    corners = [(xmin, ymin), (xmax, ymin), (xmax, ymax), (xmin, ymax)]
    border = []
    for k in range(4):
        border.append(_border_points(corners[k], corners[(k + 1) % 4], res_fn))
    border = np.concatenate(border)
    # exact border coordinates (the walk relies on x==xmin etc.)
    border[np.isclose(border[:, 0], xmin, atol=1e-6 * W), 0] = xmin
    border[np.isclose(border[:, 0], xmax, atol=1e-6 * W), 0] = xmax
    border[np.isclose(border[:, 1], ymin, atol=1e-6 * H), 1] = ymin
    border[np.isclose(border[:, 1], ymax, atol=1e-6 * H), 1] = ymax
    generate_points.last_n_border = len(border)
    return np.concatenate([border, interior])


generate_points.last_n_border = 0


def circumcentres(mesh):
    """Circumcentres of the triangles (nTri x 2)."""
    V = np.asarray(mesh.V)
    T = np.asarray(mesh.Tri) - 1
    a, b, c = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
    d = 2.0 * (a[:, 0] * (b[:, 1] - c[:, 1]) + b[:, 0] * (c[:, 1] - a[:, 1]) + c[:, 0] * (a[:, 1] - b[:, 1]))
    na, nb, nc = (a * a).sum(1), (b * b).sum(1), (c * c).sum(1)
    ux = (na * (b[:, 1] - c[:, 1]) + nb * (c[:, 1] - a[:, 1]) + nc * (a[:, 1] - b[:, 1])) / d
    uy = (na * (c[:, 0] - b[:, 0]) + nb * (a[:, 0] - c[:, 0]) + nc * (b[:, 0] - a[:, 0])) / d
    return np.c_[ux, uy]


def connection_triangles(mesh):
    """For every connection (vi, ci): the one or two triangles of the edge from vi to C(vi, ci),
    0-based (nV x nC_mem x 2, -1 where there is none)."""
    T = np.asarray(mesh.Tri, dtype=np.int64) - 1
    nV = mesh.nV
    ends = np.r_[T[:, [0, 1]], T[:, [1, 2]], T[:, [2, 0]]]
    tri = np.tile(np.arange(mesh.nTri), 3)
    key = np.minimum(ends[:, 0], ends[:, 1]) * nV + np.maximum(ends[:, 0], ends[:, 1])
    order = np.argsort(key, kind="stable")
    key, tri = key[order], tri[order]
    out = -np.ones((nV, mesh.nC_mem, 2), np.int64)
    C = np.asarray(mesh.C, dtype=np.int64) - 1
    for ci in range(mesh.nC_mem):
        live = np.arange(nV)[ci < mesh.nC]
        vj = C[live, ci]
        k = np.minimum(live, vj) * nV + np.maximum(live, vj)
        i0 = np.searchsorted(key, k)
        out[live, ci, 0] = tri[i0]
        two = (i0 + 1 < key.size) & (key[np.minimum(i0 + 1, key.size - 1)] == k)
        out[live[two], ci, 1] = tri[i0[two] + 1]
    return out


def voronoi_geometry(mesh):
    """The Voronoi geometry of type_mesh that the ice-thickness equation reads: cell areas A (nV)
    and, per connection, the length Cw of the Voronoi boundary the two cells share (nV x nC_mem,
    column-major like C).  Cells are bounded by the circumcentres of the vertex's triangles; on
    the domain border by the border edges' midpoints and the vertex itself.  A boundary shared
    across an interior edge runs between the circumcentres of its two triangles, across a border
    edge from the circumcentre to the edge's midpoint.  Areas are signed polygon areas, so the
    cells tile the domain exactly even where a circumcentre lies outside its triangle."""
    V = np.asarray(mesh.V)
    cc = circumcentres(mesh)
    ct = connection_triangles(mesh)
    nV, nC = mesh.nV, np.asarray(mesh.nC)
    C = np.asarray(mesh.C, dtype=np.int64) - 1
    Cw = np.zeros((nV, mesh.nC_mem))
    for ci in range(mesh.nC_mem):
        live = np.arange(nV)[ci < nC]
        t1, t2 = ct[live, ci, 0], ct[live, ci, 1]
        mid = 0.5 * (V[live] + V[C[live, ci]])
        far = np.where((t2 >= 0)[:, None], cc[np.maximum(t2, 0)], mid)
        Cw[live, ci] = np.hypot(*(cc[t1] - far).T)
    # areas: the polygon of each cell, walked counter-clockwise
    iT = np.asarray(mesh.iTri, dtype=np.int64) - 1
    niT = np.asarray(mesh.niTri)
    A = np.zeros(nV)
    border = np.asarray(mesh.VBI) > 0
    for k in range(mesh.nC_mem):
        live = np.arange(nV)[(k < niT) & ~border]
        a = cc[iT[live, k]]
        b = cc[iT[live, (k + 1) % niT[live]]]
        A[live] += 0.5 * (a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1])
    for vi in np.nonzero(border)[0]:
        poly = [V[vi], 0.5 * (V[vi] + V[C[vi, 0]])]
        poly += [cc[iT[vi, k]] for k in range(niT[vi])]
        poly += [0.5 * (V[vi] + V[C[vi, nC[vi] - 1]])]
        P = np.array(poly)
        A[vi] = 0.5 * np.sum(P[:, 0] * np.roll(P[:, 1], -1) - np.roll(P[:, 0], -1) * P[:, 1])
    return A, np.asfortranarray(Cw)


def triangulate(points, xmin, xmax, ymin, ymax, nz=12, zeta=None):
    """Delaunay triangulation of the points into a :class:`Mesh`."""
    from scipy.spatial import Delaunay

    dl = Delaunay(points)
    if getattr(dl, "coplanar", np.empty((0,))).size:
        raise ValueError("Qhull dropped coplanar points")
    tri = dl.simplices.astype(np.int64).copy()
    nbr = dl.neighbors.astype(np.int64).copy()
    p = points
    area2 = ((p[tri[:, 1], 0] - p[tri[:, 0], 0]) * (p[tri[:, 2], 1] - p[tri[:, 0], 1])
             - (p[tri[:, 1], 1] - p[tri[:, 0], 1]) * (p[tri[:, 2], 0] - p[tri[:, 0], 0]))
    flip = area2 < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    nbr[flip] = nbr[flip][:, [0, 2, 1]]
    if np.any(np.abs(area2) <= 1e-9 * np.abs(area2).max()):
        raise ValueError("degenerate triangle in the triangulation")
    return Mesh(points, tri, nbr, xmin, xmax, ymin, ymax, nz=nz, zeta=zeta)


def smooth_points(points, n_border, n_iter=4):
    """Lloyd-type smoothing: move every interior point to the area-weighted centroid of its
    incident triangles (the reference smooths its meshes with Lloyd iterations as well)."""
    from scipy.spatial import Delaunay

    p = points.copy()
    for _ in range(n_iter):
        tri = Delaunay(p).simplices
        a, b, c = p[tri[:, 0]], p[tri[:, 1]], p[tri[:, 2]]
        area = 0.5 * np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
        cen = (a + b + c) / 3.0
        acc = np.zeros_like(p)
        w = np.zeros(len(p))
        for k in range(3):
            np.add.at(acc, tri[:, k], cen * area[:, None])
            np.add.at(w, tri[:, k], area)
        new = acc / w[:, None]
        new[:n_border] = p[:n_border]
        p = new
    return p


def generate_mesh(xmin, xmax, ymin, ymax, res_fn, seed=0, nz=12, zeta=None, smooth_iters=4):
    pts = generate_points(xmin, xmax, ymin, ymax, res_fn, seed=seed)
    if smooth_iters:
        nb = generate_points.last_n_border
        pts = smooth_points(pts, nb, smooth_iters)
    return triangulate(pts, xmin, xmax, ymin, ymax, nz=nz, zeta=zeta)


def uniform_mesh(L=100e3, res=20e3, seed=0, nz=12):
    """A small square mesh with uniform resolution (test meshes)."""
    return generate_mesh(-L / 2, L / 2, -L / 2, L / 2, lambda x, y: np.full(np.shape(x), res), seed=seed, nz=nz)
