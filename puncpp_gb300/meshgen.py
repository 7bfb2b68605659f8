"""Synthetic tetrahedral meshes for the particle engine.

PUNC++ reads gmsh-made DOLFIN meshes (punc/src/mesh.cpp:62-92); no mesh files
ship with it, so the workloads here are built from structured boxes:

* every sub-cube is split into the 6 Kuhn (Freudenthal) tetrahedra that share
  its main diagonal, which is conforming across neighbouring cubes;
* cells whose centroid lies inside a sphere can be removed, which leaves a
  spherical object hole (the probe geometry of the reference's test/sphere.geo);
* boundary facets are tagged like Mesh::Mesh relabels them
  (punc/src/mesh.cpp:41-60): 1 = exterior boundary, 2 = first object.

The output is plain arrays: vertex coordinates, cell vertex ids, boundary
facets with tags and, for periodic meshes, the vertex-to-dof map that a
periodic CG1 space uses (punc/src/poisson.cpp:225-258).
"""
from __future__ import annotations

import dataclasses
import numpy as np

# The 6 Kuhn tetrahedra of the unit cube: each walks from corner (0,0,0) to
# (1,1,1) adding one unit vector per step, in one of the 6 axis orders.
_PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


@dataclasses.dataclass
class MeshArrays:
    """A tetrahedral mesh as flat arrays (the input of pg_create)."""
    coords: np.ndarray          # (Nv, 3) float64
    cells: np.ndarray           # (Nc, 4) int64 vertex ids
    bfacets: np.ndarray         # (Nb, 3) int64 vertex ids of boundary facets
    btags: np.ndarray           # (Nb,) int32, 1 = exterior, 2.. = objects
    vertex_to_dof: np.ndarray | None = None   # (Nv,) int64 for periodic meshes
    n_dofs: int = 0
    Ld: tuple = (1.0, 1.0, 1.0)   # box size (for move_periodic)
    origin: tuple = (0.0, 0.0, 0.0)
    n_objects: int = 0

    @property
    def n_vertices(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_cells(self) -> int:
        return int(self.cells.shape[0])


def _kuhn_cells(n: int) -> np.ndarray:
    """Cell vertex ids (in grid numbering) of an n^3 Kuhn box."""
    m = n + 1
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i = i.ravel(); j = j.ravel(); k = k.ravel()
    out = np.empty((n * n * n, 6, 4), dtype=np.int64)
    for t, perm in enumerate(_PERMS):
        p = [i.copy(), j.copy(), k.copy()]
        out[:, t, 0] = (p[0] * m + p[1]) * m + p[2]
        for s, ax in enumerate(perm):
            p[ax] = p[ax] + 1
            out[:, t, s + 1] = (p[0] * m + p[1]) * m + p[2]
    return out.reshape(-1, 4)


def _boundary_facets(cells: np.ndarray, n_vertices: int):
    """Facets that belong to exactly one cell, as sorted vertex triples."""
    sc = np.sort(cells, axis=1)
    tri = np.concatenate([sc[:, [1, 2, 3]], sc[:, [0, 2, 3]],
                          sc[:, [0, 1, 3]], sc[:, [0, 1, 2]]], axis=0)
    nv = np.int64(n_vertices)
    key = (tri[:, 0] * nv + tri[:, 1]) * nv + tri[:, 2]
    uniq, counts = np.unique(key, return_counts=True)
    bkeys = uniq[counts == 1]
    a = bkeys // (nv * nv)
    b = (bkeys // nv) % nv
    c = bkeys % nv
    return np.stack([a, b, c], axis=1)


def kuhn_box(n: int, lo: float = 0.0, hi: float = 1.0,
             hole_radius: float | None = None, periodic: bool = False) -> MeshArrays:
    """Box [lo,hi]^3 of n^3 sub-cubes x 6 tetrahedra.

    hole_radius: remove cells whose centroid is within this distance of the
    box centre; the hole's facets get tag 2 (one object).
    periodic: build the periodic vertex-to-dof map (box must start at 0,
    like move_periodic assumes, punc/include/punc/pusher.h:664-681).
    """
    m = n + 1
    h = (hi - lo) / n
    g = np.arange(m, dtype=np.float64)
    gx, gy, gz = np.meshgrid(g, g, g, indexing="ij")
    coords = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1) * h + lo
    cells = _kuhn_cells(n)
    n_objects = 0
    if hole_radius is not None:
        centre = 0.5 * (lo + hi)
        cen = coords[cells].mean(axis=1) - centre
        keep = np.einsum("ij,ij->i", cen, cen) >= hole_radius * hole_radius
        cells = cells[keep]
        used = np.zeros(coords.shape[0], dtype=bool)
        used[cells.ravel()] = True
        remap = -np.ones(coords.shape[0], dtype=np.int64)
        remap[used] = np.arange(int(used.sum()), dtype=np.int64)
        coords = coords[used]
        cells = remap[cells]
        n_objects = 1
    bf = _boundary_facets(cells, coords.shape[0])
    fx = coords[bf]                                  # (Nb, 3, 3)
    on_outer = np.zeros(bf.shape[0], dtype=bool)
    eps = 1e-9 * max(1.0, abs(hi - lo))
    for ax in range(3):
        for wall in (lo, hi):
            on_outer |= np.all(np.abs(fx[:, :, ax] - wall) < eps, axis=1)
    btags = np.where(on_outer, 1, 2).astype(np.int32)
    v2d = None
    n_dofs = coords.shape[0]
    if periodic:
        if hole_radius is not None:
            raise ValueError("periodic meshes have no object hole")
        idx = np.rint((coords - lo) / h).astype(np.int64) % n
        v2d = (idx[:, 0] * n + idx[:, 1]) * n + idx[:, 2]
        n_dofs = n * n * n
    L = hi - lo
    return MeshArrays(coords=np.ascontiguousarray(coords), cells=np.ascontiguousarray(cells),
                      bfacets=np.ascontiguousarray(bf), btags=btags,
                      vertex_to_dof=v2d, n_dofs=int(n_dofs), Ld=(L, L, L),
                      origin=(lo, lo, lo), n_objects=n_objects)


def spherical_shell(n: int, r_inner: float, r_outer: float, snap: bool = False) -> MeshArrays:
    """Cells of a [-R,R]^3 Kuhn box whose centroid radius lies in [r, R): a
    staircase spherical shell.  Inner surface = object (tag 2), outer surface =
    exterior (tag 1), as in the concentric-sphere capacitor of
    demo/capacitance/capacitance.cpp.  snap=True moves the boundary vertices
    onto the spheres (a body-fitted mesh)."""
    base = kuhn_box(n, -r_outer, r_outer)
    coords, cells = base.coords, base.cells
    cen = coords[cells].mean(axis=1)
    rad = np.sqrt(np.einsum("ij,ij->i", cen, cen))
    cells = cells[(rad >= r_inner) & (rad < r_outer)]
    used = np.zeros(coords.shape[0], dtype=bool)
    used[cells.ravel()] = True
    remap = -np.ones(coords.shape[0], dtype=np.int64)
    remap[used] = np.arange(int(used.sum()), dtype=np.int64)
    coords = coords[used]
    cells = remap[cells]
    bf = _boundary_facets(cells, coords.shape[0])
    fr = np.sqrt((coords[bf].mean(axis=1) ** 2).sum(axis=1))
    btags = np.where(fr < 0.5 * (r_inner + r_outer), 2, 1).astype(np.int32)
    if snap:
        # Move the boundary vertices radially onto the two spheres; refuse the
        # result if any cell changes orientation.
        def signed_vol(co):
            p = co[cells]
            return np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))
        v0 = signed_vol(coords)
        coords = coords.copy()
        for tag, rad_to in ((2, r_inner), (1, r_outer)):
            vid = np.unique(bf[btags == tag].ravel())
            rr = np.sqrt((coords[vid] ** 2).sum(axis=1))
            coords[vid] *= (rad_to / rr)[:, None]
        v1 = signed_vol(coords)
        if np.any(np.sign(v0) != np.sign(v1)) or np.any(np.abs(v1) < 1e-3 * np.abs(v0)):
            raise ValueError("snapping inverted or flattened a cell; use another resolution")
    L = 2 * r_outer
    return MeshArrays(coords=np.ascontiguousarray(coords), cells=np.ascontiguousarray(cells),
                      bfacets=np.ascontiguousarray(bf), btags=btags, n_dofs=int(coords.shape[0]),
                      Ld=(L, L, L), origin=(-r_outer,) * 3, n_objects=1)


def mapped_sphere_shell(n: int, k_inner: int, r_inner: float, r_outer: float) -> MeshArrays:
    """Body-fitted shell between spheres r_inner and r_outer.

    A Kuhn box [-1,1]^3 of n^3 sub-cubes (n even) loses its central cube of
    half-width s = 2*k_inner/n; every vertex v is then moved to the sphere of
    radius r_inner + (|v|_inf - s)/(1 - s) * (r_outer - r_inner) along v, which
    maps the cube shells |v|_inf = const onto spheres.  Inner surface = object
    (tag 2), outer surface = exterior (tag 1)."""
    if n % 2 or not (0 < 2 * k_inner < n):
        raise ValueError("n must be even and 0 < 2*k_inner < n")
    base = kuhn_box(n, -1.0, 1.0)
    coords, cells = base.coords, base.cells
    s = 2.0 * k_inner / n
    cen = coords[cells].mean(axis=1)
    cells = cells[np.abs(cen).max(axis=1) > s]
    used = np.zeros(coords.shape[0], dtype=bool)
    used[cells.ravel()] = True
    remap = -np.ones(coords.shape[0], dtype=np.int64)
    remap[used] = np.arange(int(used.sum()), dtype=np.int64)
    coords = coords[used]
    cells = remap[cells]
    bf = _boundary_facets(cells, coords.shape[0])
    linf = np.abs(coords).max(axis=1)
    btags = np.where(linf[bf].max(axis=1) < 0.5 * (1.0 + s), 2, 1).astype(np.int32)
    rad = r_inner + (linf - s) / (1.0 - s) * (r_outer - r_inner)
    coords = coords * (rad / np.sqrt((coords ** 2).sum(axis=1)))[:, None]
    L = 2 * r_outer
    return MeshArrays(coords=np.ascontiguousarray(coords), cells=np.ascontiguousarray(cells),
                      bfacets=np.ascontiguousarray(bf), btags=btags, n_dofs=int(coords.shape[0]),
                      Ld=(L, L, L), origin=(-r_outer,) * 3, n_objects=1)


def icosphere(level: int):
    """Unit-sphere triangulation: the icosahedron, each triangle split into 4
    level times, vertices projected onto the sphere.  Returns (vertices
    (10*4^level + 2, 3), triangles (20*4^level, 3))."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
    tris = [tuple(x) for x in f]
    for _ in range(level):
        mid = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nxt = []
        for a, b, c in tris:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nxt += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        tris = nxt
    return np.array(verts), np.array(tris, dtype=np.int64)


def sphere_shell(r_inner: float, r_outer: float, level: int = 3) -> MeshArrays:
    """Body-fitted tetrahedral shell between the spheres r_inner (the object,
    tag 2) and r_outer (the exterior boundary, tag 1): the geometry of the
    reference's test/sphere.geo.

    The icosphere of the given level is extruded radially through layers
    whose radii grow geometrically, so that a layer's thickness matches the
    triangles' edge length at its radius (resolution proportional to r, as the
    .geo file's 0.2 at r = 1 growing to 6 at r = 20).  Every triangle x layer
    prism splits into 3 tetrahedra by the order of its vertices' ids (sorted
    a < b < c below, a' < b' < c' above: (a,b,c,a'), (b,c,a',b'), (c,a',b',c')),
    which cuts every quadrilateral side face along the diagonal from its
    larger bottom vertex to its smaller top vertex; the neighbouring prism
    cuts the shared face the same way, so the mesh is conforming.  Radial
    extrusion keeps those side faces planar."""
    if not 0.0 < r_inner < r_outer:
        raise ValueError("need 0 < r_inner < r_outer")
    u, tri = icosphere(level)
    nu = u.shape[0]
    e = u[tri]
    edge = np.mean(np.linalg.norm(e[:, 0] - e[:, 1], axis=1))
    layers = max(1, int(np.ceil(np.log(r_outer / r_inner) / np.log1p(edge))))
    radii = r_inner * (r_outer / r_inner) ** (np.arange(layers + 1) / layers)
    coords = (radii[:, None, None] * u[None, :, :]).reshape(-1, 3)
    a, b, c = np.sort(tri, axis=1).T
    cells = []
    for k in range(layers):
        lo, hi = k * nu, (k + 1) * nu
        cells.append(np.stack([a + lo, b + lo, c + lo, a + hi], axis=1))
        cells.append(np.stack([b + lo, c + lo, a + hi, b + hi], axis=1))
        cells.append(np.stack([c + lo, a + hi, b + hi, c + hi], axis=1))
    cells = np.concatenate(cells)
    bf = np.concatenate([tri, tri + layers * nu])
    btags = np.concatenate([np.full(len(tri), 2, np.int32), np.full(len(tri), 1, np.int32)])
    L = 2 * r_outer
    return MeshArrays(coords=np.ascontiguousarray(coords), cells=np.ascontiguousarray(cells),
                      bfacets=np.ascontiguousarray(bf), btags=btags, n_dofs=int(coords.shape[0]),
                      Ld=(L, L, L), origin=(-r_outer,) * 3, n_objects=1)


def langmuir_cube(n: int = 16) -> MeshArrays:
    """Periodic unit cube, n^3 x 6 cells (n=16: 24,576 cells, 4,096 dofs)."""
    return kuhn_box(n, 0.0, 1.0, periodic=True)


def probe_box(n: int = 80, half: float = 10.0, radius: float = 1.0) -> MeshArrays:
    """Cube [-half,half]^3, n^3 x 6 cells, centroid-in-sphere cells removed."""
    return kuhn_box(n, -half, half, hole_radius=radius)
