"""DOLFIN XML mesh ingest: the reference's `Mesh(fname)` (punc/src/mesh.cpp:
41-84) reads `name.xml` (vertices and tetrahedra) and
`name_facet_region.xml` (a facet function of boundary tags), then relabels the
sorted distinct tags to 0, 1, 2, ... (mesh.cpp:47-56): the smallest tag (the
interior facets) becomes 0, the next (the exterior boundary) 1, the rest
objects 2, 3, ...  `read_mesh` does the same and returns the flat arrays the
engine's mesh builder takes.

Facet tags are read in either form DOLFIN 2019.1 writes:

* a mesh value collection, cell-relative (`<value cell_index=..
  local_entity=.. value=../>`, local facet i opposite local vertex i);
* a mesh function indexed by DOLFIN's global facet numbering (`<mesh_function
  dim="2"><entity index=.. value=../>`), the form dolfin-convert writes for
  gmsh meshes.  In a serial mesh DOLFIN numbers the facets by key matching
  (TopologyComputation::compute_entities_by_key_matching): each facet's
  global vertex ids are sorted into a key, the keys of all cells' facets are
  sorted lexicographically, and facet k is the k-th distinct key.
  `dolfin_facet_numbering` restates that.

HDF5 meshes (mesh.cpp:75-84) are refused: no HDF5 library is present.

`write_mesh` writes the same two files from a mesh, tags in either form, e.g.
to hand a generated mesh to the reference.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET

import numpy as np

from .meshgen import MeshArrays, _boundary_facets


def _stem(fname: str) -> str:
    root, ext = os.path.splitext(str(fname))
    if ext not in ("", ".xml"):
        raise ValueError(f"{fname}: only DOLFIN .xml meshes are read here")
    return root


def _local(tag: str) -> str:
    return tag.rsplit("}", 1)[-1]


def _sizes(path: str):
    """Sizes of <vertices> and <cells> (read from their start tags)."""
    nv = nc = None
    for ev, el in ET.iterparse(path, events=("start",)):
        t = _local(el.tag)
        if t == "vertices":
            nv = int(el.get("size"))
        elif t == "cells":
            nc = int(el.get("size"))
        if nv is not None and nc is not None:
            break
    if nv is None or nc is None:
        raise ValueError(f"{path}: no <vertices size=..> / <cells size=..>")
    return nv, nc


def _read_cells_vertices(path: str):
    nv, nc = _sizes(path)
    coords = np.zeros((nv, 3))
    cells = np.zeros((nc, 4), dtype=np.int64)
    seen_v = np.zeros(nv, dtype=bool)
    seen_c = np.zeros(nc, dtype=bool)
    for _, el in ET.iterparse(path, events=("end",)):
        t = _local(el.tag)
        if t == "vertex":
            i = int(el.get("index"))
            coords[i] = (float(el.get("x", 0.0)), float(el.get("y", 0.0)), float(el.get("z", 0.0)))
            seen_v[i] = True
            el.clear()
        elif t == "tetrahedron":
            i = int(el.get("index"))
            cells[i] = (int(el.get("v0")), int(el.get("v1")), int(el.get("v2")), int(el.get("v3")))
            seen_c[i] = True
            el.clear()
        elif t == "mesh" and el.get("celltype") not in (None, "tetrahedron"):
            raise ValueError(f"{path}: celltype {el.get('celltype')} (only tetrahedra)")
    if not seen_v.all() or not seen_c.all():
        raise ValueError(f"{path}: missing vertices or cells")
    return coords, cells


def dolfin_facet_numbering(cells: np.ndarray) -> np.ndarray:
    """The facets of a tetrahedral mesh in DOLFIN's serial numbering
    (TopologyComputation::compute_entities_by_key_matching, DOLFIN 2019.1):
    row k holds the ascending global vertex ids of facet k; the rows are the
    distinct sorted vertex triples of all cells' facets in lexicographic
    order."""
    sc = np.sort(np.asarray(cells, np.int64), axis=1)
    tri = np.concatenate([sc[:, [1, 2, 3]], sc[:, [0, 2, 3]], sc[:, [0, 1, 3]], sc[:, [0, 1, 2]]], axis=0)
    return np.unique(tri, axis=0)


def _read_facet_tags(path: str, cells: np.ndarray):
    """(sorted vertex triples, tag values) of the listed facets."""
    tri, vals = [], []
    glob_idx, glob_vals = [], []
    for _, el in ET.iterparse(path, events=("end",)):
        t = _local(el.tag)
        if t == "value":
            c, i, v = int(el.get("cell_index")), int(el.get("local_entity")), int(el.get("value"))
            verts = [int(x) for k, x in enumerate(cells[c]) if k != i]
            tri.append(sorted(verts))
            vals.append(v)
            el.clear()
        elif t == "entity":
            glob_idx.append(int(el.get("index")))
            glob_vals.append(int(el.get("value")))
            el.clear()
        elif t in ("mesh_function", "mesh_value_collection") and el.get("dim") not in (None, "2"):
            raise ValueError(f"{path}: facet tags must have dim 2")
    if glob_idx:
        facets = dolfin_facet_numbering(cells)
        idx = np.asarray(glob_idx, np.int64)
        if idx.min() < 0 or idx.max() >= len(facets):
            raise ValueError(f"{path}: facet index out of range (the mesh has {len(facets)} facets)")
        tri += facets[idx].tolist()
        vals += glob_vals
    return np.array(tri, dtype=np.int64).reshape(-1, 3), np.array(vals, dtype=np.int64)


def read_mesh(fname: str, periodic_box=None) -> MeshArrays:
    """Read name.xml + name_facet_region.xml and relabel the tags as
    punc/src/mesh.cpp:41-60.  periodic_box = (lo[3], L[3]): identify vertices
    whose coordinates differ by multiples of L (a periodic box has no tagged
    boundary)."""
    stem = _stem(fname)
    coords, cells = _read_cells_vertices(stem + ".xml")
    bf = _boundary_facets(cells, coords.shape[0])
    v2d, n_dofs = None, coords.shape[0]
    Ld, origin = tuple(np.ptp(coords, axis=0)), tuple(coords.min(axis=0))
    if periodic_box is not None:
        lo, L = np.asarray(periodic_box[0], float), np.asarray(periodic_box[1], float)
        frac = (coords - lo) / L
        frac = frac - np.floor(frac + 1e-9)          # the far faces map to the near ones
        key = np.round(frac * 1e9).astype(np.int64)
        _, v2d = np.unique(key, axis=0, return_inverse=True)
        v2d = v2d.astype(np.int64).ravel()
        n_dofs = int(v2d.max()) + 1
        Ld, origin = tuple(L), tuple(lo)
        return MeshArrays(coords=np.ascontiguousarray(coords), cells=np.ascontiguousarray(cells),
                          bfacets=np.zeros((0, 3), np.int64), btags=np.zeros(0, np.int32), vertex_to_dof=v2d,
                          n_dofs=n_dofs, Ld=Ld, origin=origin, n_objects=0)
    tri, vals = _read_facet_tags(stem + "_facet_region.xml", cells)
    # relabel: sorted distinct tags including the implicit interior value 0
    labels = np.unique(np.concatenate([vals, [0]]))
    relabel = {int(t): k for k, t in enumerate(labels)}
    nv = np.int64(coords.shape[0])
    bkey = (bf[:, 0] * nv + bf[:, 1]) * nv + bf[:, 2]
    tkey = (tri[:, 0] * nv + tri[:, 1]) * nv + tri[:, 2]
    tag_of = dict(zip(tkey.tolist(), (relabel[int(v)] for v in vals)))
    btags = np.array([tag_of.get(int(k), 0) for k in bkey], dtype=np.int32)
    if np.any(btags == 0):
        raise ValueError(f"{stem}_facet_region.xml: {int((btags == 0).sum())} boundary facets carry no boundary tag")
    return MeshArrays(coords=np.ascontiguousarray(coords), cells=np.ascontiguousarray(cells),
                      bfacets=np.ascontiguousarray(bf), btags=btags, vertex_to_dof=None, n_dofs=int(n_dofs),
                      Ld=Ld, origin=origin, n_objects=len(labels) - 2)


def write_mesh(fname: str, ma: MeshArrays, tag_values=None, facet_form: str = "cell"):
    """Write name.xml and name_facet_region.xml.  facet_form "cell": boundary
    tags as a cell-relative mesh value collection; "global": a mesh function
    over every facet in DOLFIN's numbering (interior facets 0), the layout
    dolfin-convert writes.  tag_values maps the mesh's tags 1, 2, .. to the
    values written, e.g. gmsh physical ids."""
    if facet_form not in ("cell", "global"):
        raise ValueError("facet_form is 'cell' or 'global'")
    stem = _stem(fname)
    with open(stem + ".xml", "w") as f:
        f.write('<?xml version="1.0"?>\n<dolfin xmlns:dolfin="http://fenicsproject.org">\n')
        f.write('  <mesh celltype="tetrahedron" dim="3">\n')
        f.write(f'    <vertices size="{ma.n_vertices}">\n')
        for i, (x, y, z) in enumerate(ma.coords.tolist()):
            f.write(f'      <vertex index="{i}" x="{x!r}" y="{y!r}" z="{z!r}" />\n')
        f.write(f'    </vertices>\n    <cells size="{ma.n_cells}">\n')
        for i, c in enumerate(ma.cells.tolist()):
            f.write(f'      <tetrahedron index="{i}" v0="{c[0]}" v1="{c[1]}" v2="{c[2]}" v3="{c[3]}" />\n')
        f.write("    </cells>\n  </mesh>\n</dolfin>\n")
    # each boundary facet as (cell, local facet opposite local vertex i)
    nv = np.int64(ma.n_vertices)
    keys, owner = [], []
    for i in range(4):
        others = np.sort(np.delete(ma.cells, i, axis=1), axis=1)
        keys.append((others[:, 0] * nv + others[:, 1]) * nv + others[:, 2])
        owner.append(np.stack([np.arange(ma.n_cells), np.full(ma.n_cells, i)], axis=1))
    keys = np.concatenate(keys)
    owner = np.concatenate(owner)
    order = np.argsort(keys, kind="stable")
    keys, owner = keys[order], owner[order]
    bf = np.sort(ma.bfacets, axis=1)
    bkeys = (bf[:, 0] * nv + bf[:, 1]) * nv + bf[:, 2]
    pos = np.searchsorted(keys, bkeys)
    if np.any(keys[np.minimum(pos, len(keys) - 1)] != bkeys):
        raise ValueError("a boundary facet is not a facet of any cell")
    cell_local = owner[pos]
    if facet_form == "global":
        facets = dolfin_facet_numbering(ma.cells)
        fkeys = (facets[:, 0] * nv + facets[:, 1]) * nv + facets[:, 2]
        values = np.zeros(len(facets), np.int64)
        at = np.searchsorted(fkeys, bkeys)
        values[at] = [tag_values[t] if tag_values is not None else t for t in ma.btags.tolist()]
        with open(stem + "_facet_region.xml", "w") as f:
            f.write('<?xml version="1.0"?>\n<dolfin xmlns:dolfin="http://fenicsproject.org">\n')
            f.write(f'  <mesh_function type="uint" dim="2" size="{len(facets)}">\n')
            for k, v in enumerate(values.tolist()):
                f.write(f'    <entity index="{k}" value="{v}" />\n')
            f.write("  </mesh_function>\n</dolfin>\n")
        return
    with open(stem + "_facet_region.xml", "w") as f:
        f.write('<?xml version="1.0"?>\n<dolfin xmlns:dolfin="http://fenicsproject.org">\n')
        f.write(f'  <mesh_value_collection type="uint" dim="2" size="{len(bkeys)}">\n')
        for (c, i), t in zip(cell_local.tolist(), ma.btags.tolist()):
            v = tag_values[t] if tag_values is not None else t
            f.write(f'    <value cell_index="{c}" local_entity="{i}" value="{v}" />\n')
        f.write("  </mesh_value_collection>\n</dolfin>\n")
