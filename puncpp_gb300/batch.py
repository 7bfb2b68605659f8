"""Batched runs: many independent probe runs (different meshes, particle counts,
biases and seeds) advancing together, every stage one launch for all of them.

The runs become one engine over the disjoint union of their meshes, with
per-run offset tables: run r's vertices, cells and dofs follow run r-1's, its
object carries its own tag (2 + r), and its exterior facets follow run r-1's in
the engine's facet order.  Nothing couples the runs: the facet walk, push and
deposit stay inside a run's cells, the Poisson matrix and its AMG hierarchy
are block-diagonal, the CircuitCM capacitance matrix is diagonal in the runs,
and each run's object has its own voltage source.  Meshes keep their own
coordinates (runs overlap in space), so particles are located inside their
run's cell range, and injection draws, per exterior facet, the random stream
of the run's standalone mesh (run-local facet index, the run's seed).

The solver's stopping test is on the whole batch (||r|| <= rtol ||b|| over all
runs); a run's potential is accurate to the batch tolerance.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import punc
from .meshgen import MeshArrays


def union(meshes):
    """The disjoint union of non-periodic meshes and its offset tables."""
    coords, cells, bf, bt = [], [], [], []
    v_off = [0]
    c_off = [0]
    o_off = [0]
    for ma in meshes:
        if ma.vertex_to_dof is not None:
            raise ValueError("batched runs need non-periodic meshes")
        coords.append(ma.coords)
        cells.append(ma.cells + v_off[-1])
        bf.append(ma.bfacets + v_off[-1])
        bt.append(np.where(ma.btags == 1, 1, ma.btags + o_off[-1]).astype(np.int32))
        v_off.append(v_off[-1] + ma.n_vertices)
        c_off.append(c_off[-1] + ma.n_cells)
        o_off.append(o_off[-1] + ma.n_objects)
    u = MeshArrays(coords=np.ascontiguousarray(np.concatenate(coords)), cells=np.ascontiguousarray(np.concatenate(cells)),
                   bfacets=np.ascontiguousarray(np.concatenate(bf)), btags=np.concatenate(bt),
                   n_dofs=int(v_off[-1]), Ld=meshes[0].Ld, origin=meshes[0].origin, n_objects=int(o_off[-1]))
    return u, {"vertex": np.array(v_off), "cell": np.array(c_off), "object": np.array(o_off)}


def facet_runs(mesh, cell_off):
    """Run and run-local index of each exterior facet of the union mesh, in
    the engine's facet order (a facet belongs to the run of its cell)."""
    ext = mesh.table(L.T_EXT_FACETS).reshape(-1, 14)
    cell = ext[:, 13].astype(np.int64)
    run = np.searchsorted(cell_off, cell, side="right") - 1
    first = np.searchsorted(run, np.arange(len(cell_off) - 1), side="left")
    return run, (np.arange(len(cell)) - first[run]).astype(np.uint32)


class Batch:
    """R runs in one engine.  Object k of run r is object o_off[r] + k of the
    batch (boundary tag 2 + o_off[r] + k)."""

    def __init__(self, meshes, **population_kwargs):
        self.meshes = list(meshes)
        self.union, self.off = union(self.meshes)
        self.mesh = punc.Mesh(self.union)
        self.pop = punc.Population(self.mesh, **population_kwargs)
        self.facet_run, self.facet_local = facet_runs(self.mesh, self.off["cell"])
        self.n_runs = len(self.meshes)

    def add_particles(self, r: int, xs, vs, q: float, m: float) -> int:
        x = np.ascontiguousarray(xs, np.float64)
        v = np.ascontiguousarray(vs, np.float64)
        n = C.c_int64()
        L.check(L.load().pg_add_particles_range(self.pop.handle, L.dptr(x), L.dptr(v), len(x), q, m,
                                                 int(self.off["cell"][r]), int(self.off["cell"][r + 1]), C.byref(n)))
        return n.value

    def create_flux(self, species, seeds):
        """Flux injection of the species on every run's exterior; run r's streams
        are keyed by seeds[r] (the key its standalone run uses with seed=seeds[r])."""
        punc.create_flux(self.pop, species)
        c1 = np.ascontiguousarray(self.facet_local, np.uint32)
        sd = np.ascontiguousarray(np.asarray(seeds, np.uint64)[self.facet_run], np.uint64)
        L.check(L.load().pg_set_injection_streams(self.pop.handle, c1.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                   sd.ctypes.data_as(C.POINTER(C.c_uint64))))

    def objects(self):
        return [punc.Object(2 + k) for k in range(int(self.off["object"][-1]))]

    def circuit(self, objects, biases, dt: float):
        """One voltage source from ground to the first object of each run."""
        vs = [(-1, int(self.off["object"][r]), float(biases[r])) for r in range(self.n_runs)]
        return punc.CircuitCM(self.pop, objects, vs, [], dt)

    def particles_per_run(self) -> np.ndarray:
        cell = self.pop.particles()["cell"]
        return np.bincount(np.searchsorted(self.off["cell"], cell, side="right") - 1, minlength=self.n_runs)

    def run_particles(self, r: int) -> dict:
        p = self.pop.particles()
        keep = (p["cell"] >= self.off["cell"][r]) & (p["cell"] < self.off["cell"][r + 1])
        out = {k: v[keep] for k, v in p.items()}
        out["cell"] = out["cell"] - self.off["cell"][r]
        return out
