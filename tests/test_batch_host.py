"""Batched runs on the host side: the union mesh's tables restricted to a run
equal the run's own tables (cells, exterior facets in the same order), which
is what lets each run draw its standalone injection streams."""
import numpy as np
import pytest

from puncpp_gb300 import _lib as L
from puncpp_gb300 import batch, meshgen, punc


def test_union_tables_restrict_to_the_runs(lib):
    meshes = [meshgen.probe_box(6, 2.0, 0.6), meshgen.probe_box(5, 2.5, 0.7), meshgen.probe_box(3, 2.0, 0.5)]
    u, off = batch.union(meshes)
    assert u.n_objects == 3 and set(np.unique(u.btags)) == {1, 2, 3, 4}
    mu = punc.Mesh(u)
    ext_u = mu.table(L.T_EXT_FACETS).reshape(-1, 14)
    start = 0
    for r, ma in enumerate(meshes):
        m = punc.Mesh(ma)
        ext = m.table(L.T_EXT_FACETS).reshape(-1, 14)
        part = ext_u[start:start + len(ext)].copy()
        part[:, 13] -= off["cell"][r]
        np.testing.assert_array_equal(part, ext)
        bary_u = mu.table(L.T_BARYCENTRIC).reshape(-1, 12)[off["cell"][r]:off["cell"][r + 1]]
        np.testing.assert_array_equal(bary_u, m.table(L.T_BARYCENTRIC).reshape(-1, 12))
        start += len(ext)
    assert start == len(ext_u)


def test_union_offsets_and_object_tags():
    meshes = [meshgen.probe_box(4, 2.0, 0.6), meshgen.probe_box(5, 2.5, 0.7)]
    u, off = batch.union(meshes)
    np.testing.assert_array_equal(off["vertex"], [0, meshes[0].n_vertices, meshes[0].n_vertices + meshes[1].n_vertices])
    np.testing.assert_array_equal(off["cell"], [0, meshes[0].n_cells, meshes[0].n_cells + meshes[1].n_cells])
    np.testing.assert_array_equal(off["object"], [0, 1, 2])
    assert u.n_dofs == u.n_vertices == off["vertex"][-1]
    nb0 = len(meshes[0].btags)
    # exterior facets keep tag 1; run r's object becomes tag 2 + r
    np.testing.assert_array_equal(u.btags[:nb0], meshes[0].btags)
    np.testing.assert_array_equal(u.btags[nb0:], np.where(meshes[1].btags == 1, 1, meshes[1].btags + 1))
    # run 1's cells and facets index run 1's vertices only
    assert u.cells[meshes[0].n_cells:].min() == off["vertex"][1]
    assert u.bfacets[nb0:].min() >= off["vertex"][1]
    np.testing.assert_array_equal(u.coords[off["vertex"][1]:], meshes[1].coords)


def test_single_run_union_is_the_mesh():
    ma = meshgen.probe_box(4, 2.0, 0.6)
    u, off = batch.union([ma])
    np.testing.assert_array_equal(u.cells, ma.cells)
    np.testing.assert_array_equal(u.btags, ma.btags)
    np.testing.assert_array_equal(off["cell"], [0, ma.n_cells])


def test_periodic_meshes_are_refused():
    with pytest.raises(ValueError):
        batch.union([meshgen.langmuir_cube(4)])


def test_facet_runs_give_run_local_streams(lib):
    meshes = [meshgen.probe_box(3, 2.0, 0.5), meshgen.probe_box(5, 2.5, 0.7), meshgen.probe_box(4, 2.0, 0.6)]
    u, off = batch.union(meshes)
    run, local = batch.facet_runs(punc.Mesh(u), off["cell"])
    assert np.all(np.diff(run) >= 0)
    for r, ma in enumerate(meshes):
        n_ext = len(punc.Mesh(ma).table(L.T_EXT_FACETS).reshape(-1, 14))
        assert (run == r).sum() == n_ext
        np.testing.assert_array_equal(local[run == r], np.arange(n_ext, dtype=np.uint32))
