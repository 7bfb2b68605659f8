"""Batched runs on the host side: the union mesh's tables restricted to a run
equal the run's own tables (cells, exterior facets in the same order), which
is what lets each run draw its standalone injection streams."""
import numpy as np

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
