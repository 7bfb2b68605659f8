"""The body-fitted spherical shell (the geometry of the reference's
test/sphere.geo: object sphere r = 1 inside the exterior sphere r = 20),
checked on the CPU: conforming (the only boundary facets are the two spheres,
each facet of the shell interior shared by exactly two cells), no degenerate
cell, volume and object area close to the exact sphere values, and accepted by
the engine's mesh builder with the object's facets tagged."""
import numpy as np

from puncpp_gb300 import _lib as L
from puncpp_gb300 import meshgen, punc


def test_sphere_shell_is_conforming_and_close_to_the_spheres(lib):
    ma = meshgen.sphere_shell(1.0, 20.0, level=3)
    co, ce = ma.coords, ma.cells
    bf = meshgen._boundary_facets(ce, co.shape[0])
    given = np.sort(ma.bfacets, axis=1)
    key = lambda f: set(map(tuple, f))
    assert key(bf) == key(given) and len(bf) == len(given) == 2 * 1280
    p = co[ce]
    vol = np.abs(np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))) / 6
    assert vol.min() > 1e-3 * np.median(vol[: 1280 * 3]) and vol.min() > 0
    exact = 4.0 / 3.0 * np.pi * (20.0 ** 3 - 1.0)
    assert abs(vol.sum() - exact) < 0.01 * exact
    r = np.linalg.norm(co[ma.bfacets], axis=2)
    assert np.allclose(r[ma.btags == 2], 1.0) and np.allclose(r[ma.btags == 1], 20.0)
    t = co[ma.bfacets[ma.btags == 2]]
    area = 0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1).sum()
    assert abs(area - 4 * np.pi) < 0.01 * 4 * np.pi
    mesh = punc.Mesh(ma)
    assert mesh.n_dofs == co.shape[0] and mesh.num_objects == 1
    of = mesh.table(L.T_OBJ_FACETS).reshape(-1, 7)
    assert len(of) == 1280 and np.all(of[:, 1] == 0)
    ef = mesh.table(L.T_EXT_FACETS).reshape(-1, 14)
    assert len(ef) == 1280 and abs(ef[:, 0].sum() - 4 * np.pi * 400) < 0.01 * 4 * np.pi * 400
