"""Host mesh tables of the engine (pg_mesh_build) against the oracle's
restatement of Population<3> / Cell<3> / element_volume / exterior_boundaries:
bit-identical, including the facet planes that decide every cell index."""
import numpy as np
import pytest

from puncpp_gb300 import meshgen, punc
from puncpp_gb300 import _lib as L

MESHES = {
    "periodic_4": lambda: meshgen.langmuir_cube(4),
    "periodic_16": lambda: meshgen.langmuir_cube(16),
    "probe_12": lambda: meshgen.probe_box(12, 3.0, 1.0),
    "probe_20_unit_hole": lambda: meshgen.probe_box(20, 10.0, 1.0),
    "shell_mapped": lambda: meshgen.mapped_sphere_shell(8, 1, 0.2, 1.0),
}


def _pairs(O):
    return [(L.T_CELL_VERTICES, O.T_CELLV), (L.T_BARYCENTRIC, O.T_BARY), (L.T_PLANES, O.T_PLANES),
            (L.T_NEIGHBOURS, O.T_NBR), (L.T_CELL_DOFS, O.T_DOFS), (L.T_VOLUME, O.T_VOLUME),
            (L.T_DV_INV, O.T_DV_INV), (L.T_CSR_ROWPTR, O.T_ROWPTR), (L.T_CSR_COL, O.T_COL),
            (L.T_STIFFNESS, O.T_K), (L.T_MASS, O.T_M), (L.T_EXT_FACETS, O.T_EXT), (L.T_BC_KIND, O.T_BC),
            (L.T_OBJ_FACETS, O.T_OFAC)]


@pytest.mark.parametrize("name", sorted(MESHES))
def test_tables_bitwise_equal_oracle(name, lib, oracle_mod):
    ma = MESHES[name]()
    m = punc.Mesh(ma)
    o = oracle_mod.Oracle(ma)
    for a, b in _pairs(oracle_mod):
        x, y = m.table(a), o.table(b)
        assert x.dtype == y.dtype and x.shape == y.shape, (a, x.shape, y.shape)
        if a in (L.T_STIFFNESS, L.T_MASS):
            # element sums accumulate in a different order (CSR search vs map)
            np.testing.assert_allclose(x, y, rtol=1e-13, atol=1e-15 * np.abs(y).max())
        else:
            assert np.array_equal(x.view(np.uint64) if x.dtype == np.float64 else x,
                                  y.view(np.uint64) if y.dtype == np.float64 else y), f"table {a} differs"


def test_planes_are_outward_unit_normals(lib):
    ma = meshgen.probe_box(6, 2.0, 0.5)
    m = punc.Mesh(ma)
    pl = m.table(L.T_PLANES).reshape(-1, 4, 4)
    cv = m.table(L.T_CELL_VERTICES).reshape(-1, 4)
    n = pl[:, :, 1:]
    np.testing.assert_allclose(np.linalg.norm(n, axis=2), 1.0, rtol=1e-14)
    P = ma.coords[cv]
    for f in range(4):
        # the opposite vertex is strictly inside (negative side), facet vertices on the plane
        d_opp = pl[:, f, 0] + np.einsum("ij,ij->i", n[:, f], P[:, f])
        assert np.all(d_opp < 0)
        for i in range(4):
            if i != f:
                d = pl[:, f, 0] + np.einsum("ij,ij->i", n[:, f], P[:, i])
                assert np.abs(d).max() < 1e-14


def test_barycentric_partition_of_unity(lib):
    ma = meshgen.probe_box(6, 2.0, 0.5)
    m = punc.Mesh(ma)
    A = m.table(L.T_BARYCENTRIC).reshape(-1, 3, 4)
    cv = m.table(L.T_CELL_VERTICES).reshape(-1, 4)
    P = ma.coords[cv]
    for i in range(4):
        lam = A[:, :, 0] + np.einsum("ijk,ik->ij", A[:, :, 1:], P[:, i])
        expect = np.zeros((A.shape[0], 3))
        if i < 3:
            expect[:, i] = 1.0
        np.testing.assert_allclose(lam, expect, atol=1e-12)


def test_neighbour_symmetry_and_tags(lib):
    ma = meshgen.probe_box(8, 4.0, 1.0)
    m = punc.Mesh(ma)
    nb = m.table(L.T_NEIGHBOURS).reshape(-1, 4)
    for c in range(nb.shape[0]):
        for f in range(4):
            t = nb[c, f]
            if t >= 0:
                assert c in nb[t]
            else:
                assert t in (-1, -2)
    assert (nb == -2).any() and (nb == -1).any()


def test_stiffness_rows_sum_to_zero_and_mass_to_volume(lib):
    ma = meshgen.langmuir_cube(6)
    m = punc.Mesh(ma)
    rp, K, M = m.table(L.T_CSR_ROWPTR), m.table(L.T_STIFFNESS), m.table(L.T_MASS)
    rows = np.add.reduceat(K, rp[:-1])
    assert np.abs(rows).max() < 1e-12
    assert abs(M.sum() - 1.0) < 1e-12


def test_untagged_boundary_facet_is_a_mesh_error(lib):
    ma = meshgen.probe_box(4, 1.0, 0.3)
    ma.bfacets = ma.bfacets[1:]
    ma.btags = ma.btags[1:]
    with pytest.raises(L.PgError) as e:
        punc.Mesh(ma)
    assert e.value.code == 3


def test_degenerate_cell_is_a_mesh_error(lib):
    ma = meshgen.probe_box(4, 1.0, 0.3)
    ma.coords = ma.coords.copy()
    c0 = ma.cells[0]
    ma.coords[c0[3]] = ma.coords[c0[0]] + 0.5 * (ma.coords[c0[1]] - ma.coords[c0[0]])
    with pytest.raises(L.PgError) as e:
        punc.Mesh(ma)
    assert e.value.code == 3


def test_repeated_vertex_is_a_mesh_error(lib):
    ma = meshgen.probe_box(4, 1.0, 0.3)
    ma.cells = ma.cells.copy()
    ma.cells[0, 1] = ma.cells[0, 0]
    with pytest.raises(L.PgError):
        punc.Mesh(ma)


def _interior_cell(ma):
    """A cell none of whose facets is a boundary facet."""
    bnd = {tuple(f) for f in np.sort(ma.bfacets, axis=1).tolist()}
    for c, cell in enumerate(ma.cells):
        faces = [tuple(sorted(int(v) for k, v in enumerate(cell) if k != i)) for i in range(4)]
        if not any(f in bnd for f in faces):
            return c
    raise AssertionError("no interior cell")


def test_facet_shared_by_three_cells_is_a_mesh_error(lib):
    ma = meshgen.probe_box(4, 1.0, 0.3)
    c = _interior_cell(ma)
    ma.cells = np.ascontiguousarray(np.concatenate([ma.cells, ma.cells[c:c + 1]]))
    with pytest.raises(L.PgError, match="shared by more than two cells") as e:
        punc.Mesh(ma)
    assert e.value.code == 3


@pytest.mark.parametrize("what", ["cell_vertex", "facet_vertex", "tag"])
def test_out_of_range_inputs_are_mesh_errors(what, lib):
    ma = meshgen.probe_box(4, 1.0, 0.3)
    if what == "cell_vertex":
        ma.cells = ma.cells.copy()
        ma.cells[3, 2] = ma.n_vertices
    elif what == "facet_vertex":
        ma.bfacets = ma.bfacets.copy()
        ma.bfacets[0, 1] = -1
    else:
        ma.btags = ma.btags.copy()
        ma.btags[0] = 0
    with pytest.raises(L.PgError) as e:
        punc.Mesh(ma)
    assert e.value.code == 3


def test_tables_do_not_depend_on_the_vertex_order_within_cells(lib):
    """Cells may list their vertices in any order (the builder sorts them into
    the ascending UFC order): permuting each cell's vertex ids and each
    boundary facet's gives bit-identical tables."""
    ma = meshgen.probe_box(5, 1.0, 0.3)
    rng = np.random.default_rng(21)
    mb = meshgen.MeshArrays(coords=ma.coords, cells=np.ascontiguousarray(rng.permuted(ma.cells, axis=1)),
                            bfacets=np.ascontiguousarray(rng.permuted(ma.bfacets, axis=1)), btags=ma.btags,
                            n_dofs=ma.n_dofs, Ld=ma.Ld, origin=ma.origin, n_objects=ma.n_objects)
    assert not np.array_equal(mb.cells, ma.cells)
    a, b = punc.Mesh(ma), punc.Mesh(mb)
    for t in (L.T_CELL_VERTICES, L.T_BARYCENTRIC, L.T_PLANES, L.T_NEIGHBOURS, L.T_CELL_DOFS, L.T_VOLUME,
              L.T_DV_INV, L.T_EXT_FACETS):
        np.testing.assert_array_equal(a.table(t), b.table(t), err_msg=str(t))


def test_tables_do_not_depend_on_the_boundary_facet_list_order(lib):
    ma = meshgen.probe_box(5, 1.0, 0.3)
    perm = np.random.default_rng(22).permutation(len(ma.btags))
    mb = meshgen.MeshArrays(coords=ma.coords, cells=ma.cells, bfacets=np.ascontiguousarray(ma.bfacets[perm]),
                            btags=np.ascontiguousarray(ma.btags[perm]), n_dofs=ma.n_dofs, Ld=ma.Ld,
                            origin=ma.origin, n_objects=ma.n_objects)
    a, b = punc.Mesh(ma), punc.Mesh(mb)
    for t in (L.T_NEIGHBOURS, L.T_EXT_FACETS, L.T_BC_KIND, L.T_OBJ_FACETS):
        np.testing.assert_array_equal(a.table(t), b.table(t), err_msg=str(t))
