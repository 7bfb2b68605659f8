"""DOLFIN XML mesh ingest (punc/src/mesh.cpp:41-84): write a generated mesh
as name.xml + name_facet_region.xml, read it back, and get the same arrays with
the tags relabelled as the reference does (sorted distinct values -> 0, 1, 2 ..)."""
import numpy as np
import pytest

from puncpp_gb300 import dolfin_xml, meshgen


def test_round_trip_with_relabelled_tags(tmp_path):
    ma = meshgen.probe_box(5, 2.0, 0.6)
    fname = tmp_path / "probe.xml"
    # write gmsh-like physical ids: exterior 17, object 31
    dolfin_xml.write_mesh(fname, ma, tag_values={1: 17, 2: 31})
    mb = dolfin_xml.read_mesh(fname)
    np.testing.assert_array_equal(mb.coords, ma.coords)
    np.testing.assert_array_equal(mb.cells, ma.cells)
    key = lambda m: {tuple(f): t for f, t in zip(np.sort(m.bfacets, axis=1).tolist(), m.btags.tolist())}
    assert key(mb) == key(ma)
    assert mb.n_objects == 1 and mb.n_dofs == ma.n_vertices


def test_dolfin_facet_numbering_by_hand():
    """Two tetrahedra sharing facet (1, 2, 3): DOLFIN's serial numbering sorts
    the distinct vertex triples lexicographically, whatever the cells' vertex
    order."""
    cells = np.array([[3, 1, 0, 2], [4, 2, 1, 3]])
    f = dolfin_xml.dolfin_facet_numbering(cells)
    assert f.tolist() == [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]]


def test_round_trip_through_the_global_facet_numbering(tmp_path):
    """The layout dolfin-convert writes: a mesh function over every facet,
    indexed by DOLFIN's facet numbering, interior facets 0.  Reading it gives
    the same boundary tags as the cell-relative form."""
    ma = meshgen.probe_box(6, 2.0, 0.6)
    # renumber the vertices so that the numbering is not the generator's order
    rng = np.random.default_rng(5)
    perm = rng.permutation(ma.n_vertices)
    coords = np.empty_like(ma.coords)
    coords[perm] = ma.coords
    mp = meshgen.MeshArrays(coords=coords, cells=perm[ma.cells], bfacets=perm[ma.bfacets], btags=ma.btags.copy(),
                            n_dofs=ma.n_dofs, Ld=ma.Ld, origin=ma.origin, n_objects=1)
    dolfin_xml.write_mesh(tmp_path / "g.xml", mp, tag_values={1: 17, 2: 31}, facet_form="global")
    text = (tmp_path / "g_facet_region.xml").read_text()
    n_facets = len(dolfin_xml.dolfin_facet_numbering(mp.cells))
    assert f'<mesh_function type="uint" dim="2" size="{n_facets}">' in text and "<entity index=" in text
    dolfin_xml.write_mesh(tmp_path / "c.xml", mp, tag_values={1: 17, 2: 31}, facet_form="cell")
    mg, mc = dolfin_xml.read_mesh(tmp_path / "g.xml"), dolfin_xml.read_mesh(tmp_path / "c.xml")
    key = lambda m: {tuple(f): t for f, t in zip(np.sort(m.bfacets, axis=1).tolist(), m.btags.tolist())}
    assert key(mg) == key(mc) == key(mp)
    assert mg.n_objects == 1


def test_global_facet_index_out_of_range_is_refused(tmp_path):
    ma = meshgen.probe_box(3, 2.0, 0.6)
    fname = tmp_path / "m.xml"
    dolfin_xml.write_mesh(fname, ma)
    n = len(dolfin_xml.dolfin_facet_numbering(ma.cells))
    (tmp_path / "m_facet_region.xml").write_text(
        '<?xml version="1.0"?>\n<dolfin><mesh_function type="uint" dim="2" size="1">'
        f'<entity index="{n}" value="1" /></mesh_function></dolfin>\n')
    with pytest.raises(ValueError, match="facet index out of range"):
        dolfin_xml.read_mesh(fname)


def test_untagged_boundary_facets_are_an_error(tmp_path):
    ma = meshgen.probe_box(3, 2.0, 0.6)
    fname = tmp_path / "m.xml"
    dolfin_xml.write_mesh(fname, ma)
    region = tmp_path / "m_facet_region.xml"
    lines = region.read_text().split("\n")
    region.write_text("\n".join(l for k, l in enumerate(lines) if not (k == 3)))
    with pytest.raises(ValueError, match="carry no boundary tag"):
        dolfin_xml.read_mesh(fname)


def test_periodic_box_identifies_opposite_faces(tmp_path):
    ma = meshgen.langmuir_cube(4)
    fname = tmp_path / "cube.xml"
    dolfin_xml.write_mesh(fname, ma)
    mb = dolfin_xml.read_mesh(fname, periodic_box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)))
    assert mb.n_dofs == ma.n_dofs == 64
    # the same vertex classes as the generator's periodic map
    pairs = {(int(a), int(b)) for a, b in zip(ma.vertex_to_dof, mb.vertex_to_dof)}
    assert len(pairs) == ma.n_dofs


def test_only_xml_meshes_are_read(tmp_path):
    with pytest.raises(ValueError, match="only DOLFIN .xml"):
        dolfin_xml.read_mesh(tmp_path / "m.h5")


def test_non_tetrahedral_cells_are_refused(tmp_path):
    ma = meshgen.probe_box(3, 2.0, 0.6)
    fname = tmp_path / "m.xml"
    dolfin_xml.write_mesh(fname, ma)
    text = fname.read_text()
    assert 'celltype="tetrahedron"' in text
    fname.write_text(text.replace('celltype="tetrahedron"', 'celltype="triangle"'))
    with pytest.raises(ValueError, match="only tetrahedra"):
        dolfin_xml.read_mesh(fname)


def test_facet_tags_of_another_dimension_are_refused(tmp_path):
    ma = meshgen.probe_box(3, 2.0, 0.6)
    fname = tmp_path / "m.xml"
    dolfin_xml.write_mesh(fname, ma)
    region = tmp_path / "m_facet_region.xml"
    text = region.read_text()
    assert 'dim="2"' in text
    region.write_text(text.replace('dim="2"', 'dim="1"'))
    with pytest.raises(ValueError, match="dim 2"):
        dolfin_xml.read_mesh(fname)


def test_missing_cells_are_an_error(tmp_path):
    ma = meshgen.probe_box(3, 2.0, 0.6)
    fname = tmp_path / "m.xml"
    dolfin_xml.write_mesh(fname, ma)
    lines = fname.read_text().split("\n")
    k = next(i for i, l in enumerate(lines) if "<tetrahedron " in l)
    fname.write_text("\n".join(lines[:k] + lines[k + 1:]))
    with pytest.raises(ValueError, match="missing vertices or cells"):
        dolfin_xml.read_mesh(fname)
