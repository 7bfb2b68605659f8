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


def test_refuses_global_facet_numbering(tmp_path):
    ma = meshgen.probe_box(3, 2.0, 0.6)
    fname = tmp_path / "m.xml"
    dolfin_xml.write_mesh(fname, ma)
    (tmp_path / "m_facet_region.xml").write_text(
        '<?xml version="1.0"?>\n<dolfin><mesh_function type="uint" dim="2" size="1">'
        '<entity index="0" value="1" /></mesh_function></dolfin>\n')
    with pytest.raises(ValueError, match="global facet numbering"):
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
