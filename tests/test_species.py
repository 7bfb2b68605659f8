"""Species weights (punc/src/population.cpp:41-80) on the host: the four ways
of giving the amount of simulation particles, the derived charge, mass,
density, count and Debye length, and min_plasma_period, in the Python front
end and the C++ front end (include/punc_gpu.hpp), which must agree bit for
bit.  No GPU: the mesh tables are built on the host."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from puncpp_gb300 import meshgen, punc
from puncpp_gb300.punc import ParticleAmountType as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
AMOUNTS = {T.in_total: 20000.0, T.per_cell: 16.0, T.per_volume: 40.0, T.phys_per_sim: 3.0}


@pytest.fixture(scope="module")
def box():
    ma = meshgen.kuhn_box(5, -1.0, 1.5)
    return ma, punc.Mesh(ma)


def test_mesh_volume_and_cells(lib, box):
    ma, mesh = box
    assert mesh.num_cells == ma.n_cells
    assert abs(mesh.volume() - 2.5 ** 3) <= 1e-13 * 2.5 ** 3


@pytest.mark.parametrize("kind", list(T))
def test_weights_follow_the_amount_type(kind, lib, box):
    ma, mesh = box
    V, Nc = mesh.volume(), mesh.num_cells
    density, amount = 100.0, AMOUNTS[kind]
    s = punc.Species.from_physical(-1.0, 1.0, density, amount, kind, mesh, vth=1.0)
    expect_w = {T.in_total: density / (amount / V), T.per_cell: density / (amount * Nc / V),
                T.per_volume: density / amount, T.phys_per_sim: amount}[kind]
    assert s.weight == pytest.approx(expect_w, rel=1e-15)
    assert s.q == -s.weight and s.m == s.weight
    assert s.n * s.weight == pytest.approx(density, rel=1e-15)
    expect_num = {T.in_total: amount, T.per_cell: amount * Nc, T.per_volume: amount * V,
                  T.phys_per_sim: density / amount * V}[kind]
    assert abs(s.num - expect_num) <= 1.0 and s.num == int(s.n * V)
    # lambda_D omega_p = vth for a Maxwellian
    wp = math.sqrt(s.q * s.q * s.n / (mesh.eps0 * s.m))
    assert s.debye * wp == pytest.approx(1.0, rel=1e-14)


def test_min_plasma_period_takes_the_fastest_species(lib, box):
    _, mesh = box
    e = punc.Species.from_physical(-1.0, 1.0, 100.0, 16.0, T.per_cell, mesh, vth=1.0)
    i = punc.Species.from_physical(1.0, 1836.0, 100.0, 16.0, T.per_cell, mesh, vth=0.05)
    wp_e = math.sqrt(100.0 / 1.0)        # physical: q^2 n / (eps0 m), weight-free
    assert punc.min_plasma_period([i, e], 1.0) == pytest.approx(2 * math.pi / wp_e, rel=1e-14)
    assert punc.min_plasma_period([i], 1.0) > punc.min_plasma_period([i, e], 1.0)


def test_cpp_front_end_agrees_bitwise(lib, box, tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    ma, mesh = box
    libdir = os.path.join(ROOT, "puncpp_gb300")
    exe = tmp_path / "species_check"
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "species_check.cpp"), "-L" + libdir, "-lpunc_gpu",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    files = []
    for name, arr, dt in (("co", ma.coords, np.float64), ("ce", ma.cells, np.int64), ("bf", ma.bfacets, np.int64),
                          ("bt", ma.btags, np.int32)):
        f = tmp_path / name
        np.ascontiguousarray(arr, dt).tofile(f)
        files.append(str(f))
    out = subprocess.run([str(exe)] + files, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().split("\n")
    assert len(lines) == 6
    species = []
    for line, kind in zip(lines, [T.in_total, T.per_cell, T.per_volume, T.phys_per_sim]):
        w, q, m, n, num, debye = line.split()
        s = punc.Species.from_physical(-1.0, 1.0, 100.0, AMOUNTS[kind], kind, mesh, vth=1.0, vd=(0.5, 0.0, -0.25))
        assert (float(w), float(q), float(m), float(n), int(num), float(debye)) == \
            (s.weight, s.q, s.m, s.n, s.num, s.debye), kind
        species += [s, punc.Species.from_physical(1.0, 1836.0, 100.0, AMOUNTS[kind], kind, mesh, vth=0.05)]
    period, volume = (float(x) for x in lines[4].split())
    assert volume == mesh.volume()
    assert period == punc.min_plasma_period(species, 1.0)
    s_dv, s_dv1 = (float(x) for x in lines[5].split())
    assert s_dv == float(np.cumsum(punc.element_volume(mesh, True))[-1])
    assert s_dv1 == float(np.cumsum(punc.element_volume(mesh, False))[-1])


@pytest.mark.parametrize("voronoi", [True, False])
def test_element_volume(voronoi, lib, box):
    """element_volume (punc/src/distributor.cpp:35-69) from the cell volumes:
    each dof's patch is the cells around its vertex."""
    ma, mesh = box
    vol = mesh.table(punc.L.T_VOLUME)
    patch = np.zeros(mesh.n_dofs)
    for k in range(4):
        np.add.at(patch, ma.cells[:, k], vol)
    dv = punc.element_volume(mesh, voronoi)
    np.testing.assert_allclose(dv, (4.0 if voronoi else 1.0) / patch, rtol=1e-13)
    # the patches cover the mesh four times
    assert np.sum((4.0 if voronoi else 1.0) / dv) == pytest.approx(4 * mesh.volume(), rel=1e-13)
