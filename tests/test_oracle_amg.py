"""The oracle's AMG-preconditioned CG, the Poisson solver of the timed CPU
baseline (the reference's solver class: Krylov + algebraic multigrid,
punc/src/poisson.cpp:297-304), checked on the CPU: the same solution as the
direct sparse solve for Dirichlet objects and for the periodic null space,
several times fewer iterations than Jacobi-PCG, and the same result for any
thread count."""
import numpy as np

from puncpp_gb300 import meshgen


def _load(o, ma, n, seed):
    rng = np.random.default_rng(seed)
    lo, L = np.asarray(ma.origin, float), np.asarray(ma.Ld, float)
    xs = lo + rng.random((n, 3)) * L
    o.add_particles(xs, rng.normal(size=xs.shape), -1.0, 1.0)
    return o.distribute_cg1()


def test_amg_pcg_matches_direct_solve_with_few_iterations(oracle_mod):
    ma = meshgen.probe_box(24, 4.0, 0.8)
    o = oracle_mod.Oracle(ma)
    rho = _load(o, ma, 40000, 1)
    xd = o.poisson_direct(rho, potentials=[-2.0])
    xa, ita = o.poisson_amg(rho, potentials=[-2.0], rtol=1e-12, atol=1e-300, max_iter=500, nthreads=4)
    xj, itj = o.poisson_pcg(rho, potentials=[-2.0], rtol=1e-12, atol=1e-300, max_iter=20000, nthreads=4)
    assert np.abs(xa - xd).max() < 1e-10 * np.abs(xd).max()
    assert ita * 4 < itj, (ita, itj)
    rows = o.amg_levels()
    assert len(rows) >= 3 and rows == sorted(rows, reverse=True) and rows[-1] <= 400
    x1, it1 = o.poisson_amg(rho, potentials=[-2.0], rtol=1e-12, atol=1e-300, max_iter=500, nthreads=1)
    assert it1 == ita and np.array_equal(x1, xa)


def test_amg_pcg_periodic_null_space(oracle_mod):
    ma = meshgen.langmuir_cube(12)
    o = oracle_mod.Oracle(ma)
    rho = _load(o, ma, 30000, 2)
    xd = o.poisson_direct(rho, periodic=True)
    xa, ita = o.poisson_amg(rho, periodic=True, rtol=1e-12, atol=1e-300, max_iter=500, nthreads=4)
    assert abs(xa.mean()) < 1e-13 * np.abs(xa).max()
    assert np.abs(xa - xd).max() < 1e-10 * np.abs(xd).max() and 0 < ita < 60
