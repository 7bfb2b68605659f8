"""Invariants of the oracle itself (CPU).  The engine is checked against the
oracle, so the oracle must be deterministic across thread counts (the timed
CPU baseline runs it on many threads), conserve charge in its deposit, keep
every particle in the cell that contains it after relocation, and draw
injection streams that depend only on (seed, step)."""
import numpy as np

from puncpp_gb300 import meshgen


def _loaded(oracle_mod, n=6000, seed=5):
    ma = meshgen.probe_box(6, 2.0, 0.6)
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(seed)
    xs = rng.uniform(-2.0, 2.0, (n, 3))
    xs = xs[np.linalg.norm(xs, axis=1) > 1.0]
    vs = rng.normal(0.0, 1.0, (len(xs), 3))
    added = o.add_particles(xs, vs, -1.0, 1.0)
    assert added == len(xs)
    return ma, o


def _step(o, phi, nthreads):
    E = o.efield(phi)
    o.boris(E, np.array([0.0, 0.0, 0.3]), 0.2, nthreads=nthreads)
    o.move(0.2, nthreads=nthreads)
    objects = [dict(bnd_id=2, charge=0.0, current=0.0, potential=0.0)]
    absorbed = o.update(objects, 0.2, nthreads=nthreads)
    return absorbed, objects, o.distribute_cg1(nthreads=nthreads)


def test_thread_count_does_not_change_the_oracle(oracle_mod):
    _, o1 = _loaded(oracle_mod)
    _, o4 = _loaded(oracle_mod)
    phi = np.random.default_rng(1).normal(0.0, 0.5, o1.ndof)
    for _ in range(3):
        a1, ob1, rho1 = _step(o1, phi, 1)
        a4, ob4, rho4 = _step(o4, phi, 4)
        np.testing.assert_array_equal(a1, a4)
        assert ob1[0]["charge"] == ob4[0]["charge"]
        p1, p4 = o1.particles(), o4.particles()
        for k in ("x", "v", "cell", "id"):
            np.testing.assert_array_equal(p1[k], p4[k])
        np.testing.assert_allclose(rho4, rho1, rtol=1e-12, atol=1e-12 * np.abs(rho1).max())


def test_deposit_conserves_charge(oracle_mod):
    _, o = _loaded(oracle_mod)
    rho = o.distribute_cg1()
    dof_volume = 1.0 / o.table(oracle_mod.T_DV_INV)
    q = o.particles()["q"]
    assert abs(rho @ dof_volume - q.sum()) <= 1e-12 * abs(q.sum())


def test_relocation_keeps_particles_in_their_cells(oracle_mod):
    _, o = _loaded(oracle_mod)
    n0 = o.num_particles()
    phi = np.random.default_rng(2).normal(0.0, 0.5, o.ndof)
    absorbed, objects, _ = _step(o, phi, 2)
    p = o.particles()
    # every particle absorbed, at the object or the exterior, or still inside
    assert n0 - len(p["q"]) == absorbed.sum()
    assert absorbed.sum() > 0
    # the object's charge is the absorbed charge at tag 2
    assert objects[0]["charge"] == -1.0 * absorbed[2]
    np.testing.assert_array_equal(o.locate(p["x"]), p["cell"])


def test_injection_streams_depend_only_on_seed_and_step(oracle_mod):
    ma = meshgen.kuhn_box(4, -1.0, 1.0)
    runs = []
    for step in (7, 7, 8):
        o = oracle_mod.Oracle(ma)
        o.create_flux([dict(q=-1.0, m=1.0, n=50.0, vth=1.0)])
        n, _ = o.inject(0.1, 99, step)
        assert n > 0
        runs.append(o.particles())
    for k in ("x", "v", "cell"):
        np.testing.assert_array_equal(runs[0][k], runs[1][k])
    assert len(runs[0]["q"]) != len(runs[2]["q"]) or not np.array_equal(runs[0]["x"], runs[2]["x"])


def test_empty_population_passes_every_stage(oracle_mod):
    ma = meshgen.probe_box(4, 2.0, 0.6)
    o = oracle_mod.Oracle(ma)
    assert o.add_particles(np.zeros((0, 3)), np.zeros((0, 3)), -1.0, 1.0) == 0
    E = o.efield(np.zeros(o.ndof))
    o.boris(E, np.array([0.0, 0.0, 1.0]), 0.1)
    o.move(0.1)
    objects = [dict(bnd_id=2, charge=0.0, current=0.0, potential=0.0)]
    assert o.update(objects, 0.1).sum() == 0
    assert objects[0]["charge"] == 0.0 and objects[0]["current"] == 0.0
    assert not o.distribute_cg1().any()
    assert o.kinetic_energy() == 0.0 and o.num_particles() == 0


def test_periodic_move_wraps_into_the_box(oracle_mod):
    ma = meshgen.langmuir_cube(4)
    o = oracle_mod.Oracle(ma)
    Ld = np.asarray(ma.Ld, float)
    rng = np.random.default_rng(4)
    xs = rng.uniform(0.0, 1.0, (500, 3)) * Ld
    vs = rng.normal(0.0, 3.0, (500, 3)) * Ld
    o.add_particles(xs, vs, -1.0, 1.0)
    p0 = o.particles()
    o.move(0.7, Ld=Ld)
    p1 = o.particles(sort=False)
    order = np.argsort(p1["id"])
    x1 = p1["x"][order]
    x0 = p0["x"][np.argsort(p0["id"])] + 0.7 * p0["v"][np.argsort(p0["id"])]
    assert np.all((x1 >= 0.0) & (x1 < Ld))
    # the wrapped position differs from the free flight by whole box lengths
    k = (x0 - x1) / Ld
    np.testing.assert_allclose(k, np.round(k), atol=1e-9)
