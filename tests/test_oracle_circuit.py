"""The oracle's CircuitCM on the CPU, against the capacitance-matrix equations
of punc/src/object_CM.cpp:221-357: with img the image-charge form
(eps0 grad(phi).n over the object's facets, punc/ufl/Charge.ufl) of the solve
with every object grounded, the objects' potentials and charges satisfy
C phi = Q + img (object_CM.cpp:234-256, 290-300); a voltage source fixes its
object's potential or the difference of the potentials it joins; charge moves
only inside a source-connected group; a current source adds I dt to its
object; and C is symmetric (reciprocity) with a positive diagonal and a
non-positive off-diagonal."""
import numpy as np
import pytest

from puncpp_gb300 import batch, meshgen


def _setup(oracle_mod, ma, n=3000, seed=3):
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(seed)
    lo, hi = np.min(ma.coords, axis=0), np.max(ma.coords, axis=0)
    xs = rng.uniform(lo, hi, (n, 3))
    xs = xs[o.locate(xs) >= 0]
    o.add_particles(xs, np.zeros_like(xs), -1.0, 1.0)
    rho = o.distribute_cg1()

    def solve(r, pots, laplace=False):
        return o.poisson_direct(np.zeros(o.ndof) if r is None else r, potentials=list(pots))

    return o, rho, solve


def _objects(charges):
    return [dict(bnd_id=2 + k, charge=float(q), current=0.0, potential=0.0) for k, q in enumerate(charges)]


def _state(objs):
    return (np.array([ob["potential"] for ob in objs]), np.array([ob["charge"] for ob in objs]))


def _grounded_image(o, rho, solve, n):
    return o.image_charges(solve(rho, np.zeros(n)))


def test_fixed_voltage(oracle_mod):
    ma = meshgen.probe_box(6, 2.0, 0.6)
    o, rho, solve = _setup(oracle_mod, ma)
    circ = oracle_mod.CircuitCM(o, [(-1, 0, -1.5)], [], 0.1, solve)
    objs = _objects([0.2])
    phi, img = circ.solve_circuit(rho, objs)
    pot, Q = _state(objs)
    assert pot[0] == -1.5
    np.testing.assert_allclose(img, _grounded_image(o, rho, solve, 1), rtol=1e-12)
    np.testing.assert_allclose(circ.cap @ pot, Q + img, rtol=1e-9)
    # the potential returned is the solve at the object's potential
    np.testing.assert_allclose(phi, solve(rho, pot), rtol=0, atol=1e-12 * abs(phi).max())


def test_current_source_on_a_floating_object(oracle_mod):
    ma = meshgen.probe_box(6, 2.0, 0.6)
    o, rho, solve = _setup(oracle_mod, ma)
    dt, current, q0 = 0.1, 0.3, 0.05
    circ = oracle_mod.CircuitCM(o, [], [(-1, 0, current)], dt, solve)
    objs = _objects([q0])
    _, img = circ.solve_circuit(rho, objs)
    pot, Q = _state(objs)
    assert abs(Q[0] - (q0 + current * dt)) <= 1e-12
    np.testing.assert_allclose(circ.cap @ pot, Q + img, rtol=1e-9)


@pytest.fixture(scope="module")
def two_objects(oracle_mod):
    u, _ = batch.union([meshgen.probe_box(5, 2.0, 0.6), meshgen.probe_box(6, 2.5, 0.7)])
    return _setup(oracle_mod, u)


def test_capacitance_matrix_is_symmetric_with_maxwell_signs(two_objects, oracle_mod):
    o, rho, solve = two_objects
    C = oracle_mod.CircuitCM(o, [], [], 0.1, solve).cap
    assert C.shape == (2, 2)
    assert abs(C[0, 1] - C[1, 0]) <= 1e-9 * abs(C).max()
    assert np.all(np.diag(C) > 0) and C[0, 1] <= 1e-9 * abs(C).max()


def test_voltage_source_between_objects(two_objects, oracle_mod):
    o, rho, solve = two_objects
    V = 0.8
    circ = oracle_mod.CircuitCM(o, [(0, 1, V)], [], 0.1, solve)
    objs = _objects([0.1, -0.25])
    _, img = circ.solve_circuit(rho, objs)
    pot, Q = _state(objs)
    assert abs(pot[1] - pot[0] - V) <= 1e-9 * V
    assert abs(Q.sum() - (0.1 - 0.25)) <= 1e-12
    np.testing.assert_allclose(circ.cap @ pot, Q + img, rtol=1e-9)


def test_separate_floating_objects_keep_their_charges(two_objects, oracle_mod):
    o, rho, solve = two_objects
    circ = oracle_mod.CircuitCM(o, [], [], 0.1, solve)
    objs = _objects([0.1, -0.25])
    _, img = circ.solve_circuit(rho, objs)
    pot, Q = _state(objs)
    np.testing.assert_allclose(Q, [0.1, -0.25], rtol=1e-12)
    np.testing.assert_allclose(circ.cap @ pot, Q + img, rtol=1e-9)
