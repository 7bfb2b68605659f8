"""Shared set-up for the tests: seeded particle loads on the synthetic meshes."""
import numpy as np


def uniform_points(ma, n, rng):
    lo = np.asarray(ma.origin, float)
    L = np.asarray(ma.Ld, float)
    return lo + rng.random((n, 3)) * L


def langmuir_load(ma, ppc, rng, amplitude=0.01):
    """Electrons uniform in the unit cube, x displaced by amplitude*sin(2 pi x),
    zero velocity (the Langmuir configuration)."""
    n = ppc * ma.n_cells
    x = rng.random((n, 3))
    x[:, 0] = x[:, 0] + amplitude * np.sin(2 * np.pi * x[:, 0])
    x[:, 0] -= np.floor(x[:, 0])
    v = np.zeros((n, 3))
    w = 1.0 / n          # physical density 1, volume 1: omega_p = 1 with eps0 = 1
    return x, v, -w, w


def maxwellian_velocities(n, vth, rng):
    return rng.normal(0.0, vth, size=(n, 3))


def compare_particles(a, b, bitwise=True):
    """a, b: dicts from Population.particles() / Oracle.particles(), sorted by (cell, id)."""
    assert np.array_equal(a["id"], b["id"]), "particle sets differ"
    assert np.array_equal(a["cell"], b["cell"]), "cell indices differ"
    if bitwise:
        assert np.array_equal(a["x"], b["x"]), f"x differs, max {np.abs(a['x'] - b['x']).max()}"
        assert np.array_equal(a["v"], b["v"]), f"v differs, max {np.abs(a['v'] - b['v']).max()}"
    assert np.array_equal(a["q"], b["q"]) and np.array_equal(a["m"], b["m"])


def sort_by_id(p):
    o = np.argsort(p["id"])
    return {k: v[o] for k, v in p.items()}
