"""The oracle's reverse sweep of K periodic Langmuir steps (the checker of the
engine's adjoint) against jump-free central differences of the oracle's own
forward, on the CPU."""
import numpy as np

from puncpp_gb300 import meshgen


def test_oracle_adjoint_matches_finite_differences(oracle_mod):
    O = oracle_mod
    ma = meshgen.langmuir_cube(4)
    rng = np.random.default_rng(4)
    n = 300
    x = rng.random((n, 3))
    v = rng.normal(0.0, 0.1, size=(n, 3))
    w = 1.0 / n
    target = rng.normal(0.0, 1.0, size=O.Oracle(ma).ndof) * 0.05
    E0 = np.array([0.01, 0.0, 0.0])
    K, dt = 6, 0.1
    loss, gv, ge, gx = O.langmuir_adjoint(ma, x, v, -w, w, E0, dt, K, target, ma.Ld)
    assert abs(loss - O.langmuir_loss(ma, x, v, -w, w, E0, dt, K, target, ma.Ld)) <= 1e-13 * loss

    def fd(perturb):
        for h in (1e-6, 1e-7, 1e-8):
            lp = O.langmuir_loss(ma, *perturb(h), dt, K, target, ma.Ld)
            lm = O.langmuir_loss(ma, *perturb(-h), dt, K, target, ma.Ld)
            dp, dm = (lp - loss) / h, (loss - lm) / h
            if abs(dp - dm) <= 1e-3 * max(abs(dp), abs(dm), 1e-12):
                return (lp - lm) / (2 * h)
        raise AssertionError("no jump-free step found")

    def dv(i, j):
        def p(h):
            vv = v.copy()
            vv[i, j] += h
            return x, vv, -w, w, E0
        return p

    def dx(i, j):
        def p(h):
            xx = x.copy()
            xx[i, j] += h
            return xx, v, -w, w, E0
        return p

    def de(j):
        def p(h):
            e = E0.copy()
            e[j] += h
            return x, v, -w, w, e
        return p

    for i, j in [(0, 0), (17, 1), (123, 2)]:
        assert abs(gv[i, j] - fd(dv(i, j))) <= 1e-4 * np.abs(gv).max()
        assert abs(gx[i, j] - fd(dx(i, j))) <= 1e-4 * np.abs(gx).max()
    for j in range(3):
        assert abs(ge[j] - fd(de(j))) <= 1e-4 * np.abs(ge).max()
