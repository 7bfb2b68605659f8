"""Batched runs (the bias-sweep configuration, here eight runs of different
mesh sizes, box sizes, object radii, particle counts, biases and seeds): one engine over
the union mesh against each run done alone.  Injection draws the standalone
streams, so per run and per step the particle counts, absorbed counts and the
object's current and charge agree, and the particles agree to the solver's
tolerance (the batch stops on the residual of the whole batch)."""
import numpy as np
import pytest

from helpers import maxwellian_velocities, uniform_points
from puncpp_gb300 import _lib as L
from puncpp_gb300 import batch, meshgen, punc

pytestmark = pytest.mark.gpu


def test_batch_equals_standalone_runs(lib):
    geo = [(6, 2.0, 0.6), (5, 2.5, 0.7), (7, 3.0, 0.9), (4, 2.0, 0.8), (8, 3.5, 1.2), (6, 2.6, 1.0), (9, 4.0, 1.5),
           (5, 1.8, 0.6)]
    meshes = [meshgen.probe_box(n, h, r) for n, h, r in geo]
    biases = [-1.0, -2.5, 0.5, 3.0, -4.0, 1.5, -0.5, 2.0]
    seeds = [11, 22, 33, 44, 55, 66, 77, 88]
    npart = [3000, 5000, 8000, 1500, 12000, 4000, 20000, 2500]
    assert len({m.n_cells for m in meshes}) == len(meshes)
    sp = [punc.Species(-1.0, 1.0, n=20.0, vth=1.0), punc.Species(1.0, 100.0, n=20.0, vth=0.1)]
    dt, steps = 0.1, 5
    cfg = dict(precision=L.PG_MIXED, pcg_rtol=1e-13, pcg_atol=1e-30, pcg_max_iter=4000)
    rng = np.random.default_rng(5)
    loads = []
    for ma, n in zip(meshes, npart):
        loads.append([(uniform_points(ma, n, rng), maxwellian_velocities(n, 1.0, rng), -1.0, 1.0),
                      (uniform_points(ma, n, rng), maxwellian_velocities(n, 0.1, rng), 1.0, 100.0)])
    # the batch
    b = batch.Batch(meshes, **cfg)
    added = [[b.add_particles(r, x, v, q, m) for x, v, q, m in loads[r]] for r in range(len(meshes))]
    b.create_flux(sp, seeds)
    objs = b.objects()
    b.circuit(objs, biases, dt)
    batch_rows = []
    for n in range(steps):
        res = punc.step(b.pop, objs, dt, first_step=(n == 0), inject=True, seed=0, step_no=n)
        batch_rows.append((b.particles_per_run(), [(o.current, o.charge, o.potential) for o in objs]))
    # the runs alone
    for r, ma in enumerate(meshes):
        mesh = punc.Mesh(ma)
        pop = punc.Population(mesh, **cfg)
        assert [pop.add_particles(x, v, q, m) for x, v, q, m in loads[r]] == added[r]
        punc.create_flux(pop, sp)
        o = [punc.Object(2)]
        punc.CircuitCM(pop, o, [(-1, 0, biases[r])], [], dt)
        for n in range(steps):
            res = punc.step(pop, o, dt, first_step=(n == 0), inject=True, seed=seeds[r], step_no=n)
            counts, objrow = batch_rows[n]
            assert counts[r] == res.n_particles, (r, n)
            cur, ch, pot = objrow[r]
            assert abs(cur - o[0].current) <= 1e-9 * max(abs(o[0].current), 1e-30), (r, n, cur, o[0].current)
            assert abs(ch - o[0].charge) <= 1e-9 * max(abs(o[0].charge), 1e-30)
            assert pot == o[0].potential == biases[r]
        pa, pb = b.run_particles(r), pop.particles()
        assert np.array_equal(pa["cell"], pb["cell"])
        np.testing.assert_allclose(pa["x"], pb["x"], rtol=0, atol=1e-6)
        np.testing.assert_allclose(pa["v"], pb["v"], rtol=0, atol=1e-5)
