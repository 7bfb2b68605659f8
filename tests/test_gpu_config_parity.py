"""The FP64 engine in lockstep with the oracle at the sizes of the reference
configurations, not only on small meshes.

* Langmuir oscillation (periodic unit cube 16^3 x 6 = 24,576 cells, 393,216
  electrons, Boris dt = 0.251, 100 fused steps): the time loop of
  demo/langmuir/langmuir.cpp:231-307 with the kinetic, potential and total
  energy of every step (the columns of its history, diagnostics.h:119-168).
* Spherical probe (80^3 x 6 Kuhn cells minus the r < 1 sphere, 3.07M cells,
  531,300 dofs, 2M electrons + 2M ions, CircuitCM bias -2 kT/e, flux
  injection, dt = 0.05): three fused steps of interaction.cpp:342-480.

Each step the oracle takes the engine's potential (the solve is compared on
its own, against the oracle's solve of the oracle's charge) and must end with
bit-identical particles: cell indices, positions, velocities, ids; absorbed
and injected counts exact.  Charge density, kinetic and potential energy and
object current within 1e-12 relative (sums in another order).  The potential
is the solver's: both sides solve the same system to a relative residual of
1e-13, so the bar on it is 1e-10 relative in the max-norm (condition number
times residual)."""
import numpy as np
import pytest

from helpers import compare_particles
from puncpp_gb300 import _lib as L
from puncpp_gb300 import punc

pytestmark = pytest.mark.gpu

RTOL = 1e-12
PHI_TOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_langmuir_16_fused_steps_in_lockstep_with_energies(lib, oracle_mod, capsys):
    import bench
    ma, x, v, q, m = bench.langmuir_load(16, 16)
    assert len(x) == 393_216 and ma.n_cells == 24_576 and ma.n_dofs == 4_096
    # FP64 end to end: FP64 Jacobi PCG (the default AMG solver runs a mixed recurrence)
    pop = punc.Population(punc.Mesh(ma), precision=L.PG_FP64, periodic=True, pcg_precond=1, pcg_rtol=1e-13,
                          pcg_atol=1e-300, pcg_max_iter=20000)
    o = oracle_mod.Oracle(ma)
    assert pop.add_particles(x, v, q, m) == o.add_particles(x, v, q, m) == len(x)
    dt, nth = 0.251, 8
    rows = []
    for n in range(100):
        rho_o = o.distribute_cg1(nth)
        res = punc.step(pop, [], dt, first_step=(n == 0), Ld=ma.Ld, potential_energy=True)
        assert rel(punc.Function(pop, "rho").vector(), rho_o) < RTOL, n
        phi = punc.Function(pop, "phi").vector()
        err_phi = rel(phi, o.poisson_direct(rho_o, periodic=True))
        assert err_phi < PHI_TOL, (n, err_phi)
        E = o.efield(phi)
        assert np.array_equal(punc.Function(pop, "E").vector(), E), n
        pe = o.potential_energy(phi)
        ke = o.boris(E, (0.0, 0.0, 0.0), dt * (0.5 if n == 0 else 1.0), nth)
        assert rel(res.PE, pe) < RTOL and rel(res.KE, ke) < RTOL, (n, res.PE, pe, res.KE, ke)
        o.move(dt, ma.Ld, nth)
        absorbed = o.update([], dt, nth)
        assert res.n_absorbed == absorbed.sum() == 0
        compare_particles(pop.particles(), o.particles())
        rows.append((n, res.KE, ke, res.PE, pe, res.KE + res.PE, ke + pe, err_phi))
    with capsys.disabled():
        print("\nlangmuir-16, FP64 engine vs oracle (step, KE engine, KE oracle, PE engine, PE oracle, "
              "total engine, total oracle, phi err):")
        for r in rows[::10] + rows[-1:]:
            print("  %3d  %.15e %.15e  %.15e %.15e  %.15e %.15e  %.1e" % r)
    ke_e = np.array([r[1] for r in rows])
    pe_e = np.array([r[3] for r in rows])
    # the oscillation exchanges kinetic and field energy at constant total
    assert np.corrcoef(ke_e[1:], pe_e[1:])[0, 1] < -0.99
    tot = ke_e[1:] + pe_e[1:]
    assert np.ptp(tot) < 0.05 * np.ptp(ke_e[1:])
    pop.close()


def test_probe_80_fused_steps_in_lockstep(lib, oracle_mod, capsys):
    import bench
    ma, species, loads = bench.make_workload(80, 2_000_000)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, precision=L.PG_FP64, capacity=int(2.6 * 4_000_000), pcg_precond=1,
                          pcg_rtol=1e-13, pcg_atol=1e-300, pcg_max_iter=20000)
    o = oracle_mod.Oracle(ma)
    for s, (x, v) in zip(species, loads):
        assert pop.add_particles(x, v, s["q"], s["m"]) == o.add_particles(x, v, s["q"], s["m"])
    assert ma.n_cells == 3_070_344 and mesh.n_dofs == 531_300
    punc.create_flux(pop, [punc.Species(s["q"], s["m"], n=s["n"], vth=s["vth"]) for s in species])
    o.create_flux(species)
    nth = 16
    objs = [punc.Object(2)]
    circ = punc.CircuitCM(pop, objs, [(-1, 0, bench.BIAS)], [], bench.DT)

    def solve(rho, pots, laplace=False):
        r = np.zeros(o.ndof) if rho is None else rho
        x, _ = o.poisson_pcg(r, potentials=list(pots), rtol=1e-13, atol=1e-300, max_iter=20000, nthreads=nth)
        return x

    ocirc = oracle_mod.CircuitCM(o, [(-1, 0, bench.BIAS)], [], bench.DT, solve)
    assert rel(circ.inv_capacitance(), ocirc.inv_cap) < PHI_TOL
    oobjs = [dict(bnd_id=2, charge=0.0, current=0.0, potential=0.0)]
    seed = 0x5EED0002
    rows = []
    for n in range(3):
        rho_o = o.distribute_cg1(nth)
        res = punc.step(pop, objs, bench.DT, first_step=(n == 0), inject=True, seed=seed, step_no=n)
        assert rel(punc.Function(pop, "rho").vector(), rho_o) < RTOL, n
        phi = punc.Function(pop, "phi").vector()
        phi_o, _ = ocirc.solve_circuit(rho_o, oobjs)
        err_phi = rel(phi, phi_o)
        assert err_phi < PHI_TOL, (n, err_phi)
        assert objs[0].potential == oobjs[0]["potential"] == bench.BIAS
        E = o.efield(phi)
        assert np.array_equal(punc.Function(pop, "E").vector(), E), n
        ke = o.boris(E, (0.0, 0.0, 0.0), bench.DT * (0.5 if n == 0 else 1.0), nth)
        assert rel(res.KE, ke) < RTOL, n
        o.move(bench.DT, None, nth)
        absorbed = o.update(oobjs, bench.DT, nth)
        assert res.n_absorbed == absorbed.sum() > 0
        assert oobjs[0]["current"] != 0.0 and rel(objs[0].current, oobjs[0]["current"]) < RTOL, n
        # the object charge: the circuit's charge of the solve plus the
        # absorbed charge of the update (the solve's accuracy bounds it)
        err_q = abs(objs[0].charge - oobjs[0]["charge"]) / abs(oobjs[0]["charge"])
        assert err_q < PHI_TOL, (n, err_q)
        # the tally per boundary tag and species: its sums over the species are
        # the oracle's per-tag counts, and the object's share per species adds
        # up to the object current
        counts, qs, _ = punc.absorbed_counts(pop)
        assert np.array_equal(counts.sum(axis=1), absorbed[:counts.shape[0]]), n
        per_species = counts[2] * qs / bench.DT
        assert rel(per_species.sum(), objs[0].current) < RTOL, n
        collected = per_species if n == 0 else collected + per_species
        ko, _ = o.inject(bench.DT, seed, n)
        assert res.n_injected == ko > 0
        a = pop.particles()
        b = o.particles()
        compare_particles(a, b)
        assert res.n_particles == len(b["id"])
        rows.append((n, res.n_particles, res.n_absorbed, res.n_injected, per_species[0], per_species[1], err_phi,
                     err_q))
    assert np.all(collected != 0.0)      # both species reach the object
    with capsys.disabled():
        print("\nprobe-80, FP64 engine vs oracle (step, N, absorbed, injected, object current of electrons, of ions, "
              "phi err, charge err):")
        for r in rows:
            print("  %d  %d  %d  %d  %.12e  %.12e  %.1e  %.1e" % r)
    pop.close()
