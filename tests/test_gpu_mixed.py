"""The mixed-precision form: FP32 particles, FP32 push and walk with an FP64
re-test near facets, int64 fixed-point deposit.

Bars: every cell decision equals the oracle's FP64 walk evaluated at the
FP32 position (bit-exact cell indices and absorbed counts); the deposit is
bitwise identical from run to run and within 1e-5 (relative to max |rho|) of
the FP64 deposit of the same FP32 positions; velocities within 1e-6 relative
of the FP64 push."""
import numpy as np
import pytest

from helpers import maxwellian_velocities, uniform_points
from puncpp_gb300 import _lib as L
from puncpp_gb300 import meshgen, punc

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def mixed_setup(oracle_mod, n=8, half=2.0, radius=0.6, n_particles=20000, seed=3, periodic=False, **cfg):
    ma = meshgen.langmuir_cube(n) if periodic else meshgen.probe_box(n, half, radius)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, precision=L.PG_MIXED, periodic=periodic, **cfg)
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(seed)
    for q, m, vth in ((-1.0, 1.0, 1.0), (1.0, 100.0, 0.1)):
        xs = uniform_points(ma, n_particles, rng)
        vs = maxwellian_velocities(n_particles, vth, rng)
        k1 = pop.add_particles(xs, vs, q, m)
        k2 = o.add_particles(f32(xs), f32(vs), q, m)
        assert k1 == k2
    return ma, mesh, pop, o, rng


def test_mixed_particles_are_the_rounded_inputs(lib, oracle_mod):
    ma, mesh, pop, o, rng = mixed_setup(oracle_mod)
    a, b = pop.particles(), o.particles()
    assert np.array_equal(a["id"], b["id"]) and np.array_equal(a["cell"], b["cell"])
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["v"], b["v"])


@pytest.mark.parametrize("periodic", [False, True])
def test_mixed_walk_equals_fp64_walk_at_fp32_positions(periodic, lib, oracle_mod):
    ma, mesh, pop, o, rng = mixed_setup(oracle_mod, periodic=periodic)
    before = pop.particles()
    dt = 0.9
    if periodic:
        punc.move_periodic(pop, dt, ma.Ld)
    else:
        punc.move(pop, dt)
    moved = pop.particles()                       # FP32 positions after the move, old cells
    assert np.array_equal(moved["cell"], before["cell"])
    o.set_particles(moved)
    objs = [] if periodic else [punc.Object(2)]
    oobjs = [] if periodic else [dict(bnd_id=2, charge=0.0, current=0.0, potential=0.0)]
    pop.update(objs, dt)
    absorbed = o.update(oobjs, dt)
    a, b = pop.particles(), o.particles()
    assert np.array_equal(a["id"], b["id"]), "absorbed sets differ"
    assert np.array_equal(a["cell"], b["cell"]), "cell indices differ"
    if not periodic:
        assert absorbed[1] > 0 and absorbed[2] > 0
        assert abs(objs[0].current - oobjs[0]["current"]) <= 1e-12 * abs(oobjs[0]["current"])


def test_mixed_deposit_is_deterministic_and_close_to_fp64(lib, oracle_mod):
    ma, mesh, pop, o, rng = mixed_setup(oracle_mod)
    r1 = punc.distribute_cg1(pop)
    r2 = punc.distribute_cg1(pop)
    assert np.array_equal(r1.view(np.uint64), r2.view(np.uint64))
    pop.sort()
    r3 = punc.distribute_cg1(pop)                 # another particle order
    assert np.array_equal(r1.view(np.uint64), r3.view(np.uint64))
    assert rel(r1, o.distribute_cg1()) < 1e-5


def test_mixed_deposit_with_millions_of_particles_on_one_dof(lib, oracle_mod):
    """10M particles of one sign packed next to one vertex of a single
    sub-cube: that dof collects more than 2^23 units of q_max.  In units of
    2^-40 q_max its int64 sum would pass 2^63; the engine's 2^-30 units (store
    bounded to 2^32 slots) keep it exact, and the charge equals the oracle's
    FP64 deposit of the same FP32 positions to 1e-7."""
    ma = meshgen.kuhn_box(1)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, precision=L.PG_MIXED, capacity=10_000_000)
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(11)
    xs = f32(0.001 + 0.049 * rng.random((10_000_000, 3)))
    vs = np.zeros_like(xs)
    assert pop.add_particles(xs, vs, -1.0, 1.0) == len(xs)
    assert o.add_particles(xs, vs, -1.0, 1.0) == len(xs)
    rho = punc.distribute_cg1(pop)
    ref = o.distribute_cg1()
    charge = ref / mesh.table(L.T_DV_INV)
    assert np.abs(charge).max() > 2 ** 23
    assert rel(rho, ref) < 1e-7
    pop.close()


def test_mixed_push_close_to_fp64(lib, oracle_mod):
    ma, mesh, pop, o, rng = mixed_setup(oracle_mod)
    phi = rng.normal(size=mesh.n_dofs)
    punc.Function(pop, "phi").set_local(phi)
    E = o.efield(phi)
    dt = 0.07
    ke_g = punc.boris(pop, punc.Function(pop, "E"), (0, 0, 0), dt)
    ke_o = o.boris(E, (0, 0, 0), dt)
    assert abs(ke_g - ke_o) < 1e-6 * abs(ke_o)
    a, b = pop.particles(), o.particles()
    assert np.array_equal(a["id"], b["id"])
    assert rel(a["v"], b["v"]) < 1e-6


def test_mixed_fused_steps_track_the_fp64_form(lib, oracle_mod):
    """Same seeded start in both forms; after each fused step the charge
    density of the mixed form stays within 1e-5 of the FP64 form's."""
    ma = meshgen.probe_box(10, 3.0, 0.8)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(5)
    xs_e = uniform_points(ma, 30000, rng); vs_e = maxwellian_velocities(30000, 1.0, rng)
    xs_i = uniform_points(ma, 30000, rng); vs_i = maxwellian_velocities(30000, 0.1, rng)
    pops = {}
    for prec in (L.PG_FP64, L.PG_MIXED):
        pop = punc.Population(mesh, precision=prec, pcg_rtol=1e-12)
        pop.add_particles(f32(xs_e), f32(vs_e), -1.0, 1.0)
        pop.add_particles(f32(xs_i), f32(vs_i), 1.0, 100.0)
        punc.create_flux(pop, [punc.Species(-1.0, 1.0, n=20.0, vth=1.0), punc.Species(1.0, 100.0, n=20.0, vth=0.1)])
        pops[prec] = pop
    objs = {p: [punc.Object(2, potential=-1.0)] for p in pops}
    for n in range(3):
        res = {p: punc.step(pops[p], objs[p], 0.1, first_step=(n == 0), inject=True, seed=9, step_no=n) for p in pops}
        rho64 = punc.Function(pops[L.PG_FP64], "rho").vector()
        rho32 = punc.Function(pops[L.PG_MIXED], "rho").vector()
        assert rel(rho32, rho64) < 1e-5, n
        assert abs(res[L.PG_MIXED].n_particles - res[L.PG_FP64].n_particles) <= 2
        assert abs(res[L.PG_MIXED].KE - res[L.PG_FP64].KE) < 1e-5 * abs(res[L.PG_FP64].KE)
    phi64 = punc.Function(pops[L.PG_FP64], "phi").vector()
    phi32 = punc.Function(pops[L.PG_MIXED], "phi").vector()
    assert rel(phi32, phi64) < 1e-5


def test_mixed_cg1_field_and_push_close_to_fp64(lib, oracle_mod):
    """Mixed form with the CG1 field: the FP32 ESolver within 1e-5 of the FP64
    one, and a fused CG1 step keeps rho within 1e-5 of the FP64 form."""
    ma = meshgen.probe_box(8, 2.0, 0.6)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(21)
    xs = uniform_points(ma, 20000, rng)
    vs = maxwellian_velocities(20000, 1.0, rng)
    xi = uniform_points(ma, 20000, rng)
    vi = maxwellian_velocities(20000, 0.05, rng)
    pops = {}
    for prec in (L.PG_FP64, L.PG_MIXED):
        pop = punc.Population(mesh, precision=prec, pcg_rtol=1e-12)
        pop.add_particles(f32(xs), f32(vs), -1.0, 1.0)
        pop.add_particles(f32(xi), f32(vi), 1.0, 100.0)
        pops[prec] = pop
    phi = rng.normal(size=mesh.n_dofs)
    E = {}
    for prec, pop in pops.items():
        punc.Function(pop, "phi").set_local(phi)
        E[prec] = punc.ESolver(pop).solve(punc.Function(pop, "E_cg1"), punc.Function(pop, "phi"))
    assert rel(E[L.PG_MIXED], E[L.PG_FP64]) < 1e-5
    objs = {p: [punc.Object(2, potential=-1.0)] for p in pops}
    for n in range(2):
        for p in pops:
            punc.step(pops[p], objs[p], 0.1, first_step=(n == 0), efield_cg1=True)
        rho64 = punc.Function(pops[L.PG_FP64], "rho").vector()
        rho32 = punc.Function(pops[L.PG_MIXED], "rho").vector()
        assert rel(rho32, rho64) < 1e-5, n


def test_mixed_diagnostics_close_to_the_oracle(lib, oracle_mod):
    """Diagnostics of the mixed form (FP32 positions and velocities) against
    the oracle on the same FP32-rounded particles."""
    ma = meshgen.probe_box(8, 2.0, 0.6)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(23)
    o = oracle_mod.Oracle(ma)
    pop = punc.Population(mesh, precision=L.PG_MIXED)
    for q, m, vth in ((-1.0, 1.0, 1.0), (1.0, 100.0, 0.1)):
        xs = f32(uniform_points(ma, 20000, rng))
        vs = f32(maxwellian_velocities(20000, vth, rng))
        pop.add_particles(xs, vs, q, m)
        o.add_particles(xs, vs, q, m)
    phi = rng.normal(size=mesh.n_dofs)
    punc.Function(pop, "phi").set_local(phi)
    assert rel(punc.particle_potential_energy_cg1(pop, punc.Function(pop, "phi")), o.potential_energy(phi)) < 1e-5
    ne, ni = punc.density_cg1(pop, 1.0, 1.0)
    re, ri = o.density_cg1(1.0, 1.0)
    assert rel(ne, re) < 1e-5 and rel(ni, ri) < 1e-5
    ne, ni = punc.density_dg0(pop, 1.0, 1.0)
    re, ri = o.density_dg0(1.0, 1.0)
    assert rel(ne, re) < 1e-12 and rel(ni, ri) < 1e-12
    assert np.allclose(pop.statistics(), o.statistics(), rtol=1e-6, atol=0)


@pytest.mark.parametrize("use_graph", [False, True])
def test_run_steps_equals_step_by_step(use_graph, lib, oracle_mod):
    """pg_run_steps (device-side bookkeeping, optionally a captured CUDA graph)
    against pg_step called step by step: the mixed form is deterministic (fixed-
    point deposit, fixed-order reductions), so particles, objects and per-step
    results agree bit for bit, across a cell sort."""
    ma = meshgen.probe_box(8, 3.0, 0.8)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(31)
    xe, ve = uniform_points(ma, 20000, rng), maxwellian_velocities(20000, 1.0, rng)
    xi, vi = uniform_points(ma, 20000, rng), maxwellian_velocities(20000, 0.1, rng)
    sp = [punc.Species(-1.0, 1.0, n=20.0, vth=1.0), punc.Species(1.0, 100.0, n=20.0, vth=0.1)]
    runs = []
    for k in range(2):
        pop = punc.Population(mesh, precision=L.PG_MIXED, pcg_rtol=1e-10, sort_interval=5)
        pop.add_particles(f32(xe), f32(ve), -1.0, 1.0)
        pop.add_particles(f32(xi), f32(vi), 1.0, 100.0)
        punc.create_flux(pop, sp)
        objs = [punc.Object(2)]
        punc.CircuitCM(pop, objs, [(-1, 0, -1.5)], [], 0.1)
        runs.append((pop, objs))
    (p1, o1), (p2, o2) = runs
    ref = [punc.step(p1, o1, 0.1, first_step=(n == 0), inject=True, seed=3, step_no=n) for n in range(8)]
    got = punc.run_steps(p2, o2, 0.1, 8, first_step=True, inject=True, seed=3, step_no=0, use_graph=use_graph)
    for a, b in zip(ref, got):
        assert (a.KE, a.n_particles, a.n_absorbed, a.n_injected, a.pcg_iterations) == \
               (b.KE, b.n_particles, b.n_absorbed, b.n_injected, b.pcg_iterations)
    assert (o1[0].charge, o1[0].current, o1[0].potential) == (o2[0].charge, o2[0].current, o2[0].potential)
    a, b = p1.particles(), p2.particles()
    for k in ("id", "cell", "x", "v"):
        assert np.array_equal(a[k], b[k]), k
    # a second call continues from where the first stopped
    ref2 = [punc.step(p1, o1, 0.1, inject=True, seed=3, step_no=n) for n in range(8, 12)]
    got2 = punc.run_steps(p2, o2, 0.1, 4, inject=True, seed=3, step_no=8, use_graph=use_graph)
    assert [r.n_particles for r in ref2] == [r.n_particles for r in got2]
    assert np.array_equal(p1.particles()["x"], p2.particles()["x"])


@pytest.mark.parametrize("pinned", [True, False])
def test_async_potential_read_back(pinned, lib, oracle_mod):
    """pg_get_phi_async after each of six graph-replayed steps, into
    alternating host buffers (page-locked or not), read after one
    pg_synchronize: each buffer holds the potential of its step (bit for bit
    that of a second handle read with pg_get_phi after every step), and the
    steps' particles are unchanged by the read-backs in flight."""
    torch = pytest.importorskip("torch")
    ma = meshgen.probe_box(8, 3.0, 0.8)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(37)
    xe, ve = f32(uniform_points(ma, 20000, rng)), f32(maxwellian_velocities(20000, 1.0, rng))
    sp = [punc.Species(-1.0, 1.0, n=20.0, vth=1.0)]
    runs = []
    for k in range(2):
        pop = punc.Population(mesh, precision=L.PG_MIXED, pcg_rtol=1e-10)
        pop.add_particles(xe, ve, -1.0, 1.0)
        punc.create_flux(pop, sp)
        objs = [punc.Object(2)]
        punc.CircuitCM(pop, objs, [(-1, 0, -1.5)], [], 0.1)
        runs.append((pop, objs))
    (p1, o1), (p2, o2) = runs
    ref = []
    for n in range(6):
        punc.run_steps(p1, o1, 0.1, 1, first_step=(n == 0), inject=True, seed=5, step_no=n)
        ref.append(punc.Function(p1, "phi").vector().copy())
    if pinned:
        bufs = [torch.zeros(mesh.n_dofs, dtype=torch.float64, pin_memory=True) for _ in range(6)]
        arrs = [b.numpy() for b in bufs]
    else:
        arrs = [np.zeros(mesh.n_dofs) for _ in range(6)]
    for n in range(6):
        punc.run_steps(p2, o2, 0.1, 1, first_step=(n == 0), inject=True, seed=5, step_no=n)
        L.check(lib.pg_get_phi_async(p2.handle, L.dptr(arrs[n])))
    L.check(lib.pg_synchronize(p2.handle))
    for n in range(6):
        assert np.array_equal(arrs[n], ref[n]), n
    assert not np.array_equal(ref[0], ref[5])
    a, b = p1.particles(), p2.particles()
    for k in ("id", "cell", "x", "v"):
        assert np.array_equal(a[k], b[k]), k
    p1.close()
    p2.close()


def test_launch_tuning_does_not_change_the_mixed_results(lib, oracle_mod):
    """The mixed form is deterministic: block size, grid size and the
    warp-aggregated deposit give the same particles and charge bit for bit;
    the autotuner returns a configuration from its search space and applies it."""
    ma = meshgen.probe_box(8, 3.0, 0.8)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(41)
    xe, ve = f32(uniform_points(ma, 30000, rng)), f32(maxwellian_velocities(30000, 1.0, rng))
    pops = []
    for tune in ({}, dict(threads=512, blocks_per_sm=2, dep_agg=1), dict(threads=128, blocks_per_sm=16, dep_agg=0)):
        pop = punc.Population(mesh, precision=L.PG_MIXED, pcg_rtol=1e-10)
        pop.add_particles(xe, ve, -1.0, 1.0)
        pop.add_particles(xe[::-1].copy(), ve * 0.1, 1.0, 100.0)
        punc.create_flux(pop, [punc.Species(-1.0, 1.0, n=20.0, vth=1.0)])
        if tune:
            punc.set_tuning(pop, **tune)
        pops.append(pop)
    objs = [[punc.Object(2, potential=-1.0)] for _ in pops]
    for n in range(3):
        for pop, o in zip(pops, objs):
            punc.step(pop, o, 0.1, first_step=(n == 0), inject=True, seed=1, step_no=n)
        rho = [punc.Function(p, "rho").vector() for p in pops]
        assert np.array_equal(rho[0], rho[1]) and np.array_equal(rho[0], rho[2])
    a = pops[0].particles()
    for p in pops[1:]:
        b = p.particles()
        assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["v"], b["v"])
    t = punc.autotune(pops[0], objs[0], 0.1, steps_per_trial=1, inject=True, seed=1, step_no=3)
    assert t["threads"] in (128, 256, 512) and t["blocks_per_sm"] in (2, 4, 8, 16)
    assert t["sort_interval"] in (5, 10, 20, 40) and t["pass_ms"] > 0 and t["sort_ms"] > 0
    g = punc.get_tuning(pops[0])
    assert (g["threads"], g["blocks_per_sm"], g["dep_agg"], g["sort_interval"]) == \
           (t["threads"], t["blocks_per_sm"], t["dep_agg"], t["sort_interval"])
