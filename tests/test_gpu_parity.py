"""Parity of the GPU engine (through the C ABI) with the oracle, stage by stage
and for the fused step, on small seeded cases.

Bars: cell indices, absorbed/injected counts, positions and velocities
bit-exact (FP64 form, same rounding order on both sides); kinetic energy,
deposited charge, object charges and currents within 1e-12 relative (sums in
a different order); potential within 1e-10 of a direct sparse solve (the
iterative solve runs to rtol 1e-14 there)."""
import numpy as np
import pytest

from helpers import compare_particles, langmuir_load, maxwellian_velocities, uniform_points
from puncpp_gb300 import _lib as L
from puncpp_gb300 import meshgen, punc

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def probe_setup(lib, oracle_mod, n=8, half=2.0, radius=0.6, n_particles=6000, seed=1, **cfg):
    ma = meshgen.probe_box(n, half, radius)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, **cfg)
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(seed)
    ve = maxwellian_velocities(n_particles, 1.0, rng)
    vi = maxwellian_velocities(n_particles // 2, 0.1, rng)
    for q, m, vs in ((-1.0, 1.0, ve), (1.0, 100.0, vi)):
        xs = uniform_points(ma, len(vs), rng)
        k1 = pop.add_particles(xs, vs, q, m)
        k2 = o.add_particles(xs, vs, q, m)
        assert k1 == k2
    return ma, mesh, pop, o, rng


def periodic_setup(lib, oracle_mod, n=6, ppc=12, seed=2, **cfg):
    ma = meshgen.langmuir_cube(n)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, periodic=True, **cfg)
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(seed)
    x, v, q, m = langmuir_load(ma, ppc, rng, amplitude=0.05)
    v = maxwellian_velocities(len(x), 0.2, rng)
    assert pop.add_particles(x, v, q, m) == o.add_particles(x, v, q, m)
    return ma, mesh, pop, o, rng


def test_locate_and_add_particles(lib, oracle_mod):
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod)
    pts = uniform_points(ma, 20000, rng) * 1.05        # some outside the box, some in the hole
    np.testing.assert_array_equal(pop.locate(pts), o.locate(pts))
    compare_particles(pop.particles(), o.particles())
    p = o.particles()
    assert pop.num_of_particles() == o.num_particles()
    assert pop.num_of_negatives() == int((p["q"] < 0).sum())
    assert pop.num_of_positives() == int((p["q"] > 0).sum())


@pytest.mark.parametrize("geom", ["probe", "periodic"])
def test_efield_push_move_bitwise(geom, lib, oracle_mod):
    setup = probe_setup if geom == "probe" else periodic_setup
    ma, mesh, pop, o, rng = setup(lib, oracle_mod)
    phi = rng.normal(size=mesh.n_dofs)
    E = punc.Function(pop, "E")
    punc.Function(pop, "phi").set_local(phi)
    Eo = o.efield(phi)
    assert np.array_equal(E.vector(), Eo)
    dt = 0.07
    ke_g = punc.boris(pop, E, (0.0, 0.0, 0.0), dt)
    ke_o = o.boris(Eo, (0.0, 0.0, 0.0), dt)
    assert rel(ke_g, ke_o) < RTOL
    compare_particles(pop.particles(), o.particles())
    B = (0.3, -0.2, 0.9)
    assert rel(punc.boris(pop, E, B, dt), o.boris(Eo, B, dt)) < RTOL
    compare_particles(pop.particles(), o.particles())
    assert rel(punc.accel(pop, E, dt), o.accel(Eo, dt)) < RTOL
    compare_particles(pop.particles(), o.particles())
    if geom == "periodic":
        punc.move_periodic(pop, 0.9, ma.Ld)
        o.move(0.9, ma.Ld)
    else:
        punc.move(pop, 0.9)
        o.move(0.9)
    # positions moved, cells not yet updated: compare by id
    a, b = pop.particles(), o.particles()
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["v"], b["v"])
    assert rel(punc.kinetic_energy(pop), o.kinetic_energy()) < RTOL


@pytest.mark.parametrize("geom", ["probe", "periodic"])
def test_update_walk_and_absorption(geom, lib, oracle_mod):
    setup = probe_setup if geom == "probe" else periodic_setup
    ma, mesh, pop, o, rng = setup(lib, oracle_mod)
    dt = 1.3           # multi-cell walks, many particles leave through both boundaries
    if geom == "periodic":
        punc.move_periodic(pop, dt, ma.Ld)
        o.move(dt, ma.Ld)
    else:
        punc.move(pop, dt)
        o.move(dt)
    objs = [punc.Object(2, charge=0.5)] if geom == "probe" else []
    oobjs = [dict(bnd_id=2, charge=0.5, current=0.0, potential=0.0)] if geom == "probe" else []
    pop.update(objs, dt)
    absorbed = o.update(oobjs, dt)
    compare_particles(pop.particles(), o.particles())
    assert pop.num_of_particles() == o.num_particles()
    if geom == "probe":
        assert absorbed[2] > 0 and absorbed[1] > 0
        assert rel(objs[0].current, oobjs[0]["current"]) < RTOL
        assert rel(objs[0].charge, oobjs[0]["charge"]) < RTOL


@pytest.mark.parametrize("geom", ["probe", "periodic"])
def test_distribute_cg1(geom, lib, oracle_mod):
    setup = probe_setup if geom == "probe" else periodic_setup
    ma, mesh, pop, o, rng = setup(lib, oracle_mod)
    rho_g = punc.distribute_cg1(pop)
    rho_o = o.distribute_cg1()
    assert rel(rho_g, rho_o) < RTOL
    np.testing.assert_array_equal(punc.Function(pop, "rho").vector(), rho_g)


PRECONDS = {"amg": 0, "jacobi": 1}


@pytest.mark.parametrize("precond", sorted(PRECONDS))
def test_poisson_dirichlet_and_objects(precond, lib, oracle_mod):
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, pcg_rtol=1e-14, pcg_atol=1e-30, pcg_max_iter=5000,
                                        pcg_precond=PRECONDS[precond])
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    solver = punc.PoissonSolver(pop, objs)
    phi_g = solver.solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
    phi_o = o.poisson_direct(rho, potentials=[-2.0])
    assert rel(phi_g, phi_o) < 1e-10
    assert solver.last_info.iterations > 0


@pytest.mark.parametrize("precond", sorted(PRECONDS))
@pytest.mark.parametrize("rtol", [1e-10, 1e-13])
def test_mixed_precision_pcg_meets_the_fp64_tolerance(rtol, precond, lib, oracle_mod):
    """FP32 recurrence with FP64 true-residual replacement: the returned FP64
    residual meets the same stopping test as the FP64 solver."""
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, pcg_rtol=rtol, pcg_atol=1e-30, pcg_max_iter=5000,
                                        pcg_precision=2, pcg_precond=PRECONDS[precond])
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    solver = punc.PoissonSolver(pop, objs)
    phi_g = solver.solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
    info = solver.last_info
    assert info.residual <= rtol * info.rhs_norm
    phi_o = o.poisson_direct(rho, potentials=[-2.0])
    assert rel(phi_g, phi_o) < 1e4 * rtol


@pytest.mark.parametrize("precond", sorted(PRECONDS))
def test_poisson_periodic_null_space(precond, lib, oracle_mod):
    ma, mesh, pop, o, rng = periodic_setup(lib, oracle_mod, pcg_rtol=1e-14, pcg_atol=1e-30, pcg_max_iter=5000,
                                           pcg_precond=PRECONDS[precond])
    rho = punc.distribute_cg1(pop)
    phi_g = punc.PoissonSolver(pop).solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"))
    phi_o = o.poisson_direct(rho, periodic=True)
    assert abs(phi_g.mean()) < 1e-13 * np.abs(phi_g).max()
    assert rel(phi_g, phi_o) < 1e-10


def test_amg_needs_far_fewer_iterations_than_jacobi(lib, oracle_mod):
    """Same system, same tolerance: the V-cycle preconditioner cuts the
    iteration count several-fold and both meet the stopping test."""
    its = {}
    for name, code in PRECONDS.items():
        ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, n=16, half=4.0, radius=0.8, n_particles=20000,
                                            pcg_rtol=1e-10, pcg_atol=1e-30, pcg_max_iter=5000, pcg_precond=code)
        punc.distribute_cg1(pop)
        objs = [punc.Object(2, potential=-2.0)]
        solver = punc.PoissonSolver(pop, objs)
        solver.solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
        info = solver.last_info
        assert info.residual <= 1e-10 * info.rhs_norm
        its[name] = info.iterations
        lay = punc.poisson_layout(pop)
        assert lay["n_rows"] == mesh.n_dofs and 0 < lay["nnz"] <= lay["sell_entries"]
        if code == 0:
            rows = [v["rows"] for v in lay["levels"]]
            assert len(rows) >= 2 and rows[0] == mesh.n_dofs and rows == sorted(rows, reverse=True)
            assert lay["levels"][-1]["nnz_p"] == 0 and all(v["nnz_p"] > 0 for v in lay["levels"][:-1])
        else:
            assert lay["levels"] == []
    assert its["amg"] * 3 < its["jacobi"], its


@pytest.mark.parametrize("resolve", [True, False])
def test_circuit_cm_fixed_voltage(resolve, lib, oracle_mod):
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, pcg_rtol=1e-14, pcg_atol=1e-30, pcg_max_iter=5000,
                                        circuit_resolve=resolve)
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, charge=0.3)]
    dt = 0.05
    vs = [(-1, 0, -2.0)]
    circ = punc.CircuitCM(pop, objs, vs, [], dt)
    solver = punc.PoissonSolver(pop, objs, circ)
    phi_g = solver.solve_circuit(punc.Function(pop, "phi"), punc.Function(pop, "rho"), mesh, objs, circ)
    # the reference re-solves; superposition of the set-up Laplace solutions needs one solve
    assert solver.last_info.solves == (2 if resolve else 1)

    def solve(r, pots, laplace=False):
        return o.poisson_direct(np.zeros(o.ndof) if r is None else r, potentials=list(pots))

    ocirc = oracle_mod.CircuitCM(o, vs, [], dt, solve)
    oobjs = [dict(bnd_id=2, charge=0.3, current=0.0, potential=0.0)]
    phi_o, _ = ocirc.solve_circuit(rho, oobjs)
    assert rel(circ.inv_capacitance(), ocirc.inv_cap) < 1e-9
    assert objs[0].potential == oobjs[0]["potential"] == -2.0
    assert rel(objs[0].charge, oobjs[0]["charge"]) < 1e-9
    assert rel(phi_g, phi_o) < 1e-10


@pytest.mark.parametrize("resolve", [True, False])
def test_circuit_cm_floating_object_with_current_source(resolve, lib, oracle_mod):
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, pcg_rtol=1e-14, pcg_atol=1e-30, pcg_max_iter=5000,
                                        circuit_resolve=resolve)
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, charge=0.05)]
    dt = 0.1
    isrc = [(-1, 0, 0.2)]
    circ = punc.CircuitCM(pop, objs, [], isrc, dt)
    phi_g = punc.PoissonSolver(pop, objs, circ).solve_circuit(punc.Function(pop, "phi"), None, mesh, objs, circ)

    def solve(r, pots, laplace=False):
        return o.poisson_direct(np.zeros(o.ndof) if r is None else r, potentials=list(pots))

    ocirc = oracle_mod.CircuitCM(o, [], isrc, dt, solve)
    oobjs = [dict(bnd_id=2, charge=0.05, current=0.0, potential=0.0)]
    phi_o, _ = ocirc.solve_circuit(rho, oobjs)
    assert rel(objs[0].charge, oobjs[0]["charge"]) < 1e-9
    assert rel(objs[0].potential, oobjs[0]["potential"]) < 1e-9
    assert rel(phi_g, phi_o) < 1e-9


def test_injection_bitwise(lib, oracle_mod):
    ma = meshgen.probe_box(6, 3.0, 0.8)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh)
    o = oracle_mod.Oracle(ma)
    sp = [punc.Species(-1.0, 1.0, n=40.0, vth=1.0, vd=(0.3, 0.0, -0.2)),
          punc.Species(1.0, 50.0, n=40.0, vth=0.2)]
    punc.create_flux(pop, sp)
    o.create_flux([dict(q=s.q, m=s.m, n=s.n, vth=s.vth, vd=s.vd) for s in sp])
    dt = 0.05
    for step in range(5):
        kg = punc.inject_particles(pop, sp, mesh.exterior_facets, dt, seed=99, step=step)
        ko, _ = o.inject(dt, 99, step)
        assert kg == ko and kg > 0
    compare_particles(pop.particles(), o.particles())


def test_fused_steps_in_lockstep_with_oracle(lib, oracle_mod):
    """pg_step against the oracle's staged sequence, resynchronised each step:
    the oracle starts from the engine's particles, pushes with the engine's
    potential, and must end bit-identical."""
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, pcg_rtol=1e-12)
    sp = [punc.Species(-1.0, 1.0, n=20.0, vth=1.0), punc.Species(1.0, 100.0, n=20.0, vth=0.1)]
    punc.create_flux(pop, sp)
    o.create_flux([dict(q=s.q, m=s.m, n=s.n, vth=s.vth) for s in sp])
    objs = [punc.Object(2, potential=-1.0)]
    dt = 0.2
    for n in range(4):
        o.set_particles(pop.particles())
        rho_o = o.distribute_cg1()
        res = punc.step(pop, objs, dt, first_step=(n == 0), inject=True, seed=5, step_no=n)
        # charge used by this step (the fused deposit of the previous step from n = 1 on)
        assert rel(punc.Function(pop, "rho").vector(), rho_o) < RTOL
        phi = punc.Function(pop, "phi").vector()
        assert rel(phi, o.poisson_direct(rho_o, potentials=[-1.0])) < 1e-8
        E = o.efield(phi)
        assert np.array_equal(punc.Function(pop, "E").vector(), E)
        ke = o.boris(E, (0, 0, 0), dt * (0.5 if n == 0 else 1.0))
        o.move(dt)
        oobjs = [dict(bnd_id=2, charge=0.0, current=0.0, potential=-1.0)]
        absorbed = o.update(oobjs, dt)
        assert res.n_absorbed == absorbed.sum() > 0
        assert rel(res.KE, ke) < RTOL
        assert rel(objs[0].current, oobjs[0]["current"]) < RTOL
        ko, _ = o.inject(dt, 5, n)
        assert res.n_injected == ko > 0
        compare_particles(pop.particles(), o.particles())
        assert res.n_particles == o.num_particles()


def test_fused_deposit_equals_distribute(lib, oracle_mod):
    ma, mesh, pop, o, rng = periodic_setup(lib, oracle_mod)
    res = punc.step(pop, [], 0.1, first_step=True, Ld=ma.Ld)
    assert res.n_absorbed == 0
    o.set_particles(pop.particles())
    rho_o = o.distribute_cg1()
    punc.step(pop, [], 0.1, Ld=ma.Ld)
    assert rel(punc.Function(pop, "rho").vector(), rho_o) < RTOL


def test_cpp_time_loop_runs(lib, tmp_path):
    """The C++ front end (include/punc_gpu.hpp) drives three reference-shaped
    steps, then two fused steps replayed from a captured graph (run_steps)."""
    import subprocess

    from test_abi import build_cpp_time_loop
    exe = build_cpp_time_loop(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("step")]
    assert len(lines) == 3 and all(l.endswith("particles 1") for l in lines)
    fused = [l for l in r.stdout.splitlines() if l.startswith("fused")]
    assert len(fused) == 2 and all(l.endswith("particles 1") for l in fused)


def test_sort_keeps_the_particle_set(lib, oracle_mod):
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod)
    punc.move(pop, 0.5)
    pop.update([punc.Object(2)], 0.5)
    before = pop.particles()
    pop.sort()
    compare_particles(pop.particles(), before)


def test_walk_limit_is_reported_and_engine_stays_usable(lib, oracle_mod):
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, max_walk_steps=1)
    punc.move(pop, 1.5)
    with pytest.raises(L.PgError) as e:
        pop.update([punc.Object(2)], 1.5)
    assert e.value.code == 5
    # the error was reported once; the engine answers further calls
    assert pop.status() == (0, 0)
    assert pop.num_of_particles() > 0


@pytest.mark.parametrize("geom", ["probe", "periodic"])
def test_esolver_matches_a_direct_solve(geom, lib, oracle_mod):
    """ESolver (CG1 projection of -grad phi): device CG on the mass matrix to
    rel 1e-12 against the oracle's direct solve of the same system."""
    setup = probe_setup if geom == "probe" else periodic_setup
    ma, mesh, pop, o, rng = setup(lib, oracle_mod)
    phi = rng.normal(size=mesh.n_dofs)
    punc.Function(pop, "phi").set_local(phi)
    E = punc.Function(pop, "E_cg1")
    es = punc.ESolver(pop)
    Eg = es.solve(E, punc.Function(pop, "phi"))
    Eo = o.esolver(phi)
    assert Eg.shape == (mesh.n_dofs, 3)
    assert rel(Eg, Eo) < 1e-10
    info = es.last_info
    assert 0 < info.iterations < 100 and info.residual <= 1e-12 * info.rhs_norm * 1.0001


@pytest.mark.parametrize("geom", ["probe", "periodic"])
def test_cg1_push_bitwise(geom, lib, oracle_mod):
    """accel_cg1 / boris_cg1 with the same vertex field: velocities bitwise."""
    setup = probe_setup if geom == "probe" else periodic_setup
    ma, mesh, pop, o, rng = setup(lib, oracle_mod)
    Ev = rng.normal(size=(mesh.n_dofs, 3))
    E = punc.Function(pop, "E_cg1")
    E.set_local(Ev)
    assert np.array_equal(E.vector(), Ev)
    dt = 0.07
    assert rel(punc.boris_cg1(pop, E, (0.0, 0.0, 0.0), dt), o.boris_cg1(Ev, (0.0, 0.0, 0.0), dt)) < RTOL
    compare_particles(pop.particles(), o.particles())
    B = (0.3, -0.2, 0.9)
    assert rel(punc.boris_cg1(pop, E, B, dt), o.boris_cg1(Ev, B, dt)) < RTOL
    compare_particles(pop.particles(), o.particles())
    assert rel(punc.accel_cg1(pop, E, dt), o.accel_cg1(Ev, dt)) < RTOL
    compare_particles(pop.particles(), o.particles())


def test_fused_cg1_steps_in_lockstep_with_oracle(lib, oracle_mod):
    """pg_step with the CG1 field (the reference time loop's default): the
    oracle starts from the engine's particles and pushes with the engine's
    vertex field; particles end bit-identical, the field within 1e-10 of the
    oracle's projection of the engine's potential."""
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, pcg_rtol=1e-12)
    sp = [punc.Species(-1.0, 1.0, n=20.0, vth=1.0), punc.Species(1.0, 100.0, n=20.0, vth=0.1)]
    punc.create_flux(pop, sp)
    o.create_flux([dict(q=s.q, m=s.m, n=s.n, vth=s.vth) for s in sp])
    objs = [punc.Object(2, potential=-1.0)]
    dt = 0.2
    for n in range(3):
        o.set_particles(pop.particles())
        res = punc.step(pop, objs, dt, first_step=(n == 0), inject=True, seed=7, step_no=n, efield_cg1=True)
        phi = punc.Function(pop, "phi").vector()
        Ev = punc.Function(pop, "E_cg1").vector()
        assert rel(Ev, o.esolver(phi)) < 1e-10
        ke = o.boris_cg1(Ev, (0, 0, 0), dt * (0.5 if n == 0 else 1.0))
        o.move(dt)
        oobjs = [dict(bnd_id=2, charge=0.0, current=0.0, potential=-1.0)]
        absorbed = o.update(oobjs, dt)
        assert res.n_absorbed == absorbed.sum()
        assert rel(res.KE, ke) < RTOL
        ko, _ = o.inject(dt, 7, n)
        assert res.n_injected == ko
        compare_particles(pop.particles(), o.particles())


@pytest.mark.parametrize("geom", ["probe", "periodic"])
def test_diagnostics_match_oracle(geom, lib, oracle_mod):
    """particle_potential_energy_cg1, density_cg1, density_dg0 and
    Population::statistics against the oracle's sequential restatements."""
    setup = probe_setup if geom == "probe" else periodic_setup
    ma, mesh, pop, o, rng = setup(lib, oracle_mod)
    phi = rng.normal(size=mesh.n_dofs)
    punc.Function(pop, "phi").set_local(phi)
    assert rel(punc.particle_potential_energy_cg1(pop, punc.Function(pop, "phi")), o.potential_energy(phi)) < RTOL
    we, wi = 0.37, 2.5
    for g, r in ((punc.density_cg1(pop, we, wi), o.density_cg1(we, wi)),
                 (punc.density_dg0(pop, we, wi), o.density_dg0(we, wi))):
        assert rel(g[0], r[0]) < RTOL and rel(g[1], r[1]) < RTOL
    st_g, st_o = pop.statistics(), o.statistics()
    assert np.all(np.abs(st_g - st_o) <= 1e-12 * np.abs(st_o)), (st_g, st_o)


@pytest.mark.parametrize("binary", [True, False])
def test_population_file_matches_reference_writer_and_round_trips(binary, lib, oracle_mod, tmp_path):
    """Population::save_file from the engine is byte-identical to the oracle's
    restatement for a freshly loaded population; load_file into a new engine
    gives back the same particles bit for bit."""
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod)
    fg, fo = tmp_path / "pop_engine.dat", tmp_path / "pop_oracle.dat"
    pop.save_file(fg, binary=binary)
    o.save_file(fo, binary=binary)
    assert fg.read_bytes() == fo.read_bytes()
    pop2 = punc.Population(mesh)
    assert pop2.load_file(fg, binary=binary) == pop.num_of_particles()
    a, b = pop.particles(), pop2.particles()
    for k in ("x", "v", "q", "m", "cell"):
        assert np.array_equal(a[k], b[k]), k


def _permuted(ma, rng):
    """The same mesh with its vertices renumbered at random (wide column spans
    in every operator row)."""
    perm = rng.permutation(ma.n_vertices)
    coords = np.empty_like(ma.coords)
    coords[perm] = ma.coords
    return meshgen.MeshArrays(coords=coords, cells=perm[ma.cells], bfacets=perm[ma.bfacets], btags=ma.btags.copy(),
                              vertex_to_dof=None, n_dofs=ma.n_dofs, Ld=ma.Ld, origin=ma.origin,
                              n_objects=ma.n_objects)


def _compressed_cycle_bytes(lay):
    """Operator bytes of one AMG-PCG iteration if every operator took 16-bit
    columns: A_0 (f32 + u16) twice, S_0 and S_l^T, A_l (l >= 1), U1 in
    binary16 + u16, G in f32 + i32."""
    lv, L = lay["levels"], len(lay["levels"]) - 1
    b = 2 * lv[0]["nnz"] * 6 + lv[0]["nnz_p"] * 4
    if L >= 2:
        b += lv[0]["nnz_p"] * 4 + lay["cycle_nnz_u1"] * 4
    for l in range(1, L):
        b += lv[l]["nnz"] * 4 + (lv[l]["nnz_p"] * 4 if l < L - 1 else 0)
    return b + lay["cycle_nnz_g"] * 8


def test_amg_operators_with_wide_column_spans(lib, oracle_mod):
    """A randomly renumbered mesh of more than 65,536 dofs: column offsets
    within an operator row span more than 16 bits, so some operators keep
    32-bit columns (more bytes than the all-16-bit layout predicts, while the
    mesh in its natural order matches it exactly), and the solution still
    matches a direct solve."""
    rng = np.random.default_rng(7)
    base = meshgen.probe_box(44, 4.0, 0.9)
    assert base.n_dofs > 65536
    ma = _permuted(base, rng)
    for m_ in (base, ma):
        pop = punc.Population(punc.Mesh(m_), pcg_rtol=1e-12, pcg_atol=1e-30, pcg_max_iter=5000)
        lay = punc.poisson_layout(pop)
        if m_ is base:
            assert lay["cycle_bytes"] == _compressed_cycle_bytes(lay)
        else:
            assert lay["cycle_bytes"] > _compressed_cycle_bytes(lay)
            o = oracle_mod.Oracle(ma)
            xs = uniform_points(ma, 20000, rng)
            vs = maxwellian_velocities(len(xs), 1.0, rng)
            assert pop.add_particles(xs, vs, -1.0, 1.0) == o.add_particles(xs, vs, -1.0, 1.0)
            rho = punc.distribute_cg1(pop)
            objs = [punc.Object(2, potential=-2.0)]
            phi_g = punc.PoissonSolver(pop, objs).solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
            phi_o, _ = o.poisson_pcg(rho, potentials=[-2.0], rtol=1e-13, atol=1e-30, max_iter=20000, nthreads=8)
            assert rel(phi_g, phi_o) < 1e-9
        pop.close()


def test_amg_pcg_reports_an_unattainable_tolerance(lib, oracle_mod):
    """rtol 1e-16 is below what the FP32 recurrence attains on 90k dofs: the
    solve ends with PG_ERR_NOT_CONVERGED ("stalled") instead of iterating to
    the cap, and the solution it leaves is still at the attainable accuracy
    (checked against the oracle's FP64 Jacobi-PCG at rtol 1e-13)."""
    ma = meshgen.probe_box(44, 4.0, 0.9)
    rng = np.random.default_rng(8)
    pop = punc.Population(punc.Mesh(ma), pcg_rtol=1e-16, pcg_atol=1e-30, pcg_max_iter=5000)
    o = oracle_mod.Oracle(ma)
    xs = uniform_points(ma, 20000, rng)
    vs = maxwellian_velocities(len(xs), 1.0, rng)
    assert pop.add_particles(xs, vs, -1.0, 1.0) == o.add_particles(xs, vs, -1.0, 1.0)
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    solver = punc.PoissonSolver(pop, objs)
    with pytest.raises(L.PgError) as err:
        solver.solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
    assert err.value.code == L.PG_ERR_NOT_CONVERGED and "stalled" in str(err.value)
    phi_g = punc.Function(pop, "phi").vector()
    phi_o, _ = o.poisson_pcg(rho, potentials=[-2.0], rtol=1e-13, atol=1e-30, max_iter=20000, nthreads=8)
    assert rel(phi_g, phi_o) < 1e-9
    pop.close()


@pytest.mark.parametrize("rtol", [1e-10, 1e-13])
def test_amg_pcg_residual_replacement_inside_the_cycle(rtol, lib, oracle_mod):
    """A hierarchy of three or more levels: the replacements between the
    start and the end of a solve take the FP64 true residual inside the
    iteration's own V-cycle; the solve still meets the FP64 stopping test
    (several replacements at rtol 1e-13) and matches a direct solve."""
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, n=24, half=4.0, radius=0.8, n_particles=20000,
                                        pcg_rtol=rtol, pcg_atol=1e-30, pcg_max_iter=5000)
    assert len(punc.poisson_layout(pop)["levels"]) >= 3
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    solver = punc.PoissonSolver(pop, objs)
    phi_g = solver.solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
    info = solver.last_info
    assert info.residual <= rtol * info.rhs_norm and info.iterations < 60
    assert rel(phi_g, o.poisson_direct(rho, potentials=[-2.0])) < 1e4 * rtol
    pop.close()


def test_amg_strength_threshold_rebuild_and_selection(lib, oracle_mod):
    """pg_amg_set_strength rebuilds the hierarchy: level 0 and 1 stay, the
    coarsest level grows (48 rows at theta 0, 281 at 0.05 on this mesh), the
    solve still matches a direct solve; a threshold outside [0, 1) is refused
    with the hierarchy kept; steps replayed from a graph captured before a
    rebuild use the new hierarchy (bitwise the same particles as a handle
    built with that threshold from the start); pg_autotune_amg applies the
    candidate it returns; a Jacobi-preconditioned handle has no threshold.
    Mixed form: its deposit and solve are deterministic, so two handles agree
    bit for bit."""
    kw = dict(n=24, half=4.0, radius=0.8, n_particles=20000, pcg_rtol=1e-13, pcg_atol=1e-30, pcg_max_iter=5000,
              precision=L.PG_MIXED)
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod, **kw)
    rows0 = [v["rows"] for v in punc.poisson_layout(pop)["levels"]]
    assert punc.amg_strength(pop) == 0.0 and rows0[-1] == 48
    punc.set_amg_strength(pop, 0.05)
    rows1 = [v["rows"] for v in punc.poisson_layout(pop)["levels"]]
    assert punc.amg_strength(pop) == 0.05 and rows1[:2] == rows0[:2] and rows1[-1] == 281
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    phi_g = punc.PoissonSolver(pop, objs).solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
    assert rel(phi_g, o.poisson_direct(rho, potentials=[-2.0])) < 1e-9
    with pytest.raises(L.PgError) as err:
        punc.set_amg_strength(pop, 1.5)
    assert err.value.code == L.PG_ERR_ARG
    assert punc.amg_strength(pop) == 0.05 and [v["rows"] for v in punc.poisson_layout(pop)["levels"]] == rows1
    # a graph captured at theta 0.05, then a rebuild at theta 0
    dt = 0.05
    punc.run_steps(pop, objs, dt, 2, first_step=True, use_graph=True)
    punc.set_amg_strength(pop, 0.0)
    punc.run_steps(pop, objs, dt, 2, step_no=2, use_graph=True)
    _, _, ref, _, _ = probe_setup(lib, oracle_mod, **kw)
    punc.set_amg_strength(ref, 0.05)
    robjs = [punc.Object(2, potential=-2.0)]
    punc.run_steps(ref, robjs, dt, 2, first_step=True, use_graph=True)
    punc.set_amg_strength(ref, 0.0)
    punc.run_steps(ref, robjs, dt, 2, step_no=2, use_graph=False)
    compare_particles(pop.particles(), ref.particles())
    np.testing.assert_array_equal(punc.Function(pop, "phi").vector(), punc.Function(ref, "phi").vector())
    res = punc.autotune_amg(pop, objs, dt, steps_per_trial=2, thetas=[0.0, 0.05], step_no=4)
    assert res["amg_theta"] in (0.0, 0.05) and res["pcg_ms"] > 0.0
    assert punc.amg_strength(pop) == res["amg_theta"]
    pop.close()
    ref.close()
    _, _, jac, _, _ = probe_setup(lib, oracle_mod, pcg_precond=1)
    with pytest.raises(L.PgError) as err:
        punc.set_amg_strength(jac, 0.01)
    assert err.value.code == L.PG_ERR_ARG
    jac.close()


def _walk_reference(planes, nbr, x, c, fast):
    """relocate_fast / relocate (punc/include/punc/population.h:454-569) in
    Python floats: plane value c0 + c1 x + c2 y + c3 z summed left to right."""
    k = 0
    while True:
        P = planes[c]
        d = [((P[4 * f] + P[4 * f + 1] * x[0]) + P[4 * f + 2] * x[1]) + P[4 * f + 3] * x[2] for f in range(4)]
        if fast:
            f = next((q for q in range(4) if d[q] > 0), -1)
        else:
            a = max(range(4), key=lambda q: (d[q], -q))
            f = -1 if d[a] < 0 else a
        if f < 0:
            return c, k
        k += 1
        if nbr[c][f] < 0:
            return int(nbr[c][f]), k
        c = int(nbr[c][f])


@pytest.mark.parametrize("fast", [True, False])
def test_single_point_relocate(fast, lib, oracle_mod):
    """pg_relocate: the walk of one point from a given cell, both of the
    reference's rules (first positive facet, largest projection) and the
    crossing count of relocate_stat, bit for bit against a Python
    restatement, for points inside and outside the mesh."""
    ma, mesh, pop, o, rng = probe_setup(lib, oracle_mod)
    planes = mesh.table(L.T_PLANES).reshape(-1, 16)
    nbr = mesh.table(L.T_NEIGHBOURS).reshape(-1, 4)
    n = 3000
    start = rng.integers(0, ma.n_cells, n)
    pts = np.asarray(ma.origin) + rng.random((n, 3)) * np.asarray(ma.Ld) * 1.1 - 0.05 * np.asarray(ma.Ld)
    got, cr = pop.relocate(pts, start, fast=fast, with_crossings=True)
    ref = [_walk_reference(planes, nbr, pts[i].tolist(), int(start[i]), fast) for i in range(n)]
    assert np.array_equal(got, [r[0] for r in ref]) and np.array_equal(cr, [r[1] for r in ref])
    assert (got < 0).any() and (got >= 0).any() and cr.max() >= 3
