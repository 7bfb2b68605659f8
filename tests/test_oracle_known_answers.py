"""Known answers of the reference's demos, checked on the oracle (CPU).

PUNC++ stores no golden vectors; these are the analytic results its demos
and integration test compare against (demo/capacitance, demo/boris,
demo/langmuir, demo/injection, test/test.py), regenerated on the synthetic
meshes.  They pin the oracle's physics; the GPU tests then pin the engine to
the oracle."""
import numpy as np

from puncpp_gb300 import meshgen
from helpers import langmuir_load


def test_capacitance_concentric_spheres(oracle_mod):
    # demo/capacitance/capacitance.cpp:40-42: C = 4 pi eps0 r R / (R - r)
    r, R = 0.2, 1.0
    exact = 4 * np.pi * r * R / (R - r)
    facet_err, react_err = [], []
    for n, k in ((8, 1), (16, 2), (24, 3)):
        o = oracle_mod.Oracle(meshgen.mapped_sphere_shell(n, k, r, R))
        phi = o.poisson_direct(np.zeros(o.ndof), potentials=[1.0])
        K, _ = o.matrices()
        kind, _ = o.dirichlet()
        facet_err.append(abs(o.image_charges(phi)[0] - exact) / exact)
        react_err.append(abs((K @ phi)[kind == 1].sum() - exact) / exact)
    # the variationally consistent charge converges at second order
    assert react_err[-1] < 0.02 and react_err[0] / react_err[1] > 3.0
    # the reference's facet-flux form (Charge.ufl) converges from below
    assert facet_err[0] > facet_err[1] > facet_err[2]


def test_boris_gyration_angle_and_speed(oracle_mod):
    # demo/boris: uniform B, no E: |v| is conserved, and with the reference's
    # t = tan(q B dt / 2m) (pusher.h:469-474) the velocity turns by exactly
    # -omega_c dt per step (2 atan(tan(x)) = 2x)
    ma = meshgen.kuhn_box(4, -50.0, 50.0)
    o = oracle_mod.Oracle(ma)
    q, m, B, dt = -1.0, 1.0, 0.7, 0.3
    o.add_particles(np.array([[0.1, 0.2, 0.3]]), np.array([[1.0, 0.0, 0.25]]), q, m)
    E = np.zeros((o.nc, 3))
    steps = 40
    for _ in range(steps):
        o.boris(E, (0.0, 0.0, B), dt)
    v = o.particles()["v"][0]
    theta = np.arctan2(v[1], v[0])
    expect = -steps * (q / m) * B * dt
    assert abs(np.angle(np.exp(1j * (theta - expect)))) < 1e-12
    assert abs(np.hypot(v[0], v[1]) - 1.0) < 1e-14 and v[2] == 0.25


def test_uniform_field_leapfrog_is_exact(oracle_mod):
    ma = meshgen.kuhn_box(4, -100.0, 100.0)
    o = oracle_mod.Oracle(ma)
    q, m, dt = 2.0, 4.0, 0.125
    E0 = np.array([0.5, -0.25, 1.0])
    o.add_particles(np.array([[0.0, 0.0, 0.0]]), np.array([[1.0, 2.0, -1.0]]), q, m)
    E = np.tile(E0, (o.nc, 1))
    n = 16
    for i in range(n):
        o.boris(E, (0.0, 0.0, 0.0), dt)
        o.move(dt)
    p = o.particles()
    a = q / m * E0
    v_expect = np.array([1.0, 2.0, -1.0]) + n * a * dt
    x_expect = np.array([1.0, 2.0, -1.0]) * n * dt + a * dt * dt * n * (n + 1) / 2
    np.testing.assert_allclose(p["v"][0], v_expect, rtol=0, atol=1e-13)
    np.testing.assert_allclose(p["x"][0], x_expect, rtol=0, atol=1e-12)


def _langmuir_omega(oracle_mod, n_cells, ppc, dt=0.1, steps=130):
    ma = meshgen.langmuir_cube(n_cells)
    o = oracle_mod.Oracle(ma)
    rng = np.random.default_rng(11)
    x, v, q, m = langmuir_load(ma, ppc, rng, amplitude=0.02)
    o.add_particles(x, v, q, m)
    Ld = (1.0, 1.0, 1.0)
    mode = []
    for n in range(steps):
        rho = o.distribute_cg1()
        phi = o.poisson_direct(rho, periodic=True)
        E = o.efield(phi)
        o.boris(E, (0, 0, 0), dt * (0.5 if n == 0 else 1.0))
        p = o.particles(sort=False)
        mode.append(np.mean(p["v"][:, 0] * np.cos(2 * np.pi * p["x"][:, 0])))
        o.move(dt, Ld)
        o.update([], dt)
    s = np.array(mode)
    k = np.where(np.sign(s[1:]) != np.sign(s[:-1]))[0]
    t0 = k + s[k] / (s[k] - s[k + 1])          # interpolated zero crossings (in steps)
    assert len(t0) >= 3
    return np.pi / (np.mean(np.diff(t0)) * dt)


def test_langmuir_oscillates_at_the_plasma_frequency(oracle_mod):
    # demo/langmuir: cold electrons over a neutralising background oscillate at
    # omega_p = 1; the grid lowers it by O((k h)^2), so it must rise toward 1
    w8 = _langmuir_omega(oracle_mod, 8, 16)
    w12 = _langmuir_omega(oracle_mod, 12, 8)
    assert w8 < w12 < 1.02
    assert abs(w12 - 1.0) < 0.06, (w8, w12)


def test_flux_injection_count_and_flux_weighted_speed(oracle_mod):
    # demo/injection/injection.cpp:88-114: injected count follows the analytic
    # Maxwellian flux n * vth / sqrt(2 pi) * area * dt
    ma = meshgen.kuhn_box(6, -3.0, 3.0)
    o = oracle_mod.Oracle(ma)
    n_dens, vth, dt = 30.0, 1.0, 0.05
    o.create_flux([dict(q=-1.0, m=1.0, n=n_dens, vth=vth)])
    area = 6 * 36.0
    expect_per_step = n_dens * vth / np.sqrt(2 * np.pi) * area * dt
    total = 0
    steps = 200
    for s in range(steps):
        k, _ = o.inject(dt, 1234, s)
        total += k
    mean = total / steps
    sigma = np.sqrt(expect_per_step / steps)
    assert abs(mean - expect_per_step) < 4 * sigma + 0.05 * expect_per_step * 0  # statistical, 4 sigma
    p = o.particles(sort=False)
    # flux-weighted normal speed of a Maxwellian: vth sqrt(pi/2).  A particle
    # injected through wall w sits at distance r*dt*(v.n_w), r in [0,1], from it.
    x = p["x"]
    d = np.stack([x + 3.0, 3.0 - x], axis=2).reshape(len(x), 6)
    normals = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float)
    vn_all = p["v"] @ normals.T
    ok = (vn_all > 0) & (d <= dt * vn_all * (1 + 1e-12) + 1e-12)
    assert np.all(ok.any(axis=1))
    vn = vn_all[np.arange(len(x)), np.argmax(ok, axis=1)]
    assert abs(vn.mean() - vth * np.sqrt(np.pi / 2)) < 4 * vth / np.sqrt(len(vn))


def test_update_absorbs_at_object_and_tallies_current(oracle_mod):
    ma = meshgen.probe_box(8, 2.0, 0.6)
    o = oracle_mod.Oracle(ma)
    # one particle heading into the hole, one out through the wall, one staying
    xs = np.array([[0.9, 0.05, 0.05], [1.9, 0.1, 0.1], [-1.2, -1.1, 1.0]])
    vs = np.array([[-1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    assert o.add_particles(xs, vs, -2.0, 1.0) == 3
    o.move(0.5)
    objs = [dict(bnd_id=2, charge=1.0, current=0.0, potential=0.0)]
    absorbed = o.update(objs, 0.5)
    assert absorbed[2] == 1 and absorbed[1] == 1
    assert objs[0]["charge"] == 1.0 - 2.0 and objs[0]["current"] == -2.0 / 0.5
    assert o.num_particles() == 1


def test_esolver_projects_a_uniform_field_exactly(oracle_mod):
    """ESolver of a linear potential: -grad(phi) is a constant, which the CG1
    L2 projection reproduces at every vertex; the CG1 push of a uniform field
    then equals the DG0 push of the same field (the barycentric weights sum
    to one)."""
    from helpers import maxwellian_velocities, uniform_points
    for ma in (meshgen.probe_box(6, 2.0, 0.6), meshgen.langmuir_cube(5)):
        o = oracle_mod.Oracle(ma)
        a = np.array([0.3, -1.2, 0.7])
        phi = np.zeros(ma.n_dofs)
        phi[ma.vertex_to_dof] = ma.coords @ a + 0.5
        if ma.n_dofs < ma.n_vertices:
            # periodic: a linear phi is not periodic; project a zero field instead
            a = np.zeros(3)
            phi[:] = 0.25
        Ev = o.esolver(phi)
        np.testing.assert_allclose(Ev, np.broadcast_to(-a, Ev.shape), rtol=0, atol=1e-12)
        rng = np.random.default_rng(11)
        x = uniform_points(ma, 2000, rng)
        v = maxwellian_velocities(2000, 1.0, rng)
        o2 = oracle_mod.Oracle(ma)
        o.add_particles(x, v, -1.0, 1.0)
        o2.add_particles(x, v, -1.0, 1.0)
        Ev = np.broadcast_to(np.array([0.2, 0.1, -0.4]), (ma.n_dofs, 3)).copy()
        Ec = np.broadcast_to(np.array([0.2, 0.1, -0.4]), (ma.n_cells, 3)).copy()
        ke1 = o.boris_cg1(Ev, (0.1, 0.0, 0.3), 0.05)
        ke2 = o2.boris(Ec, (0.1, 0.0, 0.3), 0.05)
        assert abs(ke1 - ke2) <= 1e-13 * abs(ke2)
        np.testing.assert_allclose(o.particles()["v"], o2.particles()["v"], rtol=0, atol=1e-14)


def test_drifting_maxwellian_flux_count(oracle_mod):
    # the flux of a drifting Maxwellian through a face whose inward normal
    # carries the drift component u: n (vth/sqrt(2 pi) exp(-u^2/2vth^2)
    # + u/2 (1 + erf(u/(sqrt(2) vth)))), summed over the box's six faces
    from math import erf
    ma = meshgen.kuhn_box(6, -3.0, 3.0)
    o = oracle_mod.Oracle(ma)
    n_dens, vth, vd, dt = 30.0, 1.0, 0.8, 0.05
    o.create_flux([dict(q=-1.0, m=1.0, n=n_dens, vth=vth, vd=(vd, 0.0, 0.0))])

    def flux(u):
        return n_dens * (vth / np.sqrt(2 * np.pi) * np.exp(-u * u / (2 * vth * vth))
                         + 0.5 * u * (1.0 + erf(u / (np.sqrt(2.0) * vth))))

    area = 36.0
    expect_per_step = area * dt * (flux(vd) + flux(-vd) + 4 * flux(0.0))
    steps = 200
    total = sum(o.inject(dt, 4321, s)[0] for s in range(steps))
    mean = total / steps
    assert abs(mean - expect_per_step) < 4 * np.sqrt(expect_per_step / steps)
    # the injected velocities carry the drift: mean v_x exceeds the
    # zero-drift value, and v_y, v_z stay centred
    v = o.particles()["v"]
    assert v[:, 0].mean() > 0.3 and abs(v[:, 1].mean()) < 4 * vth / np.sqrt(len(v))


def test_boris_e_cross_b_drift(oracle_mod):
    # uniform E perpendicular to B: the gyro-averaged velocity is the drift
    # E x B / B^2 for either charge sign (demo/boris with an electric field)
    ma = meshgen.kuhn_box(4, -500.0, 500.0)
    E0, B = np.array([0.1, 0.0, 0.0]), np.array([0.0, 0.0, 1.0])
    drift = np.cross(E0, B) / (B @ B)
    for q in (-1.0, 1.0):
        o = oracle_mod.Oracle(ma)
        o.add_particles(np.zeros((1, 3)), np.array([[0.5, 0.0, 0.0]]), q, 1.0)
        E = np.tile(E0, (o.nc, 1))
        dt, steps = 0.05, 4000
        vs = []
        for _ in range(steps):
            o.boris(E, B, dt)
            vs.append(o.particles()["v"][0].copy())
        # average over a whole number of gyro-periods (omega_c = 1)
        per = int(round(2 * np.pi / dt))
        k = (steps // per) * per
        v_mean = np.mean(vs[:k], axis=0)
        np.testing.assert_allclose(v_mean, drift, atol=3e-3)


def test_langmuir_energy_exchange(oracle_mod):
    # demo/langmuir (langmuir.cpp:291-307 writes KE, PE, TE): the field and
    # the electrons trade energy back and forth while KE + PE stays constant
    ma = meshgen.langmuir_cube(8)
    o = oracle_mod.Oracle(ma)
    x, v, q, m = langmuir_load(ma, 16, np.random.default_rng(11), amplitude=0.02)
    o.add_particles(x, v, q, m)
    dt, KE, PE = 0.1, [], []
    for n in range(70):
        phi = o.poisson_direct(o.distribute_cg1(), periodic=True)
        PE.append(o.potential_energy(phi))
        KE.append(o.boris(o.efield(phi), (0, 0, 0), dt * (0.5 if n == 0 else 1.0)))
        o.move(dt, (1.0, 1.0, 1.0))
        o.update([], dt)
    KE, PE = np.array(KE[1:]), np.array(PE[1:])
    TE = KE + PE
    swing = KE.max() - KE.min()
    assert KE.min() < 0.05 * KE.max() and PE.min() < 0.05 * PE.max()   # full exchange
    assert np.corrcoef(KE, PE)[0, 1] < -0.999
    assert TE.max() - TE.min() < 0.01 * swing
