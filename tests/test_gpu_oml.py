"""The reference's one integration check, run on the engine.

test/test.py reads the object current (history column 7) of the run set up
by test/test.ini on the mesh of test/sphere.geo and passes when its average
over steps 500..2000 is within 3% of I_OML = -0.13579559 A, the orbital-motion-
limited electron current to a sphere of radius 1 m at +2 kT/e in a plasma of
1e10 m^-3 electrons and protons with T_i = T_e.  The inputs below are the
values of test.ini: a spherical probe of radius 1 inside an exterior sphere
of radius 20 (lengths in metres), 5e5 simulation electrons and 5e5 protons
loaded uniformly with Maxwellian velocities, flux injection through the outer
sphere, the object held at 361.90256041589 V by a voltage source to ground,
dt = 0.0159 plasma periods, 2000 steps, the interaction program's default
field path (ESolver CG1 field and accel_cg1) and Poisson tolerances (rel
1e-10, abs 1e-12).

The run is made in plasma units (Debye length, inverse electron plasma
frequency, electron thermal speed, kT_e/e; eps0 = 1) and the mean current is
converted to amperes.  The mesh is the engine's body-fitted shell
(meshgen.sphere_shell: an icosphere of 1280 triangles on the object, graded
radial layers) in place of gmsh's mesh of sphere.geo, which cannot be made
here (no gmsh).  Both precision forms must pass the reference's 3% bar."""
import math

import numpy as np
import pytest

from puncpp_gb300 import _lib as L
from puncpp_gb300 import meshgen, punc

pytestmark = pytest.mark.gpu

# CODATA 2018
E_CHARGE = 1.602176634e-19
M_E = 9.1093837015e-31
AMU = 1.66053906660e-27
EPS0 = 8.8541878128e-12
# test/test.ini and test/test.py
DENSITY = 1.0e10
VTH_E = 5641460.226981773
VTH_I = 131654.93286648966
AMOUNT = 5e5
V_BIAS = 361.90256041589
DT_PLASMA = 0.0159
STOP = 2000
R_INNER, R_OUTER = 1.0, 20.0
I_TRUE = -0.13579559


def run_probe(precision, seed):
    wp = math.sqrt(DENSITY * E_CHARGE ** 2 / (EPS0 * M_E))
    debye = VTH_E / wp
    kT_over_e = M_E * VTH_E ** 2 / E_CHARGE
    ma = meshgen.sphere_shell(R_INNER / debye, R_OUTER / debye, level=3)
    mesh = punc.Mesh(ma)
    species = [punc.Species.from_physical(-1.0, 1.0, 1.0, AMOUNT, punc.ParticleAmountType.in_total, mesh, vth=1.0),
               punc.Species.from_physical(1.0, AMU / M_E, 1.0, AMOUNT, punc.ParticleAmountType.in_total, mesh,
                                           vth=VTH_I / VTH_E)]
    # read_timestep (interaction/io.cpp:129-169): dt_plasma plasma periods, unless
    # a particle at the largest speed would cross the smallest cell in less
    dt = DT_PLASMA * punc.min_plasma_period(species, 1.0)
    p = ma.coords[ma.cells]
    h = np.max([np.linalg.norm(p[:, i] - p[:, j], axis=1) for i in range(4) for j in range(i + 1, 4)], axis=0)
    v_max = max(math.sqrt((0.0 + 1.0 * s.vth) ** 2) for s in species)
    dt = min(dt, h.min() / v_max)
    pop = punc.Population(mesh, precision=precision, capacity=2_000_000, pcg_rtol=1e-10, pcg_atol=1e-12,
                          pcg_max_iter=4000)
    added = punc.load_particles(pop, species, seed=seed)
    assert all(abs(a - AMOUNT) <= 1 for a in added), added
    punc.create_flux(pop, species)
    objs = [punc.Object(2)]
    punc.CircuitCM(pop, objs, [(-1, 0, V_BIAS / kT_over_e)], [], dt)
    currents = []
    for n in range(STOP):
        punc.step(pop, objs, dt, first_step=(n == 0), inject=True, seed=seed, step_no=n, efield_cg1=True)
        currents.append(objs[0].current)
    n_end = pop.num_of_particles()
    pop.close()
    # history line n holds the current of the update of step n - 1 (0 on line
    # 0); test.py averages lines 500..2000
    hist = np.concatenate([[0.0], currents])
    amperes = E_CHARGE * DENSITY * debye ** 2 * VTH_E      # current unit: e n0 lambda_D^2 v_th
    return float(np.mean(hist[500:])) * amperes, dt, n_end


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_oml_probe_current_within_three_percent(form, capsys):
    prec = L.PG_FP64 if form == "fp64" else L.PG_MIXED
    I_mean, dt, n_end = run_probe(prec, seed=0x0E1)
    err = (I_TRUE - I_mean) / I_mean
    with capsys.disabled():
        print(f"\nOML check ({form}): dt = {dt:.6f} / omega_pe, {n_end} particles at the end, "
              f"simulated current {I_mean:.6g} A, true {I_TRUE:g} A, relative error {100 * err:.2f}%")
    assert abs(err) < 0.03
