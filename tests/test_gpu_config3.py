"""Mixed-precision form against the FP64 form on the probe geometry (the
40^3-120^3 configuration, here at 40^3 with 4M particles): same seeded
particles, same injection seed, 100 fused steps with the object biased through
CircuitCM.  Every step records the charge density error in the L2 norm and the
max-norm over dofs, both over all dofs and over the interior dofs (those of no
cell with a facet on the exterior boundary), the potential error, both forms'
collected current, and whether the step is a boundary event: a step whose
absorbed or injected counts, particle counts or object currents differ between
the forms (a particle within rounding distance of a boundary absorbed by one
form and kept by the other).  The ids of the particles alive in one form only
are recorded at the first event steps.  The table is printed for the record.

A boundary event changes the charge of the dofs of one boundary cell, which
dominates the all-dof error of that step (about 1e-3 in L2); the interior
error separates it from the drift of the FP32 trajectories away from the FP64
ones (rounding of the position and velocity updates), which grows with the
steps.

Bars:
* step 0 deposits the loaded particles, identical up to the FP32 rounding of
  the inputs: 1e-5 relative in the max-norm over all dofs;
* the interior charge density within 1e-5 relative in the L2 norm for the
  first HORIZON steps (the drift horizon; the first step above it is printed);
* every step: potential within 1e-3 relative in the max-norm, particle counts
  within 1e-4;
* the collected object current equal in both forms on at least 95% of the
  steps, and its mean over the run within 1% and non-zero."""
import numpy as np
import pytest

from puncpp_gb300 import _lib as L
from puncpp_gb300 import punc

pytestmark = pytest.mark.gpu

STEPS = 100
HORIZON = 10
ID_RECORDS = 5


def rel_max(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def rel_l2(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def interior_dofs(mesh):
    """Dofs of no cell that has a facet on the exterior boundary (tag 1)."""
    nbr = mesh.table(L.T_NEIGHBOURS).reshape(-1, 4)
    dofs = mesh.table(L.T_CELL_DOFS).reshape(-1, 4)
    keep = np.ones(mesh.n_dofs, bool)
    keep[np.unique(dofs[(nbr == -1).any(axis=1)])] = False
    return keep


def test_mixed_form_errors_on_the_probe_at_40_cubed(capsys):
    import bench
    ma, species, loads = bench.make_workload(40, 2_000_000)
    mesh = punc.Mesh(ma)
    inner = interior_dofs(mesh)
    assert 0.5 * mesh.n_dofs < inner.sum() < mesh.n_dofs
    runs = {}
    for prec in (L.PG_FP64, L.PG_MIXED):
        pop = punc.Population(mesh, precision=prec, capacity=int(2.6 * 4_000_000), pcg_rtol=1e-10, pcg_atol=1e-12,
                              pcg_max_iter=4000)
        for s, (x, v) in zip(species, loads):
            pop.add_particles(x, v, s["q"], s["m"])
        punc.create_flux(pop, [punc.Species(s["q"], s["m"], n=s["n"], vth=s["vth"]) for s in species])
        objs = [punc.Object(2)]
        circ = punc.CircuitCM(pop, objs, [(-1, 0, bench.BIAS)], [], bench.DT)
        runs[prec] = (pop, objs, circ)
    p64, o64, _ = runs[L.PG_FP64]
    p32, o32, _ = runs[L.PG_MIXED]
    rows = []
    id_records = 0
    for n in range(STEPS):
        a = punc.step(p64, o64, bench.DT, first_step=(n == 0), inject=True, seed=0x5EED0003, step_no=n)
        b = punc.step(p32, o32, bench.DT, first_step=(n == 0), inject=True, seed=0x5EED0003, step_no=n)
        r64, r32 = punc.Function(p64, "rho").vector(), punc.Function(p32, "rho").vector()
        f64, f32 = punc.Function(p64, "phi").vector(), punc.Function(p32, "phi").vector()
        event = (a.n_absorbed != b.n_absorbed or a.n_injected != b.n_injected or a.n_particles != b.n_particles
                 or o64[0].current != o32[0].current)
        ids = None
        if event and id_records < ID_RECORDS:
            ids = np.setxor1d(p64.particles(fields=("id",))["id"], p32.particles(fields=("id",))["id"])
            id_records += 1
        rows.append(dict(n=n, l2=rel_l2(r32, r64), mx=rel_max(r32, r64), l2i=rel_l2(r32[inner], r64[inner]),
                         mxi=rel_max(r32[inner], r64[inner]), phi=rel_max(f32, f64),
                         c64=o64[0].current, c32=o32[0].current, N64=a.n_particles, N32=b.n_particles,
                         event=event, ids=ids))
    over = [r["n"] for r in rows if r["l2i"] > 1e-5]
    first_over = over[0] if over else None
    with capsys.disabled():
        print("\nprobe-40, 4M particles, mixed vs FP64 over %d steps (step, rho L2, rho max, interior rho L2, "
              "interior rho max, phi max, current FP64, current mixed, N FP64, N mixed, event, ids alive in one "
              "form only):" % STEPS)
        for r in rows:
            ids = "" if r["ids"] is None else "%d %s" % (len(r["ids"]), [int(k) for k in r["ids"][:4]])
            print("  %3d  %.2e  %.2e  %.2e  %.2e  %.2e  %+.6e  %+.6e  %8d  %8d  %s  %s" % (
                r["n"], r["l2"], r["mx"], r["l2i"], r["mxi"], r["phi"], r["c64"], r["c32"], r["N64"], r["N32"],
                "event" if r["event"] else "-", ids))
        print("  first step with the interior rho L2 error above 1e-5:", first_over,
              "; event steps:", sum(r["event"] for r in rows))
    assert rows[0]["mx"] < 1e-5, rows[0]
    for r in rows[:HORIZON]:
        assert r["l2i"] < 1e-5, r
    for r in rows:
        assert r["phi"] < 1e-3 and abs(r["N64"] - r["N32"]) <= 1e-4 * r["N64"], r
    assert sum(r["c64"] == r["c32"] for r in rows) >= 0.95 * STEPS
    mean64 = np.mean([r["c64"] for r in rows])
    mean32 = np.mean([r["c32"] for r in rows])
    assert mean64 != 0.0 and abs(mean32 - mean64) < 1e-2 * abs(mean64), (mean32, mean64)
    for pop, _, _ in runs.values():
        pop.close()
