"""pg_pcg_solve_noalloc: the CG entry point for callers that cannot allocate
device memory (their host application owns every GPU buffer, or they run
inside another framework's memory pool).  It must give the same potential as
the engine's own solver (pg_poisson_solve, which works in buffers allocated
at pg_create) on the same Poisson system, call after call, although every call
reuses the same static device scratch array, and match the oracle's direct
sparse solve; a smaller system solved after the larger one, from a non-zero
initial guess, must not pick up what the larger one left in the scratch."""
import ctypes as C

import numpy as np
import pytest

from helpers import maxwellian_velocities, uniform_points
from puncpp_gb300 import _lib as L
from puncpp_gb300 import meshgen, punc

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def reduced_system(mesh, rho, potentials):
    """The Dirichlet-eliminated P1 system the engine solves (identity rows for
    boundary dofs, their columns moved to the right-hand side)."""
    rp, col = mesh.table(L.T_CSR_ROWPTR), mesh.table(L.T_CSR_COL)
    K, M = mesh.table(L.T_STIFFNESS), mesh.table(L.T_MASS)
    kind = mesh.table(L.T_BC_KIND)
    n = len(kind)
    g = np.zeros(n)
    for k, v in enumerate(potentials):
        g[kind == k + 1] = v
    rows, cols, vals = [0], [], []
    b = np.zeros(n)
    for i in range(n):
        s, e = rp[i], rp[i + 1]
        if kind[i] >= 0:
            cols.append(i); vals.append(1.0); b[i] = g[i]
        else:
            acc = float(np.dot(M[s:e], rho[col[s:e]]))
            for k in range(s, e):
                j = col[k]
                if kind[j] < 0:
                    cols.append(j); vals.append(K[k])
                else:
                    acc -= K[k] * g[j]
            b[i] = acc
        rows.append(len(cols))
    return (np.array(rows, np.int32), np.array(cols, np.int32), np.array(vals, np.float64), b)


def _call(lib, n, rowptr, col, val, b, x, rtol, atol, max_iter):
    it, res = C.c_int32(), C.c_double()
    rc = lib.pg_pcg_solve_noalloc(n, rowptr.data_ptr(), col.data_ptr(), val.data_ptr(), b.data_ptr(), x.data_ptr(),
                                  rtol, atol, max_iter, None, C.byref(it), C.byref(res))
    return rc, it.value, res.value


def test_no_alloc_solve_matches_the_engine_solver_on_two_calls(lib, oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    ma = meshgen.probe_box(10, 2.0, 0.6)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, pcg_rtol=RTOL, pcg_atol=1e-30, pcg_max_iter=5000)
    rng = np.random.default_rng(21)
    xs_e = uniform_points(ma, 8000, rng)
    vs_e = maxwellian_velocities(8000, 1.0, rng)
    xs_i = uniform_points(ma, 4000, rng)
    vs_i = maxwellian_velocities(4000, 0.1, rng)
    pop.add_particles(xs_e, vs_e, -1.0, 1.0)
    pop.add_particles(xs_i, vs_i, 1.0, 100.0)
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    phi_ref = punc.PoissonSolver(pop, objs).solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)
    # an independent reference: the oracle's direct sparse solve of the same system
    o = oracle_mod.Oracle(ma)
    o.add_particles(xs_e, vs_e, -1.0, 1.0)
    o.add_particles(xs_i, vs_i, 1.0, 100.0)
    phi_direct = o.poisson_direct(o.distribute_cg1(), potentials=[-2.0])

    rowptr, col, val, b = reduced_system(mesh, rho, [-2.0])
    n = len(b)
    dev = torch.device("cuda:0")
    d_row = torch.from_numpy(rowptr).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(val).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    for call in range(2):
        d_x = torch.zeros(n, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc, it, res = _call(lib, n, d_row, d_col, d_val, d_b, d_x, RTOL, 1e-30, 5000)
        L.check(rc)
        x = d_x.cpu().numpy()
        assert it > 0 and res <= RTOL * np.linalg.norm(b)
        err = np.abs(x - phi_ref).max() / np.abs(phi_ref).max()
        assert err < 1e-9, (call, err)
        err_direct = np.abs(x - phi_direct).max() / np.abs(phi_direct).max()
        assert err_direct < 1e-10, (call, err_direct)

    # the iteration cap is reported, with the iterations done
    d_x = torch.zeros(n, dtype=torch.float64, device=dev)
    rc, it, res = _call(lib, n, d_row, d_col, d_val, d_b, d_x, RTOL, 1e-30, 1)
    assert rc == L.PG_ERR_NOT_CONVERGED and it == 1 and res > RTOL * np.linalg.norm(b)
    assert b"iteration cap" in lib.pg_last_error()

    # a smaller system after the larger one, from a non-zero initial guess:
    # nothing left in the shared scratch past its n rows may leak in
    m = 999
    main = np.full(m, 2.0) + np.linspace(0.0, 1.0, m)
    rows = [0]
    cols, vals = [], []
    for i in range(m):
        for j, v in ((i - 1, -1.0), (i, main[i]), (i + 1, -1.0)):
            if 0 <= j < m:
                cols.append(j); vals.append(v)
        rows.append(len(cols))
    A = np.diag(main) - np.diag(np.ones(m - 1), 1) - np.diag(np.ones(m - 1), -1)
    bs = rng.normal(size=m)
    x0 = rng.normal(size=m)
    s_row = torch.tensor(rows, dtype=torch.int32, device=dev)
    s_col = torch.tensor(cols, dtype=torch.int32, device=dev)
    s_val = torch.tensor(vals, dtype=torch.float64, device=dev)
    s_b = torch.from_numpy(bs).to(dev)
    s_x = torch.from_numpy(x0.copy()).to(dev)
    torch.cuda.synchronize()
    rc, it, res = _call(lib, m, s_row, s_col, s_val, s_b, s_x, 1e-13, 1e-30, 5000)
    L.check(rc)
    ref = np.linalg.solve(A, bs)
    assert np.abs(s_x.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-11
    assert it > 0 and res <= 1e-13 * np.linalg.norm(bs)

    # sizes beyond the static scratch are refused before any work is queued
    rc = lib.pg_pcg_solve_noalloc((1 << 19) + 1, d_row.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                  d_b.data_ptr(), d_x.data_ptr(), RTOL, 1e-30, 10, None, None, None)
    assert rc == 1 and b"static scratch" in lib.pg_last_error()
    pop.close()
