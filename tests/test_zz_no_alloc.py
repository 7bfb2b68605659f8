"""pg_pcg_solve_noalloc: the CG entry point for callers that cannot allocate
device memory (their host application owns every GPU buffer, or they run
inside another framework's memory pool).  It must give the same potential as
the engine's own solver (pg_poisson_solve, which works in buffers allocated
at pg_create) on the same Poisson system, call after call, although every call
reuses the same static device scratch array."""
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


def test_no_alloc_solve_matches_the_engine_solver_on_two_calls(lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    ma = meshgen.probe_box(10, 2.0, 0.6)
    mesh = punc.Mesh(ma)
    pop = punc.Population(mesh, pcg_rtol=RTOL, pcg_atol=1e-30, pcg_max_iter=5000)
    rng = np.random.default_rng(21)
    pop.add_particles(uniform_points(ma, 8000, rng), maxwellian_velocities(8000, 1.0, rng), -1.0, 1.0)
    pop.add_particles(uniform_points(ma, 4000, rng), maxwellian_velocities(4000, 0.1, rng), 1.0, 100.0)
    rho = punc.distribute_cg1(pop)
    objs = [punc.Object(2, potential=-2.0)]
    phi_ref = punc.PoissonSolver(pop, objs).solve(punc.Function(pop, "phi"), punc.Function(pop, "rho"), objs)

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
        it, res = C.c_int32(), C.c_double()
        rc = lib.pg_pcg_solve_noalloc(n, d_row.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), d_b.data_ptr(),
                                      d_x.data_ptr(), RTOL, 1e-30, 5000, None, C.byref(it), C.byref(res))
        L.check(rc)
        x = d_x.cpu().numpy()
        assert it.value > 0 and res.value <= RTOL * np.linalg.norm(b)
        err = np.abs(x - phi_ref).max() / np.abs(phi_ref).max()
        assert err < 1e-9, (call, err)

    # sizes beyond the static scratch are refused before any work is queued
    rc = lib.pg_pcg_solve_noalloc((1 << 19) + 1, d_row.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                  d_b.data_ptr(), d_x.data_ptr(), RTOL, 1e-30, 10, None, None, None)
    assert rc == 1 and b"static scratch" in lib.pg_last_error()
    pop.close()
