"""Host-side smoothed-aggregation hierarchy of the Poisson preconditioner
(puncpp_gb300/csrc/amg.cpp), checked on the CPU: Galerkin coarse operators,
R = P^T, the coarsest inverse, the constant null space of periodic meshes,
and the iteration count of CG preconditioned by the same V-cycle the device
kernel runs (restated here in FP64 numpy)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from puncpp_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "puncpp_gb300", "csrc")


@pytest.fixture(scope="module")
def amgd(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("amg") / "libamgd.so"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-I" + CSRC,
                        os.path.join(ROOT, "tests", "cpp", "amg_dump.cpp"), os.path.join(CSRC, "amg.cpp"),
                        "-o", str(so)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = C.CDLL(str(so))
    d.amgd_setup.restype = C.c_void_p
    d.amgd_setup.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double,
                             C.c_int64, C.POINTER(C.c_int)]
    d.amgd_levels.argtypes = [C.c_void_p]
    d.amgd_shape.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    d.amgd_copy.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    d.amgd_omega.argtypes = [C.c_void_p, C.c_int]
    d.amgd_omega.restype = C.c_double
    d.amgd_coarse_inv.argtypes = [C.c_void_p, C.c_void_p]
    d.amgd_free.argtypes = [C.c_void_p]
    d.amgd_cycle.restype = C.c_void_p
    d.amgd_cycle.argtypes = [C.c_void_p]
    d.amgd_cycle_shape.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    d.amgd_cycle_copy.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    d.amgd_cycle_offsets.argtypes = [C.c_void_p, C.c_void_p]
    d.amgd_cycle_free.argtypes = [C.c_void_p]
    return d


def _csr_out(shape_fn, copy_fn):
    shape = np.zeros(3, np.int64)
    shape_fn(shape.ctypes.data)
    n, m, nnz = (int(x) for x in shape)
    if n == 0:
        return None
    orp = np.zeros(n + 1, np.int64)
    oci = np.zeros(max(nnz, 1), np.int32)
    ov = np.zeros(max(nnz, 1))
    copy_fn(orp.ctypes.data, oci.ctypes.data, ov.ctypes.data)
    return sp.csr_matrix((ov[:nnz], oci[:nnz], orp), shape=(n, m))


def hierarchy(d, A, nullspace=False, theta=-1.0, theta_factor=0.0, coarse_max=0, cycle=None):
    """Levels and coarsest inverse; fills `cycle` (a dict) with the device
    cycle's operators G, U1 and the stack offsets when given."""
    A = sp.csr_matrix(A)
    A.sort_indices()
    rp = A.indptr.astype(np.int64)
    ci = A.indices.astype(np.int32)
    v = A.data.astype(np.float64)
    rc = C.c_int(-1)
    h = d.amgd_setup(A.shape[0], rp.ctypes.data, ci.ctypes.data, v.ctypes.data, 1 if nullspace else 0, theta,
                     theta_factor, coarse_max, C.byref(rc))
    try:
        assert rc.value == 0
        levels = []
        for l in range(d.amgd_levels(h)):
            ops = {}
            for which, name in enumerate(["A", "P", "R", "S", "ST"]):
                M = _csr_out(lambda o: d.amgd_shape(h, l, which, o), lambda a, b, c: d.amgd_copy(h, l, which, a, b, c))
                if M is not None:
                    ops[name] = M
            ops["omega"] = d.amgd_omega(h, l)
            levels.append(ops)
        nc = levels[-1]["A"].shape[0]
        cinv = np.zeros(nc * nc)
        d.amgd_coarse_inv(h, cinv.ctypes.data)
        if cycle is not None:
            c = d.amgd_cycle(h)
            try:
                for which, name in enumerate(["G", "U1"]):
                    cycle[name] = _csr_out(lambda o: d.amgd_cycle_shape(c, which, o),
                                           lambda a, b, cc: d.amgd_cycle_copy(c, which, a, b, cc))
                off = np.zeros(len(levels) + 1, np.int64)
                cycle["off"] = off[:d.amgd_cycle_offsets(c, off.ctypes.data)]
            finally:
                d.amgd_cycle_free(c)
        return levels, cinv.reshape(nc, nc)
    finally:
        d.amgd_free(h)


def reduced_operator(oracle_mod, ma, periodic=False):
    """The solver's matrix: Dirichlet rows and columns replaced by identity."""
    o = oracle_mod.Oracle(ma)
    K, _ = o.matrices()
    kind, _ = o.dirichlet(periodic)
    free = (kind < 0).astype(float)
    A = sp.diags(free) @ K @ sp.diags(free) + sp.diags(1.0 - free)
    A = sp.csr_matrix(A)
    A.eliminate_zeros()
    return A


def vcycle_textbook(levels, cinv, b, l=0):
    """One V-cycle: a weighted-Jacobi sweep from zero, restriction, coarse
    correction, prolongation, one more sweep."""
    L = levels[l]
    if l == len(levels) - 1:
        return cinv @ b
    dinv = 1.0 / L["A"].diagonal()
    x = L["omega"] * dinv * b
    r = b - L["A"] @ x
    x = x + L["P"] @ vcycle_textbook(levels, cinv, L["R"] @ r, l + 1)
    return x + L["omega"] * dinv * (b - L["A"] @ x)


def vcycle(levels, cinv, b, l=0):
    """The same V-cycle as the device applies it: B b = W b + S B_c S^T b with
    W = w D^-1 (2 I - A w D^-1) and S = (I - w D^-1 A) P."""
    L = levels[l]
    if l == len(levels) - 1:
        return cinv @ b
    m = L["omega"] / L["A"].diagonal()
    t = m * (2.0 * b - L["A"] @ (m * b))
    return t + L["S"] @ vcycle(levels, cinv, L["ST"] @ b, l + 1)


def vcycle_collapsed(levels, cinv, cyc, b):
    """The cycle as the device kernel runs it: one down-sweep phase per level
    (t_l = W_l b_l and the restriction; the last one G b = C^-1 S^T b), the
    up-sweep of levels >= 1 in one product with U1, then level 0."""
    L = len(levels) - 1
    if L == 0:
        return cinv @ b
    t, bl = [], b
    for l in range(L):
        m = levels[l]["omega"] / levels[l]["A"].diagonal()
        t.append(m * (2.0 * bl - levels[l]["A"] @ (m * bl)))
        if l < L - 1:
            bl = levels[l]["ST"] @ bl
        else:
            yL = cyc["G"] @ bl
    if L >= 2:
        y1 = t[1] + cyc["U1"] @ np.concatenate(t[2:L] + [yL])
    else:
        y1 = yL
    return t[0] + levels[0]["S"] @ y1


def pcg(A, b, prec, rtol):
    x = np.zeros_like(b)
    r = b.copy()
    z = prec(r)
    p = z.copy()
    rz = r @ z
    tol = rtol * np.linalg.norm(b)
    for it in range(1, 5000):
        Ap = A @ p
        a = rz / (p @ Ap)
        x += a * p
        r -= a * Ap
        if np.linalg.norm(r) <= tol:
            return x, it
        z = prec(r)
        rz, rz_old = r @ z, rz
        p = z + (rz / rz_old) * p
    raise AssertionError("no convergence")


@pytest.fixture(scope="module")
def probe(oracle_mod):
    ma = meshgen.probe_box(14, 4.0, 0.8)
    return ma, reduced_operator(oracle_mod, ma)


def test_levels_coarsen_and_are_galerkin(amgd, probe):
    ma, A = probe
    levels, cinv = hierarchy(amgd, A)
    assert len(levels) >= 2
    sizes = [L["A"].shape[0] for L in levels]
    assert sizes[-1] <= 400
    assert all(sizes[k + 1] * 4 < sizes[k] for k in range(len(sizes) - 1)), sizes
    for k in range(len(levels) - 1):
        L, N = levels[k], levels[k + 1]
        assert abs(L["R"] - L["P"].T).max() == 0.0
        G = L["R"] @ L["A"] @ L["P"]
        assert abs(G - N["A"]).max() <= 1e-12 * abs(N["A"]).max()
        assert abs(N["A"] - N["A"].T).max() <= 1e-12 * abs(N["A"]).max()
        assert 0.0 < L["omega"] < 2.0
    Ac = levels[-1]["A"].toarray()
    np.testing.assert_allclose(cinv @ Ac, np.eye(len(Ac)), atol=1e-9)


def test_transfer_operators_give_the_textbook_vcycle(amgd, probe):
    ma, A = probe
    levels, cinv = hierarchy(amgd, A)
    for L in levels[:-1]:
        m = L["omega"] / L["A"].diagonal()
        S = L["P"] - sp.diags(m) @ (L["A"] @ L["P"])
        assert abs(S - L["S"]).max() <= 1e-12 * abs(L["P"]).max()
        assert abs(L["ST"] - L["S"].T).max() == 0.0
    b = np.random.default_rng(7).standard_normal(A.shape[0])
    np.testing.assert_allclose(vcycle(levels, cinv, b), vcycle_textbook(levels, cinv, b), rtol=0, atol=1e-10)


@pytest.fixture(scope="module")
def probe22(oracle_mod):
    ma = meshgen.probe_box(22, 4.0, 0.8)
    return ma, reduced_operator(oracle_mod, ma)


@pytest.mark.parametrize("coarse_max,depth", [(3000, 1), (400, 2), (10, 3)])
def test_collapsed_cycle_equals_the_vcycle(coarse_max, depth, amgd, probe22):
    """G = C^-1 S^T and U1 = [S_1 | S_1 S_2 | ...] reproduce the V-cycle for
    hierarchies with 1, 2 and 3 levels above the coarsest."""
    ma, A = probe22
    cyc = {}
    levels, cinv = hierarchy(amgd, A, coarse_max=coarse_max, cycle=cyc)
    L = len(levels) - 1
    assert L == depth
    G = cyc["G"]
    assert G.shape == (levels[L]["A"].shape[0], levels[L - 1]["A"].shape[0])
    np.testing.assert_allclose(G.toarray(), cinv @ levels[L - 1]["ST"].toarray(), atol=1e-12 * abs(cinv).max())
    if L >= 2:
        assert cyc["U1"].shape == (levels[1]["A"].shape[0], sum(levels[l]["A"].shape[0] for l in range(2, L + 1)))
    else:
        assert cyc["U1"] is None
    b = np.random.default_rng(8).standard_normal(A.shape[0])
    ref = vcycle_textbook(levels, cinv, b)
    np.testing.assert_allclose(vcycle_collapsed(levels, cinv, cyc, b), ref, rtol=0, atol=1e-10 * abs(ref).max())


def test_strength_threshold_coarsens_less_from_level_one(amgd, probe22):
    """A strength threshold (the engine's pg_amg_set_strength): the Kuhn
    Laplacian's couplings are all 1/6 of the diagonal, so level 0's aggregates
    and level 1 do not change; below that weak couplings are dropped and the
    coarser levels grow.  The collapsed cycle still equals the textbook
    V-cycle and the preconditioned CG meets the tolerance in a similar count."""
    ma, A = probe22
    b = np.random.default_rng(11).standard_normal(A.shape[0])
    its = {}
    sizes = {}
    for theta in (0.0, 0.05):
        cyc = {}
        levels, cinv = hierarchy(amgd, A, theta=theta, theta_factor=1.0, cycle=cyc)
        sizes[theta] = [L["A"].shape[0] for L in levels]
        ref = vcycle_textbook(levels, cinv, b)
        np.testing.assert_allclose(vcycle_collapsed(levels, cinv, cyc, b), ref, rtol=0, atol=1e-10 * abs(ref).max())
        x, its[theta] = pcg(A, b, lambda r: vcycle(levels, cinv, r), 1e-10)
        assert np.linalg.norm(b - A @ x) <= 1e-10 * np.linalg.norm(b)
    assert sizes[0.05][:2] == sizes[0.0][:2], sizes
    assert sizes[0.05][-1] > sizes[0.0][-1], sizes
    assert its[0.05] <= its[0.0] + 2, its


def test_vcycle_preconditioner_beats_jacobi(amgd, probe):
    ma, A = probe
    levels, cinv = hierarchy(amgd, A)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(A.shape[0])
    x, it_amg = pcg(A, b, lambda r: vcycle(levels, cinv, r), 1e-10)
    assert np.linalg.norm(b - A @ x) <= 1e-10 * np.linalg.norm(b)
    dinv = 1.0 / A.diagonal()
    _, it_jac = pcg(A, b, lambda r: dinv * r, 1e-10)
    assert it_amg < 25 and it_amg * 4 < it_jac, (it_amg, it_jac)


def test_periodic_constant_null_space(amgd, oracle_mod):
    ma = meshgen.langmuir_cube(10)
    A = reduced_operator(oracle_mod, ma, periodic=True)
    assert abs(A @ np.ones(A.shape[0])).max() < 1e-12 * abs(A).max()
    levels, cinv = hierarchy(amgd, A, nullspace=True)
    for L in levels[:-1]:
        ones_c = np.ones(L["P"].shape[1])
        np.testing.assert_allclose(L["P"] @ ones_c, 1.0, atol=1e-12)
    Ac = levels[-1]["A"].toarray()
    nc = len(Ac)
    assert abs(Ac @ np.ones(nc)).max() < 1e-10 * abs(Ac).max()
    reg = Ac + np.trace(Ac) / nc ** 2 * np.ones((nc, nc))
    np.testing.assert_allclose(cinv @ reg, np.eye(nc), atol=1e-9)
    # singular but consistent: CG on the mean-free right-hand side converges
    rng = np.random.default_rng(4)
    b = rng.standard_normal(A.shape[0])
    b -= b.mean()
    x, it = pcg(A, b, lambda r: vcycle(levels, cinv, r), 1e-10)
    assert it < 25


def test_hierarchy_is_deterministic(amgd, probe):
    """Two set-ups of the same matrix give identical operators, so a run's
    solver iterations and potentials are reproducible."""
    ma, A = probe
    c1, c2 = {}, {}
    l1, i1 = hierarchy(amgd, A, cycle=c1)
    l2, i2 = hierarchy(amgd, A, cycle=c2)
    assert len(l1) == len(l2)
    for a, b in zip(l1, l2):
        for k in ("A", "P", "S", "ST"):
            if k in a:
                assert (a[k] != b[k]).nnz == 0
        assert a["omega"] == b["omega"]
    assert np.array_equal(i1, i2)
    for k in ("G", "U1"):
        if c1[k] is not None:
            assert (c1[k] != c2[k]).nnz == 0


@pytest.mark.parametrize("coarse_max", [400, 10])
def test_collapsed_preconditioner_is_symmetric_positive_definite(coarse_max, amgd, probe22):
    """CG needs a symmetric positive definite preconditioner: x.By = y.Bx and
    x.Bx > 0 for the cycle the device applies."""
    ma, A = probe22
    cyc = {}
    levels, cinv = hierarchy(amgd, A, coarse_max=coarse_max, cycle=cyc)
    rng = np.random.default_rng(11)
    B = lambda v: vcycle_collapsed(levels, cinv, cyc, v)
    for _ in range(8):
        x, y = rng.standard_normal(A.shape[0]), rng.standard_normal(A.shape[0])
        bx, by = B(x), B(y)
        assert abs(x @ by - y @ bx) <= 1e-11 * np.linalg.norm(x) * np.linalg.norm(by)
        assert x @ bx > 0.0


def _setup_rc(d, A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    rp, ci, v = A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data.astype(np.float64)
    rc = C.c_int(-1)
    h = d.amgd_setup(A.shape[0], rp.ctypes.data, ci.ctypes.data, v.ctypes.data, 0, -1.0, 0.0, 0, C.byref(rc))
    d.amgd_free(h)
    return rc.value


def test_setup_reports_stalled_coarsening_and_a_singular_coarsest_operator(amgd):
    """Set-up errors the engine turns into status codes: coarsening that stops
    above the dense-inverse limit (4096 rows; 9, PG_ERR_ARG) and a singular
    coarsest operator (8, PG_ERR_SINGULAR)."""
    assert _setup_rc(amgd, sp.identity(5000, format="csr")) == 9
    assert _setup_rc(amgd, sp.csr_matrix(np.array([[1.0, 1.0], [1.0, 1.0]]))) == 8
    assert _setup_rc(amgd, sp.csr_matrix(np.array([[2.0, -1.0], [-1.0, 2.0]]))) == 0
