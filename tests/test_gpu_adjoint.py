"""Adjoint of K fused steps (push, deposit, Poisson) on the periodic Langmuir
configuration with Gaussian initial velocities and a uniform external field,
loss = ||rho_K - rho_target||^2 on the CG1 charge vector.

The gradients with respect to the initial velocities and the external field
come from pg_adjoint_forward / pg_adjoint_backward (cells fixed from the
forward pass, checkpoints every C steps, Poisson adjoint as a second PCG), and
are exposed to torch through a torch.autograd.Function.  They are checked
against central finite differences of the FP64 forward, the reference gradient
of the same FP64 computation.

The loss is piecewise smooth: a particle that changes cell sees a different
DG0 field, and a perturbation of the uniform field moves every particle, so
one of 4000 particles crossing a facet inside +-1e-6 already puts a jump into
a difference quotient.  The step h is therefore shrunk (1e-6 down to 1e-9)
until the forward and backward one-sided quotients agree, i.e. until no jump
lies within +-h, and the central quotient at that h is the check."""
import os

import numpy as np
import pytest

from puncpp_gb300 import _lib as L
from puncpp_gb300 import meshgen, punc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class Langmuir:
    """A fresh FP64 engine for each evaluation: electrons uniform in the unit
    cube (seeded), velocities v0, external field E0, K steps with checkpoints."""

    def __init__(self, n_side, n_part, K, C, dt, seed):
        self.ma = meshgen.langmuir_cube(n_side)
        self.mesh = punc.Mesh(self.ma)
        rng = np.random.default_rng(seed)
        self.x = rng.random((n_part, 3))
        self.v0 = rng.normal(0.0, 0.1, size=(n_part, 3))
        self.w = 1.0 / n_part
        self.K, self.C, self.dt = K, C, dt
        self.target = rng.normal(0.0, 1.0, size=self.mesh.n_dofs) * 0.05
        self.pop = None

    def loss(self, v0, E0):
        if self.pop is not None:
            self.pop.close()
        self.pop = punc.Population(self.mesh, periodic=True, pcg_rtol=1e-13, pcg_atol=1e-30, pcg_max_iter=5000)
        assert self.pop.add_particles(self.x, np.ascontiguousarray(v0), -self.w, self.w) == len(self.x)
        return punc.adjoint_forward(self.pop, [], self.dt, self.K, self.C, self.target, first_step=True,
                                    E0=tuple(E0), Ld=self.ma.Ld)

    def grads(self):
        gv, ge, _ = punc.adjoint_backward(self.pop, len(self.x))
        return gv, ge

    def oracle_adjoint(self, oracle_mod):
        """(loss, grad_v0, grad_E0) of the same K steps by the oracle's reverse sweep"""
        loss, gv, ge, _ = oracle_mod.langmuir_adjoint(self.ma, self.x, self.v0, -self.w, self.w,
                                                      np.array([0.01, 0.0, 0.0]), self.dt, self.K, self.target,
                                                      self.ma.Ld, nthreads=os.cpu_count() or 1)
        return loss, gv, ge


class AdjointLoss(torch.autograd.Function):
    """loss(v0, E0) with the engine's adjoint as the backward."""

    @staticmethod
    def forward(ctx, v0, E0, model):
        loss = model.loss(v0.detach().cpu().numpy(), E0.detach().cpu().numpy())
        ctx.model = model
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, g):
        gv, ge = ctx.model.grads()
        return g * torch.from_numpy(gv), g * torch.from_numpy(ge), None


@pytest.mark.parametrize("n_side,n_part,K,C", [(6, 4000, 12, 4), (16, 200_000, 20, 5)])
def test_adjoint_gradients_match_finite_differences(n_side, n_part, K, C, oracle_mod):
    model = Langmuir(n_side, n_part, K, C, dt=0.1, seed=n_side)
    v0 = torch.tensor(model.v0, requires_grad=True)
    E0 = torch.tensor([0.01, 0.0, 0.0], dtype=torch.float64, requires_grad=True)
    loss = AdjointLoss.apply(v0, E0, model)
    loss.backward()
    gv, ge = v0.grad.numpy(), E0.grad.numpy()
    assert np.all(np.isfinite(gv)) and np.abs(gv).max() > 0

    # the oracle's reverse sweep of the same computation
    lo, gvo, geo = model.oracle_adjoint(oracle_mod)
    assert abs(float(loss.detach()) - lo) <= 1e-10 * abs(lo)
    assert np.abs(gv - gvo).max() <= 1e-8 * np.abs(gvo).max()
    assert np.abs(ge - geo).max() <= 1e-8 * np.abs(geo).max()

    base_v, base_e = model.v0.copy(), np.array([0.01, 0.0, 0.0])
    base_loss = model.loss(base_v, base_e)

    def smooth_fd(perturbed):
        """central difference at the largest h with no jump within +-h"""
        for h in (1e-6, 1e-7, 1e-8, 1e-9):
            lp, lm = perturbed(h), perturbed(-h)
            dp, dm = (lp - base_loss) / h, (base_loss - lm) / h
            if abs(dp - dm) <= 1e-3 * max(abs(dp), abs(dm), 1e-12):
                return (lp - lm) / (2 * h)
        raise AssertionError("no jump-free step found")

    def fd_v(i, j):
        def f(h):
            v = base_v.copy()
            v[i, j] += h
            return model.loss(v, base_e)
        return smooth_fd(f)

    def fd_e(j):
        def f(h):
            e = base_e.copy()
            e[j] += h
            return model.loss(base_v, e)
        return smooth_fd(f)

    rng = np.random.default_rng(1)
    top = int(np.argmax(np.abs(gv).sum(axis=1)))
    picks = [(top, int(np.argmax(np.abs(gv[top]))))]
    picks += [(int(i), int(j)) for i, j in zip(rng.integers(0, n_part, 3), rng.integers(0, 3, 3))]
    scale_v = np.abs(gv).max()
    for i, j in picks:
        fd = fd_v(i, j)
        assert abs(gv[i, j] - fd) <= 1e-5 * scale_v + 1e-4 * abs(fd), (i, j, gv[i, j], fd)
    for j in range(3):
        fd = fd_e(j)
        assert abs(ge[j] - fd) <= 1e-4 * max(abs(fd), np.abs(ge).max()), (j, ge[j], fd)


def test_adjoint_full_size(oracle_mod):
    """Periodic Langmuir mesh of 32^3 sub-cubes x 6 tetrahedra, 2M electrons,
    K = 50 steps with a checkpoint every 10.  The gradients are checked against
    the oracle's reverse sweep of the same steps (all 6M velocity components
    and E0), and single velocity components against jump-free central
    differences.  A difference quotient in E0 is not taken at this size: E0
    moves all 2M particles, and at every step h that FP64 still resolves some
    of them cross a facet within +-h (the quotient then measures the jumps of
    the piecewise-smooth loss, not its derivative)."""
    model = Langmuir(32, 2_000_000, 50, 10, dt=0.1, seed=32)
    loss = model.loss(model.v0, np.array([0.01, 0.0, 0.0]))
    gv, ge = model.grads()
    lo, gvo, geo = model.oracle_adjoint(oracle_mod)
    assert abs(loss - lo) <= 1e-10 * abs(lo)
    assert np.abs(gv - gvo).max() <= 1e-8 * np.abs(gvo).max()
    assert np.abs(ge - geo).max() <= 1e-8 * np.abs(geo).max()

    base_e = np.array([0.01, 0.0, 0.0])
    for i, j in [(int(np.argmax(np.abs(gv).sum(axis=1))), 0), (12345, 2)]:
        def f(h):
            v = model.v0.copy()
            v[i, j] += h
            return model.loss(v, base_e)
        for h in (1e-6, 1e-7, 1e-8):
            lp, lm = f(h), f(-h)
            dp, dm = (lp - loss) / h, (loss - lm) / h
            if abs(dp - dm) <= 1e-3 * max(abs(dp), abs(dm), 1e-12):
                break
        else:
            raise AssertionError("no jump-free step found")
        fd = (lp - lm) / (2 * h)
        assert abs(gv[i, j] - fd) <= 1e-5 * np.abs(gv).max() + 1e-4 * abs(fd), (i, j, gv[i, j], fd)


def test_adjoint_object_potential_gradient():
    """Probe mesh with its object held at a fixed potential V (the object
    bias): d loss / d V from the adjoint (sum over the steps of <phibar, L>,
    L the unit-potential Laplace solution) against jump-free central
    differences in V.  Slow particles away from the object and the box faces,
    so that none is absorbed during the K steps."""
    from helpers import uniform_points

    ma = meshgen.probe_box(8, 2.0, 0.6)
    mesh = punc.Mesh(ma)
    rng = np.random.default_rng(11)
    pts = uniform_points(ma, 4000, rng)
    r = np.linalg.norm(pts, axis=1)
    x = pts[(r > 0.9) & (np.abs(pts).max(axis=1) < 1.5)][:600]
    v0 = rng.normal(0.0, 0.02, size=x.shape)
    K, C, dt = 4, 2, 0.1
    target = rng.normal(0.0, 1.0, size=mesh.n_dofs) * 0.05
    state = {}

    def loss(V):
        if "pop" in state:
            state["pop"].close()
        pop = punc.Population(mesh, pcg_rtol=1e-13, pcg_atol=1e-30, pcg_max_iter=5000)
        state["pop"] = pop
        assert pop.add_particles(x, v0, -1.0 / len(x), 1.0 / len(x)) == len(x)
        return punc.adjoint_forward(pop, [punc.Object(2, potential=V)], dt, K, C, target, first_step=True)

    V0 = -0.5
    base = loss(V0)
    gv, ge, gx = punc.adjoint_backward(state["pop"], len(x))
    gpot = punc.adjoint_potential_gradient(state["pop"], 1)
    assert np.all(np.isfinite(gv)) and gpot.shape == (1,)
    for h in (1e-6, 1e-7, 1e-8):
        lp, lm = loss(V0 + h), loss(V0 - h)
        dp, dm = (lp - base) / h, (base - lm) / h
        if abs(dp - dm) <= 1e-3 * max(abs(dp), abs(dm), 1e-12):
            break
    else:
        raise AssertionError("no jump-free step found")
    fd = (lp - lm) / (2 * h)
    assert abs(gpot[0] - fd) <= 1e-4 * abs(fd) + 1e-9, (gpot[0], fd)
    state["pop"].close()
