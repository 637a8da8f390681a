"""Adjoint of the DFSPH step on the GPU (dfsph_adjoint_*), FP64 and FP32.

Loss of the differentiable drop: L = mean_i |x_T,i - target_i|^2 with the target
the initial block shifted by (0.1, 0, 0) m (held fixed). Checks, on the
4913-particle puddle block with N(0, 0.1^2) initial velocities and fixed 2
divergence + 4 density iterations:
  * against the forward-mode (dual number) FP64 oracle: <grad, direction> for
    random directions in x0, v0 and the XSPH coefficient (exact derivatives of
    the same step; tolerance 1e-7 relative);
  * against central finite differences with eps = 1e-3 (20 steps; 1e-3 relative).
    Over longer horizons the reference's 27-cell stencil, which is narrower
    than the kernel support, makes the loss jump whenever a pair at distance
    between h and 2h crosses a cell face; a finite difference then measures the
    jumps as well, so the exact check above is the tight one;
  * the FP32 adjoint against the FP64 one (1e-4 relative);
  * checkpoint spacing does not change a single bit of the gradient;
  * the torch.autograd.Function wrapper returns the same gradients.
"""
import numpy as np
import pytest

from oracle import oracle as O
from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import solver_for

pytestmark = pytest.mark.gpu

SHIFT = np.array([0.1, 0.0, 0.0])


def _target(sc):
    return sc.fluid.astype(np.float64) + SHIFT


def _rollout(s, sc, x0, v0, steps, every=20):
    s.adjoint_set_state(x0, v0)
    s.adjoint_forward(sc.dt, steps, every)
    xT, _ = s.adjoint_state()
    d = xT.astype(np.float64) - _target(sc)
    return float((d * d).sum() / sc.n), xT, 2.0 * d / sc.n


def _gradients(sc, precision, steps, every=20):
    s = solver_for(sc, precision=precision)
    rd = s.real_dtype
    L, xT, xbar = _rollout(s, sc, sc.fluid.astype(rd), sc.velocity.astype(rd), steps, every)
    gx, gv, ge = s.adjoint_backward(xbar)
    return s, L, xT, gx, gv, ge


@pytest.fixture(scope="module")
def puddle40():
    return scenes.adjoint_puddle(steps=40)


@pytest.fixture(scope="module")
def fp64_grad(puddle40):
    return _gradients(puddle40, _lib.PRECISION_FP64, 40)


def test_adjoint_equals_forward_mode_oracle(puddle40, fp64_grad):
    sc = puddle40
    s, L, xT, gx, gv, ge = fp64_grad
    assert np.isfinite(gx).all() and np.isfinite(gv).all() and np.isfinite(ge)
    oc = O.config_from(sc.config(precision=_lib.PRECISION_FP64))
    rng = np.random.default_rng(17)
    dx = rng.standard_normal((sc.n, 3)) * 1e-2
    dv = rng.standard_normal((sc.n, 3))
    tgt = _target(sc)
    for kind, kw, adj in (("x0", {"dx": dx}, float((gx * dx).sum())),
                          ("v0", {"dv": dv}, float((gv * dv).sum())),
                          ("xsph", {"d_xsph": 1.0}, ge)):
        d = O.DualOracle(oc, sc.fluid, sc.velocity, sc.boundary, **kw)
        d.step(sc.dt, 40)
        x, _, tx, _ = d.state()
        if kind == "x0":
            # same trajectory as the GPU FP64 rollout
            assert np.abs(x - xT).max() < 1e-9
        jvp = float((2.0 * (x - tgt) / sc.n * tx).sum())
        assert abs(adj - jvp) <= 1e-7 * abs(jvp), (kind, adj, jvp)


def test_one_lane_reverse_passes_equal_forward_mode_oracle():
    # scenes of at most 4 x 128 particles per SM run the reverse neighbour
    # passes with two lanes per particle (the puddle above); this block is
    # just above that size, so they run one lane per particle
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    side = int(np.ceil((4 * 128 * sms + 1) ** (1 / 3)))
    sc = scenes.falling_block((side,) * 3, seed=41, radius=0.009, corner=(0.1, 0.1, 0.1), velocity_sigma=0.1)
    sc.max_divergence_iters = 2
    assert sc.n > 4 * 128 * sms
    steps = 5
    s, L, xT, gx, gv, ge = _gradients(sc, _lib.PRECISION_FP64, steps)
    oc = O.config_from(sc.config(precision=_lib.PRECISION_FP64))
    rng = np.random.default_rng(18)
    dx = rng.standard_normal((sc.n, 3)) * 1e-2
    dv = rng.standard_normal((sc.n, 3))
    tgt = _target(sc)
    for kind, kw, adj in (("x0", {"dx": dx}, float((gx * dx).sum())),
                          ("v0", {"dv": dv}, float((gv * dv).sum())),
                          ("xsph", {"d_xsph": 1.0}, ge)):
        d = O.DualOracle(oc, sc.fluid, sc.velocity, sc.boundary, **kw)
        d.step(sc.dt, steps)
        x, _, tx, _ = d.state()
        jvp = float((2.0 * (x - tgt) / sc.n * tx).sum())
        assert abs(adj - jvp) <= 1e-7 * abs(jvp), (kind, adj, jvp)


def test_central_differences_eps_1e3():
    sc = scenes.adjoint_puddle(steps=20)
    s, L, xT, gx, gv, ge = _gradients(sc, _lib.PRECISION_FP64, 20)
    x0 = sc.fluid.astype(np.float64)
    v0 = sc.velocity.astype(np.float64)
    h = 1e-3
    rng = np.random.default_rng(5)
    d = rng.standard_normal((sc.n, 3))
    fd = (_rollout(s, sc, x0, v0 + h * d, 20)[0] - _rollout(s, sc, x0, v0 - h * d, 20)[0]) / (2 * h)
    an = float((gv * d).sum())
    assert abs(fd - an) <= 1e-3 * abs(an), (fd, an)
    for i, a in ((0, 0), (2500, 1), (4000, 2)):
        vp, vm = v0.copy(), v0.copy()
        vp[i, a] += h
        vm[i, a] -= h
        fd = (_rollout(s, sc, x0, vp, 20)[0] - _rollout(s, sc, x0, vm, 20)[0]) / (2 * h)
        assert abs(fd - gv[i, a]) <= 1e-3 * abs(gv[i, a]), (i, a, fd, gv[i, a])
    e0 = np.float32(sc.viscosity)
    ep, em = np.float32(e0 + h), np.float32(e0 - h)
    s.set_xsph(float(ep))
    lp = _rollout(s, sc, x0, v0, 20)[0]
    s.set_xsph(float(em))
    lm = _rollout(s, sc, x0, v0, 20)[0]
    s.set_xsph(float(e0))
    fd = (lp - lm) / (float(ep) - float(em))
    assert abs(fd - ge) <= 1e-3 * abs(ge), (fd, ge)


def test_fp32_adjoint_against_fp64(puddle40, fp64_grad):
    _, L64, _, gx64, gv64, ge64 = fp64_grad
    _, L32, _, gx32, gv32, ge32 = _gradients(puddle40, _lib.PRECISION_FP32, 40)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)  # noqa: E731
    assert abs(L32 - L64) <= 1e-6 * L64
    assert rel(gv32, gv64) < 1e-4
    assert rel(gx32, gx64) < 1e-4
    assert abs(ge32 - ge64) < 1e-4 * abs(ge64)


def test_checkpoint_spacing_is_bit_invariant(puddle40, fp64_grad):
    sc = puddle40
    s, _, _, gx, gv, ge = fp64_grad
    for every in (1, 7, 40):
        _, _, xbar = _rollout(s, sc, sc.fluid.astype(np.float64), sc.velocity.astype(np.float64), 40, every)
        gx2, gv2, ge2 = s.adjoint_backward(xbar)
        assert np.array_equal(gx2, gx) and np.array_equal(gv2, gv) and ge2 == ge


def test_backward_leaves_final_state_and_repeats(puddle40):
    sc = puddle40
    s = solver_for(sc, precision=_lib.PRECISION_FP32)
    L, xT, xbar = _rollout(s, sc, sc.fluid, sc.velocity, 40)
    g1 = s.adjoint_backward(xbar)
    x_after, _ = s.adjoint_state()
    assert np.array_equal(x_after, xT)
    g2 = s.adjoint_backward(xbar)
    assert np.array_equal(g1[0], g2[0]) and np.array_equal(g1[1], g2[1]) and g1[2] == g2[2]


def test_torch_autograd_wrapper(puddle40):
    torch = pytest.importorskip("torch")
    from water_simulation_gb300.adjoint import drop_loss, rollout

    sc = puddle40
    s = solver_for(sc, precision=_lib.PRECISION_FP32)
    dev = torch.device("cuda:0")
    x0 = torch.tensor(sc.fluid, device=dev, requires_grad=True)
    v0 = torch.tensor(sc.velocity, device=dev, requires_grad=True)
    eps = torch.tensor(float(sc.viscosity), dtype=torch.float64, requires_grad=True)
    target = torch.tensor(sc.fluid, device=dev) + torch.tensor(SHIFT, dtype=torch.float32, device=dev)
    xT, vT = rollout(s, x0, v0, eps, sc.dt, 40, 20)
    loss = drop_loss(xT, target)
    loss.backward()
    # the same adjoint through the host API, fed with the loss gradient torch saw
    xbar = (2.0 * (xT - target) / sc.n).detach().cpu().numpy()
    s2 = solver_for(sc, precision=_lib.PRECISION_FP32)
    _, xT2, _ = _rollout(s2, sc, sc.fluid, sc.velocity, 40)
    gx, gv, ge = s2.adjoint_backward(xbar)
    assert np.array_equal(xT.detach().cpu().numpy(), xT2)
    close = lambda a, b: np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6 * np.abs(b).max())  # noqa: E731
    close(v0.grad.cpu().numpy(), gv)
    close(x0.grad.cpu().numpy(), gx)  # the target is a constant here
    assert abs(float(eps.grad) - ge) <= 1e-5 * abs(ge)


def test_adjoint_argument_and_state_errors(puddle40):
    sc = puddle40
    s = solver_for(sc, precision=_lib.PRECISION_FP32)
    with pytest.raises(_lib.DfsphError):
        s.adjoint_backward(np.zeros((sc.n, 3), np.float32))  # no recorded rollout
    adaptive = scenes.puddle()
    s2 = solver_for(adaptive)
    with pytest.raises(_lib.DfsphError):
        s2.adjoint_forward(adaptive.dt, 2, 1)  # adaptive iteration counts
    with pytest.raises(_lib.DfsphError):
        s.adjoint_forward(sc.dt, 0, 1)
