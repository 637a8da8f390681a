"""The forward-mode (dual number) oracle that checks the GPU adjoint.

Solver<Dual> must take exactly the FP64 oracle's trajectory (its values are
computed by the same code) and its derivatives must match central finite
differences of the FP64 oracle where the loss is smooth (20 steps of the
4913-particle puddle block with N(0, 0.1^2) velocities).
"""
import numpy as np
import pytest

from oracle import oracle as O
from water_simulation_gb300 import scenes

STEPS = 20


@pytest.fixture(scope="module")
def case():
    sc = scenes.adjoint_puddle(steps=STEPS)
    oc = O.config_from(sc.config())
    tgt = sc.fluid.astype(np.float64) + np.array([0.1, 0.0, 0.0])
    return sc, oc, tgt


def _loss(x, tgt):
    d = x - tgt
    return float((d * d).sum() / x.shape[0])


def _oracle_loss(oc, sc, tgt, vel):
    o = O.Oracle(oc, sc.fluid, vel, sc.boundary, precision=64)
    o.step(sc.dt, STEPS)
    return _loss(o.field(O.F_POSITION), tgt)


def test_dual_values_are_the_fp64_trajectory(case):
    sc, oc, tgt = case
    d = O.DualOracle(oc, sc.fluid, sc.velocity, sc.boundary, dv=np.ones((sc.n, 3)))
    d.step(sc.dt, STEPS)
    x, v, _, _ = d.state()
    o = O.Oracle(oc, sc.fluid, sc.velocity, sc.boundary, precision=64)
    o.step(sc.dt, STEPS)
    assert np.array_equal(x, o.field(O.F_POSITION))
    assert np.array_equal(v, o.field(O.F_VELOCITY))


def test_dual_derivative_matches_central_differences(case):
    sc, oc, tgt = case
    for i, a in ((0, 0), (2500, 1)):
        e = np.zeros((sc.n, 3))
        e[i, a] = 1.0
        d = O.DualOracle(oc, sc.fluid, sc.velocity, sc.boundary, dv=e)
        d.step(sc.dt, STEPS)
        x, _, dx, _ = d.state()
        jvp = float((2.0 * (x - tgt) / sc.n * dx).sum())
        # the oracle takes float32 input: step by an exactly representable amount
        h = 2.0 ** -10
        vp, vm = sc.velocity.copy(), sc.velocity.copy()
        vp[i, a] += np.float32(h)
        vm[i, a] -= np.float32(h)
        hh = float(vp[i, a]) - float(vm[i, a])
        fd = (_oracle_loss(oc, sc, tgt, vp) - _oracle_loss(oc, sc, tgt, vm)) / hh
        assert abs(fd - jvp) <= 1e-4 * abs(jvp), (i, a, fd, jvp)


def test_dual_xsph_derivative_matches_central_differences(case):
    sc, oc, tgt = case
    d = O.DualOracle(oc, sc.fluid, sc.velocity, sc.boundary, d_xsph=1.0)
    d.step(sc.dt, STEPS)
    x, _, dx, _ = d.state()
    jvp = float((2.0 * (x - tgt) / sc.n * dx).sum())
    cfg = sc.config()
    ls, es = [], []
    for e in (np.float32(sc.viscosity + 1e-4), np.float32(sc.viscosity - 1e-4)):
        cfg.viscosity = float(e)
        ls.append(_oracle_loss(O.config_from(cfg), sc, tgt, sc.velocity))
        es.append(float(e))
    fd = (ls[0] - ls[1]) / (es[0] - es[1])
    assert abs(fd - jvp) <= 1e-5 * abs(jvp), (fd, jvp)
