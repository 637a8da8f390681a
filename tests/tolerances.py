"""Field tolerances shared by the parity tests.

The pressure fields of a Jacobi iteration (density_change_kernel,
solvers/dfsph/src/dfsph_kernels.cu:176-232):

    rho*  = rho + dt * rho_dot
    kappa = max(0, rho* - rho0) * alpha / dt^2

rho* is compared like the density, as an absolute error relative to rho0.
kappa is a difference of two numbers near rho0 scaled by alpha / dt^2, so its
error is rho*'s absolute error times alpha / dt^2, plus alpha's relative error
times kappa: the bound below is exactly that, per particle. It also covers the
max(0, .) clamp: a particle whose rho* lies within the tolerance of rho0 may be
clamped on one side only.
"""
from __future__ import annotations

import numpy as np

RHO0 = 1000.0


def pressure_field_errors(kappa, rho_adv, kappa_ref, rho_adv_ref, alpha_ref, dt, rho0=RHO0):
    """(max |d rho*| / rho0, max |d kappa| / (alpha / dt^2 * rho0) after the
    alpha term is taken out): the two numbers the tolerances apply to."""
    kappa = np.asarray(kappa, np.float64)
    kappa_ref = np.asarray(kappa_ref, np.float64)
    a = np.abs(np.asarray(alpha_ref, np.float64))
    e_adv = float(np.abs(np.asarray(rho_adv, np.float64) - np.asarray(rho_adv_ref, np.float64)).max()) / rho0
    scale = np.maximum(a / (dt * dt) * rho0, 1e-30)
    resid = np.maximum(np.abs(kappa - kappa_ref) - 1e-4 * np.abs(kappa_ref), 0.0)
    e_kap = float((resid / scale).max())
    return e_adv, e_kap


def assert_pressure_fields_close(kappa, rho_adv, kappa_ref, rho_adv_ref, alpha_ref, dt, rho_tol, ctx=""):
    """rho* within rho_tol * rho0 of the reference value; kappa within
    alpha / dt^2 * rho_tol * rho0 + 1e-4 |kappa| of it, per particle."""
    e_adv, e_kap = pressure_field_errors(kappa, rho_adv, kappa_ref, rho_adv_ref, alpha_ref, dt)
    assert e_adv < rho_tol, f"{ctx} rho*: max |d rho*| / rho0 = {e_adv:.3e} (tolerance {rho_tol:.1e})"
    assert e_kap < rho_tol, f"{ctx} kappa: error / (alpha rho0 / dt^2) = {e_kap:.3e} (tolerance {rho_tol:.1e})"
    return e_adv, e_kap
