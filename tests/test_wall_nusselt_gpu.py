"""The wall Nusselt numbers of mglc_nusselt (no counterpart in the reference,
whose calNuRe has only the volume Nu) against closed-form limits.

* Conduction: a cavity heated from below and cooled from above below the
  onset of convection (Ra = 1000; the onset in a rigid cube lies above
  Rayleigh-Benard's 1708) settles to the linear profile T = T_hot - dT (z -
  1/2) / N with no flow, whose Nusselt number is 1 at both walls and in the
  volume.  The second-order wall gradient (9 T_1 - T_2 - 8 T_w) / 3 is exact
  for a linear profile; what remains is the anti-bounce-back wall's small
  offset (|Nu - 1| is about 1e-4 at 16 nodes).  The device's wall sums are
  also checked against the definition applied to the oracle's field.
* Energy balance: a side-heated cavity at steady state passes the same heat
  through the hot and the cold wall; the two wall estimates agree to the
  order of their second-order discretisation (h^2 = 1/N^2).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _wall_nusselt(T, t_hot, t_cold):
    """The wall Nusselt numbers of a z-heated field T[z, y, x], restated from
    their definition: -L/dT times the wall-averaged second-order gradient
    (9 T_1 - T_2 - 8 T_w) / 3 at the halfway walls."""
    n, dT = T.shape[0], t_hot - t_cold
    hot = -n / dT * (((9.0 * T[0] - T[1]).mean() - 8.0 * t_hot) / 3.0)
    cold = n / dT * (((9.0 * T[-1] - T[-2]).mean() - 8.0 * t_cold) / 3.0)
    return hot, cold


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fx64", 1e-9), ("fp32", 1e-4)])
def test_conduction_limit_wall_nusselt(mg, precision, tol):
    import os
    from oracle import oracle as O
    n, steps = 16, 30000  # more than 7 diffusion times L^2 / kappa
    with mg.BuoyancyCavity(n, rayleigh=1000.0, t_hot=0.5, t_cold=-0.5, bc_y_const_t=False,
                           bc_z_const_t=True, precision=precision) as c:
        c.initial()
        c.step(steps)
        nu_vol, _, nu_hot, nu_cold = c.nusselt()
        rho, u, v, w, T = c.macro()
    o = O.ThermalOracle(n, n, n, 1000.0, 0.71, 0.1, 0.0, 0.5, -0.5, 0.0, bc_y=0, bc_z=1)
    o.run(steps, nthreads=os.cpu_count() or 1)
    ref_hot, ref_cold = _wall_nusselt(o.T, 0.5, -0.5)
    # the device sums agree with the definition applied to the oracle's field
    assert abs(nu_hot - ref_hot) < tol and abs(nu_cold - ref_cold) < tol, (nu_hot, ref_hot)
    # the conduction limit: no convection (what moves is the forcing scheme's
    # wall current, far below the free-fall velocity sqrt(g beta N dT) ~ 0.06) ...
    assert max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max()) < 1e-4
    z = np.arange(1, n + 1) - 0.5
    assert np.abs(T - (0.5 - z / n)[:, None, None]).max() < 2e-3  # ... a linear profile ...
    for nu in (nu_hot, nu_cold, nu_vol):  # ... and Nusselt numbers of 1
        assert abs(nu - 1.0) < 2e-3, (nu_hot, nu_cold, nu_vol)


def test_side_heated_steady_state_balances_wall_fluxes(mg):
    n = 20
    with mg.BuoyancyCavity(n, rayleigh=1e4, t_hot=0.5, t_cold=-0.5) as c:
        c.initial()
        c.step(150000)
        eu, et = c.check()
        c.step(2000)
        eu, et = c.check()
        _, _, nu_hot, nu_cold = c.nusselt()
    assert eu < 1e-6 and et < 1e-6, (eu, et)  # steady
    assert nu_hot > 1.3  # convection raises the heat flux above conduction's
    assert abs(nu_hot - nu_cold) / nu_hot < 2.0 / n ** 2, (nu_hot, nu_cold)
