"""Physics checks of the boundary code against closed-form flows, on the
oracle (CPU) and on the GPU path (same cases, same tolerances; the FP64 GPU
path equals the oracle to 1e-10, so the analytic bar carries over):

* duct Poiseuille: the 3-D particle channel with no particles (periodic x,
  halfway bounce-back walls in y and z, body force along x through the forced
  MRT source) against the series solution for a rectangular duct; second-order
  accurate, ~1e-3 relative at 16-24 nodes across;
* Couette: the 2-D case1 shear channel with no circles (walls moving at
  -uwall and +uwall, periodic x) against the linear profile, which the lattice
  reproduces to round-off, in both the stationary and the moving frame."""
import numpy as np
import pytest

from oracle import oracle as O

DUCTS = [(1.0, 16, 16, 2000), (0.8, 16, 24, 4000)]  # tau, ny, nz, steps (~22 e-folds of the slowest mode)
COUETTES = [(1.0, 32, 20000, False), (0.7, 24, 30000, False), (1.0, 32, 20000, True)]
G = 1e-5  # body-force acceleration along x
DUCT_NX, DUCT_R = 8, 1.0  # the particle context needs nx >= 2 ceil(R) + 6 even without particles
UWALL, U0 = 0.05, 0.02


def duct_profile(ny, nz, g, nu, terms=201):
    """u(z, y) of fully developed flow in a duct |y| <= ny/2, |z| <= nz/2
    driven by the force density g (rho = 1): the classical cosine/cosh
    series; nodes j = 1..ny sit at y = j - (ny + 1)/2 (halfway walls)."""
    a, b = ny / 2.0, nz / 2.0
    y = np.arange(1, ny + 1) - (ny + 1) / 2.0
    z = np.arange(1, nz + 1) - (nz + 1) / 2.0
    Y, Z = np.meshgrid(y, z, indexing="xy")
    u = np.zeros_like(Y)
    for i in range(1, terms, 2):
        u += ((-1) ** ((i - 1) // 2) / i ** 3 * np.cos(i * np.pi * Y / (2 * a))
              * (1 - np.cosh(i * np.pi * Z / (2 * a)) / np.cosh(i * np.pi * b / (2 * a))))
    return 16 * a * a * g / (nu * np.pi ** 3) * u


def couette_profile(ny, moving_frame):
    y = np.arange(1, ny + 1) - (ny + 1) / 2.0
    return UWALL * y / (ny / 2.0) - (U0 if moving_frame else 0.0)


def check_duct(u_plane, tau, ny, nz):
    ua = duct_profile(ny, nz, G, (tau - 0.5) / 3.0)
    err = np.abs(u_plane - ua).max() / ua.max()
    assert err < 2e-3, err


def check_couette(u, ny, moving_frame):
    err = np.abs(u - couette_profile(ny, moving_frame)[:, None]).max() / UWALL
    assert err < 1e-10, err


@pytest.mark.parametrize("tau,ny,nz,steps", DUCTS)
def test_duct_poiseuille_oracle(tau, ny, nz, steps):
    O.build()
    o = O.ParticleOracle(np.zeros((0, 3)), dim=3, nx=DUCT_NX, ny=ny, nz=nz, periodic_x=1,
                         tauf=tau, radius=DUCT_R, body_force=(G, 0.0, 0.0))
    o.step(steps)
    check_duct(o.get()["u"][:, :, 1], tau, ny, nz)


@pytest.mark.parametrize("tau,ny,steps,moving_frame", COUETTES)
def test_couette_oracle(tau, ny, steps, moving_frame):
    O.build()
    o = O.ShearOracle(np.zeros((0, 2)), 8, ny, 5.0, tauf=tau, uwall=UWALL, u0=U0,
                      moving_frame=moving_frame)
    o.step(steps)
    check_couette(o.get()["u"], ny, moving_frame)


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


@pytest.mark.gpu
@pytest.mark.parametrize("tau,ny,nz,steps", DUCTS)
def test_duct_poiseuille_gpu(mg, tau, ny, nz, steps):
    # 20 nodes in x, like the particle channel the edge tests run without
    # particles (the profile does not depend on the periodic length)
    with mg.ParticleFlow(20, ny, nz, np.zeros((0, 3)), DUCT_R, tauf=tau, periodic_x=True,
                         body_force=(G, 0.0, 0.0), precision="fp64") as c:
        c.initial()
        c.step(steps)
        _, u, _, _ = c.macro()
    check_duct(u[:, :, 1], tau, ny, nz)


@pytest.mark.gpu
@pytest.mark.parametrize("tau,ny,steps,moving_frame", COUETTES)
def test_couette_gpu(mg, tau, ny, steps, moving_frame):
    with mg.ShearFlow2D(8, ny, np.zeros((0, 2)), 5.0, tauf=tau, uwall=UWALL, u0=U0,
                        moving_frame=moving_frame) as c:
        c.initial()
        c.step(steps)
        _, u, _ = c.macro()
    check_couette(u, ny, moving_frame)
