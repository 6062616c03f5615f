"""Size-independent properties at the benchmark sizes (the oracle comparisons
at those sizes are in test_config_parity_gpu.py): the closed cavity conserves mass, the lid flow is
mirror-symmetric about y = ny/2, the 64-bit index path (19 * cells >= 2^31)
agrees with those properties, the heated cavity is centro-symmetric, and the
FP32 particle channel tracks the FP64 one at full size and runs its full
step count."""
import numpy as np
import pytest

from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _lid_props(mg, n, form, steps, sym_tol, mass_tol):
    with mg.LidDrivenCavity(n, reynolds=1000.0, u0=0.1, top_layer_u0=False, precision=form) as c:
        c.initial()
        c.step(1)
        m0, _, _ = c.totals()
        c.step(steps - 1)
        m1, e1, _ = c.totals()
        rho, u, v, w = c.macro()
    assert np.isfinite(u).all() and np.isfinite(rho).all()
    assert abs(m1 - m0) / m0 < mass_tol, (m0, m1)
    assert e1 > 0
    # mirror y -> ny-1-y: u, w even, v odd (arrays are [z, y, x])
    assert np.abs(u - u[:, ::-1, :]).max() <= sym_tol
    assert np.abs(w - w[:, ::-1, :]).max() <= sym_tol
    assert np.abs(v + v[:, ::-1, :]).max() <= sym_tol
    assert np.abs(u).max() > 0.05  # the lid drives the top layer


@pytest.mark.parametrize("form", ["fp64", "fx64"])
def test_lid_384_cubed_properties(mg, form):
    _lid_props(mg, 384, form, 100, 1e-13, 1e-12)


def test_lid_64bit_index_path_properties(mg):
    """484^3 cells: 19 * cells exceeds 2^31, so the kernels use 64-bit indices."""
    n = 484
    assert 19 * n ** 3 >= 2 ** 31
    _lid_props(mg, n, "fp16", 60, 2e-4, 1e-4)


def test_heated_cavity_128_cubed_is_centro_symmetric(mg):
    """Hot wall +0.5 at y = 0, cold wall -0.5 at y = ny-1, T_ref = 0, gravity
    along -z: the point reflection through the centre maps the solution to
    itself with T -> -T and u -> -u."""
    with mg.BuoyancyCavity(128, rayleigh=1e5, t_hot=0.5, t_cold=-0.5) as c:
        c.initial()
        c.step(400)
        rho, u, v, w, T = c.macro()
    r = lambda a: a[::-1, ::-1, ::-1]
    assert np.isfinite(T).all()
    assert np.abs(T + r(T)).max() <= 1e-10
    for a in (u, v, w):
        assert np.abs(a + r(a)).max() <= 1e-10
    assert np.abs(w).max() > 1e-4  # convection has started


def test_particle_channel_full_size_fp32_tracks_fp64(mg):
    import bench
    wl = bench.WORKLOADS["particles"]
    out = {}
    for form in ("fp64", "fp32"):
        with bench.make_solve(mg, wl, form) as s:
            s.initial()
            s.step(60)
            st = s.state()
            rho, u, v, w = s.macro()
            out[form] = (st, np.stack([u, v, w]), s.mask())
    st64, U64, m64 = out["fp64"]
    st32, U32, m32 = out["fp32"]
    assert np.isfinite(U32).all()
    assert (m64 == m32).mean() > 0.9999  # owner masks agree (nodes at the surface may differ)
    assert rel_l2(U32, U64) <= 1e-4
    assert rel_l2(st32["uc"], st64["uc"]) <= 1e-3
    assert np.abs(st32["xc"] - st64["xc"]).max() <= 1e-6


def test_particle_channel_fp32_runs_its_10000_steps(mg):
    """The channel's own step count in FP32 with no particle status: where a
    link's FP32 ray-sphere root is near a range end (q near 0 or 1) or the ray
    is nearly tangent, the link takes the FP64 root, so FP32 rounding cannot
    put q outside [0, 1] and stop the run (it did, once, before that rule)."""
    import bench
    wl = bench.WORKLOADS["particles"]
    with bench.make_solve(mg, wl, "fp32") as s:
        s.initial()
        for _ in range(wl["error_steps"] // 1000):
            s.step(1000)  # raises on a particle status
        u = s.macro()[1]
        xc = s.state()["xc"]
    assert np.isfinite(u).all() and np.isfinite(xc).all()
    assert 1e-3 < np.abs(u).max() < 0.1  # the body force drives a channel flow
