"""Moving spheres (D3Q19): the CUDA particle path against the 3-D oracle.

The reference's particle code is 2-D only, so no reference-executed fixture
exists for spheres: the oracle's 3-D mode generalises the reference's case4
algorithm, and it is pinned through its 2-D parent (the 2-D mode reproduces
the reference's own statements bit for bit).  Both use the analytic
ray-sphere q (calQ2).  FP64: relative L2 <= 1e-10 on the fluid populations and
1e-9 on the particle state after 60 steps; FP32 storage/arithmetic: 1e-4."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu

CASE = dict(nx=40, ny=24, nz=22, radius=3.5, tauf=0.65, rho_solid=1.2, periodic_x=1,
            gravity=(0.0, 0.0, -2e-5), body_force=(1e-5, 0.0, 0.0), threshold_wall=2.0,
            threshold_particle=2.0, spring_scale_wall=1e-3, spring_scale_particle=1e-3)
CENTERS = [[9.3, 11.7, 10.9], [21.6, 12.4, 12.2], [33.2, 10.8, 11.5]]


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _gpu(mg, precision, centers=CENTERS, **over):
    kw = dict(CASE)
    kw.update(over)
    return mg.ParticleFlow(kw["nx"], kw["ny"], kw["nz"], centers, kw["radius"], tauf=kw["tauf"],
                           rho_solid=kw["rho_solid"], periodic_x=bool(kw["periodic_x"]),
                           gravity=kw["gravity"], body_force=kw["body_force"],
                           threshold_wall=kw["threshold_wall"],
                           threshold_particle=kw["threshold_particle"],
                           spring_scale_wall=kw["spring_scale_wall"],
                           spring_scale_particle=kw["spring_scale_particle"], precision=precision)


@pytest.fixture(scope="module")
def oracle60():
    o = O.ParticleOracle(np.array(CENTERS), dim=3, qmode=1, **CASE)
    assert o.step(60) == 0
    return o.get()


@pytest.mark.parametrize("prec,tf,tp", [("fp64", 1e-10, 1e-9), ("fp32", 1e-4, 1e-4)])
def test_particles_match_oracle(mg, oracle60, prec, tf, tp):
    with _gpu(mg, prec) as c:
        c.initial()
        c.step(60)
        st = c.state()
        mask = c.mask()
        f = c.get_f()
    o = oracle60
    fluid = o["obst"] == 0
    assert np.array_equal(mask < 0, fluid)
    assert rel_l2(f[fluid], o["f"][fluid]) <= tf
    assert rel_l2(st["xc"] - np.array(CENTERS), o["xc"] - np.array(CENTERS)) <= max(tp, 1e-9)
    for k_gpu, k_ora in (("uc", "uc"), ("omega", "om"), ("force", "force"), ("torque", "torque")):
        assert rel_l2(st[k_gpu], o[k_ora]) <= tp * 10, k_gpu
    # the body force drives the spheres downstream
    assert (st["uc"][:, 0] > 0).all()


# Two pairs of spheres whose surfaces are 1.2 and 2.3 lattice units apart: their
# boundary links have interpolation nodes inside the neighbouring sphere, so
# the linear and simple bounce-back fall-backs run (springs keep them apart).
THIN = [[9.0, 11.6, 10.7], [17.2, 12.1, 11.0], [27.3, 11.4, 10.8], [35.5, 12.6, 11.3]]


@pytest.mark.parametrize("prec,tf,tp", [("fp64", 1e-10, 1e-9), ("fp32", 1e-4, 1e-4)])
def test_thin_gaps_match_oracle(mg, prec, tf, tp):
    d = np.array(THIN)
    gaps = [np.linalg.norm(d[1] - d[0]) - 2 * CASE["radius"], np.linalg.norm(d[3] - d[2]) - 2 * CASE["radius"]]
    assert 1.0 < min(gaps) and max(gaps) < 2.5
    o = O.ParticleOracle(d, dim=3, qmode=1, **CASE)
    assert o.step(40) == 0
    r = o.get()
    with _gpu(mg, prec, centers=THIN) as c:
        c.initial()
        c.step(40)
        st = c.state()
        mask = c.mask()
        f = c.get_f()
    fluid = r["obst"] == 0
    assert np.array_equal(mask < 0, fluid)
    assert rel_l2(f[fluid], r["f"][fluid]) <= tf
    for k_gpu, k_ora in (("uc", "uc"), ("omega", "om"), ("force", "force"), ("torque", "torque")):
        assert rel_l2(st[k_gpu], r[k_ora]) <= tp * 10, k_gpu


def test_steps_are_deterministic(mg):
    out = []
    for _ in range(2):
        with _gpu(mg, "fp32", centers=THIN) as c:
            c.initial()
            c.step(25)
            out.append((c.get_f(), c.state()["torque"]))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_macro_marks_solid_nodes(mg):
    with _gpu(mg, "fp64") as c:
        c.initial()
        c.step(5)
        rho, u, v, w = c.macro()
        m = c.mask()
    assert np.all(rho[m >= 0] == CASE["rho_solid"]) and np.all(u[m >= 0] == 0.0)
    assert np.all(np.abs(rho[m < 0] - 1.0) < 1e-3)


def test_overlap_is_reported_not_faulted(mg):
    centers = [[10.0, 12.0, 11.0], [15.0, 12.0, 11.0]]  # 5 apart < 2R
    with _gpu(mg, "fp64", centers=centers) as c:
        c.initial()
        with pytest.raises(mg.MglcError) as ei:
            c.step(3)
        assert ei.value.code == 7 and "interpenetration" in str(ei.value)
        # the state froze at the failing step: later calls still work
        st = c.state()
        assert np.isfinite(st["xc"]).all()


def test_wall_penetration_is_reported(mg):
    centers = [[10.0, 4.2, 11.0]]  # y - R - 1 < 0
    with _gpu(mg, "fp64", centers=centers) as c:
        c.initial()
        with pytest.raises(mg.MglcError) as ei:
            c.step(2)
        assert ei.value.code == 7 and "wall" in str(ei.value)
