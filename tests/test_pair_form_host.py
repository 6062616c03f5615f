"""The pair form of the collision equals the reference's moment form.

The step kernels evaluate the lid-driven and heated-cavity collisions as a
two-relaxation-time update of opposite-direction pairs (trt_collide_lid,
trt_collide_forced, trt_collide_t in mglc_gb300/csrc/lbm_common.cuh).  This
is exact algebra, not an approximation, because the reference relaxes every
even non-conserved moment at Snu and every odd one at Sq
(mpi_3d_blocked/collision.f90:94-112, bouyancy3d_mpi.F90:723-741; D3Q7:
evolution_g.F90:1-57).  Here the reference's moment-space collision (its M,
meq with the lid's meq(12) quirk, its fSource, its s) is applied literally in
FP64 and compared with the pair-form formulas the kernels use, on random
states, to 1e-15: for the lid (absolute and scaled deviation storage), for the
forced heated cavity with the force carried from the previous step, for D3Q7,
and for the first step after initial or load, whose rho, u and T come from
macro arrays that need not agree with the populations."""
import numpy as np
import pytest

EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
EY = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]
E = np.array([EX, EY, EZ], float).T
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
PAIRS = [(1, 2), (3, 4), (5, 6), (7, 10), (9, 8), (11, 14), (13, 12), (15, 18), (17, 16)]


def moment_matrix():
    """The reference's D3Q19 basis (collision.f90:20-70), row by row."""
    e2 = (E ** 2).sum(1)
    x, y, z = E.T
    return np.array([np.ones(19), 19 * e2 - 30, (21 * e2 ** 2 - 53 * e2 + 24) / 2,
                     x, (5 * e2 - 9) * x, y, (5 * e2 - 9) * y, z, (5 * e2 - 9) * z,
                     3 * x ** 2 - e2, (3 * e2 - 5) * (3 * x ** 2 - e2),
                     y ** 2 - z ** 2, (3 * e2 - 5) * (y ** 2 - z ** 2),
                     x * y, y * z, x * z,
                     (y ** 2 - z ** 2) * x, (z ** 2 - x ** 2) * y, (x ** 2 - y ** 2) * z])


M = moment_matrix()


def rates(snu, sq):
    return np.array([0, snu, snu, 0, sq, 0, sq, 0, sq] + [snu] * 7 + [sq] * 3)


def meq(rho, u, lid):
    ux, uy, uz = u
    usq = u @ u
    p9, p11 = 2 * ux * ux - uy * uy - uz * uz, uy * uy - uz * uz
    return np.array([rho, rho * (-11 + 19 * usq), rho * (3 - 5.5 * usq),
                     rho * ux, -2 / 3 * rho * ux, rho * uy, -2 / 3 * rho * uy,
                     rho * uz, -2 / 3 * rho * uz, rho * p9, -0.5 * rho * p9, rho * p11,
                     -0.5 * p11 if lid else -0.5 * rho * p11,  # the lid's meq(12) quirk
                     rho * ux * uy, rho * uy * uz, rho * ux * uz, 0, 0, 0])


def fsource(u, F):
    ux, uy, uz = u
    fx, fy, fz = F
    uf = u @ F
    return np.array([0, 38 * uf, -11 * uf, fx, -2 / 3 * fx, fy, -2 / 3 * fy, fz, -2 / 3 * fz,
                     4 * ux * fx - 2 * uy * fy - 2 * uz * fz, -2 * ux * fx + uy * fy + uz * fz,
                     2 * uy * fy - 2 * uz * fz, -uy * fy + uz * fz, ux * fy + uy * fx,
                     uy * fz + uz * fy, ux * fz + uz * fx, 0, 0, 0])


def moment_form(f, rho, u, snu, sq, lid, F=None):
    """m_post = m - s (m - meq) + (1 - s/2) S, then f = M^-1 m_post."""
    m = M @ f
    s = rates(snu, sq)
    mp = m - s * (m - meq(rho, u, lid))
    if F is not None:
        mp = mp + (1 - s / 2) * fsource(u, F)
    return np.linalg.solve(M, mp)


def pair_update(f, snu, sq, e0, EO):
    out = f.copy()
    out[0] = f[0] - snu * (f[0] - e0)
    for (a, b), (Ea, Oa) in zip(PAIRS, EO):
        ne = f[a] + f[b] - Ea
        no = f[a] - f[b] - Oa
        out[a] = f[a] - sq / 2 * no - snu / 2 * ne
        out[b] = f[b] + sq / 2 * no - snu / 2 * ne
    return out


def pair_lid(f, rho_m, rhos, u, snu, sq, msc=1.0, dr=0.0, dj=(0.0, 0.0, 0.0)):
    """trt_collide_lid: E, O per pair from the polynomial equilibrium, the
    quirk's moment-12 term, and (first step) the conserved projections."""
    ux, uy, uz = u
    base = rho_m - 1.5 * rhos * (u @ u)
    q6 = (uy * uy - uz * uz) * (rhos - msc) / 12
    d19 = 2 * dr / 19
    EO = []
    for a, _ in PAIRS:
        e = E[a]
        eu = e @ u
        axis = abs(e).sum() == 1
        Ea = (base / 9 + rhos / 2 * eu * eu) if axis else (base / 18 + rhos / 4 * eu * eu)
        Ea += M[12][a] * q6 / 2 + d19  # M_12 = -2, +2, +1, -1, 0 by class
        Oa = (rhos / 3 if axis else rhos / 6) * eu + 0.2 * (e @ np.asarray(dj))
        EO.append((Ea, Oa))
    return pair_update(f, snu, sq, base / 3 + d19 / 2, EO)


def pair_forced(f, rho_m, rhos, u, F, dF, snu, sq, dr=0.0):
    """trt_collide_forced: the relaxed source folded into V and W; dF carries
    F - F_prev (or F + 2 (j - rho u) on the first step)."""
    le, lo = snu / 2, sq / 2
    V = rhos * u + (1 - le) / le * F
    Wv = rhos * u + (1 - lo) / (2 * lo) * F
    base = rho_m - 1.5 * (u @ V)
    d19 = 2 * dr / 19
    EO = []
    for a, _ in PAIRS:
        e = E[a]
        axis = abs(e).sum() == 1
        Ea = (base / 9 + 0.5 * (e @ u) * (e @ V)) if axis else (base / 18 + 0.25 * (e @ u) * (e @ V))
        Oa = e @ ((Wv / 3 if axis else Wv / 6) + dF / 10)
        EO.append((Ea + d19, Oa))
    return pair_update(f, snu, sq, base / 3 + d19 / 2, EO)


N7 = np.array([[1] * 7, [0, 1, -1, 0, 0, 0, 0], [0, 0, 0, 1, -1, 0, 0], [0, 0, 0, 0, 0, 1, -1],
               [-6, 1, 1, 1, 1, 1, 1], [0, 2, 2, -1, -1, -1, -1], [0, 0, 0, 1, 1, -1, -1]], float)


def moment_form_t(g, T, u, pa, qd, qnu):
    n = N7 @ g
    neq = np.array([T, T * u[0], T * u[1], T * u[2], T * pa, 0, 0])
    s = np.array([0, qd, qd, qd, qnu, qnu, qnu])
    return np.linalg.solve(N7, n - s * (n - neq))


def pair_t(g, T, u, pa, qd, qnu, dT=0.0):
    """trt_collide_t."""
    e0 = T * (1 - pa) / 7 + dT / 7
    Ep = T * (6 + pa) / 21 + 2 * dT / 7
    out = g.copy()
    out[0] = g[0] - qnu * (g[0] - e0)
    for (a, b), ua in zip(((1, 2), (3, 4), (5, 6)), u):
        ne, no = g[a] + g[b] - Ep, g[a] - g[b] - T * ua
        out[a] = g[a] - qd / 2 * no - qnu / 2 * ne
        out[b] = g[b] + qd / 2 * no - qnu / 2 * ne
    return out


def state(rng):
    rho = 1 + 0.02 * rng.standard_normal()
    u = 0.05 * rng.standard_normal(3)
    eu = E @ u
    f = W * rho * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * u @ u) + 1e-3 * W * rng.standard_normal(19)
    return f


def tau_rates(tau):
    return 1 / tau, 8 * (2 * tau - 1) / (8 * tau - 1)


@pytest.mark.parametrize("seed", range(4))
def test_lid_pair_form_equals_moment_form(seed):
    rng = np.random.default_rng(seed)
    snu, sq = tau_rates(0.5 + 3 * rng.random())
    f = state(rng)
    rho = f.sum()
    u = (E.T @ f) / rho
    ref = moment_form(f, rho, u, snu, sq, lid=True)
    assert np.abs(pair_lid(f, rho, rho, u, snu, sq) - ref).max() < 1e-15
    # deviation storage f - w rho0 scaled by 256 (the 16-bit forms' units)
    sc = 256.0
    fd = (f - W) * sc
    got = pair_lid(fd, fd.sum(), rho * sc, u, snu, sq, msc=sc) / sc + W
    assert np.abs(got - ref).max() < 1e-15


@pytest.mark.parametrize("seed", range(4))
def test_lid_first_step_with_macro_arrays(seed):
    """rho and u from the macro arrays (not the populations' sums): the
    moment form leaves sum f and sum f e alone; the pair form adds the
    projections back."""
    rng = np.random.default_rng(10 + seed)
    snu, sq = tau_rates(0.6 + rng.random())
    f = state(rng)
    rho_a = 1.0 + 0.01 * rng.standard_normal()
    u_a = (E.T @ f) / f.sum() + 0.01 * rng.standard_normal(3)
    ref = moment_form(f, rho_a, u_a, snu, sq, lid=True)
    got = pair_lid(f, rho_a, rho_a, u_a, snu, sq, dr=f.sum() - rho_a,
                   dj=E.T @ f - rho_a * u_a)
    assert np.abs(got - ref).max() < 1e-15
    assert abs(got.sum() - f.sum()) < 1e-15


@pytest.mark.parametrize("rot", [False, True])
@pytest.mark.parametrize("seed", range(3))
def test_forced_pair_form_with_carried_force(seed, rot):
    """u = (j + F_prev / 2) / rho, source from this step's F: the odd part
    keeps e.(F - F_prev)/10."""
    rng = np.random.default_rng(20 + seed)
    snu, sq = tau_rates(0.5 + rng.random())
    f = state(rng)
    Fp = 1e-3 * rng.standard_normal(3)
    F = Fp + 1e-4 * rng.standard_normal(3)
    if not rot:
        Fp[:2] = 0.0
        F[:2] = 0.0
    rho = f.sum()
    u = (E.T @ f + Fp / 2) / rho
    ref = moment_form(f, rho, u, snu, sq, lid=False, F=F)
    assert np.abs(pair_forced(f, rho, rho, u, F, F - Fp, snu, sq) - ref).max() < 1e-15
    sc = 256.0
    fd = (f - W) * sc
    got = pair_forced(fd, fd.sum(), rho * sc, u, F * sc, (F - Fp) * sc, snu, sq) / sc + W
    assert np.abs(got - ref).max() < 1e-15


def test_forced_first_step_with_macro_arrays():
    rng = np.random.default_rng(30)
    snu, sq = tau_rates(0.57)
    f = state(rng)
    rho_a = 1.0
    u_a = 0.05 * rng.standard_normal(3)
    F = 1e-3 * rng.standard_normal(3)
    ref = moment_form(f, rho_a, u_a, snu, sq, lid=False, F=F)
    dj = E.T @ f - rho_a * u_a
    got = pair_forced(f, rho_a, rho_a, u_a, F, F + 2 * dj, snu, sq, dr=f.sum() - rho_a)
    assert np.abs(got - ref).max() < 1e-15


@pytest.mark.parametrize("seed", range(3))
def test_d3q7_pair_form(seed):
    rng = np.random.default_rng(40 + seed)
    g = 0.1 + rng.random(7)
    u = 0.05 * rng.standard_normal(3)
    pa, qd, qnu = -0.3 + 0.2 * rng.random(), 0.5 + rng.random(), 0.5 + rng.random()
    T = g.sum()
    assert np.abs(pair_t(g, T, u, pa, qd, qnu) - moment_form_t(g, T, u, pa, qd, qnu)).max() < 1e-15
    Ta = T + 0.01  # first step: T from the macro array
    got = pair_t(g, Ta, u, pa, qd, qnu, dT=T - Ta)
    assert np.abs(got - moment_form_t(g, Ta, u, pa, qd, qnu)).max() < 1e-15
