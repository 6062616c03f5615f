"""The FP32 particle form's link fraction q (k_plinks, mglc_gb300/csrc/k_particle.cu).

q is the smaller root of the ray-sphere equation along a boundary link
(calQ2, case4/mpi_particle/particle_bounceback.F90:144-185):
    q = (-cb - sqrt(cb^2 - 4 |e|^2 cc)) / (2 |e|^2),
    cb = 2 e.(x - X),  cc = |x - X|^2 - R^2 (computed in FP64).
The FP32 form evaluates the root in FP32 and keeps it only where
    delta > 1e-2 cb^2 + 1e-3   and   1e-3 < q < 1 - 1e-3;
every other link (a nearly tangent ray, or q near the range ends that the
range check tests) takes the FP64 root.  Here the kernel's FP32 arithmetic is
emulated with numpy float32 on about 700,000 boundary links of a sphere of
radius 5 at 400 random centres: every FP32 root kept lies inside [0, 1] and
within 2e-5 of the FP64 root, so the FP32 and FP64 forms accept and reject
the same links."""
import numpy as np

E = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1],
              [1, 0, -1], [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], float)


def boundary_links(rng, R=5.0):
    """Fluid nodes x (|x - X| > R) whose neighbour x + e is inside the sphere."""
    X = rng.uniform(10.0, 11.0, size=3)
    lo = np.floor(X - R - 2).astype(int)
    g = np.stack(np.meshgrid(*[np.arange(lo[k], lo[k] + int(2 * R) + 5) for k in range(3)],
                             indexing="ij"), -1).reshape(-1, 3).astype(float)
    out = []
    for e in E:
        o = g - X
        inside_next = ((o + e) ** 2).sum(1) < R * R
        fluid = (o ** 2).sum(1) >= R * R
        sel = fluid & inside_next
        out.append((o[sel], np.broadcast_to(e, (sel.sum(), 3))))
    o = np.concatenate([a for a, _ in out])
    e = np.concatenate([b for _, b in out])
    return o, e


def test_fp32_roots_kept_agree_with_fp64():
    rng = np.random.default_rng(7)
    R = 5.0
    kept = taken = 0
    worst = 0.0
    for _ in range(400):  # ~1800 links per random centre
        o, e = boundary_links(rng, R)
        s = (o * e).sum(1)  # e.(x - X)
        cc = (o ** 2).sum(1) - R * R
        m2 = (np.abs(e).sum(1) == 1)  # axis (|e|^2 = 1) or edge (2)
        e2 = np.where(m2, 1.0, 2.0)
        # FP64 root (the FP64 form and the fallback)
        cb = 2.0 * s
        q64 = (-cb - np.sqrt(cb * cb - 4.0 * e2 * cc)) / (2.0 * e2)
        assert (q64 >= 0.0).all() and (q64 <= 1.0).all()
        # FP32 root as the kernel forms it
        cbf = np.float32(2.0) * s.astype(np.float32)
        fourc = np.where(m2, np.float32(4.0), np.float32(8.0)).astype(np.float32)
        delta = cbf * cbf - fourc * cc.astype(np.float32)
        half = np.where(m2, np.float32(0.5), np.float32(0.25)).astype(np.float32)
        qf = (-cbf - np.sqrt(np.maximum(delta, np.float32(0.0)))) * half
        keep = (delta > np.float32(1e-2) * cbf * cbf + np.float32(1e-3)) & \
               (qf > np.float32(1e-3)) & (qf < np.float32(1.0 - 1e-3))
        assert ((qf[keep] > 0.0) & (qf[keep] < 1.0)).all()
        if keep.any():
            worst = max(worst, float(np.abs(qf[keep].astype(np.float64) - q64[keep]).max()))
        kept += int(keep.sum())
        taken += int((~keep).sum())
    assert worst < 2e-5, worst
    assert kept > 10 * taken  # the FP32 root serves most links
