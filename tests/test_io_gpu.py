"""Output, checkpoint/restart and statistics through a context on the GPU.

The reload test follows the reference's restart: backupData's records are read
back with rho = 1 (bouyancy3d.F90:289, 367-379) and the run continues from
them; the oracle is given the same arrays.  FP64 relative L2 <= 1e-10."""
import numpy as np
import pytest

from oracle import io_oracle as IO
from oracle import oracle as O
from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu
KW = dict(rayleigh=1e5, prandtl=0.71, mach=0.1, t_hot=0.5, t_cold=-0.5)


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def test_thermal_backup_reload_continues_like_the_reference(mg, tmp_path):
    nx, ny, nz = 12, 10, 11
    path = tmp_path / "backupFile-40.bin"
    with mg.BuoyancyCavity(nx, ny, nz, **KW) as c:
        c.initial()
        c.step(40)
        c.save_backup(path)
        rho40, u40, v40, w40, T40 = c.macro()
        f40, g40 = c.get_f()
    recs = IO.read_records(path.read_bytes())
    assert len(recs) == 6
    back = [np.frombuffer(r, "<f8") for r in recs]
    for got, ref in zip(back[:4], (u40, v40, w40, T40)):
        assert np.array_equal(got.reshape(ref.shape), ref)
    assert np.array_equal(back[4].reshape(f40.shape), f40)
    assert np.array_equal(back[5].reshape(g40.shape), g40)
    o = O.ThermalOracle(nx, ny, nz, KW["rayleigh"], KW["prandtl"], KW["mach"], 0.0, 0.5, -0.5, 0.0,
                        total_nz=nz)
    o.f[...] = f40
    o.g[...] = g40
    o.rho[...] = 1.0
    o.u[...], o.v[...], o.w[...], o.T[...] = u40, v40, w40, T40
    o.run(30)
    with mg.BuoyancyCavity(nx, ny, nz, **KW) as c:
        c.load_backup(path)
        c.step(30)
        f, g = c.get_f()
        r = c.macro()
    assert rel_l2(f, o.f) <= 1e-10 and rel_l2(g, o.g) <= 1e-10
    assert rel_l2(r[4], o.T) <= 1e-10 and rel_l2(r[1], o.u) <= 1e-10


def test_lid_backup_round_trip_and_outputs(mg, tmp_path):
    with mg.LidDrivenCavity(9, 8, 7, reynolds=200.0, u0=0.1) as c:
        c.initial()
        c.step(25)
        c.save_backup(tmp_path / "b.bin")
        c.write_tecplot(tmp_path / "MRTcavity-000000025.plt")
        c.write_binary(tmp_path / "MRTcavity-25.bin")
        c.write_profiles(tmp_path / "u-z_000000025.dat", tmp_path / "x-w_000000025.dat")
        rho, u, v, w = c.macro()
        f = c.get_f()
    assert (tmp_path / "MRTcavity-000000025.plt").read_bytes() == IO.tecplot_bytes(u, v, w, rho, 0)
    recs = IO.read_records((tmp_path / "MRTcavity-25.bin").read_bytes())
    for r, ref in zip(recs, (u, v, rho)):  # output_binary writes u, v, rho
        assert np.array_equal(np.frombuffer(r, "<f8").reshape(ref.shape), ref)
    uz, xw = IO.profiles(u, w, 0.1)
    assert np.array_equal(np.loadtxt(tmp_path / "u-z_000000025.dat"), np.array(uz))
    assert np.array_equal(np.loadtxt(tmp_path / "x-w_000000025.dat"), np.array(xw))
    with mg.LidDrivenCavity(9, 8, 7, reynolds=200.0, u0=0.1) as c:
        c.load_backup(tmp_path / "b.bin")
        assert np.array_equal(c.get_f(), f)
        c.step(5)
        assert np.isfinite(c.get_f()).all()


def test_backup_of_another_geometry_is_rejected(mg, tmp_path):
    with mg.LidDrivenCavity(8, reynolds=200.0) as c:
        c.initial()
        c.save_backup(tmp_path / "b8.bin")
    with mg.LidDrivenCavity(9, reynolds=200.0) as c:
        with pytest.raises(mg.MglcError):
            c.load_backup(tmp_path / "b8.bin")


def test_nure_samples_the_device_statistics(mg):
    with mg.BuoyancyCavity(16, **KW) as c:
        c.initial()
        m = mg.NuReMonitor()
        for _ in range(3):
            c.step(20)
            st = m.sample(c)
            nu, re, _, _ = c.nusselt()
            assert st.nu == nu and st.re == re
        assert st.time == 3 and st.stationary == 0
        m.close()
