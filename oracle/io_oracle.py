"""Oracle (test infrastructure only) for the host-side output, checkpoint and
statistics routines: a literal Python restatement of the reference's writers
and of calNuRe, used by the tests to check the library's C++ versions.

References (MGLC repository paths):
  output_Tecplot  MPI/Lid_driven_cavity/fortran/3d/mpi_3d_blocked/output.f90:175-296
                  (dumpstring :298-313); heated variant
                  MPI/Buoyancy_driven_cavity/fortran/3d/seq/bouyancy3d.F90:1034-1182
  getVelocity     output.f90:318-347
  backupData      bouyancy3d.F90:1011-1030, reload :367-379
  calNuRe         bouyancy3d.F90:1185-1321
Unformatted sequential records follow gfortran's documented layout (4-byte
length markers; subrecords of at most 2^31-9 bytes; a negative leading marker
announces a following subrecord, a negative trailing marker a preceding one).
"""
from __future__ import annotations

import struct

import numpy as np

MAX_SUBRECORD = 2 ** 31 - 9


# ----------------------------------------------------------------- Tecplot --
def tecplot_bytes(u, v, w, s, thermal):
    """The byte stream of output_Tecplot for fields shaped (nz, ny, nx)."""
    nz, ny, nx = u.shape
    out = bytearray()
    i4 = lambda x: out.extend(struct.pack("<i", x))
    r4 = lambda x: out.extend(struct.pack("<f", x))

    def dumpstring(t):  # output.f90:298-313
        for ch in t.rstrip():
            i4(ord(ch))
        i4(0)

    out.extend(b"#!TDV101")                     # :196
    i4(1)                                       # :199
    dumpstring("MyFirst")                       # :201-202
    i4(7)                                       # :205
    for name in ("X", "Y", "Z", "U", "V", "W", "T" if thermal else "Pressure"):
        dumpstring(name)                        # :208-221
    r4(299.0)                                   # :226 zone marker
    dumpstring("ZONE 001")                      # :229-230
    i4(-1)                                      # :233 zone colour
    i4(0)                                       # :236 zone type
    i4(1)                                       # :239 point packing
    i4(0)                                       # :243 var location
    i4(0)                                       # :247 face neighbours
    i4(nx); i4(ny); i4(nz)                      # :250-252
    i4(0)                                       # :256 no aux data
    r4(357.0)                                   # :257 end of header
    r4(299.0)                                   # :260
    for _ in range(7):
        i4(1)                                   # :263-269 float
    i4(0)                                       # :272 no sharing
    i4(-1)                                      # :276 no connectivity sharing
    x = np.arange(1, nx + 1) - 0.5              # initial.f90:18-21
    y = np.arange(1, ny + 1) - 0.5
    z = np.arange(1, nz + 1) - 0.5
    for k in range(nz):                         # :279-291
        for j in range(ny):
            for i in range(nx):
                last = s[k, j, i] if thermal else s[k, j, i] / 3.0
                for val in (x[i], y[j], z[k], u[k, j, i], v[k, j, i], w[k, j, i], last):
                    r4(np.float32(val))
    return bytes(out)


def profiles(u, w, u0):
    """getVelocity's two tables: (u(nxh,nyh,k)/U0, z_k/nz) and (x_i/nx, w(i,nyh,nzh)/U0)."""
    nz, ny, nx = u.shape
    ih, jh, kh = (nx - 1) // 2, (ny - 1) // 2, (nz - 1) // 2   # (n-1)/2+1, 0-based
    uz = [(u[k, jh, ih] / u0, (k + 1 - 0.5) / nz) for k in range(nz)]
    xw = [((i + 1 - 0.5) / nx, w[kh, jh, i] / u0) for i in range(nx)]
    return uz, xw


# ---------------------------------------------------- unformatted records --
def record_bytes(payload: bytes, max_sub=MAX_SUBRECORD) -> bytes:
    out = bytearray()
    pos, first = 0, True
    while True:
        n = min(max_sub, len(payload) - pos)
        more = len(payload) - pos > n
        out.extend(struct.pack("<i", -n if more else n))
        out.extend(payload[pos:pos + n])
        out.extend(struct.pack("<i", n if first else -n))
        pos += n
        first = False
        if not more:
            return bytes(out)


def read_records(data: bytes):
    """Split a file into logical records (subrecords joined)."""
    recs, pos = [], 0
    while pos < len(data):
        cur = bytearray()
        first = True
        while True:
            lead, = struct.unpack_from("<i", data, pos)
            n = abs(lead)
            cur.extend(data[pos + 4:pos + 4 + n])
            trail, = struct.unpack_from("<i", data, pos + 4 + n)
            assert abs(trail) == n and ((trail > 0) == first), "bad trailing marker"
            pos += n + 8
            first = False
            if lead >= 0:
                break
        recs.append(bytes(cur))
    return recs


def backup_bytes(u, v, w, T, f, g, max_sub=MAX_SUBRECORD):
    """backupData: u, v, w, T, f(0:18,i,j,k), g(0:6,i,j,k) -- f, g shaped
    (nz, ny, nx, Q), i.e. alpha fastest as in the Fortran array."""
    parts = [u, v, w] + ([T] if T is not None else []) + [f] + ([g] if g is not None else [])
    return b"".join(record_bytes(np.ascontiguousarray(a, dtype="<f8").tobytes(), max_sub)
                    for a in parts)


# ----------------------------------------------------------------- calNuRe --
class CalNuRe:
    """bouyancy3d.F90:1185-1321, one call per time unit."""

    def __init__(self, flow_reversal=0, flow_reversal_time=0):
        self.fr, self.frt = flow_reversal, flow_reversal_time
        self.nu, self.re = [0.0], [0.0]
        self.nu_mean, self.re_mean = [0.0], [0.0]
        self.stationary = 0
        self.stationary_time = 0
        self.converged = 0

    def push(self, nu, re):
        self.nu.append(nu)
        self.re.append(re)
        t = len(self.nu) - 1                                  # :1195
        s = 0.0
        for i in range(1, t + 1):                             # :1214-1216
            s = s + self.nu[i]
        self.nu_mean.append(s / float(t))
        s = 0.0
        for i in range(1, t + 1):                             # :1238-1241
            s = s + self.re[i]
        self.re_mean.append(s / float(t))
        if self.stationary == 1 and (t - self.stationary_time) % 200 == 0:   # :1244-1245
            t0 = self.stationary_time
            half = (t0 + t) // 2
            n1 = r1 = 0.0
            for i in range(t0, half + 1):
                n1 = n1 + self.nu[i]
                r1 = r1 + self.re[i]
            n1 = n1 / float(half - t0 + 1)
            r1 = r1 / float(half - t0 + 1)
            n2 = r2 = 0.0
            for i in range(half, t + 1):
                n2 = n2 + self.nu[i]
                r2 = r2 + self.re[i]
            n2 = n2 / float(t - half + 1)
            r2 = r2 / float(t - half + 1)
            if abs((n1 - n2) / n2) <= 0.01 and abs((r1 - r2) / r2) <= 0.01:   # :1267-1268
                if self.fr == 0:
                    self.converged = 1
                elif t >= t0 + self.frt:
                    self.converged = 1
        if self.stationary == 0 and t % 100 == 0:             # :1295-1297
            a = abs((self.nu_mean[t] - self.nu_mean[t - 100]) / self.nu_mean[t])
            b = abs((self.re_mean[t] - self.re_mean[t - 100]) / self.re_mean[t])
            if a <= 0.01 and b <= 0.01:
                self.stationary = 1
                self.stationary_time = t
        return dict(time=t, nu_mean=self.nu_mean[t], re_mean=self.re_mean[t],
                    stationary=self.stationary, stationary_time=self.stationary_time,
                    converged=self.converged)
