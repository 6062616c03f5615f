"""Benchmark of the MGLC lattice-Boltzmann step on GB300 (one JSON line).

Default workload: the large lid-driven cavity, D3Q19 MRT, 384^3 cells,
Re=1000, U=0.1, FP64 plain method (the drop-in).  A "step" is one fused time
step over the whole lattice.  ``value`` is MLUPS with the state resident in
HBM; ``e2e`` is the same metric through the C-ABI with host buffers (initial
state uploaded from pinned host memory, K steps, macroscopic fields read back)
inside the timed region.  The other forms (FX64: FP64 storage with the
fixed-point collision; FP32 / FP16 / BF16 deviations with FP32 arithmetic) are
timed on the same workload and reported under ``forms``.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mglc|reference]
                    [--workload lid384|lid64|thermal128|particles]
                    [--form fp64|fx64|fp32|fp16|bf16]

Multi-GPU: replicas only (one independent cavity per GPU, no inter-GPU
traffic); launched by torchrun, rank 0 prints max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS, %HBM roofline: mixed vs FP64 plain at ≤1e-3 err; serve p50/p99 ms"

WORKLOADS = {
    "lid384": dict(kind="lid", n=384, reynolds=1000.0, u0=0.1, error_steps=1000,
                   desc="lid-driven cavity D3Q19 MRT 384^3 Re=1000 U=0.1"),
    "lid64": dict(kind="lid", n=64, reynolds=400.0, u0=0.1, error_steps=2000,
                  desc="lid-driven cavity D3Q19 MRT 64^3 Re=400 U=0.1"),
    "thermal128": dict(kind="thermal", n=128, rayleigh=1e5, prandtl=0.71, mach=0.1, error_steps=20000,
                       desc="differentially heated cavity D3Q19+D3Q7 128^3 Ra=1e5 Pr=0.71"),
    "particles": dict(kind="particle", n=(256, 128, 128), np=200, radius=5.0, ratio=1.2,
                      body_force=1e-6, tauf=0.65, seed=2026, launches_per_step=11,
                      error_steps=10000,
                      data="synthetic (seeded sphere placement, fluid at rest, no dataset)",
                      desc="particle-laden channel D3Q19 256x128x128, 200 spheres R=5, "
                           "density ratio 1.2, body force 1e-6 along x, periodic x"),
}


def place_spheres(nx, ny, nz, npart, R, seed):
    """Seeded rejection sampling: centre gap >= 2R+2, wall gap >= R+2."""
    rng = np.random.default_rng(seed)
    out = []
    tries = 0
    while len(out) < npart:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place the spheres")
        c = np.array([rng.uniform(0.5, nx + 0.5), rng.uniform(R + 2 + 1, ny - R - 2),
                      rng.uniform(R + 2 + 1, nz - R - 2)])
        ok = True
        for o in out:
            d = c - o
            d[0] -= nx * np.round(d[0] / nx)
            if np.dot(d, d) < (2 * R + 2) ** 2:
                ok = False
                break
        if ok:
            out.append(c)
    return np.array(out)


def cells_of(wl):
    n = wl["n"]
    return n[0] * n[1] * n[2] if isinstance(n, tuple) else n ** 3


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    """Per-cell DRAM bytes of the step kernels from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return {}
    return {}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak():
    """Measured FP64 instruction rate of this GPU (the probe in
    mglc_gb300/roof/fp64_rate.cu): the best of DFMA, DADD and DMUL chains,
    instructions per second."""
    import ctypes
    from mglc_gb300 import build as B
    L = ctypes.CDLL(B.build_roof())
    L.mglc_roof_fp64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_double)]
    out = {}
    for mode, name in ((0, "dfma"), (1, "dadd"), (2, "dmul")):
        r, ms = ctypes.c_double(), ctypes.c_double()
        rc = L.mglc_roof_fp64(mode, 4096, ctypes.byref(r), ctypes.byref(ms))  # mode 0..2
        if rc != 0:
            raise RuntimeError(f"FP64 rate probe failed (CUDA error {rc})")
        out[name] = r.value
    return out


def load_fp64_instr():
    """FP64 instructions per cell-update of each FP64 step kernel, counted by
    ncu (profiles/fp64_instr.json)."""
    p = os.path.join(ROOT, "profiles", "fp64_instr.json")
    if not os.path.exists(p):
        return {}
    with open(p) as fh:
        return json.load(fh)


def fp64_roof(kind, form, mlups, probe):
    """The compute roof of an FP64 kernel: its FP64 instructions per cell
    (ncu count) times cells per second, against the measured FP64 rate."""
    tab = load_fp64_instr().get(f"{kind}_{form}")
    if not tab or not probe:
        return None
    ipc = tab["fp64_instr_per_cell"]
    peak = max(probe.values()) / 1e9
    ach = ipc * mlups * 1e6 / 1e9
    # the rate this kernel's own instruction mix allows: DADD and DMUL issue
    # at their measured rates, DFMA and the other FP64-pipe work at DFMA's
    other = ipc - tab["dadd"] - tab["dfma"] - tab["dmul"]
    ns_per_cell = (tab["dadd"] / probe["dadd"] + tab["dmul"] / probe["dmul"] +
                   (tab["dfma"] + other) / probe["dfma"]) * 1e9
    mix_mlups = 1e3 / ns_per_cell
    return {"fp64_achieved": round(ach, 1), "fp64_peak": round(peak, 1),
            "fp64_unit": "G FP64 instr/s", "fp64_frac": round(ach / peak, 4),
            "fp64_mix_roof_mlups": round(mix_mlups, 1),
            "fp64_mix_frac": round(mlups / mix_mlups, 4),
            "fp64_instr_per_cell": ipc, "fp64_peak_kind": "measured (mglc_gb300/roof/fp64_rate.cu, "
            "best of DFMA/DADD/DMUL chains, same run)", "fp64_instr_source": tab["source"],
            "fp64_probe_g_per_s": {k: round(v / 1e9, 1) for k, v in probe.items()}}


def make_solve(mg, wl, form, in_place=False):
    n = wl["n"]
    if wl["kind"] == "particle":
        nx, ny, nz = n
        cen = place_spheres(nx, ny, nz, wl["np"], wl["radius"], wl["seed"])
        return mg.ParticleFlow(nx, ny, nz, cen, wl["radius"], tauf=wl["tauf"],
                               rho_solid=wl["ratio"], periodic_x=True,
                               body_force=(wl["body_force"], 0.0, 0.0), threshold_wall=2.0,
                               threshold_particle=2.0, spring_scale_wall=1.0,
                               spring_scale_particle=1.0, precision=form)
    if wl["kind"] == "lid":
        return mg.LidDrivenCavity(n, reynolds=wl["reynolds"], u0=wl["u0"], top_layer_u0=False,
                                  precision=form, in_place=in_place)
    return mg.BuoyancyCavity(n, rayleigh=wl["rayleigh"], prandtl=wl["prandtl"], mach=wl["mach"],
                             t_hot=0.5, t_cold=-0.5, ekman=0.0, precision=form, in_place=in_place)


def alg_bytes(kind, form):
    """Algorithmic bytes per cell-update of a one-solve step kernel (what the
    context's mglc_get_info reports): every stored population read and
    written once, plus the owner mask (particles) or the temperature
    populations and the carried force (heated cavity, no rotation)."""
    pb = {"fp64": 8, "fx64": 8, "fp32": 4}.get(form, 2)
    if kind == "lid":
        return 2.0 * 19 * pb
    if kind == "particle":
        return 2.0 * 19 * pb + 4.0
    cb = 8.0 if form in ("fp64", "fx64") else 4.0
    return 2.0 * 19 * pb + 2.0 * 7 * cb + 2.0 * cb


def replica_command(n, argv, port):
    """torchrun command that runs this script as n replica ranks (one GPU
    each, rendezvous on 127.0.0.1)."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
            "--master-addr", "127.0.0.1", "--master-port", str(port),
            os.path.join(ROOT, "bench.py"), *argv]


def free_port():
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def world_check(gpus):
    """(spawn, error): spawn N replica ranks when --gpus N > 1 is given
    without a launcher; an error when a launcher's WORLD_SIZE differs from N."""
    env = os.environ.get("WORLD_SIZE")
    if env is not None:
        if int(env) != gpus:
            return False, (f"bench.py: WORLD_SIZE={env} but --gpus {gpus}; run one rank per GPU "
                           f"with --gpus equal to the world size")
        return False, None
    return gpus > 1, None


def l2_note(resident_bytes):
    """How the timed region treats L2: the ping-pong state (read + written
    each step) is the resident working set."""
    mb = resident_bytes / 1e6
    if mb > 129.0:
        return f"inputs larger than L2 ({mb:.0f} MB state > 129 MB L2), no flush"
    return f"state fits in L2 ({mb:.0f} MB): parity-size workload, not a headline number"


def max_over_ranks(torch, dist, x, device="cuda"):
    """The slowest rank's time (replicas: the job finishes with its last rank)."""
    if not dist:
        return x
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class CudaClock:
    """CUDA events recorded on the stream the kernels are launched on."""

    def __init__(self, torch, stream):
        self.torch, self.stream = torch, stream
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def sync(self):
        self.torch.cuda.synchronize()

    def start(self):
        self.e0.record(self.stream)

    def stop(self):
        self.e1.record(self.stream)

    def ms(self):
        return self.e0.elapsed_time(self.e1)


class HostClock:
    """Wall clock for a host-side run (the CPU test of the replica path)."""

    def sync(self):
        pass

    def start(self):
        self.t0 = time.perf_counter()

    def stop(self):
        self.t1 = time.perf_counter()

    def ms(self):
        return (self.t1 - self.t0) * 1e3


def timed_replica(torch, dist, run, steps, warmup, clock, device="cuda"):
    """One replica's timed region: `warmup` untimed steps, a barrier with the
    device synchronised on both sides, `steps` steps between the clock's
    marks; returns the slowest rank's milliseconds."""
    run(warmup)
    clock.sync()
    if dist:
        dist.barrier()
    clock.sync()
    clock.start()
    run(steps)
    clock.stop()
    clock.sync()
    return max_over_ranks(torch, dist, clock.ms(), device)


def replica_mlups(world, cells, steps, ms):
    """Whole-job throughput: every rank advanced its own `cells` cavity."""
    return world * cells * steps / (ms * 1e-3) / 1e6


def time_device(torch, mg, wl, form, steps, warmup, dist=None, in_place=False):
    """Device-resident MLUPS: state in HBM, K fused steps between CUDA events."""
    s = make_solve(mg, wl, form, in_place)
    # the context runs on a dedicated (non-default) stream; the CUDA events
    # are recorded on that same stream
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    s.initial()
    ms = timed_replica(torch, dist, s.step, steps, warmup, CudaClock(torch, stream))
    s.set_stream(None)
    info = s.info()
    s.close()
    return ms, info


def time_e2e(torch, mg, wl, form, steps, dist=None):
    """End to end through the C-ABI: pinned host state -> device, K steps,
    macroscopic fields -> pinned host, residual check."""
    s = make_solve(mg, wl, form)
    n = wl["n"]
    cells = cells_of(wl)
    q_g = 7 if wl["kind"] == "thermal" else 0
    if wl["kind"] == "particle":  # state upload is not part of the particle API: time steps + readback
        return time_e2e_particles(torch, s, wl, steps, dist)
    f_h = torch.empty((n, n, n, 19), dtype=torch.float64, pin_memory=True).numpy()
    g_h = torch.empty((n, n, n, 7), dtype=torch.float64, pin_memory=True).numpy() if q_g else None
    fields = [torch.empty((n, n, n), dtype=torch.float64, pin_memory=True).numpy()
              for _ in range(5 if q_g else 4)]
    s.initial()
    got = s.get_f()
    if q_g:
        f_h[...] = got[0]
        g_h[...] = got[1]
    else:
        f_h[...] = got
    del got
    import ctypes
    from mglc_gb300 import capi
    L = capi.lib()
    ptr = lambda a: None if a is None else a.ctypes.data
    # one untimed pass of the same calls (warm-up of the copy path and buffers)
    capi.check(s.handle, L.mglc_load_state(s.handle, ptr(f_h), ptr(g_h), None, None, None, None, None))
    capi.check(s.handle, L.mglc_step(s.handle, 1))
    capi.check(s.handle, L.mglc_get_macros(s.handle, *[ptr(a) for a in fields[:4]],
                                           ptr(fields[4]) if q_g else None))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    capi.check(s.handle, L.mglc_load_state(s.handle, ptr(f_h), ptr(g_h), None, None, None, None, None))
    torch.cuda.synchronize()  # phase mark only: the copies are asynchronous from pinned memory
    t_load = time.perf_counter()
    capi.check(s.handle, L.mglc_step(s.handle, steps))
    capi.check(s.handle, L.mglc_get_macros(s.handle, *[ptr(a) for a in fields[:4]],
                                           ptr(fields[4]) if q_g else None))
    eu = ctypes.c_double()
    capi.check(s.handle, L.mglc_check(s.handle, ctypes.byref(eu), None))
    t1 = time.perf_counter()
    dt = t1 - t0
    dt = max_over_ranks(torch, dist, dt)
    s.close()
    h2d = 8 * (19 + q_g) * cells
    d2h = 8 * len(fields) * cells + 8
    phases = {"load_state_s": round(t_load - t0, 4), "steps_and_readback_s": round(t1 - t_load, 4),
              "h2d_gbs": round(h2d / max(t_load - t0, 1e-9) / 1e9, 1)}
    return dt, h2d / steps, d2h / steps, float(eu.value), phases


def time_e2e_particles(torch, s, wl, steps, dist=None):
    import ctypes
    from mglc_gb300 import capi
    nx, ny, nz = wl["n"]
    cells = nx * ny * nz
    fields = [torch.empty((nz, ny, nx), dtype=torch.float64, pin_memory=True).numpy()
              for _ in range(4)]
    st = [np.zeros((wl["np"], 3)) for _ in range(5)]
    L = capi.lib()
    ptr = lambda a: a.ctypes.data
    s.initial()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    capi.check(s.handle, L.mglc_step(s.handle, steps))
    capi.check(s.handle, L.mglc_get_macros(s.handle, *[ptr(a) for a in fields], None))
    capi.check(s.handle, L.mglc_particle_state(s.handle, *[ptr(a) for a in st]))
    dt = max_over_ranks(torch, dist, time.perf_counter() - t0)
    s.close()
    return dt, 0, (8 * 4 * cells + 8 * 15 * wl["np"]) / steps, 0.0, {}


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def form_errors(mg, wl, forms, steps):
    """Velocity (and temperature, wall Nusselt) error of each form against
    the FP64 plain method on the workload's own grid, after `steps` steps
    from the same initial state."""
    def run(form):
        s = make_solve(mg, wl, form)
        s.initial()
        s.step(steps)
        r = s.macro()
        out = {"U": np.stack(r[1:4])}
        if wl["kind"] == "thermal":
            out["T"] = r[4]
            out["nu"] = s.nusselt()
        s.close()
        return out
    ref = run("fp64")
    res = {}
    for fm in forms:
        try:
            got = run(fm)
            e = {"u_rel_l2_vs_fp64": rel_l2(got["U"], ref["U"])}
            if wl["kind"] == "thermal":
                e["T_rel_l2_vs_fp64"] = rel_l2(got["T"], ref["T"])
                e["nu_hot_rel_vs_fp64"] = abs(got["nu"][2] - ref["nu"][2]) / abs(ref["nu"][2])
                e["nu_cold_rel_vs_fp64"] = abs(got["nu"][3] - ref["nu"][3]) / abs(ref["nu"][3])
                e["nu_hot_fp64"] = ref["nu"][2]
                e["nu_cold_fp64"] = ref["nu"][3]
            res[fm] = e
        except Exception as ex:  # report, never hide
            res[fm] = {"error_run_failed": str(ex)}
    return res


def particle_errors(mg, wl, steps):
    """FP32 particle channel against FP64 after `steps` steps from the same
    initial state: fluid velocity, particle displacement, force and torque."""
    def run(form):
        s = make_solve(mg, wl, form)
        s.initial()
        s.step(steps)
        r = s.macro()
        st = s.state()
        m = s.mask()
        s.close()
        return np.stack(r[1:4]), st, m
    u64, st64, m64 = run("fp64")
    u32, st32, m32 = run("fp32")
    x0 = place_spheres(*wl["n"], wl["np"], wl["radius"], wl["seed"])
    fluid = (m64 < 0) & (m32 < 0)
    R = wl["radius"]
    f_rms = float(np.sqrt((st64["force"] ** 2).sum(axis=1).mean()))
    return {"error_steps": steps,
            "u_rel_l2_vs_fp64": rel_l2(u32[:, fluid], u64[:, fluid]),
            "displacement_rel_l2_vs_fp64": rel_l2(st32["xc"] - x0, st64["xc"] - x0),
            "force_rel_l2_vs_fp64": rel_l2(st32["force"], st64["force"]),
            "torque_rel_l2_vs_fp64": rel_l2(st32["torque"], st64["torque"]),
            # the torques nearly cancel (rms far below force x radius), so their
            # relative error is large; against the natural scale |F| R it is small
            "force_rms_fp64": f_rms,
            "torque_rms_fp64": float(np.sqrt((st64["torque"] ** 2).sum(axis=1).mean())),
            "torque_err_rms_over_force_rms_x_radius":
                float(np.sqrt(((st32["torque"] - st64["torque"]) ** 2).sum(axis=1).mean())) /
                (f_rms * R),
            "mask_nodes_differing": int((m64 != m32).sum())}


# the forms timed for each side workload (the first is the workload's own)
SIDE_FORMS = {"thermal128": ("fp64", "fx64", "fp32", "fp16", "fp16s", "fp16_in_place",
                             "fp16s_in_place", "fp32_in_place"),
              "particles": ("fp32", "fp64")}
# Algorithmic bytes per cell of an alternative layout of the same form (a
# carried 3-vector, and 16-bit g for the 16-bit heated cavity; a one-byte mask
# for the channel), reported beside what the kernels here move
SIDE_SPEC_BYTES = {"thermal128": {"fp64": 464, "fp16s": 128}, "particles": {"fp32": 153}}


def side_workload(torch, mg, key, steps, warmup, peak, probe, cpu=True, errors=True):
    """A workload of its own beside the headline one: device MLUPS of each
    form (CUDA events on the context's stream), HBM (and, for FP64, FP64-pipe)
    roofline, error of the reduced forms against FP64 after the workload's
    own step count, and the oracle on the host cores on a bounded sample."""
    wl = dict(WORKLOADS[key])
    cells = cells_of(wl)
    kind = wl["kind"]
    forms = SIDE_FORMS[key]
    out = {"workload": wl["desc"], "cells": cells, "unit": "MLUPS", "steps": steps,
           "warmup": warmup, "l2": l2_note(cells * alg_bytes(kind, forms[0])), "forms": {}}
    traffic_tab = load_traffic()
    for fm in forms:
        try:
            ip = fm.endswith("_in_place")
            ms, info = time_device(torch, mg, wl, fm[:-len("_in_place")] if ip else fm, steps,
                                   warmup, in_place=ip)
            v = cells * steps / (ms * 1e-3) / 1e6
            bpc = info.bytes_per_cell_step
            ach = bpc * cells / (ms / steps * 1e-3) / 1e9
            ent = {"value": round(v, 3), "ms_per_step": round(ms / steps, 4),
                   "bytes_per_cell": bpc, "achieved_gbs": round(ach, 1),
                   "frac": round(ach / peak, 4)}
            if fm in SIDE_SPEC_BYTES.get(key, {}):
                ent["alt_layout_bytes_per_cell"] = SIDE_SPEC_BYTES[key][fm]
            if fm == "fp64":
                fr = fp64_roof(kind, fm, v, probe)
                if fr:
                    ent.update(fr)
            tk = f"{kind}_{fm}"
            if tk in traffic_tab:
                ent["traffic_bytes_per_cell"] = traffic_tab[tk]["dram_bytes_per_cell"]
                ent["traffic_source"] = traffic_tab[tk]["source"]
            out["forms"][fm] = ent
        except Exception as e:  # report, never hide
            out["forms"][fm] = {"error": str(e)}
    head = out["forms"].get(forms[0], {})
    if "value" in head:
        out.update(form=forms[0], value=head["value"], ms_per_step=head["ms_per_step"],
                   gpu_launches=steps * wl.get("launches_per_step", 1))
        rf = {"bound": "fp64" if "fp64_frac" in head else "hbm", "achieved": head["achieved_gbs"],
              "peak": peak, "unit": "GB/s", "frac": head["frac"],
              "bytes_per_cell": head["bytes_per_cell"],
              "kernel": "particle step (k_pbulk + 10 small kernels)" if kind == "particle"
              else f"k_thermal_step<{forms[0]}>"}
        for k in ("fp64_achieved", "fp64_peak", "fp64_unit", "fp64_frac", "fp64_mix_roof_mlups",
                  "fp64_mix_frac", "fp64_instr_per_cell", "alt_layout_bytes_per_cell"):
            if k in head:
                rf[k] = head[k]
        out["roofline"] = rf
    if errors:
        try:
            if kind == "thermal":
                es = wl["error_steps"]
                errs = form_errors(mg, wl, [f for f in forms if f != "fp64" and
                                            not f.endswith("_in_place")], es)
                for fm, e in errs.items():
                    out["forms"].setdefault(fm, {}).update(e)
                    out["forms"][fm]["error_steps"] = es
                    if "u_rel_l2_vs_fp64" in e:
                        out["forms"][fm]["within_1e-3"] = e["u_rel_l2_vs_fp64"] <= 1e-3
            else:
                out["forms"]["fp32"].update(particle_errors(mg, wl, wl["error_steps"]))
        except Exception as e:  # report, never hide
            out["error_runs_failed"] = str(e)
    if kind == "thermal":
        mx = out["forms"].get("fp16s", {})
        base = out["forms"].get("fp64", {}).get("value")
        if "value" in mx and base:
            out["mixed"] = {"form": "fp16 storage of f - w rho0 (stochastic rounding), fp32 "
                                    "arithmetic, fp32 g",
                            "value": mx["value"], "frac": mx["frac"],
                            "speedup_vs_fp64_plain": round(mx["value"] / base, 2),
                            **{k: mx.get(k) for k in ("u_rel_l2_vs_fp64", "T_rel_l2_vs_fp64",
                                                      "nu_hot_rel_vs_fp64", "nu_cold_rel_vs_fp64",
                                                      "error_steps")}}
    if cpu:
        out["cpu_baseline"] = cpu_sample(wl)
    return out


def serve_bench(torch, mg, n_req=24, rate=50.0, seed=1234, max_steps=50000, tol=1e-6, K=100,
                precision="fp32", sample_steps=400, full_serial_budget_s=120.0):
    """Batched serving stream: Poisson arrivals of lid-driven and heated-cavity
    solves (grids from {32,48,64,96,128}, Re ~ U[100,1000] or Ra log-uniform in
    [1e3,1e5]), each run to max|du|/U < tol (checked every K steps) or
    max_steps, through the solve server (FP32 deviation storage by default:
    the 16-bit states keep moving at the 1e-6 level, so they would never
    retire on convergence).

    Serial baselines run the same requests one after another through the
    one-solve contexts: with the server's own storage form, each request for
    its full served step count (sampled over `sample_steps` steps and scaled
    only if the whole serial run would exceed `full_serial_budget_s`), and
    with the FP64 plain context, each request sampled over `sample_steps`
    steps after a warm-up and scaled to its served step count."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    arrivals -= arrivals[0]
    sizes = rng.choice([32, 48, 64, 96, 128], n_req)
    lid = rng.random(n_req) < 0.5
    re = rng.uniform(100.0, 1000.0, n_req)
    ra = 10.0 ** rng.uniform(3.0, 5.0, n_req)
    with mg.SolveServer(hbm_budget_gb=32.0, max_active=64, precision=precision,
                        steps_per_iteration=K, tol=tol, max_steps=max_steps, autotune=True,
                        keep_results=False) as srv:
        ids = [srv.submit("lid" if lid[q] else "thermal", int(sizes[q]), reynolds=float(re[q]),
                          rayleigh=float(ra[q]), arrival_s=float(arrivals[q])) for q in range(n_req)]
        srv.run()
        res = {r["id"]: r for r in srv.results()}
        st = srv.stats()
    lat = np.array([(res[i]["finish_s"] - res[i]["arrival_s"]) * 1e3 for i in ids])
    conv = np.array([bool(res[i]["converged"]) for i in ids])
    span = max(r["finish_s"] for r in res.values()) - float(arrivals[0])
    cells_done = st["cell_updates"]

    def one(q, form):
        n = int(sizes[q])
        return (mg.LidDrivenCavity(n, reynolds=float(re[q]), u0=0.1, top_layer_u0=False,
                                   precision=form) if lid[q] else
                mg.BuoyancyCavity(n, rayleigh=float(ra[q]), t_hot=0.5, t_cold=-0.5, precision=form))

    def serial(form, sample):
        """Seconds for the requests one at a time; sample=None runs each for
        its full served step count."""
        tot = 0.0
        for q, i in enumerate(ids):
            steps = int(res[i]["steps"])
            with one(q, form) as c:
                c.initial()
                m = steps if sample is None else min(steps, sample)
                if sample is not None:
                    c.step(4)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                c.step(m)
                torch.cuda.synchronize()
                tot += (time.perf_counter() - t0) * steps / m
        return tot

    agg = cells_done / span / 1e6
    t_same_est = serial(precision, sample_steps)
    same_full = t_same_est <= full_serial_budget_s
    t_same = serial(precision, None) if same_full else t_same_est
    t_plain = serial("fp64", sample_steps)
    lat_c = lat[conv]
    return {"requests": n_req, "rate_per_s": rate, "seed": seed, "max_steps": max_steps,
            "tol": tol, "steps_per_iteration": K, "precision": precision,
            "steps_mean": round(float(np.mean([res[i]["steps"] for i in ids])), 1),
            "converged": int(conv.sum()), "at_step_cap": int((~conv).sum()),
            "p50_ms": round(float(np.percentile(lat, 50)), 2),
            "p99_ms": round(float(np.percentile(lat, 99)), 2),
            "p50_ms_converged": round(float(np.percentile(lat_c, 50)), 2) if lat_c.size else None,
            "p99_ms_converged": round(float(np.percentile(lat_c, 99)), 2) if lat_c.size else None,
            "aggregate_mlups": round(agg, 1),
            "busy_mlups": round(cells_done / st["busy_s"] / 1e6, 1),
            "serial_same_form_mlups": round(cells_done / t_same / 1e6, 1),
            "serial_same_form_timing": "full served step counts" if same_full else
            f"{sample_steps}-step samples scaled to the served step counts",
            "speedup_vs_serial_same_form": round(agg / (cells_done / t_same / 1e6), 2),
            "serial_plain_fp64_mlups": round(cells_done / t_plain / 1e6, 1),
            "serial_plain_timing": f"{sample_steps}-step samples scaled to the served step counts",
            "speedup_vs_serial_plain": round(agg / (cells_done / t_plain / 1e6), 2),
            "per_request": [{"kind": "lid" if lid[q] else "heated", "n": int(sizes[q]),
                             "re_or_ra": round(float(re[q] if lid[q] else ra[q]), 1),
                             "steps": int(res[i]["steps"]), "converged": bool(conv[q]),
                             "latency_ms": round(float(lat[q]), 1)} for q, i in enumerate(ids)],
            "peak_active": st["peak_active"], "peak_device_bytes": st["peak_device_bytes"],
            "tile": {"threads": st["tile_threads"], "rows": st["tile_rows"],
                     "ctas_per_sm": st["ctas_per_sm"]}}


def lid2d_bench(torch, mg, n=1024, steps=400, warmup=20, cpu_s=3.0, cpu=True):
    """The D2Q9 lid cavity (the reference's 2-D code; FP64, bitwise the
    reference's statements) at n^2: device MLUPS between CUDA events on the
    context's stream, and the oracle on all host cores for a bounded sample.
    The kernel is bound by the FP64 pipe, not by HBM (144 B per node)."""
    c = mg.LidDrivenCavity2D(n, reynolds=1000.0, u0=0.1)
    stream = torch.cuda.Stream()
    c.set_stream(stream.cuda_stream)
    c.initial()
    c.step(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    c.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    c.set_stream(None)
    c.close()
    v = n * n * steps / (ms * 1e-3) / 1e6
    out = {"workload": f"D2Q9 MRT lid cavity {n}^2, Re=1000 (2d_revised/mpi_blocked), FP64 bitwise",
           "value": round(v, 1), "unit": "MLUPS", "steps": steps,
           "ms_per_step": round(ms / steps, 4), "bound": "fp64 pipe",
           "hbm_gbs": round(144.0 * n * n / (ms / steps * 1e-3) / 1e9, 1),
           "gpu_launches": steps}
    if not cpu:
        return out
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    o = O.Lid2DOracle(n, n, 1000.0, 0.1)
    t0, k = time.perf_counter(), 0
    while time.perf_counter() - t0 < cpu_s:
        o.run(2, nthreads=threads)
        k += 2
    cv = n * n * k / (time.perf_counter() - t0) / 1e6
    out["cpu_baseline"] = {"value": round(cv, 1), "unit": "MLUPS", "cores": threads, "kind": "port",
                           "sample": f"{k} steps of the same {n}^2 cavity (oracle, OpenMP)"}
    return out


def particles2d_bench(torch, mg, steps=200, warmup=10, cpu_steps=20, cpu=True):
    """The D2Q9 moving-particle steps of the reference's 2-D programs (FP64,
    bitwise the reference's statements): case4's three settling circles at
    400x800 and case1's circle in a sheared channel at 800x400.  Device ms per
    step between CUDA events on the context's stream; the oracle (single
    thread, like the reference's sequential build) on a bounded sample."""
    cen = [[100.3, 600.7], [200.9, 650.2], [300.1, 610.4]]
    cases = (("circles2d", "case4: 3 settling circles, 400x800, R=10, FP64 bitwise",
              lambda: mg.ParticleFlow2D(400, 800, cen, 10.0, tauf=0.7, gravity=0.01)),
             ("shear2d", "case1: 1 circle in a sheared channel, 800x400, R=12.6, FP64 bitwise",
              lambda: mg.ShearFlow2D(800, 400, [[200.4, 201.3]], 12.6)))
    out = {}
    for key, desc, make in cases:
        c = make()
        stream = torch.cuda.Stream()
        c.set_stream(stream.cuda_stream)
        c.initial()
        c.step(warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        c.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        dev = c.info().device_bytes
        c.set_stream(None)
        c.close()
        out[key] = {"workload": desc, "value": round(320000 * steps / (ms * 1e-3) / 1e6, 1),
                    "unit": "MLUPS", "steps": steps, "ms_per_step": round(ms / steps, 4),
                    "l2": f"device state {dev / 1e6:.0f} MB, of which populations "
                          f"{144 * 320000 / 1e6:.0f} MB, against the 129 MB L2: the "
                          "reference's own grid size, no flush between steps"}
    if cpu:
        import numpy as np
        from oracle import oracle as O
        o = O.ParticleOracle(np.array([[x, y, 0.0] for x, y in cen]), dim=2, nx=400, ny=800, nz=1,
                             tauf=0.7, rho_solid=1.01, radius=10.0, gravity=(0.0, -0.01, 0.0),
                             qmode=0)
        t0 = time.perf_counter()
        o.step(cpu_steps)
        dt = time.perf_counter() - t0
        out["circles2d"]["cpu_baseline"] = {
            "value": round(320000 * cpu_steps / dt / 1e6, 2), "unit": "MLUPS", "cores": 1,
            "kind": "port", "ms_per_step": round(dt / cpu_steps * 1e3, 3),
            "sample": f"{cpu_steps} steps of the same case (oracle, one thread)"}
    return out


def kernel_tour(torch, mg, steps=3):
    """One small run of every step-kernel family (profiling runs: a launch list
    of this covers all of them): lid and heated cavities in every form with two
    buffers and in place, spheres, the 2-D cases and the server.  Sizes keep
    each state above or near the 129 MB L2 while the whole tour holds a few GB."""
    jobs = []
    for form in ("fp64", "fx64", "fp32", "fp16", "fp16s", "bf16"):
        for ip in (False, True):
            jobs.append(("lid", form, ip, lambda f=form, i=ip: mg.LidDrivenCavity(
                160, reynolds=1000.0, u0=0.1, top_layer_u0=False, precision=f, in_place=i)))
    for form in ("fp64", "fx64", "fp32", "fp16", "fp16s"):
        for ip in (False, True):
            jobs.append(("heated", form, ip, lambda f=form, i=ip: mg.BuoyancyCavity(
                128, rayleigh=1e5, t_hot=0.5, t_cold=-0.5, precision=f, in_place=i)))
    cen = place_spheres(256, 128, 128, 200, 5.0, 2026)
    for form in ("fp64", "fp32"):
        jobs.append(("spheres", form, False, lambda f=form: mg.ParticleFlow(
            256, 128, 128, cen, 5.0, tauf=0.65, rho_solid=1.2, periodic_x=True,
            body_force=(1e-6, 0.0, 0.0), precision=f)))
    jobs.append(("circles2d", "fp64", False, lambda: mg.ParticleFlow2D(
        400, 800, [[100.3, 600.7], [200.9, 650.2], [300.1, 610.4]], 10.0, tauf=0.7, gravity=0.01)))
    jobs.append(("shear2d", "fp64", False, lambda: mg.ShearFlow2D(
        800, 400, [[200.4, 201.3]], 12.6)))
    jobs.append(("lid2d", "fp64", False, lambda: mg.LidDrivenCavity2D(1024, reynolds=1000.0)))
    done = []
    for kind, form, ip, make in jobs:
        with make() as c:
            c.initial()
            c.step(steps)
            c.macro()
        torch.cuda.synchronize()
        done.append(f"{kind}:{form}{':in_place' if ip else ''}")
    with mg.SolveServer(hbm_budget_gb=2.0, max_active=8, precision="fp16", steps_per_iteration=4,
                        tol=1e-12, max_steps=8, autotune=False) as srv:
        srv.submit("lid", 64, reynolds=400.0)
        srv.submit("thermal", 48, rayleigh=1e4)
        srv.run()
    done.append("serve:fp16")
    return done


def cpu_sample(wl, target_s=10.0):
    """The oracle (restatement of the reference's CPU code) with OpenMP on all
    host cores, on a bounded sample of the workload."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    n = wl["n"]
    if wl["kind"] == "particle":
        # the particle oracle is single-threaded: time a 64x32x32 slice with 6 spheres
        nx, ny, nz = 64, 32, 32
        cen = place_spheres(nx, ny, nz, 6, wl["radius"], wl["seed"])
        o = O.ParticleOracle(cen, dim=3, nx=nx, ny=ny, nz=nz, periodic_x=1, tauf=wl["tauf"],
                             rho_solid=wl["ratio"], radius=wl["radius"],
                             body_force=(wl["body_force"], 0.0, 0.0), threshold_wall=2.0,
                             threshold_particle=2.0, spring_scale_wall=1.0,
                             spring_scale_particle=1.0, qmode=1)
        t0 = time.perf_counter()
        o.step(2)
        per = max((time.perf_counter() - t0) / 2, 1e-3)
        k = int(max(2, min(50, target_s / per)))
        t0 = time.perf_counter()
        o.step(k)
        dt = time.perf_counter() - t0
        return {"value": nx * ny * nz * k / dt / 1e6, "unit": "MLUPS", "cores": 1, "kind": "port",
                "sample": f"64x32x32 channel with 6 spheres R={wl['radius']}: {k} steps, particle "
                          f"oracle (3-D generalisation of the reference's case4 loop), 1 thread"}
    if wl["kind"] == "lid":
        o = O.LidOracle(n, n, n, wl["reynolds"], wl["u0"], top_layer_u0=False)
        run = lambda k: o.run(k, nthreads=threads)
    else:
        o = O.ThermalOracle(n, n, n, wl["rayleigh"], wl["prandtl"], wl["mach"], 0.0, 0.5, -0.5, 0.0)
        run = lambda k: o.run(k, nthreads=threads)
    t0 = time.perf_counter()
    run(1)  # first touch + warm-up
    t1 = time.perf_counter()
    per = max(t1 - t0, 1e-3)
    k = int(max(1, min(20, target_s / per)))
    t0 = time.perf_counter()
    run(k)
    dt = time.perf_counter() - t0
    return {"value": n ** 3 * k / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{wl['desc']}: {k} steps after 1 warm-up step, oracle (C restatement of "
                      f"the reference's Fortran loops) with {threads} OpenMP threads"}


def mglc_config(wl, form, world, in_place=False):
    """The config object of the bench line (both arms print the same one)."""
    cells = cells_of(wl)
    return {"workload": wl["desc"], "form": form + ("_in_place" if in_place else ""),
            "cells": cells, "parallelism": f"replicas{world}" if world > 1 else "single",
            "l2": l2_note(cells * alg_bytes(wl["kind"], form))}


def reference_arm(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    n = wl["n"]
    if wl["kind"] == "particle":
        cb = cpu_sample(wl, target_s=60.0)
        line = {"impl": "reference", "metric": METRIC, "value": round(cb["value"], 3), "unit": "MLUPS",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": mglc_config(wl, args.form, world),
                "cpu_baseline": cb,
                "e2e": {"value": round(cb["value"], 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    # size the per-step sample so that warmup+steps finish within ~150 s
    probe_n = min(n, 128)
    if wl["kind"] == "lid":
        mk = lambda m: O.LidOracle(m, m, m, wl["reynolds"], wl["u0"], top_layer_u0=False)
    else:
        mk = lambda m: O.ThermalOracle(m, m, m, wl["rayleigh"], wl["prandtl"], wl["mach"], 0.0,
                                       0.5, -0.5, 0.0)
    p = mk(probe_n)
    t0 = time.perf_counter()
    p.run(2, nthreads=threads)
    rate = probe_n ** 3 * 2 / (time.perf_counter() - t0)
    del p
    total = args.steps + args.warmup
    m = n
    while m > 32 and total * m ** 3 / rate > 150.0:
        m = int(m * 0.8) // 8 * 8
    o = mk(m)
    o.run(args.warmup, nthreads=threads)
    t0 = time.perf_counter()
    o.run(args.steps, nthreads=threads)
    dt = time.perf_counter() - t0
    val = m ** 3 * args.steps / dt / 1e6
    sample = (f"{wl['desc'].replace(str(n) + '^3', str(m) + '^3')}: {args.steps} timed steps after "
              f"{args.warmup} warm-up, C restatement of the reference's Fortran loops "
              f"(no Fortran compiler here), {threads} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": round(val, 3), "unit": "MLUPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": mglc_config(wl, args.form, world),
            "cpu_baseline": {"value": round(val, 3), "unit": "MLUPS", "cores": threads,
                             "kind": "port", "sample": sample, "sample_cells": m ** 3,
                             "workload_cells": n ** 3},
            "e2e": {"value": round(val, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mglc", choices=["mglc", "reference"])
    ap.add_argument("--workload", default="lid384", choices=sorted(WORKLOADS))
    ap.add_argument("--form", default="fp64",
                    choices=["fp64", "fx64", "fp32", "fp16", "fp16s", "bf16", "bf16s"])
    ap.add_argument("--no-forms", action="store_true", help="skip timing the other storage forms")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--n", type=int, default=0, help="override the cube size (profiling runs)")
    ap.add_argument("--no-serve", action="store_true", help="skip the batched-serving stream")
    ap.add_argument("--no-error", action="store_true",
                    help="skip measuring each form's error against FP64")
    ap.add_argument("--error-steps", type=int, default=0,
                    help="steps for the error runs (default: the workload's own count)")
    ap.add_argument("--no-lid2d", action="store_true", help="skip the D2Q9 lid cavity line")
    ap.add_argument("--only-particles2d", action="store_true",
                    help="time only the D2Q9 particle cases (--steps/--warmup; no CPU sample)")
    ap.add_argument("--kernel-tour", action="store_true",
                    help="run every step-kernel family once on a small case (profiling runs)")
    ap.add_argument("--in-place", action="store_true",
                    help="time the main line with the in-place (AA-pattern, one-buffer) kernels")
    ap.add_argument("--only-lid2d", type=int, default=0, metavar="N",
                    help="time only the D2Q9 lid cavity at N^2 (--steps/--warmup; profiling runs)")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-max-steps", type=int, default=50000)
    ap.add_argument("--serve-precision", default="fp32", choices=["fp32", "fp16", "fp16s", "bf16"],
                    help="storage form of the served solves")
    ap.add_argument("--no-side", action="store_true",
                    help="skip the heated-cavity and particle-channel entries")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    wl = dict(WORKLOADS[args.workload])
    if args.n and wl["kind"] != "particle":
        wl["desc"] = wl["desc"].replace(f"{wl['n']}^3", f"{args.n}^3")
        wl["n"] = args.n
    if wl["kind"] == "particle" and args.form == "fp64" and "--form" not in sys.argv:
        args.form = "fp32"  # the channel workload is specified with FP32 arithmetic

    spawn, err = world_check(args.gpus)
    if err:
        sys.stderr.write(err + "\n")
        return 2
    if args.impl == "reference":
        return reference_arm(args, wl)  # rank 0 alone times the CPU path

    import torch
    if spawn:
        have = torch.cuda.device_count()
        if have < args.gpus:
            sys.stderr.write(f"bench.py: --gpus {args.gpus} but {have} GPU(s) visible\n")
            return 2
        # one replica rank per GPU; rank 0 prints the line
        return subprocess.run(replica_command(args.gpus, sys.argv[1:], free_port())).returncode
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import mglc_gb300
    from mglc_gb300 import build as B
    B.build()
    mglc_gb300.lib()

    if args.only_particles2d:
        print(json.dumps({"particles2d": particles2d_bench(torch, mglc_gb300, steps=args.steps,
                                                           warmup=args.warmup, cpu=False)}))
        return 0
    if args.kernel_tour:
        print(json.dumps({"kernel_tour": kernel_tour(torch, mglc_gb300)}))
        return 0
    if args.only_lid2d:
        print(json.dumps({"lid2d": lid2d_bench(torch, mglc_gb300, n=args.only_lid2d,
                                               steps=args.steps, warmup=args.warmup,
                                               cpu=not args.no_cpu)}))
        return 0
    cells = cells_of(wl)
    peak, peak_kind = load_peaks()
    with ClockSampler(local) as clk:
        ms, info = time_device(torch, mglc_gb300, wl, args.form, args.steps, args.warmup, dist,
                               in_place=args.in_place)
    clocks = clk.summary()
    value = replica_mlups(world, cells, args.steps, ms)
    ms_step = ms / args.steps
    bpc = info.bytes_per_cell_step
    achieved = bpc * cells / (ms_step * 1e-3) / 1e9
    traffic_tab = load_traffic()
    tkey = f"{wl['kind']}_{args.form}"
    traffic = None
    if tkey in traffic_tab:
        traffic = traffic_tab[tkey]["dram_bytes_per_cell"] * cells
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fx64": "i64 Q55 fixed point (f64 storage)"}.get(args.form, "f32"),
        "data": wl.get("data", "synthetic (analytic cavity initial state, no dataset)"),
        "config": mglc_config(wl, args.form, world, args.in_place),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "traffic_source": traffic_tab.get(tkey, {}).get("source"),
                     "peak_kind": f"hbm_gbs of {peak_kind}",
                     "bytes_per_cell": bpc, "kernel": f"k_{wl['kind']}_step<{args.form}>"},
        "clocks": clocks,
        "gpu_launches": args.steps * wl.get("launches_per_step", 1),
    }
    probe = None
    if args.form == "fp64":
        # the FP64 kernels are bound by the FP64 pipe: report that roof beside HBM's
        probe = fp64_peak()
        fr = fp64_roof(wl["kind"], args.form, value / world, probe)
        if fr:
            line["roofline"].update(fr)
            line["roofline"]["bound"] = "fp64"
    if not args.no_e2e:  # every rank runs its replica end to end; the slowest one counts
        dt, h2d, d2h, eu, phases = time_e2e(torch, mglc_gb300, wl, args.form, args.steps, dist)
        line["e2e"] = {"value": round(world * cells * args.steps / dt / 1e6, 3), "unit": "MLUPS",
                       "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                       "what": "mglc_load_state(host f) + mglc_step(K) + mglc_get_macros(host) "
                               "+ mglc_check, wall clock", "phases": phases}
    if rank == 0 and not args.no_forms:
        forms = {}
        fms = {"particle": ("fp64", "fp32"),
               "thermal": ("fp64", "fx64", "fp32", "fp16", "fp16s", "bf16", "bf16s"),
               "lid": ("fp64", "fx64", "fp32", "fp16", "fp16s", "bf16", "bf16s")}[wl["kind"]]
        for fm in fms:
            if fm == args.form:
                continue
            try:
                m2, inf2 = time_device(torch, mglc_gb300, wl, fm, args.steps, args.warmup)
                v2 = cells * args.steps / (m2 * 1e-3) / 1e6
                a2 = inf2.bytes_per_cell_step * cells / (m2 / args.steps * 1e-3) / 1e9
                forms[fm] = {"value": round(v2, 3), "ms_per_step": round(m2 / args.steps, 4),
                             "bytes_per_cell": inf2.bytes_per_cell_step,
                             "achieved_gbs": round(a2, 1), "frac": round(a2 / peak, 4)}
            except Exception as e:  # report, never hide
                forms[fm] = {"error": str(e)}
        if wl["kind"] == "lid":  # the in-place (AA-pattern, one buffer) kernels
            for fm in ("fp64", "fx64", "fp32", "fp16", "fp16s"):
                try:
                    m2, inf2 = time_device(torch, mglc_gb300, wl, fm, args.steps, args.warmup,
                                           in_place=True)
                    v2 = cells * args.steps / (m2 * 1e-3) / 1e6
                    a2 = inf2.bytes_per_cell_step * cells / (m2 / args.steps * 1e-3) / 1e9
                    forms[fm + "_in_place"] = {"value": round(v2, 3),
                                               "ms_per_step": round(m2 / args.steps, 4),
                                               "achieved_gbs": round(a2, 1),
                                               "frac": round(a2 / peak, 4),
                                               "device_bytes": inf2.device_bytes}
                except Exception as e:  # report, never hide
                    forms[fm + "_in_place"] = {"error": str(e)}
        if not args.no_error and wl["kind"] in ("lid", "thermal"):
            esteps = args.error_steps or wl.get("error_steps", 1000)
            errs = form_errors(mglc_gb300, wl, [f for f in fms if f != "fp64"], esteps)
            for fm, e in errs.items():
                forms.setdefault(fm, {}).update(e)
                forms[fm]["error_steps"] = esteps
                if "u_rel_l2_vs_fp64" in e:  # the metric's accuracy bar for the reduced forms
                    forms[fm]["within_1e-3"] = e["u_rel_l2_vs_fp64"] <= 1e-3
        line["forms"] = forms
        # the metric's "mixed" form: FP16 deviation storage (stochastic
        # rounding), FP32 arithmetic
        mx = forms.get("fp16s", {})
        base = value if args.form == "fp64" else forms.get("fp64", {}).get("value")
        if "value" in mx and base:
            # the in-place kernels compute the same bits; report the faster streaming
            ip = forms.get("fp16s_in_place", {})
            best, streaming = mx, "two buffers"
            if ip.get("value", 0.0) > mx["value"]:
                best, streaming = ip, "in place (AA pattern, one buffer)"
            line["mixed"] = {"form": "fp16 storage of f - w rho0 (stochastic rounding), fp32 arithmetic",
                             "streaming": streaming,
                             "value": best["value"], "unit": "MLUPS", "frac": best["frac"],
                             "speedup_vs_fp64_plain": round(best["value"] / base, 2),
                             "u_rel_l2_vs_fp64": mx.get("u_rel_l2_vs_fp64"),
                             "error_steps": mx.get("error_steps"),
                             "within_1e-3": (mx["u_rel_l2_vs_fp64"] <= 1e-3)
                             if "u_rel_l2_vs_fp64" in mx else None}
    if rank == 0 and not args.no_serve and wl["kind"] == "lid":
        line["serve"] = serve_bench(torch, mglc_gb300, n_req=args.serve_requests,
                                    max_steps=args.serve_max_steps,
                                    precision=args.serve_precision)
    if rank == 0 and not args.no_lid2d and wl["kind"] == "lid":
        line["lid2d"] = lid2d_bench(torch, mglc_gb300)
        line["particles2d"] = particles2d_bench(torch, mglc_gb300)
    if rank == 0 and not args.no_side and wl["kind"] == "lid":
        # the heated cavity (128^3, 20000-step errors) and the particle channel
        # (256x128x128, 200 spheres, 10000-step errors) as entries of their own
        pk = probe if probe else fp64_peak()
        line["thermal128"] = side_workload(torch, mglc_gb300, "thermal128", 200, 5, peak, pk,
                                           cpu=world == 1 and not args.no_cpu,
                                           errors=not args.no_error)
        line["particles"] = side_workload(torch, mglc_gb300, "particles", 200, 5, peak, pk,
                                          cpu=world == 1 and not args.no_cpu,
                                          errors=not args.no_error)
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(wl)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
