"""Benchmark of the GB300 DNS time step (one JSON line on stdout).

Workload: plane Poiseuille flow at constant bulk velocity (Ubulk = 2/3,
Re_centreline = 4000, nu = 1/4000), box Lx = 4 pi, Lz = 2 pi, grid
128 x 97 x 128, CNAB2 with SMRK2 start-up, dt = 0.01, rotational
nonlinearity with 2/3-rule dealiasing; initial field = laminar profile plus a
seeded divergence-free perturbation of L2 norm 0.3 (synthetic, see
channelflow_gb300/fields.py).  A "step" is one CNAB2 time step of that field.

GPU arm (default):  value = steps/s of the mixed-precision path (FP32
transforms and nonlinear term, FP64 state and tau solves) with the fields
resident in HBM, device-timed with CUDA events on the library's stream over
the graph-replayed steps a caller runs (the per-phase times come from a
second pass with events between the phases).
The plain FP64 path is timed the same way ("fp64" block), the end-to-end
number goes through cfgpu_dns_advance with host buffers every step ("e2e"),
and the mixed-vs-FP64 relative L2 difference after T = 10 is reported
("accuracy").  With torchrun, every rank runs an independent replica on its
own GPU (the DNS of one field does not shard); value aggregates all ranks.

Reference arm (--impl reference): the reference's algorithm restated on the
CPU (oracle/cf_oracle.py, NumPy/SciPy, FFTs on every host thread) on the same
workload; each timed step is one full CNAB2 step of the 128 x 97 x 128 field.
"""

from __future__ import annotations

import argparse
import contextlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DNS steps/s 128x97x128: FP32-mixed vs FP64 at stated L2 err; serve p50/p99"
NX, NY, NZ = 128, 97, 128
LX, LZ = 4 * math.pi, 2 * math.pi
NU, DT, UBULK = 1.0 / 4000.0, 0.01, 2.0 / 3.0
WORKLOAD = ("plane Poiseuille 128x97x128 (Lx=4pi, Lz=2pi), CNAB2 + SMRK2 start-up, dt=0.01, bulk velocity "
            "Ubulk=2/3, Re_c=4000, rotational NL, 2/3 dealiasing, seeded perturbation L2=0.3")
CNAB2, SMRK2, LaminarBase, BulkVelocity = 1, 3, 3, 1
# DRAM bytes (read + write) per step of the mixed-path phases from `ncu --set full` captures of this workload
# (one steady-state step: the tau solve's right-hand side, pressure/v and u/w kernels; the nonlinear pass's
# curl/inverse Chebyshev kernel, the three x/z kernels plain runs of this grid choose, and the tensor-core
# forward Chebyshev kernel).  Cold-cache replay: in the step the x/z intermediates stay in L2.  The z-pass
# figure is the Stockham kernel's; the register-FFT z pass reads and writes the same arrays.
NCU_TRAFFIC = {"tau_solve": (38.06 + 0.59 + 63.62 + 2.34 + 31.63 + 0.07) * 1e6,
               "nonlinear_pass": (16.32 + 0.00 + 17.74 + 1.43 + 25.13 + 0.00 + 12.60 + 0.00 + 8.26 + 0.00) * 1e6}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def current_gpu_bus_id():
    """PCI bus id of the CUDA device this process computes on (the runtime's current device).

    nvidia-smi numbers GPUs physically and ignores CUDA_VISIBLE_DEVICES, so the clock sampler names the GPU
    by bus id; None when the runtime cannot say (the sampler then records nothing)."""
    import ctypes
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            rt = None
    if rt is None:
        return None
    dev = ctypes.c_int(0)
    buf = ctypes.create_string_buffer(64)
    if rt.cudaGetDevice(ctypes.byref(dev)) != 0 or rt.cudaDeviceGetPCIBusId(buf, 64, dev) != 0:
        return None
    return buf.value.decode() or None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region, for the GPU with the given PCI bus id."""

    def __init__(self, index=None):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        if self.index is None:
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, smax, reasons = [], [], set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(smax), reasons=sorted(reasons),
                       samples=len(sm))
        return out


def make_flags():
    from channelflow_gb300 import DNSFlags
    return DNSFlags(nu=NU, dt=DT, timestepping=CNAB2, initstepping=SMRK2, baseflow=LaminarBase,
                    constraint=BulkVelocity, Ubulk=UBULK)


def initial_field(seed=1):
    from channelflow_gb300.fields import random_divfree_field
    return random_divfree_field(NX, NY, NZ, LX, LZ, seed=seed, norm=0.3, zero_mean_u=True)


def bytes_per_step(Md, prec):
    """Algorithmic HBM bytes of one CNAB2 step (fixed by formula, independent of the implementation).

    A = Ny*Md complex values per component.  Nonlinear pass (read u, write
    y-physical u and omega; read 6, write f; read 3, write N):
        B_NL = 2A (6*8 + 18*s_w)
    Tau pass (read u, q (FP64), N_j, N_j-1 (s_w), per-mode tables 14 Ny
    doubles; write u, q):  B_tau = 2A (4*8 + 6*s_w + 4*8) + 14*8*A
    """
    A = NY * Md
    sw = 4 if prec == "mixed" else 8
    bnl = 2 * A * (6 * 8 + 18 * sw)
    btau = 2 * A * (4 * 8 + 6 * sw + 4 * 8) + 14 * 8 * A
    return bnl, btau


def flops_per_step(Md):
    """Algorithmic FP64-roofline FLOPs of one step (fixed by formula, independent of the implementation):
    9 component transforms (6 inverse, 3 forward), each Ny planes x 2.5 NxNz log2(NxNz) for x-z plus
    2 Md lines x 2.5 (2(Ny-1)) log2(2(Ny-1)) for y, and about 150 Ny flops per mode for the tau solve."""
    xz = NY * 2.5 * NX * NZ * math.log2(NX * NZ)
    y = 2 * Md * 2.5 * 2 * (NY - 1) * math.log2(2 * (NY - 1))
    return 9 * (xz + y), 150.0 * NY * Md


def fp64_peak():
    """FP64 FMA throughput of this GPU in TFLOP/s (cfgpu_measure_fp64: 8 independent chains per thread)."""
    import ctypes as C
    from channelflow_gb300 import _lib as L
    tf, cyc = C.c_double(), C.c_double()
    L.check(L.load().cfgpu_measure_fp64(C.byref(tf), C.byref(cyc)))
    return tf.value, cyc.value


def pin_forms(args, prec):
    """Chebyshev forms of the DNS objects created next: the library's timed choice unless pinned on the command
    line (profiling runs pin the timed run's choices, since timing under a profiler can choose differently);
    prec None restores the defaults."""
    from channelflow_gb300 import _lib as L
    lib = L.load()
    fft = {"mixed": args.cheb_fft_mixed, "fp64": args.cheb_fft_fp64}.get(prec, -1)
    L.check(lib.cfgpu_set_cheb_fft(1 if fft < 0 else fft))
    L.check(lib.cfgpu_set_cheb_tensor(CHEB_TENSOR_DEFAULT if (prec is None or args.cheb_tensor < 0) else
                                      args.cheb_tensor))
    L.check(lib.cfgpu_set_fused_xz(1 if (prec is None or args.fused_xz < 0) else args.fused_xz))


def run_gpu(args, rank, world):
    import ctypes  # noqa: F401
    from channelflow_gb300 import DNS, Grid
    from channelflow_gb300 import build as b
    from channelflow_gb300.dns import PinnedHost
    from channelflow_gb300.fields import l2norm

    b.build()
    from channelflow_gb300.replicas import Replicas
    reps = Replicas(rank, world)  # independent DNS per rank; barriers and the slowest rank's time only
    barrier, max_over_ranks = reps.barrier, reps.max_over_ranks

    grid = Grid(NX, NY, NZ, LX, LZ)
    u0 = initial_field(seed=1 + rank)
    q0 = np.zeros((1,) + u0.shape[1:], dtype=np.complex128)
    results = {}
    hbm, peak_kind = peaks()
    for prec in ("mixed", "fp64"):
        u, q = u0.copy(), q0.copy()
        pin_forms(args, prec)
        dns = DNS(u, grid, make_flags(), precision=prec)
        dns.set_fields(u, q)
        dns.advance_resident(args.warmup)
        K = args.steps if prec == "mixed" else max(3, args.steps // 4)
        l0 = dns.kernel_launches()
        barrier()
        with ClockSampler(current_gpu_bus_id()) as cs:
            ms = dns.advance_timed(K)          # the production path: graph-replayed steps, no phase events
        ms = max_over_ranks(ms)
        launches = dns.kernel_launches() - l0
        # phase breakdown in a second pass of K steps (events between the phases: eager launches, slower)
        dns.set_profiling(True)
        dns.phase_times()
        dns.advance_timed(K)
        nl_ms, nl_n, tau_ms, tau_n = dns.phase_times()
        dns.set_profiling(False)
        results[prec] = dict(ms=ms, K=K, launches=launches, clocks=cs.summary(), nl_ms=nl_ms, nl_n=nl_n,
                             tau_ms=tau_ms, tau_n=tau_n, Md=dns.num_modes(), bytes=dns.device_bytes(),
                             cheb_fft=dns.cheb_fft(), cheb_tensor=dns.cheb_tensor())
        if True:
            # end-to-end through the public API: host buffers in, host buffers out, every step; the caller's
            # FlowField buffers page-locked once (as a caller that keeps them does), and for comparison as plain
            # pageable memory
            Ke = max(3, min(args.steps, 50))
            for pinned in (True, False):
                ue, qe = u0.copy(), q0.copy()
                dns_e = DNS(ue, grid, make_flags(), precision=prec)
                pin_forms(args, None)
                with (PinnedHost(ue, qe) if pinned else contextlib.nullcontext()):
                    dns_e.advance(ue, qe, args.warmup)
                    barrier()
                    t0 = time.perf_counter()
                    for _ in range(Ke):
                        dns_e.advance(ue, qe, 1)
                    te = max_over_ranks(time.perf_counter() - t0)
                Md = dns_e.num_modes()
                key = ("e2e" if prec == "mixed" else "e2e_fp64") + ("" if pinned else "_pageable")
                results[key] = dict(s=te, K=Ke, h2d=4 * NY * Md * 16, d2h=4 * NY * Md * 16)
                dns_e.close()
        dns.close()
    acc = None
    if args.accuracy_steps > 0 and rank == 0:
        # Mixed vs plain FP64 from the same field.  With dt = 0.01 the workload itself becomes unstable at
        # t ~ 5.1 (the CPU restatement of the reference algorithm blows up between steps 510 and 520 on the
        # same trajectory), so the error is stated at t = 4.5 for dt = 0.01 and at T = 10 with dt = 0.005.
        acc = {"norm": "Chebyshev-weighted L2 over all modes (diffops.cpp:415-487), relative to the FP64 path"}
        for dt, steps, key in ((DT, 450, "t4.5_dt0.01"), (DT / 2, 2 * args.accuracy_steps, "T10_dt0.005")):
            outs = {}
            for prec in ("mixed", "fp64"):
                u, q = u0.copy(), q0.copy()
                fl = make_flags()
                fl.dt = dt
                d = DNS(u, grid, fl, precision=prec)
                d.set_fields(u, q)
                d.advance_resident(steps)
                d.get_fields(u, q)
                d.close()
                outs[prec] = u
            acc[key] = l2norm(outs["mixed"] - outs["fp64"], NX, NZ) / l2norm(outs["fp64"], NX, NZ)
        outs0_fp64 = outs["fp64"]
        acc["rel_l2_mixed_vs_fp64"] = acc["T10_dt0.005"]
        # The T = 10 figure is one trajectory of a chaotic flow: any change of rounding reshuffles it.  Two
        # more realizations from the initial field perturbed at 1e-15 (FP64 and mixed both rerun) state the
        # spread.
        reals = [acc["T10_dt0.005"]]
        for r in (1, 2):
            rng = np.random.default_rng(100 + r)
            up = u0 * (1.0 + 1e-15 * rng.standard_normal(u0.shape))
            outs = {}
            for prec in ("mixed", "fp64"):
                u, q = np.ascontiguousarray(up.copy()), q0.copy()
                fl = make_flags()
                fl.dt = DT / 2
                d = DNS(u, grid, fl, precision=prec)
                d.set_fields(u, q)
                d.advance_resident(2 * args.accuracy_steps)
                d.get_fields(u, q)
                d.close()
                outs[prec] = u
            reals.append(l2norm(outs["mixed"] - outs["fp64"], NX, NZ) / l2norm(outs["fp64"], NX, NZ))
        acc["T10_dt0.005_realizations"] = reals
        # the mixed path with its Chebyshev transforms through the FFT (the matrix products are the mixed
        # path's default where they are faster), same field and horizon
        from channelflow_gb300 import _lib as L
        lib = L.load()
        u, q = u0.copy(), q0.copy()
        fl = make_flags()
        fl.dt = DT / 2
        L.check(lib.cfgpu_set_cheb_fft(2))
        try:
            d = DNS(u, grid, fl, precision="mixed")
        finally:
            L.check(lib.cfgpu_set_cheb_fft(1))
        d.set_fields(u, q)
        d.advance_resident(2 * args.accuracy_steps)
        d.get_fields(u, q)
        d.close()
        fp64_first = outs0_fp64
        acc["T10_dt0.005_mixed_cheb_fft"] = l2norm(u - fp64_first, NX, NZ) / l2norm(fp64_first, NX, NZ)
        # the mixed path with its forward Chebyshev transform as compensated FP32 matrix products (the tensor
        # cores take it by default where they are faster)
        u, q = u0.copy(), q0.copy()
        L.check(lib.cfgpu_set_cheb_fft(0))
        L.check(lib.cfgpu_set_cheb_tensor(0))
        try:
            d = DNS(u, grid, fl, precision="mixed")
        finally:
            L.check(lib.cfgpu_set_cheb_fft(1))
            L.check(lib.cfgpu_set_cheb_tensor(CHEB_TENSOR_DEFAULT))
        d.set_fields(u, q)
        d.advance_resident(2 * args.accuracy_steps)
        d.get_fields(u, q)
        d.close()
        acc["T10_dt0.005_mixed_matrix_forward"] = l2norm(u - fp64_first, NX, NZ) / l2norm(fp64_first, NX, NZ)
        # Control: the same FP64 run from the initial field rounded to FP32 (one FP32 rounding of the input,
        # what the mixed path's first transform does) -- how far the flow itself carries a 2^-24 input change.
        u, q = u0.copy(), q0.copy()
        u = (u.real.astype(np.float32).astype(np.float64) + 1j * u.imag.astype(np.float32).astype(np.float64))
        u = np.ascontiguousarray(u)
        fl = make_flags()
        fl.dt = DT / 2
        d = DNS(u, grid, fl, precision="fp64")
        d.set_fields(u, q)
        d.advance_resident(2 * args.accuracy_steps)
        d.get_fields(u, q)
        d.close()
        acc["T10_dt0.005_fp64_from_fp32_rounded_input"] = l2norm(u - outs["fp64"], NX, NZ) / l2norm(outs["fp64"], NX,
                                                                                                      NZ)
    return results, acc, hbm, peak_kind


CHEB_TENSOR_DEFAULT = 1  # the library's default mode of cfgpu_set_cheb_tensor


def run_cheb_forms(args):
    """The nonlinear term's Chebyshev transforms as dense matrix products and through the FFT, both
    precisions, on the benchmark field: device ms per step and per nonlinear pass (CUDA events)."""
    from channelflow_gb300 import DNS, Grid
    from channelflow_gb300 import _lib as L
    lib = L.load()
    grid = Grid(NX, NY, NZ, LX, LZ)
    u0 = initial_field(seed=1)
    out = {}
    for prec in ("mixed", "fp64"):
        out[prec] = {}
        forms = ((0, 0, "matrix"), (2, 0, "fft")) + (((0, 2, "tensor_forward"),) if prec == "mixed" else ())
        for mode, tc, name in forms:
            u, q = u0.copy(), np.zeros((1,) + u0.shape[1:], dtype=np.complex128)
            L.check(lib.cfgpu_set_cheb_fft(mode))
            L.check(lib.cfgpu_set_cheb_tensor(tc))
            try:
                d = DNS(u, grid, make_flags(), precision=prec)
            finally:
                L.check(lib.cfgpu_set_cheb_fft(1))
                L.check(lib.cfgpu_set_cheb_tensor(CHEB_TENSOR_DEFAULT))
            if (mode == 2 and not d.cheb_fft()) or (tc == 2 and not d.cheb_tensor()):
                d.close()
                continue
            d.set_fields(u, q)
            d.advance_resident(args.warmup)
            K = max(3, args.steps // (4 if prec == "fp64" else 2))
            d.set_profiling(True)
            d.phase_times()
            ms = d.advance_timed(K)
            nl_ms, nl_n, _, _ = d.phase_times()
            d.close()
            out[prec][name] = {"step_ms": ms / K, "nl_avg_ms": nl_ms / max(1, nl_n), "steps": K}
    return out


def serve_requests(n, seed, horizon=(5.0, 50.0)):
    """Mixed-grid f^T(u) requests: Nx, Nz in {32, 48, 64, 96}, Ny in {33, 49, 65}, Re U[300, 2000],
    Couette or Poiseuille (box Lx = 2pi/1.14, Lz = 2pi/2.5), T U[horizon], SBDF3 with SMRK2 start-up,
    seeded divergence-free fields of L2 norm U[0.05, 0.3]; each evaluated as cfDSI's f(u, T) with the
    reference's default CFL-adapted TimeStep started at dt = 0.02 (dT = 1, CFL in [0.4, 0.6],
    dt in [0.001, 0.2])."""
    from channelflow_gb300 import DNSFlags, Grid
    from channelflow_gb300.fields import random_divfree_field
    rng = np.random.default_rng(seed)
    lx, lz = 2 * math.pi / 1.14, 2 * math.pi / 2.5
    out = []
    for k in range(n):
        nx, nz = (int(v) for v in rng.choice([32, 48, 64, 96], size=2))
        ny = int(rng.choice([33, 49, 65]))
        re = float(rng.uniform(300, 2000))
        couette = bool(rng.random() < 0.5)
        T = float(rng.uniform(*horizon))
        if couette:
            fl = DNSFlags(nu=1 / re, dt=0.02, baseflow=LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
        else:
            fl = DNSFlags(nu=1 / re, dt=0.02, baseflow=LaminarBase, ulowerwall=0.0, uupperwall=0.0,
                          constraint=BulkVelocity, Ubulk=2 / 3)
        u = random_divfree_field(nx, ny, nz, lx, lz, seed=seed * 1000 + k, norm=float(rng.uniform(0.05, 0.3)),
                                 zero_mean_u=not couette)
        out.append((Grid(nx, ny, nz, lx, lz), fl, T, np.ascontiguousarray(u)))
    return out


def serve_timestep():
    from channelflow_gb300.dsi import TimeStep
    return TimeStep(dt=0.02, dtmin=0.001, dtmax=0.2, dT=1.0, CFLmin=0.4, CFLmax=0.6, variable=True)


def run_alone(req, precision="fp64"):
    """One request alone: f^T(u) through cfgpu_ft (a DNS built per call, as cfDSI::f does)."""
    from channelflow_gb300._lib import CfgpuError
    from channelflow_gb300.dsi import ft
    g, fl, T, u0 = req
    try:
        return ft(np.ascontiguousarray(u0), g, fl, serve_timestep(), T, precision=precision)[0]
    except CfgpuError:  # non-finite result
        return np.full_like(u0, np.nan)


def run_serve(args):
    """Served stream vs one-at-a-time plain FP64 solves of the same requests."""
    from channelflow_gb300.fields import l2norm
    from channelflow_gb300._lib import CfgpuError
    from channelflow_gb300.server import DONE, Server
    reqs = serve_requests(args.serve_requests, seed=7)
    # one at a time, plain FP64 (the reference's pattern: build a DNS per f^T(u) call)
    run_alone(serve_requests(1, seed=99, horizon=(1.0, 1.0))[0])  # warm-up: library, context
    t0 = time.perf_counter()
    alone = [run_alone(r) for r in reqs]
    t_alone = time.perf_counter() - t0
    # the same requests alone in the server's precision: a served result must equal its request run alone
    t0 = time.perf_counter()
    alone_p = [run_alone(r, args.serve_precision) for r in reqs]
    t_alone_p = time.perf_counter() - t0
    out = {"requests": len(reqs),
           "one_at_a_time_fp64": {"s": t_alone, "requests_per_s": len(reqs) / t_alone,
                                  "non_finite": int(sum(not np.all(np.isfinite(a)) for a in alone))},
           "one_at_a_time_" + args.serve_precision: {
               "s": t_alone_p, "requests_per_s": len(reqs) / t_alone_p,
               "non_finite": int(sum(not np.all(np.isfinite(a)) for a in alone_p))}, "rates": []}
    for rate in args.serve_rates:
        rng = np.random.default_rng(11)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(reqs))) if rate > 0 else np.zeros(len(reqs))
        srv = Server(max_bytes=64 << 30, slots=args.serve_slots, precision=args.serve_precision)
        ids = [None] * len(reqs)
        nxt = 0
        start = time.perf_counter()
        while True:
            now = time.perf_counter() - start
            while nxt < len(reqs) and arrivals[nxt] <= now:
                g, fl, T, u = reqs[nxt]
                ids[nxt] = srv.submit_ft(g, fl, serve_timestep(), T, u)
                nxt += 1
            active = srv.pump(args.serve_pump_steps)
            if nxt == len(reqs) and active == 0:
                break
            if active == 0 and nxt < len(reqs):
                time.sleep(max(0.0, arrivals[nxt] - (time.perf_counter() - start)))
        makespan = time.perf_counter() - start
        lat, errs, same, failed = [], [], [], 0
        for k, rid in enumerate(ids):
            try:
                st, res, t = srv.poll(rid)
            except CfgpuError:  # the field blew up (non-finite result), as it may alone
                failed += 1
                continue
            assert st == DONE
            lat.append(t[2] - t[0])
            g = reqs[k][0]
            if np.all(np.isfinite(alone[k])):
                errs.append(l2norm(res - alone[k], g.Nx, g.Nz) / l2norm(alone[k], g.Nx, g.Nz))
            if np.all(np.isfinite(alone_p[k])):
                same.append(float(np.max(np.abs(res - alone_p[k]))))
        stats = srv.stats()
        srv.close()
        out["rates"].append({
            "offered_per_s": rate, "makespan_s": makespan, "requests_per_s": len(reqs) / makespan,
            "field_steps_per_s": stats["field_steps"] / makespan, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "vs_one_at_a_time_fp64": (len(reqs) / makespan) / (len(reqs) / t_alone),
            "vs_one_at_a_time_same_precision": (len(reqs) / makespan) / (len(reqs) / t_alone_p),
            # requests whose field blew up (non-finite) count in the makespan; the completed ones alone:
            "blown_up": failed, "completed_per_s": (len(reqs) - failed) / makespan,
            "max_rel_l2_vs_alone_fp64": float(max(errs)) if errs else None,
            "median_rel_l2_vs_alone_fp64": float(np.median(errs)) if errs else None,
            "rel_l2_vs_alone_fp64_sorted": [float("%.2g" % e) for e in sorted(errs)],
            "max_abs_diff_vs_alone_same_precision": float(max(same)) if same else None, "failed": failed,
            "ensembles": stats["ensembles"], "ensemble_steps": stats["ensemble_steps"],
            "field_steps": stats["field_steps"], "chunks": stats["chunks"], "dt_changes": stats["dt_changes"],
            "host_s_admission": stats["admit_us"] / 1e6, "host_s_interval_ends": stats["interval_us"] / 1e6,
            "host_s_create": stats["create_us"] / 1e6, "host_s_params": stats["params_us"] / 1e6,
            "host_s_stage": stats["stage_us"] / 1e6, "host_s_load": stats["load_us"] / 1e6})
    out.update(precision=args.serve_precision, slots=args.serve_slots, pump_steps=args.serve_pump_steps,
               workload="f^T(u) requests: Nx,Nz in {32,48,64,96}, Ny in {33,49,65}, Re U[300,2000], Couette or "
                        "Poiseuille, T U[5,50], CFL-adapted TimeStep from dt=0.02 (dT=1, CFL 0.4-0.6), SBDF3 + "
                        "SMRK2 start-up, seeded fields L2 U[0.05,0.3], Poisson arrivals")
    return out


def run_ensemble(args):
    """64 plane Couette trajectories (Re 400, 48x49x48, box Lx = 2pi/1.14, Lz = 2pi/2.5, SBDF3 + SMRK2
    start-up, dt = 0.02), each from its own seeded perturbation with L2 norm U[0.05, 0.3], integrated to
    T = 200 (10,000 steps) as one ensemble (every kernel launch covers all 64 fields, graph-replayed steps),
    in both precisions, against the same fields run one after another as single-field FP64 DNS (timed on
    a sample of fields and steps; field 0 compared with the FP64 ensemble over the whole run)."""
    from channelflow_gb300 import DNS, DNSFlags, Ensemble, Grid
    from channelflow_gb300.fields import l2norm, random_divfree_field
    nf, K = args.ensemble_fields, args.ensemble_steps
    lx, lz = 2 * math.pi / 1.14, 2 * math.pi / 2.5
    g = Grid(48, 49, 48, lx, lz)
    fl = DNSFlags(nu=1 / 400, dt=0.02, baseflow=LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    rng = np.random.default_rng(3)
    us = [random_divfree_field(48, 49, 48, lx, lz, seed=4000 + k, norm=float(rng.uniform(0.05, 0.3)))
          for k in range(nf)]
    U = np.ascontiguousarray(np.stack(us))
    Q = np.zeros((nf, 1) + us[0].shape[1:], dtype=np.complex128)
    out = {"workload": "64 plane Couette 48x49x48 Re=400 SBDF3, dt=0.02, perturbation L2 U[0.05,0.3], "
                       "T = %g (%d steps)" % (K * 0.02, K),
           "fields": nf, "steps": K}
    for prec in ("mixed", "fp64"):
        e = Ensemble(g, fl, nf, precision=prec)
        e.set_fields(U.copy(), Q.copy())
        e.advance_resident(3)
        ms = e.advance_timed(K)
        out[prec] = {"ms_per_step": ms / K, "field_steps_per_s": nf * K / (ms / 1e3),
                     "grid_point_steps_per_s": nf * K / (ms / 1e3) * 48 * 49 * 48, "seconds": ms / 1e3,
                     "trajectories_per_s": nf / (ms / 1e3)}
        if prec == "fp64":
            Ue, Qe = np.zeros_like(U), np.zeros_like(Q)
            e.get_fields(Ue, Qe)
        e.close()
    # serial single-field FP64 runs (the reference's pattern), timed on a subset of the fields
    ns = min(nf, args.ensemble_serial_fields)
    Ks = min(K, args.ensemble_serial_steps)
    t_dev = 0.0
    for k in range(ns):
        d = DNS(us[k].copy(), g, fl, precision="fp64")
        d.set_fields(us[k].copy(), Q[0].copy())
        d.advance_resident(3)
        t_dev += d.advance_timed(Ks)
        if k == 0:
            d.advance_resident(K - Ks)
            u0, q0 = us[k].copy(), Q[0].copy()
            d.get_fields(u0, q0)
            out["rel_l2_field0_ensemble_vs_single_fp64"] = l2norm(Ue[0] - u0, 48, 48) / l2norm(u0, 48, 48)
        d.close()
    per_field = t_dev / ns / Ks
    out["serial_fp64"] = {"ms_per_field_step": per_field, "field_steps_per_s": 1e3 / per_field,
                          "fields_timed": ns, "steps_timed": Ks,
                          "seconds_for_all_fields_estimated": per_field * K * nf / 1e3}
    out["speedup_mixed_vs_serial_fp64"] = out["mixed"]["field_steps_per_s"] / out["serial_fp64"]["field_steps_per_s"]
    out["speedup_fp64_vs_serial_fp64"] = out["fp64"]["field_steps_per_s"] / out["serial_fp64"]["field_steps_per_s"]
    return out


def run_config0(args):
    """The 32x33x32 plane Couette configuration (Re 400, box 2pi/1.14 x 2pi/2.5, SBDF3 + SMRK2 start-up,
    dt = 0.02, seeded perturbation of L2 norm 0.1): steps/s of both precisions over 500 steps (T = 10), fields
    resident, CUDA events on the library's stream; and end to end through cfgpu_dns_advance with host buffers."""
    from channelflow_gb300 import DNS, DNSFlags, Grid
    from channelflow_gb300.fields import random_divfree_field
    lx, lz = 2 * math.pi / 1.14, 2 * math.pi / 2.5
    g = Grid(32, 33, 32, lx, lz)
    fl = DNSFlags(nu=1 / 400, dt=0.02, baseflow=LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    u0 = random_divfree_field(32, 33, 32, lx, lz, seed=1, norm=0.1)
    q0 = np.zeros((1,) + u0.shape[1:], dtype=np.complex128)
    out = {"workload": "plane Couette 32x33x32 Re=400 SBDF3, dt=0.02, 500 steps (T=10), perturbation L2 0.1"}
    for prec in ("mixed", "fp64"):
        u, q = u0.copy(), q0.copy()
        d = DNS(u, g, fl, precision=prec)
        d.set_fields(u, q)
        d.advance_resident(5)
        ms = d.advance_timed(500)
        d.close()
        ue, qe = u0.copy(), q0.copy()
        de = DNS(ue, g, fl, precision=prec)
        de.advance(ue, qe, 5)
        t0 = time.perf_counter()
        for _ in range(100):
            de.advance(ue, qe, 1)
        te = time.perf_counter() - t0
        de.close()
        out[prec] = {"steps_per_s": 500 / (ms / 1e3), "ms_per_step": ms / 500,
                     "e2e_steps_per_s": 100 / te}
    return out


def run_newton(args):
    """Newton-Krylov-hookstep searches (nsolver's algorithm on the host, every f^T(u) on the GPU).

    search: the equilibrium-search configuration: plane Couette Re = 400, 32x35x32, box 2pi/1.14 x 2pi/2.5,
    initial guess a seeded perturbation symmetrised with the shift-reflect symmetry (u + sigma u)/2,
    sigma = (1, 1, -1, 1/2, 0), rescaled to L2 norm 0.2; G(u) = (f^T(u) - u)/T with T = 10, fixed dt = 0.02
    (500 steps per f^T); GMRES dimension <= 100, hookstep; f^T in mixed precision for the search, then Newton
    steps with FP64 f^T from where the search stopped.
    travelling_wave: the reference's equilibrium data (tests/data/eq, a travelling wave, 24x33x24) times
    1.001 with its x shift times 1.001, searched with the shift as an unknown, FP64 f^T: the FP64 residual
    a converged search reaches."""
    from channelflow_gb300 import DNSFlags, Grid
    from channelflow_gb300.cfdsi import CFDSI, NewtonSearchFlags, hookstep_search
    from channelflow_gb300.dsi import TimeStep
    from channelflow_gb300.fields import l2norm, random_divfree_field
    from channelflow_gb300.symmetry import FieldSymmetry, apply
    lx, lz = 2 * math.pi / 1.14, 2 * math.pi / 2.5
    fl = DNSFlags(nu=1 / 400, dt=0.02, baseflow=LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    ts = TimeStep(dt=0.02, dtmin=0.02, dtmax=0.02, dT=10.0, CFLmin=0.0, CFLmax=1.0, variable=False)
    out = {}
    # --- equilibrium search (32x35x32) --------------------------------------------------------------------
    g = Grid(32, 35, 32, lx, lz)
    u = random_divfree_field(32, 35, 32, lx, lz, seed=3, norm=0.2)
    u = apply(u, g, FieldSymmetry(1, 1, -1, 0.5, 0.0, 1), project=True)
    u = np.ascontiguousarray(u * (0.2 / l2norm(u, 32, 32)))
    res = {}
    x = None
    for prec, nn in (("mixed", args.newton_steps), ("fp64", args.newton_polish_steps)):
        dsi = CFDSI(g, fl, ts, 10.0, precision=prec)
        x0 = dsi.make_vector(u) if x is None else x
        flags = NewtonSearchFlags(Nnewton=nn, Nsolver=100, epsSolver=1e-3 if prec == "mixed" else 1e-8)
        t0 = time.perf_counter()
        x, Gx, info = hookstep_search(dsi, x0, flags)
        secs = time.perf_counter() - t0
        res[prec] = {"newton_steps": len(info["gx"]) - 1, "gx": [float("%.4g" % v) for v in info["gx"]],
                     "gmres_dims": info["gmres"], "f_evaluations": dsi.fcount, "seconds": secs,
                     "s_per_newton_step": secs / max(1, len(info["gx"]) - 1),
                     "ms_per_f_evaluation": 1e3 * secs / max(1, dsi.fcount), "stop": info["reason"],
                     "converged": info["converged"]}
    uf = CFDSI(g, fl, ts, 10.0)._split(x)[0]
    res["L2Norm_u_final"] = l2norm(uf, 32, 32)
    res["workload"] = ("plane Couette 32x35x32 Re=400, shift-reflect symmetric seeded guess L2 0.2, f^T T=10 "
                       "dt=0.02 SBDF3, GMRES<=100, hookstep; mixed-precision search then FP64 Newton steps")
    out["search"] = res
    # --- travelling wave from the reference's data (FP64) ---------------------------------------------------
    z = np.load(os.path.join(ROOT, "tests", "golden", "eq.npz"))
    from channelflow_gb300.fields import io_to_spectral
    ueq = io_to_spectral(z["eq"], int(z["eq_Nx"]), int(z["eq_Nz"]))
    sb = z["sigmabest"]
    g2 = Grid(int(z["eq_Nx"]), int(z["eq_Ny"]), int(z["eq_Nz"]), float(z["eq_Lx"]), float(z["eq_Lz"]))
    sig = FieldSymmetry(int(sb[1]), int(sb[2]), int(sb[3]), float(sb[4]) * 1.001, float(sb[5]), int(sb[0]))
    dsi = CFDSI(g2, fl, ts, 10.0, sigma=sig, xrelative=True)
    t0 = time.perf_counter()
    x, Gx, info = hookstep_search(dsi, dsi.make_vector(np.ascontiguousarray(ueq * 1.001)),
                                  NewtonSearchFlags(epsSearch=1e-13, Nnewton=8, epsSolver=1e-9, Nsolver=120))
    secs = time.perf_counter() - t0
    out["travelling_wave"] = {"gx": [float("%.4g" % v) for v in info["gx"]], "converged": info["converged"],
                              "final_residual_fp64": float(np.linalg.norm(Gx)), "ax": float(x[-1]),
                              "f_evaluations": dsi.fcount, "seconds": secs,
                              "ms_per_f_evaluation": 1e3 * secs / max(1, dsi.fcount),
                              "workload": "reference tests/data/eq travelling wave 24x33x24 x1.001, x shift "
                                          "unknown, T=10 dt=0.02, FP64"}
    return out


def cpu_sample(nsteps):
    """The oracle (reference algorithm restated in NumPy) on the same workload: nsteps CNAB2 steps."""
    from oracle import cf_oracle as O
    g = O.Grid(NX, NY, NZ, LX, LZ)
    fl = O.DNSFlags(nu=NU, dt=DT, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    constraint=O.BulkVelocity, Ubulk=UBULK)
    u = initial_field()
    q = np.zeros((1,) + u.shape[1:], dtype=np.complex128)
    dns = O.DNS(u, q, g, fl)
    u, q = dns.advance(u, q, 1)  # SMRK2 start-up step (untimed)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        u, q = dns.advance(u, q, 1)
    dt = time.perf_counter() - t0
    return nsteps / dt, dt, O.WORKERS


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--accuracy-steps", type=int, default=1000, help="steps for the mixed-vs-FP64 error (T=10)")
    ap.add_argument("--cpu-steps", type=int, default=12, help="oracle steps in the cpu_baseline sample")
    ap.add_argument("--grid", default=None, help="Nx,Ny,Nz override for small profiling cases (not a bench line)")
    ap.add_argument("--serve-requests", type=int, default=48, help="requests in the serving stream (0: skip)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[4.0, 16.0, 0.0],
                    help="offered request rates per second (0: all at once)")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-pump-steps", type=int, default=25)
    ap.add_argument("--serve-precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--ensemble-fields", type=int, default=64, help="ensemble block fields (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=10000, help="ensemble steps (10000: T = 200)")
    ap.add_argument("--ensemble-serial-fields", type=int, default=8)
    ap.add_argument("--ensemble-serial-steps", type=int, default=200, help="steps timed per serial field")
    ap.add_argument("--config0", type=int, default=1, help="32x33x32 Couette block (0: skip)")
    ap.add_argument("--newton-steps", type=int, default=3, help="mixed-precision Newton steps of the search "
                                                                 "block (0: skip the Newton block)")
    ap.add_argument("--newton-polish-steps", type=int, default=2)
    ap.add_argument("--cheb-forms", type=int, default=1, help="matrix vs FFT Chebyshev transform block (0: skip)")
    ap.add_argument("--cheb-fft-mixed", type=int, default=-1, help="pin cfgpu_set_cheb_fft for the mixed DNS "
                                                                    "(-1: timed choice)")
    ap.add_argument("--cheb-fft-fp64", type=int, default=-1, help="pin cfgpu_set_cheb_fft for the FP64 DNS")
    ap.add_argument("--cheb-tensor", type=int, default=-1, help="pin cfgpu_set_cheb_tensor (-1: timed choice)")
    ap.add_argument("--fused-xz", type=int, default=-1, help="pin cfgpu_set_fused_xz (-1: timed choice; 2: the "
                                                               "fused x/z kernel wherever the grid allows)")
    args = ap.parse_args()
    if args.grid:
        global NX, NY, NZ
        NX, NY, NZ = (int(v) for v in args.grid.split(","))
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))

    if args.impl == "reference":
        if rank != 0:
            return
        warm = max(0, min(args.warmup, 3))
        from oracle import cf_oracle as O  # noqa: F401
        n = max(1, min(args.steps, 20))
        sps, secs, cores = cpu_sample(n)
        line = {"metric": METRIC, "impl": "reference", "value": sps, "unit": "steps/s", "n_gpus": args.gpus,
                "steps": n, "warmup": warm, "ms_per_step": 1000.0 / sps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "grid": [NX, NY, NZ]},
                "cpu_baseline": {"value": sps, "unit": "steps/s", "cores": cores, "kind": "port",
                                 "sample": "%d full CNAB2 steps of the 128x97x128 field after 1 SMRK2 start-up "
                                           "step (NumPy/SciPy restatement of the reference, FFTs and DCTs on "
                                           "%d host threads)" % (n, cores)},
                "e2e": {"value": sps, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    res, acc, hbm, peak_kind = run_gpu(args, rank, world)
    forms = run_cheb_forms(args) if (args.cheb_forms and rank == 0) else None
    serve = run_serve(args) if (args.serve_requests > 0 and rank == 0) else None
    ens = run_ensemble(args) if (args.ensemble_fields > 0 and rank == 0) else None
    cfg0 = run_config0(args) if (args.config0 and rank == 0) else None
    newton = run_newton(args) if (args.newton_steps > 0 and rank == 0) else None
    if rank != 0:
        return
    m = res["mixed"]
    Md = m["Md"]
    sps = world * m["K"] / (m["ms"] / 1000.0)
    f = res["fp64"]
    sps64 = world * f["K"] / (f["ms"] / 1000.0)
    bnl, btau = bytes_per_step(Md, "mixed")
    nl_avg = m["nl_ms"] / max(1, m["nl_n"])
    tau_avg = m["tau_ms"] / max(1, m["tau_n"])
    phases = {"nonlinear_pass": (nl_avg, bnl, m["nl_ms"]), "tau_solve": (tau_avg, btau, m["tau_ms"])}
    dom = max(phases, key=lambda k: phases[k][2])
    t_avg, bts, _ = phases[dom]
    ach = bts / (t_avg / 1000.0) / 1e9
    e = res["e2e"]
    cpu = None
    if world == 1 and args.cpu_steps > 0:
        cps, csecs, cores = cpu_sample(args.cpu_steps)
        cpu = {"value": cps, "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": "%d full CNAB2 steps of the 128x97x128 field (after 1 untimed SMRK2 start-up step), "
                         "NumPy/SciPy restatement of the reference, FFTs and DCTs on %d host threads of %d, "
                         "%.1f s" % (args.cpu_steps, cores, os.cpu_count() or 1, csecs)}
    bnl64, btau64 = bytes_per_step(Md, "fp64")
    ftr, ftau = flops_per_step(Md)
    pk64, cyc64 = fp64_peak()
    tau64 = f["tau_ms"] / max(1, f["tau_n"])
    line = {
        "metric": METRIC, "value": sps, "unit": "steps/s", "n_gpus": world, "steps": m["K"],
        "warmup": args.warmup, "ms_per_step": m["ms"] / m["K"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64 (FP32 transforms/NL, FP64 state and tau solves)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "mixed", "grid": [NX, NY, NZ], "solved_modes": Md,
                   "grid_point_steps_per_s": sps * NX * NY * NZ,
                   "l2": "no flush: per-step working set %.0f MB > 129 MB L2" % (m["bytes"] / 1e6),
                   "parallelism": "replicas" if world > 1 else "single",
                   "cheb_transforms": "fft" if m["cheb_fft"] else "matrix",
                   "forward_cheb_on_tensor_cores": m["cheb_tensor"]},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s",
                     "frac": ach / hbm, "peak_source": peak_kind,
                     "traffic": NCU_TRAFFIC.get(dom) if (NX, NY, NZ) == (128, 97, 128) else None,
                     "algorithmic_bytes": bts, "avg_launch_ms": t_avg},
        "phases": {"nonlinear_pass": {"avg_ms": nl_avg, "launches": m["nl_n"], "alg_bytes": bnl,
                                      "achieved_gbs": bnl / (nl_avg / 1e3) / 1e9 if nl_avg else None,
                                      "frac": (bnl / (nl_avg / 1e3) / 1e9) / hbm if nl_avg else None},
                   "tau_solve": {"avg_ms": tau_avg, "launches": m["tau_n"], "alg_bytes": btau,
                                 "achieved_gbs": btau / (tau_avg / 1e3) / 1e9 if tau_avg else None}},
        "fp64": {"value": sps64, "unit": "steps/s", "ms_per_step": f["ms"] / f["K"], "steps": f["K"],
                 "nl_avg_ms": f["nl_ms"] / max(1, f["nl_n"]), "tau_avg_ms": f["tau_ms"] / max(1, f["tau_n"]),
                 "nl_alg_bytes": bnl64, "tau_alg_bytes": btau64,
                 "cheb_transforms": "fft" if f["cheb_fft"] else "matrix"},
        # FP64 roofline (the tau solve of both paths and the whole plain-FP64 step compute in FP64): algorithmic
        # FLOPs by formula over the FP64 FMA throughput measured on this GPU in this run
        "roofline_fp64": {"peak_tflops": pk64, "dependent_dfma_cycles": cyc64,
                          "peak_source": "cfgpu_measure_fp64 (FMA microbenchmark, this run)",
                          "tau_solve_mixed": {"flops": ftau, "achieved_tflops": ftau / (tau_avg / 1e3) / 1e12,
                                              "frac": ftau / (tau_avg / 1e3) / 1e12 / pk64},
                          "tau_solve_fp64": {"flops": ftau, "achieved_tflops": ftau / (tau64 / 1e3) / 1e12,
                                             "frac": ftau / (tau64 / 1e3) / 1e12 / pk64},
                          "fp64_step": {"flops": ftr + ftau,
                                        "achieved_tflops": (ftr + ftau) / (f["ms"] / f["K"] / 1e3) / 1e12,
                                        "frac": (ftr + ftau) / (f["ms"] / f["K"] / 1e3) / 1e12 / pk64}},
        "accuracy": acc,
        "e2e": {"value": world * e["K"] / e["s"], "unit": "steps/s", "h2d_bytes_per_step": e["h2d"],
                "d2h_bytes_per_step": e["d2h"],
                "path": "cfgpu_dns_advance(u, q, 1) per step with host FlowField buffers",
                "host_memory": "page-locked once before the timed steps (cfgpu_host_register)",
                "fp64": world * res["e2e_fp64"]["K"] / res["e2e_fp64"]["s"],
                "pageable": {"mixed": world * res["e2e_pageable"]["K"] / res["e2e_pageable"]["s"],
                             "fp64": world * res["e2e_fp64_pageable"]["K"] / res["e2e_fp64_pageable"]["s"]}},
        "gpu_launches": m["launches"],
        "clocks": m["clocks"],
        "cpu_baseline": cpu,
        "serve": serve,
        "ensemble": ens,
        "config0": cfg0,
        "newton": newton,
        "cheb_forms": forms,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
