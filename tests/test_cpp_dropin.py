"""The C++ drop-in (include/cfgpu.hpp) compiled against stand-in types with the reference's member names and
linked with libcfgpu.so: it compiles and links on the CPU; on the GPU its DNS, TauSolver, HelmholtzSolver and
FlowField transforms agree with the oracle (channelflow/dns.cpp:22-163, tausolver.cpp:81-402,
helmholtz.cpp:18-213, flowfield.cpp:1850-1997)."""

import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, oracle_run, rel_l2, solved_mask

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp")
LIBDIR = os.path.join(ROOT, "channelflow_gb300")


def compile_dropin(outdir):
    from channelflow_gb300 import build
    build.build()
    gxx = shutil.which("g++") or shutil.which("c++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = os.path.join(outdir, "dropin_test")
    cuda_lib = [d for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
                            "/usr/local/cuda/targets/x86_64-linux/lib") if os.path.isdir(d)]
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", SRC, "-o", exe, "-L", LIBDIR, "-lcfgpu", "-Wl,-rpath," + LIBDIR]
    for d in cuda_lib:
        cmd += ["-L", d, "-Wl,-rpath," + d]
    cmd += ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "warning" not in r.stderr, r.stderr
    return exe


def test_dropin_compiles_and_links(tmp_path):
    exe = compile_dropin(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_dropin_matches_oracle(tmp_path):
    from tests.test_oracle_golden import tau_case
    exe = compile_dropin(str(tmp_path))
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    nsteps, nu, dt, rot = 12, 1 / 400, 0.02, 0.1
    u0 = O.random_divfree_field(g, seed=12, norm=0.1)
    rng = np.random.default_rng(4)
    c = tau_case(rng, N=g.Ny)
    lam_tau = c["lam_t"] + 4 * math.pi ** 2 * nu * ((c["kx"] / g.Lx) ** 2 + (c["kz"] / g.Lz) ** 2)
    hl, hnu, ua, ub, umean = 3.0, 0.7, 0.25, -0.5, 0.1
    f = rng.standard_normal(g.Ny) * 0.5 ** np.arange(g.Ny)
    phys = rng.standard_normal((g.Ny, g.Nx, g.Nz))
    case = os.path.join(str(tmp_path), "case.bin")
    with open(case, "wb") as fh:
        np.array([g.Nx, g.Ny, g.Nz, nsteps], np.int32).tofile(fh)
        np.array([g.Lx, g.Lz, nu, dt, rot], np.float64).tofile(fh)
        np.ascontiguousarray(u0, np.complex128).tofile(fh)
        np.array([c["kx"], c["kz"]], np.int32).tofile(fh)
        np.array([lam_tau], np.float64).tofile(fh)
        np.concatenate([c["Rx"], c["Ry"], c["Rz"]]).astype(np.complex128).tofile(fh)
        np.array([hl, hnu, ua, ub, umean], np.float64).tofile(fh)
        f.astype(np.float64).tofile(fh)
        phys.astype(np.float64).tofile(fh)
    out = os.path.join(str(tmp_path), "out.bin")
    r = subprocess.run([exe, case, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    d = np.fromfile(out, dtype=np.uint8)
    pos = 0

    def take(dtype, n):
        nonlocal pos
        b = np.dtype(dtype).itemsize * n
        v = d[pos:pos + b].view(dtype)
        pos += b
        return v

    shp = (g.Ny, g.Nx, g.Mz)
    gu = take(np.complex128, 3 * np.prod(shp)).reshape((3,) + shp)
    gq = take(np.complex128, np.prod(shp)).reshape((1,) + shp)
    t, cfl, ubulk, dpdx = take(np.float64, 4)
    fl = O.DNSFlags(nu=nu, dt=dt, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, rotation=rot)
    ou, oq, _ = oracle_run(u0, g, fl, nsteps, chunks=[nsteps // 2, nsteps - nsteps // 2])
    m = solved_mask(g)
    ou[:, :, ~m] = 0
    oq[:, :, ~m] = 0
    assert rel_l2(gu, ou, g) <= 1e-10
    assert rel_l2(gq, oq, g) <= 1e-8
    assert abs(t - nsteps * dt) < 1e-12 and cfl > 0 and math.isfinite(ubulk) and math.isfinite(dpdx)

    tu, tv, tw, tP = [take(np.complex128, g.Ny) for _ in range(4)]
    ts = O.TauSolver([c["kx"]], [c["kz"]], g.Lx, g.Lz, -1.0, 1.0, [lam_tau], nu, g.Ny)
    col = lambda x: x[:, None]
    ru, rv, rw, rP = ts.solve(col(c["Rx"]), col(c["Ry"]), col(c["Rz"]))
    for got, ref in ((tu, ru), (tv, rv), (tw, rw), (tP, rP)):
        assert np.abs(got - ref[:, 0]).max() <= 1e-11 * max(1.0, np.abs(ref).max())

    hu = take(np.float64, g.Ny)
    hm = take(np.float64, g.Ny)
    mu = take(np.float64, 1)[0]
    hs = O.HelmholtzSolver(g.Ny, -1.0, 1.0, np.array([hl]), hnu)
    ref_u = hs.solve(f[:, None], ua, ub)[:, 0]
    ref_m, ref_mu = hs.solve_mean(f[:, None], np.array([umean]), ua, ub)
    assert np.abs(hu - ref_u).max() <= 1e-12 * max(1.0, np.abs(ref_u).max())
    assert np.abs(hm - ref_m[:, 0]).max() <= 1e-12 * max(1.0, np.abs(ref_m).max())
    assert abs(mu - float(np.ravel(ref_mu)[0])) <= 1e-11 * max(1.0, abs(float(np.ravel(ref_mu)[0])))

    nzp = 2 * g.Mz
    spec = take(np.float64, g.Ny * g.Nx * nzp).view(np.complex128).reshape(1, g.Ny, g.Nx, g.Mz)
    back = take(np.float64, g.Ny * g.Nx * nzp).reshape(g.Ny, g.Nx, nzp)[:, :, : g.Nz]
    ref = O.make_spectral(phys[None], g)
    assert np.abs(spec - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(back - phys).max() <= 1e-13 * np.abs(phys).max()
    assert "dropin ok" in r.stdout
