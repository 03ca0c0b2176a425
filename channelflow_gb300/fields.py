"""Host-side field preparation: seeded synthetic initial fields and spectral norms.

The workloads start from a laminar base flow plus a seeded divergence-free,
no-slip perturbation whose Fourier-Chebyshev coefficients decay like
0.5^(|kx|+|kz|) * 0.7^n, scaled to a target L2 norm -- the role of the
reference's tools/randomfield.cpp (randomfield generates, fixdivnoslip
projects, flowfield.cpp:4762-4766).  Construction per (kx, kz) mode:
v = (1-y^2)^2 g(y) and wall-normal vorticity eta = (1-y^2) h(y) from random
coefficients, u and w from continuity, so div u = 0 and u = v = w = dv/dy = 0
at y = +-1 hold exactly.  The kz = 0 plane is Hermitian, (0,0) is real.

Fields are complex128 arrays (Nd, Ny, Nx, Nz//2+1) in the reference's serial
spectral FlowField layout.
"""

from __future__ import annotations

import math

import numpy as np
import scipy.fft as sfft


def chebypoints(N: int) -> np.ndarray:
    return np.cos(np.arange(N) * math.pi / (N - 1))


def chebyfft(x: np.ndarray, axis: int = 0) -> np.ndarray:
    """Values at Gauss-Lobatto points -> Chebyshev coefficients (DCT-I scaling of chebyshev.cpp:262-284)."""
    N = x.shape[axis]
    y = sfft.dct(x, type=1, axis=axis) / (N - 1)
    idx = [slice(None)] * y.ndim
    for e in (0, N - 1):
        idx[axis] = e
        y[tuple(idx)] *= 0.5
    return y


def ichebyfft(c: np.ndarray, axis: int = 0) -> np.ndarray:
    N = c.shape[axis]
    x = np.array(c, copy=True)
    idx = [slice(None)] * x.ndim
    idx[axis] = slice(1, N - 1)
    x[tuple(idx)] *= 0.5
    return sfft.dct(x, type=1, axis=axis)


def cdiff(u: np.ndarray, L: float = 2.0) -> np.ndarray:
    """Chebyshev-coefficient derivative along axis 0 (chebyshev.cpp:672-697)."""
    N = u.shape[0]
    d = np.zeros_like(u)
    scale = 4.0 / L
    d[N - 2] = (scale * (N - 1)) * u[N - 1]
    for n in range(N - 3, -1, -1):
        d[n] = d[n + 2] + (scale * (n + 1)) * u[n + 1]
    d[0] *= 0.5
    return d


def _l2_weights(N: int) -> np.ndarray:
    m = np.arange(N)[:, None]
    n = np.arange(N)[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        W = (1 - m * m - n * n) / ((1 + m - n) * (1 - m + n) * (1 + m + n) * (1 - m - n))
    W[(m + n) % 2 == 1] = 0.0
    return W


def l2norm(u: np.ndarray, Nx: int, Nz: int) -> float:
    """Normalised L2 norm of a spectral field (diffops.cpp:415-487), kz > 0 counted twice."""
    Ny = u.shape[1]
    W = _l2_weights(Ny)
    cz = np.where(np.arange(Nz // 2 + 1) == 0, 1.0, 2.0)
    s = 0.0
    for part in (u.real, u.imag):
        q = np.einsum("mn,imxz,inxz->ixz", W, part, part)
        s += float(np.sum(q * cz[None, None, :]))
    return math.sqrt(s)


def random_divfree_field(Nx: int, Ny: int, Nz: int, Lx: float, Lz: float, seed: int, norm: float,
                         zero_mean_u: bool = False, decay_k: float = 0.5, decay_n: float = 0.7) -> np.ndarray:
    """Seeded divergence-free, no-slip perturbation on the 2/3-rule mode set, scaled to ``norm``."""
    rng = np.random.default_rng(seed)
    Mz = Nz // 2 + 1
    y = chebypoints(Ny)
    w1 = 1.0 - y * y
    u = np.zeros((3, Ny, Nx, Mz), dtype=complex)
    nn = np.arange(Ny)
    Kx, Kz = Nx // 3 - 1, Nz // 3 - 1

    def coeffs(kx, kz, nmax):
        c = (rng.standard_normal(Ny) + 1j * rng.standard_normal(Ny)) * (decay_k ** (abs(kx) + abs(kz))) * (
            decay_n ** nn)
        c[nmax:] = 0.0
        return c

    for kx in range(0, Kx + 1):
        for sgn in ((1,) if kx == 0 else (1, -1)):
            k = sgn * kx
            for kz in range(0, Kz + 1):
                if kz == 0 and k < 0:
                    continue
                mx = k if k >= 0 else k + Nx
                if k == 0 and kz == 0:
                    hu = ichebyfft(coeffs(0, 0, Ny - 2).real)
                    hw = ichebyfft(coeffs(0, 0, Ny - 2).real)
                    uc = chebyfft(w1 * hu)
                    wc = chebyfft(w1 * hw)
                    if zero_mean_u:
                        mean = uc[0] - sum(uc[n] / (n * n - 1) for n in range(2, Ny, 2))
                        uc = uc - mean / (2.0 / 3.0) * chebyfft(w1)
                    u[0, :, 0, 0] = uc
                    u[2, :, 0, 0] = wc
                    continue
                g = ichebyfft(coeffs(k, kz, Ny - 4))
                h = ichebyfft(coeffs(k, kz, Ny - 2))
                vc = chebyfft(w1 * w1 * g)
                eta = chebyfft(w1 * h)
                vy = cdiff(vc)
                al, ga = 2 * math.pi * k / Lx, 2 * math.pi * kz / Lz
                k2 = al * al + ga * ga
                u[0, :, mx, kz] = (al * (1j * vy) + ga * (-1j * eta)) / k2
                u[1, :, mx, kz] = vc
                u[2, :, mx, kz] = (ga * (1j * vy) - al * (-1j * eta)) / k2
                if kz == 0:
                    u[:, :, (-k) % Nx, 0] = np.conj(u[:, :, mx, 0])
    return u * (norm / l2norm(u, Nx, Nz))


def io_to_spectral(phys_io: np.ndarray, Nx: int, Nz: int) -> np.ndarray:
    """Spectral field (Nd, Ny, Nx, Nz//2+1) from physical data on a file's unpadded I/O grid.

    The role of FlowField::readNetCDF followed by the padded-mode fill (channelflow/flowfield.cpp:3605-3826):
    phys_io is [i][nz][ny][nx] on the 2(Nx/3) x Ny x 2(Nz/3) grid; its xz Fourier coefficients (scaled by
    1/(nx nz)) fill the kx >= 0 and kx < 0 blocks of the Nx x Nz spectral grid, the remaining modes are zero,
    and the values at the Gauss-Lobatto points become Chebyshev coefficients."""
    Nd, Nz_io, Ny, Nx_io = phys_io.shape
    p = np.transpose(phys_io, (0, 2, 3, 1))  # [i][ny][nx][nz]
    c = np.fft.rfft2(p, axes=(2, 3)) * (1.0 / (Nx_io * Nz_io))
    out = np.zeros((Nd, Ny, Nx, Nz // 2 + 1), dtype=np.complex128)
    h = Nx_io // 2 + 1
    out[:, :, :h, : Nz_io // 2 + 1] = c[:, :, :h, :]
    out[:, :, h + (Nx - Nx_io): Nx, : Nz_io // 2 + 1] = c[:, :, h:, :]
    return np.ascontiguousarray(chebyfft(out, axis=1))
