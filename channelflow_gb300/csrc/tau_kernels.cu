// Per-(kx,kz) tau / Helmholtz kernels of the DNS step, FP64.
//
// Reference functions restated (channelflow project paths):
//   BandedTridiag::ULdecomp / ULsolveStrided / multiplyStrided
//                                        channelflow/bandedtridiag.cpp:212-333
//   HelmholtzSolver ctor / solve / solve(mean)  channelflow/helmholtz.cpp:18-95, 158-213
//   TauSolver ctor                      channelflow/tausolver.cpp:81-176
//   TauSolver::influenceCorrection      channelflow/tausolver.cpp:178-191
//   TauSolver::solve_P_and_v            channelflow/tausolver.cpp:193-251
//   TauSolver::solve (+ bulk variant)   channelflow/tausolver.cpp:347-450
//   NSE::linear / NSE::solve            channelflow/nse.cpp:393-575
//   multistep / CNAB / RK right-hand sides  channelflow/dnsalgo.cpp:217-224, 448-455, 668-673
//
// Every per-mode quantity lives in global memory as a "line" of N values
// with a fixed stride between consecutive Chebyshev indices, so a warp of
// threads (consecutive modes) touches consecutive addresses at each step.
#include "kernels.h"

struct Ln {
  double* p;
  size_t s;
  __device__ __forceinline__ double& operator[](int i) const { return p[(size_t)i * s]; }
};

// Helmholtz UL factors of one mode, packed by Chebyshev index n: even rows
// of the even matrix at n = 2i, odd matrix rows at n = 2i+1.
struct HelmFac {
  Ln band, up, lo, inv;
};

__device__ __forceinline__ int nE_of(int N) { return (N - 1) / 2 + 1; }
__device__ __forceinline__ int nO_of(int N) { return (N - 1) / 2; }

// u = A^{-1} B f with u(a)=ua, u(b)=ub (HelmholtzSolver::solve).  f and u must differ.
__device__ void helm_solve(const HelmFac& F, const HelmB& hb, int N, Ln f, Ln u, double ua, double ub) {
  for (int q = 0; q < 2; ++q) {
    const int M = q == 0 ? nE_of(N) : nO_of(N);
    // multiplyStrided: row 0 of B is e0, rows 1..M-2 tridiagonal, last row lo+diag
    u[q] = f[q];
    for (int i = 1; i < M - 1; ++i) {
      const int n = 2 * i + q;
      u[n] = hb.lo[n] * f[n - 2] + hb.di[n] * f[n] + hb.up[n] * f[n + 2];
    }
    {
      const int n = 2 * (M - 1) + q;
      u[n] = hb.lo[n] * f[n - 2] + hb.di[n] * f[n];
    }
  }
  u[0] = (ub + ua) / 2;
  u[1] = (ub - ua) / 2;
  for (int q = 0; q < 2; ++q) {
    const int M = q == 0 ? nE_of(N) : nO_of(N);
    int i;
    for (i = M - 2; i > 0; --i) {
      const int n = 2 * i + q;
      u[n] -= F.up[n] * u[n + 2];
    }
    double b0 = u[q];
    for (int j = 1; j < M; ++j) b0 -= F.band[2 * j + q] * u[2 * j + q];
    b0 /= F.band[q];
    u[q] = b0;
    double prev = b0;
    for (i = 1; i < M; ++i) {
      const int n = 2 * i + q;
      const double v = (u[n] - F.lo[n] * prev) * F.inv[n];
      u[n] = v;
      prev = v;
    }
  }
}

// d = diff(x) (chebyshev.cpp:672-697); x and d must differ.
__device__ void cheb_diff(int N, double scale, Ln x, Ln d) {
  const int Nb = N - 1;
  d[Nb] = 0.0;
  double d2 = 0.0, d1 = (scale * Nb) * x[Nb];
  d[Nb - 1] = d1;
  for (int n = Nb - 2; n >= 0; --n) {
    const double v = d2 + (scale * (n + 1)) * x[n + 1];
    d[n] = v;
    d2 = d1;
    d1 = v;
  }
  d[0] = d[0] * 0.5;
}

__device__ double eval_b(int N, Ln x) {
  double s = 0.0;
  for (int n = N - 1; n >= 0; --n) s += x[n];
  return s;
}
__device__ double eval_a(int N, Ln x) {
  double s = 0.0;
  for (int n = N - 1; n >= 0; --n) s += (n % 2 == 0) ? x[n] : -x[n];
  return s;
}
__device__ double cheb_mean(int N, Ln x) {
  double s = x[0];
  for (int n = 2; n < N; n += 2) s -= x[n] / (double)(n * n - 1);
  return s;
}

// Build Ae/Ao (band = 1, tridiagonal rows from helmholtz.cpp:35-70) and UL-factor them.
__device__ void helm_build(int N, double a, double b, double lambda, double nu, HelmFac F) {
  const int N_ = N - 1;
  const double nuscaled = nu / (((b - a) / 2) * ((b - a) / 2));
  for (int q = 0; q < 2; ++q) {
    const int M = q == 0 ? nE_of(N) : nO_of(N);
    for (int i = 0; i < M; ++i) {
      const int n = 2 * i + q;
      F.band[n] = 1.0;
      F.up[n] = 0.0;
      F.lo[n] = 0.0;
    }
    for (int i = 1; i < M; ++i) {
      const int n = 2 * i + q;
      const int nn = n * n;
      const int cn2 = (n - 2 == 0 || n - 2 == N_) ? 2 : 1;
      const int beta_n = (n > N_ - 2) ? 0 : 1;
      const int beta_n2 = (n + 2 > N_ - 2) ? 0 : 1;
      F.lo[n] = -(cn2 * lambda) / (4 * n * (n - 1));
      F.inv[n] = nuscaled + (beta_n * lambda) / (2 * (nn - 1));  // diag stored in inv until factorised
      if (beta_n2) F.up[n] = -lambda / (4 * n * (n + 1));
    }
    // ULdecomp (bandedtridiag.cpp:212-229); diag(k) lives in F.inv[2k+q]
    for (int k = M - 1; k > 1; --k) {
      const int nk = 2 * k + q, nk1 = 2 * (k - 1) + q;
      const double Akk = F.inv[nk];
      const double w = F.lo[nk];
      F.up[nk1] = F.up[nk1] / Akk;
      F.inv[nk1] = F.inv[nk1] - w * F.up[nk1];
      F.band[nk] = F.band[nk] / Akk;
      F.band[nk1] = F.band[nk1] - w * F.band[nk];
    }
    {
      const int n1 = 2 + q, n0 = q;
      F.band[n1] = F.band[n1] / F.inv[n1];
      F.band[n0] = F.band[n0] - F.lo[n1] * F.band[n1];
    }
    F.inv[q] = 1.0 / F.band[q];
    for (int i = 1; i < M; ++i) F.inv[2 * i + q] = 1.0 / F.inv[2 * i + q];
  }
}

__device__ __forceinline__ int n_func(int k, int Nb) {
  if (k == 0) return Nb - 1;
  if (k == Nb) return 0;
  if (k % 2 == 0) return 2 * (Nb - 1);
  return 2 * Nb;
}

// One thread per mode: the TauSolver constructor for lambda = lambda_t + nu kappa^2.
__global__ void k_tau_setup(GridDev g, int N, double lambda_t, double nu, HelmB hb, TauTable tt, double* scratch) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.Md) return;
  const size_t Md = g.Md;
  const size_t FN = (size_t)N * Md;
  auto T = [&](int f) { return Ln{tt.f + f * FN + m, Md}; };
  auto S = [&](int k) { return Ln{scratch + k * FN + m, Md}; };
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const double Lx = g.Lx, Lz = g.Lz, a = g.a, b = g.b;
  const double kappa2 = 4 * (M_PI * M_PI) * ((kx / Lx) * (kx / Lx) + (kz / Lz) * (kz / Lz));
  const double c4 = 4.0 * (M_PI * M_PI) * nu;
  const double lambda = lambda_t + c4 * ((kx / Lx) * (kx / Lx) + (kz / Lz) * (kz / Lz));
  const double scale = 4.0 / (b - a);
  const int Nb = N - 1;
  HelmFac PH{T(TF_PBAND), T(TF_PUP), T(TF_PLO), T(TF_PINV)};
  HelmFac VH{T(TF_VBAND), T(TF_VUP), T(TF_VLO), T(TF_VINV)};
  helm_build(N, a, b, kappa2, 1.0, PH);
  helm_build(N, a, b, lambda, nu, VH);
  Ln z = S(0), d = S(1), d2 = S(2);
  for (int n = 0; n < N; ++n) z[n] = 0.0;
  Ln Pp = T(TF_PP), Vp = T(TF_VP), Pm = T(TF_PM), Vm = T(TF_VM), P0 = T(TF_P0), V0 = T(TF_V0);
  helm_solve(PH, hb, N, z, Pp, 0.0, 1.0);
  cheb_diff(N, scale, Pp, d);
  helm_solve(VH, hb, N, d, Vp, 0.0, 0.0);
  helm_solve(PH, hb, N, z, Pm, 1.0, 0.0);
  cheb_diff(N, scale, Pm, d);
  helm_solve(VH, hb, N, d, Vm, 0.0, 0.0);
  cheb_diff(N, scale, Vp, d);
  const double A = eval_b(N, d), C = eval_a(N, d);
  cheb_diff(N, scale, Vm, d);
  const double B = eval_b(N, d), D = eval_a(N, d);
  const bool zero = (kx == 0 && kz == 0);
  const double disc = A * D - B * C;
  double i00 = 0, i01 = 0, i10 = 0, i11 = 0;
  if (!zero) {
    i00 = D / disc;
    i01 = -B / disc;
    i10 = -C / disc;
    i11 = A / disc;
  }
  const double c = 2 / (b - a);
  for (int n = 0; n < N; ++n) z[n] = c * n_func(n, Nb);
  helm_solve(PH, hb, N, z, P0, 0.0, 0.0);
  cheb_diff(N, scale, P0, d2);  // dP0dy (before the influence correction, as the reference)
  helm_solve(VH, hb, N, d2, V0, 0.0, 0.0);
  if (!zero) {
    cheb_diff(N, scale, V0, d);
    const double plus = eval_b(N, d), minus = eval_a(N, d);
    const double dp = -i00 * plus - i01 * minus;
    const double dm = -i10 * plus - i11 * minus;
    for (int n = 0; n < N; ++n) {
      P0[n] += dp * Pp[n] + dm * Pm[n];
      V0[n] += dp * Vp[n] + dm * Vm[n];
    }
  }
  // v0yy at Nb-1, Nb is identically zero (two downward recurrences from d[Nb] = 0)
  cheb_diff(N, scale, V0, d);
  Ln d3 = S(3);
  cheb_diff(N, scale, d, d3);
  const double s0Nb1 = lambda * V0[Nb - 1] + d2[Nb - 1] - nu * d3[Nb - 1];
  const double s0Nb = lambda * V0[Nb] + d2[Nb] - nu * d3[Nb];
  // mean-constrained helper (helmholtz.cpp:193-205): mean of the solution of nu u'' - lambda u = nu
  for (int n = 0; n < N; ++n) z[n] = 0.0;
  z[0] = nu;
  helm_solve(VH, hb, N, z, d, 0.0, 0.0);
  const double ucmean = cheb_mean(N, d);
  double* s = tt.s + m;
  s[TS_I00 * Md] = i00;
  s[TS_I01 * Md] = i01;
  s[TS_I10 * Md] = i10;
  s[TS_I11 * Md] = i11;
  s[TS_S0NB1 * Md] = s0Nb1;
  s[TS_S0NB * Md] = s0Nb;
  s[TS_UCMEAN * Md] = ucmean;
  s[TS_LAMBDA * Md] = lambda;
}

cudaError_t launch_tau_setup(const GridDev& g, int N, double lambda_t, double nu, const HelmB& hb, TauTable tt,
                             double* scratch, cudaStream_t st) {
  const int T = 64;
  k_tau_setup<<<(g.Md + T - 1) / T, T, 0, st>>>(g, N, lambda_t, nu, hb, tt, scratch);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Step solve: thread (m, part) with part 0 = real, 1 = imaginary.  Builds the
// scheme's right-hand side, solves the tau problem, writes u and q.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128) k_tau_solve(GridDev g, int N, SolveParams sp, SolvePtrs P, HelmB hb,
                                                   TauTable tt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int Md = g.Md;
  const bool active = t < 2 * Md;
  const int m = active ? t >> 1 : 0;
  const int part = t & 1;
  const size_t row = 2 * (size_t)Md;       // state / scratch row stride
  const size_t comp = row * N;              // component stride
  const size_t off = 2 * (size_t)m + part;  // my element in a row
  const size_t poff = 2 * (size_t)m + (1 - part);
  const size_t FN = (size_t)N * Md;
  auto T = [&](int f) { return Ln{tt.f + f * FN + m, (size_t)Md}; };
  auto SC = [&](int k) { return Ln{P.scratch + k * comp + off, row}; };
  auto SCp = [&](int k) { return Ln{P.scratch + k * comp + poff, row}; };
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = (kx == 0 && kz == 0);
  const double kxL = 2 * M_PI * kx / g.Lx;
  const double kzL = 2 * M_PI * kz / g.Lz;
  const double scale = 4.0 / (g.b - g.a);
  const double nu = sp.nu;
  const int Nb = N - 1;
  const double lambda = tt.s[TS_LAMBDA * Md + m];
  HelmFac PH{T(TF_PBAND), T(TF_PUP), T(TF_PLO), T(TF_PINV)};
  HelmFac VH{T(TF_VBAND), T(TF_VUP), T(TF_VLO), T(TF_VINV)};
  Ln Rx = SC(0), Ry = SC(1), Rz = SC(2);

  // ---- A: right-hand side (my part) --------------------------------------
  if (active) {
    if (sp.kind == 0) {
      for (int n = 0; n < N; ++n) {
        const size_t o = n * row + off;
        for (int c = 0; c < 3; ++c) {
          double acc = 0.0;
          for (int j = 0; j < sp.order; ++j) {
            const double uj = P.uin[j][c * comp + o];
            const double Nj = (double)static_cast<const R*>(P.nin[j])[c * comp + o];
            acc += sp.a[j] * uj + sp.b[j] * Nj;
          }
          SC(c)[n] = acc;
        }
      }
    } else {
      // linear term L = nu u'' - kappa^2 nu u - grad q  (NSE::linear)
      const double kappa2 = 4 * M_PI * M_PI * ((kx / g.Lx) * (kx / g.Lx) + (kz / g.Lz) * (kz / g.Lz));
      const double Dx = 2 * M_PI * kx / g.Lx * (kx == g.kxmax ? 0.0 : 1.0);
      const double Dz = 2 * M_PI * kz / g.Lz * (kz == g.kzmax ? 0.0 : 1.0);
      Ln uk = SC(3), d1 = SC(4), d2 = SC(5);
      Ln qm{const_cast<double*>(P.qin) + off, row};
      Ln qp{const_cast<double*>(P.qin) + poff, row};
      for (int c = 0; c < 3; ++c) {
        Ln uc{const_cast<double*>(P.uin[0]) + c * comp + off, row};
        for (int n = 0; n < N; ++n) uk[n] = nu * uc[n];
        cheb_diff(N, scale, uk, d1);
        cheb_diff(N, scale, d1, d2);
        double wall = 0.0;
        if (m00 && part == 0 && sp.constraint == 1 && c != 1) {
          // actual dPdx from wall shear of nu*u (nse.cpp:452-466), first term
          const double Ly = g.b - g.a;
          wall = (eval_b(N, d1) - eval_a(N, d1)) / Ly;
        }
        if (c == 1) cheb_diff(N, scale, qm, d1);  // q' for the y component
        for (int n = 0; n < N; ++n) {
          double gq;
          if (c == 0) gq = part == 0 ? -(Dx * qp[n]) : Dx * qp[n];
          else if (c == 2) gq = part == 0 ? -(Dz * qp[n]) : Dz * qp[n];
          else gq = d1[n];
          double L = d2[n] - kappa2 * uk[n] - gq;
          if (m00 && part == 0 && c != 1) {
            L += nu * (c == 0 ? P.Ubaseyy[n] : P.Wbaseyy[n]);
            if (n == 0) {
              if (sp.constraint == 0) L -= (c == 0 ? sp.dPdxRef : sp.dPdzRef);
              else L -= wall + sp.baseShear[c == 0 ? 0 : 1];
            }
          }
          const double u0 = uc[n];
          double Nj = (double)static_cast<const R*>(P.nin[0])[c * comp + n * row + off];
          double rhs;
          if (sp.kind == 1) {
            const double Nj1 = (double)static_cast<const R*>(P.nin[1])[c * comp + n * row + off];
            rhs = (u0 * sp.lam + sp.a_b * L) + ((-sp.g_b) * Nj + (-sp.z_b) * Nj1);
          } else {
            R* Q = static_cast<R*>(P.Q) + c * comp + n * row + off;
            const double Qn = (double)(*Q) * sp.rkA - Nj;
            *Q = (R)Qn;
            rhs = L + (sp.lam * u0 + sp.B_C * Qn);
          }
          SC(c)[n] = rhs;
        }
      }
    }
    if (m00 && part == 0) {
      // (0,0): NSE::solve adds nu Ubase'' (and the pressure gradient) to the RHS
      for (int n = 0; n < N; ++n) {
        Rx[n] += nu * P.Ubaseyy[n];
        Rz[n] += nu * P.Wbaseyy[n];
      }
      if (sp.constraint == 0) {
        Rx[0] -= sp.dPdxRef;
        Rz[0] -= sp.dPdzRef;
      }
    }
  }
  __syncwarp();
  // ---- B/C: pressure and wall-normal velocity (solve_P_and_v) -----------
  Ln rr = SC(3), t1 = SC(4), t2 = SC(5);
  Ln Pl{P.qout + off, row};
  Ln Vl{P.uout + comp + off, row};
  if (active) {
    cheb_diff(N, scale, Ry, rr);
    Ln Rxp = SCp(0), Rzp = SCp(2);
    for (int n = 0; n < N; ++n) {
      if (part == 0) rr[n] = rr[n] - (kxL * Rxp[n] + kzL * Rzp[n]);
      else rr[n] = rr[n] + (kxL * Rxp[n] + kzL * Rzp[n]);
    }
    helm_solve(PH, hb, N, rr, Pl, 0.0, 0.0);
    if (m00) {
      for (int n = 0; n < N; ++n) Vl[n] = 0.0;
    } else {
      cheb_diff(N, scale, Pl, t1);
      for (int n = 0; n < N; ++n) t1[n] -= Ry[n];
      helm_solve(VH, hb, N, t1, Vl, 0.0, 0.0);
      // influence correction
      cheb_diff(N, scale, Vl, t2);
      const double plus = eval_b(N, t2), minus = eval_a(N, t2);
      const double* s = tt.s + m;
      const double i00 = s[TS_I00 * Md], i01 = s[TS_I01 * Md], i10 = s[TS_I10 * Md], i11 = s[TS_I11 * Md];
      const double dp = -i00 * plus - i01 * minus;
      const double dm = -i10 * plus - i11 * minus;
      Ln Pp = T(TF_PP), Vp = T(TF_VP), Pm = T(TF_PM), Vm = T(TF_VM);
      for (int n = 0; n < N; ++n) {
        Pl[n] += dp * Pp[n] + dm * Pm[n];
        Vl[n] += dp * Vp[n] + dm * Vm[n];
      }
      if (sp.taucorrection) {
        // nu v''[Nb], nu v''[Nb-1] and P'[Nb] vanish identically; P'[Nb-1] = scale*Nb*P[Nb]
        double s1Nb = lambda * Vl[Nb] - nu * 0.0 - Ry[Nb];
        double s1Nb1 = lambda * Vl[Nb - 1] - nu * 0.0 - Ry[Nb - 1];
        s1Nb += 0.0;
        s1Nb1 += (scale * Nb) * Pl[Nb];
        const double sNb = s1Nb / (1.0 - s[TS_S0NB * Md]);
        const double sNb1 = s1Nb1 / (1.0 - s[TS_S0NB1 * Md]);
        Ln P0 = T(TF_P0), V0 = T(TF_V0);
        for (int n = 0; n <= Nb; ++n) {
          Pl[n] += ((n % 2 == 0) ? sNb1 : sNb) * P0[n];
          Vl[n] += ((n % 2 == 0) ? sNb : sNb1) * V0[n];
        }
      }
    }
  }
  __syncwarp();
  // ---- D: streamwise and spanwise velocity -------------------------------
  if (active) {
    Ln Pp{P.qout + poff, row};  // partner's pressure part
    Ln Ul{P.uout + off, row};
    Ln Wl{P.uout + 2 * comp + off, row};
    for (int c = 0; c < 2; ++c) {
      const double kL = c == 0 ? kxL : kzL;
      Ln Rc = c == 0 ? Rx : Rz;
      Ln out = c == 0 ? Ul : Wl;
      for (int n = 0; n < N; ++n) rr[n] = part == 0 ? -(kL * Pp[n]) - Rc[n] : kL * Pp[n] - Rc[n];
      if (m00 && part == 0 && sp.constraint == 1) {
        // mean-constrained solve (helmholtz.cpp:158-213): returns mu = dPdx
        helm_solve(VH, hb, N, rr, out, 0.0, 0.0);
        const double amean = cheb_mean(N, out);
        const double ucmean = tt.s[TS_UCMEAN * Md + m];
        const double target = c == 0 ? sp.umean : sp.wmean;
        const double mu = nu * (target - amean) / ucmean;
        rr[0] = rr[0] + mu;
        helm_solve(VH, hb, N, rr, out, 0.0, 0.0);
        if (P.dPdx_out) P.dPdx_out[c] = mu;
      } else {
        helm_solve(VH, hb, N, rr, out, 0.0, 0.0);
      }
    }
  }
  __syncwarp();
  if (active && m00 && part == 1 && sp.force_real00) {
    // (0,0) must be real (nse.cpp:555-564)
    for (int n = 0; n < N; ++n) {
      P.uout[n * row + off] = 0.0;
      P.uout[comp + n * row + off] = 0.0;
      P.uout[2 * comp + n * row + off] = 0.0;
      P.qout[n * row + off] = 0.0;
    }
  }
}

template <typename R>
cudaError_t launch_tau_solve(const GridDev& g, int N, const SolveParams& sp, const SolvePtrs& p, const HelmB& hb,
                             TauTable tt, cudaStream_t st) {
  const int T = 64;
  k_tau_solve<R><<<(2 * g.Md + T - 1) / T, T, 0, st>>>(g, N, sp, p, hb, tt);
  return cudaGetLastError();
}

template cudaError_t launch_tau_solve<float>(const GridDev&, int, const SolveParams&, const SolvePtrs&, const HelmB&,
                                             TauTable, cudaStream_t);
template cudaError_t launch_tau_solve<double>(const GridDev&, int, const SolveParams&, const SolvePtrs&, const HelmB&,
                                              TauTable, cudaStream_t);
