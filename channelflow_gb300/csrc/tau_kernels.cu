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
#include <atomic>
#include <type_traits>

#include "kernels.h"


// Exact FP32 -> FP64 conversion by integer operations only (the conversion instruction runs on the FP64 pipe,
// 64 cycles per warp instruction on GB300, and a conversion kept for rare lanes still takes the whole warp's
// slot).  Normal numbers re-bias the exponent; a subnormal m 2^-149 with its leading one at bit p becomes
// 1.f 2^(p-149); infinities and NaNs keep their payload.  FP64 values pass through.
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sgn = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned e = (u >> 23) & 0xFFu;
  unsigned mant = u & 0x7FFFFFu;
  unsigned ex = e + 896u;
  if (e == 0xFFu) {
    ex = 0x7FFu;
  } else if (e == 0) {
    const int p = 31 - __clz(mant | 1u);  // mant = 0 (zero): p = 0, mant stays 0, exponent field 0
    ex = mant ? (unsigned)(p + 874) : 0u;
    mant = (mant << (23 - p)) & 0x7FFFFFu;
  }
  const unsigned long long bits = sgn | ((unsigned long long)ex << 52) | ((unsigned long long)mant << 29);
  return __longlong_as_double((long long)bits);
}

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

// One thread per mode: the TauSolver constructor for lambda = lambda_t + nu kappa^2,
// for modes m0 .. m0+mcount-1.
// blockIdx.y selects one of tb's tables (its lambda_t; 4 scratch lines of its own).
__global__ void k_tau_setup(GridDev g, int N, TauSetupBatch tb, double nu, HelmB hb, double* scratch, int m0,
                            int mcount) {
  const int m = m0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= m0 + mcount || m >= g.Md) return;
  const size_t Md = g.Md;
  const size_t FN = (size_t)N * Md;
  const double lambda_t = tb.lambda_t[blockIdx.y];
  const TauTable tt = tb.tab[blockIdx.y];
  scratch += (size_t)blockIdx.y * 4 * FN;
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
  // segment products of the UL sweeps of both factorisations (four segments of L rows per parity)
  {
    const int L = tau_seg_rows(N);
    const HelmFac* fac[2] = {&PH, &VH};
    Ln Hs[2] = {T(TF_PH), T(TF_VH)}, Gs[2] = {T(TF_PG), T(TF_VG)};
    for (int f = 0; f < 2; ++f)
      for (int q = 0; q < 2; ++q) {
        const int M = q == 0 ? nE_of(N) : nO_of(N);
        Hs[f][q] = 1.0;
        Gs[f][q] = 1.0;
        for (int i0 = 0; i0 < M; i0 += L) {
          const int ia = i0 > 1 ? i0 : 1, ib = i0 + L < M ? i0 + L : M;
          double h = 1.0;
          for (int i = ib - 1; i >= ia; --i) {
            h = -fac[f]->up[2 * i + q] * h;
            Hs[f][2 * i + q] = h;
          }
          double gg = 1.0;
          for (int i = ia; i < ib; ++i) {
            gg = (-fac[f]->lo[2 * i + q] * gg) * fac[f]->inv[2 * i + q];
            Gs[f][2 * i + q] = gg;
          }
        }
      }
  }
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
  s[TS_KXL * Md] = 2 * M_PI * kx / Lx;
  s[TS_KZL * Md] = 2 * M_PI * kz / Lz;
  s[TS_DX * Md] = 2 * M_PI * kx / Lx * (kx == g.kxmax ? 0.0 : 1.0);
  s[TS_DZ * Md] = 2 * M_PI * kz / Lz * (kz == g.kzmax ? 0.0 : 1.0);
  s[TS_KAPPA2 * Md] = kappa2;
  s[TS_RS0NB1 * Md] = zero ? 0.0 : 1.0 / (1.0 - s0Nb1);
  s[TS_RS0NB * Md] = zero ? 0.0 : 1.0 / (1.0 - s0Nb);
}

cudaError_t launch_tau_setup_batch(const GridDev& g, int N, const TauSetupBatch& tb, int ntab, double nu,
                                   const HelmB& hb, double* scratch, cudaStream_t st, int m0, int mcount) {
  const int T = 64;
  if (mcount <= 0) {
    m0 = 0;
    mcount = g.Md;
  }
  if (ntab < 1 || ntab > 4) return cudaErrorInvalidValue;
  k_tau_setup<<<dim3((mcount + T - 1) / T, ntab), T, 0, st>>>(g, N, tb, nu, hb, scratch, m0, mcount);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched HelmholtzSolver (helmholtz.cpp:18-95, 158-213): one thread per system
// nu u'' - lambda_s u = f_s (+ mu_s), u(a) = ua_s, u(b) = ub_s, with the
// mean-constrained variant when umean is given.  Lines are [n][nsys] (W holds
// 7 work lines: 4 UL factors, 2 scratch, f copy).
// ---------------------------------------------------------------------------
__global__ void k_helmholtz(int N, int nsys, double a, double b, const double* __restrict__ lambda, double nu,
                           HelmB hb, const double* __restrict__ f, const double* __restrict__ ua,
                           const double* __restrict__ ub, const double* __restrict__ umean, double* __restrict__ u,
                           double* __restrict__ mu, double* __restrict__ W) {
  const int sidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (sidx >= nsys) return;
  const size_t s = nsys, FN = (size_t)N * nsys;
  auto L = [&](double* base) { return Ln{base + sidx, s}; };
  HelmFac F{L(W), L(W + FN), L(W + 2 * FN), L(W + 3 * FN)};
  helm_build(N, a, b, lambda[sidx], nu, F);
  Ln fl = Ln{const_cast<double*>(f) + sidx, s}, ul = L(u), t0 = L(W + 4 * FN), t1 = L(W + 5 * FN);
  const double A = ua ? ua[sidx] : 0.0, B = ub ? ub[sidx] : 0.0;
  if (!umean) {
    helm_solve(F, hb, N, fl, ul, A, B);
    return;
  }
  // mean-constrained: mu = nu (umean - mean(u_f)) / mean(u_1), u_1 solving nu u'' - lambda u = nu
  helm_solve(F, hb, N, fl, t0, A, B);
  const double uamean = cheb_mean(N, t0);
  for (int n = 0; n < N; ++n) t1[n] = 0.0;
  t1[0] = nu;
  helm_solve(F, hb, N, t1, t0, 0.0, 0.0);
  const double ucmean = cheb_mean(N, t0);
  const double m = nu * (umean[sidx] - uamean) / ucmean;
  Ln fc = L(W + 6 * FN);
  for (int n = 0; n < N; ++n) fc[n] = fl[n];
  fc[0] = fc[0] + m;
  helm_solve(F, hb, N, fc, ul, A, B);
  if (mu) mu[sidx] = m;
}

cudaError_t launch_helmholtz(int N, int nsys, double a, double b, const double* lambda, double nu, const HelmB& hb,
                             const double* f, const double* ua, const double* ub, const double* umean, double* u,
                             double* mu, double* W, cudaStream_t st) {
  if (nsys <= 0) return cudaSuccess;
  k_helmholtz<<<(nsys + 127) / 128, 128, 0, st>>>(N, nsys, a, b, lambda, nu, hb, f, ua, ub, umean, u, mu, W);
  return cudaGetLastError();
}

cudaError_t launch_tau_setup(const GridDev& g, int N, double lambda_t, double nu, const HelmB& hb, TauTable tt,
                             double* scratch, cudaStream_t st, int m0, int mcount) {
  TauSetupBatch tb{};
  tb.lambda_t[0] = lambda_t;
  tb.tab[0] = tt;
  return launch_tau_setup_batch(g, N, tb, 1, nu, hb, scratch, st, m0, mcount);
}

// ---------------------------------------------------------------------------
// Step solve.  Four threads per mode: (part, q) = (real/imaginary part,
// Chebyshev parity).  Even and odd Chebyshev coefficients decouple in every
// Helmholtz solve (helmholtz.cpp:79-95: Ae/Ao, Be/Bo), so thread q owns the
// coefficients n = 2i + q of every line.  Derivative recurrences read the
// other parity (written by the neighbour lane before a group barrier);
// boundary sums are combined with a shuffle.  Lines live in global memory in
// the [n][2*Md] layout; every loop prefetches a chunk of independent loads
// before the dependent arithmetic so no load sits on a recurrence chain.
// ---------------------------------------------------------------------------
#define TCH 8

// parity-local line: element i <-> Chebyshev index n = 2i + q
struct PLn {
  double* p;
  int s;  // elements between i and i+1 (= 2 * full-line stride)
  __device__ __forceinline__ double& operator[](int i) const { return p[(size_t)i * s]; }
};

// u = A^{-1} B f for one parity system of M rows (row 0 of the system carries the boundary value bc).
// Descending pass: B-multiply on the fly, back-substitution, row-0 accumulation; ascending pass: L solve.
__device__ void helm_par(int M, int q, const double* __restrict__ hlo, const double* __restrict__ hdi,
                         const double* __restrict__ hup, PLn band, PLn up, PLn lo, PLn inv, PLn f, PLn u,
                         double bc) {
  const int nM = 2 * (M - 1) + q;
  double fi = f[M - 1], fm = f[M - 2];
  double unext = __ldg(hlo + nM) * fm + __ldg(hdi + nM) * fi;
  u[M - 1] = unext;
  double acc = bc - band[M - 1] * unext;
  double fi1 = fi;
  fi = fm;
  for (int i = M - 2; i >= 1; i -= TCH) {
    double fp[TCH], upv[TCH], bv[TCH];
#pragma unroll
    for (int k = 0; k < TCH; ++k)
      if (i - k >= 1) {
        fp[k] = f[i - k - 1];
        upv[k] = up[i - k];
        bv[k] = band[i - k];
      }
#pragma unroll
    for (int k = 0; k < TCH; ++k)
      if (i - k >= 1) {
        const int n = 2 * (i - k) + q;
        const double bf = (__ldg(hlo + n) * fp[k] + __ldg(hdi + n) * fi) + __ldg(hup + n) * fi1;
        const double ui = bf - upv[k] * unext;
        u[i - k] = ui;
        unext = ui;
        acc -= bv[k] * ui;
        fi1 = fi;
        fi = fp[k];
      }
  }
  double prev = acc / band[0];
  u[0] = prev;
  for (int i = 1; i < M; i += TCH) {
    double uv[TCH], lv[TCH], iv[TCH];
#pragma unroll
    for (int k = 0; k < TCH; ++k)
      if (i + k < M) {
        uv[k] = u[i + k];
        lv[k] = lo[i + k];
        iv[k] = inv[i + k];
      }
#pragma unroll
    for (int k = 0; k < TCH; ++k)
      if (i + k < M) {
        prev = (uv[k] - lv[k] * prev) * iv[k];
        u[i + k] = prev;
      }
  }
}

// Parity q of d = diff(x) (chebyshev.cpp:672-697): d[n] = d[n+2] + (scale (n+1)) x[n+1], descending,
// d[0] *= 1/2.  xo is the other parity of x.  Optionally stores d (dst) and returns the partial sum of
// d over this parity (for boundary values).
__device__ double diff_par(int M, int q, int N, double scale, PLn xo, PLn* dst) {
  double dn2 = 0.0, sum = 0.0;
  int i = M - 1;
  if (q == 0) {
    // top even index n = N-1: x[N] = 0
    const double v = dn2 + (scale * N) * 0.0;
    if (dst) (*dst)[i] = v;
    sum += v;
    dn2 = v;
    i--;
  }
  for (; i >= 0; i -= TCH) {
    double xv[TCH];
#pragma unroll
    for (int k = 0; k < TCH; ++k)
      if (i - k >= 0) xv[k] = xo[i - k + q];
#pragma unroll
    for (int k = 0; k < TCH; ++k)
      if (i - k >= 0) {
        const int n = 2 * (i - k) + q;
        double v = dn2 + (scale * (n + 1)) * xv[k];
        dn2 = v;
        if (n == 0) v *= 0.5;
        if (dst) (*dst)[i - k] = v;
        sum += v;
      }
  }
  return sum;
}

template <typename R>
__global__ void __launch_bounds__(128) k_tau_solve(GridDev g, int N, SolveParams sp, SolvePtrs P, HelmB hb,
                                                   TauTable tt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int Md = g.Md;
  const bool act = (t >> 2) < Md;
  const int m = act ? (t >> 2) : Md - 1;
  const int part = (t >> 1) & 1, q = t & 1;
  const int lane = threadIdx.x & 31;
  const unsigned gmask = 0xFu << (lane & 28);
  const int row = 2 * Md;
  const size_t comp = (size_t)row * N;
  const int off = 2 * m + part, poff = 2 * m + (1 - part);
  const size_t FN = (size_t)N * Md;
  const int M = q ? (N - 1) / 2 : (N - 1) / 2 + 1;
  const int Nb = N - 1;
  // full-line base (n = 0) of component/array at my element; parity views
  auto mine = [&](double* base) { return PLn{base + off + q * row, 2 * row}; };
  auto other = [&](double* base) { return PLn{base + off + (1 - q) * row, 2 * row}; };
  auto ppart = [&](double* base) { return PLn{base + poff + q * row, 2 * row}; };
  auto TB = [&](int f) { return PLn{tt.f + f * FN + m + q * Md, 2 * Md}; };
  double* SC[6];
  for (int k = 0; k < 6; ++k) SC[k] = P.scratch + k * comp;
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = (kx == 0 && kz == 0);
  const double kxL = 2 * M_PI * kx / g.Lx;
  const double kzL = 2 * M_PI * kz / g.Lz;
  const double scale = 4.0 / (g.b - g.a);
  const int fld = mode_field(g, m);
  if (P.slot) apply_slot(sp, P.slot[fld]);
  const size_t fb = (size_t)P.base_stride * fld;
  const double nu = sp.nu;
  const double lambda = tt.s[TS_LAMBDA * Md + m];
  const double* __restrict__ hlo = hb.lo;
  const double* __restrict__ hdi = hb.di;
  const double* __restrict__ hup = hb.up;

  // ---- A: right-hand side (my part, my parity) ----------------------------
  if (sp.kind == 0) {
    for (int i = 0; i < M; ++i) {
      const size_t o = (size_t)(2 * i + q) * row + off;
      for (int c = 0; c < 3; ++c) {
        double acc = 0.0;
        for (int j = 0; j < sp.order; ++j)
          acc += sp.a[j] * P.uin[j][c * comp + o] + sp.b[j] * (double)static_cast<const R*>(P.nin[j])[c * comp + o];
        if (m00 && part == 0 && c != 1) {
          acc += nu * (c == 0 ? P.Ubaseyy[fb + 2 * i + q] : P.Wbaseyy[fb + 2 * i + q]);
          if (2 * i + q == 0 && sp.constraint == 0) acc -= (c == 0 ? sp.dPdxRef : sp.dPdzRef);
        }
        if (act) SC[c][o] = acc;
      }
    }
  } else {
    // per-mode constants from the tables (no FP64 divisions here)
    const double kappa2 = tt.s[TS_KAPPA2 * Md + m];
    const double Dx = tt.s[TS_DX * Md + m];
    const double Dz = tt.s[TS_DZ * Md + m];
    double* uin0 = const_cast<double*>(P.uin[0]);
    double* qin = const_cast<double*>(P.qin);
    for (int c = 0; c < 3; ++c) {
      __syncwarp(gmask);
      PLn uc = mine(uin0 + c * comp);
      PLn uk = mine(SC[3]);
      for (int i = 0; i < M; ++i)
        if (act) uk[i] = nu * uc[i];
      __syncwarp(gmask);
      PLn d1 = mine(SC[4]);
      const double s = diff_par(M, q, N, scale, other(SC[3]), act ? &d1 : nullptr);
      const double so = __shfl_xor_sync(gmask, s, 1);
      double wall = 0.0;
      if (m00 && part == 0 && sp.constraint == 1 && c != 1) {
        // actual dPdx from the wall shear of nu*u (nse.cpp:452-466): (eval_b - eval_a)/Ly
        const double s0 = q == 0 ? s : so, s1 = q == 0 ? so : s;
        wall = ((s0 + s1) - (s0 - s1)) / (g.b - g.a);
      }
      __syncwarp(gmask);
      // descending: d2 = D(d1), dq = D(q) (c == 1), L and the scheme's rhs
      PLn d1o = other(SC[4]);
      PLn qo = other(qin);
      PLn qp = ppart(qin);
      PLn out = mine(SC[c]);
      const R* Nj = static_cast<const R*>(P.nin[0]) + c * comp + off + q * row;
      const R* Nj1 = sp.kind == 1 ? static_cast<const R*>(P.nin[1]) + c * comp + off + q * row : nullptr;
      R* Q = sp.kind == 2 ? static_cast<R*>(P.Q) + c * comp + off + q * row : nullptr;
      double d2n2 = 0.0, dqn2 = 0.0;
      for (int i = M - 1; i >= 0; --i) {
        const int n = 2 * i + q;
        const double x1 = (n + 1 <= Nb) ? d1o[i + q] : 0.0;
        double d2 = d2n2 + (scale * (n + 1)) * x1;
        d2n2 = d2;
        if (n == 0) d2 *= 0.5;
        double gq;
        if (c == 1) {
          const double y1 = (n + 1 <= Nb) ? qo[i + q] : 0.0;
          double dq = dqn2 + (scale * (n + 1)) * y1;
          dqn2 = dq;
          if (n == 0) dq *= 0.5;
          gq = dq;
        } else {
          const double kD = c == 0 ? Dx : Dz;
          gq = part == 0 ? -(kD * qp[i]) : kD * qp[i];
        }
        double L = d2 - kappa2 * uk[i] - gq;
        if (m00 && part == 0 && c != 1) {
          L += nu * (c == 0 ? P.Ubaseyy[fb + n] : P.Wbaseyy[fb + n]);
          if (n == 0) L -= sp.constraint == 0 ? (c == 0 ? sp.dPdxRef : sp.dPdzRef)
                                              : wall + sp.baseShear[c == 0 ? 0 : 1];
        }
        const double u0 = uc[i];
        const double nj = (double)Nj[(size_t)i * 2 * row];
        double rhs;
        if (sp.kind == 1) {
          const double nj1 = (double)Nj1[(size_t)i * 2 * row];
          rhs = (u0 * sp.lam + sp.a_b * L) + ((-sp.g_b) * nj + (-sp.z_b) * nj1);
        } else {
          const double Qn = (double)Q[(size_t)i * 2 * row] * sp.rkA - nj;
          if (act) Q[(size_t)i * 2 * row] = (R)Qn;
          rhs = L + (sp.lam * u0 + sp.B_C * Qn);
        }
        if (m00 && part == 0 && c != 1) {
          rhs += nu * (c == 0 ? P.Ubaseyy[fb + n] : P.Wbaseyy[fb + n]);
          if (n == 0 && sp.constraint == 0) rhs -= (c == 0 ? sp.dPdxRef : sp.dPdzRef);
        }
        if (act) out[i] = rhs;
      }
    }
  }
  __syncwarp(gmask);

  // ---- B/C: pressure and wall-normal velocity (solve_P_and_v) ------------
  PLn Ry = mine(SC[1]);
  PLn rr = mine(SC[3]);
  {
    // rr = D(Ry) -/+ (kx Rx' + kz Rz') with ' the other part
    PLn Rxp = ppart(SC[0]), Rzp = ppart(SC[2]);
    PLn* dst = act ? &rr : nullptr;
    diff_par(M, q, N, scale, other(SC[1]), dst);
    for (int i = 0; i < M; ++i) {
      const double x = kxL * Rxp[i] + kzL * Rzp[i];
      if (act) rr[i] = part == 0 ? rr[i] - x : rr[i] + x;
    }
  }
  PLn Pl = mine(P.qout);
  PLn Vl = mine(P.uout + comp);
  PLn PH_band = TB(TF_PBAND), PH_up = TB(TF_PUP), PH_lo = TB(TF_PLO), PH_inv = TB(TF_PINV);
  PLn VH_band = TB(TF_VBAND), VH_up = TB(TF_VUP), VH_lo = TB(TF_VLO), VH_inv = TB(TF_VINV);
  // dummy sink for inactive lanes (never stored)
  if (act) helm_par(M, q, hlo, hdi, hup, PH_band, PH_up, PH_lo, PH_inv, rr, Pl, 0.0);
  __syncwarp(gmask);
  if (m00) {
    if (act)
      for (int i = 0; i < M; ++i) Vl[i] = 0.0;
  } else {
    PLn tmp = mine(SC[4]);
    diff_par(M, q, N, scale, other(P.qout), act ? &tmp : nullptr);
    if (act) {
      for (int i = 0; i < M; ++i) tmp[i] -= Ry[i];
      helm_par(M, q, hlo, hdi, hup, VH_band, VH_up, VH_lo, VH_inv, tmp, Vl, 0.0);
    }
  }
  __syncwarp(gmask);
  {
    // influence correction (tausolver.cpp:178-191) and tau correction (tausolver.cpp:221-247)
    const double s = m00 ? 0.0 : diff_par(M, q, N, scale, other(P.uout + comp), nullptr);
    const double so = __shfl_xor_sync(gmask, s, 1);
    const double s0 = q == 0 ? s : so, s1 = q == 0 ? so : s;
    const double plus = s0 + s1, minus = s0 - s1;
    const double* sc = tt.s + m;
    const double i00 = sc[TS_I00 * Md], i01 = sc[TS_I01 * Md], i10 = sc[TS_I10 * Md], i11 = sc[TS_I11 * Md];
    const double dp = -i00 * plus - i01 * minus;
    const double dm = -i10 * plus - i11 * minus;
    PLn Pp = TB(TF_PP), Vp = TB(TF_VP), Pm = TB(TF_PM), Vm = TB(TF_VM);
    if (!m00 && act)
      for (int i = 0; i < M; ++i) {
        Pl[i] += dp * Pp[i] + dm * Pm[i];
        Vl[i] += dp * Vp[i] + dm * Vm[i];
      }
    // Nb = N-1 is even (q = 0 holds v[Nb], P[Nb]); Nb-1 is odd (q = 1)
    const int itop = M - 1;
    double x0 = 0.0, y0 = 0.0;
    if (!m00) {
      x0 = lambda * Vl[itop] - nu * 0.0 - Ry[itop];
      y0 = q == 0 ? (scale * Nb) * Pl[itop] : 0.0;
    }
    const double ox = __shfl_xor_sync(gmask, x0, 1);
    const double oy = __shfl_xor_sync(gmask, y0, 1);
    if (!m00 && sp.taucorrection) {
      const double s1Nb = (q == 0 ? x0 : ox) + 0.0;
      const double s1Nb1 = q == 0 ? ox + y0 : x0 + oy;
      const double sNb = s1Nb / (1.0 - sc[TS_S0NB * Md]);
      const double sNb1 = s1Nb1 / (1.0 - sc[TS_S0NB1 * Md]);
      PLn P0 = TB(TF_P0), V0 = TB(TF_V0);
      const double fP = q == 0 ? sNb1 : sNb, fV = q == 0 ? sNb : sNb1;
      if (act)
        for (int i = 0; i < M; ++i) {
          Pl[i] += fP * P0[i];
          Vl[i] += fV * V0[i];
        }
    }
  }
  __syncwarp(gmask);

  // ---- D: streamwise and spanwise velocity -------------------------------
  PLn Ppt = ppart(P.qout);
  for (int c = 0; c < 2; ++c) {
    const double kL = c == 0 ? kxL : kzL;
    PLn Rc = mine(SC[c == 0 ? 0 : 2]);
    PLn out = mine(P.uout + (c == 0 ? 0 : 2) * comp);
    PLn r = mine(SC[3]);
    if (act) {
      for (int i = 0; i < M; ++i) r[i] = part == 0 ? -(kL * Ppt[i]) - Rc[i] : kL * Ppt[i] - Rc[i];
      helm_par(M, q, hlo, hdi, hup, VH_band, VH_up, VH_lo, VH_inv, r, out, 0.0);
    }
    if (m00 && sp.constraint == 1) {
      // mean-constrained solve of the real part (helmholtz.cpp:158-213); the mean involves even n only
      double amean = 0.0;
      if (q == 0) {
        amean = out[0];
        for (int i = 1; i < M; ++i) amean -= out[i] / (double)((2 * i) * (2 * i) - 1);
      }
      const double ucmean = tt.s[TS_UCMEAN * Md + m];
      const double target = c == 0 ? sp.umean : sp.wmean;
      const double mu = nu * (target - amean) / ucmean;
      if (part == 0 && q == 0 && act) {
        r[0] = r[0] + mu;
        helm_par(M, q, hlo, hdi, hup, VH_band, VH_up, VH_lo, VH_inv, r, out, 0.0);
        if (P.dPdx_out) P.dPdx_out[2 * mode_field(g, m) + c] = mu;
      }
    }
  }
  __syncwarp(gmask);
  if (act && m00 && part == 1 && sp.force_real00) {
    PLn u0 = mine(P.uout), v0 = mine(P.uout + comp), w0 = mine(P.uout + 2 * comp), p0 = mine(P.qout);
    for (int i = 0; i < M; ++i) u0[i] = v0[i] = w0[i] = p0[i] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Per-lane working lines in shared memory, laid out [i][lane] (32 lanes per
// warp), so the re-reads between passes and the neighbour-lane reads cost
// shared-memory latency instead of L2 round trips.
// ---------------------------------------------------------------------------
struct SLn {
  double* p;
  __device__ __forceinline__ double& operator[](int i) const { return p[i * 32]; }
};

// Parity q of d = diff(x) with ct[n] = scale*(n+1); xo is the other parity of x; returns the parity's sum.
__device__ double diff_s(int M, int q, const double* ct, SLn xo, SLn* dst) {
  double dn2 = 0.0, sum = 0.0;
  int i = M - 1;
  if (q == 0) {  // top even index n = N-1: x[N] = 0
    if (dst) (*dst)[i] = 0.0;
    i--;
  }
  for (; i >= 0; --i) {
    const double v = dn2 + ct[2 * i + q] * xo[i + q];
    dn2 = v;
    if (dst) (*dst)[i] = v;
    sum += v;
  }
  // the n = 0 coefficient is halved (q = 0: the last one summed, dn2)
  if (q == 0) {
    if (dst) (*dst)[0] = 0.5 * dn2;
    sum -= 0.5 * dn2;
  }
  return sum;
}

// ---------------------------------------------------------------------------
// Table-staged variant (the one launched).  Before each
// Helmholtz solve the warp copies the four UL-factor lines of its 8 modes into
// shared memory with one burst of independent coalesced loads, so the
// dependent sweeps read factors at shared-memory latency.  Rx and Rz, which
// are only streamed, live in global scratch.  Shared memory per warp:
// recurrence constants, 4 working lines per lane, 4 staged factor lines.
// Slots: 0 = Ry then v, 1 = P, 2 and 3 = scratch.
// ---------------------------------------------------------------------------
struct TLn {
  const double* p;
  __device__ __forceinline__ double operator[](int i) const { return p[i * 16]; }
};
// staged factor line of the u/w kernel: [4 fields][N][4 modes]
struct TLn4 {
  const double* p;
  __device__ __forceinline__ double operator[](int i) const { return p[i * 8]; }
};

template <typename TL>
__device__ void helm_t(int M, int q, const double* __restrict__ hlo, const double* __restrict__ hdi,
                       const double* __restrict__ hup, TL band, TL up, TL lo, TL inv, SLn f, SLn u, double bc) {
  const int nM = 2 * (M - 1) + q;
  double fi = f[M - 1], fm = f[M - 2];
  double unext = __ldg(hlo + nM) * fm + __ldg(hdi + nM) * fi;
  u[M - 1] = unext;
  double acc = bc - band[M - 1] * unext;
  double fi1 = fi;
  fi = fm;
#pragma unroll 4
  for (int i = M - 2; i >= 1; --i) {
    const int n = 2 * i + q;
    const double fm1 = f[i - 1];
    const double bf = (__ldg(hlo + n) * fm1 + __ldg(hdi + n) * fi) + __ldg(hup + n) * fi1;
    const double ui = bf - up[i] * unext;
    u[i] = ui;
    unext = ui;
    acc -= band[i] * ui;
    fi1 = fi;
    fi = fm1;
  }
  double prev = acc / band[0];
  u[0] = prev;
#pragma unroll 4
  for (int i = 1; i < M; ++i) {
    prev = (u[i] - lo[i] * prev) * inv[i];
    u[i] = prev;
  }
}

// ---------------------------------------------------------------------------
// Right-hand side of the step solve (NSE::linear and the scheme's combination,
// nse.cpp:393-477, dnsalgo.cpp:202-253, 641-697, 419-470) for the table-staged
// solve: one group of four lanes (re/im part, Chebyshev parity) per (mode,
// component), one component per grid row (blockIdx.y), writing Rx, Ry, Rz to
// the scratch lines 0, 2 and 1 (the solve reads them back).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(32, 10) k_tau_rhs(GridDev g, int N, SolveParams sp, SolvePtrs P, TauTable tt) {
  extern __shared__ double sm[];
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x;
  const int t = blockIdx.x * 32 + lane;
  const int Md = g.Md;
  // one component per grid row: the eight lane groups of a warp read eight consecutive modes of one plane
  const int grp = t >> 2;
  const bool act = grp < Md;
  const int m = act ? grp : Md - 1;
  const int cc = blockIdx.y;
  const int part = (t >> 1) & 1, q = t & 1;
  const unsigned gmask = 0xFu << (lane & 28);
  const int row = 2 * Md;
  const size_t comp = (size_t)row * N;
  const int off = 2 * m + part, poff = 2 * m + (1 - part);
  const int M0 = (N - 1) / 2 + 1;
  const int M = q ? (N - 1) / 2 : M0;
  const int Nb = N - 1;
  const double scale = 4.0 / (g.b - g.a);
  double* ct = sm;
  double* lines = sm + ((N + 1) & ~1);
  for (int n = lane; n < N; n += 32) ct[n] = scale * (n + 1);
  __syncwarp();
  auto S = [&](int slot) { return SLn{lines + (size_t)slot * M0 * 32 + lane}; };
  auto So = [&](int slot) { return SLn{lines + (size_t)slot * M0 * 32 + (lane ^ 1)}; };
  auto G = [&](const double* base) { return PLn{const_cast<double*>(base) + off + q * row, 2 * row}; };
  auto Go = [&](const double* base) { return PLn{const_cast<double*>(base) + off + (1 - q) * row, 2 * row}; };
  auto Gp = [&](const double* base) { return PLn{const_cast<double*>(base) + poff + q * row, 2 * row}; };
  double* Rxg = P.scratch;
  double* Rzg = P.scratch + comp;
  double* Ryg = P.scratch + 2 * comp;
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = (kx == 0 && kz == 0);
  const int fld = mode_field(g, m);
  if (P.slot) apply_slot(sp, P.slot[fld]);
  const size_t fb = (size_t)P.base_stride * fld;
  const double nu = sp.nu;

  // ---- A: right-hand side -------------------------------------------------
  if (sp.kind == 0) {
    PLn outx = G(Rxg), outz = G(Rzg);
    PLn outy = G(Ryg);
    for (int c = cc; c <= cc; ++c) {
      for (int i0 = 0; i0 < M; i0 += TCH) {
        double acc[TCH];
#pragma unroll
        for (int k = 0; k < TCH; ++k) acc[k] = 0.0;
        for (int j = 0; j < sp.order; ++j) {
          const double* uj = P.uin[j] + c * comp;
          const R* nj = static_cast<const R*>(P.nin[j]) + c * comp;
          double uv[TCH], nv[TCH];
#pragma unroll
          for (int k = 0; k < TCH; ++k)
            if (i0 + k < M) {
              const size_t o = (size_t)(2 * (i0 + k) + q) * row + off;
              uv[k] = __ldg(uj + o);
              nv[k] = (double)__ldg(nj + o);
            }
#pragma unroll
          for (int k = 0; k < TCH; ++k)
            if (i0 + k < M) acc[k] += sp.a[j] * uv[k] + sp.b[j] * nv[k];
        }
#pragma unroll
        for (int k = 0; k < TCH; ++k)
          if (i0 + k < M) {
            const int i = i0 + k, n = 2 * i + q;
            double a = acc[k];
            if (m00 && part == 0 && c != 1) {
              a += nu * (c == 0 ? P.Ubaseyy[fb + n] : P.Wbaseyy[fb + n]);
              if (n == 0 && sp.constraint == 0) a -= (c == 0 ? sp.dPdxRef : sp.dPdzRef);
            }
            if (act) (c == 0 ? outx : (c == 1 ? outy : outz))[i] = a;
          }
      }
    }
  } else {
    // rows per batch of the streamed lines (two batches in registers: 6 rows when the nonlinear terms are FP64)
    constexpr int RB = sizeof(R) == 8 ? 6 : TCH;
    // per-mode constants from the tables (no FP64 divisions here)
    const double kappa2 = tt.s[TS_KAPPA2 * Md + m];
    const double Dx = tt.s[TS_DX * Md + m];
    const double Dz = tt.s[TS_DZ * Md + m];
    const int c = cc;
    PLn uc = G(P.uin[0] + c * comp);
    PLn uo = Go(P.uin[0] + c * comp);
    SLn d1 = S(0);
    __syncwarp(gmask);
    // first derivative of this lane's parity from the other parity's coefficients (descending recurrence,
    // without the factor nu); the n = 0 coefficient is halved after the sweep
    // Both sweeps stream their lines in batches of RB rows with the next batch's loads issued before the
    // current batch's recurrence runs (two register buffers), so a warp waits for memory once per sweep
    // rather than once per batch.
    {
      double dn2 = 0.0;
      int i = M - 1;
      if (q == 0) {
        d1[i] = 0.0;
        i--;
      }
      double xa[RB], xb[RB];
      auto ld = [&](int i0, double(&xv)[RB]) {
#pragma unroll
        for (int k = 0; k < RB; ++k)
          if (i0 - k >= 0) xv[k] = uo[i0 - k + q];
      };
      auto run = [&](int i0, const double(&xv)[RB]) {
#pragma unroll
        for (int k = 0; k < RB; ++k)
          if (i0 - k >= 0) {
            const double v = dn2 + ct[2 * (i0 - k) + q] * xv[k];
            dn2 = v;
            d1[i0 - k] = v;
          }
      };
      if (i >= 0) ld(i, xa);
      for (; i >= 0; i -= 2 * RB) {
        if (i - RB >= 0) ld(i - RB, xb);
        run(i, xa);
        if (i - RB < 0) break;
        if (i - 2 * RB >= 0) ld(i - 2 * RB, xa);
        run(i - RB, xb);
      }
      if (q == 0) d1[0] = 0.5 * d1[0];
    }
    // wall shear of the (0,0) mode's u and w (bulk-velocity constraint): the sum of u' over the
    // coefficients of each parity, combined across the lane pair
    const bool shear = m00 && part == 0 && sp.constraint == 1 && c != 1;
    double s = 0.0;
    if (shear)
      for (int i = M - 1; i >= 0; --i) s += d1[i];
    const double so = __shfl_xor_sync(gmask, s, 1);
    double wall = 0.0;
    if (shear) {
      const double s0 = nu * (q == 0 ? s : so), s1 = nu * (q == 0 ? so : s);
      wall = ((s0 + s1) - (s0 - s1)) / (g.b - g.a);
    }
    __syncwarp(gmask);
    SLn d1o = So(0);
    PLn qo = Go(P.qin);
    PLn qp = Gp(P.qin);
    PLn out = G(c == 0 ? Rxg : (c == 1 ? Ryg : Rzg));
    const R* Nj = static_cast<const R*>(P.nin[0]) + c * comp + off + q * row;
    const R* Nj1 = sp.kind == 1 ? static_cast<const R*>(P.nin[1]) + c * comp + off + q * row : nullptr;
    R* Q = sp.kind == 2 ? static_cast<R*>(P.Q) + c * comp + off + q * row : nullptr;
    // L = nu (u'' - kappa^2 u) - grad q; CNAB: rhs = lam u + a_b L - g_b N_j - z_b N_{j-1}; CNRK2:
    // rhs = L + lam u + B_C Q.  Both as rhs = cu u + cd u'' + cg g + Nc with g = q (u, w: times the sign of
    // i k of the part) or q' (v), the constants folded per mode; the n = 0 row takes the halved derivative.
    const double kD = c == 0 ? Dx : Dz;
    const double aL = sp.kind == 1 ? sp.a_b : 1.0;
    const double cu = sp.lam - aL * (nu * kappa2);
    const double cd = aL * nu;
    const double cg = c == 1 ? -aL : (part == 0 ? aL * kD : -(aL * kD));
    const double cd0 = 0.5 * cd, cg0 = c == 1 ? 0.5 * cg : cg;
    const R gN = (R)(-sp.g_b), zN = (R)(-sp.z_b), rA = (R)sp.rkA;
    const double BC = sp.B_C;
    // the (0,0) mode's extra terms of u and w: nu U'' of the base flow in L and in the scheme's constant,
    // and the pressure-gradient / bulk-velocity term of the n = 0 row
    const bool extra = m00 && part == 0 && c != 1;
    const double dP = c == 0 ? sp.dPdxRef : sp.dPdzRef;
    const double e0L = sp.constraint == 0 ? dP : wall + sp.baseShear[c == 0 ? 0 : 1];
    const double e0 = aL * e0L + (sp.constraint == 0 ? dP : 0.0);
    const double* Byy = c == 0 ? P.Ubaseyy + fb : P.Wbaseyy + fb;
    // The (0,0) mode's terms are compiled only into the sweep of the warp that holds that mode: lanes whose
    // predicate is off still take the warp's FP64 slot of a predicated instruction.
    auto sweep = [&](auto KIND, auto EXTRA) {
      constexpr int kind = decltype(KIND)::value;
      constexpr bool has_extra = decltype(EXTRA)::value;
      double d2n2 = 0.0, dqn2 = 0.0;
      struct Batch {
        double uv[RB], qv[RB];
        R nv[RB], n1v[RB];
      };
      auto ld = [&](int i0, Batch& b) {
#pragma unroll
        for (int k = 0; k < RB; ++k) {
          const int i = i0 - k;
          if (i >= 0) {
            const int n = 2 * i + q;
            b.uv[k] = uc[i];
            b.qv[k] = c == 1 ? ((n + 1 <= Nb) ? qo[i + q] : 0.0) : qp[i];
            b.nv[k] = Nj[(size_t)i * 2 * row];
            b.n1v[k] = kind == 1 ? Nj1[(size_t)i * 2 * row] : Q[(size_t)i * 2 * row];
          }
        }
      };
      auto run = [&](int i0, const Batch& b) {
#pragma unroll
        for (int k = 0; k < RB; ++k) {
          const int i = i0 - k;
          if (i >= 0) {
            const double* uv = b.uv;
            const double* qv = b.qv;
            const R* nv = b.nv;
            const R* n1v = b.n1v;
            const int n = 2 * i + q;
            const double x1 = (n + 1 <= Nb) ? d1o[i + q] : 0.0;
            const double d2 = d2n2 + ct[n] * x1;
            d2n2 = d2;
            double gv = qv[k];
            if (c == 1) {
              gv = dqn2 + ct[n] * qv[k];
              dqn2 = gv;
            }
            // the nonlinear terms are combined at their own precision R (FP32 on the mixed path)
            double Nc;
            if (kind == 1) {
              Nc = widen(gN * nv[k] + zN * n1v[k]);
            } else {
              const R Qn = n1v[k] * rA - nv[k];
              if (act) Q[(size_t)i * 2 * row] = Qn;
              Nc = BC * widen(Qn);
            }
            const bool n0 = n == 0;
            double rhs = fma(cu, uv[k], fma(n0 ? cd0 : cd, d2, fma(n0 ? cg0 : cg, gv, Nc)));
            if (has_extra && extra) rhs += (aL + 1.0) * (nu * Byy[n]) - (n0 ? e0 : 0.0);
            if (act) out[i] = rhs;
          }
        }
      };
      Batch A, B;
      ld(M - 1, A);
      for (int i0 = M - 1; i0 >= 0; i0 -= 2 * RB) {
        if (i0 - RB >= 0) ld(i0 - RB, B);
        run(i0, A);
        if (i0 - RB < 0) break;
        if (i0 - 2 * RB >= 0) ld(i0 - 2 * RB, A);
        run(i0 - RB, B);
      }
    };
    const bool warp_extra = __any_sync(0xffffffffu, extra);
    if (sp.kind == 1) {
      if (warp_extra)
        sweep(std::integral_constant<int, 1>{}, std::true_type{});
      else
        sweep(std::integral_constant<int, 1>{}, std::false_type{});
    } else {
      if (warp_extra)
        sweep(std::integral_constant<int, 2>{}, std::true_type{});
      else
        sweep(std::integral_constant<int, 2>{}, std::false_type{});
    }
  }
  __syncwarp(gmask);
  __threadfence_block();

}

template <typename R>
__global__ void __launch_bounds__(32) k_tau_solve_t(GridDev g, int N, SolveParams sp, SolvePtrs P, HelmB hb,
                                                    TauTable tt) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x;
  const int t = blockIdx.x * 32 + lane;
  const int Md = g.Md;
  const bool act = (t >> 2) < Md;
  const int m = act ? (t >> 2) : Md - 1;
  const int mi = lane >> 2;  // mode within the warp
  const int mbase = blockIdx.x * 8;
  const int part = (t >> 1) & 1, q = t & 1;
  const unsigned gmask = 0xFu << (lane & 28);
  const int row = 2 * Md;
  const size_t comp = (size_t)row * N;
  const int off = 2 * m + part, poff = 2 * m + (1 - part);
  const size_t FN = (size_t)N * Md;
  const int M0 = (N - 1) / 2 + 1;
  const int M = q ? (N - 1) / 2 : M0;
  const int Nb = N - 1;
  const double scale = 4.0 / (g.b - g.a);
  double* ct = sm;
  double* lines = sm + ((N + 1) & ~1);
  double* tab = lines + (size_t)4 * M0 * 32;  // [4][N][8]
  for (int n = lane; n < N; n += 32) ct[n] = scale * (n + 1);
  __syncwarp();
  auto S = [&](int slot) { return SLn{lines + (size_t)slot * M0 * 32 + lane}; };
  auto So = [&](int slot) { return SLn{lines + (size_t)slot * M0 * 32 + (lane ^ 1)}; };
  auto Sp = [&](int slot) { return SLn{lines + (size_t)slot * M0 * 32 + (lane ^ 2)}; };
  auto G = [&](const double* base) { return PLn{const_cast<double*>(base) + off + q * row, 2 * row}; };
  auto Go = [&](const double* base) { return PLn{const_cast<double*>(base) + off + (1 - q) * row, 2 * row}; };
  auto Gp = [&](const double* base) { return PLn{const_cast<double*>(base) + poff + q * row, 2 * row}; };
  auto TS = [&](int k) { return TLn{tab + ((size_t)k * N + q) * 8 + mi}; };
  // stage factor fields f0..f3 of this warp's 8 modes into tab
  // (lane l copies mode mbase + l % 8 of rows n = l / 8 + 4 j: entry [k][n][l % 8] = tab[k N 8 + l + 32 j])
  // All copies of a staging are issued asynchronously (cp.async, zero fill past the last mode) and waited
  // for together: one memory latency per staging instead of one per batch of loads.
  auto stage = [&](int f0, int nf) {
    __syncwarp();
    const bool mok = mbase + (lane & 7) < Md;
    const int nb = mok ? 8 : 0;
    for (int k = 0; k < nf; ++k) {
      const double* src = mok ? tt.f + (size_t)(f0 + k) * FN + mbase + (lane & 7) + (size_t)(lane >> 3) * Md : tt.f;
      const size_t step = mok ? (size_t)4 * Md : 0;
      double* dst = tab + (size_t)k * N * 8 + lane;
      for (int n = lane >> 3; n < N; n += 4) {
        cp_async8(dst, src, nb);
        src += step;
        dst += 32;
      }
    }
    cp_async_wait_all();
    __syncwarp();
  };
  double* Rxg = P.scratch;          // global scratch lines for Rx and Rz
  double* Rzg = P.scratch + comp;
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = (kx == 0 && kz == 0);
  const double kxL = 2 * M_PI * kx / g.Lx;
  const double kzL = 2 * M_PI * kz / g.Lz;
  const int fld = mode_field(g, m);
  if (P.slot) apply_slot(sp, P.slot[fld]);
  const double nu = sp.nu;
  const double lambda = tt.s[TS_LAMBDA * Md + m];
  const double* __restrict__ hlo = hb.lo;
  const double* __restrict__ hdi = hb.di;
  const double* __restrict__ hup = hb.up;

  // ---- A: right-hand side (k_tau_rhs): Rx, Rz in scratch lines 0, 1; Ry (line 2) into slot 0 ------
  {
    // batches of 2 TCH loads in flight (one warp per SM sub-partition: nothing else hides their latency)
    PLn Ryg = G(P.scratch + 2 * comp);
    SLn outy = S(0);
    for (int i = 0; i < M; i += 2 * TCH) {
      double v[2 * TCH];
#pragma unroll
      for (int k = 0; k < 2 * TCH; ++k)
        if (i + k < M) v[k] = Ryg[i + k];
#pragma unroll
      for (int k = 0; k < 2 * TCH; ++k)
        if (i + k < M) outy[i + k] = v[k];
    }
  }
  __syncwarp(gmask);
  __threadfence_block();

  // ---- B: pressure ---------------------------------------------------------
  stage(TF_PBAND, 4);
  {
    SLn rr = S(2);
    diff_s(M, q, ct, So(0), &rr);
    PLn Rxp = Gp(Rxg), Rzp = Gp(Rzg);
    for (int i = 0; i < M; i += 2 * TCH) {
      double xa[2 * TCH], za[2 * TCH];
#pragma unroll
      for (int k = 0; k < 2 * TCH; ++k)
        if (i + k < M) {
          xa[k] = Rxp[i + k];
          za[k] = Rzp[i + k];
        }
#pragma unroll
      for (int k = 0; k < 2 * TCH; ++k)
        if (i + k < M) {
          const double x = kxL * xa[k] + kzL * za[k];
          rr[i + k] = part == 0 ? rr[i + k] - x : rr[i + k] + x;
        }
    }
    helm_t(M, q, hlo, hdi, hup, TS(0), TS(1), TS(2), TS(3), rr, S(1), 0.0);
  }
  stage(TF_VBAND, 4);
  // ---- C: wall-normal velocity, influence and tau corrections -------------
  SLn Pl = S(1), Vl = S(0);
  const double RyTop = S(0)[M - 1];
  if (m00) {
    for (int i = 0; i < M; ++i) Vl[i] = 0.0;
  } else {
    SLn tmp = S(3);
    diff_s(M, q, ct, So(1), &tmp);
    SLn Ry = S(0);
    for (int i = 0; i < M; ++i) tmp[i] -= Ry[i];
    helm_t(M, q, hlo, hdi, hup, TS(0), TS(1), TS(2), TS(3), tmp, Vl, 0.0);
  }
  __syncwarp(gmask);
  {
    const double s = m00 ? 0.0 : diff_s(M, q, ct, So(0), nullptr);
    const double so = __shfl_xor_sync(gmask, s, 1);
    const double s0 = q == 0 ? s : so, s1 = q == 0 ? so : s;
    const double plus = s0 + s1, minus = s0 - s1;
    const double* sc = tt.s + m;
    const double i00 = sc[TS_I00 * Md], i01 = sc[TS_I01 * Md], i10 = sc[TS_I10 * Md], i11 = sc[TS_I11 * Md];
    const double dp = -i00 * plus - i01 * minus;
    const double dm = -i10 * plus - i11 * minus;
    // influence solutions P+-, V+- staged like the factors (the V factors are no longer needed)
    stage(TF_PP, 4);
    const TLn Pp = TS(0), Vp = TS(1), Pm = TS(2), Vm = TS(3);
    if (!m00)
      for (int i = 0; i < M; i += TCH) {
        double a[TCH], b[TCH], c2[TCH], d[TCH];
#pragma unroll
        for (int k = 0; k < TCH; ++k)
          if (i + k < M) {
            a[k] = Pp[i + k];
            b[k] = Pm[i + k];
            c2[k] = Vp[i + k];
            d[k] = Vm[i + k];
          }
#pragma unroll
        for (int k = 0; k < TCH; ++k)
          if (i + k < M) {
            Pl[i + k] += dp * a[k] + dm * b[k];
            Vl[i + k] += dp * c2[k] + dm * d[k];
          }
      }
    const int itop = M - 1;
    double x0 = 0.0, y0 = 0.0;
    if (!m00) {
      x0 = lambda * Vl[itop] - nu * 0.0 - RyTop;
      y0 = q == 0 ? ct[Nb - 1] * Pl[itop] : 0.0;
    }
    const double ox = __shfl_xor_sync(gmask, x0, 1);
    const double oy = __shfl_xor_sync(gmask, y0, 1);
    if (sp.taucorrection) stage(TF_P0, 2);  // tau-correction solutions P0, V0
    if (!m00 && sp.taucorrection) {
      const double s1Nb = (q == 0 ? x0 : ox) + 0.0;
      const double s1Nb1 = q == 0 ? ox + y0 : x0 + oy;
      const double sNb = s1Nb / (1.0 - sc[TS_S0NB * Md]);
      const double sNb1 = s1Nb1 / (1.0 - sc[TS_S0NB1 * Md]);
      const TLn P0 = TS(0), V0 = TS(1);
      const double fP = q == 0 ? sNb1 : sNb, fV = q == 0 ? sNb : sNb1;
      for (int i = 0; i < M; i += TCH) {
        double a[TCH], b[TCH];
#pragma unroll
        for (int k = 0; k < TCH; ++k)
          if (i + k < M) {
            a[k] = P0[i + k];
            b[k] = V0[i + k];
          }
#pragma unroll
        for (int k = 0; k < TCH; ++k)
          if (i + k < M) {
            Pl[i + k] += fP * a[k];
            Vl[i + k] += fV * b[k];
          }
      }
    }
  }
  __syncwarp(gmask);
  // ---- D: streamwise and spanwise velocity in k_tau_uw (reads q from qout) ----
  const bool zero_im = m00 && part == 1 && sp.force_real00;
  if (act) {
    PLn gq = G(P.qout), gv = G(P.uout + comp);
    for (int i = 0; i < M; ++i) {
      gq[i] = zero_im ? 0.0 : Pl[i];
      gv[i] = zero_im ? 0.0 : Vl[i];
    }
  }
}

// ---------------------------------------------------------------------------
// Streamwise and spanwise velocity of the step solve (the u and w Helmholtz
// solves of TauSolver::solve, tausolver.cpp:347-402, and the mean-constrained
// solve of the (0,0) mode, helmholtz.cpp:158-213): one group of four lanes per
// (mode, u or w), four modes per warp, from the pressure the solve kernel wrote
// to qout and Rx, Rz in the scratch lines.  The solves run in place in one
// shared-memory line per lane; the velocity factors of the warp's modes are
// staged in shared memory.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(32) k_tau_uw(GridDev g, int N, SolveParams sp, SolvePtrs P, HelmB hb,
                                               TauTable tt) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x;
  const int t = blockIdx.x * 32 + lane;
  const int Md = g.Md;
  const int grp = t >> 2;
  const bool act = grp < 2 * Md;
  const int m = act ? grp >> 1 : Md - 1;
  const int cu = act ? (grp & 1) : 0;  // 0: u, 1: w
  const int mi = lane >> 3;            // mode within the warp
  const int mbase = blockIdx.x * 4;
  const int part = (t >> 1) & 1, q = t & 1;
  const int row = 2 * Md;
  const size_t comp = (size_t)row * N;
  const int off = 2 * m + part, poff = 2 * m + (1 - part);
  const size_t FN = (size_t)N * Md;
  const int M0 = (N - 1) / 2 + 1;
  const int M = q ? (N - 1) / 2 : M0;
  double* tab = sm + (size_t)M0 * 32;  // [4][N][4]
  {
    // lane l copies mode mbase + l % 4 of rows n = l / 4 + 8 j: entry [k][n][l % 4] = tab[k N 4 + l + 32 j];
    // all copies asynchronous (cp.async, zero fill past the last mode), waited for together
    const bool mok = mbase + (lane & 3) < Md;
    const int nb = mok ? 8 : 0;
    for (int k = 0; k < 4; ++k) {
      const double* src =
          mok ? tt.f + (size_t)(TF_VBAND + k) * FN + mbase + (lane & 3) + (size_t)(lane >> 2) * Md : tt.f;
      const size_t step = mok ? (size_t)8 * Md : 0;
      double* dst = tab + (size_t)k * N * 4 + lane;
      for (int n = lane >> 2; n < N; n += 8) {
        cp_async8(dst, src, nb);
        src += step;
        dst += 32;
      }
    }
    cp_async_wait_all();
  }
  __syncwarp();
  auto TS = [&](int k) { return TLn4{tab + ((size_t)k * N + q) * 4 + mi}; };
  auto G = [&](const double* base) { return PLn{const_cast<double*>(base) + off + q * row, 2 * row}; };
  auto Gp = [&](const double* base) { return PLn{const_cast<double*>(base) + poff + q * row, 2 * row}; };
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = (kx == 0 && kz == 0);
  const int fld = mode_field(g, m);
  if (P.slot) apply_slot(sp, P.slot[fld]);
  const double nu = sp.nu;
  const double kL = cu == 0 ? 2 * M_PI * kx / g.Lx : 2 * M_PI * kz / g.Lz;
  const bool zero_im = m00 && part == 1 && sp.force_real00;
  SLn r{sm + lane};
  PLn Rc = G(P.scratch + (cu == 0 ? 0 : comp));
  PLn Pp = Gp(P.qout);
  const double sk = part == 0 ? -kL : kL;  // the part's sign of i k
  auto fill = [&]() {
    for (int i = 0; i < M; i += 2 * TCH) {
      double rv[2 * TCH], pv[2 * TCH];
#pragma unroll
      for (int k = 0; k < 2 * TCH; ++k)
        if (i + k < M) {
          rv[k] = Rc[i + k];
          pv[k] = Pp[i + k];
        }
#pragma unroll
      for (int k = 0; k < 2 * TCH; ++k)
        if (i + k < M) r[i + k] = fma(sk, pv[k], -rv[k]);
    }
  };
  fill();
  helm_t(M, q, hb.lo, hb.di, hb.up, TS(0), TS(1), TS(2), TS(3), r, r, 0.0);
  if (m00 && sp.constraint == 1 && part == 0 && q == 0) {
    // mean-constrained solve of the real part (the mean involves even n only)
    double amean = r[0];
    for (int i = 1; i < M; ++i) amean -= r[i] / (double)((2 * i) * (2 * i) - 1);
    const double ucmean = tt.s[TS_UCMEAN * Md + m];
    const double target = cu == 0 ? sp.umean : sp.wmean;
    const double mu = nu * (target - amean) / ucmean;
    fill();
    r[0] = r[0] + mu;
    helm_t(M, q, hb.lo, hb.di, hb.up, TS(0), TS(1), TS(2), TS(3), r, r, 0.0);
    if (act && P.dPdx_out) P.dPdx_out[2 * mode_field(g, m) + cu] = mu;
  }
  if (act) {
    PLn gout = G(P.uout + (cu == 0 ? 0 : 2) * comp);
    for (int i = 0; i < M; ++i) gout[i] = zero_im ? 0.0 : r[i];
  }
}

static size_t tau_t_smem(int N) {
  const int M0 = (N - 1) / 2 + 1;
  return sizeof(double) * (((N + 1) & ~1) + (size_t)4 * M0 * 32 + (size_t)4 * N * 8);
}

int tau_solve_launches(int N) { return tau_t_smem(N) <= 227 * 1024 ? 3 : 1; }

static std::atomic<int> g_tau_seg{1};
void set_tau_segmented(int enable) { g_tau_seg.store(enable ? 1 : 0); }

template <typename R>
cudaError_t launch_tau_solve(const GridDev& g, int N, const SolveParams& sp, const SolvePtrs& p, const HelmB& hb,
                             TauTable tt, cudaStream_t st) {
  const int M0 = (N - 1) / 2 + 1;
  const size_t smem_t = tau_t_smem(N);
  if (g_tau_seg.load() != 0 && tau_seg_rows(N) <= 17) {
    // right-hand side (one lane per parity sweep: its derivative recurrences cost twice the FP64 operations
    // when segmented, and it is FP64-bound already), then the pressure / v and the u / w passes with
    // segmented sweeps (tau_seg.cu)
    static const bool attr = [] {
      cudaFuncSetAttribute(k_tau_rhs<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      return true;
    }();
    (void)attr;
    const size_t smem_r = sizeof(double) * (((N + 1) & ~1) + (size_t)M0 * 32);
    cudaError_t e = launch_pdl(k_tau_rhs<R>, dim3((4 * g.Md + 31) / 32, 3), dim3(32), smem_r, st, g, N, sp, p, tt);
    if (e != cudaSuccess) return e;
    return launch_tau_pvuw_seg(g, N, sp, p, hb, tt, st);
  }
  if (smem_t <= 227 * 1024) {
    // kernel attributes set once per process (thread-safe static initialisation)
    static const bool attr = [] {
      cudaFuncSetAttribute(k_tau_solve_t<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      // tall grids take more than the default 48 KB in the right-hand-side and u/w kernels too
      cudaFuncSetAttribute(k_tau_rhs<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      cudaFuncSetAttribute(k_tau_uw<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      return true;
    }();
    (void)attr;
    const size_t smem_r = sizeof(double) * (((N + 1) & ~1) + (size_t)M0 * 32);
    k_tau_rhs<R><<<dim3((4 * g.Md + 31) / 32, 3), 32, smem_r, st>>>(g, N, sp, p, tt);
    k_tau_solve_t<R><<<(4 * g.Md + 31) / 32, 32, smem_t, st>>>(g, N, sp, p, hb, tt);
    const size_t smem_u = sizeof(double) * ((size_t)M0 * 32 + (size_t)4 * N * 4);
    k_tau_uw<R><<<(8 * g.Md + 31) / 32, 32, smem_u, st>>>(g, N, sp, p, hb, tt);
    return cudaGetLastError();
  }
  const int T = 64;
  k_tau_solve<R><<<(4 * g.Md + T - 1) / T, T, 0, st>>>(g, N, sp, p, hb, tt);
  return cudaGetLastError();
}

template cudaError_t launch_tau_solve<float>(const GridDev&, int, const SolveParams&, const SolvePtrs&, const HelmB&,
                                             TauTable, cudaStream_t);
template cudaError_t launch_tau_solve<double>(const GridDev&, int, const SolveParams&, const SolvePtrs&, const HelmB&,
                                              TauTable, cudaStream_t);
