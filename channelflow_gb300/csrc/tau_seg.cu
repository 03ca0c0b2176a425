// Step solve of the DNS (TauSolver::solve per mode) with every parity sweep split over four lanes.
//
// Restates, for the pressure / wall-normal velocity pass and the streamwise / spanwise velocity pass:
//   HelmholtzSolver::solve                 channelflow/helmholtz.cpp:79-95, solve(mean) 158-213
//   BandedTridiag::ULsolveStrided          channelflow/bandedtridiag.cpp:232-277
//   TauSolver::solve_P_and_v / solve       channelflow/tausolver.cpp:193-251, 347-402
//   TauSolver::influenceCorrection         channelflow/tausolver.cpp:178-191
//   diff (Chebyshev derivative)            channelflow/chebyshev.cpp:672-697
// The UL factors, influence and tau-correction solutions of every mode are precomputed (k_tau_setup).
//
// GB300 mapping.  The FP64 pipe takes 64 cycles per warp instruction, and a serial sweep of N/2 rows per lane
// leaves one warp per SM sub-partition at the benchmark size, so the solve is bound by the latency of one
// warp's dependent chain.  Here 16 lanes work on a mode: (re/im part) x (parity) x 4 segments of the parity's
// rows.  Each sweep is a first-order linear recurrence x_i = c_i - a_i x_{i+-1} with known a_i: a segment
// runs it from a zero start (particular part p) together with the product of the -a_i (homogeneous part h),
// the segments' boundary values follow from three shuffle rounds, and x_i = p_i + h_i X (X: the boundary value
// below / above the segment).  The derivative recurrence d_n = d_{n+2} + (4/L)(n+1) x_{n+1} is a suffix sum:
// segment totals are combined by shuffles.  Vectors live in registers (L rows per lane); a per-warp shared
// line of N values per (mode, part) carries the neighbour rows a lane reads (B multiply, derivative, the
// other parity) and stages coalesced global loads and stores.  With the segment products precomputed per mode
// (k_tau_setup), 9 FP64 operations per row per Helmholtz solve against 7 for the serial sweep, on four times
// the lanes and a quarter of the chain.
#include "kernels.h"

namespace {

constexpr int SEG = 4;  // segments per parity system

// This lane's part of a parity system: parity q, segment s, rows i0 .. i0 + L - 1 (of the M rows).
struct Seg {
  int q, s, M, i0, N;
};

// Sum over the four segment lanes.
__device__ __forceinline__ double seg_sum(double v, unsigned mask) {
  v += __shfl_xor_sync(mask, v, 1);
  v += __shfl_xor_sync(mask, v, 2);
  return v;
}

// Sum of v over the segments above this one (s + 1 .. SEG - 1).
__device__ __forceinline__ double seg_above(double v, int s, unsigned mask) {
  double x = __shfl_down_sync(mask, v, 1, SEG);
  x = s + 1 < SEG ? x : 0.0;
  double t = __shfl_down_sync(mask, x, 1, SEG);
  if (s + 1 < SEG) x += t;
  t = __shfl_down_sync(mask, x, 2, SEG);
  if (s + 2 < SEG) x += t;
  return x;
}

// This lane's rows of x into the (mode, part) line (index n = 2 i + q).
template <int L>
__device__ __forceinline__ void put(const Seg& c, double* line, const double (&x)[L], unsigned mask) {
  __syncwarp(mask);
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const int i = c.i0 + k;
    if (i < c.M) line[2 * i + c.q] = x[k];
  }
  __syncwarp(mask);
}

// d = diff(x) on this lane's rows, x (both parities) in line; ct[n] = (4/L)(n + 1).
template <int L>
__device__ __forceinline__ void seg_diff(const Seg& c, const double* line, const double* ct, double (&d)[L],
                                         unsigned mask) {
  double acc = 0.0;
#pragma unroll
  for (int k = L - 1; k >= 0; --k) {
    const int i = c.i0 + k, n = 2 * i + c.q;
    if (i < c.M && n + 1 < c.N) acc = fma(ct[n], line[n + 1], acc);
    d[k] = acc;
  }
  const double off = seg_above(acc, c.s, mask);
#pragma unroll
  for (int k = 0; k < L; ++k) d[k] += off;
  if (c.q == 0 && c.s == 0) d[0] *= 0.5;
}

// u = A^{-1} B f for this lane's rows of the parity system (HelmholtzSolver::solve with u(a) = u(b) = 0 and
// row 0 of the system set to bc): f (this parity) in line; band/up/lo/inv: the mode's UL-factor columns, H/G
// their segment products, element n at [n * ts].
template <int L>
__device__ __forceinline__ void seg_helm(const Seg& c, const double* line, const HelmB& hb, const double* band,
                                         const double* up, const double* lo, const double* inv, const double* H,
                                         const double* G, size_t ts, double bc, double (&u)[L], unsigned mask) {
  // descending: u_i = (B f)_i - up_i u_{i+1}, rows M-1 .. 1, from zero above the segment
  double p = 0.0;
  int nf = -1;  // first (lowest) row of the segment in the sweep
#pragma unroll
  for (int k = L - 1; k >= 0; --k) {
    const int i = c.i0 + k, n = 2 * i + c.q;
    u[k] = 0.0;
    if (i >= 1 && i < c.M) {
      const double bf =
          fma(__ldg(hb.up + n), line[n + 2], fma(__ldg(hb.di + n), line[n], __ldg(hb.lo + n) * line[n - 2]));
      p = fma(-__ldg(up + n * ts), p, bf);
      u[k] = p;
      nf = n;
    }
  }
  const double hf = nf >= 0 ? __ldg(H + nf * ts) : 1.0;
  double X = 0.0;  // u at the first row of the segment above
#pragma unroll
  for (int r = 0; r < SEG - 1; ++r) {
    const double t = __shfl_down_sync(mask, fma(hf, X, p), 1, SEG);
    X = c.s + 1 < SEG ? t : 0.0;
  }
  double bs = 0.0;
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const int i = c.i0 + k, n = 2 * i + c.q;
    if (i >= 1 && i < c.M) {
      u[k] = fma(__ldg(H + n * ts), X, u[k]);
      bs = fma(__ldg(band + n * ts), u[k], bs);
    }
  }
  bs = seg_sum(bs, mask);
  // row 0 (inv holds 1 / band at row 0), then ascending: u_i = (u_i - lo_i u_{i-1}) inv_i from zero below the
  // segment
  double pa = 0.0;
  if (c.s == 0) {
    u[0] = (bc - bs) * __ldg(inv + c.q * ts);
    pa = u[0];
  }
  int nl = -1;  // last row of the segment in the sweep
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const int i = c.i0 + k, n = 2 * i + c.q;
    if (i >= 1 && i < c.M) {
      pa = fma(-__ldg(lo + n * ts), pa, u[k]) * __ldg(inv + n * ts);
      u[k] = pa;
      nl = n;
    }
  }
  const double gl = c.s > 0 && nl >= 0 ? __ldg(G + nl * ts) : 1.0;
  X = 0.0;  // u at the last row of the segment below
#pragma unroll
  for (int r = 0; r < SEG - 1; ++r) {
    const double t = __shfl_up_sync(mask, fma(gl, X, pa), 1, SEG);
    X = c.s > 0 ? t : 0.0;
  }
  if (c.s > 0) {
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const int i = c.i0 + k, n = 2 * i + c.q;
      if (i < c.M) u[k] = fma(__ldg(G + n * ts), X, u[k]);
    }
  }
}

// Asynchronous copy of the solved-mode lines of modes mbase, mbase + 1 (both parts) of a [n][2 Md] array into
// the warp's four lines [(mode, part)][stride ls] (cp.async, zero fill past the last mode); the caller waits.
__device__ __forceinline__ void stage_lines(const double* src, int Md, int mbase, int N, double* lines, size_t ls,
                                            int lane) {
  const size_t row = 2 * (size_t)Md;
  for (int idx = lane; idx < 4 * N; idx += 32) {
    const int n = idx >> 2, cc = idx & 3, m = mbase + (cc >> 1);
    cp_async8(lines + cc * ls + n, m < Md ? src + n * row + 2 * (size_t)m + (cc & 1) : src, m < Md ? 8 : 0);
  }
}
// zero[j]: mode mbase + j is a (0,0) mode whose imaginary part is set to zero.
__device__ __forceinline__ void store_lines(double* dst, int Md, int mbase, int N, const double* lines, size_t ls,
                                            int lane, const bool (&zero)[2]) {
  __syncwarp();
  const size_t row = 2 * (size_t)Md;
  for (int idx = lane; idx < 4 * N; idx += 32) {
    const int n = idx >> 2, cc = idx & 3, m = mbase + (cc >> 1);
    if (m < Md) dst[n * row + 2 * (size_t)m + (cc & 1)] = (zero[cc >> 1] && (cc & 1)) ? 0.0 : lines[cc * ls + n];
  }
}

// ---------------------------------------------------------------------------
// Pressure and wall-normal velocity (TauSolver::solve_P_and_v for the real and imaginary parts) from the
// right-hand sides Rx, Rz, Ry in scratch lines 0, 1, 2; writes q and v.  One warp: two modes (lanes 16 ml +
// 8 part + 4 q + s).
// ---------------------------------------------------------------------------
template <int L>
__global__ void __launch_bounds__(32, 12) k_tau_pv_seg(GridDev g, int N, SolveParams sp, SolvePtrs P, HelmB hb,
                                                   TauTable tt) {
  extern __shared__ double sm[];
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x;
  const int ml = lane >> 4, part = (lane >> 3) & 1, q = (lane >> 2) & 1, s = lane & 3;
  const int Md = g.Md;
  const int mbase = blockIdx.x * 2;
  const int m = min(mbase + ml, Md - 1);
  const unsigned full = 0xffffffffu;
  const size_t NL = (size_t)N + 2;
  const size_t comp = 2 * (size_t)Md * N;
  const size_t FN = (size_t)N * Md;
  double* ct = sm;
  double* lA = ct + NL;      // [4][NL]: per (mode, part)
  double* lB = lA + 4 * NL;  // [4][NL]
  double* lC = lB + 4 * NL;  // [4][NL]
  double* sc = lC + 4 * NL;  // [4][4] top-row scalars
  const int cc = ml * 2 + part;
  double* a = lA + cc * NL;
  double* b = lB + cc * NL;
  // Ry, Rx, Rz of the warp's modes in flight together; the lines' two padding entries are zero
  stage_lines(P.scratch + 2 * comp, Md, mbase, N, lA, NL, lane);
  stage_lines(P.scratch, Md, mbase, N, lB, NL, lane);
  stage_lines(P.scratch + comp, Md, mbase, N, lC, NL, lane);
  const double scale = 4.0 / (g.b - g.a);
  for (int n = lane; n < N; n += 32) ct[n] = scale * (n + 1);
  if (lane < 24) lA[(lane >> 1) * NL + N + (lane & 1)] = 0.0;
  cp_async_wait_all();
  __syncwarp();
  const Seg c{q, s, q ? (N - 1) / 2 : (N + 1) / 2, s * L, N};
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = kx == 0 && kz == 0;
  const double* ts = tt.s + m;
  // the part's sign of i k folded into the wavenumbers (one FP64 add per row below, not two and a select)
  const double kxL = part == 0 ? -ts[TS_KXL * Md] : ts[TS_KXL * Md];
  const double kzL = part == 0 ? -ts[TS_KZL * Md] : ts[TS_KZL * Md];

  // right-hand sides: Ry (own part) and -/+ (kx Rx + kz Rz) of the other part
  double ry[L], x[L], w[L];
#pragma unroll
  for (int k = 0; k < L; ++k) ry[k] = c.i0 + k < c.M ? a[2 * (c.i0 + k) + q] : 0.0;
  const double ryTop = a[2 * (c.M - 1) + q];
  const double* bo = lB + (cc ^ 1) * NL;
  const double* co = lC + (cc ^ 1) * NL;
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const int n = 2 * (c.i0 + k) + q;
    w[k] = c.i0 + k < c.M ? fma(kzL, co[n], kxL * bo[n]) : 0.0;
  }
  // rr = diff(Ry) -/+ (kx Rx + kz Rz) of the other part
  seg_diff<L>(c, a, ct, x, full);
#pragma unroll
  for (int k = 0; k < L; ++k) x[k] += w[k];
  // P = pH^{-1} rr
  put<L>(c, b, x, full);
  const double* tf = tt.f + m;
  seg_helm<L>(c, b, hb, tf + TF_PBAND * FN, tf + TF_PUP * FN, tf + TF_PLO * FN, tf + TF_PINV * FN,
              tf + TF_PH * FN, tf + TF_PG * FN, Md, 0.0, w, full);
  // v = vH^{-1} (diff(P) - Ry)
  put<L>(c, b, w, full);
  seg_diff<L>(c, b, ct, x, full);
#pragma unroll
  for (int k = 0; k < L; ++k) x[k] -= ry[k];
  put<L>(c, a, x, full);
  seg_helm<L>(c, a, hb, tf + TF_VBAND * FN, tf + TF_VUP * FN, tf + TF_VLO * FN, tf + TF_VINV * FN,
              tf + TF_VH * FN, tf + TF_VG * FN, Md, 0.0, ry, full);  // ry now holds v
  // influence correction: the wall values of diff(v) (sums over each parity)
  put<L>(c, b, ry, full);
  seg_diff<L>(c, b, ct, x, full);
  double sq = 0.0;
#pragma unroll
  for (int k = 0; k < L; ++k)
    if (c.i0 + k < c.M) sq += x[k];
  sq = seg_sum(sq, full);
  const double so = __shfl_xor_sync(full, sq, 4);
  const double s0 = q == 0 ? sq : so, s1 = q == 0 ? so : sq;
  const double plus = s0 + s1, minus = s0 - s1;
  const double dp = -ts[TS_I00 * Md] * plus - ts[TS_I01 * Md] * minus;
  const double dm = -ts[TS_I10 * Md] * plus - ts[TS_I11 * Md] * minus;
  // (the (0,0) mode has no influence or tau correction and v = 0)
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const int i = c.i0 + k, n = 2 * i + q;
    if (i < c.M && !m00) {
      const size_t o = (size_t)n * Md;
      w[k] = fma(dm, __ldg(tf + TF_PM * FN + o), fma(dp, __ldg(tf + TF_PP * FN + o), w[k]));
      ry[k] = fma(dm, __ldg(tf + TF_VM * FN + o), fma(dp, __ldg(tf + TF_VP * FN + o), ry[k]));
    }
  }
  // tau correction from the top rows of both parities
  if (sp.taucorrection) {
    const int itop = c.M - 1;
    if (itop >= c.i0 && itop < c.i0 + L) {
#pragma unroll
      for (int k = 0; k < L; ++k)
        if (c.i0 + k == itop) {
          sc[cc * 4 + q * 2] = ts[TS_LAMBDA * Md] * ry[k] - ryTop;
          sc[cc * 4 + q * 2 + 1] = q == 0 ? ct[N - 2] * w[k] : 0.0;
        }
    }
    __syncwarp();
    const double sNb = sc[cc * 4] * ts[TS_RS0NB * Md];
    const double sNb1 = (sc[cc * 4 + 2] + sc[cc * 4 + 1]) * ts[TS_RS0NB1 * Md];
    const double fP = q == 0 ? sNb1 : sNb, fV = q == 0 ? sNb : sNb1;
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const int i = c.i0 + k, n = 2 * i + q;
      if (i < c.M && !m00) {
        const size_t o = (size_t)n * Md;
        w[k] += fP * __ldg(tf + TF_P0 * FN + o);
        ry[k] += fV * __ldg(tf + TF_V0 * FN + o);
      }
    }
  }
  if (m00)
#pragma unroll
    for (int k = 0; k < L; ++k) ry[k] = 0.0;
  put<L>(c, a, w, full);
  put<L>(c, b, ry, full);
  bool zero[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int mj = min(mbase + j, Md - 1);
    zero[j] = sp.force_real00 && mode_kx(g, mj) == 0 && mode_kz(g, mj) == 0;
  }
  store_lines(P.qout, Md, mbase, N, lA, NL, lane, zero);
  store_lines(P.uout + comp, Md, mbase, N, lB, NL, lane, zero);
}

// ---------------------------------------------------------------------------
// Streamwise and spanwise velocity (the u and w Helmholtz solves of TauSolver::solve; the mean-constrained
// solve of the (0,0) mode's real part under the bulk-velocity constraint) from q and Rx, Rz.  One warp: one
// mode, u (lanes 0-15) and w (16-31).
// ---------------------------------------------------------------------------
template <int L>
__global__ void __launch_bounds__(32, 16) k_tau_uw_seg(GridDev g, int N, SolveParams sp, SolvePtrs P, HelmB hb,
                                                   TauTable tt) {
  extern __shared__ double sm[];
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x;
  const int cu = lane >> 4, part = (lane >> 3) & 1, q = (lane >> 2) & 1, s = lane & 3;
  const int Md = g.Md;
  const int m = blockIdx.x;
  const unsigned full = 0xffffffffu;
  const size_t NL = (size_t)N + 2;
  const size_t comp = 2 * (size_t)Md * N;
  const size_t FN = (size_t)N * Md;
  const size_t row = 2 * (size_t)Md;
  double* ql = sm;            // [2 parts][NL]: q
  double* rl = ql + 2 * NL;   // [2 comps][2 parts][NL]: right-hand side of the solve
  double* ol = rl + 4 * NL;   // [2 comps][2 parts][NL]: solution
  // q and Rx, Rz of the mode in flight together; the right-hand-side lines' padding entries are zero
  for (int idx = lane; idx < 2 * N; idx += 32) {
    const int n = idx >> 1, pt = idx & 1;
    cp_async8(ql + pt * NL + n, P.qout + n * row + 2 * (size_t)m + pt, 8);
  }
  for (int idx = lane; idx < 4 * N; idx += 32) {
    const int n = idx >> 2, c2 = idx >> 1 & 1, pt = idx & 1;
    cp_async8(rl + (c2 * 2 + pt) * NL + n, P.scratch + c2 * comp + n * row + 2 * (size_t)m + pt, 8);
  }
  if (lane < 8) rl[(lane >> 1) * NL + N + (lane & 1)] = 0.0;
  cp_async_wait_all();
  __syncwarp();
  const Seg c{q, s, q ? (N - 1) / 2 : (N + 1) / 2, s * L, N};
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const bool m00 = kx == 0 && kz == 0;
  if (P.slot) apply_slot(sp, P.slot[mode_field(g, m)]);
  const double kL = tt.s[(cu == 0 ? TS_KXL : TS_KZL) * Md + m];
  const double sk = part == 0 ? -kL : kL;  // the part's sign of i k
  double* r = rl + (cu * 2 + part) * NL;
  const double* qo = ql + (1 - part) * NL;
  // right-hand side i k q - R in place (this lane's rows), then the solve
  double u[L];
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const int n = 2 * (c.i0 + k) + q;
    u[k] = c.i0 + k < c.M ? fma(sk, qo[n], -r[n]) : 0.0;
  }
  put<L>(c, r, u, full);
  const double* tf = tt.f + m;
  // the mean-constrained solve of the (0,0) mode's real part (bulk velocity) solves again with row 0 of the
  // right-hand side raised by mu (the mean involves the even coefficients only); the whole warp repeats the
  // solve, the other parts and parities with unchanged right-hand sides
  const bool mean = m00 && sp.constraint == 1;
#pragma unroll 1
  for (int pass = 0; pass < (mean ? 2 : 1); ++pass) {
    seg_helm<L>(c, r, hb, tf + TF_VBAND * FN, tf + TF_VUP * FN, tf + TF_VLO * FN, tf + TF_VINV * FN,
                tf + TF_VH * FN, tf + TF_VG * FN, Md, 0.0, u, full);
    if (pass == 0 && mean) {
      double am = 0.0;
#pragma unroll
      for (int k = 0; k < L; ++k) {
        const int i = c.i0 + k;
        if (i >= 1 && i < c.M) am -= u[k] / (double)((2 * i) * (2 * i) - 1);
      }
      am = seg_sum(am, full);
      const double amean = __shfl_sync(full, u[0], lane & 28) + am;
      const double mu = sp.nu * ((cu == 0 ? sp.umean : sp.wmean) - amean) / tt.s[TS_UCMEAN * Md + m];
      __syncwarp();
      if (part == 0 && q == 0 && s == 0) {
        r[0] += mu;
        if (P.dPdx_out) P.dPdx_out[2 * mode_field(g, m) + cu] = mu;
      }
      __syncwarp();
    }
  }
  put<L>(c, ol + (cu * 2 + part) * NL, u, full);
  __syncwarp();
  const bool zero_im = m00 && sp.force_real00;
  for (int idx = lane; idx < 4 * N; idx += 32) {
    const int n = idx >> 2, c2 = idx >> 1 & 1, pt = idx & 1;
    P.uout[(c2 ? 2 : 0) * comp + n * row + 2 * (size_t)m + pt] = (zero_im && pt) ? 0.0 : ol[(c2 * 2 + pt) * NL + n];
  }
}

template <int L>
cudaError_t run_seg(const GridDev& g, int N, const SolveParams& sp, const SolvePtrs& p, const HelmB& hb,
                    TauTable tt, cudaStream_t st) {
  const size_t NL = (size_t)N + 2;
  const size_t smem_pv = sizeof(double) * (13 * NL + 16);
  const size_t smem_uw = sizeof(double) * (10 * NL);
  static const bool attr = [] {
    cudaFuncSetAttribute(k_tau_pv_seg<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    cudaFuncSetAttribute(k_tau_uw_seg<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    return true;
  }();
  (void)attr;
  cudaError_t e = launch_pdl(k_tau_pv_seg<L>, dim3((g.Md + 1) / 2), dim3(32), smem_pv, st, g, N, sp, p, hb, tt);
  if (e != cudaSuccess) return e;
  return launch_pdl(k_tau_uw_seg<L>, dim3(g.Md), dim3(32), smem_uw, st, g, N, sp, p, hb, tt);
}

}  // namespace

cudaError_t launch_tau_pvuw_seg(const GridDev& g, int N, const SolveParams& sp, const SolvePtrs& p,
                                const HelmB& hb, TauTable tt, cudaStream_t st) {
  switch (tau_seg_rows(N)) {
    case 2: return run_seg<2>(g, N, sp, p, hb, tt, st);
    case 3: return run_seg<3>(g, N, sp, p, hb, tt, st);
    case 4: return run_seg<4>(g, N, sp, p, hb, tt, st);
    case 5: return run_seg<5>(g, N, sp, p, hb, tt, st);
    case 6: return run_seg<6>(g, N, sp, p, hb, tt, st);
    case 7: return run_seg<7>(g, N, sp, p, hb, tt, st);
    case 8: return run_seg<8>(g, N, sp, p, hb, tt, st);
    case 9: return run_seg<9>(g, N, sp, p, hb, tt, st);
    case 10: return run_seg<10>(g, N, sp, p, hb, tt, st);
    case 11: return run_seg<11>(g, N, sp, p, hb, tt, st);
    case 12: return run_seg<12>(g, N, sp, p, hb, tt, st);
    case 13: return run_seg<13>(g, N, sp, p, hb, tt, st);
    case 14: return run_seg<14>(g, N, sp, p, hb, tt, st);
    case 15: return run_seg<15>(g, N, sp, p, hb, tt, st);
    case 16: return run_seg<16>(g, N, sp, p, hb, tt, st);
    case 17: return run_seg<17>(g, N, sp, p, hb, tt, st);
    default: return cudaErrorInvalidValue;
  }
}
