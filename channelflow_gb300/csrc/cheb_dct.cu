// Chebyshev transforms along y through the FFT (DCT-I), and the spectral curl that feeds the inverse one.
//
// Both directions of the Chebyshev transform on the Gauss-Lobatto grid y_j = cos(pi j / M), M = N - 1, are a
// DCT-I of the N values of a line (chebyfft / ichebyfft, chebyshev.cpp:262-303, which call FFTW's REDFT00):
//   inverse  u_k = sum_n a_n cos(pi n k / M)
//   forward  a_n = (c_n / M) [u_0 + (-1)^n u_M + 2 sum_{j=1}^{M-1} u_j cos(pi n j / M)],  c_0 = c_M = 1/2.
// With y_j = w_j x_j (w = 2 in the interior; 1 (forward) or 2 (inverse) at the ends) both are
//   X_k = y_0 + (-1)^k y_M + sum_{j=1}^{M-1} y_j cos(pi j k / M),
// scaled by c_k / M (forward) or 1/2 (inverse).  X is computed with one complex FFT of length M per mode:
//   a_j = s_j + sin(pi j / M) d_j,  a_{M-j} = s_j - sin(pi j / M) d_j   (s_j = x_j + x_{M-j}, d_j = x_j - x_{M-j},
//   a_0 = y_0 + y_M, a_{M/2} = y_{M/2}),  Z = DFT_M(a)  (sign -1),
//   X_{2k} = (Z_k + Z_{M-k}) / 2,
//   X_1 = y_0 - y_M + sum_{j=1}^{M/2-1} 2 cos(pi j / M) d_j,  X_{2k+1} = X_{2k-1} - i (Z_k - Z_{M-k}).
// (The sine term makes Re Z carry the even outputs and the odd outputs differences of Im Z; the relation is
// linear and real, so the real and imaginary parts of a complex mode are two real lines packed in one FFT.)
// Cost per real line: one complex FFT of length M shared by two lines plus O(M) pre- and post-processing,
// against (M/2)^2 fused multiply-adds per line for the parity-split matrix product.
#include <cmath>
#include <vector>

#include "fft_steps.cuh"
#include "kernels.h"

namespace {

using namespace fsr;

constexpr int DCT_THREADS = 256, DCT_NW = 8, DCT_TM = 32;  // 8 warps, 32 modes (one per lane) per block

// Sequence pitch (complex): at least 8 (N1 + 1) and 1 mod 8 (FP64) or 1 mod 16 (FP32), so lanes on
// consecutive sequences hit consecutive bank groups.
template <typename R, int N1>
__host__ __device__ constexpr int dct_pitch() {
  return 8 * (N1 + 1) + (((1 - 8 * (N1 + 1)) % (sizeof(R) == 8 ? 8 : 16)) + (sizeof(R) == 8 ? 8 : 16)) %
                            (sizeof(R) == 8 ? 8 : 16);
}

template <typename R, int N1>
__host__ __device__ constexpr size_t dct_smem() {
  return sizeof(cpx<R>) * ((size_t)DCT_TM * dct_pitch<R, N1>() + 8 * N1 + 4 * N1 + 1 + 2 * DCT_NW * DCT_TM);
}

// One block: 32 modes x one component (blockIdx.y) of a field; blocks never straddle fields (lpf modes each),
// so a block uses its field's version of the table.  Element (n, m) of a component at in[n ld_in + m].
// tab: exp(-2 pi i e / M), e < M, then (2 cos(pi j / M), sin(pi j / M)), j <= M / 2.
template <typename R, int N1, bool INV>
__global__ void __launch_bounds__(DCT_THREADS, 2)
    k_dct(int nmodes, int lpf, const cpx<R>* __restrict__ in, size_t ld_in, size_t cs_in, cpx<R>* __restrict__ out,
          size_t ld_out, size_t cs_out, const cpx<R>* __restrict__ tab, Dither dt) {
  constexpr int M = 8 * N1, H = M / 2, P = dct_pitch<R, N1>();
  constexpr int JI = (H + DCT_NW) / DCT_NW;  // point pairs (j, M - j), j <= H, per warp
  constexpr int KS = (H + DCT_NW) / DCT_NW;  // output pairs (2k, 2k + 1), k <= H, per warp
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<R>* seq = reinterpret_cast<cpx<R>*>(smem_raw);  // [32][P]
  cpx<R>* tw = seq + DCT_TM * P;                      // [M]
  cpx<R>* cs = tw + M;                                // [H + 1]
  cpx<R>* csp = cs + H + 1;                           // [8][32] X_1 partial sums
  cpx<R>* segt = csp + DCT_NW * DCT_TM;               // [8][32] odd-output segment sums
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int bpf = (lpf + DCT_TM - 1) / DCT_TM, fld = blockIdx.x / bpf;
  const int gm = fld * lpf + (blockIdx.x - fld * bpf) * DCT_TM + lane;
  const bool ok = gm < min(nmodes, (fld + 1) * lpf);
  const int ver = dither_ver(dt, fld);
  tab = dither_ptr(tab, ver, dt.S);
  for (int i = tid; i < M + H + 1; i += DCT_THREADS) tw[i] = tab[i];
  in += blockIdx.y * cs_in + gm;
  out += blockIdx.y * cs_out + gm;

  // this thread's point pairs: all loads in flight before any arithmetic
  cpx<R> xa[JI], xb[JI];
#pragma unroll
  for (int i = 0; i < JI; ++i) {
    const int j = warp + DCT_NW * i;
    xa[i] = xb[i] = cmk<R>(0, 0);
    if (ok && j <= H) {
      xa[i] = in[(size_t)j * ld_in];
      if (j < H) xb[i] = in[(size_t)(M - j) * ld_in];
    }
  }
  __syncthreads();  // tables staged

  cpx<R>* sq = seq + lane * P;
  cpx<R> x1 = cmk<R>(0, 0);
#pragma unroll
  for (int i = 0; i < JI; ++i) {
    const int j = warp + DCT_NW * i;
    if (j > H) break;  // uniform over the warp
    const cpx<R> s = cadd(xa[i], xb[i]), d = csub(xa[i], xb[i]);
    if (j == 0) {
      const R e = INV ? (R)2 : (R)1;
      sq[0] = cscale(s, e);
      x1 = cscale(d, e);
    } else if (j == H) {
      sq[pos_perm<N1>(H)] = cscale(xa[i], (R)2);
    } else {
      const cpx<R> c = cs[j];
      const cpx<R> t = cscale(d, c.y);
      sq[pos_perm<N1>(j)] = cadd(s, t);
      sq[pos_perm<N1>(M - j)] = csub(s, t);
      x1.x = fma(c.x, d.x, x1.x);
      x1.y = fma(c.x, d.y, x1.y);
    }
  }
  csp[warp * DCT_TM + lane] = x1;
  __syncthreads();
  pass_b<R, N1, -1>(seq, DCT_TM, SeqLinear{P}, tw, tid, DCT_THREADS);
  __syncthreads();
  pass_s<R, N1, -1>(seq, DCT_TM, SeqLinear{P}, tw, tid, DCT_THREADS);
  __syncthreads();

  // outputs k = 2 kk, 2 kk + 1 for kk in this warp's segment [k0, k0 + KS)
  const int k0 = warp * KS;
  const R so = INV ? (R)0.5 : (R)(1.0 / M);
  cpx<R> inc[KS];
  cpx<R> tot = cmk<R>(0, 0);
#pragma unroll
  for (int i = 0; i < KS; ++i) {
    const int kk = k0 + i;
    inc[i] = cmk<R>(0, 0);
    if (kk <= H) {
      const cpx<R> zk = sq[pos_nat<N1>(kk)], zm = sq[pos_nat<N1>(kk == 0 ? 0 : M - kk)];
      const R se = INV ? (R)0.25 : (R)((kk == 0 || kk == H ? 0.25 : 0.5) / M);
      if (ok) out[(size_t)(2 * kk) * ld_out] = cscale(cadd(zk, zm), se);
      if (kk >= 1 && kk < H) {
        inc[i] = cmk<R>(zk.y - zm.y, zm.x - zk.x);  // -i (Z_k - Z_{M-k})
        tot = cadd(tot, inc[i]);
      }
    }
  }
  segt[warp * DCT_TM + lane] = tot;
  __syncthreads();
  cpx<R> run = cmk<R>(0, 0);
#pragma unroll
  for (int w = 0; w < DCT_NW; ++w) run = cadd(run, csp[w * DCT_TM + lane]);
  for (int w = 0; w < warp; ++w) run = cadd(run, segt[w * DCT_TM + lane]);
#pragma unroll
  for (int i = 0; i < KS; ++i) {
    const int kk = k0 + i;
    run = cadd(run, inc[i]);
    if (ok && kk < H) out[(size_t)(2 * kk + 1) * ld_out] = cscale(run, so);
  }
}

template <typename R, int N1, bool INV>
cudaError_t run_dct(dim3 grid, cudaStream_t st, int nmodes, int lpf, const cpx<R>* in, size_t ld_in, size_t cs_in,
                    cpx<R>* out, size_t ld_out, size_t cs_out, const cpx<R>* tab, const Dither& dt) {
  constexpr size_t sm = dct_smem<R, N1>();
  static const bool attr = [] {
    cudaFuncSetAttribute(k_dct<R, N1, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    return true;
  }();
  (void)attr;
  k_dct<R, N1, INV><<<grid, DCT_THREADS, sm, st>>>(nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
  return cudaGetLastError();
}

template <typename R, int N1>
cudaError_t run_dct_dir(bool inverse, dim3 grid, cudaStream_t st, int nmodes, int lpf, const cpx<R>* in,
                        size_t ld_in, size_t cs_in, cpx<R>* out, size_t ld_out, size_t cs_out, const cpx<R>* tab,
                        const Dither& dt) {
  return inverse ? run_dct<R, N1, true>(grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt)
                 : run_dct<R, N1, false>(grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
}

// ---------------------------------------------------------------------------
// Spectral curl (rotationalNL's curl, diffops.cpp:2229-2334, in coefficient space).  Per solved mode: the
// Chebyshev coefficients of u, v, w (the base flow added to the (0,0) mode, -Vsuck on its v_0) and of
//   omega = (dw/dy - i kz v,  i kz u - i kx w,  i kx v - du/dy),
// d/dy by the coefficient relation of diff (chebyshev.cpp:672-697): d_n = (4/L) sum_{k > n, k - n odd} k x_k,
// d_0 halved.  Block: 32 modes (lanes) x 8 warps; warp w owns the rows [w NS, (w + 1) NS), and the suffix sums
// of k x_k (one per parity of k) run within a warp's rows and are joined through the segment totals.
// C6[c][n][mode], c = u, v, w, ox, oy, oz (re/im interleaved, R).  Per-field base flows: Ub/Wb + field *
// bstride.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_curl_coef(GridDev g, int N, const double* __restrict__ U,
                                                   R* __restrict__ C6, const double* __restrict__ Ub,
                                                   const double* __restrict__ Wb, int bstride, double Vsuck) {
  __shared__ cpx<double> tot[DCT_NW][4][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m = blockIdx.x * 32 + lane;
  const bool ok = m < g.Md;
  const int NS = (N + DCT_NW - 1) / DCT_NW, n0 = min(N, warp * NS), n1 = min(N, n0 + NS);
  const size_t row = (size_t)g.Md, comp = row * N;  // complex values
  const cpx<double>* Uc = reinterpret_cast<const cpx<double>*>(U);
  double dx = 0.0, dz = 0.0;
  bool m00 = false;
  if (ok) {
    const int kx = mode_kx(g, m), kz = mode_kz(g, m);
    dx = 2.0 * M_PI * kx / g.Lx * (kx == g.kxmax ? 0.0 : 1.0);
    dz = 2.0 * M_PI * kz / g.Lz * (kz == g.kzmax ? 0.0 : 1.0);
    m00 = kx == 0 && kz == 0;
    const int f = mode_field(g, m);
    Ub += (size_t)f * bstride;
    Wb += (size_t)f * bstride;
  }
  // segment totals of k u_k and k w_k by parity of k (e: even k, o: odd k)
  cpx<double> sue = cmk(0.0, 0.0), suo = sue, swe = sue, swo = sue;
  if (ok) {
#pragma unroll 4
    for (int n = n0; n < n1; ++n) {
      cpx<double> u = Uc[n * row + m], w = Uc[2 * comp + n * row + m];
      if (m00) {
        u.x += Ub[n];
        w.x += Wb[n];
      }
      if (n & 1) {
        suo = cadd(suo, cscale(u, (double)n));
        swo = cadd(swo, cscale(w, (double)n));
      } else {
        sue = cadd(sue, cscale(u, (double)n));
        swe = cadd(swe, cscale(w, (double)n));
      }
    }
  }
  tot[warp][0][lane] = sue;
  tot[warp][1][lane] = suo;
  tot[warp][2][lane] = swe;
  tot[warp][3][lane] = swo;
  __syncthreads();
  if (!ok) return;
  // the later segments' sums, then this segment's rows from the top down
  sue = suo = swe = swo = cmk(0.0, 0.0);
  for (int w = warp + 1; w < DCT_NW; ++w) {
    sue = cadd(sue, tot[w][0][lane]);
    suo = cadd(suo, tot[w][1][lane]);
    swe = cadd(swe, tot[w][2][lane]);
    swo = cadd(swo, tot[w][3][lane]);
  }
  const double scale = 4.0 / (g.b - g.a);
  const size_t orow = 2 * row, ocomp = orow * N;  // R values
#pragma unroll 4
  for (int n = n1 - 1; n >= n0; --n) {
    cpx<double> u = Uc[n * row + m], v = Uc[comp + n * row + m], w = Uc[2 * comp + n * row + m];
    if (m00) {
      u.x += Ub[n];
      w.x += Wb[n];
      if (n == 0) v.x -= Vsuck;
    }
    // d_n sums k x_k over k > n of the other parity than n
    const double h = n == 0 ? 0.5 * scale : scale;
    const bool odd = n & 1;
    const cpx<double> Du = cscale(odd ? sue : suo, h), Dw = cscale(odd ? swe : swo, h);
    if (odd) {
      suo = cadd(suo, cscale(u, (double)n));
      swo = cadd(swo, cscale(w, (double)n));
    } else {
      sue = cadd(sue, cscale(u, (double)n));
      swe = cadd(swe, cscale(w, (double)n));
    }
    const cpx<double> ox = cmk(Dw.x + dz * v.y, Dw.y - dz * v.x);
    const cpx<double> oy = cmk(-dz * u.y + dx * w.y, dz * u.x - dx * w.x);
    const cpx<double> oz = cmk(-dx * v.y - Du.x, dx * v.x - Du.y);
    R* o = C6 + n * orow + 2 * (size_t)m;
    o[0] = (R)u.x; o[1] = (R)u.y;
    o[ocomp] = (R)v.x; o[ocomp + 1] = (R)v.y;
    o[2 * ocomp] = (R)w.x; o[2 * ocomp + 1] = (R)w.y;
    o[3 * ocomp] = (R)ox.x; o[3 * ocomp + 1] = (R)ox.y;
    o[4 * ocomp] = (R)oy.x; o[4 * ocomp + 1] = (R)oy.y;
    o[5 * ocomp] = (R)oz.x; o[5 * ocomp + 1] = (R)oz.y;
  }
}

}  // namespace

bool dct_supported(int N) {
  const int M = N - 1;
  if (M % 8) return false;
  const int n1 = M / 8;
  return n1 == 4 || n1 == 6 || n1 == 8 || n1 == 12 || n1 == 16;
}

std::vector<double> dct_table(int N) {
  const int M = N - 1, H = M / 2;
  const long double PI_L = 3.14159265358979323846264338327950288L;
  auto snap = [](long double v) -> double {
    if (fabsl(v) < 1e-18L) return 0.0;
    if (fabsl(v - 1.0L) < 1e-18L) return 1.0;
    if (fabsl(v + 1.0L) < 1e-18L) return -1.0;
    return (double)v;
  };
  std::vector<double> t(2 * (size_t)(M + H + 1));
  for (int e = 0; e < M; ++e) {
    const long double a = 2.0L * PI_L * e / M;
    t[2 * e] = snap(cosl(a));
    t[2 * e + 1] = snap(-sinl(a));
  }
  for (int j = 0; j <= H; ++j) {
    const long double a = PI_L * j / M;
    t[2 * (M + j)] = 2.0 * snap(cosl(a));
    t[2 * (M + j) + 1] = snap(sinl(a));
  }
  return t;
}

template <typename R>
size_t dct_smem_bytes(int N) {
  switch ((N - 1) / 8) {
    case 4: return dct_smem<R, 4>();
    case 6: return dct_smem<R, 6>();
    case 8: return dct_smem<R, 8>();
    case 12: return dct_smem<R, 12>();
    case 16: return dct_smem<R, 16>();
    default: return 0;
  }
}

template <typename R>
cudaError_t launch_dct(int N, bool inverse, int nmodes, int ncomp, const cpx<R>* in, size_t ld_in, size_t cs_in,
                       cpx<R>* out, size_t ld_out, size_t cs_out, const cpx<R>* tab, cudaStream_t st,
                       const Dither& dt) {
  if (!dct_supported(N)) return cudaErrorInvalidValue;
  const int nf = dt.nb > 0 ? dt.nb : 1, lpf = (nmodes + nf - 1) / nf;
  const dim3 grid(nf * ((lpf + DCT_TM - 1) / DCT_TM), ncomp, 1);
  switch ((N - 1) / 8) {
    case 4: return run_dct_dir<R, 4>(inverse, grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
    case 6: return run_dct_dir<R, 6>(inverse, grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
    case 8: return run_dct_dir<R, 8>(inverse, grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
    case 12:
      return run_dct_dir<R, 12>(inverse, grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
    default:
      return run_dct_dir<R, 16>(inverse, grid, st, nmodes, lpf, in, ld_in, cs_in, out, ld_out, cs_out, tab, dt);
  }
}

template <typename R>
cudaError_t launch_curl_base(const GridDev& g, const double* U, R* C6, const double* Ub, const double* Wb,
                             int bstride, double Vsuck, cudaStream_t st) {
  k_curl_coef<R><<<(g.Md + 31) / 32, 256, 0, st>>>(g, g.Ny, U, C6, Ub, Wb, bstride, Vsuck);
  return cudaGetLastError();
}

#define CFGPU_DCT_INST(R)                                                                                      \
  template size_t dct_smem_bytes<R>(int);                                                                      \
  template cudaError_t launch_dct<R>(int, bool, int, int, const cpx<R>*, size_t, size_t, cpx<R>*, size_t,      \
                                     size_t, const cpx<R>*, cudaStream_t, const Dither&);                      \
  template cudaError_t launch_curl_base<R>(const GridDev&, const double*, R*, const double*, const double*, int, \
                                           double, cudaStream_t);
CFGPU_DCT_INST(float)
CFGPU_DCT_INST(double)
