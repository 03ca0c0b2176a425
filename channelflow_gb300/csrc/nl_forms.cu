// Nonlinear-term forms beyond the fused rotational kernel: the velocity
// gradient (convection, skew-symmetric) and velocity-only (divergence) inverse
// Chebyshev kernels, a physical-space z pass for any form, and the forward
// Chebyshev transform with the divergence combination.
//
// Reference functions restated (channelflow project paths):
//   convectionNL -> dotgrad        channelflow/diffops.cpp:2883-2885, 3586-3643
//   divergenceNL                   channelflow/diffops.cpp:3110-3134 (outer + div)
//   skewsymmetricNL                channelflow/diffops.cpp:3142-3286
//   grad (d/dx_j u_i, index 3i+j)  channelflow/diffops.cpp:1784-1941
// Forms (NL_*): rotational (omega x u), convection (u.grad u), divergence
// (div(u u)), skew-symmetric (1/2 (u.grad u + div(u u))).
#include "fft.cuh"
#include "kernels.h"

#define GC_TL 32
#define GC_PT 7

// ---------------------------------------------------------------------------
// Inverse Chebyshev of u, v, w (+ base flow) with, for MODE = 1, the nine
// gradient components G[3i+j] = d u_i / d x_j (d/dx, d/dz spectral, d/dy via
// the (2/L) T'_n half-matrices).  MODE = 2 outputs u, v, w only.
// Output W[c][j][line]: c = 0..2 velocity, 3 + 3i + j gradient.
// ---------------------------------------------------------------------------
template <typename R, int MODE>
__global__ void __launch_bounds__(256) k_grad_cheb(GridDev g, int N, const double* __restrict__ U, R* __restrict__ W,
                                                   const R* __restrict__ CA, const R* __restrict__ CB,
                                                   const R* __restrict__ DA, const R* __restrict__ DB,
                                                   const R* __restrict__ basey, double Vsuck,
                                                   int bstride, Dither dt, int lpf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typedef typename Vec16<R>::T V;
  constexpr int VW = 16 / sizeof(R);
  const int P = (N + 1) / 2, KA = (N + 1) / 2, KB = (N - 1) / 2, J = (N - 1) / 2;
  // coefficient rows padded to whole 16-byte vectors (zero-filled): the matrices are read VW columns per load
  const int KAp = (KA + VW - 1) / VW * VW, KBp = (KB + VW - 1) / VW * VW, NP = KAp + KBp;
  R* xs = reinterpret_cast<R*>(smem_raw);  // [3][NP][TL]: even coefs rows 0..KAp-1, odd KAp..NP-1
  R* sCA = xs + 3 * NP * GC_TL;
  R* sCB = sCA + P * KAp;
  R* sDA = sCB + P * KBp;
  R* sDB = sDA + P * KAp;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t row = 2 * (size_t)g.Md, comp = row * N;
  // blocks never straddle two fields (lpf lines each): a block uses its field's version of the constants
  const int bpf = (lpf + GC_TL - 1) / GC_TL, fld = blockIdx.x / bpf;
  const int nlines = (fld + 1) * lpf;  // one past this field's last line
  const int l0 = fld * lpf + (blockIdx.x - fld * bpf) * GC_TL;
  const int ver = dither_ver(dt, fld);
  CA = dither_ptr(CA, ver, dt.S);
  CB = dither_ptr(CB, ver, dt.S);
  DA = dither_ptr(DA, ver, dt.S);
  DB = dither_ptr(DB, ver, dt.S);
#pragma unroll 8
  for (int i = tid; i < P * KAp; i += blockDim.x) {
    const int pp = i / KAp, k = i - pp * KAp;
    sCA[i] = k < KA ? CA[pp * KA + k] : (R)0;
    if (MODE == 1) sDA[i] = k < KA ? DA[pp * KA + k] : (R)0;
  }
#pragma unroll 8
  for (int i = tid; i < P * KBp; i += blockDim.x) {
    const int pp = i / KBp, k = i - pp * KBp;
    sCB[i] = k < KB ? CB[pp * KB + k] : (R)0;
    if (MODE == 1) sDB[i] = k < KB ? DB[pp * KB + k] : (R)0;
  }
  for (int i = tid; i < 3 * (NP - N) * GC_TL; i += blockDim.x) {  // padding rows
    const int l = i % GC_TL, t = i / GC_TL, c = t / (NP - N), e = t % (NP - N);
    const int r = e < KAp - KA ? KA + e : KAp + KB + (e - (KAp - KA));
    xs[(c * NP + r) * GC_TL + l] = (R)0;
  }
#pragma unroll 4
  for (int i = tid; i < 3 * N * GC_TL; i += blockDim.x) {
    const int l = i % GC_TL, n = (i / GC_TL) % N, c = i / (GC_TL * N);
    const int gl = l0 + l;
    const R v = gl < nlines ? (R)U[c * comp + (size_t)n * row + gl] : (R)0;
    const int r = (n & 1) ? KAp + (n >> 1) : (n >> 1);
    xs[(c * NP + r) * GC_TL + l] = v;
  }
  __syncthreads();
  constexpr int NT = MODE == 1 ? 6 : 3;  // transforms: C u_c (3) and, for the gradient, CD u_c (3)
  R ae[NT][GC_PT], bo[NT][GC_PT];        // even-coefficient and odd-coefficient partial sums
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int i = 0; i < GC_PT; ++i) ae[t][i] = bo[t][i] = 0;
  // high n first (the small terms are summed before the large), VW columns per matrix load
  for (int kb = KAp / VW - 1; kb >= 0; --kb) {
    R x[3][VW];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int e = 0; e < VW; ++e) x[c][e] = xs[(c * NP + kb * VW + e) * GC_TL + lane];
#pragma unroll
    for (int i = 0; i < GC_PT; ++i) {
      const int p = warp + 8 * i;
      if (p < P) {
        const V c4 = *reinterpret_cast<const V*>(sCA + p * KAp + kb * VW);
        const R* cc = reinterpret_cast<const R*>(&c4);
#pragma unroll
        for (int e = VW - 1; e >= 0; --e)
#pragma unroll
          for (int c = 0; c < 3; ++c) ae[c][i] += cc[e] * x[c][e];
        if (MODE == 1) {
          const V d4 = *reinterpret_cast<const V*>(sDA + p * KAp + kb * VW);
          const R* d = reinterpret_cast<const R*>(&d4);
#pragma unroll
          for (int e = VW - 1; e >= 0; --e)
#pragma unroll
            for (int c = 0; c < 3; ++c) ae[3 + c][i] += d[e] * x[c][e];
        }
      }
    }
  }
  for (int kb = KBp / VW - 1; kb >= 0; --kb) {
    R x[3][VW];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int e = 0; e < VW; ++e) x[c][e] = xs[(c * NP + KAp + kb * VW + e) * GC_TL + lane];
#pragma unroll
    for (int i = 0; i < GC_PT; ++i) {
      const int p = warp + 8 * i;
      if (p < P) {
        const V c4 = *reinterpret_cast<const V*>(sCB + p * KBp + kb * VW);
        const R* cc = reinterpret_cast<const R*>(&c4);
#pragma unroll
        for (int e = VW - 1; e >= 0; --e)
#pragma unroll
          for (int c = 0; c < 3; ++c) bo[c][i] += cc[e] * x[c][e];
        if (MODE == 1) {
          const V d4 = *reinterpret_cast<const V*>(sDB + p * KBp + kb * VW);
          const R* d = reinterpret_cast<const R*>(&d4);
#pragma unroll
          for (int e = VW - 1; e >= 0; --e)
#pragma unroll
            for (int c = 0; c < 3; ++c) bo[3 + c][i] += d[e] * x[c][e];
        }
      }
    }
  }
  const int gl = l0 + lane;
  const int m = min(gl, nlines - 1) >> 1;
  const int part = gl & 1;
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const R dx = k_dx<R>(dt, ver, g, kx);
  const R dz = k_dz<R>(dt, ver, g, kz);
  const R vs = k_misc<R>(dt, ver, 1, Vsuck);
  const bool base = (kx == 0 && kz == 0 && part == 0);
  const R* __restrict__ by = dither_ptr(basey, ver, dt.Sb) + (size_t)bstride * mode_field(g, m);  // this field's base flow
#pragma unroll
  for (int i = 0; i < GC_PT; ++i) {
    const int p = warp + 8 * i;
    if (p >= P) continue;  // uniform per warp
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (h == 1 && p >= J) continue;
      const int j = h == 0 ? p : N - 1 - p;
      const R sg = h == 0 ? (R)1 : (R)-1;
      R u[3], dy[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) u[c] = ae[c][i] + sg * bo[c][i];
      if (MODE == 1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) dy[c] = bo[3 + c][i] + sg * ae[3 + c][i];
      }
      if (base) {
        u[0] += by[j];
        u[2] += by[2 * N + j];
        u[1] -= vs;
        if (MODE == 1) {
          dy[0] += by[N + j];
          dy[2] += by[3 * N + j];
        }
      }
      R* o = W + (size_t)j * row + gl;
      if (MODE == 1) {
        R ou[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) ou[c] = __shfl_xor_sync(0xffffffffu, u[c], 1);
        if (gl < nlines) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            // (i k) f: re = -k f_im, im = k f_re
            const R gx = part == 0 ? -dx * ou[c] : dx * ou[c];
            const R gz = part == 0 ? -dz * ou[c] : dz * ou[c];
            o[(size_t)c * comp] = u[c];
            o[(size_t)(3 + 3 * c + 0) * comp] = gx;
            o[(size_t)(3 + 3 * c + 1) * comp] = dy[c];
            o[(size_t)(3 + 3 * c + 2) * comp] = gz;
          }
        }
      } else if (gl < nlines) {
#pragma unroll
        for (int c = 0; c < 3; ++c) o[(size_t)c * comp] = u[c];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// z pass for any form.  Real sequence k of the block (row r = k / NC,
// component c = k % NC) is half of complex sequence k/2 (real part for even
// k, imaginary for odd k): one complex FFT transforms two real rows.
// ---------------------------------------------------------------------------
template <int FORM>
struct FormIO;
template <>
struct FormIO<NL_ROTATIONAL> { static constexpr int NC = 6, NO = 3; };
template <>
struct FormIO<NL_CONVECTION> { static constexpr int NC = 12, NO = 3; };
template <>
struct FormIO<NL_DIVERGENCE> { static constexpr int NC = 3, NO = 6; };
template <>
struct FormIO<NL_SKEW> { static constexpr int NC = 12, NO = 9; };

template <typename R, int FORM>
__device__ __forceinline__ void phys_products(const R* c, R* f) {
  if constexpr (FORM == NL_ROTATIONAL) {
    // c = u, v, w, ox, oy, oz ; f = omega x u
    f[0] = c[4] * c[2] - c[5] * c[1];
    f[1] = c[5] * c[0] - c[3] * c[2];
    f[2] = c[3] * c[1] - c[4] * c[0];
  } else if constexpr (FORM == NL_DIVERGENCE) {
    f[0] = c[0] * c[0];
    f[1] = c[0] * c[1];
    f[2] = c[0] * c[2];
    f[3] = c[1] * c[1];
    f[4] = c[1] * c[2];
    f[5] = c[2] * c[2];
  } else {
    // u_j d u_i / d x_j
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      R s = 0;
#pragma unroll
      for (int j = 0; j < 3; ++j) s += c[j] * c[3 + 3 * i + j];
      f[i] = s;
    }
    if constexpr (FORM == NL_SKEW) {
      f[3] = c[0] * c[0];
      f[4] = c[0] * c[1];
      f[5] = c[0] * c[2];
      f[6] = c[1] * c[1];
      f[7] = c[1] * c[2];
      f[8] = c[2] * c[2];
    }
  }
}

template <typename R, int FORM>
__global__ void __launch_bounds__(256) k_zphys(GridDev g, FftPlan pz, const cpx<R>* __restrict__ twz, int RP,
                                               const cpx<R>* __restrict__ X, cpx<R>* __restrict__ Z, Dither dt) {
  constexpr int NC = FormIO<FORM>::NC, NO = FormIO<FORM>::NO;
  extern __shared__ unsigned char smem_raw[];
  pdl_wait();  // launched with launch_pdl: the previous kernel's output is read from here on
  twz = dither_ptr(twz, dither_ver(dt, blockIdx.y % dt.nb), dt.S);  // plane blockIdx.y -> its field's twiddles
  const int Nz = g.Nz, ss = Nz + 1, NKz = g.NKz;
  const int nseq = ((NC > NO ? NC : NO) * RP) / 2;
  const int ninv = NC * RP / 2, nfwd = NO * RP / 2;
  cpx<R>* A = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* B = A + (size_t)nseq * ss;
  const int ny = blockIdx.y;
  const int x0 = blockIdx.x * RP;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const size_t plane = (size_t)g.Nx * NKz;
  // the pack below writes bins 0..NKz-1 and Nz-NKz+1..Nz-1 of every inverse sequence: zero the gap
  const float invk = 1.0f / NKz;
  {
    const int G = Nz - 2 * NKz + 1;
    const float invg = 1.0f / G;
    for (int i = tid; i < ninv * G; i += nthr) {
      int sq, z;
      divmod_small(i, G, invg, sq, z);
      A[(size_t)sq * ss + NKz + z] = cmk<R>(0, 0);
    }
  }
#pragma unroll 4
  for (int i = tid; i < ninv * NKz; i += nthr) {
    int s, iz;
    divmod_small(i, NKz, invk, s, iz);
    const int k0 = 2 * s, k1 = 2 * s + 1;
    const int r0 = k0 / NC, c0 = k0 % NC, r1 = k1 / NC, c1 = k1 % NC;
    cpx<R> ca = cmk<R>(0, 0), cb = cmk<R>(0, 0);
    if (x0 + r0 < g.Nx) ca = X[((size_t)c0 * g.Ny + ny) * plane + (size_t)(x0 + r0) * NKz + iz];
    if (x0 + r1 < g.Nx) cb = X[((size_t)c1 * g.Ny + ny) * plane + (size_t)(x0 + r1) * NKz + iz];
    cpx<R>* sq = A + (size_t)s * ss;
    if (iz == 0) {
      sq[0] = cmk<R>(ca.x, cb.x);
    } else {
      sq[iz] = cmk<R>(ca.x - cb.y, ca.y + cb.x);        // A_k + i B_k
      sq[Nz - iz] = cmk<R>(ca.x + cb.y, -ca.y + cb.x);  // conj(A_k) + i conj(B_k)
    }
  }
  __syncthreads();
  fft_batch<R>(A, B, ninv, ss, pz, twz, +1);
  R* Br = reinterpret_cast<R*>(B);
  for (int i = tid; i < RP * Nz; i += nthr) {
    const int z = i % Nz, r = i / Nz;
    R c[NC], f[NO];
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      const int k = r * NC + q;
      const cpx<R> v = A[(size_t)(k >> 1) * ss + z];
      c[q] = (k & 1) ? v.y : v.x;
    }
    phys_products<R, FORM>(c, f);
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      const int k = r * NO + o;
      Br[2 * ((size_t)(k >> 1) * ss + z) + (k & 1)] = f[o];
    }
  }
  __syncthreads();
  fft_batch<R>(B, A, nfwd, ss, pz, twz, -1);
#pragma unroll 4
  for (int i = tid; i < nfwd * NKz; i += nthr) {
    int s, iz;
    divmod_small(i, NKz, invk, s, iz);
    const cpx<R>* sq = B + (size_t)s * ss;
    const cpx<R> zk = sq[iz];
    const cpx<R> zm = sq[iz == 0 ? 0 : Nz - iz];
    const cpx<R> Pk = cmk<R>((R)0.5 * (zk.x + zm.x), (R)0.5 * (zk.y - zm.y));
    const cpx<R> Qk = cmk<R>((R)0.5 * (zk.y + zm.y), (R)0.5 * (zm.x - zk.x));
    const int k0 = 2 * s, k1 = 2 * s + 1;
    const int r0 = k0 / NO, o0 = k0 % NO, r1 = k1 / NO, o1 = k1 % NO;
    if (x0 + r0 < g.Nx) Z[((size_t)o0 * g.Ny + ny) * plane + (size_t)(x0 + r0) * NKz + iz] = Pk;
    if (x0 + r1 < g.Nx) Z[((size_t)o1 * g.Ny + ny) * plane + (size_t)(x0 + r1) * NKz + iz] = Qk;
  }
}

// ---------------------------------------------------------------------------
// Forward Chebyshev transform with the divergence combination for one output
// component i:  N_i = wF F(pF) + wK (i kx F(pKx) + i kz F(pKz)) + wD DF(pD)
// where F maps values at the Gauss-Lobatto points to Chebyshev coefficients
// (chebyfft) and DF = diff o F.  Parity split: with s_j = x_j + x_{N-1-j},
// d_j = x_j - x_{N-1-j}: F even = FA s, F odd = FB d, DF even = DFA d,
// DF odd = DFB s.  pF may be null (divergence form).
// ---------------------------------------------------------------------------
#define CF_TL 32
#define CF_PT 9

template <typename R>
__global__ void __launch_bounds__(256) k_cheb_fwd_div(GridDev g, int N, const R* __restrict__ pF,
                                                      const R* __restrict__ pKx, const R* __restrict__ pKz,
                                                      const R* __restrict__ pD, R wF, R wK, R wD, R* __restrict__ out,
                                                      const R* __restrict__ FA, const R* __restrict__ FB,
                                                      const R* __restrict__ DFA, const R* __restrict__ DFB, Dither dt,
                                                      int lpf) {
  extern __shared__ unsigned char smem_raw[];
  const int P = (N + 1) / 2, J = (N - 1) / 2, KA = J + 1, KB = J;
  R* xs = reinterpret_cast<R*>(smem_raw);  // [4 inputs][KA s-rows + KB d-rows][TL]
  R* sFA = xs + 4 * N * CF_TL;
  R* sFB = sFA + P * KA;
  R* sDA = sFB + P * KB;  // P x KB (acts on d)
  R* sDB = sDA + P * KB;  // P x KA (acts on s)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t row = 2 * (size_t)g.Md;
  // blocks never straddle two fields (lpf lines each): a block uses its field's version of the constants
  const int bpf = (lpf + CF_TL - 1) / CF_TL, fld = blockIdx.x / bpf;
  const int nlines = (fld + 1) * lpf;  // one past this field's last line
  const int l0 = fld * lpf + (blockIdx.x - fld * bpf) * CF_TL;
  const int ver = dither_ver(dt, fld);
  FA = dither_ptr(FA, ver, dt.S);
  FB = dither_ptr(FB, ver, dt.S);
  DFA = dither_ptr(DFA, ver, dt.S);
  DFB = dither_ptr(DFB, ver, dt.S);
#pragma unroll 8
  for (int i = tid; i < P * KA; i += blockDim.x) {
    sFA[i] = FA[i];
    sDB[i] = DFB[i];
  }
#pragma unroll 8
  for (int i = tid; i < P * KB; i += blockDim.x) {
    sFB[i] = FB[i];
    sDA[i] = DFA[i];
  }
  const R* ins[4] = {pF, pKx, pKz, pD};
#pragma unroll 4
  for (int i = tid; i < 4 * KA * CF_TL; i += blockDim.x) {
    const int l = i % CF_TL, j = (i / CF_TL) % KA, c = i / (CF_TL * KA);
    const int gl = l0 + l;
    const R* src = ins[c];
    R v1 = 0, v2 = 0;
    if (src && gl < nlines) {
      v1 = src[(size_t)j * row + gl];
      v2 = src[(size_t)(N - 1 - j) * row + gl];
    }
    if (j < J) {
      xs[(c * N + j) * CF_TL + l] = v1 + v2;
      xs[(c * N + KA + j) * CF_TL + l] = v1 - v2;
    } else {
      xs[(c * N + j) * CF_TL + l] = v1;  // middle point
    }
  }
  __syncthreads();
  R fe[3][CF_PT], fo[3][CF_PT], de[CF_PT], dd[CF_PT];
#pragma unroll
  for (int i = 0; i < CF_PT; ++i) {
    de[i] = dd[i] = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) fe[c][i] = fo[c][i] = 0;
  }
  // s rows: F even (inputs 0..2) and DF odd (input 3)
  for (int k = 0; k < KA; ++k) {
    R x[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = xs[(c * N + k) * CF_TL + lane];
#pragma unroll
    for (int i = 0; i < CF_PT; ++i) {
      const int p = warp + 8 * i;
      if (p < P) {
        const R a = sFA[p * KA + k];
#pragma unroll
        for (int c = 0; c < 3; ++c) fe[c][i] += a * x[c];
        dd[i] += sDB[p * KA + k] * x[3];
      }
    }
  }
  // d rows: F odd (inputs 0..2) and DF even (input 3)
  for (int k = 0; k < KB; ++k) {
    R x[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = xs[(c * N + KA + k) * CF_TL + lane];
#pragma unroll
    for (int i = 0; i < CF_PT; ++i) {
      const int p = warp + 8 * i;
      if (p < P) {
        const R b = sFB[p * KB + k];
#pragma unroll
        for (int c = 0; c < 3; ++c) fo[c][i] += b * x[c];
        de[i] += sDA[p * KB + k] * x[3];
      }
    }
  }
  const int gl = l0 + lane;
  const int m = min(gl, nlines - 1) >> 1;
  const int part = gl & 1;
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const R dx = k_dx<R>(dt, ver, g, kx);
  const R dz = k_dz<R>(dt, ver, g, kz);
#pragma unroll
  for (int i = 0; i < CF_PT; ++i) {
    const int p = warp + 8 * i;
    if (p >= P) continue;  // uniform per warp
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int n = 2 * p + h;
      if (n >= N) continue;  // uniform per warp
      const R vF = h == 0 ? fe[0][i] : fo[0][i];
      const R vX = h == 0 ? fe[1][i] : fo[1][i];
      const R vZ = h == 0 ? fe[2][i] : fo[2][i];
      const R vD = h == 0 ? de[i] : dd[i];
      const R t = dx * vX + dz * vZ;                    // (kx F(pKx) + kz F(pKz)) of my part
      const R tp = __shfl_xor_sync(0xffffffffu, t, 1);  // same of the other part
      const R ik = part == 0 ? -tp : tp;                // i * (...)
      const R val = wF * vF + wK * ik + wD * vD;
      if (gl < nlines) out[(size_t)n * row + gl] = val;
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <typename R>
size_t grad_cheb_smem_bytes(int N) {
  const int VW = 16 / sizeof(R);
  const int P = (N + 1) / 2, KAp = ((N + 1) / 2 + VW - 1) / VW * VW, KBp = ((N - 1) / 2 + VW - 1) / VW * VW;
  return sizeof(R) * ((size_t)3 * (KAp + KBp) * GC_TL + 2 * (size_t)P * (KAp + KBp));
}

template <typename R>
cudaError_t launch_grad_cheb(const GridDev& g, int N, bool gradient, const double* U, R* W, const R* CA, const R* CB,
                             const R* DA, const R* DB, const R* basey, double Vsuck, cudaStream_t st,
                             int bstride, const Dither& dt) {
  if ((N + 1) / 2 > 8 * GC_PT) return cudaErrorInvalidValue;
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_grad_cheb<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_grad_cheb<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr_set;
  const int nf = dt.nb > 0 ? dt.nb : 1, lpf = 2 * g.Md / nf;
  const dim3 grid(nf * ((lpf + GC_TL - 1) / GC_TL));
  if (gradient)
    k_grad_cheb<R, 1><<<grid, 256, grad_cheb_smem_bytes<R>(N), st>>>(g, N, U, W, CA, CB, DA, DB, basey, Vsuck, bstride,
                                                                     dt, lpf);
  else
    k_grad_cheb<R, 2><<<grid, 256, grad_cheb_smem_bytes<R>(N), st>>>(g, N, U, W, CA, CB, DA, DB, basey, Vsuck, bstride,
                                                                     dt, lpf);
  return cudaGetLastError();
}

template <typename R>
size_t zphys_smem_bytes(const GridDev& g, int form, int RP) {
  int nc = 6, no = 3;
  if (form == NL_CONVECTION) { nc = 12; no = 3; }
  if (form == NL_DIVERGENCE) { nc = 3; no = 6; }
  if (form == NL_SKEW) { nc = 12; no = 9; }
  const int nseq = ((nc > no ? nc : no) * RP) / 2;
  return 2 * sizeof(cpx<R>) * (size_t)nseq * (g.Nz + 1);
}

template <typename R, int FORM>
static cudaError_t launch_zphys_t(const GridDev& g, const FftPlan& pz, const cpx<R>* twz, int RP, const cpx<R>* X,
                                  cpx<R>* Z, cudaStream_t st, const Dither& dt) {
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_zphys<R, FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr_set;
  return launch_pdl(k_zphys<R, FORM>, dim3((g.Nx + RP - 1) / RP, g.Ny), dim3(256), zphys_smem_bytes<R>(g, FORM, RP),
                    st, g, pz, twz, RP, X, Z, dt);
}

template <typename R>
cudaError_t launch_zphys(const GridDev& g, int form, const FftPlan& pz, const cpx<R>* twz, int RP, const cpx<R>* X,
                         cpx<R>* Z, cudaStream_t st, const Dither& dt, const cpx<R>* twzf) {
  // FP32 only: in FP64 the register FFTs made the step slower (1.086 against 1.055 ms at 128x97x128), the FP64
  // pipe favouring the Stockham kernel's radix-4 stages
  if constexpr (sizeof(R) == 4) {
    if (form == NL_ROTATIONAL && twzf) {
      const cudaError_t e = launch_zrot(g, RP, X, Z, twzf, st, dt);
      if (e != cudaErrorNotSupported) return e;
    }
  }
  switch (form) {
    case NL_ROTATIONAL: return launch_zphys_t<R, NL_ROTATIONAL>(g, pz, twz, RP, X, Z, st, dt);
    case NL_CONVECTION: return launch_zphys_t<R, NL_CONVECTION>(g, pz, twz, RP, X, Z, st, dt);
    case NL_DIVERGENCE: return launch_zphys_t<R, NL_DIVERGENCE>(g, pz, twz, RP, X, Z, st, dt);
    default: return launch_zphys_t<R, NL_SKEW>(g, pz, twz, RP, X, Z, st, dt);
  }
}

template <typename R>
size_t cheb_fwd_div_smem_bytes(int N) {
  const int P = (N + 1) / 2, J = (N - 1) / 2;
  return sizeof(R) * ((size_t)4 * N * CF_TL + (size_t)P * (J + 1) * 2 + (size_t)P * J * 2);
}

template <typename R>
cudaError_t launch_cheb_fwd_div(const GridDev& g, int N, const R* pF, const R* pKx, const R* pKz, const R* pD, R wF,
                                R wK, R wD, R* out, const R* FA, const R* FB, const R* DFA, const R* DFB,
                                cudaStream_t st, const Dither& dt) {
  if ((N + 1) / 2 > 8 * CF_PT) return cudaErrorInvalidValue;
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_cheb_fwd_div<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr_set;
  const int nf = dt.nb > 0 ? dt.nb : 1, lpf = 2 * g.Md / nf;
  k_cheb_fwd_div<R><<<nf * ((lpf + CF_TL - 1) / CF_TL), 256, cheb_fwd_div_smem_bytes<R>(N), st>>>(
      g, N, pF, pKx, pKz, pD, wF, wK, wD, out, FA, FB, DFA, DFB, dt, lpf);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// LinearAboutProfile: linearizedNL (channelflow/diffops.cpp:3288-3361),
//   f = (U d/dx + W d/dz) u + v (U', 0, W'),
// per mode at the Gauss-Lobatto points: Y holds u, v, w there ([c][j][2*Md], the
// output of k_grad_cheb without base flow), basey the base profiles U, U', W, W'
// at the points ([4][N] per field, field stride bstride).  Nyquist derivatives
// are zero (no solved mode is a Nyquist mode).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_linprof(GridDev g, int N, const R* __restrict__ Y, const R* __restrict__ basey, int bstride,
                          R* __restrict__ F, Dither dt) {
  const size_t row = 2 * (size_t)g.Md, comp = row * N;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)g.Md * N) return;
  const int m = (int)(t % g.Md), j = (int)(t / g.Md);
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const int ver = dither_ver(dt, mode_field(g, m));
  const R dx = k_dx<R>(dt, ver, g, kx), dz = k_dz<R>(dt, ver, g, kz);
  const R* by = dither_ptr(basey, ver, dt.Sb) + (size_t)bstride * mode_field(g, m);
  const R U = by[j], Uy = by[N + j], W = by[2 * N + j], Wy = by[3 * N + j];
  const R d = U * dx + W * dz;  // (U d/dx + W d/dz) = i d
  const size_t o = (size_t)j * row + 2 * (size_t)m;
  const R ur = Y[o], ui = Y[o + 1], vr = Y[comp + o], vi = Y[comp + o + 1];
  const R wr = Y[2 * comp + o], wi = Y[2 * comp + o + 1];
  F[o] = -d * ui + Uy * vr;
  F[o + 1] = d * ur + Uy * vi;
  F[comp + o] = -d * vi;
  F[comp + o + 1] = d * vr;
  F[2 * comp + o] = -d * wi + Wy * vr;
  F[2 * comp + o + 1] = d * wr + Wy * vi;
}

template <typename R>
cudaError_t launch_linprof(const GridDev& g, int N, const R* Y, const R* basey, int bstride, R* F, cudaStream_t st,
                           const Dither& dt) {
  const size_t total = (size_t)g.Md * N;
  k_linprof<R><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g, N, Y, basey, bstride, F, dt);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Rotation about z (navierstokesNL, channelflow/nse.cpp:62-78): f -= rot e_z x (u + U):
//   f_x -= rot (v - Vsuck on the (0,0) mode),  f_y += rot (u + U on the (0,0) mode),
// linear in u, so added to the Chebyshev coefficients of N (the reference adds it at the
// grid points and transforms back).  U: base coefficients [field][N] (stride ustride).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_rotation(GridDev g, int N, const double* __restrict__ U, const double* __restrict__ Ub,
                           int ustride, double rot, double Vsuck, R* __restrict__ F) {
  const size_t row = 2 * (size_t)g.Md, comp = row * N;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= row * N) return;
  const int l = (int)(t % row), n = (int)(t / row);
  const int m = l >> 1, part = l & 1;
  const bool m00 = mode_kx(g, m) == 0 && mode_kz(g, m) == 0 && part == 0;
  double u = U[t], v = U[comp + t];
  if (m00) {
    u += Ub[(size_t)ustride * mode_field(g, m) + n];
    if (n == 0) v -= Vsuck;
  }
  F[t] = (R)((double)F[t] - rot * v);
  F[comp + t] = (R)((double)F[comp + t] + rot * u);
}

template <typename R>
cudaError_t launch_rotation(const GridDev& g, int N, const double* U, const double* Ub, int ustride, double rot,
                            double Vsuck, R* F, cudaStream_t st) {
  const size_t total = 2 * (size_t)g.Md * N;
  k_rotation<R><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g, N, U, Ub, ustride, rot, Vsuck, F);
  return cudaGetLastError();
}

#define INST_FORMS(R)                                                                                              \
  template cudaError_t launch_linprof<R>(const GridDev&, int, const R*, const R*, int, R*, cudaStream_t,           \
                                         const Dither&);                                                          \
  template cudaError_t launch_rotation<R>(const GridDev&, int, const double*, const double*, int, double, double,   \
                                          R*, cudaStream_t);                                                       \
  template size_t grad_cheb_smem_bytes<R>(int);                                                                    \
  template cudaError_t launch_grad_cheb<R>(const GridDev&, int, bool, const double*, R*, const R*, const R*,      \
                                           const R*, const R*, const R*, double, cudaStream_t, int, const Dither&); \
  template size_t zphys_smem_bytes<R>(const GridDev&, int, int);                                                   \
  template cudaError_t launch_zphys<R>(const GridDev&, int, const FftPlan&, const cpx<R>*, int, const cpx<R>*,      \
                                       cpx<R>*, cudaStream_t, const Dither&, const cpx<R>*);                       \
  template size_t cheb_fwd_div_smem_bytes<R>(int);                                                                 \
  template cudaError_t launch_cheb_fwd_div<R>(const GridDev&, int, const R*, const R*, const R*, const R*, R, R, R, \
                                              R*, const R*, const R*, const R*, const R*, cudaStream_t, const Dither&);

INST_FORMS(float)
INST_FORMS(double)

// Advance every field's constant version after a nonlinear evaluation (one thread per field).
__global__ void k_dither_bump(int* ver, int nb) {
  pdl_wait();
  pdl_trigger();
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < nb) ver[f] = (ver[f] + 1) % DITHER_V;
}

cudaError_t launch_dither_bump(int* ver, int nb, cudaStream_t st) {
  return launch_pdl(k_dither_bump, dim3((nb + 127) / 128), dim3(128), 0, st, ver, nb);
}
