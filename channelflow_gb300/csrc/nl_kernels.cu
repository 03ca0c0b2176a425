// Nonlinear-term kernels of the DNS step: dense Chebyshev (y) transforms (the
// spectral curl fused in) and the x/z FFT passes with the physical-space cross product.
//
// Reference functions restated (channelflow project paths):
//   curl               channelflow/diffops.cpp:2229-2334
//   cross              channelflow/diffops.cpp:2560-2611
//   rotationalNL       channelflow/diffops.cpp:2852-2881
//   navierstokesNL     channelflow/nse.cpp:12-91 (base flow added to (0,0))
//   makePhysical_y / makeSpectral_y   channelflow/flowfield.cpp:1888-1987
//   makePhysical_xz / makeSpectral_xz channelflow/flowfield.cpp:1850-1886
//   zeroPaddedModes    channelflow/flowfield.cpp:2235-2255 (only solved modes
//                      are ever stored, so truncation is implicit)
#include "fft.cuh"
#include "kernels.h"

// ---------------------------------------------------------------------------
// Chebyshev transform along y of many real lines, parity split.
// Lines are the interleaved re/im reals of a component: element (n, l) at
// base[c*cstride + n*ld + l].  One block: 64 lines x all N rows.
//   inverse (coefficients -> values at y_j = cos(pi j/(N-1))):
//       E_j = sum_k a_{2k} cos(pi 2k j/(N-1)),  O_j = sum_k a_{2k+1} cos(pi (2k+1) j/(N-1))
//       u_j = E_j + O_j,  u_{N-1-j} = E_j - O_j        (ichebyfft, chebyshev.cpp:286-303)
//   forward (values -> coefficients, chebyfft, chebyshev.cpp:262-284):
//       a_{2k} = sum_j Fe[k][j] (u_j + u_{N-1-j}),  a_{2k+1} = sum_j Fo[k][j] (u_j - u_{N-1-j})
// A (P x KA) and B (P x KB) hold the two half matrices (host-built in double).
// CS (FP32 forward transforms): the sum runs over groups of eight terms (two
// matrix vector loads), each group summed with FMAs and added to the running
// sum with an error-free two-sum whose errors are accumulated separately
// (compensated summation): the forward sums add terms of similar size, so the
// plain running sum's rounding would grow with the number of terms.
// ---------------------------------------------------------------------------
#define CHEB_TL 64
#define CHEB_WARPS 8
#define CHEB_PT 9

// s + t = s1 + err exactly (Knuth's two-sum; needs IEEE rounding of each operation, so the library is built
// without fast-math); err is added to the running compensation c.
template <typename R>
__device__ __forceinline__ void two_sum_acc(R& s, R t, R& c) {
  const R s1 = s + t;
  const R bp = s1 - s;
  c += (s - (s1 - bp)) + (t - bp);
  s = s1;
}

template <typename TI, typename R, typename TO, bool CS, int PT>
__global__ void __launch_bounds__(256, CS ? 3 : 1) k_cheb(int N, int inverse, int nlines, const TI* __restrict__ in, size_t ld_in,
                                              size_t cs_in, TO* __restrict__ out, size_t ld_out, size_t cs_out,
                                              const R* __restrict__ Amat, const R* __restrict__ Bmat, int P, int KA,
                                              int KB, Dither dt, int lpf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typedef typename VecLds<R>::T V;
  constexpr int VW = VecLds<R>::W;
  // rows padded to whole 16-byte vectors (zero-filled): the matrices are read VW columns per load
  const int KAp = (KA + VW - 1) / VW * VW, KBp = (KB + VW - 1) / VW * VW;
  R* xa = reinterpret_cast<R*>(smem_raw);
  R* xb = xa + (size_t)KAp * CHEB_TL;
  // output rows p0 .. p0 + PB of this block (blockIdx.z: row blocks of tall grids; one block covers P otherwise)
  constexpr int PB = CHEB_WARPS * PT;
  const int p0 = blockIdx.z * PB, np = min(PB, P - p0);
  R* As = xb + (size_t)KBp * CHEB_TL;
  R* Bs = As + (size_t)np * KAp;
  const int tid = threadIdx.x;
  // blocks never straddle two fields (lpf lines each): a block uses its field's version of the matrices
  const int bpf = (lpf + CHEB_TL - 1) / CHEB_TL, fld = blockIdx.x / bpf;
  const int l0 = fld * lpf + (blockIdx.x - fld * bpf) * CHEB_TL;
  nlines = min(nlines, (fld + 1) * lpf);
  const int ver = dither_ver(dt, fld);
  Amat = dither_ptr(Amat, ver, dt.S);
  Bmat = dither_ptr(Bmat, ver, dt.S);
  const int c = blockIdx.y;
  in += c * cs_in;
  out += c * cs_out;
  const int J = (N - 1) / 2;
  {
    const float invA = 1.0f / KAp, invB = 1.0f / KBp;
#pragma unroll 8
    for (int i = tid; i < np * KAp; i += blockDim.x) {
      int p, k;
      divmod_small(i, KAp, invA, p, k);
      As[i] = k < KA ? Amat[(p0 + p) * KA + k] : (R)0;
    }
#pragma unroll 8
    for (int i = tid; i < np * KBp; i += blockDim.x) {
      int p, k;
      divmod_small(i, KBp, invB, p, k);
      Bs[i] = k < KB ? Bmat[(p0 + p) * KB + k] : (R)0;
    }
  }
  for (int i = tid; i < (KAp - KA) * CHEB_TL; i += blockDim.x) xa[KA * CHEB_TL + i] = (R)0;
  for (int i = tid; i < (KBp - KB) * CHEB_TL; i += blockDim.x) xb[KB * CHEB_TL + i] = (R)0;
  // stage inputs
#pragma unroll 4
  for (int i = tid; i < N * CHEB_TL; i += blockDim.x) {
    const int n = i / CHEB_TL, l = i % CHEB_TL;
    const int gl = l0 + l;
    if (inverse) {
      R v = gl < nlines ? (R)in[n * ld_in + gl] : (R)0;
      if (n & 1) xb[(n >> 1) * CHEB_TL + l] = v;
      else xa[(n >> 1) * CHEB_TL + l] = v;
    } else if (n <= J) {
      R v1 = gl < nlines ? (R)in[n * ld_in + gl] : (R)0;
      R v2 = gl < nlines ? (R)in[(N - 1 - n) * ld_in + gl] : (R)0;
      if (n < J) {
        xa[n * CHEB_TL + l] = v1 + v2;
        xb[n * CHEB_TL + l] = v1 - v2;
      } else {
        xa[n * CHEB_TL + l] = v1;  // middle point
      }
    }
  }
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5;
  R accA[PT][2], cmpA[PT][2];  // even sums and their compensation terms (CS)
#pragma unroll
  for (int i = 0; i < PT; ++i) accA[i][0] = accA[i][1] = cmpA[i][0] = cmpA[i][1] = (R)0;
  // high n first (the small terms are summed before the large), VW columns per matrix load; the compensated
  // form adds groups of CG matrix loads (2 VW terms) to the running sum
  constexpr int CG = CS ? 2 : 1;
  for (int kb = KAp / VW - 1; kb >= 0; kb -= CG) {
    R x0[CG][VW], x1[CG][VW];
#pragma unroll
    for (int gq = 0; gq < CG; ++gq)
#pragma unroll
      for (int e = 0; e < VW; ++e) {
        const int k = (kb - gq) * VW + e;
        x0[gq][e] = k >= 0 ? xa[k * CHEB_TL + lane] : (R)0;
        x1[gq][e] = k >= 0 ? xa[k * CHEB_TL + lane + 32] : (R)0;
      }
#pragma unroll
    for (int i = 0; i < PT; ++i) {
      const int p = warp + CHEB_WARPS * i;  // row of the block
      if (p < np) {
        if (CS) {
          R t0 = (R)0, t1 = (R)0;
#pragma unroll
          for (int gq = 0; gq < CG; ++gq) {
            if (kb - gq < 0) break;  // uniform over the block
            const V a4 = *reinterpret_cast<const V*>(As + p * KAp + (kb - gq) * VW);
            const R* a = reinterpret_cast<const R*>(&a4);
#pragma unroll
            for (int e = VW - 1; e >= 0; --e) {
              t0 += a[e] * x0[gq][e];
              t1 += a[e] * x1[gq][e];
            }
          }
          two_sum_acc(accA[i][0], t0, cmpA[i][0]);
          two_sum_acc(accA[i][1], t1, cmpA[i][1]);
        } else {
          const V a4 = *reinterpret_cast<const V*>(As + p * KAp + kb * VW);
          const R* a = reinterpret_cast<const R*>(&a4);
#pragma unroll
          for (int e = VW - 1; e >= 0; --e) {
            accA[i][0] += a[e] * x0[0][e];
            accA[i][1] += a[e] * x1[0][e];
          }
        }
      }
    }
  }
  if constexpr (CS) {
    // forward: the even coefficients are complete; store them before the odd sums
#pragma unroll
    for (int i = 0; i < PT; ++i) {
      const int p = warp + CHEB_WARPS * i;
      if (p >= np) continue;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int gl = l0 + lane + 32 * h;
        if (gl < nlines) out[(2 * (p0 + p)) * ld_out + gl] = (TO)(accA[i][h] + cmpA[i][h]);
      }
    }
  }
  R accB[PT][2], cmpB[PT][2];  // odd sums
#pragma unroll
  for (int i = 0; i < PT; ++i) accB[i][0] = accB[i][1] = cmpB[i][0] = cmpB[i][1] = (R)0;
  for (int kb = KBp / VW - 1; kb >= 0; kb -= CG) {
    R x0[CG][VW], x1[CG][VW];
#pragma unroll
    for (int gq = 0; gq < CG; ++gq)
#pragma unroll
      for (int e = 0; e < VW; ++e) {
        const int k = (kb - gq) * VW + e;
        x0[gq][e] = k >= 0 ? xb[k * CHEB_TL + lane] : (R)0;
        x1[gq][e] = k >= 0 ? xb[k * CHEB_TL + lane + 32] : (R)0;
      }
#pragma unroll
    for (int i = 0; i < PT; ++i) {
      const int p = warp + CHEB_WARPS * i;
      if (p < np) {
        if (CS) {
          R t0 = (R)0, t1 = (R)0;
#pragma unroll
          for (int gq = 0; gq < CG; ++gq) {
            if (kb - gq < 0) break;  // uniform over the block
            const V b4 = *reinterpret_cast<const V*>(Bs + p * KBp + (kb - gq) * VW);
            const R* b = reinterpret_cast<const R*>(&b4);
#pragma unroll
            for (int e = VW - 1; e >= 0; --e) {
              t0 += b[e] * x0[gq][e];
              t1 += b[e] * x1[gq][e];
            }
          }
          two_sum_acc(accB[i][0], t0, cmpB[i][0]);
          two_sum_acc(accB[i][1], t1, cmpB[i][1]);
        } else {
          const V b4 = *reinterpret_cast<const V*>(Bs + p * KBp + kb * VW);
          const R* b = reinterpret_cast<const R*>(&b4);
#pragma unroll
          for (int e = VW - 1; e >= 0; --e) {
            accB[i][0] += b[e] * x0[0][e];
            accB[i][1] += b[e] * x1[0][e];
          }
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < PT; ++i) {
    const int pl = warp + CHEB_WARPS * i;
    if (pl >= np) continue;
    const int p = p0 + pl;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int gl = l0 + lane + 32 * h;
      if (gl >= nlines) continue;
      if (inverse) {
        // p = j in [0, J]
        out[p * ld_out + gl] = (TO)(accA[i][h] + accB[i][h]);
        if (p < J) out[(N - 1 - p) * ld_out + gl] = (TO)(accA[i][h] - accB[i][h]);
      } else {
        // p = k: even coefficient 2k (stored above by the compensated form), odd coefficient 2k+1
        if (!CS) out[(2 * p) * ld_out + gl] = (TO)accA[i][h];
        if (2 * p + 1 < N) out[(2 * p + 1) * ld_out + gl] = (TO)(CS ? accB[i][h] + cmpB[i][h] : accB[i][h]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Fused spectral curl + inverse Chebyshev transform (rotationalNL's curl and
// makePhysical_y, diffops.cpp:2229-2334, flowfield.cpp:1939-1987).
// For each real line (re or im part of one mode) the kernel evaluates, at the
// Gauss-Lobatto points y_j and y_{N-1-j}:
//   u, v, w                  from  CA (even n) / CB (odd n):  u_j = E_j + O_j, u_{N-1-j} = E_j - O_j
//   du/dy, dw/dy             from  DA (even n) / DB (odd n) with DA[j][k] = (2/L) T'_{2k}(y_j),
//                                  DB[j][k] = (2/L) T'_{2k+1}(y_j): d_j = DB.x_odd + DA.x_even,
//                                  d_{N-1-j} = DB.x_odd - DA.x_even
// adds the base flow (U, U', W, W' at y_j; -Vsuck on v) to the (0,0) mode and
// forms omega = curl(u) pointwise in y, pairing the re/im lines of a mode
// through a lane shuffle.  Output: W6[c][j][line], c = u, v, w, ox, oy, oz.
// Block: 256 threads (8 warps) x 32 lines x one half of the output rows
// (blockIdx.y): warp w handles p = 8 (2i + half) + w, i < CC_PT, and the block
// stages only those matrix rows.
// ---------------------------------------------------------------------------
#define CC_TL 32
#define CC_PT 4  // output rows per warp and block half: P <= 8 warps * 4 * 2 halves = 64

template <typename R>
__global__ void __launch_bounds__(256) k_curl_cheb(GridDev g, int N, const double* __restrict__ U, R* __restrict__ W6,
                                                   const R* __restrict__ CA, const R* __restrict__ CB,
                                                   const R* __restrict__ DA, const R* __restrict__ DB,
                                                   const R* __restrict__ basey, double Vsuck,
                                                   int bstride, Dither dt, int lpf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_wait();
  pdl_trigger();
  typedef typename Vec16<R>::T V;
  constexpr int VW = 16 / sizeof(R);
  const int P = (N + 1) / 2, KA = (N + 1) / 2, KB = (N - 1) / 2, J = (N - 1) / 2;
  // coefficient rows padded to whole 16-byte vectors (zero-filled): the matrices are read VW columns per load
  const int KAp = (KA + VW - 1) / VW * VW, KBp = (KB + VW - 1) / VW * VW, NP = KAp + KBp;
  constexpr int PL = 8 * CC_PT;  // matrix rows of this block half: local row r <-> p = 8 (2 (r / 8) + half) + r % 8
  const int half = blockIdx.y;
  R* xs = reinterpret_cast<R*>(smem_raw);  // [3][NP][CC_TL]: even coefs rows 0..KAp-1, odd KAp..NP-1
  R* sCA = xs + 3 * NP * CC_TL;
  R* sCB = sCA + PL * KAp;
  R* sDA = sCB + PL * KBp;
  R* sDB = sDA + PL * KAp;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t row = 2 * (size_t)g.Md, comp = row * N;
  // blocks never straddle two fields (lpf lines each): a block uses its field's version of the constants
  const int bpf = (lpf + CC_TL - 1) / CC_TL, fld = blockIdx.x / bpf;
  const int nlines = (fld + 1) * lpf;  // one past this field's last line
  const int l0 = fld * lpf + (blockIdx.x - fld * bpf) * CC_TL;
  const int ver = dither_ver(dt, fld);
  CA = dither_ptr(CA, ver, dt.S);
  CB = dither_ptr(CB, ver, dt.S);
  DA = dither_ptr(DA, ver, dt.S);
  DB = dither_ptr(DB, ver, dt.S);
  const float invKA = 1.0f / KAp, invKB = 1.0f / KBp;
#pragma unroll 8
  for (int i = tid; i < PL * KAp; i += blockDim.x) {
    int r, k;
    divmod_small(i, KAp, invKA, r, k);
    const int pp = 8 * (2 * (r >> 3) + half) + (r & 7);
    const bool in = k < KA && pp < P;
    sCA[i] = in ? CA[pp * KA + k] : (R)0;
    sDA[i] = in ? DA[pp * KA + k] : (R)0;
  }
#pragma unroll 8
  for (int i = tid; i < PL * KBp; i += blockDim.x) {
    int r, k;
    divmod_small(i, KBp, invKB, r, k);
    const int pp = 8 * (2 * (r >> 3) + half) + (r & 7);
    const bool in = k < KB && pp < P;
    sCB[i] = in ? CB[pp * KB + k] : (R)0;
    sDB[i] = in ? DB[pp * KB + k] : (R)0;
  }
  for (int i = tid; i < 3 * (NP - N) * CC_TL; i += blockDim.x) {  // padding rows
    const int l = i % CC_TL, t = i / CC_TL, c = t / (NP - N), e = t % (NP - N);
    const int r = e < KAp - KA ? KA + e : KAp + KB + (e - (KAp - KA));
    xs[(c * NP + r) * CC_TL + l] = (R)0;
  }
  {
    // lane l stages line l0 + l; warp w takes the coefficients n = w, w + 8, ... of each component
    const int gl = l0 + lane;
    const bool ok = gl < nlines;
    for (int c = 0; c < 3; ++c) {
      const double* uc = U + c * comp + gl;
#pragma unroll 4
      for (int n = warp; n < N; n += 8) {
        const R v = ok ? (R)uc[(size_t)n * row] : (R)0;
        const int r = (n & 1) ? KAp + (n >> 1) : (n >> 1);
        xs[(c * NP + r) * CC_TL + lane] = v;
      }
    }
  }
  __syncthreads();
  R aCu[CC_PT], aCv[CC_PT], aCw[CC_PT], aDu[CC_PT], aDw[CC_PT];   // even-coefficient sums
  R bCu[CC_PT], bCv[CC_PT], bCw[CC_PT], bDu[CC_PT], bDw[CC_PT];   // odd-coefficient sums
#pragma unroll
  for (int i = 0; i < CC_PT; ++i) aCu[i] = aCv[i] = aCw[i] = aDu[i] = aDw[i] = bCu[i] = bCv[i] = bCw[i] = bDu[i] = bDw[i] = 0;
  const R* xu = xs + lane;
  const R* xv = xs + NP * CC_TL + lane;
  const R* xw = xs + 2 * NP * CC_TL + lane;
  // high n first (the small terms are summed before the large), VW coefficients per matrix load
  for (int kb = KAp / VW - 1; kb >= 0; --kb) {
    R u[VW], v[VW], w[VW];
#pragma unroll
    for (int e = 0; e < VW; ++e) {
      const int k = kb * VW + e;
      u[e] = xu[k * CC_TL];
      v[e] = xv[k * CC_TL];
      w[e] = xw[k * CC_TL];
    }
#pragma unroll
    for (int i = 0; i < CC_PT; ++i) {
      const int p = 8 * (2 * i + half) + warp, r = warp + 8 * i;
      if (p < P) {
        const V c4 = *reinterpret_cast<const V*>(sCA + r * KAp + kb * VW);
        const V d4 = *reinterpret_cast<const V*>(sDA + r * KAp + kb * VW);
        const R* c = reinterpret_cast<const R*>(&c4);
        const R* d = reinterpret_cast<const R*>(&d4);
#pragma unroll
        for (int e = VW - 1; e >= 0; --e) {
          aCu[i] += c[e] * u[e]; aCv[i] += c[e] * v[e]; aCw[i] += c[e] * w[e];
          aDu[i] += d[e] * u[e]; aDw[i] += d[e] * w[e];
        }
      }
    }
  }
  for (int kb = KBp / VW - 1; kb >= 0; --kb) {
    R u[VW], v[VW], w[VW];
#pragma unroll
    for (int e = 0; e < VW; ++e) {
      const int k = KAp + kb * VW + e;
      u[e] = xu[k * CC_TL];
      v[e] = xv[k * CC_TL];
      w[e] = xw[k * CC_TL];
    }
#pragma unroll
    for (int i = 0; i < CC_PT; ++i) {
      const int p = 8 * (2 * i + half) + warp, r = warp + 8 * i;
      if (p < P) {
        const V c4 = *reinterpret_cast<const V*>(sCB + r * KBp + kb * VW);
        const V d4 = *reinterpret_cast<const V*>(sDB + r * KBp + kb * VW);
        const R* c = reinterpret_cast<const R*>(&c4);
        const R* d = reinterpret_cast<const R*>(&d4);
#pragma unroll
        for (int e = VW - 1; e >= 0; --e) {
          bCu[i] += c[e] * u[e]; bCv[i] += c[e] * v[e]; bCw[i] += c[e] * w[e];
          bDu[i] += d[e] * u[e]; bDw[i] += d[e] * w[e];
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
  for (int i = 0; i < CC_PT; ++i) {
    const int p = 8 * (2 * i + half) + warp;
    if (p >= P) continue;  // uniform per warp
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (h == 1 && p >= J) continue;  // middle point written once
      const int j = h == 0 ? p : N - 1 - p;
      const R sg = h == 0 ? (R)1 : (R)-1;
      R u = aCu[i] + sg * bCu[i], v = aCv[i] + sg * bCv[i], w = aCw[i] + sg * bCw[i];
      R du = bDu[i] + sg * aDu[i], dw = bDw[i] + sg * aDw[i];
      if (base) {
        u += by[j];
        du += by[N + j];
        w += by[2 * N + j];
        dw += by[3 * N + j];
        v -= vs;
      }
      const R ou = __shfl_xor_sync(0xffffffffu, u, 1);
      const R ov = __shfl_xor_sync(0xffffffffu, v, 1);
      const R ow = __shfl_xor_sync(0xffffffffu, w, 1);
      R ox, oy, oz;
      if (part == 0) {
        ox = dw + dz * ov;
        oy = -dz * ou + dx * ow;
        oz = -dx * ov - du;
      } else {
        ox = dw - dz * ov;
        oy = dz * ou - dx * ow;
        oz = dx * ov - du;
      }
      if (gl < nlines) {
        R* o = W6 + (size_t)j * row + gl;
        o[0] = u;
        o[comp] = v;
        o[2 * comp] = w;
        o[3 * comp] = ox;
        o[4 * comp] = oy;
        o[5 * comp] = oz;
      }
    }
  }
}

template <typename R>
size_t curl_cheb_smem_bytes(int N) {
  const int VW = 16 / sizeof(R);
  const int KAp = ((N + 1) / 2 + VW - 1) / VW * VW, KBp = ((N - 1) / 2 + VW - 1) / VW * VW;
  return sizeof(R) * ((size_t)3 * (KAp + KBp) * CC_TL + 2 * (size_t)(8 * CC_PT) * (KAp + KBp));
}

template <typename R>
cudaError_t launch_curl_cheb(const GridDev& g, int N, const double* U, R* W6, const R* CA, const R* CB, const R* DA,
                             const R* DB, const R* basey, double Vsuck, cudaStream_t st,
                             int bstride, const Dither& dt) {
  if ((N + 1) / 2 > 16 * CC_PT) return cudaErrorInvalidValue;
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_curl_cheb<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr_set;
  const int nf = dt.nb > 0 ? dt.nb : 1, lpf = 2 * g.Md / nf;
  return launch_pdl(k_curl_cheb<R>, dim3(nf * ((lpf + CC_TL - 1) / CC_TL), 2), dim3(256), curl_cheb_smem_bytes<R>(N),
                    st, g, N, U, W6, CA, CB, DA, DB, basey, Vsuck, bstride, dt, lpf);
}
template cudaError_t launch_curl_cheb<float>(const GridDev&, int, const double*, float*, const float*, const float*,
                                             const float*, const float*, const float*, double, cudaStream_t, int,
                                             const Dither&);
template cudaError_t launch_curl_cheb<double>(const GridDev&, int, const double*, double*, const double*,
                                              const double*, const double*, const double*, const double*, double,
                                              cudaStream_t, int, const Dither&);
template size_t curl_cheb_smem_bytes<float>(int);
template size_t curl_cheb_smem_bytes<double>(int);

// ---------------------------------------------------------------------------
// x-direction inverse FFT of the solved (kx, kz) block of one y-plane and
// component: column kz of the compact input is placed at x-wavenumber
// positions (kx >= 0 -> kx, kx < 0 -> Nx + kx), zero elsewhere, and
// transformed with exp(+2 pi i kx x/Nx).  Output X[c][ny][x][iz].
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_xinv(GridDev g, FftPlan px, const cpx<R>* __restrict__ twx,
                                              const cpx<R>* __restrict__ W, cpx<R>* __restrict__ X, int czc,
                                              Dither dt) {
  extern __shared__ unsigned char smem_raw[];
  pdl_wait();  // launched with launch_pdl: the previous kernel's output is read from here on
  twx = dither_ptr(twx, dither_ver(dt, blockIdx.x % dt.nb), dt.S);  // plane blockIdx.x -> its field's twiddles
  const int ss = g.Nx + 1;
  const int iz0 = blockIdx.z * czc;
  const int nc = min(czc, g.NKz - iz0);
  const float invc = 1.0f / nc;
  cpx<R>* a = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* b = a + (size_t)czc * ss;
  const int ny = blockIdx.x, c = blockIdx.y;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const cpx<R>* src = W + ((size_t)c * g.Ny + ny) * g.Md;
  for (int i = tid; i < nc * ss; i += nthr) a[i] = cmk<R>(0, 0);
  __syncthreads();
#pragma unroll 4
  for (int i = tid; i < g.NKx * nc; i += nthr) {
    int ix, jz;
    divmod_small(i, nc, invc, ix, jz);
    const int kx = ix <= g.Kx ? ix : ix - g.NKx;
    const int pos = kx >= 0 ? kx : g.Nx + kx;
    a[jz * ss + pos] = src[ix * g.NKz + iz0 + jz];
  }
  __syncthreads();
  fft_batch<R>(a, b, nc, ss, px, twx, +1);
  cpx<R>* dst = X + ((size_t)c * g.Ny + ny) * (size_t)g.Nx * g.NKz;
  for (int i = tid; i < g.Nx * nc; i += nthr) {
    int x, jz;
    divmod_small(i, nc, invc, x, jz);
    dst[x * g.NKz + iz0 + jz] = a[jz * ss + x];
  }
}

// ---------------------------------------------------------------------------
// x-direction forward FFT of the kz columns of one plane/component, keeping
// the solved kx and applying the 1/(Nx Nz) scale of makeSpectral_xz.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_xfwd(GridDev g, FftPlan px, const cpx<R>* __restrict__ twx,
                                              const cpx<R>* __restrict__ Z, cpx<R>* __restrict__ F, double scale_d,
                                              int czc, Dither dt) {
  extern __shared__ unsigned char smem_raw[];
  pdl_wait();  // launched with launch_pdl: the previous kernel's output is read from here on
  const int ver = dither_ver(dt, blockIdx.x % dt.nb);  // plane blockIdx.x -> its field's constants
  twx = dither_ptr(twx, ver, dt.S);
  const R scale = k_misc<R>(dt, ver, 0, scale_d);
  const int ss = g.Nx + 1;
  const int iz0 = blockIdx.z * czc;
  const int nc = min(czc, g.NKz - iz0);
  const float invc = 1.0f / nc;
  cpx<R>* a = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* b = a + (size_t)czc * ss;
  const int ny = blockIdx.x, c = blockIdx.y;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const cpx<R>* src = Z + ((size_t)c * g.Ny + ny) * (size_t)g.Nx * g.NKz;
#pragma unroll 4
  for (int i = tid; i < g.Nx * nc; i += nthr) {
    int x, jz;
    divmod_small(i, nc, invc, x, jz);
    a[jz * ss + x] = src[x * g.NKz + iz0 + jz];
  }
  __syncthreads();
  fft_batch<R>(a, b, nc, ss, px, twx, -1);
  cpx<R>* dst = F + ((size_t)c * g.Ny + ny) * g.Md;
#pragma unroll 4
  for (int i = tid; i < g.NKx * nc; i += nthr) {
    int ix, jz;
    divmod_small(i, nc, invc, ix, jz);
    const int kx = ix <= g.Kx ? ix : ix - g.NKx;
    const int pos = kx >= 0 ? kx : g.Nx + kx;
    dst[ix * g.NKz + iz0 + jz] = cscale(a[jz * ss + pos], scale);
  }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
// Output rows per block: all P while they fit one block's warps (CHEB_WARPS x CHEB_PT); taller grids run row
// blocks of CHEB_WARPS x CHEB_PT rows (FP32) or CHEB_WARPS x 4 rows (FP64, whose matrix rows take twice the
// shared memory).
int cheb_rows_per_block(int N, size_t rsize) {
  const int P = (N + 1) / 2;
  if (P <= CHEB_WARPS * CHEB_PT) return P;
  return rsize == 4 ? CHEB_WARPS * CHEB_PT : CHEB_WARPS * 4;
}

size_t cheb_smem_bytes(int N, size_t rsize) {
  const int VW = rsize == 4 ? VecLds<float>::W : VecLds<double>::W;
  const int KAp = ((N + 1) / 2 + VW - 1) / VW * VW, KBp = ((N - 1) / 2 + VW - 1) / VW * VW;
  return rsize * ((size_t)(KAp + KBp) * CHEB_TL + (size_t)cheb_rows_per_block(N, rsize) * (KAp + KBp));
}

// One launch of k_cheb with PT output rows per warp.
template <typename TI, typename R, typename TO, bool CS, int PT>
cudaError_t launch_cheb_pt(dim3 grid, size_t sm, cudaStream_t st, int N, int inverse, int nlines, const TI* in,
                           size_t ld_in, size_t cs_in, TO* out, size_t ld_out, size_t cs_out, const R* A, const R* B,
                           int P, int KA, int KB, const Dither& dt, int lpf) {
  // kernel attributes set once per process and instantiation (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_cheb<TI, R, TO, CS, PT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return true;
  }();
  (void)attr_set;
  k_cheb<TI, R, TO, CS, PT><<<grid, 32 * CHEB_WARPS, sm, st>>>(N, inverse, nlines, in, ld_in, cs_in, out, ld_out,
                                                               cs_out, A, B, P, KA, KB, dt, lpf);
  return cudaGetLastError();
}

template <typename TI, typename R, typename TO, bool CS>
cudaError_t launch_cheb_cs(dim3 grid, size_t sm, cudaStream_t st, int N, int inverse, int nlines, const TI* in,
                           size_t ld_in, size_t cs_in, TO* out, size_t ld_out, size_t cs_out, const R* A, const R* B,
                           int P, int KA, int KB, const Dither& dt, int lpf) {
  // the fewest rows per warp that cover P (registers: two sums per row and line)
  const int pt = (P + CHEB_WARPS - 1) / CHEB_WARPS;
  if (pt <= 4)
    return launch_cheb_pt<TI, R, TO, CS, 4>(grid, sm, st, N, inverse, nlines, in, ld_in, cs_in, out, ld_out, cs_out,
                                            A, B, P, KA, KB, dt, lpf);
  if (pt <= 7)
    return launch_cheb_pt<TI, R, TO, CS, 7>(grid, sm, st, N, inverse, nlines, in, ld_in, cs_in, out, ld_out, cs_out,
                                            A, B, P, KA, KB, dt, lpf);
  return launch_cheb_pt<TI, R, TO, CS, CHEB_PT>(grid, sm, st, N, inverse, nlines, in, ld_in, cs_in, out, ld_out,
                                                cs_out, A, B, P, KA, KB, dt, lpf);
}

template <typename TI, typename R, typename TO>
cudaError_t launch_cheb(int N, bool inverse, int nlines, int ncomp, const TI* in, size_t ld_in, size_t cs_in, TO* out,
                        size_t ld_out, size_t cs_out, const R* A, const R* B, cudaStream_t st, const Dither& dt) {
  const int P = (N + 1) / 2;
  const int KA = (N + 1) / 2, KB = (N - 1) / 2;
  const size_t sm = cheb_smem_bytes(N, sizeof(R));
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  const int PB = cheb_rows_per_block(N, sizeof(R));
  const int nf = dt.nb > 0 ? dt.nb : 1, lpf = (nlines + nf - 1) / nf;
  dim3 grid(nf * ((lpf + CHEB_TL - 1) / CHEB_TL), ncomp, (P + PB - 1) / PB);
  if (grid.z > 1) {
    // row blocks: the rows per warp that make one block's PB rows
    if constexpr (sizeof(R) == 4) {
      if (!inverse)
        return launch_cheb_pt<TI, R, TO, true, CHEB_PT>(grid, sm, st, N, 0, nlines, in, ld_in, cs_in, out, ld_out,
                                                        cs_out, A, B, P, KA, KB, dt, lpf);
      return launch_cheb_pt<TI, R, TO, false, CHEB_PT>(grid, sm, st, N, 1, nlines, in, ld_in, cs_in, out, ld_out,
                                                       cs_out, A, B, P, KA, KB, dt, lpf);
    } else {
      return launch_cheb_pt<TI, R, TO, false, 4>(grid, sm, st, N, inverse ? 1 : 0, nlines, in, ld_in, cs_in, out,
                                                 ld_out, cs_out, A, B, P, KA, KB, dt, lpf);
    }
  }
  // compensated sums for the FP32 forward transforms
  if constexpr (sizeof(R) == 4) {
    if (!inverse)
      return launch_cheb_cs<TI, R, TO, true>(grid, sm, st, N, 0, nlines, in, ld_in, cs_in, out, ld_out, cs_out, A, B,
                                             P, KA, KB, dt, lpf);
  }
  return launch_cheb_cs<TI, R, TO, false>(grid, sm, st, N, inverse ? 1 : 0, nlines, in, ld_in, cs_in, out, ld_out,
                                          cs_out, A, B, P, KA, KB, dt, lpf);
}

// Columns per block of the x passes: all NKz when they fit in shared memory.
template <typename R>
int xfft_cols(const GridDev& g) {
  const size_t per = 2 * sizeof(cpx<R>) * (size_t)(g.Nx + 1);
  int c = (int)((200 * 1024) / per);
  if (c > g.NKz) c = g.NKz;
  if (c < 1) c = 1;
  return c;
}
template <typename R>
size_t xfft_smem_bytes(const GridDev& g, int czc) {
  return 2 * sizeof(cpx<R>) * (size_t)(czc > 0 ? czc : xfft_cols<R>(g)) * (g.Nx + 1);
}

template <typename R>
cudaError_t launch_xinv(const GridDev& g, const FftPlan& px, const cpx<R>* twx, const cpx<R>* W, cpx<R>* X, int ncomp,
                        cudaStream_t st, int czc, const Dither& dt) {
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_xinv<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr_set;
  if (czc <= 0 || czc > g.NKz) czc = xfft_cols<R>(g);
  return launch_pdl(k_xinv<R>, dim3(g.Ny, ncomp, (g.NKz + czc - 1) / czc), dim3(256), xfft_smem_bytes<R>(g, czc), st,
                    g, px, twx, W, X, czc, dt);
}

template <typename R>
cudaError_t launch_xfwd(const GridDev& g, const FftPlan& px, const cpx<R>* twx, const cpx<R>* Z, cpx<R>* F, int ncomp,
                        cudaStream_t st, int czc, const Dither& dt) {
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_xfwd<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr_set;
  const double scale = 1.0 / ((double)g.Nx * (double)g.Nz);
  if (czc <= 0 || czc > g.NKz) czc = xfft_cols<R>(g);
  return launch_pdl(k_xfwd<R>, dim3(g.Ny, ncomp, (g.NKz + czc - 1) / czc), dim3(256), xfft_smem_bytes<R>(g, czc), st,
                    g, px, twx, Z, F, scale, czc, dt);
}

#define INST_R(R)                                                                                                   \
  template cudaError_t launch_xinv<R>(const GridDev&, const FftPlan&, const cpx<R>*, const cpx<R>*, cpx<R>*, int,   \
                                      cudaStream_t, int, const Dither&);                                            \
  template cudaError_t launch_xfwd<R>(const GridDev&, const FftPlan&, const cpx<R>*, const cpx<R>*, cpx<R>*, int,   \
                                      cudaStream_t, int, const Dither&);                                            \
  template size_t xfft_smem_bytes<R>(const GridDev&, int);

INST_R(float)
INST_R(double)

template cudaError_t launch_cheb<double, double, double>(int, bool, int, int, const double*, size_t, size_t, double*,
                                                         size_t, size_t, const double*, const double*, cudaStream_t,
                                                         const Dither&);
template cudaError_t launch_cheb<float, float, float>(int, bool, int, int, const float*, size_t, size_t, float*, size_t,
                                                      size_t, const float*, const float*, cudaStream_t, const Dither&);
template cudaError_t launch_cheb<float, float, double>(int, bool, int, int, const float*, size_t, size_t, double*,
                                                       size_t, size_t, const float*, const float*, cudaStream_t, const Dither&);
