// Batched mixed-radix (2,3,4,5; other primes as direct DFTs) Stockham FFT on sequences held in shared memory.
//
// One thread block transforms `nseq` sequences of length L together: every
// stage is a sweep over nseq*L/R radix-R butterflies shared by all threads,
// with a __syncthreads() between stages and ping-pong buffers a <-> b.
// Unnormalised; sign = -1 is the forward transform exp(-2 pi i jk/L) (the
// FFTW convention), sign = +1 the inverse.
//
// Stage s with radix R and Ns = product of the earlier radices maps
//   butterfly j (0 <= j < L/R), k = j mod Ns:
//     x_r = src[j + r L/R] * w^{r k},  w = exp(sign 2 pi i / (Ns R))
//     dst[(j - k) R + k + p Ns] = sum_r x_r exp(sign 2 pi i r p / R)
// (the self-sorting Stockham formulation).  Twiddles come from a table built
// on the host in double precision: entry twoff[s] + k*(R-1) + (r-1) holds
// exp(-2 pi i r k/(Ns R)); the inverse uses its conjugate.
#pragma once

#include "common.cuh"

#define FFT_MAX_STAGES 12
#define FFT_MAX_RADIX 127  // largest prime factor of a length (radices above 5 run as direct DFTs)

struct FftPlan {
  int L;
  int nst;
  int radix[FFT_MAX_STAGES];
  int Ns[FFT_MAX_STAGES];
  int twoff[FFT_MAX_STAGES];
  int rootoff[FFT_MAX_STAGES];  // radix > 5: offset of exp(-2 pi i e / R), e < R, in the table; else -1
  int twlen;  // total twiddle entries
};

template <typename R>
__device__ __forceinline__ void dft2(cpx<R>* x) {
  cpx<R> t = x[0];
  x[0] = cadd(t, x[1]);
  x[1] = csub(t, x[1]);
}

// multiply by sign*i
template <typename R>
__device__ __forceinline__ cpx<R> mul_si(cpx<R> a, int sign) {
  return sign < 0 ? cmk<R>(a.y, -a.x) : cmk<R>(-a.y, a.x);
}

template <typename R>
__device__ __forceinline__ void dft4(cpx<R>* x, int sign) {
  cpx<R> a0 = cadd(x[0], x[2]);
  cpx<R> a1 = csub(x[0], x[2]);
  cpx<R> a2 = cadd(x[1], x[3]);
  cpx<R> a3 = mul_si(csub(x[1], x[3]), sign);
  x[0] = cadd(a0, a2);
  x[2] = csub(a0, a2);
  x[1] = cadd(a1, a3);
  x[3] = csub(a1, a3);
}

template <typename R>
__device__ __forceinline__ void dft3(cpx<R>* x, int sign) {
  const R h = (R)0.86602540378443864676;  // sqrt(3)/2
  cpx<R> s = cadd(x[1], x[2]);
  cpx<R> d = csub(x[1], x[2]);
  cpx<R> m = cmk<R>(x[0].x - (R)0.5 * s.x, x[0].y - (R)0.5 * s.y);
  cpx<R> t = mul_si(cscale(d, h), sign);
  x[0] = cadd(x[0], s);
  x[1] = cadd(m, t);
  x[2] = csub(m, t);
}

template <typename R>
__device__ __forceinline__ void dft5(cpx<R>* x, int sign) {
  const R c1 = (R)0.30901699437494742410;   // cos(2pi/5)
  const R c2 = (R)-0.80901699437494742410;  // cos(4pi/5)
  const R s1 = (R)0.95105651629515357212;   // sin(2pi/5)
  const R s2 = (R)0.58778525229247312917;   // sin(4pi/5)
  cpx<R> a1 = cadd(x[1], x[4]), b1 = csub(x[1], x[4]);
  cpx<R> a2 = cadd(x[2], x[3]), b2 = csub(x[2], x[3]);
  cpx<R> m1 = cmk<R>(x[0].x + c1 * a1.x + c2 * a2.x, x[0].y + c1 * a1.y + c2 * a2.y);
  cpx<R> m2 = cmk<R>(x[0].x + c2 * a1.x + c1 * a2.x, x[0].y + c2 * a1.y + c1 * a2.y);
  cpx<R> t1 = mul_si(cmk<R>(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y), sign);
  cpx<R> t2 = mul_si(cmk<R>(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y), sign);
  x[0] = cmk<R>(x[0].x + a1.x + a2.x, x[0].y + a1.y + a2.y);
  x[1] = cadd(m1, t1);
  x[4] = csub(m1, t1);
  x[2] = cadd(m2, t2);
  x[3] = csub(m2, t2);
}

// Transforms nseq sequences (stride `ss` complex elements apart, unit element
// stride) in place; the result is left in `a` (the routine copies back after
// an odd number of stages).  Must be called by all threads of the block.
template <typename R>
__device__ void fft_batch_generic(cpx<R>* a, cpx<R>* b, int nseq, int ss, const FftPlan& p, const cpx<R>* __restrict__ tw,
                          int sign) {
  const int L = p.L;
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  cpx<R>* src = a;
  cpx<R>* dst = b;
  for (int s = 0; s < p.nst; ++s) {
    const int Rr = p.radix[s];
    const int Ns = p.Ns[s];
    const int LR = L / Rr;
    const int total = nseq * LR;
    const cpx<R>* twt = tw + p.twoff[s];
    if (Rr > 5) {
      // direct DFT of a prime radix: the butterfly's inputs (read by no other butterfly of the stage) are
      // twiddled in place, then every output sums over them with the stage's DFT matrix entries
      const cpx<R>* rt = tw + p.rootoff[s];
      for (int idx = tid; idx < total; idx += nthr) {
        const int q = idx / LR;
        const int j = idx - q * LR;
        const int k = j % Ns;
        cpx<R>* sp = src + q * ss + j;
        for (int r = 1; r < Rr; ++r) {
          cpx<R> w = twt[k * (Rr - 1) + (r - 1)];
          if (sign > 0) w.y = -w.y;
          sp[r * LR] = cmul(sp[r * LR], w);
        }
        cpx<R>* dp = dst + q * ss + (j - k) * Rr + k;
        for (int o = 0; o < Rr; ++o) {
          cpx<R> acc = sp[0];
          int e = 0;
          for (int r = 1; r < Rr; ++r) {
            e += o;
            if (e >= Rr) e -= Rr;
            cpx<R> w = rt[e];
            if (sign > 0) w.y = -w.y;
            acc = cadd(acc, cmul(sp[r * LR], w));
          }
          dp[o * Ns] = acc;
        }
      }
      __syncthreads();
      cpx<R>* t = src;
      src = dst;
      dst = t;
      continue;
    }
    for (int idx = tid; idx < total; idx += nthr) {
      const int q = idx / LR;
      const int j = idx - q * LR;
      const int k = j % Ns;
      const cpx<R>* sp = src + q * ss + j;
      cpx<R> x[5];
      x[0] = sp[0];
      for (int r = 1; r < Rr; ++r) {
        cpx<R> w = twt[k * (Rr - 1) + (r - 1)];
        if (sign > 0) w.y = -w.y;
        x[r] = cmul(sp[r * LR], w);
      }
      switch (Rr) {
        case 2: dft2(x); break;
        case 3: dft3(x, sign); break;
        case 4: dft4(x, sign); break;
        default: dft5(x, sign); break;
      }
      cpx<R>* dp = dst + q * ss + (j - k) * Rr + k;
      for (int r = 0; r < Rr; ++r) dp[r * Ns] = x[r];
    }
    __syncthreads();
    cpx<R>* t = src;
    src = dst;
    dst = t;
  }
  if (src != a) {
    const int total = nseq * ss;
    for (int idx = tid; idx < total; idx += nthr) a[idx] = src[idx];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Compile-time-length variant.  The radix of each stage is chosen as the host
// plan does (all 4s, then one 2, then 3s, then 5s), so the twiddle offsets
// TWOFF accumulate exactly like FftPlan::twoff.
// ---------------------------------------------------------------------------
template <int REM>
struct RadixOf {
  static constexpr int v = REM % 4 == 0 ? 4 : (REM % 2 == 0 ? 2 : (REM % 3 == 0 ? 3 : 5));
};

template <typename R, int RAD>
__device__ __forceinline__ void dft_fixed(cpx<R>* x, int sign) {
  if constexpr (RAD == 2) dft2(x);
  else if constexpr (RAD == 3) dft3(x, sign);
  else if constexpr (RAD == 4) dft4(x, sign);
  else dft5(x, sign);
}

template <typename R, int L, int Ns, int TWOFF, int PARITY>
__device__ __forceinline__ void fft_fixed_stages(cpx<R>* src, cpx<R>* dst, cpx<R>* a, int nseq, int ss,
                                                 const cpx<R>* __restrict__ tw, int sign, int tid, int nthr) {
  if constexpr (Ns >= L) {
    if constexpr (PARITY == 1) {
      // result is in src (== b); copy back to a
      const int total = nseq * ss;
      for (int idx = tid; idx < total; idx += nthr) a[idx] = src[idx];
      __syncthreads();
    }
  } else {
    constexpr int RAD = RadixOf<L / Ns>::v;
    constexpr int LR = L / RAD;
    const int total = nseq * LR;
    for (int idx = tid; idx < total; idx += nthr) {
      const int qq = idx / LR;
      const int j = idx - qq * LR;
      const int k = j % Ns;
      const cpx<R>* sp = src + qq * ss + j;
      cpx<R> x[RAD];
#pragma unroll
      for (int r = 0; r < RAD; ++r) x[r] = sp[r * LR];
      if constexpr (Ns > 1) {
#pragma unroll
        for (int r = 1; r < RAD; ++r) {
          cpx<R> w = tw[TWOFF + k * (RAD - 1) + (r - 1)];
          if (sign > 0) w.y = -w.y;
          x[r] = cmul(x[r], w);
        }
      }
      dft_fixed<R, RAD>(x, sign);
      cpx<R>* dp = dst + qq * ss + (j - k) * RAD + k;
#pragma unroll
      for (int r = 0; r < RAD; ++r) dp[r * Ns] = x[r];
    }
    __syncthreads();
    fft_fixed_stages<R, L, Ns * RAD, TWOFF + Ns * (RAD - 1), 1 - PARITY>(dst, src, a, nseq, ss, tw, sign, tid, nthr);
  }
}

// Dispatch to a compile-time length when the plan length is one of the common grid sizes.
template <typename R>
__device__ void fft_batch(cpx<R>* a, cpx<R>* b, int nseq, int ss, const FftPlan& p, const cpx<R>* __restrict__ tw,
                          int sign) {
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
#define FFT_CASE(LL)                                                              \
  case LL:                                                                        \
    fft_fixed_stages<R, LL, 1, 0, 0>(a, b, a, nseq, ss, tw, sign, tid, nthr);      \
    return;
  switch (p.L) {
    FFT_CASE(4)
    FFT_CASE(8)
    FFT_CASE(12)
    FFT_CASE(16)
    FFT_CASE(24)
    FFT_CASE(32)
    FFT_CASE(48)
    FFT_CASE(64)
    FFT_CASE(96)
    FFT_CASE(128)
    FFT_CASE(192)
    FFT_CASE(256)
    default:
      fft_batch_generic<R>(a, b, nseq, ss, p, tw, sign);
  }
#undef FFT_CASE
}
