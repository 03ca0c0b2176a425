// Batched mixed-radix (2,3,4,5) Stockham FFT on sequences held in shared memory.
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

struct FftPlan {
  int L;
  int nst;
  int radix[FFT_MAX_STAGES];
  int Ns[FFT_MAX_STAGES];
  int twoff[FFT_MAX_STAGES];
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
__device__ void fft_batch(cpx<R>* a, cpx<R>* b, int nseq, int ss, const FftPlan& p, const cpx<R>* __restrict__ tw,
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
