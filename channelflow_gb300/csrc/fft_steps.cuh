// Register-resident four-step FFT building blocks (compile-time lengths, radices 4, 2 and 3).
//
// A sequence of length L = 8 N1 (N1 in {4, 6, 8, 12, 16}) sits in shared memory with one padding slot per
// N1 points (index p -> p + p / N1), at a per-sequence offset given by a functor.  Pass "S" (stride): N1
// threads per sequence, 8 points each at stride N1; pass "B" (block): 8 threads per sequence, N1 contiguous
// points each.  Every thread transforms its points in registers (mixed-radix decimation in frequency), so a
// transform costs two shared-memory round trips:
//   sign +1: natural order in -> out at pos(k) = (N1 + 1) (k % 8) + k / 8      (pass S, then pass B)
//   sign -1: in at pos(x) -> natural order out (padded)                         (pass B, then pass S)
// Twiddles come from a full-circle table exp(-2 pi i e / L), e < L.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace fsr {

__host__ __device__ constexpr int dif_radix(int L) {
  return L % 4 == 0 && L != 8 ? 4 : (L % 2 == 0 ? 2 : (L % 3 == 0 ? 3 : 1));
}
// Frequency index held at register position pos after the in-place DIF of length L.
__host__ __device__ constexpr int dif_out(int pos, int L) {
  return L == 1 ? 0 : pos / (L / dif_radix(L)) + dif_radix(L) * dif_out(pos % (L / dif_radix(L)), L / dif_radix(L));
}

// f(integral_constant<int, I>) for I = B .. E-1, so that per-index constants fold at compile time.
template <int B, int E, class Fn>
__device__ __forceinline__ void static_for(Fn&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

template <typename R, int SIGN>
__device__ __forceinline__ cpx<R> twd(const cpx<R>* tw, int e) {
  cpx<R> w = tw[e];
  if (SIGN > 0) w.y = -w.y;
  return w;
}

// r-point DFT of a[0..r) with sign SIGN (-1 forward, +1 inverse); e3 = table index of exp(-2 pi i / 3).
template <typename R, int RAD, int SIGN>
__device__ __forceinline__ void small_dft(cpx<R>* a, const cpx<R>* tw, int e3) {
  if constexpr (RAD == 2) {
    const cpx<R> t = a[0];
    a[0] = cadd(t, a[1]);
    a[1] = csub(t, a[1]);
  } else if constexpr (RAD == 4) {
    const cpx<R> s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
    const cpx<R> s13 = cadd(a[1], a[3]), d13 = csub(a[1], a[3]);
    // SIGN * i * d13
    const cpx<R> id = SIGN > 0 ? cmk<R>(-d13.y, d13.x) : cmk<R>(d13.y, -d13.x);
    a[0] = cadd(s02, s13);
    a[2] = csub(s02, s13);
    a[1] = cadd(d02, id);
    a[3] = csub(d02, id);
  } else {
    static_assert(RAD == 3, "radix");
    // omega = exp(SIGN 2 pi i / 3) = -1/2 + SIGN i h, h = sqrt(3)/2 = -Im(table[L/3])
    const R h = -tw[e3].y;
    const cpx<R> s = cadd(a[1], a[2]), d = csub(a[1], a[2]);
    const cpx<R> m = cmk<R>(a[0].x - (R)0.5 * s.x, a[0].y - (R)0.5 * s.y);
    const cpx<R> t = SIGN > 0 ? cmk<R>(-h * d.y, h * d.x) : cmk<R>(h * d.y, -h * d.x);
    a[0] = cadd(a[0], s);
    a[1] = cadd(m, t);
    a[2] = csub(m, t);
  }
}

template <typename R, int L, int OFF, int SIGN>
__device__ __forceinline__ void dif_reg(cpx<R>* x, const cpx<R>* tw, int ts);

template <typename R, int M, int OFF, int SIGN, int J, int RR>
__device__ __forceinline__ void dif_sub(cpx<R>* x, const cpx<R>* tw, int ts) {
  if constexpr (J < RR) {
    dif_reg<R, M, OFF + J * M, SIGN>(x, tw, ts);
    dif_sub<R, M, OFF, SIGN, J + 1, RR>(x, tw, ts);
  }
}

// In-place decimation-in-frequency DFT of x[OFF .. OFF+L) held in registers; the table entry of
// exp(-2 pi i / L) is tw[ts] (ts = table length / L).  Output frequency dif_out(p, L) at position OFF + p.
template <typename R, int L, int OFF, int SIGN>
__device__ __forceinline__ void dif_reg(cpx<R>* x, const cpx<R>* tw, int ts) {
  if constexpr (L > 1) {
    constexpr int RAD = dif_radix(L), M = L / RAD;
    static_assert(RAD > 1, "length must factor into 2 and 3");
#pragma unroll
    for (int i = 0; i < M; ++i) {
      cpx<R> a[RAD];
#pragma unroll
      for (int q = 0; q < RAD; ++q) a[q] = x[OFF + i + q * M];
      small_dft<R, RAD, SIGN>(a, tw, ts * M);
#pragma unroll
      for (int j = 1; j < RAD; ++j)
        if (i * j != 0) a[j] = cmul(a[j], twd<R, SIGN>(tw, i * j * ts));
#pragma unroll
      for (int j = 0; j < RAD; ++j) x[OFF + i + j * M] = a[j];
    }
    dif_sub<R, M, OFF, SIGN, 0, RAD>(x, tw, ts * RAD);
  }
}

// Sequences for the passes: seq(s) -> offset of sequence s (pitch 8 (N1 + 1)).
struct SeqLinear {
  int pitch;
  __device__ __forceinline__ int operator()(int s) const { return s * pitch; }
};
// Pass S: N1 threads per sequence; thread n1 owns points n1 + N1 n2 (n2 < 8), padded n1 + (N1 + 1) n2.
//   inverse (SIGN +1): 8-point DFT over n2, times w^(n1 k2), stored at n1 + (N1+1) k2.
//   forward (SIGN -1): 8-point DFT over a, stored at natural k = b + N1 s (padded b + (N1+1) s).
template <typename R, int N1, int SIGN, class SEQ>
__device__ __forceinline__ void pass_s(cpx<R>* base, int nseq, SEQ seq, const cpx<R>* tw, int tid, int nthr) {
  for (int t = tid; t < nseq * N1; t += nthr) {
    const int s = t / N1, n1 = t - s * N1;
    cpx<R>* q = base + seq(s) + n1;
    cpx<R> y[8];
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) y[n2] = q[(N1 + 1) * n2];
    dif_reg<R, 8, 0, SIGN>(y, tw, N1);
    static_for<0, 8>([&](auto P) {
      constexpr int p = decltype(P)::value, k2 = dif_out(p, 8);
      cpx<R> v = y[p];
      if constexpr (SIGN > 0 && k2 != 0) {
        if (n1 != 0) v = cmul(v, twd<R, SIGN>(tw, n1 * k2));
      }
      q[(N1 + 1) * k2] = v;
    });
  }
}

// Pass B: 8 threads per sequence; thread a owns the contiguous block (N1 + 1) a .. + N1.
//   inverse: N1-point DFT of the block, output k1 at block offset k1 (final layout pos(k)).
//   forward: N1-point DFT of the block, times w^(a b), output b at block offset b.
template <typename R, int N1, int SIGN, class SEQ>
__device__ __forceinline__ void pass_b(cpx<R>* base, int nseq, SEQ seq, const cpx<R>* tw, int tid, int nthr) {
  for (int t = tid; t < nseq * 8; t += nthr) {
    const int s = t >> 3, a = t & 7;
    cpx<R>* q = base + seq(s) + (N1 + 1) * a;
    cpx<R> z[N1];
#pragma unroll
    for (int n = 0; n < N1; ++n) z[n] = q[n];
    dif_reg<R, N1, 0, SIGN>(z, tw, 8);
    static_for<0, N1>([&](auto P) {
      constexpr int p = decltype(P)::value, k = dif_out(p, N1);
      cpx<R> v = z[p];
      if constexpr (SIGN < 0 && k != 0) {
        if (a != 0) v = cmul(v, twd<R, SIGN>(tw, a * k));
      }
      q[k] = v;
    });
  }
}

// Forward-transform sequences of the z phase: rows' slot 0 (f0 + i f1), then the even rows' slot 1
// (f2 of the row pair).
struct SeqZf {
  int nr, pitch;
  __device__ __forceinline__ int operator()(int s) const {
    return s < nr ? (3 * s) * pitch : (3 * (2 * (s - nr)) + 1) * pitch;
  }
};

// Asynchronous global -> shared copy of one complex value (cp.async; 8 bytes FP32, 16 bytes FP64).
template <typename R>
__device__ __forceinline__ void cp_async_cpx(cpx<R>* dst_smem, const cpx<R>* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
  if constexpr (sizeof(cpx<R>) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

template <int N1>
__device__ __forceinline__ int pos_perm(int k) {
  return (N1 + 1) * (k & 7) + (k >> 3);
}
template <int N1>
__device__ __forceinline__ int pos_nat(int k) {
  return k + k / N1;
}

}  // namespace fsr
