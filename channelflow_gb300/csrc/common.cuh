// Shared device/host definitions for the channelflow GB300 DNS step.
//
// Data layout in HBM (all per-DNS arrays):
//   A "mode" m is one (kx, kz) pair of the solved set: kx in [-Kx, Kx],
//   kz in [0, Kz], stored as m = ix*(Kz+1) + kz with ix = kx (kx >= 0) or
//   ix = kx + 2Kx+1 (kx < 0).  Md = (2Kx+1)(Kz+1).  m = 0 is (0,0).
//   A spectral component is complex [ny][m]  (Chebyshev index or y point
//   outermost, mode fastest), i.e. a real array [ny][2*Md] with re/im
//   interleaved.  Thread-per-mode kernels read one ny row per step, which is
//   a contiguous, coalesced 2*Md-element row.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

// ---------------------------------------------------------------------------
// Programmatic dependent launch between the kernels of a step.  A kernel launched by launch_pdl may be
// scheduled while the previous kernel of its stream is still finishing (its launch latency and CTA placement
// overlap that kernel's tail); it must call pdl_wait() before it reads or writes any global memory, which
// returns once the previous kernel has completed and its writes are visible.  pdl_trigger() lets the next
// kernel be scheduled as soon as every CTA of this one has issued it.  Both are no-ops for a kernel launched
// without the attribute.  The legacy and per-thread default streams keep plain launches.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// cfgpu_set_pdl: programmatic dependent launch on (the default) or off for launches made afterwards
int pdl_enabled();

inline bool pdl_stream(cudaStream_t st) {
  return pdl_enabled() && st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_stream(st) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// 8-byte (FP32) / 16-byte (FP64) aligned, so a complex moves with one vector load or store.
template <typename R>
struct alignas(2 * sizeof(R)) cpx {
  R x, y;
};

template <typename R>
__host__ __device__ __forceinline__ cpx<R> cmk(R a, R b) {
  cpx<R> c;
  c.x = a;
  c.y = b;
  return c;
}
template <typename R>
__host__ __device__ __forceinline__ cpx<R> cadd(cpx<R> a, cpx<R> b) { return cmk<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> csub(cpx<R> a, cpx<R> b) { return cmk<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> cmul(cpx<R> a, cpx<R> b) {
  return cmk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R>
__host__ __device__ __forceinline__ cpx<R> cconj(cpx<R> a) { return cmk<R>(a.x, -a.y); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> cscale(cpx<R> a, R s) { return cmk<R>(a.x * s, a.y * s); }

// Grid and mode-set description passed by value to kernels.
struct GridDev {
  int Nx, Ny, Nz;
  int Kx, Kz;      // solved set: |kx| <= Kx, 0 <= kz <= Kz
  int NKx;         // 2*Kx+1
  int NKz;         // Kz+1
  int Md;          // NKx*NKz
  int kxmax, kzmax;  // Nx/2, Nz/2 (Nyquist; never in the solved set)
  double Lx, Lz, a, b;
  const int* kxs;  // optional explicit mode list (batched tau solves, field batches); null = compact mapping
  const int* kzs;
  int Mf;          // modes per field when Md spans a batch of fields (m / Mf = field); 0 = one field
};

// Field (batch slot) that mode m belongs to.
__host__ __device__ __forceinline__ int mode_field(const GridDev& g, int m) { return g.Mf > 0 ? m / g.Mf : 0; }

__host__ __device__ __forceinline__ int mode_kx(const GridDev& g, int m) {
  if (g.kxs) return g.kxs[m];
  int ix = m / g.NKz;
  return ix <= g.Kx ? ix : ix - g.NKx;
}
__host__ __device__ __forceinline__ int mode_kz(const GridDev& g, int m) {
  if (g.kzs) return g.kzs[m];
  return m % g.NKz;
}

#define CFG_MAX_NY 1025

// ---------------------------------------------------------------------------
// Dithered FP32 constants (mixed precision).  Every constant the FP32 passes
// use (Chebyshev matrices, FFT twiddles, base-flow values, wavenumbers,
// scales) is a fixed operator: its rounding error is the same at every step,
// so it accumulates linearly in time while arithmetic rounding of the
// changing data accumulates like a random walk.  Each constant therefore
// exists in DITHER_V (64) roundings, a stratified stochastic rounding between the
// two floats lo < x < hi that bracket it: with f = (x - lo)/(hi - lo),
// version k is hi when f > 1 - t_k and lo otherwise, for the thresholds
// t_k = (r_k + 1/2)/V where r_k = bitrev(k) with its top bit flipped (a
// low-discrepancy order whose version 0 is round-to-nearest up to 1/(2V)).
// Over a cycle of V nonlinear evaluations the mean of the versions equals x
// to about ulp/(2V), and constants that are floats (1, the FFT scale 2^-m,
// unit twiddles, integer derivative weights) are exact in every version: an
// offset rounding of x + s ulp(x) instead would move powers of two down in
// the versions with s < -1/4 (the float spacing below 2^e is half the
// spacing above), a bias that does not average out.  Each field carries its
// own version index (state that moves with the field), advanced after every
// nonlinear evaluation.
// Version blocks are `S` bytes apart (constant tables) and `Sb` bytes apart
// (base-flow values).
// ---------------------------------------------------------------------------
#define DITHER_BITS 6
#define DITHER_V (1 << DITHER_BITS)

struct Dither {
  const int* ver;  // per-field version index; null: version 0 of undithered tables
  long long S;     // bytes between versions of the constant tables
  long long Sb;    // bytes between versions of the base-flow values
  int nb;          // fields interleaved in the plane index of the x/z passes (plane p -> field p % nb)
  // FP32 passes: version 0 of the tables of d/dx by solved kx index, d/dz by kz, and {1/(Nx Nz), Vsuck}
  // (host-built, so kernels do no FP64 arithmetic to dither them); unused by FP64 passes
  const float* kdx;
  const float* kdz;
  const float* kmisc;
};

// Threshold t_k of version k: (r + 1/2)/V with r the DITHER_BITS-bit reversal of k, top bit flipped.
__host__ __device__ __forceinline__ double dither_threshold(int k) {
  int r = 0;
  for (int b = 0; b < DITHER_BITS; ++b) r |= ((k >> b) & 1) << (DITHER_BITS - 1 - b);
  return ((r ^ (DITHER_V / 2)) + 0.5) / DITHER_V;
}

// Version k of x in FP32: the bracketing float chosen by the stratified threshold.
__host__ __device__ __forceinline__ float dither_round(double x, int k) {
  float lo = (float)x;  // nearest
  if ((double)lo == x) return lo;
  float hi;
  if ((double)lo > x) {
    hi = lo;
    lo = nextafterf(hi, -3.0e38f);
  } else {
    hi = nextafterf(lo, 3.0e38f);
  }
  const double f = (x - (double)lo) / ((double)hi - (double)lo);
  return f > 1.0 - dither_threshold(k) ? hi : lo;
}

__device__ __forceinline__ int dither_ver(const Dither& dt, int f) { return dt.ver ? __ldg(dt.ver + f) : 0; }

template <typename T>
__host__ __device__ __forceinline__ const T* dither_ptr(const T* p, int v, long long stride_bytes) {
  return reinterpret_cast<const T*>(reinterpret_cast<const char*>(p) + (long long)v * stride_bytes);
}

// Version k of the constant x in R (FP64: x itself).
template <typename R>
__device__ __forceinline__ R dither_const(double x, int k);
template <>
__device__ __forceinline__ double dither_const<double>(double x, int) {
  return x;
}
template <>
__device__ __forceinline__ float dither_const<float>(double x, int k) {
  return dither_round(x, k);
}

// Asynchronous 8-byte global -> shared copy (cp.async, no register staging); nbytes = 0 writes zeros.
__device__ __forceinline__ void cp_async8(double* dst_smem, const double* src, int nbytes) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(nbytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// 16-byte vector of R (LDS.128): four floats or two doubles.
template <typename R>
struct Vec16;
template <>
struct Vec16<float> {
  typedef float4 T;
};
template <>
struct Vec16<double> {
  typedef double2 T;
};

// Matrix loads of the dense Chebyshev kernels whose FP64 form is bound by FP64 arithmetic: 16-byte vectors
// for FP32 (fewer shared-memory instructions), scalars for FP64 (fewer registers).
template <typename R>
struct VecLds;
template <>
struct VecLds<float> {
  typedef float4 T;
  static constexpr int W = 4;
};
template <>
struct VecLds<double> {
  typedef double T;
  static constexpr int W = 1;
};

// q = i / d, r = i % d for 0 <= i < 2^22 and d >= 1, with inv = 1.0f / d: a float reciprocal and one
// correction step (the float product is within one of the quotient in that range).
__device__ __forceinline__ void divmod_small(int i, int d, float inv, int& q, int& r) {
  q = __float2int_rz(__int2float_rn(i) * inv);
  r = i - q * d;
  if (r >= d) {
    ++q;
    r -= d;
  } else if (r < 0) {
    --q;
    r += d;
  }
}

// d/dx and d/dz factors of mode (kx, kz) and the scalar constants for version ver: FP32 passes read the
// dithered tables, FP64 passes compute them (Nyquist derivatives are zero).
// Without tables (launches outside the nonlinear pass: CFL, autotuning) FP32 passes round on the fly.
template <typename R>
__device__ __forceinline__ R k_dx(const Dither& dt, int ver, const GridDev& g, int kx) {
  if constexpr (sizeof(R) == 4) {
    if (dt.kdx) return dither_ptr(dt.kdx, ver, dt.S)[kx >= 0 ? kx : kx + g.NKx];
    return dither_const<R>(2.0 * M_PI * kx / g.Lx * (kx == g.kxmax ? 0.0 : 1.0), ver);
  } else {
    return 2.0 * M_PI * kx / g.Lx * (kx == g.kxmax ? 0.0 : 1.0);
  }
}
template <typename R>
__device__ __forceinline__ R k_dz(const Dither& dt, int ver, const GridDev& g, int kz) {
  if constexpr (sizeof(R) == 4) {
    if (dt.kdz) return dither_ptr(dt.kdz, ver, dt.S)[kz];
    return dither_const<R>(2.0 * M_PI * kz / g.Lz * (kz == g.kzmax ? 0.0 : 1.0), ver);
  } else {
    return 2.0 * M_PI * kz / g.Lz * (kz == g.kzmax ? 0.0 : 1.0);
  }
}
// idx 0: 1/(Nx Nz), 1: Vsuck (value: the exact constant)
template <typename R>
__device__ __forceinline__ R k_misc(const Dither& dt, int ver, int idx, double value) {
  if constexpr (sizeof(R) == 4) {
    if (dt.kmisc) return dither_ptr(dt.kmisc, ver, dt.S)[idx];
    return dither_const<R>(value, ver);
  } else {
    return value;
  }
}
