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

template <typename R>
struct cpx {
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
