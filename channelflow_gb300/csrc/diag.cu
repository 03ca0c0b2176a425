// Diagnostics computed on the device: the CFL factor and the L2 norm.
//
// Reference functions restated (channelflow project paths):
//   FlowField::CFLfactor(Ubase, Wbase)   channelflow/flowfield.cpp:4035-4068
//       max over points and components of (u_i + U_i)/dx_i -- a signed maximum,
//       dx = Lx/Nx, Lz/Nz, and in y (y[ny-1]-y[ny+1])/2 ((y0-y1) at the walls)
//   DNSAlgorithm::CFL                     channelflow/dnsalgo.cpp:63-67
//   L2Norm2(FlowField, normalize=true)    channelflow/diffops.cpp:417-487 with the
//       Chebyshev quadratic form of L2Norm2(ChebyCoeff), chebyshev.cpp:758-773
#include "fft.cuh"
#include "kernels.h"

// Order-preserving map of doubles onto unsigned 64-bit integers (for atomicMax).
__device__ __forceinline__ unsigned long long dbl_key(double v) {
  const unsigned long long b = __double_as_longlong(v);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double key_dbl(unsigned long long k) {
  const unsigned long long b = (k & 0x8000000000000000ull) ? (k & ~0x8000000000000000ull) : ~k;
  double d;
  memcpy(&d, &b, sizeof(d));
  return d;
}

// z pass for the CFL factor: c2r along z of u, v, w (x-transformed planes,
// two real rows per complex FFT) and the signed maximum of u_i/dx_i.  With a
// batch of nslot fields the planes are [y][field]: plane ny belongs to field
// ny % nslot at Chebyshev point ny / nslot, and each field has its own maximum.
template <typename R>
__global__ void __launch_bounds__(256) k_zcfl(GridDev g, FftPlan pz, const cpx<R>* __restrict__ twz, int RP,
                                              const cpx<R>* __restrict__ X, const double* __restrict__ dyc, double dx,
                                              double dz, int nslot, unsigned long long* __restrict__ out) {
  extern __shared__ unsigned char smem_raw[];
  const int Nz = g.Nz, ss = Nz + 1, NKz = g.NKz;
  const int nseq = 3 * RP / 2;
  cpx<R>* A = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* B = A + (size_t)nseq * ss;
  __shared__ unsigned long long bmax;
  const int ny = blockIdx.y, x0 = blockIdx.x * RP;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const size_t plane = (size_t)g.Nx * NKz;
  if (tid == 0) bmax = 0ull;
  for (int i = tid; i < nseq * ss; i += nthr) A[i] = cmk<R>(0, 0);
  __syncthreads();
  for (int i = tid; i < nseq * NKz; i += nthr) {
    const int iz = i % NKz, s = i / NKz;
    const int k0 = 2 * s, k1 = 2 * s + 1;
    const int r0 = k0 / 3, c0 = k0 % 3, r1 = k1 / 3, c1 = k1 % 3;
    cpx<R> ca = cmk<R>(0, 0), cb = cmk<R>(0, 0);
    if (x0 + r0 < g.Nx) ca = X[((size_t)c0 * g.Ny + ny) * plane + (size_t)(x0 + r0) * NKz + iz];
    if (x0 + r1 < g.Nx) cb = X[((size_t)c1 * g.Ny + ny) * plane + (size_t)(x0 + r1) * NKz + iz];
    cpx<R>* sq = A + (size_t)s * ss;
    if (iz == 0) {
      sq[0] = cmk<R>(ca.x, cb.x);
    } else {
      sq[iz] = cmk<R>(ca.x - cb.y, ca.y + cb.x);
      sq[Nz - iz] = cmk<R>(ca.x + cb.y, -ca.y + cb.x);
    }
  }
  __syncthreads();
  fft_batch<R>(A, B, nseq, ss, pz, twz, +1);
  const double inv[3] = {1.0 / dx, 1.0 / dyc[ny / nslot], 1.0 / dz};
  double m = -1e300;
  for (int i = tid; i < RP * Nz; i += nthr) {
    const int z = i % Nz, r = i / Nz;
    if (x0 + r >= g.Nx) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int k = r * 3 + c;
      const cpx<R> v = A[(size_t)(k >> 1) * ss + z];
      const double val = (double)((k & 1) ? v.y : v.x);
      m = fmax(m, val * inv[c]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((tid & 31) == 0) atomicMax(&bmax, dbl_key(m));
  __syncthreads();
  if (tid == 0) atomicMax(out + ny % nslot, bmax);
}

// L2Norm2 over the solved modes: one thread per (component, mode, part) line;
// out[field] for a batch of fields (mode_field).
__global__ void k_l2norm2(GridDev g, int N, int ncomp, const double* __restrict__ U, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lines = 2 * g.Md;
  double s = 0.0;
  int field = 0;
  if (t < ncomp * lines) {
    field = mode_field(g, (t % lines) >> 1);
    const int c = t / lines, l = t % lines;
    const int m = l >> 1;
    const size_t row = (size_t)lines;
    const double* u = U + (size_t)c * row * N + l;
    for (int a = 0; a < N; ++a) {
      const double ua = u[(size_t)a * row];
      double ps = 0.0;
      for (int b = a % 2; b < N; b += 2) {
        const double w = (double)(1 - a * a - b * b) /
                         ((double)(1 + a - b) * (double)(1 - a + b) * (double)(1 + a + b) * (double)(1 - a - b));
        ps += u[(size_t)b * row] * w;
      }
      s += ua * ps;
    }
    s *= (mode_kz(g, m) == 0) ? 1.0 : 2.0;
  }
  if (g.Mf > 0) {
    if (s != 0.0) atomicAdd(out + field, s);
    return;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(out, s);
}

template <typename R>
cudaError_t launch_zcfl(const GridDev& g, const FftPlan& pz, const cpx<R>* twz, int RP, const cpx<R>* X,
                        const double* dyc, double dx, double dz, int nslot, unsigned long long* out, cudaStream_t st) {
  // kernel attributes set once per process (thread-safe static initialisation)
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_zcfl<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaGetLastError();
    return true;
  }();
  (void)attr_set;
  const size_t smem = 2 * sizeof(cpx<R>) * (size_t)(3 * RP / 2) * (g.Nz + 1);
  k_zcfl<R><<<dim3((g.Nx + RP - 1) / RP, g.Ny), 256, smem, st>>>(g, pz, twz, RP, X, dyc, dx, dz, nslot, out);
  return cudaGetLastError();
}

cudaError_t launch_l2norm2(const GridDev& g, int N, int ncomp, const double* U, double* out, cudaStream_t st) {
  const int T = 128, total = ncomp * 2 * g.Md;
  k_l2norm2<<<(total + T - 1) / T, T, 0, st>>>(g, N, ncomp, U, out);
  return cudaGetLastError();
}

double cfl_key_to_double(unsigned long long k) { return key_dbl(k); }

template cudaError_t launch_zcfl<float>(const GridDev&, const FftPlan&, const cpx<float>*, int, const cpx<float>*,
                                        const double*, double, double, int, unsigned long long*, cudaStream_t);
template cudaError_t launch_zcfl<double>(const GridDev&, const FftPlan&, const cpx<double>*, int,
                                         const cpx<double>*, const double*, double, double, int, unsigned long long*,
                                         cudaStream_t);

// ---------------------------------------------------------------------------
// FP64 pipe microbenchmark: the roofline denominator of the FP64 kernels.
// k_dfma_tput: every thread runs 8 independent FMA chains (a*x + b with |a| < 1,
// so values stay bounded); k_dfma_chain: one thread, one dependent chain.
// ---------------------------------------------------------------------------
__global__ void k_dfma_tput(int iters, double a, double b, double* out) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(a, x[k], b);
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

__global__ void k_dfma_chain(int iters, double a, double b, double* out, long long* cycles) {
  double x = threadIdx.x * 1e-3;
  const long long t0 = clock64();
  for (int it = 0; it < iters; ++it) x = fma(a, x, b);
  const long long t1 = clock64();
  out[0] = x;
  cycles[0] = t1 - t0;
}

int measure_fp64(int device_sms, double* tflops, double* cycles_per_fma) {
  double* d = nullptr;
  long long* c = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return 1;
  if (cudaMalloc(&c, sizeof(long long)) != cudaSuccess) { cudaFree(d); return 1; }
  const int iters = 4096, blocks = device_sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_tput<<<blocks, threads>>>(64, 0.999, 1e-3, d);  // warm-up
  cudaEventRecord(e0);
  k_dfma_tput<<<blocks, threads>>>(iters, 0.999, 1e-3, d);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  k_dfma_chain<<<1, 1>>>(iters, 0.999, 1e-3, d, c);
  long long cyc = 0;
  cudaMemcpy(&cyc, c, sizeof(cyc), cudaMemcpyDeviceToHost);
  *cycles_per_fma = (double)cyc / iters;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  cudaFree(c);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

// ---------------------------------------------------------------------------
// FieldSymmetry on spectral fields: FlowField::operator*=(FieldSymmetry) and
// FlowField::project(FieldSymmetry) (channelflow/flowfield.cpp:1095-1272).
// sigma (u,v,w)(x,y,z) = s (sx u, sy v, sz w)(sx x + ax Lx, sy y, sz z + az Lz).
// In coefficients: the image at (kx, kz) is
//   c(kx, kz, n) * X(u(sx sz kx, kz, n)),   X = conjugate when sz = -1,
//   c = s * s_i * (-1)^n [sy = -1, n odd] * exp(2 pi i (ax sx kx + az sz kz)),
// s_i = (sx, sy, sz) for the velocity components and 1 for scalars; project
// replaces u by (u + sigma u)/2.  Fields are [c][n][field][m] (nb fields).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_symmetry(GridDev g, int nb, int N, int ncomp, SymmetryDev sy, int project,
                           const cpx<R>* __restrict__ in, cpx<R>* __restrict__ out) {
  const size_t Mf = g.Md;
  const size_t total = (size_t)ncomp * N * nb * Mf;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int m = (int)(t % Mf);
  size_t r = t / Mf;
  r /= nb;  // field index does not enter the map
  const int n = (int)(r % N);
  const int c = (int)(r / N);
  const int kx = mode_kx(g, m), kz = mode_kz(g, m);
  const int skx = sy.sx * sy.sz * kx;
  const int ix = skx >= 0 ? skx : skx + g.NKx;
  const size_t src = t - m + (size_t)ix * g.NKz + kz;  // same (c, n, field), source mode
  const int si = ncomp == 3 ? (c == 0 ? sy.sx : (c == 1 ? sy.sy : sy.sz)) : 1;
  const double sign = (double)(sy.s * si * ((sy.sy == -1 && (n & 1)) ? -1 : 1));
  double sn, cs;
  sincospi(2.0 * (sy.ax * sy.sx * kx + sy.az * sy.sz * kz), &sn, &cs);
  cpx<R> v = in[src];
  const double vx = (double)v.x, vy = sy.sz == -1 ? -(double)v.y : (double)v.y;
  double wx = sign * (cs * vx - sn * vy), wy = sign * (cs * vy + sn * vx);
  if (project) {
    const cpx<R> a = in[t];
    wx = 0.5 * ((double)a.x + wx);
    wy = 0.5 * ((double)a.y + wy);
  }
  out[t] = cmk<R>((R)wx, (R)wy);
}

template <typename R>
cudaError_t launch_symmetry(const GridDev& g, int nb, int N, int ncomp, const SymmetryDev& sy, int project,
                            const void* in, void* out, cudaStream_t st) {
  const size_t total = (size_t)ncomp * N * nb * g.Md;
  const int T = 256;
  k_symmetry<R><<<(unsigned)((total + T - 1) / T), T, 0, st>>>(g, nb, N, ncomp, sy, project,
                                                              (const cpx<R>*)in, (cpx<R>*)out);
  return cudaGetLastError();
}

template cudaError_t launch_symmetry<float>(const GridDev&, int, int, int, const SymmetryDev&, int, const void*, void*,
                                            cudaStream_t);
template cudaError_t launch_symmetry<double>(const GridDev&, int, int, int, const SymmetryDev&, int, const void*,
                                             void*, cudaStream_t);

// ---------------------------------------------------------------------------
// Direct host access (devices whose kernels reach pageable host memory through the host page tables,
// as GB300 does over NVLink-C2C): FlowField buffers in host memory ([field][c][ny][mx][mz] complex,
// channelflow/flowfield.h layout) are read into / written from the solved-mode layout
// ([c][ny][field][m] complex) by one kernel, without host-side gathers or staging copies.  Consecutive
// threads take consecutive kz of one (c, ny, kx) row: contiguous on both sides.  VEC: 16-byte accesses.
// ---------------------------------------------------------------------------
template <bool TO_DEVICE, bool VEC>
__global__ void __launch_bounds__(256) k_host_modes(GridDev g, int Nd, int nf, int f0, int fstride,
                                                    const double* __restrict__ src, double* __restrict__ dst) {
  const int Mz = g.Nz / 2 + 1;
  const size_t hfield = (size_t)2 * Nd * g.Ny * g.Nx * Mz;
  const size_t total = (size_t)nf * Nd * g.Ny * g.Md;
  const size_t step = (size_t)gridDim.x * blockDim.x;
  for (size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t0 < total; t0 += 4 * step) {
    size_t so[4], dof[4];
    bool ok[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const size_t t = t0 + k * step;
      ok[k] = t < total;
      const size_t tt = ok[k] ? t : 0;
      const int iz = (int)(tt % g.NKz);
      size_t r = tt / g.NKz;
      const int ix = (int)(r % g.NKx);
      r /= g.NKx;
      const int ny = (int)(r % g.Ny);
      r /= g.Ny;
      const int c = (int)(r % Nd);
      const int f = (int)(r / Nd);
      const int kx = ix <= g.Kx ? ix : ix - g.NKx;
      const int mx = kx >= 0 ? kx : kx + g.Nx;
      const size_t h = f * hfield + 2 * ((((size_t)c * g.Ny + ny) * g.Nx + mx) * Mz + iz);
      const size_t dv = 2 * ((((size_t)c * g.Ny + ny) * fstride + (f0 + f)) * g.Md + (size_t)ix * g.NKz + iz);
      so[k] = TO_DEVICE ? h : dv;
      dof[k] = TO_DEVICE ? dv : h;
    }
    if (VEC) {
      double2 v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (ok[k]) v[k] = *reinterpret_cast<const double2*>(src + so[k]);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (ok[k]) *reinterpret_cast<double2*>(dst + dof[k]) = v[k];
    } else {
      double a[4], b[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (ok[k]) {
          a[k] = src[so[k]];
          b[k] = src[so[k] + 1];
        }
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (ok[k]) {
          dst[dof[k]] = a[k];
          dst[dof[k] + 1] = b[k];
        }
    }
  }
}

cudaError_t launch_host_modes(const GridDev& g, bool to_device, int Nd, int nf, int f0, int fstride, const double* src,
                              double* dst, cudaStream_t st) {
  const size_t total = (size_t)nf * Nd * g.Ny * g.Md;
  if (total == 0) return cudaSuccess;
  const size_t need = (total + 4 * 256 - 1) / (4 * 256);
  const unsigned blocks = (unsigned)(need < 152 * 16 ? need : 152 * 16);
  const bool vec = (((uintptr_t)src | (uintptr_t)dst) & 15) == 0;
  if (to_device) {
    if (vec) k_host_modes<true, true><<<blocks, 256, 0, st>>>(g, Nd, nf, f0, fstride, src, dst);
    else k_host_modes<true, false><<<blocks, 256, 0, st>>>(g, Nd, nf, f0, fstride, src, dst);
  } else {
    if (vec) k_host_modes<false, true><<<blocks, 256, 0, st>>>(g, Nd, nf, f0, fstride, src, dst);
    else k_host_modes<false, false><<<blocks, 256, 0, st>>>(g, Nd, nf, f0, fstride, src, dst);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// field2vector / vector2field (channelflow/flowfield.cpp:4448-4760) on a field in the solved-mode layout
// (field f of a batch of fstride fields).  The vector holds the independent real coefficients of a
// divergence-free no-slip velocity: the (0,0) block (u, w real, n = 2..Ny-1), then one block of 4Ny-12
// per mode in the reference's order ((kx,0) kx = 1..Kx; (0,kz) kz = 1..Kz; (kx,kz) kx = -Kx..Kx, kx != 0,
// kz = 1..Kz): first component cA at n = 2..Ny-1, then cB at n = 3..Ny-2, re/im interleaved, with
// (cA, cB) = (w, u) for the (kx,0) modes and (u, w) otherwise.  ord[j] = solved-mode index of block j;
// blk[m] = block of mode m (-1: the (0,0) mode; -(j+2): the conjugate of block j, kz = 0 and kx < 0).
// ---------------------------------------------------------------------------
struct CLine {  // complex Chebyshev line of one mode: element n at p + n*s (re), +1 (im)
  double* p;
  size_t s;
  __device__ __forceinline__ double& re(int n) const { return p[(size_t)n * s]; }
  __device__ __forceinline__ double& im(int n) const { return p[(size_t)n * s + 1]; }
};

__global__ void k_field2vector(GridDev g, int f, int fstride, const int* __restrict__ ord, int nblk,
                               const double* __restrict__ U, double* __restrict__ v) {
  const int Ny = g.Ny, B = 4 * Ny - 12, off0 = 2 * (Ny - 2);
  const size_t total = (size_t)off0 + (size_t)nblk * B;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= total) return;
  const size_t row = 2 * (size_t)g.Md * fstride, comp = row * Ny, fo = 2 * (size_t)g.Md * f;
  if (t < (size_t)off0) {  // (0,0): u then w, real parts, n = 2..Ny-1
    const int c = t < (size_t)(Ny - 2) ? 0 : 2, n = 2 + (int)(t % (Ny - 2));
    v[t] = U[c * comp + n * row + fo];
    return;
  }
  const size_t r = t - off0;
  const int j = (int)(r / B), e = (int)(r % B);
  const int m = ord[j];
  const bool kz0 = mode_kz(g, m) == 0;
  int c, n;
  if (e < 2 * (Ny - 2)) {
    c = kz0 ? 2 : 0;
    n = 2 + e / 2;
  } else {
    c = kz0 ? 0 : 2;
    n = 3 + (e - 2 * (Ny - 2)) / 2;
  }
  v[t] = U[c * comp + n * row + fo + 2 * (size_t)m + (e & 1)];
}

__device__ void cl_eval(const CLine& L, int N, double* a_re, double* a_im, double* b_re, double* b_im) {
  double sar = 0, sai = 0, sbr = 0, sbi = 0;
  for (int n = N - 1; n >= 0; --n) {
    const double r = L.re(n), i = L.im(n);
    sbr += r;
    sbi += i;
    if (n % 2 == 0) {
      sar += r;
      sai += i;
    } else {
      sar -= r;
      sai -= i;
    }
  }
  *a_re = sar, *a_im = sai, *b_re = sbr, *b_im = sbi;
}
__device__ void cl_mean(const CLine& L, int N, double* re, double* im) {
  double sr = L.re(0), si = L.im(0);
  for (int n = 2; n < N; n += 2) {
    sr -= L.re(n) / (double)(n * n - 1);
    si -= L.im(n) / (double)(n * n - 1);
  }
  *re = sr, *im = si;
}
__device__ void cl_fix_diri(const CLine& L, int N) {
  double ar, ai, br, bi;
  cl_eval(L, N, &ar, &ai, &br, &bi);
  L.re(0) -= 0.5 * (br + ar), L.im(0) -= 0.5 * (bi + ai);
  L.re(1) -= 0.5 * (br - ar), L.im(1) -= 0.5 * (bi - ai);
}
// f(a) = f(b) = 0 and mean(f) + extra = 0 through f[0..2] (fixDiriMean with extra = 0)
__device__ void cl_fix_diri_mean(const CLine& L, int N, double xr, double xi) {
  double ar, ai, br, bi, mr, mi;
  cl_eval(L, N, &ar, &ai, &br, &bi);
  cl_mean(L, N, &mr, &mi);
  mr += xr, mi += xi;
  L.re(0) -= 0.125 * (ar + br) + 0.75 * mr, L.im(0) -= 0.125 * (ai + bi) + 0.75 * mi;
  L.re(1) -= 0.5 * (br - ar), L.im(1) -= 0.5 * (bi - ai);
  L.re(2) -= 0.375 * (ar + br) - 0.75 * mr, L.im(2) -= 0.375 * (ai + bi) - 0.75 * mi;
}
// u = integrate(du) (zero mean), then u[0] -= (u(a) + u(b))/2, then u *= (0, k)
__device__ void cl_integrate_v(const CLine& du, const CLine& u, int N, double h2, double k) {
  u.re(1) = h2 * (du.re(0) - du.re(2) / 2), u.im(1) = h2 * (du.im(0) - du.im(2) / 2);
  for (int n = 2; n < N - 1; ++n) {
    u.re(n) = h2 * (du.re(n - 1) - du.re(n + 1)) / (2 * n);
    u.im(n) = h2 * (du.im(n - 1) - du.im(n + 1)) / (2 * n);
  }
  u.re(N - 1) = h2 * du.re(N - 2) / (2 * (N - 1)), u.im(N - 1) = h2 * du.im(N - 2) / (2 * (N - 1));
  u.re(0) = 0.0, u.im(0) = 0.0;
  double mr, mi;
  cl_mean(u, N, &mr, &mi);
  u.re(0) = -mr, u.im(0) = -mi;
  double ar, ai, br, bi;
  cl_eval(u, N, &ar, &ai, &br, &bi);
  u.re(0) -= 0.5 * (ar + br), u.im(0) -= 0.5 * (ai + bi);
  if (k != 1.0)
    for (int n = 0; n < N; ++n) {
      const double r = u.re(n), i = u.im(n);
      u.re(n) = -k * i, u.im(n) = k * r;
    }
}

__global__ void k_vector2field(GridDev g, int f, int fstride, const int* __restrict__ blk,
                               const double* __restrict__ v, double* __restrict__ U, double* __restrict__ W) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.Md) return;
  const int Ny = g.Ny, B = 4 * Ny - 12, off0 = 2 * (Ny - 2);
  const size_t row = 2 * (size_t)g.Md * fstride, comp = row * Ny, fo = 2 * (size_t)g.Md * f + 2 * (size_t)m;
  const CLine Lu{U + fo, row}, Lv{U + comp + fo, row}, Lw{U + 2 * comp + fo, row};
  const CLine Ls{W + 2 * (size_t)m, 2 * (size_t)g.Md};  // scratch line of this mode
  const double h2 = (g.b - g.a) / 2;
  const int b = blk[m];
  for (int n = 0; n < Ny; ++n) {
    Lu.re(n) = Lu.im(n) = Lv.re(n) = Lv.im(n) = Lw.re(n) = Lw.im(n) = 0.0;
  }
  if (b == -1) {  // (0,0): u and w real, v = 0
    for (int n = 2; n < Ny; ++n) {
      Lu.re(n) = v[n - 2];
      Lw.re(n) = v[(Ny - 2) + n - 2];
    }
    cl_fix_diri(Lu, Ny);
    cl_fix_diri(Lw, Ny);
    return;
  }
  const int j = b >= 0 ? b : -(b + 2);
  const double* a = v + off0 + (size_t)j * B;
  const int kx = b >= 0 ? mode_kx(g, m) : -mode_kx(g, m), kz = mode_kz(g, m);
  const double ax = 2 * M_PI * kx / g.Lx, gz = 2 * M_PI * kz / g.Lz;
  const CLine& LA = kz == 0 ? Lw : Lu;  // first block part: n = 2..Ny-1
  const CLine& LB = kz == 0 ? Lu : Lw;  // second part: n = 3..Ny-2
  for (int n = 2; n < Ny; ++n) {
    LA.re(n) = a[2 * (n - 2)];
    LA.im(n) = a[2 * (n - 2) + 1];
  }
  cl_fix_diri(LA, Ny);
  for (int n = 3; n < Ny - 1; ++n) {
    LB.re(n) = a[2 * (Ny - 2) + 2 * (n - 3)];
    LB.im(n) = a[2 * (Ny - 2) + 2 * (n - 3) + 1];
  }
  if (kz == 0 || kx == 0) {
    cl_fix_diri_mean(LB, Ny, 0.0, 0.0);
    cl_integrate_v(LB, Lv, Ny, h2, kz == 0 ? -ax : -gz);  // v = int(-d/dx u) or int(-d/dz w)
  } else {
    const double r = (double)(kx * g.Lz) / (kz * g.Lx);
    Lw.re(Ny - 1) = -Lu.re(Ny - 1) * r, Lw.im(Ny - 1) = -Lu.im(Ny - 1) * r;
    double mr, mi;
    cl_mean(Lu, Ny, &mr, &mi);
    cl_fix_diri_mean(Lw, Ny, r * mr, r * mi);
    // v = int(-i ax u - i gz w) dy
    for (int n = 0; n < Ny; ++n) {
      Ls.re(n) = ax * Lu.im(n) + gz * Lw.im(n);
      Ls.im(n) = -(ax * Lu.re(n) + gz * Lw.re(n));
    }
    cl_integrate_v(Ls, Lv, Ny, h2, 1.0);
  }
  if (b < -1)  // kz = 0, kx < 0: the conjugate of (|kx|, 0)
    for (int n = 0; n < Ny; ++n) Lu.im(n) = -Lu.im(n), Lv.im(n) = -Lv.im(n), Lw.im(n) = -Lw.im(n);
}

cudaError_t launch_field2vector(const GridDev& g, int f, int fstride, const int* ord, int nblk, const double* U,
                                double* v, cudaStream_t st) {
  const size_t total = 2 * (size_t)(g.Ny - 2) + (size_t)nblk * (4 * g.Ny - 12);
  k_field2vector<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g, f, fstride, ord, nblk, U, v);
  return cudaGetLastError();
}

cudaError_t launch_vector2field(const GridDev& g, int f, int fstride, const int* blk, const double* v, double* U,
                                double* W, cudaStream_t st) {
  k_vector2field<<<(g.Md + 63) / 64, 64, 0, st>>>(g, f, fstride, blk, v, U, W);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// GMRES orthogonalisation in FP64 (the Arnoldi step of nsolver/gmres.cpp:47-83): w is made orthogonal to
// the k rows of V (k x n) by classical Gram-Schmidt applied twice, h_j = sum of both passes' projections,
// h_k = |w| afterwards, w /= h_k.  Reductions are deterministic: per-block partial sums in a fixed order,
// then one block sums the partials in index order.
// ---------------------------------------------------------------------------
#define ORTHO_T 256
__device__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = ORTHO_T / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// partial[j * nb + b] = sum over block b's slice of V[j][i] w[i] (j < k), or of w[i]^2 (j == k, V unused)
__global__ void __launch_bounds__(ORTHO_T) k_ortho_dots(int n, int k, const double* __restrict__ V,
                                                        const double* __restrict__ w, int norm_only,
                                                        double* __restrict__ partial) {
  __shared__ double sh[ORTHO_T];
  const int nb = gridDim.x, b = blockIdx.x;
  const int j = blockIdx.y;  // row (or the norm when norm_only)
  const size_t per = ((size_t)n + nb - 1) / nb, i0 = (size_t)b * per, i1 = min((size_t)n, i0 + per);
  double s = 0.0;
  for (size_t i = i0 + threadIdx.x; i < i1; i += ORTHO_T) s += norm_only ? w[i] * w[i] : V[(size_t)j * n + i] * w[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[(size_t)j * nb + b] = s;
}

__global__ void __launch_bounds__(ORTHO_T) k_ortho_reduce(int nb, int rows, const double* __restrict__ partial,
                                                          double* __restrict__ out, int accumulate) {
  __shared__ double sh[ORTHO_T];
  const int j = blockIdx.x;
  if (j >= rows) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += ORTHO_T) s += partial[(size_t)j * nb + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[j] = accumulate ? out[j] + s : s;
}

// w[i] -= sum_j c[j] V[j][i]
__global__ void k_ortho_update(int n, int k, const double* __restrict__ V, const double* __restrict__ c,
                               double* __restrict__ w) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n) return;
  double s = w[i];
  for (int j = 0; j < k; ++j) s -= c[j] * V[(size_t)j * n + i];
  w[i] = s;
}

__global__ void k_ortho_scale(int n, const double* __restrict__ nrm2, double* __restrict__ w, double* __restrict__ h,
                              int k) {
  const double nrm = sqrt(nrm2[0]);
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i == 0) h[k] = nrm;
  if (i < (size_t)n && nrm > 0.0) w[i] /= nrm;
}

// work: (k + 1) * 64 + k + 1 doubles
cudaError_t launch_orthogonalize(int n, int k, const double* V, double* w, double* h, double* work,
                                 cudaStream_t st) {
  const int nb = 64;
  double* partial = work;
  double* c = work + (size_t)(k + 1) * nb;
  for (int pass = 0; pass < 2 && k > 0; ++pass) {
    k_ortho_dots<<<dim3(nb, k), ORTHO_T, 0, st>>>(n, k, V, w, 0, partial);
    k_ortho_reduce<<<k, ORTHO_T, 0, st>>>(nb, k, partial, c, 0);
    k_ortho_reduce<<<k, ORTHO_T, 0, st>>>(nb, k, partial, h, pass);  // h = pass 1 + pass 2 projections
    k_ortho_update<<<(unsigned)(((size_t)n + 255) / 256), 256, 0, st>>>(n, k, V, c, w);
  }
  k_ortho_dots<<<dim3(nb, 1), ORTHO_T, 0, st>>>(n, 0, V, w, 1, partial);
  k_ortho_reduce<<<1, ORTHO_T, 0, st>>>(nb, 1, partial, c, 0);
  k_ortho_scale<<<(unsigned)(((size_t)n + 255) / 256), 256, 0, st>>>(n, c, w, h, k);
  return cudaGetLastError();
}
