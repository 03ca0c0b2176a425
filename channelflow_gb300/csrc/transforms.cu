// FlowField transforms on the GPU: makePhysical / makeSpectral and their
// xz and y halves, on a whole FlowField buffer in the reference's serial
// layout (every mode, Nyquist included), FP64.
//
// Reference functions restated (channelflow project paths):
//   FlowField::makeSpectral_xz / makePhysical_xz   channelflow/flowfield.cpp:1850-1886
//       (FFTW r2c / c2r over (x, z) per (y, component), 1/(Nx Nz) on the forward transform)
//   FlowField::makeSpectral_y / makePhysical_y     channelflow/flowfield.cpp:1888-1987
//       (REDFT00 along y per (x, z, component); chebyfft/ichebyfft scaling, chebyshev.cpp:262-303)
//   FlowField::makeSpectral / makePhysical         channelflow/flowfield.cpp:1989-1997
//   the (xzstate, ystate) bookkeeping              channelflow/flowfield.h:280-282
//
// Buffer layout (flowfield.h:370-400): Nd*Ny*Nx*Nzpad doubles, Nzpad = 2*(Nz/2+1).
//   xz-physical:  real u(nx, ny, nz, i) at nz + Nzpad*(nx + Nx*(ny + Ny*i)), nz < Nz
//   xz-spectral:  complex u(mx, my, mz, i) at mz + Mz*(mx + Nx*(my + Ny*i)), Mz = Nz/2+1
// The y transforms act on the reals along y (stride Nx*Nzpad) in either xz state, so a y transform of an
// xz-spectral field transforms the real and imaginary parts of every mode.
//
// Kernels (not on the DNS step's hot path, which keeps only solved modes and fuses its transforms into the
// nonlinear pass):
//   k_cheb_full   dense Ny x Ny FP64 product per y-line, 32 x 32 output tiles staged through shared memory
//   k_xcols       complex FFT along x of kz columns of one (y, component) plane, in place
//   k_zrows       z transform of x rows: c2r (Hermitian completion, FFTW's convention of taking only the
//                 real parts of the kz = 0 and Nz/2 terms) or r2c, in place
// The FFTs are the library's shared-memory Stockham FFT (fft.cuh) with twiddles built in long double.
#include "../../include/cfgpu.h"
#include "kernels.h"

#include <cmath>
#include <complex>
#include <string>
#include <vector>

bool cfgpu_fft_plan(int L, FftPlan& p, std::vector<std::complex<long double>>& tw);

namespace {

int tf_fail(int code, const std::string& m) { return cfgpu_record_error(code, m); }

#define TF_CK(x)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess) return tf_fail(CFGPU_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr int CT = 32;  // tile edge of the Chebyshev product

// out[c][j][l] = sum_n M[j][n] in[c][n][l] for j < N, l < nl; blocks: (line tiles, row tiles, components).
__global__ void __launch_bounds__(256) k_cheb_full(int N, int nl, size_t cs, const double* __restrict__ M,
                                                   const double* __restrict__ in, double* __restrict__ out) {
  __shared__ double sM[CT][CT + 1];
  __shared__ double sX[CT][CT + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads, 4 rows each
  const int l = blockIdx.x * CT + tx;
  const int j0 = blockIdx.y * CT;
  const double* src = in + blockIdx.z * cs;
  double* dst = out + blockIdx.z * cs;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int n0 = 0; n0 < N; n0 += CT) {
    for (int r = ty; r < CT; r += 8) {
      const int j = j0 + r, n = n0 + tx;
      sM[r][tx] = (j < N && n < N) ? M[(size_t)j * N + n] : 0.0;
      const int nn = n0 + r;
      sX[r][tx] = (nn < N && l < nl) ? src[(size_t)nn * nl + l] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < CT; ++k) {
      const double x = sX[k][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(sM[ty + 8 * q][k], x, acc[q]);
    }
    __syncthreads();
  }
  if (l < nl)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = j0 + ty + 8 * q;
      if (j < N) dst[(size_t)j * nl + l] = acc[q];
    }
}

// Complex FFT along x of columns [z0, z0 + cols) of plane (ny, i) = (blockIdx.x, blockIdx.y); column chunk
// blockIdx.z.  Spectral plane: complex [mx][mz], Mz columns.  Forward (sign -1) scales by `scale`.
__global__ void __launch_bounds__(256) k_xcols(int Nx, int Mz, int cols, FftPlan px, const cpx<double>* __restrict__ tw,
                                               int sign, double scale, cpx<double>* __restrict__ data, int Ny) {
  extern __shared__ unsigned char smem_raw[];
  const int ss = Nx + 1;
  cpx<double>* a = reinterpret_cast<cpx<double>*>(smem_raw);
  cpx<double>* b = a + (size_t)cols * ss;
  const int z0 = blockIdx.z * cols;
  const int nc = min(cols, Mz - z0);
  cpx<double>* plane = data + ((size_t)blockIdx.y * Ny + blockIdx.x) * (size_t)Nx * Mz;
  for (int i = threadIdx.x; i < nc * Nx; i += blockDim.x) {
    const int x = i / nc, c = i - x * nc;
    a[c * ss + x] = plane[(size_t)x * Mz + z0 + c];
  }
  __syncthreads();
  fft_batch<double>(a, b, nc, ss, px, tw, sign);
  for (int i = threadIdx.x; i < nc * Nx; i += blockDim.x) {
    const int x = i / nc, c = i - x * nc;
    plane[(size_t)x * Mz + z0 + c] = cscale(a[c * ss + x], scale);
  }
}

// z transform of rows [x0, x0 + rows) of plane (ny, i) = (blockIdx.y, blockIdx.z), row chunk blockIdx.x.
// c2r (inverse): row = Mz complex in, Nz reals out (first Nz of its Nzpad slots); r2c: the reverse.
__global__ void __launch_bounds__(256) k_zrows(int Nx, int Nz, int rows, FftPlan pz, const cpx<double>* __restrict__ tw,
                                               int inverse, double* __restrict__ data, int Ny) {
  extern __shared__ unsigned char smem_raw[];
  const int Mz = Nz / 2 + 1, Nzpad = 2 * Mz, ss = Nz + 1;
  cpx<double>* a = reinterpret_cast<cpx<double>*>(smem_raw);
  cpx<double>* b = a + (size_t)rows * ss;
  const int x0 = blockIdx.x * rows;
  const int nr = min(rows, Nx - x0);
  double* plane = data + ((size_t)blockIdx.z * Ny + blockIdx.y) * (size_t)Nx * Nzpad;
  if (inverse) {
    for (int i = threadIdx.x; i < nr * Nz; i += blockDim.x) {
      const int r = i / Nz, k = i - r * Nz;
      const double* row = plane + (size_t)(x0 + r) * Nzpad;
      cpx<double> v;
      if (k < Mz) {
        v = cmk<double>(row[2 * k], row[2 * k + 1]);
        if (k == 0 || 2 * k == Nz) v.y = 0.0;  // c2r uses only the real parts of these terms
      } else {
        v = cmk<double>(row[2 * (Nz - k)], -row[2 * (Nz - k) + 1]);  // Hermitian completion
      }
      a[r * ss + k] = v;
    }
  } else {
    for (int i = threadIdx.x; i < nr * Nz; i += blockDim.x) {
      const int r = i / Nz, z = i - r * Nz;
      a[r * ss + z] = cmk<double>(plane[(size_t)(x0 + r) * Nzpad + z], 0.0);
    }
  }
  __syncthreads();
  fft_batch<double>(a, b, nr, ss, pz, tw, inverse ? +1 : -1);
  if (inverse) {
    for (int i = threadIdx.x; i < nr * Nzpad; i += blockDim.x) {
      const int r = i / Nzpad, z = i - r * Nzpad;
      plane[(size_t)(x0 + r) * Nzpad + z] = z < Nz ? a[r * ss + z].x : 0.0;
    }
  } else {
    for (int i = threadIdx.x; i < nr * Mz; i += blockDim.x) {
      const int r = i / Mz, k = i - r * Mz;
      double* row = plane + (size_t)(x0 + r) * Nzpad;
      row[2 * k] = a[r * ss + k].x;
      row[2 * k + 1] = a[r * ss + k].y;
    }
  }
}

long double cospi_frac(long long m, long long d) {  // cos(pi m / d), argument reduced over the integers
  long long r = m % (2 * d);
  if (r < 0) r += 2 * d;
  return cosl(3.14159265358979323846264338327950288L * (long double)r / (long double)d);
}

}  // namespace

struct cfgpu_flowfield_s {
  int Nx = 0, Ny = 0, Nz = 0, Nd = 0;
  double Lx = 0, Lz = 0, a = -1, b = 1;
  int xzstate = CFGPU_SPECTRAL, ystate = CFGPU_SPECTRAL;
  size_t n = 0;  // doubles
  double* data = nullptr;
  double* work = nullptr;
  double* Mfwd = nullptr;  // [n][j] chebyfft
  double* Minv = nullptr;  // [j][n] ichebyfft
  cpx<double>* twx = nullptr;
  cpx<double>* twz = nullptr;
  FftPlan px{}, pz{};
  cudaStream_t st = nullptr;
};

namespace {

template <typename T>
int tf_upload(const std::vector<T>& h, T** d, cudaStream_t st) {
  TF_CK(cudaMalloc((void**)d, h.size() * sizeof(T)));
  TF_CK(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return CFGPU_OK;
}

int y_transform(cfgpu_flowfield f, bool to_spectral) {
  if (f->Ny < 2) return CFGPU_OK;
  const int nl = f->Nx * 2 * (f->Nz / 2 + 1);
  const size_t cs = (size_t)f->Ny * nl;
  dim3 grid((nl + CT - 1) / CT, (f->Ny + CT - 1) / CT, f->Nd);
  k_cheb_full<<<grid, 256, 0, f->st>>>(f->Ny, nl, cs, to_spectral ? f->Mfwd : f->Minv, f->data, f->work);
  TF_CK(cudaGetLastError());
  TF_CK(cudaMemcpyAsync(f->data, f->work, f->n * sizeof(double), cudaMemcpyDeviceToDevice, f->st));
  return CFGPU_OK;
}

int xz_transform(cfgpu_flowfield f, bool to_spectral) {
  const int Mz = f->Nz / 2 + 1;
  const size_t xc = 2 * sizeof(cpx<double>) * (size_t)(f->Nx + 1);  // per column
  const size_t zr = 2 * sizeof(cpx<double>) * (size_t)(f->Nz + 1);  // per row
  int cols = (int)((96 * 1024) / xc), rows = (int)((96 * 1024) / zr);
  if (cols < 1 || rows < 1) return tf_fail(CFGPU_ENOTSUP, "Nx or Nz too large for the shared-memory FFT");
  cols = cols > Mz ? Mz : (cols > 16 ? 16 : cols);
  rows = rows > f->Nx ? f->Nx : (rows > 16 ? 16 : rows);
  static const bool attr = [] {
    cudaFuncSetAttribute(k_xcols, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_zrows, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return true;
  }();
  (void)attr;
  const dim3 gx(f->Ny, f->Nd, (Mz + cols - 1) / cols), gz((f->Nx + rows - 1) / rows, f->Ny, f->Nd);
  cpx<double>* cd = reinterpret_cast<cpx<double>*>(f->data);
  if (to_spectral) {
    k_zrows<<<gz, 256, rows * zr, f->st>>>(f->Nx, f->Nz, rows, f->pz, f->twz, 0, f->data, f->Ny);
    TF_CK(cudaGetLastError());
    k_xcols<<<gx, 256, cols * xc, f->st>>>(f->Nx, Mz, cols, f->px, f->twx, -1, 1.0 / ((double)f->Nx * f->Nz), cd,
                                           f->Ny);
    TF_CK(cudaGetLastError());
  } else {
    k_xcols<<<gx, 256, cols * xc, f->st>>>(f->Nx, Mz, cols, f->px, f->twx, +1, 1.0, cd, f->Ny);
    TF_CK(cudaGetLastError());
    k_zrows<<<gz, 256, rows * zr, f->st>>>(f->Nx, f->Nz, rows, f->pz, f->twz, 1, f->data, f->Ny);
    TF_CK(cudaGetLastError());
  }
  return CFGPU_OK;
}

int finish(cfgpu_flowfield f, int st) {
  if (st != CFGPU_OK) {
    (void)cudaStreamSynchronize(f->st);
    return st;
  }
  TF_CK(cudaStreamSynchronize(f->st));
  return CFGPU_OK;
}

}  // namespace

extern "C" {

cfgpu_status cfgpu_flowfield_create(const cfgpu_grid* g, int Nd, cfgpu_flowfield* out) {
  if (!g || !out || Nd < 1 || g->Nx < 2 || g->Nz < 2 || g->Ny < 2 || g->Nx % 2 || g->Nz % 2 || !(g->b > g->a) ||
      g->Lx <= 0 || g->Lz <= 0)
    return tf_fail(CFGPU_EINVAL, "bad argument");
  *out = nullptr;
  auto* f = new cfgpu_flowfield_s();
  f->Nx = g->Nx;
  f->Ny = g->Ny;
  f->Nz = g->Nz;
  f->Nd = Nd;
  f->Lx = g->Lx;
  f->Lz = g->Lz;
  f->a = g->a;
  f->b = g->b;
  f->n = (size_t)Nd * g->Ny * g->Nx * 2 * (g->Nz / 2 + 1);
  std::vector<std::complex<long double>> twx, twz;
  int st = CFGPU_OK;
  if (!cfgpu_fft_plan(g->Nx, f->px, twx) || !cfgpu_fft_plan(g->Nz, f->pz, twz))
    st = tf_fail(CFGPU_ENOTSUP, "Nx and Nz must factor into primes <= " + std::to_string(FFT_MAX_RADIX));
  if (st == CFGPU_OK && cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking) != cudaSuccess)
    st = tf_fail(CFGPU_ECUDA, "cudaStreamCreate failed");
  if (st == CFGPU_OK) {
    cudaError_t e = cudaMalloc((void**)&f->data, f->n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&f->work, f->n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(f->data, 0, f->n * sizeof(double), f->st);
    if (e != cudaSuccess) st = tf_fail(CFGPU_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  if (st == CFGPU_OK) {
    const int N = g->Ny;
    std::vector<double> Mf((size_t)N * N), Mi((size_t)N * N);
    for (int n = 0; n < N; ++n)
      for (int j = 0; j < N; ++j) {
        const long double cn = (n == 0 || n == N - 1) ? 0.5L : 1.0L;
        const long double w = (j == 0 || j == N - 1) ? 1.0L : 2.0L;
        Mf[(size_t)n * N + j] = (double)(w * cn * cospi_frac((long long)n * j, N - 1) / (N - 1));
        Mi[(size_t)j * N + n] = (double)cospi_frac((long long)n * j, N - 1);
      }
    std::vector<cpx<double>> tx(twx.size() ? twx.size() : 1), tz(twz.size() ? twz.size() : 1);
    for (size_t i = 0; i < twx.size(); ++i) tx[i] = cmk<double>((double)twx[i].real(), (double)twx[i].imag());
    for (size_t i = 0; i < twz.size(); ++i) tz[i] = cmk<double>((double)twz[i].real(), (double)twz[i].imag());
    st = tf_upload(Mf, &f->Mfwd, f->st);
    if (st == CFGPU_OK) st = tf_upload(Mi, &f->Minv, f->st);
    if (st == CFGPU_OK) st = tf_upload(tx, &f->twx, f->st);
    if (st == CFGPU_OK) st = tf_upload(tz, &f->twz, f->st);
    // the host vectors go out of scope: wait for the copies
    if (st == CFGPU_OK && cudaStreamSynchronize(f->st) != cudaSuccess) st = tf_fail(CFGPU_ECUDA, "stream sync");
  }
  if (st != CFGPU_OK) {
    cfgpu_flowfield_destroy(f);
    return st;
  }
  *out = f;
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_destroy(cfgpu_flowfield f) {
  if (!f) return CFGPU_OK;
  if (f->st) cudaStreamSynchronize(f->st);
  cudaFree(f->data);
  cudaFree(f->work);
  cudaFree(f->Mfwd);
  cudaFree(f->Minv);
  cudaFree(f->twx);
  cudaFree(f->twz);
  if (f->st) cudaStreamDestroy(f->st);
  delete f;
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_size(cfgpu_flowfield f, long long* ndoubles) {
  if (!f || !ndoubles) return tf_fail(CFGPU_EINVAL, "bad argument");
  *ndoubles = (long long)f->n;
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_data(cfgpu_flowfield f, double** device_ptr) {
  if (!f || !device_ptr) return tf_fail(CFGPU_EINVAL, "bad argument");
  *device_ptr = f->data;
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_upload(cfgpu_flowfield f, const double* host, int xzstate, int ystate) {
  if (!f || !host || (xzstate != CFGPU_SPECTRAL && xzstate != CFGPU_PHYSICAL) ||
      (ystate != CFGPU_SPECTRAL && ystate != CFGPU_PHYSICAL))
    return tf_fail(CFGPU_EINVAL, "bad argument");
  TF_CK(cudaMemcpyAsync(f->data, host, f->n * sizeof(double), cudaMemcpyHostToDevice, f->st));
  TF_CK(cudaStreamSynchronize(f->st));
  f->xzstate = xzstate;
  f->ystate = ystate;
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_download(cfgpu_flowfield f, double* host) {
  if (!f || !host) return tf_fail(CFGPU_EINVAL, "bad argument");
  TF_CK(cudaMemcpyAsync(host, f->data, f->n * sizeof(double), cudaMemcpyDeviceToHost, f->st));
  TF_CK(cudaStreamSynchronize(f->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_state(cfgpu_flowfield f, int* xzstate, int* ystate) {
  if (!f || !xzstate || !ystate) return tf_fail(CFGPU_EINVAL, "bad argument");
  *xzstate = f->xzstate;
  *ystate = f->ystate;
  return CFGPU_OK;
}

cfgpu_status cfgpu_flowfield_make_spectral_xz(cfgpu_flowfield f) {
  if (!f) return tf_fail(CFGPU_EINVAL, "bad argument");
  if (f->xzstate == CFGPU_SPECTRAL) return CFGPU_OK;
  const int st = finish(f, xz_transform(f, true));
  if (st == CFGPU_OK) f->xzstate = CFGPU_SPECTRAL;
  return st;
}

cfgpu_status cfgpu_flowfield_make_physical_xz(cfgpu_flowfield f) {
  if (!f) return tf_fail(CFGPU_EINVAL, "bad argument");
  if (f->xzstate == CFGPU_PHYSICAL) return CFGPU_OK;
  const int st = finish(f, xz_transform(f, false));
  if (st == CFGPU_OK) f->xzstate = CFGPU_PHYSICAL;
  return st;
}

cfgpu_status cfgpu_flowfield_make_spectral_y(cfgpu_flowfield f) {
  if (!f) return tf_fail(CFGPU_EINVAL, "bad argument");
  if (f->ystate == CFGPU_SPECTRAL) return CFGPU_OK;
  const int st = finish(f, y_transform(f, true));
  if (st == CFGPU_OK) f->ystate = CFGPU_SPECTRAL;
  return st;
}

cfgpu_status cfgpu_flowfield_make_physical_y(cfgpu_flowfield f) {
  if (!f) return tf_fail(CFGPU_EINVAL, "bad argument");
  if (f->ystate == CFGPU_PHYSICAL) return CFGPU_OK;
  const int st = finish(f, y_transform(f, false));
  if (st == CFGPU_OK) f->ystate = CFGPU_PHYSICAL;
  return st;
}

// makeSpectral: xz first, then y; makePhysical: y first, then xz (flowfield.cpp:1989-1997).
cfgpu_status cfgpu_flowfield_make_spectral(cfgpu_flowfield f) {
  cfgpu_status s = cfgpu_flowfield_make_spectral_xz(f);
  return s == CFGPU_OK ? cfgpu_flowfield_make_spectral_y(f) : s;
}

cfgpu_status cfgpu_flowfield_make_physical(cfgpu_flowfield f) {
  cfgpu_status s = cfgpu_flowfield_make_physical_y(f);
  return s == CFGPU_OK ? cfgpu_flowfield_make_physical_xz(f) : s;
}

}  // extern "C"
