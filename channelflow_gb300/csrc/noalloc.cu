// Allocation-free variant of the batched tau solve.
//
// cfgpu_tau_solve_batched() obtains its device working memory (per-mode
// tables, re-laid-out inputs and outputs, scratch lines) with cudaMalloc on
// every call.  Some callers cannot do that: a process whose GPU memory is
// already fully reserved by another allocator (a framework's caching pool or
// a fixed budget on a shared GPU), where a raw cudaMalloc would fail or
// break the budget, or a latency-sensitive loop that must not pay for
// allocation and synchronising frees.  cfgpu_tau_solve_batched_noalloc()
// gives them the same solve with all device working memory taken from the
// file-scope array below, which is part of this file's device module.  The
// module, and with it the array's CFGPU_NOALLOC_BYTES, is reserved on a
// device when the module is loaded there: with the CUDA runtime's default
// lazy module loading that is the first call of this entry point on the
// device (the symbol lookup below); with CUDA_MODULE_LOADING=EAGER it is the
// creation of the context.  From then on the device holds the array until
// the process exits.  A caller whose GPU memory will be taken over by another
// allocator therefore makes one (small) call before that allocator reserves
// the memory.
//
// The kernels are the ones cfgpu_tau_solve_batched() launches (k_tau_setup,
// k_tau_solve); only where their memory comes from differs.
#include "../../include/cfgpu.h"
#include "kernels.h"

#include <atomic>
#include <string>

namespace {

// 16 MiB of device working memory shared by every call on a device.
constexpr size_t kNoallocDoubles = (size_t)CFGPU_NOALLOC_BYTES / sizeof(double);
static __device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

constexpr int kMaxDevices = 64;
// Device address of g_noalloc_scratch, per device.  Several host threads may look it up at once; they all
// store the same value, and the atomics make that well defined.
std::atomic<double*> g_scratch_ptr[kMaxDevices] = {};

// Device words a call with these sizes needs (must match the carving below).
size_t noalloc_words(int N, int nmodes) {
  const size_t cl = 2 * (size_t)N * nmodes;  // one complex component line set
  const size_t FN = (size_t)N * nmodes;
  return 7 * cl                               // raw inputs (3) and raw outputs (4)
         + 3 * cl + 3 * cl + cl               // R3, U3, Q1 in the solve layout
         + 6 * cl                             // solve scratch lines
         + (size_t)TF_NFIELDS * FN            // per-mode tables
         + (size_t)TS_NSCALARS * nmodes       // per-mode scalars
         + 4 * (size_t)N                      // B rows (lo, di, up) and a zero profile
         + (size_t)nmodes;                    // kx, kz (two ints per word)
}

// Helmholtz right-hand-side rows Be/Bo packed by n (helmholtz.cpp:35-70), built on the device.
__global__ void k_helm_b_rows(int N, double* lo, double* di, double* up, double* zero) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int N_ = N - 1;
  auto beta = [&](int k) { return (k > N_ - 2) ? 0 : 1; };
  auto c = [&](int k) { return (k == 0 || k == N_) ? 2 : 1; };
  double l = 0.0, d = 0.0, u = 0.0;
  if (n >= 2) {
    const int nn = n * n;
    l = ((double)c(n - 2)) / (4 * n * (n - 1));
    d = -((double)beta(n)) / (2 * (nn - 1));
    if (beta(n + 2)) u = 1.0 / (4 * n * (n + 1));
  } else {
    d = 1.0;
  }
  lo[n] = l;
  di[n] = d;
  up[n] = u;
  zero[n] = 0.0;
}

// [k][n] complex (caller layout) <-> [c][n][2*nmodes] (solve layout); c = blockIdx.y
__global__ void k_gather(int N, int nmodes, const double* __restrict__ raw, double* __restrict__ lay) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t per = 2 * (size_t)N * nmodes;
  if (i >= per) return;
  const int c = blockIdx.y;
  const int part = (int)(i & 1);
  const size_t kn = i >> 1;
  const int k = (int)(kn / N), n = (int)(kn % N);
  lay[c * per + (size_t)n * 2 * nmodes + 2 * k + part] = raw[c * per + i];
}

__global__ void k_scatter(int N, int nmodes, const double* __restrict__ lay, double* __restrict__ raw) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t per = 2 * (size_t)N * nmodes;
  if (i >= per) return;
  const int c = blockIdx.y;
  const int part = (int)(i & 1);
  const size_t kn = i >> 1;
  const int k = (int)(kn / N), n = (int)(kn % N);
  raw[c * per + i] = lay[c * per + (size_t)n * 2 * nmodes + 2 * k + part];
}

int na_fail(int code, const std::string& m) { return cfgpu_record_error(code, m); }

}  // namespace

extern "C" cfgpu_status cfgpu_tau_solve_batched_noalloc(int N, int nmodes, const int* kx, const int* kz, double Lx,
                                                        double Lz, double a, double b, double lambda_t, double nu,
                                                        int taucorrection, const double* Rx, const double* Ry,
                                                        const double* Rz, double* u, double* v, double* w,
                                                        double* P) {
  if (N < 5 || N % 2 == 0 || nmodes <= 0 || !kx || !kz || !Rx || !Ry || !Rz || !u || !v || !w || !P)
    return na_fail(CFGPU_EINVAL, "bad argument");
  if (!(b > a) || Lx <= 0 || Lz <= 0) return na_fail(CFGPU_EINVAL, "bad geometry");
  if ((N + 1) / 2 > 1024) return na_fail(CFGPU_EINVAL, "N too large");
  if (noalloc_words(N, nmodes) > kNoallocDoubles)
    return na_fail(CFGPU_EINVAL, "N * nmodes too large for the static working array (" +
                                     std::to_string(noalloc_words(N, nmodes) * sizeof(double)) + " bytes needed, " +
                                     std::to_string((size_t)CFGPU_NOALLOC_BYTES) + " available)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(CFGPU_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return na_fail(CFGPU_ENOTSUP, "device ordinal beyond the supported range");
  double* base = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!base) {
    // First call on this device (current device): look up where the static array lives.  Under lazy module
    // loading this loads the module and so reserves the array; that can fail when the device's memory is
    // already taken.
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e == cudaErrorMemoryAllocation)
      return na_fail(CFGPU_ENOMEM, "the static working array (" + std::to_string((size_t)CFGPU_NOALLOC_BYTES) +
                                       " bytes) could not be reserved on this device: make the first call before "
                                       "another allocator takes the GPU's memory, or load modules eagerly "
                                       "(CUDA_MODULE_LOADING=EAGER)");
    if (e != cudaSuccess || !p)
      return na_fail(CFGPU_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    base = static_cast<double*>(p);
    g_scratch_ptr[dev].store(base, std::memory_order_release);
  }
  const size_t cl = 2 * (size_t)N * nmodes, FN = (size_t)N * nmodes;
  double* raw_in = base;             // 3 cl
  double* raw_out = raw_in + 3 * cl;  // 4 cl
  double* R3 = raw_out + 4 * cl;
  double* U3 = R3 + 3 * cl;
  double* Q1 = U3 + 3 * cl;
  double* scr = Q1 + cl;              // 6 cl
  TauTable t{};
  t.f = scr + 6 * cl;
  t.s = t.f + (size_t)TF_NFIELDS * FN;
  double* hlo = t.s + (size_t)TS_NSCALARS * nmodes;
  double* hdi = hlo + N;
  double* hup = hdi + N;
  double* zero = hup + N;
  int* dkx = reinterpret_cast<int*>(zero + N);
  int* dkz = dkx + nmodes;
  cudaStream_t st = 0;
  const size_t cb = cl * sizeof(double);
  // On an error after the first enqueue, wait for the work already queued (its copies into the caller's
  // buffers and its use of the shared array) before returning, so that nothing of this call runs on after it.
#define NA_CK(x)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (x);                                                                            \
    if (e_ != cudaSuccess) {                                                                         \
      (void)cudaStreamSynchronize(st);                                                               \
      return na_fail(CFGPU_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_));                  \
    }                                                                                                \
  } while (0)
  NA_CK(cudaMemcpyAsync(dkx, kx, nmodes * sizeof(int), cudaMemcpyHostToDevice, st));
  NA_CK(cudaMemcpyAsync(dkz, kz, nmodes * sizeof(int), cudaMemcpyHostToDevice, st));
  NA_CK(cudaMemcpyAsync(raw_in, Rx, cb, cudaMemcpyHostToDevice, st));
  NA_CK(cudaMemcpyAsync(raw_in + cl, Ry, cb, cudaMemcpyHostToDevice, st));
  NA_CK(cudaMemcpyAsync(raw_in + 2 * cl, Rz, cb, cudaMemcpyHostToDevice, st));
  k_helm_b_rows<<<(N + 127) / 128, 128, 0, st>>>(N, hlo, hdi, hup, zero);
  NA_CK(cudaGetLastError());
  k_gather<<<dim3((unsigned)((cl + 255) / 256), 3), 256, 0, st>>>(N, nmodes, raw_in, R3);
  NA_CK(cudaGetLastError());
  GridDev g{};
  g.Nx = g.Nz = 4;
  g.Ny = N;
  g.Md = nmodes;
  g.NKx = nmodes;
  g.NKz = 1;
  g.kxmax = g.kzmax = 1 << 30;
  g.Lx = Lx;
  g.Lz = Lz;
  g.a = a;
  g.b = b;
  g.kxs = dkx;
  g.kzs = dkz;
  HelmB hb{hlo, hdi, hup};
  NA_CK(launch_tau_setup(g, N, lambda_t, nu, hb, t, scr, st));
  SolveParams sp{};
  sp.kind = 0;
  sp.order = 1;
  sp.a[0] = 1.0;
  sp.b[0] = 0.0;
  sp.nu = nu;
  sp.constraint = CFGPU_PressureGradient;
  sp.taucorrection = taucorrection;
  sp.force_real00 = 0;
  SolvePtrs p{};
  p.uin[0] = R3;
  p.nin[0] = R3;
  p.uout = U3;
  p.qout = Q1;
  p.Ubaseyy = zero;
  p.Wbaseyy = zero;
  p.scratch = scr;
  NA_CK(launch_tau_solve<double>(g, N, sp, p, hb, t, st));
  k_scatter<<<dim3((unsigned)((cl + 255) / 256), 3), 256, 0, st>>>(N, nmodes, U3, raw_out);
  NA_CK(cudaGetLastError());
  k_scatter<<<dim3((unsigned)((cl + 255) / 256), 1), 256, 0, st>>>(N, nmodes, Q1, raw_out + 3 * cl);
  NA_CK(cudaGetLastError());
  NA_CK(cudaMemcpyAsync(u, raw_out, cb, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(v, raw_out + cl, cb, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(w, raw_out + 2 * cl, cb, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(P, raw_out + 3 * cl, cb, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
#undef NA_CK
  return CFGPU_OK;
}
