// Host runtime of the GB300 DNS step and the C ABI declared in include/cfgpu.h.
//
// A cfgpu_dns owns, on one CUDA device and stream:
//   * the multistep history ring (u, q and the nonlinear term N per slot),
//     or the CNAB / CNRK2 state, in the solved-mode layout of common.cuh;
//   * the per-substep tau tables of the main and of the initialisation
//     scheme (TauSolver constructor work, done once by k_tau_setup);
//   * FFT plans/twiddles and the Chebyshev transform matrices;
//   * work arrays of the nonlinear-term pipeline.
// Scheme logic follows channelflow/dnsalgo.cpp (MultistepDNS, CNABstyleDNS,
// RungeKuttaDNS) and the DNS facade channelflow/dns.cpp:22-163.
#include <climits>
#include <cmath>
#include <atomic>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cfgpu.h"
#include "kernels.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(x)                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) return fail(CFGPU_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CKS(x)                 \
  do {                         \
    int s_ = (x);              \
    if (s_ != CFGPU_OK) return s_; \
  } while (0)

// ---------------------------------------------------------------------------
// Host-side Chebyshev helpers (chebyshev.cpp) for base flows and constraints
// ---------------------------------------------------------------------------
std::vector<double> cheb_diff_h(const std::vector<double>& u, double L) {
  const int N = (int)u.size();
  std::vector<double> d(N, 0.0);
  if (N < 2) return d;
  const int Nb = N - 1;
  const double scale = 4.0 / L;
  d[Nb] = 0.0;
  d[Nb - 1] = scale * Nb * u[Nb];
  for (int n = Nb - 2; n >= 0; --n) d[n] = d[n + 2] + scale * (n + 1) * u[n + 1];
  d[0] *= 0.5;
  return d;
}
double eval_b_h(const std::vector<double>& u) {
  double s = 0.0;
  for (int n = (int)u.size() - 1; n >= 0; --n) s += u[n];
  return s;
}
double eval_a_h(const std::vector<double>& u) {
  double s = 0.0;
  for (int n = (int)u.size() - 1; n >= 0; --n) s += u[n] * ((n % 2 == 0) ? 1 : -1);
  return s;
}
double mean_h(const std::vector<double>& u) {
  double s = u[0];
  for (size_t n = 2; n < u.size(); n += 2) s -= u[n] / (double)(n * n - 1);
  return s;
}
// cos(pi m / d) with the argument reduced exactly first
long double cospi_ratio(long long m, long long d) {
  long long r = m % (2 * d);
  if (r < 0) r += 2 * d;
  return cosl(3.14159265358979323846264338327950288L * (long double)r / (long double)d);
}
// Values at Gauss-Lobatto points -> Chebyshev coefficients (chebyfft, chebyshev.cpp:262-284), direct sum.
std::vector<double> chebyfft_h(const std::vector<double>& x) {
  const int N = (int)x.size();
  std::vector<double> a(N);
  for (int n = 0; n < N; ++n) {
    long double Y = (long double)x[0] + ((n % 2 == 0) ? 1.0L : -1.0L) * x[N - 1];
    for (int j = 1; j < N - 1; ++j) Y += 2.0L * x[j] * cospi_ratio((long long)n * j, N - 1);
    long double c = Y / (N - 1);
    if (n == 0 || n == N - 1) c *= 0.5L;
    a[n] = (double)c;
  }
  return a;
}

// laminarProfile (channelflow/nse.cpp:823-943)
std::vector<double> laminar_profile(double nu, int constraint, double dPdx, double Ubulk, double Vsuck, double a,
                                    double b, double ua, double ub, int Ny) {
  std::vector<double> u(Ny, 0.0);
  const double H = b - a;
  double mu = Vsuck * H / nu;
  if (std::fabs(mu) == 0.0) {
    if (constraint == CFGPU_BulkVelocity) {
      u[0] = 0.125 * (ub + ua) + 0.75 * Ubulk;
      u[1] = 0.5 * (ub - ua);
      u[2] = 0.375 * (ub + ua) - 0.75 * Ubulk;
    } else {
      dPdx *= ((b - a) / 2) * ((b - a) / 2);
      u[0] = 0.5 * (ub + ua) - 0.25 * dPdx / nu;
      u[1] = 0.5 * (ub - ua);
      u[2] = 0.25 * dPdx / nu;
    }
    return u;
  }
  mu = H * Vsuck / nu;
  const double ub_ua = ub - ua;
  const double expm1_mu = std::expm1(-mu);
  double dPdx_HH_nu = dPdx * H * H / nu;
  std::vector<double> phys(Ny);
  const double piN = M_PI / (Ny - 1), radius = (b - a) / 2, center = (b + a) / 2;
  if (std::fabs(mu) > 1e-01) {
    if (constraint == CFGPU_BulkVelocity) {
      const double k = -1.0 / expm1_mu - 1 / mu;
      dPdx_HH_nu = mu * (Ubulk - ua - ub_ua * k) / (0.5 - k);
    }
    for (int i = 0; i < Ny; ++i) {
      const double y = center + radius * std::cos(i * piN);
      const double yhat = (y - a) / H;
      const double e = std::expm1(-mu * yhat);
      phys[i] = ua + ub_ua * e / expm1_mu + dPdx_HH_nu * (yhat - e / expm1_mu) / mu;
    }
  } else {
    if (constraint == CFGPU_BulkVelocity) {
      const double mu2 = mu * mu, A = ub - ua, B = ua + ub - 2 * Ubulk;
      dPdx_HH_nu = 6 * B + mu * (A + mu * (B / 10 + mu2 * (-B / 1400 + mu2 * B / 126000)));
    }
    const double one_2 = 1.0 / 2, one_12 = 1.0 / 12, one_24 = 1.0 / 24, one_720 = 1.0 / 720, one_1440 = 1.0 / 1440,
                 one_30240 = 1.0 / 30240, one_120960 = 1.0 / 120960;
    for (int i = 0; i < Ny; ++i) {
      const double y = center + radius * std::cos(i * piN);
      const double yh = (y - a) / H, yh2 = yh * yh, yh3 = yh2 * yh, yh4 = yh3 * yh, yh_1 = yh - 1;
      const double sq = (yh * yh_1) * (yh * yh_1);
      const double t1 =
          yh + mu * (-one_2 * yh * yh_1 +
                     mu * (one_12 * yh * yh_1 * (2 * yh - 1) +
                           mu * (-one_24 * sq + mu * (one_720 * yh * yh_1 * (2 * yh - 1) * (3 * yh2 - 3 * yh - 1) +
                                                      mu * (-one_1440 * sq * (2 * yh2 - 2 * yh - 1) +
                                                            mu * (one_30240 * yh * yh_1 * (2 * yh - 1) *
                                                                  (3 * yh4 - 6 * yh3 + 3 * yh + 1)))))));
      const double t2 =
          one_2 * yh * yh_1 +
          mu * (-one_12 * yh * yh_1 * (2 * yh - 1) +
                mu * (one_24 * sq +
                      mu * (-one_720 * yh * yh_1 * (2 * yh - 1) * (3 * yh2 - 3 * yh - 1) +
                            mu * (one_1440 * sq * (2 * yh2 - 2 * yh - 1) +
                                  mu * (-one_30240 * yh * yh_1 * (2 * yh - 1) * (3 * yh4 - 6 * yh3 + 3 * yh + 1) +
                                        mu * (one_120960 * sq * (3 * yh4 - 6 * yh3 + 4 * yh + 2)))))));
      phys[i] = ua + ub_ua * t1 + dPdx_HH_nu * t2;
    }
  }
  return chebyfft_h(phys);
}

// ---------------------------------------------------------------------------
// FFT plans and Chebyshev matrices
// ---------------------------------------------------------------------------
bool make_fft_plan(int L, FftPlan& p, std::vector<std::complex<long double>>& tw) {
  std::vector<int> rs;
  int n = L;
  while (n % 4 == 0) { rs.push_back(4); n /= 4; }
  while (n % 2 == 0) { rs.push_back(2); n /= 2; }
  while (n % 3 == 0) { rs.push_back(3); n /= 3; }
  while (n % 5 == 0) { rs.push_back(5); n /= 5; }
  // any other prime factor is a direct-DFT stage (FFTW takes every length; such grids are rare, so these
  // stages favour generality over speed)
  for (int f = 7; n > 1 && f <= FFT_MAX_RADIX; f += 2)
    while (n % f == 0) { rs.push_back(f); n /= f; }
  if (n != 1 || rs.empty() || (int)rs.size() > FFT_MAX_STAGES) return false;
  memset(&p, 0, sizeof(p));
  p.L = L;
  p.nst = (int)rs.size();
  int Ns = 1, off = 0;
  tw.clear();
  const long double PI_L = 3.14159265358979323846264338327950288L;
  for (int s = 0; s < p.nst; ++s) {
    const int R = rs[s];
    p.radix[s] = R;
    p.Ns[s] = Ns;
    p.twoff[s] = off;
    for (int k = 0; k < Ns; ++k)
      for (int r = 1; r < R; ++r) {
        // exp(-2 pi i r k / (Ns R)), argument reduced over the integer r*k
        const long long num = (long long)r * k, den = (long long)Ns * R;
        const long double ang = -2.0L * PI_L * (long double)(num % den) / (long double)den;
        tw.emplace_back(cosl(ang), sinl(ang));
      }
    off += Ns * (R - 1);
    p.rootoff[s] = -1;
    if (R > 5) {
      // the stage's DFT matrix entries exp(-2 pi i e / R), e = 0 .. R-1
      p.rootoff[s] = off;
      for (int e = 0; e < R; ++e) {
        const long double ang = -2.0L * PI_L * (long double)e / (long double)R;
        tw.emplace_back(e == 0 ? 1.0L : cosl(ang), e == 0 ? 0.0L : sinl(ang));
      }
      off += R;
    }
    Ns *= R;
  }
  p.twlen = off;
  return true;
}

// exp(-2 pi i e / L) for e < L, re/im interleaved; quarter-circle points exact (0, +-1).
std::vector<double> circle_table(int L) {
  std::vector<double> t(2 * (size_t)L);
  const long double PI_L = 3.14159265358979323846264338327950288L;
  auto snap = [](long double v) -> double {
    if (fabsl(v) < 1e-18L) return 0.0;
    if (fabsl(v - 1.0L) < 1e-18L) return 1.0;
    if (fabsl(v + 1.0L) < 1e-18L) return -1.0;
    return (double)v;
  };
  for (int e = 0; e < L; ++e) {
    const long double ang = 2.0L * PI_L * (long double)e / (long double)L;
    t[2 * (size_t)e] = snap(cosl(ang));
    t[2 * (size_t)e + 1] = snap(-sinl(ang));
  }
  return t;
}

struct ChebMats {
  std::vector<double> invA, invB, fwdA, fwdB;  // P x KA, P x KB (row-major)
  std::vector<double> derA, derB;              // (2/L) T'_n at y_j for even / odd n
  std::vector<double> dfA, dfB;                // diff o chebyfft: even coefs from d (P x KB), odd from s (P x KA)
};

long double sinpi_ratio(long long m, long long d) {
  long long r = m % (2 * d);
  if (r < 0) r += 2 * d;
  return sinl(3.14159265358979323846264338327950288L * (long double)r / (long double)d);
}

// T'_n(y_j) at y_j = cos(pi j/(N-1)): n sin(n theta)/sin(theta), n^2 at j = 0
long double cheb_deriv_at(int n, int j, int N) {
  if (j == 0) return (long double)n * n;
  if (2 * j == 2 * (N - 1)) return (n % 2 ? 1.0L : -1.0L) * n * n;
  return n * sinpi_ratio((long long)n * j, N - 1) / sinpi_ratio(j, N - 1);
}

ChebMats make_cheb_mats(int N) {
  ChebMats M;
  const int P = (N + 1) / 2, KA = (N + 1) / 2, KB = (N - 1) / 2, J = (N - 1) / 2;
  M.invA.assign((size_t)P * KA, 0.0);
  M.invB.assign((size_t)P * KB, 0.0);
  M.fwdA.assign((size_t)P * KA, 0.0);
  M.fwdB.assign((size_t)P * KB, 0.0);
  for (int j = 0; j < P; ++j) {
    for (int k = 0; k < KA; ++k) M.invA[j * KA + k] = (double)cospi_ratio(2LL * k * j, N - 1);
    for (int k = 0; k < KB; ++k) M.invB[j * KB + k] = (double)cospi_ratio((2LL * k + 1) * j, N - 1);
  }
  M.derA.assign((size_t)P * KA, 0.0);
  M.derB.assign((size_t)P * KB, 0.0);
  for (int j = 0; j < P; ++j) {
    for (int k = 0; k < KA; ++k) M.derA[j * KA + k] = (double)(cheb_deriv_at(2 * k, j, N));
    for (int k = 0; k < KB; ++k) M.derB[j * KB + k] = (double)(cheb_deriv_at(2 * k + 1, j, N));
  }
  {
    // full forward matrix F[n][j] and coefficient derivative D (diff, chebyshev.cpp:672-697, L = 2 here;
    // the 2/L factor is applied by the caller), DF = D F split by parity
    std::vector<long double> F((size_t)N * N), D((size_t)N * N, 0.0L), DF((size_t)N * N, 0.0L);
    for (int n = 0; n < N; ++n) {
      const long double cn = (n == 0 || n == N - 1) ? 0.5L : 1.0L;
      for (int j = 0; j < N; ++j) {
        const long double w = (j == 0 || j == N - 1) ? 1.0L : 2.0L;
        F[(size_t)n * N + j] = w * cospi_ratio((long long)n * j, N - 1) * cn / (N - 1);
      }
    }
    for (int n = 0; n < N; ++n)
      for (int m2 = n + 1; m2 < N; m2 += 2) D[(size_t)n * N + m2] = (n == 0 ? 1.0L : 2.0L) * m2;
    for (int n = 0; n < N; ++n)
      for (int mm = 0; mm < N; ++mm) {
        const long double dv = D[(size_t)n * N + mm];
        if (dv == 0.0L) continue;
        for (int j = 0; j < N; ++j) DF[(size_t)n * N + j] += dv * F[(size_t)mm * N + j];
      }
    M.dfA.assign((size_t)P * KB, 0.0);
    M.dfB.assign((size_t)P * KA, 0.0);
    for (int k = 0; k < P; ++k) {
      for (int j = 0; j < KB; ++j) M.dfA[k * KB + j] = (double)DF[(size_t)(2 * k) * N + j];
      if (2 * k + 1 < N)
        for (int j = 0; j <= J; ++j) M.dfB[k * KA + j] = (double)DF[(size_t)(2 * k + 1) * N + j];
    }
  }
  for (int k = 0; k < P; ++k) {
    const int n = 2 * k;
    const long double cn = (n == 0 || n == N - 1) ? 0.5L : 1.0L;
    for (int j = 0; j <= J; ++j) {
      const long double w = (j == 0) ? 1.0L : 2.0L;
      M.fwdA[k * KA + j] = (double)(w * cospi_ratio((long long)n * j, N - 1) * cn / (N - 1));
    }
    const int no = 2 * k + 1;
    if (no < N)
      for (int j = 0; j < J; ++j) {
        const long double w = (j == 0) ? 1.0L : 2.0L;
        M.fwdB[k * KB + j] = (double)(w * cospi_ratio((long long)no * j, N - 1) / (N - 1));
      }
  }
  return M;
}

// Be/Bo rows packed by Chebyshev index (helmholtz.cpp:35-70)
void make_helm_b(int N, std::vector<double>& lo, std::vector<double>& di, std::vector<double>& up) {
  const int N_ = N - 1;
  lo.assign(N, 0.0);
  di.assign(N, 0.0);
  up.assign(N, 0.0);
  auto beta = [&](int n) { return (n > N_ - 2) ? 0 : 1; };
  auto c = [&](int n) { return (n == 0 || n == N_) ? 2 : 1; };
  for (int n = 2; n < N; ++n) {
    const int nn = n * n;
    lo[n] = ((double)c(n - 2)) / (4 * n * (n - 1));
    di[n] = -((double)beta(n)) / (2 * (nn - 1));
    if (beta(n + 2)) up[n] = 1.0 / (4 * n * (n + 1));
  }
  di[0] = di[1] = 1.0;
}

template <typename T>
int dalloc(T** p, size_t n, long long& bytes);

// Device memory comes from the device's stream-ordered pool, which keeps freed memory reserved, so that DNS
// objects created and destroyed at serving rates allocate in microseconds.  Allocations and frees are issued
// on one internal stream per device; an allocation is complete when dalloc returns.
cudaStream_t pool_stream() {
  static std::mutex mu;
  static std::map<int, cudaStream_t> streams;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = streams.find(dev);
  if (it != streams.end()) return it->second;
  cudaStream_t st = nullptr;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  streams[dev] = st;
  return st;
}

template <typename T>
int dalloc(T** p, size_t n, long long& bytes) {
  if (n == 0) n = 1;
  cudaStream_t ps = pool_stream();
  cudaError_t e = cudaMallocAsync((void**)p, n * sizeof(T), ps);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ps);
  if (e != cudaSuccess) return fail(CFGPU_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  bytes += (long long)(n * sizeof(T));
  return CFGPU_OK;
}

// Back to the pool; the caller has synchronized every stream that used p.
void dfree(void* p) {
  if (p) cudaFreeAsync(p, pool_stream());
}

// Page-locked host buffers come from a process-wide cache by power-of-two size class: page-locked
// allocation is slow and can serialize the streams of other DNS objects running concurrently, so blocks
// are allocated once and reused.
std::mutex g_pin_mu;
std::map<size_t, std::vector<void*>> g_pin_free;  // size class -> free blocks
std::map<void*, size_t> g_pin_class;

template <typename T>
int pinned_alloc(T** p, size_t bytes) {
  size_t c = 256;
  while (c < bytes) c <<= 1;
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto& v = g_pin_free[c];
    if (!v.empty()) {
      *p = (T*)v.back();
      v.pop_back();
      return CFGPU_OK;
    }
  }
  void* q = nullptr;
  const cudaError_t e = cudaMallocHost(&q, c);
  if (e != cudaSuccess) return fail(CFGPU_ENOMEM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_class[q] = c;
  *p = (T*)q;
  return CFGPU_OK;
}

void pinned_free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free[g_pin_class[p]].push_back(p);
}

}  // namespace

// programmatic dependent launch between the kernels of a step (cfgpu_set_pdl; declared in common.cuh)
static std::atomic<int> g_pdl_on{1};
int pdl_enabled() { return g_pdl_on.load(std::memory_order_relaxed); }

int cfgpu_record_error(int code, const std::string& msg) { return fail(code, msg); }

bool cfgpu_fft_plan(int L, FftPlan& p, std::vector<std::complex<long double>>& tw) { return make_fft_plan(L, p, tw); }

// ---------------------------------------------------------------------------
// The DNS object
// ---------------------------------------------------------------------------
struct Scheme {
  int method = CFGPU_SBDF3;
  int family = 0;  // 0 multistep, 1 CNAB-style, 2 RK
  int order = 0, nsub = 1, ninit = 0;
  double eta = 1;
  double alpha[4] = {0}, beta[4] = {0};          // multistep
  double ca[3] = {0}, cb[3] = {0}, cg[3] = {0}, cz[3] = {0};  // CNAB-style
  double rA[3] = {0}, rB[3] = {0}, rC[3] = {0};  // RK
  std::vector<double> lambda_t;
  int countdown = 0;
  bool full = true;
  double t = 0;
  std::vector<TauTable> tau;
};

static int setup_scheme(Scheme& s, int method, double dt) {
  s.method = method;
  switch (method) {
    case CFGPU_CNFE1:
    case CFGPU_SBDF1:
      s.family = 0; s.order = 1; s.eta = 1.0; s.alpha[0] = -1.0; s.beta[0] = 1.0; break;
    case CFGPU_SBDF2:
      s.family = 0; s.order = 2; s.eta = 1.5; s.alpha[0] = -2.0; s.alpha[1] = 0.5; s.beta[0] = 2.0; s.beta[1] = -1.0;
      break;
    case CFGPU_SBDF3:
      s.family = 0; s.order = 3; s.eta = 11.0 / 6.0;
      s.alpha[0] = -3.0; s.alpha[1] = 1.5; s.alpha[2] = -1.0 / 3.0;
      s.beta[0] = 3.0; s.beta[1] = -3.0; s.beta[2] = 1.0;
      break;
    case CFGPU_SBDF4:
      s.family = 0; s.order = 4; s.eta = 25.0 / 12.0;
      s.alpha[0] = -4.0; s.alpha[1] = 3.0; s.alpha[2] = -4.0 / 3.0; s.alpha[3] = 0.25;
      s.beta[0] = 4.0; s.beta[1] = -6.0; s.beta[2] = 4.0; s.beta[3] = -1.0;
      break;
    case CFGPU_CNAB2:
      s.family = 1; s.order = 2; s.nsub = 1; s.ninit = 1;
      s.ca[0] = 0.5; s.cb[0] = 0.5; s.cg[0] = 1.5; s.cz[0] = -0.5;
      break;
    case CFGPU_SMRK2:
      s.family = 1; s.order = 2; s.nsub = 3; s.ninit = 0;
      s.ca[0] = 29.0 / 96.0; s.ca[1] = -3.0 / 40.0; s.ca[2] = 1.0 / 6.0;
      s.cb[0] = 37.0 / 160.0; s.cb[1] = 5.0 / 24.0; s.cb[2] = 1.0 / 6.0;
      s.cg[0] = 8.0 / 15.0; s.cg[1] = 5.0 / 12.0; s.cg[2] = 3.0 / 4.0;
      s.cz[0] = 0.0; s.cz[1] = -17.0 / 60.0; s.cz[2] = -5.0 / 12.0;
      break;
    case CFGPU_CNRK2:
      s.family = 2; s.order = 2; s.nsub = 3; s.ninit = 0;
      s.rA[0] = 0.0; s.rA[1] = -5.0 / 9.0; s.rA[2] = -153.0 / 128.0;
      s.rB[0] = 1.0 / 3.0; s.rB[1] = 15.0 / 16.0; s.rB[2] = 8.0 / 15.0;
      s.rC[0] = 1.0 / 6.0; s.rC[1] = 5.0 / 24.0; s.rC[2] = 1.0 / 8.0;
      break;
    default:
      return fail(CFGPU_EINVAL, "unknown time-stepping method");
  }
  s.lambda_t.clear();
  if (s.family == 0) {
    s.ninit = s.order - 1;
    s.lambda_t.push_back(s.eta / dt);
    s.countdown = s.ninit;
    s.full = (s.countdown == 0);
  } else if (s.family == 1) {
    for (int j = 0; j < s.nsub; ++j) s.lambda_t.push_back(1.0 / (s.cb[j] * dt));
    s.full = (method == CFGPU_SMRK2);
  } else {
    for (int j = 0; j < s.nsub; ++j) s.lambda_t.push_back(1.0 / (s.rC[j] * dt));
    s.full = true;
  }
  return CFGPU_OK;
}

// Base flow and constraint of one field: NSE::createCFBaseFlow (nse.cpp:589-632) and
// NSE::initCFConstraint (nse.cpp:634-671), plus the base profiles at the Gauss-Lobatto
// points used by the nonlinear kernels (U, U', W, W').
struct BaseFlow {
  std::vector<double> Ubase, Wbase, Ubaseyy, Wbaseyy, basey;
  double UbulkBase = 0, WbulkBase = 0, dPdxRef = 0, dPdzRef = 0, UbulkRef = 0, WbulkRef = 0;
  double dPdxAct = 0, dPdzAct = 0;
  double baseShear[2] = {0, 0};
};

int compute_base(const cfgpu_flags& f, const double* Ub, const double* Wb, int Ny, double a, double b, BaseFlow& B) {
  if (Ub && Wb) {
    B.Ubase.assign(Ub, Ub + Ny);
    B.Wbase.assign(Wb, Wb + Ny);
  } else {
    B.Ubase.assign(Ny, 0.0);
    B.Wbase.assign(Ny, 0.0);
    switch (f.baseflow) {
      case CFGPU_ZeroBase: break;
      case CFGPU_LinearBase: B.Ubase[1] = 1; break;
      case CFGPU_ParabolicBase: B.Ubase[0] = 0.5; B.Ubase[2] = -0.5; break;
      case CFGPU_SuctionBase:
        B.Ubase = laminar_profile(f.nu, CFGPU_PressureGradient, 0, f.Ubulk, f.Vsuck, a, b, -0.5, 0.5, Ny);
        break;
      case CFGPU_LaminarBase:
        B.Ubase = laminar_profile(f.nu, f.constraint, f.dPdx, f.Ubulk, f.Vsuck, a, b, f.ulowerwall, f.uupperwall, Ny);
        B.Wbase = laminar_profile(f.nu, f.constraint, f.dPdz, f.Wbulk, f.Vsuck, a, b, f.wlowerwall, f.wupperwall, Ny);
        break;
      default:
        return fail(CFGPU_EINVAL, "ArbitraryBase requires Ubase and Wbase");
    }
  }
  const double L = b - a;
  B.UbulkBase = mean_h(B.Ubase);
  B.Ubaseyy = cheb_diff_h(cheb_diff_h(B.Ubase, L), L);
  B.WbulkBase = mean_h(B.Wbase);
  B.Wbaseyy = cheb_diff_h(cheb_diff_h(B.Wbase, L), L);
  {
    std::vector<double> Uy = cheb_diff_h(B.Ubase, L), Wy = cheb_diff_h(B.Wbase, L);
    B.baseShear[0] = f.nu * (eval_b_h(Uy) - eval_a_h(Uy)) / L;
    B.baseShear[1] = f.nu * (eval_b_h(Wy) - eval_a_h(Wy)) / L;
  }
  if (f.constraint == CFGPU_BulkVelocity) {
    B.UbulkRef = f.Ubulk;
    B.WbulkRef = f.Wbulk;
  } else {
    B.dPdxAct = B.dPdxRef = f.dPdx;
    B.dPdzAct = B.dPdzRef = f.dPdz;
  }
  B.basey.assign(4 * (size_t)Ny, 0.0);
  for (int j = 0; j < Ny; ++j) {
    long double U = 0, Uy = 0, W = 0, Wy = 0;
    for (int n = 0; n < Ny; ++n) {
      const long double c = cospi_ratio((long long)n * j, Ny - 1);
      const long double dd = cheb_deriv_at(n, j, Ny) * (2.0L / (b - a));
      U += B.Ubase[n] * c;
      Uy += B.Ubase[n] * dd;
      W += B.Wbase[n] * c;
      Wy += B.Wbase[n] * dd;
    }
    B.basey[j] = (double)U;
    B.basey[Ny + j] = (double)Uy;
    B.basey[2 * Ny + j] = (double)W;
    B.basey[3 * Ny + j] = (double)Wy;
  }
  return CFGPU_OK;
}

SlotParams slot_params(const cfgpu_flags& f, const BaseFlow& B) {
  SlotParams p{};
  p.nu = f.nu;
  p.constraint = f.constraint;
  p.dPdxRef = B.dPdxRef;
  p.dPdzRef = B.dPdzRef;
  p.umean = B.UbulkRef - B.UbulkBase;
  p.wmean = B.WbulkRef - B.WbulkBase;
  p.baseShear[0] = B.baseShear[0];
  p.baseShear[1] = B.baseShear[1];
  // scheme coefficients at this field's dt, computed as a single-field DNS computes them
  Scheme m{}, i{};
  if (setup_scheme(m, f.timestepping, f.dt) == CFGPU_OK) {
    if (m.family == 0)
      for (int j = 0; j < m.order; ++j) p.a[j] = -m.alpha[j] / f.dt;
    else
      for (int j = 0; j < m.nsub && j < 3; ++j) p.lam[0][j] = m.lambda_t[j];
  }
  if (f.initstepping != f.timestepping && setup_scheme(i, f.initstepping, f.dt) == CFGPU_OK && i.family != 0)
    for (int j = 0; j < i.nsub && j < 3; ++j) p.lam[1][j] = i.lambda_t[j];
  return p;
}

// lambda_t of substep j of scheme `method` at dt (the tau tables of a field with that dt).
double lambda_at(int method, double dt, int j) {
  Scheme s{};
  if (setup_scheme(s, method, dt) != CFGPU_OK || j >= (int)s.lambda_t.size()) return 0.0;
  return s.lambda_t[j];
}

struct cfgpu_dns_s {
  int device = 0;
  cudaStream_t st = nullptr;
  GridDev g{};   // one field
  // A batch of nb fields of the same grid and flags is stored interleaved,
  // component arrays [c][ny][field][m]: the per-mode kernels see nb*Md modes
  // (gm, explicit mode lists, Mf = Md) and the per-plane x/z kernels see nb*Ny
  // planes (gp).  nb = 1: gm = gp = g.
  int nb = 1;
  GridDev gm{}, gp{};
  int* dmodes = nullptr;  // kx then kz lists of gm
  // Heterogeneous batch: per-field nu, base flow and constraint (set by cfgpu_ensemble_set_params).
  bool hetero = false;
  std::vector<cfgpu_flags> sfl;      // per-field flags
  SlotParams* dslot = nullptr;       // [nb]
  double* dbaseS = nullptr;          // [4][nb][N]: Ubase, Wbase, Ubaseyy, Wbaseyy
  void* baseyS = nullptr;            // R-typed [nb][4N]
  int N = 0;  // Ny
  int precision = CFGPU_FP64;
  cfgpu_flags fl{};
  long long bytes = 0;
  long long launches = 0;
  // base flow and constraint (NSE::initCFConstraint)
  std::vector<double> Ubase, Wbase, Ubaseyy, Wbaseyy;
  double UbulkBase = 0, WbulkBase = 0, dPdxRef = 0, dPdzRef = 0, UbulkRef = 0, WbulkRef = 0;
  double dPdxAct = 0, dPdzAct = 0;
  double UbulkAct = 0, WbulkAct = 0;  // NSE::UbulkAct_ (nse.cpp:645): set from the initial field at construction
  double baseShear[2] = {0, 0};
  double *dUbase = nullptr, *dWbase = nullptr, *dUbaseyy = nullptr, *dWbaseyy = nullptr;
  double* ddPdx = nullptr;  // [2]
  // Helmholtz B rows
  double *hb_lo = nullptr, *hb_di = nullptr, *hb_up = nullptr;
  // transforms
  FftPlan px{}, pz{};
  void *twx = nullptr, *twz = nullptr;  // R-typed complex
  // fused x/z pass (rotational form): full-circle twiddle tables exp(-2 pi i e/L), cluster shape
  void *twxf = nullptr, *twzf = nullptr;
  bool xzf = false;
  int xzC = 0, xzRC = 0;
  // Chebyshev transforms of the rotational form through the FFT (dct_table(Ny), R-typed): chosen at creation
  void* cdct = nullptr;
  bool ydct = false;
  // forward Chebyshev transform of the mixed path on the tensor cores (cheb_tc_matrix(Ny), BF16 splits)
  void* ctc = nullptr;
  int* dtcerr = nullptr;
  bool ytc = false;
  void *cinvA = nullptr, *cinvB = nullptr, *cfwdA = nullptr, *cfwdB = nullptr;
  void *cderA = nullptr, *cderB = nullptr, *basey = nullptr;  // fused curl: (2/L) T'_n(y_j); U, U', W, W' at y_j
  void *cdfA = nullptr, *cdfB = nullptr;                       // (2/L) diff o chebyfft, parity split
  void* zbasey = nullptr;  // zero base profiles [nb][4N] (LinearAboutProfile: u, v, w without base flow)
  // Mixed precision: the FP32 constant tables above live in one block of DITHER_V dithered versions (cS bytes
  // apart; the pointers above address version 0), basey/baseyS likewise; dver holds each field's version.
  void* cblock = nullptr;
  long long cS = 0;
  const float *kdx = nullptr, *kdz = nullptr, *kmisc = nullptr;  // dithered d/dx, d/dz, {1/(Nx Nz), Vsuck}
  int* dver = nullptr;  // [nb]
  double* dyc = nullptr;           // CFL grid spacing in y per Gauss-Lobatto point
  unsigned long long* dred = nullptr;  // reduction scratch (CFL key, L2 sum)
  unsigned long long* cfl_host = nullptr;  // pinned copy of the CFL keys (asynchronous CFL passes)
  double* stage1 = nullptr;                 // pinned staging of one field (slot transfers)
  bool direct = false;  // kernels read/write the caller's FlowField buffers in host memory directly
  int alt[2] = {0, 0};  // Alternating state of the main (0) and init (1) NSE: 0 = next is divergence
  // state: current fields
  double *Ucur = nullptr, *Qcur = nullptr;
  // multistep ring
  double *Uh[4] = {nullptr}, *Qh[4] = {nullptr};
  void* Nh[4] = {nullptr};
  int perm[4] = {0, 1, 2, 3};
  // CNAB-style (main or init): fj, fj1 per scheme; RK accumulator
  void *fj[2] = {nullptr, nullptr}, *fj1[2] = {nullptr, nullptr};
  void* rkQ[2] = {nullptr, nullptr};
  void* rkN = nullptr;
  // NL work
  void *C6 = nullptr, *W6 = nullptr, *X6 = nullptr, *Z3 = nullptr, *F3 = nullptr;
  double* scratch = nullptr;
  int RP = 8;     // x rows per block of the z pass (autotuned)
  int xcols = 0;  // kz columns per block of the x passes (autotuned; 0 = all that fit)
  // schemes
  Scheme main, init;
  bool has_init = false;
  // host staging (pinned)
  double* stage = nullptr;
  size_t stage_elems = 0;
  // DNSFlags::symmetries / symmetryprojectioninterval (velocity; the pressure's symmetry is the identity)
  std::vector<SymmetryDev> syms;
  int sym_interval = 100;
  // CUDA graphs of one main-scheme step, keyed by the step's buffer rotation state
  bool use_graphs = true;
  bool autotune = true;  // block shapes of the FFT passes timed at creation (cached per grid)
  struct StepGraph {
    int key;
    cudaGraphExec_t exec;
    long long launches;
  };
  std::vector<StepGraph> graphs;
  bool graph_warm = false;  // one eager main step ran since the graphs were last dropped
  // phase profiling: event pairs recorded around NL passes (0) and tau solves (1)
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_used;

  size_t rowc() const { return 2 * (size_t)g.Md * nb; }      // doubles per row (all fields)
  size_t compc() const { return rowc() * (size_t)N; }         // doubles per component
  size_t rsz() const { return precision == CFGPU_FP64 ? 8 : 4; }
};

namespace {

cudaEvent_t take_event(cfgpu_dns d) {
  if (d->ev_pool.empty()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t e = d->ev_pool.back();
  d->ev_pool.pop_back();
  return e;
}

struct PhaseScope {
  cfgpu_dns d;
  int phase;
  cudaEvent_t a = nullptr;
  PhaseScope(cfgpu_dns d_, int p) : d(d_), phase(p) {
    if (d->profiling) {
      a = take_event(d);
      cudaEventRecord(a, d->st);
    }
  }
  ~PhaseScope() {
    if (d->profiling) {
      cudaEvent_t b = take_event(d);
      cudaEventRecord(b, d->st);
      d->ev_used.push_back({phase, {a, b}});
    }
  }
};

int build_tables(cfgpu_dns d, Scheme& s) {
  const size_t FN = (size_t)d->N * d->gm.Md;
  HelmB hb{d->hb_lo, d->hb_di, d->hb_up};
  if (!s.tau.empty()) CK(cudaStreamSynchronize(d->st));  // no queued step still reads the old tables
  for (auto& t : s.tau) {
    dfree(t.f);
    dfree(t.s);
  }
  s.tau.clear();
  const int nt = (int)s.lambda_t.size();
  if (nt > 4) return fail(CFGPU_EINVAL, "more than 4 substeps");
  TauSetupBatch tb{};
  for (int j = 0; j < nt; ++j) {
    TauTable t{};
    CKS(dalloc(&t.f, FN * TF_NFIELDS, d->bytes));
    CKS(dalloc(&t.s, (size_t)d->gm.Md * TS_NSCALARS, d->bytes));
    s.tau.push_back(t);
    tb.tab[j] = t;
    tb.lambda_t[j] = s.lambda_t[j];
  }
  // all substep tables in one launch (per field when the fields have their own nu and dt)
  if (d->hetero) {
    for (int f = 0; f < d->nb; ++f) {
      for (int j = 0; j < nt; ++j) tb.lambda_t[j] = lambda_at(s.method, d->sfl[f].dt, j);
      CK(launch_tau_setup_batch(d->gm, d->N, tb, nt, d->sfl[f].nu, hb, d->scratch, d->st, f * d->g.Md, d->g.Md));
      d->launches++;
    }
  } else {
    CK(launch_tau_setup_batch(d->gm, d->N, tb, nt, d->fl.nu, hb, d->scratch, d->st));
    d->launches++;
  }
  return CFGPU_OK;
}

// Rebuild one field's part of every tau table (its nu changed).
// A DNS running main-scheme steps only (its start-up done, fields arriving through
// cfgpu_ensemble_load_slot) needs no start-up tables: those are rebuilt by the next restart.
int build_slot_tables(cfgpu_dns d, int f) {
  HelmB hb{d->hb_lo, d->hb_di, d->hb_up};
  for (Scheme* s : {&d->main, &d->init}) {
    if (s == &d->init && (!d->has_init || d->main.full)) continue;
    TauSetupBatch tb{};
    const int nt = (int)s->tau.size();
    for (int j = 0; j < nt; ++j) {
      tb.lambda_t[j] = lambda_at(s->method, d->sfl[f].dt, j);
      tb.tab[j] = s->tau[j];
    }
    CK(launch_tau_setup_batch(d->gm, d->N, tb, nt, d->sfl[f].nu, hb, d->scratch, d->st, f * d->g.Md, d->g.Md));
    d->launches++;
  }
  return CFGPU_OK;
}

// Constant versions of the nonlinear pass (mixed precision; FP64 uses its exact tables).
Dither dither_of(cfgpu_dns d) {
  Dither dt{};
  dt.ver = d->precision == CFGPU_FP64 ? nullptr : d->dver;
  dt.S = d->cS;
  dt.Sb = (long long)4 * d->N * (d->hetero ? d->nb : 1) * (long long)d->rsz();
  dt.nb = d->nb;
  dt.kdx = d->precision == CFGPU_FP64 ? nullptr : d->kdx;
  dt.kdz = d->precision == CFGPU_FP64 ? nullptr : d->kdz;
  dt.kmisc = d->precision == CFGPU_FP64 ? nullptr : d->kmisc;
  return dt;
}

// Nonlinear term N(u) of the fields in U (solved-mode layout) into Nout (R-typed):
// navierstokesNL (nse.cpp:12-91) for the form selected by the flags; `which`
// selects the NSE (0 main, 1 init) whose Alternating state is advanced.
template <typename R>
int nonlinear_impl(cfgpu_dns d, const double* U, void* Nout, int form) {
  const GridDev& g = d->gm;   // per-mode kernels
  const GridDev& gp = d->gp;  // per-plane x/z kernels
  const int N = d->N;
  R* C6 = (R*)d->C6;
  R* W = (R*)d->W6;
  const size_t row = d->rowc(), comp = d->compc();
  int nin = 6, nout = 3;
  const void* by = d->hetero ? d->baseyS : d->basey;
  const int bstride = d->hetero ? 4 * N : 0;
  const Dither dt = dither_of(d);
  Dither dt0 = dt;  // zero base profiles: one version
  dt0.Sb = 0;
  if (form == CFGPU_LinearAboutProfile) {
    // linearizedNL: u, v, w at the points (no base flow), (U d/dx + W d/dz) u + v (U', 0, W'), forward y
    if ((N + 1) / 2 > 56) return fail(CFGPU_ENOTSUP, "Ny > 111 with LinearAboutProfile");
    CK(launch_grad_cheb<R>(g, N, false, U, W, (const R*)d->cinvA, (const R*)d->cinvB, (const R*)d->cderA,
                           (const R*)d->cderB, (const R*)d->zbasey, 0.0, d->st, bstride, dt0));
    CK(launch_linprof<R>(g, N, W, (const R*)by, bstride, (R*)d->F3, d->st, dt));
    CK((launch_cheb<R, R, R>(N, false, (int)row, 3, (const R*)d->F3, row, comp, (R*)Nout, row, comp,
                             (const R*)d->cfwdA, (const R*)d->cfwdB, d->st, dt)));
    d->launches += 3;
    return CFGPU_OK;
  }
  const double* bU = d->hetero ? d->dbaseS : d->dUbase;
  const double* bW = d->hetero ? d->dbaseS + (size_t)d->nb * N : d->dWbase;
  if (form == NL_ROTATIONAL && d->ydct) {
    // spectral curl, then the inverse transform of u, v, w, ox, oy, oz through the FFT
    CK(launch_curl_base<R>(g, U, C6, bU, bW, d->hetero ? N : 0, d->fl.Vsuck, d->st));
    CK(launch_dct<R>(N, true, g.Md, 6, (const cpx<R>*)C6, row / 2, comp / 2, (cpx<R>*)W, row / 2, comp / 2,
                     (const cpx<R>*)d->cdct, d->st, dt));
    d->launches += 2;
  } else if (form == NL_ROTATIONAL) {
    if ((N + 1) / 2 <= 56) {
      CK(launch_curl_cheb<R>(g, N, U, W, (const R*)d->cinvA, (const R*)d->cinvB, (const R*)d->cderA,
                             (const R*)d->cderB, (const R*)(d->hetero ? d->baseyS : d->basey), d->fl.Vsuck, d->st,
                             d->hetero ? 4 * N : 0, dt));
      d->launches += 1;
    } else {
      CK(launch_curl_base<R>(g, U, C6, bU, bW, d->hetero ? N : 0, d->fl.Vsuck, d->st));
      CK((launch_cheb<R, R, R>(N, true, (int)row, 6, C6, row, comp, W, row, comp, (const R*)d->cinvA,
                               (const R*)d->cinvB, d->st, dt)));
      d->launches += 2;
    }
  } else {
    if ((N + 1) / 2 > 56) return fail(CFGPU_ENOTSUP, "Ny > 111 with a gradient nonlinear form");
    const bool gradient = form != NL_DIVERGENCE;
    CK(launch_grad_cheb<R>(g, N, gradient, U, W, (const R*)d->cinvA, (const R*)d->cinvB, (const R*)d->cderA,
                           (const R*)d->cderB, (const R*)(d->hetero ? d->baseyS : d->basey), d->fl.Vsuck, d->st,
                           d->hetero ? 4 * N : 0, dt));
    d->launches += 1;
    nin = gradient ? 12 : 3;
    nout = form == NL_CONVECTION ? 3 : (form == NL_DIVERGENCE ? 6 : 9);
  }
  if (form == NL_ROTATIONAL && d->xzf) {
    CK(launch_xz_rot(gp, d->xzC, d->xzRC, (const cpx<R>*)W, (cpx<R>*)d->F3, (const cpx<R>*)d->twxf,
                     (const cpx<R>*)d->twzf, d->st, dt));
    d->launches += 1;
  } else {
    CK(launch_xinv<R>(gp, d->px, (const cpx<R>*)d->twx, (const cpx<R>*)W, (cpx<R>*)d->X6, nin, d->st, d->xcols,
                      dt));
    CK(launch_zphys<R>(gp, form, d->pz, (const cpx<R>*)d->twz, d->RP, (const cpx<R>*)d->X6, (cpx<R>*)d->Z3, d->st,
                       dt, (const cpx<R>*)d->twzf));
    CK(launch_xfwd<R>(gp, d->px, (const cpx<R>*)d->twx, (const cpx<R>*)d->Z3, (cpx<R>*)d->F3, nout, d->st,
                      d->xcols, dt));
    d->launches += 3;
  }
  const R* F = (const R*)d->F3;
  if constexpr (sizeof(R) == 4) {
    if ((form == NL_ROTATIONAL || form == NL_CONVECTION) && d->ytc) {
      CK(launch_cheb_tc(N, (int)row, 3, (const float*)F, row, comp, (float*)Nout, d->ctc, d->dtcerr, d->st));
      d->launches += 1;
      return CFGPU_OK;
    }
  }
  if (form == NL_ROTATIONAL && d->ydct) {
    CK(launch_dct<R>(N, false, g.Md, 3, (const cpx<R>*)F, row / 2, comp / 2, (cpx<R>*)Nout, row / 2, comp / 2,
                     (const cpx<R>*)d->cdct, d->st, dt));
    d->launches += 1;
  } else if (form == NL_ROTATIONAL || form == NL_CONVECTION) {
    CK((launch_cheb<R, R, R>(N, false, (int)row, 3, F, row, comp, (R*)Nout, row, comp, (const R*)d->cfwdA,
                             (const R*)d->cfwdB, d->st, dt)));
    d->launches += 1;
  } else {
    // products p_ij (ij = uu, uv, uw, vv, vw, ww) follow the convection term for the skew form
    const R* p = form == NL_SKEW ? F + 3 * comp : F;
    const int pij[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    const R half = (R)0.5;
    for (int i = 0; i < 3; ++i) {
      const R* pF = form == NL_SKEW ? F + i * comp : nullptr;
      const R wF = form == NL_SKEW ? half : (R)0, w = form == NL_SKEW ? half : (R)1;
      CK(launch_cheb_fwd_div<R>(g, N, pF, p + pij[i][0] * comp, p + pij[i][2] * comp, p + pij[i][1] * comp, wF, w,
                                w, (R*)Nout + i * comp, (const R*)d->cfwdA, (const R*)d->cfwdB,
                                (const R*)d->cdfA, (const R*)d->cdfB, d->st, dt));
    }
    d->launches += 3;
  }
  return CFGPU_OK;
}

template <typename R>
int rotation_term(cfgpu_dns d, const double* U, void* Nout) {
  const double* Ub = d->hetero ? d->dbaseS : d->dUbase;
  CK(launch_rotation<R>(d->gm, d->N, U, Ub, d->hetero ? d->N : 0, d->fl.rotation, d->fl.Vsuck, (R*)Nout, d->st));
  d->launches++;
  return CFGPU_OK;
}

int nonlinear(cfgpu_dns d, const double* U, void* Nout, int which = 0) {
  PhaseScope ps(d, 0);
  int form = d->fl.nonlinearity;
  if (form == CFGPU_Alternating || form == CFGPU_Alternating_) {
    // navierstokesNL flips the NSE's flag on every call (nse.cpp:50-57): divergence, then convection, ...
    form = d->alt[which] == 0 ? NL_DIVERGENCE : NL_CONVECTION;
    d->alt[which] ^= 1;
  }
  const bool fp64 = d->precision == CFGPU_FP64;
  CKS(fp64 ? nonlinear_impl<double>(d, U, Nout, form) : nonlinear_impl<float>(d, U, Nout, form));
  // rotation about z (nse.cpp:62-78; not with LinearAboutProfile)
  if (d->fl.rotation != 0.0 && form != CFGPU_LinearAboutProfile)
    CKS(fp64 ? rotation_term<double>(d, U, Nout) : rotation_term<float>(d, U, Nout));
  if (!fp64) {
    CK(launch_dither_bump(d->dver, d->nb, d->st));  // next evaluation: next version of the FP32 constants
    d->launches++;
  }
  return CFGPU_OK;
}

SolveParams base_params(cfgpu_dns d) {
  SolveParams sp{};
  sp.nu = d->fl.nu;
  sp.constraint = d->fl.constraint;
  sp.dPdxRef = d->dPdxRef;
  sp.dPdzRef = d->dPdzRef;
  sp.umean = d->UbulkRef - d->UbulkBase;
  sp.wmean = d->WbulkRef - d->WbulkBase;
  sp.baseShear[0] = d->baseShear[0];
  sp.baseShear[1] = d->baseShear[1];
  sp.taucorrection = d->fl.taucorrection;
  sp.force_real00 = 1;
  return sp;
}

SolvePtrs base_ptrs(cfgpu_dns d) {
  SolvePtrs p{};
  p.Ubaseyy = d->dUbaseyy;
  p.Wbaseyy = d->dWbaseyy;
  p.Ubase = d->dUbase;
  p.Wbase = d->dWbase;
  p.scratch = d->scratch;
  p.dPdx_out = d->ddPdx;
  if (d->hetero) {
    const size_t nN = (size_t)d->nb * d->N;
    p.Ubase = d->dbaseS;
    p.Wbase = d->dbaseS + nN;
    p.Ubaseyy = d->dbaseS + 2 * nN;
    p.Wbaseyy = d->dbaseS + 3 * nN;
    p.slot = d->dslot;
    p.base_stride = d->N;
  }
  return p;
}

int tau_solve(cfgpu_dns d, const SolveParams& sp, const SolvePtrs& p, const TauTable& tt) {
  PhaseScope ps(d, 1);
  HelmB hb{d->hb_lo, d->hb_di, d->hb_up};
  if (d->precision == CFGPU_FP64) {
    CK(launch_tau_solve<double>(d->gm, d->N, sp, p, hb, tt, d->st));
  } else {
    CK(launch_tau_solve<float>(d->gm, d->N, sp, p, hb, tt, d->st));
  }
  d->launches += tau_solve_launches(d->N);
  return CFGPU_OK;
}

size_t state_bytes(cfgpu_dns d) { return d->compc() * sizeof(double); }

// ---- multistep (dnsalgo.cpp:202-315) ---------------------------------------
void ms_shift(cfgpu_dns d) {
  const int K = d->main.order;
  const int last = d->perm[K - 1];
  for (int j = K - 1; j > 0; --j) d->perm[j] = d->perm[j - 1];
  d->perm[0] = last;
}

int ms_push(cfgpu_dns d) {
  ms_shift(d);
  if (d->main.order > 1) {
    const int s1 = d->perm[1];
    CK(cudaMemcpyAsync(d->Uh[s1], d->Ucur, 3 * state_bytes(d), cudaMemcpyDeviceToDevice, d->st));
    CK(cudaMemcpyAsync(d->Qh[s1], d->Qcur, state_bytes(d), cudaMemcpyDeviceToDevice, d->st));
    CKS(nonlinear(d, d->Uh[s1], d->Nh[s1]));
  }
  d->main.t += d->fl.dt;
  d->main.countdown--;
  d->main.full = (d->main.countdown == 0);
  return CFGPU_OK;
}

// One multistep step on the ring (rhs from u_j, N_j; solve into the oldest slot; rotate).
int ms_step(cfgpu_dns d) {
  Scheme& s = d->main;
  const int K = s.order, J = K - 1;
  const double dt = d->fl.dt;
  CKS(nonlinear(d, d->Uh[d->perm[0]], d->Nh[d->perm[0]]));
  SolveParams sp = base_params(d);
  sp.kind = 0;
  sp.order = K;
  SolvePtrs p = base_ptrs(d);
  for (int j = 0; j < K; ++j) {
    sp.a[j] = -s.alpha[j] / dt;
    sp.b[j] = -s.beta[j];
    p.uin[j] = d->Uh[d->perm[j]];
    p.nin[j] = d->Nh[d->perm[j]];
  }
  p.uout = d->Uh[d->perm[J]];
  p.qout = d->Qh[d->perm[J]];
  CKS(tau_solve(d, sp, p, s.tau[0]));
  ms_shift(d);
  s.t += dt;
  return CFGPU_OK;
}

int main_step(cfgpu_dns d);

// Host-side state changes of one main step (replayed beside a graph launch).
void main_step_host(cfgpu_dns d) {
  Scheme& s = d->main;
  if (s.family == 0) {
    ms_shift(d);
  } else if (s.family == 1) {
    for (int j = 0; j < s.nsub; ++j) std::swap(d->fj[0], d->fj1[0]);
  }
  s.t += d->fl.dt;
}

// Rotation state that selects a step graph: ring phase (multistep) or fj/fj1 order (CNAB).
int main_step_key(cfgpu_dns d) {
  if (d->main.family == 0) return d->perm[0];
  if (d->main.family == 1) return d->fj[0] < d->fj1[0] ? 0 : 1;
  return 0;
}

void drop_graphs(cfgpu_dns d) {
  for (auto& g : d->graphs) cudaGraphExecDestroy(g.exec);
  d->graphs.clear();
  d->graph_warm = false;
}

// One main-scheme step, replayed from a captured CUDA graph when one exists for this rotation state.
// The first step of each state runs eagerly (first-use kernel attributes are set outside any
// capture), the second is captured.
int main_step_graph(cfgpu_dns d) {
  const bool alternating = d->fl.nonlinearity == CFGPU_Alternating || d->fl.nonlinearity == CFGPU_Alternating_;
  if (!d->use_graphs || d->profiling || alternating) return main_step(d);
  const int key = main_step_key(d);
  for (auto& g : d->graphs)
    if (g.key == key) {
      CK(cudaGraphLaunch(g.exec, d->st));
      d->launches += g.launches;
      main_step_host(d);
      return CFGPU_OK;
    }
  if (!d->graph_warm) {
    d->graph_warm = true;
    return main_step(d);
  }
  const long long l0 = d->launches;
  CK(cudaStreamBeginCapture(d->st, cudaStreamCaptureModeThreadLocal));
  const int st = main_step(d);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(d->st, &graph);
  if (st != CFGPU_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return fail(CFGPU_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e2 = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e2 != cudaSuccess) return fail(CFGPU_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e2));
  d->graphs.push_back({key, exec, d->launches - l0});
  CK(cudaGraphLaunch(exec, d->st));  // the captured step has not run yet
  return CFGPU_OK;
}

int ms_advance(cfgpu_dns d, int nsteps) {
  if (nsteps <= 0) return CFGPU_OK;
  CK(cudaMemcpyAsync(d->Uh[d->perm[0]], d->Ucur, 3 * state_bytes(d), cudaMemcpyDeviceToDevice, d->st));
  CK(cudaMemcpyAsync(d->Qh[d->perm[0]], d->Qcur, state_bytes(d), cudaMemcpyDeviceToDevice, d->st));
  for (int step = 0; step < nsteps; ++step) CKS(main_step_graph(d));
  CK(cudaMemcpyAsync(d->Ucur, d->Uh[d->perm[0]], 3 * state_bytes(d), cudaMemcpyDeviceToDevice, d->st));
  CK(cudaMemcpyAsync(d->Qcur, d->Qh[d->perm[0]], state_bytes(d), cudaMemcpyDeviceToDevice, d->st));
  return CFGPU_OK;
}

// ---- CNAB-style (dnsalgo.cpp:608-697); which = 0 main, 1 init --------------
int cnab_push(cfgpu_dns d, int which) {
  std::swap(d->fj[which], d->fj1[which]);
  CKS(nonlinear(d, d->Ucur, d->fj[which], which));
  Scheme& s = which == 0 ? d->main : d->init;
  s.t += d->fl.dt;
  s.full = true;
  return CFGPU_OK;
}

int cnab_step(cfgpu_dns d, int which) {
  Scheme& s = which == 0 ? d->main : d->init;
  {
    for (int j = 0; j < s.nsub; ++j) {
      std::swap(d->fj[which], d->fj1[which]);
      CKS(nonlinear(d, d->Ucur, d->fj[which], which));
      SolveParams sp = base_params(d);
      sp.kind = 1;
      sp.scheme = which;
      sp.substep = j;
      sp.lam = s.lambda_t[j];
      sp.a_b = s.ca[j] / s.cb[j];
      sp.g_b = s.cg[j] / s.cb[j];
      sp.z_b = s.cz[j] / s.cb[j];
      SolvePtrs p = base_ptrs(d);
      p.uin[0] = d->Ucur;
      p.nin[0] = d->fj[which];
      p.nin[1] = d->fj1[which];
      p.qin = d->Qcur;
      p.uout = d->Ucur;
      p.qout = d->Qcur;
      CKS(tau_solve(d, sp, p, s.tau[j]));
    }
    s.t += d->fl.dt;
  }
  return CFGPU_OK;
}

// ---- CNRK2 (dnsalgo.cpp:419-470) -------------------------------------------
int rk_step(cfgpu_dns d, int which) {
  Scheme& s = which == 0 ? d->main : d->init;
  {
    for (int j = 0; j < s.nsub; ++j) {
      CKS(nonlinear(d, d->Ucur, d->rkN, which));
      SolveParams sp = base_params(d);
      sp.kind = 2;
      sp.scheme = which;
      sp.substep = j;
      sp.lam = s.lambda_t[j];
      sp.rkA = s.rA[j];
      sp.B_C = s.rB[j] / s.rC[j];
      SolvePtrs p = base_ptrs(d);
      p.uin[0] = d->Ucur;
      p.nin[0] = d->rkN;
      p.Q = d->rkQ[which];
      p.qin = d->Qcur;
      p.uout = d->Ucur;
      p.qout = d->Qcur;
      CKS(tau_solve(d, sp, p, s.tau[j]));
    }
    s.t += d->fl.dt;
  }
  return CFGPU_OK;
}

int main_step(cfgpu_dns d) {
  if (d->main.family == 0) return ms_step(d);
  if (d->main.family == 1) return cnab_step(d, 0);
  return rk_step(d, 0);
}

// One step of an order-1 multistep start-up scheme (SBDF1 / CNFE1; MultistepDNS::advance, dnsalgo.cpp:202-251
// with order 1): rhs = -alpha_0/dt u_n - beta_0 N(u_n), solved with lambda_t = eta/dt.
int ms1_init_step(cfgpu_dns d) {
  Scheme& s = d->init;
  CKS(nonlinear(d, d->Ucur, d->fj[1], 1));
  SolveParams sp = base_params(d);
  sp.kind = 0;
  sp.order = 1;
  sp.scheme = 1;
  sp.a[0] = -s.alpha[0] / d->fl.dt;
  sp.b[0] = -s.beta[0];
  SolvePtrs p = base_ptrs(d);
  p.uin[0] = d->Ucur;  // the right-hand side is complete before the solve writes u
  p.nin[0] = d->fj[1];
  p.uout = d->Ucur;
  p.qout = d->Qcur;
  CKS(tau_solve(d, sp, p, s.tau[0]));
  s.t += d->fl.dt;
  return CFGPU_OK;
}

int scheme_advance(cfgpu_dns d, int which, int nsteps) {
  Scheme& s = which == 0 ? d->main : d->init;
  if (which == 0 && s.family == 0) return ms_advance(d, nsteps);
  for (int n = 0; n < nsteps; ++n) {
    if (which == 0) {
      CKS(main_step_graph(d));
    } else {
      CKS(s.family == 0 ? ms1_init_step(d) : (s.family == 1 ? cnab_step(d, 1) : rk_step(d, 1)));
    }
  }
  return CFGPU_OK;
}

int scheme_push(cfgpu_dns d) {
  if (d->main.family == 0) return ms_push(d);
  if (d->main.family == 1) return cnab_push(d, 0);
  return CFGPU_OK;
}

// DNS::advance (dns.cpp:135-163)
// sigma (or its projection) on ncomp components of the resident array a (element type size esz).
int symmetry_on(cfgpu_dns d, void* a, size_t esz, int ncomp, const SymmetryDev& sy, int project) {
  const size_t bytes = (size_t)ncomp * d->compc() * esz;
  if (esz == 8) {
    CK(launch_symmetry<double>(d->g, d->nb, d->N, ncomp, sy, project, a, d->scratch, d->st));
  } else {
    CK(launch_symmetry<float>(d->g, d->nb, d->N, ncomp, sy, project, a, d->scratch, d->st));
  }
  d->launches++;
  CK(cudaMemcpyAsync(a, d->scratch, bytes, cudaMemcpyDeviceToDevice, d->st));
  return CFGPU_OK;
}

// DNS::advance's projection (dns.cpp:151-155): the velocity and the main algorithm's stored fields
// (MultistepDNS::project, dnsalgo.cpp:255-262: u_j and N_j; CNABstyleDNS::project, :628-632: f_j).
int project_symmetries(cfgpu_dns d) {
  const size_t rs = d->rsz();
  for (const SymmetryDev& sy : d->syms) {
    CKS(symmetry_on(d, d->Ucur, 8, 3, sy, 1));
    if (d->main.family == 0) {
      for (int j = 0; j < d->main.order; ++j) {
        CKS(symmetry_on(d, d->Uh[j], 8, 3, sy, 1));
        CKS(symmetry_on(d, d->Nh[j], rs, 3, sy, 1));
      }
    } else if (d->main.family == 1) {
      CKS(symmetry_on(d, d->fj[0], rs, 3, sy, 1));
    }
  }
  return CFGPU_OK;
}

int dns_advance_device(cfgpu_dns d, int nsteps) {
  if (!d->syms.empty() && ((int)d->main.t) % d->sym_interval == 0) CKS(project_symmetries(d));
  int n = 0;
  while (!d->main.full && n < nsteps) {
    if (!d->has_init) return fail(CFGPU_EINVAL, "main algorithm uninitialized and no init algorithm");
    CKS(scheme_push(d));
    CKS(scheme_advance(d, 1, 1));
    ++n;
  }
  return scheme_advance(d, 0, nsteps - n);
}

// host serial layout <-> solved-mode layout.  The host side holds nf
// consecutive FlowFields (Nd components each, fields f0 .. f0+nf-1 of the
// batch); the device side is [i][my][field][m] with nb fields (fstride = nb),
// or one field's compact [i][my][m] (fstride = 1, f0 = 0).
// Row-parallel loop over (field, component, y) rows: one contiguous run of Kz+1 complex values per solved kx
// in both layouts.  Large transfers are split over host threads.
template <typename F>
void for_rows(size_t nrows, size_t row_bytes, const F& body) {
  const size_t total = nrows * row_bytes;
  unsigned nt = total > (8u << 20) ? std::min(8u, std::max(1u, std::thread::hardware_concurrency())) : 1u;
  if (nt <= 1 || nrows < 2 * nt) {
    for (size_t r = 0; r < nrows; ++r) body(r);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      for (size_t r = t; r < nrows; r += nt) body(r);
    });
  for (auto& x : th) x.join();
}

void gather_modes(cfgpu_dns d, const double* h, int Nd, double* out, int f0 = 0, int nf = -1, int fstride = -1) {
  const GridDev& g = d->g;
  const int Mz = g.Nz / 2 + 1;
  if (nf < 0) nf = d->nb;
  if (fstride < 0) fstride = d->nb;
  const size_t hfield = (size_t)2 * Nd * g.Ny * g.Nx * Mz;
  const size_t nrows = (size_t)nf * Nd * g.Ny;
  for_rows(nrows, (size_t)16 * g.Md, [&](size_t r) {
    const int my = (int)(r % g.Ny), i = (int)((r / g.Ny) % Nd), f = (int)(r / ((size_t)g.Ny * Nd));
    const double* src = h + f * hfield + 2 * (((size_t)i * g.Ny + my) * g.Nx) * Mz;
    double* dst = out + 2 * ((((size_t)i * g.Ny + my) * fstride + (f0 + f)) * g.Md);
    for (int ix = 0; ix < g.NKx; ++ix) {
      const int kx = ix <= g.Kx ? ix : ix - g.NKx;
      const int mx = kx >= 0 ? kx : kx + g.Nx;
      memcpy(dst + 2 * (size_t)ix * g.NKz, src + 2 * (size_t)mx * Mz, 16 * (size_t)g.NKz);
    }
  });
}
void scatter_modes(cfgpu_dns d, const double* in, int Nd, double* h, int f0 = 0, int nf = -1, int fstride = -1) {
  const GridDev& g = d->g;
  const int Mz = g.Nz / 2 + 1;
  if (nf < 0) nf = d->nb;
  if (fstride < 0) fstride = d->nb;
  const size_t hfield = (size_t)2 * Nd * g.Ny * g.Nx * Mz;
  const size_t nrows = (size_t)nf * Nd * g.Ny;
  for_rows(nrows, (size_t)16 * g.Md, [&](size_t r) {
    const int my = (int)(r % g.Ny), i = (int)((r / g.Ny) % Nd), f = (int)(r / ((size_t)g.Ny * Nd));
    double* dst = h + f * hfield + 2 * (((size_t)i * g.Ny + my) * g.Nx) * Mz;
    const double* src = in + 2 * ((((size_t)i * g.Ny + my) * fstride + (f0 + f)) * g.Md);
    for (int ix = 0; ix < g.NKx; ++ix) {
      const int kx = ix <= g.Kx ? ix : ix - g.NKx;
      const int mx = kx >= 0 ? kx : kx + g.Nx;
      memcpy(dst + 2 * (size_t)mx * Mz, src + 2 * (size_t)ix * g.NKz, 16 * (size_t)g.NKz);
    }
  });
}

int ensure_stage(cfgpu_dns d) {
  if (!d->stage) CKS(pinned_alloc(&d->stage, d->stage_elems * sizeof(double)));
  return CFGPU_OK;
}

int set_fields(cfgpu_dns d, const double* u, const double* q) {
  if (d->direct) {
    if (u) CK(launch_host_modes(d->g, true, 3, d->nb, 0, d->nb, u, d->Ucur, d->st));
    if (q) CK(launch_host_modes(d->g, true, 1, d->nb, 0, d->nb, q, d->Qcur, d->st));
    return CFGPU_OK;  // the caller synchronizes before the buffers may change
  }
  CKS(ensure_stage(d));
  const size_t cd = d->compc();
  if (u) {
    gather_modes(d, u, 3, d->stage);
    CK(cudaMemcpyAsync(d->Ucur, d->stage, 3 * cd * sizeof(double), cudaMemcpyHostToDevice, d->st));
  }
  if (q) {
    gather_modes(d, q, 1, d->stage + 3 * cd);
    CK(cudaMemcpyAsync(d->Qcur, d->stage + 3 * cd, cd * sizeof(double), cudaMemcpyHostToDevice, d->st));
  }
  return CFGPU_OK;
}

int get_fields(cfgpu_dns d, double* u, double* q) {
  if (d->direct) {
    if (u) CK(launch_host_modes(d->g, false, 3, d->nb, 0, d->nb, d->Ucur, u, d->st));
    if (q) CK(launch_host_modes(d->g, false, 1, d->nb, 0, d->nb, d->Qcur, q, d->st));
    CK(cudaStreamSynchronize(d->st));
    return CFGPU_OK;
  }
  CKS(ensure_stage(d));
  const size_t cd = d->compc();
  CK(cudaMemcpyAsync(d->stage, d->Ucur, 3 * cd * sizeof(double), cudaMemcpyDeviceToHost, d->st));
  CK(cudaMemcpyAsync(d->stage + 3 * cd, d->Qcur, cd * sizeof(double), cudaMemcpyDeviceToHost, d->st));
  CK(cudaStreamSynchronize(d->st));
  if (u) scatter_modes(d, d->stage, 3, u);
  if (q) scatter_modes(d, d->stage + 3 * cd, 1, q);
  return CFGPU_OK;
}

// One field (slot) of a batch: the rows [c][ny] of that field are strided by nb*Md modes on the device.
int ensure_stage1(cfgpu_dns d) {
  if (!d->stage1) CKS(pinned_alloc(&d->stage1, 4 * 2 * (size_t)d->g.Md * d->N * sizeof(double)));
  return CFGPU_OK;
}

int set_slot(cfgpu_dns d, int slot, const double* u, const double* q) {
  if (d->direct) {
    if (u) CK(launch_host_modes(d->g, true, 3, 1, slot, d->nb, u, d->Ucur, d->st));
    if (q) CK(launch_host_modes(d->g, true, 1, 1, slot, d->nb, q, d->Qcur, d->st));
    CK(cudaStreamSynchronize(d->st));
    return CFGPU_OK;
  }
  CKS(ensure_stage1(d));
  double* stage = d->stage1;
  const size_t w = 2 * (size_t)d->g.Md, pitch = w * d->nb, cd1 = w * d->N;
  if (u) {
    gather_modes(d, u, 3, stage, 0, 1, 1);
    CK(cudaMemcpy2DAsync(d->Ucur + slot * w, pitch * sizeof(double), stage, w * sizeof(double),
                         w * sizeof(double), 3 * (size_t)d->N, cudaMemcpyHostToDevice, d->st));
  }
  if (q) {
    gather_modes(d, q, 1, stage + 3 * cd1, 0, 1, 1);
    CK(cudaMemcpy2DAsync(d->Qcur + slot * w, pitch * sizeof(double), stage + 3 * cd1, w * sizeof(double),
                         w * sizeof(double), (size_t)d->N, cudaMemcpyHostToDevice, d->st));
  }
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

int get_slot(cfgpu_dns d, int slot, double* u, double* q) {
  if (d->direct) {
    if (u) CK(launch_host_modes(d->g, false, 3, 1, slot, d->nb, d->Ucur, u, d->st));
    if (q) CK(launch_host_modes(d->g, false, 1, 1, slot, d->nb, d->Qcur, q, d->st));
    CK(cudaStreamSynchronize(d->st));
    return CFGPU_OK;
  }
  CKS(ensure_stage1(d));
  double* stage = d->stage1;
  const size_t w = 2 * (size_t)d->g.Md, pitch = w * d->nb, cd1 = w * d->N;
  CK(cudaMemcpy2DAsync(stage, w * sizeof(double), d->Ucur + slot * w, pitch * sizeof(double),
                       w * sizeof(double), 3 * (size_t)d->N, cudaMemcpyDeviceToHost, d->st));
  CK(cudaMemcpy2DAsync(stage + 3 * cd1, w * sizeof(double), d->Qcur + slot * w, pitch * sizeof(double),
                       w * sizeof(double), (size_t)d->N, cudaMemcpyDeviceToHost, d->st));
  CK(cudaStreamSynchronize(d->st));
  if (u) scatter_modes(d, stage, 3, u, 0, 1, 1);
  if (q) scatter_modes(d, stage + 3 * cd1, 1, q, 0, 1, 1);
  return CFGPU_OK;
}

// Host rounding of x to float with dither offset k (the device's dither_const<float>).
float dither_round_host(double x, int k) { return dither_round(x, k); }

// DITHER_V versions of the tables (tables[i] at float offset off[i] of each S-float version) in one block.
int upload_dithered(const std::vector<std::vector<double>>& tables, const std::vector<size_t>& off, size_t S,
                    void** dst, long long& bytes, cudaStream_t st) {
  std::vector<float> h((size_t)DITHER_V * S, 0.0f);
  for (int v = 0; v < DITHER_V; ++v)
    for (size_t i = 0; i < tables.size(); ++i)
      for (size_t e = 0; e < tables[i].size(); ++e) h[(size_t)v * S + off[i] + e] = dither_round_host(tables[i][e], v);
  float* p;
  CKS(dalloc(&p, h.size(), bytes));
  CK(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));  // h is a local
  *dst = p;
  return CFGPU_OK;
}

template <typename R>
int upload_as(const std::vector<double>& v, void** dst, long long& bytes, cudaStream_t st) {
  std::vector<R> t(v.begin(), v.end());
  R* p;
  CKS(dalloc(&p, t.size(), bytes));
  CK(cudaMemcpyAsync(p, t.data(), t.size() * sizeof(R), cudaMemcpyHostToDevice, st));
  *dst = p;
  return CFGPU_OK;
}

template <typename R>
int upload_tw(const std::vector<std::complex<long double>>& tw, void** dst, long long& bytes, cudaStream_t st) {
  std::vector<cpx<R>> t(tw.size() ? tw.size() : 1);
  for (size_t i = 0; i < tw.size(); ++i) t[i] = cmk<R>((R)tw[i].real(), (R)tw[i].imag());
  cpx<R>* p;
  CKS(dalloc(&p, t.size(), bytes));
  CK(cudaMemcpyAsync(p, t.data(), t.size() * sizeof(cpx<R>), cudaMemcpyHostToDevice, st));
  *dst = p;
  return CFGPU_OK;
}

// Autotuner of the FFT passes' block shapes: kz columns per block of the x passes and x rows per block of
// the z pass, timed with CUDA events on this DNS's own work arrays (their contents do not change the
// work), the fastest kept; choices are cached per (grid, planes, precision, form).
struct TuneKey {
  int Nx, planes, Nz, NKz, prec, form;
  bool operator<(const TuneKey& o) const {
    return std::tie(Nx, planes, Nz, NKz, prec, form) < std::tie(o.Nx, o.planes, o.Nz, o.NKz, o.prec, o.form);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, int>> g_tune;
std::atomic<int> g_autotune{1};
std::atomic<int> g_fused_xz{1};
std::atomic<int> g_host_access{1};  // direct host-buffer access when the device supports it

template <typename R>
float time_ms(cfgpu_dns d, const std::function<cudaError_t()>& f) {
  cudaEvent_t a = take_event(d), b = take_event(d);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, d->st);
    if (f() != cudaSuccess) {
      cudaGetLastError();
      best = 1e30f;
      break;
    }
    cudaEventRecord(b, d->st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0) best = std::min(best, ms);  // first run warms up
  }
  d->ev_pool.push_back(a);
  d->ev_pool.push_back(b);
  return best;
}

template <typename R>
int autotune(cfgpu_dns d, int form, int nin, int nout) {
  const GridDev& gp = d->gp;
  const TuneKey key{gp.Nx, gp.Ny, gp.Nz, gp.NKz, (int)sizeof(R), form};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      d->xcols = it->second.first;
      d->RP = it->second.second;
      return CFGPU_OK;
    }
  }
  // small grids are launch-bound: keep the defaults
  if ((long long)gp.Ny * gp.Nx * gp.NKz < 200000) return CFGPU_OK;
  const cpx<R>* tw = (const cpx<R>*)d->twx;
  float best = 1e30f;
  int bestc = d->xcols;
  for (int div : {1, 2, 3, 4, 6}) {
    const int c = (gp.NKz + div - 1) / div;
    if (c < 2 || xfft_smem_bytes<R>(gp, c) > 200 * 1024) continue;
    const float t = time_ms<R>(d, [&]() {
      cudaError_t e = launch_xinv<R>(gp, d->px, tw, (const cpx<R>*)d->W6, (cpx<R>*)d->X6, nin, d->st, c);
      if (e != cudaSuccess) return e;
      return launch_xfwd<R>(gp, d->px, tw, (const cpx<R>*)d->Z3, (cpx<R>*)d->F3, nout, d->st, c);
    });
    if (t < best) {
      best = t;
      bestc = c;
    }
  }
  d->xcols = bestc;
  if (form >= 0) {
    best = 1e30f;
    int bestr = d->RP;
    for (int rp = d->RP; rp >= 2; rp /= 2) {
      if (zphys_smem_bytes<R>(gp, form, rp) > 200 * 1024) continue;
      const float t = time_ms<R>(d, [&]() {
        return launch_zphys<R>(gp, form, d->pz, (const cpx<R>*)d->twz, rp, (const cpx<R>*)d->X6, (cpx<R>*)d->Z3,
                               d->st, kNoDither, (const cpx<R>*)d->twzf);
      });
      if (t < best) {
        best = t;
        bestr = rp;
      }
    }
    d->RP = bestr;
  }
  CK(cudaStreamSynchronize(d->st));
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = {d->xcols, d->RP};
  return CFGPU_OK;
}

// Launch shape of the fused x/z pass: the candidates the device can run, timed with CUDA events on this DNS's
// own work arrays (contents do not change the work) when autotuning is on, else the model's first choice;
// cached per (grid, planes, precision).
std::map<TuneKey, std::pair<int, int>> g_tune_xz;

template <typename R>
int tune_xz(cfgpu_dns d) {
  // keyed and timed on one field's planes, so that a batch and a single field of the same grid take the same
  // form (the forms agree to rounding, not bit for bit)
  GridDev gp = d->gp;
  gp.Ny = d->g.Ny;
  const TuneKey key{gp.Nx, gp.Ny, gp.Nz, gp.NKz, (int)sizeof(R), NL_ROTATIONAL};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_xz.find(key);
    if (it != g_tune_xz.end()) {
      d->xzC = it->second.first;
      d->xzRC = it->second.second;
      d->xzf = d->xzC > 0;
      return CFGPU_OK;
    }
  }
  const std::vector<XzShape> cand = xz_fused_candidates(gp, sizeof(R) == 8);
  d->xzC = d->xzRC = 0;
  if (!cand.empty()) {
    d->xzC = cand[0].C;
    d->xzRC = cand[0].RC;
    if (d->autotune && cand.size() > 1) {
      float best = 1e30f;
      for (const XzShape& c : cand) {
        const float t = time_ms<R>(d, [&]() {
          return launch_xz_rot(gp, c.C, c.RC, (const cpx<R>*)d->W6, (cpx<R>*)d->F3, (const cpx<R>*)d->twxf,
                               (const cpx<R>*)d->twzf, d->st, kNoDither);
        });
        if (t < best) {
          best = t;
          d->xzC = c.C;
          d->xzRC = c.RC;
        }
      }
      // the three-kernel path (x inverse, z pass, x forward) with its own tuned shapes, if faster
      const float t3 = time_ms<R>(d, [&]() {
        cudaError_t e = launch_xinv<R>(gp, d->px, (const cpx<R>*)d->twx, (const cpx<R>*)d->W6, (cpx<R>*)d->X6, 6,
                                       d->st, d->xcols);
        if (e == cudaSuccess)
          e = launch_zphys<R>(gp, NL_ROTATIONAL, d->pz, (const cpx<R>*)d->twz, d->RP, (const cpx<R>*)d->X6,
                              (cpx<R>*)d->Z3, d->st, kNoDither, (const cpx<R>*)d->twzf);
        if (e == cudaSuccess)
          e = launch_xfwd<R>(gp, d->px, (const cpx<R>*)d->twx, (const cpx<R>*)d->Z3, (cpx<R>*)d->F3, 3, d->st,
                             d->xcols);
        return e;
      });
      if (best >= 1e30f || (t3 < best && g_fused_xz.load() != 2)) d->xzC = d->xzRC = 0;
    }
  }
  d->xzf = d->xzC > 0;
  CK(cudaStreamSynchronize(d->st));
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_xz[key] = {d->xzC, d->xzRC};
  return CFGPU_OK;
}

// Chebyshev transforms of the rotational form: dense matrix products (fused curl + inverse, forward) or the
// FFT form (spectral curl, inverse and forward through the FFT), timed with CUDA events on this DNS's own
// arrays when the mode is automatic; cached per (grid, planes, precision).
std::atomic<int> g_cheb_fft{1};
std::map<TuneKey, int> g_tune_cheb;

template <typename R>
int tune_cheb(cfgpu_dns d) {
  d->ydct = false;
  const int mode = g_cheb_fft.load();
  if (mode == 0 || !d->cdct || !dct_supported(d->N)) return CFGPU_OK;
  if (mode == 2) {
    d->ydct = true;
    return CFGPU_OK;
  }
  // keyed and timed on one field (its modes), so that a batch and a single field take the same form
  GridDev g = d->gm;
  g.Md = d->g.Md;
  const TuneKey key{d->g.Nx, d->g.Ny, d->g.Nz, d->g.NKz, (int)sizeof(R), 100};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cheb.find(key);
    if (it != g_tune_cheb.end()) {
      d->ydct = it->second != 0;
      return CFGPU_OK;
    }
  }
  const int N = d->N;
  const size_t row = d->rowc(), comp = d->compc();
  const int nl1 = 2 * d->g.Md;  // one field's real lines
  R* C6 = (R*)d->C6;
  R* W = (R*)d->W6;
  const float tdense = time_ms<R>(d, [&]() {
    cudaError_t e;
    if ((N + 1) / 2 <= 56) {
      e = launch_curl_cheb<R>(g, N, d->Ucur, W, (const R*)d->cinvA, (const R*)d->cinvB, (const R*)d->cderA,
                              (const R*)d->cderB, (const R*)d->basey, 0.0, d->st);
    } else {
      e = launch_curl_base<R>(g, d->Ucur, C6, d->dUbase, d->dWbase, 0, 0.0, d->st);
      if (e == cudaSuccess)
        e = launch_cheb<R, R, R>(N, true, nl1, 6, C6, row, comp, W, row, comp, (const R*)d->cinvA,
                                 (const R*)d->cinvB, d->st);
    }
    if (e == cudaSuccess)
      e = launch_cheb<R, R, R>(N, false, nl1, 3, (const R*)d->F3, row, comp, C6, row, comp, (const R*)d->cfwdA,
                               (const R*)d->cfwdB, d->st);
    return e;
  });
  const float tfft = time_ms<R>(d, [&]() {
    cudaError_t e = launch_curl_base<R>(g, d->Ucur, C6, d->dUbase, d->dWbase, 0, 0.0, d->st);
    if (e == cudaSuccess)
      e = launch_dct<R>(N, true, g.Md, 6, (const cpx<R>*)C6, row / 2, comp / 2, (cpx<R>*)W, row / 2, comp / 2,
                        (const cpx<R>*)d->cdct, d->st);
    if (e == cudaSuccess)
      e = launch_dct<R>(N, false, g.Md, 3, (const cpx<R>*)d->F3, row / 2, comp / 2, (cpx<R>*)C6, row / 2,
                        comp / 2, (const cpx<R>*)d->cdct, d->st);
    return e;
  });
  d->ydct = tfft < 1e30f && tfft < tdense;
  CK(cudaStreamSynchronize(d->st));
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cheb[key] = d->ydct ? 1 : 0;
  return CFGPU_OK;
}

// Forward Chebyshev transform of the mixed path on the tensor cores or as compensated FP32 matrix products:
// mode 0 never, 1 timed on the DNS's own arrays (cached per grid shape), 2 wherever supported.
std::atomic<int> g_cheb_tc{1};
std::map<TuneKey, int> g_tune_tc;

int tune_cheb_tc(cfgpu_dns d) {
  d->ytc = false;
  const int mode = g_cheb_tc.load();
  if (mode == 0 || !d->ctc || d->ydct) return CFGPU_OK;
  if (mode == 2) {
    d->ytc = true;
    return CFGPU_OK;
  }
  const TuneKey key{d->g.Nx, d->g.Ny, d->g.Nz, d->g.NKz, 4, 101};  // one field's grid (see tune_cheb)
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_tc.find(key);
    if (it != g_tune_tc.end()) {
      d->ytc = it->second != 0;
      return CFGPU_OK;
    }
  }
  const int N = d->N;
  const size_t row = d->rowc(), comp = d->compc();
  float* out = (float*)d->C6;
  const int nl1 = 2 * d->g.Md;  // one field's real lines
  const float tm = time_ms<float>(d, [&]() {
    return launch_cheb<float, float, float>(N, false, nl1, 3, (const float*)d->F3, row, comp, out, row, comp,
                                            (const float*)d->cfwdA, (const float*)d->cfwdB, d->st);
  });
  const float tt = time_ms<float>(d, [&]() {
    return launch_cheb_tc(N, nl1, 3, (const float*)d->F3, row, comp, out, d->ctc, d->dtcerr, d->st);
  });
  d->ytc = tt < 1e30f && tt < tm;
  CK(cudaStreamSynchronize(d->st));
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_tc[key] = d->ytc ? 1 : 0;
  return CFGPU_OK;
}

int dns_create_impl(cfgpu_dns d, const cfgpu_grid* grid, const cfgpu_flags* flags, const double* Ub, const double* Wb,
                    const double* u0, int nb = 1) {
  d->fl = *flags;
  const cfgpu_flags& f = d->fl;
  const int Nx = grid->Nx, Ny = grid->Ny, Nz = grid->Nz;
  if (Nx < 4 || Nz < 4 || Nx % 2 || Nz % 2) return fail(CFGPU_EINVAL, "Nx and Nz must be even and >= 4");
  if (Ny < 5 || Ny % 2 == 0) return fail(CFGPU_EINVAL, "Ny must be odd and >= 5 (HelmholtzSolver asserts odd N)");
  if (Ny > 257) return fail(CFGPU_ENOTSUP, "Ny > 257 not supported by the Chebyshev transform kernels");
  if ((Ny + 1) / 2 > 56 && f.nonlinearity != CFGPU_Rotational)
    return fail(CFGPU_ENOTSUP, "Ny > 111 needs the rotational nonlinear form");
  if (!(grid->b > grid->a) || grid->Lx <= 0 || grid->Lz <= 0) return fail(CFGPU_EINVAL, "bad box");
  if (f.dt <= 0 || f.nu <= 0) return fail(CFGPU_EINVAL, "dt and nu must be positive");
  if (f.nonlinearity < CFGPU_Rotational || f.nonlinearity > CFGPU_LinearAboutProfile)
    return fail(CFGPU_EINVAL, "unknown nonlinearity");
  if (f.dealiasing == CFGPU_DealiasY || f.dealiasing == CFGPU_DealiasXYZ)
    return fail(CFGPU_ENOTSUP, "DealiasY is not implemented on the device path");
  const bool dxz = (f.dealiasing == CFGPU_DealiasXZ);
  GridDev& g = d->g;
  g.Nx = Nx;
  g.Ny = Ny;
  g.Nz = Nz;
  g.kxmax = Nx / 2;
  g.kzmax = Nz / 2;
  g.Kx = dxz ? Nx / 3 - 1 : Nx / 2 - 1;
  g.Kz = dxz ? Nz / 3 - 1 : Nz / 2 - 1;
  g.NKx = 2 * g.Kx + 1;
  g.NKz = g.Kz + 1;
  g.Md = g.NKx * g.NKz;
  g.Lx = grid->Lx;
  g.Lz = grid->Lz;
  g.a = grid->a;
  g.b = grid->b;
  g.kxs = g.kzs = nullptr;
  g.Mf = 0;
  d->N = Ny;
  d->nb = nb;
  d->gm = g;
  d->gp = g;
  d->alt[0] = d->alt[1] = (f.nonlinearity == CFGPU_Alternating_) ? 1 : 0;
  CK(cudaGetDevice(&d->device));
  CK(cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking));
  {
    // kernels may touch pageable host memory through the host page tables (no migration, no faults
    // to service): FlowField buffers are then read and written in place
    int ats = 0;
    if (cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, d->device) != cudaSuccess)
      ats = 0;
    d->direct = ats == 1 && g_host_access.load() != 0;
  }

  // base flow and constraint (NSE::createCFBaseFlow, nse.cpp:589-632; NSE::initCFConstraint, nse.cpp:634-671)
  const double a = g.a, b = g.b;
  BaseFlow bf;
  CKS(compute_base(f, Ub, Wb, Ny, a, b, bf));
  d->Ubase = bf.Ubase;
  d->Wbase = bf.Wbase;
  d->Ubaseyy = bf.Ubaseyy;
  d->Wbaseyy = bf.Wbaseyy;
  d->UbulkBase = bf.UbulkBase;
  d->WbulkBase = bf.WbulkBase;
  d->baseShear[0] = bf.baseShear[0];
  d->baseShear[1] = bf.baseShear[1];
  d->UbulkRef = bf.UbulkRef;
  d->WbulkRef = bf.WbulkRef;
  d->dPdxAct = bf.dPdxAct;
  d->dPdxRef = bf.dPdxRef;
  d->dPdzAct = bf.dPdzAct;
  d->dPdzRef = bf.dPdzRef;
  if (u0) {
    // getUbulk / getWbulk (diffops.cpp:3839-3867): mean over y of the (0,0) mode of u and w
    const size_t plane = 2 * (size_t)Nx * (Nz / 2 + 1), comp = plane * Ny;
    double su = u0[0], sw = u0[2 * comp];
    for (int n = 2; n < Ny; n += 2) {
      su -= u0[n * plane] / (double)(n * n - 1);
      sw -= u0[2 * comp + n * plane] / (double)(n * n - 1);
    }
    d->UbulkAct = bf.UbulkBase + su;
    d->WbulkAct = bf.WbulkBase + sw;
  }
  long long& B = d->bytes;
  CKS(dalloc(&d->dUbase, Ny, B));
  CKS(dalloc(&d->dWbase, Ny, B));
  CKS(dalloc(&d->dUbaseyy, Ny, B));
  CKS(dalloc(&d->dWbaseyy, Ny, B));
  CKS(dalloc(&d->ddPdx, 2 * (size_t)nb, B));
  CKS(dalloc(&d->dred, 2 * (size_t)nb, B));
  if (nb > 1) {
    // mode lists of the batched mode view and the plane view of the x/z passes
    std::vector<int> ml(2 * (size_t)nb * g.Md);
    for (int f = 0; f < nb; ++f)
      for (int m = 0; m < g.Md; ++m) {
        ml[(size_t)f * g.Md + m] = mode_kx(g, m);
        ml[(size_t)nb * g.Md + (size_t)f * g.Md + m] = mode_kz(g, m);
      }
    CKS(dalloc(&d->dmodes, ml.size(), B));
    CK(cudaMemcpyAsync(d->dmodes, ml.data(), ml.size() * sizeof(int), cudaMemcpyHostToDevice, d->st));
    d->gm.Md = nb * g.Md;
    d->gm.Mf = g.Md;
    d->gm.kxs = d->dmodes;
    d->gm.kzs = d->dmodes + (size_t)nb * g.Md;
    d->gp.Ny = nb * Ny;
  }
  {
    // FlowField::CFLfactor spacing (flowfield.cpp:4046-4052)
    std::vector<double> y(Ny), dy(Ny);
    for (int j = 0; j < Ny; ++j) y[j] = (b + a) / 2 + (b - a) / 2 * std::cos(j * M_PI / (Ny - 1));
    for (int j = 0; j < Ny; ++j) dy[j] = (j == 0 || j == Ny - 1) ? y[0] - y[1] : (y[j - 1] - y[j + 1]) / 2.0;
    CKS(dalloc(&d->dyc, Ny, B));
    CK(cudaMemcpyAsync(d->dyc, dy.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
  }
  CK(cudaMemcpyAsync(d->dUbase, d->Ubase.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
  CK(cudaMemcpyAsync(d->dWbase, d->Wbase.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
  CK(cudaMemcpyAsync(d->dUbaseyy, d->Ubaseyy.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
  CK(cudaMemcpyAsync(d->dWbaseyy, d->Wbaseyy.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
  {
    std::vector<double> init(2 * (size_t)nb);
    for (int f = 0; f < nb; ++f) {
      init[2 * f] = d->dPdxAct;
      init[2 * f + 1] = d->dPdzAct;
    }
    CK(cudaMemcpyAsync(d->ddPdx, init.data(), init.size() * sizeof(double), cudaMemcpyHostToDevice, d->st));
  }
  // Helmholtz B rows
  {
    std::vector<double> lo, di, up;
    make_helm_b(Ny, lo, di, up);
    CKS(dalloc(&d->hb_lo, Ny, B));
    CKS(dalloc(&d->hb_di, Ny, B));
    CKS(dalloc(&d->hb_up, Ny, B));
    CK(cudaMemcpyAsync(d->hb_lo, lo.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
    CK(cudaMemcpyAsync(d->hb_di, di.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
    CK(cudaMemcpyAsync(d->hb_up, up.data(), Ny * sizeof(double), cudaMemcpyHostToDevice, d->st));
  }
  // FFT plans, twiddles, Chebyshev matrices
  std::vector<std::complex<long double>> twx, twz;
  if (!make_fft_plan(Nx, d->px, twx) || !make_fft_plan(Nz, d->pz, twz))
    return fail(CFGPU_ENOTSUP, "Nx and Nz must factor into primes <= " + std::to_string(FFT_MAX_RADIX));
  ChebMats cm = make_cheb_mats(Ny);
  for (auto& v : cm.derA) v *= 2.0 / (b - a);
  for (auto& v : cm.derB) v *= 2.0 / (b - a);
  for (auto& v : cm.dfA) v *= 2.0 / (b - a);
  for (auto& v : cm.dfB) v *= 2.0 / (b - a);
  const std::vector<double>& basey = bf.basey;
  const bool fp64 = d->precision == CFGPU_FP64;
  const std::vector<double> circx = circle_table(Nx), circz = circle_table(Nz);
  if (fp64) {
    CKS(upload_tw<double>(twx, &d->twx, B, d->st));
    CKS(upload_tw<double>(twz, &d->twz, B, d->st));
    CKS(upload_as<double>(circx, &d->twxf, B, d->st));
    CKS(upload_as<double>(circz, &d->twzf, B, d->st));
    CKS(upload_as<double>(cm.invA, &d->cinvA, B, d->st));
    CKS(upload_as<double>(cm.invB, &d->cinvB, B, d->st));
    CKS(upload_as<double>(cm.fwdA, &d->cfwdA, B, d->st));
    CKS(upload_as<double>(cm.fwdB, &d->cfwdB, B, d->st));
    CKS(upload_as<double>(cm.derA, &d->cderA, B, d->st));
    CKS(upload_as<double>(cm.derB, &d->cderB, B, d->st));
    CKS(upload_as<double>(basey, &d->basey, B, d->st));
    CKS(upload_as<double>(cm.dfA, &d->cdfA, B, d->st));
    CKS(upload_as<double>(cm.dfB, &d->cdfB, B, d->st));
    if (dct_supported(Ny)) CKS(upload_as<double>(dct_table(Ny), &d->cdct, B, d->st));
  } else {
    // DITHER_V dithered versions of every FP32 constant table in one block (16-byte aligned tables)
    std::vector<std::vector<double>> tabs = {cm.invA, cm.invB, cm.fwdA, cm.fwdB, cm.derA, cm.derB, cm.dfA, cm.dfB};
    for (const auto* tw : {&twx, &twz}) {
      std::vector<double> t(2 * (tw->size() ? tw->size() : 1), 0.0);
      for (size_t i = 0; i < tw->size(); ++i) {
        t[2 * i] = (double)(*tw)[i].real();
        t[2 * i + 1] = (double)(*tw)[i].imag();
      }
      tabs.push_back(t);
    }
    {
      // d/dx by solved kx index, d/dz by kz, {1/(Nx Nz), Vsuck}
      std::vector<double> tx(g.NKx), tz(g.NKz), tm(4, 0.0);
      for (int ix = 0; ix < g.NKx; ++ix) {
        const int kx = ix <= g.Kx ? ix : ix - g.NKx;
        tx[ix] = 2.0 * M_PI * kx / g.Lx * (kx == g.kxmax ? 0.0 : 1.0);
      }
      for (int iz = 0; iz < g.NKz; ++iz) tz[iz] = 2.0 * M_PI * iz / g.Lz * (iz == g.kzmax ? 0.0 : 1.0);
      tm[0] = 1.0 / ((double)Nx * (double)Nz);
      tm[1] = f.Vsuck;
      tabs.push_back(tx);
      tabs.push_back(tz);
      tabs.push_back(tm);
    }
    tabs.push_back(circx);
    tabs.push_back(circz);
    tabs.push_back(dct_supported(Ny) ? dct_table(Ny) : std::vector<double>(2, 0.0));
    std::vector<size_t> off(tabs.size());
    size_t S = 0;
    for (size_t i = 0; i < tabs.size(); ++i) {
      off[i] = S;
      S += (tabs[i].size() + 3) & ~(size_t)3;
    }
    CKS(upload_dithered(tabs, off, S, &d->cblock, B, d->st));
    float* c0 = (float*)d->cblock;
    void** dst[10] = {&d->cinvA, &d->cinvB, &d->cfwdA, &d->cfwdB, &d->cderA, &d->cderB, &d->cdfA, &d->cdfB,
                      &d->twx, &d->twz};
    for (size_t i = 0; i < 10; ++i) *dst[i] = c0 + off[i];
    d->kdx = c0 + off[10];
    d->kdz = c0 + off[11];
    d->kmisc = c0 + off[12];
    d->twxf = c0 + off[13];
    d->twzf = c0 + off[14];
    if (dct_supported(Ny)) d->cdct = c0 + off[15];
    if (cheb_tc_supported(Ny)) {
      // full forward matrix F[n][j] = w_j cos(pi n j / (N-1)) c_n / (N-1) (chebyfft), four BF16 splits
      std::vector<double> Fm((size_t)Ny * Ny);
      for (int n = 0; n < Ny; ++n)
        for (int j = 0; j < Ny; ++j) {
          const long double cn = (n == 0 || n == Ny - 1) ? 0.5L : 1.0L;
          const long double w = (j == 0 || j == Ny - 1) ? 1.0L : 2.0L;
          Fm[(size_t)n * Ny + j] = (double)(w * cospi_ratio((long long)n * j, Ny - 1) * cn / (Ny - 1));
        }
      const std::vector<uint16_t> tcm = cheb_tc_matrix(Fm, Ny);
      CKS(dalloc(&d->ctc, tcm.size() * sizeof(uint16_t), B));
      CK(cudaMemcpyAsync(d->ctc, tcm.data(), tcm.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, d->st));
      CKS(dalloc(&d->dtcerr, 1, B));
      CK(cudaMemsetAsync(d->dtcerr, 0, sizeof(int), d->st));
    }
    d->cS = (long long)(S * sizeof(float));
    CKS(upload_dithered({basey}, {0}, basey.size(), &d->basey, B, d->st));
  }
  CKS(dalloc(&d->dver, nb, B));
  CK(cudaMemsetAsync(d->dver, 0, nb * sizeof(int), d->st));
  // state and work arrays
  const size_t cd = d->compc();
  const size_t rs = d->rsz();
  CKS(dalloc(&d->Ucur, 3 * cd, B));
  CKS(dalloc(&d->Qcur, cd, B));
  CK(cudaMemsetAsync(d->Ucur, 0, 3 * cd * sizeof(double), d->st));
  CK(cudaMemsetAsync(d->Qcur, 0, cd * sizeof(double), d->st));
  unsigned char* tmp;
  CKS(dalloc(&tmp, 6 * cd * rs, B));
  d->C6 = tmp;
  const bool rot = (f.nonlinearity == CFGPU_Rotational);
  const int nin = rot ? 6 : 12, nout = rot ? 3 : 9;  // y-physical components in / physical outputs
  CKS(dalloc(&tmp, nin * cd * rs, B));
  d->W6 = tmp;
  const size_t plane = (size_t)Nx * g.NKz * 2;  // reals per plane per component
  CKS(dalloc(&tmp, nin * plane * Ny * nb * rs, B));
  d->X6 = tmp;
  CKS(dalloc(&tmp, nout * plane * Ny * nb * rs, B));
  d->Z3 = tmp;
  CKS(dalloc(&tmp, nout * cd * rs, B));
  d->F3 = tmp;
  CKS(dalloc(&d->scratch, 8 * cd, B));
  if (f.nonlinearity == CFGPU_LinearAboutProfile) {
    CKS(dalloc(&tmp, 4 * (size_t)Ny * nb * rs, B));
    d->zbasey = tmp;
    CK(cudaMemsetAsync(d->zbasey, 0, 4 * (size_t)Ny * nb * rs, d->st));
  }
  d->RP = fp64 ? 8 : 16;
  auto zbytes = [&](int form, int rp) {
    return fp64 ? zphys_smem_bytes<double>(g, form, rp) : zphys_smem_bytes<float>(g, form, rp);
  };
  const int zform = rot ? NL_ROTATIONAL : NL_SKEW;  // skew needs the most shared memory of the gradient forms
  while (d->RP > 2 && zbytes(zform, d->RP) > 200 * 1024) d->RP -= 2;
  if ((fp64 ? xfft_smem_bytes<double>(g) : xfft_smem_bytes<float>(g)) > 227 * 1024 || zbytes(zform, d->RP) > 227 * 1024)
    return fail(CFGPU_ENOTSUP, "grid too large for the shared-memory FFT passes");
  if (cheb_smem_bytes(Ny, rs) > 200 * 1024) return fail(CFGPU_ENOTSUP, "Ny too large for the Chebyshev kernel");
  d->autotune = g_autotune.load() != 0;
  if (d->autotune) {
    const int tform = f.nonlinearity == CFGPU_LinearAboutProfile
                          ? -1
                          : (rot ? NL_ROTATIONAL : (f.nonlinearity == CFGPU_SkewSymmetric ? NL_SKEW : NL_CONVECTION));
    CKS(fp64 ? autotune<double>(d, tform, nin, nout) : autotune<float>(d, tform, nin, nout));
  }

  // fused x/z pass for the rotational form (thread-block clusters over a y-plane)
  d->xzf = false;
  if (rot && g_fused_xz.load() != 0 && xz_fused_supported(d->gp)) CKS(fp64 ? tune_xz<double>(d) : tune_xz<float>(d));
  // Chebyshev transforms of the rotational form: dense or through the FFT
  if (rot) CKS(fp64 ? tune_cheb<double>(d) : tune_cheb<float>(d));
  if (!fp64 && (rot || f.nonlinearity == CFGPU_Convection)) CKS(tune_cheb_tc(d));

  // schemes (DNS::DNS, dns.cpp:22-39)
  CKS(setup_scheme(d->main, f.timestepping, f.dt));
  d->main.t = f.t0;
  d->has_init = false;
  if (!d->main.full && f.initstepping != f.timestepping) {
    CKS(setup_scheme(d->init, f.initstepping, f.dt));
    d->init.t = f.t0;
    // a multistep start-up scheme must start itself (DNS::DNS warns that it "needs initialization itself"
    // otherwise, dns.cpp:34-37): order 1, SBDF1 or CNFE1
    if (d->init.family == 0 && d->init.order > 1)
      return fail(CFGPU_ENOTSUP, "a multistep start-up scheme must be of order 1 (SBDF1 or CNFE1)");
    d->has_init = true;
  }
  auto alloc_scheme = [&](Scheme& s, int which) -> int {
    if (s.family == 0 && which == 1) {
      // order-1 multistep start-up: its nonlinear term only (u_n is the current field)
      CKS(dalloc(&tmp, 3 * cd * rs, B));
      d->fj[1] = tmp;
      CK(cudaMemsetAsync(d->fj[1], 0, 3 * cd * rs, d->st));
    } else if (s.family == 0) {
      for (int j = 0; j < s.order; ++j) {
        CKS(dalloc(&d->Uh[j], 3 * cd, B));
        CKS(dalloc(&d->Qh[j], cd, B));
        CKS(dalloc(&tmp, 3 * cd * rs, B));
        d->Nh[j] = tmp;
        CK(cudaMemsetAsync(d->Uh[j], 0, 3 * cd * sizeof(double), d->st));
        CK(cudaMemsetAsync(d->Qh[j], 0, cd * sizeof(double), d->st));
        CK(cudaMemsetAsync(d->Nh[j], 0, 3 * cd * rs, d->st));
      }
    } else if (s.family == 1) {
      CKS(dalloc(&tmp, 3 * cd * rs, B));
      d->fj[which] = tmp;
      CKS(dalloc(&tmp, 3 * cd * rs, B));
      d->fj1[which] = tmp;
      CK(cudaMemsetAsync(d->fj[which], 0, 3 * cd * rs, d->st));
      CK(cudaMemsetAsync(d->fj1[which], 0, 3 * cd * rs, d->st));
    } else {
      CKS(dalloc(&tmp, 3 * cd * rs, B));
      d->rkQ[which] = tmp;
      CK(cudaMemsetAsync(d->rkQ[which], 0, 3 * cd * rs, d->st));
      if (!d->rkN) {
        CKS(dalloc(&tmp, 3 * cd * rs, B));
        d->rkN = tmp;
      }
    }
    return CFGPU_OK;
  };
  CKS(alloc_scheme(d->main, 0));
  if (d->has_init) CKS(alloc_scheme(d->init, 1));
  CKS(build_tables(d, d->main));
  if (d->has_init) CKS(build_tables(d, d->init));
  d->stage_elems = 4 * cd;  // pinned host staging, allocated on first host transfer (ensure_stage)
  CKS(pinned_alloc(&d->cfl_host, (size_t)nb * sizeof(unsigned long long)));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

void dns_free(cfgpu_dns d) {
  if (!d) return;
  if (d->st) cudaStreamSynchronize(d->st);
  auto F = [](void* p) { dfree(p); };
  if (d->cblock) {
    // the FP32 constant tables live inside one block (all versions): freed once, below
    d->twx = d->twz = d->cinvA = d->cinvB = d->cfwdA = d->cfwdB = d->cderA = d->cderB = d->cdfA = d->cdfB = nullptr;
    d->twxf = d->twzf = d->cdct = nullptr;
  }
  F(d->twxf); F(d->twzf); F(d->cdct); F(d->ctc); F(d->dtcerr);
  F(d->dUbase); F(d->dWbase); F(d->dUbaseyy); F(d->dWbaseyy); F(d->ddPdx);
  F(d->hb_lo); F(d->hb_di); F(d->hb_up);
  F(d->twx); F(d->twz); F(d->cinvA); F(d->cinvB); F(d->cfwdA); F(d->cfwdB);
  F(d->cderA); F(d->cderB); F(d->basey); F(d->cdfA); F(d->cdfB); F(d->dyc); F(d->dred); F(d->dmodes);
  F(d->dslot); F(d->dbaseS); F(d->baseyS); F(d->zbasey); F(d->cblock); F(d->dver);
  F(d->Ucur); F(d->Qcur);
  for (int j = 0; j < 4; ++j) { F(d->Uh[j]); F(d->Qh[j]); F(d->Nh[j]); }
  for (int w = 0; w < 2; ++w) { F(d->fj[w]); F(d->fj1[w]); F(d->rkQ[w]); }
  F(d->rkN);
  F(d->C6); F(d->W6); F(d->X6); F(d->Z3); F(d->F3); F(d->scratch);
  for (Scheme* s : {&d->main, &d->init})
    for (auto& t : s->tau) { F(t.f); F(t.s); }
  pinned_free(d->stage);
  pinned_free(d->cfl_host);
  pinned_free(d->stage1);
  for (auto& e : d->ev_pool) cudaEventDestroy(e);
  for (auto& u : d->ev_used) {
    cudaEventDestroy(u.second.first);
    cudaEventDestroy(u.second.second);
  }
  drop_graphs(d);
  if (d->st) cudaStreamDestroy(d->st);
  delete d;
}

}  // namespace

namespace {
// DNSAlgorithm::CFL of every field of the batch: the pass is enqueued on the DNS's stream and its CFL keys
// copied to pinned host memory (cfl_enqueue); cfl_finish converts them once the stream has reached that point.
template <typename R>
int cfl_enqueue(cfgpu_dns d) {
  const GridDev& g = d->gm;
  R* W = (R*)d->W6;
  if ((d->N + 1) / 2 > 56 || d->ydct) {
    // tall grids, or transforms through the FFT: u + base flow as Chebyshev coefficients (the curl pass's
    // first three components), then the inverse transform to the Gauss-Lobatto points
    const size_t row = d->rowc(), comp = d->compc(), nN = (size_t)d->nb * d->N;
    CK(launch_curl_base<R>(g, d->Ucur, (R*)d->C6, d->hetero ? d->dbaseS : d->dUbase,
                           d->hetero ? d->dbaseS + nN : d->dWbase, d->hetero ? d->N : 0, 0.0, d->st));
    if (d->ydct)
      CK(launch_dct<R>(d->N, true, g.Md, 3, (const cpx<R>*)d->C6, row / 2, comp / 2, (cpx<R>*)W, row / 2, comp / 2,
                       (const cpx<R>*)d->cdct, d->st));
    else
      CK((launch_cheb<R, R, R>(d->N, true, (int)row, 3, (const R*)d->C6, row, comp, W, row, comp,
                               (const R*)d->cinvA, (const R*)d->cinvB, d->st)));
    d->launches += 2;
  } else {
    CK(launch_grad_cheb<R>(g, d->N, false, d->Ucur, W, (const R*)d->cinvA, (const R*)d->cinvB, (const R*)d->cderA,
                           (const R*)d->cderB, (const R*)(d->hetero ? d->baseyS : d->basey), 0.0, d->st,
                           d->hetero ? 4 * d->N : 0));
  }
  CK(launch_xinv<R>(d->gp, d->px, (const cpx<R>*)d->twx, (const cpx<R>*)W, (cpx<R>*)d->X6, 3, d->st, d->xcols));
  CK(cudaMemsetAsync(d->dred, 0, d->nb * sizeof(unsigned long long), d->st));
  CK(launch_zcfl<R>(d->gp, d->pz, (const cpx<R>*)d->twz, d->RP, (const cpx<R>*)d->X6, d->dyc, g.Lx / g.Nx,
                    g.Lz / g.Nz, d->nb, d->dred, d->st));
  d->launches += 3;
  CK(cudaMemcpyAsync(d->cfl_host, d->dred, d->nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost, d->st));
  return CFGPU_OK;
}

void cfl_finish(cfgpu_dns d, double* cfl) {
  const bool dxz = d->fl.dealiasing == CFGPU_DealiasXZ || d->fl.dealiasing == CFGPU_DealiasXYZ;
  for (int f = 0; f < d->nb; ++f) {
    const double dt = d->hetero ? d->sfl[f].dt : d->fl.dt;
    cfl[f] = cfl_key_to_double(d->cfl_host[f]) * (dxz ? 2.0 * M_PI / 3.0 * dt : M_PI * dt);
  }
}

template <typename R>
int cfl_impl(cfgpu_dns d, double* cfl) {
  CKS(cfl_enqueue<R>(d));
  CK(cudaStreamSynchronize(d->st));
  cfl_finish(d, cfl);
  return CFGPU_OK;
}

int l2norm_impl(cfgpu_dns d, int field, double* l2) {
  double* out = reinterpret_cast<double*>(d->dred) + d->nb;
  CK(cudaMemsetAsync(out, 0, d->nb * sizeof(double), d->st));
  CK(launch_l2norm2(d->gm, d->N, field == 0 ? 3 : 1, field == 0 ? d->Ucur : d->Qcur, out, d->st));
  d->launches++;
  std::vector<double> s(d->nb);
  CK(cudaMemcpyAsync(s.data(), out, d->nb * sizeof(double), cudaMemcpyDeviceToHost, d->st));
  CK(cudaStreamSynchronize(d->st));
  for (int f = 0; f < d->nb; ++f) l2[f] = std::sqrt(s[f]);
  return CFGPU_OK;
}
}  // namespace

#include "timestep.h"

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// Runtime hooks used by the request server (server.cu); not part of the C ABI.
namespace cfgpu_rt {
// CFL pass enqueued on the DNS's stream (results readable with cfl_collect once the stream passed it).
int cfl_async(cfgpu_dns d) { return d->precision == CFGPU_FP64 ? cfl_enqueue<double>(d) : cfl_enqueue<float>(d); }
void cfl_collect(cfgpu_dns d, double* out) { cfl_finish(d, out); }

// Recreate the DNS's stream with a scheduling priority (cudaDeviceGetStreamPriorityRange).
int set_priority(cfgpu_dns d, int prio) {
  CK(cudaStreamSynchronize(d->st));
  cudaStream_t ns = nullptr;
  CK(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
  cudaStreamDestroy(d->st);
  d->st = ns;
  return CFGPU_OK;
}

int advance_async(cfgpu_dns d, int nsteps) { return dns_advance_device(d, nsteps); }
cudaStream_t stream(cfgpu_dns d) { return d->st; }
long long bytes(cfgpu_dns d) { return d->bytes; }
int nfields(cfgpu_dns d) { return d->nb; }

// Steps DNS::advance takes with the start-up scheme before the main scheme runs alone.
int startup_steps(cfgpu_dns d) {
  if (d->main.full) return 0;
  return d->main.family == 0 ? d->main.countdown : 1;
}

// Copy velocity and pressure of field `slot` of d into the one-field DNS dst (its only field).
int store_slot(cfgpu_dns d, int slot, cfgpu_dns dst) {
  if (dst->nb != 1 || d->g.Md != dst->g.Md || d->N != dst->N) return fail(CFGPU_EINVAL, "store_slot: shapes differ");
  const size_t w = 2 * (size_t)d->g.Md, pitch = w * d->nb, N = d->N;
  CK(cudaStreamSynchronize(dst->st));
  CK(cudaMemcpy2DAsync(dst->Ucur, w * 8, d->Ucur + slot * w, pitch * 8, w * 8, 3 * N, cudaMemcpyDeviceToDevice,
                       d->st));
  CK(cudaMemcpy2DAsync(dst->Qcur, w * 8, d->Qcur + slot * w, pitch * 8, w * 8, N, cudaMemcpyDeviceToDevice, d->st));
  CK(cudaMemcpyAsync(dst->dver, d->dver + slot, sizeof(int), cudaMemcpyDeviceToDevice, d->st));  // constant version
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

// Field `slot` starts over as a fresh DNS does: version 0 of the dithered FP32 constants.
int reset_version(cfgpu_dns d, int slot) {
  CK(cudaMemsetAsync(d->dver + slot, 0, sizeof(int), d->st));
  return CFGPU_OK;
}

// Back to the state of a fresh DNS (time t0, start-up steps pending) without rebuilding tables.
int restart(cfgpu_dns d) {
  for (Scheme* s : {&d->main, &d->init}) {
    if (s == &d->init && !d->has_init) continue;
    std::vector<TauTable> keep = s->tau;
    CKS(setup_scheme(*s, s->method, d->fl.dt));
    s->tau = keep;
    s->t = d->fl.t0;
  }
  d->alt[0] = d->alt[1] = (d->fl.nonlinearity == CFGPU_Alternating_) ? 1 : 0;
  for (int j = 0; j < 4; ++j) d->perm[j] = j;
  const size_t cd = d->compc(), rs = d->rsz();
  for (int w = 0; w < 2; ++w)
    if (d->rkQ[w]) CK(cudaMemsetAsync(d->rkQ[w], 0, 3 * cd * rs, d->st));  // 0 * stale NaN would stay NaN
  return CFGPU_OK;
}

// Device bytes a DNS of nb fields with these flags allocates (the allocations of dns_create_impl).
long long estimate_bytes(const cfgpu_grid& grid, const cfgpu_flags& f, int nb, int precision) {
  const bool dxz = f.dealiasing == CFGPU_DealiasXZ;
  const long long Kx = dxz ? grid.Nx / 3 - 1 : grid.Nx / 2 - 1, Kz = dxz ? grid.Nz / 3 - 1 : grid.Nz / 2 - 1;
  const long long Md = (2 * Kx + 1) * (Kz + 1), N = grid.Ny;
  const long long cd = 2 * Md * N * nb, rs = precision == CFGPU_FP64 ? 8 : 4;
  const bool rot = f.nonlinearity == CFGPU_Rotational;
  const long long nin = rot ? 6 : 12, nout = rot ? 3 : 9, plane = 2LL * grid.Nx * (Kz + 1) * N * nb;
  long long b = 4 * cd * 8 + 6 * cd * rs + nin * cd * rs + nin * plane * rs + nout * plane * rs + nout * cd * rs +
                8 * cd * 8;
  Scheme m{}, i{};
  if (setup_scheme(m, f.timestepping, f.dt) != CFGPU_OK) return -1;
  int ntab = (int)m.lambda_t.size();
  auto hist = [&](const Scheme& s) -> long long {
    if (s.family == 0) return s.order * (4 * cd * 8 + 3 * cd * rs);
    if (s.family == 1) return 6 * cd * rs;
    return 6 * cd * rs;
  };
  b += hist(m);
  if (!m.full && f.initstepping != f.timestepping && setup_scheme(i, f.initstepping, f.dt) == CFGPU_OK) {
    b += hist(i);
    ntab += (int)i.lambda_t.size();
  }
  b += ntab * (TF_NFIELDS * N * Md * nb + TS_NSCALARS * Md * nb) * 8;
  return b + (1 << 20);
}
}  // namespace cfgpu_rt

namespace {
// Upload the per-field parameter arrays of a heterogeneous batch from d->sfl.
template <typename R>
int upload_slot(cfgpu_dns d, int f, const BaseFlow& B) {
  const size_t N = d->N, nN = (size_t)d->nb * N;
  const SlotParams sp = slot_params(d->sfl[f], B);
  CK(cudaMemcpyAsync(d->dslot + f, &sp, sizeof(sp), cudaMemcpyHostToDevice, d->st));
  const std::vector<double>* arrs[4] = {&B.Ubase, &B.Wbase, &B.Ubaseyy, &B.Wbaseyy};
  for (int k = 0; k < 4; ++k)
    CK(cudaMemcpyAsync(d->dbaseS + k * nN + f * N, arrs[k]->data(), N * sizeof(double), cudaMemcpyHostToDevice,
                       d->st));
  const int nver = sizeof(R) == sizeof(double) ? 1 : DITHER_V;
  std::vector<R> by((size_t)nver * 4 * N);
  for (int v = 0; v < nver; ++v)
    for (size_t e = 0; e < 4 * N; ++e)
      by[v * 4 * N + e] = sizeof(R) == sizeof(double) ? (R)B.basey[e] : (R)dither_round_host(B.basey[e], v);
  for (int v = 0; v < nver; ++v)
    CK(cudaMemcpyAsync((R*)d->baseyS + (size_t)v * nN * 4 + f * 4 * N, by.data() + (size_t)v * 4 * N,
                       4 * N * sizeof(R), cudaMemcpyHostToDevice, d->st));
  const double init[2] = {B.dPdxAct, B.dPdzAct};
  CK(cudaMemcpyAsync(d->ddPdx + 2 * f, init, sizeof(init), cudaMemcpyHostToDevice, d->st));
  CK(cudaStreamSynchronize(d->st));  // host sources are locals
  return CFGPU_OK;
}

int ensure_hetero(cfgpu_dns d) {
  if (d->hetero) return CFGPU_OK;
  if (d->has_init && d->init.family == 0)
    return fail(CFGPU_ENOTSUP, "per-field parameters with a multistep start-up scheme");
  const size_t N = d->N, nb = d->nb;
  CKS(dalloc(&d->dslot, nb, d->bytes));
  CKS(dalloc(&d->dbaseS, 4 * nb * N, d->bytes));
  unsigned char* tmp;
  const size_t nver = d->precision == CFGPU_FP64 ? 1 : DITHER_V;  // dithered versions (mixed precision)
  CKS(dalloc(&tmp, nver * 4 * nb * N * d->rsz(), d->bytes));
  d->baseyS = tmp;
  d->sfl.assign(nb, d->fl);
  drop_graphs(d);  // the solve and nonlinear kernels switch to per-field parameter arrays
  BaseFlow B;
  CKS(compute_base(d->fl, d->fl.baseflow == CFGPU_ArbitraryBase ? d->Ubase.data() : nullptr,
                   d->fl.baseflow == CFGPU_ArbitraryBase ? d->Wbase.data() : nullptr, d->N, d->g.a, d->g.b, B));
  d->hetero = true;
  for (int f = 0; f < d->nb; ++f)
    CKS(d->precision == CFGPU_FP64 ? upload_slot<double>(d, f, B) : upload_slot<float>(d, f, B));
  return CFGPU_OK;
}
}  // namespace

extern "C" {

const char* cfgpu_version(void) { return "cfgpu 0.1 (sm_103a)"; }

cfgpu_status cfgpu_dither_versions(double x, float* versions) {
  static_assert(DITHER_V == CFGPU_DITHER_VERSIONS, "version count of the C ABI");
  if (!versions) return fail(CFGPU_EINVAL, "null argument");
  for (int k = 0; k < DITHER_V; ++k) versions[k] = dither_round_host(x, k);
  return CFGPU_OK;
}

cfgpu_status cfgpu_measure_fp64(double* tflops, double* cycles_per_fma) {
  if (!tflops || !cycles_per_fma) return fail(CFGPU_EINVAL, "null argument");
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (measure_fp64(sms, tflops, cycles_per_fma) != 0) return fail(CFGPU_ECUDA, "FP64 microbenchmark failed");
  return CFGPU_OK;
}
const char* cfgpu_last_error(void) { return g_err.c_str(); }

cfgpu_status cfgpu_flags_default(cfgpu_flags* f) {
  if (!f) return fail(CFGPU_EINVAL, "null flags");
  memset(f, 0, sizeof(*f));
  f->nu = 0.0025;
  f->dt = 0.03125;
  f->baseflow = CFGPU_LaminarBase;
  f->constraint = CFGPU_PressureGradient;
  f->timestepping = CFGPU_SBDF3;
  f->initstepping = CFGPU_SMRK2;
  f->nonlinearity = CFGPU_Rotational;
  f->dealiasing = CFGPU_DealiasXZ;
  f->taucorrection = 1;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_create(const cfgpu_grid* grid, const cfgpu_flags* flags, const double* Ubase,
                              const double* Wbase, const double* u, int precision, cfgpu_dns* out) {
  if (!grid || !flags || !out) return fail(CFGPU_EINVAL, "null argument");
  if (precision != CFGPU_FP64 && precision != CFGPU_MIXED) return fail(CFGPU_EINVAL, "bad precision");
  if ((Ubase == nullptr) != (Wbase == nullptr)) return fail(CFGPU_EINVAL, "Ubase and Wbase must both be given");
  *out = nullptr;
  cfgpu_dns d = new cfgpu_dns_s();
  d->precision = precision;
  int s = dns_create_impl(d, grid, flags, Ubase, Wbase, u);
  if (s != CFGPU_OK) {
    std::string keep = g_err;
    dns_free(d);
    g_err = keep;
    return s;
  }
  *out = d;
  return CFGPU_OK;
}

cfgpu_status cfgpu_ensemble_create(const cfgpu_grid* grid, const cfgpu_flags* flags, int nfields, int precision,
                                   cfgpu_dns* out) {
  if (!grid || !flags || !out || nfields < 1) return fail(CFGPU_EINVAL, "bad argument");
  if (precision != CFGPU_FP64 && precision != CFGPU_MIXED) return fail(CFGPU_EINVAL, "bad precision");
  *out = nullptr;
  cfgpu_dns d = new cfgpu_dns_s();
  d->precision = precision;
  int s = dns_create_impl(d, grid, flags, nullptr, nullptr, nullptr, nfields);
  if (s != CFGPU_OK) {
    std::string keep = g_err;
    dns_free(d);
    g_err = keep;
    return s;
  }
  *out = d;
  return CFGPU_OK;
}


cfgpu_status cfgpu_ensemble_set_params(cfgpu_dns d, int slot, const cfgpu_flags* f, const double* Ubase,
                                       const double* Wbase) {
  if (!d || !f || slot < 0 || slot >= d->nb) return fail(CFGPU_EINVAL, "bad argument");
  if ((Ubase == nullptr) != (Wbase == nullptr)) return fail(CFGPU_EINVAL, "Ubase and Wbase must both be given");
  const cfgpu_flags& e = d->fl;
  if (f->timestepping != e.timestepping || f->initstepping != e.initstepping ||
      f->nonlinearity != e.nonlinearity || f->dealiasing != e.dealiasing || f->taucorrection != e.taucorrection ||
      f->Vsuck != e.Vsuck)
    return fail(CFGPU_EINVAL,
                "per-field flags may change nu, dt, base flow, walls and constraint only (schemes, nonlinearity, "
                "dealiasing, taucorrection and Vsuck are shared)");
  if (f->nu <= 0 || f->dt <= 0) return fail(CFGPU_EINVAL, "nu and dt must be positive");
  if ((d->N + 1) / 2 > 56) return fail(CFGPU_ENOTSUP, "per-field parameters need Ny <= 111");
  CKS(ensure_hetero(d));
  BaseFlow B;
  CKS(compute_base(*f, Ubase, Wbase, d->N, d->g.a, d->g.b, B));
  d->sfl[slot] = *f;
  CKS(d->precision == CFGPU_FP64 ? upload_slot<double>(d, slot, B) : upload_slot<float>(d, slot, B));
  CKS(build_slot_tables(d, slot));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_ensemble_load_slot(cfgpu_dns d, int slot, cfgpu_dns src) {
  if (!d || !src || slot < 0 || slot >= d->nb || src->nb != 1) return fail(CFGPU_EINVAL, "bad argument");
  const GridDev &a = d->g, &b = src->g;
  if (a.Nx != b.Nx || a.Ny != b.Ny || a.Nz != b.Nz || a.Md != b.Md || a.Lx != b.Lx || a.Lz != b.Lz ||
      a.a != b.a || a.b != b.b || d->precision != src->precision || d->device != src->device)
    return fail(CFGPU_EINVAL, "source DNS has another grid, precision or device");
  const double dt_slot = d->hetero ? d->sfl[slot].dt : d->fl.dt, dt_src = src->hetero ? src->sfl[0].dt : src->fl.dt;
  if (d->fl.timestepping != src->fl.timestepping || dt_slot != dt_src ||
      d->fl.nonlinearity != src->fl.nonlinearity || d->alt[0] != src->alt[0])
    return fail(CFGPU_EINVAL, "source DNS has another scheme, dt or nonlinearity state");
  if (!src->main.full) return fail(CFGPU_EINVAL, "the source DNS must be past its start-up steps");
  if (!d->main.full) {
    // the ensemble's fields arrive through this call, already started: its scheme runs main steps from now on
    d->main.countdown = 0;
    d->main.full = true;
  }
  CK(cudaStreamSynchronize(src->st));
  const size_t w = 2 * (size_t)a.Md, pitch = w * d->nb, N = d->N;
  auto copy = [&](void* dst, const void* srcp, size_t esz, size_t rows) -> int {
    CK(cudaMemcpy2DAsync((unsigned char*)dst + slot * w * esz, pitch * esz, srcp, w * esz, w * esz, rows,
                         cudaMemcpyDeviceToDevice, d->st));
    return CFGPU_OK;
  };
  const size_t rs = d->rsz();
  CKS(copy(d->Ucur, src->Ucur, 8, 3 * N));
  CKS(copy(d->Qcur, src->Qcur, 8, N));
  const Scheme& m = d->main;
  if (m.family == 0) {
    for (int j = 1; j < m.order; ++j) {
      CKS(copy(d->Uh[d->perm[j]], src->Uh[src->perm[j]], 8, 3 * N));
      CKS(copy(d->Qh[d->perm[j]], src->Qh[src->perm[j]], 8, N));
      CKS(copy(d->Nh[d->perm[j]], src->Nh[src->perm[j]], rs, 3 * N));
    }
  } else if (m.family == 1) {
    CKS(copy(d->fj[0], src->fj[0], rs, 3 * N));
    CKS(copy(d->fj1[0], src->fj1[0], rs, 3 * N));
  } else {
    CKS(copy(d->rkQ[0], src->rkQ[0], rs, 3 * N));
  }
  CK(cudaMemcpyAsync(d->ddPdx + 2 * slot, src->ddPdx, 2 * sizeof(double), cudaMemcpyDeviceToDevice, d->st));
  CK(cudaMemcpyAsync(d->dver + slot, src->dver, sizeof(int), cudaMemcpyDeviceToDevice, d->st));  // constant version
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_ensemble_size(cfgpu_dns d, int* nfields) {
  if (!d || !nfields) return fail(CFGPU_EINVAL, "bad argument");
  *nfields = d->nb;
  return CFGPU_OK;
}

cfgpu_status cfgpu_ensemble_set_field(cfgpu_dns d, int slot, const double* u, const double* q) {
  if (!d || slot < 0 || slot >= d->nb) return fail(CFGPU_EINVAL, "bad argument");
  return set_slot(d, slot, u, q);
}

cfgpu_status cfgpu_ensemble_get_field(cfgpu_dns d, int slot, double* u, double* q) {
  if (!d || slot < 0 || slot >= d->nb) return fail(CFGPU_EINVAL, "bad argument");
  return get_slot(d, slot, u, q);
}

cfgpu_status cfgpu_ensemble_cfl(cfgpu_dns d, double* cfl) {
  if (!d || !cfl) return fail(CFGPU_EINVAL, "bad argument");
  return d->precision == CFGPU_FP64 ? cfl_impl<double>(d, cfl) : cfl_impl<float>(d, cfl);
}

cfgpu_status cfgpu_ensemble_l2norm(cfgpu_dns d, int field, double* l2) {
  if (!d || !l2 || (field != 0 && field != 1)) return fail(CFGPU_EINVAL, "bad argument");
  return l2norm_impl(d, field, l2);
}

cfgpu_status cfgpu_ensemble_dPdx(cfgpu_dns d, double* dPdx) {
  if (!d || !dPdx) return fail(CFGPU_EINVAL, "bad argument");
  std::vector<double> v(2 * (size_t)d->nb);
  CK(cudaMemcpyAsync(v.data(), d->ddPdx, v.size() * sizeof(double), cudaMemcpyDeviceToHost, d->st));
  CK(cudaStreamSynchronize(d->st));
  for (int f = 0; f < d->nb; ++f) dPdx[f] = v[2 * f];
  return CFGPU_OK;
}

}  // extern "C"

// A field on the GPU in the solved-mode layout of its grid (2/3-dealiased modes): Nd components, complex
// [c][ny][m]; the C ABI's FlowField handle.
struct cfgpu_field_s {
  cfgpu_dns_s g;  // mode set, staging and stream only (no DNS is built)
  int Nd = 3;
  double* data = nullptr;
  long long bytes = 0;
};

namespace {
int f2v_grid(const cfgpu_grid* grid, cfgpu_dns_s& tmp);

int field_transfer(cfgpu_field f, const double* host_in, double* host_out) {
  cfgpu_dns_s& t = f->g;
  const size_t n = (size_t)f->Nd * t.compc();
  if (t.direct) {
    if (host_in) CK(launch_host_modes(t.g, true, f->Nd, 1, 0, 1, host_in, f->data, t.st));
    if (host_out) CK(launch_host_modes(t.g, false, f->Nd, 1, 0, 1, f->data, host_out, t.st));
    CK(cudaStreamSynchronize(t.st));
    return CFGPU_OK;
  }
  std::vector<double> h(n);
  if (host_in) {
    gather_modes(&t, host_in, f->Nd, h.data());
    CK(cudaMemcpyAsync(f->data, h.data(), n * sizeof(double), cudaMemcpyHostToDevice, t.st));
    CK(cudaStreamSynchronize(t.st));
  }
  if (host_out) {
    CK(cudaMemcpyAsync(h.data(), f->data, n * sizeof(double), cudaMemcpyDeviceToHost, t.st));
    CK(cudaStreamSynchronize(t.st));
    scatter_modes(&t, h.data(), f->Nd, host_out);
  }
  return CFGPU_OK;
}

// The field's grid and mode set must be the DNS's (one field of it).
bool field_matches(cfgpu_dns d, cfgpu_field f, int Nd) {
  const GridDev &a = d->g, &b = f->g.g;
  return f->Nd == Nd && a.Nx == b.Nx && a.Ny == b.Ny && a.Nz == b.Nz && a.Md == b.Md && a.Lx == b.Lx &&
         a.Lz == b.Lz && a.a == b.a && a.b == b.b;
}
}  // namespace

extern "C" {

cfgpu_status cfgpu_field_create(const cfgpu_grid* grid, int Nd, cfgpu_field* out) {
  if (!out || (Nd != 1 && Nd != 3)) return fail(CFGPU_EINVAL, "bad argument");
  *out = nullptr;
  auto* f = new cfgpu_field_s();
  int st = f2v_grid(grid, f->g);
  if (st == CFGPU_OK) {
    f->Nd = Nd;
    int ats = 0, dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) ats = 0;
    f->g.direct = ats == 1 && g_host_access.load() != 0;
    if (cudaStreamCreateWithFlags(&f->g.st, cudaStreamNonBlocking) != cudaSuccess)
      st = fail(CFGPU_ECUDA, "cudaStreamCreate failed");
  }
  const size_t n = (size_t)Nd * f->g.compc();
  if (st == CFGPU_OK) st = dalloc(&f->data, n, f->bytes);
  if (st == CFGPU_OK && cudaMemsetAsync(f->data, 0, n * sizeof(double), f->g.st) != cudaSuccess)
    st = fail(CFGPU_ECUDA, "cudaMemset failed");
  if (st == CFGPU_OK && cudaStreamSynchronize(f->g.st) != cudaSuccess) st = fail(CFGPU_ECUDA, "stream sync");
  if (st != CFGPU_OK) {
    cfgpu_field_destroy(f);
    return st;
  }
  *out = f;
  return CFGPU_OK;
}

cfgpu_status cfgpu_field_upload(cfgpu_field f, const double* u) {
  if (!f || !u) return fail(CFGPU_EINVAL, "bad argument");
  return field_transfer(f, u, nullptr);
}

cfgpu_status cfgpu_field_download(cfgpu_field f, double* u) {
  if (!f || !u) return fail(CFGPU_EINVAL, "bad argument");
  const GridDev& g = f->g.g;
  memset(u, 0, sizeof(double) * f->Nd * 2 * (size_t)g.Ny * g.Nx * (g.Nz / 2 + 1));
  return field_transfer(f, nullptr, u);
}

cfgpu_status cfgpu_field_destroy(cfgpu_field f) {
  if (!f) return CFGPU_OK;
  if (f->g.st) cudaStreamSynchronize(f->g.st);
  dfree(f->data);
  if (f->g.st) cudaStreamDestroy(f->g.st);
  f->g.st = nullptr;
  delete f;
  return CFGPU_OK;
}

// The DNS's current velocity / pressure (field 0 of an ensemble: slot) from / into GPU fields (device to
// device; either may be null).
cfgpu_status cfgpu_dns_set_fields_device(cfgpu_dns d, int slot, cfgpu_field u, cfgpu_field q) {
  if (!d || slot < 0 || slot >= d->nb || (u && !field_matches(d, u, 3)) || (q && !field_matches(d, q, 1)))
    return fail(CFGPU_EINVAL, "bad argument (fields must have the DNS's grid and 2/3-dealiased modes)");
  const size_t w = 2 * (size_t)d->g.Md, pitch = w * d->nb, N = d->N;
  if (u) CK(cudaStreamSynchronize(u->g.st));
  if (q) CK(cudaStreamSynchronize(q->g.st));
  if (u) CK(cudaMemcpy2DAsync(d->Ucur + slot * w, pitch * 8, u->data, w * 8, w * 8, 3 * N, cudaMemcpyDeviceToDevice, d->st));
  if (q) CK(cudaMemcpy2DAsync(d->Qcur + slot * w, pitch * 8, q->data, w * 8, w * 8, N, cudaMemcpyDeviceToDevice, d->st));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_get_fields_device(cfgpu_dns d, int slot, cfgpu_field u, cfgpu_field q) {
  if (!d || slot < 0 || slot >= d->nb || (u && !field_matches(d, u, 3)) || (q && !field_matches(d, q, 1)))
    return fail(CFGPU_EINVAL, "bad argument (fields must have the DNS's grid and 2/3-dealiased modes)");
  const size_t w = 2 * (size_t)d->g.Md, pitch = w * d->nb, N = d->N;
  if (u) CK(cudaMemcpy2DAsync(u->data, w * 8, d->Ucur + slot * w, pitch * 8, w * 8, 3 * N, cudaMemcpyDeviceToDevice, d->st));
  if (q) CK(cudaMemcpy2DAsync(q->data, w * 8, d->Qcur + slot * w, pitch * 8, w * 8, N, cudaMemcpyDeviceToDevice, d->st));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_set_fields(cfgpu_dns d, const double* u, const double* q) {
  if (!d) return fail(CFGPU_EINVAL, "null dns");
  CKS(set_fields(d, u, q));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_get_fields(cfgpu_dns d, double* u, double* q) {
  if (!d) return fail(CFGPU_EINVAL, "null dns");
  return get_fields(d, u, q);
}

cfgpu_status cfgpu_dns_advance_resident(cfgpu_dns d, int nsteps) {
  if (!d || nsteps < 0) return fail(CFGPU_EINVAL, "bad argument");
  CKS(dns_advance_device(d, nsteps));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_advance(cfgpu_dns d, double* u, double* q, int nsteps) {
  if (!d || !u || !q || nsteps < 0) return fail(CFGPU_EINVAL, "bad argument");
  CKS(set_fields(d, u, q));
  CKS(dns_advance_device(d, nsteps));
  return get_fields(d, u, q);
}

cfgpu_status cfgpu_dns_reset_dt(cfgpu_dns d, double dt) {
  if (!d || dt <= 0) return fail(CFGPU_EINVAL, "bad argument");
  d->fl.dt = dt;
  drop_graphs(d);  // tables and step coefficients change
  // MultistepDNS/CNABstyleDNS/RungeKuttaDNS::reset_dt (dnsalgo.cpp:191-200, 404-413, 589-606)
  for (Scheme* s : {&d->main, &d->init}) {
    if (s == &d->init && !d->has_init) continue;
    const double t = s->t;
    std::vector<TauTable> keep = s->tau;
    CKS(setup_scheme(*s, s->method, dt));
    s->t = t;
    s->tau = keep;
    CKS(build_tables(d, *s));
  }
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_reset_time(cfgpu_dns d, double t) {
  if (!d) return fail(CFGPU_EINVAL, "bad argument");
  d->main.t = t;
  if (d->has_init) d->init.t = t;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_reset_gradp(cfgpu_dns d, double dPdx, double dPdz) {
  if (!d) return fail(CFGPU_EINVAL, "bad argument");
  if (d->hetero) return fail(CFGPU_ENOTSUP, "per-field parameters: set the constraint with cfgpu_ensemble_set_params");
  d->fl.constraint = CFGPU_PressureGradient;
  d->fl.dPdx = dPdx, d->fl.dPdz = dPdz, d->fl.Ubulk = 0.0, d->fl.Wbulk = 0.0;
  d->dPdxRef = dPdx, d->dPdzRef = dPdz, d->UbulkRef = 0.0, d->WbulkRef = 0.0;
  drop_graphs(d);  // the step parameters change
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_reset_bulkv(cfgpu_dns d, double Ubulk, double Wbulk) {
  if (!d) return fail(CFGPU_EINVAL, "bad argument");
  if (d->hetero) return fail(CFGPU_ENOTSUP, "per-field parameters: set the constraint with cfgpu_ensemble_set_params");
  d->fl.constraint = CFGPU_BulkVelocity;
  d->fl.Ubulk = Ubulk, d->fl.Wbulk = Wbulk, d->fl.dPdx = 0.0, d->fl.dPdz = 0.0;
  d->UbulkRef = Ubulk, d->WbulkRef = Wbulk, d->dPdxRef = 0.0, d->dPdzRef = 0.0;
  drop_graphs(d);
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_constraint(cfgpu_dns d, double* v) {
  if (!d || !v) return fail(CFGPU_EINVAL, "bad argument");
  v[0] = d->UbulkAct, v[1] = d->WbulkAct, v[2] = d->UbulkRef, v[3] = d->WbulkRef, v[4] = d->dPdxRef, v[5] = d->dPdzRef;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_time(cfgpu_dns d, double* t) {
  if (!d || !t) return fail(CFGPU_EINVAL, "bad argument");
  *t = d->main.t;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_dPdx(cfgpu_dns d, double* dPdx) {
  if (!d || !dPdx) return fail(CFGPU_EINVAL, "bad argument");
  double v[2];
  CK(cudaMemcpyAsync(v, d->ddPdx, sizeof(v), cudaMemcpyDeviceToHost, d->st));
  CK(cudaStreamSynchronize(d->st));
  *dPdx = v[0];
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_base(cfgpu_dns d, double* Ubase, double* Wbase) {
  if (!d) return fail(CFGPU_EINVAL, "null dns");
  if (Ubase) memcpy(Ubase, d->Ubase.data(), d->N * sizeof(double));
  if (Wbase) memcpy(Wbase, d->Wbase.data(), d->N * sizeof(double));
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_num_modes(cfgpu_dns d, int* n) {
  if (!d || !n) return fail(CFGPU_EINVAL, "bad argument");
  *n = d->g.Md;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_device_bytes(cfgpu_dns d, long long* b) {
  if (!d || !b) return fail(CFGPU_EINVAL, "bad argument");
  *b = d->bytes;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_kernel_launches(cfgpu_dns d, long long* n) {
  if (!d || !n) return fail(CFGPU_EINVAL, "bad argument");
  *n = d->launches;
  return CFGPU_OK;
}


// navierstokesNL (channelflow/nse.cpp:12-91) followed by NSE::nonlinear's zeroPaddedModes
// (nse.cpp:383-391): f = N(u) for the FlowField buffers u (nb velocity fields, spectral), computed by the
// DNS's own kernels in its precision; the DNS's state is untouched (an Alternating form flips as in
// navierstokesNL).
cfgpu_status cfgpu_dns_nonlinear(cfgpu_dns d, const double* u, double* f) {
  if (!d || !u || !f) return fail(CFGPU_EINVAL, "bad argument");
  CKS(ensure_stage(d));
  const size_t cd = d->compc(), rs = d->rsz();
  long long B = 0;
  double* Ud = nullptr;
  unsigned char* Nd = nullptr;
  CKS(dalloc(&Ud, 3 * cd, B));
  int st = dalloc(&Nd, 3 * cd * rs, B);
  std::vector<double> out(3 * cd);
  std::vector<int> ver(d->nb);  // the evaluation advances the constant versions: put them back afterwards
  if (st == CFGPU_OK) {
    gather_modes(d, u, 3, d->stage);
    cudaError_t e = cudaMemcpyAsync(ver.data(), d->dver, d->nb * sizeof(int), cudaMemcpyDeviceToHost, d->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Ud, d->stage, 3 * cd * sizeof(double), cudaMemcpyHostToDevice, d->st);
    if (e == cudaSuccess && (st = nonlinear(d, Ud, Nd, 0)) == CFGPU_OK) {
      e = cudaMemcpyAsync(d->dver, ver.data(), d->nb * sizeof(int), cudaMemcpyHostToDevice, d->st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d->stage, Nd, 3 * cd * rs, cudaMemcpyDeviceToHost, d->st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
    }
    if (e != cudaSuccess) st = fail(CFGPU_ECUDA, std::string("nonlinear: ") + cudaGetErrorString(e));
  }
  cudaStreamSynchronize(d->st);
  dfree(Ud);
  dfree(Nd);
  if (st != CFGPU_OK) return st;
  if (rs == sizeof(double)) {
    memcpy(out.data(), d->stage, 3 * cd * sizeof(double));
  } else {
    const float* p = reinterpret_cast<const float*>(d->stage);
    for (size_t i = 0; i < 3 * cd; ++i) out[i] = p[i];
  }
  const GridDev& g = d->g;
  memset(f, 0, sizeof(double) * 3 * (size_t)d->nb * 2 * g.Ny * g.Nx * (g.Nz / 2 + 1));
  scatter_modes(d, out.data(), 3, f);
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_cfl(cfgpu_dns d, double* cfl) {
  if (!d || !cfl) return fail(CFGPU_EINVAL, "bad argument");
  std::vector<double> v(d->nb);
  CKS(d->precision == CFGPU_FP64 ? cfl_impl<double>(d, v.data()) : cfl_impl<float>(d, v.data()));
  *cfl = v[0];
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_l2norm(cfgpu_dns d, int field, double* l2) {
  if (!d || !l2 || (field != 0 && field != 1)) return fail(CFGPU_EINVAL, "bad argument");
  std::vector<double> v(d->nb);
  CKS(l2norm_impl(d, field, v.data()));
  *l2 = v[0];
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_advance_timed(cfgpu_dns d, int nsteps, double* ms) {
  if (!d || nsteps < 0 || !ms) return fail(CFGPU_EINVAL, "bad argument");
  cudaEvent_t a = take_event(d), b = take_event(d);
  CK(cudaStreamSynchronize(d->st));  // the timed region starts on an idle stream
  CK(cudaEventRecord(a, d->st));
  CKS(dns_advance_device(d, nsteps));
  CK(cudaEventRecord(b, d->st));
  CK(cudaEventSynchronize(b));
  float t = 0;
  CK(cudaEventElapsedTime(&t, a, b));
  *ms = t;
  d->ev_pool.push_back(a);
  d->ev_pool.push_back(b);
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_set_profiling(cfgpu_dns d, int enable) {
  if (!d) return fail(CFGPU_EINVAL, "null dns");
  d->profiling = enable != 0;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_set_symmetries(cfgpu_dns d, const cfgpu_symmetry* syms, int n, int interval) {
  if (!d || n < 0 || (n > 0 && !syms) || interval < 1) return fail(CFGPU_EINVAL, "bad argument");
  d->syms.clear();
  for (int i = 0; i < n; ++i) {
    const cfgpu_symmetry& y = syms[i];
    if (std::abs(y.s) != 1 || std::abs(y.sx) != 1 || std::abs(y.sy) != 1 || std::abs(y.sz) != 1)
      return fail(CFGPU_EINVAL, "symmetry signs must be +1 or -1");
    d->syms.push_back({y.s, y.sx, y.sy, y.sz, y.ax, y.az});
  }
  d->sym_interval = interval;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_symmetry(cfgpu_dns d, const cfgpu_symmetry* y, int project) {
  if (!d || !y) return fail(CFGPU_EINVAL, "bad argument");
  if (std::abs(y->s) != 1 || std::abs(y->sx) != 1 || std::abs(y->sy) != 1 || std::abs(y->sz) != 1)
    return fail(CFGPU_EINVAL, "symmetry signs must be +1 or -1");
  CKS(symmetry_on(d, d->Ucur, 8, 3, SymmetryDev{y->s, y->sx, y->sy, y->sz, y->ax, y->az}, project ? 1 : 0));
  CK(cudaStreamSynchronize(d->st));
  return CFGPU_OK;
}

}  // extern "C"

namespace {
// Block order of the field <-> vector map (flowfield.cpp:4480-4557) over the solved set of g (dealiased):
// ord[j] = solved-mode index of block j; blk[m] = block of mode m (-1: the (0,0) mode; -(j+2): kz = 0,
// kx < 0, the conjugate of block j).
void f2v_tables(const GridDev& g, std::vector<int>& ord, std::vector<int>& blk) {
  auto midx = [&](int kx, int kz) { return (kx >= 0 ? kx : kx + g.NKx) * g.NKz + kz; };
  ord.clear();
  blk.assign(g.Md, -1);
  for (int kx = 1; kx <= g.Kx; ++kx) {
    blk[midx(kx, 0)] = (int)ord.size();
    blk[midx(-kx, 0)] = -((int)ord.size() + 2);
    ord.push_back(midx(kx, 0));
  }
  for (int kz = 1; kz <= g.Kz; ++kz) {
    blk[midx(0, kz)] = (int)ord.size();
    ord.push_back(midx(0, kz));
  }
  for (int kx = -g.Kx; kx <= g.Kx; ++kx) {
    if (kx == 0) continue;
    for (int kz = 1; kz <= g.Kz; ++kz) {
      blk[midx(kx, kz)] = (int)ord.size();
      ord.push_back(midx(kx, kz));
    }
  }
}

long long f2v_size(int Ny, int Kx, int Kz) {
  return 2LL * (Ny - 2) + (long long)(Kx + Kz + 2 * Kx * Kz) * (4LL * Ny - 12);
}

// field f of a batch of fstride fields (device, solved-mode layout) -> vector in host memory
int f2v_device(const GridDev& g, int f, int fstride, const double* U, double* v, cudaStream_t st) {
  std::vector<int> ord, blk;
  f2v_tables(g, ord, blk);
  const size_t n = (size_t)f2v_size(g.Ny, g.Kx, g.Kz);
  long long B = 0;
  int* dord = nullptr;
  double* dv = nullptr;
  int status = CFGPU_OK;
  auto body = [&]() -> int {
    CKS(dalloc(&dord, ord.size(), B));
    CKS(dalloc(&dv, n, B));
    CK(cudaMemcpyAsync(dord, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(launch_field2vector(g, f, fstride, dord, (int)ord.size(), U, dv, st));
    CK(cudaMemcpyAsync(v, dv, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CFGPU_OK;
  };
  status = body();
  cudaStreamSynchronize(st);
  dfree(dord);
  dfree(dv);
  return status;
}

// vector in host memory -> field f of a batch (device); every coefficient of that field's solved modes is set
int v2f_device(const GridDev& g, int f, int fstride, const double* v, double* U, cudaStream_t st) {
  std::vector<int> ord, blk;
  f2v_tables(g, ord, blk);
  const size_t n = (size_t)f2v_size(g.Ny, g.Kx, g.Kz);
  long long B = 0;
  int* dblk = nullptr;
  double *dv = nullptr, *W = nullptr;
  int status = CFGPU_OK;
  auto body = [&]() -> int {
    CKS(dalloc(&dblk, blk.size(), B));
    CKS(dalloc(&dv, n, B));
    CKS(dalloc(&W, 2 * (size_t)g.Md * g.Ny, B));
    CK(cudaMemcpyAsync(dblk, blk.data(), blk.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv, v, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(launch_vector2field(g, f, fstride, dblk, dv, U, W, st));
    CK(cudaStreamSynchronize(st));
    return CFGPU_OK;
  };
  status = body();
  cudaStreamSynchronize(st);
  dfree(dblk);
  dfree(dv);
  dfree(W);
  return status;
}

int f2v_grid(const cfgpu_grid* grid, cfgpu_dns_s& tmp) {
  if (!grid || grid->Nx < 6 || grid->Nz < 6 || grid->Ny < 5 || grid->Nx % 2 || grid->Nz % 2)
    return fail(CFGPU_EINVAL, "bad grid (Nx, Nz even >= 6, Ny >= 5)");
  GridDev& g = tmp.g;
  g.Nx = grid->Nx; g.Ny = grid->Ny; g.Nz = grid->Nz;
  g.Kx = grid->Nx / 3 - 1;
  g.Kz = grid->Nz / 3 - 1;
  g.NKx = 2 * g.Kx + 1;
  g.NKz = g.Kz + 1;
  g.Md = g.NKx * g.NKz;
  g.kxmax = grid->Nx / 2;
  g.kzmax = grid->Nz / 2;
  g.Lx = grid->Lx; g.Lz = grid->Lz; g.a = grid->a; g.b = grid->b;
  tmp.N = grid->Ny;
  tmp.nb = 1;
  return CFGPU_OK;
}
}  // namespace

extern "C" {

cfgpu_status cfgpu_orthogonalize(int n, int k, const double* V, double* w, double* h) {
  if (n < 1 || k < 0 || !w || !h || (k > 0 && !V)) return fail(CFGPU_EINVAL, "bad argument");
  cudaStream_t st = nullptr;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  long long B = 0;
  double *dV = nullptr, *dw = nullptr, *dh = nullptr, *work = nullptr;
  auto body = [&]() -> int {
    if (k > 0) CKS(dalloc(&dV, (size_t)k * n, B));
    CKS(dalloc(&dw, n, B));
    CKS(dalloc(&dh, (size_t)k + 1, B));
    CKS(dalloc(&work, (size_t)(k + 1) * 64 + k + 1, B));
    if (k > 0) CK(cudaMemcpyAsync(dV, V, (size_t)k * n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dw, w, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(launch_orthogonalize(n, k, dV, dw, dh, work, st));
    CK(cudaMemcpyAsync(w, dw, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(h, dh, ((size_t)k + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CFGPU_OK;
  };
  const int status = body();
  cudaStreamSynchronize(st);
  for (double* p : {dV, dw, dh, work}) dfree(p);
  cudaStreamDestroy(st);
  return status;
}

cfgpu_status cfgpu_field2vector_size(const cfgpu_grid* grid, long long* n) {
  cfgpu_dns_s tmp;
  if (!n) return fail(CFGPU_EINVAL, "bad argument");
  CKS(f2v_grid(grid, tmp));
  *n = f2v_size(tmp.g.Ny, tmp.g.Kx, tmp.g.Kz);
  return CFGPU_OK;
}

cfgpu_status cfgpu_field2vector(const cfgpu_grid* grid, const double* u, double* v) {
  cfgpu_dns_s tmp;  // mode set only; no DNS is built
  if (!u || !v) return fail(CFGPU_EINVAL, "bad argument");
  CKS(f2v_grid(grid, tmp));
  const size_t n = 3 * tmp.compc();
  std::vector<double> h(n);
  gather_modes(&tmp, u, 3, h.data());
  cudaStream_t st = nullptr;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  long long B = 0;
  double* U = nullptr;
  int status = dalloc(&U, n, B);
  if (status == CFGPU_OK) {
    const cudaError_t e = cudaMemcpyAsync(U, h.data(), n * sizeof(double), cudaMemcpyHostToDevice, st);
    status = e == cudaSuccess ? f2v_device(tmp.g, 0, 1, U, v, st) : fail(CFGPU_ECUDA, cudaGetErrorString(e));
  }
  cudaStreamSynchronize(st);
  dfree(U);
  cudaStreamDestroy(st);
  return status;
}

cfgpu_status cfgpu_vector2field(const cfgpu_grid* grid, const double* v, double* u) {
  cfgpu_dns_s tmp;
  if (!u || !v) return fail(CFGPU_EINVAL, "bad argument");
  CKS(f2v_grid(grid, tmp));
  const size_t n = 3 * tmp.compc();
  std::vector<double> h(n);
  cudaStream_t st = nullptr;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  long long B = 0;
  double* U = nullptr;
  int status = dalloc(&U, n, B);
  if (status == CFGPU_OK) status = v2f_device(tmp.g, 0, 1, v, U, st);
  if (status == CFGPU_OK) {
    cudaError_t e = cudaMemcpyAsync(h.data(), U, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) status = fail(CFGPU_ECUDA, cudaGetErrorString(e));
  }
  cudaStreamSynchronize(st);
  dfree(U);
  cudaStreamDestroy(st);
  if (status != CFGPU_OK) return status;
  const GridDev& g = tmp.g;
  memset(u, 0, sizeof(double) * 3 * 2 * (size_t)g.Ny * g.Nx * (g.Nz / 2 + 1));
  scatter_modes(&tmp, h.data(), 3, u);
  return CFGPU_OK;
}

cfgpu_status cfgpu_ensemble_field2vector(cfgpu_dns d, int slot, double* v) {
  if (!d || !v || slot < 0 || slot >= d->nb) return fail(CFGPU_EINVAL, "bad argument");
  if (d->g.Kx != d->g.Nx / 3 - 1 || d->g.Kz != d->g.Nz / 3 - 1 || d->N < 5)
    return fail(CFGPU_ENOTSUP, "field2vector needs the 2/3-dealiased mode set");
  CK(cudaStreamSynchronize(d->st));
  return f2v_device(d->g, slot, d->nb, d->Ucur, v, d->st);
}

cfgpu_status cfgpu_ensemble_vector2field(cfgpu_dns d, int slot, const double* v) {
  if (!d || !v || slot < 0 || slot >= d->nb) return fail(CFGPU_EINVAL, "bad argument");
  if (d->g.Kx != d->g.Nx / 3 - 1 || d->g.Kz != d->g.Nz / 3 - 1 || d->N < 5)
    return fail(CFGPU_ENOTSUP, "vector2field needs the 2/3-dealiased mode set");
  CK(cudaStreamSynchronize(d->st));
  return v2f_device(d->g, slot, d->nb, v, d->Ucur, d->st);
}

cfgpu_status cfgpu_field_symmetry(const cfgpu_grid* grid, int dealias, int Nd, const cfgpu_symmetry* y, int project,
                                  double* u) {
  if (!grid || !y || !u || (Nd != 1 && Nd != 3) || grid->Nx < 4 || grid->Nz < 4 || grid->Ny < 2)
    return fail(CFGPU_EINVAL, "bad argument");
  if (std::abs(y->s) != 1 || std::abs(y->sx) != 1 || std::abs(y->sy) != 1 || std::abs(y->sz) != 1)
    return fail(CFGPU_EINVAL, "symmetry signs must be +1 or -1");
  cfgpu_dns_s tmp;  // a field's mode set and staging only; no DNS is built
  GridDev& g = tmp.g;
  g.Nx = grid->Nx; g.Ny = grid->Ny; g.Nz = grid->Nz;
  g.Kx = dealias ? grid->Nx / 3 - 1 : grid->Nx / 2 - 1;
  g.Kz = dealias ? grid->Nz / 3 - 1 : grid->Nz / 2 - 1;
  g.NKx = 2 * g.Kx + 1;
  g.NKz = g.Kz + 1;
  g.Md = g.NKx * g.NKz;
  g.kxmax = grid->Nx / 2;
  g.kzmax = grid->Nz / 2;
  tmp.N = grid->Ny;
  const size_t n = (size_t)Nd * tmp.compc();
  std::vector<double> h(n);
  gather_modes(&tmp, u, Nd, h.data());
  double *a = nullptr, *b = nullptr;
  cudaError_t e = cudaMalloc(&a, 2 * n * sizeof(double));
  if (e != cudaSuccess) return fail(CFGPU_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  b = a + n;
  int st = CFGPU_OK;
  do {
    if ((e = cudaMemcpy(a, h.data(), n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) break;
    if ((e = launch_symmetry<double>(g, 1, grid->Ny, Nd, SymmetryDev{y->s, y->sx, y->sy, y->sz, y->ax, y->az},
                                     project ? 1 : 0, a, b, 0)) != cudaSuccess)
      break;
    if ((e = cudaMemcpy(h.data(), b, n * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess) break;
  } while (false);
  cudaFree(a);
  if (e != cudaSuccess) st = fail(CFGPU_ECUDA, std::string("symmetry: ") + cudaGetErrorString(e));
  if (st == CFGPU_OK) scatter_modes(&tmp, h.data(), Nd, u);
  return st;
}

cfgpu_status cfgpu_set_register_zpass(int enable) {
  set_zpass_register(enable);
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_pdl(int enable) {
  g_pdl_on.store(enable ? 1 : 0);
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_fused_xz(int enable) {
  if (enable < 0 || enable > 2) return fail(CFGPU_EINVAL, "fused x/z mode must be 0, 1 or 2");
  {
    // the cached choices were made under the previous mode
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_xz.clear();
  }
  g_fused_xz.store(enable);
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_tau_segmented(int enable) {
  set_tau_segmented(enable);
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_cheb_tensor(int mode) {
  if (mode < 0 || mode > 2) return fail(CFGPU_EINVAL, "mode must be 0 (never), 1 (timed) or 2 (always)");
  g_cheb_tc.store(mode);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_tc.clear();
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_cheb_tensor(cfgpu_dns dns, int* on) {
  if (!dns || !on) return fail(CFGPU_EINVAL, "null argument");
  *on = dns->ytc ? 1 : 0;
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_cheb_fft(int mode) {
  if (mode < 0 || mode > 2) return fail(CFGPU_EINVAL, "mode must be 0 (matrix), 1 (automatic) or 2 (FFT)");
  g_cheb_fft.store(mode);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cheb.clear();
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_cheb_fft(cfgpu_dns dns, int* fft) {
  if (!dns || !fft) return fail(CFGPU_EINVAL, "null argument");
  *fft = dns->ydct ? 1 : 0;
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_autotune(int enable) {
  g_autotune.store(enable ? 1 : 0);
  if (!enable) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
    g_tune_xz.clear();
    g_tune_cheb.clear();
    g_tune_tc.clear();
  }
  return CFGPU_OK;
}

cfgpu_status cfgpu_set_host_access(int enable) {
  g_host_access.store(enable ? 1 : 0);
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_host_access(cfgpu_dns d, int* direct) {
  if (!d || !direct) return fail(CFGPU_EINVAL, "bad argument");
  *direct = d->direct ? 1 : 0;
  return CFGPU_OK;
}

// Page-locking a caller's FlowField buffer (portable, mapped).  The host-buffer transfers do not change path for
// it; on GB300 the direct kernels read and write pinned and pageable buffers at the same rate.  Host memory
// only: no device memory is taken.
cfgpu_status cfgpu_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return fail(CFGPU_EINVAL, "null pointer or zero size");
  const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterPortable | cudaHostRegisterMapped);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(e == cudaErrorHostMemoryAlreadyRegistered ? CFGPU_EINVAL : CFGPU_ECUDA,
                std::string("cudaHostRegister: ") + cudaGetErrorString(e));
  }
  return CFGPU_OK;
}

cfgpu_status cfgpu_host_unregister(void* ptr) {
  if (!ptr) return fail(CFGPU_EINVAL, "null pointer");
  const cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(e == cudaErrorHostMemoryNotRegistered ? CFGPU_EINVAL : CFGPU_ECUDA,
                std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
  }
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_set_graphs(cfgpu_dns d, int enable) {
  if (!d) return fail(CFGPU_EINVAL, "null dns");
  d->use_graphs = enable != 0;
  if (!d->use_graphs) drop_graphs(d);
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_phase_times(cfgpu_dns d, double* nl_ms, long long* nl_count, double* tau_ms,
                                   long long* tau_count) {
  if (!d) return fail(CFGPU_EINVAL, "null dns");
  CK(cudaStreamSynchronize(d->st));
  double t[2] = {0, 0};
  long long n[2] = {0, 0};
  for (auto& u : d->ev_used) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, u.second.first, u.second.second));
    t[u.first] += ms;
    n[u.first] += 1;
    d->ev_pool.push_back(u.second.first);
    d->ev_pool.push_back(u.second.second);
  }
  d->ev_used.clear();
  if (nl_ms) *nl_ms = t[0];
  if (nl_count) *nl_count = n[0];
  if (tau_ms) *tau_ms = t[1];
  if (tau_count) *tau_count = n[1];
  return CFGPU_OK;
}

cfgpu_status cfgpu_timestep_adjust_for_T(cfgpu_timestep* ts, double T, int* n, int* N, double* dt) {
  if (!ts || T < 0) return fail(CFGPU_EINVAL, "bad argument");
  cfgpu_rt::TimeStepH h;
  CKS(h.init(*ts));
  h.adjust_for_T(T);
  ts->dt = h.dt;
  ts->dT = h.dT;
  if (n) *n = h.n;
  if (N) *N = h.N;
  if (dt) *dt = h.value();
  return CFGPU_OK;
}

cfgpu_status cfgpu_timestep_adjust(cfgpu_timestep* ts, double cfl, int* n, int* adjusted) {
  if (!ts) return fail(CFGPU_EINVAL, "bad argument");
  cfgpu_rt::TimeStepH h;
  CKS(h.init(*ts));
  const int adj = h.adjust(cfl) ? 1 : 0;
  ts->dt = h.dt;
  if (n) *n = h.n;
  if (adjusted) *adjusted = adj;
  return CFGPU_OK;
}

// f^T(u): cfDSI's f(u, T, ...) without a Poincare section (channelflow/cfdsi.cpp:705-775).
cfgpu_status cfgpu_ft(const cfgpu_grid* grid, const cfgpu_flags* flags, const cfgpu_timestep* timestep, double T,
                      const double* u, double* fu, double* cfl_out, int precision) {
  if (!grid || !flags || !timestep || !u || !fu) return fail(CFGPU_EINVAL, "null argument");
  const size_t ncplx = 3 * (size_t)grid->Ny * grid->Nx * (grid->Nz / 2 + 1);
  for (size_t i = 0; i < 2 * ncplx; ++i)
    if (!std::isfinite(u[i])) return fail(CFGPU_ENONFINITE, "f: u is not finite");
  memcpy(fu, u, 2 * ncplx * sizeof(double));
  if (T < 0) {
    for (size_t i = 0; i < 2 * ncplx; ++i) fu[i] *= 1 + std::fabs(T);
    return CFGPU_OK;
  }
  if (T == 0) return CFGPU_OK;
  cfgpu_rt::TimeStepH dt;
  CKS(dt.init(*timestep));
  dt.adjust_for_T(T);
  cfgpu_flags fl = *flags;
  fl.dt = dt.value();
  std::vector<double> q((size_t)2 * grid->Ny * grid->Nx * (grid->Nz / 2 + 1), 0.0);
  cfgpu_dns d = nullptr;
  CKS(cfgpu_dns_create(grid, &fl, nullptr, nullptr, u, precision, &d));
  int st = CFGPU_OK;
  double cfl = 0;
  do {
    if ((st = set_fields(d, fu, q.data())) != CFGPU_OK) break;
    if (dt.variable) {
      // one step to measure the CFL number, then restart from u with the adjusted dt
      if ((st = dns_advance_device(d, 1)) != CFGPU_OK) break;
      if ((st = cfgpu_dns_cfl(d, &cfl)) != CFGPU_OK) break;
      dt.adjust(cfl);
      if ((st = cfgpu_dns_reset_dt(d, dt.value())) != CFGPU_OK) break;
      if ((st = set_fields(d, u, nullptr)) != CFGPU_OK) break;
    }
    for (int s = 1; s <= dt.N; ++s) {
      if ((st = cfgpu_dns_cfl(d, &cfl)) != CFGPU_OK) break;
      if ((st = dns_advance_device(d, dt.n)) != CFGPU_OK) break;
      if (dt.variable && dt.adjust(cfl))
        if ((st = cfgpu_dns_reset_dt(d, dt.value())) != CFGPU_OK) break;
    }
    if (st != CFGPU_OK) break;
    st = get_fields(d, fu, q.data());
  } while (false);
  std::string keep = g_err;
  cfgpu_dns_destroy(d);
  g_err = keep;
  if (st != CFGPU_OK) return st;
  for (size_t i = 0; i < 2 * ncplx; ++i)
    if (!std::isfinite(fu[i])) return fail(CFGPU_ENONFINITE, "f: f^T(u) is not finite");
  if (cfl_out) *cfl_out = cfl;
  return CFGPU_OK;
}

cfgpu_status cfgpu_dns_destroy(cfgpu_dns d) {
  if (!d) return CFGPU_OK;
  cudaStreamSynchronize(d->st);
  dns_free(d);
  return CFGPU_OK;
}

}  // extern "C"

namespace {
// HelmholtzSolver(N, a, b, lambda_s, nu).solve for nsys systems at once (helmholtz.cpp:18-95); with umean the
// mean-constrained solve (helmholtz.cpp:158-213).  Host arrays [nsys][N] (ChebyCoeff data per system).
int helmholtz_batched(int N, int nsys, double a, double b, const double* lambda, double nu, const double* f,
                      const double* ua, const double* ub, const double* umean, double* u, double* mu) {
  if (N < 3 || N % 2 == 0) return fail(CFGPU_EINVAL, "N must be odd and >= 3 (HelmholtzSolver asserts odd N)");
  if (nsys < 1 || !lambda || !f || !u || !(b > a) || nu == 0.0) return fail(CFGPU_EINVAL, "bad argument");
  const size_t FN = (size_t)N * nsys;
  std::vector<double> ft(FN), hbv;
  for (int sy = 0; sy < nsys; ++sy)
    for (int n = 0; n < N; ++n) ft[(size_t)n * nsys + sy] = f[(size_t)sy * N + n];
  std::vector<double> lo, di, up;
  make_helm_b(N, lo, di, up);
  long long B = 0;
  double *dl = nullptr, *df = nullptr, *dua = nullptr, *dub = nullptr, *dum = nullptr, *du = nullptr, *dmu = nullptr;
  double *dW = nullptr, *dhb = nullptr;
  cudaStream_t st = nullptr;
  int status = CFGPU_OK;
  auto body = [&]() -> int {
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CKS(dalloc(&dl, nsys, B));
    CKS(dalloc(&df, FN, B));
    CKS(dalloc(&du, FN, B));
    CKS(dalloc(&dW, 7 * FN, B));
    CKS(dalloc(&dhb, 3 * (size_t)N, B));
    CK(cudaMemcpyAsync(dl, lambda, nsys * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(df, ft.data(), FN * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dhb, lo.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dhb + N, di.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dhb + 2 * N, up.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    if (ua) {
      CKS(dalloc(&dua, nsys, B));
      CK(cudaMemcpyAsync(dua, ua, nsys * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    if (ub) {
      CKS(dalloc(&dub, nsys, B));
      CK(cudaMemcpyAsync(dub, ub, nsys * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    if (umean) {
      CKS(dalloc(&dum, nsys, B));
      CKS(dalloc(&dmu, nsys, B));
      CK(cudaMemcpyAsync(dum, umean, nsys * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    HelmB hb{dhb, dhb + N, dhb + 2 * N};
    CK(launch_helmholtz(N, nsys, a, b, dl, nu, hb, df, dua, dub, dum, du, dmu, dW, st));
    CK(cudaMemcpyAsync(ft.data(), du, FN * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (umean && mu) CK(cudaMemcpyAsync(mu, dmu, nsys * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CFGPU_OK;
  };
  status = body();
  if (st) cudaStreamSynchronize(st);
  for (double* p : {dl, df, dua, dub, dum, du, dmu, dW, dhb}) dfree(p);
  if (st) cudaStreamDestroy(st);
  if (status != CFGPU_OK) return status;
  for (int sy = 0; sy < nsys; ++sy)
    for (int n = 0; n < N; ++n) u[(size_t)sy * N + n] = ft[(size_t)n * nsys + sy];
  return CFGPU_OK;
}
}  // namespace

extern "C" {

cfgpu_status cfgpu_helmholtz_solve_batched(int N, int nsys, double a, double b, const double* lambda, double nu,
                                           const double* f, const double* ua, const double* ub, double* u) {
  return helmholtz_batched(N, nsys, a, b, lambda, nu, f, ua, ub, nullptr, u, nullptr);
}

cfgpu_status cfgpu_helmholtz_solve_mean_batched(int N, int nsys, double a, double b, const double* lambda, double nu,
                                                const double* f, const double* umean, const double* ua,
                                                const double* ub, double* u, double* mu) {
  if (!umean) return fail(CFGPU_EINVAL, "bad argument");
  return helmholtz_batched(N, nsys, a, b, lambda, nu, f, ua, ub, umean, u, mu);
}

cfgpu_status cfgpu_tau_solve_batched(int N, int nmodes, const int* kx, const int* kz, double Lx, double Lz, double a,
                                     double b, double lambda_t, double nu, int taucorrection, const double* Rx,
                                     const double* Ry, const double* Rz, double* u, double* v, double* w, double* P) {
  if (N < 5 || N % 2 == 0 || nmodes <= 0 || !kx || !kz || !Rx || !Ry || !Rz || !u || !v || !w || !P)
    return fail(CFGPU_EINVAL, "bad argument");
  if (!(b > a) || Lx <= 0 || Lz <= 0) return fail(CFGPU_EINVAL, "bad geometry");
  GridDev g{};
  g.Nx = g.Nz = 4;
  g.Ny = N;
  g.Md = nmodes;
  g.NKx = nmodes;
  g.NKz = 1;
  g.kxmax = g.kzmax = 1 << 30;  // no Nyquist zeroing for explicit lists
  g.Lx = Lx;
  g.Lz = Lz;
  g.a = a;
  g.b = b;
  long long bytes = 0;
  int *dkx = nullptr, *dkz = nullptr;
  double *R3 = nullptr, *U3 = nullptr, *Q1 = nullptr, *scr = nullptr, *zero = nullptr, *hlo = nullptr,
         *hdi = nullptr, *hup = nullptr;
  TauTable t{};
  cudaStream_t st = nullptr;
  int status = CFGPU_OK;
  const size_t row = 2 * (size_t)nmodes, comp = row * N;
  std::vector<double> h(3 * comp), hq(comp);
  auto body = [&]() -> int {
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CKS(dalloc(&dkx, nmodes, bytes));
    CKS(dalloc(&dkz, nmodes, bytes));
    CK(cudaMemcpyAsync(dkx, kx, nmodes * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dkz, kz, nmodes * sizeof(int), cudaMemcpyHostToDevice, st));
    g.kxs = dkx;
    g.kzs = dkz;
    CKS(dalloc(&R3, 3 * comp, bytes));
    CKS(dalloc(&U3, 3 * comp, bytes));
    CKS(dalloc(&Q1, comp, bytes));
    CKS(dalloc(&scr, 8 * comp, bytes));
    CKS(dalloc(&zero, N, bytes));
    CK(cudaMemsetAsync(zero, 0, N * sizeof(double), st));
    std::vector<double> lo, di, up;
    make_helm_b(N, lo, di, up);
    CKS(dalloc(&hlo, N, bytes));
    CKS(dalloc(&hdi, N, bytes));
    CKS(dalloc(&hup, N, bytes));
    CK(cudaMemcpyAsync(hlo, lo.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(hdi, di.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(hup, up.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
    HelmB hb{hlo, hdi, hup};
    CKS(dalloc(&t.f, (size_t)N * nmodes * TF_NFIELDS, bytes));
    CKS(dalloc(&t.s, (size_t)nmodes * TS_NSCALARS, bytes));
    CK(launch_tau_setup(g, N, lambda_t, nu, hb, t, scr, st));
    const double* Rs[3] = {Rx, Ry, Rz};
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < nmodes; ++k)
        for (int n = 0; n < N; ++n) {
          h[c * comp + n * row + 2 * k] = Rs[c][2 * ((size_t)k * N + n)];
          h[c * comp + n * row + 2 * k + 1] = Rs[c][2 * ((size_t)k * N + n) + 1];
        }
    CK(cudaMemcpyAsync(R3, h.data(), 3 * comp * sizeof(double), cudaMemcpyHostToDevice, st));
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
    CK(launch_tau_solve<double>(g, N, sp, p, hb, t, st));
    CK(cudaMemcpyAsync(h.data(), U3, 3 * comp * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hq.data(), Q1, comp * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double* outs[4] = {u, v, w, P};
    for (int c = 0; c < 4; ++c)
      for (int k = 0; k < nmodes; ++k)
        for (int n = 0; n < N; ++n) {
          const double* src = c < 3 ? &h[c * comp] : hq.data();
          outs[c][2 * ((size_t)k * N + n)] = src[n * row + 2 * k];
          outs[c][2 * ((size_t)k * N + n) + 1] = src[n * row + 2 * k + 1];
        }
    return CFGPU_OK;
  };
  status = body();
  if (st) cudaStreamSynchronize(st);
  for (void* p : {(void*)dkx, (void*)dkz, (void*)R3, (void*)U3, (void*)Q1, (void*)scr, (void*)zero, (void*)hlo,
                  (void*)hdi, (void*)hup, (void*)t.f, (void*)t.s})
    dfree(p);
  if (st) cudaStreamDestroy(st);
  return status;
}

}  // extern "C"
