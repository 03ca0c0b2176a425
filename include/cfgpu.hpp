/*
 * C++ drop-in for channelflow's DNS, TauSolver, HelmholtzSolver and FlowField transforms over the C ABI
 * of libcfgpu.so (cfgpu.h).  Header-only; link with -lcfgpu (and the CUDA runtime it depends on).
 *
 * The classes are templates over the caller's own types, so the header needs none of channelflow's
 * headers and a maintainer instantiates them with the reference's classes:
 *
 *     #include "cfgpu.hpp"
 *     using DNS = cfgpu::DNS<chflow::FlowField, chflow::DNSFlags>;          // channelflow/dns.h:30-97
 *     DNS dns(fields, flags);                  // DNS::DNS(fields, flags), dns.cpp:22-39
 *     dns.advance(fields, n);                  // DNS::advance(fields, nSteps), dns.cpp:135-163
 *
 * What the templates use of the types (all present in the reference):
 *   FlowField   Nx() Ny() Nz() Nd() Lx() Lz() a() b(), makeSpectral(), cmplx(mx, my, mz, i) -> complex&
 *               (spectral data in the serial layout complex [i][my][mx][mz], flowfield.h:383-402)
 *   DNSFlags    the public members of dnsflags.h:84-140: nu dPdx dPdz Ubulk Wbulk ulowerwall uupperwall
 *               wlowerwall wupperwall Vsuck t0 dt baseflow constraint timestepping initstepping
 *               nonlinearity dealiasing taucorrection rotation (enum values as in dnsflags.h:24-38)
 *   ChebyCoeff  N(), operator[](n) -> double& (chebyshev.h:70-110)
 *   ComplexChebyCoeff  N(), operator[](n) -> complex, set(n, complex) (chebyshev.h:112-180)
 *
 * Errors: every failing call throws cfgpu::Error with the library's message.  The reference reports
 * failures through cferror() (print and exit(1), cfbasics/cfbasics.h:272-278); a caller that wants that
 * behaviour catches cfgpu::Error and calls cferror(e.what()).
 */
#ifndef CFGPU_HPP
#define CFGPU_HPP

#include <cmath>
#include <complex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cfgpu.h"

namespace cfgpu {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(cfgpu_status s) {
  if (s != CFGPU_OK) {
    const char* m = cfgpu_last_error();
    throw Error(s, std::string("cfgpu: ") + (m ? m : "error"));
  }
}

// Every DNSFlags member the time step reads (dnsflags.h:84-140), rotation included (nse.cpp:62-78).
template <class Flags>
cfgpu_flags to_cfgpu_flags(const Flags& f) {
  cfgpu_flags c;
  check(cfgpu_flags_default(&c));
  c.nu = f.nu;
  c.dPdx = f.dPdx;
  c.dPdz = f.dPdz;
  c.Ubulk = f.Ubulk;
  c.Wbulk = f.Wbulk;
  c.ulowerwall = f.ulowerwall;
  c.uupperwall = f.uupperwall;
  c.wlowerwall = f.wlowerwall;
  c.wupperwall = f.wupperwall;
  c.Vsuck = f.Vsuck;
  c.t0 = f.t0;
  c.dt = f.dt;
  c.baseflow = static_cast<int>(f.baseflow);
  c.constraint = static_cast<int>(f.constraint);
  c.timestepping = static_cast<int>(f.timestepping);
  c.initstepping = static_cast<int>(f.initstepping);
  c.nonlinearity = static_cast<int>(f.nonlinearity);
  c.dealiasing = static_cast<int>(f.dealiasing);
  c.taucorrection = f.taucorrection ? 1 : 0;
  c.rotation = f.rotation;
  return c;
}

template <class FlowField>
cfgpu_grid grid_of(const FlowField& u) {
  cfgpu_grid g;
  g.Nx = u.Nx();
  g.Ny = u.Ny();
  g.Nz = u.Nz();
  g.Lx = u.Lx();
  g.Lz = u.Lz();
  g.a = u.a();
  g.b = u.b();
  return g;
}

// The FlowField's spectral buffer (made spectral first, as DNS::advance does, dns.cpp:135-163).
template <class FlowField>
double* spectral_data(FlowField& u) {
  u.makeSpectral();
  return reinterpret_cast<double*>(&u.cmplx(0, 0, 0, 0));
}

// DNS (channelflow/dns.h:30-97) with the time step on the GPU.  precision: CFGPU_FP64 (the reference's
// arithmetic) or CFGPU_MIXED (FP32 transforms and nonlinear term, FP64 state and solves).
template <class FlowField, class DNSFlags>
class DNS {
 public:
  DNS(const std::vector<FlowField>& fields, const DNSFlags& flags, int precision = CFGPU_FP64) {
    create(fields, flags, nullptr, nullptr, precision);
  }
  // DNS(fields, base, flags) (dns.cpp:41-62): base = {Ubase, Wbase} Chebyshev coefficients.
  template <class ChebyCoeff>
  DNS(const std::vector<FlowField>& fields, const std::vector<ChebyCoeff>& base, const DNSFlags& flags,
      int precision = CFGPU_FP64) {
    if (base.size() < 2) throw Error(CFGPU_EINVAL, "cfgpu: base needs {Ubase, Wbase}");
    std::vector<double> U(base[0].N()), W(base[1].N());
    for (int n = 0; n < base[0].N(); ++n) U[n] = base[0][n];
    for (int n = 0; n < base[1].N(); ++n) W[n] = base[1][n];
    create(fields, flags, U.data(), W.data(), precision);
  }
  ~DNS() {
    if (h_) cfgpu_dns_destroy(h_);
  }
  DNS(const DNS&) = delete;
  DNS& operator=(const DNS&) = delete;
  DNS(DNS&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }

  // fields[0] = velocity, fields[1] = modified pressure q; both overwritten in place.
  void advance(std::vector<FlowField>& fields, int nSteps) {
    check(cfgpu_dns_advance(h_, spectral_data(fields[0]), spectral_data(fields[1]), nSteps));
  }
  void reset_dt(double dt) { check(cfgpu_dns_reset_dt(h_, dt)); }
  void reset_time(double t) { check(cfgpu_dns_reset_time(h_, t)); }
  void reset_gradp(double dPdx, double dPdz) { check(cfgpu_dns_reset_gradp(h_, dPdx, dPdz)); }
  void reset_bulkv(double Ubulk, double Wbulk) { check(cfgpu_dns_reset_bulkv(h_, Ubulk, Wbulk)); }
  double time() const { return query(cfgpu_dns_time); }
  double dPdx() const { return query(cfgpu_dns_dPdx); }
  // CFL number of the velocity after the last advance (DNSAlgorithm::CFL, dnsalgo.cpp:62-66).
  double CFL() const { return query(cfgpu_dns_cfl); }
  double Ubulk() const { return constraint(0); }
  double Wbulk() const { return constraint(1); }
  double UbulkRef() const { return constraint(2); }
  double WbulkRef() const { return constraint(3); }
  double dPdxRef() const { return constraint(4); }
  double dPdzRef() const { return constraint(5); }
  // Base flow profiles (NSE::Ubase / Wbase), Ny coefficients each.
  void base(std::vector<double>& U, std::vector<double>& W) const {
    U.assign(Ny_, 0.0);
    W.assign(Ny_, 0.0);
    check(cfgpu_dns_base(h_, U.data(), W.data()));
  }
  cfgpu_dns handle() const { return h_; }

 private:
  void create(const std::vector<FlowField>& fields, const DNSFlags& flags, const double* U, const double* W,
              int precision) {
    if (fields.empty()) throw Error(CFGPU_EINVAL, "cfgpu: DNS needs the velocity field");
    FlowField us(fields[0]);
    cfgpu_grid g = grid_of(us);
    cfgpu_flags c = to_cfgpu_flags(flags);
    if (U && W) c.baseflow = 5;  // ArbitraryBase, as DNS(fields, base, flags) sets it (dns.cpp:44)
    Ny_ = g.Ny;
    check(cfgpu_dns_create(&g, &c, U, W, spectral_data(us), precision, &h_));
  }
  double query(cfgpu_status (*fn)(cfgpu_dns, double*)) const {
    double v = 0.0;
    check(fn(h_, &v));
    return v;
  }
  double constraint(int k) const {
    double v[6];
    check(cfgpu_dns_constraint(h_, v));
    return v[k];
  }
  cfgpu_dns h_ = nullptr;
  int Ny_ = 0;
};

// TauSolver (channelflow/tausolver.h:30-50) for one (kx, kz) mode, solved on the GPU.  lambda is the full
// value the reference passes, lambda_t + 4 pi^2 nu (kx^2/Lx^2 + kz^2/Lz^2) (nse.cpp:683-700); the library
// takes lambda_t and rebuilds lambda the same way (equal to round-off).  Solving many modes at once through
// cfgpu_tau_solve_batched is the efficient form; this class keeps the reference's per-mode interface.
class TauSolver {
 public:
  TauSolver(int kx, int kz, double Lx, double Lz, double a, double b, double lambda, double nu, int Ny,
            bool tauCorrection = true)
      : kx_(kx), kz_(kz), N_(Ny), Lx_(Lx), Lz_(Lz), a_(a), b_(b), nu_(nu), tau_(tauCorrection) {
    const double pi = 3.14159265358979323846;
    lambda_t_ = lambda - 4.0 * pi * pi * nu * ((kx / Lx) * (kx / Lx) + (kz / Lz) * (kz / Lz));
  }
  // solve(u, v, w, P, Rx, Ry, Rz) (tausolver.cpp:347-402) for ComplexChebyCoeff-like profiles.
  template <class CCC>
  void solve(CCC& u, CCC& v, CCC& w, CCC& P, const CCC& Rx, const CCC& Ry, const CCC& Rz) const {
    std::vector<std::complex<double>> in(3 * (size_t)N_), out(4 * (size_t)N_);
    for (int n = 0; n < N_; ++n) {
      in[n] = Rx[n];
      in[N_ + n] = Ry[n];
      in[2 * N_ + n] = Rz[n];
    }
    solve_raw(in.data(), in.data() + N_, in.data() + 2 * N_, out.data(), out.data() + N_, out.data() + 2 * N_,
              out.data() + 3 * N_);
    for (int n = 0; n < N_; ++n) {
      u.set(n, out[n]);
      v.set(n, out[N_ + n]);
      w.set(n, out[2 * N_ + n]);
      P.set(n, out[3 * N_ + n]);
    }
  }
  // The same on raw complex Chebyshev coefficient arrays of length Ny.
  void solve_raw(const std::complex<double>* Rx, const std::complex<double>* Ry, const std::complex<double>* Rz,
                 std::complex<double>* u, std::complex<double>* v, std::complex<double>* w,
                 std::complex<double>* P) const {
    check(cfgpu_tau_solve_batched(N_, 1, &kx_, &kz_, Lx_, Lz_, a_, b_, lambda_t_, nu_, tau_ ? 1 : 0, d(Rx), d(Ry),
                                  d(Rz), d(u), d(v), d(w), d(P)));
  }

 private:
  static const double* d(const std::complex<double>* p) { return reinterpret_cast<const double*>(p); }
  static double* d(std::complex<double>* p) { return reinterpret_cast<double*>(p); }
  int kx_, kz_, N_;
  double Lx_, Lz_, a_, b_, nu_, lambda_t_;
  bool tau_;
};

// HelmholtzSolver (channelflow/helmholtz.h:29-38): nu u'' - lambda u = f with Dirichlet values, and the
// mean-constrained form nu u'' - lambda u - mu = f, mean(u) = umean; solved on the GPU.
class HelmholtzSolver {
 public:
  HelmholtzSolver(int numberModes, double a, double b, double lambda, double nu = 1.0)
      : N_(numberModes), a_(a), b_(b), lambda_(lambda), nu_(nu) {}
  double lambda() const { return lambda_; }

  template <class ChebyCoeff>
  void solve(ChebyCoeff& u, const ChebyCoeff& f, double ua, double ub) const {
    std::vector<double> fv(N_), uv(N_);
    for (int n = 0; n < N_; ++n) fv[n] = f[n];
    check(cfgpu_helmholtz_solve_batched(N_, 1, a_, b_, &lambda_, nu_, fv.data(), &ua, &ub, uv.data()));
    for (int n = 0; n < N_; ++n) u[n] = uv[n];
  }
  template <class ChebyCoeff>
  void solve(ChebyCoeff& u, double& mu, const ChebyCoeff& f, double umean, double ua, double ub) const {
    std::vector<double> fv(N_), uv(N_);
    for (int n = 0; n < N_; ++n) fv[n] = f[n];
    check(cfgpu_helmholtz_solve_mean_batched(N_, 1, a_, b_, &lambda_, nu_, fv.data(), &umean, &ua, &ub, uv.data(),
                                             &mu));
    for (int n = 0; n < N_; ++n) u[n] = uv[n];
  }

 private:
  int N_;
  double a_, b_, lambda_, nu_;
};

// A FlowField's data transformed on the GPU: makePhysical / makeSpectral of flowfield.cpp:1850-1997 on a
// whole FlowField buffer (Nd*Ny*Nx*2*(Nz/2+1) doubles in the reference's serial layout), in place.
class FlowFieldTransforms {
 public:
  FlowFieldTransforms(int Nx, int Ny, int Nz, int Nd, double Lx, double Lz, double a = -1.0, double b = 1.0) {
    cfgpu_grid g;
    g.Nx = Nx;
    g.Ny = Ny;
    g.Nz = Nz;
    g.Lx = Lx;
    g.Lz = Lz;
    g.a = a;
    g.b = b;
    check(cfgpu_flowfield_create(&g, Nd, &f_));
    long long n = 0;
    check(cfgpu_flowfield_size(f_, &n));
    n_ = (size_t)n;
  }
  ~FlowFieldTransforms() {
    if (f_) cfgpu_flowfield_destroy(f_);
  }
  FlowFieldTransforms(const FlowFieldTransforms&) = delete;
  FlowFieldTransforms& operator=(const FlowFieldTransforms&) = delete;
  size_t size() const { return n_; }
  // data: the FlowField's buffer in state (xzstate, ystate) (CFGPU_PHYSICAL / CFGPU_SPECTRAL)
  void makePhysical(double* data, int xzstate, int ystate) {
    check(cfgpu_flowfield_upload(f_, data, xzstate, ystate));
    check(cfgpu_flowfield_make_physical(f_));
    check(cfgpu_flowfield_download(f_, data));
  }
  void makeSpectral(double* data, int xzstate, int ystate) {
    check(cfgpu_flowfield_upload(f_, data, xzstate, ystate));
    check(cfgpu_flowfield_make_spectral(f_));
    check(cfgpu_flowfield_download(f_, data));
  }
  cfgpu_flowfield handle() const { return f_; }

 private:
  cfgpu_flowfield f_ = nullptr;
  size_t n_ = 0;
};

}  // namespace cfgpu

#endif  // CFGPU_HPP
