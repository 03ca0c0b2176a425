// Links libcfgpu.so through include/cfgpu.hpp the way channelflow code would: cfgpu::DNS over FlowField and
// DNSFlags types, the TauSolver and HelmholtzSolver drop-ins over ChebyCoeff types, and the FlowField
// transforms.  The stand-in types below carry exactly the members of the reference's classes that the
// header uses (flowfield.h, dnsflags.h, chebyshev.h), with the reference's names.
//
// usage: dropin_test <case.bin> <out.bin>
//   case.bin: int32 Nx Ny Nz nsteps, float64 Lx Lz nu dt rotation, then the initial velocity
//             (complex [3][Ny][Nx][Nz/2+1]), then tau inputs (int32 kx kz, float64 lambda, complex Rx Ry Rz [Ny]),
//             then Helmholtz inputs (float64 lambda nu ua ub umean, f [Ny]), then a physical field [Ny][Nx][Nz]
//   out.bin:  u and q after nsteps (spectral), DNS time, CFL, Ubulk, dPdx; tau u v w P; Helmholtz u, u_mean, mu;
//             the physical field after makeSpectral (spectral buffer) and after makePhysical again.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "cfgpu.hpp"

typedef std::complex<double> Complex;

// channelflow/dnsflags.h:24-38
enum BaseFlow { ZeroBase, LinearBase, ParabolicBase, LaminarBase, SuctionBase, ArbitraryBase };
enum MeanConstraint { PressureGradient, BulkVelocity };
enum TimeStepMethod { CNFE1, CNAB2, CNRK2, SMRK2, SBDF1, SBDF2, SBDF3, SBDF4 };
enum NonlinearMethod { Rotational, Convection, Divergence, SkewSymmetric, Alternating, Alternating_, LinearAboutProfile };
enum Dealiasing { NoDealiasing, DealiasXZ, DealiasY, DealiasXYZ };

struct DNSFlags {  // the members of dnsflags.h:84-140 with the reference's defaults
  BaseFlow baseflow = LaminarBase;
  MeanConstraint constraint = PressureGradient;
  TimeStepMethod timestepping = SBDF3;
  TimeStepMethod initstepping = SMRK2;
  NonlinearMethod nonlinearity = Rotational;
  Dealiasing dealiasing = DealiasXZ;
  bool taucorrection = true;
  double nu = 0.0025, Vsuck = 0.0, rotation = 0.0, theta = 0.0, dPdx = 0.0, dPdz = 0.0, Ubulk = 0.0, Wbulk = 0.0;
  double Uwall = 1.0, ulowerwall = 0.0, uupperwall = 0.0, wlowerwall = 0.0, wupperwall = 0.0;
  double t0 = 0.0, dt = 0.03125;
};

class FlowField {  // spectral storage in the serial layout complex [i][my][mx][mz]
 public:
  FlowField(int Nx, int Ny, int Nz, int Nd, double Lx, double Lz, double a = -1, double b = 1)
      : Nx_(Nx), Ny_(Ny), Nz_(Nz), Nd_(Nd), Lx_(Lx), Lz_(Lz), a_(a), b_(b),
        data_((size_t)Nd * Ny * Nx * (Nz / 2 + 1)) {}
  int Nx() const { return Nx_; }
  int Ny() const { return Ny_; }
  int Nz() const { return Nz_; }
  int Nd() const { return Nd_; }
  double Lx() const { return Lx_; }
  double Lz() const { return Lz_; }
  double a() const { return a_; }
  double b() const { return b_; }
  void makeSpectral() {}
  Complex& cmplx(int mx, int my, int mz, int i) {
    return data_[(((size_t)i * Ny_ + my) * Nx_ + mx) * (Nz_ / 2 + 1) + mz];
  }
  std::vector<Complex>& data() { return data_; }

 private:
  int Nx_, Ny_, Nz_, Nd_;
  double Lx_, Lz_, a_, b_;
  std::vector<Complex> data_;
};

class ChebyCoeff {
 public:
  explicit ChebyCoeff(int N) : d_(N) {}
  int N() const { return (int)d_.size(); }
  double& operator[](int n) { return d_[n]; }
  double operator[](int n) const { return d_[n]; }

 private:
  std::vector<double> d_;
};

class ComplexChebyCoeff {
 public:
  explicit ComplexChebyCoeff(int N) : d_(N) {}
  int N() const { return (int)d_.size(); }
  Complex operator[](int n) const { return d_[n]; }
  void set(int n, Complex c) { d_[n] = c; }

 private:
  std::vector<Complex> d_;
};

template <class T>
static void rd(std::ifstream& in, T* p, size_t n) {
  in.read(reinterpret_cast<char*>(p), n * sizeof(T));
  if (!in) {
    std::cerr << "short input\n";
    std::exit(2);
  }
}
template <class T>
static void wr(std::ofstream& out, const T* p, size_t n) {
  out.write(reinterpret_cast<const char*>(p), n * sizeof(T));
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::cerr << "usage: dropin_test case.bin out.bin\n";
    return 2;
  }
  std::ifstream in(argv[1], std::ios::binary);
  std::ofstream out(argv[2], std::ios::binary);
  int dims[4];
  double par[5];
  rd(in, dims, 4);
  rd(in, par, 5);
  const int Nx = dims[0], Ny = dims[1], Nz = dims[2], nsteps = dims[3];
  try {
    // --- DNS: plane Couette, SBDF3 with SMRK2 start-up --------------------------------------------------
    DNSFlags flags;
    flags.nu = par[2];
    flags.dt = par[3];
    flags.rotation = par[4];
    flags.ulowerwall = -1.0;
    flags.uupperwall = 1.0;
    std::vector<FlowField> fields = {FlowField(Nx, Ny, Nz, 3, par[0], par[1]), FlowField(Nx, Ny, Nz, 1, par[0], par[1])};
    rd(in, fields[0].data().data(), fields[0].data().size());
    cfgpu::DNS<FlowField, DNSFlags> dns(fields, flags);
    dns.advance(fields, nsteps / 2);
    dns.advance(fields, nsteps - nsteps / 2);
    wr(out, fields[0].data().data(), fields[0].data().size());
    wr(out, fields[1].data().data(), fields[1].data().size());
    const double scal[4] = {dns.time(), dns.CFL(), dns.Ubulk(), dns.dPdx()};
    wr(out, scal, 4);

    // --- TauSolver ----------------------------------------------------------------------------------------
    int kk[2];
    double lam;
    rd(in, kk, 2);
    rd(in, &lam, 1);
    ComplexChebyCoeff Rx(Ny), Ry(Ny), Rz(Ny), u(Ny), v(Ny), w(Ny), P(Ny);
    std::vector<Complex> buf(3 * (size_t)Ny);
    rd(in, buf.data(), buf.size());
    for (int n = 0; n < Ny; ++n) {
      Rx.set(n, buf[n]);
      Ry.set(n, buf[Ny + n]);
      Rz.set(n, buf[2 * Ny + n]);
    }
    cfgpu::TauSolver tau(kk[0], kk[1], par[0], par[1], -1.0, 1.0, lam, flags.nu, Ny);
    tau.solve(u, v, w, P, Rx, Ry, Rz);
    for (const ComplexChebyCoeff* c : {&u, &v, &w, &P})
      for (int n = 0; n < Ny; ++n) {
        const Complex z = (*c)[n];
        wr(out, &z, 1);
      }

    // --- HelmholtzSolver ------------------------------------------------------------------------------------
    double hp[5];
    rd(in, hp, 5);
    ChebyCoeff f(Ny), hu(Ny), hm(Ny);
    std::vector<double> fb(Ny);
    rd(in, fb.data(), Ny);
    for (int n = 0; n < Ny; ++n) f[n] = fb[n];
    cfgpu::HelmholtzSolver helm(Ny, -1.0, 1.0, hp[0], hp[1]);
    helm.solve(hu, f, hp[2], hp[3]);
    double mu = 0.0;
    helm.solve(hm, mu, f, hp[4], hp[2], hp[3]);
    for (int n = 0; n < Ny; ++n) wr(out, &hu[n], 1);
    for (int n = 0; n < Ny; ++n) wr(out, &hm[n], 1);
    wr(out, &mu, 1);

    // --- FlowField transforms ---------------------------------------------------------------------------
    cfgpu::FlowFieldTransforms tf(Nx, Ny, Nz, 1, par[0], par[1]);
    const int Nzpad = 2 * (Nz / 2 + 1);
    std::vector<double> phys((size_t)Ny * Nx * Nz), buf2(tf.size(), 0.0);
    rd(in, phys.data(), phys.size());
    for (int ny = 0; ny < Ny; ++ny)
      for (int nx = 0; nx < Nx; ++nx)
        for (int nz = 0; nz < Nz; ++nz) buf2[((size_t)ny * Nx + nx) * Nzpad + nz] = phys[((size_t)ny * Nx + nx) * Nz + nz];
    tf.makeSpectral(buf2.data(), CFGPU_PHYSICAL, CFGPU_PHYSICAL);
    wr(out, buf2.data(), buf2.size());
    tf.makePhysical(buf2.data(), CFGPU_SPECTRAL, CFGPU_SPECTRAL);
    wr(out, buf2.data(), buf2.size());

    // --- errors come back as exceptions ---------------------------------------------------------------
    bool threw = false;
    try {
      cfgpu::HelmholtzSolver bad(4, -1.0, 1.0, 1.0);  // even N is rejected by the library
      ChebyCoeff x(4), y(4);
      bad.solve(x, y, 0.0, 0.0);
    } catch (const cfgpu::Error& e) {
      threw = e.code() == CFGPU_EINVAL;
    }
    if (!threw) {
      std::cerr << "expected cfgpu::Error\n";
      return 1;
    }
  } catch (const cfgpu::Error& e) {
    std::cerr << e.what() << "\n";
    return 1;
  }
  std::cout << "dropin ok\n";
  return 0;
}
