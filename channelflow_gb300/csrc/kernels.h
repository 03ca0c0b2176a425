// Internal launcher declarations shared by the kernel translation units and
// the host runtime (not part of the public C ABI).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fft.cuh"

// Records the message returned by cfgpu_last_error() on this thread; returns code.
int cfgpu_record_error(int code, const std::string& msg);

// Undithered constants (version 0 only; one field).
constexpr Dither kNoDither{nullptr, 0, 0, 1, nullptr, nullptr, nullptr};

// Spectral curl (cheb_dct.cu): C6 = u, v, w, ox, oy, oz as Chebyshev coefficients, base flow (per field:
// Ub/Wb + field * bstride) added to the (0,0) mode.
template <typename R>
cudaError_t launch_curl_base(const GridDev& g, const double* U, R* C6, const double* Ub, const double* Wb,
                             int bstride, double Vsuck, cudaStream_t st);

// Chebyshev transforms along y through one complex FFT of length N - 1 per mode (cheb_dct.cu), for
// N - 1 = 8 N1, N1 in {4, 6, 8, 12, 16}.  Element (n, mode) of component c at in[c cs_in + n ld_in + mode]
// (complex units); modes split evenly over dt.nb fields.  tab = dct_table(N) (one version per field version).
bool dct_supported(int N);
std::vector<double> dct_table(int N);
template <typename R>
size_t dct_smem_bytes(int N);
template <typename R>
cudaError_t launch_dct(int N, bool inverse, int nmodes, int ncomp, const cpx<R>* in, size_t ld_in, size_t cs_in,
                       cpx<R>* out, size_t ld_out, size_t cs_out, const cpx<R>* tab, cudaStream_t st,
                       const Dither& dt = kNoDither);


size_t cheb_smem_bytes(int N, size_t rsize);

template <typename R>
size_t curl_cheb_smem_bytes(int N);
template <typename R>
cudaError_t launch_curl_cheb(const GridDev& g, int N, const double* U, R* W6, const R* CA, const R* CB, const R* DA,
                             const R* DB, const R* basey, double Vsuck, cudaStream_t st,
                             int bstride = 0, const Dither& dt = kNoDither);

// Lines split evenly over dt.nb fields (no block straddles two) when dithered.
template <typename TI, typename R, typename TO>
cudaError_t launch_cheb(int N, bool inverse, int nlines, int ncomp, const TI* in, size_t ld_in, size_t cs_in, TO* out,
                        size_t ld_out, size_t cs_out, const R* A, const R* B, cudaStream_t st,
                        const Dither& dt = kNoDither);

// Forward Chebyshev transform of FP32 lines on the tensor cores (cheb_tc.cu), N <= 128: Ag = cheb_tc_matrix
// (four BF16 splits of the N x N forward matrix, uploaded); err: device flag set if an MMA wait timed out.
bool cheb_tc_supported(int N);
std::vector<uint16_t> cheb_tc_matrix(const std::vector<double>& F, int N);
cudaError_t launch_cheb_tc(int N, int nlines, int ncomp, const float* in, size_t ld, size_t cs, float* out,
                           const void* Ag, int* err, cudaStream_t st);

// Nonlinear forms (values of the reference's NonlinearMethod enum, dnsflags.h:28-35)
enum { NL_ROTATIONAL = 0, NL_CONVECTION = 1, NL_DIVERGENCE = 2, NL_SKEW = 3 };

template <typename R>
size_t grad_cheb_smem_bytes(int N);
template <typename R>
cudaError_t launch_grad_cheb(const GridDev& g, int N, bool gradient, const double* U, R* W, const R* CA, const R* CB,
                             const R* DA, const R* DB, const R* basey, double Vsuck, cudaStream_t st,
                             int bstride = 0, const Dither& dt = kNoDither);
template <typename R>
size_t zphys_smem_bytes(const GridDev& g, int form, int RP);
// z pass of the x/z path (c2r, the form's products, r2c).  With twzf (the full-circle twiddle table
// exp(-2 pi i e / Nz), e < Nz) the FP32 rotational form runs with register-resident FFTs where Nz allows
// (launch_zrot, csrc/z_reg.cu), else the generic Stockham kernel.
template <typename R>
cudaError_t launch_zphys(const GridDev& g, int form, const FftPlan& pz, const cpx<R>* twz, int RP, const cpx<R>* X,
                         cpx<R>* Z, cudaStream_t st, const Dither& dt = kNoDither, const cpx<R>* twzf = nullptr);
// Rotational z pass with register FFTs, FP32 (Nz in {32, 48, 64, 96, 128}, RC x rows per CTA);
// cudaErrorNotSupported, with nothing launched, for other lengths or when switched off (set_zpass_register(0)).
cudaError_t launch_zrot(const GridDev& g, int RC, const cpx<float>* X, cpx<float>* Z, const cpx<float>* twzf,
                        cudaStream_t st, const Dither& dt);
void set_zpass_register(int enable);
template <typename R>
size_t cheb_fwd_div_smem_bytes(int N);
template <typename R>
cudaError_t launch_cheb_fwd_div(const GridDev& g, int N, const R* pF, const R* pKx, const R* pKz, const R* pD, R wF,
                                R wK, R wD, R* out, const R* FA, const R* FB, const R* DFA, const R* DFB,
                                cudaStream_t st, const Dither& dt = kNoDither);

// LinearAboutProfile term from u, v, w at the Gauss-Lobatto points (k_grad_cheb without base flow).
template <typename R>
cudaError_t launch_linprof(const GridDev& g, int N, const R* Y, const R* basey, int bstride, R* F, cudaStream_t st,
                           const Dither& dt = kNoDither);
// Rotation term added to the Chebyshev coefficients of N from the FP64 state U.
template <typename R>
cudaError_t launch_rotation(const GridDev& g, int N, const double* U, const double* Ub, int ustride, double rot,
                            double Vsuck, R* F, cudaStream_t st);

template <typename R>
size_t xfft_smem_bytes(const GridDev& g, int czc = 0);  // czc <= 0: all solved kz columns that fit

// x passes: czc kz columns per block (0: as many as fit in shared memory)
template <typename R>
cudaError_t launch_xinv(const GridDev& g, const FftPlan& px, const cpx<R>* twx, const cpx<R>* W, cpx<R>* X, int ncomp,
                        cudaStream_t st, int czc = 0, const Dither& dt = kNoDither);
template <typename R>
cudaError_t launch_xfwd(const GridDev& g, const FftPlan& px, const cpx<R>* twx, const cpx<R>* Z, cpx<R>* F, int ncomp,
                        cudaStream_t st, int czc = 0, const Dither& dt = kNoDither);

// Fused x/z pass of the rotational form (xz_fused.cu, xz_fused.cuh): one thread-block cluster of C CTAs per
// plane of gp, RC x rows per z chunk; W = u, v, w, ox, oy, oz at the Gauss-Lobatto points ([c][plane][mode]),
// F = the transformed product ([c][plane][mode]); twxf/twzf = full-circle tables exp(-2 pi i e/L) (version 0).
struct XzShape {
  int C = 0, RC = 0;
  double cost = 0.0;
};
bool xz_fused_supported(const GridDev& gp);
size_t xz_fused_smem(const GridDev& gp, int C, int RC, bool fp64);
std::vector<XzShape> xz_fused_candidates(const GridDev& gp, bool fp64);
cudaError_t launch_xz_rot(const GridDev& gp, int C, int RC, const cpx<float>* W, cpx<float>* F,
                          const cpx<float>* twxf, const cpx<float>* twzf, cudaStream_t st, const Dither& dt);
cudaError_t launch_xz_rot(const GridDev& gp, int C, int RC, const cpx<double>* W, cpx<double>* F,
                          const cpx<double>* twxf, const cpx<double>* twzf, cudaStream_t st, const Dither& dt);

// field2vector / vector2field on field f of a batch of fstride fields in the solved-mode layout (one-field
// grid g, dealiased): ord = solved-mode index of each vector block, blk = block of each mode; W: 2 Md Ny
// doubles of scratch.
cudaError_t launch_field2vector(const GridDev& g, int f, int fstride, const int* ord, int nblk, const double* U,
                                double* v, cudaStream_t st);
cudaError_t launch_vector2field(const GridDev& g, int f, int fstride, const int* blk, const double* v, double* U,
                                double* W, cudaStream_t st);

// Arnoldi step in FP64: w orthogonalised against the k rows of V (k x n, device), h[0..k-1] the projections,
// h[k] = |w|, w normalised.  work: (k + 1) * 64 + k + 1 doubles.
cudaError_t launch_orthogonalize(int n, int k, const double* V, double* w, double* h, double* work, cudaStream_t st);

// Advance every field's constant version (after a nonlinear evaluation).
cudaError_t launch_dither_bump(int* ver, int nb, cudaStream_t st);

// FlowField buffer(s) in host memory (nf fields of Nd components) <-> solved modes of fields f0.. of a
// batch of fstride fields on the device, read/written by the GPU directly (pageable memory through the
// host page tables).  g: the one-field grid.
cudaError_t launch_host_modes(const GridDev& g, bool to_device, int Nd, int nf, int f0, int fstride, const double* src,
                              double* dst, cudaStream_t st);

// ---------------------------------------------------------------------------
// Tau / Helmholtz per-mode tables (FP64), layout [field][n][m] with m the
// compact mode index (stride Md), plus per-mode scalars [s][m].
// ---------------------------------------------------------------------------
enum TauField {
  TF_PBAND = 0, TF_PUP, TF_PLO, TF_PINV,  // pressure Helmholtz UL factors (lambda = kappa^2, nu = 1)
  TF_VBAND, TF_VUP, TF_VLO, TF_VINV,      // velocity Helmholtz UL factors (lambda, nu)
  TF_PP, TF_VP, TF_PM, TF_VM, TF_P0, TF_V0,
  // segment products of the UL sweeps (tau_seg.cu; four segments of tau_seg_rows(N) rows per parity): H[n] =
  // prod of -up over rows i .. the segment's top, G[n] = prod of -lo inv over the segment's first row .. i
  TF_PH, TF_PG, TF_VH, TF_VG,
  TF_NFIELDS
};
enum TauScalar {
  TS_I00 = 0, TS_I01, TS_I10, TS_I11, TS_S0NB1, TS_S0NB, TS_UCMEAN, TS_LAMBDA,
  TS_KXL, TS_KZL,      // 2 pi kx / Lx, 2 pi kz / Lz
  TS_DX, TS_DZ,        // the same with the Nyquist modes' derivatives zero
  TS_KAPPA2,           // 4 pi^2 ((kx / Lx)^2 + (kz / Lz)^2)
  TS_RS0NB1, TS_RS0NB, // 1 / (1 - sigma0_Nb1), 1 / (1 - sigma0_Nb) (0 for the (0,0) mode)
  TS_NSCALARS
};

struct TauTable {
  double* f;  // [TF_NFIELDS][N][Md]
  double* s;  // [TS_NSCALARS][Md]
};

// Mode-independent Helmholtz right-hand-side matrices Be/Bo, packed by n:
// brow[n] holds the row of B that produces u[n]: lo, diag, up; row 0 is e0.
struct HelmB {
  const double* lo;
  const double* di;
  const double* up;
};

// Batched HelmholtzSolver: nsys systems, lines [n][nsys]; umean null: plain solve, else mean-constrained
// (mu out).  W: 7 N nsys doubles of work space.
cudaError_t launch_helmholtz(int N, int nsys, double a, double b, const double* lambda, double nu, const HelmB& hb,
                             const double* f, const double* ua, const double* ub, const double* umean, double* u,
                             double* mu, double* W, cudaStream_t st);

// Tables of modes m0 .. m0+mcount-1 of g (mcount <= 0: all modes) for lambda_t and nu.
cudaError_t launch_tau_setup(const GridDev& g, int N, double lambda_t, double nu, const HelmB& hb, TauTable tt,
                             double* scratch, cudaStream_t st, int m0 = 0, int mcount = 0);
// Up to 4 tables (the substeps of a scheme) in one launch; scratch holds 4 lines of N*Md doubles per table.
struct TauSetupBatch {
  double lambda_t[4];
  TauTable tab[4];
};
cudaError_t launch_tau_setup_batch(const GridDev& g, int N, const TauSetupBatch& tb, int ntab, double nu,
                                   const HelmB& hb, double* scratch, cudaStream_t st, int m0 = 0, int mcount = 0);

// Per-mode solve parameters for one substep.
struct SolveParams {
  int kind;          // 0 = multistep (SBDF/CNFE), 1 = CNAB-style substep, 2 = CNRK2 substep
  int order;         // multistep order
  double a[4], b[4]; // multistep: rhs = sum_j a_j u_j + b_j N_j
  // CNAB: rhs = lambda u + a_b L(u,q) - g_b N_j - z_b N_{j-1}
  double lam, a_b, g_b, z_b;
  // CNRK2: Q = A_j Q - N(u);  rhs = L(u,q) + lam u + B_C Q
  double rkA, B_C;
  double nu;
  int constraint;    // 0 = PressureGradient, 1 = BulkVelocity
  double dPdxRef, dPdzRef, umean, wmean;
  double baseShear[2];  // nu (U'(b) - U'(a)) / Ly and the same for W (bulk-velocity linear term)
  int taucorrection;
  int force_real00;  // NSE::solve keeps only the real part of the (0,0) mode
  int scheme;        // 0 main scheme, 1 start-up scheme (selects per-field coefficients)
  int substep;       // CNAB/RK substep j
};

// Per-field parameters of a heterogeneous field batch (one entry per field);
// they replace the SolveParams fields of the same names for that field's modes.
struct SlotParams {
  double nu, dPdxRef, dPdzRef, umean, wmean, baseShear[2];
  double a[4];       // multistep rhs coefficients -alpha_j / dt of this field's dt
  double lam[2][3];  // CNAB/RK lambda_t per substep of the main (0) and start-up (1) scheme at this dt
  int constraint;
  int pad;
};

#ifdef __CUDACC__
// A heterogeneous batch's per-field parameters over the launch-wide ones.
__device__ __forceinline__ void apply_slot(SolveParams& sp, const SlotParams& s) {
  sp.nu = s.nu;
  sp.constraint = s.constraint;
  sp.dPdxRef = s.dPdxRef;
  sp.dPdzRef = s.dPdzRef;
  sp.umean = s.umean;
  sp.wmean = s.wmean;
  sp.baseShear[0] = s.baseShear[0];
  sp.baseShear[1] = s.baseShear[1];
  if (sp.kind == 0) {
    for (int j = 0; j < 4; ++j) sp.a[j] = s.a[j];
  } else {
    sp.lam = s.lam[sp.scheme][sp.substep];
  }
}
#endif

struct SolvePtrs {
  const double* uin[4];  // multistep history u_j (3 comps each, complex [3][N][Md])
  const void* nin[4];    // N_j (R-typed, [3][N][Md] complex)
  const double* qin;     // pressure q (CNAB/RK linear term)
  double* uout;          // solution u (may alias uin[0] for CNAB/RK)
  double* qout;          // solution q
  void* Q;               // CNRK2 accumulator (R-typed)
  const double* Ubaseyy;
  const double* Wbaseyy;
  const double* Ubase;   // for the bulk-velocity linear term
  const double* Wbase;
  double* scratch;       // [8][N][2Md]
  double* dPdx_out;      // device scalars: actual dPdx, dPdz after solve ([field][2] for a batch)
  const SlotParams* slot;  // per-field parameters (null: SolveParams holds them for every field)
  int base_stride;         // 0: one base flow for all fields; N: Ubase/Wbase/Ubaseyy/Wbaseyy are [field][N]
};

// Kernel launches one launch_tau_solve makes for Ny = N (the right-hand-side kernel and the solve).
int tau_solve_launches(int N);
// Pressure / v and u / w passes of the step solve with segmented parity sweeps (tau_seg.cu), for
// tau_seg_rows(N) <= 17 (rows per segment lane); the right-hand sides Rx, Rz, Ry in scratch lines 0, 1, 2.
// set_tau_segmented(0) keeps the one-lane sweeps.
__host__ __device__ inline int tau_seg_rows(int N) { return ((N + 1) / 2 + 3) / 4; }
cudaError_t launch_tau_pvuw_seg(const GridDev& g, int N, const SolveParams& sp, const SolvePtrs& p,
                                const HelmB& hb, TauTable tt, cudaStream_t st);
void set_tau_segmented(int enable);
template <typename R>
cudaError_t launch_tau_solve(const GridDev& g, int N, const SolveParams& sp, const SolvePtrs& p, const HelmB& hb,
                             TauTable tt, cudaStream_t st);

// FieldSymmetry (s, sx, sy, sz, ax, az) (channelflow/symmetry.h) on [c][n][field][m] spectral fields of the
// per-field grid g (compact mode mapping); project = 1 gives (u + sigma u)/2.  out must not alias in.
struct SymmetryDev {
  int s, sx, sy, sz;
  double ax, az;
};
template <typename R>
cudaError_t launch_symmetry(const GridDev& g, int nb, int N, int ncomp, const SymmetryDev& sy, int project,
                            const void* in, void* out, cudaStream_t st);

// Diagnostics (diag.cu)
template <typename R>
cudaError_t launch_zcfl(const GridDev& g, const FftPlan& pz, const cpx<R>* twz, int RP, const cpx<R>* X,
                        const double* dyc, double dx, double dz, int nslot, unsigned long long* out, cudaStream_t st);
cudaError_t launch_l2norm2(const GridDev& g, int N, int ncomp, const double* U, double* out, cudaStream_t st);
double cfl_key_to_double(unsigned long long k);
int measure_fp64(int device_sms, double* tflops, double* cycles_per_fma);
