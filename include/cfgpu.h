/*
 * cfgpu.h -- C ABI of the GB300-native channelflow DNS time step.
 *
 * The library replaces the hot path of channelflow's C++ API: the DNS time
 * step (DNS / DNSFlags / NSE / TauSolver / HelmholtzSolver) with hand-written
 * sm_103a CUDA kernels.  Plain C types only: pointers, sizes, doubles.
 *
 * Field buffers exchanged with the host use the reference's serial
 * FlowField spectral layout (channelflow/flowfield.h:383-402): complex
 * values (re, im interleaved doubles) indexed [i][my][mx][mz], with
 * Mz = Nz/2+1, my the Chebyshev index, i the vector component.  Velocity
 * has Nd = 3, pressure q has Nd = 1.
 *
 * Only the (kx, kz) modes that the reference's NSE::solve updates (its
 * "solved set": |kx| <= Nx/3-1, kz <= Nz/3-1 with DealiasXZ; all but the
 * Nyquist modes without dealiasing) are held on the device.  Those modes are
 * read from the input buffers and written back; every other mode of the
 * caller's buffers is left untouched.  The nonlinear term is evaluated from
 * the solved modes only (the reference also uses any nonzero unsolved modes
 * of the input; they are zero for every field the reference's own DNS
 * produces from a padded field).
 *
 * Errors: every entry point returns a cfgpu_status; the reference's
 * cferror() exits the process instead (cfbasics/cfbasics.h:272-278).
 * cfgpu_last_error() returns a message for the last failure on the calling
 * thread.
 */
#ifndef CFGPU_H
#define CFGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int cfgpu_status;
enum {
  CFGPU_OK = 0,
  CFGPU_EINVAL = 1,    /* invalid argument (bad grid, flags, null pointer) */
  CFGPU_ENOMEM = 2,    /* device allocation failed */
  CFGPU_ECUDA = 3,     /* CUDA runtime error */
  CFGPU_ENOTSUP = 4,   /* option not implemented on the device path */
  CFGPU_ENONFINITE = 5 /* NaN or Inf detected in the state */
};

/* Arithmetic of the nonlinear term and transforms. */
enum { CFGPU_FP64 = 0, CFGPU_MIXED = 1 };

/* Enumerations with the reference's values (channelflow/dnsflags.h:24-38). */
enum { CFGPU_ZeroBase = 0, CFGPU_LinearBase, CFGPU_ParabolicBase, CFGPU_LaminarBase, CFGPU_SuctionBase,
       CFGPU_ArbitraryBase };
enum { CFGPU_PressureGradient = 0, CFGPU_BulkVelocity };
enum { CFGPU_CNFE1 = 0, CFGPU_CNAB2, CFGPU_CNRK2, CFGPU_SMRK2, CFGPU_SBDF1, CFGPU_SBDF2, CFGPU_SBDF3, CFGPU_SBDF4 };
enum { CFGPU_Rotational = 0, CFGPU_Convection, CFGPU_Divergence, CFGPU_SkewSymmetric, CFGPU_Alternating,
       CFGPU_Alternating_, CFGPU_LinearAboutProfile };
enum { CFGPU_NoDealiasing = 0, CFGPU_DealiasXZ, CFGPU_DealiasY, CFGPU_DealiasXYZ };

/* Geometry of a FlowField (FlowField(Nx,Ny,Nz,Nd,Lx,Lz,a,b), flowfield.h:60-70). */
typedef struct cfgpu_grid {
  int Nx, Ny, Nz;
  double Lx, Lz, a, b;
} cfgpu_grid;

/* The DNSFlags members used by the time step (channelflow/dnsflags.h:84-140). */
typedef struct cfgpu_flags {
  double nu, dPdx, dPdz, Ubulk, Wbulk;
  double ulowerwall, uupperwall, wlowerwall, wupperwall;
  double Vsuck, t0, dt;
  int baseflow, constraint, timestepping, initstepping, nonlinearity, dealiasing, taucorrection;
  double rotation; /* DNSFlags::rotation: dimensionless rotation about z (nse.cpp:62-78) */
} cfgpu_flags;

typedef struct cfgpu_dns_s* cfgpu_dns;

/*
 * FlowField on the GPU (channelflow/flowfield.h:52-345: construction, the spectral data, upload/download in
 * the serial layout complex [i][my][mx][mz]): the 2/3-dealiased modes of Nd = 1 or 3 components, in the
 * layout the DNS kernels use.  download zeroes the other modes.  cfgpu_dns_set/get_fields_device move a
 * DNS's velocity (Nd = 3) and pressure (Nd = 1) from/to such fields on the device (field `slot` of an
 * ensemble; either may be null).
 */
typedef struct cfgpu_field_s* cfgpu_field;
cfgpu_status cfgpu_field_create(const cfgpu_grid* grid, int Nd, cfgpu_field* out);
cfgpu_status cfgpu_field_upload(cfgpu_field f, const double* u);
cfgpu_status cfgpu_field_download(cfgpu_field f, double* u);
cfgpu_status cfgpu_field_destroy(cfgpu_field f);
cfgpu_status cfgpu_dns_set_fields_device(cfgpu_dns dns, int slot, cfgpu_field u, cfgpu_field q);
cfgpu_status cfgpu_dns_get_fields_device(cfgpu_dns dns, int slot, cfgpu_field u, cfgpu_field q);

/*
 * A whole FlowField on the GPU (every mode, Nyquist included) with the reference's transforms:
 * FlowField::makePhysical / makeSpectral and their _xz / _y halves (channelflow/flowfield.cpp:1850-1997),
 * in place, FP64.  The buffer is the reference's serial FlowField buffer (flowfield.h:370-400):
 * Nd*Ny*Nx*Nzpad doubles with Nzpad = 2*(Nz/2+1); xz-spectral data is complex [i][my][mx][mz], xz-physical
 * data real [i][ny][nx][nz] with rows of Nzpad.  The (xzstate, ystate) pair follows the reference
 * (fieldstate, cfbasics/mathdefs.h:77: Physical = 0, Spectral = 1); a transform to the current state does
 * nothing, makeSpectral runs xz then y, makePhysical y then xz.  Forward xz scales by 1/(Nx Nz); y uses the
 * chebyfft/ichebyfft scaling (chebyshev.cpp:262-303).  cfgpu_flowfield_data gives the device buffer.
 * Nx and Nz even, with no prime factor above 127 (factors 2, 3, 5 run as radix-2/3/4/5 stages, larger
 * primes as direct DFTs: FFTW takes every length).
 */
enum { CFGPU_PHYSICAL = 0, CFGPU_SPECTRAL = 1 };
typedef struct cfgpu_flowfield_s* cfgpu_flowfield;
cfgpu_status cfgpu_flowfield_create(const cfgpu_grid* grid, int Nd, cfgpu_flowfield* out);
cfgpu_status cfgpu_flowfield_destroy(cfgpu_flowfield f);
cfgpu_status cfgpu_flowfield_size(cfgpu_flowfield f, long long* ndoubles);
cfgpu_status cfgpu_flowfield_data(cfgpu_flowfield f, double** device_ptr);
cfgpu_status cfgpu_flowfield_upload(cfgpu_flowfield f, const double* host, int xzstate, int ystate);
cfgpu_status cfgpu_flowfield_download(cfgpu_flowfield f, double* host);
cfgpu_status cfgpu_flowfield_state(cfgpu_flowfield f, int* xzstate, int* ystate);
cfgpu_status cfgpu_flowfield_make_physical(cfgpu_flowfield f);
cfgpu_status cfgpu_flowfield_make_spectral(cfgpu_flowfield f);
cfgpu_status cfgpu_flowfield_make_physical_xz(cfgpu_flowfield f);
cfgpu_status cfgpu_flowfield_make_spectral_xz(cfgpu_flowfield f);
cfgpu_status cfgpu_flowfield_make_physical_y(cfgpu_flowfield f);
cfgpu_status cfgpu_flowfield_make_spectral_y(cfgpu_flowfield f);

/* TimeStep parameters (channelflow/dnsflags.h:166-198): dt within [dtmin, dtmax], dT = n dt the CFL-check
 * interval, CFL kept within [CFLmin, CFLmax] when variable != 0. */
typedef struct cfgpu_timestep {
  double dt, dtmin, dtmax, dT, CFLmin, CFLmax;
  int variable;
} cfgpu_timestep;

/* DNSFlags() defaults (channelflow/dnsflags.h:84-92, dnsflags.cpp:110-158). */
cfgpu_status cfgpu_flags_default(cfgpu_flags* flags);

/*
 * Builds a DNS on the current CUDA device: base flow, mean constraint,
 * per-mode tau tables for the main and the initialisation scheme.
 * Replaces DNS::DNS(fields, flags) (channelflow/dns.cpp:22-39) and, when
 * Ubase/Wbase are non-null (Ny Chebyshev coefficients each),
 * DNS::DNS(fields, base, flags) (channelflow/dns.cpp:41-62).  `u` is the
 * initial velocity in the layout above; it fixes the initial bulk velocity
 * and dPdx (NSE::initCFConstraint, channelflow/nse.cpp:634-671) but is not
 * stored: every advance call passes the fields.
 */
cfgpu_status cfgpu_dns_create(const cfgpu_grid* grid, const cfgpu_flags* flags, const double* Ubase,
                              const double* Wbase, const double* u, int precision, cfgpu_dns* out);

/*
 * DNS::advance(fields, nSteps) (channelflow/dns.cpp:135-163): copies u and q
 * (host buffers) to the device, takes nsteps steps (initialisation steps of
 * the init scheme first while the multistep history is not full), and
 * copies the new u and q back into the same buffers.
 */
cfgpu_status cfgpu_dns_advance(cfgpu_dns dns, double* u, double* q, int nsteps);

/* Device-resident variant: set the fields once, advance without host copies, read them back. */
cfgpu_status cfgpu_dns_set_fields(cfgpu_dns dns, const double* u, const double* q);
cfgpu_status cfgpu_dns_advance_resident(cfgpu_dns dns, int nsteps);
cfgpu_status cfgpu_dns_get_fields(cfgpu_dns dns, double* u, double* q);

/* DNS::reset_dt (channelflow/dns.cpp:191-196): rebuilds tau tables, restarts initialisation. */
cfgpu_status cfgpu_dns_reset_dt(cfgpu_dns dns, double dt);

/* DNS::time(), DNS::dPdx(), DNS::Ubulk() style queries (channelflow/dns.h:55-75). */
cfgpu_status cfgpu_dns_time(cfgpu_dns dns, double* t);
/* DNS::reset_time (channelflow/dns.cpp:199-205); reset_gradp / reset_bulkv (dns.cpp:221-232, NSE
 * nse.cpp:724-745): switch to the pressure-gradient or bulk-velocity constraint from the next step on,
 * keeping the base flow (not for ensembles with per-field parameters).  cfgpu_dns_constraint: v[6] =
 * {Ubulk, Wbulk (NSE::UbulkAct_, set from the initial field at construction, nse.cpp:645), UbulkRef,
 * WbulkRef, dPdxRef, dPdzRef} (dns.cpp:306-330). */
cfgpu_status cfgpu_dns_reset_time(cfgpu_dns dns, double t);
cfgpu_status cfgpu_dns_reset_gradp(cfgpu_dns dns, double dPdx, double dPdz);
cfgpu_status cfgpu_dns_reset_bulkv(cfgpu_dns dns, double Ubulk, double Wbulk);
cfgpu_status cfgpu_dns_constraint(cfgpu_dns dns, double* v);
cfgpu_status cfgpu_dns_dPdx(cfgpu_dns dns, double* dPdx);

/*
 * DNS::CFL(u) (channelflow/dnsalgo.cpp:63-67 with FlowField::CFLfactor,
 * flowfield.cpp:4035-4068) of the current velocity: the signed maximum over
 * grid points and components of (u_i + U_i)/dx_i, times 2 pi/3 dt with
 * DealiasXZ (pi dt otherwise).  Needs Ny <= 111.
 */
cfgpu_status cfgpu_dns_cfl(cfgpu_dns dns, double* cfl);
/* navierstokesNL (channelflow/nse.h:20, nse.cpp:12-91) plus NSE::nonlinear's zeroPaddedModes
 * (nse.cpp:383-391): f = N(u) with the DNS's base flow, nonlinearity, Vsuck and rotation flags, in its
 * precision.  u and f: FlowField buffers of the DNS's nfields velocity fields; the DNS's own fields are not
 * touched (an Alternating form flips, as the reference's flag does). */
cfgpu_status cfgpu_dns_nonlinear(cfgpu_dns dns, const double* u, double* f);

/*
 * field2vector / vector2field (channelflow/flowfield.h:617-620, flowfield.cpp:4448-4760): the vector of the
 * independent real coefficients of a divergence-free, no-slip velocity field (2/3-dealiased modes), the
 * unknowns of cfDSI's Newton-Krylov searches (cfdsi.cpp:52-61).  vector2field rebuilds the other
 * coefficients from the wall conditions and continuity and zeroes every other mode.  The _ensemble forms
 * act on a field resident on the GPU (slot of an ensemble or the field of a DNS; the pressure is kept).
 */
/* The Arnoldi step of GMRES in FP64 on the GPU (nsolver/gmres.cpp:47-83 orthogonalises the new Krylov
 * vector against the basis): w (n) is orthogonalised against the k rows of V (k x n, row-major) by classical
 * Gram-Schmidt applied twice; h[j] = w.V_j summed over both passes (j < k), h[k] = |w| after, and w is
 * normalised (unless h[k] == 0).  Host arrays. */
cfgpu_status cfgpu_orthogonalize(int n, int k, const double* V, double* w, double* h);
cfgpu_status cfgpu_field2vector_size(const cfgpu_grid* grid, long long* n);
cfgpu_status cfgpu_field2vector(const cfgpu_grid* grid, const double* u, double* v);
cfgpu_status cfgpu_vector2field(const cfgpu_grid* grid, const double* v, double* u);
cfgpu_status cfgpu_ensemble_field2vector(cfgpu_dns dns, int slot, double* v);
cfgpu_status cfgpu_ensemble_vector2field(cfgpu_dns dns, int slot, const double* v);

/* L2Norm(field, normalize=true) (channelflow/diffops.cpp:415-487) of the current u (field 0) or q (field 1). */
cfgpu_status cfgpu_dns_l2norm(cfgpu_dns dns, int field, double* l2);

/* Base flow Chebyshev coefficients (NSE::Ubase/Wbase, channelflow/nse.cpp:766-767); Ny doubles each. */
cfgpu_status cfgpu_dns_base(cfgpu_dns dns, double* Ubase, double* Wbase);

/* Number of solved (kx, kz) modes held on the device. */
cfgpu_status cfgpu_dns_num_modes(cfgpu_dns dns, int* nmodes);

/* Device bytes held by this DNS. */
cfgpu_status cfgpu_dns_device_bytes(cfgpu_dns dns, long long* bytes);

/* Launch count of the library's kernels since create (diagnostics). */
cfgpu_status cfgpu_dns_kernel_launches(cfgpu_dns dns, long long* launches);

cfgpu_status cfgpu_dns_destroy(cfgpu_dns dns);

/*
 * Timing (no reference counterpart; the reference times dns.advance with
 * gettimeofday, tools/benchmark.cpp:122-149).  cfgpu_dns_advance_timed runs
 * cfgpu_dns_advance_resident bracketed by CUDA events on the DNS's stream and
 * returns the device time in milliseconds.  With profiling enabled, every
 * nonlinear-term pass and every tau solve is bracketed by events too;
 * cfgpu_dns_phase_times returns their accumulated milliseconds and counts
 * since the last reset (and resets them).
 */
cfgpu_status cfgpu_dns_advance_timed(cfgpu_dns dns, int nsteps, double* ms);
/*
 * FieldSymmetry (channelflow/symmetry.h): sigma (u,v,w)(x,y,z) = s (sx u, sy v, sz w)(sx x + ax Lx, sy y,
 * sz z + az Lz), signs +-1, ax and az shifts in units of Lx and Lz.
 */
typedef struct cfgpu_symmetry {
  int s, sx, sy, sz;
  double ax, az;
} cfgpu_symmetry;

/* DNSFlags::symmetries and symmetryprojectioninterval: DNS::advance projects the velocity and the scheme's
 * stored fields onto the symmetric subspace when (int)time % interval == 0 (channelflow/dns.cpp:151-155,
 * dnsalgo.cpp:255-262, 628-632).  n = 0 removes them. */
cfgpu_status cfgpu_dns_set_symmetries(cfgpu_dns dns, const cfgpu_symmetry* syms, int n, int interval);
/* u <- sigma u (project = 0, FlowField::operator*=) or (u + sigma u)/2 (project = 1, FlowField::project)
 * for the resident velocity of every field (channelflow/flowfield.cpp:1095-1272). */
cfgpu_status cfgpu_dns_symmetry(cfgpu_dns dns, const cfgpu_symmetry* sym, int project);
/* The same on a host FlowField buffer (Nd = 1 or 3, spectral layout), over the modes |kx| <= Nx/3-1,
 * kz <= Nz/3-1 (dealias != 0, a padded field) or all but the Nyquist modes; other modes are untouched. */
cfgpu_status cfgpu_field_symmetry(const cfgpu_grid* grid, int dealias, int Nd, const cfgpu_symmetry* sym,
                                  int project, double* u);

/*
 * Steady-state main-scheme steps are captured once per buffer-rotation state as CUDA graphs and replayed
 * (one launch per step); enable = 0 launches every kernel eagerly.  Default on; graphs are not used while
 * profiling is on or with the Alternating nonlinearity.
 */
cfgpu_status cfgpu_dns_set_graphs(cfgpu_dns dns, int enable);

/* Block shapes of the FFT passes (kz columns per block of the x passes, x rows per block of the z pass) are
 * chosen at DNS creation by timing candidates on the DNS's own arrays, cached per grid shape, for grids with
 * Ny * Nx * (Kz+1) >= 200000 planes' worth of work; results do not depend on the choice.  enable = 0 makes
 * later DNS objects use the defaults and clears the cache. */
cfgpu_status cfgpu_set_autotune(int enable);
/* No reference counterpart: DNS objects created while enable != 0 (the default) run the rotational form's
 * x and z transforms and product as one fused kernel per step (a thread-block cluster per y-plane,
 * distributed shared memory) when the grid allows (Nx, Nz in {32, 48, 64, 96, 128}); otherwise as three
 * kernels. Both give the same results to rounding.  With enable == 1 the fused kernel's launch shapes are
 * timed against the three kernels and the faster kept; enable == 2 keeps the fused kernel wherever the grid
 * allows (its shapes still timed), e.g. for profiling runs, whose timings can favour the other form. */
cfgpu_status cfgpu_set_fused_xz(int enable);
/* No reference counterpart: programmatic dependent launch between the kernels of a step (a kernel's launch
 * and set-up overlap the previous kernel's tail; it waits for that kernel's results before reading them).
 * On by default; applies to launches made afterwards (a DNS captures its step graphs on its first steps). */
cfgpu_status cfgpu_set_pdl(int enable);
/* No reference counterpart: the mixed path's rotational z pass in the three-kernel x/z path with
 * register-resident four-step FFTs (enable != 0, the default; Nz in {32, 48, 64, 96, 128}) or with the generic
 * shared-memory Stockham FFT (always in FP64).  Both give the same results to rounding.  Applies to launches
 * made afterwards; a DNS replays the step graphs it captured on its first steps, so set it before creating
 * the DNS objects whose results are to be compared bit for bit. */
cfgpu_status cfgpu_set_register_zpass(int enable);
/* No reference counterpart: the Chebyshev transforms of the rotational form's nonlinear term (the inverse
 * transform of u and curl u, the forward transform of the product) run either as dense parity-split matrix
 * products or through one complex FFT of length Ny - 1 per mode (Ny - 1 in {32, 48, 64, 96, 128}).  For DNS
 * objects created afterwards: mode 0 matrix products; 1 (the default) both timed at creation on the DNS's own
 * arrays, the faster kept (cached per grid shape and precision); 2 the FFT wherever the grid allows.  Both
 * give the same results to rounding.  cfgpu_dns_cheb_fft reports a DNS's choice (1 FFT, 0 matrix). */
cfgpu_status cfgpu_set_cheb_fft(int mode);
/* No reference counterpart: the per-mode step solve (TauSolver::solve) runs its parity sweeps split over
 * four lanes each (first-order recurrences joined across segments; the default, for Ny <= 135) or one lane
 * per sweep (enable = 0).  Both give the same results to rounding.  Affects solves launched afterwards (a
 * DNS captures its step graphs on its first steps). */
cfgpu_status cfgpu_set_tau_segmented(int enable);
/* No reference counterpart: the mixed path's forward Chebyshev transform (rotational and convection forms,
 * Ny <= 128) on the tensor cores (BF16 splits of the FP32 data and of the constant matrix, FP32 accumulation)
 * instead of compensated FP32 matrix products.  For DNS objects created afterwards: mode 0 never, 1 (the
 * default) timed against the matrix products at creation (cached per grid shape), 2 always.
 * cfgpu_dns_cheb_tensor reports a DNS's choice. */
cfgpu_status cfgpu_set_cheb_tensor(int mode);
cfgpu_status cfgpu_dns_cheb_tensor(cfgpu_dns dns, int* on);
cfgpu_status cfgpu_dns_cheb_fft(cfgpu_dns dns, int* fft);
/* Host FlowField buffers: on devices whose kernels reach pageable host memory through the host page
 * tables (GB300 over NVLink-C2C), DNS objects created while enable != 0 (the default) read and write the
 * caller's buffers with one kernel each way; otherwise through host-side gathers and pinned staging
 * copies.  cfgpu_dns_host_access reports which path a DNS uses (1 direct, 0 staged). */
cfgpu_status cfgpu_set_host_access(int enable);
cfgpu_status cfgpu_dns_host_access(cfgpu_dns dns, int* direct);
/* No reference counterpart (the reference's FlowField data is plain pageable memory): page-lock a caller's
 * host buffer (e.g. a FlowField's data array kept for many advance calls) and map it for every device
 * (cudaHostRegister, portable and mapped); unregister before freeing the buffer.  The host-buffer transfers of
 * cfgpu_dns_advance / set_fields / get_fields take the same path for it (direct kernels where the device
 * reaches pageable memory, staged copies elsewhere); on GB300 the two run at the same rate.  Takes no device
 * memory.  Registering a buffer twice, or unregistering one that was not registered, is CFGPU_EINVAL. */
cfgpu_status cfgpu_host_register(void* ptr, size_t bytes);
cfgpu_status cfgpu_host_unregister(void* ptr);
cfgpu_status cfgpu_dns_set_profiling(cfgpu_dns dns, int enable);
cfgpu_status cfgpu_dns_phase_times(cfgpu_dns dns, double* nl_ms, long long* nl_count, double* tau_ms,
                                   long long* tau_count);

/*
 * Ensembles: nfields independent fields with one grid and one set of flags
 * (the same base flow, constraint, nu and dt) advanced together, every kernel
 * launch covering all of them (no reference counterpart; the reference runs
 * one DNS per field, e.g. programs/edgetracking.cpp:488-525).  The handle is
 * a cfgpu_dns: cfgpu_dns_set_fields/get_fields/advance then take nfields
 * consecutive FlowField buffers, cfgpu_dns_advance_resident advances all of
 * them, and cfgpu_dns_reset_dt/time apply to all.  Each field's arithmetic is
 * the same as in a single-field DNS.  The per-field accessors below address
 * one slot (0 <= slot < nfields); cfl, l2 and dPdx receive nfields values.
 * Multistep schemes share one start-up phase: fields written into a slot
 * after the first step join the running history (use the whole-ensemble
 * setters, or a self-starting scheme, to restart them cleanly).
 */
cfgpu_status cfgpu_ensemble_create(const cfgpu_grid* grid, const cfgpu_flags* flags, int nfields, int precision,
                                   cfgpu_dns* out);
cfgpu_status cfgpu_ensemble_size(cfgpu_dns dns, int* nfields);
cfgpu_status cfgpu_ensemble_set_field(cfgpu_dns dns, int slot, const double* u, const double* q);
cfgpu_status cfgpu_ensemble_get_field(cfgpu_dns dns, int slot, double* u, double* q);
cfgpu_status cfgpu_ensemble_cfl(cfgpu_dns dns, double* cfl);
cfgpu_status cfgpu_ensemble_l2norm(cfgpu_dns dns, int field, double* l2);
cfgpu_status cfgpu_ensemble_dPdx(cfgpu_dns dns, double* dPdx);

/*
 * Per-field parameters: field `slot` gets its own nu, dt, base flow (from flags->baseflow and the
 * walls, or Ubase/Wbase Chebyshev coefficients when both are non-null) and constraint (type,
 * dPdx/dPdz or Ubulk/Wbulk), as NSE::createCFBaseFlow / initCFConstraint (channelflow/nse.cpp:589-671)
 * compute them for a DNS with those flags; that field's tau tables and scheme coefficients are
 * recomputed for its nu and dt exactly as a single-field DNS computes them.  The schemes, the
 * nonlinearity, dealiasing, taucorrection and Vsuck stay those of the ensemble (CFGPU_EINVAL
 * otherwise); the ensemble's time (cfgpu_dns_time) advances by the ensemble's dt.  Changing a field's
 * dt does not restart its start-up steps (restart it through a one-field DNS and
 * cfgpu_ensemble_load_slot).  Needs Ny <= 111.
 */
cfgpu_status cfgpu_ensemble_set_params(cfgpu_dns dns, int slot, const cfgpu_flags* flags, const double* Ubase,
                                       const double* Wbase);

/*
 * Continuous batching: copy the complete time-stepping state of the single-field DNS `src` (velocity,
 * pressure, multistep history or CNAB nonlinear terms, dPdx) into field `slot`.  src must have the
 * ensemble's grid, precision, scheme, dt and nonlinearity, and both must be past their start-up
 * steps (DNS::advance's init stepping, channelflow/dns.cpp:156-160): a request starts alone, then
 * joins the batch, and its later steps are the steps it would have taken alone.  Set the slot's
 * parameters (cfgpu_ensemble_set_params) to src's flags first.  An ensemble that has not run its own
 * start-up steps runs main-scheme steps from the first load on (its fields are expected to arrive
 * through this call).
 */
cfgpu_status cfgpu_ensemble_load_slot(cfgpu_dns dns, int slot, cfgpu_dns src);

/*
 * Request server (no reference counterpart; it serves the DNS integrations and f^T(u) evaluations
 * that programs/simulateflow.cpp, cfDSI::f (channelflow/cfdsi.cpp:705-775) and the nsolver drivers
 * run one at a time).  A request is nsteps fixed-dt steps of one field from the FlowField buffer u
 * (cfgpu_server_submit), or f^T(u) with a TimeStep (cfgpu_server_submit_ft).  Requests with the same
 * grid, schemes, nonlinearity, dealiasing, taucorrection and Vsuck share field ensembles of up to
 * `slots` fields (per-field nu, dt, base flow and constraint; a new ensemble is sized to the requests
 * of its key waiting at that moment); new requests are
 * admitted into free slots while others run (continuous batching), new ensembles only while their
 * estimated device bytes fit in max_bytes.  Each ensemble is driven by its own host thread, which
 * loads new requests into its slots (start-up steps in a one-field staging DNS), advances its fields in
 * chunks of at most max_steps steps on its own stream and handles interval ends and finished requests;
 * cfgpu_server_pump is the admission round (it waits up to 2 ms for progress) and sets max_steps;
 * *active = requests queued or running.  cfgpu_server_poll: *status 0 queued, 1 running, 2 done,
 * 3 failed (returns CFGPU_ENONFINITE); u receives the result when done; times = {submit, start, done}
 * in seconds of a monotonic clock.  stats = {device bytes, ensembles, slots, running, queued,
 * ensemble steps, field steps, chunks enqueued, dt changes, microseconds in admission, microseconds in
 * interval ends, microseconds creating ensembles, setting staging parameters, running staging steps,
 * loading slots} (15 values; "ensembles" counts those created; host times are summed over the server's
 * threads).  The calls take the server's lock; one thread at a time may call destroy.
 */
typedef struct cfgpu_server_s* cfgpu_server;
cfgpu_status cfgpu_server_create(long long max_bytes, int slots, int precision, cfgpu_server* out);
cfgpu_status cfgpu_server_submit(cfgpu_server srv, const cfgpu_grid* grid, const cfgpu_flags* flags, int nsteps,
                                 const double* u, long long* id);
/* f^T(u) request: the result equals cfgpu_ft(grid, flags, timestep, T, u, ...) run alone (CFL probe and
 * dT-interval dt adjustments included when timestep->variable). T > 0. */
cfgpu_status cfgpu_server_submit_ft(cfgpu_server srv, const cfgpu_grid* grid, const cfgpu_flags* flags,
                                    const cfgpu_timestep* timestep, double T, const double* u, long long* id);
cfgpu_status cfgpu_server_pump(cfgpu_server srv, int max_steps, int* active);
cfgpu_status cfgpu_server_poll(cfgpu_server srv, long long id, int* status, double* u, double* times);
cfgpu_status cfgpu_server_release(cfgpu_server srv, long long id);
cfgpu_status cfgpu_server_stats(cfgpu_server srv, long long* stats);
cfgpu_status cfgpu_server_destroy(cfgpu_server srv);

/*
 * TimeStep::adjust_for_T (channelflow/dnsflags.cpp:912-965): fits dT and dt to the horizon T; returns
 * n (steps per dT), N (dT intervals) and dt = dT/n, and updates ts->dt, ts->dT.
 */
cfgpu_status cfgpu_timestep_adjust_for_T(cfgpu_timestep* ts, double T, int* n, int* N, double* dt);

/*
 * TimeStep::adjust(CFL) (channelflow/dnsflags.cpp:811-859): when variable and CFL is outside
 * [CFLmin, CFLmax], moves dt = dT/n so that the CFL number returns to the middle of the range;
 * updates ts->dt, returns n and whether it changed.
 */
cfgpu_status cfgpu_timestep_adjust(cfgpu_timestep* ts, double cfl, int* n, int* adjusted);

/*
 * f^T(u): the time-T map used by the Newton-Krylov, Arnoldi and continuation
 * drivers, cfDSI's f(u, T, ...) without a Poincare section
 * (channelflow/cfdsi.cpp:705-775): adjust dt to T, build a DNS, optionally
 * probe the CFL number with one step and restart from u with the adjusted dt,
 * then advance N intervals of n steps, adjusting dt from the CFL number of
 * each interval when timestep->variable.  u and fu are velocity buffers in
 * the FlowField layout; the final CFL number is returned in *cfl (may be null).
 */
cfgpu_status cfgpu_ft(const cfgpu_grid* grid, const cfgpu_flags* flags, const cfgpu_timestep* timestep, double T,
                      const double* u, double* fu, double* cfl, int precision);

/*
 * channelflow's binary FlowField format (.ff): FlowField::binarySave and the
 * FlowField(filebase) constructor's binary branch (channelflow/flowfield.cpp:2642-2723, 216-356).
 * data is the FlowField's spectral storage, complex [Nd][Ny][Nx][Nz/2+1] (2*Nd*Ny*Nx*(Nz/2+1) doubles).
 * padded != 0 writes only the 2/3-rule modes (the caller's aliased modes must be zero).
 * cfgpu_ff_read_header returns dims = {Nx, Ny, Nz, Nd}, geom = {Lx, Lz, a, b}, the padded flag and the
 * two state characters ('S' spectral, 'P' physical); cfgpu_ff_read reads spectral-state files only
 * (CFGPU_ENOTSUP otherwise) and zero-fills the modes a padded file omits.
 */
cfgpu_status cfgpu_ff_write(const char* path, int Nx, int Ny, int Nz, int Nd, double Lx, double Lz, double a,
                            double b, int padded, const double* data);
cfgpu_status cfgpu_ff_read_header(const char* path, int* dims, double* geom, int* padded, char* state);
cfgpu_status cfgpu_ff_read(const char* path, double* data, size_t ndoubles);

/*
 * HelmholtzSolver(N, a, b, lambda_s, nu).solve(u_s, f_s, ua_s, ub_s) (channelflow/helmholtz.h:29-38,
 * helmholtz.cpp:18-95) for nsys systems at once: nu u'' - lambda_s u = f_s, u(a) = ua_s, u(b) = ub_s (ua/ub
 * may be null: zero).  f and u are [nsys][N] Chebyshev coefficients (ChebyCoeff data per system); N odd.
 * The _mean variant is solve(u, mu, f, umean, ua, ub) (helmholtz.cpp:158-213): mu_s is chosen so that
 * mean(u_s) = umean_s with nu u'' - lambda u = f + mu.
 */
cfgpu_status cfgpu_helmholtz_solve_batched(int N, int nsys, double a, double b, const double* lambda, double nu,
                                           const double* f, const double* ua, const double* ub, double* u);
cfgpu_status cfgpu_helmholtz_solve_mean_batched(int N, int nsys, double a, double b, const double* lambda, double nu,
                                                const double* f, const double* umean, const double* ua,
                                                const double* ub, double* u, double* mu);

/*
 * Batched TauSolver (channelflow/tausolver.cpp:81-176 constructor and
 * 347-402 solve): for nmodes modes (kx[k], kz[k]) of one geometry, solves
 *   nu (u'' - kappa^2 u) - lambda u - grad P = -R,  div u = 0,  u(a)=u(b)=0
 * with lambda = lambda_t + nu kappa^2 (NSE::reset_lambda, nse.cpp:683-700).
 * Profiles are complex Chebyshev coefficients [k][n] (re, im interleaved),
 * N odd.  The (0,0) mode uses the reference's degenerate branch (v = 0).
 */
cfgpu_status cfgpu_tau_solve_batched(int N, int nmodes, const int* kx, const int* kz, double Lx, double Lz, double a,
                                     double b, double lambda_t, double nu, int taucorrection, const double* Rx,
                                     const double* Ry, const double* Rz, double* u, double* v, double* w, double* P);

/*
 * Batched tau solve that allocates nothing (no counterpart in the reference:
 * channelflow solves per mode on the CPU and never touches GPU memory).
 *
 * Same arguments, host buffers and results as cfgpu_tau_solve_batched, but
 * it calls no cudaMalloc/cudaFree: all device working memory comes from one
 * static array of CFGPU_NOALLOC_BYTES (16 MiB) in the library's device code.
 * It is for callers that must not allocate GPU memory: processes whose GPU
 * memory is fully reserved by another allocator (a framework's pool, a fixed
 * budget on a shared GPU), and latency-sensitive loops that cannot pay for
 * allocation.
 *
 * When the array is reserved: with the CUDA runtime's default lazy module
 * loading, at the first call of this function on a device; with
 * CUDA_MODULE_LOADING=EAGER, when the context is created.  From then on that
 * device holds it until the process exits.  Make the first call (any size)
 * before another allocator takes the device's memory; if the array cannot be
 * reserved the call returns CFGPU_ENOMEM and says so in cfgpu_last_error().
 *
 * Limit: 54*N*nmodes + 9*nmodes + 4*N doubles must fit in the array, e.g.
 * N = 49 allows nmodes <= 789, N = 97 allows nmodes <= 399; larger requests
 * return CFGPU_EINVAL with the sizes in cfgpu_last_error().
 * The first call on a device (with that device current) looks up the array's
 * device address; make that first call before any stream capture.  Every
 * call on a device reuses the same array, and calls run on the legacy
 * default stream: calls that overlap on the GPU (from several host threads)
 * race on it.
 */
#define CFGPU_NOALLOC_BYTES (16u << 20)
cfgpu_status cfgpu_tau_solve_batched_noalloc(int N, int nmodes, const int* kx, const int* kz, double Lx, double Lz,
                                             double a, double b, double lambda_t, double nu, int taucorrection,
                                             const double* Rx, const double* Ry, const double* Rz, double* u,
                                             double* v, double* w, double* P);

/*
 * FP64 microbenchmark of the current device (no reference counterpart):
 * sustained FMA throughput in TFLOP/s (8 independent chains per thread, 8
 * blocks per SM) and the latency of one dependent FMA chain in cycles.  The
 * FP64 kernels' roofline denominator.
 */
cfgpu_status cfgpu_measure_fp64(double* tflops, double* cycles_per_fma);

/*
 * The CFGPU_DITHER_VERSIONS FP32 versions of the constant x that the mixed
 * precision passes cycle through, one per nonlinear evaluation (no reference
 * counterpart; host only, no device call): a stratified stochastic rounding
 * between the two floats that bracket x, whose mean is x to 1/(2 V) of the
 * float spacing.  versions holds CFGPU_DITHER_VERSIONS floats.
 */
#define CFGPU_DITHER_VERSIONS 64
cfgpu_status cfgpu_dither_versions(double x, float* versions);

/* Library version string. */
const char* cfgpu_version(void);

/* Message for the last error on the calling thread. */
const char* cfgpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* CFGPU_H */
