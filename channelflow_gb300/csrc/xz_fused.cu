// Fused x/z pass of the rotational nonlinear term: one thread-block cluster per y-plane.
//
// Restates, for the solved modes of one y-plane (makePhysical_xz, the pointwise cross product of
// rotationalNL and makeSpectral_xz; channelflow/flowfield.cpp:1850-1886, diffops.cpp:2560-2611, 2852-2881):
//   six components u, v, w, ox, oy, oz (complex, solved (kx, kz), at one Gauss-Lobatto point y)
//   -> inverse complex FFT along x of every solved kz column
//   -> c2r along z of every x row (two real rows packed in one complex FFT), f = omega x u pointwise,
//      r2c along z (again two real rows per complex FFT), kz <= Kz kept
//   -> forward complex FFT along x, solved kx kept, scaled by 1/(Nx Nz).
//
// GB300 mapping.  A cluster of C CTAs (thread-block cluster, distributed shared memory) holds the plane:
//   phase 1  CTA r transforms the kz columns it owns (all six components) along x, in its own shared memory;
//   phase 2  CTA r takes the x rows it owns, gathers their kz bins from every CTA of the cluster (DSMEM
//            loads), does the z transforms and the product, and scatters the three result components back
//            into the owning CTAs' shared memory, over the very slots it read (each slot is read by exactly
//            one CTA, so the overwrite is safe without extra barriers);
//   phase 3  CTA r transforms its columns of the result along x and writes the solved modes to HBM.
// The plane is read from HBM once and the result written once; nothing in between leaves the cluster.
//
// FFTs: four-step, L = N1 * 8 (N1 in {4, 6, 8, 12, 16}: L in {32, 48, 64, 96, 128}).  Pass "S" (stride):
// N1 threads per sequence, 8 points each at stride N1; pass "B" (block): 8 threads per sequence, N1
// contiguous points each.  Every thread transforms its points in registers (compile-time mixed-radix DIF,
// radices 4, 2, 3), so a transform costs two shared-memory round trips.  Sequences are padded by one slot
// per N1 (index p -> p + p / N1) so the stride-N1 and the block accesses are free of bank conflicts.
//   inverse: natural order in -> out at pos(k) = (N1 + 1) (k % 8) + k / 8      (pass S, then pass B)
//   forward: in at pos(x) -> natural order out (padded)                        (pass B, then pass S)
// Twiddles come from a full-circle table exp(-2 pi i e / L), e < L, staged in shared memory per field:
// on the mixed path it is one of the DITHER_V dithered versions (the field's current one), so every
// non-trivial constant of the transform, the internal ones of the radix-3 DFT included, is dithered.
#include <cooperative_groups.h>

#include <type_traits>

#include "kernels.h"

namespace cg = cooperative_groups;

namespace {

constexpr int XZ_THREADS = 512;
constexpr int XZ_MAX_NKZ = 64;

__host__ __device__ constexpr int dif_radix(int L) {
  return L % 4 == 0 && L != 8 ? 4 : (L % 2 == 0 ? 2 : (L % 3 == 0 ? 3 : 1));
}
// Frequency index held at register position pos after the in-place DIF of length L.
__host__ __device__ constexpr int dif_out(int pos, int L) {
  return L == 1 ? 0 : pos / (L / dif_radix(L)) + dif_radix(L) * dif_out(pos % (L / dif_radix(L)), L / dif_radix(L));
}

// f(integral_constant<int, I>) for I = B .. E-1, so that per-index constants fold at compile time.
template <int B, int E, class Fn>
__device__ __forceinline__ void static_for(Fn&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

template <typename R, int SIGN>
__device__ __forceinline__ cpx<R> twd(const cpx<R>* tw, int e) {
  cpx<R> w = tw[e];
  if (SIGN > 0) w.y = -w.y;
  return w;
}

// r-point DFT of a[0..r) with sign SIGN (-1 forward, +1 inverse); e3 = table index of exp(-2 pi i / 3).
template <typename R, int RAD, int SIGN>
__device__ __forceinline__ void small_dft(cpx<R>* a, const cpx<R>* tw, int e3) {
  if constexpr (RAD == 2) {
    const cpx<R> t = a[0];
    a[0] = cadd(t, a[1]);
    a[1] = csub(t, a[1]);
  } else if constexpr (RAD == 4) {
    const cpx<R> s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
    const cpx<R> s13 = cadd(a[1], a[3]), d13 = csub(a[1], a[3]);
    // SIGN * i * d13
    const cpx<R> id = SIGN > 0 ? cmk<R>(-d13.y, d13.x) : cmk<R>(d13.y, -d13.x);
    a[0] = cadd(s02, s13);
    a[2] = csub(s02, s13);
    a[1] = cadd(d02, id);
    a[3] = csub(d02, id);
  } else {
    static_assert(RAD == 3, "radix");
    // omega = exp(SIGN 2 pi i / 3) = -1/2 + SIGN i h, h = sqrt(3)/2 = -Im(table[L/3])
    const R h = -tw[e3].y;
    const cpx<R> s = cadd(a[1], a[2]), d = csub(a[1], a[2]);
    const cpx<R> m = cmk<R>(a[0].x - (R)0.5 * s.x, a[0].y - (R)0.5 * s.y);
    const cpx<R> t = SIGN > 0 ? cmk<R>(-h * d.y, h * d.x) : cmk<R>(h * d.y, -h * d.x);
    a[0] = cadd(a[0], s);
    a[1] = cadd(m, t);
    a[2] = csub(m, t);
  }
}

template <typename R, int L, int OFF, int SIGN>
__device__ __forceinline__ void dif_reg(cpx<R>* x, const cpx<R>* tw, int ts);

template <typename R, int M, int OFF, int SIGN, int J, int RR>
__device__ __forceinline__ void dif_sub(cpx<R>* x, const cpx<R>* tw, int ts) {
  if constexpr (J < RR) {
    dif_reg<R, M, OFF + J * M, SIGN>(x, tw, ts);
    dif_sub<R, M, OFF, SIGN, J + 1, RR>(x, tw, ts);
  }
}

// In-place decimation-in-frequency DFT of x[OFF .. OFF+L) held in registers; the table entry of
// exp(-2 pi i / L) is tw[ts] (ts = table length / L).  Output frequency dif_out(p, L) at position OFF + p.
template <typename R, int L, int OFF, int SIGN>
__device__ __forceinline__ void dif_reg(cpx<R>* x, const cpx<R>* tw, int ts) {
  if constexpr (L > 1) {
    constexpr int RAD = dif_radix(L), M = L / RAD;
    static_assert(RAD > 1, "length must factor into 2 and 3");
#pragma unroll
    for (int i = 0; i < M; ++i) {
      cpx<R> a[RAD];
#pragma unroll
      for (int q = 0; q < RAD; ++q) a[q] = x[OFF + i + q * M];
      small_dft<R, RAD, SIGN>(a, tw, ts * M);
#pragma unroll
      for (int j = 1; j < RAD; ++j)
        if (i * j != 0) a[j] = cmul(a[j], twd<R, SIGN>(tw, i * j * ts));
#pragma unroll
      for (int j = 0; j < RAD; ++j) x[OFF + i + j * M] = a[j];
    }
    dif_sub<R, M, OFF, SIGN, 0, RAD>(x, tw, ts * RAD);
  }
}

// Sequences for the passes: seq(s) -> offset of sequence s (pitch 8 (N1 + 1)).
struct SeqLinear {
  int pitch;
  __device__ __forceinline__ int operator()(int s) const { return s * pitch; }
};
// The columns this CTA owns: s = c * ks + kl -> column (c, kl) of the [c][KS][PX] array.
struct SeqCols {
  int ks, KS, pitch;
  __device__ __forceinline__ int operator()(int s) const {
    const int c = s / ks;
    return ((c * KS) + (s - c * ks)) * pitch;
  }
};

// Pass S: N1 threads per sequence; thread n1 owns points n1 + N1 n2 (n2 < 8), padded n1 + (N1 + 1) n2.
//   inverse (SIGN +1): 8-point DFT over n2, times w^(n1 k2), stored at n1 + (N1+1) k2.
//   forward (SIGN -1): 8-point DFT over a, stored at natural k = b + N1 s (padded b + (N1+1) s).
template <typename R, int N1, int SIGN, class SEQ>
__device__ __forceinline__ void pass_s(cpx<R>* base, int nseq, SEQ seq, const cpx<R>* tw, int tid, int nthr) {
  for (int t = tid; t < nseq * N1; t += nthr) {
    const int s = t / N1, n1 = t - s * N1;
    cpx<R>* q = base + seq(s) + n1;
    cpx<R> y[8];
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) y[n2] = q[(N1 + 1) * n2];
    dif_reg<R, 8, 0, SIGN>(y, tw, N1);
    static_for<0, 8>([&](auto P) {
      constexpr int p = decltype(P)::value, k2 = dif_out(p, 8);
      cpx<R> v = y[p];
      if constexpr (SIGN > 0 && k2 != 0) {
        if (n1 != 0) v = cmul(v, twd<R, SIGN>(tw, n1 * k2));
      }
      q[(N1 + 1) * k2] = v;
    });
  }
}

// Pass B: 8 threads per sequence; thread a owns the contiguous block (N1 + 1) a .. + N1.
//   inverse: N1-point DFT of the block, output k1 at block offset k1 (final layout pos(k)).
//   forward: N1-point DFT of the block, times w^(a b), output b at block offset b.
template <typename R, int N1, int SIGN, class SEQ>
__device__ __forceinline__ void pass_b(cpx<R>* base, int nseq, SEQ seq, const cpx<R>* tw, int tid, int nthr) {
  for (int t = tid; t < nseq * 8; t += nthr) {
    const int s = t >> 3, a = t & 7;
    cpx<R>* q = base + seq(s) + (N1 + 1) * a;
    cpx<R> z[N1];
#pragma unroll
    for (int n = 0; n < N1; ++n) z[n] = q[n];
    dif_reg<R, N1, 0, SIGN>(z, tw, 8);
    static_for<0, N1>([&](auto P) {
      constexpr int p = decltype(P)::value, k = dif_out(p, N1);
      cpx<R> v = z[p];
      if constexpr (SIGN < 0 && k != 0) {
        if (a != 0) v = cmul(v, twd<R, SIGN>(tw, a * k));
      }
      q[k] = v;
    });
  }
}

template <typename R, int SIGN, class SEQ>
__device__ void pass_s_any(int N1, cpx<R>* base, int nseq, SEQ seq, const cpx<R>* tw, int tid, int nthr) {
  switch (N1) {
    case 4: pass_s<R, 4, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    case 6: pass_s<R, 6, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    case 8: pass_s<R, 8, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    case 12: pass_s<R, 12, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    default: pass_s<R, 16, SIGN>(base, nseq, seq, tw, tid, nthr); break;
  }
}
template <typename R, int SIGN, class SEQ>
__device__ void pass_b_any(int N1, cpx<R>* base, int nseq, SEQ seq, const cpx<R>* tw, int tid, int nthr) {
  switch (N1) {
    case 4: pass_b<R, 4, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    case 6: pass_b<R, 6, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    case 8: pass_b<R, 8, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    case 12: pass_b<R, 12, SIGN>(base, nseq, seq, tw, tid, nthr); break;
    default: pass_b<R, 16, SIGN>(base, nseq, seq, tw, tid, nthr); break;
  }
}

// Position of inverse-transform output k (and of forward-transform input x): (N1 + 1) (k % 8) + k / 8.
__device__ __forceinline__ int pos_perm(int k, int N1) { return (N1 + 1) * (k & 7) + (k >> 3); }
// Padded position of natural index k.
__device__ __forceinline__ int pos_nat(int k, int N1) { return k + k / N1; }

// Forward-transform sequences of the z phase: rows' slot 0 (f0 + i f1), then the even rows' slot 1
// (f2 of the row pair).
struct SeqZf {
  int nr, pitch;
  __device__ __forceinline__ int operator()(int s) const {
    return s < nr ? (3 * s) * pitch : (3 * (2 * (s - nr)) + 1) * pitch;
  }
};

template <typename R>
__global__ void __launch_bounds__(XZ_THREADS, 1)
    k_xz_rot(GridDev g, int C, int KS, int RC, const cpx<R>* __restrict__ W, cpx<R>* __restrict__ F,
             const cpx<R>* __restrict__ twxf, const cpx<R>* __restrict__ twzf, double scale_d, Dither dt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int plane = blockIdx.y;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int NX = g.Nx, NZ = g.Nz, NKz = g.NKz, NKx = g.NKx;
  const int N1x = NX >> 3, N1z = NZ >> 3;
  const int PX = NX + 8, PZ = NZ + 8;
  cpx<R>* X = reinterpret_cast<cpx<R>*>(smem_raw);  // [6][KS][PX]
  cpx<R>* Zs = X + (size_t)6 * KS * PX;               // [RC][3][PZ]
  cpx<R>* twX = Zs + (size_t)RC * 3 * PZ;             // [NX]
  cpx<R>* twZ = twX + NX;                             // [NZ]
  int* owner = reinterpret_cast<int*>(twZ + NZ);      // [NKz]
  int* local = owner + XZ_MAX_NKZ;                    // [NKz]

  const int ver = dither_ver(dt, plane % dt.nb);
  const cpx<R>* twx = dither_ptr(twxf, ver, dt.S);
  const cpx<R>* twz = dither_ptr(twzf, ver, dt.S);
  const R scale = k_misc<R>(dt, ver, 0, scale_d);
  for (int i = tid; i < NX; i += nthr) twX[i] = twx[i];
  for (int i = tid; i < NZ; i += nthr) twZ[i] = twz[i];
  for (int kz = tid; kz < NKz; kz += nthr) {
    int o = 0;
    while (o + 1 < C && (o + 1) * NKz / C <= kz) ++o;
    owner[kz] = o;
    local[kz] = kz - o * NKz / C;
  }
  const int kz0 = r * NKz / C, ks = (r + 1) * NKz / C - kz0;
  const int x0 = r * NX / C, x1 = (r + 1) * NX / C;
  const size_t Mf = g.Md;  // modes per field (per plane)

  // ---- phase 1: inverse x transform of my kz columns (6 components) --------------------------------------
  for (int t = tid; t < 6 * NX * ks; t += nthr) {
    const int kl = t % ks, rem = t / ks, p = rem % NX, c = rem / NX;
    const int kx = p <= NX / 2 ? p : p - NX;
    cpx<R> v = cmk<R>(0, 0);
    if (kx >= -g.Kx && kx <= g.Kx) {
      const int ix = kx >= 0 ? kx : kx + NKx;
      v = W[((size_t)c * gridDim.y + plane) * Mf + (size_t)ix * NKz + kz0 + kl];
    }
    X[((size_t)c * KS + kl) * PX + pos_nat(p, N1x)] = v;
  }
  __syncthreads();
  {
    const SeqCols sq{ks, KS, PX};
    pass_s_any<R, +1>(N1x, X, 6 * ks, sq, twX, tid, nthr);
    __syncthreads();
    pass_b_any<R, +1>(N1x, X, 6 * ks, sq, twX, tid, nthr);
  }
  cluster.sync();

  // ---- phase 2: z transforms and the product for my x rows ------------------------------------------------
  for (int xc = x0; xc < x1; xc += RC) {
    const int nr = min(RC, x1 - xc);
    // gather: three packed sequences per row, (u + i v), (w + i ox), (oy + i oz), natural kz order
    for (int t = tid; t < nr * 3 * NZ; t += nthr) {
      const int k = t % NZ, rem = t / NZ, qd = rem % 3, row = rem / 3;
      cpx<R> v = cmk<R>(0, 0);
      if (k < NKz || k > NZ - NKz) {
        const int kk = k < NKz ? k : NZ - k;
        const cpx<R>* Xr = cluster.map_shared_rank(X, owner[kk]);
        const size_t o = (size_t)local[kk] * PX + pos_perm(xc + row, N1x);
        const cpx<R> A = Xr[(size_t)(2 * qd) * KS * PX + o];
        const cpx<R> B = Xr[(size_t)(2 * qd + 1) * KS * PX + o];
        if (k == 0)
          v = cmk<R>(A.x, B.x);
        else if (k < NKz)
          v = cmk<R>(A.x - B.y, A.y + B.x);  // A_k + i B_k
        else
          v = cmk<R>(A.x + B.y, -A.y + B.x);  // conj(A_k) + i conj(B_k)
      }
      Zs[(size_t)(row * 3 + qd) * PZ + pos_nat(k, N1z)] = v;
    }
    __syncthreads();
    const SeqLinear sz{PZ};
    pass_s_any<R, +1>(N1z, Zs, nr * 3, sz, twZ, tid, nthr);
    __syncthreads();
    pass_b_any<R, +1>(N1z, Zs, nr * 3, sz, twZ, tid, nthr);
    __syncthreads();
    // f = omega x u at every z (positions pos(z)); row pairs share the f2 sequence
    const int npair = (nr + 1) >> 1;
    for (int t = tid; t < npair * NZ; t += nthr) {
      const int z = t % NZ, pr = t / NZ;
      const int ra = 2 * pr, rb = 2 * pr + 1;
      const int pz = pos_perm(z, N1z);
      R f2[2] = {0, 0};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = h == 0 ? ra : rb;
        if (row < nr) {
          cpx<R>* s0 = Zs + (size_t)(row * 3) * PZ + pz;
          const cpx<R> a = s0[0], b = s0[PZ], c = s0[2 * PZ];
          // a = (u, v), b = (w, ox), c = (oy, oz)
          const R f0 = c.x * b.x - c.y * a.y;
          const R f1 = c.y * a.x - b.y * b.x;
          f2[h] = b.y * a.y - c.x * a.x;
          s0[0] = cmk<R>(f0, f1);
        }
      }
      Zs[(size_t)(ra * 3 + 1) * PZ + pz] = cmk<R>(f2[0], f2[1]);
    }
    __syncthreads();
    const SeqZf sf{nr, PZ};
    const int nf = nr + npair;
    pass_b_any<R, -1>(N1z, Zs, nf, sf, twZ, tid, nthr);
    __syncthreads();
    pass_s_any<R, -1>(N1z, Zs, nf, sf, twZ, tid, nthr);
    __syncthreads();
    // unpack the r2c results and scatter f0, f1, f2 to the owners' shared memory (over the slots read above)
    for (int t = tid; t < nr * NKz; t += nthr) {
      const int k = t % NKz, row = t / NKz;
      const int km = k == 0 ? 0 : NZ - k;
      const cpx<R>* s0 = Zs + (size_t)(row * 3) * PZ;
      const cpx<R>* s1 = Zs + (size_t)((row & ~1) * 3 + 1) * PZ;
      const cpx<R> zk = s0[pos_nat(k, N1z)], zm = s0[pos_nat(km, N1z)];
      const cpx<R> yk = s1[pos_nat(k, N1z)], ym = s1[pos_nat(km, N1z)];
      const R hf = (R)0.5;
      const cpx<R> P0 = cmk<R>(hf * (zk.x + zm.x), hf * (zk.y - zm.y));
      const cpx<R> P1 = cmk<R>(hf * (zk.y + zm.y), hf * (zm.x - zk.x));
      const cpx<R> P2 = (row & 1) ? cmk<R>(hf * (yk.y + ym.y), hf * (ym.x - yk.x))
                                  : cmk<R>(hf * (yk.x + ym.x), hf * (yk.y - ym.y));
      cpx<R>* Xr = cluster.map_shared_rank(X, owner[k]);
      const size_t o = (size_t)local[k] * PX + pos_perm(xc + row, N1x);
      Xr[o] = P0;
      Xr[(size_t)KS * PX + o] = P1;
      Xr[(size_t)2 * KS * PX + o] = P2;
    }
    __syncthreads();
  }
  cluster.sync();

  // ---- phase 3: forward x transform of my columns of f, solved kx out ------------------------------------
  {
    const SeqCols sq{ks, KS, PX};
    pass_b_any<R, -1>(N1x, X, 3 * ks, sq, twX, tid, nthr);
    __syncthreads();
    pass_s_any<R, -1>(N1x, X, 3 * ks, sq, twX, tid, nthr);
    __syncthreads();
  }
  for (int t = tid; t < 3 * NKx * ks; t += nthr) {
    const int kl = t % ks, rem = t / ks, ix = rem % NKx, c = rem / NKx;
    const int kx = ix <= g.Kx ? ix : ix - NKx;
    const int p = kx >= 0 ? kx : NX + kx;
    F[((size_t)c * gridDim.y + plane) * Mf + (size_t)ix * NKz + kz0 + kl] =
        cscale(X[((size_t)c * KS + kl) * PX + pos_nat(p, N1x)], scale);
  }
}

}  // namespace

bool xz_fused_supported(const GridDev& gp) {
  auto ok = [](int L) { return L == 32 || L == 48 || L == 64 || L == 96 || L == 128; };
  return ok(gp.Nx) && ok(gp.Nz) && gp.NKz <= XZ_MAX_NKZ && gp.NKz >= 1 && gp.kxs == nullptr;
}

template <typename R>
size_t xz_fused_smem(const GridDev& gp, int C, int RC) {
  const int KS = (gp.NKz + C - 1) / C;
  return sizeof(cpx<R>) * ((size_t)6 * KS * (gp.Nx + 8) + (size_t)RC * 3 * (gp.Nz + 8) + gp.Nx + gp.Nz) +
         2 * XZ_MAX_NKZ * sizeof(int);
}

template <typename R>
cudaLaunchConfig_t xz_config(const GridDev& gp, int C, int RC, cudaStream_t st, cudaLaunchAttribute* at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, gp.Ny, 1);
  cfg.blockDim = dim3(XZ_THREADS, 1, 1);
  cfg.dynamicSmemBytes = xz_fused_smem<R>(gp, C, RC);
  cfg.stream = st;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

template <typename R>
void xz_set_attributes() {
  static const bool attr = [] {
    cudaFuncSetAttribute(k_xz_rot<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr;
}

// Cluster size and rows per z chunk: the largest row chunk that fits, and among cluster sizes 2..8 that the
// device can schedule (cudaOccupancyMaxActiveClusters > 0) the one whose CTAs fill whole waves of one CTA
// per SM best (ties: the smaller cluster).
template <typename R>
int xz_fused_shape(const GridDev& gp, int nsm, int& C, int& RC) {
  xz_set_attributes<R>();
  double best = -1.0;
  C = RC = 0;
  const int rcmax = sizeof(R) == 4 ? 16 : 8;
  for (int c = 2; c <= 8; ++c) {
    if (c > gp.NKz) break;
    const int rows = (gp.Nx + c - 1) / c;
    int rc = rcmax < rows ? rcmax : rows;
    rc += rc & 1;
    while (rc > 2 && xz_fused_smem<R>(gp, c, rc) > 227 * 1024) rc -= 2;
    if (xz_fused_smem<R>(gp, c, rc) > 227 * 1024) continue;
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = xz_config<R>(gp, c, rc, 0, at);
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_xz_rot<R>, &cfg) != cudaSuccess || nclusters < 1) {
      (void)cudaGetLastError();
      continue;
    }
    const long long ctas = (long long)c * gp.Ny;
    const long long waves = (ctas + nsm - 1) / nsm;
    const double eff = (double)ctas / (double)(waves * nsm) - 0.002 * c;
    if (eff > best) {
      best = eff;
      C = c;
      RC = rc;
    }
  }
  return C > 0 ? 0 : -1;
}

template <typename R>
cudaError_t launch_xz_rot(const GridDev& gp, int C, int RC, const cpx<R>* W, cpx<R>* F, const cpx<R>* twxf,
                          const cpx<R>* twzf, cudaStream_t st, const Dither& dt) {
  xz_set_attributes<R>();
  const int KS = (gp.NKz + C - 1) / C;
  cudaLaunchAttribute at[1];
  cudaLaunchConfig_t cfg = xz_config<R>(gp, C, RC, st, at);
  const double scale = 1.0 / ((double)gp.Nx * (double)gp.Nz);
  return cudaLaunchKernelEx(&cfg, k_xz_rot<R>, gp, C, KS, RC, W, F, twxf, twzf, scale, dt);
}

template size_t xz_fused_smem<float>(const GridDev&, int, int);
template size_t xz_fused_smem<double>(const GridDev&, int, int);
template int xz_fused_shape<float>(const GridDev&, int, int&, int&);
template int xz_fused_shape<double>(const GridDev&, int, int&, int&);
template cudaError_t launch_xz_rot<float>(const GridDev&, int, int, const cpx<float>*, cpx<float>*,
                                          const cpx<float>*, const cpx<float>*, cudaStream_t, const Dither&);
template cudaError_t launch_xz_rot<double>(const GridDev&, int, int, const cpx<double>*, cpx<double>*,
                                           const cpx<double>*, const cpx<double>*, cudaStream_t, const Dither&);
