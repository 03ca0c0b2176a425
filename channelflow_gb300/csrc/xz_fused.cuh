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
#pragma once

#include <cooperative_groups.h>

#include <type_traits>

#include "fft_steps.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace xzf {

constexpr int XZ_THREADS = 256;
constexpr int XZ_MAX_NKZ = 64;

using namespace fsr;

// Dynamic shared memory of k_xz_rot: owned columns [6 ks][NX + 9], z rows [RC][3][NZ + 8], the two
// twiddle tables, and the kz -> (owner, column, owner's column count) tables.
template <typename R>
__host__ __device__ inline size_t smem_bytes(int Nx, int Nz, int NKz, int C, int RC) {
  const int KS = (NKz + C - 1) / C;
  return sizeof(cpx<R>) * ((size_t)6 * KS * (Nx + 9) + (size_t)RC * 3 * (Nz + 8) + Nx + Nz) +
         3 * XZ_MAX_NKZ * sizeof(int);
}

template <typename R, int N1X, int N1Z>
__global__ void __launch_bounds__(XZ_THREADS, 2)
    k_xz_rot(GridDev g, int C, int RC, const cpx<R>* __restrict__ W, cpx<R>* __restrict__ F,
             const cpx<R>* __restrict__ twxf, const cpx<R>* __restrict__ twzf, double scale_d, Dither dt) {
  constexpr int NX = 8 * N1X, NZ = 8 * N1Z;
  constexpr int PX = NX + 9;  // odd pitch: lanes on consecutive columns hit distinct banks
  constexpr int PZ = NZ + 8;  // 8 mod 16: the two sequences of a half-warp in pass B hit distinct banks
  constexpr int NW = XZ_THREADS / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int plane = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int NKz = g.NKz, NKx = g.NKx, Kx = g.Kx;
  const int KS = (NKz + C - 1) / C;
  cpx<R>* X = reinterpret_cast<cpx<R>*>(smem_raw);  // owned columns, (c ks + kl) PX
  cpx<R>* Zs = X + (size_t)6 * KS * PX;               // [RC][3][PZ]
  cpx<R>* twX = Zs + (size_t)RC * 3 * PZ;             // [NX]
  cpx<R>* twZ = twX + NX;                             // [NZ]
  int* own = reinterpret_cast<int*>(twZ + NZ);        // kz -> rank of the CTA owning its column
  int* col = own + XZ_MAX_NKZ;                        // kz -> its column index in the owner (c = 0)
  int* oks = col + XZ_MAX_NKZ;                        // kz -> the owner's columns per component

  const int ver = dither_ver(dt, plane % dt.nb);
  const cpx<R>* twx = dither_ptr(twxf, ver, dt.S);
  const cpx<R>* twz = dither_ptr(twzf, ver, dt.S);
  const R scale = k_misc<R>(dt, ver, 0, scale_d);
  for (int i = tid; i < NX; i += XZ_THREADS) twX[i] = twx[i];
  for (int i = tid; i < NZ; i += XZ_THREADS) twZ[i] = twz[i];
  for (int kz = tid; kz < NKz; kz += XZ_THREADS) {
    int o = 0;
    while (o + 1 < C && (o + 1) * NKz / C <= kz) ++o;
    own[kz] = o;
    col[kz] = kz - o * NKz / C;
    oks[kz] = (o + 1) * NKz / C - o * NKz / C;
  }
  const int kz0 = r * NKz / C, ks = (r + 1) * NKz / C - kz0;
  const int x0 = r * NX / C, x1 = (r + 1) * NX / C;
  const size_t Mf = g.Md;                      // modes per field (per plane)
  const size_t cstr = (size_t)gridDim.y * Mf;  // component stride of W and F
  // lane groups of 2^lks lanes on the owned columns (ks <= 32): RW groups per warp
  const int lks = ks <= 8 ? 3 : (ks <= 16 ? 4 : 5);
  const int RW = 32 >> lks, sub = lane >> lks, kl = lane & ((1 << lks) - 1);
  const bool kok = kl < ks;

  // ---- phase 1: the owned kz columns of u, v, w, ox, oy, oz, inverse transform along x ------------------
  // every solved value is copied asynchronously (all copies of the CTA in flight at once), the rest zeroed
  if (kok) {
    const cpx<R>* Wp = W + (size_t)plane * Mf + kz0 + kl;
    for (int u = warp * RW + sub; u < 6 * NX; u += NW * RW) {
      const int c = u / NX, p = u - c * NX;
      const int kx = p <= NX / 2 ? p : p - NX;
      cpx<R>* dst = X + (c * ks + kl) * PX + pos_nat<N1X>(p);
      if (kx >= -Kx && kx <= Kx)
        cp_async_cpx<R>(dst, Wp + c * cstr + (size_t)(kx >= 0 ? kx : kx + NKx) * NKz);
      else
        *dst = cmk<R>(0, 0);
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  pass_s<R, N1X, +1>(X, 6 * ks, SeqLinear{PX}, twX, tid, XZ_THREADS);
  __syncthreads();
  pass_b<R, N1X, +1>(X, 6 * ks, SeqLinear{PX}, twX, tid, XZ_THREADS);
  cluster.sync();

  // ---- phase 2: z transforms and omega x u for the owned x rows, RC rows at a time ------------------------
  for (int xc = x0; xc < x1; xc += RC) {
    const int nr = min(RC, x1 - xc);
    // gather: one warp per (row, pair) sequence, two sequences at a time, lanes over kz bins, columns read
    // from their owners (DSMEM); all loads of both sequences are issued before the stores
    for (int rq0 = warp; rq0 < nr * 3; rq0 += 2 * NW) {
      constexpr int KI = (NZ + 31) / 32;
      cpx<R> val[2][KI];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int rq = rq0 + h * NW;
        const int row = rq / 3, qd = rq - 3 * row;
        const int px = pos_perm<N1X>(xc + row);
#pragma unroll
        for (int i = 0; i < KI; ++i) {
          const int k = lane + 32 * i;
          cpx<R> v = cmk<R>(0, 0);
          if (rq < nr * 3 && k < NZ && (k < NKz || k > NZ - NKz)) {
            const int kk = k < NKz ? k : NZ - k;
            const int ow = oks[kk];
            const cpx<R>* Xr = cluster.map_shared_rank(X, own[kk]);
            const int ia = (2 * qd * ow + col[kk]) * PX + px;
            const cpx<R> A = Xr[ia], B = Xr[ia + ow * PX];
            if (k == 0)
              v = cmk<R>(A.x, B.x);
            else if (k < NKz)
              v = cmk<R>(A.x - B.y, A.y + B.x);  // A_k + i B_k
            else
              v = cmk<R>(A.x + B.y, -A.y + B.x);  // conj(A_k) + i conj(B_k)
          }
          val[h][i] = v;
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int rq = rq0 + h * NW;
        if (rq < nr * 3) {
          cpx<R>* zs = Zs + (size_t)rq * PZ;
#pragma unroll
          for (int i = 0; i < KI; ++i) {
            const int k = lane + 32 * i;
            if (k < NZ) zs[pos_nat<N1Z>(k)] = val[h][i];
          }
        }
      }
    }
    __syncthreads();
    pass_s<R, N1Z, +1>(Zs, nr * 3, SeqLinear{PZ}, twZ, tid, XZ_THREADS);
    __syncthreads();
    pass_b<R, N1Z, +1>(Zs, nr * 3, SeqLinear{PZ}, twZ, tid, XZ_THREADS);
    __syncthreads();
    // f = omega x u at every z (positions pos(z)); row pairs share the f2 sequence
    const int npair = (nr + 1) >> 1;
    for (int t = tid; t < npair * NZ; t += XZ_THREADS) {
      const int pr = t / NZ, z = t - pr * NZ;
      const int ra = 2 * pr, rb = 2 * pr + 1;
      const int pz = pos_perm<N1Z>(z);
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
    pass_b<R, N1Z, -1>(Zs, nf, sf, twZ, tid, XZ_THREADS);
    __syncthreads();
    pass_s<R, N1Z, -1>(Zs, nf, sf, twZ, tid, XZ_THREADS);
    __syncthreads();
    // unpack the r2c results; f0, f1, f2 go to the owners' columns, over the slots gathered above
    for (int row = warp; row < nr; row += NW) {
      const int px = pos_perm<N1X>(xc + row);
      const cpx<R>* s0 = Zs + (size_t)(row * 3) * PZ;
      const cpx<R>* s1 = Zs + (size_t)((row & ~1) * 3 + 1) * PZ;
      const bool odd = row & 1;
      for (int k = lane; k < NKz; k += 32) {
        const int km = k == 0 ? 0 : NZ - k;
        const cpx<R> zk = s0[pos_nat<N1Z>(k)], zm = s0[pos_nat<N1Z>(km)];
        const cpx<R> yk = s1[pos_nat<N1Z>(k)], ym = s1[pos_nat<N1Z>(km)];
        const R hf = (R)0.5;
        const cpx<R> P0 = cmk<R>(hf * (zk.x + zm.x), hf * (zk.y - zm.y));
        const cpx<R> P1 = cmk<R>(hf * (zk.y + zm.y), hf * (zm.x - zk.x));
        const cpx<R> P2 = odd ? cmk<R>(hf * (yk.y + ym.y), hf * (ym.x - yk.x))
                              : cmk<R>(hf * (yk.x + ym.x), hf * (yk.y - ym.y));
        const int ow = oks[k];
        cpx<R>* Xr = cluster.map_shared_rank(X, own[k]);
        const int ia = col[k] * PX + px;
        Xr[ia] = P0;
        Xr[ia + ow * PX] = P1;
        Xr[ia + 2 * ow * PX] = P2;
      }
    }
    __syncthreads();
  }
  cluster.sync();

  // ---- phase 3: forward transform along x of the owned columns of f, solved kx to HBM ---------------------
  pass_b<R, N1X, -1>(X, 3 * ks, SeqLinear{PX}, twX, tid, XZ_THREADS);
  __syncthreads();
  pass_s<R, N1X, -1>(X, 3 * ks, SeqLinear{PX}, twX, tid, XZ_THREADS);
  __syncthreads();
  if (kok) {
    cpx<R>* Fp = F + (size_t)plane * Mf + kz0 + kl;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      for (int ix = warp * RW + sub; ix < NKx; ix += NW * RW) {
        const int kx = ix <= Kx ? ix : ix - NKx;
        const int p = kx >= 0 ? kx : NX + kx;
        Fp[c * cstr + (size_t)ix * NKz] = cscale(X[(c * ks + kl) * PX + pos_nat<N1X>(p)], scale);
      }
  }
}

inline cudaLaunchConfig_t launch_config(const GridDev& gp, size_t smem, int C, cudaStream_t st,
                                        cudaLaunchAttribute* at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, gp.Ny, 1);
  cfg.blockDim = dim3(XZ_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

// Launch (max_clusters == nullptr) or occupancy query (clusters that fit at once) of k_xz_rot<R, N1X, N1Z>.
template <typename R, int N1X, int N1Z>
cudaError_t run_xz(const GridDev& gp, int C, int RC, const cpx<R>* W, cpx<R>* F, const cpx<R>* twxf,
                   const cpx<R>* twzf, cudaStream_t st, const Dither& dt, int* max_clusters) {
  static const bool attr = [] {
    cudaFuncSetAttribute(k_xz_rot<R, N1X, N1Z>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr;
  cudaLaunchAttribute at[2];
  cudaLaunchConfig_t cfg = launch_config(gp, smem_bytes<R>(gp.Nx, gp.Nz, gp.NKz, C, RC), C, st, at);
  if (max_clusters) return cudaOccupancyMaxActiveClusters(max_clusters, k_xz_rot<R, N1X, N1Z>, &cfg);
  // launched without programmatic dependent launch: with it the step ran 20% slower (128x97x128 mixed,
  // graph-replayed: 0.387 against 0.322 ms per step), without it the fused and the three-kernel forms are level
  const double scale = 1.0 / ((double)gp.Nx * (double)gp.Nz);
  return cudaLaunchKernelEx(&cfg, k_xz_rot<R, N1X, N1Z>, gp, C, RC, W, F, twxf, twzf, scale, dt);
}

template <typename R, int N1X>
cudaError_t run_xz_z(int n1z, const GridDev& gp, int C, int RC, const cpx<R>* W, cpx<R>* F, const cpx<R>* twxf,
                     const cpx<R>* twzf, cudaStream_t st, const Dither& dt, int* mc) {
  switch (n1z) {
    case 4: return run_xz<R, N1X, 4>(gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 6: return run_xz<R, N1X, 6>(gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 8: return run_xz<R, N1X, 8>(gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 12: return run_xz<R, N1X, 12>(gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 16: return run_xz<R, N1X, 16>(gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    default: return cudaErrorInvalidValue;
  }
}

// Dispatch over the compile-time x and z lengths (8 N1, N1 in {4, 6, 8, 12, 16}).
template <typename R>
cudaError_t run_xz_any(const GridDev& gp, int C, int RC, const cpx<R>* W, cpx<R>* F, const cpx<R>* twxf,
                       const cpx<R>* twzf, cudaStream_t st, const Dither& dt, int* mc) {
  const int n1z = gp.Nz / 8;
  switch (gp.Nx / 8) {
    case 4: return run_xz_z<R, 4>(n1z, gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 6: return run_xz_z<R, 6>(n1z, gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 8: return run_xz_z<R, 8>(n1z, gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 12: return run_xz_z<R, 12>(n1z, gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    case 16: return run_xz_z<R, 16>(n1z, gp, C, RC, W, F, twxf, twzf, st, dt, mc);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace xzf
