// z pass of the rotational nonlinear term with register-resident FFTs (the three-kernel x/z path).
//
// Restates, for the x rows of one y-plane (the z half of makePhysical_xz, the pointwise cross product of
// rotationalNL and the z half of makeSpectral_xz; channelflow/flowfield.cpp:1850-1886,
// diffops.cpp:2560-2611, 2852-2881):
//   six components u, v, w, ox, oy, oz of each x row (complex, kz <= Kz, after the inverse x transform)
//   -> c2r along z, two real rows packed in one complex sequence (A_k + i B_k)
//   -> f = omega x u at every z
//   -> r2c along z (f0 + i f1 per row, f2 of two rows per sequence), kz <= Kz kept, unscaled.
// Input X[c][plane][x][kz], output Z[c][plane][x][kz] as the generic z pass (k_zphys) reads and writes them.
//
// The transforms are the four-step FFTs of fft_steps.cuh (L = 8 N1, compile-time lengths 32 ... 128): every
// thread transforms 8 or N1 points in registers, so a transform costs two shared-memory round trips, against
// one per radix stage for the generic Stockham FFT; sequences are padded by one slot per N1 points.  Twiddles:
// the full-circle table exp(-2 pi i e / Nz), e < Nz, in the field's dithered version on the mixed path.  One
// CTA takes RC x rows of one plane (the DNS's tuned z-pass row count).  FP32 (mixed path) only: in FP64 the
// Stockham kernel's radix-4 stages take fewer FP64-pipe slots and were faster.
#include "fft_steps.cuh"
#include "kernels.h"

#include <atomic>

namespace {

using namespace fsr;

constexpr int ZR_THREADS = 256;

std::atomic<int> g_zreg{1};

template <typename R>
size_t zreg_smem(int Nz, int RC) {
  return sizeof(cpx<R>) * ((size_t)RC * 3 * (Nz + 8) + Nz);
}

template <typename R, int N1Z>
__global__ void __launch_bounds__(ZR_THREADS) k_zrot(GridDev g, int RC, const cpx<R>* __restrict__ X,
                                                     cpx<R>* __restrict__ Z, const cpx<R>* __restrict__ twzf,
                                                     Dither dt) {
  constexpr int NZ = 8 * N1Z;
  constexpr int PZ = NZ + 8;  // 8 mod 16: the two sequences of a half-warp in pass B hit distinct banks
  constexpr int NW = ZR_THREADS / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<R>* Zs = reinterpret_cast<cpx<R>*>(smem_raw);  // [RC][3][PZ]: sequence (row, pair) at (3 row + pair) PZ
  cpx<R>* twZ = Zs + (size_t)RC * 3 * PZ;             // [NZ]
  pdl_wait();  // launched with launch_pdl: the previous kernel's output is read from here on
  const int ny = blockIdx.y;
  const int xc = blockIdx.x * RC;
  const int nr = min(RC, g.Nx - xc);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int NKz = g.NKz;
  const size_t plane = (size_t)g.Nx * NKz;
  const size_t cstr = (size_t)g.Ny * plane;  // component stride of X and Z
  const cpx<R>* Xp = X + (size_t)ny * plane + (size_t)xc * NKz;
  cpx<R>* Zp = Z + (size_t)ny * plane + (size_t)xc * NKz;
  const cpx<R>* twz = dither_ptr(twzf, dither_ver(dt, ny % dt.nb), dt.S);  // plane ny -> its field's twiddles
  for (int i = tid; i < NZ; i += ZR_THREADS) twZ[i] = twz[i];

  // pack: sequence (row, pair q) holds components 2q and 2q + 1 of the row as A_k + i B_k (k < NKz) and
  // conj(A_k) + i conj(B_k) at Nz - k; the other bins (the Nyquist bin among them) are zero
#pragma unroll 4
  for (int t = tid; t < nr * 3 * NZ; t += ZR_THREADS) {
    const int rq = t / NZ, k = t - rq * NZ;
    const int row = rq / 3, q = rq - 3 * row;
    cpx<R> v = cmk<R>(0, 0);
    if (k < NKz || k > NZ - NKz) {
      const int kk = k < NKz ? k : NZ - k;
      const size_t o = (size_t)row * NKz + kk;
      const cpx<R> A = Xp[(size_t)(2 * q) * cstr + o], B = Xp[(size_t)(2 * q + 1) * cstr + o];
      if (k == 0)
        v = cmk<R>(A.x, B.x);
      else if (k < NKz)
        v = cmk<R>(A.x - B.y, A.y + B.x);  // A_k + i B_k
      else
        v = cmk<R>(A.x + B.y, -A.y + B.x);  // conj(A_k) + i conj(B_k)
    }
    Zs[(size_t)rq * PZ + pos_nat<N1Z>(k)] = v;
  }
  __syncthreads();
  pass_s<R, N1Z, +1>(Zs, nr * 3, SeqLinear{PZ}, twZ, tid, ZR_THREADS);
  __syncthreads();
  pass_b<R, N1Z, +1>(Zs, nr * 3, SeqLinear{PZ}, twZ, tid, ZR_THREADS);
  __syncthreads();
  // f = omega x u at every z (positions pos(z)); a = (u, v), b = (w, ox), c = (oy, oz); row pairs share the f2
  // sequence (slot 1 of the pair's even row)
  const int npair = (nr + 1) >> 1;
  for (int t = tid; t < npair * NZ; t += ZR_THREADS) {
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
  pass_b<R, N1Z, -1>(Zs, nf, sf, twZ, tid, ZR_THREADS);
  __syncthreads();
  pass_s<R, N1Z, -1>(Zs, nf, sf, twZ, tid, ZR_THREADS);
  __syncthreads();
  // unpack the r2c results of f0, f1 (slot 0 of the row) and f2 (slot 1 of the pair's even row)
  for (int row = warp; row < nr; row += NW) {
    const cpx<R>* s0 = Zs + (size_t)(row * 3) * PZ;
    const cpx<R>* s1 = Zs + (size_t)((row & ~1) * 3 + 1) * PZ;
    const bool odd = row & 1;
    for (int k = lane; k < NKz; k += 32) {
      const int km = k == 0 ? 0 : NZ - k;
      const cpx<R> zk = s0[pos_nat<N1Z>(k)], zm = s0[pos_nat<N1Z>(km)];
      const cpx<R> yk = s1[pos_nat<N1Z>(k)], ym = s1[pos_nat<N1Z>(km)];
      const R hf = (R)0.5;
      const size_t o = (size_t)row * NKz + k;
      Zp[o] = cmk<R>(hf * (zk.x + zm.x), hf * (zk.y - zm.y));
      Zp[cstr + o] = cmk<R>(hf * (zk.y + zm.y), hf * (zm.x - zk.x));
      Zp[2 * cstr + o] = odd ? cmk<R>(hf * (yk.y + ym.y), hf * (ym.x - yk.x))
                             : cmk<R>(hf * (yk.x + ym.x), hf * (yk.y - ym.y));
    }
  }
}

template <typename R, int N1Z>
cudaError_t run_zrot(const GridDev& g, int RC, const cpx<R>* X, cpx<R>* Z, const cpx<R>* twzf, cudaStream_t st,
                     const Dither& dt) {
  static const bool attr = [] {
    cudaFuncSetAttribute(k_zrot<R, N1Z>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr;
  return launch_pdl(k_zrot<R, N1Z>, dim3((g.Nx + RC - 1) / RC, g.Ny), dim3(ZR_THREADS), zreg_smem<R>(g.Nz, RC), st,
                    g, RC, X, Z, twzf, dt);
}

}  // namespace

void set_zpass_register(int enable) { g_zreg.store(enable ? 1 : 0); }

cudaError_t launch_zrot(const GridDev& g, int RC, const cpx<float>* X, cpx<float>* Z, const cpx<float>* twzf,
                        cudaStream_t st, const Dither& dt) {
  using R = float;
  if (!g_zreg.load() || !twzf || RC < 1 || g.NKz > g.Nz / 2 || zreg_smem<R>(g.Nz, RC) > 227 * 1024)
    return cudaErrorNotSupported;
  switch (g.Nz) {
    case 32: return run_zrot<R, 4>(g, RC, X, Z, twzf, st, dt);
    case 48: return run_zrot<R, 6>(g, RC, X, Z, twzf, st, dt);
    case 64: return run_zrot<R, 8>(g, RC, X, Z, twzf, st, dt);
    case 96: return run_zrot<R, 12>(g, RC, X, Z, twzf, st, dt);
    case 128: return run_zrot<R, 16>(g, RC, X, Z, twzf, st, dt);
    default: return cudaErrorNotSupported;
  }
}

