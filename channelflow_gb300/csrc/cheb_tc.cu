// Forward Chebyshev transform (values at the Gauss-Lobatto points -> coefficients, chebyfft,
// chebyshev.cpp:262-284) of the mixed path on the 5th-generation tensor cores.
//
// out[n][l] = sum_j F[n][j] in[j][l] for every real line l of a component: a GEMM with M = Ny output rows
// (padded to 128), K = Ny points (padded to a multiple of 16) and N = lines.  Operands in BF16 with FP32
// accumulation in tensor memory (tcgen05.mma kind::f16, one CTA, M = 128, N = 64 lines per CTA):
//   the constant matrix is split into four BF16 parts, F = F1 + F2 + F3 + F4 (host-built, about 32 bits of
//   the FP64 value), and every FP32 input into three, x = x1 + x2 + x3 (exact: each part takes the next 8 of
//   the 24 significand bits); the nine products Fi xj with i + j <= 5 carry every term down to 2^-24 of the
//   leading one, so the result is the FP32 transform of the FP32 data with the constants exact to well below
//   FP32 rounding.
// Operands sit in shared memory in the canonical no-swizzle K-major layout: 8 x 16-byte core matrices, the two
// of a 16-wide K slice 128 bytes apart (leading-dimension offset), row groups of 8 rows 256 bytes apart
// (stride-dimension offset).  One thread issues the MMAs and commits them to an mbarrier; every warp then
// reads its 32 rows (TMEM lanes) with tcgen05.ld.
#include <cuda_bf16.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "kernels.h"

namespace {

constexpr int TC_M = 128, TC_NT = 64, TC_THREADS = 512;
constexpr int TC_ASPLIT = 4, TC_BSPLIT = 3, TC_NPROD = 9;

// Element offset of (row r, column k) in one split of a K-major operand of R rows.
__host__ __device__ constexpr int kmaj_off(int r, int k, int R) {
  return (k >> 4) * (R * 16) + (r >> 3) * 128 + ((k >> 3) & 1) * 64 + (r & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start address, leading / stride byte offsets, version 1, no
// swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// 4-byte asynchronous global -> shared copy; nbytes = 0 writes zero.
__device__ __forceinline__ void cp_async4(void* dst_smem, const void* src, int nbytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_u32(dst_smem)), "l"(src), "r"(nbytes)
               : "memory");
}

// s + t = s1 + err exactly (two-sum); err added to the compensation c.
__device__ __forceinline__ void two_sum_c(float& s, float t, float& c) {
  const float s1 = s + t;
  const float bp = s1 - s;
  c += (s - (s1 - bp)) + (t - bp);
  s = s1;
}

// Persistent: one CTA per SM loads the constant matrix once (bulk copy) and walks the tiles (64 lines of one
// component) with stride gridDim.x; the next tile's FP32 lines are copied (cp.async) while the current one is
// split, multiplied and written.  Shared memory: constant matrix, BF16 tile, two FP32 tiles (the current one
// also stages the output rows, XOR-swizzled), barriers.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_cheb_tc(int N, int KS, int nlines, int ncomp, const float* __restrict__ in, size_t ld, size_t cs,
              float* __restrict__ out, const __nv_bfloat16* __restrict__ Ag, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int KP = 16 * KS;                       // padded K
  const int asz = TC_M * KP, bsz = TC_NT * KP;  // elements per split
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(smem_raw);
  __nv_bfloat16* Bs = As + TC_ASPLIT * asz;
  float* Xs = reinterpret_cast<float*>(Bs + TC_BSPLIT * bsz);  // [2][KP][64] FP32 tiles
  uint64_t* mbar = reinterpret_cast<uint64_t*>(Xs + 2 * KP * TC_NT);  // [0]: constant matrix, [1]: MMAs done
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tpc = (nlines + TC_NT - 1) / TC_NT, ntiles = tpc * ncomp;
  const uint32_t abytes = (uint32_t)(TC_ASPLIT * asz * 2);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar + 1)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  __syncthreads();
  if (tid == 0) {
    // the constant matrix (all splits, already in the operand layout) by the bulk-copy engine, 16 KB pieces
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(abytes)
                 : "memory");
    for (uint32_t o = 0; o < abytes; o += 16384) {
      const uint32_t sz = abytes - o < 16384 ? abytes - o : 16384;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
              smem_u32(reinterpret_cast<unsigned char*>(As) + o)),
          "l"(reinterpret_cast<const unsigned char*>(Ag) + o), "r"(sz), "r"(smem_u32(mbar))
          : "memory");
    }
  }
  // FP32 lines of a tile into X, all copies in flight (zero past the last line and in the K padding)
  auto issue = [&](int tile, float* X) {
    const int comp = tile / tpc, l0 = (tile - comp * tpc) * TC_NT;
    const float* src = in + comp * cs;
    for (int i = tid; i < KP * TC_NT; i += TC_THREADS) {
      const int k = i / TC_NT, c = i - k * TC_NT;
      const bool okc = k < N && l0 + c < nlines;
      cp_async4(X + i, okc ? src + (size_t)k * ld + l0 + c : src, okc ? 4 : 0);
    }
  };
  const uint32_t tmem = *tslot;
  // the set-up above (barriers, tensor memory, the constant matrix) overlaps the previous kernel's tail; its
  // output is read from here on
  pdl_wait();
  pdl_trigger();
  if (blockIdx.x < ntiles) issue(blockIdx.x, Xs);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  bool ok = true;
  int it = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
    float* X = Xs + (it & 1) * KP * TC_NT;
    if (t + (int)gridDim.x < ntiles) issue(t + gridDim.x, Xs + ((it + 1) & 1) * KP * TC_NT);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this tile's copies have landed
    __syncthreads();
    // split every value into three BF16 parts in the operand layout: a thread takes one line and eight
    // consecutive k (one 16-byte core-matrix row per split)
    for (int i = tid; i < (KP / 8) * TC_NT; i += TC_THREADS) {
      const int kg = i / TC_NT, c = i - kg * TC_NT;
      uint32_t p1[4], p2[4], p3[4];
#pragma unroll
      for (int e = 0; e < 8; e += 2) {
        __nv_bfloat16 b1[2], b2[2], b3[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float x = X[(8 * kg + e + h) * TC_NT + c];
          b1[h] = __float2bfloat16_rn(x);
          const float r1 = x - __bfloat162float(b1[h]);
          b2[h] = __float2bfloat16_rn(r1);
          b3[h] = __float2bfloat16_rn(r1 - __bfloat162float(b2[h]));
        }
        p1[e >> 1] = (uint32_t)__bfloat16_as_ushort(b1[0]) | ((uint32_t)__bfloat16_as_ushort(b1[1]) << 16);
        p2[e >> 1] = (uint32_t)__bfloat16_as_ushort(b2[0]) | ((uint32_t)__bfloat16_as_ushort(b2[1]) << 16);
        p3[e >> 1] = (uint32_t)__bfloat16_as_ushort(b3[0]) | ((uint32_t)__bfloat16_as_ushort(b3[1]) << 16);
      }
      const int o = kmaj_off(c, 8 * kg, TC_NT);
      *reinterpret_cast<uint4*>(Bs + o) = make_uint4(p1[0], p1[1], p1[2], p1[3]);
      *reinterpret_cast<uint4*>(Bs + bsz + o) = make_uint4(p2[0], p2[1], p2[2], p2[3]);
      *reinterpret_cast<uint4*>(Bs + 2 * bsz + o) = make_uint4(p3[0], p3[1], p3[2], p3[3]);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (tid == 0) {
      if (it == 0) {
        bool got = false;
        for (int w = 0; w < (1 << 20); ++w)
          if (mbar_try_wait(smem_u32(mbar), 0)) {
            got = true;
            break;
          }
        if (!got) {
          ok = false;
          if (err) atomicExch(err, 1);
        }
      }
      if (ok) {
        // D f32, A and B BF16, both K-major, N = 64, M = 128
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_NT >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);
        // one accumulator (64 TMEM columns) per K slice; the products Fi xj (i + j <= 5) smallest first, so the
        // leading product is added last to the slice's sum
        const int pa[TC_NPROD] = {1, 2, 3, 0, 1, 2, 0, 1, 0};
        const int pb[TC_NPROD] = {2, 1, 0, 2, 1, 0, 1, 0, 0};
        const uint32_t a0 = smem_u32(As), b0 = smem_u32(Bs);
        for (int ks = 0; ks < KS; ++ks)
          for (int p = 0; p < TC_NPROD; ++p) {
            const uint64_t da = umma_desc(a0 + 2u * (uint32_t)(pa[p] * asz + ks * TC_M * 16), 128, 256);
            const uint64_t db = umma_desc(b0 + 2u * (uint32_t)(pb[p] * bsz + ks * TC_NT * 16), 128, 256);
            mma_bf16(tmem + (uint32_t)(ks * TC_NT), da, db, idesc, p != 0);
          }
      }
      // arrive on the MMA barrier in every case (after the MMAs when they were issued)
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(mbar + 1))
                   : "memory");
    }
    bool done = false;
    for (int w = 0; w < (1 << 20); ++w)
      if (mbar_try_wait(smem_u32(mbar + 1), (uint32_t)(it & 1))) {
        done = true;
        break;
      }
    if (!done && err) atomicExch(err, 1);
    ok = __syncthreads_and(ok && done) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its sub-partition's) and columns 16 (w / 4) .. + 15;
    // the K-slice sums are combined with error-free two-sums and the rows staged over this tile's FP32 lines
    // (row r, column c at r 64 + (c ^ (r mod 32)): conflict-free both ways)
    float* Os = X;
    const int n = 32 * (warp & 3) + lane;
    {
      const int cb = 16 * (warp >> 2);
      float sum[16], cmp[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) sum[j] = cmp[j] = 0.0f;
#pragma unroll 1
      for (int ks = 0; ks < KS; ++ks) {
        uint32_t v[16];
        const uint32_t ta = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(ks * TC_NT + cb);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) two_sum_c(sum[j], __uint_as_float(v[j]), cmp[j]);
      }
      if (n < N) {
#pragma unroll
        for (int j = 0; j < 16; ++j) Os[n * TC_NT + ((cb + j) ^ (n & 31))] = sum[j] + cmp[j];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (ok) {
      const int comp = t / tpc, l0 = (t - comp * tpc) * TC_NT;
      float* dst = out + comp * cs;
      for (int i = tid; i < N * TC_NT; i += TC_THREADS) {
        const int r = i / TC_NT, c = i - r * TC_NT;
        if (l0 + c < nlines) dst[(size_t)r * ld + l0 + c] = Os[r * TC_NT + (c ^ (r & 31))];
      }
    }
    __syncthreads();
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512));
}

}  // namespace

int cheb_tc_kslices(int N) { return (N + 15) / 16; }

// K slices of 16 (one 64-column TMEM accumulator each, at most 7 with the persistent kernel's shared memory:
// constant matrix, BF16 tile and two FP32 tiles) bound N.
bool cheb_tc_supported(int N) { return N >= 9 && cheb_tc_kslices(N) <= 7; }

size_t cheb_tc_smem_bytes(int N) {
  const size_t KP = 16 * (size_t)cheb_tc_kslices(N);
  return 2 * (TC_ASPLIT * TC_M * KP + TC_BSPLIT * TC_NT * KP) + 2 * 4 * KP * TC_NT + 32;
}

// Four BF16 splits of the forward matrix F (N x N, row-major FP64) in the kernel's operand layout (BF16 bits).
std::vector<uint16_t> cheb_tc_matrix(const std::vector<double>& F, int N) {
  const int KS = cheb_tc_kslices(N), KP = 16 * KS, asz = TC_M * KP;
  std::vector<uint16_t> out((size_t)TC_ASPLIT * asz, 0);
  auto to_bf16 = [](double v, double* back) -> uint16_t {
    // round to nearest even in BF16 via FP32 (exact for the residuals, which carry < 24 bits)
    const float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t r = u + 0x7FFFu + ((u >> 16) & 1u);
    const uint16_t h = (uint16_t)(r >> 16);
    const uint32_t hb = (uint32_t)h << 16;
    float g;
    std::memcpy(&g, &hb, 4);
    *back = (double)g;
    return h;
  };
  for (int n = 0; n < N; ++n)
    for (int k = 0; k < N; ++k) {
      double rem = F[(size_t)n * N + k];
      for (int s = 0; s < TC_ASPLIT; ++s) {
        double b;
        out[(size_t)s * asz + kmaj_off(n, k, TC_M)] = to_bf16(rem, &b);
        rem -= b;
      }
    }
  return out;
}

cudaError_t launch_cheb_tc(int N, int nlines, int ncomp, const float* in, size_t ld, size_t cs, float* out,
                           const void* Ag, int* err, cudaStream_t st) {
  if (!cheb_tc_supported(N)) return cudaErrorInvalidValue;
  const size_t sm = cheb_tc_smem_bytes(N);
  static const bool attr = [] {
    cudaFuncSetAttribute(k_cheb_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return true;
  }();
  (void)attr;
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  const int ntiles = ((nlines + TC_NT - 1) / TC_NT) * ncomp;
  return launch_pdl(k_cheb_tc, dim3(ntiles < sms ? ntiles : sms), dim3(TC_THREADS), sm, st, N, cheb_tc_kslices(N),
                    nlines, ncomp, in, ld, cs, out, static_cast<const __nv_bfloat16*>(Ag), err);
}
