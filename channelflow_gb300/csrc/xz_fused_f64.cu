// FP64 instances of the fused x/z pass (xz_fused.cuh).
#include "xz_fused.cuh"

cudaError_t launch_xz_rot(const GridDev& gp, int C, int RC, const cpx<double>* W, cpx<double>* F, const cpx<double>* twxf,
                          const cpx<double>* twzf, cudaStream_t st, const Dither& dt) {
  return xzf::run_xz_any<double>(gp, C, RC, W, F, twxf, twzf, st, dt, nullptr);
}

int xz_max_clusters_f64(const GridDev& gp, int C, int RC) {
  int n = 0;
  if (xzf::run_xz_any<double>(gp, C, RC, nullptr, nullptr, nullptr, nullptr, 0, Dither{}, &n) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}
