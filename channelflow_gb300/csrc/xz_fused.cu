// Host side of the fused x/z pass (kernels in xz_fused.cuh, instances in xz_fused_f32.cu / xz_fused_f64.cu):
// which grids it covers and the launch shapes (cluster size C, x rows per z chunk RC) that fit the device.
#include <algorithm>
#include <vector>

#include "xz_fused.cuh"

int xz_max_clusters_f32(const GridDev& gp, int C, int RC);
int xz_max_clusters_f64(const GridDev& gp, int C, int RC);

bool xz_fused_supported(const GridDev& gp) {
  auto ok = [](int L) { return L == 32 || L == 48 || L == 64 || L == 96 || L == 128; };
  return ok(gp.Nx) && ok(gp.Nz) && gp.NKz >= 2 && gp.NKz <= xzf::XZ_MAX_NKZ && gp.kxs == nullptr;
}

size_t xz_fused_smem(const GridDev& gp, int C, int RC, bool fp64) {
  return fp64 ? xzf::smem_bytes<double>(gp.Nx, gp.Nz, gp.NKz, C, RC)
              : xzf::smem_bytes<float>(gp.Nx, gp.Nz, gp.NKz, C, RC);
}

// Every shape the device can run: C in 2..8 with at most 32 owned kz columns per CTA, RC in {4, 8, 16}
// (bounded by the rows a CTA owns), shared memory within 227 KB and at least one cluster resident.  Sorted
// by a model of the launch: waves of resident clusters times the phases per CTA (fewer chunks first).
std::vector<XzShape> xz_fused_candidates(const GridDev& gp, bool fp64) {
  std::vector<XzShape> out;
  for (int C = 2; C <= 8; ++C) {
    if (C > gp.NKz || (gp.NKz + C - 1) / C > 32) continue;
    const int rows = (gp.Nx + C - 1) / C;
    for (int RC : {4, 8, 16}) {
      if (RC > 4 && RC / 2 >= rows) continue;
      if (xz_fused_smem(gp, C, RC, fp64) > 227 * 1024) continue;
      const int mc = fp64 ? xz_max_clusters_f64(gp, C, RC) : xz_max_clusters_f32(gp, C, RC);
      if (mc < 1) continue;
      XzShape s;
      s.C = C;
      s.RC = RC;
      const long long waves = ((long long)gp.Ny + mc - 1) / mc;
      const int chunks = (rows + RC - 1) / RC;
      // phases of one CTA: ~8 for the x transforms, 7 per z chunk; a CTA's phases shrink with C
      s.cost = (double)waves * (8.0 + 7.0 * chunks) * (1.0 + 1.0 / C);
      out.push_back(s);
    }
  }
  std::sort(out.begin(), out.end(), [](const XzShape& a, const XzShape& b) { return a.cost < b.cost; });
  return out;
}
