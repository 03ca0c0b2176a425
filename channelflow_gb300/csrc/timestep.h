// TimeStep (channelflow/dnsflags.cpp:736-972) on the host, shared by the f^T(u) entry point and the
// request server.
#pragma once

#include <algorithm>
#include <climits>
#include <string>

#include "../../include/cfgpu.h"

int cfgpu_record_error(int code, const std::string& msg);

// ---------------------------------------------------------------------------
// TimeStep (channelflow/dnsflags.cpp:736-972): dt within [dtmin, dtmax] with
// dT = n dt, CFL kept within [CFLmin, CFLmax] by adjust(); same arithmetic.
// ---------------------------------------------------------------------------
namespace cfgpu_rt {
inline int iround_h(double x) { return int(x > 0.0 ? x + 0.5 : x - 0.5); }

struct TimeStepH {
  int n = 0, N = 0;
  double dt = 0, dtmin = 0, dtmax = 0, dT = 0, T = 0, CFLmin = 0, CFL = 0, CFLmax = 0;
  bool variable = false;
  double value() const { return dT / n; }  // TimeStep::operator Real

  int init(const cfgpu_timestep& t) {
    dt = t.dt; dtmin = t.dtmin; dtmax = t.dtmax; dT = t.dT; CFLmin = t.CFLmin; CFLmax = t.CFLmax;
    variable = t.variable != 0;
    CFL = (CFLmax + CFLmin) / 2;
    if (dtmin < 0 || dt < dtmin || dtmax < dt) return cfgpu_record_error(CFGPU_EINVAL, "TimeStep: 0 <= dtmin <= dt <= dtmax");
    if (CFLmin < 0 || CFLmax < CFLmin) return cfgpu_record_error(CFGPU_EINVAL, "TimeStep: 0 <= CFLmin <= CFLmax");
    if (dT < dtmin) return cfgpu_record_error(CFGPU_EINVAL, "TimeStep: dT < dtmin");
    n = std::max(iround_h(dT / dt), 1);
    dt = dT / n;
    while (dt < dtmin && n >= 2 && dT != 0) dt = dT / --n;
    while (dt > dtmax && n <= INT_MAX && dT != 0) dt = dT / ++n;
    return CFGPU_OK;
  }
  bool adjust(double c) {
    CFL = c;
    if (variable && (c <= CFLmin || c >= CFLmax)) return adjust_to_middle(c);
    return false;
  }
  bool adjust_to_middle(double c) {
    if (dtmin == dtmax || dT == 0.0) return false;
    int nn = std::max(iround_h(2 * n * c / (CFLmax + CFLmin)), 1);
    double d = dT / nn;
    while (d < dtmin && d < dT) d = dT / --nn;
    while (d > dtmax && nn <= INT_MAX) d = dT / ++nn;
    c *= d / dt;
    const bool adj = nn != n;
    if (adj) {
      n = nn;
      dt = d;
      CFL = c;
    }
    return adj;
  }
  bool adjust_for_T(double TT) {
    T = TT;
    if (TT == 0) {
      const bool adj = dt != 0;
      dt = 0; n = 0; dT = 0; T = 0;
      return adj;
    }
    const int NN = std::max(iround_h(TT / dT), 1);
    const double dTT = TT / NN;
    int nn = std::max(iround_h(dTT / dt), 1);
    double d = dTT / nn;
    while (d < dtmin && nn > 2 && dTT != 0) d = dTT / --nn;
    while (d > dtmax && nn <= INT_MAX && dTT != 0) d = dTT / ++nn;
    const double c = d * CFL / dt;
    const bool adj = d != dt;
    n = nn; N = NN; dt = d; dT = dTT; CFL = c;
    return adj;
  }
};
}  // namespace cfgpu_rt
