// Move-size settings and proposal arithmetic shared by the chain kernels.
#pragma once

#include "gb_mc.h"

#include <cmath>

namespace gb {

// ===========================================================================
// Move settings, identical on host and device
// ===========================================================================
GB_HD double bound_d(double v, double lo, double hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

// MoveSettings::AdjustMoves / Adjust / AdjustMultiParticle
// (src/MoveSettings.cpp:157-265), called at the start of every step.
GB_HD void settings_adjust(Settings &s, long long step) {
  if ((step + 1) % s.adj != 0)
    return;
  for (int mv = 0; mv < 3; ++mv) {
    if (mv < 2) {
      if (s.tempTries[mv] > 0) {
        double currentAccept =
            (double)s.tempAccepted[mv] / (double)s.tempTries[mv];
        double fract = currentAccept / 0.5;
        if (fract > 0.0)
          s.scale[mv] *= fract;
        else
          s.scale[mv] *= 0.5;
      }
      if (mv == 0)
        s.scale[0] = bound_d(s.scale[0], 1.0e-10, (s.amin * 0.5) - 1.0e-7);
      else
        s.scale[1] = bound_d(s.scale[1], 1.0e-6, M_PI - 1.0e-7);
    }
    s.tempTries[mv] = 0;
    s.tempAccepted[mv] = 0;
  }
  for (int t = 0; t < 2; ++t) {
    if (s.mp_itries[t] > 0) {
      s.mp_tries[t] += s.mp_itries[t];
      s.mp_acc[t] += s.mp_iacc[t];
      double fTot = ((double)s.mp_acc[t] / (double)s.mp_tries[t]) / 0.3;
      double fInt = ((double)s.mp_iacc[t] / (double)s.mp_itries[t]) / 0.3;
      double &mx = (t == 0) ? s.mp_t_max : s.mp_r_max;
      if (fInt == 0.0)
        mx *= 0.5;
      else if (fabs(fInt - 0.3) > 0.1)
        mx *= ((1.0 - 0.2) * fTot + 0.2 * fInt);
      if (t == 0)
        mx = bound_d(mx, 0.001, (s.amin * 0.5) - 0.001);
      else
        mx = bound_d(mx, 0.001, M_PI - 0.001);
      s.mp_iacc[t] = 0;
      s.mp_itries[t] = 0;
    }
  }
}

// MoveSettings::Update (src/MoveSettings.cpp:100-155), one molecule kind
GB_HD void settings_update(Settings &s, int mv, int accepted) {
  s.tries[mv]++;
  s.tempTries[mv]++;
  if (accepted) {
    s.tempAccepted[mv]++;
    s.accepted[mv]++;
    s.singleMoveAccepted = 1;
  }
  if (mv == 2)
    s.singleMoveAccepted = 0;
}

// Rotation matrix from an angle and a unit axis
// (RotationMatrix::FromAxisAngle, src/TransformMatrix.h:165-214).
__device__ __forceinline__ void axis_angle_matrix(double theta, const double *u,
                                                  double *r) {
  double c = cos(theta);
  double s = sin(theta);
  double cross[9] = {0.0, -(u[2]), u[1], u[2], 0.0, -(u[0]), -(u[1]), u[0], 0.0};
  double omc = 1 - c;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = __dmul_rn(u[i], u[j]);
      double add = __dadd_rn(__dmul_rn(s, cross[3 * i + j]), __dmul_rn(omc, t));
      r[3 * i + j] = __dadd_rn(i == j ? c : 0.0, add);
    }
}

// Proposal of one move for the current scales: shift (3) or matrix (9).
__device__ __forceinline__ void make_proposal(const MoveRec &r,
                                              const Settings &s, double *prop) {
  if (r.kind == 0) {
    double bnd = s.scale[0];
    double b2 = 2.0 * bnd;
    for (int d = 0; d < 3; ++d)
      prop[d] = __dadd_rn(__dmul_rn(r.u[d], b2), -bnd);
  } else if (r.kind == 1) {
    double mx = s.scale[1];
    double theta = __dadd_rn(__dmul_rn(r.u[0], 2.0 * mx), -mx);
    axis_angle_matrix(theta, r.ax, prop);
  }
}

}  // namespace gb
