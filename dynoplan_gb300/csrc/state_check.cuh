// state_check.cuh -- validity of single states in FP64 (the oracle's
// definitions, oracle/oracle.c): positions inside the bounds (inclusive),
// and the separating-axis gap to every obstacle > 0 (touching collides).
#pragma once

#include "expand_kernels.cuh"

namespace dpg {

template <int KIND>
__device__ bool state_in_bounds64(const EnvView &ev, const double *x) {
  using R = Robot<KIND>;
#pragma unroll
  for (int d = 0; d < R::POSD; d++)
    if (!(x[d] >= ev.lo[d] && x[d] <= ev.hi[d])) return false;
  return true;
}

template <int KIND>
__device__ bool state_collides64(const RobotParams &rp, const EnvView &ev, const double *x) {
  using R = Robot<KIND>;
  if constexpr (R::SPHERE) {
    const Obs3<double> *ob = static_cast<const Obs3<double> *>(ev.obs64);
    for (int o = 0; o < ev.n_obs; o++) {
      const double dx = fabs(x[0] - ob[o].cx) - ob[o].hx, dy = fabs(x[1] - ob[o].cy) - ob[o].hy,
                   dz = fabs(x[2] - ob[o].cz) - ob[o].hz;
      const double m = fmax(dx, fmax(dy, dz));
      const double ux = fmax(dx, 0.0), uy = fmax(dy, 0.0), uz = fmax(dz, 0.0);
      if ((m <= 0 ? m : sqrt(ux * ux + uy * uy + uz * uz)) - rp.radius <= 0.0) return true;
    }
  } else {
    double px[2], py[2], pc[2], ps[2];
    sincos(x[2], &ps[0], &pc[0]);
    px[0] = x[0];
    py[0] = x[1];
    if (R::PARTS > 1) {
      sincos(x[3], &ps[1], &pc[1]);
      px[1] = x[0] - rp.hitch * pc[1];
      py[1] = x[1] - rp.hitch * ps[1];
    }
    const Obs2<double> *ob = static_cast<const Obs2<double> *>(ev.obs64);
    const double a = rp.half_len, b = rp.half_wid;
    for (int o = 0; o < ev.n_obs; o++)
#pragma unroll
      for (int q = 0; q < R::PARTS; q++) {
        const double ac = fabs(pc[q]), as = fabs(ps[q]);
        const double dx = px[q] - ob[o].cx, dy = py[q] - ob[o].cy;
        const double gx = fabs(dx) - (a * ac + b * as + ob[o].hx);
        const double gy = fabs(dy) - (a * as + b * ac + ob[o].hy);
        const double du = dx * pc[q] + dy * ps[q], dv = -dx * ps[q] + dy * pc[q];
        const double gu = fabs(du) - (a + ob[o].hx * ac + ob[o].hy * as);
        const double gv = fabs(dv) - (b + ob[o].hx * as + ob[o].hy * ac);
        if (fmax(fmax(gx, gy), fmax(gu, gv)) <= 0.0) return true;
      }
  }
  return false;
}

template <int KIND>
__device__ bool state_free64(const RobotParams &rp, const EnvView &ev, const double *x) {
  return state_in_bounds64<KIND>(ev, x) && !state_collides64<KIND>(rp, ev, x);
}

}  // namespace dpg
