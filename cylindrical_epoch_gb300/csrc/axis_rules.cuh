// axis_rules.cuh -- the r = 0 axis rules of update_e_field / update_b_field
// and the boundary constants shared by the field kernels (fields.cu) and the
// FP32 bulk updates that apply the axis rules inside their own launches
// (fields_fp32.cu).
#pragma once
#include <type_traits>

#include "cyl_common.cuh"
#include "cyl_kernels.cuh"

namespace cyl {

// Axis rules of update_e_field (fields.f90:116-180) and update_b_field
// (fields.f90:249-310).  Per column and mode they are one short sequence on
// the axis row (task 0) and the r < 0 ghost-row mirrors by mode parity
// (tasks 1 .. ng-1, ghost row ir = -task).  The mirrors read rows >= 1 (E)
// or >= 1 (B) that the axis sequence does not write (it writes row 0, and
// row 1 of Er only for m > 1, which no mirror reads), so every
// (column, mode, task) is an independent work item.
// a / d: the exact IEEE division for the FP64 form (its results must be the
// reference's), a multiplication by the host-rounded 1/d for the mixed
// form, whose E and B are FP32 anyway.
template <typename T>
__device__ __forceinline__ cplx div_form(cplx a, double d, double inv_d) {
  if constexpr (std::is_same<T, cplxf>::value) return a * inv_d;
  else return a / d;
}

static inline BcConst bc_const(const RunConst& rc, double dt) {
  BcConst k;
  const double c2 = CLIGHT * CLIGHT;
  k.c4dy = 4.0 * c2 / rc.dy;
  k.inv_eps0 = 1.0 / EPS0;
  k.inv_dx = 1.0 / rc.dx;
  k.inv_dy = 1.0 / rc.dy;
  k.inv_9 = 1.0 / 9.0;
  const double dtc2 = dt * c2;
  k.lx = dtc2 / rc.dx;
  k.lr = dtc2 / rc.dy;
  k.sum = 1.0 / (k.lx + CLIGHT);
  k.diff = k.lx - CLIGHT;
  k.dt_eps = dt / EPS0;
  const double dtc2r = dt * CLIGHT * CLIGHT;
  k.rx_lx = dtc2r / rc.dx;
  k.rx_inv_r = 1.0 / ((double)((float)rc.ny - 1.5f) * rc.dy + rc.y_grid_min);
  k.rx_dtc2_4r = 0.25 * dtc2r * k.rx_inv_r;
  k.rx_icdt_2r = ((0.5 * IMAGI) * CLIGHT) * dt * k.rx_inv_r;
  k.rx_ly = dtc2r / rc.dy;
  k.rx_sum_x = 1.0 / (k.rx_ly + CLIGHT);
  k.rx_sum_t = 1.0 / ((k.rx_ly + CLIGHT) + k.rx_dtc2_4r);
  k.rx_dt_2eps = 0.5 * dt / EPS0;
  k.rx_lx_c = (0.5 * k.rx_lx) / CLIGHT;
  return k;
}

// mode_sign of the reference for m >= 2: +1 at m = 2, alternating.
__device__ __forceinline__ double mode_sign_of(int im) { return ((im - 2) & 1) ? -1.0 : 1.0; }

template <typename T>
__device__ __forceinline__ void e_axis_item(FViewT<T> ex, FViewT<T> er, FViewT<T> et, FView jx, FViewT<T> bt,
                                            const RunConst& rc, const BcConst& K, int ix, int im, int task) {
  const double dt = rc.dt;
  if (task == 0) {
    if (im == 0) {
      ex(ix, 0, 0) = ex(ix, 0, 0) + (K.c4dy * bt(ix, 1, 0) - div_form<T>(jx(ix, 0, 0), EPS0, K.inv_eps0)) * 0.5 * dt;
      et(ix, 0, 0) = mk(0.0, 0.0);
      er(ix, 0, 0) = -er(ix, 1, 0);
    } else if (im == 1) {
      ex(ix, 0, 1) = mk(0.0, 0.0);
      er(ix, 0, 1) = (2.0 * IMAGI) * et(ix, 0, 1) - er(ix, 1, 1);
      et(ix, 0, 1) = (-IMAGI / 8.0) * (9.0 * er(ix, 1, 1) - er(ix, 2, 1));
    } else {
      ex(ix, 0, im) = mk(0.0, 0.0);
      et(ix, 0, im) = mk(0.0, 0.0);
      er(ix, 0, im) = -er(ix, 1, im);
      er(ix, 1, im) = div_form<T>(er(ix, 2, im), 9.0, K.inv_9);
    }
    return;
  }
  const int ir = -task;
  if (im == 0) {
    et(ix, ir, 0) = -et(ix, -ir, 0);
    er(ix, ir, 0) = -er(ix, -ir + 1, 0);
    ex(ix, ir, 0) = ex(ix, -ir, 0);
  } else if (im == 1) {
    et(ix, ir, 1) = et(ix, -ir, 1);
    er(ix, ir, 1) = er(ix, -ir + 1, 1);
    ex(ix, ir, 1) = -ex(ix, -ir, 1);
  } else {
    const double ms = mode_sign_of(im);
    et(ix, ir, im) = (-ms) * et(ix, -ir, im);
    er(ix, ir, im) = (-ms) * er(ix, -ir + 1, im);
    ex(ix, ir, im) = ms * ex(ix, -ir, im);
  }
}

template <typename T>
__device__ __forceinline__ void b_axis_item(FViewT<T> bx, FViewT<T> br, FViewT<T> bt, FViewT<T> ex, FViewT<T> et,
                                            const RunConst& rc, const BcConst& K, int ix, int im, int task) {
  const double dx = rc.dx, dt = rc.dt;
  if (task == 0) {
    if (im == 0) {
      br(ix, 0, 0) = mk(0.0, 0.0);
      bx(ix, 0, 0) = bx(ix, 1, 0);
      bt(ix, 0, 0) = -bt(ix, 1, 0);
    } else if (im == 1) {
      bx(ix, 0, 1) = -bx(ix, 1, 1);
      if (ix >= 2 - NG)
        br(ix, 0, 1) = br(ix, 0, 1) +
            (mk(0.0, K.inv_dy) * ex(ix, 0, 1) + div_form<T>(et(ix, 0, 1) - et(ix - 1, 0, 1), dx, K.inv_dx)) * 0.5 *
                dt;
      bt(ix, 0, 1) = (-2.0 * IMAGI) * br(ix, 0, 1) - bt(ix, 1, 1);
    } else {
      bx(ix, 0, im) = -bx(ix, 1, im);
      br(ix, 0, im) = mk(0.0, 0.0);
      bt(ix, 0, im) = -bt(ix, 1, im);
    }
    return;
  }
  const int ir = -task;
  if (im == 0) {
    bt(ix, ir, 0) = -bt(ix, -ir + 1, 0);
    br(ix, ir, 0) = -br(ix, -ir, 0);
    bx(ix, ir, 0) = bx(ix, -ir + 1, 0);
  } else if (im == 1) {
    bt(ix, ir, 1) = bt(ix, -ir + 1, 1);
    br(ix, ir, 1) = br(ix, -ir, 1);
    bx(ix, ir, 1) = -bx(ix, -ir + 1, 1);
  } else {
    const double ms = mode_sign_of(im);
    bt(ix, ir, im) = (-ms) * bt(ix, -ir + 1, im);
    br(ix, ir, im) = (-ms) * br(ix, -ir, im);
    bx(ix, ir, im) = ms * bx(ix, -ir + 1, im);
  }
}

}  // namespace cyl
