// push_fp64.cu -- plain FP64 form of the fused gather + Boris push +
// charge-conserving per-mode deposit (push_particles, particles.F90:28-734,
// with the triangle shape includes src/include/triangle/{gx,hx_dcell,
// e_part,b_part}.inc), followed in the same pass by particle_bcs
// (boundary.F90:1541-1889) for each particle.
//
// Compiled with --fmad=false: every operation below rounds once, in the
// reference's order, so positions, momenta and cell indices are bit-exact
// against the FP64 restatement when the fields are identical.  The current
// adds are FP64 atomics, whose order is the only source of difference in J.
#include "cyl_common.cuh"
#include "cyl_kernels.cuh"
#include "../../include/cyl_math.h"

namespace cyl {

__device__ __forceinline__ void catomic_add(cplx* p, cplx v) {
  atomicAdd(&p->re, v.re);
  atomicAdd(&p->im, v.im);
}

// particle_bcs for one particle (boundary.F90:1584-1860, one rank).
// Returns true when the particle leaves the system (open boundary).
__device__ __forceinline__ bool particle_bc_one(double& x, double& y, double& z, double& px,
                                                double& py, double& pz, const int* bc,
                                                double x_min, double x_max, double x_min_local,
                                                double x_max_local, const RunConst& rc) {
  const double bshift_x = rc.dx * (double)((1 + PNG + 0) / 2);
  const double x_min_outer = x_min - bshift_x, x_max_outer = x_max + bshift_x;
  const double x_shift = rc.length_x + 2.0 * rc.dx * 0.0;
  const double bshift_y = rc.dy * (double)((1 + PNG + 0) / 2);
  const double y_max_outer = rc.y_max + bshift_y;
  const double y_shift = rc.length_y + 2.0 * rc.dy * 0.0;
  bool oob = false;
  int b = 0;
  double part_pos = x;
  if (part_pos < x_min_local) {
    b = bc[CYL_BD_X_MIN];
    if (b == CYL_BC_REFLECT) {
      x = 2.0 * x_min - part_pos;
      px = -px;
    } else if (b == CYL_BC_PERIODIC) {
      x = part_pos - (-1.0) * x_shift;
    }
    if (part_pos < x_min_outer && b != CYL_BC_PERIODIC) oob = true;
  }
  if (part_pos >= x_max_local) {
    b = bc[CYL_BD_X_MAX];
    if (b == CYL_BC_REFLECT) {
      x = 2.0 * x_max - part_pos;
      px = -px;
    } else if (b == CYL_BC_PERIODIC) {
      x = part_pos - 1.0 * x_shift;
    }
    if (part_pos >= x_max_outer && b != CYL_BC_PERIODIC) oob = true;
  }
  part_pos = sqrt(y * y + z * z);
  if (part_pos >= rc.y_max_local) {
    b = bc[CYL_BD_Y_MAX];
    if (b == CYL_BC_REFLECT) {
      const double rr = 2.0 * rc.y_max / part_pos - 1.0;
      y = y * rr;
      z = z * rr;
      const double inv_final_r = 1.0 / sqrt(y * y + z * z);
      const double ct = y * inv_final_r, st = z * inv_final_r;
      const double ppr = py * ct + pz * st;
      const double ppt = (-py) * st + pz * ct;
      py = (-ppr) * ct - ppt * st;
      pz = (-ppr) * st + ppt * ct;
    } else if (b == CYL_BC_PERIODIC) {
      y = part_pos - 1.0 * y_shift;
    }
    if (part_pos >= y_max_outer && b != CYL_BC_PERIODIC) oob = true;
  }
  return oob;
}

// Three-point weighted sum of one row pair orientation, as e_part.inc:
// sum_{jj} wa(jj) * (wb(-1) F(ca-1) + wb(0) F(ca) + wb(1) F(ca+1)), row cb+jj.
__device__ __forceinline__ cplx stencil3(const FView& f, const double* wa, const double* wb, int ca,
                                         int cb, int m) {
  cplx acc;
#pragma unroll
  for (int jj = -1; jj <= 1; ++jj) {
    const cplx inner = (wb[1] * f(ca - 1, cb + jj, m) + wb[2] * f(ca, cb + jj, m)) +
                       wb[3] * f(ca + 1, cb + jj, m);
    if (jj == -1) acc = wa[jj + 2] * inner;
    else acc = acc + wa[jj + 2] * inner;
  }
  return acc;
}

__global__ void __launch_bounds__(256) k_push_fp64(FieldSet F, GeomTables g, SpeciesPtrs sp,
                                                   SpeciesCounters* cnt, const StepRec* rec,
                                                   RunConst rc, int apply_bcs, int* err) {
  const int64_t n = cnt->n_used;
  const double fac = 0.25;  // (0.5)**c_ndims
  const double dt = rc.dt;
  const double idx = 1.0 / rc.dx, idy = 1.0 / rc.dy, idt = 1.0 / dt;
  const double dto2 = dt / 2.0, dtco2 = CLIGHT * dto2;
  const double dtfac = 0.5 * dt * fac;
  const double third = 1.0 / 3.0, sixth = 0.5 * third;
  const double x_grid_min_local = rec->x_grid_min, y_grid_min_local = rc.y_grid_min;
  const double part_q = sp.charge;
  const double part_mc = CLIGHT * sp.mass;
  const double ipart_mc = 1.0 / part_mc;
  const double cmratio = (part_q * dtfac) * ipart_mc;
  const double ccmratio = CLIGHT * cmratio;
  const int M = rc.M;
  const double x_min = rec->x_min, x_max = rec->x_max;
  const double x_min_local = rec->x_min_local, x_max_local = rec->x_max_local;
  int bc[4] = {sp.bc[0], sp.bc[1], sp.bc[2], sp.bc[3]};
  int64_t ndead_local = 0;

  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double part_x = sp.x[i];
    if (isnan(part_x)) continue;  // removed particle (hole)
    double part_y = sp.y[i], part_z = sp.z[i];
    const double part_weight = sp.w[i];
    double part_ux = sp.px[i] * ipart_mc;
    double part_uy = sp.py[i] * ipart_mc;
    double part_uz = sp.pz[i] * ipart_mc;

    double gamma_rel = sqrt(((part_ux * part_ux + part_uy * part_uy) + part_uz * part_uz) + 1.0);
    double root = dtco2 / gamma_rel;
    part_x = part_x + part_ux * root;
    part_y = part_y + part_uy * root;
    part_z = part_z + part_uz * root;

    double part_x_local = part_x - x_grid_min_local;
    double part_r = sqrt(part_y * part_y + part_z * part_z);
    double part_r_local = part_r - y_grid_min_local;
    const cplx exp_min_itheta = mk(part_y / part_r, (-part_z) / part_r);
    const double theta_05 = cyl_atan2(part_z, part_y);
    const cplx exp_itheta_05 = crecip(exp_min_itheta);

    double gx[5] = {0, 0, 0, 0, 0}, gy[5] = {0, 0, 0, 0, 0};
    double hx[5] = {0, 0, 0, 0, 0}, hy[5] = {0, 0, 0, 0, 0};
    double cell_x_r = part_x_local * idx;
    double cell_y_r = part_r_local * idy;
    int cell_x1 = (int)floor(cell_x_r + 0.5);
    double cell_frac_x = (double)cell_x1 - cell_x_r;
    cell_x1 = cell_x1 + 1;
    int cell_y1 = (int)floor(cell_y_r + 0.5);
    double cell_frac_y = (double)cell_y1 - cell_y_r;
    cell_y1 = cell_y1 + 1;
    double cf2 = cell_frac_x * cell_frac_x;
    gx[1] = (0.25 + cf2) + cell_frac_x;
    gx[2] = 1.5 - 2.0 * cf2;
    gx[3] = (0.25 + cf2) - cell_frac_x;
    cf2 = cell_frac_y * cell_frac_y;
    gy[1] = (0.25 + cf2) + cell_frac_y;
    gy[2] = 1.5 - 2.0 * cf2;
    gy[3] = (0.25 + cf2) - cell_frac_y;

    int cell_x2 = (int)floor(cell_x_r);
    cell_frac_x = ((double)cell_x2 - cell_x_r) + 0.5;
    cell_x2 = cell_x2 + 1;
    int cell_y2 = (int)floor(cell_y_r);
    cell_frac_y = ((double)cell_y2 - cell_y_r) + 0.5;
    cell_y2 = cell_y2 + 1;
    cf2 = cell_frac_x * cell_frac_x;
    hx[1] = (0.25 + cf2) + cell_frac_x;
    hx[2] = 1.5 - 2.0 * cf2;
    hx[3] = (0.25 + cf2) - cell_frac_x;
    cf2 = cell_frac_y * cell_frac_y;
    hy[1] = (0.25 + cf2) + cell_frac_y;
    hy[2] = 1.5 - 2.0 * cf2;
    hy[3] = (0.25 + cf2) - cell_frac_y;

    // The gather stencil and the deposit footprint (cells cell_*2-2 .. +3)
    // must stay inside the ghosted arrays; flag and skip otherwise.
    if (cell_x1 < 2 - NG || cell_x1 > rc.nx + NG - 1 || cell_x2 < 3 - NG || cell_x2 > rc.nx + NG - 3 ||
        cell_y1 < 2 - NG || cell_y1 > rc.ny + NG - 1 || cell_y2 < 3 - NG || cell_y2 > rc.ny + NG - 3) {
      atomicOr(err, ERR_CELL_RANGE);
      continue;
    }

    // e_part.inc / b_part.inc
    double ex_part = 0.0, er_part = 0.0, et_part = 0.0;
    double bx_part = 0.0, br_part = 0.0, bt_part = 0.0;
    cplx emi = mk(1.0, 0.0);
    for (int im = 0; im < M; ++im) {
      ex_part = ex_part + (emi * stencil3(F.ex, hy, gx, cell_x1, cell_y2, im)).re;
      er_part = er_part + (emi * stencil3(F.er, gy, hx, cell_x2, cell_y1, im)).re;
      et_part = et_part + (emi * stencil3(F.et, hy, hx, cell_x2, cell_y2, im)).re;
      emi = emi * exp_min_itheta;
    }
    const double ey_part = er_part * exp_min_itheta.re + et_part * exp_min_itheta.im;
    const double ez_part = (-er_part) * exp_min_itheta.im + et_part * exp_min_itheta.re;
    emi = mk(1.0, 0.0);
    for (int im = 0; im < M; ++im) {
      bx_part = bx_part + (emi * stencil3(F.bx, gy, hx, cell_x2, cell_y1, im)).re;
      br_part = br_part + (emi * stencil3(F.br, hy, gx, cell_x1, cell_y2, im)).re;
      bt_part = bt_part + (emi * stencil3(F.bt, gy, gx, cell_x1, cell_y1, im)).re;
      emi = emi * exp_min_itheta;
    }
    const double by_part = br_part * exp_min_itheta.re + bt_part * exp_min_itheta.im;
    const double bz_part = (-br_part) * exp_min_itheta.im + bt_part * exp_min_itheta.re;

    // Boris rotation (particles.F90:404-451)
    const double uxm = part_ux + cmratio * ex_part;
    const double uym = part_uy + cmratio * ey_part;
    const double uzm = part_uz + cmratio * ez_part;
    gamma_rel = sqrt(((uxm * uxm + uym * uym) + uzm * uzm) + 1.0);
    root = ccmratio / gamma_rel;
    const double taux = bx_part * root, tauy = by_part * root, tauz = bz_part * root;
    const double taux2 = taux * taux, tauy2 = tauy * tauy, tauz2 = tauz * tauz;
    const double tau = 1.0 / (((1.0 + taux2) + tauy2) + tauz2);
    const double uxp = ((((1.0 + taux2) - tauy2) - tauz2) * uxm +
                        2.0 * ((taux * tauy + tauz) * uym + (taux * tauz - tauy) * uzm)) * tau;
    const double uyp = ((((1.0 - taux2) + tauy2) - tauz2) * uym +
                        2.0 * ((tauy * tauz + taux) * uzm + (tauy * taux - tauz) * uxm)) * tau;
    const double uzp = ((((1.0 - taux2) - tauy2) + tauz2) * uzm +
                        2.0 * ((tauz * taux + tauy) * uxm + (tauz * tauy - taux) * uym)) * tau;
    part_ux = uxp + cmratio * ex_part;
    part_uy = uyp + cmratio * ey_part;
    part_uz = uzp + cmratio * ez_part;

    const double part_u2 = (part_ux * part_ux + part_uy * part_uy) + part_uz * part_uz;
    gamma_rel = sqrt(part_u2 + 1.0);
    const double igamma = 1.0 / gamma_rel;
    root = dtco2 * igamma;
    const double delta_x = part_ux * root, delta_y = part_uy * root, delta_z = part_uz * root;
    part_x = part_x + delta_x;
    part_y = part_y + delta_y;
    part_z = part_z + delta_z;
    double nx_ = part_x, ny_ = part_y, nz_ = part_z;
    double npx = part_mc * part_ux, npy = part_mc * part_uy, npz = part_mc * part_uz;

    const double part_vy = (part_uy * CLIGHT) * igamma;
    const double part_vz = (part_uz * CLIGHT) * igamma;
    part_r = sqrt(part_y * part_y + part_z * part_z);
    const cplx exp_itheta_10 = mk(part_y / part_r, part_z / part_r);
    const double part_vt = (-part_vy) * exp_itheta_10.im + part_vz * exp_itheta_10.re;

    // deposit from the t+dt/2 to the t+3dt/2 shape (particles.F90:515-665)
    part_x_local = (part_x + delta_x) - x_grid_min_local;
    part_y = part_y + delta_y;
    part_z = part_z + delta_z;
    part_r = sqrt(part_y * part_y + part_z * part_z);
    part_r_local = part_r - y_grid_min_local;
    const cplx exp_itheta_15 = mk(part_y / part_r, part_z / part_r);
    const double theta_15 = cyl_atan2(part_z, part_y);
    const cplx exp_idtheta = exp_itheta_15 * exp_min_itheta;
    const double dtheta = theta_15 - theta_05;
#pragma unroll
    for (int k = 0; k < 5; ++k) { gx[k] = hx[k]; gy[k] = hy[k]; }
    cell_x_r = part_x_local * idx;
    cell_y_r = part_r_local * idy;
    int cell_x3 = (int)floor(cell_x_r);
    cell_frac_x = ((double)cell_x3 - cell_x_r) + 0.5;
    cell_x3 = cell_x3 + 1;
    int cell_y3 = (int)floor(cell_y_r);
    cell_frac_y = ((double)cell_y3 - cell_y_r) + 0.5;
    cell_y3 = cell_y3 + 1;
    const int dcellx = cell_x3 - cell_x2, dcelly = cell_y3 - cell_y2;
    if (dcellx < -1 || dcellx > 1 || dcelly < -1 || dcelly > 1) {
      atomicOr(err, ERR_CELL_RANGE);
      continue;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) { hx[k] = 0.0; hy[k] = 0.0; }
    cf2 = cell_frac_x * cell_frac_x;
    hx[dcellx - 1 + 2] = (0.25 + cf2) + cell_frac_x;
    hx[dcellx + 2] = 1.5 - 2.0 * cf2;
    hx[dcellx + 1 + 2] = (0.25 + cf2) - cell_frac_x;
    cf2 = cell_frac_y * cell_frac_y;
    hy[dcelly - 1 + 2] = (0.25 + cf2) + cell_frac_y;
    hy[dcelly + 2] = 1.5 - 2.0 * cf2;
    hy[dcelly + 1 + 2] = (0.25 + cf2) - cell_frac_y;
#pragma unroll
    for (int k = 0; k < 5; ++k) { hx[k] = hx[k] - gx[k]; hy[k] = hy[k] - gy[k]; }

    const int xmin = -1 + (dcellx - 1) / 2, xmax = 1 + (dcellx + 1) / 2;
    const int ymin = -1 + (dcelly - 1) / 2, ymax = 1 + (dcelly + 1) / 2;
    const double q_weight_fac = (part_q * part_weight) * fac;
    const double fcx = q_weight_fac * idt, fcy = q_weight_fac * idt, fcz = q_weight_fac * part_vt;

    cplx exp_imtheta0 = mk(1, 0), exp_imdtheta = mk(1, 0);
    cplx m_fac_2 = mk(0, 0), m_fac_3 = mk(0, 0), m_fac_4 = mk(0, 0);
    double inv_mdth = 0.0, inv_m2dth2 = 0.0;
    for (int im = 0; im < M; ++im) {
      const double mdth = (double)im * dtheta;
      const double m2dth2 = mdth * mdth;
      const bool small = fabs(mdth) < 1.0e-4;
      if (!small && im > 0) {
        inv_mdth = 1.0 / mdth;
        inv_m2dth2 = inv_mdth * inv_mdth;
      }
      if (im > 0) {
        exp_imtheta0 = exp_imtheta0 * exp_itheta_05;
        exp_imdtheta = exp_imdtheta * exp_idtheta;
        if (small) {
          const cplx m_fac_1 = 2.0 * exp_imtheta0;
          m_fac_2 = m_fac_1 * ((mk(1.0, 0.0) + (0.5 * IMAGI) * mdth) - sixth * m2dth2);
          m_fac_3 = m_fac_1 * ((mk(0.5, 0.0) + (third * IMAGI) * mdth) - 0.125 * m2dth2);
          m_fac_4 = m_fac_1 * ((mk(third, 0.0) + (0.25 * IMAGI) * mdth) - 0.1 * m2dth2);
        } else {
          const cplx m_fac_1 = (2.0 * inv_mdth) * exp_imtheta0;
          m_fac_2 = m_fac_1 * ((-IMAGI) * (exp_imdtheta - 1.0));
          m_fac_3 = m_fac_1 * (inv_mdth * ((exp_imdtheta * (mk(1.0, 0.0) - IMAGI * mdth)) - 1.0));
          m_fac_4 = m_fac_1 * ((IMAGI * inv_m2dth2) *
                               ((exp_imdtheta * (((-m2dth2) - (2.0 * IMAGI) * mdth) + 2.0)) - 2.0));
        }
      }
      cplx jyh[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) jyh[k] = mk(0, 0);
      for (int iy = ymin; iy <= ymax; ++iy) {
        const int cy = cell_y2 + iy;
        cplx w_rt, ym_fac_1;
        if (im == 0) {
          w_rt = mk(gy[iy + 2] + 0.5 * hy[iy + 2], 0.0);
          ym_fac_1 = mk(0.5 * gy[iy + 2] + third * hy[iy + 2], 0.0);
        } else {
          w_rt = m_fac_2 * gy[iy + 2] + m_fac_3 * hy[iy + 2];
          ym_fac_1 = m_fac_3 * gy[iy + 2] + m_fac_4 * hy[iy + 2];
        }
        const double fjx = fcx * g.inv_area_rt[cy - (1 - JNG)];
        const double fjy = (fcy * hy[iy + 2]) * g.inv_area_xt[cy - (0 - JNG)];
        const double fjz = fcz * g.inv_volume[cy - (1 - JNG)];
        const double rat = g.ratio_area_xt[cy - (1 - JNG)];
        cplx jxh = mk(0, 0);
        for (int ix = xmin; ix <= xmax; ++ix) {
          const int cx = cell_x2 + ix;
          cplx w_xt;
          if (im == 0) w_xt = mk(gx[ix + 2] + 0.5 * hx[ix + 2], 0.0);
          else w_xt = m_fac_2 * gx[ix + 2] + m_fac_3 * hx[ix + 2];
          const cplx w_xr = gx[ix + 2] * w_rt + hx[ix + 2] * ym_fac_1;
          jxh = jxh - (fjx * hx[ix + 2]) * w_rt;
          jyh[ix + 2] = jyh[ix + 2] * rat - fjy * w_xt;
          const cplx jzh = fjz * w_xr;
          catomic_add(F.jx.ptr(cx + 1, cy, im), jxh);
          catomic_add(F.jr.ptr(cx, cy + 1, im), jyh[ix + 2]);
          catomic_add(F.jt.ptr(cx, cy, im), jzh);
        }
      }
    }

    bool dead = false;
    if (apply_bcs)
      dead = particle_bc_one(nx_, ny_, nz_, npx, npy, npz, bc, x_min, x_max, x_min_local, x_max_local, rc);
    if (dead) {
      nx_ = __longlong_as_double(0x7ff8000000000000LL);
      ndead_local++;
    }
    sp.x[i] = nx_;
    sp.y[i] = ny_;
    sp.z[i] = nz_;
    sp.px[i] = npx;
    sp.py[i] = npy;
    sp.pz[i] = npz;
  }
  if (ndead_local) atomicAdd((unsigned long long*)&cnt->n_dead, (unsigned long long)ndead_local);
}

// The FP64 kernel's atan2 (include/cyl_math.h) on n arguments, for the test
// that the device evaluates it bit for bit as the host does.
__global__ void k_eval_atan2(const double* y, const double* x, double* out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = cyl_atan2(y[i], x[i]);
}

void launch_eval_atan2(cudaStream_t s, const double* y, const double* x, double* out, int64_t n) {
  k_eval_atan2<<<1216, 256, 0, s>>>(y, x, out, n);
}

void launch_push_fp64(cudaStream_t s, const FieldSet& F, const GeomTables& g, const SpeciesPtrs& sp,
                      SpeciesCounters* cnt, const StepRec* rec, const RunConst& rc, int apply_bcs,
                      int* err, int nblocks) {
  k_push_fp64<<<nblocks, 256, 0, s>>>(F, g, sp, cnt, rec, rc, apply_bcs, err);
}

}  // namespace cyl
