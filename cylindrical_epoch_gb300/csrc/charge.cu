// charge.cu -- per-mode charge density of the deposit's staggered shape, the
// diagnostic behind the discrete continuity (charge-conservation) residual.
//
// push_particles (particles.F90:515-665) deposits, per particle and mode, the
// current whose x and r differences equal the change of the particle's
// staggered-shape charge between t + dt/2 and t + 3 dt/2.  This kernel
// deposits that charge for the current state: the half-drifted position
// x + u c dt/2 / gamma (particles.F90:304-312), the cell cell_x2 and the
// h weights of particles.F90:369-388 (the ones the next push starts from),
// the 2 e^{i m theta} factor of m_fac_1 for m > 0 (particles.F90:595-611) and
// the inv_volume of each row (particles.F90:661).  Both particle layouts are
// evaluated in FP64 (the mixed layout's integer cell + FP32 offset converts
// exactly), so the residual of the mixed form measures its own error.
// Compiled without FMA contraction: on the FP64 layout every operation
// matches the oracle's.
#include "cyl_common.cuh"
#include "cyl_kernels.cuh"

namespace cyl {

template <bool MIXED>
__global__ void __launch_bounds__(256) k_charge_density(SpeciesPtrs sp, const SpeciesCounters* cnt,
                                                        const double* inv_volume, RunConst rc,
                                                        double x_grid_min, int nsh, FView rho) {
  const int64_t n = cnt->n_used;
  const double fac = 0.25;
  const double idx = 1.0 / rc.dx, idy = 1.0 / rc.dy;
  const double dtco2 = CLIGHT * (rc.dt / 2.0);
  const double ipart_mc = 1.0 / (CLIGHT * sp.mass);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double cell_x_r, part_y, part_z, w;
    if (MIXED) {
      const int32_t kx = sp.kx[i];
      if (kx == INT32_MIN) continue;
      const double ux = f2d_bits(sp.ux[i]), uy = f2d_bits(sp.uy[i]), uz = f2d_bits(sp.uz[i]);
      const double gamma_rel = sqrt(((ux * ux + uy * uy) + uz * uz) + 1.0);
      const double root = dtco2 / gamma_rel;
      cell_x_r = ((double)(kx - nsh) + f2d_bits(sp.fx[i])) + ux * root * idx;
      part_y = f2d_bits(sp.fy[i]) * rc.dy + uy * root;
      part_z = f2d_bits(sp.fz[i]) * rc.dy + uz * root;
      w = f2d_bits(sp.fw[i]);
    } else {
      const double x = sp.x[i];
      if (isnan(x)) continue;
      const double ux = sp.px[i] * ipart_mc, uy = sp.py[i] * ipart_mc, uz = sp.pz[i] * ipart_mc;
      const double gamma_rel = sqrt(((ux * ux + uy * uy) + uz * uz) + 1.0);
      const double root = dtco2 / gamma_rel;
      const double part_x = x + ux * root;
      part_y = sp.y[i] + uy * root;
      part_z = sp.z[i] + uz * root;
      cell_x_r = (part_x - x_grid_min) * idx;
      w = sp.w[i];
    }
    const double part_r = sqrt(part_y * part_y + part_z * part_z);
    const cplx exp_itheta = crecip(mk(part_y / part_r, (-part_z) / part_r));
    const double cell_y_r = (part_r - rc.y_grid_min) * idy;
    int cell_x2 = (int)floor(cell_x_r);
    const double fx = ((double)cell_x2 - cell_x_r) + 0.5;
    cell_x2 = cell_x2 + 1;
    int cell_y2 = (int)floor(cell_y_r);
    const double fy = ((double)cell_y2 - cell_y_r) + 0.5;
    cell_y2 = cell_y2 + 1;
    if (cell_x2 - 1 < 1 - NG || cell_x2 + 1 > rc.nx + NG || cell_y2 - 1 < 1 - NG || cell_y2 + 1 > rc.ny + NG)
      continue;  // outside the ghosted grid: no cell of the residual sees it
    double hx[3], hy[3];
    double cf2 = fx * fx;
    hx[0] = (0.25 + cf2) + fx;
    hx[1] = 1.5 - 2.0 * cf2;
    hx[2] = (0.25 + cf2) - fx;
    cf2 = fy * fy;
    hy[0] = (0.25 + cf2) + fy;
    hy[1] = 1.5 - 2.0 * cf2;
    hy[2] = (0.25 + cf2) - fy;
    const double qwf = sp.charge * w * fac;
    cplx mf = mk(1.0, 0.0), e_m = mk(1.0, 0.0);
    for (int im = 0; im < rc.M; ++im) {
      if (im > 0) {
        e_m = e_m * exp_itheta;
        mf = 2.0 * e_m;
      }
      for (int iy = -1; iy <= 1; ++iy) {
        const int cy = cell_y2 + iy;
        const double fr = qwf * hy[iy + 1] * inv_volume[cy - (1 - JNG)];
        for (int ix = -1; ix <= 1; ++ix) {
          const cplx v = (fr * hx[ix + 1]) * mf;
          cplx* d = rho.ptr(cell_x2 + ix, cy, im);
          atomicAdd(&d->re, v.re);
          if (im > 0) atomicAdd(&d->im, v.im);
        }
      }
    }
  }
}

// calc_number_density_modes (calc_df.F90:588-661): cell-centred weights
// (particle_to_grid.inc, triangle/gxfac.inc with gy folded for r < dy), the
// macro particle volume 2 pi dx dy r (partlist.F90:999-1013), mode factor
// 2 e^{i m theta}; FP64 atomics into the output.  Same operation order as
// the reference on the FP64 layout.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_number_density(SpeciesPtrs sp, const SpeciesCounters* cnt, RunConst rc,
                                                        double x_grid_min, int nsh, FView out) {
  const int64_t n = cnt->n_used;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double cell_x_r, y, z, wdata;
    if (MIXED) {
      const int32_t kx = sp.kx[i];
      if (kx == INT32_MIN) continue;
      cell_x_r = (double)(kx - nsh) + f2d_bits(sp.fx[i]);
      y = f2d_bits(sp.fy[i]) * rc.dy;
      z = f2d_bits(sp.fz[i]) * rc.dy;
      wdata = f2d_bits(sp.fw[i]);
    } else {
      const double x = sp.x[i];
      if (isnan(x)) continue;
      cell_x_r = (x - x_grid_min) / rc.dx;
      y = sp.y[i];
      z = sp.z[i];
      wdata = sp.w[i];
    }
    const double part_r = sqrt(y * y + z * z);
    const double cell_y_r = (part_r - rc.y_grid_min) / rc.dy;
    int cell_x = (int)floor(cell_x_r + 0.5), cell_y = (int)floor(cell_y_r + 0.5);
    const double fx = (double)cell_x - cell_x_r, fy = (double)cell_y - cell_y_r;
    cell_x = cell_x + 1;
    cell_y = cell_y + 1;
    if (cell_x - 1 < 1 - NG || cell_x + 1 > rc.nx + NG || cell_y - 1 < 1 - NG || cell_y + 1 > rc.ny + NG) continue;
    double gx[3], gy[3];
    double c2 = fx * fx;
    gx[0] = 0.5 * ((0.25 + c2) + fx);
    gx[1] = 0.75 - c2;
    gx[2] = 0.5 * ((0.25 + c2) - fx);
    c2 = fy * fy;
    gy[0] = 0.5 * ((0.25 + c2) + fy);
    gy[1] = 0.75 - c2;
    gy[2] = 0.5 * ((0.25 + c2) - fy);
    if (part_r < rc.dy) {
      gy[1] = gy[1] + gy[0];
      gy[0] = 0.0;
    }
    const double macro_part_volume = ((2.0 * PI) * rc.dx) * rc.dy * part_r;
    const double part_num_dens = wdata / macro_part_volume;
    const cplx exp_itheta = mk(y / part_r, z / part_r);
    cplx exp_imtheta = mk(1.0, 0.0), mode_fac = mk(1.0, 0.0);
    for (int im = 0; im < rc.M; ++im) {
      if (im > 0) {
        exp_imtheta = exp_imtheta * exp_itheta;
        mode_fac = 2.0 * exp_imtheta;
      }
      for (int iy = -1; iy <= 1; ++iy)
        for (int ix = -1; ix <= 1; ++ix) {
          const cplx v = ((gx[ix + 1] * gy[iy + 1]) * part_num_dens) * mode_fac;
          cplx* d = out.ptr(cell_x + ix, cell_y + iy, im);
          atomicAdd(&d->re, v.re);
          if (im > 0) atomicAdd(&d->im, v.im);
        }
    }
  }
}

// calc_boundary_modes (calc_df.F90:35-55) and field_mode_zero_gradient on the
// four boundaries, centre stagger (boundary.F90:654-707): reflecting folds
// (particle_reflection_bcs without flip, boundary.F90:833-915), periodic
// sums (particle_periodic_bcs, boundary.F90:1019-1100), then the
// zero-gradient ghost fill.  One CTA, the reference's phase order.
__global__ void k_number_density_bcs(FView f, RunConst rc, int4 bcf) {
  const int nx = rc.nx, ny = rc.ny, M = rc.M, nxg = rc.nxg, nyg = rc.nyg;
  const int bcx0 = rc.bc_allspecies[CYL_BD_X_MIN], bcx1 = rc.bc_allspecies[CYL_BD_X_MAX];
  const int bcy1 = rc.bc_allspecies[CYL_BD_Y_MAX];
  const cplx Z = mk(0.0, 0.0);
  if (bcx0 == CYL_BC_REFLECT)
    for (int t = threadIdx.x; t < (NG - 1) * nyg * M; t += blockDim.x) {
      const int i = 1 + t % (NG - 1), j = 1 - NG + (t / (NG - 1)) % nyg, m = t / ((NG - 1) * nyg);
      f(i, j, m) = (cplx)f(i, j, m) + (cplx)f(1 - i, j, m);
      f(1 - i, j, m) = Z;
    }
  __syncthreads();
  if (bcx1 == CYL_BC_REFLECT)
    for (int t = threadIdx.x; t < NG * nyg * M; t += blockDim.x) {
      const int i = 1 + t % NG, j = 1 - NG + (t / NG) % nyg, m = t / (NG * nyg);
      f(nx + 1 - i, j, m) = (cplx)f(nx + 1 - i, j, m) + (cplx)f(nx + i, j, m);
      f(nx + i, j, m) = Z;
    }
  __syncthreads();
  if (bcy1 == CYL_BC_REFLECT)
    for (int t = threadIdx.x; t < NG * nxg * M; t += blockDim.x) {
      const int i = 1 + t % NG, ix = 1 - NG + (t / NG) % nxg, m = t / (NG * nxg);
      f(ix, ny + 1 - i, m) = (cplx)f(ix, ny + 1 - i, m) + (cplx)f(ix, ny + i, m);
      f(ix, ny + i, m) = Z;
    }
  __syncthreads();
  if (bcx0 == CYL_BC_PERIODIC) {
    for (int t = threadIdx.x; t < NG * nyg * M; t += blockDim.x) {
      const int i = 1 + t % NG, j = 1 - NG + (t / NG) % nyg, m = t / (NG * nyg);
      f(i, j, m) = (cplx)f(i, j, m) + (cplx)f(nx + i, j, m);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < NG * nyg * M; t += blockDim.x) {
      const int i = 1 + t % NG, j = 1 - NG + (t / NG) % nyg, m = t / (NG * nyg);
      f(nx - NG + i, j, m) = (cplx)f(nx - NG + i, j, m) + (cplx)f(i - NG, j, m);
    }
  }
  __syncthreads();
  // zero gradient, centre stagger: ghosts copy the mirrored interior cells
  if (bcf.x != CYL_BC_PERIODIC)
    for (int t = threadIdx.x; t < NG * nyg * M; t += blockDim.x) {
      const int i = 1 + t % NG, j = 1 - NG + (t / NG) % nyg, m = t / (NG * nyg);
      f(i - NG, j, m) = (cplx)f(NG + 1 - i, j, m);
    }
  __syncthreads();
  if (bcf.y != CYL_BC_PERIODIC)
    for (int t = threadIdx.x; t < NG * nyg * M; t += blockDim.x) {
      const int i = 1 + t % NG, j = 1 - NG + (t / NG) % nyg, m = t / (NG * nyg);
      f(nx + i, j, m) = (cplx)f(nx + 1 - i, j, m);
    }
  __syncthreads();
  if (bcf.w != CYL_BC_PERIODIC)
    for (int t = threadIdx.x; t < NG * nxg * M; t += blockDim.x) {
      const int i = 1 + t % NG, ix = 1 - NG + (t / NG) % nxg, m = t / (NG * nxg);
      f(ix, ny + i, m) = (cplx)f(ix, ny + 1 - i, m);
    }
}

void launch_number_density(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, const RunConst& rc,
                           double x_grid_min, int nsh, bool mixed, const FView& out, int nblocks) {
  if (mixed)
    k_number_density<true><<<nblocks, 256, 0, s>>>(sp, cnt, rc, x_grid_min, nsh, out);
  else
    k_number_density<false><<<nblocks, 256, 0, s>>>(sp, cnt, rc, x_grid_min, nsh, out);
}

void launch_number_density_bcs(cudaStream_t s, const FView& out, const RunConst& rc, const int* bc_field) {
  k_number_density_bcs<<<1, 1024, 0, s>>>(out, rc, make_int4(bc_field[0], bc_field[1], bc_field[2], bc_field[3]));
}

void launch_charge_density(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt,
                           const double* inv_volume, const RunConst& rc, double x_grid_min, int nsh,
                           bool mixed, const FView& rho, int nblocks) {
  if (mixed)
    k_charge_density<true><<<nblocks, 256, 0, s>>>(sp, cnt, inv_volume, rc, x_grid_min, nsh, rho);
  else
    k_charge_density<false><<<nblocks, 256, 0, s>>>(sp, cnt, inv_volume, rc, x_grid_min, nsh, rho);
}

}  // namespace cyl
