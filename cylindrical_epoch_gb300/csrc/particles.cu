// particles.cu -- particle boundary pass, moving-window particle work,
// diagnostics reductions and the counting sort by cell.
//
// Particles live in SoA arrays (x, y, z, px, py, pz, w, id), one set per
// species.  A particle removed by an open boundary becomes a hole (x = NaN)
// that every kernel skips; the counting sort drops holes and orders the
// survivors by cell so the push reads neighbouring fields and writes
// neighbouring currents.
#include "cyl_common.cuh"
#include "cyl_kernels.cuh"

namespace cyl {

__device__ __forceinline__ double nan_hole() { return __longlong_as_double(0x7ff8000000000000LL); }

// particle_bcs (boundary.F90:1584-1860) for one particle, one rank
__device__ __forceinline__ bool pbc_one(double& x, double& y, double& z, double& px, double& py,
                                        double& pz, const int* bc, double x_min, double x_max,
                                        double x_min_local, double x_max_local, const RunConst& rc) {
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

// Standalone particle_bcs pass.  after_shift selects the grid of the
// moving window after this step's shift; then particles behind the new
// x_min are removed first (remove_particles, window.F90:304-325).
__global__ void k_particle_bcs(SpeciesPtrs sp, SpeciesCounters* cnt, const StepRec* rec,
                               int after_shift, RunConst rc) {
  if (after_shift && rec->nshift == 0) return;
  const int64_t n = cnt->n_used;
  const double x_min = after_shift ? rec->x_min_after : rec->x_min;
  const double x_max = after_shift ? rec->x_max_after : rec->x_max;
  const double xl = after_shift ? rec->x_min_local_after : rec->x_min_local;
  const double xh = after_shift ? rec->x_max_local_after : rec->x_max_local;
  int bc[4] = {sp.bc[0], sp.bc[1], sp.bc[2], sp.bc[3]};
  int64_t dead = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double x = sp.x[i];
    if (isnan(x)) continue;
    if (after_shift && x < x_min) {
      sp.x[i] = nan_hole();
      dead++;
      continue;
    }
    double y = sp.y[i], z = sp.z[i], px = sp.px[i], py = sp.py[i], pz = sp.pz[i];
    const double x0 = x, y0 = y, z0 = z, px0 = px, py0 = py, pz0 = pz;
    bool oob = pbc_one(x, y, z, px, py, pz, bc, x_min, x_max, xl, xh, rc);
    if (oob) {
      sp.x[i] = nan_hole();
      dead++;
      continue;
    }
    if (x != x0) sp.x[i] = x;
    if (y != y0) sp.y[i] = y;
    if (z != z0) sp.z[i] = z;
    if (px != px0) sp.px[i] = px;
    if (py != py0) sp.py[i] = py;
    if (pz != pz0) sp.pz[i] = pz;
  }
  if (dead) atomicAdd((unsigned long long*)&cnt->n_dead, (unsigned long long)dead);
}

// Append this step's injected particles (insert_particles, window.F90:157-300,
// generated on the host by the KISS stream); 8 doubles per particle:
// x, y, z, px, py, pz, w, id (bit pattern).
__global__ void k_append(SpeciesPtrs sp, SpeciesCounters* cnt, const double* inject,
                         const StepRec* rec, int isp, int* err) {
  const int64_t off = rec->inject_off[isp], k = rec->inject_cnt[isp];
  const int64_t base = cnt->n_used;
  if (base + k > sp.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERR_CAPACITY);
    return;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double* q = inject + (off + i) * 8;
    const int64_t d = base + i;
    sp.x[d] = q[0];
    sp.y[d] = q[1];
    sp.z[d] = q[2];
    sp.px[d] = q[3];
    sp.py[d] = q[4];
    sp.pz[d] = q[5];
    sp.w[d] = q[6];
    sp.id[d] = __double_as_longlong(q[7]);
  }
}
__global__ void k_append_commit(SpeciesPtrs sp, SpeciesCounters* cnt, const StepRec* rec, int isp) {
  const int64_t k = rec->inject_cnt[isp];
  if (cnt->n_used + k <= sp.cap) cnt->n_used += k;
}

void launch_particle_bcs(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                         const StepRec* rec, int after_shift, const RunConst& rc, int nblocks) {
  k_particle_bcs<<<nblocks, 256, 0, s>>>(sp, cnt, rec, after_shift, rc);
}

void launch_window_particles(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                             const double* inject, const StepRec* rec, int isp, const RunConst& rc,
                             int* err, int nblocks) {
  k_append<<<64, 256, 0, s>>>(sp, cnt, inject, rec, isp, err);
  k_append_commit<<<1, 1, 0, s>>>(sp, cnt, rec, isp);
  k_particle_bcs<<<nblocks, 256, 0, s>>>(sp, cnt, rec, 1, rc);
}

// Cell-sort indices of split_particle.F90:61-62 for every slot; live[i] = 0
// marks a hole.
__global__ void k_cell_indices(SpeciesPtrs sp, const SpeciesCounters* cnt, double x_grid_min,
                               RunConst rc, int32_t* cx, int32_t* cy, int32_t* live) {
  const int64_t n = cnt->n_used;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = sp.x[i];
    if (isnan(x)) {
      live[i] = 0;
      continue;
    }
    const double y = sp.y[i], z = sp.z[i];
    const double part_r = sqrt(y * y + z * z);
    cx[i] = (int32_t)floor((x - x_grid_min) / rc.dx + 1.5);
    cy[i] = (int32_t)floor((part_r - rc.y_grid_min) / rc.dy + 1.5);
    live[i] = 1;
  }
}

void launch_cell_indices(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt,
                         double x_grid_min, const RunConst& rc, int32_t* cx, int32_t* cy,
                         int32_t* live, int nblocks) {
  k_cell_indices<<<nblocks, 256, 0, s>>>(sp, cnt, x_grid_min, rc, cx, cy, live);
}

// Kinetic energy sum w m c^2 (gamma - 1), gamma - 1 = u^2/(gamma + 1)
// (calc_df.F90:1246-1291); out[0] += energy, out[1] += live count.
__global__ void k_energy(SpeciesPtrs sp, const SpeciesCounters* cnt, double* out) {
  const int64_t n = cnt->n_used;
  const double mc = CLIGHT * sp.mass, mc2 = CLIGHT * mc;
  double e = 0.0, c = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (isnan(sp.x[i])) continue;
    const double ux = sp.px[i] / mc, uy = sp.py[i] / mc, uz = sp.pz[i] / mc;
    const double u2 = ux * ux + uy * uy + uz * uz;
    e += sp.w[i] * mc2 * (u2 / (sqrt(u2 + 1.0) + 1.0));
    c += 1.0;
  }
  double v[2] = {e, c};
  block_sum_add<2>(v, out);
}

void launch_energy(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, double* out,
                   int nblocks) {
  k_energy<<<nblocks, 256, 0, s>>>(sp, cnt, out);
}

// Per-mode field energy over the interior: m = 0 contributes |F_0|^2, m >= 1
// contributes |F_m|^2 / 2 (F = Re sum F_m e^{-im theta}), cell volume 2 pi r dx dr.
// Blocks stride over the interior cells of mode blockIdx.y; one atomic per
// block and sum.
template <typename T>
__global__ void k_field_energy(FieldSetT<T> F, RunConst rc, double* out) {
  const int m = blockIdx.y;
  const int ncell = rc.nx * rc.ny;
  const double mf = (m == 0) ? 1.0 : 0.5;
  auto a2 = [](cplx v) { return v.re * v.re + v.im * v.im; };
  double v[3] = {0.0, 0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
    const int iy = 1 + c / rc.nx, ix = 1 + (c - (iy - 1) * rc.nx);
    const double r = (double)iy * rc.dy;
    const double vol = 2.0 * PI * r * rc.dx * rc.dy;
    v[0] += mf * vol * (a2(F.ex(ix, iy, m)) + a2(F.er(ix, iy, m)) + a2(F.et(ix, iy, m)));
    v[1] += mf * vol * (a2(F.bx(ix, iy, m)) + a2(F.br(ix, iy, m)) + a2(F.bt(ix, iy, m)));
    v[2] += sqrt(a2(F.jx(ix, iy, m))) + sqrt(a2(F.jr(ix, iy, m))) + sqrt(a2(F.jt(ix, iy, m)));
  }
  block_sum_add<3>(v, out);
}

template <typename T>
void launch_field_energy(cudaStream_t s, const FieldSetT<T>& F, const RunConst& rc, double* out) {
  const int ncell = rc.nx * rc.ny;
  int bx = (ncell + 255) / 256;
  if (bx > 152 * 4) bx = 152 * 4;
  dim3 blk(256), grd(bx, rc.M);
  k_field_energy<T><<<grd, blk, 0, s>>>(F, rc, out);
}
template void launch_field_energy<cplx>(cudaStream_t, const FieldSet&, const RunConst&, double*);
template void launch_field_energy<cplxf>(cudaStream_t, const FieldSetF&, const RunConst&, double*);

// ------------------------------------------------------------- sorting

// Key of a particle: its cell (cell_x1, cell_y1 of the push) in the ghosted
// grid; holes get the sentinel ncells so they sort last and are dropped.
__global__ void k_sort_keys(SpeciesPtrs sp, const SpeciesCounters* cnt, const double* xgm,
                            RunConst rc, int32_t* keys, int32_t* hist, int ncells) {
  const int64_t n = cnt->n_used;
  const double x_grid_min = *xgm;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = sp.x[i];
    int key = ncells;
    if (!isnan(x)) {
      const double r = sqrt(sp.y[i] * sp.y[i] + sp.z[i] * sp.z[i]);
      int cx = (int)floor((x - x_grid_min) / rc.dx + 0.5) + NG;  // 0-based ghosted column
      int cy = (int)floor((r - rc.y_grid_min) / rc.dy + 0.5) + NG;
      cx = cx < 0 ? 0 : (cx >= rc.nxg ? rc.nxg - 1 : cx);
      cy = cy < 0 ? 0 : (cy >= rc.nyg ? rc.nyg - 1 : cy);
      key = cy * rc.nxg + cx;
    }
    keys[i] = key;
    atomicAdd(&hist[key], 1);
  }
}

// Exclusive scan of hist[0..n) in place, three kernels (block sums, scan of
// the block sums in one CTA, add back).
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;

__device__ int block_exclusive_scan(int v, int* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  int prefix = (warp > 0) ? sh[warp - 1] : 0;
  int total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  sh[32] = total;
  return prefix + x - v;
}

__global__ void k_scan_local(int* data, int n, int* block_sums) {
  __shared__ int sh[40];
  const int base = blockIdx.x * SCAN_BLOCK * SCAN_ITEMS + threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int tsum = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = (base + k < n) ? data[base + k] : 0;
    tsum += v[k];
  }
  int ex = block_exclusive_scan(tsum, sh);
  __syncthreads();
  int run = ex;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    if (base + k < n) data[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = sh[32];
}

__global__ void k_scan_sums(int* block_sums, int nb) {
  __shared__ int sh[40];
  // one CTA, sequential chunks of blockDim.x
  int carry = 0;
  for (int base = 0; base < nb; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = (i < nb) ? block_sums[i] : 0;
    int ex = block_exclusive_scan(v, sh);
    int tot = sh[32];
    __syncthreads();
    if (i < nb) block_sums[i] = ex + carry;
    carry += tot;
    __syncthreads();
  }
}

__global__ void k_scan_add(int* data, int n, const int* block_sums) {
  const int base = blockIdx.x * SCAN_BLOCK * SCAN_ITEMS + threadIdx.x * SCAN_ITEMS;
  const int add = block_sums[blockIdx.x];
  for (int k = 0; k < SCAN_ITEMS; ++k)
    if (base + k < n) data[base + k] += add;
}

void scan_exclusive(cudaStream_t s, int32_t* data, int n, int32_t* block_sums) {
  const int per = SCAN_BLOCK * SCAN_ITEMS;
  const int nb = (n + per - 1) / per;
  k_scan_local<<<nb, SCAN_BLOCK, 0, s>>>(data, n, block_sums);
  k_scan_sums<<<1, SCAN_BLOCK, 0, s>>>(block_sums, nb);
  k_scan_add<<<nb, SCAN_BLOCK, 0, s>>>(data, n, block_sums);
}

__global__ void k_sort_copy_out(SpeciesPtrs sp, const SpeciesCounters* cnt, double* tmp,
                                int64_t* tmp_id, int64_t cap) {
  const int64_t n = cnt->n_used;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    tmp[i] = sp.x[i];
    tmp[cap + i] = sp.y[i];
    tmp[2 * cap + i] = sp.z[i];
    tmp[3 * cap + i] = sp.px[i];
    tmp[4 * cap + i] = sp.py[i];
    tmp[5 * cap + i] = sp.pz[i];
    tmp[6 * cap + i] = sp.w[i];
    tmp_id[i] = sp.id[i];
  }
}

__global__ void k_sort_scatter(SpeciesPtrs sp, const SpeciesCounters* cnt, const double* tmp,
                               const int64_t* tmp_id, int64_t cap, const int32_t* keys,
                               int32_t* offs, int ncells) {
  const int64_t n = cnt->n_used;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int key = keys[i];
    if (key >= ncells) continue;
    const int64_t d = atomicAdd(&offs[key], 1);
    sp.x[d] = tmp[i];
    sp.y[d] = tmp[cap + i];
    sp.z[d] = tmp[2 * cap + i];
    sp.px[d] = tmp[3 * cap + i];
    sp.py[d] = tmp[4 * cap + i];
    sp.pz[d] = tmp[5 * cap + i];
    sp.w[d] = tmp[6 * cap + i];
    sp.id[d] = tmp_id[i];
  }
}

__global__ void k_sort_commit(SpeciesCounters* cnt, const int32_t* offs_end, int ncells) {
  // after the scatter, offs[ncells-1] is the end of the last live cell
  cnt->n_used = offs_end[ncells - 1];
  cnt->n_dead = 0;
}

void sort_species(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, SortScratch& sc,
                  const double* x_grid_min, const RunConst& rc, int nblocks) {
  const int nc = sc.ncells;
  cudaMemsetAsync(sc.hist, 0, sizeof(int32_t) * (nc + 1), s);
  k_sort_keys<<<nblocks, 256, 0, s>>>(sp, cnt, x_grid_min, rc, sc.keys, sc.hist, nc);
  const int n = nc + 1;
  const int per = SCAN_BLOCK * SCAN_ITEMS;
  const int nb = (n + per - 1) / per;
  int32_t* block_sums = (int32_t*)sc.perm;  // reuse scratch as int buffer
  k_scan_local<<<nb, SCAN_BLOCK, 0, s>>>(sc.hist, n, block_sums);
  k_scan_sums<<<1, SCAN_BLOCK, 0, s>>>(block_sums, nb);
  k_scan_add<<<nb, SCAN_BLOCK, 0, s>>>(sc.hist, n, block_sums);
  k_sort_copy_out<<<nblocks, 256, 0, s>>>(sp, cnt, sc.tmp, sc.tmp_id, sc.cap);
  k_sort_scatter<<<nblocks, 256, 0, s>>>(sp, cnt, sc.tmp, sc.tmp_id, sc.cap, sc.keys, sc.hist, nc);
  k_sort_commit<<<1, 1, 0, s>>>(cnt, sc.hist, nc);
}

}  // namespace cyl
