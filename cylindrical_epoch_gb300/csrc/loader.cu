// loader.cu -- particle loading and window injection on the device, drawn
// from the counter stream (counter_rng.cuh) instead of the reference's
// serial KISS stream.
//
// The structure is the reference's:
//  - load_particles (helper.F90:669-811): floor(npart_per_cell) particles in
//    every valid cell, in the order iy outer, ix inner; the remaining
//    floor(npart_per_cell * nvalid) - floor(npart_per_cell) nvalid particles
//    in valid cells chosen as valid(INT(U (nvalid - 1)) + 1); position
//    x = x(ix) + (U - 1/2) dx, r = y(iy) + (U - 1/2) dy, theta = 2 pi U;
//  - weights (helper.F90:707-782): the density interpolated with the
//    particle's triangle shape (gxfac fold below r = dy, neighbours outside
//    the valid map replaced by the nearer cell), times the cell volume
//    2 pi dx dy r, divided by the particles found in the particle's cell;
//  - momenta (particle_temperature.F90:30-81, 388-398): per direction a
//    normal deviate with the shape-interpolated temperature's
//    sqrt(kB T m) and the drift as mean;
//  - insert_particles (window.F90:157-300): per valid row of the new x_max
//    column, floor(npart_per_cell) particles plus one with probability
//    frac(npart_per_cell), r = y(iy) - (1/2 - U) dy, x = x0 + U dx, the
//    weight from the row-interpolated density, temperature and drift.
// Each particle is one thread: its random numbers are Philox outputs of its
// own counter, and the normal deviates come from the plain Box-Muller
// transform of two uniforms (the reference's polar rejection form would make
// the number of draws per particle random).
#include <cstdint>

#include "../../include/cyl_math.h"
#include "counter_rng.cuh"
#include "cyl_common.cuh"
#include "cyl_kernels.cuh"

namespace cyl {

namespace {

__device__ __forceinline__ int64_t map_at(const LoadParams& P, int ix, int iy) {
  return (int64_t)(ix + NG - 1) + (int64_t)P.W * (int64_t)(iy + NG - 1);
}

// three normal deviates from one Philox output (Box-Muller; the angles
// through cyl_sincos_turn, which the CPU restatement shares)
__device__ __forceinline__ void normals3(const U4& r, double& n0, double& n1, double& n2) {
  const double rho1 = sqrt(-2.0 * log(u01(r.v[0])));
  double s1, c1, s2, c2;
  cyl_sincos_turn(u01(r.v[1]), &s1, &c1);
  const double rho2 = sqrt(-2.0 * log(u01(r.v[2])));
  cyl_sincos_turn(u01(r.v[3]), &s2, &c2);
  n0 = rho1 * c1;
  n1 = rho1 * s1;
  n2 = rho2 * c2;
}

__global__ void k_load_positions(LoadParams P, const int32_t* __restrict__ valid, LoadOut o, int* npic) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const U4 r = philox4x32_10((uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)P.species, TAG_LOAD_POS,
                             P.seed);
  int64_t v;
  if (p < P.nppc * P.nvalid) v = p / P.nppc;
  else v = (int64_t)(u01(r.v[3]) * (double)(P.nvalid - 1));
  const int32_t cell = valid[v];
  const int cy = cell / P.nx, cx = cell - P.nx * cy;
  const int ix = cx + 1, iy = cy + 1;
  const double x = (P.x_grid_min + (double)(ix - 1) * P.dx) + (u01(r.v[0]) - 0.5) * P.dx;
  const double pr = (P.y_grid_min + (double)(iy - 1) * P.dy) + (u01(r.v[1]) - 0.5) * P.dy;
  double sn, cs;
  cyl_sincos_turn(u01(r.v[2]), &sn, &cs);  // theta = 2 pi U
  const double y = pr * cs, z = pr * sn;
  o.x[p] = x;
  o.y[p] = y;
  o.z[p] = z;
  // counted in the cell of the particle's shape (particle_to_grid), read
  // back below with the cell-sort formula, as the reference does
  const double part_r = sqrt(y * y + z * z);
  const int ax = (int)floor((x - P.x_grid_min) / P.dx + 0.5) + 1;
  const int ay = (int)floor((part_r - P.y_grid_min) / P.dy + 0.5) + 1;
  atomicAdd(&npic[map_at(P, ax, ay)], 1);
}

__global__ void k_load_weights(LoadParams P, const double* __restrict__ dens, const int8_t* __restrict__ dmap,
                               const int* __restrict__ npic, LoadOut o, uint32_t* wmax_bits) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const double x = o.x[p], y = o.y[p], z = o.z[p];
  const double part_r = sqrt(y * y + z * z);
  const double cxr = (x - P.x_grid_min) / P.dx, cyr = (part_r - P.y_grid_min) / P.dy;
  const int cx0 = (int)floor(cxr + 0.5), cy0 = (int)floor(cyr + 0.5);
  const double fx = (double)cx0 - cxr, fy = (double)cy0 - cyr;
  const int scx = cx0 + 1, scy = cy0 + 1;
  const double x2 = fx * fx, y2 = fy * fy;
  double gx[3], gy[3];
  gx[0] = 0.5 * ((0.25 + x2) + fx);
  gx[1] = 0.75 - x2;
  gx[2] = 0.5 * ((0.25 + x2) - fx);
  gy[0] = 0.5 * ((0.25 + y2) + fy);
  gy[1] = 0.75 - y2;
  gy[2] = 0.5 * ((0.25 + y2) - fy);
  if (part_r < P.dy) {
    gy[1] = gy[1] + gy[0];
    gy[0] = 0.0;
  }
  double wd = 0.0;
  for (int sy = -1; sy <= 1; ++sy) {
    int i = scx, j = scy + sy;
    if (!dmap[map_at(P, i, j)]) j = scy + sy / 2;
    for (int sx = -1; sx <= 1; ++sx) {
      i = scx + sx;
      if (!dmap[map_at(P, i, j)]) i = scx + sx / 2;
      wd = wd + (gx[sx + 1] * gy[sy + 1]) * dens[map_at(P, i, j)];
    }
  }
  const int ax = (int)floor((x - P.x_grid_min) / P.dx + 1.5);
  const int ay = (int)floor((part_r - P.y_grid_min) / P.dy + 1.5);
  const double vol = 2.0 * PI * P.dx * P.dy * part_r;
  const double w = wd * vol / (double)npic[map_at(P, ax, ay)];
  o.w[p] = w;
  double nrm[3];
  normals3(philox4x32_10((uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)P.species, TAG_LOAD_MOM, P.seed),
           nrm[0], nrm[1], nrm[2]);
  double* const pp[3] = {o.px, o.py, o.pz};
  for (int dir = 0; dir < 3; ++dir) {
    double tl = 0.0, dl = 0.0;
    for (int sy = -1; sy <= 1; ++sy)
      for (int sx = -1; sx <= 1; ++sx) {
        tl = tl + (gx[sx + 1] * gy[sy + 1]) * P.temp[dir];
        dl = dl + (gx[sx + 1] * gy[sy + 1]) * P.drift[dir];
      }
    pp[dir][p] = nrm[dir] * sqrt(tl * KB * P.mass) + dl;
  }
  o.id[p] = P.id_base + p;
  atomicMax(wmax_bits, __float_as_uint(fabsf(__double2float_rn(w))));
}

// Window injection in two passes, so that the particles' FP64 arithmetic is
// spread over the GPU rather than one SM per (shift, species):
//  1. k_inject_rows, one block per (shift, species): per row its count
//     (floor(ppc) plus the row's fraction bit), a block-wide exclusive scan
//     for the rows' places, and for every particle slot of the step's batch
//     its (shift, species, row), packed as c << 28 | s << 24 | row;
//  2. k_inject_particles, a grid-stride loop over the step's batch: each
//     thread makes the particle of one slot from its counter.
constexpr int INJ_THREADS = 256;
constexpr int INJ_PART_THREADS = 128, INJ_PART_BLOCKS = 64;

__device__ __forceinline__ int64_t inj_count(const InjSpecies& S, int iy, uint32_t shift, int s, uint64_t seed) {
  int64_t bit = 0;
  if (S.frac > 0.0 && u01(philox4x32_10((uint32_t)iy, shift, (uint32_t)s, TAG_INJ_COUNT, seed).v[0]) < S.frac)
    bit = 1;
  return S.nppc + bit;
}

__global__ void __launch_bounds__(INJ_THREADS) k_inject_rows(const StepRec* __restrict__ rec,
                                                             const InjSpecies* __restrict__ isp, int nsp, int ny,
                                                             uint64_t seed, int32_t* __restrict__ rowmap) {
  // blocks: MAX_INJ_SHIFTS x nsp; rows 1..ny in chunks of the block
  const int c = blockIdx.x / nsp, s = blockIdx.x - c * nsp;
  if (!rec->inj_counter || c >= rec->inj_nshift) return;
  const int64_t n = rec->inj_n[c][s];
  if (n <= 0) return;
  const InjSpecies& S = isp[s];
  const uint32_t shift = (uint32_t)rec->inj_shift[c];
  const int64_t base = rec->inj_base[c][s];
  __shared__ int64_t scan[INJ_THREADS];
  __shared__ int64_t run;
  if (threadIdx.x == 0) run = 0;
  __syncthreads();
  for (int r0 = 1; r0 <= ny; r0 += INJ_THREADS) {
    const int iy = r0 + (int)threadIdx.x;
    const int64_t cnt = iy <= ny ? inj_count(S, iy, shift, s, seed) : 0;
    scan[threadIdx.x] = cnt;
    __syncthreads();
    for (int d = 1; d < INJ_THREADS; d <<= 1) {  // inclusive Hillis-Steele scan
      const int64_t add = threadIdx.x >= (unsigned)d ? scan[threadIdx.x - d] : 0;
      __syncthreads();
      scan[threadIdx.x] += add;
      __syncthreads();
    }
    const int64_t j0 = run + scan[threadIdx.x] - cnt;
    const int32_t tag = (int32_t)(((uint32_t)c << 28) | ((uint32_t)s << 24) | (uint32_t)iy);
    for (int64_t ip = 0; ip < cnt && j0 + ip < n; ++ip) rowmap[base + j0 + ip] = tag;
    __syncthreads();
    if (threadIdx.x == INJ_THREADS - 1) run += scan[INJ_THREADS - 1];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(INJ_PART_THREADS) k_inject_particles(const StepRec* __restrict__ rec,
                                                                       const InjSpecies* __restrict__ isp, int nsp,
                                                                       double dx, double dy, double y_grid_min,
                                                                       uint64_t seed, const int32_t* __restrict__ rowmap,
                                                                       double* __restrict__ inj) {
  if (!rec->inj_counter) return;
  const int64_t g0 = rec->inject_off[0];
  int64_t total = 0;
  for (int s = 0; s < nsp; ++s) total += rec->inject_cnt[s];
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = g0 + t;
    const uint32_t tag = (uint32_t)rowmap[g];
    const int c = (int)(tag >> 28), s = (int)((tag >> 24) & 15u), iy = (int)(tag & 0xFFFFFFu);
    const InjSpecies& S = isp[s];
    const uint32_t shift = (uint32_t)rec->inj_shift[c];
    const int64_t j = g - rec->inj_base[c][s];
    const int64_t cnt = inj_count(S, iy, shift, s, seed);
    const double dens = rec->inj_dens[c][s];
    const double yg = y_grid_min + (double)(iy - 1) * dy;
    const U4 r = philox4x32_10((uint32_t)j, shift, (uint32_t)s, TAG_INJ_POS, seed);
    const double cell_frac_y = 0.5 - u01(r.v[0]);
    const double part_r = yg - cell_frac_y * dy;
    double sn, cs;
    cyl_sincos_turn(u01(r.v[1]), &sn, &cs);  // theta = 2 pi U
    const double px0 = rec->inj_x0[c] + u01(r.v[2]) * dx;
    const double wdata = (2.0 * PI * dx * dy * part_r) / (double)cnt;
    const double cy2 = cell_frac_y * cell_frac_y;
    const double gyv[3] = {0.5 * ((0.25 + cy2) + cell_frac_y), 0.75 - cy2, 0.5 * ((0.25 + cy2) - cell_frac_y)};
    double nrm[3];
    normals3(philox4x32_10((uint32_t)j, shift, (uint32_t)s, TAG_INJ_MOM, seed), nrm[0], nrm[1], nrm[2]);
    double* q = inj + g * 8;
    q[0] = px0;
    q[1] = part_r * cs;
    q[2] = part_r * sn;
    for (int i = 0; i < 3; ++i) {
      double tl = 0.0, dl = 0.0;
      for (int k = 0; k < 3; ++k) {
        tl = tl + gyv[k] * S.temp[i];
        dl = dl + gyv[k] * S.drift[i];
      }
      q[3 + i] = nrm[i] * sqrt(tl * KB * S.mass) + dl;
    }
    double wl = 0.0;
    for (int k = 0; k < 3; ++k) wl = wl + gyv[k] * dens;
    q[6] = wl * wdata;
    const int64_t id = rec->inj_id0[c][s] + j;
    q[7] = __longlong_as_double(id);
  }
}

}  // namespace

void launch_load_particles(cudaStream_t s, const LoadParams& P, const int32_t* valid, const double* dens,
                           const int8_t* dmap, int* npic, LoadOut o, uint32_t* wmax_bits) {
  if (P.n <= 0) return;
  const int T = 256;
  const unsigned blocks = (unsigned)((P.n + T - 1) / T);
  k_load_positions<<<blocks, T, 0, s>>>(P, valid, o, npic);
  k_load_weights<<<blocks, T, 0, s>>>(P, dens, dmap, npic, o, wmax_bits);
}

void launch_inject_counter(cudaStream_t s, const StepRec* rec, const InjSpecies* isp, int nsp, const RunConst& rc,
                           uint64_t seed, int32_t* rowmap, double* inj) {
  k_inject_rows<<<MAX_INJ_SHIFTS * nsp, INJ_THREADS, 0, s>>>(rec, isp, nsp, rc.ny, seed, rowmap);
  k_inject_particles<<<INJ_PART_BLOCKS, INJ_PART_THREADS, 0, s>>>(rec, isp, nsp, rc.dx, rc.dy, rc.y_grid_min, seed,
                                                                  rowmap, inj);
}

}  // namespace cyl
