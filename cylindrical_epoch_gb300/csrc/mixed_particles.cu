// mixed_particles.cu -- particle kernels of the mixed-precision form that
// depend on its layout: conversion from/to the FP64 Cartesian form at the
// C ABI, moving-window append + removal + particle_bcs, kinetic energy,
// cell-sort indices and the counting sort by tile.
#include <climits>

#include "cyl_common.cuh"
#include "cyl_kernels.cuh"
#include "push_mixed.cuh"

namespace cyl {

void scan_exclusive(cudaStream_t s, int32_t* data, int n, int32_t* block_sums);  // particles.cu

MixedParams mixed_params(const SpeciesPtrs& sp, const RunConst& rc) {
  MixedParams P{};
  const double fac = 0.25;
  P.cdt2_dx = (float)(CLIGHT * rc.dt / 2.0 / rc.dx);
  P.cdt2_dy = (float)(CLIGHT * rc.dt / 2.0 / rc.dy);
  const double cm = sp.charge * (0.5 * rc.dt * fac) / (CLIGHT * sp.mass);
  P.cmratio = (float)cm;
  P.ccmratio = (float)(CLIGHT * cm);
  P.q_fac = (float)(sp.charge * fac);
  P.idt = (float)(1.0 / rc.dt);
  P.c = (float)CLIGHT;
  P.r_hi = (float)(rc.y_max_local / rc.dy);
  P.r_sys = (float)(rc.y_max / rc.dy);
  P.r_out = (float)((rc.y_max + rc.dy * 2.0) / rc.dy);
  return P;
}



__global__ void k_from_double(SpeciesPtrs sp, const double* st, int64_t n, int64_t cap, double xg0,
                              RunConst rc) {
  const MixedScale k = mixed_scale(sp, rc);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    to_mixed(sp, i, st[i], st[cap + i], st[2 * cap + i], st[3 * cap + i], st[4 * cap + i], st[5 * cap + i],
             st[6 * cap + i], xg0, k);
    sp.id[i] = __double_as_longlong(st[7 * cap + i]);
  }
}

__global__ void k_to_double(SpeciesPtrs sp, double* st, int64_t n, int64_t cap, double xg0, RunConst rc) {
  const double mc = sp.mass * CLIGHT;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = sp.kx[i];
    st[i] = (k == INT32_MIN) ? __longlong_as_double(0x7ff8000000000000LL)
                             : xg0 + ((double)k + (double)sp.fx[i]) * rc.dx;
    st[cap + i] = (double)sp.fy[i] * rc.dy;
    st[2 * cap + i] = (double)sp.fz[i] * rc.dy;
    st[3 * cap + i] = (double)sp.ux[i] * mc;
    st[4 * cap + i] = (double)sp.uy[i] * mc;
    st[5 * cap + i] = (double)sp.uz[i] * mc;
    st[6 * cap + i] = (double)sp.fw[i];
    st[7 * cap + i] = __longlong_as_double(sp.id[i]);
  }
}

void mixed_from_double(cudaStream_t s, const SpeciesPtrs& sp, const double* stage, int64_t n, int64_t cap,
                       double xg0, const RunConst& rc) {
  k_from_double<<<1024, 256, 0, s>>>(sp, stage, n, cap, xg0, rc);
}
void mixed_to_double(cudaStream_t s, const SpeciesPtrs& sp, double* stage, int64_t n, int64_t cap,
                     double xg0, const RunConst& rc) {
  k_to_double<<<1024, 256, 0, s>>>(sp, stage, n, cap, xg0, rc);
}

// FP32 values widened to FP64 (exact), for the downloads of the mixed form's
// FP32 field arrays.
__global__ void k_widen(const float* src, double* dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

void widen_f32(cudaStream_t s, const float* src, double* dst, int64_t n) {
  k_widen<<<1024, 256, 0, s>>>(src, dst, n);
}

// What an upload of n particles (weights w, ids id, on the device) adds to
// its species' counters: the largest |w| rounded to FP32 (its bits, which
// order as the non-negative values do) into cnt->wmax_bits, and the largest
// id into *max_id (the caller sets both to their starting values).
__global__ void k_upload_stats(const double* w, const int64_t* id, int64_t n, SpeciesCounters* cnt,
                               long long* max_id) {
  unsigned wb = 0u;
  long long mid = -1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned b = __float_as_uint(fabsf((float)w[i]));
    wb = b > wb ? b : wb;
    const long long v = (long long)id[i];
    mid = v > mid ? v : mid;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned wo = __shfl_down_sync(0xffffffffu, wb, o);
    const long long mo = __shfl_down_sync(0xffffffffu, mid, o);
    wb = wo > wb ? wo : wb;
    mid = mo > mid ? mo : mid;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&cnt->wmax_bits, wb);
    atomicMax(max_id, mid);
  }
}

void upload_stats(cudaStream_t s, const double* w, const int64_t* id, int64_t n, SpeciesCounters* cnt,
                  long long* max_id) {
  if (n > 0) k_upload_stats<<<256, 256, 0, s>>>(w, id, n, cnt, max_id);
}

// particle_bcs in the cell units of a grid whose cell_x_r origin is
// x_grid_min: xc = kx - nsh + fx (boundary.F90:1584-1860).
__device__ __forceinline__ bool mixed_bc(const SpeciesPtrs& sp, int64_t i, int nsh, float xlo, float xhi,
                                         float xs_lo, float xs_hi, float xo_lo, float xo_hi, float r_hi,
                                         float r_sys, float r_out, int nx) {
  int k = sp.kx[i] - nsh;
  float f = sp.fx[i];
  const float xc = (float)k + f;
  float ux = sp.ux[i];
  bool dead = false, changed = false;
  if (xc < xlo) {
    const int b = sp.bc[CYL_BD_X_MIN];
    if (b == CYL_BC_REFLECT) {
      const float v = 2.0f * xs_lo - xc;
      k = (int)floorf(v); f = v - (float)k; ux = -ux; changed = true;
    } else if (b == CYL_BC_PERIODIC) {
      k += nx; changed = true;
    }
    if (xc < xo_lo && b != CYL_BC_PERIODIC) dead = true;
  }
  if (xc >= xhi) {
    const int b = sp.bc[CYL_BD_X_MAX];
    if (b == CYL_BC_REFLECT) {
      const float v = 2.0f * xs_hi - xc;
      k = (int)floorf(v); f = v - (float)k; ux = -ux; changed = true;
    } else if (b == CYL_BC_PERIODIC) {
      k -= nx; changed = true;
    }
    if (xc >= xo_hi && b != CYL_BC_PERIODIC) dead = true;
  }
  float y = sp.fy[i], z = sp.fz[i];
  const float rn = sqrtf(y * y + z * z);
  if (rn >= r_hi) {
    const int b = sp.bc[CYL_BD_Y_MAX];
    if (b == CYL_BC_REFLECT) {
      const float fr = 2.0f * r_sys / rn - 1.0f;
      y *= fr; z *= fr;
      const float rr = sqrtf(y * y + z * z);
      const float cc = y / rr, ss = z / rr;
      const float uy = sp.uy[i], uz = sp.uz[i];
      const float pr = uy * cc + uz * ss, pt = -uy * ss + uz * cc;
      sp.uy[i] = -pr * cc - pt * ss;
      sp.uz[i] = -pr * ss + pt * cc;
      sp.fy[i] = y;
      sp.fz[i] = z;
    }
    if (rn >= r_out && b != CYL_BC_PERIODIC) dead = true;
  }
  if (dead) {
    sp.kx[i] = INT32_MIN;
    return true;
  }
  if (changed) {
    sp.kx[i] = k + nsh;
    sp.fx[i] = f;
    sp.ux[i] = ux;
  }
  return false;
}

// bid, nb: the block index and block count of the grid-stride loop
__device__ __forceinline__ void mixed_bcs_body(const SpeciesPtrs& sp, SpeciesCounters* cnt, const StepRec* rec,
                                               int after, const MixedParams& P, const RunConst& rc, int bid,
                                               int nb) {
  if (after && rec->nshift == 0) return;
  const int64_t n = cnt->n_used;
  const int nsh = after ? rec->nshift_total_after : rec->nshift_total;
  const double xgm = after ? rec->x_grid_min_after : rec->x_grid_min;
  const float xs_lo = (float)(((after ? rec->x_min_after : rec->x_min) - xgm) / rc.dx);
  const float xs_hi = (float)(((after ? rec->x_max_after : rec->x_max) - xgm) / rc.dx);
  const float xlo = -0.5f, xhi = (float)rc.nx - 0.5f;
  int64_t dead = 0;
  for (int64_t i = (int64_t)bid * blockDim.x + threadIdx.x; i < n; i += (int64_t)nb * blockDim.x) {
    if (sp.kx[i] == INT32_MIN) continue;
    if (after && ((float)(sp.kx[i] - nsh) + sp.fx[i]) < xs_lo) {  // remove_particles (window.F90:304-325)
      sp.kx[i] = INT32_MIN;
      dead++;
      continue;
    }
    if (mixed_bc(sp, i, nsh, xlo, xhi, xs_lo, xs_hi, xs_lo - 2.0f, xs_hi + 2.0f, P.r_hi, P.r_sys, P.r_out,
                 rc.nx))
      dead++;
  }
  if (dead) atomicAdd((unsigned long long*)&cnt->n_dead, (unsigned long long)dead);
}
__global__ void k_mixed_bcs(SpeciesPtrs sp, SpeciesCounters* cnt, const StepRec* rec, int after, MixedParams P,
                            RunConst rc) {
  mixed_bcs_body(sp, cnt, rec, after, P, rc, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void mixed_append_body(const SpeciesPtrs& sp, SpeciesCounters* cnt, const double* inject,
                                                  const StepRec* rec, int isp, double xg0, const RunConst& rc,
                                                  int* err, int bid, int nb) {
  const int64_t off = rec->inject_off[isp], k = rec->inject_cnt[isp];
  const int64_t base = cnt->n_used;
  if (base + k > sp.cap) {
    if (bid == 0 && threadIdx.x == 0) atomicOr(err, ERR_CAPACITY);
    return;
  }
  unsigned wb = 0u;  // bits of the largest |FP32 weight| (positive floats order as integers)
  for (int64_t i = (int64_t)bid * blockDim.x + threadIdx.x; i < k; i += (int64_t)nb * blockDim.x) {
    const double* q = inject + (off + i) * 8;
    to_mixed(sp, base + i, q[0], q[1], q[2], q[3], q[4], q[5], q[6], xg0, rc);
    sp.id[base + i] = __double_as_longlong(q[7]);
    wb = max(wb, __float_as_uint(fabsf(sp.fw[base + i])));
  }
  wb = __reduce_max_sync(0xffffffffu, wb);
  if ((threadIdx.x & 31) == 0 && wb != 0u) atomicMax(&cnt->wmax_bits, wb);
}
__global__ void k_mixed_append(SpeciesPtrs sp, SpeciesCounters* cnt, const double* inject, const StepRec* rec,
                               int isp, double xg0, RunConst rc, int* err) {
  mixed_append_body(sp, cnt, inject, rec, isp, xg0, rc, err, blockIdx.x, gridDim.x);
}
__device__ __forceinline__ void mixed_append_commit_body(const SpeciesPtrs& sp, SpeciesCounters* cnt,
                                                         const StepRec* rec, int isp) {
  const int64_t k = rec->inject_cnt[isp];
  if (cnt->n_used + k <= sp.cap) cnt->n_used += k;
}
__global__ void k_mixed_append_commit(SpeciesPtrs sp, SpeciesCounters* cnt, const StepRec* rec, int isp) {
  mixed_append_commit_body(sp, cnt, rec, isp);
}

// The same three stages of the window for every (run, species) of a batch:
// blockIdx.y is the WindowJob.
__global__ void k_mixed_append_batch(const WindowJob* __restrict__ jobs) {
  const WindowJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  mixed_append_body(J.sp, J.cnt, J.inject, J.rec, J.isp, J.xg0, rc, J.err, blockIdx.x, gridDim.x);
}
__global__ void k_mixed_append_commit_batch(const WindowJob* __restrict__ jobs, int njobs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  const WindowJob& J = jobs[j];
  mixed_append_commit_body(J.sp, J.cnt, J.rec, J.isp);
}
__global__ void k_mixed_bcs_batch(const WindowJob* __restrict__ jobs) {
  const WindowJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  const MixedParams P = J.P;
  mixed_bcs_body(J.sp, J.cnt, J.rec, 1, P, rc, blockIdx.x, gridDim.x);
}

void batch_window_particles(cudaStream_t s, const WindowJob* jobs, int njobs, int nblocks) {
  if (njobs == 0) return;
  k_mixed_append_batch<<<dim3(64, njobs), 256, 0, s>>>(jobs);
  k_mixed_append_commit_batch<<<(njobs + 63) / 64, 64, 0, s>>>(jobs, njobs);
  k_mixed_bcs_batch<<<dim3(nblocks, njobs), 256, 0, s>>>(jobs);
}

void mixed_window_particles(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, const double* inject,
                            const StepRec* rec, int isp, double xg0, const RunConst& rc, int* err, int nblocks) {
  k_mixed_append<<<64, 256, 0, s>>>(sp, cnt, inject, rec, isp, xg0, rc, err);
  k_mixed_append_commit<<<1, 1, 0, s>>>(sp, cnt, rec, isp);
  k_mixed_bcs<<<nblocks, 256, 0, s>>>(sp, cnt, rec, 1, mixed_params(sp, rc), rc);
}

void mixed_particle_bcs(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, const StepRec* rec,
                        const RunConst& rc, int nblocks) {
  k_mixed_bcs<<<nblocks, 256, 0, s>>>(sp, cnt, rec, 0, mixed_params(sp, rc), rc);
}

__global__ void k_mixed_energy(SpeciesPtrs sp, const SpeciesCounters* cnt, double* out) {
  const int64_t n = cnt->n_used;
  const double mc2 = sp.mass * CLIGHT * CLIGHT;
  double e = 0.0, c = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (sp.kx[i] == INT32_MIN) continue;
    const double ux = sp.ux[i], uy = sp.uy[i], uz = sp.uz[i];
    const double u2 = ux * ux + uy * uy + uz * uz;
    e += (double)sp.fw[i] * mc2 * (u2 / (sqrt(u2 + 1.0) + 1.0));
    c += 1.0;
  }
  double v[2] = {e, c};
  block_sum_add<2>(v, out);
}
void mixed_energy(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, double* out, int nblocks) {
  k_mixed_energy<<<nblocks, 256, 0, s>>>(sp, cnt, out);
}

__global__ void k_mixed_cells(SpeciesPtrs sp, const SpeciesCounters* cnt, double xg0, double xgm, RunConst rc,
                              int32_t* cx, int32_t* cy, int32_t* live) {
  const int64_t n = cnt->n_used;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = sp.kx[i];
    if (k == INT32_MIN) {
      live[i] = 0;
      continue;
    }
    const double x = xg0 + ((double)k + (double)sp.fx[i]) * rc.dx;
    const double y = (double)sp.fy[i] * rc.dy, z = (double)sp.fz[i] * rc.dy;
    cx[i] = (int32_t)floor((x - xgm) / rc.dx + 1.5);
    cy[i] = (int32_t)floor((sqrt(y * y + z * z) - rc.y_grid_min) / rc.dy + 1.5);
    live[i] = 1;
  }
}
void mixed_cell_indices(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, double xg0,
                        double x_grid_min, const RunConst& rc, int32_t* cx, int32_t* cy, int32_t* live,
                        int nblocks) {
  k_mixed_cells<<<nblocks, 256, 0, s>>>(sp, cnt, xg0, x_grid_min, rc, cx, cy, live);
}

// --------------------------------------------------------- sort by tile

__device__ __forceinline__ int floordiv(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

__global__ void k_tile_layout(TileTable* tt, const StepRec* rec, RunConst rc, int64_t* start, int32_t* order,
                              int tile_x, int tile_y) {
  const int nsh = rec->nshift_total_after;
  tt->tile_x = tile_x;
  tt->tile_y = tile_y;
  tt->tx_min = floordiv(nsh, tile_x) - 1;
  tt->ntx = rc.nx / tile_x + 3;
  tt->nty = rc.ny / tile_y + 2;
  tt->ntiles = tt->ntx * tt->nty;
  tt->start = start;
  tt->order = order;
}

__global__ void k_tile_keys(SpeciesPtrs sp, const SpeciesCounters* cnt, const TileTable* tt, int32_t* keys,
                            int32_t* hist) {
  const int64_t n = cnt->n_used;
  const int ntiles = tt->ntiles, ntx = tt->ntx, nty = tt->nty, txm = tt->tx_min;
  const int tile_x = tt->tile_x, tile_y = tt->tile_y;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int key = ntiles;  // holes sort last and are dropped
    if (i < n) {
      const int32_t k = sp.kx[i];
      if (k != INT32_MIN) {
        int tx = floordiv(k, tile_x) - txm;
        const float y = sp.fy[i], z = sp.fz[i];
        int ky = (int)floorf(sqrtf(y * y + z * z) - 0.5f);
        int ty = ky < 0 ? 0 : ky / tile_y;
        tx = tx < 0 ? 0 : (tx >= ntx ? ntx - 1 : tx);
        ty = ty >= nty ? nty - 1 : ty;
        key = ty * ntx + tx;
      }
      keys[i] = key;
    }
    // warp-aggregated histogram increment
    const unsigned act = __ballot_sync(0xffffffffu, i < n);
    if (i < n) {
      const unsigned peers = __match_any_sync(act, key);
      const int leader = __ffs(peers) - 1;
      if ((threadIdx.x & 31) == leader) atomicAdd(&hist[key], __popc(peers));
    }
  }
}

__global__ void k_tile_starts(const int32_t* offs, int64_t* start, TileTable* tt, int ntiles_max) {
  const int nt = tt->ntiles;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= nt; t += gridDim.x * blockDim.x) start[t] = offs[t];
  if (blockIdx.x == 0 && threadIdx.x == 0) tt->n_sorted = offs[nt];
}

__global__ void k_tile_copy_out(SpeciesPtrs sp, const SpeciesCounters* cnt, double* tmp, int64_t* tmp_id,
                                int64_t cap) {
  const int64_t n = cnt->n_used;
  int32_t* tk = (int32_t*)tmp;
  float* tf = (float*)(tmp + cap / 2 + 1);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    tk[i] = sp.kx[i];
    tf[i] = sp.fx[i];
    tf[cap + i] = sp.fy[i];
    tf[2 * cap + i] = sp.fz[i];
    tf[3 * cap + i] = sp.ux[i];
    tf[4 * cap + i] = sp.uy[i];
    tf[5 * cap + i] = sp.uz[i];
    tf[6 * cap + i] = sp.fw[i];
    tmp_id[i] = sp.id[i];
  }
}

__global__ void k_tile_scatter(SpeciesPtrs sp, const SpeciesCounters* cnt, const double* tmp,
                               const int64_t* tmp_id, int64_t cap, const int32_t* keys, int32_t* offs,
                               const TileTable* tt) {
  const int64_t n = cnt->n_used;
  const int ntiles = tt->ntiles;
  const int32_t* tk = (const int32_t*)tmp;
  const float* tf = (const float*)(tmp + cap / 2 + 1);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const bool valid = i < n;
    const int key = valid ? keys[i] : ntiles;
    const unsigned act = __ballot_sync(0xffffffffu, valid && key < ntiles);
    if (!(valid && key < ntiles)) continue;
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&offs[key], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    const int64_t d = base + __popc(peers & ((1u << lane) - 1u));
    sp.kx[d] = tk[i];
    sp.fx[d] = tf[i];
    sp.fy[d] = tf[cap + i];
    sp.fz[d] = tf[2 * cap + i];
    sp.ux[d] = tf[3 * cap + i];
    sp.uy[d] = tf[4 * cap + i];
    sp.uz[d] = tf[5 * cap + i];
    sp.fw[d] = tf[6 * cap + i];
    sp.id[d] = tmp_id[i];
  }
}

// The push's tile schedule: tiles by decreasing particle count, bucketed by
// count / 8 (counts of 8 * (ORDER_BUCKETS - 1) and more share the top
// bucket).  One CTA: a histogram of the buckets, an exclusive scan from the
// top bucket down, and a scatter of the tile indices.  Every tile appears
// exactly once; the order inside a bucket follows the shared-memory atomics.
constexpr int ORDER_BUCKETS = 1024;
__global__ void __launch_bounds__(ORDER_BUCKETS) k_tile_order(const TileTable* tt, const int64_t* start,
                                                               int32_t* order) {
  __shared__ int hist[ORDER_BUCKETS];
  __shared__ int warp_tot[ORDER_BUCKETS / 32];
  const int nt = tt->ntiles;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  hist[tid] = 0;
  __syncthreads();
  auto bucket = [&](int t) {
    const int64_t c = (start[t + 1] - start[t]) >> 3;
    // descending: the fullest tiles get the lowest bucket index
    return ORDER_BUCKETS - 1 - (int)(c < ORDER_BUCKETS - 1 ? c : ORDER_BUCKETS - 1);
  };
  for (int t = tid; t < nt; t += ORDER_BUCKETS) atomicAdd(&hist[bucket(t)], 1);
  __syncthreads();
  // exclusive scan of hist over the 1024 buckets (thread = bucket)
  const int v = hist[tid];
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = warp_tot[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    warp_tot[lane] = s;  // inclusive sums of the warp totals
  }
  __syncthreads();
  hist[tid] = x - v + (w > 0 ? warp_tot[w - 1] : 0);  // first slot of this bucket
  __syncthreads();
  for (int t = tid; t < nt; t += ORDER_BUCKETS) order[atomicAdd(&hist[bucket(t)], 1)] = t;
}

__global__ void k_tile_commit(SpeciesCounters* cnt, const TileTable* tt) {
  cnt->n_used = tt->n_sorted;
  cnt->n_dead = 0;
}

void mixed_sort(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, SortScratch& sc, TileTable* tt,
                int64_t* tile_start, int32_t* tile_order, int tile_x, int tile_y, const StepRec* rec,
                const RunConst& rc, int nblocks) {
  const int ntiles_max = ntiles_max_of(rc.nx, rc.ny);
  k_tile_layout<<<1, 1, 0, s>>>(tt, rec, rc, tile_start, tile_order, tile_x, tile_y);
  cudaMemsetAsync(sc.hist, 0, sizeof(int32_t) * (ntiles_max + 1), s);
  k_tile_keys<<<nblocks, 256, 0, s>>>(sp, cnt, tt, sc.keys, sc.hist);
  scan_exclusive(s, sc.hist, ntiles_max + 1, (int32_t*)sc.perm);
  k_tile_starts<<<64, 256, 0, s>>>(sc.hist, tile_start, tt, ntiles_max);
  k_tile_copy_out<<<nblocks, 256, 0, s>>>(sp, cnt, sc.tmp, sc.tmp_id, sc.cap);
  k_tile_scatter<<<nblocks, 256, 0, s>>>(sp, cnt, sc.tmp, sc.tmp_id, sc.cap, sc.keys, sc.hist, tt);
  k_tile_order<<<1, ORDER_BUCKETS, 0, s>>>(tt, tile_start, tile_order);
  k_tile_commit<<<1, 1, 0, s>>>(cnt, tt);
}

// ------------------------------------------------- batched push

// The work table of a batched push: every non-empty tile of every job as a
// (job, tile) item, in decreasing order of particle count (the bucketing of
// k_tile_order, over all jobs).  One CTA.
__global__ void __launch_bounds__(ORDER_BUCKETS) k_batch_schedule(const BatchJob* jobs, int njobs, int2* work,
                                                                   int* nwork) {
  __shared__ int hist[ORDER_BUCKETS];
  __shared__ int warp_tot[ORDER_BUCKETS / 32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  hist[tid] = 0;
  __syncthreads();
  auto bucket = [&](const int64_t* start, int t) {
    const int64_t c = (start[t + 1] - start[t]) >> 3;
    return ORDER_BUCKETS - 1 - (int)(c < ORDER_BUCKETS - 1 ? c : ORDER_BUCKETS - 1);
  };
  for (int j = 0; j < njobs; ++j) {
    const TileTable* tt = jobs[j].tt;
    const int nt = tt->ntiles;
    const int64_t* start = tt->start;
    for (int t = tid; t < nt; t += ORDER_BUCKETS)
      if (start[t + 1] > start[t]) atomicAdd(&hist[bucket(start, t)], 1);
  }
  __syncthreads();
  const int v = hist[tid];
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = warp_tot[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    warp_tot[lane] = s;
  }
  __syncthreads();
  hist[tid] = x - v + (w > 0 ? warp_tot[w - 1] : 0);
  if (tid == ORDER_BUCKETS - 1) *nwork = x + (w > 0 ? warp_tot[w - 1] : 0);
  __syncthreads();
  for (int j = 0; j < njobs; ++j) {
    const TileTable* tt = jobs[j].tt;
    const int nt = tt->ntiles;
    const int64_t* start = tt->start;
    for (int t = tid; t < nt; t += ORDER_BUCKETS)
      if (start[t + 1] > start[t]) work[atomicAdd(&hist[bucket(start, t)], 1)] = make_int2(j, t);
  }
}

// Clear the deferred-list counters of a batch's jobs (one step's table).
__global__ void k_batch_reset(const BatchJob* jobs, int njobs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < njobs) *jobs[j].P.fb_count = 0;
}

void batch_schedule(cudaStream_t s, const BatchJob* jobs, int njobs, int2* work, int* nwork) {
  k_batch_schedule<<<1, ORDER_BUCKETS, 0, s>>>(jobs, njobs, work, nwork);
}
void batch_reset(cudaStream_t s, const BatchJob* jobs, int njobs) {
  k_batch_reset<<<(njobs + 127) / 128, 128, 0, s>>>(jobs, njobs);
}

// ------------------------------------------------- push tile shapes

PushMixedFns push_mixed_fns_16x8();
PushMixedFns push_mixed_fns_8x16();
PushMixedFns push_mixed_fns_8x8();
PushMixedFns push_mixed_fns_16x4();
PushMixedFns push_mixed_fns_8x4();

const PushMixedFns& push_mixed_fns(int shape) {
  static const PushMixedFns table[N_TILE_SHAPES] = {push_mixed_fns_16x8(), push_mixed_fns_8x16(),
                                                    push_mixed_fns_8x8(), push_mixed_fns_16x4(),
                                                    push_mixed_fns_8x4()};
  return table[shape < 0 || shape >= N_TILE_SHAPES ? 0 : shape];
}

}  // namespace cyl
