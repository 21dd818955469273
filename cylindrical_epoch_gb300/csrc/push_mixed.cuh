// push_mixed.cuh -- mixed-precision form: tile table, push parameters and
// the particle kernels that know the mixed particle layout.
#pragma once

#include "cyl_common.cuh"
#include "cyl_kernels.cuh"

namespace cyl {

// Tile shapes (cells along x, cells along r) the mixed push is built for;
// push_mixed.cu is compiled once per shape.  Shape 0 is the default;
// cyl_tune_tiles picks another per run.
constexpr int N_TILE_SHAPES = CYL_N_TILE_SHAPES;
constexpr int TILE_SHAPES[N_TILE_SHAPES][2] = {{16, 8}, {8, 16}, {8, 8}, {16, 4}, {8, 4}};
constexpr int TILE_MIN_X = 8, TILE_MIN_Y = 4;  // the smallest extents: tile-table sizes
inline int ntiles_max_of(int nx, int ny) { return (nx / TILE_MIN_X + 3) * (ny / TILE_MIN_Y + 2); }

// Particles sorted by tile: tile t owns slots [start[t], start[t+1]);
// slots [n_sorted, n_used) were appended after the sort.  order[] lists the
// tiles by decreasing particle count (the push deals them to its CTAs
// round-robin in that order, a longest-first static schedule).
struct TileTable {
  int tile_x, tile_y;  // the tile shape of the last sort
  int ntiles;
  int ntx, nty;
  int tx_min;     // absolute tile column of tile 0
  int64_t n_sorted;
  int64_t* start;  // ntiles + 1
  int32_t* order;  // ntiles
};

struct MixedParams {
  float cdt2_dx, cdt2_dy;   // c dt / 2 in cells along x and r
  float cmratio, ccmratio;  // q dt fac / (2 m c) and c times it
  float q_fac, idt, c;
  // particle boundaries in cell units of the step's grid (set per launch)
  float x_lo, x_hi, x_sys_lo, x_sys_hi, x_out_lo, x_out_hi;
  float r_hi, r_sys, r_out;
  int* err;
  // FP32 copies of the geometric factors (rows 1-jng.., 0-jng.., 1-jng..)
  const float *g_rt, *g_xt, *g_vol;
  // particles deferred to the global-memory pass
  int* fb_list;
  int* fb_count;
  // first particle that raised the device error word: reason, index and
  // state (diagnostic record read by cyl_debug_record)
  float* dbg;
};

MixedParams mixed_params(const SpeciesPtrs& sp, const RunConst& rc);

// One run of a batched push (one entry per run and step of a chunk): the
// run's fields (J of the step's parity), particles, counters, step record,
// constants, push parameters and tile table.
struct BatchJob {
  FieldSetF F;
  SpeciesPtrs sp;
  SpeciesCounters* cnt;
  const StepRec* rec;
  RunConst rc;
  MixedParams P;
  TileTable* tt;
  int apply_bcs;
};

// The push of one tile shape (push_mixed.cu built for that shape):
// shared memory per CTA, resident CTAs per SM (also sets the kernel's
// shared-memory attributes; call before the first launch), and the launch
// of the tile kernel and the global-path kernel.
struct PushMixedFns {
  size_t (*smem)(int M);
  int (*blocks_per_sm)(int M);
  // (count_zeroed: the deferred-particle count P.fb_count is already 0)
  void (*launch)(cudaStream_t s, const FieldSetF& F, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                 const StepRec* rec, const RunConst& rc, int apply_bcs, int nblocks_tiles, int nblocks_global,
                 const MixedParams& P, TileTable* tt, int count_zeroed);
  // the batched push: jobs[0, njobs) of one step, work = (job, tile) items
  void (*launch_batch)(cudaStream_t s, int M, const BatchJob* jobs, int njobs, const int2* work, const int* nwork,
                       int nblocks_tiles, int nblocks_global);
};
const PushMixedFns& push_mixed_fns(int shape);

// mixed_particles.cu: the (job, tile) work table of a batched push, and the
// per-step reset of the jobs' deferred-list counters.
void batch_schedule(cudaStream_t s, const BatchJob* jobs, int njobs, int2* work, int* nwork);
void batch_reset(cudaStream_t s, const BatchJob* jobs, int njobs);

// mixed_particles.cu
void mixed_from_double(cudaStream_t s, const SpeciesPtrs& sp, const double* stage, int64_t n, int64_t cap,
                       double xg0, const RunConst& rc);
void mixed_to_double(cudaStream_t s, const SpeciesPtrs& sp, double* stage, int64_t n, int64_t cap,
                     double xg0, const RunConst& rc);
// Reciprocals of the mixed form's units (the cell sizes, m c of the
// species), computed once by a thread and used by all its conversions.
struct MixedScale {
  double idx, idy, imc;
};
__device__ __forceinline__ MixedScale mixed_scale(const SpeciesPtrs& sp, const RunConst& rc) {
  return MixedScale{1.0 / rc.dx, 1.0 / rc.dy, 1.0 / (sp.mass * CLIGHT)};
}

// One particle from FP64 state into the mixed form's storage at slot d
// (integer cell + FP32 offset of x from xg0, y and z in units of dy,
// normalised momenta, FP32 weight; a NaN x marks a hole).  Products with
// the reciprocals instead of divisions: the FP64 pipe is narrow, and every
// result but the cell index is rounded to FP32 at once.
__device__ __forceinline__ void to_mixed(const SpeciesPtrs& sp, int64_t d, double x, double y, double z,
                                         double px, double py, double pz, double w, double xg0,
                                         const MixedScale& k) {
  if (isnan(x)) {
    sp.kx[d] = INT32_MIN;
    return;
  }
  const double xi = (x - xg0) * k.idx;
  double kf = floor(xi);
  float f = (float)(xi - kf);
  if (f >= 1.0f) {
    f = 0.0f;
    kf += 1.0;
  }
  sp.kx[d] = (int32_t)kf;
  sp.fx[d] = f;
  sp.fy[d] = (float)(y * k.idy);
  sp.fz[d] = (float)(z * k.idy);
  sp.ux[d] = (float)(px * k.imc);
  sp.uy[d] = (float)(py * k.imc);
  sp.uz[d] = (float)(pz * k.imc);
  sp.fw[d] = (float)w;
}
__device__ __forceinline__ void to_mixed(const SpeciesPtrs& sp, int64_t d, double x, double y, double z,
                                         double px, double py, double pz, double w, double xg0,
                                         const RunConst& rc) {
  to_mixed(sp, d, x, y, z, px, py, pz, w, xg0, mixed_scale(sp, rc));
}

// One (run, species) of a batch in one step, for the window's particle
// stages (append the step's injected particles, commit, particle_bcs after
// the shift and remove_particles) of every member in one launch each.
struct WindowJob {
  SpeciesPtrs sp;
  SpeciesCounters* cnt;
  const double* inject;
  const StepRec* rec;
  MixedParams P;
  RunConst rc;
  double xg0;
  int isp;
  int* err;
};
void batch_window_particles(cudaStream_t s, const WindowJob* jobs, int njobs, int nblocks);
void widen_f32(cudaStream_t s, const float* src, double* dst, int64_t n);
void upload_stats(cudaStream_t s, const double* w, const int64_t* id, int64_t n, SpeciesCounters* cnt,
                  long long* max_id);
void mixed_window_particles(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, const double* inject,
                            const StepRec* rec, int isp, double xg0, const RunConst& rc, int* err, int nblocks);
void mixed_particle_bcs(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, const StepRec* rec,
                        const RunConst& rc, int nblocks);
void mixed_energy(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, double* out, int nblocks);
void mixed_sort(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, SortScratch& sc, TileTable* tt,
                int64_t* tile_start, int32_t* tile_order, int tile_x, int tile_y, const StepRec* rec,
                const RunConst& rc, int nblocks);
void mixed_cell_indices(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, double xg0,
                        double x_grid_min, const RunConst& rc, int32_t* cx, int32_t* cy, int32_t* live,
                        int nblocks);

}  // namespace cyl
