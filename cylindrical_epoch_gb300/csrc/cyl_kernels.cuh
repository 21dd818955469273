// cyl_kernels.cuh -- launch interface between the C ABI layer and the kernels.
#pragma once

#include "cyl_common.cuh"

namespace cyl {

// The mode arrays of one step: E, B and B_old in the form's storage type T
// (FP64 for the plain form, FP32 for the mixed form); J and J_old are FP64
// in both forms.
template <typename T>
struct FieldSetT {
  FViewT<T> ex, er, et, bx, br, bt;
  FView jx, jr, jt;
  FViewT<T> bxo, bro, bto;
  FView jxo, jro, jto;
};
using FieldSet = FieldSetT<cplx>;
using FieldSetF = FieldSetT<cplxf>;

// Scalars of the axis, laser and r_max kernels, rounded once on the host
// in the order the kernels used to evaluate them (no FMA contraction on
// either side, so the FP64 form's values are unchanged).
struct BcConst {
  double c4dy;                 // 4 c^2 / dy
  double inv_eps0, inv_dx, inv_dy, inv_9;
  double lx, lr, sum, diff, dt_eps;  // k_laser_x
  double rx_lx, rx_inv_r, rx_dtc2_4r, rx_ly, rx_sum_x, rx_sum_t, rx_dt_2eps, rx_lx_c;  // k_rmax_b
  cplx rx_icdt_2r;
};

// Coefficients of the first radial cell (ir = 1) of the mixed form's Yee
// updates in FP64, precomputed on the host so that the row needs no FP64
// division (h = dt/2, r_d, r_p of ir = 1):
// E: a = c^2/r_p h/2, bm = c^2/r_p h (times i m), c = c^2/dy h, cx = c^2/dx h,
//    d = h/eps0, erm = c^2/r_d h (times i m);
// B: p = h/r_d (times i m), q = h/(2 r_d), r = h/dy, s = h/r_p (times i m),
//    t = h/dx.
struct Row1E {
  double a, bm, c, cx, d, erm;
};
struct Row1B {
  double p, q, r, s, t;
};

// One run of a batch in one step, for the batched field and boundary stages
// (one launch per stage for every run of the batch, blockIdx.y = run): the
// field sets of the step's first half (F0, J of the step before) and of the
// push (F1, after the J swap), the step's record and laser sources, and the
// run's constants with the host-rounded coefficients of each stage.
struct StageJob {
  FieldSetF F0, F1;
  const StepRec* rec;
  const double* src;
  const cplx* cols;
  const float4* rowtab;
  RunConst rc;
  BcConst K;
  Row1E r1e;
  Row1B r1b;
  float cdx, cdy, cj, hdx, hdy;
};
// The host-rounded constants of a stage job from its rc (K in fields.cu,
// the Yee coefficients in fields_fp32.cu).
void stage_job_bc_consts(StageJob& J);
void stage_job_yee_consts(StageJob& J);
// Grid extents of a batch: the largest nx, ny of its runs (one M for all).
struct StageDims {
  int nx_max, ny_max, M;
};
// The mixed form's step stages for all runs of a batch (jobs: njobs
// consecutive StageJobs of one step).  use_f1 selects F1 over F0.
void batch_update_e_f32(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, const StageDims& d);
void batch_update_b_f32(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, int save_old,
                        const StageDims& d);
// k_e_axis and efield_bcs; k_b_axis and the halo of bfield_bcs (the
// update_eb_fields_half sequence); bc_mask_any: the OR of the runs' masks
void batch_e_axis_bcs(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, int bc_mask_any,
                      const StageDims& d);
void batch_b_axis_bcs(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, int bc_mask_any,
                      const StageDims& d);
// update_b_field's axis rules and bfield_final_bcs, on F1
void batch_b_final_bcs(cudaStream_t s, const StageJob* jobs, int njobs, int bc_mask_any, const StageDims& d);
// current_bcs_r_min_final on F1; J = 0 of F1 (the swap's zeroing)
void batch_j_rmin(cudaStream_t s, const StageJob* jobs, int njobs, const StageDims& d);
void batch_zero_j(cudaStream_t s, const StageJob* jobs, int njobs, const StageDims& d);
// current_finish's folding and halo pass of the runs that need it (reflecting
// or periodic boundaries: stage_finish_needed), on F1
void batch_current_finish(cudaStream_t s, const StageJob* jobs, int njobs);
bool stage_finish_needed(const RunConst& rc);
// shift_fields of a window shift (which = the shift's index in the step), on F1
void batch_shift_fields(cudaStream_t s, const StageJob* jobs, int njobs, int which, const StageDims& d);

// Geometry tables of push_particles (particles.F90:189-217), run constant.
struct GeomTables {
  const double* inv_area_rt;    // index iy - (1-jng)
  const double* inv_area_xt;    // index iy - (0-jng)
  const double* inv_volume;     // index iy - (1-jng)
  const double* ratio_area_xt;  // index iy - (1-jng)
};

// Per-species counters kept on the device.
struct SpeciesCounters {
  int64_t n_used;  // slots in use (live + removed holes)
  int64_t n_dead;  // removed particles still occupying a slot
  uint32_t wmax_bits;  // mixed form: FP32 bits of the largest weight uploaded or injected
  uint32_t pad;
};

// loader.cu: particle loading and window injection from the counter stream
// (counter_rng.cuh).  The density map is the (nx + 2ng) x (ny + 2ng) grid of
// setup_particle_density with row length W; valid lists the valid interior
// cells as (ix - 1) + nx (iy - 1), iy outer.
struct LoadParams {
  int nx, ny, W;
  double dx, dy, x_grid_min, y_grid_min;
  int64_t nppc, nvalid, n, id_base;
  uint64_t seed;
  int species;
  double temp[3], drift[3], mass;
};
struct LoadOut {
  double *x, *y, *z, *px, *py, *pz, *w;
  int64_t* id;
};
struct InjSpecies {  // per species: what insert_particles needs besides the column density
  int64_t nppc;
  double frac;
  double temp[3], drift[3], mass;
};
void launch_load_particles(cudaStream_t s, const LoadParams& P, const int32_t* valid, const double* dens,
                           const int8_t* dmap, int* npic, LoadOut o, uint32_t* wmax_bits);
void launch_inject_counter(cudaStream_t s, const StepRec* rec, const InjSpecies* isp, int nsp, const RunConst& rc,
                           uint64_t seed, int32_t* rowmap, double* inj);

// fields.cu (E/B boundary and axis kernels for either storage type)
void launch_update_e(cudaStream_t s, const FieldSet& F, const RunConst& rc);
void launch_update_b(cudaStream_t s, const FieldSet& F, int save_old, const RunConst& rc);
template <typename T>
int launch_e_axis_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc);
template <typename T>
int launch_efield_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc);
template <typename T>
int launch_old_field_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc);
template <typename T>
int launch_b_axis_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc);
template <typename T>
int launch_b_final_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const double* src,
                        const cplx* cols, int do_axis, double dt, const RunConst& rc);
template <typename T>
int launch_current_finish(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc,
                           int smooth, int its, int comp_its, int stride, FView wk, int parts = 7);
// The zeroing at the start of a step's push: J = 0 of the three current
// arrays (the J swap of update_eb_fields_half) and up to MAX_SPECIES int
// counters (the mixed push's deferred-particle counts), in one launch.
struct ZeroCounts {
  int* p[MAX_SPECIES];
  int n;
};
template <typename T>
void launch_zero_step(cudaStream_t s, const FieldSetT<T>& F, const RunConst& rc, const ZeroCounts& zc);
template <typename T>
void launch_shift_fields(cudaStream_t s, const FieldSetT<T>& F, const cplx* cols, const StepRec* rec,
                         int which, const RunConst& rc);

// fields_fp32.cu (bulk Yee updates of the mixed form, FP32 storage)
void launch_update_e_f32(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc);
// Two consecutive E half-steps (the closing half of a step, then the E
// boundary rules, then the opening half of the next step): the edge cells'
// first half with the axis row's rule, then (after the ghost phases) the
// edge cells' second half and both halves of every other cell, with the
// axis rules (fields_fp32.cu).  Each is followed by the ghost phases alone.
void launch_update_e_f32_edge_axis(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc);
void launch_update_e_f32_fused_axis(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc);
void launch_update_b_f32(cudaStream_t s, const FieldSetF& F, int save_old, const double* rowtab,
                         const RunConst& rc);
// The opening B half-step (B_old saved) together with launch_zero_step's
// zeroing of Fz's currents and the counts zc, in one launch.
void launch_update_b_f32_zero(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc,
                              const FieldSetF& Fz, const ZeroCounts& zc);

// push_fp64.cu
void launch_push_fp64(cudaStream_t s, const FieldSet& F, const GeomTables& g, const SpeciesPtrs& sp,
                      SpeciesCounters* cnt, const StepRec* rec, const RunConst& rc, int apply_bcs,
                      int* err, int nblocks);
void launch_eval_atan2(cudaStream_t s, const double* y, const double* x, double* out, int64_t n);

// ionise.cu: field ionisation of the FP64 form.  Per species the deck's data
// and the constants of initialise_ionisation (ionise.F90:51-286): n_exp is
// 2 n* - 1.5, k_photons_exponent 4 K - 2, fields in atomic units.
struct IonSpecies {
  int32_t ionise, ionise_to, release, l;
  double energy, released_mass_fraction, n_exp, adk_scaling, ionisation_constant, smallest_e_mag;
  double bsi_constant, bsi_scaling, bsi_threshold, adk_maximum, adk_bsi_cap;
  double keldysh, multi_constant, k_photons_energy, k_photons_exponent, adk_multiphoton_cap;
};
struct IonParams {
  IonSpecies s[MAX_SPECIES];
  int32_t model, nsp;
  uint64_t seed;
};
void ionisation_constants(const cyl_ionisation_species* io, const cyl_species_desc* sd, int n, int model,
                          double omega, IonSpecies* out);
void launch_ionise(cudaStream_t s, const FieldSet& F, const SpeciesPtrs* sp, int nsp, SpeciesCounters* cnt,
                   const IonParams& P, const StepRec* rec, const RunConst& rc, int64_t* snap, const int64_t* caps,
                   int* err, int nblocks);
// The mixed form's storage (xg0: its x origin); J stays FP64 in both forms.
void launch_ionise(cudaStream_t s, const FieldSetF& F, const SpeciesPtrs* sp, int nsp, SpeciesCounters* cnt,
                   const IonParams& P, const StepRec* rec, const RunConst& rc, int64_t* snap, const int64_t* caps,
                   int* err, int nblocks, double xg0);

// charge.cu (continuity-residual and number-density diagnostics)
void launch_number_density(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, const RunConst& rc,
                           double x_grid_min, int nsh, bool mixed, const FView& out, int nblocks);
void launch_number_density_bcs(cudaStream_t s, const FView& out, const RunConst& rc, const int* bc_field);
void launch_charge_density(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt,
                           const double* inv_volume, const RunConst& rc, double x_grid_min, int nsh,
                           bool mixed, const FView& rho, int nblocks);

// particles.cu
void launch_particle_bcs(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                         const StepRec* rec, int after_shift, const RunConst& rc, int nblocks);
void launch_window_particles(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                             const double* inject, const StepRec* rec, int isp, const RunConst& rc,
                             int* err, int nblocks);
void launch_cell_indices(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt,
                         double x_grid_min, const RunConst& rc, int32_t* cx, int32_t* cy,
                         int32_t* live, int nblocks);
void launch_energy(cudaStream_t s, const SpeciesPtrs& sp, const SpeciesCounters* cnt, double* out,
                   int nblocks);
template <typename T>
void launch_field_energy(cudaStream_t s, const FieldSetT<T>& F, const RunConst& rc, double* out);
// Counting sort of one species by cell; scratch holds the keys, histogram and
// a second copy of the particle arrays.  Removes dead slots.
struct SortScratch {
  int32_t* keys;
  int32_t* hist;     // ncells + 1
  int64_t* perm;
  double* tmp;       // 7 * cap doubles
  int64_t* tmp_id;
  int64_t cap;
  int ncells;
};
void sort_species(cudaStream_t s, const SpeciesPtrs& sp, SpeciesCounters* cnt, SortScratch& sc,
                  const double* x_grid_min, const RunConst& rc, int nblocks);

}  // namespace cyl
