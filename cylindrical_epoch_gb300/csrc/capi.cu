// capi.cu -- the C ABI of include/cylpic.h: run handle, host-side scalar
// bookkeeping and the per-step kernel sequence.
//
// The Fortran module scalars that the hot path reads (time, grid position of
// the moving window, field boundary codes, laser phases) are advanced on the
// host in the reference's order and shipped to the GPU as one StepRec per
// step, together with the laser source vectors and the particles the window
// injects.  All array state (fields, currents, particles) stays resident in
// HBM.  Steps are enqueued in chunks; a chunk of CHUNK steps can be captured
// once into a CUDA graph and replayed.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "cyl_common.cuh"
#include "counter_rng.cuh"
#include "cyl_kernels.cuh"
#include "host_pool.h"
#include "host_deck.h"
#include "push_mixed.cuh"

namespace cyl {

constexpr int CHUNK = 16;

#define CK(call)                                  \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) {                      \
      h->last_cuda_error = e_;                    \
      return CYL_ERR_CUDA;                        \
    }                                             \
  } while (0)

struct HostLaser {
  cyl_laser_desc d;
  std::vector<double> profile, phase;
  double current_integral_phase = 0.0;
};


// Where a handle stands (Handle::at_output): between full steps, at the
// output point inside a step, or loaded from a restart dump taken there.
enum { AT_OUTPUT_NONE = 0, AT_OUTPUT_STEP = 1, AT_OUTPUT_RESTART = 2 };

struct Handle {
  uint64_t serial = 0;  // unique per handle in the process (never reused, unlike the address)
  uint64_t topo_epoch = 0;  // bumped when the kernels of a step change (captured graphs are stale)
  int device = 0;
  cudaStream_t st = nullptr;
  cudaError_t last_cuda_error = cudaSuccess;
  cyl_grid_desc gd;
  HostGrid g;
  RunConst rc;
  int prec = CYL_PREC_FP64;
  size_t fcount = 0;  // complex elements per mode array
  cplx* fbuf = nullptr;
  cplx* F[16] = {};   // 15 arrays + smoothing work array
  cplxf* ffbuf = nullptr;  // mixed form: E, B, B_old in FP32
  cplxf* Ff[9] = {};
  float4* rowtab = nullptr;   // per-row FP32 Yee coefficients of the mixed form
  float* gtab_f = nullptr;    // FP32 geometric factors of the mixed deposit
  int* fb_buf = nullptr;      // mixed form: deferred-particle lists + counters
  float* d_dbg = nullptr;     // diagnostic record of the first flagged particle
  int jpar = 0;       // 0: J in slots 6..8, J_old in 12..14; 1: swapped
  cplx* cols = nullptr;
  double* geom_buf = nullptr;
  GeomTables geom;
  int nsp = 0;
  cyl_species_desc sd[MAX_SPECIES];
  SpeciesPtrs sp[MAX_SPECIES];
  SpeciesCounters* d_cnt = nullptr;
  SortScratch sc;
  double* sort_buf = nullptr;
  int64_t next_id = 0;
  // window injection: 0 = the host KISS stream (reference order), 1 = the
  // device counter stream keyed by inj_seed (cyl_set_injection_stream)
  int inj_counter = 0;
  uint64_t inj_seed = 0;
  InjSpecies* d_injsp = nullptr;
  int32_t* d_injrow = nullptr;  // (shift, species, row) of every injection slot (inj_cap)
  // diagnostics read without a stream sync: a ring of two pinned slots, each
  // the 8 reductions plus the device error word, with an event
  struct DiagSlot {
    double* h = nullptr;  // pinned: 8 doubles, then the error word
    cudaEvent_t ev = nullptr;
    bool pending = false;
  } diag_slot[2];
  int diag_head = 0, diag_count = 0;  // oldest pending slot, slots pending
  // host bookkeeping (module globals)
  double time = 0.0;
  int64_t step = 0;
  int bc_deck[4], bc_field[4], add_laser[4], bc_after_move[4];
  int bc_allspecies[4];
  bool move_window = false, window_started = false;
  double window_v_x = 0, window_start_time = 0, window_stop_time = 0, wsf = 0;
  int64_t n_shifts = 0;
  // Output point (cyl_step_to_output, cyl_restart_sdf): AT_OUTPUT_STEP after
  // the first part of a step (through current_finish), AT_OUTPUT_RESTART after
  // a restart dump was loaded; out_rec holds that step's record so far.  The
  // next stepping call finishes the step first.
  int at_output = 0;
  StepRec out_rec;
  // ic_from_restart: a window that starts keeps the restored shift fraction
  // (window.F90:347)
  bool from_restart = false;
  bool restart_wsf = false;  // the loaded dump held window_shift_fraction
  std::vector<HostLaser> lasers;
  // deck-expression callbacks (cyl_set_deck_fns); cb_failed is raised by a
  // callback's error while a step is prepared and read by its caller
  cyl_deck_fns fns{};
  bool cb_failed = false;
  // field ionisation (cyl_set_ionisation): constants, device snapshot of the
  // species' counts at the routine's start, capacities
  IonParams ion{};
  bool ion_on = false;
  int64_t* d_ion = nullptr;  // [0, MAX_SPECIES) snapshot, [MAX_SPECIES, 2 MAX_SPECIES) capacities
  KissRng rng;
  // staging
  StepRec* h_rec = nullptr;
  StepRec* d_rec = nullptr;
  double* h_src = nullptr;
  double* d_src = nullptr;
  double* h_inj = nullptr;
  double* d_inj = nullptr;
  int64_t inj_cap = 0;  // particles per chunk
  size_t src_per_step = 0;
  cudaEvent_t ev_copy = nullptr;
  bool copy_pending = false;
  int* d_err = nullptr;
  double* d_red = nullptr;
  // graph
  cudaGraphExec_t gexec = nullptr;
  int graph_parity = -1;
  bool graph_window = true;  // the captured chunk has the window's kernels
  bool merge_e = true;       // mixed form: merged E half-steps inside a chunk (cyl_set_merge_e_halves)
  // timing of the push kernel (events around each push in eager mode and in graphs)
  cudaEvent_t ev_push[CHUNK][2];
  int push_events_used = 0;
  double push_ms_sum = 0.0;
  int64_t push_launches = 0;
  int timing_pending = 0;  // steps of the last chunk whose push events are not yet read
  int nblocks = 152 * 8;
  int nblocks_mixed = 152 * 4;               // push CTAs of the current tile shape
  int tile_shape = 0;                         // index into TILE_SHAPES (mixed form)
  int nblocks_by_shape[N_TILE_SHAPES] = {};   // resident push CTAs per shape
  double xg0 = 0.0;  // x_grid_min at creation: origin of the mixed form's cell index
  MixedParams mp[MAX_SPECIES];
  TileTable* d_tiles = nullptr;     // one per species
  int64_t* d_tile_start = nullptr;  // (ntiles_max + 1) per species
  int32_t* d_tile_order = nullptr;  // ntiles_max per species (push schedule)
  int ntiles_max = 0;
  int64_t kernel_launches = 0;
  int64_t graph_launches = 0;
};

static int map_field_bc(int b) {
  // boundary.F90:30-75
  if (b == CYL_BC_OTHER) b = CYL_BC_CLAMP;
  if (b == CYL_BC_REFLECT) b = CYL_BC_CLAMP;
  if (b == CYL_BC_OPEN) b = CYL_BC_SIMPLE_OUTFLOW;
  return b;
}

static void setup_boundaries(Handle* h) {
  for (int i = 0; i < 4; ++i) {
    h->add_laser[i] = h->bc_deck[i] == CYL_BC_SIMPLE_LASER;
    h->bc_field[i] = map_field_bc(h->bc_deck[i]);
  }
}

// Field bc kinds a run can meet: the deck's bcs and, with a moving window,
// the bcs after it starts.
static int bc_mask_of(const int* deck, const int* after, bool window) {
  int mask = 0;
  for (int pass = 0; pass < (window ? 2 : 1); ++pass) {
    for (int i = 0; i < 4; ++i) {
      if (i == CYL_BD_Y_MIN) continue;
      const int b = map_field_bc(pass == 0 ? deck[i] : after[i]);
      if (b == CYL_BC_PERIODIC && i != CYL_BD_Y_MAX) mask |= BCM_PERIODIC_X;
      if (b == CYL_BC_CONDUCT) mask |= BCM_CONDUCT;
      if (b == CYL_BC_CLAMP || b == CYL_BC_SIMPLE_LASER || b == CYL_BC_SIMPLE_OUTFLOW ||
          b == CYL_BC_ZERO_GRADIENT)
        mask |= BCM_OTHER;
    }
  }
  return mask;
}

static int map_particle_bc(int b) {
  // setup_particle_boundary (boundary.F90:100-140)
  if (b == CYL_BC_OTHER || b == CYL_BC_CONDUCT) b = CYL_BC_REFLECT;
  if (b == CYL_BC_SIMPLE_LASER || b == CYL_BC_SIMPLE_OUTFLOW) b = CYL_BC_OPEN;
  return b;
}

template <typename T>
static FieldSetT<T> fieldset_t(const Handle* h, int jpar);

static FieldSet fieldset(const Handle* h, int jpar) {
  auto v = [&](int k) { return FView{h->F[k], h->rc.nxg, h->rc.nyg}; };
  FieldSet F;
  F.ex = v(0); F.er = v(1); F.et = v(2);
  F.bx = v(3); F.br = v(4); F.bt = v(5);
  F.bxo = v(9); F.bro = v(10); F.bto = v(11);
  const int j0 = jpar ? 12 : 6, jo = jpar ? 6 : 12;
  F.jx = v(j0); F.jr = v(j0 + 1); F.jt = v(j0 + 2);
  F.jxo = v(jo); F.jro = v(jo + 1); F.jto = v(jo + 2);
  return F;
}

// Mixed form: E, B and B_old live in the FP32 buffer, J and J_old in the
// FP64 one (same parity rule).
static FieldSetF fieldset_f(const Handle* h, int jpar) {
  auto v = [&](int k) { return FViewF{h->Ff[k], h->rc.nxg, h->rc.nyg}; };
  auto d = [&](int k) { return FView{h->F[k], h->rc.nxg, h->rc.nyg}; };
  FieldSetF F;
  F.ex = v(0); F.er = v(1); F.et = v(2);
  F.bx = v(3); F.br = v(4); F.bt = v(5);
  F.bxo = v(6); F.bro = v(7); F.bto = v(8);
  const int j0 = jpar ? 12 : 6, jo = jpar ? 6 : 12;
  F.jx = d(j0); F.jr = d(j0 + 1); F.jt = d(j0 + 2);
  F.jxo = d(jo); F.jro = d(jo + 1); F.jto = d(jo + 2);
  return F;
}
template <>
FieldSet fieldset_t<cplx>(const Handle* h, int jpar) { return fieldset(h, jpar); }
template <>
FieldSetF fieldset_t<cplxf>(const Handle* h, int jpar) { return fieldset_f(h, jpar); }

// Slot of a public field index under the current J parity.
static int field_slot(const Handle* h, int which) {
  if (h->jpar && which >= 6 && which <= 8) return which + 6;
  if (h->jpar && which >= 12 && which <= 14) return which - 6;
  return which;
}

// update_laser_omegas (laser.f90:276-328) at the handle's current time, dt_eff
// the step's dt (dt/2 at the start-up half step): a deck-function omega is
// evaluated and its phase integrated, the others' phase is omega * time.
static void update_laser_omegas(Handle* h, double dt_eff) {
  for (size_t i = 0; i < h->lasers.size(); ++i) {
    HostLaser& L = h->lasers[i];
    if (h->fns.laser_omega && ((h->fns.omega_fn_mask >> i) & 1u)) {
      double om = L.d.omega;
      if (h->fns.laser_omega(h->fns.user, (int32_t)i, h->time, &om) != 0) h->cb_failed = true;
      L.d.omega = om;
      L.current_integral_phase = L.current_integral_phase + om * dt_eff;
    } else {
      L.current_integral_phase = L.d.omega * h->time;
    }
  }
}

// Laser sources at the handle's current time (laser.f90:444-461), after
// update_laser_omegas: out[side*2*(ny+1) + {0, ny+1} + ir] = source1, source2.
// A laser whose phase or profile is a function of time has it re-evaluated
// first (laser.f90:449-450), then its time profile.
static void laser_sources(Handle* h, double* out, double dt_eff) {
  const int ny = h->g.ny;
  std::memset(out, 0, sizeof(double) * 4 * (ny + 1));
  update_laser_omegas(h, dt_eff);
  for (int side = 0; side < 2; ++side) {
    const int bd = side == 0 ? CYL_BD_X_MIN : CYL_BD_X_MAX;
    if (!h->add_laser[bd]) continue;
    double* s1 = out + side * 2 * (ny + 1);
    double* s2 = s1 + (ny + 1);
    for (size_t i = 0; i < h->lasers.size(); ++i) {
      HostLaser& L = h->lasers[i];
      if (L.d.boundary != bd) continue;
      if (h->time >= L.d.t_start && h->time <= L.d.t_end) {
        const cyl_deck_fns& f = h->fns;
        if (f.laser_phase && ((f.phase_fn_mask >> i) & 1u) &&
            f.laser_phase(f.user, (int32_t)i, h->time, L.phase.data()) != 0)
          h->cb_failed = true;
        if (f.laser_profile && ((f.profile_fn_mask >> i) & 1u) &&
            f.laser_profile(f.user, (int32_t)i, h->time, L.profile.data()) != 0)
          h->cb_failed = true;
        double tp = 1.0;
        if (f.laser_time) {
          if (f.laser_time(f.user, (int32_t)i, h->time, &tp) != 0) h->cb_failed = true;
        } else if (L.d.t_profile == 1) {
          const double v = (h->time - L.d.t0) / L.d.tw;
          tp = std::exp(-(v * v));
        }
        const double t_env = tp * L.d.amp;
        for (int ir = 0; ir <= ny; ++ir) {
          const double base = t_env * L.profile[ir] * std::sin(L.current_integral_phase + L.phase[ir]);
          s1[ir] = s1[ir] + base * std::cos(L.d.pol_angle);
          s2[ir] = s2[ir] + base * std::sin(L.d.pol_angle);
        }
      }
    }
  }
}

// insert_particles' columns of species s from the caller's callback (or
// none: the descriptor's closed forms), at the grid before the shift.
static const InjectColumns* inject_columns(Handle* h, int s, InjectColumns& cols) {
  if (!h->fns.inject) return nullptr;
  const int ny = h->g.ny;
  cols.density.assign((size_t)ny + 2, 0.0);
  cols.temperature.assign(3 * ((size_t)ny + 2), 0.0);
  cols.drift.assign(3 * ((size_t)ny + 2), 0.0);
  if (h->fns.inject(h->fns.user, s, h->time, h->g.xg(h->g.nx), cols.density.data(), cols.temperature.data(),
                    cols.drift.data()) != 0)
    h->cb_failed = true;
  return &cols;
}

static void fill_grid(StepRec& r, const HostGrid& g, bool after) {
  if (!after) {
    r.x_grid_min = g.x_grid_min;
    r.x_min = g.x_min;
    r.x_max = g.x_max;
    r.x_min_local = g.x_min_local;
    r.x_max_local = g.x_max_local;
  } else {
    r.x_grid_min_after = g.x_grid_min;
    r.x_min_after = g.x_min;
    r.x_max_after = g.x_max;
    r.x_min_local_after = g.x_min_local;
    r.x_max_local_after = g.x_max_local;
  }
}

// Advance the host scalars through one driver-loop iteration and describe it
// (epoch2d.F90:213-265 with moving_window, window.F90:330-376).
// The window shifts of one step with the injection drawn on the device
// (k_inject_counter): per shift the column's left edge x_grid_max + dx/2
// and global shift index, per species the clamped column density
// (insert_particles evaluates the profile at pack_ix = nx) and the count --
// floor(ppc) per row plus the rows' fraction bits, recomputed here from the
// same counter stream -- then the grid shift.  Ids are handed out shift by
// shift, species by species, and the batch holds each species' particles
// together, as in the host path.  At most MAX_INJ_SHIFTS shifts per step
// (cyl_set_injection_stream checks the deck allows no more).
static void inject_counter_step(Handle* h, StepRec& r, int cells, int64_t& inj_used) {
  r.inj_counter = 1;
  r.inj_nshift = cells;
  int64_t cnt[MAX_INJ_SHIFTS][MAX_SPECIES] = {};
  for (int c = 0; c < cells && c < MAX_INJ_SHIFTS; ++c) {
    r.inj_x0[c] = h->g.x_grid_max + 0.5 * h->g.dx;
    r.inj_shift[c] = h->n_shifts;
    for (int s = 0; s < h->nsp; ++s) {
      const cyl_species_desc& d = h->sd[s];
      double dens = species_density(d, h->g.xg(h->g.nx));
      if (dens > d.density_max) dens = d.density_max;
      if (dens < d.density_min) dens = 0.0;
      int64_t n = 0;
      if (!d.immobile && dens >= d.density_min) {
        const int64_t nppc = (int64_t)std::floor(d.npart_per_cell);
        const double frac = d.npart_per_cell - (double)nppc;
        for (int iy = 1; iy <= h->g.ny; ++iy) {
          n += nppc;
          if (frac > 0.0 &&
              u01(philox4x32_10((uint32_t)iy, (uint32_t)h->n_shifts, (uint32_t)s, TAG_INJ_COUNT, h->inj_seed)
                      .v[0]) < frac)
            n += 1;
        }
      }
      r.inj_dens[c][s] = dens;
      r.inj_id0[c][s] = h->next_id;
      r.inj_n[c][s] = n;
      cnt[c][s] = n;
      h->next_id += n;
    }
    h->g.x_grid_min = h->g.xg(1) + h->g.dx;
    h->g.xb_min = h->g.xb_min + h->g.dx;
    h->g.x_min = h->g.xb_min + h->g.dx * 0.0;
    h->g.x_max = (h->g.xb_min + (double)(h->g.nx + 1 - 1) * h->g.dx) - h->g.dx * 0.0;
    h->g.setup_grid_x();
    h->n_shifts++;
  }
  for (int s = 0; s < h->nsp; ++s) {
    r.inject_off[s] = inj_used;
    for (int c = 0; c < cells && c < MAX_INJ_SHIFTS; ++c) {
      r.inj_base[c][s] = inj_used;
      inj_used += cnt[c][s];
    }
    r.inject_cnt[s] = inj_used - r.inject_off[s];
  }
}

// The record fields of a step that its first part (update_eb_fields_half,
// the push, current_finish) reads: the grid and boundaries before the step's
// window shift.
static void step_head_fields(Handle* h, StepRec& r) {
  std::memset(&r, 0, sizeof(r));
  r.time_half = h->time;
  r.step = h->step;
  r.nshift_total = (int32_t)h->n_shifts;
  fill_grid(r, h->g, false);
  for (int i = 0; i < 4; ++i) {
    r.bc_field[i] = h->bc_field[i];
    r.add_laser[i] = h->add_laser[i];
  }
}

// A step up to the reference's output point (epoch2d.F90:259-262): the
// record's first part, step = step + 1, time = time + dt/2.
static void step_head(Handle* h, StepRec& r) {
  step_head_fields(h, r);
  h->step++;
  h->time = h->time + h->g.dt / 2.0;
}

static void step_tail(Handle* h, int k, int64_t& inj_used);

static void prepare_step(Handle* h, int k, int64_t& inj_used) {
  step_head(h, h->h_rec[k]);
  step_tail(h, k, inj_used);
}

// The rest of a step from the output point: time = time + dt/2
// (epoch2d.F90:263), the laser sources of update_eb_fields_final and
// moving_window's host part (window.F90:330-376).
static void step_tail(Handle* h, int k, int64_t& inj_used) {
  StepRec& r = h->h_rec[k];
  h->time = h->time + h->g.dt / 2.0;
  r.time_final = h->time;
  r.src_off = (int64_t)k * (int64_t)h->src_per_step;
  laser_sources(h, h->h_src + r.src_off, h->g.dt);
  for (int s = 0; s < h->nsp; ++s) {
    r.inject_off[s] = inj_used;
    r.inject_cnt[s] = 0;
  }
  int nshift = 0;
  if (h->move_window) {
    if (!h->window_started) {
      if (h->time >= h->window_start_time && h->time < h->window_stop_time) {
        for (int i = 0; i < 4; ++i) h->bc_deck[i] = h->bc_after_move[i];
        setup_boundaries(h);
        if (!h->from_restart) h->wsf = 0.0;
        h->window_started = true;
      }
    }
    if (h->window_started && !(h->time >= h->window_stop_time) && h->window_v_x > 0.0) {
      h->wsf = h->wsf + h->g.dt * h->window_v_x / h->g.dx;
      const int cells = (int)std::floor(h->wsf);
      if (cells > 0 && h->inj_counter) {
        inject_counter_step(h, r, cells, inj_used);
        nshift = cells;
        h->wsf = h->wsf - (double)cells;
      } else if (cells > 0) {
        std::vector<HostParticle> batch;
        // one buffer region per species: inject all species for every shift
        std::vector<std::vector<HostParticle>> per(h->nsp);
        InjectColumns cols;
        for (int c = 0; c < cells; ++c) {
          for (int s = 0; s < h->nsp; ++s)
            host_insert_particles(h->g, h->sd[s], h->rng, h->next_id, per[s], inject_columns(h, s, cols));
          h->g.x_grid_min = h->g.xg(1) + h->g.dx;
          h->g.xb_min = h->g.xb_min + h->g.dx;
          h->g.x_min = h->g.xb_min + h->g.dx * 0.0;
          h->g.x_max = (h->g.xb_min + (double)(h->g.nx + 1 - 1) * h->g.dx) - h->g.dx * 0.0;
          h->g.setup_grid_x();
          h->n_shifts++;
          nshift++;
        }
        for (int s = 0; s < h->nsp; ++s) {
          r.inject_off[s] = inj_used;
          r.inject_cnt[s] = (int64_t)per[s].size();
          for (auto& p : per[s]) {
            double* q = h->h_inj + inj_used * 8;
            for (int t = 0; t < 7; ++t) q[t] = p.v[t];
            std::memcpy(&q[7], &p.id, 8);
            inj_used++;
          }
        }
        h->wsf = h->wsf - (double)cells;
      }
    }
  }
  r.nshift = nshift;
  r.nshift_total_after = (int32_t)h->n_shifts;
  for (int i = 0; i < 4; ++i) r.bc_field_after[i] = h->bc_field[i];
  fill_grid(r, h->g, true);
}

static void count_launch(Handle* h, int n) { h->kernel_launches += n; }


// Enqueue the kernels of one step; rec/src point at this step's records.
// Bulk Yee updates: exact FP64 kernels for the plain form, FP32 for the mixed form.
static void bulk_e(Handle* h, cudaStream_t s, const FieldSet& F) { launch_update_e(s, F, h->rc); }
static void bulk_e(Handle* h, cudaStream_t s, const FieldSetF& F) {
  launch_update_e_f32(s, F, (const double*)h->rowtab, h->rc);
}
// An E half-step and the E boundary rules after it (the axis rules and
// efield_bcs).  At a step boundary inside a chunk (mixed form), `half` 1 is
// the closing half of a step (its edge cells alone), 2 the opening half of
// the next (see launch_update_e_f32_edge_axis / _fused_axis, which apply the
// axis rules themselves); 0 is a plain half-step.  Returns the launches.
template <typename T>
static int e_half_and_bcs(Handle* h, cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, int half) {
  if constexpr (std::is_same<T, cplxf>::value) {
    if (half == 1) {
      launch_update_e_f32_edge_axis(s, F, (const double*)h->rowtab, h->rc);
      return 1 + launch_efield_bcs(s, F, rec, h->rc);
    }
    if (half == 2) {
      launch_update_e_f32_fused_axis(s, F, (const double*)h->rowtab, h->rc);
      return 1 + launch_efield_bcs(s, F, rec, h->rc);
    }
  }
  bulk_e(h, s, F);
  return 1 + launch_e_axis_bcs(s, F, rec, h->rc);
}
static void bulk_b(Handle* h, cudaStream_t s, const FieldSet& F, int save_old) {
  launch_update_b(s, F, save_old, h->rc);
}
static void bulk_b(Handle* h, cudaStream_t s, const FieldSetF& F, int save_old) {
  launch_update_b_f32(s, F, save_old, (const double*)h->rowtab, h->rc);
}
static void push_all(Handle* h, cudaStream_t s, const FieldSet& F, const StepRec* rec, int apply_bcs,
                     int = 0) {
  for (int i = 0; i < h->nsp; ++i) {
    if (h->sp[i].immobile) continue;
    launch_push_fp64(s, F, h->geom, h->sp[i], h->d_cnt + i, rec, h->rc, apply_bcs, h->d_err, h->nblocks);
    count_launch(h, 1);
  }
}
// count_zeroed: the step's zeroing launch already cleared the deferred counts
static void push_all(Handle* h, cudaStream_t s, const FieldSetF& F, const StepRec* rec, int apply_bcs,
                     int count_zeroed = 0) {
  for (int i = 0; i < h->nsp; ++i) {
    if (h->sp[i].immobile) continue;
    push_mixed_fns(h->tile_shape)
        .launch(s, F, h->sp[i], h->d_cnt + i, rec, h->rc, apply_bcs, h->nblocks_mixed, h->nblocks / 4, h->mp[i],
                h->d_tiles + i, count_zeroed);
    count_launch(h, 2);
  }
}

// The kernels of one step before the push: update_eb_fields_half
// (fields.f90:316-337), then J_old = J, J = 0 (particles.F90:163-169) by
// buffer swap.  Returns the field set of the push.
template <typename T>
static FieldSetT<T> enqueue_step_pre(Handle* h, cudaStream_t s, const StepRec* rec, bool fused_in = false) {
  const RunConst& rc = h->rc;
  FieldSetT<T> F = fieldset_t<T>(h, h->jpar);
  int n = e_half_and_bcs<T>(h, s, F, rec, fused_in ? 2 : 0);
  // J = 0 of the field set after the swap (its J held the step before's
  // J_old, which nothing reads any more), and the mixed push's deferred
  // counts: in the mixed form inside the B half-step's launch, else in one
  // launch of their own
  const FieldSetT<T> Fn = fieldset_t<T>(h, h->jpar ^ 1);
  ZeroCounts zc{};
  if constexpr (std::is_same<T, cplxf>::value) {
    for (int i = 0; i < h->nsp; ++i)
      if (!h->sp[i].immobile) zc.p[zc.n++] = h->mp[i].fb_count;
    launch_update_b_f32_zero(s, F, (const double*)h->rowtab, rc, Fn, zc);
  } else {
    bulk_b(h, s, F, 1);
  }
  n += 1 + launch_b_axis_bcs(s, F, rec, rc);
  if constexpr (!std::is_same<T, cplxf>::value) {
    launch_zero_step(s, Fn, rc, zc);
    ++n;
  }
  count_launch(h, n);
  h->jpar ^= 1;
  return Fn;
}

// The kernels of one step after the push up to the output point:
// current_bcs_r_min_final and current_finish.
template <typename T>
static void enqueue_current_finish(Handle* h, cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec) {
  const RunConst& rc = h->rc;
  FView wk{h->F[15], rc.nxg, rc.nyg};
  const int stride = h->gd.smooth_stride > 0 ? h->gd.smooth_stride : 1;
  if (h->ion_on) {
    // push_particles ends with current_bcs_r_min_final; ionise_particles
    // runs before current_finish (epoch2d.F90:218-252)
    int n = launch_current_finish(s, F, rec, rc, h->gd.smooth_currents, h->gd.smooth_its, h->gd.smooth_comp_its,
                                  stride, wk, 1);
    if constexpr (std::is_same<T, cplx>::value)
      launch_ionise(s, F, h->sp, h->nsp, h->d_cnt, h->ion, rec, rc, h->d_ion, h->d_ion + MAX_SPECIES, h->d_err,
                    h->nblocks);
    else
      launch_ionise(s, F, h->sp, h->nsp, h->d_cnt, h->ion, rec, rc, h->d_ion, h->d_ion + MAX_SPECIES, h->d_err,
                    h->nblocks, h->xg0);
    n += launch_current_finish(s, F, rec, rc, h->gd.smooth_currents, h->gd.smooth_its, h->gd.smooth_comp_its,
                               stride, wk, 6);
    int nion = 0;
    for (int i = 0; i < h->nsp; ++i) nion += h->ion.s[i].ionise;
    count_launch(h, n + 2 + nion);  // the ionisation: a count snapshot, a kernel per species, the clamp
    return;
  }
  count_launch(h, launch_current_finish(s, F, rec, rc, h->gd.smooth_currents, h->gd.smooth_its,
                                        h->gd.smooth_comp_its, stride, wk));
}

// The kernels of a step after the output point: update_eb_fields_final
// (fields.f90:341-353) and moving_window.
template <typename T>
static void enqueue_step_final(Handle* h, cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec,
                               const double* src, bool window = true, bool fused_out = false) {
  const RunConst& rc = h->rc;
  bulk_b(h, s, F, 0);
  int n = 1 + launch_b_final_bcs(s, F, rec, src, h->cols, 1, rc.dt, rc);
  n += e_half_and_bcs<T>(h, s, F, rec, fused_out ? 1 : 0);
  count_launch(h, n);
  // window: false when no step of the chunk shifts (the window's kernels
  // would do nothing: no injected particles, no removals, no field shift)
  if (h->move_window && window) {
    if (h->inj_counter) {
      launch_inject_counter(s, rec, h->d_injsp, h->nsp, rc, h->inj_seed, h->d_injrow, h->d_inj);
      count_launch(h, 1);
    }
    for (int i = 0; i < h->nsp; ++i) {
      if (h->prec == CYL_PREC_MIXED)
        mixed_window_particles(s, h->sp[i], h->d_cnt + i, h->d_inj, rec, i, h->xg0, rc, h->d_err, h->nblocks);
      else
        launch_window_particles(s, h->sp[i], h->d_cnt + i, h->d_inj, rec, i, rc, h->d_err, h->nblocks);
      count_launch(h, 3);
    }
    launch_shift_fields(s, F, h->cols, rec, 0, rc);
    launch_shift_fields(s, F, h->cols, rec, 1, rc);
    count_launch(h, 2);
  }
}

// The kernels of one step after the push.
template <typename T>
static void enqueue_step_post(Handle* h, cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec,
                              const double* src, bool window = true, bool fused_out = false) {
  enqueue_current_finish<T>(h, s, F, rec);
  enqueue_step_final<T>(h, s, F, rec, src, window, fused_out);
}

// Enqueue the kernels of one step; rec/src point at this step's records.
// fused_in: the step before left its closing E half-step to this step's
// opening one (bulk_e_half); fused_out: this step leaves it to the next.
template <typename T>
static void enqueue_step_t(Handle* h, const StepRec* rec, const double* src, int k_in_chunk, bool timing,
                           bool capturing, bool window, bool fused_in, bool fused_out) {
  const unsigned evflag = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  cudaStream_t s = h->st;
  const FieldSetT<T> F = enqueue_step_pre<T>(h, s, rec, fused_in);
  if (timing) cudaEventRecordWithFlags(h->ev_push[k_in_chunk][0], s, evflag);
  push_all(h, s, F, rec, 1, 1);
  if (timing) cudaEventRecordWithFlags(h->ev_push[k_in_chunk][1], s, evflag);
  enqueue_step_post<T>(h, s, F, rec, src, window, fused_out);
}

// Step i of a chunk of k steps.  In the mixed form, a chunk whose steps do
// not shift the window (no field shift between a step's closing E half-step
// and the next step's opening one) merges those two half-steps at each step
// boundary inside the chunk; the chunk's last step ends with a whole E
// half-step, so the state between chunks is the plain one.
static void enqueue_chunk_step(Handle* h, int i, int k, bool timing, bool capturing, bool window) {
  const StepRec* rec = h->d_rec + i;
  const double* src = h->d_src + h->src_per_step * i;
  const bool fuse = h->prec == CYL_PREC_MIXED && h->merge_e && !window;
  if (h->prec == CYL_PREC_MIXED)
    enqueue_step_t<cplxf>(h, rec, src, i, timing, capturing, window, fuse && i > 0, fuse && i < k - 1);
  else
    enqueue_step_t<cplx>(h, rec, src, i, timing, capturing, window, false, false);
}

// Counting sort of every species by cell; xgm points at the device copy of
// the current x_grid_min (the grid moves with the window).
static void enqueue_sort(Handle* h, const StepRec* rec) {
  for (int i = 0; i < h->nsp; ++i) {
    if (h->sp[i].immobile) continue;
    if (h->prec == CYL_PREC_MIXED) {
      mixed_sort(h->st, h->sp[i], h->d_cnt + i, h->sc, h->d_tiles + i,
                 h->d_tile_start + (size_t)i * (h->ntiles_max + 1), h->d_tile_order + (size_t)i * h->ntiles_max,
                 TILE_SHAPES[h->tile_shape][0], TILE_SHAPES[h->tile_shape][1], rec, h->rc, h->nblocks);
      count_launch(h, 9);
    } else {
      sort_species(h->st, h->sp[i], h->d_cnt + i, h->sc, &rec->x_grid_min_after, h->rc, h->nblocks);
      count_launch(h, 7);
    }
  }
}

static int alloc_species(Handle* h, int i, const cyl_species_desc& d) {
  SpeciesPtrs& p = h->sp[i];
  const int64_t cap = d.capacity > 0 ? d.capacity : 1;
  double* buf = nullptr;
  if (cudaMalloc(&buf, (size_t)cap * 8 * sizeof(double)) != cudaSuccess) return CYL_ERR_OUT_OF_MEMORY;
  p.x = buf;
  p.y = buf + cap;
  p.z = buf + 2 * cap;
  p.px = buf + 3 * cap;
  p.py = buf + 4 * cap;
  p.pz = buf + 5 * cap;
  p.w = buf + 6 * cap;
  p.id = (int64_t*)(buf + 7 * cap);
  p.kx = (int32_t*)buf;
  float* fb = (float*)buf + cap;
  p.fx = fb;
  p.fy = fb + cap;
  p.fz = fb + 2 * cap;
  p.ux = fb + 3 * cap;
  p.uy = fb + 4 * cap;
  p.uz = fb + 5 * cap;
  p.fw = fb + 6 * cap;
  p.cap = cap;
  p.charge = d.charge;
  p.mass = d.mass;
  p.immobile = d.immobile;
  for (int k = 0; k < 4; ++k) p.bc[k] = map_particle_bc(d.bc_particle[k]);
  return CYL_OK;
}

// Geometry tables of push_particles (particles.F90:189-217)
static void make_geom(const HostGrid& g, std::vector<double>& out) {
  const int ny = g.ny, n1 = ny + 2 * JNG, n0 = ny + 2 * JNG + 1;
  out.assign((size_t)n1 * 3 + n0, 0.0);
  double* rt = out.data();
  double* xt = rt + n1;
  double* vol = xt + n0;
  double* rat = vol + n1;
  const double dy = g.dy, dx = g.dx;
  double r_low = g.y_grid_min - JNG * dy;
  xt[0] = 1.0 / (2.0 * PI * std::fabs(r_low) * dx);
  for (int iy = 1 - JNG; iy <= ny + JNG; ++iy) {
    if (std::nearbyint(2.0 * r_low / dy) == -1.0)
      rt[iy - (1 - JNG)] = 1.0 / (PI * ((0.5 * dy) * (0.5 * dy)));
    else
      rt[iy - (1 - JNG)] = 1.0 / (PI * std::fabs((r_low + dy) * (r_low + dy) - r_low * r_low));
    xt[iy - (0 - JNG)] = 1.0 / (2.0 * PI * std::fabs(r_low + dy) * dx);
    r_low = r_low + dy;
  }
  for (int iy = 1 - JNG; iy <= ny + JNG; ++iy) {
    vol[iy - (1 - JNG)] = rt[iy - (1 - JNG)] / dx;
    rat[iy - (1 - JNG)] = xt[iy - (0 - JNG)] / xt[iy - 1 - (0 - JNG)];
  }
}

// Host waits on the device.  The library's waits for a run's work poll the
// stream or event and give up after the process-wide limit
// (cyl_set_wait_timeout, 600 s unless set) with CYL_ERR_TIMEOUT: the work
// stays queued, the handle's bookkeeping is left as it was before the wait,
// and a later call waits for the same work again.  The first 2 ms are polled
// with yields, later polls are 50 us apart.
static std::atomic<double> g_wait_timeout_s{600.0};

template <class Query>
static int poll_device(Query query, cudaError_t* err) {
  const double lim = g_wait_timeout_s.load();
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    const cudaError_t e = query();
    if (e != cudaErrorNotReady) {
      *err = e;
      return e == cudaSuccess ? CYL_OK : CYL_ERR_CUDA;
    }
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (lim > 0.0 && el > lim) {
      *err = cudaSuccess;
      return CYL_ERR_TIMEOUT;
    }
    if (el < 2e-3)
      std::this_thread::yield();
    else
      std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

static int wait_stream(Handle* h, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  const int rc = poll_device([s] { return cudaStreamQuery(s); }, &e);
  if (rc == CYL_ERR_CUDA) h->last_cuda_error = e;
  return rc;
}

static int wait_event(Handle* h, cudaEvent_t ev) {
  cudaError_t e = cudaSuccess;
  const int rc = poll_device([ev] { return cudaEventQuery(ev); }, &e);
  if (rc == CYL_ERR_CUDA) h->last_cuda_error = e;
  return rc;
}

// The end of copies to or from host memory that the caller or this frame
// owns.  The stream's earlier work has been waited for with the limit before
// the copies were queued, so this wait is for the copies alone; it is not
// cut short, because the memory must stay valid until they are done.
static int copies_done(Handle* h, cudaStream_t s) {
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    h->last_cuda_error = e;
    return CYL_ERR_CUDA;
  }
  return CYL_OK;
}

#define WAIT(call)                    \
  do {                                \
    if (int rc_ = (call)) return rc_; \
  } while (0)

static int flush_push_timing(Handle* h);

static int sync_and_check(Handle* h) {
  WAIT(wait_stream(h, h->st));
  if (int r = flush_push_timing(h)) return r;
  int err = 0;
  CK(cudaMemcpy(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return CYL_ERR_DEVICE_FLAG;
  return CYL_OK;
}

static void collect_push_timing(Handle* h, int nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev_push[k][0], h->ev_push[k][1]) == cudaSuccess) {
      h->push_ms_sum += ms;
      h->push_launches += 1;
    }
  }
}

// Read the push events of the last chunk (they are re-recorded by the next).
static int flush_push_timing(Handle* h) {
  if (h->timing_pending > 0) {
    WAIT(wait_event(h, h->ev_push[h->timing_pending - 1][1]));
    collect_push_timing(h, h->timing_pending);
    h->timing_pending = 0;
  }
  return CYL_OK;
}

// Capture the CHUNK steps of a chunk that starts at the current J parity
// (with or without the window's kernels) and the sort after them into a
// graph, and instantiate it.  Nothing runs: the host state that enqueueing
// moves (J parity, the launch count) is put back.  The graph reads the
// chunk's step records and laser sources from the staging buffers when it
// is launched.  The stream may still hold earlier work: the capture does
// not depend on it, and the graph's launch is ordered after it.
static int capture_chunk_graph(Handle* h, bool window) {
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  const int par0 = h->jpar;
  const int64_t launches0 = h->kernel_launches;
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < CHUNK; ++i) enqueue_chunk_step(h, i, CHUNK, true, true, window);
  enqueue_sort(h, h->d_rec + (CHUNK - 1));
  h->graph_launches = h->kernel_launches - launches0;
  h->kernel_launches = launches0;
  h->jpar = par0;
  CK(cudaStreamEndCapture(h->st, &graph));
  const cudaError_t e = cudaGraphInstantiate(&h->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    h->gexec = nullptr;
    return CYL_ERR_CUDA;
  }
  h->graph_parity = par0;
  h->graph_window = window;
  return CYL_OK;
}

static int run_chunk(Handle* h, int k, bool use_graph) {
  // staging buffers are reused: wait until the previous chunk's copies are done
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  // the push events of the previous chunk are read (and re-recorded by this
  // one); both waits come before the host state moves, so a wait that runs
  // out leaves the run as it was.  The previous chunk's field stages and
  // sort still run on the device while this chunk is prepared and queued.
  if (int r = flush_push_timing(h)) return r;
  int64_t inj_used = 0;
  h->cb_failed = false;
  for (int i = 0; i < k; ++i) prepare_step(h, i, inj_used);
  if (h->cb_failed) return CYL_ERR_CALLBACK;
  CK(cudaMemcpyAsync(h->d_rec, h->h_rec, sizeof(StepRec) * k, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_src, h->h_src, sizeof(double) * h->src_per_step * k, cudaMemcpyHostToDevice, h->st));
  if (inj_used > 0 && !h->inj_counter)
    CK(cudaMemcpyAsync(h->d_inj, h->h_inj, sizeof(double) * 8 * inj_used, cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->ev_copy, h->st));
  h->copy_pending = true;
  const StepRec* last = h->d_rec + (k - 1);
  // whether any step of the chunk shifts the window (the host has just
  // prepared their records): a chunk without shifts leaves out the window's
  // kernels, which would find nothing to inject, remove or shift
  bool window = false;
  for (int i = 0; i < k; ++i) window = window || h->h_rec[i].nshift > 0;
  const bool have_graph = h->gexec && h->graph_parity == h->jpar && h->graph_window == window;
  if (use_graph && k == CHUNK && have_graph) {
    CK(cudaGraphLaunch(h->gexec, h->st));
    h->kernel_launches += h->graph_launches;
    // a chunk swaps J and J_old CHUNK times
    h->jpar = h->graph_parity ^ (CHUNK & 1);
  } else {
    // a launch that cannot start (a bad configuration) reports only through
    // the thread's last error: clear it before the launches, read it after
    (void)cudaGetLastError();
    for (int i = 0; i < k; ++i) enqueue_chunk_step(h, i, k, true, false, window);
    enqueue_sort(h, last);
    CK(cudaGetLastError());
    // No graph of this chunk's kind (J parity, window kernels) yet: the chunk
    // ran from single launches, and the graph of the next chunk of the same
    // kind is captured and instantiated now, while the device works through
    // this one.  Built before the launch instead, the capture and the
    // instantiation (about a millisecond of host time) would leave the
    // stream idle.
    // the chunk is queued: its push events are read with the next chunk
    // even when the capture fails
    h->timing_pending = k;
    if (use_graph && k == CHUNK)
      if (int r = capture_chunk_graph(h, window)) return r;
    return CYL_OK;
  }
  h->timing_pending = k;
  return CYL_OK;
}

// ---------------------------------------------------------------------------
// Cell-sort indices without allocation (cyl_cell_indices_noalloc).
//
// cyl_cell_indices takes a device scratch of 12 bytes per particle slot from
// cudaMalloc on every call.  Callers that cannot allocate per call -- a
// diagnostics hook run between queued steps, where cudaMalloc/cudaFree would
// synchronise the device and stall the steps behind it, and runs admitted
// against a fully committed HBM budget, where the allocation could fail --
// use this fixed scratch instead: a file-scope device array reserved when the
// library is loaded, 5 int32 words per slot:
//   [0, N)   cell_x of every slot      [N, 2N)  cell_y      [2N, 3N) live flag
//   [3N, 4N) compacted cell_x          [4N, 5N) compacted cell_y
//   [5N]     number of live slots
// with N = CYL_NOALLOC_MAX_PARTICLES.  Nothing in it needs to start at zero:
// every word a call reads was written earlier in the same call.  The scratch
// is shared by every handle of the process, so calls that overlap in time
// race on it.
static __device__ __align__(256) int32_t g_cell_scratch[5 * (size_t)CYL_NOALLOC_MAX_PARTICLES + 64];

constexpr int MAX_SCRATCH_DEVICES = 64;
static int32_t* g_cell_scratch_ptr[MAX_SCRATCH_DEVICES] = {};
static std::mutex g_cell_scratch_mu;

// Device address of the scratch on device `dev`, which must be the current
// device; looked up by the first call on each device (the lookup can load
// the module, so that first call should come before any stream capture).
static int cell_scratch(int dev, int32_t** out) {
  if (dev < 0 || dev >= MAX_SCRATCH_DEVICES) return CYL_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_cell_scratch_mu);
  if (!g_cell_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_cell_scratch);
    if (e != cudaSuccess || !p) return CYL_ERR_CUDA;
    g_cell_scratch_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_cell_scratch_ptr[dev];
  return CYL_OK;
}

// Order-preserving compaction of the live slots' (cell_x, cell_y) by one CTA
// of 1024 threads: a block-wide exclusive scan of the live flags per chunk of
// 1024 slots.  Writes the live count to *count.
__global__ void __launch_bounds__(1024) k_compact_cells(const int32_t* cx, const int32_t* cy, const int32_t* live,
                                                        int64_t n, int32_t* ocx, int32_t* ocy, int32_t* count) {
  __shared__ int warp_sums[32];
  __shared__ int base_s;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < n; c0 += 1024) {
    const int64_t i = c0 + threadIdx.x;
    const int f = (i < n && live[i]) ? 1 : 0;
    int v = f;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, d);
      if (lane >= d) v += t;
    }
    if (lane == 31) warp_sums[w] = v;
    __syncthreads();
    if (w == 0) {
      int s = warp_sums[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d) s += t;
      }
      warp_sums[lane] = s;
    }
    __syncthreads();
    const int base = base_s;
    const int excl = base + (v - f) + (w > 0 ? warp_sums[w - 1] : 0);
    if (f) {
      ocx[excl] = cx[i];
      ocy[excl] = cy[i];
    }
    __syncthreads();
    if (threadIdx.x == 1023) base_s = excl + f;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = base_s;
}

}  // namespace cyl

using namespace cyl;

struct cyl_handle_s {
  Handle h;
};

// A batch: mixed-form runs with the same number of modes stepped together,
// their pushes one launch per step over a shared (job, tile) work table (a
// job is one mobile species of one run).  The stages before and after the
// push stay per run, on each run's own stream, forked from and joined to the
// batch stream around the push; a chunk of 16 steps is one CUDA graph,
// captured again when the membership or a run's current parity changes.
struct cyl_batch_s {
  int device = 0;
  int cap_runs = 0, cap_jobs = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_sched = nullptr, ev_push = nullptr, ev_done = nullptr, ev_jobs = nullptr;
  std::vector<cudaEvent_t> ev_run;  // one per run slot
  BatchJob* h_jobs = nullptr;       // pinned, CHUNK x cap_jobs (step-major)
  BatchJob* d_jobs = nullptr;
  StageJob* h_stage = nullptr;      // pinned, CHUNK x cap_runs (step-major)
  StageJob* d_stage = nullptr;
  WindowJob* h_win = nullptr;       // pinned, CHUNK x cap_jobs (step-major)
  WindowJob* d_win = nullptr;
  int2* d_work = nullptr;
  int* d_nwork = nullptr;
  int64_t work_cap = 0;
  bool jobs_pending = false;
  cudaGraphExec_t gexec = nullptr;
  std::vector<uint64_t> g_runs;  // membership (handle serials, step epochs) and parities of the captured graph
  std::vector<int> g_par;
  int g_jobs = 0;
  std::unique_ptr<HostPool> pool;  // per-run host preparation of a chunk
};

namespace cyl {

struct JobRef {
  Handle* h;
  int isp;
};

// The extents and boundary kinds of a batch's runs (one M for all).
static StageDims stage_dims(const std::vector<Handle*>& runs, int* mask_any, bool* any_window) {
  StageDims d{0, 0, runs[0]->rc.M};
  *mask_any = 0;
  *any_window = false;
  for (Handle* h : runs) {
    d.nx_max = std::max(d.nx_max, h->rc.nx);
    d.ny_max = std::max(d.ny_max, h->rc.ny);
    *mask_any |= h->rc.bc_mask;
    *any_window = *any_window || h->move_window;
  }
  return d;
}

// The kernels of k steps of a batch on b->st: per step, each field and
// boundary stage of every run in one launch from the chunk's stage table
// (update_eb_fields_half, the J swap, the (run, tile) push, current_finish,
// update_eb_fields_final, the window's particle stages and field shift), the
// stages that only some runs have (current smoothing, counter injection) per
// run on the same stream; the chunk's (job, tile) table first, every run's
// sort last on its own stream.  The step's node count depends on the number
// of runs with those extra stages, not on the number of runs.
static void enqueue_batch_chunk(cyl_batch_s* b, const std::vector<Handle*>& runs, int njobs, int nwin, int k,
                                int M, const std::vector<int>& par0) {
  const PushMixedFns& fns = push_mixed_fns(0);
  const int nbt = runs[0]->nblocks_by_shape[0], nbg = runs[0]->nblocks;
  const int nr = (int)runs.size();
  int mask_any = 0;
  bool any_window = false;
  const StageDims d = stage_dims(runs, &mask_any, &any_window);
  bool any_finish = false;
  for (Handle* h : runs) any_finish = any_finish || stage_finish_needed(h->rc);
  batch_schedule(b->st, b->d_jobs, njobs, b->d_work, b->d_nwork);
  int launches = 1;
  for (int i = 0; i < k; ++i) {
    const StageJob* st = b->d_stage + (size_t)i * b->cap_runs;
    batch_update_e_f32(b->st, st, nr, 0, d);
    batch_e_axis_bcs(b->st, st, nr, 0, mask_any, d);
    batch_update_b_f32(b->st, st, nr, 0, 1, d);
    batch_b_axis_bcs(b->st, st, nr, 0, mask_any, d);
    batch_zero_j(b->st, st, nr, d);
    const BatchJob* tab = b->d_jobs + (size_t)i * b->cap_jobs;
    batch_reset(b->st, tab, njobs);
    fns.launch_batch(b->st, M, tab, njobs, b->d_work, b->d_nwork, nbt, nbg);
    batch_j_rmin(b->st, st, nr, d);
    launches += 10;
    if (any_finish) {
      batch_current_finish(b->st, st, nr);
      launches += 1;
    }
    for (int r = 0; r < nr; ++r) {
      Handle* h = runs[(size_t)r];
      if (!h->gd.smooth_currents) continue;
      // smoothing (rare): per run
      const FieldSetF F1 = fieldset_f(h, par0[(size_t)r] ^ ((i + 1) & 1));
      const RunConst& rc = h->rc;
      FView wk{h->F[15], rc.nxg, rc.nyg};
      const int stride = h->gd.smooth_stride > 0 ? h->gd.smooth_stride : 1;
      launch_current_finish(b->st, F1, h->d_rec + i, rc, h->gd.smooth_currents, h->gd.smooth_its,
                            h->gd.smooth_comp_its, stride, wk, 4);
      launches += 1;
    }
    batch_update_b_f32(b->st, st, nr, 1, 0, d);
    batch_b_final_bcs(b->st, st, nr, mask_any, d);
    batch_update_e_f32(b->st, st, nr, 1, d);
    batch_e_axis_bcs(b->st, st, nr, 1, mask_any, d);
    launches += 8;
    if (any_window) {
      for (Handle* h : runs)
        if (h->move_window && h->inj_counter) {
          launch_inject_counter(b->st, h->d_rec + i, h->d_injsp, h->nsp, h->rc, h->inj_seed, h->d_injrow,
                                h->d_inj);
          launches += 1;
        }
      batch_window_particles(b->st, b->d_win + (size_t)i * b->cap_jobs, nwin, nbg);
      batch_shift_fields(b->st, st, nr, 0, d);
      batch_shift_fields(b->st, st, nr, 1, d);
      launches += 5;
    }
  }
  runs[0]->kernel_launches += launches;
  cudaEventRecord(b->ev_push, b->st);
  for (size_t r = 0; r < runs.size(); ++r) {
    Handle* h = runs[r];
    cudaStreamWaitEvent(h->st, b->ev_push, 0);
    enqueue_sort(h, h->d_rec + (k - 1));
    cudaEventRecord(b->ev_run[r], h->st);
    cudaStreamWaitEvent(b->st, b->ev_run[r], 0);
  }
  // the chunk advanced each run's J parity by k
  for (Handle* h : runs) h->jpar ^= (k & 1);
}

}  // namespace cyl

extern "C" {

int cyl_estimate_device_bytes(const cyl_grid_desc* gd, const cyl_species_desc* spd, int32_t nsp,
                              int64_t* out) {
  // the allocations of cyl_create below, from the descriptors alone
  if (!gd || !out || (nsp > 0 && !spd) || nsp < 0 || nsp > MAX_SPECIES) return CYL_ERR_BAD_ARG;
  if (gd->nx < 8 || gd->ny < 8 || gd->n_mode < 1 || gd->n_mode > MAX_MODES) return CYL_ERR_BAD_ARG;
  const int64_t nxg = gd->nx + 2 * NG, nyg = gd->ny + 2 * NG, M = gd->n_mode;
  const int64_t fcount = nxg * nyg * M;
  int64_t b = fcount * 16 * (int64_t)sizeof(cplx);                 // 15 mode arrays + work array
  if (gd->precision == CYL_PREC_MIXED) b += fcount * 9 * (int64_t)sizeof(cplxf);  // FP32 E, B, B_old
  b += (gd->ny + 2 * NG) * M * 12 * (int64_t)sizeof(cplx);         // boundary columns
  int64_t maxcap = 1, fbtot = 0, per_step_inj = 0;
  const double dx = (gd->x_max - gd->x_min) / (double)gd->nx;
  const double shifts_max = std::floor(gd->dt * std::fabs(gd->window_v_x) / dx) + 1.0;
  for (int i = 0; i < nsp; ++i) {
    const int64_t cap = spd[i].capacity > 0 ? spd[i].capacity : 1;
    b += cap * 8 * (int64_t)sizeof(double);                        // particle SoA
    maxcap = std::max(maxcap, cap);
    fbtot += cap + 1;
    per_step_inj += (int64_t)(shifts_max * (double)gd->ny * (std::floor(spd[i].npart_per_cell) + 1.0));
  }
  if (gd->precision == CYL_PREC_MIXED) b += fbtot * (int64_t)sizeof(int);  // deferred lists
  const int64_t ntiles_max = ntiles_max_of(gd->nx, gd->ny);
  b += (ntiles_max + 1) * MAX_SPECIES * 8 + ntiles_max * MAX_SPECIES * 4;
  const int64_t ncells = nxg * nyg;
  b += maxcap * (4 + 8 * 8) + (ncells + 2) * 4 + ((ncells + 4096) / 4096 + 64) * 8;  // sort scratch
  const int64_t inj_cap = gd->move_window ? per_step_inj * CHUNK + 1 : 1;
  b += inj_cap * 8 * (int64_t)sizeof(double) + (int64_t)4 * (gd->ny + 1) * CHUNK * 8 +
       (int64_t)sizeof(StepRec) * (CHUNK + 1);
  b += 1 << 20;  // small tables, counters, allocation granularity
  *out = b;
  return CYL_OK;
}

int cyl_create(const cyl_grid_desc* gd, const cyl_species_desc* spd, int32_t nsp,
               const cyl_laser_desc* las, int32_t nlas, const cyl_rng_state* rng, cyl_handle* out) {
  if (!gd || !out || (nsp > 0 && !spd) || (nlas > 0 && !las)) return CYL_ERR_BAD_ARG;
  if (gd->nx < 8 || gd->ny < 8 || gd->n_mode < 1 || gd->n_mode > MAX_MODES) return CYL_ERR_BAD_ARG;
  if (nsp < 0 || nsp > MAX_SPECIES || nlas < 0 || nlas > MAX_LASERS) return CYL_ERR_BAD_ARG;
  if (!(gd->dt > 0.0) || !(gd->x_max > gd->x_min) || !(gd->y_max > 0.0)) return CYL_ERR_BAD_ARG;
  if (gd->precision != CYL_PREC_FP64 && gd->precision != CYL_PREC_MIXED) return CYL_ERR_BAD_ARG;

  for (int i = 0; i < nlas; ++i) {
    if (las[i].boundary != CYL_BD_X_MIN && las[i].boundary != CYL_BD_X_MAX) return CYL_ERR_UNSUPPORTED;
    if (!las[i].profile || !las[i].phase) return CYL_ERR_BAD_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CYL_ERR_NO_DEVICE;
  static std::atomic<uint64_t> next_serial{1};
  cyl_handle_s* hs = new cyl_handle_s();
  Handle* h = &hs->h;
  h->serial = next_serial.fetch_add(1);
  cudaGetDevice(&h->device);
  h->gd = *gd;
  h->prec = gd->precision;
  h->g.init(*gd);
  RunConst& rc = h->rc;
  rc.nx = gd->nx;
  rc.ny = gd->ny;
  rc.M = gd->n_mode;
  rc.nxg = gd->nx + 2 * NG;
  rc.nyg = gd->ny + 2 * NG;
  rc.dx = h->g.dx;
  rc.dy = h->g.dy;
  rc.dt = gd->dt;
  rc.y_grid_min = h->g.y_grid_min;
  rc.y_max = h->g.y_max;
  rc.y_max_local = h->g.y_max_local;
  rc.length_x = h->g.length_x;
  rc.length_y = h->g.length_y;
  for (int i = 0; i < 4; ++i) {
    h->bc_deck[i] = gd->bc_field[i];
    h->bc_after_move[i] = gd->bc_after_move[i];
  }
  setup_boundaries(h);
  h->move_window = gd->move_window != 0;
  rc.bc_mask = bc_mask_of(gd->bc_field, gd->bc_after_move, h->move_window);
  h->window_v_x = gd->window_v_x;
  h->window_start_time = gd->window_start_time;
  h->window_stop_time = gd->window_stop_time;
  h->nsp = nsp;
  int rcode = CYL_OK;
  for (int i = 0; i < nsp; ++i) {
    h->sd[i] = spd[i];
    for (int k = 0; k < 4; ++k) {
      int b = map_particle_bc(spd[i].bc_particle[k]);
      if (k != CYL_BD_Y_MIN && b != CYL_BC_PERIODIC && b != CYL_BC_REFLECT && b != CYL_BC_OPEN)
        rcode = CYL_ERR_UNSUPPORTED;
    }
  }
  // bc_allspecies (deck_species_block.F90:182-199)
  for (int idx = 0; idx < 4; ++idx) {
    h->bc_allspecies[idx] = CYL_BC_OPEN;
    for (int i = 0; i < nsp; ++i) {
      int b = map_particle_bc(spd[i].bc_particle[idx]);
      if (b != CYL_BC_REFLECT && b != CYL_BC_PERIODIC) b = CYL_BC_OPEN;
      if (i == 0) h->bc_allspecies[idx] = b;
      else if (h->bc_allspecies[idx] != b) rcode = CYL_ERR_UNSUPPORTED;  // mixed per-species bcs
    }
    rc.bc_allspecies[idx] = h->bc_allspecies[idx];
  }
  if (rcode != CYL_OK) {
    delete hs;
    return rcode;
  }
  for (int i = 0; i < nlas; ++i) {
    HostLaser L;
    L.d = las[i];
    L.profile.assign(las[i].profile, las[i].profile + gd->ny + 1);
    L.phase.assign(las[i].phase, las[i].phase + gd->ny + 1);
    L.d.profile = nullptr;
    L.d.phase = nullptr;
    h->lasers.push_back(L);
  }
  if (rng) h->rng.from_state(rng);
  else h->rng.seed(7842432);

  cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete hs;
    return CYL_ERR_CUDA;
  }
  // first failing CUDA call of the set-up (its code is checked at the end)
  cudaError_t first_err = cudaSuccess;
  auto ok = [&first_err](cudaError_t e) {
    if (e != cudaSuccess && first_err == cudaSuccess) first_err = e;
  };
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device);
  h->nblocks = nsm * 8;
  ok(cudaMalloc(&h->d_err, sizeof(int)));
  ok(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
  ok(cudaMalloc(&h->d_dbg, 16 * sizeof(float)));
  ok(cudaMemsetAsync(h->d_dbg, 0, 16 * sizeof(float), h->st));
  // fields: 15 arrays + one work array, one allocation
  h->fcount = (size_t)rc.nxg * rc.nyg * rc.M;
  if (cudaMalloc(&h->fbuf, h->fcount * 16 * sizeof(cplx)) != cudaSuccess) {
    cyl_destroy((cyl_handle)hs);
    return CYL_ERR_OUT_OF_MEMORY;
  }
  ok(cudaMemsetAsync(h->fbuf, 0, h->fcount * 16 * sizeof(cplx), h->st));
  for (int k = 0; k < 16; ++k) h->F[k] = h->fbuf + h->fcount * k;
  const size_t ncolv = (size_t)(rc.ny + 2 * NG) * rc.M;
  ok(cudaMalloc(&h->cols, ncolv * 12 * sizeof(cplx)));
  ok(cudaMemsetAsync(h->cols, 0, ncolv * 12 * sizeof(cplx), h->st));
  // host sources of the set-up copies, alive until the stream is synchronised
  std::vector<double> geo;
  std::vector<float4> rt;
  std::vector<float> gf;
  make_geom(h->g, geo);
  ok(cudaMalloc(&h->geom_buf, geo.size() * sizeof(double)));
  ok(cudaMemcpyAsync(h->geom_buf, geo.data(), geo.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  {
    const int n1 = rc.ny + 2 * JNG, n0 = n1 + 1;
    h->geom.inv_area_rt = h->geom_buf;
    h->geom.inv_area_xt = h->geom_buf + n1;
    h->geom.inv_volume = h->geom_buf + n1 + n0;
    h->geom.ratio_area_xt = h->geom_buf + 2 * n1 + n0;
  }
  if (h->prec == CYL_PREC_MIXED) {
    // FP32 E, B, B_old
    if (cudaMalloc(&h->ffbuf, h->fcount * 9 * sizeof(cplxf)) != cudaSuccess) {
      cyl_destroy((cyl_handle)hs);
      return CYL_ERR_OUT_OF_MEMORY;
    }
    ok(cudaMemsetAsync(h->ffbuf, 0, h->fcount * 9 * sizeof(cplxf), h->st));
    for (int k = 0; k < 9; ++k) h->Ff[k] = h->ffbuf + h->fcount * k;
    // per-row Yee coefficients: c^2/r_p dt/2, c^2/r_d dt/2, dt/2/r_d, dt/2/r_p
    rt.resize(rc.ny + 2);
    for (int ir = 0; ir <= rc.ny + 1; ++ir) {
      const double r_d = std::fabs((double)(ir - 1) * rc.dy + rc.y_grid_min);
      const double r_p = r_d + 0.5 * rc.dy;
      const double hh2 = 0.5 * rc.dt, c2 = CLIGHT * CLIGHT;
      rt[ir] = make_float4((float)(c2 / r_p * hh2), (float)(c2 / r_d * hh2), (float)(hh2 / r_d), (float)(hh2 / r_p));
    }
    ok(cudaMalloc(&h->rowtab, rt.size() * sizeof(float4)));
    ok(cudaMemcpyAsync(h->rowtab, rt.data(), rt.size() * sizeof(float4), cudaMemcpyHostToDevice, h->st));
    gf.resize(geo.size());
    for (size_t k = 0; k < geo.size(); ++k) gf[k] = (float)geo[k];
    ok(cudaMalloc(&h->gtab_f, gf.size() * sizeof(float)));
    ok(cudaMemcpyAsync(h->gtab_f, gf.data(), gf.size() * sizeof(float), cudaMemcpyHostToDevice, h->st));
  }
  int64_t maxcap = 1;
  for (int i = 0; i < nsp; ++i) {
    if (alloc_species(h, i, spd[i]) != CYL_OK) {
      cyl_destroy((cyl_handle)hs);
      return CYL_ERR_OUT_OF_MEMORY;
    }
    if (h->sp[i].cap > maxcap) maxcap = h->sp[i].cap;
  }
  h->xg0 = h->g.x_grid_min;
  h->ntiles_max = ntiles_max_of(rc.nx, rc.ny);
  ok(cudaMalloc(&h->d_tiles, sizeof(TileTable) * MAX_SPECIES));
  ok(cudaMemsetAsync(h->d_tiles, 0, sizeof(TileTable) * MAX_SPECIES, h->st));
  ok(cudaMalloc(&h->d_tile_start, sizeof(int64_t) * (h->ntiles_max + 1) * MAX_SPECIES));
  ok(cudaMemsetAsync(h->d_tile_start, 0, sizeof(int64_t) * (h->ntiles_max + 1) * MAX_SPECIES, h->st));
  ok(cudaMalloc(&h->d_tile_order, sizeof(int32_t) * h->ntiles_max * MAX_SPECIES));
  if (h->prec == CYL_PREC_MIXED) {
    int64_t fbtot = 0;
    for (int i = 0; i < nsp; ++i) fbtot += h->sp[i].cap + 1;
    if (cudaMalloc(&h->fb_buf, sizeof(int) * (size_t)fbtot) != cudaSuccess) {
      cyl_destroy((cyl_handle)hs);
      return CYL_ERR_OUT_OF_MEMORY;
    }
    int64_t off = 0;
    const int n1 = rc.ny + 2 * JNG, n0 = n1 + 1;
    for (int i = 0; i < nsp; ++i) {
      h->mp[i] = mixed_params(h->sp[i], rc);
      h->mp[i].err = h->d_err;
      h->mp[i].g_rt = h->gtab_f;
      h->mp[i].g_xt = h->gtab_f + n1;
      h->mp[i].g_vol = h->gtab_f + n1 + n0;
      h->mp[i].fb_count = h->fb_buf + off;
      h->mp[i].fb_list = h->fb_buf + off + 1;
      h->mp[i].dbg = h->d_dbg;
      off += h->sp[i].cap + 1;
    }
  }
  if (h->prec == CYL_PREC_MIXED) {
    for (int k = 0; k < N_TILE_SHAPES; ++k) h->nblocks_by_shape[k] = nsm * push_mixed_fns(k).blocks_per_sm(rc.M);
    h->nblocks_mixed = h->nblocks_by_shape[h->tile_shape];
  }
  ok(cudaMalloc(&h->d_cnt, sizeof(SpeciesCounters) * MAX_SPECIES));
  ok(cudaMemsetAsync(h->d_cnt, 0, sizeof(SpeciesCounters) * MAX_SPECIES, h->st));
  // sort scratch: keys, histogram, block sums, 7 doubles + id per particle
  h->sc.ncells = rc.nxg * rc.nyg;
  h->sc.cap = maxcap;
  const size_t sort_bytes = (size_t)maxcap * (4 + 8 * 8) + (size_t)(h->sc.ncells + 2) * 4 +
                            (size_t)((h->sc.ncells + 4096) / 4096 + 64) * 8;
  if (cudaMalloc(&h->sort_buf, sort_bytes) != cudaSuccess) {
    cyl_destroy((cyl_handle)hs);
    return CYL_ERR_OUT_OF_MEMORY;
  }
  {
    char* p = (char*)h->sort_buf;
    h->sc.tmp = (double*)p;
    p += (size_t)maxcap * 7 * 8;
    h->sc.tmp_id = (int64_t*)p;
    p += (size_t)maxcap * 8;
    h->sc.perm = (int64_t*)p;
    p += (size_t)((h->sc.ncells + 4096) / 4096 + 64) * 8;
    h->sc.keys = (int32_t*)p;
    p += (size_t)maxcap * 4;
    h->sc.hist = (int32_t*)p;
  }
  ok(cudaMalloc(&h->d_red, 8 * sizeof(double)));
  // staging for CHUNK steps
  h->src_per_step = (size_t)4 * (rc.ny + 1);
  int64_t per_step_inj = 0;
  const double shifts_max = std::floor(gd->dt * std::fabs(gd->window_v_x) / h->g.dx) + 1.0;
  for (int i = 0; i < nsp; ++i)
    per_step_inj += (int64_t)(shifts_max * (double)rc.ny * (std::floor(spd[i].npart_per_cell) + 1.0));
  h->inj_cap = h->move_window ? per_step_inj * CHUNK + 1 : 1;
  ok(cudaMallocHost(&h->h_rec, sizeof(StepRec) * CHUNK));
  ok(cudaMalloc(&h->d_rec, sizeof(StepRec) * (CHUNK + 1)));
  ok(cudaMallocHost(&h->h_src, sizeof(double) * h->src_per_step * CHUNK));
  ok(cudaMalloc(&h->d_src, sizeof(double) * h->src_per_step * CHUNK));
  ok(cudaMallocHost(&h->h_inj, sizeof(double) * 8 * h->inj_cap));
  ok(cudaMalloc(&h->d_inj, sizeof(double) * 8 * h->inj_cap));
  ok(cudaEventCreateWithFlags(&h->ev_copy, cudaEventDisableTiming));
  for (int k = 0; k < CHUNK; ++k) {
    ok(cudaEventCreate(&h->ev_push[k][0]));
    ok(cudaEventCreate(&h->ev_push[k][1]));
  }
  // Only this handle's stream is synchronised: a device-wide synchronisation
  // is invalid while another thread's stream is being captured into a graph
  // (the request loop creates handles while other runs capture their steps).
  ok(cudaStreamSynchronize(h->st));
  if (first_err != cudaSuccess) {
    cyl_destroy((cyl_handle)hs);
    return first_err == cudaErrorMemoryAllocation ? CYL_ERR_OUT_OF_MEMORY : CYL_ERR_CUDA;
  }
  *out = (cyl_handle)hs;
  return CYL_OK;
}

int cyl_set_wait_timeout(double seconds) {
  if (std::isnan(seconds)) return CYL_ERR_BAD_ARG;
  g_wait_timeout_s.store(seconds);
  return CYL_OK;
}

int cyl_destroy(cyl_handle hh) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  cudaFree(h->d_injsp);
  cudaFree(h->d_injrow);
  for (auto& d : h->diag_slot) {
    if (d.h) cudaFreeHost(d.h);
    if (d.ev) cudaEventDestroy(d.ev);
  }
  for (int i = 0; i < h->nsp; ++i)
    if (h->sp[i].x) cudaFree(h->sp[i].x);
  cudaFree(h->fbuf);
  cudaFree(h->cols);
  cudaFree(h->geom_buf);
  cudaFree(h->d_cnt);
  cudaFree(h->d_tiles);
  cudaFree(h->ffbuf);
  cudaFree(h->rowtab);
  cudaFree(h->gtab_f);
  cudaFree(h->fb_buf);
  cudaFree(h->d_ion);
  cudaFree(h->d_dbg);
  cudaFree(h->d_tile_start);
  cudaFree(h->d_tile_order);
  cudaFree(h->sort_buf);
  cudaFree(h->d_err);
  cudaFree(h->d_red);
  cudaFreeHost(h->h_rec);
  cudaFree(h->d_rec);
  cudaFreeHost(h->h_src);
  cudaFree(h->d_src);
  cudaFreeHost(h->h_inj);
  cudaFree(h->d_inj);
  if (h->ev_copy) cudaEventDestroy(h->ev_copy);
  for (int k = 0; k < CHUNK; ++k) {
    if (h->ev_push[k][0]) cudaEventDestroy(h->ev_push[k][0]);
    if (h->ev_push[k][1]) cudaEventDestroy(h->ev_push[k][1]);
  }
  if (h->st) cudaStreamDestroy(h->st);
  delete hh;
  return CYL_OK;
}

int cyl_upload_particles(cyl_handle hh, int32_t isp, const double* x, const double* y, const double* z,
                         const double* px, const double* py, const double* pz, const double* w,
                         const int64_t* id, int64_t n) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (isp < 0 || isp >= h->nsp || n < 0) return CYL_ERR_BAD_ARG;
  if (n > 0 && (!x || !y || !z || !px || !py || !pz || !w || !id)) return CYL_ERR_BAD_ARG;
  SpeciesPtrs& p = h->sp[isp];
  if (n > p.cap) return CYL_ERR_CAPACITY;
  cudaStream_t s = h->st;
  WAIT(wait_stream(h, s));
  const size_t b = (size_t)n * 8;
  if (n > 0 && h->prec == CYL_PREC_MIXED) {
    // stage the FP64 arrays in the sort scratch, convert on the device
    double* st = h->sc.tmp;
    const int64_t cap = h->sc.cap;
    const double* srcs[7] = {x, y, z, px, py, pz, w};
    for (int k = 0; k < 7; ++k) CK(cudaMemcpyAsync(st + (size_t)k * cap, srcs[k], b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(st + (size_t)7 * cap, id, b, cudaMemcpyHostToDevice, s));
    mixed_from_double(s, p, st, n, cap, h->xg0, h->rc);
  } else if (n > 0) {
    CK(cudaMemcpyAsync(p.x, x, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.y, y, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.z, z, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.px, px, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.py, py, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.pz, pz, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.w, w, b, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(p.id, id, b, cudaMemcpyHostToDevice, s));
  }
  // the counters, with the largest FP32 weight (the mixed form's fixed-point
  // deposit scale) and the largest id (the next id of window injection)
  // reduced on the device from the copied arrays
  SpeciesCounters c{n, 0, 0u, 0u};
  long long max_id = -1;
  long long* d_max = reinterpret_cast<long long*>(h->d_red);  // reduction scratch
  CK(cudaMemcpyAsync(h->d_cnt + isp, &c, sizeof(c), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_max, &max_id, sizeof(max_id), cudaMemcpyHostToDevice, s));
  if (h->prec == CYL_PREC_MIXED)
    upload_stats(s, h->sc.tmp + (size_t)6 * h->sc.cap, reinterpret_cast<const int64_t*>(h->sc.tmp + (size_t)7 * h->sc.cap),
                 n, h->d_cnt + isp, d_max);
  else
    upload_stats(s, p.w, p.id, n, h->d_cnt + isp, d_max);
  CK(cudaGetLastError());
  WAIT(copies_done(h, s));
  CK(cudaMemcpy(&max_id, d_max, sizeof(max_id), cudaMemcpyDeviceToHost));
  if (max_id >= h->next_id) h->next_id = max_id + 1;
  return CYL_OK;
}

int cyl_load_species_device(cyl_handle hh, int32_t isp, uint64_t seed, int64_t id_base, int64_t* n_out) {
  if (!hh || !n_out) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (isp < 0 || isp >= h->nsp || id_base < 0) return CYL_ERR_BAD_ARG;
  const cyl_species_desc& d = h->sd[isp];
  if (d.immobile) return CYL_ERR_BAD_ARG;
  SpeciesPtrs& p = h->sp[isp];
  std::vector<double> dens;
  std::vector<char> dmap;
  std::vector<int32_t> valid;
  host_density_map(h->g, h->gd, d, dens, dmap, valid);
  const int64_t nvalid = (int64_t)valid.size();
  const int64_t n = (int64_t)std::floor(d.npart_per_cell * (double)nvalid);
  if (n > p.cap) return CYL_ERR_CAPACITY;
  cudaStream_t s = h->st;
  WAIT(wait_stream(h, s));
  // every copy below is on the handle's stream, so the kernels on it see
  // them (a cudaMemcpy from pageable memory may return before its DMA lands,
  // and it is not ordered with a non-blocking stream)
  SpeciesCounters c{n, 0, 0u, 0u};
  CK(cudaMemcpyAsync(h->d_cnt + isp, &c, sizeof(c), cudaMemcpyHostToDevice, s));
  if (n == 0) WAIT(copies_done(h, s));
  if (n > 0) {
    double* d_dens = nullptr;
    int8_t* d_dmap = nullptr;
    int32_t* d_valid = nullptr;
    int* d_npic = nullptr;
    const size_t cells = dens.size();
    auto release = [&]() {
      cudaFree(d_dens);
      cudaFree(d_dmap);
      cudaFree(d_valid);
      cudaFree(d_npic);
    };
    if (cudaMalloc(&d_dens, cells * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&d_dmap, cells) != cudaSuccess ||
        cudaMalloc(&d_valid, (size_t)nvalid * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&d_npic, cells * sizeof(int)) != cudaSuccess) {
      release();
      return CYL_ERR_OUT_OF_MEMORY;
    }
    std::vector<int8_t> dm(cells);
    for (size_t k = 0; k < cells; ++k) dm[k] = (int8_t)dmap[k];
    cudaError_t e = cudaMemcpyAsync(d_dens, dens.data(), cells * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_dmap, dm.data(), cells, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_valid, valid.data(), (size_t)nvalid * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_npic, 0, cells * sizeof(int), s);
    LoadParams P{};
    P.nx = h->g.nx;
    P.ny = h->g.ny;
    P.W = h->g.nx + 2 * NG;
    P.dx = h->g.dx;
    P.dy = h->g.dy;
    P.x_grid_min = h->g.x_grid_min;
    P.y_grid_min = h->g.y_grid_min;
    P.nppc = (int64_t)std::floor(d.npart_per_cell);
    P.nvalid = nvalid;
    P.n = n;
    P.id_base = id_base;
    P.seed = seed;
    P.species = isp;
    for (int k = 0; k < 3; ++k) {
      P.temp[k] = d.temp[k];
      P.drift[k] = d.drift[k];
    }
    P.mass = d.mass;
    // the FP64 form loads into the particle arrays, the mixed form into the
    // FP64 staging of cyl_upload_particles, converted on the device after
    LoadOut o;
    double* st = h->sc.tmp;
    const int64_t cap = h->sc.cap;
    if (h->prec == CYL_PREC_MIXED)
      o = LoadOut{st, st + cap, st + 2 * cap, st + 3 * cap, st + 4 * cap, st + 5 * cap, st + 6 * cap,
                  (int64_t*)(st + 7 * cap)};
    else
      o = LoadOut{p.x, p.y, p.z, p.px, p.py, p.pz, p.w, p.id};
    if (e == cudaSuccess) {
      launch_load_particles(s, P, d_valid, d_dens, d_dmap, d_npic, o, &h->d_cnt[isp].wmax_bits);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && h->prec == CYL_PREC_MIXED) {
      mixed_from_double(s, p, st, n, cap, h->xg0, h->rc);
      e = cudaGetLastError();
    }
    // the host buffers above and the temporaries stay alive until the
    // stream has used them
    const cudaError_t es = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = es;
    release();
    if (e != cudaSuccess) {
      h->last_cuda_error = e;
      return e == cudaErrorMemoryAllocation ? CYL_ERR_OUT_OF_MEMORY : CYL_ERR_CUDA;
    }
  }
  if (id_base + n > h->next_id) h->next_id = id_base + n;
  *n_out = n;
  return CYL_OK;
}

int cyl_counter_block(uint64_t seed, const uint32_t* ctr4, uint32_t* out4) {
  if (!ctr4 || !out4) return CYL_ERR_BAD_ARG;
  const U4 r = philox4x32_10(ctr4[0], ctr4[1], ctr4[2], ctr4[3], seed);
  for (int k = 0; k < 4; ++k) out4[k] = r.v[k];
  return CYL_OK;
}

int cyl_set_injection_stream(cyl_handle hh, int32_t mode, uint64_t seed) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (mode != CYL_RNG_KISS && mode != CYL_RNG_COUNTER) return CYL_ERR_BAD_ARG;
  if (mode == CYL_RNG_COUNTER && h->fns.inject) return CYL_ERR_UNSUPPORTED;
  if (mode == CYL_RNG_COUNTER && h->move_window) {
    const double shifts_max = std::floor(h->g.dt * std::fabs(h->window_v_x) / h->g.dx) + 1.0;
    if (shifts_max > (double)MAX_INJ_SHIFTS) return CYL_ERR_UNSUPPORTED;
  }
  if (mode == CYL_RNG_COUNTER && !h->d_injsp) {
    InjSpecies tab[MAX_SPECIES] = {};
    for (int s = 0; s < h->nsp; ++s) {
      const cyl_species_desc& d = h->sd[s];
      tab[s].nppc = (int64_t)std::floor(d.npart_per_cell);
      tab[s].frac = d.npart_per_cell - (double)tab[s].nppc;
      for (int k = 0; k < 3; ++k) {
        tab[s].temp[k] = d.temp[k];
        tab[s].drift[k] = d.drift[k];
      }
      tab[s].mass = d.mass;
    }
    WAIT(wait_stream(h, h->st));
    if (cudaMalloc(&h->d_injsp, sizeof(tab)) != cudaSuccess) return CYL_ERR_OUT_OF_MEMORY;
    if (cudaMalloc(&h->d_injrow, sizeof(int32_t) * (size_t)h->inj_cap) != cudaSuccess) {
      cudaFree(h->d_injsp);
      h->d_injsp = nullptr;
      return CYL_ERR_OUT_OF_MEMORY;
    }
    CK(cudaMemcpyAsync(h->d_injsp, tab, sizeof(tab), cudaMemcpyHostToDevice, h->st));
    WAIT(copies_done(h, h->st));
  }
  h->inj_counter = mode == CYL_RNG_COUNTER;
  h->inj_seed = seed;
  // the step's kernels change: a captured step graph is rebuilt
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  h->topo_epoch++;
  return CYL_OK;
}

int cyl_write_sdf(cyl_handle hh, const char* path, int32_t restart, const char* const* species_names) {
  if (!hh || !path) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (restart && !h->at_output) return CYL_ERR_BAD_ARG;
  if (species_names)
    for (int s = 0; s < h->nsp; ++s)
      if (!species_names[s] || !species_names[s][0]) return CYL_ERR_BAD_ARG;
  const int nf = restart ? CYL_NFIELDS : CYL_F_JTM + 1;
  std::vector<std::vector<double>> host((size_t)nf, std::vector<double>(h->fcount * 2));
  const double* arrays[CYL_NFIELDS] = {};
  for (int k = 0; k < nf; ++k) {
    if (int r = cyl_download_field(hh, k, host[(size_t)k].data())) return r;
    arrays[k] = host[(size_t)k].data();
  }
  cyl_sdf_desc d{};
  d.nx = h->g.nx;
  d.ny = h->g.ny;
  d.n_mode = h->rc.M;
  d.step = (int32_t)h->step;
  d.time = h->time;
  d.xb_min = h->g.xb_min;
  d.dx = h->g.dx;
  d.dy = h->g.dy;
  d.restart = restart ? 1 : 0;
  d.dt = h->g.dt;
  d.x_grid_min = h->g.x_grid_min;
  // a run loaded from a dump restarts its window at its first moving_window;
  // until then the loaded shift fraction is still the one to keep
  const bool started = h->window_started || (h->at_output == AT_OUTPUT_RESTART && h->restart_wsf);
  d.window_started = h->move_window && started ? 1 : 0;
  d.window_shift_fraction = h->wsf;
  // the live particles of every species, in device order
  const int nsp = species_names ? h->nsp : 0;
  std::vector<std::vector<double>> pd((size_t)nsp);
  std::vector<std::vector<int64_t>> pid((size_t)nsp);
  std::vector<cyl_sdf_species> sp((size_t)nsp);
  for (int s = 0; s < nsp; ++s) {
    int64_t n = 0;
    if (int r = cyl_download_particles(hh, s, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                       &n))
      return r;
    pd[(size_t)s].resize((size_t)n * 7 + 1);
    pid[(size_t)s].resize((size_t)n + 1);
    double* b = pd[(size_t)s].data();
    const size_t un = (size_t)n;
    if (int r = cyl_download_particles(hh, s, b, b + un, b + 2 * un, b + 3 * un, b + 4 * un, b + 5 * un, b + 6 * un,
                                       pid[(size_t)s].data(), &n))
      return r;
    cyl_sdf_species& e = sp[(size_t)s];
    e.name = species_names[s];
    e.n = n;
    e.x = b;
    e.y = b + un;
    e.z = b + 2 * un;
    e.px = b + 3 * un;
    e.py = b + 4 * un;
    e.pz = b + 5 * un;
    e.w = b + 6 * un;
    e.id = pid[(size_t)s].data();
  }
  return cyl_sdf_write(path, &d, arrays, sp.data(), nsp);
}

// restart_data (setup.F90:777-1569) and the restart branch of the start-up
// (epoch2d.F90:116-153) for this path's state.
int cyl_restart_sdf(cyl_handle hh, const char* path, const char* const* species_names) {
  if (!hh || !path) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->at_output || h->step != 0) return CYL_ERR_BAD_ARG;
  for (int s = 0; s < h->nsp; ++s) {
    int64_t n = 0;
    if (int r = cyl_download_particles(hh, s, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                       nullptr, &n))
      return r;
    if (n != 0) return CYL_ERR_BAD_ARG;
    if (species_names && (!species_names[s] || !species_names[s][0])) return CYL_ERR_BAD_ARG;
  }
  cyl_sdf_file f = nullptr;
  if (int r = cyl_sdf_open(path, &f)) return r;
  struct Closer {
    cyl_sdf_file f;
    ~Closer() { cyl_sdf_close(f); }
  } closer{f};
  cyl_sdf_info info;
  if (int r = cyl_sdf_get_info(f, &info)) return r;
  // setup.F90:811-830: a restart dump of this code, grid as the deck's
  if (!info.restart || std::strcmp(info.code_name, "Epoch2d") != 0) return CYL_ERR_BAD_ARG;
  if (info.nx != h->g.nx || info.ny != h->g.ny || info.n_mode != h->rc.M) return CYL_ERR_BAD_ARG;
  if (info.has_dt && info.dt > 0.0 && info.dt != h->g.dt) return CYL_ERR_BAD_ARG;
  if (info.step == 0) return CYL_ERR_UNSUPPORTED;
  // the mode arrays: zero, then the file's interiors (setup.F90:939-953, 1222-1390)
  std::vector<double> buf(h->fcount * 2);
  for (int k = 0; k < CYL_NFIELDS; ++k) {
    if (int r = cyl_sdf_read_field(f, k, buf.data())) return r;
    if (int r = cyl_upload_field(hh, k, buf.data())) return r;
  }
  // the particles of every named species (ids continue after the largest)
  for (int s = 0; species_names && s < h->nsp; ++s) {
    int64_t n = -1;
    if (int r = cyl_sdf_species_count(f, species_names[s], &n)) return r;
    if (n <= 0) continue;
    std::vector<double> v((size_t)n * 7);
    std::vector<int64_t> id((size_t)n);
    const size_t un = (size_t)n;
    double* b = v.data();
    int64_t got = n;
    if (int r = cyl_sdf_read_particles(f, species_names[s], b, b + un, b + 2 * un, b + 3 * un, b + 4 * un,
                                       b + 5 * un, b + 6 * un, id.data(), &got))
      return r;
    if (int r = cyl_upload_particles(hh, s, b, b + un, b + 2 * un, b + 3 * un, b + 4 * un, b + 5 * un, b + 6 * un,
                                     id.data(), got))
      return r;
  }
  // the grid: a window that has moved puts the first edge elsewhere; the
  // grid is then rebuilt from it and x_grid_min as a window shift builds it
  if (info.has_grid && info.grid_x0 != h->g.xb_min) {
    const int64_t shifts = (int64_t)std::llround((info.grid_x0 - h->g.xb_min) / h->g.dx);
    h->g.xb_min = info.grid_x0;
    h->g.x_grid_min = info.has_x_grid_min ? info.x_grid_min : h->g.xb_min + 0.5 * h->g.dx;
    h->g.x_min = h->g.xb_min + h->g.dx * 0.0;
    h->g.x_max = (h->g.xb_min + (double)(h->g.nx + 1 - 1) * h->g.dx) - h->g.dx * 0.0;
    h->g.setup_grid_x();
    h->n_shifts += shifts;
  }
  if (info.has_window_shift_fraction) h->wsf = info.window_shift_fraction;
  h->restart_wsf = info.has_window_shift_fraction != 0;
  h->from_restart = true;
  h->window_started = false;
  h->step = info.step;
  h->time = info.time;
  step_head_fields(h, h->out_rec);
  h->at_output = AT_OUTPUT_RESTART;
  WAIT(wait_stream(h, h->st));
  return CYL_OK;
}

int cyl_download_particles(cyl_handle hh, int32_t isp, double* x, double* y, double* z, double* px,
                           double* py, double* pz, double* w, int64_t* id, int64_t* n_inout) {
  if (!hh || !n_inout) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (isp < 0 || isp >= h->nsp) return CYL_ERR_BAD_ARG;
  WAIT(wait_stream(h, h->st));
  SpeciesCounters c;
  CK(cudaMemcpy(&c, h->d_cnt + isp, sizeof(c), cudaMemcpyDeviceToHost));
  const int64_t n = c.n_used;
  SpeciesPtrs& p = h->sp[isp];
  // the count alone: live = slots in use - removed holes (the counters the
  // push, the window and the sort keep)
  if (!x) {
    *n_inout = n - c.n_dead;
    return CYL_OK;
  }
  if (!y || !z || !px || !py || !pz || !w || !id) return CYL_ERR_BAD_ARG;
  if (c.n_dead == 0) {
    // no holes (as after every chunk's sort): straight into the caller's arrays
    if (*n_inout < n) return CYL_ERR_CAPACITY;
    double* dst[7] = {x, y, z, px, py, pz, w};
    const size_t b = (size_t)n * 8;
    if (h->prec == CYL_PREC_MIXED) {
      double* st = h->sc.tmp;
      const int64_t cap = h->sc.cap;
      mixed_to_double(h->st, p, st, n, cap, h->xg0, h->rc);
      for (int k = 0; k < 7 && n > 0; ++k)
        CK(cudaMemcpyAsync(dst[k], st + (size_t)k * cap, b, cudaMemcpyDeviceToHost, h->st));
      if (n > 0) CK(cudaMemcpyAsync(id, st + (size_t)7 * cap, b, cudaMemcpyDeviceToHost, h->st));
    } else {
      const double* srcs[7] = {p.x, p.y, p.z, p.px, p.py, p.pz, p.w};
      for (int k = 0; k < 7 && n > 0; ++k) CK(cudaMemcpyAsync(dst[k], srcs[k], b, cudaMemcpyDeviceToHost, h->st));
      if (n > 0) CK(cudaMemcpyAsync(id, p.id, b, cudaMemcpyDeviceToHost, h->st));
    }
    WAIT(copies_done(h, h->st));
    *n_inout = n;
    return CYL_OK;
  }
  std::unique_ptr<double[]> buf(new double[(size_t)n * 8]);
  if (h->prec == CYL_PREC_MIXED) {
    double* st = h->sc.tmp;
    const int64_t cap = h->sc.cap;
    mixed_to_double(h->st, p, st, n, cap, h->xg0, h->rc);
    for (int k = 0; k < 8; ++k)
      CK(cudaMemcpyAsync(buf.get() + (size_t)k * n, st + (size_t)k * cap, (size_t)n * 8, cudaMemcpyDeviceToHost,
                         h->st));
    WAIT(copies_done(h, h->st));
  } else {
    double* srcs[7] = {p.x, p.y, p.z, p.px, p.py, p.pz, p.w};
    for (int k = 0; k < 7; ++k)
      CK(cudaMemcpy(buf.get() + (size_t)k * n, srcs[k], (size_t)n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(buf.get() + (size_t)7 * n, p.id, (size_t)n * 8, cudaMemcpyDeviceToHost));
  }
  int64_t live = 0;
  for (int64_t i = 0; i < n; ++i)
    if (!std::isnan(buf[i])) live++;
  if (*n_inout < live) return CYL_ERR_CAPACITY;
  int64_t k = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (std::isnan(buf[i])) continue;
    x[k] = buf[i];
    y[k] = buf[n + i];
    z[k] = buf[2 * n + i];
    px[k] = buf[3 * n + i];
    py[k] = buf[4 * n + i];
    pz[k] = buf[5 * n + i];
    w[k] = buf[6 * n + i];
    std::memcpy(&id[k], &buf[7 * n + i], 8);
    ++k;
  }
  *n_inout = k;
  return CYL_OK;
}

// Mixed form: slot of an E / B / B_old array in the FP32 buffer, else -1.
static int f32_slot(const Handle* h, int which) {
  if (h->prec != CYL_PREC_MIXED) return -1;
  if (which >= 0 && which <= 5) return which;
  if (which >= 9 && which <= 11) return which - 3;
  return -1;
}

int cyl_upload_field(cyl_handle hh, int32_t which, const double* data) {
  if (!hh || !data || which < 0 || which >= CYL_NFIELDS) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  WAIT(wait_stream(h, h->st));
  const int fs = f32_slot(h, which);
  if (fs >= 0) {
    std::vector<float> tmp(h->fcount * 2);
    for (size_t i = 0; i < tmp.size(); ++i) tmp[i] = (float)data[i];
    // after the stream's earlier work on the array, before its later work
    CK(cudaMemcpyAsync(h->Ff[fs], tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice, h->st));
    WAIT(copies_done(h, h->st));
    return CYL_OK;
  }
  CK(cudaMemcpyAsync(h->F[field_slot(h, which)], data, h->fcount * sizeof(cplx), cudaMemcpyHostToDevice,
                     h->st));
  WAIT(copies_done(h, h->st));
  return CYL_OK;
}

int cyl_download_field(cyl_handle hh, int32_t which, double* data) {
  if (!hh || !data || which < 0 || which >= CYL_NFIELDS) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  WAIT(wait_stream(h, h->st));
  const int fs = f32_slot(h, which);
  if (fs >= 0) {
    const int64_t nval = (int64_t)h->fcount * 2;
    if (nval <= h->sc.cap * 7) {
      // widened on the device into the sort scratch, then one copy into the
      // caller's array (no host-side pass over the values)
      widen_f32(h->st, reinterpret_cast<const float*>(h->Ff[fs]), h->sc.tmp, nval);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(data, h->sc.tmp, (size_t)nval * sizeof(double), cudaMemcpyDeviceToHost, h->st));
      WAIT(copies_done(h, h->st));
      return CYL_OK;
    }
    std::vector<float> tmp(h->fcount * 2);
    CK(cudaMemcpy(tmp.data(), h->Ff[fs], tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < tmp.size(); ++i) data[i] = (double)tmp[i];
    return CYL_OK;
  }
  CK(cudaMemcpy(data, h->F[field_slot(h, which)], h->fcount * sizeof(cplx), cudaMemcpyDeviceToHost));
  return CYL_OK;
}

int cyl_initialise(cyl_handle hh) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->at_output) return CYL_ERR_BAD_ARG;
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  StepRec& r = h->h_rec[0];
  std::memset(&r, 0, sizeof(r));
  fill_grid(r, h->g, false);
  fill_grid(r, h->g, true);
  for (int i = 0; i < 4; ++i) {
    r.bc_field[i] = h->bc_field[i];
    r.add_laser[i] = h->add_laser[i];
    r.bc_field_after[i] = h->bc_field[i];
  }
  r.nshift_total = r.nshift_total_after = (int32_t)h->n_shifts;
  // epoch2d.F90:157-161: dt halved, time advanced by it, bfield_final_bcs
  const double dt_half = h->g.dt / 2.0;
  h->time = h->time + dt_half;
  r.time_final = h->time;
  h->cb_failed = false;
  laser_sources(h, h->h_src, dt_half);
  if (h->cb_failed) return CYL_ERR_CALLBACK;
  CK(cudaMemcpyAsync(h->d_rec, h->h_rec, sizeof(StepRec), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_src, h->h_src, sizeof(double) * h->src_per_step, cudaMemcpyHostToDevice, h->st));
  for (int i = 0; i < h->nsp; ++i) {
    if (h->prec == CYL_PREC_MIXED)
      mixed_particle_bcs(h->st, h->sp[i], h->d_cnt + i, h->d_rec, h->rc, h->nblocks);
    else
      launch_particle_bcs(h->st, h->sp[i], h->d_cnt + i, h->d_rec, 0, h->rc, h->nblocks);
  }
  if (h->prec == CYL_PREC_MIXED) {
    FieldSetF F = fieldset_f(h, h->jpar);
    launch_efield_bcs(h->st, F, h->d_rec, h->rc);
    launch_b_final_bcs(h->st, F, h->d_rec, h->d_src, h->cols, 0, dt_half, h->rc);
    enqueue_sort(h, h->d_rec);
  } else {
    FieldSet F = fieldset(h, h->jpar);
    launch_efield_bcs(h->st, F, h->d_rec, h->rc);
    launch_b_final_bcs(h->st, F, h->d_rec, h->d_src, h->cols, 0, dt_half, h->rc);
  }
  CK(cudaEventRecord(h->ev_copy, h->st));
  h->copy_pending = true;
  return sync_and_check(h);
}

// ---------------------------------------------------------------------------
// The output point inside a step (cyl_step_to_output) and the restart from a
// dump taken there (cyl_restart_sdf).

extern "C++" {
// A step's kernels up to the output point: update_eb_fields_half, the push,
// current_finish.
template <typename T>
static void enqueue_step_head(Handle* h, const StepRec* rec) {
  cudaStream_t s = h->st;
  const FieldSetT<T> F = enqueue_step_pre<T>(h, s, rec);
  push_all(h, s, F, rec, 1, 1);
  enqueue_current_finish<T>(h, s, F, rec);
}

// The rest of the step stopped at the output point.  After a restart dump
// was loaded, first the restart start-up of epoch2d.F90:143-153 (particle_bcs,
// efield_bcs, old_field_bcs), then update_eb_fields_final and moving_window,
// and the sort that ends every chunk.
template <typename T>
static void enqueue_finish(Handle* h, bool restart) {
  cudaStream_t s = h->st;
  const FieldSetT<T> F = fieldset_t<T>(h, h->jpar);
  if (restart) {
    for (int i = 0; i < h->nsp; ++i) {
      if (h->prec == CYL_PREC_MIXED)
        mixed_particle_bcs(s, h->sp[i], h->d_cnt + i, h->d_rec, h->rc, h->nblocks);
      else
        launch_particle_bcs(s, h->sp[i], h->d_cnt + i, h->d_rec, 0, h->rc, h->nblocks);
      count_launch(h, 1);
    }
    launch_efield_bcs(s, F, h->d_rec, h->rc);
    launch_old_field_bcs(s, F, h->d_rec, h->rc);
    count_launch(h, 2);
  }
  enqueue_step_final<T>(h, s, F, h->d_rec, h->d_src);
  enqueue_sort(h, h->d_rec);
}
}  // extern "C++"

static int finish_output(Handle* h) {
  if (h->at_output == AT_OUTPUT_NONE) return CYL_OK;
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  if (int r = flush_push_timing(h)) return r;
  const bool restart = h->at_output == AT_OUTPUT_RESTART;
  h->h_rec[0] = h->out_rec;
  int64_t inj_used = 0;
  h->cb_failed = false;
  step_tail(h, 0, inj_used);
  if (h->cb_failed) return CYL_ERR_CALLBACK;
  CK(cudaMemcpyAsync(h->d_rec, h->h_rec, sizeof(StepRec), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_src, h->h_src, sizeof(double) * h->src_per_step, cudaMemcpyHostToDevice, h->st));
  if (inj_used > 0 && !h->inj_counter)
    CK(cudaMemcpyAsync(h->d_inj, h->h_inj, sizeof(double) * 8 * inj_used, cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->ev_copy, h->st));
  h->copy_pending = true;
  h->at_output = AT_OUTPUT_NONE;
  (void)cudaGetLastError();
  if (h->prec == CYL_PREC_MIXED) enqueue_finish<cplxf>(h, restart);
  else enqueue_finish<cplx>(h, restart);
  CK(cudaGetLastError());
  return CYL_OK;
}

static int step_impl(cyl_handle hh, int32_t nsteps, bool graph, bool sync = true) {
  if (!hh || nsteps < 0) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (int r = finish_output(h)) return r;
  while (nsteps > 0) {
    const int k = nsteps < CHUNK ? nsteps : CHUNK;
    int r = run_chunk(h, k, graph);
    if (r != CYL_OK) return r;
    nsteps -= k;
  }
  if (!sync) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      h->last_cuda_error = e;
      return CYL_ERR_CUDA;
    }
    return CYL_OK;
  }
  return sync_and_check(h);
}

int cyl_step_to_output(cyl_handle hh, int32_t nsteps) {
  if (!hh || nsteps < 1) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (int r = step_impl(hh, nsteps - 1, true, false)) return r;
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  if (int r = flush_push_timing(h)) return r;
  StepRec& r = h->h_rec[0];
  step_head(h, r);
  h->out_rec = r;
  CK(cudaMemcpyAsync(h->d_rec, h->h_rec, sizeof(StepRec), cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->ev_copy, h->st));
  h->copy_pending = true;
  h->at_output = AT_OUTPUT_STEP;
  (void)cudaGetLastError();
  if (h->prec == CYL_PREC_MIXED) enqueue_step_head<cplxf>(h, h->d_rec);
  else enqueue_step_head<cplx>(h, h->d_rec);
  CK(cudaGetLastError());
  return sync_and_check(h);
}

int cyl_step(cyl_handle hh, int32_t nsteps) { return step_impl(hh, nsteps, false); }
int cyl_step_graph(cyl_handle hh, int32_t nsteps) { return step_impl(hh, nsteps, true); }
int cyl_step_async(cyl_handle hh, int32_t nsteps) { return step_impl(hh, nsteps, true, false); }

int cyl_push_only(cyl_handle hh) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (int r = finish_output(h)) return r;
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  if (int r = flush_push_timing(h)) return r;
  StepRec& r = h->h_rec[0];
  std::memset(&r, 0, sizeof(r));
  fill_grid(r, h->g, false);
  fill_grid(r, h->g, true);
  for (int i = 0; i < 4; ++i) r.bc_field[i] = r.bc_field_after[i] = h->bc_field[i];
  CK(cudaMemcpyAsync(h->d_rec, h->h_rec, sizeof(StepRec), cudaMemcpyHostToDevice, h->st));
  h->jpar ^= 1;
  FieldSet F = fieldset(h, h->jpar);
  const size_t bytes = h->fcount * sizeof(cplx);
  cudaMemsetAsync(F.jx.p, 0, bytes, h->st);
  cudaMemsetAsync(F.jr.p, 0, bytes, h->st);
  cudaMemsetAsync(F.jt.p, 0, bytes, h->st);
  CK(cudaEventRecord(h->ev_push[0][0], h->st));
  if (h->prec == CYL_PREC_MIXED) push_all(h, h->st, fieldset_f(h, h->jpar), h->d_rec, 0);
  else push_all(h, h->st, F, h->d_rec, 0);
  CK(cudaEventRecord(h->ev_push[0][1], h->st));
  WAIT(wait_event(h, h->ev_push[0][1]));
  collect_push_timing(h, 1);
  return sync_and_check(h);
}

int cyl_ionisation_constants(const cyl_ionisation_species* io, const cyl_species_desc* sp, int32_t n,
                             int32_t model, double laser_omega, double* out) {
  if (!io || !sp || !out || n < 1 || n > MAX_SPECIES) return CYL_ERR_BAD_ARG;
  for (int i = 0; i < n; ++i)
    if (io[i].ionise && (io[i].ionise_to < 0 || io[i].ionise_to >= n || io[i].release < -1 || io[i].release >= n))
      return CYL_ERR_BAD_ARG;
  IonSpecies c[MAX_SPECIES];
  ionisation_constants(io, sp, n, model, laser_omega, c);
  for (int i = 0; i < n; ++i) {
    const double v[CYL_ION_NCONST] = {c[i].released_mass_fraction, c[i].n_exp, c[i].adk_scaling,
                                      c[i].ionisation_constant, c[i].smallest_e_mag, c[i].bsi_constant,
                                      c[i].bsi_scaling, c[i].bsi_threshold, c[i].adk_maximum, c[i].adk_bsi_cap,
                                      c[i].keldysh, c[i].multi_constant, c[i].k_photons_energy,
                                      c[i].k_photons_exponent, c[i].adk_multiphoton_cap};
    for (int k = 0; k < CYL_ION_NCONST; ++k) out[i * CYL_ION_NCONST + k] = v[k];
  }
  return CYL_OK;
}

int cyl_set_ionisation(cyl_handle hh, const cyl_ionisation_species* io, int32_t n, int32_t model,
                       uint64_t seed) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (n == 0) {
    h->ion_on = false;
  } else {
    if (!io || n != h->nsp) return CYL_ERR_BAD_ARG;
    for (int i = 0; i < n; ++i)
      if (io[i].ionise && (io[i].ionise_to < 0 || io[i].ionise_to >= n || io[i].release < -1 ||
                           io[i].release >= n || io[i].energy <= 0.0))
        return CYL_ERR_BAD_ARG;
    double omega = 0.0;
    if (model & CYL_IONISE_MULTIPHOTON) {
      // one laser frequency on the x boundaries (ionise.F90:56-123)
      if (h->lasers.empty()) return CYL_ERR_UNSUPPORTED;
      omega = h->lasers[0].d.omega;
      for (const auto& L : h->lasers)
        if (std::fabs(L.d.omega - omega) > 2.2250738585072014e-308) return CYL_ERR_UNSUPPORTED;
    }
    IonParams P{};
    ionisation_constants(io, h->sd, n, model, omega, P.s);
    P.model = model;
    P.nsp = n;
    P.seed = seed;
    if (!h->d_ion) {
      if (cudaMalloc(&h->d_ion, sizeof(int64_t) * 2 * MAX_SPECIES) != cudaSuccess) return CYL_ERR_OUT_OF_MEMORY;
      int64_t caps[2 * MAX_SPECIES] = {};
      for (int i = 0; i < h->nsp; ++i) caps[MAX_SPECIES + i] = h->sp[i].cap;
      CK(cudaMemcpy(h->d_ion, caps, sizeof(caps), cudaMemcpyHostToDevice));
    }
    h->ion = P;
    h->ion_on = true;
  }
  // the step's kernels change: a captured step graph is rebuilt
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  h->topo_epoch++;
  return CYL_OK;
}

int cyl_set_merge_e_halves(cyl_handle hh, int32_t on) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  h->merge_e = on != 0;
  // the step's kernels change: a captured step graph is rebuilt
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  h->topo_epoch++;
  return CYL_OK;
}

int cyl_set_deck_fns(cyl_handle hh, const cyl_deck_fns* fns) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (!fns) {
    h->fns = cyl_deck_fns{};
    return CYL_OK;
  }
  const size_t nl = h->lasers.size();
  const uint32_t valid = nl >= 32 ? 0xffffffffu : ((1u << nl) - 1u);
  for (uint32_t m : {fns->omega_fn_mask, fns->profile_fn_mask, fns->phase_fn_mask})
    if (m & ~valid) return CYL_ERR_BAD_ARG;
  if ((fns->omega_fn_mask && !fns->laser_omega) || (fns->profile_fn_mask && !fns->laser_profile) ||
      (fns->phase_fn_mask && !fns->laser_phase))
    return CYL_ERR_BAD_ARG;
  if (fns->inject && h->inj_counter) return CYL_ERR_UNSUPPORTED;
  h->fns = *fns;
  return CYL_OK;
}

int cyl_eval_atan2(int64_t n, const double* y, const double* x, double* out) {
  if (n < 0 || (n > 0 && (!y || !x || !out))) return CYL_ERR_BAD_ARG;
  if (n == 0) return CYL_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CYL_ERR_NO_DEVICE;
  const size_t bytes = (size_t)n * sizeof(double);
  double* d = nullptr;
  if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) return CYL_ERR_OUT_OF_MEMORY;
  cudaError_t e = cudaMemcpy(d, y, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, x, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    launch_eval_atan2(0, d, d + n, d + 2 * n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * n, bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? CYL_OK : CYL_ERR_CUDA;
}

int cyl_get_stream(cyl_handle hh, void** stream_out) {
  if (!hh || !stream_out) return CYL_ERR_BAD_ARG;
  *stream_out = (void*)hh->h.st;
  return CYL_OK;
}

int cyl_kernel_timing(cyl_handle hh, double* push_ms_avg, int64_t* launches) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (push_ms_avg) *push_ms_avg = h->push_launches ? h->push_ms_sum / (double)h->push_launches : 0.0;
  if (launches) *launches = h->kernel_launches;
  h->push_ms_sum = 0.0;
  h->push_launches = 0;
  h->kernel_launches = 0;
  return CYL_OK;
}

int cyl_get_run_state(cyl_handle hh, cyl_run_state* out) {
  if (!hh || !out) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  WAIT(wait_stream(h, h->st));
  std::memset(out, 0, sizeof(*out));
  out->time = h->time;
  out->step = h->step;
  out->x_grid_min = h->g.x_grid_min;
  out->xb_min = h->g.xb_min;
  out->x_min = h->g.x_min;
  out->x_max = h->g.x_max;
  out->window_shift_fraction = h->wsf;
  out->window_started = h->window_started ? 1 : 0;
  for (int i = 0; i < 4; ++i) out->bc_field[i] = h->bc_field[i];
  SpeciesCounters c[MAX_SPECIES];
  CK(cudaMemcpy(c, h->d_cnt, sizeof(SpeciesCounters) * MAX_SPECIES, cudaMemcpyDeviceToHost));
  for (int i = 0; i < h->nsp && i < 8; ++i) out->n_live[i] = c[i].n_used - c[i].n_dead;
  out->n_shifts = h->n_shifts;
  return CYL_OK;
}

// The diagnostic reductions of the current state into d_red (8 doubles).
static void enqueue_diag_reductions(Handle* h) {
  cudaMemsetAsync(h->d_red, 0, 8 * sizeof(double), h->st);
  for (int i = 0; i < h->nsp; ++i) {
    if (h->prec == CYL_PREC_MIXED) mixed_energy(h->st, h->sp[i], h->d_cnt + i, h->d_red, h->nblocks);
    else launch_energy(h->st, h->sp[i], h->d_cnt + i, h->d_red, h->nblocks);
  }
  if (h->prec == CYL_PREC_MIXED) launch_field_energy(h->st, fieldset_f(h, h->jpar), h->rc, h->d_red + 2);
  else launch_field_energy(h->st, fieldset(h, h->jpar), h->rc, h->d_red + 2);
}

static void fill_diag(const double* red, int err, cyl_diag* out) {
  out->kinetic_energy = red[0];
  out->n_live = (int64_t)(red[1] + 0.5);
  out->field_energy_e = 0.5 * EPS0 * red[2];
  out->field_energy_b = 0.5 / (4.0e-7 * PI) * red[3];
  out->jsum_abs = red[4];
  out->device_error = err;
}

int cyl_diagnostics(cyl_handle hh, cyl_diag* out) {
  if (!hh || !out) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  WAIT(wait_stream(h, h->st));
  enqueue_diag_reductions(h);
  double red[8];
  CK(cudaMemcpyAsync(red, h->d_red, sizeof(red), cudaMemcpyDeviceToHost, h->st));
  WAIT(copies_done(h, h->st));
  int err = 0;
  CK(cudaMemcpy(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  fill_diag(red, err, out);
  return CYL_OK;
}

int cyl_diagnostics_async(cyl_handle hh) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->diag_count >= 2) return CYL_ERR_BAD_ARG;  // read one first
  Handle::DiagSlot& d = h->diag_slot[(h->diag_head + h->diag_count) % 2];
  if (!d.h) {
    CK(cudaMallocHost(&d.h, 9 * sizeof(double)));
    CK(cudaEventCreateWithFlags(&d.ev, cudaEventDisableTiming));
  }
  enqueue_diag_reductions(h);
  CK(cudaMemcpyAsync(d.h, h->d_red, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(d.h + 8, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaEventRecord(d.ev, h->st));
  d.pending = true;
  h->diag_count++;
  return CYL_OK;
}

int cyl_diagnostics_read(cyl_handle hh, cyl_diag* out) {
  if (!hh || !out) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->diag_count == 0) return CYL_ERR_BAD_ARG;
  Handle::DiagSlot& d = h->diag_slot[h->diag_head];
  WAIT(wait_event(h, d.ev));
  int err = 0;
  std::memcpy(&err, d.h + 8, sizeof(int));
  fill_diag(d.h, err, out);
  d.pending = false;
  h->diag_head = (h->diag_head + 1) % 2;
  h->diag_count--;
  return CYL_OK;
}

int cyl_debug_record(cyl_handle hh, float* out16) {
  if (!hh || !out16) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  WAIT(wait_stream(h, h->st));
  CK(cudaMemcpy(out16, h->d_dbg, 16 * sizeof(float), cudaMemcpyDeviceToHost));
  return CYL_OK;
}

int cyl_get_rng_state(cyl_handle hh, cyl_rng_state* out) {
  if (!hh || !out) return CYL_ERR_BAD_ARG;
  hh->h.rng.to_state(out);
  return CYL_OK;
}

int cyl_sort_particles(cyl_handle hh) {
  if (!hh) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  StepRec& r = h->h_rec[0];
  std::memset(&r, 0, sizeof(r));
  fill_grid(r, h->g, false);
  fill_grid(r, h->g, true);
  r.nshift_total = r.nshift_total_after = (int32_t)h->n_shifts;
  CK(cudaMemcpyAsync(h->d_rec + CHUNK, h->h_rec, sizeof(StepRec), cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->ev_copy, h->st));
  h->copy_pending = true;
  enqueue_sort(h, h->d_rec + CHUNK);
  return sync_and_check(h);
}

int cyl_number_density(cyl_handle hh, int32_t isp, double* out) {
  if (!hh || !out) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (isp >= h->nsp) return CYL_ERR_BAD_ARG;
  // the work array is free between steps
  cplx* dst = h->F[15];
  const FView v{dst, h->rc.nxg, h->rc.nyg};
  CK(cudaMemsetAsync(dst, 0, h->fcount * sizeof(cplx), h->st));
  for (int i = 0; i < h->nsp; ++i) {
    if (isp >= 0 && i != isp) continue;
    launch_number_density(h->st, h->sp[i], h->d_cnt + i, h->rc, h->g.x_grid_min, (int)h->n_shifts,
                          h->prec == CYL_PREC_MIXED, v, h->nblocks);
  }
  launch_number_density_bcs(h->st, v, h->rc, h->bc_field);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dst, h->fcount * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
  return sync_and_check(h);
}

int cyl_tile_shape(int32_t shape, int32_t* tx, int32_t* ty) {
  if (shape < 0 || shape >= N_TILE_SHAPES || !tx || !ty) return CYL_ERR_BAD_ARG;
  *tx = TILE_SHAPES[shape][0];
  *ty = TILE_SHAPES[shape][1];
  return CYL_OK;
}

// Use tile shape k for the mixed push from the next sort on; a captured step
// graph holds the old shape's launches and is rebuilt.
static void set_tile_shape(Handle* h, int k) {
  h->tile_shape = k;
  h->nblocks_mixed = h->nblocks_by_shape[k];
  h->topo_epoch++;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
}

// The step record of the current grid (no step in progress) at d_rec + CHUNK.
static int current_rec(Handle* h) {
  if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
  StepRec& r = h->h_rec[0];
  std::memset(&r, 0, sizeof(r));
  fill_grid(r, h->g, false);
  fill_grid(r, h->g, true);
  for (int i = 0; i < 4; ++i) r.bc_field[i] = r.bc_field_after[i] = h->bc_field[i];
  r.nshift_total = r.nshift_total_after = (int32_t)h->n_shifts;
  CK(cudaMemcpyAsync(h->d_rec + CHUNK, h->h_rec, sizeof(StepRec), cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->ev_copy, h->st));
  h->copy_pending = true;
  return CYL_OK;
}

int cyl_tune_tiles(cyl_handle hh, int32_t mode, int32_t* shape) {
  if (!hh || !shape) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (h->prec != CYL_PREC_MIXED) return CYL_ERR_UNSUPPORTED;
  if (int r = finish_output(h)) return r;
  if (mode == CYL_TUNE_SET) {
    if (*shape < 0 || *shape >= N_TILE_SHAPES) return CYL_ERR_BAD_ARG;
    set_tile_shape(h, *shape);
    return cyl_sort_particles(hh);
  }
  if (mode != CYL_TUNE_TIME) return CYL_ERR_BAD_ARG;
  if (int r = flush_push_timing(h)) return r;
  if (int r = current_rec(h)) return r;
  const StepRec* rec = h->d_rec + CHUNK;
  WAIT(wait_stream(h, h->st));
  // Copy of the state a push changes: the mixed particle words of every
  // species (kx, fx, fy, fz, ux, uy, uz, fw: bytes [0, 32 cap) of the species
  // buffer; id: bytes [56 cap, 64 cap)) and the counters.  The trial pushes
  // deposit into three scratch current arrays behind the copy.
  size_t bytes = 0;
  for (int i = 0; i < h->nsp; ++i) bytes += (size_t)h->sp[i].cap * 40;
  const size_t jbytes = h->fcount * sizeof(cplx);
  char* snap = nullptr;
  if (cudaMalloc(&snap, bytes + 3 * jbytes) != cudaSuccess) return CYL_ERR_OUT_OF_MEMORY;
  std::vector<SpeciesCounters> cnt0(MAX_SPECIES);
  int rcode = CYL_OK;
  auto run = [&](cudaError_t e) {
    if (e != cudaSuccess && rcode == CYL_OK) {
      h->last_cuda_error = e;
      rcode = CYL_ERR_CUDA;
    }
  };
  auto copy_state = [&](bool save) {
    size_t off = 0;
    for (int i = 0; i < h->nsp; ++i) {
      char* buf = reinterpret_cast<char*>(h->sp[i].x);
      const size_t cap = (size_t)h->sp[i].cap;
      char* a = save ? snap + off : buf;
      const char* b = save ? buf : snap + off;
      run(cudaMemcpyAsync(a, b, 32 * cap, cudaMemcpyDeviceToDevice, h->st));
      a = save ? snap + off + 32 * cap : buf + 56 * cap;
      b = save ? buf + 56 * cap : snap + off + 32 * cap;
      run(cudaMemcpyAsync(a, b, 8 * cap, cudaMemcpyDeviceToDevice, h->st));
      off += 40 * cap;
    }
    if (save)
      run(cudaMemcpyAsync(cnt0.data(), h->d_cnt, sizeof(SpeciesCounters) * MAX_SPECIES, cudaMemcpyDeviceToHost,
                          h->st));
    else
      run(cudaMemcpyAsync(h->d_cnt, cnt0.data(), sizeof(SpeciesCounters) * MAX_SPECIES, cudaMemcpyHostToDevice,
                          h->st));
    run(cudaStreamSynchronize(h->st));
  };
  copy_state(true);
  FieldSetF F = fieldset_f(h, h->jpar);
  cplx* jscr = reinterpret_cast<cplx*>(snap + bytes);
  F.jx.p = jscr;
  F.jr.p = jscr + h->fcount;
  F.jt.p = jscr + 2 * h->fcount;
  float best_ms[N_TILE_SHAPES];
  for (int k = 0; k < N_TILE_SHAPES; ++k) best_ms[k] = 1e30f;
  for (int rep = 0; rep < 2 && rcode == CYL_OK; ++rep) {
    for (int k = 0; k < N_TILE_SHAPES && rcode == CYL_OK; ++k) {
      copy_state(false);
      set_tile_shape(h, k);
      enqueue_sort(h, rec);
      run(cudaMemsetAsync(jscr, 0, 3 * jbytes, h->st));
      run(cudaEventRecord(h->ev_push[0][0], h->st));
      push_all(h, h->st, F, rec, 0);
      run(cudaEventRecord(h->ev_push[0][1], h->st));
      run(cudaEventSynchronize(h->ev_push[0][1]));
      float ms = 0.f;
      run(cudaEventElapsedTime(&ms, h->ev_push[0][0], h->ev_push[0][1]));
      if (ms < best_ms[k]) best_ms[k] = ms;
    }
  }
  int best = 0;
  for (int k = 1; k < N_TILE_SHAPES; ++k)
    if (best_ms[k] < best_ms[best]) best = k;
  copy_state(false);
  cudaFree(snap);
  set_tile_shape(h, best);
  if (rcode != CYL_OK) return rcode;
  enqueue_sort(h, rec);
  *shape = best;
  return sync_and_check(h);
}

int cyl_charge_density(cyl_handle hh, double* rho) {
  if (!hh || !rho) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  // the work array is free between steps
  cplx* dst = h->F[15];
  const FView v{dst, h->rc.nxg, h->rc.nyg};
  CK(cudaMemsetAsync(dst, 0, h->fcount * sizeof(cplx), h->st));
  for (int i = 0; i < h->nsp; ++i) {
    if (h->sp[i].immobile) continue;
    launch_charge_density(h->st, h->sp[i], h->d_cnt + i, h->geom.inv_volume, h->rc, h->g.x_grid_min,
                          (int)h->n_shifts, h->prec == CYL_PREC_MIXED, v, h->nblocks);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(rho, dst, h->fcount * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
  return sync_and_check(h);
}

// The body of cyl_cell_indices_noalloc, with the handle's device current.
static int cell_indices_noalloc(Handle* h, int32_t isp, int32_t* cx, int32_t* cy, int64_t* n_inout) {
  int32_t* sc = nullptr;
  if (int r = cell_scratch(h->device, &sc)) return r;
  WAIT(wait_stream(h, h->st));
  SpeciesCounters c;
  CK(cudaMemcpy(&c, h->d_cnt + isp, sizeof(c), cudaMemcpyDeviceToHost));
  const int64_t n = c.n_used;
  if (!cx) {
    *n_inout = n - c.n_dead;
    return CYL_OK;
  }
  if (n > CYL_NOALLOC_MAX_PARTICLES) return CYL_ERR_SCRATCH;
  if (n == 0) {
    *n_inout = 0;
    return CYL_OK;
  }
  const int64_t N = CYL_NOALLOC_MAX_PARTICLES;
  if (h->prec == CYL_PREC_MIXED)
    mixed_cell_indices(h->st, h->sp[isp], h->d_cnt + isp, h->xg0, h->g.x_grid_min, h->rc, sc, sc + N, sc + 2 * N,
                       h->nblocks);
  else
    launch_cell_indices(h->st, h->sp[isp], h->d_cnt + isp, h->g.x_grid_min, h->rc, sc, sc + N, sc + 2 * N,
                        h->nblocks);
  k_compact_cells<<<1, 1024, 0, h->st>>>(sc, sc + N, sc + 2 * N, n, sc + 3 * N, sc + 4 * N, sc + 5 * N);
  CK(cudaGetLastError());
  int32_t k = 0;
  CK(cudaMemcpyAsync(&k, sc + 5 * N, sizeof(int32_t), cudaMemcpyDeviceToHost, h->st));
  WAIT(copies_done(h, h->st));
  if (k > *n_inout) return CYL_ERR_CAPACITY;
  if (k > 0) {
    CK(cudaMemcpyAsync(cx, sc + 3 * N, (size_t)k * sizeof(int32_t), cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(cy, sc + 4 * N, (size_t)k * sizeof(int32_t), cudaMemcpyDeviceToHost, h->st));
    WAIT(copies_done(h, h->st));
  }
  *n_inout = k;
  return CYL_OK;
}

int cyl_cell_indices_noalloc(cyl_handle hh, int32_t isp, int32_t* cx, int32_t* cy, int64_t* n_inout) {
  if (!hh || !n_inout || (!cx) != (!cy)) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (isp < 0 || isp >= h->nsp) return CYL_ERR_BAD_ARG;
  // the scratch address and the launches belong to the handle's device,
  // whatever device the caller has current; the caller's is restored
  int prev = 0;
  CK(cudaGetDevice(&prev));
  if (prev != h->device) CK(cudaSetDevice(h->device));
  const int r = cell_indices_noalloc(h, isp, cx, cy, n_inout);
  if (prev != h->device && cudaSetDevice(prev) != cudaSuccess && r == CYL_OK) return CYL_ERR_CUDA;
  return r;
}

int cyl_cell_indices(cyl_handle hh, int32_t isp, int32_t* cx, int32_t* cy, int64_t* n_inout) {
  if (!hh || !n_inout || (!cx) != (!cy)) return CYL_ERR_BAD_ARG;
  Handle* h = &hh->h;
  if (isp < 0 || isp >= h->nsp) return CYL_ERR_BAD_ARG;
  WAIT(wait_stream(h, h->st));
  SpeciesCounters c;
  CK(cudaMemcpy(&c, h->d_cnt + isp, sizeof(c), cudaMemcpyDeviceToHost));
  const int64_t n = c.n_used;
  if (!cx) {
    *n_inout = n - c.n_dead;
    return CYL_OK;
  }
  int32_t* d = nullptr;
  CK(cudaMalloc(&d, (size_t)n * 12 + 16));
  if (h->prec == CYL_PREC_MIXED)
    mixed_cell_indices(h->st, h->sp[isp], h->d_cnt + isp, h->xg0, h->g.x_grid_min, h->rc, d, d + n, d + 2 * n,
                       h->nblocks);
  else
    launch_cell_indices(h->st, h->sp[isp], h->d_cnt + isp, h->g.x_grid_min, h->rc, d, d + n, d + 2 * n,
                        h->nblocks);
  std::vector<int32_t> b((size_t)n * 3);
  cudaError_t e = cudaMemcpyAsync(b.data(), d, (size_t)n * 12, cudaMemcpyDeviceToHost, h->st);
  cudaStreamSynchronize(h->st);
  cudaFree(d);
  if (e != cudaSuccess) return CYL_ERR_CUDA;
  int64_t k = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!b[2 * n + i]) continue;
    if (k >= *n_inout) return CYL_ERR_CAPACITY;
    cx[k] = b[i];
    cy[k] = b[n + i];
    ++k;
  }
  *n_inout = k;
  return CYL_OK;
}

int cyl_batch_create(int32_t max_runs, cyl_batch* out) {
  if (!out || max_runs < 1 || max_runs > 1024) return CYL_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CYL_ERR_NO_DEVICE;
  auto* b = new cyl_batch_s();
  cudaError_t e = cudaGetDevice(&b->device);
  b->cap_runs = max_runs;
  b->cap_jobs = max_runs * MAX_SPECIES;
  auto ok = [&e](cudaError_t r) {
    if (r != cudaSuccess && e == cudaSuccess) e = r;
  };
  ok(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
  for (cudaEvent_t* ev : {&b->ev_sched, &b->ev_push, &b->ev_done, &b->ev_jobs})
    ok(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  b->ev_run.assign((size_t)max_runs, nullptr);
  for (auto& ev : b->ev_run) ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  const size_t tab = sizeof(BatchJob) * (size_t)CHUNK * b->cap_jobs;
  ok(cudaMallocHost(&b->h_jobs, tab));
  ok(cudaMalloc(&b->d_jobs, tab));
  const size_t stab = sizeof(StageJob) * (size_t)CHUNK * b->cap_runs;
  ok(cudaMallocHost(&b->h_stage, stab));
  ok(cudaMalloc(&b->d_stage, stab));
  const size_t wtab = sizeof(WindowJob) * (size_t)CHUNK * b->cap_jobs;
  ok(cudaMallocHost(&b->h_win, wtab));
  ok(cudaMalloc(&b->d_win, wtab));
  ok(cudaMalloc(&b->d_nwork, sizeof(int)));
  const int hw = (int)std::thread::hardware_concurrency();
  b->pool.reset(new HostPool(std::max(0, std::min({max_runs - 1, hw / 2, 8}))));
  if (e != cudaSuccess) {
    cyl_batch_destroy(b);
    return e == cudaErrorMemoryAllocation ? CYL_ERR_OUT_OF_MEMORY : CYL_ERR_CUDA;
  }
  *out = b;
  return CYL_OK;
}

int cyl_batch_step(cyl_batch b, const cyl_handle* hs, int32_t n, int32_t nsteps) {
  if (!b || !hs || n < 1 || n > b->cap_runs || nsteps < 0) return CYL_ERR_BAD_ARG;
  std::vector<Handle*> runs;
  std::vector<JobRef> jobs;
  int M = -1;
  int64_t need = 0;
  for (int r = 0; r < n; ++r) {
    if (!hs[r]) return CYL_ERR_BAD_ARG;
    Handle* h = &hs[r]->h;
    if (h->prec != CYL_PREC_MIXED) return CYL_ERR_UNSUPPORTED;
    if (h->ion_on) return CYL_ERR_UNSUPPORTED;  // the batched stages have no ionisation
    if (h->device != b->device) return CYL_ERR_BAD_ARG;
    if (M < 0) M = h->rc.M;
    if (h->rc.M != M) return CYL_ERR_UNSUPPORTED;
    for (Handle* q : runs)
      if (q == h) return CYL_ERR_BAD_ARG;
    runs.push_back(h);
    for (int i = 0; i < h->nsp; ++i)
      if (!h->sp[i].immobile) {
        jobs.push_back({h, i});
        need += h->ntiles_max;
      }
  }
  const int nj = (int)jobs.size();
  if (nj > b->cap_jobs) return CYL_ERR_BAD_ARG;
  // a run stopped at the output point finishes its step on its own stream
  for (Handle* h : runs)
    if (h->at_output != AT_OUTPUT_NONE) {
      if (int rc = finish_output(h)) return rc;
      WAIT(wait_stream(h, h->st));
    }
  // every run on the batch kernel's tile shape (shape 0), sorted for it
  for (int r = 0; r < n; ++r)
    if (runs[r]->tile_shape != 0) {
      int32_t shape = 0;
      if (int rc = cyl_tune_tiles(hs[r], CYL_TUNE_SET, &shape)) return rc;
    }
  if (need > b->work_cap) {
    cudaStreamSynchronize(b->st);
    cudaFree(b->d_work);
    b->d_work = nullptr;
    if (cudaMalloc(&b->d_work, sizeof(int2) * (size_t)need) != cudaSuccess) return CYL_ERR_OUT_OF_MEMORY;
    b->work_cap = need;
    if (b->gexec) {
      cudaGraphExecDestroy(b->gexec);
      b->gexec = nullptr;
    }
  }
  int32_t done = 0;
  while (done < nsteps) {
    const int k = nsteps - done < CHUNK ? nsteps - done : CHUNK;
    // the waits of the chunk come first, so that a wait that runs out
    // returns before any run's host state has moved: every run's staging
    // buffers and push events of the previous chunk, and the job table
    for (Handle* h : runs) {
      if (h->copy_pending) WAIT(wait_event(h, h->ev_copy));
      if (int rc = flush_push_timing(h)) return rc;
    }
    if (b->jobs_pending) {
      cudaError_t e = cudaSuccess;
      if (int rc = poll_device([b] { return cudaEventQuery(b->ev_jobs); }, &e)) return rc;
    }
    // each run's step records and host inputs (as run_chunk), copied on its
    // stream; runs share no host state, so the pool prepares them in parallel
    std::vector<int> prep_err(runs.size(), CYL_OK);
    b->pool->run((int)runs.size(), [&](int r) {
      Handle* h = runs[(size_t)r];
      cudaSetDevice(h->device);
      int64_t inj_used = 0;
      h->cb_failed = false;
      for (int i = 0; i < k; ++i) prepare_step(h, i, inj_used);
      if (h->cb_failed) {
        prep_err[(size_t)r] = CYL_ERR_CALLBACK;
        return;
      }
      cudaError_t e = cudaMemcpyAsync(h->d_rec, h->h_rec, sizeof(StepRec) * k, cudaMemcpyHostToDevice, h->st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_src, h->h_src, sizeof(double) * h->src_per_step * k, cudaMemcpyHostToDevice,
                            h->st);
      if (e == cudaSuccess && inj_used > 0 && !h->inj_counter)
        e = cudaMemcpyAsync(h->d_inj, h->h_inj, sizeof(double) * 8 * inj_used, cudaMemcpyHostToDevice, h->st);
      if (e == cudaSuccess) e = cudaEventRecord(h->ev_copy, h->st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, h->ev_copy, 0);
      if (e != cudaSuccess) {
        prep_err[(size_t)r] = CYL_ERR_CUDA;
        return;
      }
      h->copy_pending = true;
      h->timing_pending = 0;
    });
    for (int rc : prep_err)
      if (rc != CYL_OK) return rc;
    // the job table of the chunk: per step, the fields of the J parity after
    // that step's swap
    std::vector<int> par0(runs.size());
    for (size_t r = 0; r < runs.size(); ++r) par0[r] = runs[r]->jpar;
    // the stage table (per step, one row per run) and the window's
    // (run, species) table
    int nwin = 0;
    for (int i = 0; i < k; ++i) {
      int w = 0;
      for (size_t r = 0; r < runs.size(); ++r) {
        Handle* h = runs[r];
        StageJob& S = b->h_stage[(size_t)i * b->cap_runs + r];
        S.F0 = fieldset_f(h, par0[r] ^ (i & 1));
        S.F1 = fieldset_f(h, par0[r] ^ ((i + 1) & 1));
        S.rec = h->d_rec + i;
        S.src = h->d_src + h->src_per_step * i;
        S.cols = h->cols;
        S.rowtab = reinterpret_cast<const float4*>(h->rowtab);
        S.rc = h->rc;
        stage_job_bc_consts(S);
        stage_job_yee_consts(S);
        if (!h->move_window) continue;
        for (int isp = 0; isp < h->nsp; ++isp) {
          WindowJob& W = b->h_win[(size_t)i * b->cap_jobs + w++];
          W.sp = h->sp[isp];
          W.cnt = h->d_cnt + isp;
          W.inject = h->d_inj;
          W.rec = h->d_rec + i;
          W.P = h->mp[isp];
          W.rc = h->rc;
          W.xg0 = h->xg0;
          W.isp = isp;
          W.err = h->d_err;
        }
      }
      nwin = w;
    }
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < nj; ++j) {
        Handle* h = jobs[j].h;
        const int isp = jobs[j].isp;
        BatchJob& J = b->h_jobs[(size_t)i * b->cap_jobs + j];
        J.F = fieldset_f(h, h->jpar ^ ((i + 1) & 1));
        J.sp = h->sp[isp];
        J.cnt = h->d_cnt + isp;
        J.rec = h->d_rec + i;
        J.rc = h->rc;
        J.P = h->mp[isp];
        J.tt = h->d_tiles + isp;
        J.apply_bcs = 1;
      }
    if (cudaMemcpyAsync(b->d_jobs, b->h_jobs, sizeof(BatchJob) * (size_t)k * b->cap_jobs, cudaMemcpyHostToDevice,
                        b->st) != cudaSuccess ||
        cudaMemcpyAsync(b->d_stage, b->h_stage, sizeof(StageJob) * (size_t)k * b->cap_runs,
                        cudaMemcpyHostToDevice, b->st) != cudaSuccess ||
        (nwin > 0 && cudaMemcpyAsync(b->d_win, b->h_win, sizeof(WindowJob) * (size_t)k * b->cap_jobs,
                                     cudaMemcpyHostToDevice, b->st) != cudaSuccess) ||
        cudaEventRecord(b->ev_jobs, b->st) != cudaSuccess)
      return CYL_ERR_CUDA;
    b->jobs_pending = true;
    if (k == CHUNK) {
      std::vector<uint64_t> serials(2 * runs.size());
      for (size_t r = 0; r < runs.size(); ++r) {
        serials[2 * r] = runs[r]->serial;
        serials[2 * r + 1] = runs[r]->topo_epoch;
      }
      const bool same = b->gexec && b->g_runs == serials && b->g_par == par0 && b->g_jobs == nj;
      if (!same) {
        // capture the chunk for the new membership; when its graph has the
        // old one's shape (a run replaced by one of the same kind), update
        // the executable graph in place instead of instantiating a new one
        // (an update does not touch launches still in flight)
        cudaGraph_t graph;
        auto drop_exec = [b]() {
          if (b->gexec) cudaGraphExecDestroy(b->gexec);
          b->gexec = nullptr;
        };
        if (cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
          drop_exec();
          return CYL_ERR_CUDA;
        }
        enqueue_batch_chunk(b, runs, nj, nwin, k, M, par0);
        if (cudaStreamEndCapture(b->st, &graph) != cudaSuccess) {
          drop_exec();
          return CYL_ERR_CUDA;
        }
        bool updated = false;
        if (b->gexec) {
          cudaGraphExecUpdateResultInfo info;
          updated = cudaGraphExecUpdate(b->gexec, graph, &info) == cudaSuccess;
          if (!updated) {
            (void)cudaGetLastError();
            drop_exec();
          }
        }
        cudaError_t e = cudaSuccess;
        if (!updated) e = cudaGraphInstantiate(&b->gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
          b->gexec = nullptr;
          return CYL_ERR_CUDA;
        }
        b->g_runs = serials;
        b->g_par = par0;
        b->g_jobs = nj;
        // the capture advanced each run's J parity by k (even): unchanged
      } else {
        for (Handle* h : runs) h->jpar ^= (k & 1);
      }
      if (cudaGraphLaunch(b->gexec, b->st) != cudaSuccess) return CYL_ERR_CUDA;
    } else {
      (void)cudaGetLastError();
      enqueue_batch_chunk(b, runs, nj, nwin, k, M, par0);
      if (cudaGetLastError() != cudaSuccess) return CYL_ERR_CUDA;
    }
    // each run's later work (its next copies, reads) comes after the chunk
    if (cudaEventRecord(b->ev_done, b->st) != cudaSuccess) return CYL_ERR_CUDA;
    for (Handle* h : runs)
      if (cudaStreamWaitEvent(h->st, b->ev_done, 0) != cudaSuccess) return CYL_ERR_CUDA;
    done += k;
  }
  {
    cudaError_t e = cudaSuccess;
    if (int rc = poll_device([b] { return cudaStreamQuery(b->st); }, &e)) return rc;
  }
  for (Handle* h : runs)
    if (int r = sync_and_check(h)) return r;
  return CYL_OK;
}

int cyl_batch_destroy(cyl_batch b) {
  if (!b) return CYL_ERR_BAD_ARG;
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  cudaFreeHost(b->h_jobs);
  cudaFree(b->d_jobs);
  cudaFreeHost(b->h_stage);
  cudaFree(b->d_stage);
  cudaFreeHost(b->h_win);
  cudaFree(b->d_win);
  cudaFree(b->d_work);
  cudaFree(b->d_nwork);
  for (cudaEvent_t ev : {b->ev_sched, b->ev_push, b->ev_done, b->ev_jobs})
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : b->ev_run)
    if (ev) cudaEventDestroy(ev);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return CYL_OK;
}

}  // extern "C"
