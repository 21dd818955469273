/*
 * cylpic.h -- C ABI of the GB300 quasi-3D (x, r, theta-mode) PIC step.
 *
 * This is the drop-in boundary for the hot path of cylindrical EPOCH
 * (epoch_axial).  In the reference the path is a set of argument-less Fortran
 * module subroutines acting on module globals, called from the driver loop
 * (epoch_axial/src/epoch2d.F90:213-265):
 *
 *   update_eb_fields_half  (epoch_axial/src/fields.f90:316)
 *   push_particles         (epoch_axial/src/particles.F90:28)
 *   current_finish         (epoch_axial/src/housekeeping/current_smooth.F90:29)
 *   update_eb_fields_final (epoch_axial/src/fields.f90:341)
 *   moving_window          (epoch_axial/src/housekeeping/window.F90:330)
 *
 * Here the state those routines share (complex mode fields, particle lists,
 * window position, laser phases) is owned by an opaque handle that lives on
 * one GPU.  Every entry point returns an int status: CYL_OK (0) or one of the
 * CYL_ERR_* codes.  Host arrays are caller-owned and are only read or written
 * during the call; no pointer is retained.  One handle per host thread.
 *
 * Units are SI throughout, exactly as in the reference.  Field arrays are
 * complex FP64 in the reference's Fortran layout
 *   F(1-ng:nx+ng, 1-ng:ny+ng, 0:n_mode-1),  ng = 5  (constants.F90:535-545)
 * i.e. x fastest, interleaved (re, im) pairs, so a Fortran caller can pass
 * C_LOC(exm) directly.
 */
#ifndef CYLPIC_H
#define CYLPIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Ghost width of every mode array (triangle shape: png=3, ng=png+2,
 * jng=MAX(ng,png); constants.F90:535-545). */
#define CYL_NG 5

/* ---- status codes (the reference aborts through abort_code(errcode),
 *      utilities.f90:261; codes constants.F90:94-130) ---------------------- */
#define CYL_OK 0
#define CYL_ERR_BAD_ARG 1        /* null pointer, size out of range          */
#define CYL_ERR_CUDA 2           /* a CUDA runtime call failed               */
#define CYL_ERR_NO_DEVICE 3      /* no CUDA device visible                   */
#define CYL_ERR_CAPACITY 4       /* particle capacity of a species exceeded  */
#define CYL_ERR_UNSUPPORTED 5    /* option outside the implemented subset    */
#define CYL_ERR_DEVICE_FLAG 6    /* a kernel raised its device error word    */
#define CYL_ERR_TIMEOUT 7        /* a bounded host wait on the GPU ran out   */
#define CYL_ERR_OUT_OF_MEMORY 8  /* device allocation failed                 */
#define CYL_ERR_SCRATCH 9        /* input larger than a fixed scratch buffer */
#define CYL_ERR_IO 10            /* a file could not be written              */
#define CYL_ERR_CALLBACK 11      /* a deck-expression callback returned an error */

/* ---- boundary codes: the values of constants.F90:56-72 ------------------- */
#define CYL_BC_PERIODIC 1
#define CYL_BC_OTHER 2
#define CYL_BC_SIMPLE_LASER 3
#define CYL_BC_SIMPLE_OUTFLOW 4
#define CYL_BC_OPEN 5
#define CYL_BC_ZERO_GRADIENT 7
#define CYL_BC_CLAMP 8
#define CYL_BC_REFLECT 9
#define CYL_BC_CONDUCT 10
#define CYL_BC_ZERO_B 16

/* Index of a boundary in the bc arrays below.  The reference numbers them
 * c_bd_x_min=1 .. c_bd_y_max=4 (constants.F90:81-84); here they are 0-based. */
#define CYL_BD_X_MIN 0
#define CYL_BD_X_MAX 1
#define CYL_BD_Y_MIN 2
#define CYL_BD_Y_MAX 3

/* Arithmetic form of the step. */
#define CYL_PREC_FP64 0   /* plain form: FP64 everywhere, no FMA contraction */
#define CYL_PREC_MIXED 1  /* int cell + FP32 offset, FP32 push/deposit      */

/* Field array selectors for cyl_upload_field / cyl_download_field.  The
 * order follows the module globals of shared_data.F90:474-478. */
#define CYL_F_EXM 0
#define CYL_F_ERM 1
#define CYL_F_ETM 2
#define CYL_F_BXM 3
#define CYL_F_BRM 4
#define CYL_F_BTM 5
#define CYL_F_JXM 6
#define CYL_F_JRM 7
#define CYL_F_JTM 8
#define CYL_F_BXM_OLD 9
#define CYL_F_BRM_OLD 10
#define CYL_F_BTM_OLD 11
#define CYL_F_JXM_OLD 12
#define CYL_F_JRM_OLD 13
#define CYL_F_JTM_OLD 14
#define CYL_NFIELDS 15

/* Grid, boundaries and moving window.  Mirrors the control, boundaries and
 * window deck blocks (deck_control_block.F90:236-476, window block
 * deck_window_block.f90) after the deck has been evaluated by the host. */
typedef struct cyl_grid_desc {
  int32_t nx, ny;          /* cells along x (axis) and r                    */
  int32_t n_mode;          /* azimuthal modes m = 0 .. n_mode-1             */
  int32_t precision;       /* CYL_PREC_*                                     */
  double x_min, x_max;     /* axial extent (m); cell-centred grid, setup.F90:164-206 */
  double y_max;            /* radial extent (m); y_min = 0 is forced (deck_control_block.F90:74-75) */
  double dt;               /* time step (s), as set_dt (setup.F90:629-670) computes it */
  int32_t bc_field[4];     /* deck field bcs, before setup_boundaries mapping */
  int32_t move_window;     /* window block: move_window                      */
  double window_v_x;       /* window speed (m/s)                             */
  double window_start_time, window_stop_time;
  int32_t bc_after_move[4];/* bc_*_after_move (deck_window_block.f90:48-55)   */
  int32_t smooth_currents; /* current_smooth.F90:37 (0 = off, the default)   */
  int32_t smooth_its, smooth_comp_its, smooth_stride;
} cyl_grid_desc;

/* Particle species (deck species block).  The density/temperature profile
 * is what insert_particles (window.F90:157-300) evaluates at the x_max
 * column when the window moves; density_kind 0 is uniform, 1 a linear
 * up-ramp n(x) = density * clamp((x - ramp_x0) / ramp_length, 0, 1). */
typedef struct cyl_species_desc {
  double charge, mass;      /* SI: C, kg                                      */
  int32_t immobile;
  int32_t bc_particle[4];   /* deck particle bcs                              */
  int64_t capacity;         /* device particle capacity (>= live count)       */
  double npart_per_cell;
  int32_t density_kind;
  double density, ramp_x0, ramp_length;
  double density_min, density_max;  /* defaults EPSILON(1.0), HUGE (helper.F90:184-185) */
  double temp[3];           /* temperature per direction (K)                   */
  double drift[3];          /* momentum drift per direction (kg m/s)           */
} cyl_species_desc;

/* A laser on an x boundary (laser deck block, deck_laser_block.f90:90-260).
 * The transverse profile and phase are the host-evaluated deck expressions
 * at y(ir), ir = 0..ny (laser.f90:230-253).  The time envelope is either
 * constant (t_profile 0) or gauss(time, t0, tw) = exp(-((time-t0)/tw)^2)
 * (evaluator_blocks.F90:988-992), evaluated on the device every step. */
typedef struct cyl_laser_desc {
  int32_t boundary;          /* CYL_BD_X_MIN or CYL_BD_X_MAX                */
  int32_t t_profile;         /* 0 = constant, 1 = gauss                     */
  double amp, omega, pol_angle, t_start, t_end;
  double t0, tw;
  const double* profile;     /* ny+1 values                                 */
  const double* phase;       /* ny+1 values                                 */
} cyl_laser_desc;

/* State of the reference's global KISS generator (random_generator.f90:28-33),
 * carried across the host loader, the handle and the window injector. */
typedef struct cyl_rng_state {
  int32_t x, y, z, w;
  int32_t box_muller_cached;
  double cached_random_value;
} cyl_rng_state;

/* Scalars of a run that the Fortran module globals hold. */
typedef struct cyl_run_state {
  double time;
  int64_t step;
  double x_grid_min, xb_min, x_min, x_max;   /* moving window bookkeeping   */
  double window_shift_fraction;
  int32_t window_started;
  int32_t bc_field[4];                       /* current, after mapping       */
  int64_t n_live[8];                         /* live particles per species   */
  int64_t n_shifts;                          /* window shifts so far         */
} cyl_run_state;

/* Diagnostics of the current state (calc_df.F90:1225-1321 for the kinetic
 * energy; the field energy is the per-mode form of the cylindrical grid). */
typedef struct cyl_diag {
  double kinetic_energy;       /* sum w m c^2 (gamma-1), FP64               */
  double field_energy_e;       /* sum over cells and modes of the E energy   */
  double field_energy_b;
  double jsum_abs;             /* sum |J| over interior (sanity)             */
  int64_t n_live;
  int32_t device_error;        /* device error word (0 = none)               */
} cyl_diag;

typedef struct cyl_handle_s* cyl_handle;

/* ---- lifetime --------------------------------------------------------- */

/* Allocate the device state of one run.  Replaces the allocation in
 * mpi_initialise (mpi_routines.F90:385-400) and setup_boundaries
 * (boundary.F90:30-75) for one GPU.  rng is the state of the global KISS
 * generator after loading (it continues into window injection). */
int cyl_create(const cyl_grid_desc* grid, const cyl_species_desc* species,
               int32_t nspecies, const cyl_laser_desc* lasers, int32_t nlasers,
               const cyl_rng_state* rng, cyl_handle* out);
int cyl_destroy(cyl_handle h);

/* Limit of every host wait of the library on a run's device work (stepping,
 * state, field and particle reads, diagnostics, batches), in seconds;
 * seconds <= 0 removes the limit.  Process-wide, 600 s unless set.  A wait
 * that runs out returns CYL_ERR_TIMEOUT before the run's host state moves:
 * the queued work continues, and a later call waits for it again.  Copies
 * into or out of caller memory are queued only after the run's earlier work
 * is done, and their own end is always waited for.  The reference has no
 * equivalent (its MPI waits are unbounded). */
int cyl_set_wait_timeout(double seconds);

/* Upload one species' particles (SoA host arrays of length n: Cartesian
 * position x, y, z (m), momentum px, py, pz (kg m/s), weight, id).  The
 * Fortran side packs these from its list (shared_data.F90:93-142). */
int cyl_upload_particles(cyl_handle h, int32_t ispecies, const double* x,
                         const double* y, const double* z, const double* px,
                         const double* py, const double* pz, const double* w,
                         const int64_t* id, int64_t n);
/* ---- SDF output of the mode fields ---------------------------------------
 * The reference's field dump of the mode arrays (write_mode_field,
 * diagnostics.F90:2033-2110, and the "grid" mesh, 870-882) in SDF, the
 * reference's file format (SDF/FORTRAN sdf_output_*.f90): per mode array
 * the blocks "<id>_real" and "<id>_imag", real8 (nx, ny, n_mode) on mesh id
 * "mode_grid" with the reference's names, units and staggers; the rows of
 * Ex, Etheta, Br, Jx, Jtheta shifted up by one so that row 1 holds the axis
 * row 0, as the reference prints them; then the mesh "grid" of the cell
 * edges.  E, B and J are written; with `restart` also B_old and J_old, and
 * the header's restart flag is set.
 * Particles follow as the reference writes them (write_particle_variable,
 * write_particle_grid): per species the point variables weight, px, py, pz
 * (real8) and id (integer8), "<var>/<species>" on mesh "grid/<species>",
 * then the 3D point mesh "grid/<species>" of the Cartesian positions.
 * cyl_sdf_write: from host arrays, arrays[CYL_F_*] in the cyl_download_field
 * layout (NULL leaves an array out), species[0..nspecies) particle arrays;
 * host only.
 * A restart dump (restart != 0) first holds the constants the restart reads
 * back (diagnostics.F90:407-416): "dt", "window_shift_fraction" (only once the
 * window has started) and "x_grid_min".
 * cyl_sdf_write: from host arrays, arrays[CYL_F_*] in the cyl_download_field
 * layout (NULL leaves an array out), species[0..nspecies) particle arrays;
 * host only.
 * cyl_write_sdf: the handle's current state (its grid, step, time and live
 * particles); species_names[i] names species i (NULL: no particles).  The
 * reference writes its dumps at the output point inside a step
 * (epoch2d.F90:259-262, see cyl_step_to_output); between full steps the
 * state is the one after moving_window instead.  A restart dump is only
 * written at the output point (CYL_ERR_BAD_ARG otherwise), since the
 * restart finishes the step it stopped in. */
typedef struct cyl_sdf_desc {
  int32_t nx, ny, n_mode;
  int32_t step;
  double time;
  double xb_min;           /* x of the first cell edge (moves with the window) */
  double dx, dy;
  int32_t restart;
  /* restart dumps only */
  int32_t window_started;  /* write window_shift_fraction */
  double dt;               /* written when > 0 */
  double x_grid_min;
  double window_shift_fraction;
} cyl_sdf_desc;
typedef struct cyl_sdf_species {
  const char* name;
  int64_t n;
  const double *x, *y, *z, *px, *py, *pz, *w;
  const int64_t* id;
} cyl_sdf_species;
int cyl_sdf_write(const char* path, const cyl_sdf_desc* desc, const double* const* arrays,
                  const cyl_sdf_species* species, int32_t nspecies);
int cyl_write_sdf(cyl_handle h, const char* path, int32_t restart, const char* const* species_names);

/* ---- SDF input: the restart reader ---------------------------------------
 * Reads the SDF files above as restart_data does (setup.F90:777-1569):
 * cyl_sdf_read_field gives a mode array in the cyl_download_field layout,
 * zero where the file has no block and in the ghost cells, the interior
 * from "<id>_real" / "<id>_imag" (the rows of the shifted arrays moved back
 * down by one, setup.F90:1237-1247); species are found by the point mesh
 * whose species id (or block id "grid/<name>") is the name, and their
 * point variables by species id or mesh id; a point variable whose count
 * differs from its mesh's is an error (setup.F90:1411-1425).  Host only.
 * Errors: CYL_ERR_IO for a file that cannot be read or is not SDF,
 * CYL_ERR_BAD_ARG for an array or species the file does not describe. */
typedef struct cyl_sdf_file_s* cyl_sdf_file;
typedef struct cyl_sdf_info {
  int32_t step, restart;
  double time;
  int32_t nx, ny, n_mode;      /* from the mode blocks (0 without any) */
  int32_t has_grid;            /* the "grid" mesh: x edges [x0, x1], y [y0, y1] */
  double grid_x0, grid_x1, grid_y0, grid_y1;
  int32_t has_dt, has_window_shift_fraction, has_x_grid_min;
  double dt, window_shift_fraction, x_grid_min;
  char code_name[33];
} cyl_sdf_info;
int cyl_sdf_open(const char* path, cyl_sdf_file* out);
int cyl_sdf_close(cyl_sdf_file f);
int cyl_sdf_get_info(cyl_sdf_file f, cyl_sdf_info* out);
int cyl_sdf_read_field(cyl_sdf_file f, int32_t which, double* data);
/* *n_out = the species' particle count, -1 when the file has none of it. */
int cyl_sdf_species_count(cyl_sdf_file f, const char* name, int64_t* n_out);
/* n_inout in: capacity; out: particles written.  Variables absent from the
 * file read as zeros. */
int cyl_sdf_read_particles(cyl_sdf_file f, const char* name, double* x, double* y, double* z,
                           double* px, double* py, double* pz, double* w, int64_t* id,
                           int64_t* n_inout);

/* Load a restart dump into a handle created from the same deck, with no
 * particles loaded, as restart_data and the restart start-up of
 * epoch2d.F90:116-153 do: the mode arrays and every named species' particles
 * from the file (species_names[i] names species i; species the file lacks
 * stay empty), step and time from the header, the window's shift fraction,
 * x_grid_min and the grid edges from their blocks.  The handle is left at
 * the output point of the dumped step; the next stepping call runs
 * particle_bcs, efield_bcs, old_field_bcs, time = time + dt/2,
 * update_eb_fields_final and moving_window, then its steps.  The window
 * restarts as in the reference (window_started false, kept shift fraction),
 * ids continue from the largest loaded id + 1, and the host random stream
 * is the one the handle was created with (the reference's non-exact
 * restart).  Errors: CYL_ERR_IO (file), CYL_ERR_BAD_ARG (not a restart dump,
 * another code, grid or mode count or dt unlike the handle's, particles
 * already loaded), CYL_ERR_UNSUPPORTED (a step-0 dump, which a fresh start
 * replaces), CYL_ERR_CAPACITY (a species larger than its capacity). */
int cyl_restart_sdf(cyl_handle h, const char* path, const char* const* species_names);

/* ---- deck expressions evaluated by the caller --------------------------
 * While it steps, the reference evaluates some deck expressions through its
 * parser (evaluate_with_parameters, parser/evaluate.F90:461):
 *  - update_laser_omegas (laser.f90:276-328, from bfield_final_bcs): every
 *    laser's omega, when it is a deck function (use_omega_function);
 *  - outflow_bcs_x_min / x_max (laser.f90:444-451): for each laser between
 *    its t_start and t_end, its phase and profile when they are functions of
 *    time (laser_update_phase / _profile, laser.f90:201-253) and its time
 *    profile (laser_time_profile, laser.f90:182-199);
 *  - insert_particles (window.F90:196-222): at every window shift, every
 *    species' temperature, drift and density along the x_max column.
 * A caller that keeps the reference's parser (the Fortran driver) registers
 * callbacks that evaluate them.  A step calls them on the calling host thread
 * while it prepares that step, in the reference's order, before any of the
 * step's work is enqueued; a chunk of steps is prepared step by step.  Each
 * returns 0, or a non-zero value that makes the step return
 * CYL_ERR_CALLBACK.  Without callbacks the descriptors' closed forms are
 * used (cyl_laser_desc.t_profile, omega, profile and phase;
 * cyl_species_desc.density_kind, temp and drift).  Lasers are numbered by
 * their place in cyl_create's array, species likewise. */

/* *t_env = laser_time_profile of laser `ilaser` at `time` (the step
 * multiplies it by amp). */
typedef int (*cyl_laser_time_fn)(void* user, int32_t ilaser, double time, double* t_env);
/* *omega = omega(time) in rad/s of a laser whose omega is a deck function
 * (laser_update_omega, laser.f90:255-272, with the freq / lambda conversion
 * done); the step integrates its phase, phase += omega dt (laser.f90:307-309).
 * The phase of the other lasers is omega * time. */
typedef int (*cyl_laser_omega_fn)(void* user, int32_t ilaser, double time, double* omega);
/* The laser's profile or phase at y(ir), ir = 0..ny, at `time`: ny+1 values
 * written over the laser's current array. */
typedef int (*cyl_laser_array_fn)(void* user, int32_t ilaser, double time, double* values);
/* insert_particles' columns of species `ispecies` at a window shift: at
 * pack_ix = nx, i.e. x = x(nx) of the grid before the shift, and `time`, for
 * rows iy = 0..ny+1: density[iy] (m^-3), temperature[iy + (ny+2) dir] (K) and
 * drift[iy + (ny+2) dir] (kg m/s), dir = 0, 1, 2 (Fortran's (0:ny+1, 1:3)).
 * The step clamps the density to density_max and zeroes it below
 * density_min, as insert_particles does. */
typedef int (*cyl_inject_fn)(void* user, int32_t ispecies, double time, double x, double* density,
                             double* temperature, double* drift);

typedef struct cyl_deck_fns {
  void* user;                     /* passed back to every callback              */
  cyl_laser_time_fn laser_time;   /* NULL: cyl_laser_desc.t_profile             */
  cyl_laser_omega_fn laser_omega; /* called for the lasers of omega_fn_mask     */
  cyl_laser_array_fn laser_profile; /* called for the lasers of profile_fn_mask */
  cyl_laser_array_fn laser_phase;   /* called for the lasers of phase_fn_mask   */
  uint32_t omega_fn_mask;         /* bit i: laser i's omega is a deck function  */
  uint32_t profile_fn_mask;       /* bit i: laser i's profile depends on time   */
  uint32_t phase_fn_mask;         /* bit i: laser i's phase depends on time     */
  cyl_inject_fn inject;           /* NULL: cyl_species_desc density_kind, temp, drift */
} cyl_deck_fns;

/* Register the callbacks of a run (fns == NULL clears them); the struct is
 * copied.  The window injection drawn on the device (CYL_RNG_COUNTER) takes
 * its columns from the descriptors: an inject callback with it is
 * CYL_ERR_UNSUPPORTED, here and in cyl_set_injection_stream.  A mask bit
 * without its callback, or a bit beyond the run's lasers, is CYL_ERR_BAD_ARG. */
int cyl_set_deck_fns(cyl_handle h, const cyl_deck_fns* fns);

/* ---- field ionisation (physics_packages/ionise.F90) -------------------
 * Per species: whether it ionises (species%ionise), the species it becomes
 * (ionise_to_species) and the species that receives the released electron
 * (release_species; -1: none), 0-based as in cyl_create; the quantum numbers
 * l and n of the electron removed and its ionisation energy in J, which the
 * reference reads from its tables for the deck's atomic_no
 * (deck_species_block.F90:1194-1310; TABLES/ionisation_energies.table,
 * ion_l.table, ion_n.table). */
typedef struct cyl_ionisation_species {
  int32_t ionise;
  int32_t ionise_to;
  int32_t release;
  int32_t l, n;
  double energy;
} cyl_ionisation_species;
#define CYL_IONISE_MULTIPHOTON 1  /* use_multiphoton (on by default in the reference) */
#define CYL_IONISE_BSI 2          /* use_bsi (on by default in the reference) */
/* Switch on field ionisation (use_field_ionisation): from the next step on,
 * ionise_particles runs after the push and current_bcs_r_min_final and
 * before current_finish (epoch2d.F90:251), with the constants of
 * initialise_ionisation (ionise.F90:51-286) computed here.  model: the
 * CYL_IONISE_* bits; both is the reference's default
 * (multiphoton_tunnelling_bsi, ionise.F90:355-657), none its plain
 * tunnelling (ionise.F90:1236-1500).  Multiphoton needs every laser at one
 * omega (ionise.F90:56-123).  The random number of each ionisation trial is
 * the counter stream's word for (particle id, step, charge state) under key
 * seed, where the reference draws from its serial KISS stream: same
 * distribution, a different sequence.  A released electron takes the id
 * 2^62 + 16 (parent id) + (index of the parent's species before the event).
 * Both forms; in the mixed form the trials read the FP32 fields and the
 * ions and electrons enter the species' unsorted tails (pushed on the
 * global path until the next sort); a batch (cyl_batch_step) refuses runs
 * with ionisation (CYL_ERR_UNSUPPORTED).  Errors:
 * CYL_ERR_BAD_ARG for species indices out of range or an ionising species
 * without a next state; CYL_ERR_UNSUPPORTED for multiphoton without lasers
 * or with lasers of different omega.  nspecies == 0 switches it off. */
int cyl_set_ionisation(cyl_handle h, const cyl_ionisation_species* species, int32_t nspecies, int32_t model,
                       uint64_t seed);
/* The per-species constants of initialise_ionisation that the step uses, for
 * the tests (host only): out[i * CYL_ION_NCONST + k] for species i, in the
 * order released mass fraction, 2 n* - 1.5, ADK field scale, ADK constant,
 * smallest usable E, BSI constant, BSI scale, BSI threshold, ADK maximum,
 * ADK cap at the BSI threshold, Keldysh field, multiphoton constant, energy
 * of the K photons, 4 K - 2, ADK cap at the multiphoton threshold (atomic
 * units where the reference uses them).  No counterpart in the reference's
 * interfaces. */
#define CYL_ION_NCONST 15
int cyl_ionisation_constants(const cyl_ionisation_species* species, const cyl_species_desc* sp,
                             int32_t nspecies, int32_t model, double laser_omega, double* out);

/* Device loading and window injection from a counter-based stream
 * (Philox4x32-10 keyed by seed, one counter per particle) instead of the
 * reference's serial KISS stream: the loader and injector of the reference
 * (helper.F90:669-811, window.F90:157-300) with each particle made by its
 * own thread; the particles differ from the KISS-stream ones but follow the
 * same distributions, counts, weights and id order.
 * cyl_load_species_device: fill species ispecies (replacing its particles)
 * on the current grid; ids id_base .. id_base + n - 1; n_out = particles
 * (floor(npart_per_cell * valid cells), as the reference loads).  Immobile
 * species: CYL_ERR_BAD_ARG.
 * cyl_set_injection_stream: window injection from the next step on comes
 * from the host KISS stream (CYL_RNG_KISS, the default, reference order) or
 * is drawn on the device (CYL_RNG_COUNTER, keyed by seed); the counter mode
 * handles at most 2 window shifts per step (CYL_ERR_UNSUPPORTED beyond). */
#define CYL_RNG_KISS 0
#define CYL_RNG_COUNTER 1
int cyl_load_species_device(cyl_handle h, int32_t ispecies, uint64_t seed, int64_t id_base, int64_t* n_out);
int cyl_set_injection_stream(cyl_handle h, int32_t mode, uint64_t seed);
/* Mixed form: inside one cyl_step call's chunk of steps that does not shift
 * the window, the closing E half-step of each step and the opening one of
 * the next see the same B and J; they are merged into one pass over the
 * bulk of the grid (on, the default), with the cells that the E boundary
 * rules touch between them updated one half at a time.  The results are
 * those of separate half-steps; on = 0 runs every half-step as its own
 * pass.  The FP64 form never merges. */
int cyl_set_merge_e_halves(cyl_handle h, int32_t on);
/* One block of the counter stream: Philox4x32-10 of counter ctr under key
 * seed (host only; for reproducing the stream outside the library). */
int cyl_counter_block(uint64_t seed, const uint32_t* ctr4, uint32_t* out4);
/* Download the live particles of one species, in device order.  n_inout in:
 * capacity of the host arrays; out: particles written.  With x == NULL only
 * the live count is returned (from the device counters, no copy).  Right
 * after a sort (every 16-step chunk ends with one) the slots hold no holes
 * and the copy goes straight into the caller's arrays (pinned arrays give
 * the full copy bandwidth). */
int cyl_download_particles(cyl_handle h, int32_t ispecies, double* x, double* y,
                           double* z, double* px, double* py, double* pz,
                           double* w, int64_t* id, int64_t* n_inout);
/* Copy one complex mode array (Fortran layout with ghosts, interleaved
 * re/im, (nx+2ng)*(ny+2ng)*n_mode complex values). */
int cyl_upload_field(cyl_handle h, int32_t which, const double* data);
int cyl_download_field(cyl_handle h, int32_t which, double* data);

/* Start-up sequence of epoch2d.F90:143-162 for a run that is not a restart:
 * particle_bcs, efield_bcs, then bfield_final_bcs with dt halved and the
 * time advanced to dt/2. */
int cyl_initialise(cyl_handle h);

/* Advance nsteps full PIC steps, i.e. nsteps iterations of the driver loop
 * body epoch2d.F90:213-265: update_eb_fields_half, push_particles (with
 * current_bcs_r_min_final and particle_bcs), current_finish,
 * update_eb_fields_final, moving_window.  Window injection is generated by
 * the handle's own KISS stream exactly as insert_particles does. */
int cyl_step(cyl_handle h, int32_t nsteps);

/* Same as cyl_step but the steps are captured once into a CUDA graph and
 * replayed (one graph launch per call after the first). */
int cyl_step_graph(cyl_handle h, int32_t nsteps);
/* As cyl_step_graph without the final stream sync: the call returns once
 * the steps are enqueued (the host work of a chunk overlaps the device work
 * of the one before, also across calls).  A device error flag raised by
 * these steps is reported by the next call that syncs (cyl_diagnostics,
 * cyl_diagnostics_read's device_error, cyl_get_run_state, downloads). */
int cyl_step_async(cyl_handle h, int32_t nsteps);
/* Advance to the reference's output point of the nsteps-th step
 * (nsteps >= 1): nsteps - 1 full steps, then of the last one
 * update_eb_fields_half, the push and current_finish, with step = step + 1
 * and time = time + dt/2 -- the state output_routines(step) sees
 * (epoch2d.F90:259-262).  Downloads, cyl_write_sdf, cyl_get_run_state and
 * diagnostics then read that state.  The next stepping call (cyl_step*,
 * cyl_batch_step, cyl_push_only, cyl_tune_tiles, with nsteps 0 too) first
 * finishes the step: time = time + dt/2, update_eb_fields_final,
 * moving_window (epoch2d.F90:263-265).  Fields and particles after
 * finishing equal those of nsteps full steps. */
int cyl_step_to_output(cyl_handle h, int32_t nsteps);

int cyl_get_run_state(cyl_handle h, cyl_run_state* out);
int cyl_diagnostics(cyl_handle h, cyl_diag* out);
/* Diagnostics without a stream sync: cyl_diagnostics_async enqueues the
 * reductions of the state after the steps enqueued so far, with their copy
 * to pinned host memory (at most two pending, else CYL_ERR_BAD_ARG);
 * cyl_diagnostics_read waits for the oldest pending one and returns it. */
int cyl_diagnostics_async(cyl_handle h);
int cyl_diagnostics_read(cyl_handle h, cyl_diag* out);
int cyl_get_rng_state(cyl_handle h, cyl_rng_state* out);

/* The first particle that raised the device error word in the mixed form:
 * out16[0] holds the reason as an int bit pattern (0 = none), out16[1] the
 * particle slot, out16[2..9] its state at the failing check.  No
 * counterpart in the reference (its debug builds trap instead). */
int cyl_debug_record(cyl_handle h, float* out16);

/* Sort each species' particles by cell tile and drop removed particles
 * (the device analogue of reorder_particles_to_grid, split_particle.F90:29-73). */
int cyl_sort_particles(cyl_handle h);

/* Cell-sort indices of the live particles, in device order:
 * cell_x = FLOOR((x - x_grid_min_local)/dx + 1.5),
 * cell_y = FLOOR((r - y_grid_min_local)/dy + 1.5)  (split_particle.F90:61-62).
 * With cell_x and cell_y both NULL, *n_inout receives the live count; passing
 * only one of them is CYL_ERR_BAD_ARG. */
int cyl_cell_indices(cyl_handle h, int32_t ispecies, int32_t* cell_x,
                     int32_t* cell_y, int64_t* n_inout);

/* Same result and arguments as cyl_cell_indices, computed without any
 * allocation: no cudaMalloc/cudaFree and no allocating library call, host or
 * device.  No counterpart in the reference.  It serves callers that cannot
 * allocate per call -- a diagnostics hook run between queued steps (cudaMalloc
 * and cudaFree synchronise the device and would stall them) and runs admitted
 * against a fully committed HBM budget (an allocation could fail).
 *
 * The scratch is one fixed device array of CYL_NOALLOC_MAX_PARTICLES slots
 * (5 int32 words per slot, 5 MiB) reserved when the library is loaded; a
 * species with more particle slots (live + removed since the last sort) is
 * rejected with CYL_ERR_SCRATCH.  The first call on a device looks the scratch
 * up (cudaGetSymbolAddress) and should come before any stream capture.  The
 * call works on the handle's device whatever device the caller has current,
 * and restores the caller's.  The scratch is shared by every handle of the
 * process: calls that overlap in time race on it. */
#define CYL_NOALLOC_MAX_PARTICLES 262144
int cyl_cell_indices_noalloc(cyl_handle h, int32_t ispecies, int32_t* cell_x,
                             int32_t* cell_y, int64_t* n_inout);

/* Per-mode charge density of the mobile species, complex FP64 in the field
 * layout (like cyl_download_field), computed from the current particle state
 * with the current deposit's own staggered shape at t + dt/2 (the half-drift
 * of particles.F90:304-312, cell_x2 and the h weights of :369-388, the
 * 2 e^{i m theta} mode factor of :595-611 and inv_volume of :661).  Between
 * two calls around one step, (rho' - rho)/dt + div J is the discrete
 * continuity residual of that step's deposit; the reference has no such
 * diagnostic (its Gauss-law consistency rests on the same identity).  The
 * mixed form evaluates it in FP64 from its stored state. */
int cyl_charge_density(cyl_handle h, double* rho);

/* Per-mode number density of species `ispecies` (every species when
 * ispecies < 0), complex FP64 in the field layout: the reference's
 * calc_number_density_modes (io/calc_df.F90:588-661) -- cell-centred triangle
 * weights with the r < dy fold (include/triangle/gxfac.inc), each particle's
 * weight over its macro-particle volume 2 pi dx dy r
 * (housekeeping/partlist.F90:999-1013), mode factor 2 e^{i m theta} for
 * m > 0, boundary sums (calc_df.F90:35-55) and zero-gradient ghosts.  The
 * mixed form evaluates it in FP64 from its stored state. */
int cyl_number_density(cyl_handle h, int32_t ispecies, double* out);

/* ---- tile shape of the mixed form's push ------------------------------
 * The mixed form keeps particles sorted by tiles of tx x ty cells and pushes
 * one tile per CTA with the tile's fields staged in shared memory.  The push
 * is built for CYL_N_TILE_SHAPES shapes; shape 0 (16 x 8) is the default.
 * No counterpart in the reference (its push walks linked lists).
 *
 * cyl_tile_shape: the cells (x, r) of shape `shape`.  Host only.
 *
 * cyl_tune_tiles (mixed form only; CYL_ERR_UNSUPPORTED for the FP64 form):
 *   mode CYL_TUNE_SET:  use shape *shape (re-sorts the particles);
 *   mode CYL_TUNE_TIME: time one push of the current state with every shape
 *     (each on a copy of the state that is restored afterwards: the run's
 *     particles and currents are unchanged) and keep the fastest; its index
 *     is returned in *shape.  The copy is a temporary device allocation of
 *     40 bytes per particle slot plus three current arrays.
 * The shape changes the order of the per-tile FP32 partial sums only; the
 * results of two shapes agree to FP32 round-off. */
#define CYL_N_TILE_SHAPES 5
#define CYL_TUNE_SET 0
#define CYL_TUNE_TIME 1
int cyl_tile_shape(int32_t shape, int32_t* tx, int32_t* ty);
int cyl_tune_tiles(cyl_handle h, int32_t mode, int32_t* shape);

/* Push-and-deposit only (the body of push_particles, particles.F90:163-734,
 * without current_bcs_r_min_final and particle_bcs): used by the parity tests
 * and by the kernel benchmark to time the dominant kernel alone. */
int cyl_push_only(cyl_handle h);

/* Average duration (ms) of the push/deposit kernel over the launches since
 * the last call, measured with CUDA events on the launching stream. */
int cyl_kernel_timing(cyl_handle h, double* push_ms_avg, int64_t* launches);

/* The CUDA stream (a cudaStream_t) every kernel and copy of the handle is
 * enqueued on, so that a caller can time the steps with its own CUDA events
 * on that stream.  No counterpart in the reference. */
int cyl_get_stream(cyl_handle h, void** stream_out);

/* out[i] = atan2(y[i], x[i]) as the FP64 form's push evaluates theta on the
 * device (the correctly rounded routine of include/cyl_math.h, which the
 * oracle also evaluates in its "shared" mode), for i < n.  Host arrays.  No
 * counterpart in the reference: it lets a test show that the device and host
 * builds of that routine agree bit for bit.  Synchronous; allocates device
 * scratch for the call. */
int cyl_eval_atan2(int64_t n, const double* y, const double* x, double* out);

/* Device bytes cyl_create would allocate for these descriptors (an upper
 * bound; used for admission against an HBM budget).  Host only. */
int cyl_estimate_device_bytes(const cyl_grid_desc* grid, const cyl_species_desc* species,
                              int32_t nspecies, int64_t* out);

/* ---- batches: several mixed-form runs stepped together ------------------
 * No counterpart in the reference (one deck per MPI job there).  A batch
 * steps n handles (mixed form, the same number of modes, any grids and
 * particle counts) through the same steps in lockstep: the push of all of
 * them is one persistent kernel per step over a shared table of (run,
 * species, tile) items in decreasing order of particle count; the field,
 * boundary and window stages stay per run, on each run's own stream, forked
 * and joined around the push, and a chunk of 16 steps is one CUDA graph
 * (captured again when the membership changes).  Membership may change from
 * one call to the next (runs join and leave between calls).  The runs use
 * tile shape 0 while batched.  Each run's results are those of stepping it
 * alone, up to the order of its FP64 current additions. */
typedef struct cyl_batch_s* cyl_batch;
int cyl_batch_create(int32_t max_runs, cyl_batch* out);
int cyl_batch_step(cyl_batch b, const cyl_handle* handles, int32_t n, int32_t nsteps);
int cyl_batch_destroy(cyl_batch b);

/* ---- serving: a request loop for parameter scans ----------------------
 * No counterpart in the reference (one deck per MPI job there).  A server
 * owns a queue of runs (jobs) and a pool of worker threads on one GPU.  Jobs
 * are admitted in arrival order while their estimated device memory fits the
 * HBM budget; each admitted job loads its species on the host (the
 * reference's loader and KISS stream, seeded per job), creates a handle on
 * its own CUDA stream, runs its steps as CUDA graphs of 16 steps and is
 * retired (its device memory freed) when done, so runs of uneven size
 * overlap on the device.  Results stay readable until the server is
 * destroyed. */
#define CYL_JOB_QUEUED 0
#define CYL_JOB_RUNNING 1
#define CYL_JOB_DONE 2
#define CYL_JOB_FAILED 3

typedef struct cyl_job_desc {
  cyl_grid_desc grid;
  int32_t nspecies;
  cyl_species_desc species[8];
  int32_t nlasers;
  cyl_laser_desc lasers[8];      /* profile / phase are copied at submit   */
  int64_t nsteps;
  int32_t seed;                  /* KISS seed of the loader (7842432 + rank in the reference) */
  int32_t rng_mode;              /* CYL_RNG_KISS: host load and injection from the KISS stream;
                                    CYL_RNG_COUNTER: device load and injection, counter stream keyed by seed */
} cyl_job_desc;

typedef struct cyl_job_result {
  int32_t status;                /* CYL_JOB_*                               */
  int32_t error;                 /* CYL_OK or the failing call's status     */
  double t_submit, t_start, t_end;  /* seconds since the server was created */
  int64_t steps_done;
  double particle_steps;         /* mean live mobile particles x steps      */
  int64_t device_bytes;          /* estimate charged to the budget          */
  cyl_diag diag;                 /* diagnostics after the last step         */
  cyl_run_state state;
} cyl_job_result;

typedef struct cyl_server_s* cyl_server;

/* hbm_budget_bytes: device memory the jobs may hold together (0: the free
 * memory of the device at creation, minus 2 GiB); workers: jobs run at the
 * same time (>= 1). */
int cyl_server_create(int64_t hbm_budget_bytes, int32_t workers, cyl_server* out);
/* The request loop with continuous batching: `loaders` threads admit jobs
 * against the budget (and while fewer than max_batch jobs are open).  A
 * mixed-form job with at most one push tile (16 x 8 cells) per SM is loaded
 * and handed to one stepper thread, which advances all such jobs with the
 * same number of modes together through one cyl_batch, by up to 16 steps
 * per pass; new jobs join at the next pass, finished ones are retired and
 * their memory freed.  Larger and FP64-form jobs fill the device alone and
 * run start to end on their loader's stream, as in cyl_server_create. */
int cyl_server_create_batched(int64_t hbm_budget_bytes, int32_t loaders, int32_t max_batch, cyl_server* out);
/* Queue a job; CYL_ERR_OUT_OF_MEMORY if it alone exceeds the budget. */
int cyl_server_submit(cyl_server s, const cyl_job_desc* job, int64_t* job_id);
/* Current state of a job (non-blocking). */
int cyl_server_poll(cyl_server s, int64_t job_id, cyl_job_result* out);
/* Wait until the job is done or failed, at most timeout_s seconds
 * (CYL_ERR_TIMEOUT when the wait runs out). */
int cyl_server_wait(cyl_server s, int64_t job_id, double timeout_s, cyl_job_result* out);
/* Jobs queued, running, and device bytes currently charged. */
int cyl_server_stats(cyl_server s, int32_t* queued, int32_t* running, int64_t* bytes_in_use);
/* Finish the running and queued jobs, join the workers, free everything. */
int cyl_server_destroy(cyl_server s);

/* ---- host-side deck helpers (stand in for the Fortran loader) ---------- */

/* KISS generator and polar Box-Muller of random_generator.f90:45-173. */
void cyl_rng_init(cyl_rng_state* s, int32_t seed);
double cyl_rng_random(cyl_rng_state* s);
double cyl_rng_box_muller(cyl_rng_state* s, double stdev, double mu);

/* Load one species the way auto_load does for a thermal species
 * (helper.F90:95-169, 373-663, 669-811; particle_temperature.F90:30-81):
 * uniform random positions per valid cell, weights from the triangle shape
 * and the macro-particle volume, Maxwellian momenta by Box-Muller.  Two
 * calls: with x == NULL it only returns the particle count in *n_inout
 * (without touching the RNG); otherwise it fills the arrays (capacity
 * *n_inout) and advances the RNG. */
int cyl_host_load_species(const cyl_grid_desc* grid, const cyl_species_desc* sp,
                          cyl_rng_state* rng, int64_t id_base, double* x,
                          double* y, double* z, double* px, double* py,
                          double* pz, double* w, int64_t* id, int64_t* n_inout);

/* cyl_host_load_species with the deck's density, temperature and drift
 * evaluated by the caller on the whole grid with ghosts, as
 * setup_particle_density (helper.F90:669-811) and the temperature and
 * drift arrays of auto_load (helper.F90:130-160, particle_temperature.F90:
 * 30-81) hold them: index (ix + ng - 1) + (nx + 2 ng)(iy + ng - 1) for
 * ix = 1-ng..nx+ng, iy = 1-ng..ny+ng (Fortran's (1-ng:nx+ng, 1-ng:ny+ng));
 * temperature (K) and drift (kg m/s) hold three such planes, x, y, z.  The
 * loader applies the density's periodic x wrap, density_max clamp and
 * density_min cut as it does to the closed form.  A NULL array takes the
 * descriptor's closed form for that quantity. */
int cyl_host_load_species_grid(const cyl_grid_desc* grid, const cyl_species_desc* sp,
                               cyl_rng_state* rng, int64_t id_base, const double* density,
                               const double* temperature, const double* drift, double* x,
                               double* y, double* z, double* px, double* py,
                               double* pz, double* w, int64_t* id, int64_t* n_inout);

#ifdef __cplusplus
}
#endif

#endif /* CYLPIC_H */
