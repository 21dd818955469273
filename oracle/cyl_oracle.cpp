// cyl_oracle.cpp -- CPU FP64 restatement of cylindrical EPOCH's PIC step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path is
// checked against.  Nothing in the product links, loads or calls it; only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
//
// Parity status: the reference (Fortran 2003 + MPI) cannot be built in this
// environment and its own tests pin no cylindrical result, so this
// restatement is pinned by the analytic current of DOCUMENTATION.pdf section
// 7.2 (example_decks/current_density_test.deck), by discrete charge
// conservation and by the Yee vacuum dispersion relation; see tests/.
//
// Every routine follows the Fortran line by line, single rank (so MPI halo
// exchanges reduce to periodic self-wraps), default compile-time options:
// triangle shape, per-particle weight, Boris push.  Operation order is kept
// and the file is compiled with -ffp-contract=off.  Citations are
// path:line inside the reference project (epoch_axial/src/...).

#include "../include/cylpic.h"
#include "../include/cyl_math.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// constants.F90:171-181
const double PI = 3.141592653589793238462643383279503;
const double C = 2.99792458e8;
const double KB = 1.3806488e-23;
const double EPS0 = 8.854187817620389850536563031710750e-12;
// constants.F90:535-548 (triangle shape)
const int SF_MIN = -1, SF_MAX = 1, PNG = 3, NG = 5, JNG = 5;

struct cplx {
  double re, im;
};
inline cplx mk(double r, double i) { return {r, i}; }
inline cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
inline cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
inline cplx operator-(cplx a) { return {-a.re, -a.im}; }
inline cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
inline cplx operator*(double s, cplx a) { return {s * a.re, s * a.im}; }
inline cplx operator*(cplx a, double s) { return {a.re * s, a.im * s}; }
inline cplx operator/(cplx a, double s) { return {a.re / s, a.im / s}; }
inline cplx operator+(cplx a, double s) { return {a.re + s, a.im}; }
inline cplx operator-(cplx a, double s) { return {a.re - s, a.im}; }
inline cplx operator-(double s, cplx a) { return {s - a.re, -a.im}; }
inline cplx operator+(double s, cplx a) { return {s + a.re, a.im}; }
// 1/z by the range-reduced (Smith) division that gfortran's Fortran complex
// rules use for a real numerator.
inline cplx crecip(cplx z) {
  double c = z.re, d = z.im;
  if (std::fabs(c) < std::fabs(d)) {
    double ratio = c / d;
    double div = c * ratio + d;
    return {(1.0 * ratio + 0.0) / div, (0.0 * ratio - 1.0) / div};
  } else {
    double ratio = d / c;
    double div = d * ratio + c;
    return {(0.0 * ratio + 1.0) / div, (0.0 - 1.0 * ratio) / div};
  }
}
const cplx IMAGI = {0.0, 1.0};

inline int ffloor(double v) { return (int)std::floor(v); }

// Complex mode array F(1-ng:nx+ng, 1-ng:ny+ng, 0:M-1), Fortran order.
struct Field {
  int nx = 0, ny = 0, M = 0, nxg = 0, nyg = 0;
  std::vector<cplx> a;
  void init(int nx_, int ny_, int M_) {
    nx = nx_; ny = ny_; M = M_;
    nxg = nx + 2 * NG; nyg = ny + 2 * NG;
    a.assign((size_t)nxg * nyg * M, cplx{0.0, 0.0});
  }
  cplx& operator()(int ix, int iy, int m) {
    return a[(size_t)(ix + NG - 1) + (size_t)nxg * ((size_t)(iy + NG - 1) + (size_t)nyg * m)];
  }
};

// Boundary column arrays *_x_min/_x_max (setup.F90:393-423): (1-ng:ny+ng, 0:M-1)
struct Col {
  int ny = 0, M = 0;
  std::vector<cplx> a;
  void init(int ny_, int M_) { ny = ny_; M = M_; a.assign((size_t)(ny + 2 * NG) * M, cplx{0, 0}); }
  cplx& operator()(int iy, int m) { return a[(size_t)(iy + NG - 1) + (size_t)(ny + 2 * NG) * m]; }
};

// KISS + Box-Muller (random_generator.f90:45-173), 32-bit wrap-around.
struct Rng {
  int32_t x, y, z, w;
  bool cached;
  double cval;
  double random() {
    x = (int32_t)((uint32_t)69069u * (uint32_t)x + (uint32_t)1327217885u);
    uint32_t a1 = (uint32_t)y;
    uint32_t a2 = a1 ^ (a1 << 13);
    uint32_t a3 = a2 ^ (a2 >> 17);
    y = (int32_t)(a3 ^ (a3 << 5));
    z = (int32_t)((uint32_t)18000u * ((uint32_t)z & 65535u) + ((uint32_t)z >> 16));
    w = (int32_t)((uint32_t)30903u * ((uint32_t)w & 65535u) + ((uint32_t)w >> 16));
    int32_t kiss = (int32_t)((uint32_t)x + (uint32_t)y + ((uint32_t)z << 16) + (uint32_t)w);
    return ((double)kiss + 2147483648.0) / 4294967296.0;
  }
  void init(int32_t seed) {
    x = (int32_t)(123456789u + (uint32_t)seed);
    y = (int32_t)(362436069u + (uint32_t)seed);
    z = (int32_t)(521288629u + (uint32_t)seed);
    w = (int32_t)(916191069u + (uint32_t)seed);
    cached = false;
    cval = 0.0;
    for (int i = 0; i < 1000; ++i) random();
  }
  double box_muller(double stdev, double mu) {
    if (cached) {
      cached = false;
      return cval * stdev + mu;
    }
    cached = true;
    double r1, r2, ww;
    for (;;) {
      r1 = random();
      r2 = random();
      r1 = 2.0 * r1 - 1.0;
      r2 = 2.0 * r2 - 1.0;
      ww = r1 * r1 + r2 * r2;
      if (ww > 2.2250738585072014e-308 && ww < 1.0) break;
    }
    ww = std::sqrt((-2.0 * std::log(ww)) / ww);
    double v = r1 * ww * stdev + mu;
    cval = r2 * ww;
    return v;
  }
};

// The counter stream of device loading and device window injection, restated
// from the published algorithm: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// SC'11).  A round multiplies words 0 and 2 by 0xD2511F53 and 0xCD9E8D57,
// takes the high halves xor the other two words and the round key as the new
// words 0 and 2, the low halves as the new 3 and 1; the key advances by
// 0x9E3779B9 / 0xBB67AE85 between rounds.  Counters and tags as the product
// documents them: (p, p >> 32, species, 1|2) for loading positions/momenta,
// (row, shift, species, 3) for the injected row's fraction bit,
// (j, shift, species, 4|5) for injected positions/momenta.
struct Ctr4 {
  uint32_t w[4];
};
Ctr4 philox10(Ctr4 c, uint64_t seed) {
  uint32_t key[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
  for (int round = 0; round < 10; ++round) {
    const uint64_t m0 = (uint64_t)0xD2511F53u * c.w[0];
    const uint64_t m1 = (uint64_t)0xCD9E8D57u * c.w[2];
    Ctr4 n;
    n.w[0] = (uint32_t)(m1 >> 32) ^ c.w[1] ^ key[0];
    n.w[1] = (uint32_t)m1;
    n.w[2] = (uint32_t)(m0 >> 32) ^ c.w[3] ^ key[1];
    n.w[3] = (uint32_t)m0;
    c = n;
    key[0] += 0x9E3779B9u;
    key[1] += 0xBB67AE85u;
  }
  return c;
}
inline double ctr_u01(uint32_t r) { return ((double)r + 0.5) * 2.3283064365386963e-10; }
// three normal deviates: Box-Muller of words (0, 1) -> cos, sin; (2, 3) ->
// cos; angles in turns through cyl_sincos_turn (shared with the kernels)
void ctr_normals(const Ctr4& r, double out[3]) {
  const double rho1 = std::sqrt(-2.0 * std::log(ctr_u01(r.w[0])));
  double s1, c1, s2, c2;
  cyl_sincos_turn(ctr_u01(r.w[1]), &s1, &c1);
  const double rho2 = std::sqrt(-2.0 * std::log(ctr_u01(r.w[2])));
  cyl_sincos_turn(ctr_u01(r.w[3]), &s2, &c2);
  out[0] = rho1 * c1;
  out[1] = rho1 * s1;
  out[2] = rho2 * c2;
}

struct Species {
  cyl_species_desc d;
  int bc[4];  // particle bcs after setup_particle_boundary
  std::vector<double> x, y, z, px, py, pz, w;
  std::vector<int64_t> id;
  size_t n() const { return x.size(); }
  void push_back(double a, double b, double c, double d1, double e, double f, double g, int64_t i) {
    x.push_back(a); y.push_back(b); z.push_back(c);
    px.push_back(d1); py.push_back(e); pz.push_back(f); w.push_back(g); id.push_back(i);
  }
  void erase_mask(const std::vector<char>& dead) {
    size_t k = 0;
    for (size_t i = 0; i < n(); ++i) {
      if (dead[i]) continue;
      x[k] = x[i]; y[k] = y[i]; z[k] = z[i];
      px[k] = px[i]; py[k] = py[i]; pz[k] = pz[i]; w[k] = w[i]; id[k] = id[i];
      ++k;
    }
    x.resize(k); y.resize(k); z.resize(k); px.resize(k); py.resize(k); pz.resize(k);
    w.resize(k); id.resize(k);
  }
};

struct Laser {
  cyl_laser_desc d;
  std::vector<double> profile, phase;  // 0..ny
  double current_integral_phase = 0.0;
};

struct Sim {
  // grid and time
  int nx, ny, M;
  double dx, dy, dt, time;
  int64_t step;
  double length_x, length_y;
  double x_min, x_max, y_max;
  double x_grid_min, xb_min, x_grid_max;
  double y_grid_min, y_grid_max;
  double x_min_local, x_max_local, y_min_local, y_max_local;
  int bc_field[4];
  int bc_deck[4];
  int bc_allspecies[4];
  bool add_laser[4];
  bool move_window, window_started;
  double window_v_x, window_start_time, window_stop_time, window_shift_fraction;
  int bc_after_move[4];
  int64_t n_shifts;
  int64_t next_id;
  bool from_restart = false;  // ic_from_restart: a starting window keeps its shift fraction
  bool inj_counter = false;  // window injection from the counter stream
  uint64_t inj_seed = 0;
  Field ex, er, et, bx, br, bt, jx, jr, jt, bx_old, br_old, bt_old, jx_old, jr_old, jt_old;
  Col ex_xmin, er_xmin, et_xmin, bx_xmin, br_xmin, bt_xmin;
  Col ex_xmax, er_xmax, et_xmax, bx_xmax, br_xmax, bt_xmax;
  std::vector<Species> sp;
  std::vector<Laser> lasers;
  cyl_deck_fns fns{};  // deck-expression callbacks (orc_set_deck_fns)
  // field ionisation (orc_set_ionisation): per-species data and constants
  bool ion_on = false;
  int ion_model = 0;
  uint64_t ion_seed = 0;
  struct IonSp {
    cyl_ionisation_species in;
    double rmf, n_exp, adk_scaling, ion_const, smallest_e, bsi_const, bsi_scaling, bsi_threshold, adk_max;
    double adk_bsi_cap, keldysh, multi_const, k_energy, k_exponent, adk_mp_cap;
  };
  std::vector<IonSp> ion;
  Rng rng;
  int smooth, smooth_its, smooth_comp_its, smooth_stride;
  std::vector<Field> thread_j;  // per-thread currents of the multi-threaded timing form

  Field* field(int which) {
    Field* t[15] = {&ex, &er, &et, &bx, &br, &bt, &jx, &jr, &jt,
                    &bx_old, &br_old, &bt_old, &jx_old, &jr_old, &jt_old};
    return (which >= 0 && which < 15) ? t[which] : nullptr;
  }

  // x(ix), y(iy): cell-centred local grid (setup.F90:189-201, utilities.f90:347-349)
  double xg(int ix) const { return x_grid_min + (double)(ix - 1) * dx; }
  double yg(int iy) const { return y_grid_min + (double)(iy - 1) * dy; }

  // setup_grid_x / setup_grid_y (utilities.f90:343-409), cpml_thickness = 0
  void setup_grid_x() {
    x_grid_max = x_grid_min + (double)(nx - 1) * dx;
    x_min_local = x_grid_min + (0.0 - 0.5) * dx;
    x_max_local = x_grid_max - (0.0 - 0.5) * dx;
  }
  void setup_grid_y() {
    y_grid_max = y_grid_min + (double)(ny - 1) * dy;
    y_min_local = y_grid_min + (0.0 - 0.5) * dy;
    y_max_local = y_grid_max - (0.0 - 0.5) * dy;
  }

  // setup_boundaries (boundary.F90:30-75): field bc mapping + add_laser
  void setup_boundaries() {
    for (int i = 0; i < 4; ++i) {
      int b = bc_deck[i];
      add_laser[i] = false;
      if (b == CYL_BC_OTHER) b = CYL_BC_CLAMP;
      if (b == CYL_BC_SIMPLE_LASER) add_laser[i] = true;
      if (b == CYL_BC_REFLECT) b = CYL_BC_CLAMP;
      if (b == CYL_BC_OPEN) b = CYL_BC_SIMPLE_OUTFLOW;
      bc_field[i] = b;
    }
  }
};

// Stagger table (setup.F90:126-136 with constants.F90:291-296):
// which = 0 exm, 1 erm, 2 etm, 3 bxm, 4 brm, 5 btm
const bool STAG_X[6] = {false, true, true, true, false, false};
const bool STAG_Y[6] = {true, false, true, false, true, false};

// ---------------------------------------------------------------- field bcs

// do_field_mpi_with_lengths_cmplx on one rank (boundary.F90:500-593): only
// the periodic-x self wrap moves data; rows [j0, j1].
void halo_x(Sim& s, Field& f, int j0, int j1) {
  if (s.bc_field[CYL_BD_X_MAX] == CYL_BC_PERIODIC) {
    for (int m = 0; m < s.M; ++m)
      for (int j = j0; j <= j1; ++j)
        for (int i = 1; i <= NG; ++i) f(s.nx + i, j, m) = f(i, j, m);
  }
  if (s.bc_field[CYL_BD_X_MIN] == CYL_BC_PERIODIC) {
    for (int m = 0; m < s.M; ++m)
      for (int j = j0; j <= j1; ++j)
        for (int i = 1 - NG; i <= 0; ++i) f(i, j, m) = f(s.nx + i, j, m);
  }
}
// field_mode_bc on an array whose ir=0 row is not a ghost: the r-shift of
// efield_bcs/bfield_bcs (boundary.F90:1362-1371) leaves row ny+ng untouched.
void halo_full(Sim& s, Field& f) { halo_x(s, f, 1 - NG, s.ny + NG); }
void halo_shifted(Sim& s, Field& f) { halo_x(s, f, 1 - NG, s.ny + NG - 1); }

// field_mode_zero_gradient (boundary.F90:654-707)
void zero_gradient(Sim& s, Field& f, int st, int bd) {
  if (s.bc_field[bd] == CYL_BC_PERIODIC) return;
  int nx = s.nx, ny = s.ny, M = s.M;
  if (bd == CYL_BD_X_MIN) {
    for (int m = 0; m < M; ++m)
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        if (STAG_X[st]) for (int i = 1; i <= NG - 1; ++i) f(i - NG, j, m) = f(NG - i, j, m);
        else for (int i = 1; i <= NG; ++i) f(i - NG, j, m) = f(NG + 1 - i, j, m);
      }
  } else if (bd == CYL_BD_X_MAX) {
    for (int m = 0; m < M; ++m)
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        if (STAG_X[st]) for (int i = 1; i <= NG - 1; ++i) f(nx + i, j, m) = f(nx - i, j, m);
        else for (int i = 1; i <= NG; ++i) f(nx + i, j, m) = f(nx + 1 - i, j, m);
      }
  } else if (bd == CYL_BD_Y_MAX) {
    for (int m = 0; m < M; ++m) {
      if (STAG_Y[st]) {
        for (int i = 1; i <= NG - 1; ++i)
          for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, ny + i, m) = f(ix, ny - i, m);
      } else {
        for (int i = 1; i <= NG; ++i)
          for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, ny + i, m) = f(ix, ny + 1 - i, m);
      }
    }
  }
}

// field_mode_clamp_zero (boundary.F90:772-829)
void clamp_zero(Sim& s, Field& f, int st, int bd) {
  if (s.bc_field[bd] == CYL_BC_PERIODIC) return;
  int nx = s.nx, ny = s.ny, M = s.M;
  const cplx Z = {0.0, 0.0};
  if (bd == CYL_BD_X_MIN) {
    for (int m = 0; m < M; ++m)
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        if (STAG_X[st]) {
          for (int i = 1; i <= NG - 1; ++i) f(i - NG, j, m) = -f(NG - i, j, m);
          f(0, j, m) = Z;
        } else {
          for (int i = 1; i <= NG; ++i) f(i - NG, j, m) = -f(NG + 1 - i, j, m);
        }
      }
  } else if (bd == CYL_BD_X_MAX) {
    for (int m = 0; m < M; ++m)
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        if (STAG_X[st]) {
          f(nx, j, m) = Z;
          for (int i = 1; i <= NG - 1; ++i) f(nx + i, j, m) = -f(nx - i, j, m);
        } else {
          for (int i = 1; i <= NG; ++i) f(nx + i, j, m) = -f(nx + 1 - i, j, m);
        }
      }
  } else if (bd == CYL_BD_Y_MAX) {
    for (int m = 0; m < M; ++m) {
      if (STAG_Y[st]) {
        for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, ny, m) = Z;
        for (int i = 1; i <= NG - 1; ++i)
          for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, ny + i, m) = -f(ix, ny - i, m);
      } else {
        for (int i = 1; i <= NG; ++i)
          for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, ny + i, m) = -f(ix, ny + 1 - i, m);
      }
    }
  }
}

// efield_bcs (boundary.F90:1355-1413)
void efield_bcs(Sim& s) {
  halo_shifted(s, s.ex);
  halo_full(s, s.er);
  halo_shifted(s, s.et);
  for (int i = CYL_BD_X_MIN; i <= CYL_BD_X_MAX; ++i) {
    if (s.bc_field[i] == CYL_BC_CONDUCT) {
      clamp_zero(s, s.ex, 0, i);
      zero_gradient(s, s.er, 1, i);
      zero_gradient(s, s.et, 2, i);
    }
  }
  if (s.bc_field[CYL_BD_Y_MAX] == CYL_BC_CONDUCT) {
    zero_gradient(s, s.ex, 0, CYL_BD_Y_MAX);
    clamp_zero(s, s.er, 1, CYL_BD_Y_MAX);
    zero_gradient(s, s.et, 2, CYL_BD_Y_MAX);
  }
  for (int i = 0; i < 4; ++i) {
    if (i == CYL_BD_Y_MIN) continue;
    int b = s.bc_field[i];
    if (b == CYL_BC_CLAMP || b == CYL_BC_SIMPLE_LASER || b == CYL_BC_SIMPLE_OUTFLOW) {
      clamp_zero(s, s.ex, 0, i);
      clamp_zero(s, s.er, 1, i);
      clamp_zero(s, s.et, 2, i);
    }
    if (b == CYL_BC_ZERO_GRADIENT) {
      zero_gradient(s, s.ex, 0, i);
      zero_gradient(s, s.er, 1, i);
      zero_gradient(s, s.et, 2, i);
    }
  }
}

// bfield_bcs (boundary.F90:1417-1476)
void bfield_bcs(Sim& s, bool mpi_only) {
  halo_full(s, s.bx);
  halo_shifted(s, s.br);
  halo_full(s, s.bt);
  if (mpi_only) return;
  for (int i = CYL_BD_X_MIN; i <= CYL_BD_X_MAX; ++i) {
    if (s.bc_field[i] == CYL_BC_CONDUCT) {
      zero_gradient(s, s.bx, 3, i);
      clamp_zero(s, s.br, 4, i);
      clamp_zero(s, s.bt, 5, i);
    }
  }
  if (s.bc_field[CYL_BD_Y_MAX] == CYL_BC_CONDUCT) {
    clamp_zero(s, s.bx, 3, CYL_BD_Y_MAX);
    zero_gradient(s, s.br, 4, CYL_BD_Y_MAX);
    clamp_zero(s, s.bt, 5, CYL_BD_Y_MAX);
  }
  for (int i = 0; i < 4; ++i) {
    if (i == CYL_BD_Y_MIN) continue;
    int b = s.bc_field[i];
    if (b == CYL_BC_CLAMP || b == CYL_BC_SIMPLE_LASER || b == CYL_BC_SIMPLE_OUTFLOW) {
      clamp_zero(s, s.bx, 3, i);
      clamp_zero(s, s.br, 4, i);
      clamp_zero(s, s.bt, 5, i);
    }
    if (b == CYL_BC_ZERO_GRADIENT) {
      zero_gradient(s, s.bx, 3, i);
      zero_gradient(s, s.br, 4, i);
      zero_gradient(s, s.bt, 5, i);
    }
  }
}

// ------------------------------------------------------------- Yee solver

// update_e_field (fields.f90:53-182); y_min_boundary is true on one rank.
void update_e_field(Sim& s) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  const double dx = s.dx, dy = s.dy, dt = s.dt, c2 = C * C;
  for (int im = 0; im < M; ++im) {
    for (int ir = 1; ir <= ny; ++ir) {
      double r_d = std::fabs((double)(ir - 1) * dy + s.y_grid_min);
      double r_p = r_d + 0.5 * dy;
      double fac_x = c2 / r_p;
      cplx im_fac_x = (IMAGI * (double)im) * fac_x;
      cplx im_fac_r = ((IMAGI * (double)im) * c2) / r_d;
      for (int ix = 0; ix <= nx; ++ix) {
        s.ex(ix, ir, im) = s.ex(ix, ir, im) +
            ((((fac_x * 0.5) * (s.bt(ix, ir + 1, im) + s.bt(ix, ir, im)) +
               im_fac_x * s.br(ix, ir, im)) +
              (c2 * (s.bt(ix, ir + 1, im) - s.bt(ix, ir, im))) / dy) -
             s.jx(ix, ir, im) / EPS0) * 0.5 * dt;
        s.er(ix, ir, im) = s.er(ix, ir, im) +
            ((-(im_fac_r * s.bx(ix, ir, im)) -
              (c2 * (s.bt(ix + 1, ir, im) - s.bt(ix, ir, im))) / dx) -
             s.jr(ix, ir, im) / EPS0) * 0.5 * dt;
        s.et(ix, ir, im) = s.et(ix, ir, im) +
            (((c2 * (s.br(ix + 1, ir, im) - s.br(ix, ir, im))) / dx -
              (c2 * (s.bx(ix, ir + 1, im) - s.bx(ix, ir, im))) / dy) -
             s.jt(ix, ir, im) / EPS0) * 0.5 * dt;
      }
    }
  }
  // r = 0 axis rules, fields.f90:116-180
  const int a = 1 - NG, b = nx + NG;
  for (int ix = a; ix <= b; ++ix) {
    s.ex(ix, 0, 0) = s.ex(ix, 0, 0) +
        ((4.0 * c2 / dy) * s.bt(ix, 1, 0) - s.jx(ix, 0, 0) / EPS0) * 0.5 * dt;
    s.et(ix, 0, 0) = mk(0.0, 0.0);
    s.er(ix, 0, 0) = -s.er(ix, 1, 0);
    for (int ir = 1 - NG; ir <= -1; ++ir) {
      s.et(ix, ir, 0) = -s.et(ix, -ir, 0);
      s.er(ix, ir, 0) = -s.er(ix, -ir + 1, 0);
      s.ex(ix, ir, 0) = s.ex(ix, -ir, 0);
    }
  }
  if (M > 1) {
    for (int ix = a; ix <= b; ++ix) {
      s.ex(ix, 0, 1) = mk(0.0, 0.0);
      s.er(ix, 0, 1) = (2.0 * IMAGI) * s.et(ix, 0, 1) - s.er(ix, 1, 1);
      s.et(ix, 0, 1) = (-IMAGI / 8.0) * (9.0 * s.er(ix, 1, 1) - s.er(ix, 2, 1));
      for (int ir = 1 - NG; ir <= -1; ++ir) {
        s.et(ix, ir, 1) = s.et(ix, -ir, 1);
        s.er(ix, ir, 1) = s.er(ix, -ir + 1, 1);
        s.ex(ix, ir, 1) = -s.ex(ix, -ir, 1);
      }
    }
  }
  if (M > 2) {
    double mode_sign = 1.0;
    for (int im = 2; im < M; ++im) {
      for (int ix = a; ix <= b; ++ix) {
        s.ex(ix, 0, im) = mk(0.0, 0.0);
        s.et(ix, 0, im) = mk(0.0, 0.0);
        s.er(ix, 0, im) = -s.er(ix, 1, im);
        s.er(ix, 1, im) = s.er(ix, 2, im) / 9.0;
        for (int ir = 1 - NG; ir <= -1; ++ir) {
          s.et(ix, ir, im) = (-mode_sign) * s.et(ix, -ir, im);
          s.er(ix, ir, im) = (-mode_sign) * s.er(ix, -ir + 1, im);
          s.ex(ix, ir, im) = mode_sign * s.ex(ix, -ir, im);
        }
      }
      mode_sign = -mode_sign;
    }
  }
}

// update_b_field (fields.f90:186-312)
void update_b_field(Sim& s) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  const double dx = s.dx, dy = s.dy, dt = s.dt;
  const int ir_max = ny - 1;  // y_max_boundary
  for (int im = 0; im < M; ++im) {
    for (int ir = 1; ir <= ir_max; ++ir) {
      double r_d = std::fabs((double)(ir - 1) * dy + s.y_grid_min);
      double r_p = r_d + 0.5 * dy;
      cplx im_fac_x = (IMAGI * (double)im) / r_d;
      cplx im_fac_r = (IMAGI * (double)im) / r_p;
      for (int ix = 0; ix <= nx; ++ix) {
        s.bx(ix, ir, im) = s.bx(ix, ir, im) -
            ((im_fac_x * s.er(ix, ir, im) +
              (0.5 * (s.et(ix, ir, im) + s.et(ix, ir - 1, im))) / r_d) +
             (s.et(ix, ir, im) - s.et(ix, ir - 1, im)) / dy) * 0.5 * dt;
        s.br(ix, ir, im) = s.br(ix, ir, im) +
            (im_fac_r * s.ex(ix, ir, im) +
             (s.et(ix, ir, im) - s.et(ix - 1, ir, im)) / dx) * 0.5 * dt;
        s.bt(ix, ir, im) = s.bt(ix, ir, im) +
            (-((s.er(ix, ir, im) - s.er(ix - 1, ir, im)) / dx) +
             (s.ex(ix, ir, im) - s.ex(ix, ir - 1, im)) / dy) * 0.5 * dt;
      }
    }
  }
  const int a = 1 - NG, b = nx + NG;
  for (int ix = a; ix <= b; ++ix) {
    s.br(ix, 0, 0) = mk(0.0, 0.0);
    s.bx(ix, 0, 0) = s.bx(ix, 1, 0);
    s.bt(ix, 0, 0) = -s.bt(ix, 1, 0);
    for (int ir = 1 - NG; ir <= -1; ++ir) {
      s.bt(ix, ir, 0) = -s.bt(ix, -ir + 1, 0);
      s.br(ix, ir, 0) = -s.br(ix, -ir, 0);
      s.bx(ix, ir, 0) = s.bx(ix, -ir + 1, 0);
    }
  }
  if (M > 1) {
    for (int ix = a; ix <= b; ++ix) s.bx(ix, 0, 1) = -s.bx(ix, 1, 1);
    // (22) Lifschitz: whole-array update, right-hand side uses old values only
    std::vector<cplx> tmp(b - a + 1);
    for (int ix = 2 - NG; ix <= b; ++ix)
      tmp[ix - a] = s.br(ix, 0, 1) +
          ((IMAGI / s.dy) * s.ex(ix, 0, 1) + (s.et(ix, 0, 1) - s.et(ix - 1, 0, 1)) / dx) * 0.5 * dt;
    for (int ix = 2 - NG; ix <= b; ++ix) s.br(ix, 0, 1) = tmp[ix - a];
    for (int ix = a; ix <= b; ++ix) {
      s.bt(ix, 0, 1) = (-2.0 * IMAGI) * s.br(ix, 0, 1) - s.bt(ix, 1, 1);
      for (int ir = 1 - NG; ir <= -1; ++ir) {
        s.bt(ix, ir, 1) = s.bt(ix, -ir + 1, 1);
        s.br(ix, ir, 1) = s.br(ix, -ir, 1);
        s.bx(ix, ir, 1) = -s.bx(ix, -ir + 1, 1);
      }
    }
  }
  if (M > 2) {
    double mode_sign = 1.0;
    for (int im = 2; im < M; ++im) {
      for (int ix = a; ix <= b; ++ix) {
        s.bx(ix, 0, im) = -s.bx(ix, 1, im);
        s.br(ix, 0, im) = mk(0.0, 0.0);
        s.bt(ix, 0, im) = -s.bt(ix, 1, im);
        for (int ir = 1 - NG; ir <= -1; ++ir) {
          s.bt(ix, ir, im) = (-mode_sign) * s.bt(ix, -ir + 1, im);
          s.br(ix, ir, im) = (-mode_sign) * s.br(ix, -ir, im);
          s.bx(ix, ir, im) = mode_sign * s.bx(ix, -ir + 1, im);
        }
      }
      mode_sign = -mode_sign;
    }
  }
}

// -------------------------------------------------------- laser / outflow

double laser_time_profile(const Laser& L, double time) {
  if (L.d.t_profile == 1) {
    double v = (time - L.d.t0) / L.d.tw;
    return std::exp(-(v * v));
  }
  return 1.0;
}

// update_laser_omegas (laser.f90:276-328): an omega that is a deck function
// (laser_update_omega, evaluated by the caller's callback) integrates the
// phase with the current dt, the others give omega * time.
void update_laser_omegas(Sim& s) {
  for (size_t i = 0; i < s.lasers.size(); ++i) {
    Laser& L = s.lasers[i];
    if (s.fns.laser_omega && ((s.fns.omega_fn_mask >> i) & 1u)) {
      double om = L.d.omega;
      s.fns.laser_omega(s.fns.user, (int32_t)i, s.time, &om);
      L.d.omega = om;
      L.current_integral_phase = L.current_integral_phase + L.d.omega * s.dt;
    } else {
      L.current_integral_phase = L.d.omega * s.time;
    }
  }
}

void laser_sources(Sim& s, int bd, std::vector<double>& s1, std::vector<double>& s2) {
  s1.assign(s.ny + 1, 0.0);
  s2.assign(s.ny + 1, 0.0);
  if (!s.add_laser[bd]) return;
  for (size_t i = 0; i < s.lasers.size(); ++i) {
    Laser& L = s.lasers[i];
    if (L.d.boundary != bd) continue;
    if (s.time >= L.d.t_start && s.time <= L.d.t_end) {
      // laser.f90:449-451: phase and profile functions, then the time profile
      const cyl_deck_fns& f = s.fns;
      if (f.laser_phase && ((f.phase_fn_mask >> i) & 1u)) f.laser_phase(f.user, (int32_t)i, s.time, L.phase.data());
      if (f.laser_profile && ((f.profile_fn_mask >> i) & 1u))
        f.laser_profile(f.user, (int32_t)i, s.time, L.profile.data());
      double tp;
      if (f.laser_time) f.laser_time(f.user, (int32_t)i, s.time, &tp);
      else tp = laser_time_profile(L, s.time);
      double t_env = tp * L.d.amp;
      for (int ir = 0; ir <= s.ny; ++ir) {
        double base = t_env * L.profile[ir] * std::sin(L.current_integral_phase + L.phase[ir]);
        s1[ir] = s1[ir] + base * std::cos(L.d.pol_angle);
        s2[ir] = s2[ir] + base * std::sin(L.d.pol_angle);
      }
    }
  }
}

// outflow_bcs_x_min (laser.f90:411-520).  The Bt line divides by the whole
// array r_d_vals(0:ny) inside a 1:ny section; element k of the section pairs
// with r_d_vals(k-1) (array elements are taken in order), reproduced here.
void outflow_bcs_x_min(Sim& s) {
  const int ny = s.ny, M = s.M;
  const double dtc2 = s.dt * (C * C), lx = dtc2 / s.dx, lr = dtc2 / s.dy;
  const double sum = 1.0 / (lx + C), diff = lx - C, dt_eps = s.dt / EPS0;
  std::vector<double> s1, s2;
  for (int m = 0; m < M; ++m)
    for (int ir = 0; ir <= ny; ++ir) s.bx(0, ir, m) = s.bx_xmin(ir, m);
  laser_sources(s, CYL_BD_X_MIN, s1, s2);
  std::vector<double> rdv(ny + 1);
  for (int ir = 0; ir <= ny; ++ir) rdv[ir] = std::fabs((double)(ir - 1) * s.dy + s.y_grid_min);
  for (int im = 0; im < M; ++im) {
    std::vector<cplx> st(ny + 1, mk(0, 0)), sr(ny + 1, mk(0, 0));
    if (im == 1)
      for (int ir = 0; ir <= ny; ++ir) {
        st[ir] = s1[ir] + IMAGI * s2[ir];
        sr[ir] = (-IMAGI) * s1[ir] + s2[ir];
      }
    cplx imc = ((IMAGI * (double)im) * (C * C)) * s.dt;
    std::vector<cplx> nbt(ny + 1);
    for (int ir = 1; ir <= ny; ++ir) {
      nbt[ir] = sum * (((((4.0 * st[ir] +
                          2.0 * (s.er_xmin(ir, im) + C * s.bt_xmin(ir, im))) -
                         2.0 * s.er(1, ir, im)) +
                        (imc * s.bx(1, ir, im)) / rdv[ir - 1]) +
                       dt_eps * s.jr(1, ir, im)) +
                      diff * s.bt(2, ir, im));
    }
    for (int ir = 1; ir <= ny; ++ir) s.bt(1, ir, im) = nbt[ir];
    const int ir_l = 1, ir_h = ny - 1;
    std::vector<cplx> nbr(ny + 1);
    for (int ir = ir_l; ir <= ir_h; ++ir) {
      nbr[ir] = sum * ((((((-4.0) * sr[ir] -
                           2.0 * (s.et_xmin(ir, im) + C * s.br_xmin(ir, im))) +
                          2.0 * s.et(1, ir, im)) -
                         lr * (s.bx(1, ir + 1, im) - s.bx(1, ir, im))) -
                        dt_eps * s.jt(1, ir, im)) +
                       diff * s.br(2, ir, im));
    }
    for (int ir = ir_l; ir <= ir_h; ++ir) s.br(1, ir, im) = nbr[ir];
  }
}

// outflow_bcs_x_max (laser.f90:524-633); the Bt line uses the whole arrays
// source_t(0:ny) and r_d_vals(0:ny) inside a 1:ny section (element k pairs
// with index k-1), reproduced here.
void outflow_bcs_x_max(Sim& s) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  const double dtc2 = s.dt * (C * C), lx = dtc2 / s.dx, lr = dtc2 / s.dy;
  const double sum = 1.0 / (lx + C), diff = lx - C, dt_eps = s.dt / EPS0;
  std::vector<double> s1, s2;
  for (int m = 0; m < M; ++m)
    for (int ir = 0; ir <= ny; ++ir) s.bx(nx, ir, m) = s.bx_xmax(ir, m);
  laser_sources(s, CYL_BD_X_MAX, s1, s2);
  std::vector<double> rdv(ny + 1);
  for (int ir = 0; ir <= ny; ++ir) rdv[ir] = std::fabs((double)(ir - 1) * s.dy + s.y_grid_min);
  for (int im = 0; im < M; ++im) {
    std::vector<cplx> st(ny + 1, mk(0, 0)), sr(ny + 1, mk(0, 0));
    if (im == 1)
      for (int ir = 0; ir <= ny; ++ir) {
        st[ir] = s1[ir] + IMAGI * s2[ir];
        sr[ir] = (-IMAGI) * s1[ir] + s2[ir];
      }
    cplx imc = ((IMAGI * (double)im) * (C * C)) * s.dt;
    std::vector<cplx> nbt(ny + 1);
    for (int ir = 1; ir <= ny; ++ir) {
      nbt[ir] = sum * ((((((-4.0) * st[ir - 1] -
                           2.0 * (s.er_xmax(ir, im) + C * s.bt_xmax(ir, im))) +
                          2.0 * s.er(nx - 1, ir, im)) -
                         (imc * s.bx(nx - 1, ir, im)) / rdv[ir - 1]) -
                        dt_eps * s.jr(nx - 1, ir, im)) +
                       diff * s.bt(nx - 1, ir, im));
    }
    for (int ir = 1; ir <= ny; ++ir) s.bt(nx, ir, im) = nbt[ir];
    const int ir_l = 1, ir_h = ny - 1;
    std::vector<cplx> nbr(ny + 1);
    for (int ir = ir_l; ir <= ir_h; ++ir) {
      nbr[ir] = sum * (((((4.0 * sr[ir] +
                          2.0 * (s.et_xmax(ir, im) + C * s.br_xmax(ir, im))) -
                         2.0 * s.et(nx - 1, ir, im)) +
                        lr * (s.bx(nx - 1, ir + 1, im) - s.bx(nx - 1, ir, im))) +
                       dt_eps * s.jt(nx - 1, ir, im)) +
                      diff * s.br(nx - 1, ir, im));
    }
    for (int ir = ir_l; ir <= ir_h; ++ir) s.br(nx, ir, im) = nbr[ir];
  }
}

// outflow_bcs_r_max (laser.f90:637-690)
void outflow_bcs_r_max(Sim& s) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  const double dt = s.dt, dtc2 = dt * (C * C);
  const double inv_r = 1.0 / ((double)((float)ny - 1.5f) * s.dy + s.y_grid_min);
  const double dtc2_4r = 0.25 * dtc2 * inv_r;
  const cplx icdt_2r = ((0.5 * IMAGI) * C) * dt * inv_r;
  const double lx = dtc2 / s.dx, ly = dtc2 / s.dy;
  const double sum_x = 1.0 / (ly + C), sum_t = 1.0 / ((ly + C) + dtc2_4r);
  const double dt_2eps = 0.5 * dt / EPS0;
  const int ix_l = 1, ix_h = nx - 1;
  for (int im = 0; im < M; ++im) {
    std::vector<cplx> nbx(nx + 2), nbt(nx + 2);
    const cplx icm = icdt_2r * (double)im;
    for (int ix = ix_l; ix <= ix_h; ++ix) {
      cplx t = (-s.bx(ix, ny - 1, im)) * (C - ly);
      t = t - s.bx_old(ix, ny, im) * ((-C) + ly);
      t = t - s.bx_old(ix, ny - 1, im) * ((-C) - ly);
      t = t - ((C * dt) * inv_r) * s.et(ix, ny - 1, im);
      t = t + (0.5 * lx) * (((s.br(ix + 1, ny - 1, im) - s.br(ix, ny - 1, im)) +
                             s.br_old(ix + 1, ny - 1, im)) - s.br_old(ix, ny - 1, im));
      t = t - icm * (s.er(ix, ny, im) + s.er(ix, ny - 1, im));
      t = t - dt_2eps * (s.jt(ix, ny - 1, im) + s.jt_old(ix, ny - 1, im));
      nbx[ix] = sum_x * t;
    }
    for (int ix = 1; ix <= nx; ++ix) {
      cplx t = (-s.bt(ix, ny - 1, im)) * ((C - ly) + dtc2_4r);
      t = t - s.bt_old(ix, ny, im) * (((-C) + ly) + dtc2_4r);
      t = t - s.bt_old(ix, ny - 1, im) * (((-C) - ly) + dtc2_4r);
      t = t - ((0.5 * lx) / C) * (((s.er(ix, ny, im) + s.er(ix, ny - 1, im)) - s.er(ix - 1, ny, im)) -
                                  s.er(ix - 1, ny - 1, im));
      t = t - (icm * C) * (s.br(ix, ny - 1, im) + s.br_old(ix, ny - 1, im));
      t = t + dt_2eps * (s.jx(ix, ny - 1, im) + s.jx_old(ix, ny - 1, im));
      nbt[ix] = sum_t * t;
    }
    for (int ix = ix_l; ix <= ix_h; ++ix) s.bx(ix, ny, im) = nbx[ix];
    for (int ix = 1; ix <= nx; ++ix) s.bt(ix, ny, im) = nbt[ix];
  }
}

// bfield_final_bcs (boundary.F90:1505-1537)
void bfield_final_bcs(Sim& s) {
  update_laser_omegas(s);
  bfield_bcs(s, false);
  if (s.add_laser[CYL_BD_X_MIN] || s.bc_field[CYL_BD_X_MIN] == CYL_BC_SIMPLE_OUTFLOW)
    outflow_bcs_x_min(s);
  if (s.add_laser[CYL_BD_X_MAX] || s.bc_field[CYL_BD_X_MAX] == CYL_BC_SIMPLE_OUTFLOW)
    outflow_bcs_x_max(s);
  if (s.bc_field[CYL_BD_Y_MAX] == CYL_BC_SIMPLE_OUTFLOW) {
    outflow_bcs_r_max(s);
  } else if (s.bc_field[CYL_BD_Y_MAX] == CYL_BC_ZERO_B) {
    for (int m = 0; m < s.M; ++m)
      for (int ix = 1 - NG; ix <= s.nx + NG; ++ix) {
        s.bx(ix, s.ny, m) = mk(0, 0);
        s.br(ix, s.ny, m) = mk(0, 0);
        s.bt(ix, s.ny, m) = mk(0, 0);
      }
  }
  bfield_bcs(s, true);
}

// ------------------------------------------------------------- currents

// current_bcs_r_min_final (boundary.F90:1909-1959)
void current_bcs_r_min_final(Sim& s) {
  const int a = 1 - NG, b = s.nx + NG;
  double mode_sign = 1.0;
  for (int im = 0; im < s.M; ++im) {
    for (int j = 2; j <= JNG; ++j) {
      for (int ix = a; ix <= b; ++ix) {
        s.jx(ix, j - 1, im) = s.jx(ix, j - 1, im) + mode_sign * s.jx(ix, 1 - j, im);
        s.jr(ix, j, im) = s.jr(ix, j, im) - mode_sign * s.jr(ix, 1 - j, im);
        s.jt(ix, j - 1, im) = s.jt(ix, j - 1, im) - mode_sign * s.jt(ix, 1 - j, im);
        s.jx(ix, 1 - j, im) = mk(0, 0);
        s.jr(ix, 1 - j, im) = mk(0, 0);
        s.jt(ix, 1 - j, im) = mk(0, 0);
      }
    }
    for (int ix = a; ix <= b; ++ix) s.jr(ix, 1, im) = s.jr(ix, 1, im) - mode_sign * s.jr(ix, 0, im);
    mode_sign = -mode_sign;
  }
  for (int im = 0; im < s.M; ++im) {
    for (int ix = a; ix <= b; ++ix) {
      if (im > 0) s.jx(ix, 0, im) = mk(0, 0);
      else s.jx(ix, 0, im) = (4.0 * s.jx(ix, 1, im) - s.jx(ix, 2, im)) / 3.0;
      if (im == 1) {
        s.jt(ix, 0, im) = ((-IMAGI) * (9.0 * s.jr(ix, 1, im) - s.jr(ix, 2, im))) / 8.0;
        s.jr(ix, 0, im) = (2.0 * IMAGI) * s.jt(ix, 0, im) - s.jr(ix, 1, im);
      } else {
        s.jt(ix, 0, im) = mk(0, 0);
        s.jr(ix, 0, im) = -s.jr(ix, 1, im);
      }
    }
  }
}

// particle_reflection_bcs_complex (boundary.F90:918-1015), flip 1=x 2=y 3=z
void reflection_bcs(Sim& s, Field& f, int flip) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  const cplx Z = mk(0, 0);
  for (int m = 0; m < M; ++m) {
    if (s.bc_allspecies[CYL_BD_X_MIN] == CYL_BC_REFLECT) {
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        if (flip == 1) {
          for (int i = 1; i <= NG - 1; ++i) { f(i, j, m) = f(i, j, m) - f(1 - i, j, m); f(1 - i, j, m) = Z; }
        } else {
          for (int i = 1; i <= NG - 1; ++i) { f(i, j, m) = f(i, j, m) + f(-i, j, m); f(-i, j, m) = Z; }
        }
      }
    }
    if (s.bc_allspecies[CYL_BD_X_MAX] == CYL_BC_REFLECT) {
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        if (flip == 1) {
          for (int i = 1; i <= NG; ++i) { f(nx + 1 - i, j, m) = f(nx + 1 - i, j, m) - f(nx + i, j, m); f(nx + i, j, m) = Z; }
        } else {
          for (int i = 1; i <= NG; ++i) { f(nx - i, j, m) = f(nx - i, j, m) + f(nx + i, j, m); f(nx + i, j, m) = Z; }
        }
      }
    }
    if (s.bc_allspecies[CYL_BD_Y_MAX] == CYL_BC_REFLECT) {
      const double r_max = s.y_grid_min + ((double)ny - 0.5) * s.dy;
      for (int i = 1; i <= NG; ++i) {
        for (int ix = 1 - NG; ix <= nx + NG; ++ix) {
          if (flip == 2) {
            f(ix, ny + 1 - i, m) = f(ix, ny + 1 - i, m) -
                (f(ix, ny + i, m) * (r_max + ((double)i - 0.5) * s.dy)) / (r_max - ((double)i - 0.5) * s.dy);
          } else if (flip == 1) {
            f(ix, ny - i, m) = f(ix, ny - i, m) +
                (f(ix, ny + i, m) * (r_max + (double)i * s.dy)) / (r_max - (double)i * s.dy);
          } else {
            f(ix, ny - i, m) = f(ix, ny - i, m) + f(ix, ny + i, m);
          }
          f(ix, ny + i, m) = Z;
        }
      }
    }
  }
}

// particle_periodic_bcs_complex on one rank (boundary.F90:1133-1245)
void periodic_sum(Sim& s, Field& f) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  for (int m = 0; m < M; ++m) {
    bool px = s.bc_allspecies[CYL_BD_X_MIN] == CYL_BC_PERIODIC;  // both sides
    for (int j = 1 - NG; j <= ny + NG; ++j) {
      for (int i = 1; i <= NG; ++i) {
        cplx t = px ? f(nx + i, j, m) : mk(0.0, 0.0);
        f(i, j, m) = f(i, j, m) + t;
      }
    }
    for (int j = 1 - NG; j <= ny + NG; ++j) {
      for (int i = 1; i <= NG; ++i) {
        cplx t = px ? f(i - NG, j, m) : mk(0.0, 0.0);
        f(nx - NG + i, j, m) = f(nx - NG + i, j, m) + t;
      }
    }
    for (int i = 1; i <= NG; ++i)
      for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, i, m) = f(ix, i, m) + mk(0.0, 0.0);
    for (int i = 1; i <= NG; ++i)
      for (int ix = 1 - NG; ix <= nx + NG; ++ix) f(ix, ny - NG + i, m) = f(ix, ny - NG + i, m) + mk(0.0, 0.0);
  }
}

// current_finish (current_smooth.F90:29-45) with current_bcs (boundary.F90:1893-1905)
void smooth_mode_array(Sim& s, Field& f);
void current_finish(Sim& s) {
  reflection_bcs(s, s.jx, 1);
  periodic_sum(s, s.jx);
  reflection_bcs(s, s.jr, 2);
  periodic_sum(s, s.jr);
  reflection_bcs(s, s.jt, 3);
  periodic_sum(s, s.jt);
  halo_full(s, s.jx);
  halo_full(s, s.jr);
  halo_full(s, s.jt);
  if (s.smooth) {
    smooth_mode_array(s, s.jx);
    smooth_mode_array(s, s.jr);
    smooth_mode_array(s, s.jt);
  }
}

// smooth_mode_array (current_smooth.F90:145-196), sng = jng
void smooth_mode_array(Sim& s, Field& f) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  Field wk;
  wk.init(nx, ny, M);
  wk.a = f.a;
  double alpha = 0.5, beta = (1.0 - alpha) * 0.25;
  const int its = s.smooth_its, comp = s.smooth_comp_its, cs = s.smooth_stride;
  for (int it = 1; it <= its + comp; ++it) {
    halo_full(s, wk);
    for (int im = 0; im < M; ++im)
      for (int iy = 1; iy <= ny; ++iy)
        for (int ix = 1; ix <= nx; ++ix)
          f(ix, iy, im) = alpha * wk(ix, iy, im) +
              (((wk(ix - cs, iy, im) + wk(ix + cs, iy, im)) + wk(ix, iy - cs, im)) + wk(ix, iy + cs, im)) * beta;
    for (int im = 0; im < M; ++im)
      for (int iy = 1; iy <= ny; ++iy)
        for (int ix = 1; ix <= nx; ++ix) wk(ix, iy, im) = f(ix, iy, im);
    if (it > its) alpha = (double)its * 0.5 + 1.0;
  }
  for (int im = 0; im < M; ++im)
    for (int iy = 1; iy <= ny; ++iy)
      for (int ix = 1; ix <= nx; ++ix) f(ix, iy, im) = wk(ix, iy, im);
}

// ------------------------------------------------------------ particles

int g_threads = 1;

// theta = ATAN2(z, y) of push_particles (particles.F90:321,522).  The
// reference calls the platform libm (gfortran's ATAN2 is the C library's
// atan2), and so does the oracle by default.  Mode 1 evaluates the shared
// correctly rounded cyl_atan2 of include/cyl_math.h instead, the routine the
// CUDA kernel runs: libm's atan2 is one ulp off on about 0.09 % of
// arguments (glibc 2.39), and the deposit's (m dtheta)^-2 factors carry such
// an ulp into J_theta (2e-12 after one push, up to 7e-9 relative after 20
// steps of a thermal plasma), so multi-step comparisons at 1e-10 use mode 1.
int g_atan2_mode = 0;
inline double theta_of(double z, double y) { return g_atan2_mode ? cyl_atan2(z, y) : std::atan2(z, y); }

struct Geom {
  std::vector<double> inv_area_rt, inv_area_xt, inv_volume, ratio_area_xt;
  int lo;  // index offset: arrays start at 1-jng (inv_area_xt at 0-jng)
};

// push_particles geometry tables (particles.F90:189-217)
void make_geom(const Sim& s, Geom& g) {
  const int ny = s.ny;
  const double dy = s.dy, dx = s.dx;
  g.inv_area_rt.assign(ny + 2 * JNG, 0.0);      // 1-jng .. ny+jng
  g.inv_area_xt.assign(ny + 2 * JNG + 1, 0.0);  // 0-jng .. ny+jng
  double r_low = s.y_grid_min - JNG * dy;
  g.inv_area_xt[0] = 1.0 / (2.0 * PI * std::fabs(r_low) * dx);
  for (int iy = 1 - JNG; iy <= ny + JNG; ++iy) {
    if (std::nearbyint(2.0 * r_low / dy) == -1.0)
      g.inv_area_rt[iy - (1 - JNG)] = 1.0 / (PI * ((0.5 * dy) * (0.5 * dy)));
    else
      g.inv_area_rt[iy - (1 - JNG)] = 1.0 / (PI * std::fabs((r_low + dy) * (r_low + dy) - r_low * r_low));
    g.inv_area_xt[iy - (0 - JNG)] = 1.0 / (2.0 * PI * std::fabs(r_low + dy) * dx);
    r_low = r_low + dy;
  }
  g.inv_volume.resize(ny + 2 * JNG);
  g.ratio_area_xt.resize(ny + 2 * JNG);
  for (int iy = 1 - JNG; iy <= ny + JNG; ++iy) {
    g.inv_volume[iy - (1 - JNG)] = g.inv_area_rt[iy - (1 - JNG)] / dx;
    g.ratio_area_xt[iy - (1 - JNG)] = g.inv_area_xt[iy - (0 - JNG)] / g.inv_area_xt[iy - 1 - (0 - JNG)];
  }
}

// Fortran integer division truncates toward zero, as C++ does.
inline int fdiv2(int v) { return v / 2; }

// The body of push_particles for one particle (particles.F90:270-665).
void push_one(Sim& s, const Geom& g, Species& spc, size_t i, double part_q, double part_mc,
              double ipart_mc, double cmratio, double ccmratio, Field& JX, Field& JR, Field& JT) {
  const double fac = 0.25;  // (0.5)**c_ndims
  const double idx = 1.0 / s.dx, idy = 1.0 / s.dy, idt = 1.0 / s.dt;
  const double dto2 = s.dt / 2.0, dtco2 = C * dto2;
  const double third = 1.0 / 3.0, sixth = 0.5 * third;
  const double x_grid_min_local = s.x_grid_min, y_grid_min_local = s.y_grid_min;
  double gx[5] = {0, 0, 0, 0, 0}, gy[5] = {0, 0, 0, 0, 0};  // index +2
  double hx[5], hy[5];
  double part_weight = spc.w[i];
  double part_x = spc.x[i], part_y = spc.y[i], part_z = spc.z[i];
  double part_ux = spc.px[i] * ipart_mc;
  double part_uy = spc.py[i] * ipart_mc;
  double part_uz = spc.pz[i] * ipart_mc;

  double gamma_rel = std::sqrt(((part_ux * part_ux + part_uy * part_uy) + part_uz * part_uz) + 1.0);
  double root = dtco2 / gamma_rel;
  part_x = part_x + part_ux * root;
  part_y = part_y + part_uy * root;
  part_z = part_z + part_uz * root;

  double part_x_local = part_x - x_grid_min_local;
  double part_r = std::sqrt(part_y * part_y + part_z * part_z);
  double part_r_local = part_r - y_grid_min_local;
  cplx exp_min_itheta = mk(part_y / part_r, (-part_z) / part_r);
  double theta_05 = theta_of(part_z, part_y);
  cplx exp_min_itheta_05 = exp_min_itheta;
  cplx exp_itheta_05 = crecip(exp_min_itheta_05);

  double cell_x_r = part_x_local * idx;
  double cell_y_r = part_r_local * idy;
  int cell_x1 = ffloor(cell_x_r + 0.5);
  double cell_frac_x = (double)cell_x1 - cell_x_r;
  cell_x1 = cell_x1 + 1;
  int cell_y1 = ffloor(cell_y_r + 0.5);
  double cell_frac_y = (double)cell_y1 - cell_y_r;
  cell_y1 = cell_y1 + 1;
  // triangle/gx.inc
  double cf2 = cell_frac_x * cell_frac_x;
  gx[1] = (0.25 + cf2) + cell_frac_x;
  gx[2] = 1.5 - 2.0 * cf2;
  gx[3] = (0.25 + cf2) - cell_frac_x;
  cf2 = cell_frac_y * cell_frac_y;
  gy[1] = (0.25 + cf2) + cell_frac_y;
  gy[2] = 1.5 - 2.0 * cf2;
  gy[3] = (0.25 + cf2) - cell_frac_y;

  int cell_x2 = ffloor(cell_x_r);
  cell_frac_x = ((double)cell_x2 - cell_x_r) + 0.5;
  cell_x2 = cell_x2 + 1;
  int cell_y2 = ffloor(cell_y_r);
  cell_frac_y = ((double)cell_y2 - cell_y_r) + 0.5;
  cell_y2 = cell_y2 + 1;
  int dcellx = 0, dcelly = 0;
  for (int k = 0; k < 5; ++k) { hx[k] = 0.0; hy[k] = 0.0; }
  // triangle/hx_dcell.inc
  cf2 = cell_frac_x * cell_frac_x;
  hx[dcellx - 1 + 2] = (0.25 + cf2) + cell_frac_x;
  hx[dcellx + 2] = 1.5 - 2.0 * cf2;
  hx[dcellx + 1 + 2] = (0.25 + cf2) - cell_frac_x;
  cf2 = cell_frac_y * cell_frac_y;
  hy[dcelly - 1 + 2] = (0.25 + cf2) + cell_frac_y;
  hy[dcelly + 2] = 1.5 - 2.0 * cf2;
  hy[dcelly + 1 + 2] = (0.25 + cf2) - cell_frac_y;

  // triangle/e_part.inc and b_part.inc
  cplx emi = mk(1.0, 0.0);
  double ex_part = 0.0, er_part = 0.0, et_part = 0.0;
  double bx_part = 0.0, br_part = 0.0, bt_part = 0.0;
  auto st3 = [&](Field& f, const double* wa, const double* wb, int ca, int cb, int m) {
    // wa weights along y (outer), wb weights along x (inner); ca = x cell, cb = y cell
    cplx acc = mk(0, 0);
    for (int jj = -1; jj <= 1; ++jj) {
      cplx inner = (wb[1] * f(ca - 1, cb + jj, m) + wb[2] * f(ca, cb + jj, m)) + wb[3] * f(ca + 1, cb + jj, m);
      if (jj == -1) acc = wa[jj + 2] * inner;
      else acc = acc + wa[jj + 2] * inner;
    }
    return acc;
  };
  for (int im = 0; im < s.M; ++im) {
    ex_part = ex_part + (emi * st3(s.ex, hy, gx, cell_x1, cell_y2, im)).re;
    er_part = er_part + (emi * st3(s.er, gy, hx, cell_x2, cell_y1, im)).re;
    et_part = et_part + (emi * st3(s.et, hy, hx, cell_x2, cell_y2, im)).re;
    emi = emi * exp_min_itheta;
  }
  double ey_part = er_part * exp_min_itheta.re + et_part * exp_min_itheta.im;
  double ez_part = (-er_part) * exp_min_itheta.im + et_part * exp_min_itheta.re;
  emi = mk(1.0, 0.0);
  for (int im = 0; im < s.M; ++im) {
    bx_part = bx_part + (emi * st3(s.bx, gy, hx, cell_x2, cell_y1, im)).re;
    br_part = br_part + (emi * st3(s.br, hy, gx, cell_x1, cell_y2, im)).re;
    bt_part = bt_part + (emi * st3(s.bt, gy, gx, cell_x1, cell_y1, im)).re;
    emi = emi * exp_min_itheta;
  }
  double by_part = br_part * exp_min_itheta.re + bt_part * exp_min_itheta.im;
  double bz_part = (-br_part) * exp_min_itheta.im + bt_part * exp_min_itheta.re;

  // Boris (particles.F90:404-451)
  double uxm = part_ux + cmratio * ex_part;
  double uym = part_uy + cmratio * ey_part;
  double uzm = part_uz + cmratio * ez_part;
  gamma_rel = std::sqrt(((uxm * uxm + uym * uym) + uzm * uzm) + 1.0);
  root = ccmratio / gamma_rel;
  double taux = bx_part * root, tauy = by_part * root, tauz = bz_part * root;
  double taux2 = taux * taux, tauy2 = tauy * tauy, tauz2 = tauz * tauz;
  double tau = 1.0 / (((1.0 + taux2) + tauy2) + tauz2);
  double uxp = ((((1.0 + taux2) - tauy2) - tauz2) * uxm +
                2.0 * ((taux * tauy + tauz) * uym + (taux * tauz - tauy) * uzm)) * tau;
  double uyp = ((((1.0 - taux2) + tauy2) - tauz2) * uym +
                2.0 * ((tauy * tauz + taux) * uzm + (tauy * taux - tauz) * uxm)) * tau;
  double uzp = ((((1.0 - taux2) - tauy2) + tauz2) * uzm +
                2.0 * ((tauz * taux + tauy) * uxm + (tauz * tauy - taux) * uym)) * tau;
  part_ux = uxp + cmratio * ex_part;
  part_uy = uyp + cmratio * ey_part;
  part_uz = uzp + cmratio * ez_part;

  double part_u2 = (part_ux * part_ux + part_uy * part_uy) + part_uz * part_uz;
  gamma_rel = std::sqrt(part_u2 + 1.0);
  double igamma = 1.0 / gamma_rel;
  root = dtco2 * igamma;
  double delta_x = part_ux * root, delta_y = part_uy * root, delta_z = part_uz * root;
  part_x = part_x + delta_x;
  part_y = part_y + delta_y;
  part_z = part_z + delta_z;
  spc.x[i] = part_x; spc.y[i] = part_y; spc.z[i] = part_z;
  spc.px[i] = part_mc * part_ux; spc.py[i] = part_mc * part_uy; spc.pz[i] = part_mc * part_uz;

  double part_vy = (part_uy * C) * igamma;
  double part_vz = (part_uz * C) * igamma;
  part_r = std::sqrt(part_y * part_y + part_z * part_z);
  cplx exp_itheta_10 = mk(part_y / part_r, part_z / part_r);
  double part_vt = (-part_vy) * exp_itheta_10.im + part_vz * exp_itheta_10.re;

  // current deposition (particles.F90:515-665)
  part_x_local = (part_x + delta_x) - x_grid_min_local;
  part_y = part_y + delta_y;
  part_z = part_z + delta_z;
  part_r = std::sqrt(part_y * part_y + part_z * part_z);
  part_r_local = part_r - y_grid_min_local;
  cplx exp_itheta_15 = mk(part_y / part_r, part_z / part_r);
  double theta_15 = theta_of(part_z, part_y);
  cplx exp_idtheta = exp_itheta_15 * exp_min_itheta_05;
  double dtheta = theta_15 - theta_05;
  for (int k = 0; k < 5; ++k) { gx[k] = hx[k]; gy[k] = hy[k]; }
  cell_x_r = part_x_local * idx;
  cell_y_r = part_r_local * idy;
  int cell_x3 = ffloor(cell_x_r);
  cell_frac_x = ((double)cell_x3 - cell_x_r) + 0.5;
  cell_x3 = cell_x3 + 1;
  int cell_y3 = ffloor(cell_y_r);
  cell_frac_y = ((double)cell_y3 - cell_y_r) + 0.5;
  cell_y3 = cell_y3 + 1;
  for (int k = 0; k < 5; ++k) { hx[k] = 0.0; hy[k] = 0.0; }
  dcellx = cell_x3 - cell_x2;
  dcelly = cell_y3 - cell_y2;
  cf2 = cell_frac_x * cell_frac_x;
  hx[dcellx - 1 + 2] = (0.25 + cf2) + cell_frac_x;
  hx[dcellx + 2] = 1.5 - 2.0 * cf2;
  hx[dcellx + 1 + 2] = (0.25 + cf2) - cell_frac_x;
  cf2 = cell_frac_y * cell_frac_y;
  hy[dcelly - 1 + 2] = (0.25 + cf2) + cell_frac_y;
  hy[dcelly + 2] = 1.5 - 2.0 * cf2;
  hy[dcelly + 1 + 2] = (0.25 + cf2) - cell_frac_y;
  for (int k = 0; k < 5; ++k) { hx[k] = hx[k] - gx[k]; hy[k] = hy[k] - gy[k]; }

  int xmin = SF_MIN + fdiv2(dcellx - 1), xmax = SF_MAX + fdiv2(dcellx + 1);
  int ymin = SF_MIN + fdiv2(dcelly - 1), ymax = SF_MAX + fdiv2(dcelly + 1);
  double q_weight_fac = (part_q * part_weight) * fac;
  double fcx = q_weight_fac * idt, fcy = q_weight_fac * idt, fcz = q_weight_fac * part_vt;

  cplx exp_imtheta0 = mk(1, 0), exp_imdtheta = mk(1, 0);
  cplx m_fac_1 = mk(0, 0), m_fac_2 = mk(0, 0), m_fac_3 = mk(0, 0), m_fac_4 = mk(0, 0);
  double inv_mdth = 0.0, inv_m2dth2 = 0.0;
  for (int im = 0; im < s.M; ++im) {
    double mdth = (double)im * dtheta;
    double m2dth2 = mdth * mdth;
    bool small = std::fabs(mdth) < 1.0e-4;
    if (!small && im > 0) {
      inv_mdth = 1.0 / mdth;
      inv_m2dth2 = inv_mdth * inv_mdth;
    }
    if (im == 0) {
      exp_imtheta0 = mk(1.0, 0.0);
      exp_imdtheta = mk(1.0, 0.0);
    } else {
      exp_imtheta0 = exp_imtheta0 * exp_itheta_05;
      exp_imdtheta = exp_imdtheta * exp_idtheta;
      if (small) {
        m_fac_1 = 2.0 * exp_imtheta0;
        m_fac_2 = m_fac_1 * ((mk(1.0, 0.0) + (0.5 * IMAGI) * mdth) - sixth * m2dth2);
        m_fac_3 = m_fac_1 * ((mk(0.5, 0.0) + (third * IMAGI) * mdth) - 0.125 * m2dth2);
        m_fac_4 = m_fac_1 * ((mk(third, 0.0) + (0.25 * IMAGI) * mdth) - 0.1 * m2dth2);
      } else {
        m_fac_1 = (2.0 * inv_mdth) * exp_imtheta0;
        m_fac_2 = m_fac_1 * ((-IMAGI) * (exp_imdtheta - 1.0));
        m_fac_3 = m_fac_1 * (inv_mdth * ((exp_imdtheta * (mk(1.0, 0.0) - IMAGI * mdth)) - 1.0));
        m_fac_4 = m_fac_1 * ((IMAGI * inv_m2dth2) *
                             ((exp_imdtheta * (((-m2dth2) - (2.0 * IMAGI) * mdth) + 2.0)) - 2.0));
      }
    }
    cplx jyh[5];
    for (int k = 0; k < 5; ++k) jyh[k] = mk(0, 0);
    for (int iy = ymin; iy <= ymax; ++iy) {
      int cy = cell_y2 + iy;
      cplx w_rt, ym_fac_1;
      if (im == 0) {
        w_rt = mk(gy[iy + 2] + 0.5 * hy[iy + 2], 0.0);
        ym_fac_1 = mk(0.5 * gy[iy + 2] + third * hy[iy + 2], 0.0);
      } else {
        w_rt = m_fac_2 * gy[iy + 2] + m_fac_3 * hy[iy + 2];
        ym_fac_1 = m_fac_3 * gy[iy + 2] + m_fac_4 * hy[iy + 2];
      }
      double fjx = fcx * g.inv_area_rt[cy - (1 - JNG)];
      double fjy = (fcy * hy[iy + 2]) * g.inv_area_xt[cy - (0 - JNG)];
      double fjz = fcz * g.inv_volume[cy - (1 - JNG)];
      double rat = g.ratio_area_xt[cy - (1 - JNG)];
      cplx jxh = mk(0, 0);
      for (int ix = xmin; ix <= xmax; ++ix) {
        int cx = cell_x2 + ix;
        cplx w_xt;
        if (im == 0) w_xt = mk(gx[ix + 2] + 0.5 * hx[ix + 2], 0.0);
        else w_xt = m_fac_2 * gx[ix + 2] + m_fac_3 * hx[ix + 2];
        cplx w_xr = gx[ix + 2] * w_rt + hx[ix + 2] * ym_fac_1;
        jxh = jxh - (fjx * hx[ix + 2]) * w_rt;
        jyh[ix + 2] = jyh[ix + 2] * rat - fjy * w_xt;
        cplx jzh = fjz * w_xr;
        JX(cx + 1, cy, im) = JX(cx + 1, cy, im) + jxh;
        JR(cx, cy + 1, im) = JR(cx, cy + 1, im) + jyh[ix + 2];
        JT(cx, cy, im) = JT(cx, cy, im) + jzh;
      }
    }
  }
}

// Per-mode charge density of the mobile species with the deposit's own
// staggered (h) shape, at the half-drifted position x + u c dt/2 / gamma: the
// t + dt/2 shape of the next push (particles.F90:304-312 for the drift,
// :369-388 for cell_x2 and the h weights, :548-571 for the same shape at
// t + 3 dt/2).  Mode m > 0 carries the 2 e^{i m theta} factor of m_fac_1
// (:595-611) and every cell the inv_volume of its row (:661), so that the
// deposit satisfies, per particle,
//   (rho' - rho)/dt + div_x J + div_r J - (i m / r_p) J_theta = 0
// exactly in its x and r parts (the theta part uses v_theta, :587).
void charge_density(Sim& s, Field& rho) {
  std::fill(rho.a.begin(), rho.a.end(), mk(0, 0));
  Geom g;
  make_geom(s, g);
  const double fac = 0.25;
  const double idx = 1.0 / s.dx, idy = 1.0 / s.dy;
  const double dtco2 = C * (s.dt / 2.0);
  for (auto& spc : s.sp) {
    if (spc.d.immobile) continue;
    const double part_q = spc.d.charge;
    const double ipart_mc = 1.0 / (C * spc.d.mass);
    for (size_t i = 0; i < spc.n(); ++i) {
      const double part_ux = spc.px[i] * ipart_mc, part_uy = spc.py[i] * ipart_mc, part_uz = spc.pz[i] * ipart_mc;
      const double gamma_rel = std::sqrt(((part_ux * part_ux + part_uy * part_uy) + part_uz * part_uz) + 1.0);
      const double root = dtco2 / gamma_rel;
      const double part_x = spc.x[i] + part_ux * root;
      const double part_y = spc.y[i] + part_uy * root;
      const double part_z = spc.z[i] + part_uz * root;
      const double part_r = std::sqrt(part_y * part_y + part_z * part_z);
      const cplx exp_itheta = crecip(mk(part_y / part_r, (-part_z) / part_r));
      const double cell_x_r = (part_x - s.x_grid_min) * idx;
      const double cell_y_r = (part_r - s.y_grid_min) * idy;
      int cell_x2 = ffloor(cell_x_r);
      const double fx = ((double)cell_x2 - cell_x_r) + 0.5;
      cell_x2 = cell_x2 + 1;
      int cell_y2 = ffloor(cell_y_r);
      const double fy = ((double)cell_y2 - cell_y_r) + 0.5;
      cell_y2 = cell_y2 + 1;
      double hx[3], hy[3];
      double cf2 = fx * fx;
      hx[0] = (0.25 + cf2) + fx; hx[1] = 1.5 - 2.0 * cf2; hx[2] = (0.25 + cf2) - fx;
      cf2 = fy * fy;
      hy[0] = (0.25 + cf2) + fy; hy[1] = 1.5 - 2.0 * cf2; hy[2] = (0.25 + cf2) - fy;
      const double qwf = part_q * spc.w[i] * fac;
      cplx mf = mk(1.0, 0.0), e_m = mk(1.0, 0.0);
      for (int im = 0; im < s.M; ++im) {
        if (im > 0) {
          e_m = e_m * exp_itheta;
          mf = 2.0 * e_m;
        }
        for (int iy = -1; iy <= 1; ++iy) {
          const int cy = cell_y2 + iy;
          const double fr = qwf * hy[iy + 1] * g.inv_volume[cy - (1 - JNG)];
          for (int ix = -1; ix <= 1; ++ix) {
            cplx& d = rho(cell_x2 + ix, cy, im);
            d = d + (fr * hx[ix + 1]) * mf;
          }
        }
      }
    }
  }
}

// particle_reflection_bcs for a real array, no flip (boundary.F90:833-915):
// the centre-staggered number density folds its ghost rows back at
// reflecting walls (applied to the real and imaginary parts alike).
void density_reflection(Sim& s, Field& f) {
  const int nx = s.nx, ny = s.ny, M = s.M;
  const cplx Z = mk(0.0, 0.0);
  for (int m = 0; m < M; ++m) {
    if (s.bc_allspecies[CYL_BD_X_MIN] == CYL_BC_REFLECT)
      for (int i = 1; i <= NG - 1; ++i)
        for (int j = 1 - NG; j <= ny + NG; ++j) {
          f(i, j, m) = f(i, j, m) + f(1 - i, j, m);
          f(1 - i, j, m) = Z;
        }
    if (s.bc_allspecies[CYL_BD_X_MAX] == CYL_BC_REFLECT)
      for (int i = 1; i <= NG; ++i)
        for (int j = 1 - NG; j <= ny + NG; ++j) {
          f(nx + 1 - i, j, m) = f(nx + 1 - i, j, m) + f(nx + i, j, m);
          f(nx + i, j, m) = Z;
        }
    if (s.bc_allspecies[CYL_BD_Y_MAX] == CYL_BC_REFLECT)
      for (int i = 1; i <= NG; ++i)
        for (int ix = 1 - NG; ix <= nx + NG; ++ix) {
          f(ix, ny + 1 - i, m) = f(ix, ny + 1 - i, m) + f(ix, ny + i, m);
          f(ix, ny + i, m) = Z;
        }
  }
}

// calc_number_density_modes (calc_df.F90:588-661) for species isp, or every
// species with particles when isp < 0: particle_to_grid.inc with
// triangle/gxfac.inc (cell-centred weights; gy folded for r < dy), the macro
// particle volume 2 pi dx dy r (partlist.F90:999-1013), the mode factor
// 2 e^{i m theta} for m > 0, then calc_boundary_modes (calc_df.F90:35-55:
// reflecting folds and periodic sums, no per-species bcs here) and
// field_mode_zero_gradient on every boundary with the centre stagger (not
// staggered along x or r, the stagger of btm).
void number_density_modes(Sim& s, Field& out, int isp) {
  std::fill(out.a.begin(), out.a.end(), mk(0, 0));
  for (size_t k = 0; k < s.sp.size(); ++k) {
    if (isp >= 0 && (int)k != isp) continue;
    const Species& spc = s.sp[k];
    for (size_t i = 0; i < spc.n(); ++i) {
      const double wdata = spc.w[i];
      const double part_r = std::sqrt(spc.y[i] * spc.y[i] + spc.z[i] * spc.z[i]);
      const double cell_x_r = (spc.x[i] - s.x_grid_min) / s.dx;
      const double cell_y_r = (part_r - s.y_grid_min) / s.dy;
      int cell_x = ffloor(cell_x_r + 0.5), cell_y = ffloor(cell_y_r + 0.5);
      const double fx = (double)cell_x - cell_x_r, fy = (double)cell_y - cell_y_r;
      cell_x = cell_x + 1;
      cell_y = cell_y + 1;
      double gx[3], gy[3];
      double c2 = fx * fx;
      gx[0] = 0.5 * ((0.25 + c2) + fx);
      gx[1] = 0.75 - c2;
      gx[2] = 0.5 * ((0.25 + c2) - fx);
      c2 = fy * fy;
      gy[0] = 0.5 * ((0.25 + c2) + fy);
      gy[1] = 0.75 - c2;
      gy[2] = 0.5 * ((0.25 + c2) - fy);
      if (part_r < s.dy) {
        gy[1] = gy[1] + gy[0];
        gy[0] = 0.0;
      }
      const double macro_part_volume = ((2.0 * PI) * s.dx) * s.dy * part_r;
      const double part_num_dens = wdata / macro_part_volume;
      const cplx exp_itheta = mk(spc.y[i] / part_r, spc.z[i] / part_r);
      cplx exp_imtheta = mk(1.0, 0.0), mode_fac = mk(1.0, 0.0);
      for (int im = 0; im < s.M; ++im) {
        if (im > 0) {
          exp_imtheta = exp_imtheta * exp_itheta;
          mode_fac = 2.0 * exp_imtheta;
        }
        for (int iy = -1; iy <= 1; ++iy)
          for (int ix = -1; ix <= 1; ++ix) {
            cplx& d = out(cell_x + ix, cell_y + iy, im);
            d = d + ((gx[ix + 1] * gy[iy + 1]) * part_num_dens) * mode_fac;
          }
      }
    }
  }
  density_reflection(s, out);
  periodic_sum(s, out);
  for (int bd = 0; bd < 4; ++bd) zero_gradient(s, out, 5, bd);
}

// push_particles without the trailing current_bcs_r_min_final / particle_bcs
void push_particles_core(Sim& s) {
  s.jx_old = s.jx; s.jr_old = s.jr; s.jt_old = s.jt;
  std::fill(s.jx.a.begin(), s.jx.a.end(), mk(0, 0));
  std::fill(s.jr.a.begin(), s.jr.a.end(), mk(0, 0));
  std::fill(s.jt.a.begin(), s.jt.a.end(), mk(0, 0));
  Geom g;
  make_geom(s, g);
  const double fac = 0.25;
  const double dtfac = 0.5 * s.dt * fac;
  for (auto& spc : s.sp) {
    if (spc.d.immobile) continue;
    double part_q = spc.d.charge;
    double part_mc = C * spc.d.mass;
    double ipart_mc = 1.0 / part_mc;
    double cmratio = (part_q * dtfac) * ipart_mc;
    double ccmratio = C * cmratio;
    if (g_threads <= 1) {
      for (size_t i = 0; i < spc.n(); ++i)
        push_one(s, g, spc, i, part_q, part_mc, ipart_mc, cmratio, ccmratio, s.jx, s.jr, s.jt);
      continue;
    }
    // Multi-threaded timing form (CPU baseline only): private current
    // arrays per thread, summed afterwards; positions are unaffected.
    const int nt = g_threads;
    std::vector<Field>& pj = s.thread_j;
    if ((int)pj.size() != 3 * nt) {
      pj.assign(3 * nt, Field());
      for (auto& f : pj) f.init(s.nx, s.ny, s.M);
    }
    const long long n = (long long)spc.n();
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int t = 0; t < nt; ++t) {
      for (int c = 0; c < 3; ++c) std::fill(pj[3 * t + c].a.begin(), pj[3 * t + c].a.end(), mk(0, 0));
      const long long a = n * t / nt, b = n * (t + 1) / nt;
      for (long long i = a; i < b; ++i)
        push_one(s, g, spc, (size_t)i, part_q, part_mc, ipart_mc, cmratio, ccmratio, pj[3 * t], pj[3 * t + 1],
                 pj[3 * t + 2]);
    }
    Field* dst[3] = {&s.jx, &s.jr, &s.jt};
    const size_t ne = s.jx.a.size();
#pragma omp parallel for num_threads(nt) schedule(static)
    for (long long e = 0; e < (long long)ne; ++e)
      for (int t = 0; t < nt; ++t)
        for (int c = 0; c < 3; ++c) dst[c]->a[e] = dst[c]->a[e] + pj[3 * t + c].a[e];
  }
}

// particle_bcs (boundary.F90:1541-1889) on one rank.  Particles sent to a
// neighbour (= this rank for periodic wraps) are appended at the list tail.
void particle_bcs(Sim& s) {
  const double bshift_x = s.dx * (double)((1 + PNG + 0) / 2);
  const double x_min_outer = s.x_min - bshift_x, x_max_outer = s.x_max + bshift_x;
  const double x_shift = s.length_x + 2.0 * s.dx * 0.0;
  const double bshift_y = s.dy * (double)((1 + PNG + 0) / 2);
  const double y_max_outer = s.y_max + bshift_y;
  const double y_shift = s.length_y + 2.0 * s.dy * 0.0;
  for (auto& spc : s.sp) {
    const size_t n = spc.n();
    std::vector<char> dead(n, 0), moved(n, 0);
    for (size_t i = 0; i < n; ++i) {
      int xbd = 0, ybd = 0;
      bool oob = false;
      int bc = 0;
      double part_pos = spc.x[i];
      if (part_pos < s.x_min_local) {
        xbd = -1;
        xbd = 0;
        bc = spc.bc[CYL_BD_X_MIN];
        if (bc == CYL_BC_REFLECT) {
          spc.x[i] = 2.0 * s.x_min - part_pos;
          spc.px[i] = -spc.px[i];
        } else if (bc == CYL_BC_PERIODIC) {
          xbd = -1;
          spc.x[i] = part_pos - (-1.0) * x_shift;
        }
        if (part_pos < x_min_outer && bc != CYL_BC_PERIODIC) oob = true;
      }
      if (part_pos >= s.x_max_local) {
        xbd = 1;
        xbd = 0;
        bc = spc.bc[CYL_BD_X_MAX];
        if (bc == CYL_BC_REFLECT) {
          spc.x[i] = 2.0 * s.x_max - part_pos;
          spc.px[i] = -spc.px[i];
        } else if (bc == CYL_BC_PERIODIC) {
          xbd = 1;
          spc.x[i] = part_pos - 1.0 * x_shift;
        }
        if (part_pos >= x_max_outer && bc != CYL_BC_PERIODIC) oob = true;
      }
      part_pos = std::sqrt(spc.y[i] * spc.y[i] + spc.z[i] * spc.z[i]);
      if (part_pos >= s.y_max_local) {
        ybd = 1;
        ybd = 0;
        bc = spc.bc[CYL_BD_Y_MAX];
        if (bc == CYL_BC_REFLECT) {
          double rr = 2.0 * s.y_max / part_pos - 1.0;
          spc.y[i] = spc.y[i] * rr;
          spc.z[i] = spc.z[i] * rr;
          double inv_final_r = 1.0 / std::sqrt(spc.y[i] * spc.y[i] + spc.z[i] * spc.z[i]);
          double ct = spc.y[i] * inv_final_r, stt = spc.z[i] * inv_final_r;
          double ppr = spc.py[i] * ct + spc.pz[i] * stt;
          double ppt = (-spc.py[i]) * stt + spc.pz[i] * ct;
          spc.py[i] = (-ppr) * ct - ppt * stt;
          spc.pz[i] = (-ppr) * stt + ppt * ct;
        } else if (bc == CYL_BC_PERIODIC) {
          ybd = 1;
          spc.y[i] = part_pos - 1.0 * y_shift;
        }
        if (part_pos >= y_max_outer && bc != CYL_BC_PERIODIC) oob = true;
      }
      if (oob) dead[i] = 1;
      else if (std::abs(xbd) + std::abs(ybd) > 0) moved[i] = 1;
    }
    // keep order: stay, then the wrapped ones appended
    Species tail;
    for (size_t i = 0; i < n; ++i)
      if (moved[i] && !dead[i])
        tail.push_back(spc.x[i], spc.y[i], spc.z[i], spc.px[i], spc.py[i], spc.pz[i], spc.w[i], spc.id[i]);
    std::vector<char> drop(n, 0);
    for (size_t i = 0; i < n; ++i) drop[i] = dead[i] || moved[i];
    spc.erase_mask(drop);
    for (size_t i = 0; i < tail.n(); ++i)
      spc.push_back(tail.x[i], tail.y[i], tail.z[i], tail.px[i], tail.py[i], tail.pz[i], tail.w[i], tail.id[i]);
  }
}

// --------------------------------------------------------- moving window

double density_at(const cyl_species_desc& d, double x) {
  if (d.density_kind == 1) {
    double f = (x - d.ramp_x0) / d.ramp_length;
    if (f < 0.0) f = 0.0;
    if (f > 1.0) f = 1.0;
    return d.density * f;
  }
  return d.density;
}

// insert_particles with the counter stream: the same rows, weights,
// temperatures and drifts, the random numbers from Philox counters instead
// of the KISS sequence; immobile species get none.
void insert_particles_counter(Sim& s) {
  const int ny = s.ny;
  const uint32_t shift = (uint32_t)s.n_shifts;
  for (size_t isp = 0; isp < s.sp.size(); ++isp) {
    Species& spc = s.sp[isp];
    const cyl_species_desc& d = spc.d;
    if (d.immobile) continue;
    const int64_t nppc = (int64_t)std::floor(d.npart_per_cell);
    const double npart_frac = d.npart_per_cell - (double)nppc;
    double dens = density_at(d, s.xg(s.nx));
    if (dens > d.density_max) dens = d.density_max;
    if (dens < d.density_min) dens = 0.0;
    if (dens < d.density_min) continue;
    const double x0 = s.x_grid_max + 0.5 * s.dx;
    int64_t j = 0;
    for (int iy = 1; iy <= ny; ++iy) {
      int64_t n_frac = 0;
      if (npart_frac > 0.0 &&
          ctr_u01(philox10(Ctr4{{(uint32_t)iy, shift, (uint32_t)isp, 3u}}, s.inj_seed).w[0]) < npart_frac)
        n_frac = 1;
      for (int64_t ip = 0; ip < nppc + n_frac; ++ip, ++j) {
        const Ctr4 r = philox10(Ctr4{{(uint32_t)j, shift, (uint32_t)isp, 4u}}, s.inj_seed);
        const double cell_frac_y = 0.5 - ctr_u01(r.w[0]);
        const double part_r = s.yg(iy) - cell_frac_y * s.dy;
        double sn, cs;
        cyl_sincos_turn(ctr_u01(r.w[1]), &sn, &cs);  // theta = 2 pi U
        const double px0 = x0 + ctr_u01(r.w[2]) * s.dx;
        const double wdata = (2.0 * PI * s.dx * s.dy * part_r) / (double)(nppc + n_frac);
        const double cy2 = cell_frac_y * cell_frac_y;
        const double gyv[3] = {0.5 * ((0.25 + cy2) + cell_frac_y), 0.75 - cy2,
                               0.5 * ((0.25 + cy2) - cell_frac_y)};
        double nrm[3];
        ctr_normals(philox10(Ctr4{{(uint32_t)j, shift, (uint32_t)isp, 5u}}, s.inj_seed), nrm);
        double pm[3];
        for (int i = 0; i < 3; ++i) {
          double tl = 0.0, dl = 0.0;
          for (int k = 0; k < 3; ++k) {
            tl = tl + gyv[k] * d.temp[i];
            dl = dl + gyv[k] * d.drift[i];
          }
          pm[i] = nrm[i] * std::sqrt(tl * KB * d.mass) + dl;
        }
        double wl = 0.0;
        for (int k = 0; k < 3; ++k) wl = wl + gyv[k] * dens;
        spc.push_back(px0, part_r * cs, part_r * sn, pm[0], pm[1], pm[2], wl * wdata, s.next_id++);
      }
    }
  }
}

// insert_particles (window.F90:157-300), thermal species
void insert_particles(Sim& s) {
  if (s.inj_counter) {
    insert_particles_counter(s);
    return;
  }
  const int ny = s.ny;
  for (auto& spc : s.sp) {
    const cyl_species_desc& d = spc.d;
    int64_t nppc = (int64_t)std::floor(d.npart_per_cell);
    double npart_frac = d.npart_per_cell - (double)nppc;
    double dmin = d.density_min, dmax = d.density_max;
    std::vector<double> density(ny + 2), temperature((ny + 2) * 3), drift((ny + 2) * 3);
    const double xpack = s.xg(s.nx);
    if (s.fns.inject) {
      // window.F90:196-212: the deck's columns at pack_ix = nx
      s.fns.inject(s.fns.user, (int32_t)(&spc - s.sp.data()), s.time, xpack, density.data(), temperature.data(),
                   drift.data());
    } else {
      for (int i = 0; i < 3; ++i)
        for (int iy = 0; iy <= ny + 1; ++iy) {
          temperature[iy + (ny + 2) * i] = d.temp[i];
          drift[iy + (ny + 2) * i] = d.drift[i];
        }
      for (int iy = 0; iy <= ny + 1; ++iy) density[iy] = density_at(d, xpack);
    }
    for (int iy = 0; iy <= ny + 1; ++iy) {
      if (density[iy] > dmax) density[iy] = dmax;
      if (density[iy] < dmin) density[iy] = 0.0;
    }
    double x0 = s.x_grid_max + 0.5 * s.dx;
    Species app;
    for (int iy = 1; iy <= ny; ++iy) {
      if (density[iy] < dmin) continue;
      int64_t n_frac = 0;
      if (npart_frac > 0.0) {
        if (s.rng.random() < npart_frac) n_frac = 1;
      }
      for (int64_t ip = 1; ip <= nppc + n_frac; ++ip) {
        double cell_frac_y = 0.5 - s.rng.random();
        double part_r = s.yg(iy) - cell_frac_y * s.dy;
        double part_theta = 2.0 * PI * s.rng.random();
        double px0 = x0 + s.rng.random() * s.dx;
        double py0 = part_r * std::cos(part_theta);
        double pz0 = part_r * std::sin(part_theta);
        double wdata = (2.0 * PI * s.dx * s.dy * part_r) / (double)(nppc + n_frac);
        double cy2 = cell_frac_y * cell_frac_y;
        double gyv[3];
        gyv[0] = 0.5 * ((0.25 + cy2) + cell_frac_y);
        gyv[1] = 0.75 - cy2;
        gyv[2] = 0.5 * ((0.25 + cy2) - cell_frac_y);
        double tl[3] = {0, 0, 0}, dl[3] = {0, 0, 0};
        for (int i = 0; i < 3; ++i)
          for (int isuby = -1; isuby <= 1; ++isuby) {
            tl[i] = tl[i] + gyv[isuby + 1] * temperature[iy + isuby + (ny + 2) * i];
            dl[i] = dl[i] + gyv[isuby + 1] * drift[iy + isuby + (ny + 2) * i];
          }
        double pm[3];
        for (int i = 0; i < 3; ++i) {
          double stdev = std::sqrt(tl[i] * KB * d.mass);
          pm[i] = s.rng.box_muller(stdev, dl[i]);
        }
        double wl = 0.0;
        for (int isuby = -1; isuby <= 1; ++isuby) wl = wl + gyv[isuby + 1] * density[iy + isuby];
        app.push_back(px0, py0, pz0, pm[0], pm[1], pm[2], wl * wdata, s.next_id++);
      }
    }
    for (size_t i = 0; i < app.n(); ++i)
      spc.push_back(app.x[i], app.y[i], app.z[i], app.px[i], app.py[i], app.pz[i], app.w[i], app.id[i]);
  }
}

// shift_field_modes (window.F90:136-153)
void shift_field_modes(Sim& s, Field& f) {
  for (int m = 0; m < s.M; ++m)
    for (int j = 1 - NG; j <= s.ny + NG; ++j)
      for (int i = 1 - NG; i <= s.nx + NG - 1; ++i) f(i, j, m) = f(i + 1, j, m);
  halo_full(s, f);
}

// shift_fields (window.F90:98-132)
void shift_fields(Sim& s) {
  shift_field_modes(s, s.ex); shift_field_modes(s, s.er); shift_field_modes(s, s.et);
  shift_field_modes(s, s.bx); shift_field_modes(s, s.br); shift_field_modes(s, s.bt);
  shift_field_modes(s, s.jx); shift_field_modes(s, s.jr); shift_field_modes(s, s.jt);
  const int nx = s.nx;
  for (int j = 1 - NG; j <= s.ny + NG; ++j)
    for (int m = 0; m < s.M; ++m) {
      s.ex(nx + 1, j, m) = s.ex_xmax(j, m);
      s.er(nx, j, m) = s.er_xmax(j, m);
      s.et(nx, j, m) = s.et_xmax(j, m);
      s.ex(nx, j, m) = 0.5 * (s.ex(nx - 1, j, m) + s.ex(nx + 1, j, m));
      s.er(nx - 1, j, m) = 0.5 * (s.er(nx - 2, j, m) + s.er(nx, j, m));
      s.et(nx - 1, j, m) = 0.5 * (s.et(nx - 2, j, m) + s.et(nx, j, m));
      s.bx(nx, j, m) = s.bx_xmax(j, m);
      s.br(nx + 1, j, m) = s.br_xmax(j, m);
      s.bt(nx + 1, j, m) = s.bt_xmax(j, m);
      s.bx(nx - 1, j, m) = 0.5 * (s.bx(nx - 2, j, m) + s.bx(nx, j, m));
      s.br(nx, j, m) = 0.5 * (s.br(nx - 1, j, m) + s.br(nx + 1, j, m));
      s.bt(nx, j, m) = 0.5 * (s.bt(nx - 1, j, m) + s.bt(nx + 1, j, m));
    }
}

// remove_particles (window.F90:304-325)
void remove_particles(Sim& s) {
  for (auto& spc : s.sp) {
    std::vector<char> dead(spc.n(), 0);
    for (size_t i = 0; i < spc.n(); ++i)
      if (spc.x[i] < s.x_min) dead[i] = 1;
    spc.erase_mask(dead);
  }
}

// shift_window (window.F90:62-94), cpml_thickness = 0
void shift_window(Sim& s, int cells) {
  for (int iw = 1; iw <= cells; ++iw) {
    insert_particles(s);
    s.x_grid_min = s.xg(1) + s.dx;
    s.xb_min = s.xb_min + s.dx;
    s.x_min = s.xb_min + s.dx * 0.0;
    s.x_max = (s.xb_min + (double)(s.nx + 1 - 1) * s.dx) - s.dx * 0.0;
    s.setup_grid_x();
    remove_particles(s);
    shift_fields(s);
    s.n_shifts++;
  }
}

// moving_window (window.F90:330-376)
void moving_window(Sim& s) {
  if (!s.move_window) return;
  if (!s.window_started) {
    if (s.time >= s.window_start_time && s.time < s.window_stop_time) {
      for (int i = 0; i < 4; ++i) s.bc_deck[i] = s.bc_after_move[i];
      s.setup_boundaries();
      if (!s.from_restart) s.window_shift_fraction = 0.0;  // window.F90:347
      s.window_started = true;
    }
  }
  if (s.window_started) {
    if (s.time >= s.window_stop_time) return;
    if (s.window_v_x <= 0.0) return;
    s.window_shift_fraction = s.window_shift_fraction + s.dt * s.window_v_x / s.dx;
    int cells = (int)std::floor(s.window_shift_fraction);
    if (cells > 0) {
      double real_cells = (double)cells;
      shift_window(s, cells);
      particle_bcs(s);
      s.window_shift_fraction = s.window_shift_fraction - real_cells;
    }
  }
}

// ------------------------------------------------------- field ionisation

// constants.F90:172-198
const double ION_Q0 = 1.602176565e-19, ION_M0 = 9.10938291e-31;
const double ION_HBAR = 1.054571725336289397963133257349698e-34;
const double ION_A0 = 5.291772101121111395947216558438464e-11;
const double ION_HARTREE = 4.359744350823120007758594450644308e-18;
const double ION_ATIME = 2.418884320905619591809404261549867e-17;
const double ION_AFIELD = 5.142206538736485312185213306837419e11;
const double ION_LARGEST_EXP = 1024.0 * 0.69314718055994530941723212145817657;
const double ION_TINY = 2.2250738585072014e-308, ION_HUGE = 1.7976931348623157e308;
const double ION_EXPONENT = -1.0 / 3.0;           // ionise.F90:27
const double ION_BESSEL = 1.5957691216057308;     // SQRT(8/pi), ionise.F90:28

// bessel_constant SQRT(x) EXP(x) RKBESL(x, 0.5, l + 1, 1): K_{l+1/2} by its
// finite closed form (Abramowitz & Stegun 10.2.15).
double ion_bessel_term(double x, int l) {
  double sum = 0.0, term = 1.0;
  for (int k = 0; k <= l; ++k) {
    if (k > 0) term = term * ((double)((l + k) * (l - k + 1)) / (double)k) / (2.0 * x);
    sum = sum + term;
  }
  const double kval = std::sqrt(PI / (2.0 * x)) * std::exp(-x) * sum;
  return std::sqrt(8.0 / PI) * std::sqrt(x) * std::exp(x) * kval;
}

// factorial, numerics.f90:24-40
double ion_factorial(double x) {
  double f = 1.0;
  for (int i = 2; i <= (int)x; ++i) {
    if (f < std::sqrt(ION_HUGE)) f = f * (double)i;
    else return ION_HUGE;
  }
  return f;
}

// initialise_ionisation (ionise.F90:51-286); GAMMA by the C library, integer
// powers expanded as gfortran expands them.
void initialise_ionisation(Sim& s, const cyl_ionisation_species* in, int n, int model, double omega) {
  const bool mp = model & CYL_IONISE_MULTIPHOTON, bsi = model & CYL_IONISE_BSI;
  const double omega_atomic = omega * ION_ATIME, c_atomic = C * ION_ATIME / ION_A0;
  s.ion.assign(n, Sim::IonSp{});
  for (int i = 0; i < n; ++i) {
    Sim::IonSp& o = s.ion[i];
    o.in = in[i];
    if (!in[i].ionise) continue;
    o.rmf = in[i].release >= 0 ? s.sp[in[i].release].d.mass / s.sp[i].d.mass : 0.0;
    const double ip = in[i].energy / ION_HARTREE;
    const double z = s.sp[in[i].ionise_to].d.charge / ION_Q0;
    double neff = z / std::sqrt(2.0 * ip);
    const double t = 2.0 * ip;
    o.adk_scaling = 2.0 * std::sqrt((t * t) * t);
    o.ion_const = std::sqrt(6.0 / PI) * ip * std::pow(2.0, 2.0 * neff) / (neff * std::tgamma(2.0 * neff));
    if (bsi) {
      o.bsi_const = ip * std::sqrt(2.0 * ip) / (2.0 * PI * z);
      o.bsi_scaling = (ip * ip) / (4.0 * z);
      const double u = 2.0 * neff, u2 = u * u;
      o.bsi_threshold = ((z * z) * z) / (u2 * u2);
      o.adk_max = std::fmax(o.adk_scaling / (3.0 * (2.0 * neff + (double)in[i].l - 1.5)), o.bsi_threshold);
    }
    if (mp) {
      const double k = (double)((int64_t)std::floor(ip / omega_atomic) + 1);
      double multi = ion_factorial(k);
      if (multi < std::sqrt(ION_HUGE)) {
        const int64_t nq = in[i].n, nq2 = nq * nq;
        multi = c_atomic * (multi * multi) * (double)((nq2 * nq2) * nq) *
                std::pow(omega_atomic, (10.0 * k - 1.0) / 3.0) * std::sqrt(k) * (2.0 * k + 1.0);
      } else {
        multi = 0.0;
      }
      if (std::fabs(multi) > ION_TINY) multi = 4.8 * std::pow(1.69 * c_atomic / (8.0 * PI * omega_atomic), k) / multi;
      o.multi_const = multi;
      o.k_energy = k * ION_HBAR * omega;
      o.k_exponent = 4.0 * k - 2.0;
    }
    neff = 2.0 * neff - 1.5;
    o.n_exp = neff;
    if (bsi) {
      const double x = o.adk_scaling / o.bsi_threshold;
      o.adk_bsi_cap = o.ion_const * std::pow(x, neff) * std::exp(ION_EXPONENT * x) * (ion_bessel_term(x, in[i].l) - 1.0);
    }
    if (mp) {
      o.keldysh = std::fmax(o.adk_scaling / (0.99472065388909858 * ION_LARGEST_EXP),
                            omega_atomic * std::sqrt(2.0 * ip) / 0.5);
      const double x = o.adk_scaling / o.keldysh;
      o.adk_mp_cap = o.ion_const * std::pow(x, neff) * std::exp(ION_EXPONENT * x) * (ion_bessel_term(x, in[i].l) - 1.0);
      if (std::fabs(o.multi_const) <= ION_TINY) o.smallest_e = ION_HUGE;
      else o.smallest_e = std::pow(ION_TINY / std::fmin(o.multi_const, 1.0), 1.0 / o.k_exponent);
    } else {
      o.smallest_e = o.adk_scaling / (0.99472065388909858 * ION_LARGEST_EXP);
    }
  }
}

// ionise_particles (ionise.F90:325-351) and its four models
// (multiphoton_tunnelling_bsi :355-657, multiphoton_tunnelling :661-950,
// tunnelling_bsi :954-1232, tunnelling :1236-1500), single rank.  The trial's
// random number is the counter stream's word (id, id >> 32, step,
// 6 + 16 species) in place of random(); released electrons take the id
// 2^62 + 16 parent id + species.
void ionise_particles(Sim& s) {
  const int nsp = (int)s.sp.size();
  const bool mp = s.ion_model & CYL_IONISE_MULTIPHOTON, bsi = s.ion_model & CYL_IONISE_BSI;
  const double fac = 0.25;
  const double idx = 1.0 / s.dx, idy = 1.0 / s.dy;
  const double dfac1 = fac * fac / (s.dt * 2.0 * PI * s.dx * s.dy);
  std::vector<Species> ionised(nsp);
  for (int i = 0; i < nsp; ++i) ionised[i].d = s.sp[i].d;
  auto st3 = [&](Field& f, const double* wa, const double* wb, int ca, int cb, int m) {
    cplx acc = mk(0, 0);
    for (int jj = -1; jj <= 1; ++jj) {
      cplx inner = (wb[1] * f(ca - 1, cb + jj, m) + wb[2] * f(ca, cb + jj, m)) + wb[3] * f(ca + 1, cb + jj, m);
      if (jj == -1) acc = wa[jj + 2] * inner;
      else acc = acc + wa[jj + 2] * inner;
    }
    return acc;
  };
  for (int i = 0; i < nsp; ++i) {
    if (!s.ion[i].in.ionise) continue;
    Species& spc = s.sp[i];
    const size_t n0 = spc.n();
    std::vector<char> gone(n0, 0);
    for (size_t p = 0; p < n0; ++p) {
      const double x0 = spc.x[p], y0 = spc.y[p], z0 = spc.z[p];
      const double part_x_local = x0 - s.x_grid_min;
      const double part_r = std::sqrt(y0 * y0 + z0 * z0);
      const double part_r_local = part_r - s.y_grid_min;
      const cplx exp_min_itheta = mk(y0 / part_r, (-z0) / part_r);
      const cplx exp_itheta = crecip(exp_min_itheta);
      const double dfac = dfac1 / part_r;
      double gx[5] = {0, 0, 0, 0, 0}, gy[5] = {0, 0, 0, 0, 0}, hx[5] = {0, 0, 0, 0, 0}, hy[5] = {0, 0, 0, 0, 0};
      const double cell_x_r = part_x_local * idx, cell_y_r = part_r_local * idy;
      int cell_x1 = ffloor(cell_x_r + 0.5);
      double cell_frac_x = (double)cell_x1 - cell_x_r;
      cell_x1 = cell_x1 + 1;
      int cell_y1 = ffloor(cell_y_r + 0.5);
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
      int cell_x2 = ffloor(cell_x_r);
      cell_frac_x = ((double)cell_x2 - cell_x_r) + 0.5;
      cell_x2 = cell_x2 + 1;
      int cell_y2 = ffloor(cell_y_r);
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
      // e_part.inc
      double ex_part = 0.0, er_part = 0.0, et_part = 0.0;
      cplx emi = mk(1.0, 0.0);
      for (int im = 0; im < s.M; ++im) {
        ex_part = ex_part + (emi * st3(s.ex, hy, gx, cell_x1, cell_y2, im)).re;
        er_part = er_part + (emi * st3(s.er, gy, hx, cell_x2, cell_y1, im)).re;
        et_part = et_part + (emi * st3(s.et, hy, hx, cell_x2, cell_y2, im)).re;
        emi = emi * exp_min_itheta;
      }
      const double ey_part = er_part * exp_min_itheta.re + et_part * exp_min_itheta.im;
      const double ez_part = (-er_part) * exp_min_itheta.im + et_part * exp_min_itheta.re;
      const double e_mag = fac * std::sqrt((ex_part * ex_part + ey_part * ey_part) + ez_part * ez_part) / ION_AFIELD;
      const int64_t pid = spc.id[p];
      double ppx = spc.px[p], ppy = spc.py[p], ppz = spc.pz[p];
      const double weight = spc.w[p];
      int cs = i;
      double time_left = s.dt / ION_ATIME, j_ion = 0.0;
      while (time_left > 0.0 && s.ion[cs].in.ionise) {
        const Sim::IonSp& q = s.ion[cs];
        bool multi = false;
        double rate;
        auto adk = [&]() {
          const double x = q.adk_scaling / e_mag;
          return q.ion_const * std::pow(x, q.n_exp) * std::exp(ION_EXPONENT * x) * (ion_bessel_term(x, q.in.l) - 1.0);
        };
        auto bsi_rate = [&]() { return q.bsi_const * (1.0 - q.bsi_scaling / e_mag) + q.adk_bsi_cap; };
        if (mp && bsi) {
          if (e_mag > q.adk_max) rate = bsi_rate();
          else if (e_mag > q.keldysh) {
            rate = adk();
            if (e_mag > q.bsi_threshold) rate = std::fmin(bsi_rate(), rate);
          } else if (e_mag > q.smallest_e) {
            rate = std::fmin(q.adk_mp_cap, q.multi_const * std::pow(e_mag, q.k_exponent));
            multi = true;
          } else break;
        } else if (mp) {
          if (e_mag > q.keldysh) rate = adk();
          else if (e_mag > q.smallest_e) {
            rate = std::fmin(q.adk_mp_cap, q.multi_const * std::pow(e_mag, q.k_exponent));
            multi = true;
          } else break;
        } else if (bsi) {
          if (e_mag > q.adk_max) rate = bsi_rate();
          else if (e_mag > q.smallest_e) {
            rate = adk();
            if (e_mag > q.bsi_threshold) rate = std::fmin(bsi_rate(), rate);
          } else break;
        } else {
          if (e_mag > q.smallest_e) rate = adk();
          else break;
        }
        const Ctr4 r = philox10(Ctr4{{(uint32_t)pid, (uint32_t)((uint64_t)pid >> 32), (uint32_t)s.step,
                                      6u | ((uint32_t)cs << 4)}}, s.ion_seed);
        const double sample = ctr_u01(r.w[0]);
        if (sample < 1.0 - std::exp(-1.0 * rate * time_left)) {
          if (q.in.release >= 0) {
            double ex_ = ppx * q.rmf, ey_ = ppy * q.rmf, ez_ = ppz * q.rmf;
            ppx = ppx - ex_;
            ppy = ppy - ey_;
            ppz = ppz - ez_;
            if (multi) {
              const double kick = std::sqrt(2.0 * ION_M0 * (q.k_energy - q.in.energy));
              const double den = e_mag * ION_AFIELD;
              ex_ = ex_ + kick * fac * ex_part / den;
              ey_ = ey_ + kick * fac * ey_part / den;
              ez_ = ez_ + kick * fac * ez_part / den;
            }
            s.sp[q.in.release].push_back(x0, y0, z0, ex_, ey_, ez_, weight,
                                         (int64_t)(((uint64_t)1 << 62) | ((uint64_t)pid << 4) | (uint64_t)cs));
          }
          time_left = time_left + std::log(1.0 - sample) / rate;
          j_ion = j_ion + (multi ? q.k_energy : q.in.energy);
          cs = q.in.ionise_to;
        } else {
          time_left = 0.0;
        }
      }
      if (cs == i) continue;
      gone[p] = 1;
      ionised[cs].push_back(x0, y0, z0, ppx, ppy, ppz, weight, pid);
      const double den = ION_AFIELD * e_mag;
      const double jf = dfac * j_ion * weight;
      const double jx_ion = jf * ex_part / (den * den), jy_ion = jf * ey_part / (den * den),
                   jz_ion = jf * ez_part / (den * den);
      if (std::fabs(jx_ion) > ION_TINY || std::fabs(jy_ion) > ION_TINY || std::fabs(jz_ion) > ION_TINY) {
        const double jr_ion = jy_ion * exp_itheta.re + jz_ion * exp_itheta.im;
        const double jt_ion = (-jy_ion) * exp_itheta.im + jz_ion * exp_itheta.re;
        cplx eim = mk(1.0, 0.0);
        for (int im = 0; im < s.M; ++im) {
          for (int iy = -1; iy <= 1; ++iy)
            for (int ix = -1; ix <= 1; ++ix) {
              s.jx(cell_x1 + ix, cell_y2 + iy, im) =
                  s.jx(cell_x1 + ix, cell_y2 + iy, im) + ((gx[ix + 2] * hy[iy + 2]) * jx_ion) * eim;
              s.jr(cell_x2 + ix, cell_y1 + iy, im) =
                  s.jr(cell_x2 + ix, cell_y1 + iy, im) + ((hx[ix + 2] * gy[iy + 2]) * jr_ion) * eim;
              s.jt(cell_x2 + ix, cell_y2 + iy, im) =
                  s.jt(cell_x2 + ix, cell_y2 + iy, im) + ((hx[ix + 2] * hy[iy + 2]) * jt_ion) * eim;
            }
          eim = eim * exp_itheta;
          if (im == 0) eim = eim * 2.0;
        }
      }
    }
    spc.erase_mask(gone);
  }
  for (int i = 0; i < nsp; ++i)
    for (size_t k = 0; k < ionised[i].n(); ++k)
      s.sp[i].push_back(ionised[i].x[k], ionised[i].y[k], ionised[i].z[k], ionised[i].px[k], ionised[i].py[k],
                        ionised[i].pz[k], ionised[i].w[k], ionised[i].id[k]);
}

// ---------------------------------------------------------------- driver

void update_eb_fields_half(Sim& s) {
  update_e_field(s);
  efield_bcs(s);
  s.bx_old = s.bx; s.br_old = s.br; s.bt_old = s.bt;
  update_b_field(s);
  bfield_bcs(s, true);
}
void update_eb_fields_final(Sim& s) {
  update_b_field(s);
  bfield_final_bcs(s);
  update_e_field(s);
  efield_bcs(s);
}

// One iteration of the driver loop up to output_routines (epoch2d.F90:213-262)
void step_to_output(Sim& s) {
  update_eb_fields_half(s);
  push_particles_core(s);
  current_bcs_r_min_final(s);
  particle_bcs(s);
  if (s.ion_on) ionise_particles(s);  // epoch2d.F90:251
  current_finish(s);
  s.step++;
  s.time = s.time + s.dt / 2.0;
}
// ... and the rest of it (epoch2d.F90:263-265)
void finish_step(Sim& s) {
  s.time = s.time + s.dt / 2.0;
  update_eb_fields_final(s);
  moving_window(s);
}
// One iteration of the driver loop (epoch2d.F90:213-265)
void one_step(Sim& s) {
  step_to_output(s);
  finish_step(s);
}

void compute_bc_allspecies(Sim& s) {
  for (int idx = 0; idx < 4; ++idx) {
    for (size_t i = 0; i < s.sp.size(); ++i) {
      int bc = s.sp[i].bc[idx];
      if (bc == CYL_BC_REFLECT) bc = CYL_BC_REFLECT;
      else if (bc != CYL_BC_PERIODIC) bc = CYL_BC_OPEN;
      if (i == 0) s.bc_allspecies[idx] = bc;
      else if (s.bc_allspecies[idx] != bc) s.bc_allspecies[idx] = 14;  // mixed
    }
    if (s.sp.empty()) s.bc_allspecies[idx] = CYL_BC_OPEN;
  }
}

int map_particle_bc(int b) {
  // setup_particle_boundary (boundary.F90:100-140)
  if (b == CYL_BC_OTHER || b == CYL_BC_CONDUCT) b = CYL_BC_REFLECT;
  if (b == CYL_BC_SIMPLE_LASER || b == CYL_BC_SIMPLE_OUTFLOW) b = CYL_BC_OPEN;
  return b;
}

// ----------------------------------------------------------------- loader

// The per-particle part of particle_to_grid.inc + gxfac.inc (triangle)
struct Shape {
  int cell_x, cell_y;
  double gx[3], gy[3];
};
Shape shape_at(const Sim& s, double px, double py, double pz) {
  Shape r;
  double part_r = std::sqrt(py * py + pz * pz);
  double cell_x_r = (px - s.x_grid_min) / s.dx;
  double cell_y_r = (part_r - s.y_grid_min) / s.dy;
  int cx = ffloor(cell_x_r + 0.5), cy = ffloor(cell_y_r + 0.5);
  double fx = (double)cx - cell_x_r, fy = (double)cy - cell_y_r;
  r.cell_x = cx + 1;
  r.cell_y = cy + 1;
  double cx2 = fx * fx;
  r.gx[0] = 0.5 * ((0.25 + cx2) + fx);
  r.gx[1] = 0.75 - cx2;
  r.gx[2] = 0.5 * ((0.25 + cx2) - fx);
  double cy2 = fy * fy;
  r.gy[0] = 0.5 * ((0.25 + cy2) + fy);
  r.gy[1] = 0.75 - cy2;
  r.gy[2] = 0.5 * ((0.25 + cy2) - fy);
  if (part_r < s.dy) {
    r.gy[1] = r.gy[1] + r.gy[0];
    r.gy[0] = 0.0;
  }
  return r;
}

// auto_load for one thermal species: setup_particle_density + load_particles
// (helper.F90:373-663, 669-811) and setup_particle_temperature x3
// (particle_temperature.F90:30-81).
// dens_in, temp_in, drift_in: the deck's density, temperature and drift on
// the ghosted grid, evaluated by the caller (NULL: the closed forms).
void load_species(Sim& s, Species& spc, const double* dens_in = nullptr, const double* temp_in = nullptr,
                  const double* drift_in = nullptr) {
  const cyl_species_desc& d = spc.d;
  const int nx = s.nx, ny = s.ny;
  const int W = nx + 2 * NG;
  auto at = [&](int ix, int iy) { return (size_t)(ix + NG - 1) + (size_t)W * (size_t)(iy + NG - 1); };
  std::vector<double> density((size_t)W * (ny + 2 * NG));
  std::vector<char> dmap(density.size(), 0);
  const size_t plane = density.size();
  for (int iy = 1 - NG; iy <= ny + NG; ++iy)
    for (int ix = 1 - NG; ix <= nx + NG; ++ix)
      density[at(ix, iy)] = dens_in ? dens_in[at(ix, iy)] : density_at(d, s.xg(ix));
  // field_bc(density): periodic x self-wrap only
  if (s.bc_field[CYL_BD_X_MAX] == CYL_BC_PERIODIC)
    for (int iy = 1 - NG; iy <= ny + NG; ++iy)
      for (int i = 1; i <= NG; ++i) density[at(nx + i, iy)] = density[at(i, iy)];
  if (s.bc_field[CYL_BD_X_MIN] == CYL_BC_PERIODIC)
    for (int iy = 1 - NG; iy <= ny + NG; ++iy)
      for (int i = 1 - NG; i <= 0; ++i) density[at(i, iy)] = density[at(nx + i, iy)];
  for (size_t k = 0; k < density.size(); ++k) {
    if (density[k] > d.density_max) density[k] = d.density_max;
    if (density[k] >= d.density_min) dmap[k] = 1;
    else density[k] = 0.0;
  }
  // load_particles: valid cells in the interior
  int64_t nvalid = 0;
  for (int iy = 1; iy <= ny; ++iy)
    for (int ix = 1; ix <= nx; ++ix)
      if (dmap[at(ix, iy)]) nvalid++;
  int64_t nppc = (int64_t)std::floor(d.npart_per_cell);
  int64_t nnew = (int64_t)std::floor(d.npart_per_cell * (double)nvalid);
  spc.x.clear(); spc.y.clear(); spc.z.clear(); spc.px.clear(); spc.py.clear(); spc.pz.clear();
  spc.w.clear(); spc.id.clear();
  int64_t left = nnew;
  if (nppc > 0) {
    for (int iy = 1; iy <= ny; ++iy)
      for (int ix = 1; ix <= nx; ++ix) {
        if (!dmap[at(ix, iy)]) continue;
        for (int64_t ip = 0; ip < nppc && (int64_t)spc.n() < nnew; ++ip) {
          double px0 = s.xg(ix) + (s.rng.random() - 0.5) * s.dx;
          double pr = s.yg(iy) + (s.rng.random() - 0.5) * s.dy;
          double th = 2.0 * PI * s.rng.random();
          spc.push_back(px0, pr * std::cos(th), pr * std::sin(th), 0, 0, 0, 0, s.next_id++);
          left--;
        }
      }
  }
  if (left > 0) {
    std::vector<int64_t> valid;
    for (int iy = 1; iy <= ny; ++iy)
      for (int ix = 1; ix <= nx; ++ix)
        if (dmap[at(ix, iy)]) valid.push_back((int64_t)(ix - 1) + (int64_t)nx * (iy - 1));
    for (int64_t i = 0; i < left; ++i) {
      int64_t ipos = (int64_t)(s.rng.random() * (double)(nvalid - 1)) + 1;
      ipos = valid[ipos - 1];
      int64_t cyy = ipos / nx;
      ipos = ipos - nx * cyy;
      int cell_y = (int)cyy + 1, cell_x = (int)ipos + 1;
      double px0 = s.xg(cell_x) + (s.rng.random() - 0.5) * s.dx;
      double pr = s.yg(cell_y) + (s.rng.random() - 0.5) * s.dy;
      double th = 2.0 * PI * s.rng.random();
      spc.push_back(px0, pr * std::cos(th), pr * std::sin(th), 0, 0, 0, 0, s.next_id++);
    }
  }
  particle_bcs(s);
  // weights (helper.F90:707-782)
  std::vector<int> npic((size_t)W * (ny + 2 * NG), 0);
  for (size_t p = 0; p < spc.n(); ++p) {
    Shape sh = shape_at(s, spc.x[p], spc.y[p], spc.z[p]);
    double wdata = 0.0;
    for (int isuby = SF_MIN; isuby <= SF_MAX; ++isuby) {
      int i = sh.cell_x;
      int j = sh.cell_y + isuby;
      if (!dmap[at(i, j)]) j = sh.cell_y + isuby / 2;
      for (int isubx = SF_MIN; isubx <= SF_MAX; ++isubx) {
        i = sh.cell_x + isubx;
        if (!dmap[at(i, j)]) i = sh.cell_x + isubx / 2;
        wdata = wdata + (sh.gx[isubx + 1] * sh.gy[isuby + 1]) * density[at(i, j)];
      }
    }
    spc.w[p] = wdata;
    npic[at(sh.cell_x, sh.cell_y)]++;
  }
  for (size_t p = 0; p < spc.n(); ++p) {
    double part_r = std::sqrt(spc.y[p] * spc.y[p] + spc.z[p] * spc.z[p]);
    int cx = ffloor((spc.x[p] - s.x_grid_min) / s.dx + 1.5);
    int cy = ffloor((part_r - s.y_grid_min) / s.dy + 1.5);
    double vol = 2.0 * PI * s.dx * s.dy * part_r;
    spc.w[p] = spc.w[p] * vol / (double)npic[at(cx, cy)];
  }
  // momenta: direction loop outer (helper.F90:139-142)
  for (int dir = 0; dir < 3; ++dir) {
    for (size_t p = 0; p < spc.n(); ++p) {
      Shape sh = shape_at(s, spc.x[p], spc.y[p], spc.z[p]);
      double tl = 0.0, dl = 0.0;
      // particle_temperature.F90:58-66: temperature(cell_x+ix, cell_y+iy)
      for (int iy = SF_MIN; iy <= SF_MAX; ++iy)
        for (int ix = SF_MIN; ix <= SF_MAX; ++ix) {
          const size_t c = at(sh.cell_x + ix, sh.cell_y + iy) + plane * (size_t)dir;
          tl = tl + (sh.gx[ix + 1] * sh.gy[iy + 1]) * (temp_in ? temp_in[c] : d.temp[dir]);
          dl = dl + (sh.gx[ix + 1] * sh.gy[iy + 1]) * (drift_in ? drift_in[c] : d.drift[dir]);
        }
      double stdev = std::sqrt(tl * KB * d.mass);
      double v = s.rng.box_muller(stdev, dl);
      if (dir == 0) spc.px[p] = v;
      else if (dir == 1) spc.py[p] = v;
      else spc.pz[p] = v;
    }
  }
}

// load_particles with the counter stream: the valid cells, counts, extra
// particles' cell rule, weights and temperatures of load_species, the random
// numbers from Philox counters (positions (p, species, 1), momenta
// (p, species, 2)); ids id_base + p.
void load_species_counter(Sim& s, Species& spc, int isp, uint64_t seed, int64_t id_base) {
  const cyl_species_desc& d = spc.d;
  const int nx = s.nx, ny = s.ny;
  const int W = nx + 2 * NG;
  auto at = [&](int ix, int iy) { return (size_t)(ix + NG - 1) + (size_t)W * (size_t)(iy + NG - 1); };
  std::vector<double> density((size_t)W * (ny + 2 * NG));
  std::vector<char> dmap(density.size(), 0);
  for (int iy = 1 - NG; iy <= ny + NG; ++iy)
    for (int ix = 1 - NG; ix <= nx + NG; ++ix) density[at(ix, iy)] = density_at(d, s.xg(ix));
  if (s.bc_field[CYL_BD_X_MAX] == CYL_BC_PERIODIC)
    for (int iy = 1 - NG; iy <= ny + NG; ++iy)
      for (int i = 1; i <= NG; ++i) density[at(nx + i, iy)] = density[at(i, iy)];
  if (s.bc_field[CYL_BD_X_MIN] == CYL_BC_PERIODIC)
    for (int iy = 1 - NG; iy <= ny + NG; ++iy)
      for (int i = 1 - NG; i <= 0; ++i) density[at(i, iy)] = density[at(nx + i, iy)];
  for (size_t k = 0; k < density.size(); ++k) {
    if (density[k] > d.density_max) density[k] = d.density_max;
    if (density[k] >= d.density_min) dmap[k] = 1;
    else density[k] = 0.0;
  }
  std::vector<std::pair<int, int>> valid;
  for (int iy = 1; iy <= ny; ++iy)
    for (int ix = 1; ix <= nx; ++ix)
      if (dmap[at(ix, iy)]) valid.push_back({ix, iy});
  const int64_t nvalid = (int64_t)valid.size();
  const int64_t nppc = (int64_t)std::floor(d.npart_per_cell);
  const int64_t nnew = (int64_t)std::floor(d.npart_per_cell * (double)nvalid);
  spc.x.clear(); spc.y.clear(); spc.z.clear(); spc.px.clear(); spc.py.clear(); spc.pz.clear();
  spc.w.clear(); spc.id.clear();
  for (int64_t p = 0; p < nnew; ++p) {
    const Ctr4 r = philox10(Ctr4{{(uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)isp, 1u}}, seed);
    const int64_t v = p < nppc * nvalid ? p / nppc : (int64_t)(ctr_u01(r.w[3]) * (double)(nvalid - 1));
    const int ix = valid[(size_t)v].first, iy = valid[(size_t)v].second;
    const double px0 = s.xg(ix) + (ctr_u01(r.w[0]) - 0.5) * s.dx;
    const double pr = s.yg(iy) + (ctr_u01(r.w[1]) - 0.5) * s.dy;
    double sn, cs;
    cyl_sincos_turn(ctr_u01(r.w[2]), &sn, &cs);  // theta = 2 pi U
    spc.push_back(px0, pr * cs, pr * sn, 0, 0, 0, 0, id_base + p);
  }
  std::vector<int> npic(density.size(), 0);
  for (size_t p = 0; p < spc.n(); ++p) {
    Shape sh = shape_at(s, spc.x[p], spc.y[p], spc.z[p]);
    npic[at(sh.cell_x, sh.cell_y)]++;
  }
  for (size_t p = 0; p < spc.n(); ++p) {
    Shape sh = shape_at(s, spc.x[p], spc.y[p], spc.z[p]);
    double wdata = 0.0;
    for (int isuby = SF_MIN; isuby <= SF_MAX; ++isuby) {
      int i = sh.cell_x;
      int j = sh.cell_y + isuby;
      if (!dmap[at(i, j)]) j = sh.cell_y + isuby / 2;
      for (int isubx = SF_MIN; isubx <= SF_MAX; ++isubx) {
        i = sh.cell_x + isubx;
        if (!dmap[at(i, j)]) i = sh.cell_x + isubx / 2;
        wdata = wdata + (sh.gx[isubx + 1] * sh.gy[isuby + 1]) * density[at(i, j)];
      }
    }
    const double part_r = std::sqrt(spc.y[p] * spc.y[p] + spc.z[p] * spc.z[p]);
    const int cx = ffloor((spc.x[p] - s.x_grid_min) / s.dx + 1.5);
    const int cy = ffloor((part_r - s.y_grid_min) / s.dy + 1.5);
    const double vol = 2.0 * PI * s.dx * s.dy * part_r;
    spc.w[p] = wdata * vol / (double)npic[at(cx, cy)];
    double nrm[3];
    ctr_normals(philox10(Ctr4{{(uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)isp, 2u}}, seed), nrm);
    for (int dir = 0; dir < 3; ++dir) {
      double tl = 0.0, dl = 0.0;
      for (int iy = SF_MIN; iy <= SF_MAX; ++iy)
        for (int ix = SF_MIN; ix <= SF_MAX; ++ix) {
          tl = tl + (sh.gx[ix + 1] * sh.gy[iy + 1]) * d.temp[dir];
          dl = dl + (sh.gx[ix + 1] * sh.gy[iy + 1]) * d.drift[dir];
        }
      const double v = nrm[dir] * std::sqrt(tl * KB * d.mass) + dl;
      if (dir == 0) spc.px[p] = v;
      else if (dir == 1) spc.py[p] = v;
      else spc.pz[p] = v;
    }
  }
  if (id_base + (int64_t)spc.n() > s.next_id) s.next_id = id_base + (int64_t)spc.n();
}

// kinetic energy (calc_df.F90:1246-1291) and per-mode field energy
void diagnostics(Sim& s, cyl_diag* out) {
  double ke = 0.0;
  int64_t n = 0;
  for (auto& spc : s.sp) {
    double mc = C * spc.d.mass, mc2 = C * mc;
    for (size_t i = 0; i < spc.n(); ++i) {
      double u2 = (spc.px[i] / mc) * (spc.px[i] / mc) + (spc.py[i] / mc) * (spc.py[i] / mc) +
                  (spc.pz[i] / mc) * (spc.pz[i] / mc);
      double gm1 = u2 / (std::sqrt(u2 + 1.0) + 1.0);
      ke += spc.w[i] * mc2 * gm1;
    }
    n += (int64_t)spc.n();
  }
  double fe = 0.0, fb = 0.0, js = 0.0;
  for (int m = 0; m < s.M; ++m) {
    double mf = (m == 0) ? 1.0 : 0.5;
    for (int iy = 1; iy <= s.ny; ++iy) {
      double r = (double)iy * s.dy;
      double vol = 2.0 * PI * r * s.dx * s.dy;
      for (int ix = 1; ix <= s.nx; ++ix) {
        auto a2 = [](cplx v) { return v.re * v.re + v.im * v.im; };
        fe += mf * vol * (a2(s.ex(ix, iy, m)) + a2(s.er(ix, iy, m)) + a2(s.et(ix, iy, m)));
        fb += mf * vol * (a2(s.bx(ix, iy, m)) + a2(s.br(ix, iy, m)) + a2(s.bt(ix, iy, m)));
        js += std::sqrt(a2(s.jx(ix, iy, m))) + std::sqrt(a2(s.jr(ix, iy, m))) + std::sqrt(a2(s.jt(ix, iy, m)));
      }
    }
  }
  out->kinetic_energy = ke;
  out->field_energy_e = 0.5 * EPS0 * fe;
  out->field_energy_b = 0.5 / (4.0e-7 * PI) * fb;
  out->jsum_abs = js;
  out->n_live = n;
  out->device_error = 0;
}

}  // namespace

// ============================================================== C API

extern "C" {

typedef struct orc_sim_s* orc_handle;

int orc_create(const cyl_grid_desc* g, const cyl_species_desc* sp, int32_t nsp,
               const cyl_laser_desc* las, int32_t nlas, int32_t seed, orc_handle* out) {
  if (!g || !out || g->nx < 4 || g->ny < 4 || g->n_mode < 1) return CYL_ERR_BAD_ARG;
  Sim* s = new Sim();
  s->nx = g->nx; s->ny = g->ny; s->M = g->n_mode;
  s->x_min = g->x_min; s->x_max = g->x_max; s->y_max = g->y_max;
  // setup_grid (setup.F90:164-206)
  s->length_x = s->x_max - s->x_min;
  s->dx = s->length_x / (double)(s->nx - 0);
  s->x_grid_min = s->x_min - s->dx * 0.0;
  s->length_y = s->y_max - 0.0;
  s->dy = s->length_y / (double)(s->ny - 0);
  s->y_grid_min = 0.0 - s->dy * 0.0;
  s->xb_min = s->x_grid_min;
  s->x_grid_min = s->x_grid_min + s->dx / 2.0;
  s->y_grid_min = s->y_grid_min + s->dy / 2.0;
  s->setup_grid_x();
  s->setup_grid_y();
  s->dt = g->dt;
  s->time = 0.0;
  s->step = 0;
  for (int i = 0; i < 4; ++i) { s->bc_deck[i] = g->bc_field[i]; s->bc_after_move[i] = g->bc_after_move[i]; }
  s->setup_boundaries();
  s->move_window = g->move_window != 0;
  s->window_started = false;
  s->window_v_x = g->window_v_x;
  s->window_start_time = g->window_start_time;
  s->window_stop_time = g->window_stop_time;
  s->window_shift_fraction = 0.0;
  s->n_shifts = 0;
  s->next_id = 0;
  s->smooth = g->smooth_currents;
  s->smooth_its = g->smooth_its;
  s->smooth_comp_its = g->smooth_comp_its;
  s->smooth_stride = g->smooth_stride > 0 ? g->smooth_stride : 1;
  Field* fs[15] = {&s->ex, &s->er, &s->et, &s->bx, &s->br, &s->bt, &s->jx, &s->jr, &s->jt,
                   &s->bx_old, &s->br_old, &s->bt_old, &s->jx_old, &s->jr_old, &s->jt_old};
  for (auto* f : fs) f->init(s->nx, s->ny, s->M);
  Col* cs[12] = {&s->ex_xmin, &s->er_xmin, &s->et_xmin, &s->bx_xmin, &s->br_xmin, &s->bt_xmin,
                 &s->ex_xmax, &s->er_xmax, &s->et_xmax, &s->bx_xmax, &s->br_xmax, &s->bt_xmax};
  for (auto* c : cs) c->init(s->ny, s->M);
  s->sp.resize(nsp);
  for (int i = 0; i < nsp; ++i) {
    s->sp[i].d = sp[i];
    for (int k = 0; k < 4; ++k) s->sp[i].bc[k] = map_particle_bc(sp[i].bc_particle[k]);
  }
  compute_bc_allspecies(*s);
  for (int i = 0; i < nlas; ++i) {
    Laser L;
    L.d = las[i];
    L.profile.assign(las[i].profile, las[i].profile + s->ny + 1);
    L.phase.assign(las[i].phase, las[i].phase + s->ny + 1);
    L.d.profile = nullptr;
    L.d.phase = nullptr;
    s->lasers.push_back(L);
  }
  s->rng.init(seed);
  *out = (orc_handle)s;
  return CYL_OK;
}

int orc_destroy(orc_handle h) {
  delete (Sim*)h;
  return CYL_OK;
}

int orc_load_species(orc_handle h, int32_t isp) {
  Sim* s = (Sim*)h;
  if (isp < 0 || isp >= (int)s->sp.size()) return CYL_ERR_BAD_ARG;
  load_species(*s, s->sp[isp]);
  return CYL_OK;
}

int orc_load_species_grid(orc_handle h, int32_t isp, const double* density, const double* temperature,
                          const double* drift) {
  Sim* s = (Sim*)h;
  if (isp < 0 || isp >= (int)s->sp.size()) return CYL_ERR_BAD_ARG;
  load_species(*s, s->sp[isp], density, temperature, drift);
  return CYL_OK;
}

int orc_set_ionisation(orc_handle h, const cyl_ionisation_species* in, int32_t n, int32_t model, uint64_t seed) {
  Sim* s = (Sim*)h;
  if (n == 0) {
    s->ion_on = false;
    return CYL_OK;
  }
  if (!in || n != (int)s->sp.size()) return CYL_ERR_BAD_ARG;
  double omega = 0.0;
  if ((model & CYL_IONISE_MULTIPHOTON) && !s->lasers.empty()) omega = s->lasers[0].d.omega;
  initialise_ionisation(*s, in, n, model, omega);
  s->ion_model = model;
  s->ion_seed = seed;
  s->ion_on = true;
  return CYL_OK;
}

// The constants of initialise_ionisation per species, in the order of
// cyl_ionisation_constants.
int orc_ionisation_constants(orc_handle h, double* out) {
  Sim* s = (Sim*)h;
  for (size_t i = 0; i < s->ion.size(); ++i) {
    const Sim::IonSp& o = s->ion[i];
    const double v[15] = {o.rmf, o.n_exp, o.adk_scaling, o.ion_const, o.smallest_e, o.bsi_const, o.bsi_scaling,
                          o.bsi_threshold, o.adk_max, o.adk_bsi_cap, o.keldysh, o.multi_const, o.k_energy,
                          o.k_exponent, o.adk_mp_cap};
    for (int k = 0; k < 15; ++k) out[i * 15 + k] = v[k];
  }
  return CYL_OK;
}

int orc_set_deck_fns(orc_handle h, const cyl_deck_fns* fns) {
  Sim* s = (Sim*)h;
  s->fns = fns ? *fns : cyl_deck_fns{};
  return CYL_OK;
}

int orc_load_species_counter(orc_handle h, int32_t isp, uint64_t seed, int64_t id_base) {
  Sim* s = (Sim*)h;
  if (isp < 0 || isp >= (int)s->sp.size() || s->sp[isp].d.immobile) return CYL_ERR_BAD_ARG;
  load_species_counter(*s, s->sp[isp], isp, seed, id_base);
  return CYL_OK;
}

int orc_counter_block(uint64_t seed, const uint32_t* ctr4, uint32_t* out4) {
  const Ctr4 r = philox10(Ctr4{{ctr4[0], ctr4[1], ctr4[2], ctr4[3]}}, seed);
  for (int k = 0; k < 4; ++k) out4[k] = r.w[k];
  return CYL_OK;
}

int orc_set_injection_stream(orc_handle h, int32_t mode, uint64_t seed) {
  Sim* s = (Sim*)h;
  if (mode != CYL_RNG_KISS && mode != CYL_RNG_COUNTER) return CYL_ERR_BAD_ARG;
  s->inj_counter = mode == CYL_RNG_COUNTER;
  s->inj_seed = seed;
  return CYL_OK;
}

int orc_set_particles(orc_handle h, int32_t isp, const double* x, const double* y, const double* z,
                      const double* px, const double* py, const double* pz, const double* w,
                      const int64_t* id, int64_t n) {
  Sim* s = (Sim*)h;
  if (isp < 0 || isp >= (int)s->sp.size()) return CYL_ERR_BAD_ARG;
  Species& spc = s->sp[isp];
  spc.x.assign(x, x + n); spc.y.assign(y, y + n); spc.z.assign(z, z + n);
  spc.px.assign(px, px + n); spc.py.assign(py, py + n); spc.pz.assign(pz, pz + n);
  spc.w.assign(w, w + n); spc.id.assign(id, id + n);
  for (int64_t i = 0; i < n; ++i)
    if (id[i] >= s->next_id) s->next_id = id[i] + 1;
  return CYL_OK;
}

int64_t orc_count(orc_handle h, int32_t isp) { return (int64_t)((Sim*)h)->sp[isp].n(); }

int orc_get_particles(orc_handle h, int32_t isp, double* x, double* y, double* z, double* px,
                      double* py, double* pz, double* w, int64_t* id) {
  Species& spc = ((Sim*)h)->sp[isp];
  size_t n = spc.n();
  std::memcpy(x, spc.x.data(), n * 8); std::memcpy(y, spc.y.data(), n * 8);
  std::memcpy(z, spc.z.data(), n * 8); std::memcpy(px, spc.px.data(), n * 8);
  std::memcpy(py, spc.py.data(), n * 8); std::memcpy(pz, spc.pz.data(), n * 8);
  std::memcpy(w, spc.w.data(), n * 8); std::memcpy(id, spc.id.data(), n * 8);
  return CYL_OK;
}

int orc_set_field(orc_handle h, int32_t which, const double* data) {
  Field* f = ((Sim*)h)->field(which);
  if (!f) return CYL_ERR_BAD_ARG;
  std::memcpy(f->a.data(), data, f->a.size() * sizeof(cplx));
  return CYL_OK;
}
int orc_get_field(orc_handle h, int32_t which, double* data) {
  Field* f = ((Sim*)h)->field(which);
  if (!f) return CYL_ERR_BAD_ARG;
  std::memcpy(data, f->a.data(), f->a.size() * sizeof(cplx));
  return CYL_OK;
}

int orc_get_rng(orc_handle h, cyl_rng_state* r) {
  Sim* s = (Sim*)h;
  r->x = s->rng.x; r->y = s->rng.y; r->z = s->rng.z; r->w = s->rng.w;
  r->box_muller_cached = s->rng.cached ? 1 : 0;
  r->cached_random_value = s->rng.cval;
  return CYL_OK;
}
int orc_set_rng(orc_handle h, const cyl_rng_state* r) {
  Sim* s = (Sim*)h;
  s->rng.x = r->x; s->rng.y = r->y; s->rng.z = r->z; s->rng.w = r->w;
  s->rng.cached = r->box_muller_cached != 0;
  s->rng.cval = r->cached_random_value;
  return CYL_OK;
}

// epoch2d.F90:143-162
int orc_initialise(orc_handle h) {
  Sim* s = (Sim*)h;
  particle_bcs(*s);
  efield_bcs(*s);
  double dt_store = s->dt;
  s->dt = s->dt / 2.0;
  s->time = s->time + s->dt;
  bfield_final_bcs(*s);
  s->dt = dt_store;
  return CYL_OK;
}

int orc_step(orc_handle h, int32_t nsteps) {
  Sim* s = (Sim*)h;
  for (int i = 0; i < nsteps; ++i) one_step(*s);
  return CYL_OK;
}

// Advance to the output point of the n-th step (n - 1 full steps, then the
// first part of the last one).
int orc_step_to_output(orc_handle h, int32_t nsteps) {
  Sim* s = (Sim*)h;
  if (nsteps < 1) return CYL_ERR_BAD_ARG;
  for (int i = 0; i < nsteps - 1; ++i) one_step(*s);
  step_to_output(*s);
  return CYL_OK;
}
int orc_finish_step(orc_handle h) {
  finish_step(*(Sim*)h);
  return CYL_OK;
}

// restart_data (setup.F90:777-1569) for the scalars, on fields and particles
// already set (orc_set_field, orc_set_particles), then the restart start-up
// (epoch2d.F90:143-153): particle_bcs, efield_bcs, old_field_bcs
// (boundary.F90:1480-1501) and the rest of the dumped step.  A window that
// has moved (xb_min differs) rebuilds the grid as a shift does.
int orc_restart(orc_handle h, int64_t step, double time, double xb_min, double x_grid_min, int32_t has_wsf,
                double wsf) {
  Sim& s = *(Sim*)h;
  if (step < 1) return CYL_ERR_UNSUPPORTED;
  if (xb_min != s.xb_min) {
    const int64_t shifts = (int64_t)std::llround((xb_min - s.xb_min) / s.dx);
    s.xb_min = xb_min;
    s.x_grid_min = x_grid_min;
    s.x_min = s.xb_min + s.dx * 0.0;
    s.x_max = (s.xb_min + (double)(s.nx + 1 - 1) * s.dx) - s.dx * 0.0;
    s.setup_grid_x();
    s.n_shifts += shifts;
  }
  if (has_wsf) s.window_shift_fraction = wsf;
  s.from_restart = true;
  s.window_started = false;
  s.step = step;
  s.time = time;
  particle_bcs(s);
  efield_bcs(s);
  halo_full(s, s.bx_old);
  halo_shifted(s, s.br_old);
  halo_full(s, s.bt_old);
  finish_step(s);
  return CYL_OK;
}

// Sub-stages, for stage-level parity tests.
int orc_stage(orc_handle h, int32_t stage) {
  Sim& s = *(Sim*)h;
  switch (stage) {
    case 0: update_e_field(s); break;
    case 1: efield_bcs(s); break;
    case 2: update_b_field(s); break;
    case 3: bfield_bcs(s, true); break;
    case 4: push_particles_core(s); break;
    case 5: current_bcs_r_min_final(s); break;
    case 6: particle_bcs(s); break;
    case 7: current_finish(s); break;
    case 8: bfield_final_bcs(s); break;
    case 9: moving_window(s); break;
    case 10: update_eb_fields_half(s); break;
    case 11: update_eb_fields_final(s); break;
    default: return CYL_ERR_BAD_ARG;
  }
  return CYL_OK;
}

int orc_get_run_state(orc_handle h, cyl_run_state* r) {
  Sim* s = (Sim*)h;
  std::memset(r, 0, sizeof(*r));
  r->time = s->time;
  r->step = s->step;
  r->x_grid_min = s->x_grid_min;
  r->xb_min = s->xb_min;
  r->x_min = s->x_min;
  r->x_max = s->x_max;
  r->window_shift_fraction = s->window_shift_fraction;
  r->window_started = s->window_started ? 1 : 0;
  for (int i = 0; i < 4; ++i) r->bc_field[i] = s->bc_field[i];
  for (size_t i = 0; i < s->sp.size() && i < 8; ++i) r->n_live[i] = (int64_t)s->sp[i].n();
  r->n_shifts = s->n_shifts;
  return CYL_OK;
}

int orc_diagnostics(orc_handle h, cyl_diag* out) {
  diagnostics(*(Sim*)h, out);
  return CYL_OK;
}

// Cell-sort indices (split_particle.F90:61-62)
int orc_cell_indices(orc_handle h, int32_t isp, int32_t* cx, int32_t* cy) {
  Sim* s = (Sim*)h;
  Species& spc = s->sp[isp];
  for (size_t i = 0; i < spc.n(); ++i) {
    double part_r = std::sqrt(spc.y[i] * spc.y[i] + spc.z[i] * spc.z[i]);
    cx[i] = ffloor((spc.x[i] - s->x_grid_min) / s->dx + 1.5);
    cy[i] = ffloor((part_r - s->y_grid_min) / s->dy + 1.5);
  }
  return CYL_OK;
}

// Per-mode charge density (complex FP64, field layout) of the current state.
int orc_charge_density(orc_handle h, double* data) {
  Sim& s = *(Sim*)h;
  Field rho;
  rho.init(s.nx, s.ny, s.M);
  charge_density(s, rho);
  std::memcpy(data, rho.a.data(), rho.a.size() * sizeof(cplx));
  return 0;
}

// Per-mode number density (complex FP64, field layout) of species isp (< 0:
// every species with particles).
int orc_number_density(orc_handle h, int32_t isp, double* data) {
  Sim& s = *(Sim*)h;
  Field nd;
  nd.init(s.nx, s.ny, s.M);
  number_density_modes(s, nd, isp);
  std::memcpy(data, nd.a.data(), nd.a.size() * sizeof(cplx));
  return 0;
}

void orc_set_threads(int32_t n) { g_threads = n < 1 ? 1 : n; }

double orc_atan2(double y, double x) { return cyl_atan2(y, x); }
void orc_atan2_many(int64_t n, const double* y, const double* x, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = cyl_atan2(y[i], x[i]);
}
void orc_set_atan2(int32_t mode) { g_atan2_mode = mode ? 1 : 0; }
void orc_sincos_turn(double u, double* s, double* c) { cyl_sincos_turn(u, s, c); }

double orc_dx(orc_handle h) { return ((Sim*)h)->dx; }
double orc_dy(orc_handle h) { return ((Sim*)h)->dy; }
double orc_time(orc_handle h) { return ((Sim*)h)->time; }

}  // extern "C"
