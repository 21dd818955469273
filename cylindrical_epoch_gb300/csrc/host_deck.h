// host_deck.h -- host-side stand-ins for the Fortran driver's deck work:
// the global KISS generator, the particle loader and the moving-window
// injector.  These run on the CPU exactly as the reference does (the
// reference evaluates deck expressions and draws random numbers serially on
// the host); the GPU receives their output.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/cylpic.h"

namespace cyl {

// KISS + polar Box-Muller (random_generator.f90:45-173)
struct KissRng {
  int32_t x = 0, y = 0, z = 0, w = 0;
  bool cached = false;
  double cval = 0.0;
  void seed(int32_t s);
  double random();
  double box_muller(double stdev, double mu);
  void to_state(cyl_rng_state* s) const;
  void from_state(const cyl_rng_state* s);
};

// Grid scalars of one run, as setup_grid / setup_grid_x / setup_grid_y
// (setup.F90:164-206, utilities.f90:343-409) compute them, cpml_thickness = 0.
struct HostGrid {
  int nx = 0, ny = 0, M = 0;
  double dx = 0, dy = 0, dt = 0;
  double length_x = 0, length_y = 0;
  double x_min = 0, x_max = 0, y_max = 0;
  double x_grid_min = 0, xb_min = 0, x_grid_max = 0;
  double y_grid_min = 0, y_grid_max = 0;
  double x_min_local = 0, x_max_local = 0, y_min_local = 0, y_max_local = 0;
  void init(const cyl_grid_desc& g);
  void setup_grid_x();
  void setup_grid_y();
  double xg(int ix) const { return x_grid_min + (double)(ix - 1) * dx; }
  double yg(int iy) const { return y_grid_min + (double)(iy - 1) * dy; }
};

// A particle produced on the host: x, y, z, px, py, pz, w, id
struct HostParticle {
  double v[7];
  int64_t id;
};

double species_density(const cyl_species_desc& d, double x);

// setup_particle_density for one species (helper.F90:373-663): the density
// on the (nx + 2ng) x (ny + 2ng) grid (index (ix + ng - 1) + W (iy + ng - 1),
// W = nx + 2ng), with the periodic x self-wrap, clamped to density_max and
// zeroed below density_min; dmap marks the cells at or above density_min.
// valid lists the valid interior cells as (ix - 1) + nx (iy - 1), iy outer.
// dens_in, when given, holds the deck's density on that grid (the caller's
// evaluation of the density expression) in place of the closed form.
void host_density_map(const HostGrid& g, const cyl_grid_desc& gd, const cyl_species_desc& sp,
                      std::vector<double>& dens, std::vector<char>& dmap, std::vector<int32_t>& valid,
                      const double* dens_in = nullptr);

// The columns insert_particles evaluates at pack_ix = nx (window.F90:196-222):
// density(0:ny+1), temperature(0:ny+1, 1:3), drift(0:ny+1, 1:3).
struct InjectColumns {
  std::vector<double> density, temperature, drift;
};

// insert_particles (window.F90:157-300) for one species at the current grid
// (before the shift): appends to out, advances rng and next_id.  cols, when
// given, holds the caller's evaluation of the deck's columns (the density
// not yet clamped); else the descriptor's closed forms are used.
void host_insert_particles(const HostGrid& g, const cyl_species_desc& d, KissRng& rng,
                           int64_t& next_id, std::vector<HostParticle>& out,
                           const InjectColumns* cols = nullptr);

}  // namespace cyl
