// host_deck.cpp -- KISS generator, thermal loader and window injector that
// stand in for the Fortran driver's host-side deck work.
#include "host_deck.h"

#include <cmath>
#include <cstring>

namespace cyl {

namespace {
const double PI_H = 3.141592653589793238462643383279503;
const double KB_H = 1.3806488e-23;
const int NG_H = CYL_NG;
}  // namespace

// ------------------------------------------------------------------ KISS

void KissRng::seed(int32_t s) {
  // random_init (random_generator.f90:82-108)
  x = (int32_t)(123456789u + (uint32_t)s);
  y = (int32_t)(362436069u + (uint32_t)s);
  z = (int32_t)(521288629u + (uint32_t)s);
  w = (int32_t)(916191069u + (uint32_t)s);
  cached = false;
  cval = 0.0;
  for (int i = 0; i < 1000; ++i) random();
}

double KissRng::random() {
  // random (random_generator.f90:45-78): 32-bit two's-complement wrap-around,
  // ISHFT with a negative count is a logical right shift.
  uint32_t ux = (uint32_t)x * 69069u + 1327217885u;
  uint32_t uy = (uint32_t)y;
  uy ^= uy << 13;
  uy ^= uy >> 17;
  uy ^= uy << 5;
  uint32_t uz = 18000u * ((uint32_t)z & 65535u) + ((uint32_t)z >> 16);
  uint32_t uw = 30903u * ((uint32_t)w & 65535u) + ((uint32_t)w >> 16);
  x = (int32_t)ux;
  y = (int32_t)uy;
  z = (int32_t)uz;
  w = (int32_t)uw;
  const int32_t kiss = (int32_t)(ux + uy + (uz << 16) + uw);
  return ((double)kiss + 2147483648.0) / 4294967296.0;
}

double KissRng::box_muller(double stdev, double mu) {
  // random_box_muller (random_generator.f90:112-173)
  if (cached) {
    cached = false;
    return cval * stdev + mu;
  }
  cached = true;
  double r1, r2, s;
  do {
    r1 = 2.0 * random() - 1.0;
    r2 = 2.0 * random() - 1.0;
    s = r1 * r1 + r2 * r2;
  } while (!(s > 2.2250738585072014e-308 && s < 1.0));
  s = std::sqrt((-2.0 * std::log(s)) / s);
  cval = r2 * s;
  return r1 * s * stdev + mu;
}

void KissRng::to_state(cyl_rng_state* s) const {
  s->x = x; s->y = y; s->z = z; s->w = w;
  s->box_muller_cached = cached ? 1 : 0;
  s->cached_random_value = cval;
}
void KissRng::from_state(const cyl_rng_state* s) {
  x = s->x; y = s->y; z = s->z; w = s->w;
  cached = s->box_muller_cached != 0;
  cval = s->cached_random_value;
}

// ------------------------------------------------------------------ grid

void HostGrid::init(const cyl_grid_desc& g) {
  nx = g.nx; ny = g.ny; M = g.n_mode;
  x_min = g.x_min; x_max = g.x_max; y_max = g.y_max;
  dt = g.dt;
  length_x = x_max - x_min;
  dx = length_x / (double)(nx - 0);
  x_grid_min = x_min - dx * 0.0;
  length_y = y_max - 0.0;
  dy = length_y / (double)(ny - 0);
  y_grid_min = 0.0 - dy * 0.0;
  xb_min = x_grid_min;
  x_grid_min = x_grid_min + dx / 2.0;
  y_grid_min = y_grid_min + dy / 2.0;
  setup_grid_x();
  setup_grid_y();
}
void HostGrid::setup_grid_x() {
  x_grid_max = x_grid_min + (double)(nx - 1) * dx;
  x_min_local = x_grid_min + (0.0 - 0.5) * dx;
  x_max_local = x_grid_max - (0.0 - 0.5) * dx;
}
void HostGrid::setup_grid_y() {
  y_grid_max = y_grid_min + (double)(ny - 1) * dy;
  y_min_local = y_grid_min + (0.0 - 0.5) * dy;
  y_max_local = y_grid_max - (0.0 - 0.5) * dy;
}

double species_density(const cyl_species_desc& d, double x) {
  if (d.density_kind == 1) {
    double f = (x - d.ramp_x0) / d.ramp_length;
    if (f < 0.0) f = 0.0;
    if (f > 1.0) f = 1.0;
    return d.density * f;
  }
  return d.density;
}

void host_density_map(const HostGrid& g, const cyl_grid_desc& gd, const cyl_species_desc& sp,
                      std::vector<double>& dens, std::vector<char>& dmap, std::vector<int32_t>& valid,
                      const double* dens_in) {
  const int nx = g.nx, ny = g.ny;
  const int W = nx + 2 * NG_H;
  auto at = [&](int ix, int iy) { return (size_t)(ix + NG_H - 1) + (size_t)W * (size_t)(iy + NG_H - 1); };
  dens.assign((size_t)W * (ny + 2 * NG_H), 0.0);
  dmap.assign(dens.size(), 0);
  for (int iy = 1 - NG_H; iy <= ny + NG_H; ++iy)
    for (int ix = 1 - NG_H; ix <= nx + NG_H; ++ix)
      dens[at(ix, iy)] = dens_in ? dens_in[at(ix, iy)] : species_density(sp, g.xg(ix));
  if (gd.bc_field[CYL_BD_X_MAX] == CYL_BC_PERIODIC)
    for (int iy = 1 - NG_H; iy <= ny + NG_H; ++iy)
      for (int i = 1; i <= NG_H; ++i) dens[at(nx + i, iy)] = dens[at(i, iy)];
  if (gd.bc_field[CYL_BD_X_MIN] == CYL_BC_PERIODIC)
    for (int iy = 1 - NG_H; iy <= ny + NG_H; ++iy)
      for (int i = 1 - NG_H; i <= 0; ++i) dens[at(i, iy)] = dens[at(nx + i, iy)];
  for (size_t k = 0; k < dens.size(); ++k) {
    if (dens[k] > sp.density_max) dens[k] = sp.density_max;
    if (dens[k] >= sp.density_min) dmap[k] = 1;
    else dens[k] = 0.0;
  }
  valid.clear();
  for (int iy = 1; iy <= ny; ++iy)
    for (int ix = 1; ix <= nx; ++ix)
      if (dmap[at(ix, iy)]) valid.push_back((int32_t)((ix - 1) + nx * (iy - 1)));
}

// ------------------------------------------------------------ injection

void host_insert_particles(const HostGrid& g, const cyl_species_desc& d, KissRng& rng,
                           int64_t& next_id, std::vector<HostParticle>& out, const InjectColumns* cols) {
  const int ny = g.ny;
  const int64_t nppc = (int64_t)std::floor(d.npart_per_cell);
  const double npart_frac = d.npart_per_cell - (double)nppc;
  const double dmin = d.density_min, dmax = d.density_max;
  // density / temperature / drift at the x_max column (pack_ix = nx)
  const double dens_col = species_density(d, g.xg(g.nx));
  std::vector<double> density(ny + 2);
  for (int iy = 0; iy <= ny + 1; ++iy) {
    double v = cols ? cols->density[iy] : dens_col;
    if (v > dmax) v = dmax;
    if (v < dmin) v = 0.0;
    density[iy] = v;
  }
  // temperature(iy, i), drift(iy, i) of the rows around iy
  auto temp_at = [&](int iy, int i) { return cols ? cols->temperature[iy + (ny + 2) * i] : d.temp[i]; };
  auto drift_at = [&](int iy, int i) { return cols ? cols->drift[iy + (ny + 2) * i] : d.drift[i]; };
  const double x0 = g.x_grid_max + 0.5 * g.dx;
  for (int iy = 1; iy <= ny; ++iy) {
    if (density[iy] < dmin) continue;
    int64_t n_frac = 0;
    if (npart_frac > 0.0 && rng.random() < npart_frac) n_frac = 1;
    for (int64_t ip = 1; ip <= nppc + n_frac; ++ip) {
      const double cell_frac_y = 0.5 - rng.random();
      const double part_r = g.yg(iy) - cell_frac_y * g.dy;
      const double part_theta = 2.0 * PI_H * rng.random();
      HostParticle p;
      p.v[0] = x0 + rng.random() * g.dx;
      p.v[1] = part_r * std::cos(part_theta);
      p.v[2] = part_r * std::sin(part_theta);
      const double wdata = (2.0 * PI_H * g.dx * g.dy * part_r) / (double)(nppc + n_frac);
      const double cy2 = cell_frac_y * cell_frac_y;
      const double gyv[3] = {0.5 * ((0.25 + cy2) + cell_frac_y), 0.75 - cy2,
                             0.5 * ((0.25 + cy2) - cell_frac_y)};
      for (int i = 0; i < 3; ++i) {
        double tl = 0.0, dl = 0.0;
        for (int k = 0; k < 3; ++k) {
          tl = tl + gyv[k] * temp_at(iy - 1 + k, i);
          dl = dl + gyv[k] * drift_at(iy - 1 + k, i);
        }
        p.v[3 + i] = rng.box_muller(std::sqrt(tl * KB_H * d.mass), dl);
      }
      double wl = 0.0;
      for (int k = -1; k <= 1; ++k) wl = wl + gyv[k + 1] * density[iy + k];
      p.v[6] = wl * wdata;
      p.id = next_id++;
      out.push_back(p);
    }
  }
}

}  // namespace cyl

// ============================================================ C ABI part

using namespace cyl;

extern "C" {

void cyl_rng_init(cyl_rng_state* s, int32_t seed) {
  KissRng r;
  r.seed(seed);
  r.to_state(s);
}

double cyl_rng_random(cyl_rng_state* s) {
  KissRng r;
  r.from_state(s);
  double v = r.random();
  r.to_state(s);
  return v;
}

double cyl_rng_box_muller(cyl_rng_state* s, double stdev, double mu) {
  KissRng r;
  r.from_state(s);
  double v = r.box_muller(stdev, mu);
  r.to_state(s);
  return v;
}

// Loader: setup_particle_density + load_particles (helper.F90:373-663,
// 669-811), then setup_particle_temperature for x, y, z
// (particle_temperature.F90:30-81).
int cyl_host_load_species(const cyl_grid_desc* gd, const cyl_species_desc* sp, cyl_rng_state* rs,
                          int64_t id_base, double* x, double* y, double* z, double* px, double* py,
                          double* pz, double* w, int64_t* id, int64_t* n_inout) {
  return cyl_host_load_species_grid(gd, sp, rs, id_base, nullptr, nullptr, nullptr, x, y, z, px, py, pz, w, id,
                                    n_inout);
}

int cyl_host_load_species_grid(const cyl_grid_desc* gd, const cyl_species_desc* sp, cyl_rng_state* rs,
                               int64_t id_base, const double* density, const double* temperature,
                               const double* drift, double* x, double* y, double* z, double* px, double* py,
                               double* pz, double* w, int64_t* id, int64_t* n_inout) {
  if (!gd || !sp || !n_inout) return CYL_ERR_BAD_ARG;
  HostGrid g;
  g.init(*gd);
  const int nx = g.nx;
  const int W = nx + 2 * NG_H;
  auto at = [&](int ix, int iy) { return (size_t)(ix + NG_H - 1) + (size_t)W * (size_t)(iy + NG_H - 1); };
  std::vector<double> dens;
  std::vector<char> dmap;
  std::vector<int32_t> valid_cells;
  host_density_map(g, *gd, *sp, dens, dmap, valid_cells, density);
  const int64_t nvalid = (int64_t)valid_cells.size();
  const int64_t nppc = (int64_t)std::floor(sp->npart_per_cell);
  const int64_t nnew = (int64_t)std::floor(sp->npart_per_cell * (double)nvalid);
  if (!x) {
    *n_inout = nnew;
    return CYL_OK;
  }
  if (*n_inout < nnew || !y || !z || !px || !py || !pz || !w || !id || !rs) return CYL_ERR_BAD_ARG;
  KissRng rng;
  rng.from_state(rs);
  int64_t n = 0;
  if (nppc > 0) {
    for (const int32_t cell : valid_cells) {
      const int iy = cell / nx + 1, ix = cell % nx + 1;
      for (int64_t ip = 0; ip < nppc && n < nnew; ++ip) {
        x[n] = g.xg(ix) + (rng.random() - 0.5) * g.dx;
        const double pr = g.yg(iy) + (rng.random() - 0.5) * g.dy;
        const double th = 2.0 * PI_H * rng.random();
        y[n] = pr * std::cos(th);
        z[n] = pr * std::sin(th);
        ++n;
      }
    }
  }
  if (n < nnew) {
    while (n < nnew) {
      int64_t ipos = (int64_t)(rng.random() * (double)(nvalid - 1)) + 1;
      ipos = valid_cells[ipos - 1];
      const int64_t cyy = ipos / nx;
      ipos = ipos - nx * cyy;
      const int cy = (int)cyy + 1, cx = (int)ipos + 1;
      x[n] = g.xg(cx) + (rng.random() - 0.5) * g.dx;
      const double pr = g.yg(cy) + (rng.random() - 0.5) * g.dy;
      const double th = 2.0 * PI_H * rng.random();
      y[n] = pr * std::cos(th);
      z[n] = pr * std::sin(th);
      ++n;
    }
  }
  // Loaded positions lie in [x_min, x_max) x [0, y_max) by construction, so
  // the particle_bcs call at the end of load_particles moves none of them.
  for (int64_t p = 0; p < n; ++p) {
    id[p] = id_base + p;
    px[p] = py[p] = pz[p] = 0.0;
  }
  // weights: particle_to_grid.inc + triangle/gxfac.inc
  struct Sh {
    int cx, cy;
    double gx[3], gy[3];
  };
  auto shape = [&](int64_t p) {
    Sh r;
    const double part_r = std::sqrt(y[p] * y[p] + z[p] * z[p]);
    const double cxr = (x[p] - g.x_grid_min) / g.dx;
    const double cyr = (part_r - g.y_grid_min) / g.dy;
    const int cx = (int)std::floor(cxr + 0.5), cy = (int)std::floor(cyr + 0.5);
    const double fx = (double)cx - cxr, fy = (double)cy - cyr;
    r.cx = cx + 1;
    r.cy = cy + 1;
    const double x2 = fx * fx, y2 = fy * fy;
    r.gx[0] = 0.5 * ((0.25 + x2) + fx);
    r.gx[1] = 0.75 - x2;
    r.gx[2] = 0.5 * ((0.25 + x2) - fx);
    r.gy[0] = 0.5 * ((0.25 + y2) + fy);
    r.gy[1] = 0.75 - y2;
    r.gy[2] = 0.5 * ((0.25 + y2) - fy);
    if (part_r < g.dy) {
      r.gy[1] = r.gy[1] + r.gy[0];
      r.gy[0] = 0.0;
    }
    return r;
  };
  std::vector<int> npic(dens.size(), 0);
  for (int64_t p = 0; p < n; ++p) {
    Sh s = shape(p);
    double wd = 0.0;
    for (int sy = -1; sy <= 1; ++sy) {
      int i = s.cx, j = s.cy + sy;
      if (!dmap[at(i, j)]) j = s.cy + sy / 2;
      for (int sx = -1; sx <= 1; ++sx) {
        i = s.cx + sx;
        if (!dmap[at(i, j)]) i = s.cx + sx / 2;
        wd = wd + (s.gx[sx + 1] * s.gy[sy + 1]) * dens[at(i, j)];
      }
    }
    w[p] = wd;
    npic[at(s.cx, s.cy)]++;
  }
  for (int64_t p = 0; p < n; ++p) {
    const double part_r = std::sqrt(y[p] * y[p] + z[p] * z[p]);
    const int cx = (int)std::floor((x[p] - g.x_grid_min) / g.dx + 1.5);
    const int cy = (int)std::floor((part_r - g.y_grid_min) / g.dy + 1.5);
    const double vol = 2.0 * PI_H * g.dx * g.dy * part_r;
    w[p] = w[p] * vol / (double)npic[at(cx, cy)];
  }
  // temperature(cell_x + sx, cell_y + sy) and drift of direction dir
  const size_t plane = dens.size();
  for (int dir = 0; dir < 3; ++dir) {
    double* pp = dir == 0 ? px : (dir == 1 ? py : pz);
    for (int64_t p = 0; p < n; ++p) {
      Sh s = shape(p);
      double tl = 0.0, dl = 0.0;
      for (int sy = -1; sy <= 1; ++sy)
        for (int sx = -1; sx <= 1; ++sx) {
          const size_t c = at(s.cx + sx, s.cy + sy) + plane * (size_t)dir;
          tl = tl + (s.gx[sx + 1] * s.gy[sy + 1]) * (temperature ? temperature[c] : sp->temp[dir]);
          dl = dl + (s.gx[sx + 1] * s.gy[sy + 1]) * (drift ? drift[c] : sp->drift[dir]);
        }
      pp[p] = rng.box_muller(std::sqrt(tl * KB_H * sp->mass), dl);
    }
  }
  rng.to_state(rs);
  *n_inout = n;
  return CYL_OK;
}

}  // extern "C"
