// ionise.cu -- field ionisation (physics_packages/ionise.F90), for both forms:
// the constants of initialise_ionisation (:51-286) on the host, and
// ionise_particles (:325-351) with its four rate models (multiphoton /
// tunnelling / barrier suppression, :355-1500) as one kernel.
//
// Per particle of an ionising species: the electric field at the particle
// (e_part.inc, the push's gather), its magnitude in atomic units, then
// ionisation trials through the charge states while time is left in the step:
// the rate of the state's regime, a uniform sample, ionisation if the sample
// falls below 1 - exp(-rate time_left), which releases an electron (momentum
// split by mass, plus the multiphoton kick) and spends time
// -log(1 - sample)/rate.  A particle that ionised moves to its final
// species and deposits the ionisation current (Mulser et al. 1998) with the
// triangle weights, per mode.
//
// The reference draws the samples from its serial KISS stream in list order.
// Here each trial takes the counter stream's word for (particle id, step,
// charge state) (counter_rng.cuh, tag TAG_IONISE), so any thread can ionise
// any particle; the oracle draws the same words.  Released electrons and
// moved ions are appended to their species with atomic slot counters; the
// order of slots differs from the reference's lists, ids do not.
//
// Compiled with --fmad=false: every FP64 operation rounds once, in the
// reference's order.  The mixed form runs the same kernel over its own
// storage (IonState<true>): particles converted to FP64 as its download does,
// fields gathered from its FP32 arrays, ions and electrons written back
// through its upload's conversion into the species' unsorted tails.
#include <cmath>
#include <cstring>
#include <type_traits>

#include "counter_rng.cuh"
#include "cyl_common.cuh"
#include "cyl_kernels.cuh"
#include "push_mixed.cuh"

namespace cyl {

namespace {

// constants.F90:172-198
constexpr double Q0 = 1.602176565e-19;
constexpr double M0 = 9.10938291e-31;
constexpr double H_BAR = 1.054571725336289397963133257349698e-34;
constexpr double A0 = 5.291772101121111395947216558438464e-11;
constexpr double HARTREE = 4.359744350823120007758594450644308e-18;
constexpr double ATOMIC_TIME = 2.418884320905619591809404261549867e-17;
constexpr double ATOMIC_E = 5.142206538736485312185213306837419e11;
constexpr double C_LOG2 = 0.69314718055994530941723212145817657;
constexpr double C_LARGEST_EXP = 1024.0 * C_LOG2;  // MAXEXPONENT(1.0_num) * c_log2
constexpr double C_TINY = 2.2250738585072014e-308;  // TINY(1.0_num)
constexpr double C_HUGE = 1.7976931348623157e308;   // HUGE(1.0_num)
// ionise.F90:27-28
constexpr double IONISATION_EXPONENT = -1.0 / 3.0;

// exp(x) K_{l+1/2}(x) sqrt(8/pi) sqrt(x): the factor of the ADK rate that
// the reference evaluates with RKBESL (numerics.f90:294-792, Cody's
// algorithm for K of any order).  For half-integer order K has the closed
// form sqrt(pi/(2x)) e^{-x} sum_{k=0..l} (l+k)!/(k!(l-k)!) (2x)^-k
// (Abramowitz & Stegun 10.2.15), evaluated here in the reference's
// arrangement bessel_constant * SQRT(x) * EXP(x) * K(x).
CYL_HD double bessel_term(double x, int l) {
  double sum = 0.0, term = 1.0;
  for (int k = 0; k <= l; ++k) {
    if (k > 0) term = term * ((double)((l + k) * (l - k + 1)) / (double)k) / (2.0 * x);
    sum = sum + term;
  }
  const double kval = sqrt(PI / (2.0 * x)) * exp(-x) * sum;
  return sqrt(8.0 / PI) * sqrt(x) * exp(x) * kval;
}

// factorial (numerics.f90:24-40)
double factorial_ref(double x) {
  double f = 1.0;
  for (int i = 2; i <= (int)x; ++i) {
    if (f < std::sqrt(C_HUGE)) f = f * (double)i;
    else {
      f = C_HUGE;
      break;
    }
  }
  return f;
}

}  // namespace

// initialise_ionisation (ionise.F90:51-286) for species desc sd[0..n), with
// the deck's ionisation data io[0..n).  omega: the lasers' common omega
// (only used with multiphoton).
void ionisation_constants(const cyl_ionisation_species* io, const cyl_species_desc* sd, int n, int model,
                          double omega, IonSpecies* out) {
  const bool mp = (model & CYL_IONISE_MULTIPHOTON) != 0, bsi = (model & CYL_IONISE_BSI) != 0;
  const double omega_atomic = omega * ATOMIC_TIME;
  const double c_atomic = CLIGHT * ATOMIC_TIME / A0;
  for (int i = 0; i < n; ++i) {
    IonSpecies& o = out[i];
    std::memset(&o, 0, sizeof(o));
    o.ionise = io[i].ionise ? 1 : 0;
    o.ionise_to = io[i].ionise_to;
    o.release = io[i].release;
    o.l = io[i].l;
    o.energy = io[i].energy;
    if (!o.ionise) continue;
    const cyl_species_desc& to = sd[io[i].ionise_to];
    o.released_mass_fraction = io[i].release >= 0 ? sd[io[i].release].mass / sd[i].mass : 0.0;
    const double ip = io[i].energy / HARTREE;
    const double z = to.charge / Q0;
    double n_eff = z / std::sqrt(2.0 * ip);
    const double t2 = 2.0 * ip;
    o.adk_scaling = 2.0 * std::sqrt((t2 * t2) * t2);  // integer powers as gfortran expands them
    o.ionisation_constant = std::sqrt(6.0 / PI) * ip * std::pow(2.0, 2.0 * n_eff) / (n_eff * std::tgamma(2.0 * n_eff));
    if (bsi) {
      o.bsi_constant = ip * std::sqrt(2.0 * ip) / (2.0 * PI * z);
      o.bsi_scaling = (ip * ip) / (4.0 * z);
      const double u = 2.0 * n_eff, u2 = u * u;
      o.bsi_threshold = ((z * z) * z) / (u2 * u2);
      o.adk_maximum = std::fmax(o.adk_scaling / (3.0 * (2.0 * n_eff + (double)io[i].l - 1.5)), o.bsi_threshold);
    }
    double kexp = 0.0;
    if (mp) {
      kexp = (double)((int64_t)std::floor(ip / omega_atomic) + 1);
      double multi = factorial_ref(kexp);
      if (multi < std::sqrt(C_HUGE)) {
        const int64_t nq = io[i].n, nq2 = nq * nq;
        multi = c_atomic * (multi * multi) * (double)((nq2 * nq2) * nq) *
                std::pow(omega_atomic, (10.0 * kexp - 1.0) / 3.0) * std::sqrt(kexp) * (2.0 * kexp + 1.0);
      } else {
        multi = 0.0;
      }
      if (std::fabs(multi) > C_TINY)
        multi = 4.8 * std::pow(1.69 * c_atomic / (8.0 * PI * omega_atomic), kexp) / multi;
      o.multi_constant = multi;
      o.k_photons_energy = kexp * H_BAR * omega;
      o.k_photons_exponent = 4.0 * kexp - 2.0;
    }
    n_eff = 2.0 * n_eff - 1.5;
    o.n_exp = n_eff;
    if (bsi) {
      const double x = o.adk_scaling / o.bsi_threshold;
      o.adk_bsi_cap = o.ionisation_constant * std::pow(x, o.n_exp) * std::exp(IONISATION_EXPONENT * x) *
                      (bessel_term(x, io[i].l) - 1.0);
    }
    if (mp) {
      o.keldysh = std::fmax(o.adk_scaling / (0.99472065388909858 * C_LARGEST_EXP),
                            omega_atomic * std::sqrt(2.0 * ip) / 0.5);
      const double x = o.adk_scaling / o.keldysh;
      o.adk_multiphoton_cap = o.ionisation_constant * std::pow(x, o.n_exp) * std::exp(IONISATION_EXPONENT * x) *
                              (bessel_term(x, io[i].l) - 1.0);
      if (std::fabs(o.multi_constant) <= C_TINY) o.smallest_e_mag = C_HUGE;
      else o.smallest_e_mag = std::pow(C_TINY / std::fmin(o.multi_constant, 1.0), 1.0 / o.k_photons_exponent);
    } else {
      o.smallest_e_mag = o.adk_scaling / (0.99472065388909858 * C_LARGEST_EXP);
    }
  }
}

namespace {

template <typename T>
__device__ __forceinline__ cplx gather3(const FViewT<T>& f, const double* wa, const double* wb, int ca, int cb,
                                       int m) {
  cplx acc;
#pragma unroll
  for (int jj = -1; jj <= 1; ++jj) {
    const cplx inner = (wb[1] * f(ca - 1, cb + jj, m) + wb[2] * f(ca, cb + jj, m)) + wb[3] * f(ca + 1, cb + jj, m);
    if (jj == -1) acc = wa[jj + 2] * inner;
    else acc = acc + wa[jj + 2] * inner;
  }
  return acc;
}

__device__ __forceinline__ double nan_slot() { return __longlong_as_double(0x7ff8000000000000LL); }

// A slot at the end of species t, or -1 when it is full (the count is
// clamped back and the run flagged after the kernel).
__device__ __forceinline__ int64_t take_slot(SpeciesCounters* cnt, const SpeciesPtrs& sp) {
  const int64_t k = (int64_t)atomicAdd((unsigned long long*)&cnt->n_used, 1ull);
  return k < sp.cap ? k : -1;
}

struct IonLaunch {
  SpeciesPtrs sp[MAX_SPECIES];
  IonParams P;
  double xg0;  // the mixed form's x origin
};

// One particle's state as the routine reads and writes it: the FP64 form's
// arrays, or the mixed form's storage (converted to FP64 on the way in, as
// the mixed form's download does, and back on the way out).
template <bool MIXED>
struct IonState;
template <>
struct IonState<false> {
  __device__ static bool load(const SpeciesPtrs& S, int64_t i, double, const RunConst&, double& x, double& y,
                              double& z) {
    x = S.x[i];
    if (isnan(x)) return false;
    y = S.y[i];
    z = S.z[i];
    return true;
  }
  __device__ static void momenta(const SpeciesPtrs& S, int64_t i, double& px, double& py, double& pz, double& w) {
    px = S.px[i];
    py = S.py[i];
    pz = S.pz[i];
    w = S.w[i];
  }
  __device__ static void store(const SpeciesPtrs& T, SpeciesCounters*, int64_t k, double x, double y, double z,
                               double px, double py, double pz, double w, int64_t id, double, const RunConst&) {
    T.x[k] = x;
    T.y[k] = y;
    T.z[k] = z;
    T.px[k] = px;
    T.py[k] = py;
    T.pz[k] = pz;
    T.w[k] = w;
    T.id[k] = id;
  }
  __device__ static void remove(const SpeciesPtrs& S, int64_t i) { S.x[i] = nan_slot(); }
};
template <>
struct IonState<true> {
  __device__ static bool load(const SpeciesPtrs& S, int64_t i, double xg0, const RunConst& rc, double& x,
                              double& y, double& z) {
    const int32_t k = S.kx[i];
    if (k == INT32_MIN) return false;
    x = xg0 + ((double)k + (double)S.fx[i]) * rc.dx;
    y = (double)S.fy[i] * rc.dy;
    z = (double)S.fz[i] * rc.dy;
    return true;
  }
  __device__ static void momenta(const SpeciesPtrs& S, int64_t i, double& px, double& py, double& pz, double& w) {
    const double mc = S.mass * CLIGHT;
    px = (double)S.ux[i] * mc;
    py = (double)S.uy[i] * mc;
    pz = (double)S.uz[i] * mc;
    w = (double)S.fw[i];
  }
  __device__ static void store(const SpeciesPtrs& T, SpeciesCounters* c, int64_t k, double x, double y, double z,
                               double px, double py, double pz, double w, int64_t id, double xg0,
                               const RunConst& rc) {
    to_mixed(T, k, x, y, z, px, py, pz, w, xg0, rc);
    T.id[k] = id;
    atomicMax(&c->wmax_bits, __float_as_uint(fabsf(T.fw[k])));
  }
  __device__ static void remove(const SpeciesPtrs& S, int64_t i) { S.kx[i] = INT32_MIN; }
};

// ionise_particles over the particles species `isp` held when the routine
// started (snap[isp]); one thread per particle.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_ionise(FieldSetT<typename std::conditional<MIXED, cplxf, cplx>::type> F,
                                                IonLaunch L, SpeciesCounters* cnt, const int64_t* snap, int isp,
                                                const StepRec* rec, RunConst rc, int* err) {
  using IO = IonState<MIXED>;
  const IonParams& P = L.P;
  const SpeciesPtrs& S = L.sp[isp];
  const int64_t n = snap[isp];
  const double fac = 0.25;  // (0.5)**c_ndims
  const double idx = 1.0 / rc.dx, idy = 1.0 / rc.dy;
  const double dfac1 = fac * fac / (rc.dt * 2.0 * PI * rc.dx * rc.dy);
  const double x_grid_min_local = rec->x_grid_min, y_grid_min_local = rc.y_grid_min;
  const int M = rc.M;
  const bool mp = (P.model & CYL_IONISE_MULTIPHOTON) != 0, bsi = (P.model & CYL_IONISE_BSI) != 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double px0, py0, pz0;
    if (!IO::load(S, i, L.xg0, rc, px0, py0, pz0)) continue;
    const double part_x_local = px0 - x_grid_min_local;
    const double part_r = sqrt(py0 * py0 + pz0 * pz0);
    const double part_r_local = part_r - y_grid_min_local;
    const cplx exp_min_itheta = mk(py0 / part_r, (-pz0) / part_r);
    const cplx exp_itheta = crecip(exp_min_itheta);
    const double dfac = dfac1 / part_r;
    double gx[5] = {0, 0, 0, 0, 0}, gy[5] = {0, 0, 0, 0, 0}, hx[5] = {0, 0, 0, 0, 0}, hy[5] = {0, 0, 0, 0, 0};
    const double cell_x_r = part_x_local * idx, cell_y_r = part_r_local * idy;
    int cell_x1 = (int)floor(cell_x_r + 0.5);
    double cell_frac_x = (double)cell_x1 - cell_x_r;
    cell_x1 = cell_x1 + 1;
    int cell_y1 = (int)floor(cell_y_r + 0.5);
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
    int cell_x2 = (int)floor(cell_x_r);
    cell_frac_x = ((double)cell_x2 - cell_x_r) + 0.5;
    cell_x2 = cell_x2 + 1;
    int cell_y2 = (int)floor(cell_y_r);
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
    if (cell_x1 < 2 - NG || cell_x1 > rc.nx + NG - 1 || cell_x2 < 2 - NG || cell_x2 > rc.nx + NG - 1 ||
        cell_y1 < 2 - NG || cell_y1 > rc.ny + NG - 1 || cell_y2 < 2 - NG || cell_y2 > rc.ny + NG - 1) {
      atomicOr(err, ERR_CELL_RANGE);
      continue;
    }
    // e_part.inc
    double ex_part = 0.0, er_part = 0.0, et_part = 0.0;
    cplx emi = mk(1.0, 0.0);
    for (int im = 0; im < M; ++im) {
      ex_part = ex_part + (emi * gather3(F.ex, hy, gx, cell_x1, cell_y2, im)).re;
      er_part = er_part + (emi * gather3(F.er, gy, hx, cell_x2, cell_y1, im)).re;
      et_part = et_part + (emi * gather3(F.et, hy, hx, cell_x2, cell_y2, im)).re;
      emi = emi * exp_min_itheta;
    }
    const double ey_part = er_part * exp_min_itheta.re + et_part * exp_min_itheta.im;
    const double ez_part = (-er_part) * exp_min_itheta.im + et_part * exp_min_itheta.re;
    const double e_part_mag = fac * sqrt((ex_part * ex_part + ey_part * ey_part) + ez_part * ez_part) / ATOMIC_E;

    const int64_t pid = S.id[i];
    double ppx, ppy, ppz, weight;
    IO::momenta(S, i, ppx, ppy, ppz, weight);
    int cs = isp;
    double time_left = rc.dt / ATOMIC_TIME;
    double j_ion = 0.0;
    while (time_left > 0.0 && P.s[cs].ionise) {
      const IonSpecies& q = P.s[cs];
      bool multiphoton_ionised = false;
      double rate;
      // the ADK rate of ionise.F90:522-530 / 1367-1375
      auto adk = [&]() {
        const double x = q.adk_scaling / e_part_mag;
        return q.ionisation_constant * pow(x, q.n_exp) * exp(IONISATION_EXPONENT * x) * (bessel_term(x, q.l) - 1.0);
      };
      if (mp && bsi) {  // multiphoton_tunnelling_bsi, ionise.F90:512-544
        if (e_part_mag > q.adk_maximum) {
          rate = q.bsi_constant * (1.0 - q.bsi_scaling / e_part_mag) + q.adk_bsi_cap;
        } else if (e_part_mag > q.keldysh) {
          rate = adk();
          if (e_part_mag > q.bsi_threshold)
            rate = fmin(q.bsi_constant * (1.0 - q.bsi_scaling / e_part_mag) + q.adk_bsi_cap, rate);
        } else if (e_part_mag > q.smallest_e_mag) {
          rate = fmin(q.adk_multiphoton_cap, q.multi_constant * pow(e_part_mag, q.k_photons_exponent));
          multiphoton_ionised = true;
        } else {
          break;
        }
      } else if (mp) {  // multiphoton_tunnelling
        if (e_part_mag > q.keldysh) {
          rate = adk();
        } else if (e_part_mag > q.smallest_e_mag) {
          rate = fmin(q.adk_multiphoton_cap, q.multi_constant * pow(e_part_mag, q.k_photons_exponent));
          multiphoton_ionised = true;
        } else {
          break;
        }
      } else if (bsi) {  // tunnelling_bsi
        if (e_part_mag > q.adk_maximum) {
          rate = q.bsi_constant * (1.0 - q.bsi_scaling / e_part_mag) + q.adk_bsi_cap;
        } else if (e_part_mag > q.smallest_e_mag) {
          rate = adk();
          if (e_part_mag > q.bsi_threshold)
            rate = fmin(q.bsi_constant * (1.0 - q.bsi_scaling / e_part_mag) + q.adk_bsi_cap, rate);
        } else {
          break;
        }
      } else {  // tunnelling
        if (e_part_mag > q.smallest_e_mag) rate = adk();
        else break;
      }
      const U4 r = philox4x32_10((uint32_t)pid, (uint32_t)((uint64_t)pid >> 32), (uint32_t)rec->step,
                                 TAG_IONISE | ((uint32_t)cs << 4), P.seed);
      const double sample = u01(r.v[0]);
      if (sample < 1.0 - exp(-1.0 * rate * time_left)) {
        if (q.release >= 0) {
          const SpeciesPtrs& E = L.sp[q.release];
          double nx_ = ppx * q.released_mass_fraction, ny_ = ppy * q.released_mass_fraction,
                 nz_ = ppz * q.released_mass_fraction;
          ppx = ppx - nx_;
          ppy = ppy - ny_;
          ppz = ppz - nz_;
          if (multiphoton_ionised) {
            const double kick = sqrt(2.0 * M0 * (q.k_photons_energy - q.energy));
            const double den = e_part_mag * ATOMIC_E;
            nx_ = nx_ + kick * fac * ex_part / den;
            ny_ = ny_ + kick * fac * ey_part / den;
            nz_ = nz_ + kick * fac * ez_part / den;
          }
          const int64_t k = take_slot(cnt + q.release, E);
          if (k >= 0) {
            IO::store(E, cnt + q.release, k, px0, py0, pz0, nx_, ny_, nz_, weight,
                      (int64_t)(((uint64_t)1 << 62) | ((uint64_t)pid << 4) | (uint64_t)cs), L.xg0, rc);
          } else {
            atomicOr(err, ERR_CAPACITY);
          }
        }
        time_left = time_left + log(1.0 - sample) / rate;
        j_ion = j_ion + (multiphoton_ionised ? q.k_photons_energy : q.energy);
        cs = q.ionise_to;
      } else {
        time_left = 0.0;
      }
    }
    if (cs == isp) continue;
    // the ion moves to its final species (ionised_list, then append_partlist)
    const SpeciesPtrs& T = L.sp[cs];
    const int64_t k = take_slot(cnt + cs, T);
    if (k >= 0) {
      IO::store(T, cnt + cs, k, px0, py0, pz0, ppx, ppy, ppz, weight, pid, L.xg0, rc);
    } else {
      atomicOr(err, ERR_CAPACITY);
    }
    IO::remove(S, i);
    atomicAdd((unsigned long long*)&cnt[isp].n_dead, 1ull);
    // ionisation current (ionise.F90:608-639)
    const double den = ATOMIC_E * e_part_mag;
    const double jf = dfac * j_ion * weight;
    const double jx_ion = jf * ex_part / (den * den), jy_ion = jf * ey_part / (den * den),
                 jz_ion = jf * ez_part / (den * den);
    if (fabs(jx_ion) > C_TINY || fabs(jy_ion) > C_TINY || fabs(jz_ion) > C_TINY) {
      const double jr_ion = jy_ion * exp_itheta.re + jz_ion * exp_itheta.im;
      const double jt_ion = (-jy_ion) * exp_itheta.im + jz_ion * exp_itheta.re;
      cplx eim = mk(1.0, 0.0);
      for (int im = 0; im < M; ++im) {
        for (int iy = -1; iy <= 1; ++iy)
          for (int ix = -1; ix <= 1; ++ix) {
            const cplx vx = ((gx[ix + 2] * hy[iy + 2]) * jx_ion) * eim;
            const cplx vr = ((hx[ix + 2] * gy[iy + 2]) * jr_ion) * eim;
            const cplx vt = ((hx[ix + 2] * hy[iy + 2]) * jt_ion) * eim;
            cplx* a = F.jx.ptr(cell_x1 + ix, cell_y2 + iy, im);
            atomicAdd(&a->re, vx.re);
            atomicAdd(&a->im, vx.im);
            a = F.jr.ptr(cell_x2 + ix, cell_y1 + iy, im);
            atomicAdd(&a->re, vr.re);
            atomicAdd(&a->im, vr.im);
            a = F.jt.ptr(cell_x2 + ix, cell_y2 + iy, im);
            atomicAdd(&a->re, vt.re);
            atomicAdd(&a->im, vt.im);
          }
        eim = eim * exp_itheta;
        if (im == 0) eim = eim * 2.0;
      }
    }
  }
}

__global__ void k_ion_snapshot(const SpeciesCounters* cnt, int nsp, int64_t* snap) {
  if (threadIdx.x < nsp) snap[threadIdx.x] = cnt[threadIdx.x].n_used;
}

// Slots taken beyond a full species are given back (the kernel flagged them).
__global__ void k_ion_clamp(SpeciesCounters* cnt, const int64_t* caps, int nsp) {
  const int s = threadIdx.x;
  if (s < nsp && cnt[s].n_used > caps[s]) cnt[s].n_used = caps[s];
}

}  // namespace

template <bool MIXED, typename FS>
static void launch_ionise_t(cudaStream_t s, const FS& F, const SpeciesPtrs* sp, int nsp, SpeciesCounters* cnt,
                            const IonParams& P, const StepRec* rec, const RunConst& rc, int64_t* snap,
                            const int64_t* caps, int* err, int nblocks, double xg0) {
  IonLaunch L;
  std::memset(&L, 0, sizeof(L));
  for (int i = 0; i < nsp && i < MAX_SPECIES; ++i) L.sp[i] = sp[i];
  L.P = P;
  L.xg0 = xg0;
  k_ion_snapshot<<<1, 32, 0, s>>>(cnt, nsp, snap);
  for (int i = 0; i < nsp; ++i)
    if (P.s[i].ionise) k_ionise<MIXED><<<nblocks, 256, 0, s>>>(F, L, cnt, snap, i, rec, rc, err);
  k_ion_clamp<<<1, 32, 0, s>>>(cnt, caps, nsp);
}

void launch_ionise(cudaStream_t s, const FieldSet& F, const SpeciesPtrs* sp, int nsp, SpeciesCounters* cnt,
                   const IonParams& P, const StepRec* rec, const RunConst& rc, int64_t* snap, const int64_t* caps,
                   int* err, int nblocks) {
  launch_ionise_t<false>(s, F, sp, nsp, cnt, P, rec, rc, snap, caps, err, nblocks, 0.0);
}
void launch_ionise(cudaStream_t s, const FieldSetF& F, const SpeciesPtrs* sp, int nsp, SpeciesCounters* cnt,
                   const IonParams& P, const StepRec* rec, const RunConst& rc, int64_t* snap, const int64_t* caps,
                   int* err, int nblocks, double xg0) {
  launch_ionise_t<true>(s, F, sp, nsp, cnt, P, rec, rc, snap, caps, err, nblocks, xg0);
}

}  // namespace cyl
