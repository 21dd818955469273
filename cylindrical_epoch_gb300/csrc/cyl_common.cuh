// cyl_common.cuh -- shared definitions of the GB300 quasi-3D PIC step.
//
// Complex arithmetic follows the operation trees of the reference Fortran
// (gfortran evaluates left to right; a real operand of a complex product is
// applied component-wise).  The FP64 kernels are compiled with --fmad=false
// so each operation rounds once, as in the reference build.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/cylpic.h"
#include "cyl_convert.cuh"

#define CYL_HD __host__ __device__ __forceinline__

namespace cyl {

constexpr int NG = CYL_NG;  // ghost width of every mode array
constexpr int JNG = CYL_NG;
constexpr int PNG = 3;
constexpr int MAX_SPECIES = 8;
constexpr int MAX_INJ_SHIFTS = 2;  // window shifts per step the device injector handles
constexpr int MAX_LASERS = 8;
constexpr int MAX_MODES = 8;

// constants.F90:171-181
constexpr double PI = 3.141592653589793238462643383279503;
constexpr double CLIGHT = 2.99792458e8;
constexpr double KB = 1.3806488e-23;
constexpr double EPS0 = 8.854187817620389850536563031710750e-12;

struct cplx {
  double re, im;
};
CYL_HD cplx mk(double r, double i) { return {r, i}; }
CYL_HD cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
CYL_HD cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
CYL_HD cplx operator-(cplx a) { return {-a.re, -a.im}; }
CYL_HD cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
CYL_HD cplx operator*(double s, cplx a) { return {s * a.re, s * a.im}; }
CYL_HD cplx operator*(cplx a, double s) { return {a.re * s, a.im * s}; }
CYL_HD cplx operator/(cplx a, double s) { return {a.re / s, a.im / s}; }
CYL_HD cplx operator+(cplx a, double s) { return {a.re + s, a.im}; }
CYL_HD cplx operator-(cplx a, double s) { return {a.re - s, a.im}; }
CYL_HD cplx operator-(double s, cplx a) { return {s - a.re, -a.im}; }
CYL_HD cplx operator+(double s, cplx a) { return {s + a.re, a.im}; }
// 1/z by range-reduced (Smith) division, real numerator 1.
CYL_HD cplx crecip(cplx z) {
  double c = z.re, d = z.im;
  if (fabs(c) < fabs(d)) {
    double ratio = c / d;
    double div = c * ratio + d;
    return {(1.0 * ratio + 0.0) / div, (0.0 * ratio - 1.0) / div};
  } else {
    double ratio = d / c;
    double div = d * ratio + c;
    return {(0.0 * ratio + 1.0) / div, (0.0 - 1.0 * ratio) / div};
  }
}
constexpr cplx IMAGI = {0.0, 1.0};

// FP32 complex, the storage of E and B in the mixed-precision form.
struct cplxf {
  float re, im;
};
// On the device the FP32 <-> FP64 conversions use the integer routines of
// cyl_convert.cuh (the conversion instructions run on the narrow FP64 pipe).
CYL_HD cplx to_c(const cplx& v) { return v; }
CYL_HD cplx to_c(const cplxf& v) {
#ifdef __CUDA_ARCH__
  return {f2d_bits(v.re), f2d_bits(v.im)};
#else
  return {(double)v.re, (double)v.im};
#endif
}
CYL_HD void from_c(cplx& d, const cplx& v) { d = v; }
CYL_HD void from_c(cplxf& d, const cplx& v) {
#ifdef __CUDA_ARCH__
  d.re = d2f_bits(v.re);
  d.im = d2f_bits(v.im);
#else
  d.re = (float)v.re;
  d.im = (float)v.im;
#endif
}

// Reference to one element of a mode array: reads convert to FP64 complex,
// writes convert back to the storage type (exact for FP64 storage).
template <typename T>
struct FRef {
  T* q;
  CYL_HD operator cplx() const { return to_c(*q); }
  CYL_HD FRef& operator=(const cplx& v) {
    from_c(*q, v);
    return *this;
  }
  CYL_HD FRef& operator=(const FRef& o) {
    from_c(*q, to_c(*o.q));
    return *this;
  }
};

// Layout of one complex mode array in HBM: Fortran order with ghosts,
// F(1-ng:nx+ng, 1-ng:ny+ng, 0:M-1), x fastest.
template <typename T>
struct FViewT {
  T* p;
  int nxg, nyg;
  CYL_HD T* ptr(int ix, int iy, int m) const {
    return p + ((int64_t)(ix + NG - 1) + (int64_t)nxg * ((int64_t)(iy + NG - 1) + (int64_t)nyg * m));
  }
  CYL_HD FRef<T> operator()(int ix, int iy, int m) const { return FRef<T>{ptr(ix, iy, m)}; }
};
using FView = FViewT<cplx>;
using FViewF = FViewT<cplxf>;

// Stagger table (setup.F90:126-136 with constants.F90:291-296).
// which: 0 exm, 1 erm, 2 etm, 3 bxm, 4 brm, 5 btm
CYL_HD bool stag_x(int w) { return w == 1 || w == 2 || w == 3; }
CYL_HD bool stag_y(int w) { return w == 0 || w == 2 || w == 4; }

// Scalars of one step, prepared on the host in the reference's order
// (the Fortran module globals time, x_grid_min, bc_field, ... at the point
// where each stage reads them).
struct StepRec {
  double time_half;          // time during update_eb_fields_half and the push
  double time_final;         // time during update_eb_fields_final
  double x_grid_min;         // grid of this step's push (before any shift)
  double x_min, x_max;       // system extent before any shift
  double x_min_local, x_max_local;
  int32_t bc_field[4];       // field bcs during this step (after mapping)
  int32_t add_laser[4];
  int32_t nshift;            // window shifts at the end of the step
  int32_t pad0;
  int32_t bc_field_after[4]; // field bcs after moving_window's start switch
  double x_grid_min_after;   // grid after the shifts
  double x_min_after, x_max_after, x_min_local_after, x_max_local_after;
  int64_t inject_off[MAX_SPECIES];  // offsets into the injection batch
  int64_t inject_cnt[MAX_SPECIES];
  int64_t src_off;           // offset of this step's laser source vectors
  int32_t nshift_total;      // window shifts before this step (mixed-form cell origin)
  int32_t nshift_total_after;
  int64_t step;              // steps completed before this one (the reference's step during the push)
  // window injection drawn on the device from the counter stream (counter_rng.cuh):
  // per shift c of this step and species s, the column's left edge, the
  // global shift index, the clamped column density, and where its particles
  // go in the injection batch (inject_off[s] + ...) with their first id
  int32_t inj_counter;       // 1: the kernel k_inject_counter makes this step's batch
  int32_t inj_nshift;
  double inj_x0[MAX_INJ_SHIFTS];
  int64_t inj_shift[MAX_INJ_SHIFTS];
  double inj_dens[MAX_INJ_SHIFTS][MAX_SPECIES];
  int64_t inj_base[MAX_INJ_SHIFTS][MAX_SPECIES];
  int64_t inj_id0[MAX_INJ_SHIFTS][MAX_SPECIES];
  int64_t inj_n[MAX_INJ_SHIFTS][MAX_SPECIES];
};

// Run-constant geometry and physics parameters (pushed by value).
struct RunConst {
  int nx, ny, M, nxg, nyg;
  double dx, dy, dt;
  double y_grid_min, y_max, y_max_local;
  double length_x, length_y;
  int bc_allspecies[4];
  int bc_mask;  // BCM_* bits: field bc kinds this run can meet (before and after the window starts)
};

// Field bc kinds present in a run, so that ghost-cell phases with nothing to
// do are not launched.
constexpr int BCM_PERIODIC_X = 1;
constexpr int BCM_CONDUCT = 2;
constexpr int BCM_OTHER = 4;  // clamp, simple_laser, simple_outflow, zero_gradient

struct SpeciesPtrs {
  // FP64 form: Cartesian position (m), momentum (kg m/s), weight
  double *x, *y, *z, *px, *py, *pz, *w;
  int64_t* id;
  int64_t cap;
  double charge, mass;
  int immobile;
  int bc[4];
  // mixed form, in the same allocation: absolute axial cell index and FP32
  // offset in [0,1) (x = x_grid_min0 + (kx + fx) dx), y and z in units of
  // dy, normalised momentum u = p/(m c), weight
  int32_t* kx;
  float *fx, *fy, *fz, *ux, *uy, *uz, *fw;
};

// Device error word bits.
constexpr int ERR_CAPACITY = 1;
constexpr int ERR_CELL_RANGE = 2;    // particle stencil left the ghosted grid
constexpr int ERR_NONFINITE = 4;
constexpr int ERR_TMA_TIMEOUT = 8;  // a TMA tile copy did not complete within its bounded wait

#ifdef __CUDACC__
// Sum K per-thread values over a 1-D block (warp shuffles, then the warps'
// partial sums through shared memory) and add the block's totals to
// out[0..K) with one atomic each.  Every thread of the block must call it.
template <int K>
__device__ __forceinline__ void block_sum_add(double (&v)[K], double* out) {
  __shared__ double part[32][K];
  for (int k = 0; k < K; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < K; ++k) part[wid][k] = v[k];
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < K; ++k) {
      double t = lane < nw ? part[lane][k] : 0.0;
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) atomicAdd(&out[k], t);
    }
  }
}
#endif

}  // namespace cyl
