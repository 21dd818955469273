// push_mixed.cu -- mixed-precision form of the fused gather + Boris push +
// per-mode deposit (push_particles, particles.F90:28-734), with particle_bcs
// (boundary.F90:1541-1889) applied in the same pass.
//
// Particles: absolute axial cell index (int32) + FP32 offset, y and z in units
// of dy (FP32), normalised momentum u = p/(m c) (FP32), FP32 weight.  They are
// kept sorted by cell tile (TX x TY cells).  One CTA works on one tile at a
// time (persistent loop):
//   1. the tile's E and B modes (+ halo) are staged in shared memory as FP32;
//   2. each particle is pushed in FP32, gathers from shared memory and
//      deposits its charge fluxes into FP32 shared-memory accumulators;
//   3. the accumulators are flushed once into the FP64 global currents, where
//      the per-row geometric factors of the reference (inv_area_rt,
//      inv_area_xt, inv_volume, particles.F90:189-217) are applied in FP64.
// The deposit uses the flux form of the reference's recursion: with
// F = jyh / inv_area_xt(cy) the radial recursion jyh = jyh*ratio - fjy*w_xt
// (particles.F90:658) becomes F(cy) = F(cy-1) - fc*hy*w_xt, so no geometric
// factor enters the FP32 sums.  Particles whose stencil leaves the staged
// region (fast particles between sorts, or appended by the moving window
// since the last sort) take the global path: FP64 field loads and FP64
// atomics per contribution.
#include <cfloat>

#include "cyl_common.cuh"
#include "cyl_kernels.cuh"
#include "push_mixed.cuh"

namespace cyl {

constexpr int DRIFT = 1;                       // cells a particle may drift from its tile
constexpr int RW = TILE_X + 2 * DRIFT + 5;     // staged region width (x)
constexpr int RH = TILE_Y + 2 * DRIFT + 5;     // staged region height (r)
constexpr int RCELLS = RW * RH;
constexpr int PUSH_THREADS = 256;

struct f2 {
  float re, im;
};
__device__ __forceinline__ f2 fm(float a, float b) { return {a, b}; }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ f2 operator*(float s, f2 a) { return {s * a.re, s * a.im}; }

// f2(phi) = -i (e^{i phi} - 1)/phi, f3 = (e^{i phi}(1 - i phi) - 1)/phi^2,
// f4 = i (e^{i phi}(2 - 2 i phi - phi^2) - 2)/phi^3: the per-mode deposit
// factors of particles.F90:603-625 without the 2 e^{i m theta0} prefactor.
// Their Taylor series sum_k c_k (i phi)^k have c_k = 1/(k+1)!,
// (k+1)/(k+2)! and (k+1)(k+2)/(k+3)!; FP32 evaluates the series below
// |phi| = 0.5 and the closed forms above.
__device__ __forceinline__ void mode_factors(float phi, f2 eip, f2& F2, f2& F3, f2& F4) {
  if (fabsf(phi) < 0.5f) {
    // Horner in z = i phi over k = 0..9
    const f2 z = fm(0.0f, phi);
    f2 a = fm(1.0f / 3628800.0f, 0.f), b = fm(10.0f / 39916800.0f, 0.f), c = fm(110.0f / 479001600.0f, 0.f);
    // coefficients for k = 8 .. 0
    const float c2[9] = {1.0f / 362880.0f, 1.0f / 40320.0f, 1.0f / 5040.0f, 1.0f / 720.0f, 1.0f / 120.0f,
                         1.0f / 24.0f, 1.0f / 6.0f, 1.0f / 2.0f, 1.0f};
    const float c3[9] = {9.0f / 3628800.0f, 8.0f / 362880.0f, 7.0f / 40320.0f, 6.0f / 5040.0f, 5.0f / 720.0f,
                         4.0f / 120.0f, 3.0f / 24.0f, 2.0f / 6.0f, 1.0f / 2.0f};
    const float c4[9] = {90.0f / 39916800.0f, 72.0f / 3628800.0f, 56.0f / 362880.0f, 42.0f / 40320.0f,
                         30.0f / 5040.0f, 20.0f / 720.0f, 12.0f / 120.0f, 6.0f / 24.0f, 2.0f / 6.0f};
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      a = a * z + fm(c2[k], 0.f);
      b = b * z + fm(c3[k], 0.f);
      c = c * z + fm(c4[k], 0.f);
    }
    F2 = a;
    F3 = b;
    F4 = c;
  } else {
    const float ip = 1.0f / phi, ip2 = ip * ip;
    const f2 em1 = fm(eip.re - 1.0f, eip.im);
    F2 = ip * fm(em1.im, -em1.re);  // -i (e - 1) / phi
    const f2 t3 = eip * fm(1.0f, -phi);
    F3 = ip2 * fm(t3.re - 1.0f, t3.im);
    const f2 t4 = eip * fm(2.0f - phi * phi, -2.0f * phi);
    const f2 u = fm(t4.re - 2.0f, t4.im);
    F4 = (ip2 * ip) * fm(-u.im, u.re);  // i * u / phi^3
  }
}

struct TileCtx {
  int x0, y0;  // Fortran indices of the staged region's first cell
};

// Shared-memory layout: fields [6][M][RCELLS] as float2, currents
// [3][M][RCELLS] as float2 (charge fluxes without geometric factors).
__device__ __forceinline__ float2* fld_s(float2* base, int comp, int m, int M, int cell) {
  return base + ((size_t)(comp * M + m) * RCELLS + cell);
}

// global-path helpers (FP64 storage)
__device__ __forceinline__ void gadd(cplx* p, double re, double im) {
  atomicAdd(&p->re, re);
  if (im != 0.0) atomicAdd(&p->im, im);
}

template <int M>
__device__ void push_particle(int64_t i, const SpeciesPtrs& sp, SpeciesCounters* cnt, const FieldSet& F,
                              const GeomTables& g, const MixedParams& P, const RunConst& rc,
                              float2* sf, float2* sj, const TileCtx& tc, bool staged, int nsh,
                              int apply_bcs) {
  int kx = sp.kx[i];
  if (kx == INT32_MIN) return;
  int k = kx - nsh;  // local 0-based floor cell index
  float fx = sp.fx[i];
  float y = sp.fy[i], z = sp.fz[i];
  float ux = sp.ux[i], uy = sp.uy[i], uz = sp.uz[i];
  const float w = sp.fw[i];

  float gam = sqrtf(ux * ux + uy * uy + uz * uz + 1.0f);
  float igm = 1.0f / gam;
  fx += ux * (P.cdt2_dx * igm);
  y += uy * (P.cdt2_dy * igm);
  z += uz * (P.cdt2_dy * igm);
  float r = sqrtf(y * y + z * z);
  float ir = (r > 0.f) ? 1.0f / r : 0.f;
  const float ct = (r > 0.f) ? y * ir : 1.f, st = (r > 0.f) ? z * ir : 0.f;  // e^{i theta}
  const float th05 = atan2f(z, y);
  const float cyr = r - 0.5f;

  // cell-centred (g) and staggered (h) weights, x2 the reference's convention
  const int a1 = (int)floorf(fx + 0.5f);
  const float frx1 = (float)a1 - fx;
  const int a2 = (int)floorf(fx);
  const float frx2 = ((float)a2 - fx) + 0.5f;
  const int cx1 = k + a1 + 1, cx2 = k + a2 + 1;  // Fortran cell indices
  const int b1 = (int)floorf(cyr + 0.5f);
  const float fry1 = (float)b1 - cyr;
  const int b2 = (int)floorf(cyr);
  const float fry2 = ((float)b2 - cyr) + 0.5f;
  const int cy1 = b1 + 1, cy2 = b2 + 1;
  float gx[3], gy[3], hx[5], hy[5];
  {
    float c2 = frx1 * frx1;
    gx[0] = 0.25f + c2 + frx1; gx[1] = 1.5f - 2.0f * c2; gx[2] = 0.25f + c2 - frx1;
    c2 = fry1 * fry1;
    gy[0] = 0.25f + c2 + fry1; gy[1] = 1.5f - 2.0f * c2; gy[2] = 0.25f + c2 - fry1;
    c2 = frx2 * frx2;
    hx[0] = 0.f; hx[1] = 0.25f + c2 + frx2; hx[2] = 1.5f - 2.0f * c2; hx[3] = 0.25f + c2 - frx2; hx[4] = 0.f;
    c2 = fry2 * fry2;
    hy[0] = 0.f; hy[1] = 0.25f + c2 + fry2; hy[2] = 1.5f - 2.0f * c2; hy[3] = 0.25f + c2 - fry2; hy[4] = 0.f;
  }
  // is the whole stencil (gather and deposit) inside the staged region?
  bool in = staged && (cx2 - 2 >= tc.x0) && (cx2 + 3 < tc.x0 + RW) && (cy2 - 2 >= tc.y0) &&
            (cy2 + 3 < tc.y0 + RH);
  if (!in) {
    if (cx2 - 2 < 1 - NG || cx2 + 3 > rc.nx + NG || cy2 - 2 < 1 - NG || cy2 + 3 > rc.ny + NG ||
        cx1 - 1 < 1 - NG || cx1 + 1 > rc.nx + NG || cy1 - 1 < 1 - NG || cy1 + 1 > rc.ny + NG) {
      atomicOr(P.err, ERR_CELL_RANGE);
      return;
    }
  }

  // gather (e_part.inc / b_part.inc): fields F = Re sum_m e^{-i m theta} F_m
  float exr = 0.f, err_ = 0.f, etr = 0.f, bxr = 0.f, brr = 0.f, btr = 0.f;
  {
    f2 emi = fm(1.f, 0.f);
    const f2 e1 = fm(ct, -st);
#pragma unroll
    for (int m = 0; m < M; ++m) {
      f2 acc[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) acc[q] = fm(0.f, 0.f);
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) {
          // (component, x index, y index, weight) for the six fields
          const int xs[6] = {cx1 - 1 + ii, cx2 - 1 + ii, cx2 - 1 + ii, cx2 - 1 + ii, cx1 - 1 + ii, cx1 - 1 + ii};
          const int ys[6] = {cy2 - 1 + jj, cy1 - 1 + jj, cy2 - 1 + jj, cy1 - 1 + jj, cy2 - 1 + jj, cy1 - 1 + jj};
          const float ws[6] = {hy[jj + 1] * gx[ii], gy[jj] * hx[ii + 1], hy[jj + 1] * hx[ii + 1],
                               gy[jj] * hx[ii + 1], hy[jj + 1] * gx[ii], gy[jj] * gx[ii]};
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            f2 v;
            if (in) {
              const float2 t = *fld_s(sf, q, m, M, (ys[q] - tc.y0) * RW + (xs[q] - tc.x0));
              v = fm(t.x, t.y);
            } else {
              const FView* fv = (q == 0) ? &F.ex : (q == 1) ? &F.er : (q == 2) ? &F.et
                              : (q == 3) ? &F.bx : (q == 4) ? &F.br : &F.bt;
              const cplx c = (*fv)(xs[q], ys[q], m);
              v = fm((float)c.re, (float)c.im);
            }
            acc[q] = acc[q] + ws[q] * v;
          }
        }
      }
      exr += (emi * acc[0]).re;
      err_ += (emi * acc[1]).re;
      etr += (emi * acc[2]).re;
      bxr += (emi * acc[3]).re;
      brr += (emi * acc[4]).re;
      btr += (emi * acc[5]).re;
      emi = emi * e1;
    }
  }
  const float eyr = err_ * ct - etr * st;
  const float ezr = err_ * st + etr * ct;
  const float byr = brr * ct - btr * st;
  const float bzr = brr * st + btr * ct;

  // Boris rotation
  const float cm = P.cmratio, ccm = P.ccmratio;
  const float uxm = ux + cm * exr, uym = uy + cm * eyr, uzm = uz + cm * ezr;
  gam = sqrtf(uxm * uxm + uym * uym + uzm * uzm + 1.0f);
  const float root = ccm / gam;
  const float tx = bxr * root, ty = byr * root, tz = bzr * root;
  const float tx2 = tx * tx, ty2 = ty * ty, tz2 = tz * tz;
  const float tau = 1.0f / (1.0f + tx2 + ty2 + tz2);
  const float uxp = ((1.0f + tx2 - ty2 - tz2) * uxm + 2.0f * ((tx * ty + tz) * uym + (tx * tz - ty) * uzm)) * tau;
  const float uyp = ((1.0f - tx2 + ty2 - tz2) * uym + 2.0f * ((ty * tz + tx) * uzm + (ty * tx - tz) * uxm)) * tau;
  const float uzp = ((1.0f - tx2 - ty2 + tz2) * uzm + 2.0f * ((tz * tx + ty) * uxm + (tz * ty - tx) * uym)) * tau;
  ux = uxp + cm * exr;
  uy = uyp + cm * eyr;
  uz = uzp + cm * ezr;
  gam = sqrtf(ux * ux + uy * uy + uz * uz + 1.0f);
  igm = 1.0f / gam;
  const float dxs = ux * (P.cdt2_dx * igm), dys = uy * (P.cdt2_dy * igm), dzs = uz * (P.cdt2_dy * igm);
  float fxn = fx + dxs;
  float yn = y + dys, zn = z + dzs;
  // v_theta at t + dt (m/s)
  float rn = sqrtf(yn * yn + zn * zn);
  float vt = 0.f;
  if (rn > 0.f) vt = (P.c * igm) * ((-uy) * (zn / rn) + uz * (yn / rn));

  // deposit: shape change from t+dt/2 to t+3dt/2
  const float fx3 = fxn + dxs, y3 = yn + dys, z3 = zn + dzs;
  const float r3 = sqrtf(y3 * y3 + z3 * z3);
  const float ir3 = (r3 > 0.f) ? 1.0f / r3 : 0.f;
  const float c3 = (r3 > 0.f) ? y3 * ir3 : 1.f, s3 = (r3 > 0.f) ? z3 * ir3 : 0.f;
  const float th15 = atan2f(z3, y3);
  const float cyr3 = r3 - 0.5f;
  const int a3 = (int)floorf(fx3);
  const float frx3 = ((float)a3 - fx3) + 0.5f;
  const int b3 = (int)floorf(cyr3);
  const float fry3 = ((float)b3 - cyr3) + 0.5f;
  const int dcx = a3 - a2, dcy = b3 - b2;
  if (dcx < -1 || dcx > 1 || dcy < -1 || dcy > 1) {
    atomicOr(P.err, ERR_CELL_RANGE);
    return;
  }
  float dhx[5], dhy[5], ogx[5], ogy[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) { ogx[q] = hx[q]; ogy[q] = hy[q]; dhx[q] = 0.f; dhy[q] = 0.f; }
  {
    float c2 = frx3 * frx3;
    const float h0 = 0.25f + c2 + frx3, h1 = 1.5f - 2.0f * c2, h2 = 0.25f + c2 - frx3;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int o = q - 2 - dcx;  // position relative to the new centre
      const float hn = (o == -1) ? h0 : (o == 0) ? h1 : (o == 1) ? h2 : 0.f;
      dhx[q] = hn - ogx[q];
    }
    c2 = fry3 * fry3;
    const float v0 = 0.25f + c2 + fry3, v1 = 1.5f - 2.0f * c2, v2 = 0.25f + c2 - fry3;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int o = q - 2 - dcy;
      const float hn = (o == -1) ? v0 : (o == 0) ? v1 : (o == 1) ? v2 : 0.f;
      dhy[q] = hn - ogy[q];
    }
  }
  const int xmin = -1 + (dcx - 1) / 2, xmax = 1 + (dcx + 1) / 2;
  const int ymin = -1 + (dcy - 1) / 2, ymax = 1 + (dcy + 1) / 2;
  const float qwf = P.q_fac * w;      // q * w * fac
  const float fc = qwf * P.idt;       // fcx = fcy
  const float fcz = qwf * vt;
  const float third = 1.0f / 3.0f;
  // e^{i theta_05}, e^{i dtheta}
  const f2 e05 = fm(ct, st);
  const f2 edt = fm(c3, s3) * fm(ct, -st);
  float dth = th15 - th05;
  f2 eimt = fm(1.f, 0.f), eimd = fm(1.f, 0.f);
#pragma unroll
  for (int m = 0; m < M; ++m) {
    f2 F2 = fm(1.f, 0.f), F3 = fm(0.5f, 0.f), F4 = fm(third, 0.f), pre = fm(1.f, 0.f);
    if (m > 0) {
      eimt = eimt * e05;
      eimd = eimd * edt;
      mode_factors((float)m * dth, eimd, F2, F3, F4);
      pre = 2.0f * eimt;
      F2 = pre * F2;
      F3 = pre * F3;
      F4 = pre * F4;
    }
    f2 qr[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) qr[q] = fm(0.f, 0.f);
    for (int iy = ymin; iy <= ymax; ++iy) {
      const float gyv = ogy[iy + 2], hyv = dhy[iy + 2];
      f2 w_rt, ym1;
      if (m == 0) {
        w_rt = fm(gyv + 0.5f * hyv, 0.f);
        ym1 = fm(0.5f * gyv + third * hyv, 0.f);
      } else {
        w_rt = gyv * F2 + hyv * F3;
        ym1 = gyv * F3 + hyv * F4;
      }
      const int cy = cy2 + iy;
      f2 qx = fm(0.f, 0.f);
      for (int ix = xmin; ix <= xmax; ++ix) {
        const float gxv = ogx[ix + 2], hxv = dhx[ix + 2];
        const f2 w_xt = (m == 0) ? fm(gxv + 0.5f * hxv, 0.f) : (gxv * F2 + hxv * F3);
        const f2 w_xr = gxv * w_rt + hxv * ym1;
        qx = qx - (fc * hxv) * w_rt;
        qr[ix + 2] = qr[ix + 2] - (fc * hyv) * w_xt;
        const f2 qt = fcz * w_xr;
        const int cx = cx2 + ix;
        if (in) {
          float2* jx = fld_s(sj, 0, m, M, (cy - tc.y0) * RW + (cx + 1 - tc.x0));
          float2* jr = fld_s(sj, 1, m, M, (cy + 1 - tc.y0) * RW + (cx - tc.x0));
          float2* jt = fld_s(sj, 2, m, M, (cy - tc.y0) * RW + (cx - tc.x0));
          atomicAdd(&jx->x, qx.re);
          atomicAdd(&jr->x, qr[ix + 2].re);
          atomicAdd(&jt->x, qt.re);
          if (m > 0) {
            atomicAdd(&jx->y, qx.im);
            atomicAdd(&jr->y, qr[ix + 2].im);
            atomicAdd(&jt->y, qt.im);
          }
        } else {
          const double fx_ = g.inv_area_rt[cy - (1 - JNG)];
          const double fr_ = g.inv_area_xt[cy - (0 - JNG)];
          const double ft_ = g.inv_volume[cy - (1 - JNG)];
          gadd(&F.jx(cx + 1, cy, m), (double)qx.re * fx_, (double)qx.im * fx_);
          gadd(&F.jr(cx, cy + 1, m), (double)qr[ix + 2].re * fr_, (double)qr[ix + 2].im * fr_);
          gadd(&F.jt(cx, cy, m), (double)qt.re * ft_, (double)qt.im * ft_);
        }
      }
    }
  }

  // store position at t + dt, then particle_bcs in cell units
  int kk = (int)floorf(fxn);
  int knew = k + kk;
  float fnew = fxn - (float)kk;
  if (fnew >= 1.0f) { fnew -= 1.0f; knew += 1; }
  if (fnew < 0.0f) { fnew = 0.0f; }
  bool dead = false;
  if (apply_bcs) {
    const float xc = (float)knew + fnew;  // cell_x_r relative to this step's grid
    const float xlo = P.x_lo, xhi = P.x_hi;  // x_min_local, x_max_local in cells
    if (xc < xlo) {
      const int b = sp.bc[CYL_BD_X_MIN];
      if (b == CYL_BC_REFLECT) {
        const float v = 2.0f * P.x_sys_lo - xc;
        knew = (int)floorf(v); fnew = v - (float)knew; ux = -ux;
      } else if (b == CYL_BC_PERIODIC) {
        knew += rc.nx;
      }
      if (xc < P.x_out_lo && b != CYL_BC_PERIODIC) dead = true;
    }
    if (xc >= xhi) {
      const int b = sp.bc[CYL_BD_X_MAX];
      if (b == CYL_BC_REFLECT) {
        const float v = 2.0f * P.x_sys_hi - xc;
        knew = (int)floorf(v); fnew = v - (float)knew; ux = -ux;
      } else if (b == CYL_BC_PERIODIC) {
        knew -= rc.nx;
      }
      if (xc >= P.x_out_hi && b != CYL_BC_PERIODIC) dead = true;
    }
    if (rn >= P.r_hi) {
      const int b = sp.bc[CYL_BD_Y_MAX];
      if (b == CYL_BC_REFLECT) {
        const float f = 2.0f * P.r_sys / rn - 1.0f;
        yn *= f; zn *= f;
        const float rr = sqrtf(yn * yn + zn * zn);
        const float cc = yn / rr, ss = zn / rr;
        const float pr = uy * cc + uz * ss, pt = -uy * ss + uz * cc;
        uy = -pr * cc - pt * ss;
        uz = -pr * ss + pt * cc;
      }
      if (rn >= P.r_out && b != CYL_BC_PERIODIC) dead = true;
    }
  }
  if (dead) {
    sp.kx[i] = INT32_MIN;
    atomicAdd((unsigned long long*)&cnt->n_dead, 1ull);
    return;
  }
  sp.kx[i] = knew + nsh;
  sp.fx[i] = fnew;
  sp.fy[i] = yn;
  sp.fz[i] = zn;
  sp.ux[i] = ux;
  sp.uy[i] = uy;
  sp.uz[i] = uz;
}

template <int M>
__global__ void __launch_bounds__(PUSH_THREADS) k_push_mixed(FieldSet F, GeomTables g, SpeciesPtrs sp,
                                                              SpeciesCounters* cnt, const StepRec* rec,
                                                              RunConst rc, MixedParams P, TileTable* tt,
                                                              int apply_bcs) {
  extern __shared__ float2 smem[];
  float2* sf = smem;                          // 6 * M * RCELLS
  float2* sj = smem + (size_t)6 * M * RCELLS;  // 3 * M * RCELLS
  __shared__ int s_tile;
  const int nsh = rec->nshift_total;
  // cell-unit boundaries of this step's grid
  P.x_lo = -0.5f;
  P.x_hi = (float)rc.nx - 0.5f;
  P.x_sys_lo = (float)((rec->x_min - rec->x_grid_min) / rc.dx);
  P.x_sys_hi = (float)((rec->x_max - rec->x_grid_min) / rc.dx);
  P.x_out_lo = P.x_sys_lo - 2.0f;
  P.x_out_hi = P.x_sys_hi + 2.0f;
  const int ntiles = tt->ntiles;
  const int64_t n_sorted = tt->n_sorted;
  const int64_t n_used = cnt->n_used;
  const int64_t ntail = n_used > n_sorted ? n_used - n_sorted : 0;
  const int ntail_chunks = (int)((ntail + PUSH_THREADS - 1) / PUSH_THREADS);
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(&tt->next, 1);
    __syncthreads();
    const int t = s_tile;
    __syncthreads();
    if (t >= ntiles + ntail_chunks) break;
    if (t >= ntiles) {
      // appended particles not yet sorted: global path
      const int64_t i = n_sorted + (int64_t)(t - ntiles) * PUSH_THREADS + threadIdx.x;
      TileCtx tc{0, 0};
      if (i < n_used) push_particle<M>(i, sp, cnt, F, g, P, rc, sf, sj, tc, false, nsh, apply_bcs);
      continue;
    }
    const int64_t p0 = tt->start[t], p1 = tt->start[t + 1];
    if (p1 <= p0) continue;
    const int tx = t % tt->ntx, ty = t / tt->ntx;
    TileCtx tc;
    tc.x0 = (tt->tx_min + tx) * TILE_X - nsh + 1 - DRIFT - 2;
    tc.y0 = ty * TILE_Y + 1 - DRIFT - 2;
    // stage fields (FP64 -> FP32) and clear the current accumulators
    const bool inside = tc.x0 >= 1 - NG && tc.x0 + RW - 1 <= rc.nx + NG && tc.y0 >= 1 - NG &&
                        tc.y0 + RH - 1 <= rc.ny + NG;
    if (inside) {
      const FView* fv[6] = {&F.ex, &F.er, &F.et, &F.bx, &F.br, &F.bt};
      for (int e = threadIdx.x; e < 6 * M * RCELLS; e += PUSH_THREADS) {
        const int cell = e % RCELLS, cm = e / RCELLS;
        const int comp = cm / M, m = cm % M;
        const cplx v = (*fv[comp])(tc.x0 + cell % RW, tc.y0 + cell / RW, m);
        sf[e] = make_float2((float)v.re, (float)v.im);
      }
      for (int e = threadIdx.x; e < 3 * M * RCELLS; e += PUSH_THREADS) sj[e] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int64_t i = p0 + threadIdx.x; i < p1; i += PUSH_THREADS)
      push_particle<M>(i, sp, cnt, F, g, P, rc, sf, sj, tc, inside, nsh, apply_bcs);
    __syncthreads();
    if (inside) {
      // flush: one FP64 add per non-zero accumulator, geometric factor per row
      for (int e = threadIdx.x; e < 3 * M * RCELLS; e += PUSH_THREADS) {
        const float2 v = sj[e];
        if (v.x == 0.f && v.y == 0.f) continue;
        const int cell = e % RCELLS, cm = e / RCELLS;
        const int comp = cm / M, m = cm % M;
        const int cx = tc.x0 + cell % RW, cy = tc.y0 + cell / RW;
        double f;
        cplx* dst;
        if (comp == 0) { f = g.inv_area_rt[cy - (1 - JNG)]; dst = &F.jx(cx, cy, m); }
        else if (comp == 1) { f = g.inv_area_xt[cy - 1 - (0 - JNG)]; dst = &F.jr(cx, cy, m); }
        else { f = g.inv_volume[cy - (1 - JNG)]; dst = &F.jt(cx, cy, m); }
        gadd(dst, (double)v.x * f, (double)v.y * f);
      }
    }
  }
}

size_t push_mixed_smem(int M) { return (size_t)9 * M * RCELLS * sizeof(float2); }

int push_mixed_blocks_per_sm(int M) {
  const size_t smem = push_mixed_smem(M);
  int nb = 1;
  switch (M) {
#define OCC(MM)                                                                                    \
  case MM:                                                                                         \
    cudaFuncSetAttribute(k_push_mixed<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_push_mixed<MM>, PUSH_THREADS, smem);      \
    break;
    OCC(1) OCC(2) OCC(3) OCC(4)
#undef OCC
    default:
      break;
  }
  return nb < 1 ? 1 : nb;
}

void launch_push_mixed(cudaStream_t s, const FieldSet& F, const GeomTables& g, const SpeciesPtrs& sp,
                       SpeciesCounters* cnt, const StepRec* rec, const RunConst& rc, int apply_bcs,
                       int* err, int nblocks, const MixedParams& P0, TileTable* tt) {
  MixedParams P = P0;
  P.err = err;
  const size_t smem = push_mixed_smem(rc.M);
  cudaMemsetAsync(&tt->next, 0, sizeof(int), s);
  switch (rc.M) {
#define CASE(MM)                                                                                   \
  case MM:                                                                                         \
    cudaFuncSetAttribute(k_push_mixed<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    k_push_mixed<MM><<<nblocks, PUSH_THREADS, smem, s>>>(F, g, sp, cnt, rec, rc, P, tt, apply_bcs); \
    break;
    CASE(1) CASE(2) CASE(3) CASE(4)
#undef CASE
    default:
      break;
  }
}

}  // namespace cyl
