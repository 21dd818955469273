// push_mixed.cu -- mixed-precision form of the fused gather + Boris push +
// per-mode deposit (push_particles, particles.F90:28-734), with particle_bcs
// (boundary.F90:1541-1889) applied in the same pass.
//
// Particles: absolute axial cell index (int32) + FP32 offset, y and z in units
// of dy (FP32), normalised momentum u = p/(m c) (FP32), FP32 weight; E and B
// are FP32, the currents FP64.  Particles are kept sorted by cell tile
// (TILE_X x TILE_Y cells).  One CTA works on one tile at a time (static
// round-robin over the tiles):
//   1. the tile's E and B modes plus a halo are staged in shared memory;
//   2. each particle is pushed in FP32, gathers from shared memory and adds
//      its charge fluxes to fixed-point (int32) shared-memory accumulators;
//   3. the accumulators are flushed once into the FP64 global currents; the
//      per-row geometric factors of the reference (inv_area_rt, inv_area_xt,
//      inv_volume, particles.F90:189-217) are applied there.
// The deposit uses the flux form of the reference's recursion: with
// F = jyh / inv_area_xt(cy) the radial recursion jyh = jyh*ratio - fjy*w_xt
// (particles.F90:658) becomes F(cy) = F(cy-1) - fc*hy*w_xt, so no geometric
// factor enters the tile sums.  A particle whose stencil leaves the staged
// region (it drifted since the last sort) is deferred to a second kernel that
// gathers from global memory and adds each contribution with an FP64 atomic;
// so are the particles the moving window appended since the last sort.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "cyl_common.cuh"
#include "cyl_convert.cuh"
#include "cyl_kernels.cuh"
#include "push_mixed.cuh"

// This file is compiled once per tile shape with -DCYL_TILE_X, -DCYL_TILE_Y,
// -DCYL_TILE_NS (the namespace of that build) and -DCYL_TILE_FNS (the name
// of its PushMixedFns accessor).
#if !defined(CYL_TILE_X) || !defined(CYL_TILE_Y) || !defined(CYL_TILE_NS) || !defined(CYL_TILE_FNS)
#error "push_mixed.cu is built per tile shape: define CYL_TILE_X, CYL_TILE_Y, CYL_TILE_NS, CYL_TILE_FNS"
#endif

namespace cyl {
namespace CYL_TILE_NS {

constexpr int TILE_X = CYL_TILE_X;          // cells per tile along x
constexpr int TILE_Y = CYL_TILE_Y;          // cells per tile along r
constexpr int DRIFT = 1;                    // cells a particle may drift from its tile
constexpr int RW = TILE_X + 2 * DRIFT + 5;  // staged region width (x)
constexpr int RH = TILE_Y + 2 * DRIFT + 5;  // staged region height (r)
constexpr int RCELLS = RW * RH;
// Modes m >= 1 are staged by TMA (cp.async.bulk.tensor) as boxes of TW x RH
// complex values: the box's first column is the staged region's first column
// rounded down to an even index (a TMA copy starts on a 16-byte boundary, two
// 8-byte complex values), so TW = RW + 1 covers the region; each plane starts
// on a 128-byte boundary.
constexpr int TW = RW + 1;
static_assert((TW * 8) % 16 == 0, "TMA box rows must be whole 16-byte units");
constexpr int TPLANE = ((TW * RH * 8 + 127) / 128) * 128 / 8;  // float2 per TMA plane
constexpr int PUSH_THREADS = 256;
// Resident CTAs per SM the register budget is sized for: 3 (at most 80
// registers a thread, 24 warps an SM) for m = 0..1, 2 (at most 128) for
// three or more modes, whose per-mode gather and deposit state spills at
// 80 registers.  Measured on the 2048x256 / 4096x512 wakefields: M = 2
// 0.433 ms with 3 against 0.510 with 2; M = 3 0.797 against 0.742; M = 4
// 15.8 ms against 14.5.
template <int M>
constexpr int push_min_blocks() {
  return M >= 3 ? 2 : 3;
}

struct f2 {
  float re, im;
};
__device__ __forceinline__ f2 fm(float a, float b) { return {a, b}; }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ f2 operator*(float s, f2 a) { return {s * a.re, s * a.im}; }

// Paired FP32 arithmetic (one FFMA2 / FMUL2 instruction for two lanes of
// FP32 work): acc + s v and s v for a scalar s and a pair v.
__device__ __forceinline__ float2 pfma(float s, float2 v, float2 acc) { return __ffma2_rn(make_float2(s, s), v, acc); }
__device__ __forceinline__ float2 pfma(float2 s, float2 v, float2 acc) { return __ffma2_rn(s, v, acc); }
__device__ __forceinline__ float2 pmul(float s, float2 v) { return __fmul2_rn(make_float2(s, s), v); }
__device__ __forceinline__ float2 P2(f2 a) { return make_float2(a.re, a.im); }
__device__ __forceinline__ f2 U2(float2 a) { return {a.x, a.y}; }

// f2(phi) = -i (e^{i phi} - 1)/phi, f3 = (e^{i phi}(1 - i phi) - 1)/phi^2,
// f4 = i (e^{i phi}(2 - 2 i phi - phi^2) - 2)/phi^3: the per-mode deposit
// factors of particles.F90:603-625 without the 2 e^{i m theta0} prefactor.
// Their Taylor series sum_k c_k (i phi)^k have c_k = 1/(k+1)!,
// (k+1)/(k+2)! and (k+1)(k+2)/(k+3)!.  Below |phi| = 0.5 (where the closed
// forms cancel) FP32 sums the series to k = 7 (the first omitted term is
// below 1e-8 of the sum) as two real polynomials in phi^2: the even terms
// give the real part, the odd terms the imaginary part.
__device__ __forceinline__ f2 series(float p2, float phi, float c0, float c1, float c2, float c3, float c4, float c5,
                                     float c6, float c7) {
  const float re = fmaf(fmaf(fmaf(-c6, p2, c4), p2, -c2), p2, c0);
  const float im = phi * fmaf(fmaf(fmaf(-c7, p2, c5), p2, -c3), p2, c1);
  return fm(re, im);
}
__device__ __forceinline__ void mode_factors(float phi, f2 eip, f2& F2, f2& F3, f2& F4) {
  if (fabsf(phi) < 0.5f) {
    const float p2 = phi * phi;
    F2 = series(p2, phi, 1.0f, 1.0f / 2.0f, 1.0f / 6.0f, 1.0f / 24.0f, 1.0f / 120.0f, 1.0f / 720.0f,
                1.0f / 5040.0f, 1.0f / 40320.0f);
    F3 = series(p2, phi, 1.0f / 2.0f, 2.0f / 6.0f, 3.0f / 24.0f, 4.0f / 120.0f, 5.0f / 720.0f, 6.0f / 5040.0f,
                7.0f / 40320.0f, 8.0f / 362880.0f);
    F4 = series(p2, phi, 2.0f / 6.0f, 6.0f / 24.0f, 12.0f / 120.0f, 20.0f / 720.0f, 30.0f / 5040.0f,
                42.0f / 40320.0f, 56.0f / 362880.0f, 72.0f / 3628800.0f);
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

// Shared-memory layout: staged fields (planes of RCELLS cells, see Gather);
// current accumulators [3][M][re, im][hi, lo][RCELLS] int32 (fixed point,
// see sadd).
struct Tile {
  const float2* sf;  // mode-0 planes (RCELLS cells each)
  const float2* tm;  // modes m >= 1: TMA planes (TPLANE float2 each, row pitch TW)
  int* sj;
  int xs;           // Fortran x index of the TMA boxes' first column
  int x0, y0;       // Fortran indices of the staged region's first cell
  float s_xr, s_t;  // accumulator units per unit of jx / jr and of jtheta flux
  int* dirty;       // set by every warp that deposits into the accumulators
};

// Fixed-point scales of a tile's current accumulators.  One particle of
// weight w and normalised momentum u after its push adds at most
//   8 |q fac| w / dt * min(2, 3 d)   to a jx or jr accumulator value, and
//   16 |q fac| w c * min(1, |u|)     to a jtheta value,
// d = (c dt / min(dx, dy)) min(1, |u|) its displacement in cells over the
// deposit's interval: the partial sums of its weight changes are the charge
// its shape moves across a cell face, at most 1.5 d (the shape's peak
// density, twice the reference's convention) and at most 2 (a whole cell
// crossed); |v| <= c min(1, |u|); the flux weights with the 2 e^{i m theta}
// prefactor are at most 4 and 8.  The tile's bound takes the tile's largest
// weight, and for |u| the largest momentum before the push plus two
// electric kicks at the largest staged field (the magnetic rotation keeps
// |u|), with a margin for FP32 rounding.  It is scaled to 2^30 / k,
// k = max(1, n / 2^16) for a tile of n particles, so that neither one add
// (|v| <= 2^30) nor the sum of at most 2^16 adds of one hi word overflows.
// The quantum is thus 2^-30 of what the tile's fastest, heaviest particle
// could deposit, not of a worst case for the species: a tile of particles
// at rest in a weak field gets a fine quantum, a tile with a relativistic
// particle the coarse one, and within a tile the relative error of an add
// grows only with the spread of the tile's currents.
struct TileBound {
  float w_max;   // largest |weight|
  float u2_max;  // largest |u|^2 before the push
  float e_sum;   // bound on |E| at a particle: 4 sum_comp sum_m max|F_m|
};
__device__ __forceinline__ void tile_scales(Tile& t, int64_t n, const TileBound& b, const MixedParams& P) {
  const float k = fmaxf(1.0f, (float)n * (1.0f / 65536.0f));
  const float u = (sqrtf(b.u2_max) + 2.0f * fabsf(P.cmratio) * b.e_sum) * 1.001f;
  const float vfac = fminf(1.0f, u);
  const float d = 2.0f * fmaxf(P.cdt2_dx, P.cdt2_dy) * vfac;
  const float qw = fabsf(P.q_fac) * b.w_max;
  const float bxr = 8.0f * qw * P.idt * k * fminf(2.0f, 3.0f * d), bt = 16.0f * qw * P.c * k * vfac;
  t.s_xr = bxr > 0.f ? 1073741824.0f / bxr : 0.f;
  t.s_t = bt > 0.f ? 1073741824.0f / bt : 0.f;
}

// Block-wide maximum of non-negative floats: their bit patterns order as
// unsigned integers.  Every thread of the CTA takes part; the result is in
// slot[0] after the next __syncthreads (slot must be 0 before).
__device__ __forceinline__ void block_max_into(unsigned* slot, float v) {
  const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(v));
  if ((threadIdx.x & 31) == 0) atomicMax(slot, m);
}

// Staged fields of a tile, in shared memory:
//   mode 0 (RCELLS cells per plane, row pitch RW):
//     plane 0: float2 {Re Ex_0, Re Br_0}   plane 1: float2 {Re Er_0, Re Bx_0}
//     plane 2: float {Re Et_0} then float {Re Bt_0} (one float2 plane)
//   modes m >= 1: float2 complex F_m of field q in TMA plane q (M-1) + m - 1
//     (TPLANE float2 each, row pitch TW, first column at Fortran x = xs)
// Mode 0 contributes Re F_0 alone; Ex and Br share their stencil (gx along
// x at cell_x1, hy along r at cell_y2), and so do Er and Bx (hx at cell_x2,
// gy at cell_y1), so each pair is gathered by one 64-bit load and one
// paired FMA.
constexpr int PLANES_M0 = 3;

template <int M, bool SHARED>
struct Gather {
  // SHARED: read from the staged tile; else from the FP32 global arrays
  __device__ __forceinline__ static FViewF view(const FieldSetF& F, int q) {
    const cplxf* base = (q == 0) ? F.ex.p : (q == 1) ? F.er.p : (q == 2) ? F.et.p : (q == 3) ? F.bx.p
                      : (q == 4) ? F.br.p : F.bt.p;
    return FViewF{const_cast<cplxf*>(base), F.ex.nxg, F.ex.nyg};
  }
  __device__ __forceinline__ static float re0(const FieldSetF& F, int q, int x, int y) {
    return view(F, q).ptr(x, y, 0)->re;
  }
  __device__ __forceinline__ static int cell(const Tile& t, int x, int y) { return (y - t.y0) * RW + (x - t.x0); }
  // {Re Ex_0, Re Br_0} at (x, y)
  __device__ __forceinline__ static float2 eb0(const FieldSetF& F, const Tile& t, int x, int y) {
    if (SHARED) return t.sf[cell(t, x, y)];
    return make_float2(re0(F, 0, x, y), re0(F, 4, x, y));
  }
  // {Re Er_0, Re Bx_0} at (x, y)
  __device__ __forceinline__ static float2 rx0(const FieldSetF& F, const Tile& t, int x, int y) {
    if (SHARED) return t.sf[RCELLS + cell(t, x, y)];
    return make_float2(re0(F, 1, x, y), re0(F, 3, x, y));
  }
  __device__ __forceinline__ static float et0(const FieldSetF& F, const Tile& t, int x, int y) {
    if (SHARED) return reinterpret_cast<const float*>(t.sf + 2 * RCELLS)[cell(t, x, y)];
    return re0(F, 2, x, y);
  }
  __device__ __forceinline__ static float bt0(const FieldSetF& F, const Tile& t, int x, int y) {
    if (SHARED) return reinterpret_cast<const float*>(t.sf + 2 * RCELLS)[RCELLS + cell(t, x, y)];
    return re0(F, 5, x, y);
  }
  // complex F_m of field q (m >= 1)
  __device__ __forceinline__ static float2 get(const FieldSetF& F, const Tile& t, int q, int m, int x, int y) {
    if (SHARED) return t.tm[(q * (M - 1) + m - 1) * TPLANE + (y - t.y0) * TW + (x - t.xs)];
    return *reinterpret_cast<const float2*>(view(F, q).ptr(x, y, m));
  }
};

__device__ __forceinline__ void record(const MixedParams& P, int reason, int64_t i, float a, float b, float c,
                                       float d, float e, float f, float g, float h) {
  if (!P.dbg) return;
  int* flag = reinterpret_cast<int*>(P.dbg);
  if (atomicCAS(flag, 0, reason) != 0) return;
  P.dbg[1] = (float)i;
  P.dbg[2] = a; P.dbg[3] = b; P.dbg[4] = c; P.dbg[5] = d;
  P.dbg[6] = e; P.dbg[7] = f; P.dbg[8] = g; P.dbg[9] = h;
}

__device__ __forceinline__ void gadd_f(cplx* p, float re, float im) {
  atomicAdd(&p->re, f2d_bits(re));
  if (im != 0.f) atomicAdd(&p->im, f2d_bits(im));
}

// 1 / gamma for a normalised momentum u (one expression for every use, so
// that consecutive steps agree on a particle's drift to the last bit).
__device__ __forceinline__ float inv_gamma(float ux, float uy, float uz) {
  return 1.0f / sqrtf(fmaf(ux, ux, fmaf(uy, uy, fmaf(uz, uz, 1.0f))));
}

// Per-mode deposit weights of particles.F90:589-665 for one particle: mode
// factors F2, F3, F4 (with the 2 e^{i m theta0} prefactor for m > 0).
template <int M>
struct ModeWalk {
  f2 eimt = {1.f, 0.f}, eimd = {1.f, 0.f};
  __device__ __forceinline__ void next(int m, f2 e05, f2 edt, float dth, f2& F2, f2& F3, f2& F4) {
    F2 = fm(1.f, 0.f);
    F3 = fm(0.5f, 0.f);
    F4 = fm(1.0f / 3.0f, 0.f);
    if (m > 0) {
      eimt = eimt * e05;
      eimd = eimd * edt;
      mode_factors((float)m * dth, eimd, F2, F3, F4);
      const f2 pre = 2.0f * eimt;
      F2 = pre * F2;
      F3 = pre * F3;
      F4 = pre * F4;
    }
  }
};

// Add one FP32 value v (in accumulator units, |v| <= 2^30) to the hi/lo pair
// of int32 accumulators at p (hi word p[0], lo word p[RCELLS]):
// v = hi 2^15 + lo with |hi| <= 2^15, |lo| <= 2^14 + 1/2, each rounded to an
// integer with the 1.5 * 2^23 offset trick (the split itself is exact).  The
// sums are exact integer sums -- independent of the order of the adds -- and,
// with at most 2^16 adds per accumulator, cannot overflow.  The error of one
// add is that of rounding v to FP32 plus at most 1/2 unit.  Integer
// shared-memory adds are single native instructions (FP32 shared-memory
// adds are not).
__device__ __forceinline__ void red_hi(int* p, int v) {
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.s32 q, %1, 0;\n\t@q red.shared.add.s32 [%0], %1;\n\t}" ::"r"(
                   (unsigned)__cvta_generic_to_shared(p)), "r"(v));
}
__device__ __forceinline__ void red_lo(int* p, int v) {
  asm volatile("red.shared.add.s32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "r"(v));
}
constexpr float FXP_MAGIC = 12582912.0f;  // 1.5 * 2^23
constexpr int FXP_MAGIC_BITS = 0x4B400000;
__device__ __forceinline__ void sadd(int* p, float v) {
  const float t = fmaf(v, 1.0f / 32768.0f, FXP_MAGIC);
  const int hi = __float_as_int(t) - FXP_MAGIC_BITS;
  const float lo = fmaf(-(t - FXP_MAGIC), 32768.0f, v);
  const int lo_i = __float_as_int(lo + FXP_MAGIC) - FXP_MAGIC_BITS;
  red_hi(p, hi);
  red_lo(p + RCELLS, lo_i);
}

// sadd for the real and imaginary parts of one complex value at once (the
// same split, computed with paired FP32 instructions).
__device__ __forceinline__ void sadd2(int* pr, int* pi, float2 v) {
  const float2 t = __ffma2_rn(v, make_float2(1.0f / 32768.0f, 1.0f / 32768.0f), make_float2(FXP_MAGIC, FXP_MAGIC));
  const int hr = __float_as_int(t.x) - FXP_MAGIC_BITS, hi = __float_as_int(t.y) - FXP_MAGIC_BITS;
  const float2 d = __fadd2_rn(t, make_float2(-FXP_MAGIC, -FXP_MAGIC));
  const float2 lo = __fadd2_rn(__ffma2_rn(d, make_float2(-32768.0f, -32768.0f), v), make_float2(FXP_MAGIC, FXP_MAGIC));
  const int lr = __float_as_int(lo.x) - FXP_MAGIC_BITS, li = __float_as_int(lo.y) - FXP_MAGIC_BITS;
  red_hi(pr, hr);
  red_lo(pr + RCELLS, lr);
  red_hi(pi, hi);
  red_lo(pi + RCELLS, li);
}

// Deposit into the tile accumulators over a WX x WY window whose first cell
// is (cx2 + x0, cy2 + y0); x0, y0 in {-2, -1} select the offsets -2..2 of the
// weight arrays (a 3-cell extent always starts at -1).  The accumulators are
// fixed-point integers (scale tile.s_xr for jx and jr, tile.s_t for jtheta):
// integer shared-memory adds are single instructions and their sums do not
// depend on the order of the adds.
template <int M, int WX, int WY>
__device__ __forceinline__ void deposit_tile(const Tile& tile, const float* og, const float* oh, const float* dgx,
                                             const float* dgy, int x0, int y0, int cx2, int cy2, float fc,
                                             float fcz, f2 e05, f2 edt, float dth) {
  float gxw[WX], hxw[WX], gyw[WY], hyw[WY];
#pragma unroll
  for (int c = 0; c < WX; ++c) {
    gxw[c] = (x0 == -2) ? og[c] : og[c + 1];
    hxw[c] = (x0 == -2) ? dgx[c] : dgx[c + 1];
  }
#pragma unroll
  for (int c = 0; c < WY; ++c) {
    gyw[c] = (y0 == -2) ? oh[c] : oh[c + 1];
    hyw[c] = (y0 == -2) ? dgy[c] : dgy[c + 1];
  }
  const float fcs = fc * tile.s_xr, fczs = fcz * tile.s_t;
  const float third = 1.0f / 3.0f;
  int* const sj = tile.sj;
  const int b0 = (cy2 + y0 - tile.y0) * RW + (cx2 + x0 - tile.x0);
  ModeWalk<M> mw;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    f2 F2, F3, F4;
    mw.next(m, e05, edt, dth, F2, F3, F4);
    // [comp][m][re, im][hi, lo][RCELLS]
    int* const ax = sj + ((0 * M + m) * 4) * RCELLS;
    int* const ar = sj + ((1 * M + m) * 4) * RCELLS;
    int* const at = sj + ((2 * M + m) * 4) * RCELLS;
    const float2 F2p = P2(F2), F3p = P2(F3), F4p = P2(F4);
    float2 qr[WX];
#pragma unroll
    for (int c = 0; c < WX; ++c) qr[c] = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < WY; ++r) {
      const float gyv = gyw[r], hyv = hyw[r];
      const float nfy = -(fcs * hyv);
      float2 w_rt, ym1;
      if (m == 0) {
        w_rt = make_float2(gyv + 0.5f * hyv, 0.f);
        ym1 = make_float2(0.5f * gyv + third * hyv, 0.f);
      } else {
        w_rt = pfma(gyv, F2p, pmul(hyv, F3p));
        ym1 = pfma(gyv, F3p, pmul(hyv, F4p));
      }
      float2 qx = make_float2(0.f, 0.f);
#pragma unroll
      for (int c = 0; c < WX; ++c) {
        const float gxv = gxw[c], hxv = hxw[c];
        const int cell = b0 + r * RW + c;
        // The window's last column (jx) and last row (jr) carry the running
        // flux sum after every weight change of the row (column), which is
        // zero up to FP32 round-off (old and new weights both sum to 2):
        // those adds are left out.
        if (m == 0) {
          const float w_xt = gxv + 0.5f * hxv;
          const float w_xr = gxv * w_rt.x + hxv * ym1.x;
          qx.x = qx.x - (fcs * hxv) * w_rt.x;
          qr[c].x = qr[c].x + nfy * w_xt;
          if (c < WX - 1) sadd(ax + cell + 1, qx.x);       // jx at (cx + 1, cy)
          if (r < WY - 1) sadd(ar + cell + RW, qr[c].x);  // jr at (cx, cy + 1)
          sadd(at + cell, fczs * w_xr);                    // jtheta at (cx, cy)
        } else {
          const float2 w_xt = pfma(gxv, F2p, pmul(hxv, F3p));
          const float2 w_xr = pfma(gxv, w_rt, pmul(hxv, ym1));
          qx = pfma(-(fcs * hxv), w_rt, qx);
          qr[c] = pfma(nfy, w_xt, qr[c]);
          if (c < WX - 1) sadd2(ax + cell + 1, ax + 2 * RCELLS + cell + 1, qx);
          if (r < WY - 1) sadd2(ar + cell + RW, ar + 2 * RCELLS + cell + RW, qr[c]);
          sadd2(at + cell, at + 2 * RCELLS + cell, pmul(fczs, w_xr));
        }
      }
    }
  }
}

// The window shape of a warp: 3 cells along a direction when no lane of the
// warp changes cell along it, else 4 (holding the reference's xmin..xmax or
// ymin..ymax range; the extra row or column carries zero flux).
template <int M>
__device__ __forceinline__ void deposit_tile_warp(const Tile& tile, const float* og, const float* oh,
                                                  const float* dgx, const float* dgy, int dcx, int dcy, int cx2,
                                                  int cy2, float fc, float fcz, f2 e05, f2 edt, float dth) {
  const unsigned am = __activemask();
  const bool wx = __any_sync(am, dcx != 0), wy = __any_sync(am, dcy != 0);
  const int x0 = dcx < 0 ? -2 : -1, y0 = dcy < 0 ? -2 : -1;
  if (!wx && !wy)
    deposit_tile<M, 3, 3>(tile, og, oh, dgx, dgy, -1, -1, cx2, cy2, fc, fcz, e05, edt, dth);
  else
    deposit_tile<M, 4, 4>(tile, og, oh, dgx, dgy, x0, y0, cx2, cy2, fc, fcz, e05, edt, dth);
}

// Deposit of a particle on the global path: FP64 atomics into the global
// currents with the geometric factor of each row, over the reference's
// xmin..xmax, ymin..ymax range.
template <int M>
__device__ __forceinline__ void deposit_global(const FieldSetF& F, const MixedParams& P, const float* og,
                                               const float* oh, const float* dgx, const float* dgy, int dcx,
                                               int dcy, int cx2, int cy2, float fc, float fcz, f2 e05, f2 edt,
                                               float dth) {
  const int xmin = -1 + (dcx - 1) / 2, xmax = 1 + (dcx + 1) / 2;
  const int ymin = -1 + (dcy - 1) / 2, ymax = 1 + (dcy + 1) / 2;
  const float third = 1.0f / 3.0f;
  ModeWalk<M> mw;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    f2 F2, F3, F4;
    mw.next(m, e05, edt, dth, F2, F3, F4);
    f2 qr[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) qr[q] = fm(0.f, 0.f);
    for (int iy = ymin; iy <= ymax; ++iy) {
      const float gyv = oh[iy + 2], hyv = dgy[iy + 2];
      f2 w_rt, ym1;
      if (m == 0) {
        w_rt = fm(gyv + 0.5f * hyv, 0.f);
        ym1 = fm(0.5f * gyv + third * hyv, 0.f);
      } else {
        w_rt = gyv * F2 + hyv * F3;
        ym1 = gyv * F3 + hyv * F4;
      }
      const int cy = cy2 + iy;
      const float gx_ = P.g_rt[cy - (1 - JNG)];
      const float gr_ = P.g_xt[cy - (0 - JNG)];
      const float gt_ = P.g_vol[cy - (1 - JNG)];
      f2 qx = fm(0.f, 0.f);
#pragma unroll
      for (int ix = -2; ix <= 2; ++ix) {
        if (ix < xmin || ix > xmax) continue;
        const float gxv = og[ix + 2], hxv = dgx[ix + 2];
        const f2 w_xt = (m == 0) ? fm(gxv + 0.5f * hxv, 0.f) : (gxv * F2 + hxv * F3);
        const f2 w_xr = gxv * w_rt + hxv * ym1;
        qx = qx - (fc * hxv) * w_rt;
        qr[ix + 2] = qr[ix + 2] - (fc * hyv) * w_xt;
        const f2 qt = fcz * w_xr;
        const int cx = cx2 + ix;
        gadd_f(F.jx.ptr(cx + 1, cy, m), qx.re * gx_, qx.im * gx_);
        gadd_f(F.jr.ptr(cx, cy + 1, m), qr[ix + 2].re * gr_, qr[ix + 2].im * gr_);
        gadd_f(F.jt.ptr(cx, cy, m), qt.re * gt_, qt.im * gt_);
      }
    }
  }
}

// Push one particle.  Returns false (and leaves the particle untouched) when
// SHARED and its stencil is not inside the staged tile.
template <int M, bool SHARED>
__device__ __forceinline__ bool push_one(int64_t i, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                                         const FieldSetF& F, const MixedParams& P, const RunConst& rc,
                                         const Tile& tile, int nsh, int apply_bcs) {
  const int kx = sp.kx[i];
  if (kx == INT32_MIN) return true;
  const int k = kx - nsh;  // local 0-based floor cell index
  float fx = sp.fx[i];
  float y = sp.fy[i], z = sp.fz[i];
  float ux = sp.ux[i], uy = sp.uy[i], uz = sp.uz[i];
  const float w = sp.fw[i];

  float igm = inv_gamma(ux, uy, uz);
  fx += ux * (P.cdt2_dx * igm);
  y += uy * (P.cdt2_dy * igm);
  z += uz * (P.cdt2_dy * igm);
  const float r = sqrtf(y * y + z * z);
  const float ir = (r > 0.f) ? 1.0f / r : 0.f;
  const float ct = (r > 0.f) ? y * ir : 1.f, st = (r > 0.f) ? z * ir : 0.f;  // e^{i theta}
  const float cyr = r - 0.5f;

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
  if (SHARED) {
    if (!((cx2 - 2 >= tile.x0) && (cx2 + 3 < tile.x0 + RW) && (cy2 - 2 >= tile.y0) && (cy2 + 3 < tile.y0 + RH)))
      return false;
  } else {
    if (cx2 - 2 < 1 - NG || cx2 + 3 > rc.nx + NG || cy2 - 2 < 1 - NG || cy2 + 3 > rc.ny + NG ||
        cx1 - 1 < 1 - NG || cx1 + 1 > rc.nx + NG || cy1 - 1 < 1 - NG || cy1 + 1 > rc.ny + NG) {
      atomicOr(P.err, ERR_CELL_RANGE);
      record(P, 1, i, (float)k, fx, y, z, (float)cx2, (float)cy2, (float)cx1, (float)cy1);
      return true;
    }
  }
  // cell-centred (g) and staggered (h) weights, x2 the reference's convention
  float gx[3], gy[3], hx[3], hy[3];
  {
    float c2 = frx1 * frx1;
    gx[0] = 0.25f + c2 + frx1; gx[1] = 1.5f - 2.0f * c2; gx[2] = 0.25f + c2 - frx1;
    c2 = fry1 * fry1;
    gy[0] = 0.25f + c2 + fry1; gy[1] = 1.5f - 2.0f * c2; gy[2] = 0.25f + c2 - fry1;
    c2 = frx2 * frx2;
    hx[0] = 0.25f + c2 + frx2; hx[1] = 1.5f - 2.0f * c2; hx[2] = 0.25f + c2 - frx2;
    c2 = fry2 * fry2;
    hy[0] = 0.25f + c2 + fry2; hy[1] = 1.5f - 2.0f * c2; hy[2] = 0.25f + c2 - fry2;
  }

  // gather (e_part.inc / b_part.inc): field = Re sum_m e^{-i m theta} F_m
  float exr, er_, etr, bxr, brr, btr;
  {
    using G = Gather<M, SHARED>;
    // mode 0: (Ex, Br), (Er, Bx) and (Et, Bt) as pairs
    float2 aEB = make_float2(0.f, 0.f), aRX = aEB, aTB = aEB;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
      float2 rEB = make_float2(0.f, 0.f), rRX = rEB, rTB = rEB;
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) {
        // Ex, Br at (cx1, cy2); Er, Bx at (cx2, cy1); Et at (cx2, cy2); Bt at (cx1, cy1)
        rEB = pfma(gx[ii], G::eb0(F, tile, cx1 - 1 + ii, cy2 - 1 + jj), rEB);
        rRX = pfma(hx[ii], G::rx0(F, tile, cx2 - 1 + ii, cy1 - 1 + jj), rRX);
        rTB = pfma(make_float2(hx[ii], gx[ii]),
                   make_float2(G::et0(F, tile, cx2 - 1 + ii, cy2 - 1 + jj), G::bt0(F, tile, cx1 - 1 + ii, cy1 - 1 + jj)),
                   rTB);
      }
      aEB = pfma(hy[jj], rEB, aEB);
      aRX = pfma(gy[jj], rRX, aRX);
      aTB = pfma(make_float2(hy[jj], gy[jj]), rTB, aTB);
    }
    exr = aEB.x; brr = aEB.y; er_ = aRX.x; bxr = aRX.y; etr = aTB.x; btr = aTB.y;
    // modes m >= 1: complex sums, then Re(e^{-i m theta} F_m)
    f2 emi = fm(1.f, 0.f);
    const f2 e1 = fm(ct, -st);
#pragma unroll
    for (int m = 1; m < M; ++m) {
      emi = emi * e1;
      float2 aex = make_float2(0.f, 0.f), aer = aex, aet = aex, abx = aex, abr = aex, abt = aex;
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        float2 rex = make_float2(0.f, 0.f), rer = rex, ret = rex, rbr = rex, rbt = rex, rbx = rex;
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) {
          rex = pfma(gx[ii], G::get(F, tile, 0, m, cx1 - 1 + ii, cy2 - 1 + jj), rex);
          rbr = pfma(gx[ii], G::get(F, tile, 4, m, cx1 - 1 + ii, cy2 - 1 + jj), rbr);
          rer = pfma(hx[ii], G::get(F, tile, 1, m, cx2 - 1 + ii, cy1 - 1 + jj), rer);
          rbx = pfma(hx[ii], G::get(F, tile, 3, m, cx2 - 1 + ii, cy1 - 1 + jj), rbx);
          ret = pfma(hx[ii], G::get(F, tile, 2, m, cx2 - 1 + ii, cy2 - 1 + jj), ret);
          rbt = pfma(gx[ii], G::get(F, tile, 5, m, cx1 - 1 + ii, cy1 - 1 + jj), rbt);
        }
        aex = pfma(hy[jj], rex, aex);
        abr = pfma(hy[jj], rbr, abr);
        aer = pfma(gy[jj], rer, aer);
        abx = pfma(gy[jj], rbx, abx);
        aet = pfma(hy[jj], ret, aet);
        abt = pfma(gy[jj], rbt, abt);
      }
      // Re(emi * a) = emi.re a.re - emi.im a.im
      exr += emi.re * aex.x - emi.im * aex.y;
      er_ += emi.re * aer.x - emi.im * aer.y;
      etr += emi.re * aet.x - emi.im * aet.y;
      bxr += emi.re * abx.x - emi.im * abx.y;
      brr += emi.re * abr.x - emi.im * abr.y;
      btr += emi.re * abt.x - emi.im * abt.y;
    }
  }
  if (!isfinite(exr + er_ + etr + bxr + brr + btr)) {
    atomicOr(P.err, ERR_NONFINITE);
    record(P, 20 + (SHARED ? 10 : 0), i, exr, er_, etr, bxr, brr, btr, (float)cx2, (float)cy2);
    return true;
  }
  const float eyr = er_ * ct - etr * st;
  const float ezr = er_ * st + etr * ct;
  const float byr = brr * ct - btr * st;
  const float bzr = brr * st + btr * ct;

  // Boris rotation (particles.F90:404-451)
  const float cm = P.cmratio;
  const float uxm = ux + cm * exr, uym = uy + cm * eyr, uzm = uz + cm * ezr;
  const float root = P.ccmratio * inv_gamma(uxm, uym, uzm);
  const float tx = bxr * root, ty = byr * root, tz = bzr * root;
  const float tx2 = tx * tx, ty2 = ty * ty, tz2 = tz * tz;
  const float tau = 1.0f / (1.0f + tx2 + ty2 + tz2);
  const float uxp = ((1.0f + tx2 - ty2 - tz2) * uxm + 2.0f * ((tx * ty + tz) * uym + (tx * tz - ty) * uzm)) * tau;
  const float uyp = ((1.0f - tx2 + ty2 - tz2) * uym + 2.0f * ((ty * tz + tx) * uzm + (ty * tx - tz) * uxm)) * tau;
  const float uzp = ((1.0f - tx2 - ty2 + tz2) * uzm + 2.0f * ((tz * tx + ty) * uxm + (tz * ty - tx) * uym)) * tau;
  ux = uxp + cm * exr;
  uy = uyp + cm * eyr;
  uz = uzp + cm * ezr;
  if (!isfinite(ux + uy + uz)) {
    atomicOr(P.err, ERR_NONFINITE);
    record(P, 40 + (SHARED ? 10 : 0), i, exr, er_, etr, bxr, brr, btr, (float)cx1, (float)cy2);
    return true;
  }
  // the same expression as the next step's half drift, so that its t + dt/2
  // position is this deposit's t + 3dt/2 one
  igm = inv_gamma(ux, uy, uz);
  const float dxs = ux * (P.cdt2_dx * igm), dys = uy * (P.cdt2_dy * igm), dzs = uz * (P.cdt2_dy * igm);
  const float fxn = fx + dxs;
  const float yn = y + dys, zn = z + dzs;
  const float rn = sqrtf(yn * yn + zn * zn);
  float vt = 0.f;  // v_theta at t + dt (m/s)
  if (rn > 0.f) vt = (P.c * igm) * ((uz * yn - uy * zn) / rn);

  // position at t + dt, then particle_bcs in the cell units of this grid.
  // The particle is stored before its deposit (whose inputs are all formed
  // above), so that its new state is not held in registers across the
  // deposit; a particle that leaves still deposits the current of its move.
  const int kk = (int)floorf(fxn);
  int knew = k + kk;
  float fnew = fxn - (float)kk;
  if (fnew >= 1.0f) { fnew -= 1.0f; knew += 1; }
  if (fnew < 0.0f) fnew = 0.0f;
  // the stored radial position (a reflection at r_max moves it); the
  // deposit below uses the unreflected move
  float ys = yn, zs = zn;
  bool dead = false;
  if (apply_bcs) {
    const float xc = (float)knew + fnew;
    if (xc < P.x_lo) {
      const int b = sp.bc[CYL_BD_X_MIN];
      if (b == CYL_BC_REFLECT) {
        const float v = 2.0f * P.x_sys_lo - xc;
        knew = (int)floorf(v); fnew = v - (float)knew; ux = -ux;
      } else if (b == CYL_BC_PERIODIC) {
        knew += rc.nx;
      }
      if (xc < P.x_out_lo && b != CYL_BC_PERIODIC) dead = true;
    }
    if (xc >= P.x_hi) {
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
        ys *= f;
        zs *= f;
        const float rr = sqrtf(ys * ys + zs * zs);
        const float cc = ys / rr, ss = zs / rr;
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
  } else {
    sp.kx[i] = knew + nsh;
    sp.fx[i] = fnew;
    sp.fy[i] = ys;
    sp.fz[i] = zs;
    sp.ux[i] = ux;
    sp.uy[i] = uy;
    sp.uz[i] = uz;
  }
  // A particle that neither moves nor turns over the deposit's interval
  // adds exactly zero to every current value (its weight changes and v_theta
  // are zero): a warp all of whose particles are such skips the deposit and its
  // preparation.
  // That is most of the plasma ahead of a laser, cold and in zero field.
  const bool moving = (dxs != 0.f) || (dys != 0.f) || (dzs != 0.f) || (vt != 0.f);
  if (SHARED) {
    if (!__any_sync(__activemask(), moving)) return true;
  } else if (!moving) {
    return true;
  }
  // deposit: shape change from t+dt/2 to t+3dt/2 (particles.F90:515-665)
  const float fx3 = fxn + dxs, y3 = yn + dys, z3 = zn + dzs;
  const float r3 = sqrtf(y3 * y3 + z3 * z3);
  const float ir3 = (r3 > 0.f) ? 1.0f / r3 : 0.f;
  const float c3 = (r3 > 0.f) ? y3 * ir3 : 1.f, s3 = (r3 > 0.f) ? z3 * ir3 : 0.f;
  // Displacements over the deposit's interval.  fx3 - fx and y3 - y, z3 - z
  // are differences of nearby FP32 values, exact; the radial one is formed
  // as (r3^2 - r^2) / (r3 + r), without the cancellation of r3 - r, whose
  // terms each carry the absolute rounding of a radius (2^-24 r, up to 3e-5
  // of a cell at r = 256 cells: the size of a slow particle's whole step).
  const float ddx = fx3 - fx;
  const float rs = r3 + r;
  const float ddr = rs > 0.f ? ((y3 - y) * (y3 + y) + (z3 - z) * (z3 + z)) / rs : 0.f;
  const float cyr3 = cyr + ddr;
  const int a3 = (int)floorf(fx3);
  const float frx3 = ((float)a3 - fx3) + 0.5f;
  const int b3 = (int)floorf(cyr3);
  const float fry3 = ((float)b3 - cyr3) + 0.5f;
  const int dcx = a3 - a2, dcy = b3 - b2;
  if (dcx < -1 || dcx > 1 || dcy < -1 || dcy > 1) {
    atomicOr(P.err, ERR_CELL_RANGE);
    record(P, 2 + (SHARED ? 10 : 0), i, (float)k, fx, fx3, cyr, cyr3, (float)dcx, (float)dcy, ux);
    return true;
  }
  // old (t+dt/2) staggered weights on offsets -2..2 and their change
  float og[5], oh[5], dgx[5], dgy[5];
  {
    const float c2x = frx3 * frx3, c2y = fry3 * fry3;
    const float nx0 = 0.25f + c2x + frx3, nx1 = 1.5f - 2.0f * c2x, nx2 = 0.25f + c2x - frx3;
    const float ny0 = 0.25f + c2y + fry3, ny1 = 1.5f - 2.0f * c2y, ny2 = 0.25f + c2y - fry3;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      og[q] = (q >= 1 && q <= 3) ? hx[q - 1] : 0.f;
      oh[q] = (q >= 1 && q <= 3) ? hy[q - 1] : 0.f;
      const int ox = q - 2 - dcx, oy = q - 2 - dcy;
      const float hnx = (ox == -1) ? nx0 : (ox == 0) ? nx1 : (ox == 1) ? nx2 : 0.f;
      const float hny = (oy == -1) ? ny0 : (oy == 0) ? ny1 : (oy == 1) ? ny2 : 0.f;
      dgx[q] = hnx - og[q];
      dgy[q] = hny - oh[q];
    }
    // Without a cell change the weight changes are formed from the
    // displacement d itself: with f' = f - d,
    //   h(-1): (f'+f+1)(f'-f) = -(p + d),  h(0): -2 (f'^2 - f^2) = 2 p,
    //   h(+1): (f'+f-1)(f'-f) = d - p,     p = d (2 f - d),
    // so each change keeps the relative precision of d (a difference of
    // new and old weights, each near 1, keeps only their absolute 2^-24).
    if (dcx == 0) {
      const float p = ddx * (2.0f * frx2 - ddx);
      dgx[1] = -(p + ddx);
      dgx[2] = 2.0f * p;
      dgx[3] = ddx - p;
    }
    if (dcy == 0) {
      const float p = ddr * (2.0f * fry2 - ddr);
      dgy[1] = -(p + ddr);
      dgy[2] = 2.0f * p;
      dgy[3] = ddr - p;
    }
  }
  const float qwf = P.q_fac * w;  // q w fac
  const float fc = qwf * P.idt;   // fcx = fcy
  const float fcz = qwf * vt;
  const f2 e05 = fm(ct, st);
  const f2 edt = fm(c3, s3) * fm(ct, -st);
  const float dth = atan2f(z3, y3) - atan2f(z, y);
  if (SHARED) {
    *tile.dirty = 1;
    deposit_tile_warp<M>(tile, og, oh, dgx, dgy, dcx, dcy, cx2, cy2, fc, fcz, e05, edt, dth);
  }
  else
    deposit_global<M>(F, P, og, oh, dgx, dgy, dcx, dcy, cx2, cy2, fc, fcz, e05, edt, dth);
  return true;
}

__device__ __forceinline__ void set_bounds(MixedParams& P, const StepRec* rec, const RunConst& rc) {
  P.x_lo = -0.5f;
  P.x_hi = (float)rc.nx - 0.5f;
  P.x_sys_lo = (float)((rec->x_min - rec->x_grid_min) / rc.dx);
  P.x_sys_hi = (float)((rec->x_max - rec->x_grid_min) / rc.dx);
  P.x_out_lo = P.x_sys_lo - 2.0f;
  P.x_out_hi = P.x_sys_hi + 2.0f;
}

// Tensor maps of the six FP32 E/B arrays (8-byte complex elements, dims
// nxg x nyg x M, box TW x RH x 1), one set per launch.
struct TmaSet {
  CUtensorMap map[6];
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for phase `parity` of the barrier, at most `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int limit) {
  for (int k = 0; k < limit; ++k) {
    if (mbar_try_wait(bar, parity)) return true;
    __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// Polls of the TMA barrier before a tile gives up (with 64 ns sleeps: about
// a second).
constexpr int TMA_WAIT_POLLS = 1 << 24;

// Shared memory of one push CTA: 128-byte aligned TMA planes, mode-0
// planes, accumulators.
template <int M>
struct TileSmem {
  float2* tm;  // 6 (M-1) TPLANE float2
  float2* sf;  // PLANES_M0 RCELLS float2
  int* sj;     // 3 M 4 RCELLS int32
  __device__ __forceinline__ explicit TileSmem(float4* smem4) {
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(smem4) + 127) & ~(uintptr_t)127);
    tm = reinterpret_cast<float2*>(base);
    sf = tm + 6 * (M - 1) * TPLANE;
    sj = reinterpret_cast<int*>(sf + PLANES_M0 * RCELLS);
  }
};

// One tile of one run: stage its fields, push and deposit its particles, and
// flush its current accumulators.  Every thread of the CTA calls it with the
// same tile, so all meet the same barriers.  Returns false when the TMA
// staging timed out (the CTA must leave).
template <int M>
__device__ __forceinline__ bool process_tile(const FieldSetF& F, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                                             const RunConst& rc, const MixedParams& P, const TileTable* tt, int t,
                                             int nsh, int apply_bcs, const TmaSet* tma, int use_tma,
                                             const TileSmem<M>& sm, uint64_t* tma_bar, int* tma_failed,
                                             unsigned* s_bound, int* s_dirty, unsigned& tma_phase) {
  float2* const tm = sm.tm;
  float2* const sf = sm.sf;
  int* const sj = sm.sj;
  const int ntx = tt->ntx;
    const int64_t p0 = tt->start[t], p1 = tt->start[t + 1];
    Tile tile;
    tile.sf = sf;
    tile.tm = tm;
    tile.sj = sj;
    tile.dirty = s_dirty;
    tile.x0 = (tt->tx_min + t % ntx) * TILE_X - nsh + 1 - DRIFT - 2;
    tile.y0 = (t / ntx) * TILE_Y + 1 - DRIFT - 2;
    tile.xs = tile.x0 - (((tile.x0 % 2) + 2) % 2);  // rounded down to even
    const bool inside = tile.x0 >= 1 - NG && tile.x0 + RW - 1 <= rc.nx + NG && tile.y0 >= 1 - NG &&
                        tile.y0 + RH - 1 <= rc.ny + NG;
    if (p1 <= p0) return true;
    if (!inside) {
      // tile partly outside the ghosted grid: every particle takes the global path
      for (int64_t i = p0 + threadIdx.x; i < p1; i += PUSH_THREADS) P.fb_list[atomicAdd(P.fb_count, 1)] = (int)i;
      return true;
    }
    // stage E and B (FP32): modes m >= 1 by TMA boxes (issued first, they
    // arrive while mode 0 is staged by plain loads as real pairs, see Gather)
    if (M > 1 && use_tma && threadIdx.x == 0) {
      mbar_expect_tx(tma_bar, (unsigned)(6 * (M - 1) * TW * RH * 8));
      for (int q = 0; q < 6; ++q)
        for (int m = 1; m < M; ++m)
          tma_load_3d(tm + (q * (M - 1) + m - 1) * TPLANE, &tma->map[q], tile.xs + NG - 1, tile.y0 + NG - 1, m,
                      tma_bar);
    }
    // inputs of the tile's fixed-point bound (tile_scales): the largest
    // weight and momentum of its particles, the largest staged E values
    float b_w = 0.f, b_u2 = 0.f, b_ex = 0.f, b_er = 0.f, b_et = 0.f, b_em = 0.f;
    for (int64_t i = p0 + threadIdx.x; i < p1; i += PUSH_THREADS) {
      const float ux = sp.ux[i], uy = sp.uy[i], uz = sp.uz[i];
      b_w = fmaxf(b_w, fabsf(sp.fw[i]));
      b_u2 = fmaxf(b_u2, fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
    }
    {
      using G = Gather<M, false>;
      float* s_t = reinterpret_cast<float*>(sf + 2 * RCELLS);
      for (int c = threadIdx.x; c < RCELLS; c += PUSH_THREADS) {
        const int x = tile.x0 + c % RW, y = tile.y0 + c / RW;
        const float ex = G::re0(F, 0, x, y), er = G::re0(F, 1, x, y), et = G::re0(F, 2, x, y);
        sf[c] = make_float2(ex, G::re0(F, 4, x, y));
        sf[RCELLS + c] = make_float2(er, G::re0(F, 3, x, y));
        s_t[c] = et;
        s_t[RCELLS + c] = G::re0(F, 5, x, y);
        b_ex = fmaxf(b_ex, fabsf(ex));
        b_er = fmaxf(b_er, fabsf(er));
        b_et = fmaxf(b_et, fabsf(et));
      }
      if (M > 1 && !use_tma) {
        // the same boxes by plain loads (row pitches that TMA cannot take)
#pragma unroll 1
        for (int q = 0; q < 6; ++q) {
          const FViewF v = G::view(F, q);
#pragma unroll 1
          for (int m = 1; m < M; ++m)
            for (int c = threadIdx.x; c < TW * RH; c += PUSH_THREADS) {
              const int x = tile.xs + c % TW, y = tile.y0 + c / TW;
              tm[(q * (M - 1) + m - 1) * TPLANE + c] =
                  x <= rc.nx + NG ? *reinterpret_cast<const float2*>(v.ptr(x, y, m)) : make_float2(0.f, 0.f);
            }
        }
      }
    }
    if (M > 1 && use_tma) {
      // every thread waits for the boxes (the barrier's completion makes the
      // copies visible to the waiting thread); a wait that runs out flags the
      // run, waits once more for copies in flight, and the CTA leaves at the
      // next barrier
      if (!mbar_wait_bounded(tma_bar, tma_phase, TMA_WAIT_POLLS)) {
        atomicOr(P.err, ERR_TMA_TIMEOUT);
        mbar_wait_bounded(tma_bar, tma_phase, TMA_WAIT_POLLS);
        *tma_failed = 1;
      }
      tma_phase ^= 1u;
    }
    if (M > 1) {
      // E_m of modes m >= 1 (TMA planes of Ex, Er, Et: q = 0, 1, 2)
      for (int e = threadIdx.x; e < 3 * (M - 1) * TW * RH; e += PUSH_THREADS) {
        const float2 v = tm[(e / (TW * RH)) * TPLANE + e % (TW * RH)];
        b_em = fmaxf(b_em, fabsf(v.x) + fabsf(v.y));
      }
    }
    block_max_into(s_bound + 0, b_w);
    block_max_into(s_bound + 1, b_u2);
    block_max_into(s_bound + 2, b_ex);
    block_max_into(s_bound + 3, b_er);
    block_max_into(s_bound + 4, b_et);
    block_max_into(s_bound + 5, b_em);
    __syncthreads();
    if (*tma_failed) return false;  // uniform: read by every thread after the barrier
    {
      TileBound b;
      b.w_max = __uint_as_float(s_bound[0]);
      b.u2_max = __uint_as_float(s_bound[1]);
      b.e_sum = 4.0f * (__uint_as_float(s_bound[2]) + __uint_as_float(s_bound[3]) + __uint_as_float(s_bound[4]) +
                        3.0f * (float)(M - 1) * __uint_as_float(s_bound[5]));
      tile_scales(tile, p1 - p0, b, P);
    }
    for (int64_t i = p0 + threadIdx.x; i < p1; i += PUSH_THREADS) {
      if (!push_one<M, true>(i, sp, cnt, F, P, rc, tile, nsh, apply_bcs))
        P.fb_list[atomicAdd(P.fb_count, 1)] = (int)i;
    }
    __syncthreads();
    // every thread read the bound before the barrier: clear it for the next tile
    if (threadIdx.x < 6) s_bound[threadIdx.x] = 0u;
    // accumulators that no warp wrote are still zero: no flush
    const bool dirty = *s_dirty != 0;
    // flush: one FP64 add per non-zero accumulator, with the geometric
    // factor of the row and the inverse fixed-point scale
    const float inv_xr = tile.s_xr > 0.f ? 1.0f / tile.s_xr : 0.f;
    const float inv_t = tile.s_t > 0.f ? 1.0f / tile.s_t : 0.f;
    for (int e = threadIdx.x; dirty && e < 3 * M * RCELLS; e += PUSH_THREADS) {
      const int cell = e % RCELLS, cm = e / RCELLS;
      const int comp = cm / M, m = cm % M;
      int* a = sj + cm * 4 * RCELLS + cell;
      const int rh = a[0], rl = a[RCELLS], ih = a[2 * RCELLS], il = a[3 * RCELLS];
      if ((rh | rl | ih | il) == 0) continue;
      // left at zero for the next tile
      a[0] = 0;
      a[RCELLS] = 0;
      a[2 * RCELLS] = 0;
      a[3 * RCELLS] = 0;
      const float vr = fmaf((float)rh, 32768.0f, (float)rl), vi = fmaf((float)ih, 32768.0f, (float)il);
      const int cx = tile.x0 + cell % RW, cy = tile.y0 + cell / RW;
      float f;
      cplx* dst;
      if (comp == 0) { f = P.g_rt[cy - (1 - JNG)] * inv_xr; dst = F.jx.ptr(cx, cy, m); }
      else if (comp == 1) { f = P.g_xt[cy - 1 - (0 - JNG)] * inv_xr; dst = F.jr.ptr(cx, cy, m); }
      else { f = P.g_vol[cy - (1 - JNG)] * inv_t; dst = F.jt.ptr(cx, cy, m); }
      gadd_f(dst, vr * f, vi * f);
    }
    __syncthreads();
    if (threadIdx.x == 0) *s_dirty = 0;  // read by every thread before the barrier above
  return true;
}

// Accumulators at zero and the dirty flag clear, before a CTA's first tile
// (each tile's flush leaves them so for the next).
template <int M>
__device__ __forceinline__ void tile_acc_init(const TileSmem<M>& sm, int* s_dirty) {
  for (int e = threadIdx.x; e < 3 * M * 4 * RCELLS; e += PUSH_THREADS) sm.sj[e] = 0;
  if (threadIdx.x == 0) *s_dirty = 0;
}

template <int M>
__global__ void __launch_bounds__(PUSH_THREADS, push_min_blocks<M>()) k_push_tiles(
    FieldSetF F, SpeciesPtrs sp, SpeciesCounters* cnt, const StepRec* rec, RunConst rc, MixedParams P, TileTable* tt,
    int apply_bcs, const __grid_constant__ TmaSet tma, int use_tma) {
  extern __shared__ float4 smem4[];
  __shared__ uint64_t tma_bar;
  __shared__ int tma_failed;
  __shared__ unsigned s_bound[6];
  __shared__ int s_dirty;
  const TileSmem<M> sm(smem4);
  if (threadIdx.x == 0) {
    tma_failed = 0;
    if (use_tma) mbar_init(&tma_bar);
  }
  if (threadIdx.x < 6) s_bound[threadIdx.x] = 0u;
  tile_acc_init<M>(sm, &s_dirty);
  __syncthreads();
  unsigned tma_phase = 0;
  const int nsh = rec->nshift_total;
  set_bounds(P, rec, rc);
  const int ntiles = tt->ntiles;
  // static round-robin over the tiles in decreasing order of particle count
  // (longest first)
  for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    if (!process_tile<M>(F, sp, cnt, rc, P, tt, tt->order[ti], nsh, apply_bcs, &tma, use_tma, sm, &tma_bar,
                         &tma_failed, s_bound, &s_dirty, tma_phase))
      return;
  }
}

// The push of several runs (a batch) in one launch: the runs' tiles form one
// table of (run, tile) items in decreasing order of particle count, dealt to
// the CTAs round-robin.  Each item reads its run's parameters from the job
// table (one entry per run and step of the chunk).  Fields are staged by
// plain loads.
template <int M>
__global__ void __launch_bounds__(PUSH_THREADS, push_min_blocks<M>()) k_push_tiles_batch(const BatchJob* jobs,
                                                                                   const int2* work,
                                                                                   const int* nwork) {
  extern __shared__ float4 smem4[];
  __shared__ int tma_failed;
  __shared__ unsigned s_bound[6];
  __shared__ int s_dirty;
  const TileSmem<M> sm(smem4);
  if (threadIdx.x == 0) tma_failed = 0;
  if (threadIdx.x < 6) s_bound[threadIdx.x] = 0u;
  tile_acc_init<M>(sm, &s_dirty);
  __syncthreads();
  unsigned tma_phase = 0;
  const int n = *nwork;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int2 jt = work[w];
    const BatchJob& J = jobs[jt.x];
    MixedParams P = J.P;
    set_bounds(P, J.rec, J.rc);
    process_tile<M>(J.F, J.sp, J.cnt, J.rc, P, J.tt, jt.y, J.rec->nshift_total, J.apply_bcs, nullptr, 0, sm,
                    nullptr, &tma_failed, s_bound, &s_dirty, tma_phase);
  }
}

// The deferred particles of every run of a batch (blockIdx.y = run).
template <int M>
__global__ void __launch_bounds__(PUSH_THREADS) k_push_global_batch(const BatchJob* jobs) {
  const BatchJob& J = jobs[blockIdx.y];
  MixedParams P = J.P;
  set_bounds(P, J.rec, J.rc);
  const int nsh = J.rec->nshift_total;
  const int64_t nlist = *P.fb_count;
  const int64_t n_sorted = J.tt->n_sorted, n_used = J.cnt->n_used;
  const int64_t ntail = n_used > n_sorted ? n_used - n_sorted : 0;
  Tile none{nullptr, nullptr, nullptr, 0, 0, 0, 0.f, 0.f};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nlist + ntail;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (t < nlist) ? (int64_t)P.fb_list[t] : n_sorted + (t - nlist);
    push_one<M, false>(i, J.sp, J.cnt, J.F, P, J.rc, none, nsh, J.apply_bcs);
  }
}

// Deferred particles (listed by k_push_tiles) and the unsorted tail that the
// moving window appended since the last sort: global gather and FP64 atomics.
template <int M>
__global__ void __launch_bounds__(PUSH_THREADS) k_push_global(FieldSetF F, SpeciesPtrs sp, SpeciesCounters* cnt,
                                                              const StepRec* rec, RunConst rc, MixedParams P,
                                                              const TileTable* tt, int apply_bcs) {
  const int nsh = rec->nshift_total;
  set_bounds(P, rec, rc);
  const int64_t nlist = *P.fb_count;
  const int64_t n_sorted = tt->n_sorted, n_used = cnt->n_used;
  const int64_t ntail = n_used > n_sorted ? n_used - n_sorted : 0;
  Tile none{nullptr, nullptr, nullptr, 0, 0, 0, 0.f, 0.f};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nlist + ntail;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (t < nlist) ? (int64_t)P.fb_list[t] : n_sorted + (t - nlist);
    push_one<M, false>(i, sp, cnt, F, P, rc, none, nsh, apply_bcs);
  }
}

size_t push_mixed_smem(int M) {
  return 128 + (size_t)6 * (M - 1) * TPLANE * sizeof(float2) + (size_t)PLANES_M0 * RCELLS * sizeof(float2) +
         (size_t)12 * M * RCELLS * sizeof(int);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (null if
// the driver does not provide it: the push then stages by plain loads).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Tensor maps of the six FP32 E/B arrays for the TMA staging.  Returns false
// (plain-load staging) when the rows cannot be described: a row pitch or base
// that is not a multiple of 16 bytes, or no encoder.
static bool make_tma_set(const FieldSetF& F, const RunConst& rc, TmaSet* out) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || rc.M < 2 || ((size_t)rc.nxg * 8) % 16 != 0) return false;
  const cplxf* bases[6] = {F.ex.p, F.er.p, F.et.p, F.bx.p, F.br.p, F.bt.p};
  const cuuint64_t dims[3] = {(cuuint64_t)rc.nxg, (cuuint64_t)rc.nyg, (cuuint64_t)rc.M};
  const cuuint64_t strides[2] = {(cuuint64_t)rc.nxg * 8, (cuuint64_t)rc.nxg * rc.nyg * 8};
  const cuuint32_t box[3] = {(cuuint32_t)TW, (cuuint32_t)RH, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  for (int q = 0; q < 6; ++q) {
    if ((reinterpret_cast<uintptr_t>(bases[q]) & 15) != 0) return false;
    if (enc(&out->map[q], CU_TENSOR_MAP_DATA_TYPE_INT64, 3, const_cast<cplxf*>(bases[q]), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

int push_mixed_blocks_per_sm(int M) {
  const size_t smem = push_mixed_smem(M);
  int nb = 1;
  switch (M) {
#define OCC(MM)                                                                                     \
  case MM:                                                                                          \
    cudaFuncSetAttribute(k_push_tiles<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    cudaFuncSetAttribute(k_push_tiles<MM>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);    \
    cudaFuncSetAttribute(k_push_tiles_batch<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                         (int)smem);                                                                 \
    cudaFuncSetAttribute(k_push_tiles_batch<MM>, cudaFuncAttributePreferredSharedMemoryCarveout,    \
                         100);                                                                       \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_push_tiles<MM>, PUSH_THREADS, smem);       \
    break;
    OCC(1) OCC(2) OCC(3) OCC(4)
#undef OCC
    default:
      break;
  }
  return nb < 1 ? 1 : nb;
}

void launch_push_mixed(cudaStream_t s, const FieldSetF& F, const SpeciesPtrs& sp, SpeciesCounters* cnt,
                       const StepRec* rec, const RunConst& rc, int apply_bcs, int nblocks_tiles,
                       int nblocks_global, const MixedParams& P, TileTable* tt, int count_zeroed) {
  const size_t smem = push_mixed_smem(rc.M);
  TmaSet tma;
  std::memset(&tma, 0, sizeof(tma));
  const int use_tma = make_tma_set(F, rc, &tma) ? 1 : 0;
  if (!count_zeroed) cudaMemsetAsync(P.fb_count, 0, sizeof(int), s);
  switch (rc.M) {
#define CASE(MM)                                                                                    \
  case MM:                                                                                          \
    k_push_tiles<MM><<<nblocks_tiles, PUSH_THREADS, smem, s>>>(F, sp, cnt, rec, rc, P, tt, apply_bcs, tma, use_tma); \
    k_push_global<MM><<<nblocks_global, PUSH_THREADS, 0, s>>>(F, sp, cnt, rec, rc, P, tt, apply_bcs);  \
    break;
    CASE(1) CASE(2) CASE(3) CASE(4)
#undef CASE
    default:
      break;
  }
}

// The push of a batch of runs with the same number of modes: the tile
// kernel over the (run, tile) table, then the deferred particles of each run.
void launch_push_mixed_batch(cudaStream_t s, int M, const BatchJob* jobs, int njobs, const int2* work,
                             const int* nwork, int nblocks_tiles, int nblocks_global) {
  const size_t smem = push_mixed_smem(M);
  switch (M) {
#define CASE(MM)                                                                                      \
  case MM:                                                                                            \
    k_push_tiles_batch<MM><<<nblocks_tiles, PUSH_THREADS, smem, s>>>(jobs, work, nwork);                \
    k_push_global_batch<MM><<<dim3(nblocks_global, njobs), PUSH_THREADS, 0, s>>>(jobs);                 \
    break;
    CASE(1) CASE(2) CASE(3) CASE(4)
#undef CASE
    default:
      break;
  }
}

}  // namespace CYL_TILE_NS

PushMixedFns CYL_TILE_FNS() {
  return {&CYL_TILE_NS::push_mixed_smem, &CYL_TILE_NS::push_mixed_blocks_per_sm, &CYL_TILE_NS::launch_push_mixed,
          &CYL_TILE_NS::launch_push_mixed_batch};
}

}  // namespace cyl
