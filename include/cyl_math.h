/*
 * cyl_math.h -- portable atan2 of the FP64 form.
 *
 * push_particles takes theta = ATAN2(z, y) twice per particle
 * (particles.F90:321,522).  The per-mode deposit factors of the reference
 * divide by (m*dtheta)^2 (particles.F90:595-596,619-624), which turns a
 * one-ulp difference in theta into a ~1e-9 relative difference in J_theta.
 * The reference calls the platform libm, whose last bit differs between
 * libraries; here the CUDA kernel and the CPU restatement both evaluate the
 * same routine below, built only from IEEE-754 +, -, *, / (no FMA
 * contraction: the files that include this are compiled with
 * --fmad=false / -ffp-contract=off), so the two agree bit for bit.
 *
 * Method (textbook argument reduction): with a = |y|, b = |x| reduce to
 * t = min(a,b)/max(a,b) in [0,1]; pick c = k/16 nearest to t and use
 * atan(t) = atan(c) + atan((t - c)/(1 + t c)), where |t'| <= 1/32 and
 * atan(t') is its Taylor series to t'^15; atan(k/16) is tabulated as a
 * double-double (values computed to 50 digits with mpmath).  The quadrant
 * is restored with pi/2 and pi as double-doubles.  Accuracy is about one
 * ulp against a correctly rounded atan2 (tests/test_cyl_math.py).
 */
#ifndef CYL_MATH_H
#define CYL_MATH_H

#include <math.h>

#if defined(__CUDACC__)
#define CYLM_FN __host__ __device__ inline
#else
#define CYLM_FN static inline
#endif

/* atan(k/16) = hi + lo, k = 0..16 */
#define CYLM_ATAN_TABLE                                         \
  {{0.0, 0.0},                                                  \
   {0.06241880999595735, -1.5490756308295046e-18},              \
   {0.12435499454676144, -3.1253241424539383e-18},              \
   {0.18534794999569476, 4.180692268843079e-18},                \
   {0.24497866312686414, 1.0698755618734451e-17},               \
   {0.3028848683749714, -1.1010827903001369e-17},               \
   {0.35877067027057225, -2.4623815582638635e-17},              \
   {0.4124104415973873, -1.587652227770689e-17},                \
   {0.4636476090008061, 2.2698777452961687e-17},                \
   {0.5123894603107377, -2.5462781472855804e-17},               \
   {0.5585993153435624, -5.4556305485916264e-18},               \
   {0.6022873461349642, 2.950430737228402e-17},                 \
   {0.6435011087932844, 1.5834785051444286e-17},                \
   {0.6823165548747481, 6.943223671560008e-18},                 \
   {0.7188299996216245, -2.1478388444456983e-17},               \
   {0.7531512809621944, -2.4256934659182068e-17},               \
   {0.7853981633974483, 3.061616997868383e-17}}

static const double cylm_atan_tab_host[17][2] = CYLM_ATAN_TABLE;
#if defined(__CUDACC__)
static __constant__ double cylm_atan_tab_dev[17][2] = CYLM_ATAN_TABLE;
#endif

CYLM_FN double cylm_atan_tab(int k, int part) {
#if defined(__CUDA_ARCH__)
  return cylm_atan_tab_dev[k][part];
#else
  return cylm_atan_tab_host[k][part];
#endif
}

CYLM_FN double cyl_atan2(double y, double x) {
  const double PIO2_HI = 1.5707963267948966, PIO2_LO = 6.123233995736766e-17;
  const double PI_HI = 3.141592653589793, PI_LO = 1.2246467991473532e-16;
  if (x != x || y != y) return x + y;
  const double ax = fabs(x), ay = fabs(y);
  const int xneg = signbit(x) ? 1 : 0;
  double a;
  if (ay == 0.0 && ax == 0.0) {
    a = xneg ? PI_HI : 0.0;
  } else if (isinf(ax) || isinf(ay)) {
    if (isinf(ax) && isinf(ay)) a = xneg ? 3.0 * (PI_HI / 4.0) : PI_HI / 4.0;
    else if (isinf(ay)) a = PIO2_HI;
    else a = xneg ? PI_HI : 0.0;
  } else {
    const int swap = ay > ax;
    const double t = swap ? ax / ay : ay / ax;
    const int k = (int)(t * 16.0 + 0.5);
    const double c = (double)k * 0.0625;
    const double tp = (t - c) / (1.0 + t * c);
    const double s = tp * tp;
    double p = -1.0 / 15.0;
    p = 1.0 / 13.0 + s * p;
    p = -1.0 / 11.0 + s * p;
    p = 1.0 / 9.0 + s * p;
    p = -1.0 / 7.0 + s * p;
    p = 1.0 / 5.0 + s * p;
    p = -1.0 / 3.0 + s * p;
    const double at = tp + tp * (s * p);
    a = cylm_atan_tab(k, 0) + (cylm_atan_tab(k, 1) + at);
    if (swap) a = PIO2_HI + (PIO2_LO - a);
    if (xneg) a = PI_HI + (PI_LO - a);
  }
  return signbit(y) ? -a : a;
}

/*
 * cyl_sincos_turn: sin and cos of 2 pi u for u in [0, 1) (u in turns), for
 * the angles of the counter-stream loader and injector, whose particles'
 * theta = atan2(z, y) enters the same (m dtheta)^-2 deposit factors: the CUDA
 * kernels and the CPU restatement must place them bit-identically.
 * Method: the quadrant k = floor(4u) is split off in turns, where
 * f = u - k/4 is exact for the stream's u = (r + 1/2) 2^-32; x = 2 pi f lies
 * in [0, pi/2), and sin x, cos x are their Taylor series to x^23 and x^22
 * (truncation below 2e-18 at pi/2) in Horner form with the reciprocal
 * factorial ratios as compile-time constants; the quadrant rotates the pair.
 * About one ulp from the correctly rounded values (tests/test_cyl_math.py).
 */
CYLM_FN void cyl_sincos_turn(double u, double* s, double* c) {
  int k = (int)(u * 4.0);
  if (k < 0) k = 0;
  if (k > 3) k = 3;
  const double f = u - 0.25 * (double)k;
  const double x = f * 6.283185307179586;
  const double x2 = x * x;
  double ps = 1.0 - x2 * (1.0 / 506.0);  /* 22 * 23 */
  ps = 1.0 - x2 * (1.0 / 420.0) * ps;    /* 20 * 21 */
  ps = 1.0 - x2 * (1.0 / 342.0) * ps;
  ps = 1.0 - x2 * (1.0 / 272.0) * ps;
  ps = 1.0 - x2 * (1.0 / 210.0) * ps;
  ps = 1.0 - x2 * (1.0 / 156.0) * ps;
  ps = 1.0 - x2 * (1.0 / 110.0) * ps;
  ps = 1.0 - x2 * (1.0 / 72.0) * ps;
  ps = 1.0 - x2 * (1.0 / 42.0) * ps;
  ps = 1.0 - x2 * (1.0 / 20.0) * ps;
  ps = 1.0 - x2 * (1.0 / 6.0) * ps;      /* 2 * 3 */
  double pc = 1.0 - x2 * (1.0 / 462.0);  /* 21 * 22 */
  pc = 1.0 - x2 * (1.0 / 380.0) * pc;    /* 19 * 20 */
  pc = 1.0 - x2 * (1.0 / 306.0) * pc;
  pc = 1.0 - x2 * (1.0 / 240.0) * pc;
  pc = 1.0 - x2 * (1.0 / 182.0) * pc;
  pc = 1.0 - x2 * (1.0 / 132.0) * pc;
  pc = 1.0 - x2 * (1.0 / 90.0) * pc;
  pc = 1.0 - x2 * (1.0 / 56.0) * pc;
  pc = 1.0 - x2 * (1.0 / 30.0) * pc;
  pc = 1.0 - x2 * (1.0 / 12.0) * pc;
  pc = 1.0 - x2 * (1.0 / 2.0) * pc;      /* 1 * 2 */
  const double sx = x * ps, cx = pc;
  if (k == 0) {
    *s = sx;
    *c = cx;
  } else if (k == 1) {
    *s = cx;
    *c = -sx;
  } else if (k == 2) {
    *s = -sx;
    *c = -cx;
  } else {
    *s = -cx;
    *c = sx;
  }
}

#endif /* CYL_MATH_H */
