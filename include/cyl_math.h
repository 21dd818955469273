/*
 * cyl_math.h -- correctly rounded atan2 of the FP64 form, and the sin/cos of
 * the counter-stream angles.
 *
 * push_particles takes theta = ATAN2(z, y) twice per particle
 * (particles.F90:321,522).  The per-mode deposit factors of the reference
 * divide by (m*dtheta)^2 (particles.F90:595-596,619-624), which turns a
 * one-ulp difference in theta into a ~1e-9 relative difference in J_theta.
 * The reference calls the platform libm.  glibc's atan2 is not correctly
 * rounded (glibc 2.39: one ulp off on about 0.035 % of random arguments),
 * so the reference's own J_theta differs in its last digits between
 * libraries.  cyl_atan2 below returns the correctly rounded result, the one
 * value every platform can agree on; it equals libm's wherever libm is
 * correctly rounded.  The CUDA kernel and the CPU restatement evaluate the
 * same code, built from IEEE-754 +, -, *, / and explicit fma() only (no FMA
 * contraction: the files that include this are compiled with --fmad=false /
 * -ffp-contract=off), so the two agree bit for bit.
 *
 * Method (table-driven argument reduction in double-double arithmetic,
 * Dekker's exact products and Knuth's two-sum): with a = |y|, b = |x|,
 * t = min(a,b)/max(a,b) in [0,1] is formed as t_hi + t_lo from a reciprocal
 * and the remainder of the product (an FMA); c = k/128 is the grid point nearest to t and
 * atan(t) = atan(c) + atan(u), u = (t - c)/(1 + t c), |u| <= 1/256 + ulp,
 * with u as a double-double (the same reciprocal-and-remainder form: the
 * routine divides twice, by max(a,b) and by 1 + t c; the narrow FP64 pipe
 * of the GPU makes each division cost about ten FP64 operations).  atan(u) = u + u q, q = -u^2/3 (double-double)
 * + u^4/5 - u^6/7 + u^8/9 - u^10/11 (double; the first omitted term is below
 * 2^-99 of q).  atan(k/128) is tabulated as a double-double (mpmath at 300
 * bits), and the quadrant is restored with pi/2 and pi as double-doubles.
 * The double-double result carries a relative error of about 2^-100, so its
 * final rounding is the correct rounding of atan2 except when the exact
 * value lies within 2^-100 of a rounding boundary (probability ~2^-47 per
 * argument).  Arguments whose ratio is below 2^-1000 return the ratio
 * min/max rounded once, which is the correctly rounded result except at an
 * exact tie between two subnormals.  Tested against mpmath
 * (tests/test_cyl_math.py).
 */
#ifndef CYL_MATH_H
#define CYL_MATH_H

#include <math.h>

#if defined(__CUDACC__)
#define CYLM_FN __host__ __device__ inline
#else
#define CYLM_FN static inline
#endif

/* atan(k/128) = hi + lo, k = 0..128 */
#define CYLM_ATAN_TABLE \
  {\
   {0.0, 0.0},  \
   {0.007812341060101111, 1.5247608492487475e-19},  \
   {0.015623728620476831, -4.913600136566304e-19},  \
   {0.023433209879467586, -1.0946924642180502e-18},  \
   {0.031239833430268277, -1.188442711587748e-18},  \
   {0.03904264995516699, 6.271263374213089e-19},  \
   {0.046840712915969654, -1.655677442254952e-19},  \
   {0.05463307923935948, -2.6698003590189837e-18},  \
   {0.06241880999595735, -1.5490756308295046e-18},  \
   {0.07019697107187052, -1.798192160322046e-18},  \
   {0.0779666338315423, 5.804551873143357e-18},  \
   {0.08572687577074481, 5.347194143502951e-18},  \
   {0.09347678115858947, -6.2844725995420954e-18},  \
   {0.10121544166746667, 5.681202558623414e-18},  \
   {0.10894195698986579, 6.8267122072409585e-18},  \
   {0.11665543544106935, 5.487925812108699e-18},  \
   {0.12435499454676144, -3.1253241424539383e-18},  \
   {0.13203976161463876, -1.2769254007099595e-17},  \
   {0.13970887428916365, -2.9579864247315813e-18},  \
   {0.14736148108865163, 5.409599147666298e-18},  \
   {0.15499674192394097, 9.585415594114324e-18},  \
   {0.16261382859794857, 7.784470643106252e-18},  \
   {0.1702119252854744, -3.541164079802125e-18},  \
   {0.17779022899267607, -4.029582100854422e-18},  \
   {0.18534794999569476, 4.180692268843079e-18},  \
   {0.19288431225797467, -7.414590176247246e-18},  \
   {0.2003985538258785, 3.1399542871844493e-18},  \
   {0.207889927202263, 7.333160666520898e-18},  \
   {0.21535769969773805, 4.738160130078733e-19},  \
   {0.22280115375939452, -5.498822172446843e-18},  \
   {0.23021958727684372, 1.2313404529142703e-17},  \
   {0.23761231386547124, 1.058231431371113e-17},  \
   {0.24497866312686414, 1.0698755618734451e-17},  \
   {0.2523179808864272, -1.9471162027087266e-17},  \
   {0.2596296294082575, 1.9238754924615304e-17},  \
   {0.26691298758740045, -1.809450026578138e-17},  \
   {0.2741674511196588, 8.261353575163773e-18},  \
   {0.28139243264917846, -7.594730074283234e-18},  \
   {0.2885873618940774, -1.428369957377257e-17},  \
   {0.29575168575043154, 1.1955271549785761e-17},  \
   {0.3028848683749714, -1.1010827903001369e-17},  \
   {0.30998639124688343, 1.4934173643675254e-17},  \
   {0.31705575320914703, -1.893928924292642e-17},  \
   {0.3240924704898717, -1.31421892240624e-17},  \
   {0.3310960767041321, -7.952610375793799e-18},  \
   {0.33806612283682547, 1.4946671397270723e-17},  \
   {0.34500217720710513, -2.2938804755578304e-17},  \
   {0.3519038254149648, -1.9886237545562348e-18},  \
   {0.35877067027057225, -2.4623815582638635e-17},  \
   {0.3656023317069669, -3.232740235706072e-18},  \
   {0.3723984466767542, 1.9612311504845653e-17},  \
   {0.3791586690334418, 2.5555409686140026e-17},  \
   {0.38588266939807375, 2.378822732491941e-17},  \
   {0.3925701350118286, 1.4769733768267405e-17},  \
   {0.39922076957525254, 2.246598105617042e-17},  \
   {0.4058342930748041, -2.4728071815164154e-17},  \
   {0.4124104415973873, -1.587652227770689e-17},  \
   {0.41894896713355284, 2.7554871436380083e-17},  \
   {0.42544963737004227, 2.3315530741892885e-17},  \
   {0.4319122354723482, 1.8301439937795217e-17},  \
   {0.43833655985795783, -2.494277030626541e-17},  \
   {0.44472242396093936, -2.0205282713454678e-17},  \
   {0.4510696559885235, -2.2703795229420475e-17},  \
   {0.4573780986703208, 1.0659281558975183e-17},  \
   {0.4636476090008061, 2.2698777452961687e-17},  \
   {0.46987805797568694, -4.052709832737995e-18},  \
   {0.4760693303227612, 1.4654487332256713e-17},  \
   {0.48222132422785374, -6.892698180647022e-18},  \
   {0.48833395105640554, -1.1373236189329585e-17},  \
   {0.49440713507127537, -2.484649204493573e-17},  \
   {0.5004408131472942, -4.7181675085518756e-17},  \
   {0.5064349344830967, 2.1662702888915918e-17},  \
   {0.5123894603107377, -2.5462781472855804e-17},  \
   {0.518304363603578, -1.4859314226587844e-17},  \
   {0.5241796287829132, 5.520094119641666e-18},  \
   {0.5300152514237931, 3.230433670398613e-20},  \
   {0.5358112379604637, -4.0637956834825575e-18},  \
   {0.541567605391845, -3.5958145539643824e-17},  \
   {0.5472843809874369, 4.923709671396255e-17},  \
   {0.5529616019940283, -7.85800765242264e-18},  \
   {0.5585993153435624, -5.4556305485916264e-18},  \
   {0.5641975773624976, -4.088689784609966e-17},  \
   {0.5697564534829784, 1.2255062085054184e-17},  \
   {0.5752760179561178, 6.3047065262415604e-18},  \
   {0.5807563535676704, -1.441464378193067e-17},  \
   {0.5861975513563606, -2.246359256161595e-18},  \
   {0.5915997103351114, 4.920495453686772e-17},  \
   {0.5969629372154015, 3.4780325041179635e-17},  \
   {0.6022873461349642, 2.950430737228402e-17},  \
   {0.6075730583890224, -4.546482020514537e-18},  \
   {0.6128202021652414, -3.1552061848586226e-17},  \
   {0.6180289122825618, -5.217936253827864e-17},  \
   {0.6231993299340659, 2.672403885140095e-17},  \
   {0.6283316024340097, 8.602534936248055e-18},  \
   {0.6334258829691446, -2.7290767436015276e-17},  \
   {0.6384823303544376, -8.503543139790755e-18},  \
   {0.6435011087932844, 1.5834785051444286e-17},  \
   {0.6484823876423006, -4.8645153510305985e-17},  \
   {0.6534263411807619, 3.5800634857340095e-17},  \
   {0.658333148384756, 1.582190586223303e-17},  \
   {0.6632029927060933, -3.076054864429649e-17},  \
   {0.6680360618560202, 4.436835183629535e-17},  \
   {0.6728325475937632, -1.899315009714705e-17},  \
   {0.6775926455199252, 4.023193265647988e-17},  \
   {0.6823165548747481, 6.943223671560008e-18},  \
   {0.687004478341245, -5.919903342770666e-18},  \
   {0.6916566218531999, -8.117151192285796e-18},  \
   {0.6962731944080236, -6.676326953941976e-18},  \
   {0.7008544078844502, -1.987626234335816e-17},  \
   {0.705400476865049, 5.1314774085494894e-17},  \
   {0.7099116184635249, -4.597166450584887e-17},  \
   {0.714388052156769, -6.065199961989827e-18},  \
   {0.7188299996216245, -2.1478388444456983e-17},  \
   {0.7232376845763179, 5.4825900866114946e-18},  \
   {0.7276113326265107, 2.569325697391839e-18},  \
   {0.7319511711159166, 3.0500950191971875e-17},  \
   {0.7362574289814281, 3.473937648299457e-17},  \
   {0.7405303366126927, -5.0144719711844464e-17},  \
   {0.7447701257160751, 3.708315849135547e-17},  \
   {0.7489770291829414, 5.5225132122615064e-17},  \
   {0.7531512809621944, -2.4256934659182068e-17},  \
   {0.7572931159369924, 8.267789465700113e-18},  \
   {0.7614027698055784, 9.850030332752822e-18},  \
   {0.7654804789661445, 1.4471913247374173e-17},  \
   {0.7695264804056583, -3.704991905602721e-17},  \
   {0.7735410115925735, 4.84248858844057e-17},  \
   {0.7775243103733478, -2.6676490951944502e-17},  \
   {0.7814766148726883, 3.907463295560081e-17},  \
   {0.7853981633974483, 3.061616997868383e-17}}

static const double cylm_atan_tab_host[129][2] = CYLM_ATAN_TABLE;
#if defined(__CUDACC__)
/* global memory (L1-cached): lanes of a warp read different rows */
static __device__ const double cylm_atan_tab_dev[129][2] = CYLM_ATAN_TABLE;
#endif

CYLM_FN double cylm_atan_tab(int k, int part) {
#if defined(__CUDA_ARCH__)
  return __ldg(&cylm_atan_tab_dev[k][part]);
#else
  return cylm_atan_tab_host[k][part];
#endif
}

CYLM_FN double cylm_fma(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(a, b, c);
#else
  return fma(a, b, c);
#endif
}

/* s + e = a + b exactly (Knuth's two-sum) */
CYLM_FN void cylm_two_sum(double a, double b, double* s, double* e) {
  const double x = a + b;
  const double bv = x - a;
  *e = (a - (x - bv)) + (b - bv);
  *s = x;
}

/* s + e = a + b exactly, for |a| >= |b| or a = 0 (Dekker's fast two-sum) */
CYLM_FN void cylm_fast_two_sum(double a, double b, double* s, double* e) {
  const double x = a + b;
  *e = b - (x - a);
  *s = x;
}

/* (h, l) = c - (a_h + a_l) for a double-double constant c = (c_h, c_l) */
CYLM_FN void cylm_dd_rsub(double c_h, double c_l, double a_h, double a_l, double* h, double* l) {
  double s, e;
  cylm_two_sum(c_h, -a_h, &s, &e);
  e = e + (c_l - a_l);
  cylm_fast_two_sum(s, e, h, l);
}

CYLM_FN double cyl_atan2(double y, double x) {
  const double PIO2_HI = 1.5707963267948966, PIO2_LO = 6.123233995736766e-17;
  const double PI_HI = 3.141592653589793, PI_LO = 1.2246467991473532e-16;
  if (x != x || y != y) return x + y;
  const double ax = fabs(x), ay = fabs(y);
  const int xneg = signbit(x) ? 1 : 0;
  double ah, al;
  if (ay == 0.0 && ax == 0.0) {
    ah = xneg ? PI_HI : 0.0;
    al = 0.0;
  } else if (isinf(ax) || isinf(ay)) {
    if (isinf(ax) && isinf(ay)) ah = xneg ? 3.0 * (PI_HI / 4.0) : PI_HI / 4.0;
    else if (isinf(ay)) ah = PIO2_HI;
    else ah = xneg ? PI_HI : 0.0;
    al = 0.0;
  } else {
    const int swap = ay > ax;
    const double num0 = swap ? ax : ay, den0 = swap ? ay : ax;
    double num = num0, den = den0;
    /* scale both by one power of two so that den lies in [1, 2): the
       remainder of the division below is then exact */
    const int e = ilogb(den);
    num = scalbn(num, -e);
    den = scalbn(den, -e);
    /* one division: th = num (1/den) need not be the rounded quotient,
       only the head of th + tl, whose tail comes from the remainder */
    const double rden = 1.0 / den;
    const double th = num * rden;
    if (th < 0x1p-1000) {
      /* atan(t) = t to far below the last bit: the ratio of the unscaled
         arguments, rounded once (also into the subnormal range) */
      ah = num0 / den0;
      al = 0.0;
    } else {
      const double tl = cylm_fma(-th, den, num) * rden;
      const int k = (int)(th * 128.0 + 0.5);
      const double c = (double)k * 0.0078125;
      double uh, ul;
      if (k == 0) {
        uh = th;
        ul = tl;
      } else {
        /* u = (t - c) / (1 + t c): th - c is exact (c/2 <= th <= 2c) */
        double nh, nl, dh, dl, p, pe;
        cylm_two_sum(th - c, tl, &nh, &nl);
        p = th * c;
        pe = cylm_fma(th, c, -p);
        cylm_fast_two_sum(1.0, p, &dh, &dl);
        dl = dl + (pe + tl * c);
        cylm_fast_two_sum(dh, dl, &dh, &dl);
        const double rdh = 1.0 / dh;
        uh = nh * rdh;
        double rem = cylm_fma(-uh, dh, nh);
        rem = (rem + nl) - uh * dl;
        ul = rem * rdh;
      }
      /* q = -u^2/3 + u^4/5 - u^6/7 + u^8/9 - u^10/11 */
      const double sh = uh * uh;
      const double sl = cylm_fma(uh, uh, -sh) + 2.0 * uh * ul;
      const double third = 1.0 / 3.0;
      const double qh = -(sh * third);
      const double qr = cylm_fma(-3.0, qh, -sh); /* -sh = 3 qh + qr exactly */
      const double ql = (qr - sl) * third;
      double q1 = 1.0 / 9.0 - sh * (1.0 / 11.0);
      q1 = 1.0 / 7.0 - sh * q1;
      q1 = 1.0 / 5.0 - sh * q1;
      q1 = (sh * sh) * q1;
      /* atan(u) = u + u q */
      const double ph = uh * qh;
      const double pl = cylm_fma(uh, qh, -ph) + (uh * (ql + q1) + ul * qh);
      double bh, bl;
      cylm_two_sum(uh, ph, &bh, &bl);
      bl = bl + (ul + pl);
      cylm_fast_two_sum(bh, bl, &bh, &bl);
      /* + atan(c) */
      double rh, rl;
      cylm_two_sum(cylm_atan_tab(k, 0), bh, &rh, &rl);
      rl = rl + (cylm_atan_tab(k, 1) + bl);
      cylm_fast_two_sum(rh, rl, &ah, &al);
    }
    if (swap) cylm_dd_rsub(PIO2_HI, PIO2_LO, ah, al, &ah, &al);
    if (xneg) cylm_dd_rsub(PI_HI, PI_LO, ah, al, &ah, &al);
  }
  const double a = ah + al;
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
