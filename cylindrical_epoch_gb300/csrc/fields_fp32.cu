// fields_fp32.cu -- bulk per-mode Yee updates of the mixed-precision form.
//
// Same equations as update_e_field / update_b_field (fields.f90:67-108,
// 203-241) with E and B stored as FP32 complex and the currents FP64.  The
// bulk rows run in FP32 with the per-row coefficients (c^2/r, dt/r, ...)
// precomputed; the first radial cell (ir = 1, where the 1/r terms are
// largest) is updated in FP64 arithmetic.  The FP64 -> FP32 conversion of
// the currents is done with integer operations (GB300's FP64 pipe is narrow).
#include <cmath>

#include "cyl_common.cuh"
#include "cyl_kernels.cuh"
#include "cyl_convert.cuh"
#include "axis_rules.cuh"

namespace cyl {

// rowtab (per ir = 0 .. ny+1, float4): x = c^2/r_p * dt/2, y = c^2/r_d * dt/2,
// z = dt/2 / r_d, w = dt/2 / r_p
__device__ __forceinline__ float2 ld2(const cplxf* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(cplxf* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
__device__ __forceinline__ float2 ldj(const cplx* p) {
  const double2 v = *reinterpret_cast<const double2*>(p);
  return make_float2(d2f_bits(v.x), d2f_bits(v.y));
}

// One cell and mode of update_e_field's bulk: (ix, ir) for ix = 0..nx,
// ir = 1..ny.  reps = 2 applies two consecutive half-step updates at once
// (the closing half of one step and the opening half of the next, which see
// the same B and J): the increment is formed once and added twice, with the
// FP32 roundings of two separate updates.  The increments are written with
// explicit roundings, so that one add and two adds of the same increment
// give the results of one and of two separate launches bit for bit.
__device__ __forceinline__ double dinc2(double s0, double c1, double v1, double c2, double v2) {
  return __fma_rn(c2, v2, __fma_rn(c1, v1, s0));
}
__device__ __forceinline__ double dinc3(double s0, double c1, double v1, double c2, double v2, double c3,
                                        double v3) {
  return __fma_rn(c3, v3, dinc2(s0, c1, v1, c2, v2));
}
__device__ __forceinline__ float inc2(float s0, float c1, float v1, float c2, float v2) {
  return __fmaf_rn(c2, v2, __fmaf_rn(c1, v1, s0));
}
__device__ __forceinline__ float inc3(float s0, float c1, float v1, float c2, float v2, float c3, float v3) {
  return __fmaf_rn(c3, v3, inc2(s0, c1, v1, c2, v2));
}
__device__ __forceinline__ void update_e_item(const FieldSetF& F, const float4* rowtab, float cdx, float cdy,
                                              float cj, const Row1E& r1, int ix, int im, int ir, int reps = 1) {
  if (ir == 1) {
    // first radial cell in FP64 arithmetic (the equations of update_e_field)
    const double m = (double)im;
    const cplx bt0 = F.bt(ix, ir, im), bt1 = F.bt(ix, ir + 1, im), btx = F.bt(ix + 1, ir, im);
    const cplx br0 = F.br(ix, ir, im), brx = F.br(ix + 1, ir, im);
    const cplx bx0 = F.bx(ix, ir, im), bx1 = F.bx(ix, ir + 1, im);
    const cplx jx = F.jx(ix, ir, im), jr = F.jr(ix, ir, im), jt = F.jt(ix, ir, im);
    const double bmm = r1.bm * m, erm = r1.erm * m;
    cplx ex = F.ex(ix, ir, im), er = F.er(ix, ir, im), et = F.et(ix, ir, im);
    // ex += a (bt1 + bt0) + i m bm br0 + c (bt1 - bt0) - d jx
    ex.re = __dadd_rn(ex.re, dinc3(__dmul_rn(r1.a, __dadd_rn(bt1.re, bt0.re)), -bmm, br0.im, r1.c,
                                   __dsub_rn(bt1.re, bt0.re), -r1.d, jx.re));
    ex.im = __dadd_rn(ex.im, dinc3(__dmul_rn(r1.a, __dadd_rn(bt1.im, bt0.im)), bmm, br0.re, r1.c,
                                   __dsub_rn(bt1.im, bt0.im), -r1.d, jx.im));
    // er += -i m erm bx0 - cx (btx - bt0) - d jr
    er.re = __dadd_rn(er.re, dinc2(__dmul_rn(erm, bx0.im), -r1.cx, __dsub_rn(btx.re, bt0.re), -r1.d, jr.re));
    er.im = __dadd_rn(er.im, dinc2(__dmul_rn(-erm, bx0.re), -r1.cx, __dsub_rn(btx.im, bt0.im), -r1.d, jr.im));
    // et += cx (brx - br0) - c (bx1 - bx0) - d jt
    et.re = __dadd_rn(et.re, dinc2(__dmul_rn(r1.cx, __dsub_rn(brx.re, br0.re)), -r1.c, __dsub_rn(bx1.re, bx0.re),
                                   -r1.d, jt.re));
    et.im = __dadd_rn(et.im, dinc2(__dmul_rn(r1.cx, __dsub_rn(brx.im, br0.im)), -r1.c, __dsub_rn(bx1.im, bx0.im),
                                   -r1.d, jt.im));
    F.ex(ix, ir, im) = ex;
    F.er(ix, ir, im) = er;
    F.et(ix, ir, im) = et;
    return;
  }
  const float4 rt = rowtab[ir];
  const float m = (float)im;
  const float2 bt0 = ld2(F.bt.ptr(ix, ir, im)), bt1 = ld2(F.bt.ptr(ix, ir + 1, im)), btx = ld2(F.bt.ptr(ix + 1, ir, im));
  const float2 br0 = ld2(F.br.ptr(ix, ir, im)), brx = ld2(F.br.ptr(ix + 1, ir, im));
  const float2 bx0 = ld2(F.bx.ptr(ix, ir, im)), bx1 = ld2(F.bx.ptr(ix, ir + 1, im));
  const float2 jx = ldj(F.jx.ptr(ix, ir, im)), jr = ldj(F.jr.ptr(ix, ir, im)), jt = ldj(F.jt.ptr(ix, ir, im));
  const float ah = __fmul_rn(rt.x, 0.5f), am = __fmul_rn(rt.x, m), b = __fmul_rn(rt.y, m);
  // ex += c^2/r_p*dt/2 * (0.5 (bt1 + bt0) + i m br0) + c^2 dt/(2 dy) (bt1 - bt0) - dt/(2 eps0) jx
  const float2 dex = make_float2(
      inc3(__fmul_rn(ah, __fadd_rn(bt1.x, bt0.x)), -am, br0.y, cdy, __fsub_rn(bt1.x, bt0.x), -cj, jx.x),
      inc3(__fmul_rn(ah, __fadd_rn(bt1.y, bt0.y)), am, br0.x, cdy, __fsub_rn(bt1.y, bt0.y), -cj, jx.y));
  // er += -i m c^2/r_d dt/2 bx0 - c^2 dt/(2 dx) (btx - bt0) - dt/(2 eps0) jr
  const float2 der = make_float2(inc2(__fmul_rn(b, bx0.y), -cdx, __fsub_rn(btx.x, bt0.x), -cj, jr.x),
                                 inc2(__fmul_rn(-b, bx0.x), -cdx, __fsub_rn(btx.y, bt0.y), -cj, jr.y));
  // et += c^2 dt/(2 dx) (brx - br0) - c^2 dt/(2 dy) (bx1 - bx0) - dt/(2 eps0) jt
  const float2 det = make_float2(
      inc2(__fmul_rn(cdx, __fsub_rn(brx.x, br0.x)), -cdy, __fsub_rn(bx1.x, bx0.x), -cj, jt.x),
      inc2(__fmul_rn(cdx, __fsub_rn(brx.y, br0.y)), -cdy, __fsub_rn(bx1.y, bx0.y), -cj, jt.y));
  float2 ex = ld2(F.ex.ptr(ix, ir, im)), er = ld2(F.er.ptr(ix, ir, im)), et = ld2(F.et.ptr(ix, ir, im));
  for (int k = 0; k < reps; ++k) {
    ex = make_float2(__fadd_rn(ex.x, dex.x), __fadd_rn(ex.y, dex.y));
    er = make_float2(__fadd_rn(er.x, der.x), __fadd_rn(er.y, der.y));
    et = make_float2(__fadd_rn(et.x, det.x), __fadd_rn(et.y, det.y));
  }
  st2(F.ex.ptr(ix, ir, im), ex);
  st2(F.er.ptr(ix, ir, im), er);
  st2(F.et.ptr(ix, ir, im), et);
}

// One cell and mode of update_b_field over the whole ghosted array (index
// i, j from the first ghost), with the optional B_old save.
__device__ __forceinline__ void update_b_item(const FieldSetF& F, int save_old, const float4* rowtab, float hdx,
                                              float hdy, const Row1B& r1, const RunConst& rc, int i, int im,
                                              int j) {
  const int ix = i + 1 - NG, ir = j + 1 - NG;
  if (save_old) {
    st2(F.bxo.ptr(ix, ir, im), ld2(F.bx.ptr(ix, ir, im)));
    st2(F.bro.ptr(ix, ir, im), ld2(F.br.ptr(ix, ir, im)));
    st2(F.bto.ptr(ix, ir, im), ld2(F.bt.ptr(ix, ir, im)));
  }
  if (ix < 0 || ix > rc.nx || ir < 1 || ir > rc.ny - 1) return;
  if (ir == 1) {
    // first radial cell in FP64 arithmetic (the equations of update_b_field)
    const double m = (double)im;
    const cplx et0 = F.et(ix, ir, im), etm1 = F.et(ix, ir - 1, im), etxm = F.et(ix - 1, ir, im);
    const cplx er0 = F.er(ix, ir, im), erxm = F.er(ix - 1, ir, im);
    const cplx ex0 = F.ex(ix, ir, im), exm1 = F.ex(ix, ir - 1, im);
    const double pm = r1.p * m, sm = r1.s * m;
    cplx bx = F.bx(ix, ir, im), br = F.br(ix, ir, im), bt = F.bt(ix, ir, im);
    // bx -= i m p er0 + q (et0 + etm1) + r (et0 - etm1)
    bx.re -= -pm * er0.im + r1.q * (et0.re + etm1.re) + r1.r * (et0.re - etm1.re);
    bx.im -= pm * er0.re + r1.q * (et0.im + etm1.im) + r1.r * (et0.im - etm1.im);
    // br += i m s ex0 + t (et0 - etxm)
    br.re += -sm * ex0.im + r1.t * (et0.re - etxm.re);
    br.im += sm * ex0.re + r1.t * (et0.im - etxm.im);
    // bt += -t (er0 - erxm) + r (ex0 - exm1)
    bt.re += -r1.t * (er0.re - erxm.re) + r1.r * (ex0.re - exm1.re);
    bt.im += -r1.t * (er0.im - erxm.im) + r1.r * (ex0.im - exm1.im);
    F.bx(ix, ir, im) = bx;
    F.br(ix, ir, im) = br;
    F.bt(ix, ir, im) = bt;
    return;
  }
  const float4 rt = rowtab[ir];
  const float m = (float)im;
  const float2 et0 = ld2(F.et.ptr(ix, ir, im)), etm1 = ld2(F.et.ptr(ix, ir - 1, im)), etxm = ld2(F.et.ptr(ix - 1, ir, im));
  const float2 er0 = ld2(F.er.ptr(ix, ir, im)), erxm = ld2(F.er.ptr(ix - 1, ir, im));
  const float2 ex0 = ld2(F.ex.ptr(ix, ir, im)), exm1 = ld2(F.ex.ptr(ix, ir - 1, im));
  // bx -= dt/2 (i m/r_d er0 + 0.5 (et0 + etm1)/r_d + (et0 - etm1)/dy)
  const float c1 = rt.z * m, c2 = rt.z * 0.5f, c3 = rt.w * m;
  float2 b = ld2(F.bx.ptr(ix, ir, im));
  b.x -= -c1 * er0.y + c2 * (et0.x + etm1.x) + hdy * (et0.x - etm1.x);
  b.y -= c1 * er0.x + c2 * (et0.y + etm1.y) + hdy * (et0.y - etm1.y);
  st2(F.bx.ptr(ix, ir, im), b);
  // br += dt/2 (i m/r_p ex0 + (et0 - etxm)/dx)
  b = ld2(F.br.ptr(ix, ir, im));
  b.x += -c3 * ex0.y + hdx * (et0.x - etxm.x);
  b.y += c3 * ex0.x + hdx * (et0.y - etxm.y);
  st2(F.br.ptr(ix, ir, im), b);
  // bt += dt/2 (-(er0 - erxm)/dx + (ex0 - exm1)/dy)
  b = ld2(F.bt.ptr(ix, ir, im));
  b.x += -hdx * (er0.x - erxm.x) + hdy * (ex0.x - exm1.x);
  b.y += -hdx * (er0.y - erxm.y) + hdy * (ex0.y - exm1.y);
  st2(F.bt.ptr(ix, ir, im), b);
}

// Grid: (columns, modes, rows), so that the FP64 first row of every mode is
// in the first wave of CTAs rather than the tail of the launch.
__global__ void k_update_e_f32(FieldSetF F, const float4* rowtab, float cdx, float cdy, float cj, Row1E r1,
                               RunConst rc) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx
  if (ix > rc.nx) return;
  update_e_item(F, rowtab, cdx, cdy, cj, r1, ix, blockIdx.y, 1 + blockIdx.z);
}

// Two consecutive E half-steps with the E boundary rules between them (the
// closing half of one step, the opening half of the next) in two launches
// instead of two bulk passes and two axis launches.  Between the halves, the
// axis rules and the ghost phases read E of rows 1 and 2, column 1 and column
// nx, and write rows <= 0 and ghost cells; inside the update range they
// write only row 1 (modes >= 2), row ny, columns 0 and nx.  These edge cells
// take the two halves one at a time: the first by k_update_e_edge_axis_f32
// before the rules, the second by k_update_e_fused_axis_f32 after them.
// Every other cell reads only its own E, so it takes both halves in
// k_update_e_fused_axis_f32.
//
// The axis rules run inside the same launches, per column: the first launch
// updates rows 1 and 2 of its column, then applies the axis row's sequence
// (task 0, which reads rows 0..2 of the column); its ghost-row mirrors
// (tasks >= 1) are left out, as every value they would write is rewritten
// by the mirrors after the second half before anything reads it.  The second
// launch updates rows 1 .. NG of its column, then applies all the column's
// axis tasks (the mirrors read rows 1 .. NG).  Both cover the ghost columns
// too, for the axis rules alone.
__device__ __forceinline__ bool e_edge_cell(int ix, int ir, const RunConst& rc) {
  return ir <= 2 || ir == rc.ny || ix <= 1 || ix == rc.nx;
}
// Items: (column 1-NG .. nx+NG) for rows 1, 2 and the axis row, then the
// other edge cells: row ny, and columns 0, 1, nx of rows 3 .. ny-1.
__global__ void k_update_e_edge_axis_f32(FieldSetF F, const float4* rowtab, float cdx, float cdy, float cj, Row1E r1,
                                         BcConst K, RunConst rc) {
  const int nx = rc.nx, ny = rc.ny, im = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncolg = nx + 2 * NG, nrow = nx + 1, ncol = 3 * (ny - 3);
  if (t < ncolg) {
    const int ix = 1 - NG + t;
    if (ix >= 0 && ix <= nx) {
      update_e_item(F, rowtab, cdx, cdy, cj, r1, ix, im, 1);
      update_e_item(F, rowtab, cdx, cdy, cj, r1, ix, im, 2);
    }
    e_axis_item<cplxf>(F.ex, F.er, F.et, F.jx, F.bt, rc, K, ix, im, 0);
    return;
  }
  int u = t - ncolg, ix, ir;
  if (u < nrow) {
    ix = u;
    ir = ny;
  } else if ((u -= nrow) < ncol) {
    const int k = u / (ny - 3);
    ir = 3 + (u - k * (ny - 3));
    ix = k == 0 ? 0 : k == 1 ? 1 : nx;
  } else {
    return;
  }
  update_e_item(F, rowtab, cdx, cdy, cj, r1, ix, im, ir);
}
// blockIdx.z = 0: per column (1-NG .. nx+NG), rows 1 .. NG, then the
// column's axis tasks; blockIdx.z = z >= 1: row NG + z of columns 0 .. nx.
__global__ void k_update_e_fused_axis_f32(FieldSetF F, const float4* rowtab, float cdx, float cdy, float cj,
                                          Row1E r1, BcConst K, RunConst rc) {
  const int nx = rc.nx, im = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.z == 0) {
    if (t >= nx + 2 * NG) return;
    const int ix = 1 - NG + t;
    if (ix >= 0 && ix <= nx)
      for (int ir = 1; ir <= NG; ++ir)
        update_e_item(F, rowtab, cdx, cdy, cj, r1, ix, im, ir, e_edge_cell(ix, ir, rc) ? 1 : 2);
    for (int task = 0; task < NG; ++task) e_axis_item<cplxf>(F.ex, F.er, F.et, F.jx, F.bt, rc, K, ix, im, task);
    return;
  }
  if (t > nx) return;
  const int ir = NG + (int)blockIdx.z;
  update_e_item(F, rowtab, cdx, cdy, cj, r1, t, im, ir, e_edge_cell(t, ir, rc) ? 1 : 2);
}

// The B updates wait on memory (long-scoreboard stalls, a third of the HBM
// bandwidth at 32 warps an SM, the register-bound occupancy): a 40-register
// cap gives 48 warps an SM (the FP64 first row's few spills are in one row
// of the grid).
constexpr int B_BLOCKS_PER_SM = 12;
__global__ void __launch_bounds__(128, B_BLOCKS_PER_SM) k_update_b_f32(FieldSetF F, int save_old,
                                                                      const float4* rowtab, float hdx, float hdy,
                                                                      Row1B r1, RunConst rc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rc.nxg) return;
  update_b_item(F, save_old, rowtab, hdx, hdy, r1, rc, i, blockIdx.y, blockIdx.z);
}
// The opening B half-step of a step (B_old saved) with the step's zeroing
// folded in: every cell of the ghosted grid also clears its values of the
// three current arrays jx, jr, jt of Fz (the push's J after the J swap,
// which nothing reads any more), and the first CTA clears the deferred
// counts.  The grid covers the current arrays' whole extent.
__global__ void __launch_bounds__(128, B_BLOCKS_PER_SM) k_update_b_f32_zero(FieldSetF F, const float4* rowtab,
                                                                           float hdx, float hdy, Row1B r1,
                                                                           RunConst rc, FView jx, FView jr,
                                                                           FView jt, ZeroCounts zc) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && (int)threadIdx.x < zc.n) *zc.p[threadIdx.x] = 0;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rc.nxg) return;
  const int ix = i + 1 - NG, ir = (int)blockIdx.z + 1 - NG, im = blockIdx.y;
  const cplx z = mk(0.0, 0.0);
  *jx.ptr(ix, ir, im) = z;
  *jr.ptr(ix, ir, im) = z;
  *jt.ptr(ix, ir, im) = z;
  update_b_item(F, 1, rowtab, hdx, hdy, r1, rc, i, blockIdx.y, blockIdx.z);
}

// The batched forms: run blockIdx.z, (mode, row) blockIdx.y = m + M row.
__global__ void k_update_e_f32_batch(const StageJob* __restrict__ jobs, int use_f1) {
  const StageJob& J = jobs[blockIdx.z];
  const int M = J.rc.M;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  const int im = blockIdx.y % M, ir = 1 + blockIdx.y / M;
  if (ix > J.rc.nx || ir > J.rc.ny) return;
  const FieldSetF F = use_f1 ? J.F1 : J.F0;
  update_e_item(F, J.rowtab, J.cdx, J.cdy, J.cj, J.r1e, ix, im, ir);
}
__global__ void __launch_bounds__(128, B_BLOCKS_PER_SM) k_update_b_f32_batch(const StageJob* __restrict__ jobs,
                                                                            int use_f1, int save_old) {
  const StageJob& J = jobs[blockIdx.z];
  const int M = J.rc.M;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int im = blockIdx.y % M, j = blockIdx.y / M;
  if (i >= J.rc.nxg || j >= J.rc.nyg) return;
  const FieldSetF F = use_f1 ? J.F1 : J.F0;
  const RunConst rc = J.rc;
  update_b_item(F, save_old, J.rowtab, J.hdx, J.hdy, J.r1b, rc, i, im, j);
}

static void yee_e_consts(const RunConst& rc, float& cdx, float& cdy, float& cj, Row1E& r1) {
  const double c2 = CLIGHT * CLIGHT, h = 0.5 * rc.dt;
  const double r_d = std::fabs(rc.y_grid_min), r_p = r_d + 0.5 * rc.dy;
  r1 = Row1E{c2 / r_p * 0.5 * h, c2 / r_p * h, c2 / rc.dy * h, c2 / rc.dx * h, h / EPS0, c2 / r_d * h};
  cdx = (float)(c2 / rc.dx * h);
  cdy = (float)(c2 / rc.dy * h);
  cj = (float)(h / EPS0);
}
static void yee_b_consts(const RunConst& rc, float& hdx, float& hdy, Row1B& r1) {
  const double h = 0.5 * rc.dt;
  const double r_d = std::fabs(rc.y_grid_min), r_p = r_d + 0.5 * rc.dy;
  r1 = Row1B{h / r_d, 0.5 * h / r_d, h / rc.dy, h / r_p, h / rc.dx};
  hdx = (float)(h / rc.dx);
  hdy = (float)(h / rc.dy);
}

void stage_job_yee_consts(StageJob& J) {
  yee_e_consts(J.rc, J.cdx, J.cdy, J.cj, J.r1e);
  yee_b_consts(J.rc, J.hdx, J.hdy, J.r1b);
}

void launch_update_e_f32(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc) {
  float cdx, cdy, cj;
  Row1E r1;
  yee_e_consts(rc, cdx, cdy, cj, r1);
  dim3 blk(128), grd((rc.nx + 1 + 127) / 128, rc.M, rc.ny);
  k_update_e_f32<<<grd, blk, 0, s>>>(F, reinterpret_cast<const float4*>(rowtab), cdx, cdy, cj, r1, rc);
}

void launch_update_e_f32_edge_axis(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc) {
  float cdx, cdy, cj;
  Row1E r1;
  yee_e_consts(rc, cdx, cdy, cj, r1);
  const int n = (rc.nx + 2 * NG) + (rc.nx + 1) + 3 * (rc.ny - 3);
  dim3 blk(128), grd((n + 127) / 128, rc.M);
  k_update_e_edge_axis_f32<<<grd, blk, 0, s>>>(F, reinterpret_cast<const float4*>(rowtab), cdx, cdy, cj, r1,
                                               bc_const(rc, rc.dt), rc);
}

void launch_update_e_f32_fused_axis(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc) {
  float cdx, cdy, cj;
  Row1E r1;
  yee_e_consts(rc, cdx, cdy, cj, r1);
  dim3 blk(128), grd((rc.nx + 2 * NG + 127) / 128, rc.M, rc.ny - NG + 1);
  k_update_e_fused_axis_f32<<<grd, blk, 0, s>>>(F, reinterpret_cast<const float4*>(rowtab), cdx, cdy, cj, r1,
                                                bc_const(rc, rc.dt), rc);
}

void launch_update_b_f32(cudaStream_t s, const FieldSetF& F, int save_old, const double* rowtab,
                         const RunConst& rc) {
  float hdx, hdy;
  Row1B r1;
  yee_b_consts(rc, hdx, hdy, r1);
  dim3 blk(128), grd((rc.nxg + 127) / 128, rc.M, rc.nyg);
  k_update_b_f32<<<grd, blk, 0, s>>>(F, save_old, reinterpret_cast<const float4*>(rowtab), hdx, hdy, r1, rc);
}

void launch_update_b_f32_zero(cudaStream_t s, const FieldSetF& F, const double* rowtab, const RunConst& rc,
                              const FieldSetF& Fz, const ZeroCounts& zc) {
  float hdx, hdy;
  Row1B r1;
  yee_b_consts(rc, hdx, hdy, r1);
  dim3 blk(128), grd((rc.nxg + 127) / 128, rc.M, rc.nyg);
  k_update_b_f32_zero<<<grd, blk, 0, s>>>(F, reinterpret_cast<const float4*>(rowtab), hdx, hdy, r1, rc, Fz.jx,
                                          Fz.jr, Fz.jt, zc);
}

void batch_update_e_f32(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, const StageDims& d) {
  dim3 blk(128), grd((d.nx_max + 1 + 127) / 128, d.M * d.ny_max, njobs);
  k_update_e_f32_batch<<<grd, blk, 0, s>>>(jobs, use_f1);
}
void batch_update_b_f32(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, int save_old,
                        const StageDims& d) {
  dim3 blk(128), grd((d.nx_max + 2 * NG + 127) / 128, d.M * (d.ny_max + 2 * NG), njobs);
  k_update_b_f32_batch<<<grd, blk, 0, s>>>(jobs, use_f1, save_old);
}

}  // namespace cyl
