// fields.cu -- per-mode r-z Yee update, r = 0 axis rules and field/current
// boundary kernels of the quasi-3D step.
//
// Bulk updates (update_e_field / update_b_field bulk loops,
// fields.f90:67-108, 203-241) are grid-wide elementwise kernels over
// (ix, ir, m), coalesced along x.  The O(perimeter) work -- axis rules
// (fields.f90:116-180, 249-310), efield_bcs / bfield_bcs / bfield_final_bcs
// (boundary.F90:1355-1537), the x boundary laser and outflow and the r_max
// outflow (laser.f90:411-690), current_bcs_r_min_final (boundary.F90:
// 1909-1959) -- runs as a sequence of multi-CTA launches, one per phase whose
// work items are independent, in the reference's order (the phases depend on
// each other at the domain corners).  current_finish (current_smooth.F90:
// 29-45), which is cheap and only active for periodic or reflecting
// particle boundaries, stays one single-CTA kernel.
#include <algorithm>
#include <cstddef>

#include <type_traits>

#include "cyl_common.cuh"
#include "cyl_kernels.cuh"
#include "axis_rules.cuh"

namespace cyl {

// ----------------------------------------------------------------- bulk

__global__ void k_update_e(FView ex, FView er, FView et, FView bx, FView br, FView bt,
                           FView jx, FView jr, FView jt, RunConst rc) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx
  const int ir = 1 + blockIdx.y;                         // 1..ny
  const int im = blockIdx.z;
  if (ix > rc.nx) return;
  const double dx = rc.dx, dy = rc.dy, dt = rc.dt, c2 = CLIGHT * CLIGHT;
  const double r_d = fabs((double)(ir - 1) * dy + rc.y_grid_min);
  const double r_p = r_d + 0.5 * dy;
  const double fac_x = c2 / r_p;
  const cplx im_fac_x = (IMAGI * (double)im) * fac_x;
  const cplx im_fac_r = ((IMAGI * (double)im) * c2) / r_d;
  const cplx bt0 = bt(ix, ir, im), bt1 = bt(ix, ir + 1, im), btx = bt(ix + 1, ir, im);
  const cplx br0 = br(ix, ir, im), brx = br(ix + 1, ir, im);
  const cplx bx0 = bx(ix, ir, im), bx1 = bx(ix, ir + 1, im);
  ex(ix, ir, im) = ex(ix, ir, im) +
      ((((fac_x * 0.5) * (bt1 + bt0) + im_fac_x * br0) + (c2 * (bt1 - bt0)) / dy) -
       jx(ix, ir, im) / EPS0) * 0.5 * dt;
  er(ix, ir, im) = er(ix, ir, im) +
      ((-(im_fac_r * bx0) - (c2 * (btx - bt0)) / dx) - jr(ix, ir, im) / EPS0) * 0.5 * dt;
  et(ix, ir, im) = et(ix, ir, im) +
      (((c2 * (brx - br0)) / dx - (c2 * (bx1 - bx0)) / dy) - jt(ix, ir, im) / EPS0) * 0.5 * dt;
}

// B update over the whole ghosted array: optionally saves B into B_old
// (fields.f90:326-328), then updates ix = 0..nx, ir = 1..ny-1 (y_max_boundary).
__global__ void k_update_b(FView ex, FView er, FView et, FView bx, FView br, FView bt,
                           FView bxo, FView bro, FView bto, int save_old, RunConst rc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nxg-1
  const int j = blockIdx.y;                             // 0..nyg-1
  const int im = blockIdx.z;
  if (i >= rc.nxg) return;
  const int ix = i + 1 - NG, ir = j + 1 - NG;
  if (save_old) {
    bxo(ix, ir, im) = bx(ix, ir, im);
    bro(ix, ir, im) = br(ix, ir, im);
    bto(ix, ir, im) = bt(ix, ir, im);
  }
  if (ix < 0 || ix > rc.nx || ir < 1 || ir > rc.ny - 1) return;
  const double dx = rc.dx, dy = rc.dy, dt = rc.dt;
  const double r_d = fabs((double)(ir - 1) * dy + rc.y_grid_min);
  const double r_p = r_d + 0.5 * dy;
  const cplx im_fac_x = (IMAGI * (double)im) / r_d;
  const cplx im_fac_r = (IMAGI * (double)im) / r_p;
  const cplx et0 = et(ix, ir, im), etm1 = et(ix, ir - 1, im), etxm = et(ix - 1, ir, im);
  const cplx er0 = er(ix, ir, im), erxm = er(ix - 1, ir, im);
  const cplx ex0 = ex(ix, ir, im), exm1 = ex(ix, ir - 1, im);
  bx(ix, ir, im) = bx(ix, ir, im) -
      ((im_fac_x * er0 + (0.5 * (et0 + etm1)) / r_d) + (et0 - etm1) / dy) * 0.5 * dt;
  br(ix, ir, im) = br(ix, ir, im) + (im_fac_r * ex0 + (et0 - etxm) / dx) * 0.5 * dt;
  bt(ix, ir, im) = bt(ix, ir, im) + (-((er0 - erxm) / dx) + (ex0 - exm1) / dy) * 0.5 * dt;
}

// ----------------------------------------------------- halo (one CTA)

constexpr int CTA_THREADS = 512;
#define CTA_FOR(var, n) for (int var = threadIdx.x; var < (n); var += blockDim.x)

// halo_x: periodic-x self wrap of rows [j0, j1] (boundary.F90:500-593 on one rank)
template <typename T>
__device__ void halo_x(FViewT<T> f, int j0, int j1, const int* bcf, const RunConst& rc) {
  const int nrow = j1 - j0 + 1;
  if (bcf[CYL_BD_X_MAX] == CYL_BC_PERIODIC) {
    CTA_FOR(t, nrow * rc.M * NG) {
      int i = 1 + t % NG, r = t / NG;
      int j = j0 + r % nrow, m = r / nrow;
      f(rc.nx + i, j, m) = f(i, j, m);
    }
  }
  __syncthreads();
  if (bcf[CYL_BD_X_MIN] == CYL_BC_PERIODIC) {
    CTA_FOR(t, nrow * rc.M * NG) {
      int i = 1 - NG + t % NG, r = t / NG;
      int j = j0 + r % nrow, m = r / nrow;
      f(i, j, m) = f(rc.nx + i, j, m);
    }
  }
  __syncthreads();
}

// ---------------------------------------------------- ghost-cell phases
//
// efield_bcs (boundary.F90:1355-1413) and bfield_bcs (boundary.F90:1417-1476)
// are, in the reference's order, five phases:
//   PH_HALO       periodic self-wrap in x (boundary.F90:500-593 on one rank)
//   PH_CONDUCT_X  conducting x boundaries      PH_CONDUCT_Y  conducting r_max
//   PH_OTHER_X    clamp / laser / outflow / zero-gradient x boundaries
//   PH_OTHER_Y    the same at r_max
// with the ghost mirrors of field_mode_clamp_zero (boundary.F90:772-829) and
// field_mode_zero_gradient (boundary.F90:654-707).  They run as one launch
// (k_ghost_all below, which composes the phases cell by cell).  Copies and
// sign flips act on the storage type, so they are exact in both forms.
enum GhostPhase { PH_HALO = 0, PH_CONDUCT_X = 1, PH_CONDUCT_Y = 2, PH_OTHER_X = 3, PH_OTHER_Y = 4 };
enum GhostKind { GK_NONE = 0, GK_CLAMP = 1, GK_ZERO_GRADIENT = 2 };

template <typename T>
__device__ __forceinline__ void gset(FViewT<T> f, int ix, int iy, int m, int kind, int sx, int sy) {
  T v = *f.ptr(sx, sy, m);
  if (kind == GK_CLAMP) {
    v.re = -v.re;
    v.im = -v.im;
  }
  *f.ptr(ix, iy, m) = v;
}
template <typename T>
__device__ __forceinline__ void gzero(FViewT<T> f, int ix, int iy, int m) {
  T v;
  v.re = 0;
  v.im = 0;
  *f.ptr(ix, iy, m) = v;
}

// Kind of ghost rule for field st (0..5 = ex er et bx br bt) on boundary bd
// in phase ph, from the mapped field bc codes.
__device__ __forceinline__ int ghost_kind(int ph, int st, int bd, const int32_t* bcf) {
  const int b = bcf[bd];
  if (b == CYL_BC_PERIODIC) return GK_NONE;
  if (ph == PH_CONDUCT_X || ph == PH_CONDUCT_Y) {
    if (b != CYL_BC_CONDUCT) return GK_NONE;
    // x: ex clamp, er et zero-gradient; bx zero-gradient, br bt clamp.
    // r_max: ex et zero-gradient, er clamp; bx bt clamp, br zero-gradient.
    static constexpr int kx[6] = {GK_CLAMP, GK_ZERO_GRADIENT, GK_ZERO_GRADIENT, GK_ZERO_GRADIENT, GK_CLAMP, GK_CLAMP};
    static constexpr int ky[6] = {GK_ZERO_GRADIENT, GK_CLAMP, GK_ZERO_GRADIENT, GK_CLAMP, GK_ZERO_GRADIENT, GK_CLAMP};
    return ph == PH_CONDUCT_X ? kx[st] : ky[st];
  }
  if (b == CYL_BC_CLAMP || b == CYL_BC_SIMPLE_LASER || b == CYL_BC_SIMPLE_OUTFLOW) return GK_CLAMP;
  if (b == CYL_BC_ZERO_GRADIENT) return GK_ZERO_GRADIENT;
  return GK_NONE;
}

template <typename T>
struct Triplet {
  FViewT<T> f[3];
};

// All phases of one efield_bcs / bfield_bcs call in one launch.  Every
// boundary has one rule per field: none, a zero, or a copy (with a sign) of
// a cell of the same row (x boundaries) or column (r_max).  The x rules
// write ghost columns (and column 0 or nx), the r_max rules rows ny..ny+NG.
// A cell in both sets (a corner) takes the copy of the cell at the x rule's
// source column and the r rule's source row, with both signs, or zero if
// either rule zeroes it: the x-then-r order of the phases gives the same
// value (the rules are separable), and so does the opposite order.  No
// rule's source cell is another rule's target, so one launch reads every
// source before any write that could concern it.
enum GhostOp { GO_NONE = 0, GO_ZERO = 1, GO_COPY = 2 };
struct GhostRule {
  int op, src;  // src: source column (x rules) or row (r_max rules)
  bool neg;
};
// The x rule of field st at the side's i-th target (i = 1..NG) in row j, and
// its target column.
__device__ __forceinline__ GhostRule ghost_x_rule(int st, int side, int i, int j, bool halo_only,
                                                  const int32_t* bcp, const RunConst& rc, int& col) {
  const int nx = rc.nx, ny = rc.ny;
  const int bd = side == 0 ? CYL_BD_X_MIN : CYL_BD_X_MAX;
  const GhostRule none{GO_NONE, 0, false};
  if (bcp[bd] == CYL_BC_PERIODIC) {
    // halo exchange: rows 1-ng .. ny+ng, one fewer for r-staggered arrays
    col = side == 0 ? i - NG : nx + i;
    if (!(rc.bc_mask & BCM_PERIODIC_X) || j > ny + NG - (stag_y(st) ? 1 : 0)) return none;
    return GhostRule{GO_COPY, side == 0 ? nx + i - NG : i, false};
  }
  const bool stag = stag_x(st);
  col = stag && i == NG ? (side == 0 ? 0 : nx) : (side == 0 ? i - NG : nx + i);
  if (halo_only) return none;
  const int ph = bcp[bd] == CYL_BC_CONDUCT ? PH_CONDUCT_X : PH_OTHER_X;
  if (!(rc.bc_mask & (ph == PH_CONDUCT_X ? BCM_CONDUCT : BCM_OTHER))) return none;
  const int kind = ghost_kind(ph, st, bd, bcp);
  if (kind == GK_NONE) return none;
  if (stag && i == NG) return kind == GK_CLAMP ? GhostRule{GO_ZERO, 0, false} : none;
  const int src = side == 0 ? (stag ? NG - i : NG + 1 - i) : (stag ? nx - i : nx + 1 - i);
  return GhostRule{GO_COPY, src, kind == GK_CLAMP};
}
// The r_max rule of field st at its i-th target (i = 1..NG), and its target
// row.
__device__ __forceinline__ GhostRule ghost_y_rule(int st, int i, bool halo_only, const int32_t* bcp,
                                                  const RunConst& rc, int& row) {
  const int ny = rc.ny;
  const GhostRule none{GO_NONE, 0, false};
  const bool stag = stag_y(st);
  row = stag && i == NG ? ny : ny + i;
  if (halo_only) return none;
  const int ph = bcp[CYL_BD_Y_MAX] == CYL_BC_CONDUCT ? PH_CONDUCT_Y : PH_OTHER_Y;
  if (!(rc.bc_mask & (ph == PH_CONDUCT_Y ? BCM_CONDUCT : BCM_OTHER))) return none;
  const int kind = ghost_kind(ph, st, CYL_BD_Y_MAX, bcp);
  if (kind == GK_NONE) return none;
  if (stag && i == NG) return kind == GK_CLAMP ? GhostRule{GO_ZERO, 0, false} : none;
  return GhostRule{GO_COPY, stag ? ny - i : ny + 1 - i, kind == GK_CLAMP};
}
// The r_max rule that targets row j (i = 0: none).
__device__ __forceinline__ int ghost_y_index(int st, int j, const RunConst& rc) {
  const int ny = rc.ny;
  if (stag_y(st)) return j == ny ? NG : (j > ny && j < ny + NG) ? j - ny : 0;
  return (j > ny && j <= ny + NG) ? j - ny : 0;
}
template <typename T>
__device__ __forceinline__ void ghost_apply(FViewT<T> f, int col, int row, int m, const GhostRule& rx,
                                            const GhostRule& ry) {
  if (rx.op == GO_ZERO || ry.op == GO_ZERO) return gzero(f, col, row, m);
  const int sc = rx.op == GO_COPY ? rx.src : col, sr = ry.op == GO_COPY ? ry.src : row;
  gset(f, col, row, m, (rx.neg != ry.neg) ? GK_CLAMP : GK_ZERO_GRADIENT, sc, sr);
}
// Items: the x targets (i = 1..NG fastest, row j, m, q, side), which take
// the corners, then the r_max targets (column fastest, i, m, q) outside the
// x target columns.
template <typename T>
__device__ __forceinline__ void ghost_all_item(const Triplet<T>& tr, int st0, bool halo_only, const int32_t* bcp,
                                               const RunConst& rc, int64_t t) {
  const int nx = rc.nx, ny = rc.ny, M = rc.M;
  const int nrow = ny + 2 * NG, ncol = nx + 2 * NG;
  const int64_t nxi = (int64_t)2 * 3 * M * nrow * NG;
  if (t < nxi) {
    const int i = 1 + (int)(t % NG);
    int r = (int)(t / NG);
    const int j = 1 - NG + r % nrow;
    r /= nrow;
    const int m = r % M;
    r /= M;
    const int q = r % 3, side = r / 3;
    const int st = st0 + q;
    int col, row;
    const GhostRule rx = ghost_x_rule(st, side, i, j, halo_only, bcp, rc, col);
    const int iy = ghost_y_index(st, j, rc);
    const GhostRule ry = iy ? ghost_y_rule(st, iy, halo_only, bcp, rc, row) : GhostRule{GO_NONE, 0, false};
    if (rx.op == GO_NONE && ry.op == GO_NONE) return;
    // a column that is an x target in some row belongs to these items
    if (rx.op == GO_NONE) {
      int c2;
      if (ghost_x_rule(st, side, i, 1, halo_only, bcp, rc, c2).op == GO_NONE) return;
    }
    ghost_apply(tr.f[q], col, j, m, rx, ry);
    return;
  }
  t -= nxi;
  if (t >= (int64_t)ncol * NG * M * 3) return;
  const int ix = 1 - NG + (int)(t % ncol);
  int r = (int)(t / ncol);
  const int i = 1 + r % NG;
  r /= NG;
  const int m = r % M, q = r / M;
  const int st = st0 + q;
  int row;
  const GhostRule ry = ghost_y_rule(st, i, halo_only, bcp, rc, row);
  if (ry.op == GO_NONE) return;
  if (ix <= 0 || ix >= nx) {
    // columns that an x rule targets (in any row) are written by the x items
    for (int side = 0; side < 2; ++side)
      for (int k = 1; k <= NG; ++k) {
        int c;
        if (ghost_x_rule(st, side, k, 1, halo_only, bcp, rc, c).op != GO_NONE && c == ix) return;
      }
  }
  ghost_apply(tr.f[q], ix, row, m, GhostRule{GO_NONE, 0, false}, ry);
}
template <typename T>
__global__ void k_ghost_all(Triplet<T> tr, int st0, int halo_only, const int32_t* bcp, RunConst rc) {
  ghost_all_item<T>(tr, st0, halo_only != 0, bcp, rc, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// Device address of a step record's field bc codes (no host dereference).
__host__ __device__ static const int32_t* bc_ptr(const StepRec* rec) {
  return reinterpret_cast<const int32_t*>(reinterpret_cast<const char*>(rec) + offsetof(StepRec, bc_field));
}

// Launch the phases of efield_bcs / bfield_bcs (halo_only: bfield_bcs(.TRUE.),
// the halo exchange alone) that this run's bc kinds can need.
// Returns the number of kernels launched (0 or 1); so do the launchers below.
template <typename T>
static int launch_ghost_bcs(cudaStream_t s, FViewT<T> a, FViewT<T> b, FViewT<T> c, int st0, bool halo_only,
                            const int32_t* bcp, const RunConst& rc) {
  const Triplet<T> tr{{a, b, c}};
  if (halo_only && !(rc.bc_mask & BCM_PERIODIC_X)) return 0;
  if (!(rc.bc_mask & (BCM_PERIODIC_X | BCM_CONDUCT | BCM_OTHER))) return 0;
  const int64_t items = (int64_t)2 * 3 * rc.M * (rc.ny + 2 * NG) * NG + (int64_t)(rc.nx + 2 * NG) * NG * rc.M * 3;
  k_ghost_all<T><<<(unsigned)((items + 255) / 256), 256, 0, s>>>(tr, st0, halo_only ? 1 : 0, bcp, rc);
  return 1;
}
// Laser source and Mur outflow at the x boundaries (outflow_bcs_x_min /
// outflow_bcs_x_max, laser.f90:411-633), one thread per (side, ir, m).  src
// holds this step's Cartesian laser sources (source1, source2 for x_min then
// x_max, each ny+1 values), which the host evaluates from the deck's time and
// transverse profiles.  cols: the boundary column arrays, 12 arrays
// [ex,er,et,bx,br,bt]_x_min then _x_max, each (1-ng:ny+ng, M).  Every read
// is of a column other than the ones written (columns 0, 1 at x_min and nx
// at x_max; nx >= 8).
template <typename T>
__device__ __forceinline__ void laser_x_item(const FieldSetT<T>& F, const StepRec* rec, const double* src,
                                             const cplx* cols, double dt, const BcConst& K, const RunConst& rc,
                                             int t) {
  const int nx = rc.nx, ny = rc.ny, M = rc.M;
  if (t >= 2 * (ny + 1) * M) return;
  const int side = t / ((ny + 1) * M);
  const int ir = t % (ny + 1), m = (t / (ny + 1)) % M;
  const int bd = side == 0 ? CYL_BD_X_MIN : CYL_BD_X_MAX;
  if (!(rec->add_laser[bd] || rec->bc_field[bd] == CYL_BC_SIMPLE_OUTFLOW)) return;
  const double c2 = CLIGHT * CLIGHT;
  const double lr = K.lr, sum = K.sum, diff = K.diff, dt_eps = K.dt_eps;
  const int ncolv = ny + 2 * NG;
  const size_t cs = (size_t)ncolv * M;
  const cplx* erb = cols + (size_t)(side * 6 + 1) * cs;
  const cplx* etb = cols + (size_t)(side * 6 + 2) * cs;
  const cplx* bxb = cols + (size_t)(side * 6 + 3) * cs;
  const cplx* brb = cols + (size_t)(side * 6 + 4) * cs;
  const cplx* btb = cols + (size_t)(side * 6 + 5) * cs;
  const size_t cj = (size_t)(ir + NG - 1) + (size_t)ncolv * m;
  F.bx(side == 0 ? 0 : nx, ir, m) = bxb[cj];
  if (ir == 0) return;
  const double* s1 = src + (size_t)side * 2 * (ny + 1);
  const double* s2 = s1 + (ny + 1);
  const cplx imc = ((IMAGI * (double)m) * c2) * dt;
  // Bt row: ir pairs with r_d_vals(ir-1) (whole array inside a 1:ny section)
  const double rdv = fabs((double)(ir - 2) * rc.dy + rc.y_grid_min);
  const double inv_rdv = 1.0 / rdv;  // used by the mixed form only
  cplx nbt;
  if (side == 0) {
    cplx st = mk(0.0, 0.0);
    if (m == 1) st = s1[ir] + IMAGI * s2[ir];
    nbt = sum * (((((4.0 * st + 2.0 * (erb[cj] + CLIGHT * btb[cj])) - 2.0 * F.er(1, ir, m)) +
                   div_form<T>(imc * F.bx(1, ir, m), rdv, inv_rdv)) +
                  dt_eps * F.jr(1, ir, m)) +
                 diff * F.bt(2, ir, m));
  } else {
    // source_t whole array (0:ny) inside the 1:ny section: index ir-1
    cplx st = mk(0.0, 0.0);
    if (m == 1) st = s1[ir - 1] + IMAGI * s2[ir - 1];
    nbt = sum * ((((((-4.0) * st - 2.0 * (erb[cj] + CLIGHT * btb[cj])) + 2.0 * F.er(nx - 1, ir, m)) -
                   div_form<T>(imc * F.bx(nx - 1, ir, m), rdv, inv_rdv)) -
                  dt_eps * F.jr(nx - 1, ir, m)) +
                 diff * F.bt(nx - 1, ir, m));
  }
  cplx nbr = mk(0.0, 0.0);
  const bool do_br = ir <= ny - 1;
  if (do_br) {
    cplx sr = mk(0.0, 0.0);
    if (m == 1) sr = (-IMAGI) * s1[ir] + s2[ir];
    if (side == 0) {
      nbr = sum * (((((((-4.0) * sr - 2.0 * (etb[cj] + CLIGHT * brb[cj])) + 2.0 * F.et(1, ir, m)) -
                      lr * (F.bx(1, ir + 1, m) - F.bx(1, ir, m))) -
                     dt_eps * F.jt(1, ir, m)) +
                    diff * F.br(2, ir, m)));
    } else {
      nbr = sum * (((((4.0 * sr + 2.0 * (etb[cj] + CLIGHT * brb[cj])) - 2.0 * F.et(nx - 1, ir, m)) +
                     lr * (F.bx(nx - 1, ir + 1, m) - F.bx(nx - 1, ir, m))) +
                    dt_eps * F.jt(nx - 1, ir, m)) +
                   diff * F.br(nx - 1, ir, m));
    }
  }
  if (side == 0) {
    F.bt(1, ir, m) = nbt;
    if (do_br) F.br(1, ir, m) = nbr;
  } else {
    F.bt(nx, ir, m) = nbt;
    if (do_br) F.br(nx, ir, m) = nbr;
  }
}
template <typename T>
__global__ void k_laser_x(FieldSetT<T> F, const StepRec* rec, const double* src, const cplx* cols, double dt,
                          BcConst K, RunConst rc) {
  laser_x_item<T>(F, rec, src, cols, dt, K, rc, blockIdx.x * blockDim.x + threadIdx.x);
}

// outflow_bcs_r_max (laser.f90:637-690) or zero_b (boundary.F90:1528-1531),
// one thread per (ix, m).  The new Bx, Bt of row ny depend on row ny-1, row
// ny of the other arrays and the B_old / J_old arrays only.
template <typename T>
__device__ __forceinline__ void rmax_b_item(const FieldSetT<T>& F, const StepRec* rec, double dt, const BcConst& K,
                                            const RunConst& rc, int t) {
  const int nx = rc.nx, ny = rc.ny, M = rc.M;
  const int b = rec->bc_field[CYL_BD_Y_MAX];
  if (b == CYL_BC_ZERO_B) {
    if (t >= (nx + 2 * NG) * M) return;
    const int ix = 1 - NG + t % (nx + 2 * NG), m = t / (nx + 2 * NG);
    F.bx(ix, ny, m) = mk(0, 0);
    F.br(ix, ny, m) = mk(0, 0);
    F.bt(ix, ny, m) = mk(0, 0);
    return;
  }
  if (b != CYL_BC_SIMPLE_OUTFLOW || t >= nx * M) return;
  const int ix = 1 + t % nx, m = t / nx;
  const double lx = K.rx_lx, inv_r = K.rx_inv_r, dtc2_4r = K.rx_dtc2_4r, ly = K.rx_ly;
  const double sum_x = K.rx_sum_x, sum_t = K.rx_sum_t, dt_2eps = K.rx_dt_2eps;
  const cplx icm = K.rx_icdt_2r * (double)m;
  if (ix <= nx - 1) {
    cplx v = (-F.bx(ix, ny - 1, m)) * (CLIGHT - ly);
    v = v - F.bxo(ix, ny, m) * ((-CLIGHT) + ly);
    v = v - F.bxo(ix, ny - 1, m) * ((-CLIGHT) - ly);
    v = v - ((CLIGHT * dt) * inv_r) * F.et(ix, ny - 1, m);
    v = v + (0.5 * lx) * (((F.br(ix + 1, ny - 1, m) - F.br(ix, ny - 1, m)) + F.bro(ix + 1, ny - 1, m)) -
                          F.bro(ix, ny - 1, m));
    v = v - icm * (F.er(ix, ny, m) + F.er(ix, ny - 1, m));
    v = v - dt_2eps * (F.jt(ix, ny - 1, m) + F.jto(ix, ny - 1, m));
    F.bx(ix, ny, m) = sum_x * v;
  }
  cplx v = (-F.bt(ix, ny - 1, m)) * ((CLIGHT - ly) + dtc2_4r);
  v = v - F.bto(ix, ny, m) * (((-CLIGHT) + ly) + dtc2_4r);
  v = v - F.bto(ix, ny - 1, m) * (((-CLIGHT) - ly) + dtc2_4r);
  v = v - K.rx_lx_c * (((F.er(ix, ny, m) + F.er(ix, ny - 1, m)) - F.er(ix - 1, ny, m)) -
                                   F.er(ix - 1, ny - 1, m));
  v = v - (icm * CLIGHT) * (F.br(ix, ny - 1, m) + F.bro(ix, ny - 1, m));
  v = v + dt_2eps * (F.jx(ix, ny - 1, m) + F.jxo(ix, ny - 1, m));
  F.bt(ix, ny, m) = sum_t * v;
}
template <typename T>
__global__ void k_rmax_b(FieldSetT<T> F, const StepRec* rec, double dt, BcConst K, RunConst rc) {
  rmax_b_item<T>(F, rec, dt, K, rc, blockIdx.x * blockDim.x + threadIdx.x);
}
// ------------------------------------------------------------- currents

// particle_reflection_bcs_complex (boundary.F90:918-1015) for one side
__device__ void reflect_side(FView f, int flip, int bd, const RunConst& rc) {
  const int nx = rc.nx, ny = rc.ny, M = rc.M;
  const cplx Z = mk(0, 0);
  if (bd == CYL_BD_X_MIN || bd == CYL_BD_X_MAX) {
    const int nrow = ny + 2 * NG;
    CTA_FOR(t, nrow * M) {
      int j = 1 - NG + t % nrow, m = t / nrow;
      if (bd == CYL_BD_X_MIN) {
        if (flip == 1) {
          for (int i = 1; i <= NG - 1; ++i) { f(i, j, m) = f(i, j, m) - f(1 - i, j, m); f(1 - i, j, m) = Z; }
        } else {
          for (int i = 1; i <= NG - 1; ++i) { f(i, j, m) = f(i, j, m) + f(-i, j, m); f(-i, j, m) = Z; }
        }
      } else {
        if (flip == 1) {
          for (int i = 1; i <= NG; ++i) { f(nx + 1 - i, j, m) = f(nx + 1 - i, j, m) - f(nx + i, j, m); f(nx + i, j, m) = Z; }
        } else {
          for (int i = 1; i <= NG; ++i) { f(nx - i, j, m) = f(nx - i, j, m) + f(nx + i, j, m); f(nx + i, j, m) = Z; }
        }
      }
    }
  } else {
    const int ncol = nx + 2 * NG;
    const double r_max = rc.y_grid_min + ((double)ny - 0.5) * rc.dy;
    CTA_FOR(t, ncol * M) {
      int ix = 1 - NG + t % ncol, m = t / ncol;
      for (int i = 1; i <= NG; ++i) {
        if (flip == 2) {
          f(ix, ny + 1 - i, m) = f(ix, ny + 1 - i, m) -
              (f(ix, ny + i, m) * (r_max + ((double)i - 0.5) * rc.dy)) / (r_max - ((double)i - 0.5) * rc.dy);
        } else if (flip == 1) {
          f(ix, ny - i, m) = f(ix, ny - i, m) +
              (f(ix, ny + i, m) * (r_max + (double)i * rc.dy)) / (r_max - (double)i * rc.dy);
        } else {
          f(ix, ny - i, m) = f(ix, ny - i, m) + f(ix, ny + i, m);
        }
        f(ix, ny + i, m) = Z;
      }
    }
  }
}

// current_bcs_r_min_final (boundary.F90:1909-1959) for one (column, mode):
// fold the r < 0 ghost rows of J into rows 1 .. jng-1 with the mode-parity
// signs, then set the axis row.  The ghost and target rows are read before
// any is written, so their loads overlap.
__device__ __forceinline__ void j_rmin_item(FView jx, FView jr, FView jt, int ix, int im) {
  const double mode_sign = (im & 1) ? -1.0 : 1.0;
  const cplx Z = mk(0, 0);
  cplx gx[JNG - 1], gr[JNG - 1], gt[JNG - 1], tx[JNG - 1], tr[JNG - 1], tt[JNG - 1];
#pragma unroll
  for (int j = 2; j <= JNG; ++j) {
    gx[j - 2] = jx(ix, 1 - j, im);
    gr[j - 2] = jr(ix, 1 - j, im);
    gt[j - 2] = jt(ix, 1 - j, im);
    tx[j - 2] = jx(ix, j - 1, im);
    tr[j - 2] = jr(ix, j, im);
    tt[j - 2] = jt(ix, j - 1, im);
  }
  const cplx r0 = jr(ix, 0, im), r1 = jr(ix, 1, im);
#pragma unroll
  for (int j = 2; j <= JNG; ++j) {
    tx[j - 2] = tx[j - 2] + mode_sign * gx[j - 2];
    tr[j - 2] = tr[j - 2] - mode_sign * gr[j - 2];
    tt[j - 2] = tt[j - 2] - mode_sign * gt[j - 2];
    jx(ix, j - 1, im) = tx[j - 2];
    jr(ix, j, im) = tr[j - 2];
    jt(ix, j - 1, im) = tt[j - 2];
    jx(ix, 1 - j, im) = Z;
    jr(ix, 1 - j, im) = Z;
    jt(ix, 1 - j, im) = Z;
  }
  const cplx r1n = r1 - mode_sign * r0;
  jr(ix, 1, im) = r1n;
  // rows 1 and 2 after the fold: jx(1) = tx[0], jx(2) = tx[1], jr(2) = tr[0]
  if (im > 0) jx(ix, 0, im) = Z;
  else jx(ix, 0, im) = (4.0 * tx[0] - tx[1]) / 3.0;
  if (im == 1) {
    const cplx t0 = ((-IMAGI) * (9.0 * r1n - tr[0])) / 8.0;
    jt(ix, 0, im) = t0;
    jr(ix, 0, im) = (2.0 * IMAGI) * t0 - r1n;
  } else {
    jt(ix, 0, im) = Z;
    jr(ix, 0, im) = -r1n;
  }
}

// particle_periodic_bcs_complex on one rank (boundary.F90:1133-1245)
__device__ void periodic_sum_dev(FView f, const RunConst& rc) {
  if (rc.bc_allspecies[CYL_BD_X_MIN] != CYL_BC_PERIODIC) return;
  const int nrow = rc.ny + 2 * NG;
  const int nx = rc.nx;
  CTA_FOR(t, nrow * rc.M * NG) {
    int i = 1 + t % NG, r = t / NG;
    int j = 1 - NG + r % nrow, m = r / nrow;
    f(i, j, m) = f(i, j, m) + f(nx + i, j, m);
  }
  __syncthreads();
  CTA_FOR(t, nrow * rc.M * NG) {
    int i = 1 + t % NG, r = t / NG;
    int j = 1 - NG + r % nrow, m = r / nrow;
    f(nx - NG + i, j, m) = f(nx - NG + i, j, m) + f(i - NG, j, m);
  }
}

// current_bcs_r_min_final, then current_finish (current_smooth.F90:29-45)
// without smoothing (one CTA).
__device__ __forceinline__ void current_finish_cta(FView jx, FView jr, FView jt, const StepRec* rec,
                                                   const RunConst& rc) {
  __shared__ int bcf[4];
  if (threadIdx.x < 4) bcf[threadIdx.x] = rec->bc_field[threadIdx.x];
  __syncthreads();
  const int bds[3] = {CYL_BD_X_MIN, CYL_BD_X_MAX, CYL_BD_Y_MAX};
  for (int k = 0; k < 3; ++k) {
    if (rc.bc_allspecies[bds[k]] == CYL_BC_REFLECT) {
      reflect_side(jx, 1, bds[k], rc);
      reflect_side(jr, 2, bds[k], rc);
      reflect_side(jt, 3, bds[k], rc);
    }
    __syncthreads();
  }
  periodic_sum_dev(jx, rc);
  periodic_sum_dev(jr, rc);
  periodic_sum_dev(jt, rc);
  __syncthreads();
  halo_x(jx, 1 - NG, rc.ny + NG, bcf, rc);
  halo_x(jr, 1 - NG, rc.ny + NG, bcf, rc);
  halo_x(jt, 1 - NG, rc.ny + NG, bcf, rc);
}
__global__ void __launch_bounds__(CTA_THREADS) k_current_finish(FView jx, FView jr, FView jt, const StepRec* rec, RunConst rc) {
  current_finish_cta(jx, jr, jt, rec, rc);
}
// The folding and halo pass has work only with a reflecting or periodic
// particle boundary or a periodic x field boundary (before or after the
// window starts); all of these are fixed for the run.
__host__ __device__ static bool finish_needed(const RunConst& rc) {
  const bool reflect = rc.bc_allspecies[CYL_BD_X_MIN] == CYL_BC_REFLECT ||
                       rc.bc_allspecies[CYL_BD_X_MAX] == CYL_BC_REFLECT ||
                       rc.bc_allspecies[CYL_BD_Y_MAX] == CYL_BC_REFLECT;
  const bool periodic = rc.bc_allspecies[CYL_BD_X_MIN] == CYL_BC_PERIODIC || (rc.bc_mask & BCM_PERIODIC_X);
  return reflect || periodic;
}

// One pass of smooth_mode_array (current_smooth.F90:172-190): the halo of wk
// is done by k_halo_rows before this; reads wk, writes f (interior).
__global__ void k_smooth_pass(FView f, FView wk, double alpha, double beta, int cs, RunConst rc) {
  const int ix = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int iy = 1 + blockIdx.y;
  const int im = blockIdx.z;
  if (ix > rc.nx) return;
  f(ix, iy, im) = alpha * wk(ix, iy, im) +
      (((wk(ix - cs, iy, im) + wk(ix + cs, iy, im)) + wk(ix, iy - cs, im)) + wk(ix, iy + cs, im)) * beta;
}
__global__ void k_copy_interior(FView dst, FView src, RunConst rc) {
  const int ix = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int iy = 1 + blockIdx.y;
  const int im = blockIdx.z;
  if (ix > rc.nx) return;
  dst(ix, iy, im) = src(ix, iy, im);
}
__global__ void __launch_bounds__(CTA_THREADS) k_halo_rows(FView f, const StepRec* rec, RunConst rc) {
  __shared__ int bcf[4];
  if (threadIdx.x < 4) bcf[threadIdx.x] = rec->bc_field[threadIdx.x];
  __syncthreads();
  halo_x(f, 1 - NG, rc.ny + NG, bcf, rc);
}

// -------------------------------------------------------- moving window

// shift_fields (window.F90:98-132): one block per (row j, mode m).  The
// in-place left shift f(i) = f(i+1) runs in chunks of blockDim.x elements
// from the left: a chunk reads its sources into registers before any of its
// writes, and the next chunk reads only beyond what this one wrote, so no
// row staging is needed whatever the row length.  The periodic self-wrap of
// shift_field_modes and the x_max column fix-ups act within the same row.
template <typename U>
__device__ void shift_row(FViewT<U> f, int j, int m, const int* bcf, const RunConst& rc) {
  const int nxg = rc.nxg, nx = rc.nx;
  __syncthreads();
  for (int c = 0; c < nxg - 1; c += blockDim.x) {
    const int i = c + threadIdx.x;
    U v;
    if (i < nxg - 1) v = *f.ptr(1 - NG + i + 1, j, m);
    __syncthreads();
    if (i < nxg - 1) *f.ptr(1 - NG + i, j, m) = v;
    __syncthreads();
  }
  // periodic self-wrap (field_mode_bc) within this row
  if (bcf[CYL_BD_X_MAX] == CYL_BC_PERIODIC)
    for (int i = 1 + (int)threadIdx.x; i <= NG; i += (int)blockDim.x) f(nx + i, j, m) = f(i, j, m);
  __syncthreads();
  if (bcf[CYL_BD_X_MIN] == CYL_BC_PERIODIC)
    for (int i = 1 - NG + (int)threadIdx.x; i <= 0; i += (int)blockDim.x) f(i, j, m) = f(nx + i, j, m);
}

// The same shift with the row held in registers: each thread loads all of
// its elements of the row (strided by the block, at most SHIFT_VPT) before
// one barrier, then stores each one place to the left (new(i) = old(i + 1)
// for i < nxg - 1; the last element keeps its value), so a row costs one
// load round trip instead of one per chunk.  Pure data movement: the FP64
// form's values are unchanged.
constexpr int SHIFT_THREADS = 512;
constexpr int SHIFT_VPT_MAX = 16;  // rows of up to 8192 cells

template <int VPT, typename U>
__device__ void shift_row_regs(FViewT<U> f, int j, int m, const int* bcf, const RunConst& rc) {
  const int nxg = rc.nxg, nx = rc.nx;
  U v[VPT];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    const int i = k * SHIFT_THREADS + (int)threadIdx.x;
    if (i >= 1 && i < nxg) v[k] = *f.ptr(1 - NG + i, j, m);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    const int i = k * SHIFT_THREADS + (int)threadIdx.x;
    if (i >= 1 && i < nxg) *f.ptr(1 - NG + i - 1, j, m) = v[k];
  }
  __syncthreads();
  if (bcf[CYL_BD_X_MAX] == CYL_BC_PERIODIC)
    for (int i = 1 + (int)threadIdx.x; i <= NG; i += (int)blockDim.x) f(nx + i, j, m) = f(i, j, m);
  __syncthreads();
  if (bcf[CYL_BD_X_MIN] == CYL_BC_PERIODIC)
    for (int i = 1 - NG + (int)threadIdx.x; i <= 0; i += (int)blockDim.x) f(i, j, m) = f(nx + i, j, m);
}

// VPT: elements per thread of the register path (0: the chunked path).
// One CTA per row j and mode m.
template <typename T, int VPT>
__device__ __forceinline__ void shift_fields_row(const FieldSetT<T>& F, const cplx* cols, const StepRec* rec,
                                                 int which, const RunConst& rc, int j, int m) {
  const int nx = rc.nx;
  __shared__ int bcf[4];
  if (threadIdx.x < 4) bcf[threadIdx.x] = rec->bc_field_after[threadIdx.x];
  if (rec->nshift <= which) return;
  if constexpr (VPT > 0) {
    shift_row_regs<VPT>(F.ex, j, m, bcf, rc);
    shift_row_regs<VPT>(F.er, j, m, bcf, rc);
    shift_row_regs<VPT>(F.et, j, m, bcf, rc);
    shift_row_regs<VPT>(F.bx, j, m, bcf, rc);
    shift_row_regs<VPT>(F.br, j, m, bcf, rc);
    shift_row_regs<VPT>(F.bt, j, m, bcf, rc);
    shift_row_regs<VPT>(F.jx, j, m, bcf, rc);
    shift_row_regs<VPT>(F.jr, j, m, bcf, rc);
    shift_row_regs<VPT>(F.jt, j, m, bcf, rc);
  } else {
    shift_row(F.ex, j, m, bcf, rc);
    shift_row(F.er, j, m, bcf, rc);
    shift_row(F.et, j, m, bcf, rc);
    shift_row(F.bx, j, m, bcf, rc);
    shift_row(F.br, j, m, bcf, rc);
    shift_row(F.bt, j, m, bcf, rc);
    shift_row(F.jx, j, m, bcf, rc);
    shift_row(F.jr, j, m, bcf, rc);
    shift_row(F.jt, j, m, bcf, rc);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int ncolv = rc.ny + 2 * NG;
    auto cv = [&](int a) { return cols[(size_t)(6 + a) * ncolv * rc.M + (j + NG - 1) + (size_t)ncolv * m]; };
    F.ex(nx + 1, j, m) = cv(0);
    F.er(nx, j, m) = cv(1);
    F.et(nx, j, m) = cv(2);
    F.ex(nx, j, m) = 0.5 * (F.ex(nx - 1, j, m) + F.ex(nx + 1, j, m));
    F.er(nx - 1, j, m) = 0.5 * (F.er(nx - 2, j, m) + F.er(nx, j, m));
    F.et(nx - 1, j, m) = 0.5 * (F.et(nx - 2, j, m) + F.et(nx, j, m));
    F.bx(nx, j, m) = cv(3);
    F.br(nx + 1, j, m) = cv(4);
    F.bt(nx + 1, j, m) = cv(5);
    F.bx(nx - 1, j, m) = 0.5 * (F.bx(nx - 2, j, m) + F.bx(nx, j, m));
    F.br(nx, j, m) = 0.5 * (F.br(nx - 1, j, m) + F.br(nx + 1, j, m));
    F.bt(nx, j, m) = 0.5 * (F.bt(nx - 1, j, m) + F.bt(nx + 1, j, m));
  }
}
template <typename T, int VPT>
__global__ void k_shift_fields(FieldSetT<T> F, const cplx* cols, const StepRec* rec, int which, RunConst rc) {
  shift_fields_row<T, VPT>(F, cols, rec, which, rc, 1 - NG + (int)blockIdx.x, blockIdx.y);
}

// Axis rules and J folding: one thread per independent work item.
template <typename T>
__global__ void k_e_axis(FViewT<T> ex, FViewT<T> er, FViewT<T> et, FView jx, FViewT<T> bt, BcConst K, RunConst rc) {
  const int ncol = rc.nx + 2 * NG;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * rc.M * NG) return;
  const int ix = 1 - NG + t % ncol, r = t / ncol;
  e_axis_item(ex, er, et, jx, bt, rc, K, ix, r % rc.M, r / rc.M);
}
template <typename T>
__global__ void k_b_axis(FViewT<T> bx, FViewT<T> br, FViewT<T> bt, FViewT<T> ex, FViewT<T> et, BcConst K,
                         RunConst rc) {
  const int ncol = rc.nx + 2 * NG;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * rc.M * NG) return;
  const int ix = 1 - NG + t % ncol, r = t / ncol;
  b_axis_item(bx, br, bt, ex, et, rc, K, ix, r % rc.M, r / rc.M);
}
__global__ void k_j_rmin(FView jx, FView jr, FView jt, RunConst rc) {
  const int ncol = rc.nx + 2 * NG;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * rc.M) return;
  j_rmin_item(jx, jr, jt, 1 - NG + t % ncol, t / ncol);
}
static int axis_blocks(const RunConst& rc) { return ((rc.nx + 2 * NG) * rc.M * NG + 127) / 128; }
static int jrmin_blocks(const RunConst& rc) { return ((rc.nx + 2 * NG) * rc.M + 127) / 128; }

// ------------------------------------------------------------ launchers

void launch_update_e(cudaStream_t s, const FieldSet& F, const RunConst& rc) {
  dim3 blk(128), grd((rc.nx + 1 + 127) / 128, rc.ny, rc.M);
  k_update_e<<<grd, blk, 0, s>>>(F.ex, F.er, F.et, F.bx, F.br, F.bt, F.jx, F.jr, F.jt, rc);
}
void launch_update_b(cudaStream_t s, const FieldSet& F, int save_old, const RunConst& rc) {
  dim3 blk(128), grd((rc.nxg + 127) / 128, rc.nyg, rc.M);
  k_update_b<<<grd, blk, 0, s>>>(F.ex, F.er, F.et, F.bx, F.br, F.bt, F.bxo, F.bro, F.bto, save_old, rc);
}
template <typename T>
int launch_e_axis_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc) {
  k_e_axis<T><<<axis_blocks(rc), 128, 0, s>>>(F.ex, F.er, F.et, F.jx, F.bt, bc_const(rc, rc.dt), rc);
  return 1 + launch_ghost_bcs<T>(s, F.ex, F.er, F.et, 0, false, bc_ptr(rec), rc);
}
template <typename T>
int launch_efield_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc) {
  return launch_ghost_bcs<T>(s, F.ex, F.er, F.et, 0, false, bc_ptr(rec), rc);
}
// old_field_bcs (boundary.F90:1480-1501): the halo exchange of B_old, Br_old
// over rows 1-ng .. ny+ng-1.
template <typename T>
int launch_old_field_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc) {
  return launch_ghost_bcs<T>(s, F.bxo, F.bro, F.bto, 3, true, bc_ptr(rec), rc);
}
template <typename T>
int launch_b_axis_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc) {
  k_b_axis<T><<<axis_blocks(rc), 128, 0, s>>>(F.bx, F.br, F.bt, F.ex, F.et, bc_const(rc, rc.dt), rc);
  return 1 + launch_ghost_bcs<T>(s, F.bx, F.br, F.bt, 3, true, bc_ptr(rec), rc);
}
// update_b_field axis rules, then bfield_final_bcs (boundary.F90:1505-1537):
// bfield_bcs, the x boundary laser / outflow, the r_max outflow or zero_b,
// and the closing halo exchange (bfield_bcs(.TRUE.)).
template <typename T>
int launch_b_final_bcs(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const double* src,
                       const cplx* cols, int do_axis, double dt, const RunConst& rc) {
  const BcConst K = bc_const(rc, dt);
  if (do_axis) k_b_axis<T><<<axis_blocks(rc), 128, 0, s>>>(F.bx, F.br, F.bt, F.ex, F.et, bc_const(rc, rc.dt), rc);
  int n = (do_axis ? 1 : 0) + launch_ghost_bcs<T>(s, F.bx, F.br, F.bt, 3, false, bc_ptr(rec), rc);
  k_laser_x<T><<<(2 * (rc.ny + 1) * rc.M + 127) / 128, 128, 0, s>>>(F, rec, src, cols, dt, K, rc);
  k_rmax_b<T><<<((rc.nx + 2 * NG) * rc.M + 127) / 128, 128, 0, s>>>(F, rec, dt, K, rc);
  return n + 2 + launch_ghost_bcs<T>(s, F.bx, F.br, F.bt, 3, true, bc_ptr(rec), rc);
}
template <typename T>
// parts: bit 0 the r_min fold (current_bcs_r_min_final, the end of
// push_particles), bits 1 and 2 current_finish (the folding and halo pass,
// the smoothing): field ionisation runs between the fold and current_finish
// (epoch2d.F90:218-252).
int launch_current_finish(cudaStream_t s, const FieldSetT<T>& F, const StepRec* rec, const RunConst& rc,
                          int smooth, int its, int comp_its, int stride, FView wk, int parts) {
  int n = 0;
  if (parts & 1) {
    k_j_rmin<<<jrmin_blocks(rc), 128, 0, s>>>(F.jx, F.jr, F.jt, rc);
    ++n;
  }
  if ((parts & 2) && finish_needed(rc)) {
    k_current_finish<<<1, CTA_THREADS, 0, s>>>(F.jx, F.jr, F.jt, rec, rc);
    ++n;
  }
  if (!(parts & 4) || !smooth) return n;
  FView js[3] = {F.jx, F.jr, F.jt};
  dim3 blk(128), grd((rc.nx + 127) / 128, rc.ny, rc.M);
  const size_t bytes = (size_t)rc.nxg * rc.nyg * rc.M * sizeof(cplx);
  for (int a = 0; a < 3; ++a) {
    cudaMemcpyAsync(wk.p, js[a].p, bytes, cudaMemcpyDeviceToDevice, s);
    double alpha = 0.5, beta = (1.0 - alpha) * 0.25;
    for (int it = 1; it <= its + comp_its; ++it) {
      k_halo_rows<<<1, CTA_THREADS, 0, s>>>(wk, rec, rc);
      k_smooth_pass<<<grd, blk, 0, s>>>(js[a], wk, alpha, beta, stride, rc);
      k_copy_interior<<<grd, blk, 0, s>>>(wk, js[a], rc);
      if (it > its) alpha = (double)its * 0.5 + 1.0;
    }
    k_copy_interior<<<grd, blk, 0, s>>>(js[a], wk, rc);
    n += 3 * (its + comp_its) + 1;
  }
  return n;
}
template <typename T>
void launch_shift_fields(cudaStream_t s, const FieldSetT<T>& F, const cplx* cols, const StepRec* rec,
                         int which, const RunConst& rc) {
  dim3 grd(rc.nyg, rc.M);
  const int vpt = (rc.nxg + SHIFT_THREADS - 1) / SHIFT_THREADS;
  if (vpt <= 4) k_shift_fields<T, 4><<<grd, SHIFT_THREADS, 0, s>>>(F, cols, rec, which, rc);
  else if (vpt <= 6) k_shift_fields<T, 6><<<grd, SHIFT_THREADS, 0, s>>>(F, cols, rec, which, rc);
  else if (vpt <= 9) k_shift_fields<T, 9><<<grd, SHIFT_THREADS, 0, s>>>(F, cols, rec, which, rc);
  else if (vpt <= SHIFT_VPT_MAX) k_shift_fields<T, SHIFT_VPT_MAX><<<grd, SHIFT_THREADS, 0, s>>>(F, cols, rec, which, rc);
  else k_shift_fields<T, 0><<<grd, 256, 0, s>>>(F, cols, rec, which, rc);
}

__global__ void k_zero_step(FView jx, FView jr, FView jt, int64_t n, ZeroCounts zc) {
  if (blockIdx.x == 0 && (int)threadIdx.x < zc.n) *zc.p[threadIdx.x] = 0;
  const cplx z = mk(0, 0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    jx.p[i] = z;
    jr.p[i] = z;
    jt.p[i] = z;
  }
}
template <typename T>
void launch_zero_step(cudaStream_t s, const FieldSetT<T>& F, const RunConst& rc, const ZeroCounts& zc) {
  const int64_t n = (int64_t)rc.nxg * rc.nyg * rc.M;
  const int nb = (int)std::min<int64_t>((n + 255) / 256, 1216);
  k_zero_step<<<nb, 256, 0, s>>>(F.jx, F.jr, F.jt, n, zc);
}

// ------------------------------------- batched stages of the mixed form
//
// One launch per stage for every run of a batch: blockIdx.y (blockIdx.z for
// the shift) is the run's StageJob, the rest of the grid covers the largest
// run, and each run's items are the single-run kernel's (the same item
// functions, so a run's arithmetic is the one it gets alone).

void stage_job_bc_consts(StageJob& J) { J.K = bc_const(J.rc, J.rc.dt); }

// which: 0 the E triplet, 1 the B triplet of the job's field set
__global__ void k_ghost_all_batch(const StageJob* __restrict__ jobs, int which, int use_f1, int st0, int halo_only) {
  const StageJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  const FieldSetF& Fr = use_f1 ? J.F1 : J.F0;
  const Triplet<cplxf> tr = which == 0 ? Triplet<cplxf>{{Fr.ex, Fr.er, Fr.et}} : Triplet<cplxf>{{Fr.bx, Fr.br, Fr.bt}};
  ghost_all_item<cplxf>(tr, st0, halo_only != 0, bc_ptr(J.rec), rc, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_e_axis_batch(const StageJob* __restrict__ jobs, int use_f1) {
  const StageJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  const int ncol = rc.nx + 2 * NG;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * rc.M * NG) return;
  const FieldSetF& F = use_f1 ? J.F1 : J.F0;
  const int ix = 1 - NG + t % ncol, r = t / ncol;
  e_axis_item(F.ex, F.er, F.et, F.jx, F.bt, rc, J.K, ix, r % rc.M, r / rc.M);
}
__global__ void k_b_axis_batch(const StageJob* __restrict__ jobs, int use_f1) {
  const StageJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  const int ncol = rc.nx + 2 * NG;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * rc.M * NG) return;
  const FieldSetF& F = use_f1 ? J.F1 : J.F0;
  const int ix = 1 - NG + t % ncol, r = t / ncol;
  b_axis_item(F.bx, F.br, F.bt, F.ex, F.et, rc, J.K, ix, r % rc.M, r / rc.M);
}
__global__ void k_laser_x_batch(const StageJob* __restrict__ jobs) {
  const StageJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  laser_x_item<cplxf>(J.F1, J.rec, J.src, J.cols, rc.dt, J.K, rc, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_rmax_b_batch(const StageJob* __restrict__ jobs) {
  const StageJob& J = jobs[blockIdx.y];
  const RunConst rc = J.rc;
  rmax_b_item<cplxf>(J.F1, J.rec, rc.dt, J.K, rc, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_j_rmin_batch(const StageJob* __restrict__ jobs) {
  const StageJob& J = jobs[blockIdx.y];
  const int ncol = J.rc.nx + 2 * NG;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * J.rc.M) return;
  j_rmin_item(J.F1.jx, J.F1.jr, J.F1.jt, 1 - NG + t % ncol, t / ncol);
}
__global__ void k_zero_j_batch(const StageJob* __restrict__ jobs) {
  const StageJob& J = jobs[blockIdx.y];
  const int64_t n = (int64_t)J.rc.nxg * J.rc.nyg * J.rc.M;
  cplx* const a = J.F1.jx.p;
  cplx* const b = J.F1.jr.p;
  cplx* const c = J.F1.jt.p;
  const cplx z = mk(0, 0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    a[i] = z;
    b[i] = z;
    c[i] = z;
  }
}
template <int VPT>
__global__ void k_shift_fields_batch(const StageJob* __restrict__ jobs, int which) {
  const StageJob& J = jobs[blockIdx.z];
  const RunConst rc = J.rc;
  if ((int)blockIdx.x >= rc.nyg) return;  // the whole CTA
  shift_fields_row<cplxf, VPT>(J.F1, J.cols, J.rec, which, rc, 1 - NG + (int)blockIdx.x, blockIdx.y);
}

// current_finish's folding and halo pass: one CTA per run (runs without it
// leave at once)
__global__ void __launch_bounds__(CTA_THREADS) k_current_finish_batch(const StageJob* __restrict__ jobs) {
  const StageJob& J = jobs[blockIdx.x];
  const RunConst rc = J.rc;
  if (!finish_needed(rc)) return;  // the whole CTA
  current_finish_cta(J.F1.jx, J.F1.jr, J.F1.jt, J.rec, rc);
}

// All ghost phases of one call for every run of the batch in one launch (as
// launch_ghost_bcs; each run's own bc codes and mask decide its rules).
static void batch_ghost(cudaStream_t s, const StageJob* jobs, int njobs, int which, int use_f1, int st0,
                        bool halo_only, int mask_any, const StageDims& d) {
  if (halo_only && !(mask_any & BCM_PERIODIC_X)) return;
  if (!(mask_any & (BCM_PERIODIC_X | BCM_CONDUCT | BCM_OTHER))) return;
  const int64_t items =
      (int64_t)2 * 3 * d.M * (d.ny_max + 2 * NG) * NG + (int64_t)(d.nx_max + 2 * NG) * NG * d.M * 3;
  k_ghost_all_batch<<<dim3((unsigned)((items + 255) / 256), njobs), 256, 0, s>>>(jobs, which, use_f1, st0,
                                                                             halo_only ? 1 : 0);
}
static dim3 batch_axis_grid(int njobs, const StageDims& d) {
  return dim3(((d.nx_max + 2 * NG) * d.M * NG + 127) / 128, njobs);
}
void batch_e_axis_bcs(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, int bc_mask_any,
                      const StageDims& d) {
  k_e_axis_batch<<<batch_axis_grid(njobs, d), 128, 0, s>>>(jobs, use_f1);
  batch_ghost(s, jobs, njobs, 0, use_f1, 0, false, bc_mask_any, d);
}
void batch_b_axis_bcs(cudaStream_t s, const StageJob* jobs, int njobs, int use_f1, int bc_mask_any,
                      const StageDims& d) {
  k_b_axis_batch<<<batch_axis_grid(njobs, d), 128, 0, s>>>(jobs, use_f1);
  batch_ghost(s, jobs, njobs, 1, use_f1, 3, true, bc_mask_any, d);
}
void batch_b_final_bcs(cudaStream_t s, const StageJob* jobs, int njobs, int bc_mask_any, const StageDims& d) {
  k_b_axis_batch<<<batch_axis_grid(njobs, d), 128, 0, s>>>(jobs, 1);
  batch_ghost(s, jobs, njobs, 1, 1, 3, false, bc_mask_any, d);
  k_laser_x_batch<<<dim3((2 * (d.ny_max + 1) * d.M + 127) / 128, njobs), 128, 0, s>>>(jobs);
  k_rmax_b_batch<<<dim3(((d.nx_max + 2 * NG) * d.M + 127) / 128, njobs), 128, 0, s>>>(jobs);
  batch_ghost(s, jobs, njobs, 1, 1, 3, true, bc_mask_any, d);
}
void batch_j_rmin(cudaStream_t s, const StageJob* jobs, int njobs, const StageDims& d) {
  k_j_rmin_batch<<<dim3(((d.nx_max + 2 * NG) * d.M + 127) / 128, njobs), 128, 0, s>>>(jobs);
}
void batch_current_finish(cudaStream_t s, const StageJob* jobs, int njobs) {
  k_current_finish_batch<<<njobs, CTA_THREADS, 0, s>>>(jobs);
}
bool stage_finish_needed(const RunConst& rc) { return finish_needed(rc); }
void batch_zero_j(cudaStream_t s, const StageJob* jobs, int njobs, const StageDims& d) {
  const int64_t n = (int64_t)(d.nx_max + 2 * NG) * (d.ny_max + 2 * NG) * d.M;
  const int nb = (int)std::min<int64_t>((n + 255) / 256, 256);
  k_zero_j_batch<<<dim3(nb, njobs), 256, 0, s>>>(jobs);
}
void batch_shift_fields(cudaStream_t s, const StageJob* jobs, int njobs, int which, const StageDims& d) {
  const dim3 grd(d.ny_max + 2 * NG, d.M, njobs);
  const int vpt = (d.nx_max + 2 * NG + SHIFT_THREADS - 1) / SHIFT_THREADS;
  if (vpt <= 4) k_shift_fields_batch<4><<<grd, SHIFT_THREADS, 0, s>>>(jobs, which);
  else if (vpt <= 6) k_shift_fields_batch<6><<<grd, SHIFT_THREADS, 0, s>>>(jobs, which);
  else if (vpt <= 9) k_shift_fields_batch<9><<<grd, SHIFT_THREADS, 0, s>>>(jobs, which);
  else if (vpt <= SHIFT_VPT_MAX) k_shift_fields_batch<SHIFT_VPT_MAX><<<grd, SHIFT_THREADS, 0, s>>>(jobs, which);
  else k_shift_fields_batch<0><<<grd, 256, 0, s>>>(jobs, which);
}

#define INST(T)                                                                                          \
  template int launch_e_axis_bcs<T>(cudaStream_t, const FieldSetT<T>&, const StepRec*, const RunConst&);  \
  template int launch_efield_bcs<T>(cudaStream_t, const FieldSetT<T>&, const StepRec*, const RunConst&);  \
  template int launch_old_field_bcs<T>(cudaStream_t, const FieldSetT<T>&, const StepRec*, const RunConst&); \
  template int launch_b_axis_bcs<T>(cudaStream_t, const FieldSetT<T>&, const StepRec*, const RunConst&);  \
  template int launch_b_final_bcs<T>(cudaStream_t, const FieldSetT<T>&, const StepRec*, const double*,    \
                                      const cplx*, int, double, const RunConst&);                          \
  template int launch_current_finish<T>(cudaStream_t, const FieldSetT<T>&, const StepRec*, const RunConst&, \
                                         int, int, int, int, FView, int);                                  \
  template void launch_shift_fields<T>(cudaStream_t, const FieldSetT<T>&, const cplx*, const StepRec*, int,  \
                                       const RunConst&);                                                  \
  template void launch_zero_step<T>(cudaStream_t, const FieldSetT<T>&, const RunConst&, const ZeroCounts&);
INST(cplx)
INST(cplxf)
#undef INST

}  // namespace cyl
