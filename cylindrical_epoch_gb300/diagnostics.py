"""Discrete charge-conservation (continuity) residual of one step.

The reference's current deposit (particles.F90:515-665) is the per-mode
Esirkepov form: for every particle the x and r current differences equal the
change of its staggered-shape charge between t + dt/2 and t + 3 dt/2, and the
theta current is q w v_theta times the path-averaged shape (particles.F90:587,
643, 659).  With rho_m the charge density of that shape (cyl_charge_density),
the residual of step n is, per mode m and cell (cx, cy),

  R = (rho_m^{n+1} - rho_m^n) / dt
      + (jx(cx+1, cy) - jx(cx, cy)) / dx
      + inv_volume(cy) (jr(cx, cy+1) / inv_area_xt(cy) - jr(cx, cy) / inv_area_xt(cy-1))
      - i m jtheta(cx, cy) / r_p(cy)

with the geometry tables of particles.F90:189-217 and r_p the radius of the
charge cell (fields.f90:76-77).  The x and r parts cancel to round-off for
every mode; the theta part is exact only in the limit of small angle steps,
so the m > 0 residual is small but not round-off.  Cells next to the x
boundaries and the axis (where current_finish and current_bcs_r_min_final
fold ghost currents) are left out.
"""
import numpy as np

from . import abi

NG = abi.NG
JNG = abi.NG


def geometry(deck):
    """inv_area_rt, inv_area_xt, inv_volume indexed by Fortran row iy as
    arrays over iy = 1-jng .. ny+jng (inv_area_xt over 0-jng .. ny+jng)."""
    dx, dy, ny = deck.dx, deck.dy, deck.ny
    y_grid_min = dy / 2.0
    r_low = y_grid_min - JNG * dy
    rt = np.zeros(ny + 2 * JNG)
    xt = np.zeros(ny + 2 * JNG + 1)
    xt[0] = 1.0 / (2.0 * np.pi * abs(r_low) * dx)
    for k, iy in enumerate(range(1 - JNG, ny + JNG + 1)):
        if round(2.0 * r_low / dy) == -1:
            rt[k] = 1.0 / (np.pi * (0.5 * dy) ** 2)
        else:
            rt[k] = 1.0 / (np.pi * abs((r_low + dy) ** 2 - r_low ** 2))
        xt[k + 1] = 1.0 / (2.0 * np.pi * abs(r_low + dy) * dx)
        r_low += dy
    return rt, xt, rt / dx


def continuity_residual(deck, rho0, rho1, jx, jr, jt, dt, margin=3):
    """Per-mode relative L2 residual ||R|| / ||(rho1 - rho0)/dt|| over the
    interior cells cx in [1+margin, nx-margin], cy in [margin, ny-margin].
    Arrays are (M, ny+2ng, nx+2ng) complex, Fortran (ix, iy) at
    [m, iy+ng-1, ix+ng-1].  Returns (list of relative residuals, list of
    absolute L2 norms of R)."""
    nx, ny, M = deck.nx, deck.ny, deck.n_mode
    _, xt, vol = geometry(deck)
    cx = np.arange(1 + margin, nx - margin + 1)
    cy = np.arange(margin, ny - margin + 1)
    X = cx + NG - 1
    Y = cy + NG - 1
    vol_c = vol[cy - (1 - JNG)][:, None]
    xt_c = xt[cy - (0 - JNG)][:, None]
    xt_m = xt[cy - 1 - (0 - JNG)][:, None]
    r_p = (np.abs((cy - 1) * deck.dy + deck.dy / 2.0) + 0.5 * deck.dy)[:, None]
    rel, ab = [], []
    for m in range(M):
        sl = np.ix_(Y, X)
        drho = (rho1[m][sl] - rho0[m][sl]) / dt
        dvx = (jx[m][np.ix_(Y, X + 1)] - jx[m][sl]) / deck.dx
        dvr = vol_c * (jr[m][np.ix_(Y + 1, X)] / xt_c - jr[m][sl] / xt_m)
        dvt = -1j * m * jt[m][sl] / r_p
        R = drho + dvx + dvr + dvt
        nR = float(np.sqrt(np.sum(np.abs(R) ** 2)))
        nD = float(np.sqrt(np.sum(np.abs(drho) ** 2)))
        rel.append(nR / nD if nD > 0 else nR)
        ab.append(nR)
    return rel, ab


def spectrum(p, mass):
    """Weighted moments of the kinetic energy (MeV) of one species."""
    mc = mass * 2.99792458e8
    u2 = (p.px ** 2 + p.py ** 2 + p.pz ** 2) / mc ** 2
    ke = mc * 2.99792458e8 * u2 / (np.sqrt(u2 + 1.0) + 1.0) / 1.602176565e-13
    w = p.w / np.sum(p.w)
    return {"mean_mev": float(np.sum(w * ke)), "rms_mev": float(np.sqrt(np.sum(w * ke ** 2))),
            "m3_mev": float(np.cbrt(np.sum(w * ke ** 3))), "max_mev": float(np.max(ke))}


def residual_step(run, deck, tries=8):
    """Continuity residual of the next step of `run` that does not shift the
    window (the charge densities must be on one grid)."""
    for _ in range(tries):
        s0 = run.state().n_shifts
        r0 = run.charge_density()
        run.step(1)
        if run.state().n_shifts != s0:
            continue
        r1 = run.charge_density()
        return continuity_residual(deck, r0, r1, run.field("jxm"), run.field("jrm"), run.field("jtm"),
                                   deck.grid_desc().dt)[0]
    return None


def compare_runs(a, b, deck, residual=True):
    """Error of run `a` against run `b` of the same deck after the same steps
    (any objects with field, particles, state, charge_density and step, e.g.
    a GPU run and the oracle): per-mode Ez relative L2, on-axis wake
    amplitude (max |Re Ez_0| on r = 0), electron kinetic-energy moments,
    particle counts and window shifts, and the continuity residual of one
    further step of each (which advances both)."""
    rel = lambda x, y: float(np.sqrt(np.sum(np.abs(x - y) ** 2) / max(np.sum(np.abs(y) ** 2), 1e-300)))
    ea, eb = a.field("exm"), b.field("exm")
    ez = [rel(ea[m], eb[m]) for m in range(deck.n_mode)]
    ax = NG - 1  # exm row ir = 0 (r = 0) is array row ng - 1
    lo, hi = abi.NG, abi.NG + deck.nx  # ix = 1 .. nx
    wa = float(np.max(np.abs(ea[0, ax, lo:hi].real)))
    wb = float(np.max(np.abs(eb[0, ax, lo:hi].real)))
    spa = spectrum(a.particles(0), deck.species[0].mass)
    spb = spectrum(b.particles(0), deck.species[0].mass)
    sa, sb = a.state(), b.state()
    out = {
        "ez_rel_l2_per_mode": ez,
        "wake_amplitude_v_per_m": {"run": wa, "against": wb, "rel_err": abs(wa - wb) / max(wb, 1e-300)},
        "electron_spectrum": {"run": spa, "against": spb,
                              "rel_err": {k: abs(spa[k] - spb[k]) / max(abs(spb[k]), 1e-300) for k in spa}},
        "n_live": {"run": int(sa.n_live[0]), "against": int(sb.n_live[0])},
        "n_shifts": {"run": int(sa.n_shifts), "against": int(sb.n_shifts)},
    }
    if residual:
        out["continuity_residual_per_mode"] = {"run": residual_step(a, deck), "against": residual_step(b, deck)}
    return out
