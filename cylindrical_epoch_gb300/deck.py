"""Deck descriptions of the runs this package is measured and tested on.

A Deck holds what the reference's Fortran driver has after it read an input
deck (control, boundaries, species, laser and window blocks) and ran set_dt:
the descriptors of include/cylpic.h plus the host-evaluated laser profile.
The builders below write the benchmark decks in the reference's deck
vocabulary; ``set_dt`` restates setup.F90:573-670.
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import abi

# constants.F90:171-181
PI = 3.141592653589793238462643383279503
Q0 = 1.602176565e-19
M0 = 9.10938291e-31
CL = 2.99792458e8
KB = 1.3806488e-23
EPS0 = 8.854187817620389850536563031710750e-12
EV = Q0
C_TINY = 2.2250738585072014e-308  # TINY(1.0_num)
C_EPS = 2.220446049250313e-16      # EPSILON(1.0_num), the density_min default
C_HUGE = 1.7976931348623157e308


@dataclass
class Species:
    name: str
    charge: float
    mass: float
    npart_per_cell: float
    density: float
    temp_k: tuple = (0.0, 0.0, 0.0)
    drift: tuple = (0.0, 0.0, 0.0)
    bc: tuple = (abi.BC_PERIODIC, abi.BC_PERIODIC, abi.BC_OTHER, abi.BC_REFLECT)
    immobile: bool = False
    density_kind: int = 0          # 0 uniform, 1 linear ramp
    ramp_x0: float = 0.0
    ramp_length: float = 1.0
    density_min: float = C_EPS
    density_max: float = C_HUGE
    capacity: int = 0

    def desc(self):
        d = abi.SpeciesDesc()
        d.charge = self.charge
        d.mass = self.mass
        d.immobile = 1 if self.immobile else 0
        for i in range(4):
            d.bc_particle[i] = self.bc[i]
        d.capacity = int(self.capacity)
        d.npart_per_cell = self.npart_per_cell
        d.density_kind = self.density_kind
        d.density = self.density
        d.ramp_x0 = self.ramp_x0
        d.ramp_length = self.ramp_length
        d.density_min = self.density_min
        d.density_max = self.density_max
        for i in range(3):
            d.temp[i] = self.temp_k[i]
            d.drift[i] = self.drift[i]
        return d

    def density_at(self, x):
        if self.density_kind == 1:
            f = (np.asarray(x, dtype=np.float64) - self.ramp_x0) / self.ramp_length
            return self.density * np.clip(f, 0.0, 1.0)
        return np.full_like(np.asarray(x, dtype=np.float64), self.density)


@dataclass
class Laser:
    boundary: int
    amp: float
    omega: float
    profile: np.ndarray            # ny+1 values at y(ir), ir = 0..ny
    phase: np.ndarray
    pol_angle: float = 0.0
    t_start: float = 0.0
    t_end: float = C_HUGE
    t_profile: int = 0             # 0 constant, 1 gauss(time, t0, tw)
    t0: float = 0.0
    tw: float = 1.0


@dataclass
class Deck:
    name: str
    nx: int
    ny: int
    n_mode: int
    x_min: float
    x_max: float
    y_max: float
    bc_field: tuple
    species: List[Species]
    lasers: List[Laser] = field(default_factory=list)
    nsteps: int = 100
    precision: int = abi.PREC_FP64
    dt_multiplier: float = 0.95
    move_window: bool = False
    window_v_x: float = 0.0
    window_start_time: float = 0.0
    window_stop_time: float = 1.0e300
    bc_after_move: Optional[tuple] = None
    smooth_currents: int = 0
    smooth_its: int = 1
    smooth_comp_its: int = 0
    smooth_stride: int = 1
    seed: int = 7842432
    dt: float = 0.0
    # Deck expressions evaluated by the driver while stepping (the parser's
    # part, cyl_deck_fns): None keeps the closed forms of the descriptors.
    #   laser_time(il, t) -> laser_time_profile; laser_omega(il, t) -> omega
    #   for the lasers in omega_fn (a set of laser indices); laser_profile /
    #   laser_phase(il, t) -> ny+1 values for the lasers in profile_fn /
    #   phase_fn; inject(isp, t, x) -> (density (ny+2,), temperature (3, ny+2),
    #   drift (3, ny+2)) at a window shift; load_grids(isp) -> (density,
    #   temperature (3, ...), drift (3, ...)) on the ghosted grid, or None.
    laser_time: Optional[object] = None
    laser_omega: Optional[object] = None
    laser_profile: Optional[object] = None
    laser_phase: Optional[object] = None
    omega_fn: frozenset = frozenset()
    profile_fn: frozenset = frozenset()
    phase_fn: frozenset = frozenset()
    inject: Optional[object] = None
    load_grids: Optional[object] = None
    # field ionisation (use_field_ionisation): per species a dict with
    # ionise, ionise_to, release (species indices, -1 none), l, n and energy
    # (J); the rate model (abi.IONISE_* bits; both = the reference's default)
    # and the counter-stream key of the ionisation trials
    ionisation: Optional[list] = None
    ionisation_model: int = abi.IONISE_MULTIPHOTON | abi.IONISE_BSI
    ionisation_seed: int = 1

    @property
    def dx(self):
        return (self.x_max - self.x_min) / float(self.nx)

    @property
    def dy(self):
        return (self.y_max - 0.0) / float(self.ny)

    def y_grid(self, ir):
        """Cell-centred radial grid y(ir) (setup.F90:196-200)."""
        ygm = (0.0 - self.dy * 0.0) + self.dy / 2.0
        return ygm + (np.asarray(ir, dtype=np.float64) - 1.0) * self.dy

    def grid_desc(self):
        g = abi.GridDesc()
        g.nx, g.ny, g.n_mode = self.nx, self.ny, self.n_mode
        g.precision = self.precision
        g.x_min, g.x_max, g.y_max = self.x_min, self.x_max, self.y_max
        g.dt = self.dt if self.dt > 0 else set_dt(self)
        for i in range(4):
            g.bc_field[i] = self.bc_field[i]
        g.move_window = 1 if self.move_window else 0
        g.window_v_x = self.window_v_x
        g.window_start_time = self.window_start_time
        g.window_stop_time = self.window_stop_time
        after = self.bc_after_move or self.bc_field
        for i in range(4):
            g.bc_after_move[i] = after[i]
        g.smooth_currents = self.smooth_currents
        g.smooth_its = self.smooth_its
        g.smooth_comp_its = self.smooth_comp_its
        g.smooth_stride = self.smooth_stride
        return g

    def species_descs(self):
        arr = (abi.SpeciesDesc * max(1, len(self.species)))()
        for i, s in enumerate(self.species):
            arr[i] = s.desc()
        return arr

    def laser_descs(self):
        """Descriptor array plus the numpy buffers it points into (keep both alive)."""
        arr = (abi.LaserDesc * max(1, len(self.lasers)))()
        keep = []
        for i, L in enumerate(self.lasers):
            prof = np.ascontiguousarray(L.profile, dtype=np.float64)
            ph = np.ascontiguousarray(L.phase, dtype=np.float64)
            keep += [prof, ph]
            d = arr[i]
            d.boundary, d.t_profile = L.boundary, L.t_profile
            d.amp, d.omega, d.pol_angle = L.amp, L.omega, L.pol_angle
            d.t_start, d.t_end, d.t0, d.tw = L.t_start, L.t_end, L.t0, L.tw
            d.profile = prof.ctypes.data_as(C.POINTER(C.c_double))
            d.phase = ph.ctypes.data_as(C.POINTER(C.c_double))
        return arr, keep

    def ionisation_descs(self):
        arr = (abi.IonisationSpecies * max(1, len(self.species)))()
        for i, d in enumerate(self.ionisation or []):
            a = arr[i]
            a.ionise = 1 if d.get("ionise") else 0
            a.ionise_to = int(d.get("ionise_to", -1))
            a.release = int(d.get("release", -1))
            a.l, a.n = int(d.get("l", 0)), int(d.get("n", 1))
            a.energy = float(d.get("energy", 0.0))
        return arr

    def has_deck_fns(self):
        return any(f is not None for f in (self.laser_time, self.laser_omega, self.laser_profile,
                                           self.laser_phase, self.inject))

    def deck_fns(self):
        """The cyl_deck_fns struct of this deck's expression hooks, plus the
        ctypes callback objects it points to (keep both alive while the run
        that holds it steps).  A Python exception in a hook is reported to
        the step as a non-zero return (CYL_ERR_CALLBACK)."""
        ny = self.ny
        keep = []

        def guard(fn):
            def wrapped(*a):
                try:
                    fn(*a)
                    return 0
                except Exception:  # reported to the step, which fails with CYL_ERR_CALLBACK
                    import traceback
                    traceback.print_exc()
                    return 1
            return wrapped

        f = abi.DeckFns()
        if self.laser_time is not None:
            def lt(user, il, t, out):
                out[0] = float(self.laser_time(int(il), t))
            f.laser_time = abi.LaserTimeFn(guard(lt))
            keep.append(f.laser_time)
        if self.laser_omega is not None:
            def lo(user, il, t, out):
                out[0] = float(self.laser_omega(int(il), t))
            f.laser_omega = abi.LaserOmegaFn(guard(lo))
            keep.append(f.laser_omega)
            f.omega_fn_mask = sum(1 << i for i in self.omega_fn)
        for name, fn, idx, mask in (("laser_profile", self.laser_profile, self.profile_fn, "profile_fn_mask"),
                                    ("laser_phase", self.laser_phase, self.phase_fn, "phase_fn_mask")):
            if fn is None:
                continue

            def la(user, il, t, out, fn=fn):
                v = np.asarray(fn(int(il), t), dtype=np.float64)
                for ir in range(ny + 1):
                    out[ir] = float(v[ir])
            cb = abi.LaserArrayFn(guard(la))
            setattr(f, name, cb)
            keep.append(cb)
            setattr(f, mask, sum(1 << i for i in idx))
        if self.inject is not None:
            def inj(user, isp, t, x, dens, temp, drift):
                d, tm, dr = self.inject(int(isp), t, x)
                d = np.asarray(d, dtype=np.float64)
                tm = np.asarray(tm, dtype=np.float64).reshape(3, ny + 2)
                dr = np.asarray(dr, dtype=np.float64).reshape(3, ny + 2)
                C.memmove(dens, d.ctypes.data, 8 * (ny + 2))
                C.memmove(temp, np.ascontiguousarray(tm).ctypes.data, 8 * 3 * (ny + 2))
                C.memmove(drift, np.ascontiguousarray(dr).ctypes.data, 8 * 3 * (ny + 2))
            f.inject = abi.InjectFn(guard(inj))
            keep.append(f.inject)
        return f, keep

    def mobile_particles_estimate(self):
        n = 0
        for s in self.species:
            if not s.immobile:
                n += int(math.floor(s.npart_per_cell)) * self.nx * self.ny
        return n


def set_dt(deck: Deck) -> float:
    """dt of set_dt (setup.F90:629-670) with set_plasma_frequency_dt
    (setup.F90:573-625) and set_laser_dt (laser.f90:368-407)."""
    dx, dy = deck.dx, deck.dy
    min_dt = 1000000.0
    k_max = 2.0 * PI / min(dx, dy)
    xg = (deck.x_min - dx * 0.0) + dx / 2.0 + (np.arange(1, deck.nx + 1) - 1.0) * dx
    for s in deck.species:
        fac1 = Q0 ** 2 / s.mass / EPS0
        fac2 = 3.0 * k_max ** 2 * KB / s.mass
        dens = s.density_at(xg)
        if s.density_max > 0:
            dens = np.minimum(dens, s.density_max)
        omega2 = fac1 * dens + fac2 * max(s.temp_k)
        omega2 = omega2[omega2 > C_TINY]
        if omega2.size:
            omega = np.sqrt(omega2)
            cand = (2.0 * PI / omega).min()
            if cand < min_dt:
                min_dt = float(cand)
    dt_plasma = min_dt / 2.0
    dt_laser = C_HUGE
    for L in deck.lasers:
        dt_laser = min(dt_laser, 2.0 * PI / L.omega)
    dt_laser = dt_laser / 2.0
    dt = 0.9 * min(dx, dy) / math.sqrt(2.0) / CL
    if dt_plasma > C_TINY:
        dt = min(dt, dt_plasma)
    if dt_laser > C_TINY:
        dt = min(dt, dt_laser)
    return deck.dt_multiplier * dt


# ---------------------------------------------------------------- decks

def thermal_plasma(nx=256, ny=64, ppc=16, n_mode=2, nsteps=200, precision=abi.PREC_FP64):
    """Uniform 1 keV thermal electron plasma, n = 1e25 m^-3, dz = dr = 50 nm,
    periodic in z, conducting outer r boundary, immobile neutralising ions
    (not loaded: they carry no current), CFL 0.95."""
    d = 0.05e-6
    t_k = 1000.0 * EV / KB  # temp_ev (deck_species_block.F90:835-844)
    e = Species("electron", -Q0, M0, ppc, 1.0e25, temp_k=(t_k, t_k, t_k),
                bc=(abi.BC_PERIODIC, abi.BC_PERIODIC, abi.BC_OTHER, abi.BC_CONDUCT))
    deck = Deck("thermal_plasma", nx, ny, n_mode, 0.0, nx * d, ny * d,
                (abi.BC_PERIODIC, abi.BC_PERIODIC, abi.BC_OTHER, abi.BC_CONDUCT),
                [e], nsteps=nsteps, precision=precision)
    e.capacity = int(ppc * nx * ny * 1.05) + 1024
    return deck


def wakefield(nx=2048, ny=256, n_mode=2, ppc=8, a0=2.0, lam=0.8e-6, waist=10.0e-6,
              t_fwhm=30.0e-15, density=1.0e24, ramp=50.0e-6, nsteps=2000,
              precision=abi.PREC_FP64, circular=False, ions=None):
    """Laser wakefield deck: Gaussian laser injected at z-min (simple_laser),
    electron plasma with a linear up-ramp, moving window at c.

    The time envelope and the window start follow the reference's own
    wakefield example deck conventions (example_decks/
    Wakefield_Lifschitz09_JCompPhys228.deck): t_profile = gauss(time, t0, wt)
    with wt = 0.60056 t_fwhm and t0 = 0.5 * 1.8226 t_fwhm; the window starts
    once the pulse has fully entered (time 2 t0) and the x boundaries become
    simple_outflow after the move."""
    dx = lam / 32.0 if nx == 2048 else lam / 32.0
    dy = lam / 8.0
    omega = 2.0 * PI * CL / lam
    amp = a0 * M0 * CL * omega / Q0
    wt = t_fwhm * 0.60056
    t0 = 0.5 * t_fwhm * 1.8226
    deck = Deck("wakefield", nx, ny, n_mode, 0.0, nx * dx, ny * dy,
                (abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN),
                [], nsteps=nsteps, precision=precision)
    yv = deck.y_grid(np.arange(0, ny + 1))
    prof = np.exp(-((yv - 0.0) / waist) ** 2)  # gauss(y, 0, waist)
    phase = np.zeros(ny + 1)
    if circular:
        deck.lasers = [
            Laser(abi.BD_X_MIN, amp / math.sqrt(2.0), omega, prof, phase, 0.0, t_profile=1, t0=t0, tw=wt),
            Laser(abi.BD_X_MIN, amp / math.sqrt(2.0), omega, prof, phase + PI / 2.0, PI / 2.0,
                  t_profile=1, t0=t0, tw=wt),
        ]
    else:
        deck.lasers = [Laser(abi.BD_X_MIN, amp, omega, prof, phase, 0.0, t_profile=1, t0=t0, tw=wt)]
    e = Species("electron", -Q0, M0, ppc, density, density_kind=1, ramp_x0=0.0, ramp_length=ramp,
                bc=(abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN))
    deck.species = [e]
    if ions is not None:
        deck.species.append(ions)
    deck.move_window = True
    deck.window_v_x = CL
    deck.window_start_time = 2.0 * t0
    deck.bc_after_move = (abi.BC_SIMPLE_OUTFLOW, abi.BC_SIMPLE_OUTFLOW, abi.BC_OTHER, abi.BC_OPEN)
    # Particle slots: the moving window injects fresh plasma at the front
    # while electrons trapped in the wake travel with the window, so a run
    # can hold more than ppc * nx * ny particles (1.10x at step 1264 on a
    # 512 x 128, a0 = 2.1 scan deck); the reference's linked lists have no
    # limit, the slots here are sized with room to spare.
    for s in deck.species:
        s.capacity = int(math.floor(s.npart_per_cell) * nx * ny * 1.5) + 4096
    return deck


def large_wakefield(precision=abi.PREC_MIXED, nsteps=3000):
    """m = 0..3, a0 = 4, circular polarisation, waist 8 um, 3e24 m^-3 electrons
    plus a mobile helium-like ion species (Z = 2, 4 amu) at 1 % of n_e,
    4096 x 512 cells, 32 electrons per cell (the ion species uses 2 per cell)."""
    ions = Species("helium2+", 2.0 * Q0, 4.0 * 1.66053886e-27, 2, 0.01 * 3.0e24, density_kind=1,
                   ramp_x0=0.0, ramp_length=50.0e-6,
                   bc=(abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN))
    return wakefield(nx=4096, ny=512, n_mode=4, ppc=32, a0=4.0, waist=8.0e-6, density=3.0e24,
                     nsteps=nsteps, precision=precision, circular=True, ions=ions)


def moving_window_deck(precision=abi.PREC_FP64):
    """The reference's own moving-window example deck
    (example_decks/moving_window.deck), with its deck expressions evaluated
    here as the Fortran parser would and passed through the deck-expression
    channel: 500 x 100 cells over 20 x 5 um, modes m = 0..1; a 1 um laser at
    1e15 W/cm^2 from x_min with a curved-wavefront phase
    2 pi / lambda0 y^2 / (2 RC) - gouy and profile gauss(y, 0, w_bnd); a
    window at 2e8 m/s from 30 to 100 fs with simple_outflow x boundaries
    after the move; one neutral species of mass 2000 m_e at 0.5 K with
    npart = 2 nx ny (2 per cell: every cell is valid) and the x-dependent
    density 0.5 + sin(x / 4 um)^2, used by the loader on the ghosted grid and
    by insert_particles at every window shift."""
    nx, ny = 500, 100
    micron = 1.0e-6
    lambda0 = 1.0 * micron
    w_0 = 0.9 * micron
    x_spot = 15.0 * micron
    x_r = PI * w_0 ** 2 / lambda0
    rc = x_spot * (1.0 + (x_r / x_spot) ** 2)
    w_bnd = w_0 * math.sqrt(1.0 + (x_spot / x_r) ** 2)
    gouy = math.atan(x_spot / x_r)
    deck = Deck("moving_window", nx, ny, 2, 0.0, 20.0e-6, 5.0e-6,
                (abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN), [], precision=precision)
    yv = deck.y_grid(np.arange(0, ny + 1))
    amp = math.sqrt(1.0e15 / (CL * EPS0 / 2.0)) * 100.0  # intensity_w_cm2 (deck_laser_block.f90:136-139)
    omega = 2.0 * PI * CL / lambda0
    deck.lasers = [Laser(abi.BD_X_MIN, amp, omega, np.exp(-((yv - 0.0) / w_bnd) ** 2),
                         2.0 * PI / lambda0 * yv ** 2 / (2.0 * rc) - gouy)]
    t_k = 0.5
    n = Species("Neutron", 0.0, 2000.0 * M0, 2.0, 1.0, temp_k=(t_k, t_k, t_k),
                bc=(abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN))
    n.capacity = int(2 * nx * ny * 1.3) + 4096
    deck.species = [n]
    deck.move_window = True
    deck.window_v_x = 2.0e8
    deck.window_start_time = 30.0e-15
    deck.window_stop_time = 100.0e-15
    deck.bc_after_move = (abi.BC_SIMPLE_OUTFLOW, abi.BC_SIMPLE_OUTFLOW, abi.BC_OTHER, abi.BC_OPEN)
    deck.nsteps = int(math.ceil(200.0e-15 / set_dt(deck)))

    def density(x):
        return 0.5 + np.sin(np.asarray(x, dtype=np.float64) / 4.0e-6) ** 2

    def load_grids(isp):
        ng = abi.NG
        ix = np.arange(1 - ng, nx + ng + 1)
        xg = (deck.x_min + deck.dx / 2.0) + (ix - 1.0) * deck.dx  # x(ix), setup.F90:189-195
        dens = np.repeat(density(xg)[None, :], ny + 2 * ng, axis=0)
        temp = np.full((3, ny + 2 * ng, nx + 2 * ng), t_k)
        return dens, temp, np.zeros_like(temp)

    def inject(isp, time, x):
        return (np.full(ny + 2, float(density(x))), np.full((3, ny + 2), t_k), np.zeros((3, ny + 2)))

    deck.load_grids = load_grids
    deck.inject = inject
    return deck


def field_ionisation_deck(precision=abi.PREC_FP64, model=None):
    """The reference's field-ionisation example deck
    (example_decks/field_ionisation.deck): 125 x 200 cells over 4 x 6.4 um,
    modes m = 0..2; a 0.8 um laser at 3e15 W/cm^2 from x_min, constant in
    time and radius; a neutral carbon slab (atomic_no 6, mass 12 x 1836.2 m_e,
    temperature 0) of 2.91e20 m^-3 for r < 125 nm and 3.05 < x < 3.3 um,
    npart = 1000 (250 nm / x_max) nx (125 nm / y_max) ny, ionisable up to C3+
    (ionise_limit 3) with one electron species per level
    (unique_electron_species).  The ionisation data of carbon are the
    reference's tables (TABLES/ionisation_energies.table, ion_l.table,
    ion_n.table, row 6): 11.2602880, 24.383154, 47.88778 eV; l = 1, 1, 0;
    n = 2, 2, 2.  Species: 0 Carbon, 1-3 Carbon1..3, 4-6 the electrons of
    each level."""
    nx, ny = 125, 200
    x_max, y_max = 4.0e-6, 6.4e-6
    deck = Deck("field_ionisation", nx, ny, 3, 0.0, x_max, y_max,
                (abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN), [], precision=precision)
    lam = 0.8e-6
    omega = 2.0 * PI * CL / lam
    amp = math.sqrt(3.0e15 / (CL * EPS0 / 2.0)) * 100.0  # intensity_w_cm2 (deck_laser_block.f90:136-139)
    deck.lasers = [Laser(abi.BD_X_MIN, amp, omega, np.ones(ny + 1), np.zeros(ny + 1))]
    bc = (abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN)
    mass_c = 12.0 * 1836.2 * M0
    npart = 1000 * (250.0e-9 / x_max) * nx * (125.0e-9 / y_max) * ny
    ng = abi.NG
    ix = np.arange(1 - ng, nx + ng + 1)
    iy = np.arange(1 - ng, ny + ng + 1)
    dx, dy = x_max / nx, y_max / ny
    xg = (dx / 2.0) + (ix - 1.0) * dx
    yg = (dy / 2.0) + (iy - 1.0) * dy
    dens = np.where(yg[:, None] < 125e-9, 2.91e20, 0.0) * np.ones((1, ix.size))
    dens = np.where((xg[None, :] > 3.05e-6) & (xg[None, :] < 3.3e-6), dens, 0.0)
    valid = int(np.count_nonzero(dens[ng:ng + ny, ng:ng + nx] >= C_EPS))
    ppc = float(int(npart)) / valid  # npart spread over the valid cells (helper.F90:522-523)
    species = [Species("Carbon", 0.0, mass_c, ppc, 2.91e20, bc=bc)]
    for k in (1, 2, 3):
        species.append(Species(f"Carbon{k}", k * Q0, mass_c - k * M0, ppc, 0.0, bc=bc))
    for k in (1, 2, 3):
        species.append(Species(f"Carbon{k}_electron", -Q0, M0, ppc, 0.0, bc=bc))
    n_load = int(npart) + 1024
    for s in species:
        s.capacity = n_load
    deck.species = species
    zero = np.zeros((ny + 2 * ng, nx + 2 * ng))
    deck.load_grids = lambda isp: (dens if isp == 0 else zero, None, None)
    ev = [11.2602880, 24.383154, 47.88778]
    ls = [1, 1, 0]
    deck.ionisation = [dict(ionise=1, ionise_to=1 + k, release=4 + k, l=ls[k], n=2, energy=ev[k] * Q0)
                       for k in range(3)] + [dict(ionise=0)] * 4
    if model is not None:
        deck.ionisation_model = model
    return deck
