"""ctypes wrapper of the CPU FP64 oracle (oracle/cyl_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py, as the test oracle.  The product never loads
it.  Parity status: the reference itself (Fortran + MPI) cannot be built
here; the oracle is pinned by the analytic current of the reference's
documentation (section 7.2), by discrete charge conservation and by the
Yee vacuum dispersion relation (tests/test_oracle_pins.py).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cyl_oracle.cpp")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

_lib = None


def build(force=False):
    """Compile the oracle with -O2 -ffp-contract=off (no FMA contraction, as
    the reference's default gfortran build on x86 and the product's FP64
    kernels)."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "..", "include", "cylpic.h"),
            os.path.join(HERE, "..", "include", "cyl_math.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-fopenmp", "-o", tmp, SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    from cylindrical_epoch_gb300 import abi  # descriptor structs only
    lib = C.CDLL(LIB)
    PD = C.POINTER(C.c_double)
    PI64 = C.POINTER(C.c_int64)
    PI32 = C.POINTER(C.c_int32)
    H = C.c_void_p
    sig = {
        "orc_create": (C.c_int, [C.POINTER(abi.GridDesc), C.POINTER(abi.SpeciesDesc), C.c_int32,
                                 C.POINTER(abi.LaserDesc), C.c_int32, C.c_int32, C.POINTER(H)]),
        "orc_destroy": (C.c_int, [H]),
        "orc_load_species": (C.c_int, [H, C.c_int32]),
        "orc_load_species_counter": (C.c_int, [H, C.c_int32, C.c_uint64, C.c_int64]),
        "orc_set_injection_stream": (C.c_int, [H, C.c_int32, C.c_uint64]),
        "orc_counter_block": (C.c_int, [C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "orc_set_particles": (C.c_int, [H, C.c_int32, PD, PD, PD, PD, PD, PD, PD, PI64, C.c_int64]),
        "orc_count": (C.c_int64, [H, C.c_int32]),
        "orc_get_particles": (C.c_int, [H, C.c_int32, PD, PD, PD, PD, PD, PD, PD, PI64]),
        "orc_set_field": (C.c_int, [H, C.c_int32, PD]),
        "orc_get_field": (C.c_int, [H, C.c_int32, PD]),
        "orc_get_rng": (C.c_int, [H, C.POINTER(abi.RngState)]),
        "orc_set_rng": (C.c_int, [H, C.POINTER(abi.RngState)]),
        "orc_initialise": (C.c_int, [H]),
        "orc_step": (C.c_int, [H, C.c_int32]),
        "orc_step_to_output": (C.c_int, [H, C.c_int32]),
        "orc_finish_step": (C.c_int, [H]),
        "orc_restart": (C.c_int, [H, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_double]),
        "orc_stage": (C.c_int, [H, C.c_int32]),
        "orc_get_run_state": (C.c_int, [H, C.POINTER(abi.RunState)]),
        "orc_diagnostics": (C.c_int, [H, C.POINTER(abi.Diag)]),
        "orc_cell_indices": (C.c_int, [H, C.c_int32, PI32, PI32]),
        "orc_charge_density": (C.c_int, [H, PD]),
        "orc_number_density": (C.c_int, [H, C.c_int32, PD]),
        "orc_atan2": (C.c_double, [C.c_double, C.c_double]),
        "orc_atan2_many": (None, [C.c_int64, PD, PD, PD]),
        "orc_set_deck_fns": (C.c_int, [H, C.POINTER(abi.DeckFns)]),
        "orc_set_ionisation": (C.c_int, [H, C.POINTER(abi.IonisationSpecies), C.c_int32, C.c_int32, C.c_uint64]),
        "orc_ionisation_constants": (C.c_int, [H, PD]),
        "orc_load_species_grid": (C.c_int, [H, C.c_int32, PD, PD, PD]),
        "orc_set_atan2": (None, [C.c_int32]),
        "orc_sincos_turn": (None, [C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "orc_set_threads": (None, [C.c_int32]),
        "orc_dx": (C.c_double, [H]),
        "orc_dy": (C.c_double, [H]),
        "orc_time": (C.c_double, [H]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


STAGE = {"update_e": 0, "efield_bcs": 1, "update_b": 2, "bfield_bcs_mpi": 3, "push": 4,
         "current_rmin": 5, "particle_bcs": 6, "current_finish": 7, "bfield_final_bcs": 8,
         "moving_window": 9, "eb_half": 10, "eb_final": 11}


ATAN2 = {"libm": 0, "shared": 1}


class Oracle:
    """One run of the CPU restatement, fed the same inputs as the GPU run.

    atan2: "libm" (default) takes theta with the platform's atan2, as the
    reference does (particles.F90:321,522); "shared" with the correctly
    rounded cyl_atan2 that the CUDA kernel evaluates (include/cyl_math.h).
    They differ where libm is not correctly rounded (about 0.09 % of
    arguments with glibc 2.39); tests that compare many steps at 1e-10 use
    "shared"."""

    def __init__(self, deck, particles=None, rng=None, load_species=False, counter_seed=None, atan2="libm"):
        from cylindrical_epoch_gb300 import abi
        self.abi = abi
        self.lib = load()
        self.atan2_mode = ATAN2[atan2]
        self.deck = deck
        g = deck.grid_desc()
        sp = deck.species_descs()
        las, self._keep = deck.laser_descs()
        h = C.c_void_p()
        rc = self.lib.orc_create(C.byref(g), sp, len(deck.species), las, len(deck.lasers), deck.seed,
                                 C.byref(h))
        if rc != 0:
            raise RuntimeError(f"orc_create failed {rc}")
        self.h = h
        self.nxg = deck.nx + 2 * abi.NG
        self.nyg = deck.ny + 2 * abi.NG
        if counter_seed is not None:
            # the counter stream for loading and window injection (ids
            # continue across the mobile species, as the host loader's)
            id_base = 0
            for i in range(len(deck.species)):
                if not deck.species[i].immobile:
                    self.lib.orc_load_species_counter(self.h, i, int(counter_seed), id_base)
                    id_base += self.lib.orc_count(self.h, i)
            self.lib.orc_set_injection_stream(self.h, abi.RNG_COUNTER, int(counter_seed))
        elif load_species:
            for i in range(len(deck.species)):
                if deck.species[i].immobile:
                    continue
                grids = deck.load_grids(i) if deck.load_grids is not None else None
                if grids is None:
                    self.lib.orc_load_species(self.h, i)
                else:
                    ga = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in grids]
                    PDc = C.POINTER(C.c_double)
                    self.lib.orc_load_species_grid(self.h, i, *[None if a is None else a.ctypes.data_as(PDc)
                                                                for a in ga])
        if deck.has_deck_fns():
            self._fns, self._fns_keep = deck.deck_fns()
            self.lib.orc_set_deck_fns(self.h, C.byref(self._fns))
        if deck.ionisation:
            arr = deck.ionisation_descs()
            if self.lib.orc_set_ionisation(self.h, arr, len(deck.species), deck.ionisation_model,
                                           deck.ionisation_seed) != 0:
                raise RuntimeError("orc_set_ionisation")
        if particles is not None:
            for i, p in enumerate(particles):
                self.set_particles(i, p)
        if rng is not None:
            self.lib.orc_set_rng(self.h, C.byref(rng))

    def ionisation_constants(self):
        out = np.zeros((len(self.deck.species), self.abi.ION_NCONST))
        self.lib.orc_ionisation_constants(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, isp, p):
        PD = C.POINTER(C.c_double)
        f = lambda a: a.ctypes.data_as(PD)
        self.lib.orc_set_particles(self.h, isp, f(p.x), f(p.y), f(p.z), f(p.px), f(p.py), f(p.pz), f(p.w),
                                   p.id.ctypes.data_as(C.POINTER(C.c_int64)), p.n)

    def particles(self, isp=0):
        from cylindrical_epoch_gb300.run import Particles
        n = self.lib.orc_count(self.h, isp)
        p = Particles(n)
        PD = C.POINTER(C.c_double)
        f = lambda a: a.ctypes.data_as(PD)
        self.lib.orc_get_particles(self.h, isp, f(p.x), f(p.y), f(p.z), f(p.px), f(p.py), f(p.pz), f(p.w),
                                   p.id.ctypes.data_as(C.POINTER(C.c_int64)))
        return p

    def field(self, name):
        which = self.abi.FIELD_INDEX[name] if isinstance(name, str) else name
        a = np.zeros((self.deck.n_mode, self.nyg, self.nxg), dtype=np.complex128)
        self.lib.orc_get_field(self.h, which, a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        return a

    def set_field(self, name, arr):
        which = self.abi.FIELD_INDEX[name] if isinstance(name, str) else name
        a = np.ascontiguousarray(arr, dtype=np.complex128)
        self.lib.orc_set_field(self.h, which, a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))

    def rng_state(self):
        r = self.abi.RngState()
        self.lib.orc_get_rng(self.h, C.byref(r))
        return r

    def initialise(self):
        self.lib.orc_set_atan2(self.atan2_mode)
        self.lib.orc_initialise(self.h)

    def step(self, n=1):
        self.lib.orc_set_atan2(self.atan2_mode)
        self.lib.orc_step(self.h, n)

    def step_to_output(self, n=1):
        self.lib.orc_set_atan2(self.atan2_mode)
        if self.lib.orc_step_to_output(self.h, n) != 0:
            raise RuntimeError("orc_step_to_output")

    def finish_step(self):
        self.lib.orc_set_atan2(self.atan2_mode)
        self.lib.orc_finish_step(self.h)

    def restart(self, step, time, xb_min, x_grid_min, window_shift_fraction=None):
        """The restart of a dump's scalars, after set_field / set_particles
        (orc_restart)."""
        rc = self.lib.orc_restart(self.h, int(step), float(time), float(xb_min), float(x_grid_min),
                                  0 if window_shift_fraction is None else 1, float(window_shift_fraction or 0.0))
        if rc != 0:
            raise RuntimeError(f"orc_restart: {rc}")

    def stage(self, name):
        self.lib.orc_set_atan2(self.atan2_mode)
        rc = self.lib.orc_stage(self.h, STAGE[name])
        if rc != 0:
            raise RuntimeError(name)

    def state(self):
        s = self.abi.RunState()
        self.lib.orc_get_run_state(self.h, C.byref(s))
        return s

    def diagnostics(self):
        d = self.abi.Diag()
        self.lib.orc_diagnostics(self.h, C.byref(d))
        return d

    def charge_density(self):
        """Per-mode charge density of the deposit's staggered shape (the
        t + dt/2 shape of the next push), complex (M, ny+2ng, nx+2ng)."""
        a = np.zeros((self.deck.n_mode, self.nyg, self.nxg), dtype=np.complex128)
        self.lib.orc_charge_density(self.h, a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        return a

    def number_density(self, isp=-1):
        """Per-mode number density (calc_number_density_modes) of species isp,
        or of every species with isp < 0; complex (M, ny+2ng, nx+2ng)."""
        a = np.zeros((self.deck.n_mode, self.nyg, self.nxg), dtype=np.complex128)
        self.lib.orc_number_density(self.h, isp, a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
        return a

    def cell_indices(self, isp=0):
        n = self.lib.orc_count(self.h, isp)
        cx = np.zeros(max(1, n), dtype=np.int32)
        cy = np.zeros(max(1, n), dtype=np.int32)
        self.lib.orc_cell_indices(self.h, isp, cx.ctypes.data_as(C.POINTER(C.c_int32)),
                                  cy.ctypes.data_as(C.POINTER(C.c_int32)))
        return cx[:n], cy[:n]
