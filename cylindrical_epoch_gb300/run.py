"""Host-side driver of one run on the GPU.

``Run`` plays the part of the reference's Fortran driver (epoch2d.F90): it
loads the species on the host (auto_load), hands particles and fields to the
C ABI, performs the start-up sequence and advances steps.  All calls go
through libcylpic.so; there is no CPU path.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .deck import Deck
from .lib import load

PD = C.POINTER(C.c_double)
PI64 = C.POINTER(C.c_int64)
PI32 = C.POINTER(C.c_int32)


def _p(a, t=PD):
    return a.ctypes.data_as(t)


class Particles:
    """SoA host copy of one species (positions m, momenta kg m/s)."""

    __slots__ = ("x", "y", "z", "px", "py", "pz", "w", "id")

    def __init__(self, n):
        for k in ("x", "y", "z", "px", "py", "pz", "w"):
            setattr(self, k, np.zeros(n, dtype=np.float64))
        self.id = np.zeros(n, dtype=np.int64)

    @property
    def n(self):
        return self.x.shape[0]

    def resize(self, n):
        for k in self.__slots__:
            setattr(self, k, getattr(self, k)[:n].copy())
        return self

    def sorted_by_id(self):
        o = np.argsort(self.id, kind="stable")
        out = Particles(0)
        for k in self.__slots__:
            setattr(out, k, getattr(self, k)[o])
        return out

    def arrays(self):
        return [getattr(self, k) for k in self.__slots__]


def set_wait_timeout(seconds):
    """Limit of every host wait of the library on device work, in seconds
    (cyl_set_wait_timeout; <= 0: no limit).  A call whose wait runs out
    raises CylError with code CYL_ERR_TIMEOUT and leaves its run as it was
    before the wait."""
    abi.check("cyl_set_wait_timeout", load().cyl_set_wait_timeout(float(seconds)))


def host_load(deck: Deck, rng=None):
    """Load every species as auto_load does; returns (list of Particles, rng)."""
    lib = load()
    if rng is None:
        rng = abi.RngState()
        lib.cyl_rng_init(C.byref(rng), deck.seed)
    g = deck.grid_desc()
    out = []
    id_base = 0
    for isp, s in enumerate(deck.species):
        d = s.desc()
        n = C.c_int64(0)
        grids = deck.load_grids(isp) if deck.load_grids is not None else None
        ga = [None, None, None]
        if grids is not None:
            ga = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in grids]
        gp = [None if a is None else _p(a) for a in ga]
        abi.check("cyl_host_load_species_grid",
                  lib.cyl_host_load_species_grid(C.byref(g), C.byref(d), C.byref(rng), id_base, *gp,
                                                 None, None, None, None, None, None, None, None, C.byref(n)))
        p = Particles(n.value)
        if s.immobile:
            out.append(Particles(0))
            continue
        abi.check("cyl_host_load_species_grid",
                  lib.cyl_host_load_species_grid(C.byref(g), C.byref(d), C.byref(rng), id_base, *gp,
                                                 _p(p.x), _p(p.y), _p(p.z), _p(p.px), _p(p.py), _p(p.pz),
                                                 _p(p.w), _p(p.id, PI64), C.byref(n)))
        p.resize(n.value)
        id_base += n.value
        out.append(p)
    return out, rng


def load_counts(deck: Deck):
    """Particles the loader makes per species (floor(ppc x valid cells); 0
    for immobile species), without loading them."""
    lib = load()
    g = deck.grid_desc()
    out = []
    for s in deck.species:
        n = C.c_int64(0)
        if not s.immobile:
            d = s.desc()
            abi.check("cyl_host_load_species",
                      lib.cyl_host_load_species(C.byref(g), C.byref(d), None, 0, None, None, None, None, None,
                                                None, None, None, C.byref(n)))
        out.append(n.value)
    return out


def sdf_write_arrays(path, nx, ny, n_mode, arrays, step=0, time=0.0, xb_min=0.0, dx=1.0, dy=1.0, restart=False,
                     species=None, dt=0.0, x_grid_min=None, window_shift_fraction=None):
    """Write mode arrays as the reference's SDF field dump (cyl_sdf_write).
    arrays: {name or CYL_F_* index: complex128 array (n_mode, ny+2ng, nx+2ng)}
    (the layout of Run.field); E, B, J and, with restart, B_old and J_old.
    species: [(name, Particles)] written as the reference's particle
    variables and point meshes.  Restart dumps also carry dt (when > 0),
    x_grid_min (default: the first cell centre) and window_shift_fraction
    (when given: the window has started)."""
    lib = load()
    d = abi.SdfDesc()
    d.nx, d.ny, d.n_mode, d.step = int(nx), int(ny), int(n_mode), int(step)
    d.time, d.xb_min, d.dx, d.dy = float(time), float(xb_min), float(dx), float(dy)
    d.restart = 1 if restart else 0
    d.dt = float(dt)
    d.x_grid_min = float(xb_min + 0.5 * dx if x_grid_min is None else x_grid_min)
    d.window_started = 0 if window_shift_fraction is None else 1
    d.window_shift_fraction = float(window_shift_fraction or 0.0)
    ptrs = (PD * abi.NFIELDS)()
    keep = []
    for name, a in arrays.items():
        k = abi.FIELD_INDEX[name] if isinstance(name, str) else int(name)
        a = np.ascontiguousarray(a, dtype=np.complex128)
        if a.shape != (n_mode, ny + 2 * abi.NG, nx + 2 * abi.NG):
            raise ValueError(f"{name}: shape {a.shape}")
        keep.append(a)
        ptrs[k] = a.view(np.float64).ctypes.data_as(PD)
    species = list(species or [])
    sp = (abi.SdfSpecies * max(1, len(species)))()
    for i, (name, p) in enumerate(species):
        e = sp[i]
        e.name = name.encode()
        e.n = p.n
        for k in ("x", "y", "z", "px", "py", "pz", "w"):
            a = np.ascontiguousarray(getattr(p, k), dtype=np.float64)
            keep.append(a)
            setattr(e, k, a.ctypes.data_as(PD))
        a = np.ascontiguousarray(p.id, dtype=np.int64)
        keep.append(a)
        e.id = a.ctypes.data_as(PI64)
    abi.check("cyl_sdf_write", lib.cyl_sdf_write(os.fsencode(path), C.byref(d), ptrs, sp, len(species)))


class SdfFile:
    """An SDF file opened by the restart reader (cyl_sdf_open): `info`
    (cyl_sdf_info), `field(name)` and `particles(species)`."""

    def __init__(self, path):
        self.lib = load()
        h = C.c_void_p()
        abi.check("cyl_sdf_open", self.lib.cyl_sdf_open(os.fsencode(path), C.byref(h)))
        self.h = h
        self.info = abi.SdfInfo()
        abi.check("cyl_sdf_get_info", self.lib.cyl_sdf_get_info(self.h, C.byref(self.info)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.cyl_sdf_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def field(self, name):
        """A mode array in the layout of Run.field (zero ghosts)."""
        which = abi.FIELD_INDEX[name] if isinstance(name, str) else int(name)
        i = self.info
        out = np.zeros((i.n_mode, i.ny + 2 * abi.NG, i.nx + 2 * abi.NG), dtype=np.complex128)
        abi.check("cyl_sdf_read_field", self.lib.cyl_sdf_read_field(self.h, which, _p(out.view(np.float64))))
        return out

    def species_count(self, name):
        n = C.c_int64(0)
        abi.check("cyl_sdf_species_count", self.lib.cyl_sdf_species_count(self.h, name.encode(), C.byref(n)))
        return n.value

    def particles(self, name):
        n = self.species_count(name)
        if n < 0:
            raise KeyError(name)
        p = Particles(n)
        got = C.c_int64(n)
        abi.check("cyl_sdf_read_particles",
                  self.lib.cyl_sdf_read_particles(self.h, name.encode(), _p(p.x), _p(p.y), _p(p.z), _p(p.px),
                                                  _p(p.py), _p(p.pz), _p(p.w), p.id.ctypes.data_as(PI64),
                                                  C.byref(got)))
        return p


class Run:
    """One simulation resident on the GPU, driven through the C ABI.

    rng_mode=abi.RNG_KISS (default): particles come from the host loader (the
    reference's KISS stream, or `particles`) and window injection replays
    the same stream.  rng_mode=abi.RNG_COUNTER: the species are loaded on the
    device and the window injects on the device, both from the counter
    stream keyed by `counter_seed` (default: the deck's seed)."""

    def __init__(self, deck: Deck, particles=None, rng=None, fields=None, initialise=True,
                 rng_mode=abi.RNG_KISS, counter_seed=None):
        self.lib = load()
        self.deck = deck
        counter = rng_mode == abi.RNG_COUNTER
        if counter:
            counts = load_counts(deck)
            if rng is None:
                rng = abi.RngState()
                self.lib.cyl_rng_init(C.byref(rng), deck.seed)
        elif particles is None:
            particles, rng = host_load(deck, rng)
        g = deck.grid_desc()
        self.dt = g.dt
        sp = deck.species_descs()
        for i, s in enumerate(deck.species):
            if counter:
                need = counts[i]
            else:
                need = particles[i].n if i < len(particles) else 0
            if sp[i].capacity < need + 1024:
                sp[i].capacity = int(need * 1.1) + 4096
        las, self._keep = deck.laser_descs()
        h = C.c_void_p()
        abi.check("cyl_create", self.lib.cyl_create(C.byref(g), sp, len(deck.species), las,
                                                    len(deck.lasers), C.byref(rng) if rng else None,
                                                    C.byref(h)))
        self.h = h
        self.nxg = deck.nx + 2 * abi.NG
        self.nyg = deck.ny + 2 * abi.NG
        if deck.has_deck_fns():
            self._fns, self._fns_keep = deck.deck_fns()
            abi.check("cyl_set_deck_fns", self.lib.cyl_set_deck_fns(self.h, C.byref(self._fns)))
        if deck.ionisation:
            abi.check("cyl_set_ionisation",
                      self.lib.cyl_set_ionisation(self.h, deck.ionisation_descs(), len(deck.species),
                                                  deck.ionisation_model, deck.ionisation_seed))
        if counter:
            seed = deck.seed if counter_seed is None else int(counter_seed)
            id_base = 0
            for i, s in enumerate(deck.species):
                if s.immobile:
                    continue
                n = C.c_int64(0)
                abi.check("cyl_load_species_device",
                          self.lib.cyl_load_species_device(self.h, i, seed, id_base, C.byref(n)))
                id_base += n.value
            abi.check("cyl_set_injection_stream", self.lib.cyl_set_injection_stream(self.h, abi.RNG_COUNTER, seed))
        else:
            for i, p in enumerate(particles):
                self.upload_particles(i, p)
        if fields:
            for name, arr in fields.items():
                self.upload_field(name, arr)
        if initialise:
            abi.check("cyl_initialise", self.lib.cyl_initialise(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.cyl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- data movement
    def upload_particles(self, isp, p: Particles):
        abi.check("cyl_upload_particles",
                  self.lib.cyl_upload_particles(self.h, isp, _p(p.x), _p(p.y), _p(p.z), _p(p.px),
                                                _p(p.py), _p(p.pz), _p(p.w), _p(p.id, PI64), p.n))

    def particles(self, isp=0, out=None):
        """The live particles of species isp (device order).  out: a
        Particles whose arrays (e.g. pinned) receive them, of at least the
        live count; the result then views its first n entries."""
        n = C.c_int64(0)
        abi.check("cyl_download_particles",
                  self.lib.cyl_download_particles(self.h, isp, None, None, None, None, None, None,
                                                  None, None, C.byref(n)))
        if out is not None:
            if out.n < n.value:
                raise ValueError(f"out holds {out.n} particles, {n.value} are live")
            n = C.c_int64(out.n)
            abi.check("cyl_download_particles",
                      self.lib.cyl_download_particles(self.h, isp, _p(out.x), _p(out.y), _p(out.z), _p(out.px),
                                                      _p(out.py), _p(out.pz), _p(out.w), _p(out.id, PI64),
                                                      C.byref(n)))
            v = Particles(0)
            for k in v.__slots__:
                setattr(v, k, getattr(out, k)[:n.value])
            return v
        p = Particles(n.value)
        abi.check("cyl_download_particles",
                  self.lib.cyl_download_particles(self.h, isp, _p(p.x), _p(p.y), _p(p.z), _p(p.px),
                                                  _p(p.py), _p(p.pz), _p(p.w), _p(p.id, PI64),
                                                  C.byref(n)))
        return p.resize(n.value)

    def field(self, name, out=None):
        """Complex mode array F(1-ng:nx+ng, 1-ng:ny+ng, 0:M-1) as numpy
        complex128 with shape (M, ny+2ng, nx+2ng) (Fortran order reversed);
        into `out` (a contiguous complex128 array of that shape) if given."""
        which = abi.FIELD_INDEX[name] if isinstance(name, str) else name
        shape = (self.deck.n_mode, self.nyg, self.nxg)
        if out is not None:
            if out.shape != shape or out.dtype != np.complex128 or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous complex128 array of shape %s" % (shape,))
            a = out
        else:
            a = np.zeros(shape, dtype=np.complex128)
        abi.check("cyl_download_field", self.lib.cyl_download_field(self.h, which, _p(a.view(np.float64))))
        return a

    def charge_density(self):
        """Per-mode charge density of the deposit's staggered shape for the
        current state (cyl_charge_density), shaped like field()."""
        a = np.zeros((self.deck.n_mode, self.nyg, self.nxg), dtype=np.complex128)
        abi.check("cyl_charge_density", self.lib.cyl_charge_density(self.h, _p(a.view(np.float64))))
        return a

    def number_density(self, isp=-1):
        """Per-mode number density of species isp, or of every species with
        isp < 0 (cyl_number_density), shaped like field()."""
        a = np.zeros((self.deck.n_mode, self.nyg, self.nxg), dtype=np.complex128)
        abi.check("cyl_number_density", self.lib.cyl_number_density(self.h, int(isp), _p(a.view(np.float64))))
        return a

    def upload_field(self, name, arr):
        which = abi.FIELD_INDEX[name] if isinstance(name, str) else name
        a = np.ascontiguousarray(arr, dtype=np.complex128)
        abi.check("cyl_upload_field", self.lib.cyl_upload_field(self.h, which, _p(a.view(np.float64))))

    # ---- stepping
    def step(self, n=1, graph=False):
        fn = self.lib.cyl_step_graph if graph else self.lib.cyl_step
        abi.check("cyl_step", fn(self.h, n))

    def step_to_output(self, n=1):
        """Advance to the reference's output point of the n-th step
        (cyl_step_to_output); the next stepping call finishes that step."""
        abi.check("cyl_step_to_output", self.lib.cyl_step_to_output(self.h, n))

    @classmethod
    def from_sdf(cls, deck: Deck, path, rng_mode=abi.RNG_KISS, counter_seed=None):
        """A run restarted from a restart dump of the same deck
        (cyl_restart_sdf), at the output point of the dumped step."""
        with SdfFile(path) as f:
            counts = [max(f.species_count(s.name), 0) for s in deck.species]
        self = cls.__new__(cls)
        self.lib = load()
        self.deck = deck
        g = deck.grid_desc()
        self.dt = g.dt
        sp = deck.species_descs()
        for i, n in enumerate(counts):
            if sp[i].capacity < n + 1024:
                sp[i].capacity = int(n * 1.1) + 4096
        las, self._keep = deck.laser_descs()
        rng = abi.RngState()
        self.lib.cyl_rng_init(C.byref(rng), deck.seed)
        h = C.c_void_p()
        abi.check("cyl_create", self.lib.cyl_create(C.byref(g), sp, len(deck.species), las, len(deck.lasers),
                                                    C.byref(rng), C.byref(h)))
        self.h = h
        self.nxg = deck.nx + 2 * abi.NG
        self.nyg = deck.ny + 2 * abi.NG
        if rng_mode == abi.RNG_COUNTER:
            seed = deck.seed if counter_seed is None else int(counter_seed)
            abi.check("cyl_set_injection_stream", self.lib.cyl_set_injection_stream(self.h, abi.RNG_COUNTER, seed))
        names = (C.c_char_p * len(deck.species))(*[s.name.encode() for s in deck.species])
        abi.check("cyl_restart_sdf", self.lib.cyl_restart_sdf(self.h, os.fsencode(path), names))
        return self

    def write_sdf(self, path, restart=False, particles=True):
        """Dump the current state as the reference's SDF output
        (cyl_write_sdf): the mode fields and, with particles, every species'
        live particles under the deck's species names."""
        names = None
        if particles:
            names = (C.c_char_p * len(self.deck.species))(*[s.name.encode() for s in self.deck.species])
        abi.check("cyl_write_sdf", self.lib.cyl_write_sdf(self.h, os.fsencode(path), 1 if restart else 0, names))

    def step_async(self, n=1):
        """Enqueue n steps (graphs) and return without waiting (cyl_step_async)."""
        abi.check("cyl_step_async", self.lib.cyl_step_async(self.h, n))

    def diagnostics_async(self):
        """Enqueue a diagnostics read of the state after the enqueued steps."""
        abi.check("cyl_diagnostics_async", self.lib.cyl_diagnostics_async(self.h))

    def diagnostics_read(self):
        """Wait for the oldest enqueued diagnostics read and return it."""
        d = abi.Diag()
        abi.check("cyl_diagnostics_read", self.lib.cyl_diagnostics_read(self.h, C.byref(d)))
        return d

    def stream(self):
        """The handle's CUDA stream (cudaStream_t as an int)."""
        st = C.c_void_p()
        abi.check("cyl_get_stream", self.lib.cyl_get_stream(self.h, C.byref(st)))
        return st.value or 0

    def push_only(self):
        abi.check("cyl_push_only", self.lib.cyl_push_only(self.h))

    def merge_e_halves(self, on=True):
        """Mixed form: merge each step's closing E half-step with the next
        step's opening one inside a chunk (the default; the results are
        those of separate half-steps).  cyl_set_merge_e_halves."""
        abi.check("cyl_set_merge_e_halves", self.lib.cyl_set_merge_e_halves(self.h, 1 if on else 0))

    def tune_tiles(self, shape=None):
        """Mixed form: with shape=None time one push of the current state with
        every tile shape and keep the fastest, else use tile shape `shape`
        (cyl_tune_tiles).  Returns (index, (cells x, cells r))."""
        k = C.c_int32(-1 if shape is None else int(shape))
        mode = abi.TUNE_TIME if shape is None else abi.TUNE_SET
        abi.check("cyl_tune_tiles", self.lib.cyl_tune_tiles(self.h, mode, C.byref(k)))
        tx, ty = C.c_int32(0), C.c_int32(0)
        abi.check("cyl_tile_shape", self.lib.cyl_tile_shape(k.value, C.byref(tx), C.byref(ty)))
        return k.value, (tx.value, ty.value)

    def sort(self):
        abi.check("cyl_sort_particles", self.lib.cyl_sort_particles(self.h))

    def state(self):
        s = abi.RunState()
        abi.check("cyl_get_run_state", self.lib.cyl_get_run_state(self.h, C.byref(s)))
        return s

    def diagnostics(self):
        d = abi.Diag()
        abi.check("cyl_diagnostics", self.lib.cyl_diagnostics(self.h, C.byref(d)))
        return d

    def rng_state(self):
        r = abi.RngState()
        abi.check("cyl_get_rng_state", self.lib.cyl_get_rng_state(self.h, C.byref(r)))
        return r

    def kernel_timing(self):
        ms = C.c_double(0.0)
        n = C.c_int64(0)
        abi.check("cyl_kernel_timing", self.lib.cyl_kernel_timing(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def cell_indices(self, isp=0):
        n = C.c_int64(0)
        abi.check("cyl_cell_indices", self.lib.cyl_cell_indices(self.h, isp, None, None, C.byref(n)))
        cx = np.zeros(max(1, n.value), dtype=np.int32)
        cy = np.zeros(max(1, n.value), dtype=np.int32)
        abi.check("cyl_cell_indices", self.lib.cyl_cell_indices(self.h, isp, _p(cx, PI32), _p(cy, PI32),
                                                                C.byref(n)))
        return cx[:n.value], cy[:n.value]


class Batch:
    """Mixed-form runs stepped together (cyl_batch_*): one push launch per
    step over all runs' tiles; the other stages per run, in one graph per
    chunk of 16 steps."""

    def __init__(self, max_runs=16):
        self.lib = load()
        self.b = C.c_void_p()
        abi.check("cyl_batch_create", self.lib.cyl_batch_create(int(max_runs), C.byref(self.b)))

    def step(self, runs, nsteps):
        hs = (C.c_void_p * len(runs))(*[r.h for r in runs])
        abi.check("cyl_batch_step", self.lib.cyl_batch_step(self.b, hs, len(runs), int(nsteps)))

    def close(self):
        if getattr(self, "b", None):
            self.lib.cyl_batch_destroy(self.b)
            self.b = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

