"""ctypes mirror of include/cylpic.h.

The structures below are field-for-field copies of the C descriptors, so a
Python caller builds exactly what a Fortran caller would pass through
ISO_C_BINDING.  Constants carry the values of the reference's
constants.F90:56-84.
"""
import ctypes as C

NG = 5

CYL_OK = 0
CYL_ERR_BAD_ARG = 1
CYL_ERR_CUDA = 2
CYL_ERR_NO_DEVICE = 3
CYL_ERR_CAPACITY = 4
CYL_ERR_UNSUPPORTED = 5
CYL_ERR_DEVICE_FLAG = 6
CYL_ERR_TIMEOUT = 7
CYL_ERR_OUT_OF_MEMORY = 8
CYL_ERR_SCRATCH = 9
CYL_ERR_IO = 10
CYL_ERR_CALLBACK = 11
NOALLOC_MAX_PARTICLES = 262144  # CYL_NOALLOC_MAX_PARTICLES
N_TILE_SHAPES = 5  # CYL_N_TILE_SHAPES
TUNE_SET = 0       # CYL_TUNE_SET
TUNE_TIME = 1      # CYL_TUNE_TIME
RNG_KISS = 0       # CYL_RNG_KISS: host KISS stream, the reference's order
RNG_COUNTER = 1    # CYL_RNG_COUNTER: device counter stream (Philox4x32-10)

ERROR_NAMES = {
    CYL_ERR_BAD_ARG: "bad argument",
    CYL_ERR_CUDA: "CUDA runtime error",
    CYL_ERR_NO_DEVICE: "no CUDA device",
    CYL_ERR_CAPACITY: "particle capacity exceeded",
    CYL_ERR_UNSUPPORTED: "unsupported option",
    CYL_ERR_DEVICE_FLAG: "device error flag raised",
    CYL_ERR_TIMEOUT: "timed out waiting for the GPU",
    CYL_ERR_OUT_OF_MEMORY: "device out of memory",
    CYL_ERR_SCRATCH: "input larger than the fixed scratch (CYL_NOALLOC_MAX_PARTICLES slots)",
    CYL_ERR_IO: "file could not be written",
    CYL_ERR_CALLBACK: "a deck-expression callback returned an error",
}

BC_PERIODIC = 1
BC_OTHER = 2
BC_SIMPLE_LASER = 3
BC_SIMPLE_OUTFLOW = 4
BC_OPEN = 5
BC_ZERO_GRADIENT = 7
BC_CLAMP = 8
BC_REFLECT = 9
BC_CONDUCT = 10
BC_ZERO_B = 16

BD_X_MIN, BD_X_MAX, BD_Y_MIN, BD_Y_MAX = 0, 1, 2, 3

PREC_FP64 = 0
PREC_MIXED = 1

FIELD_NAMES = ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm",
               "bxm_old", "brm_old", "btm_old", "jxm_old", "jrm_old", "jtm_old"]
FIELD_INDEX = {n: i for i, n in enumerate(FIELD_NAMES)}
NFIELDS = len(FIELD_NAMES)  # CYL_NFIELDS


class GridDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("n_mode", C.c_int32),
        ("precision", C.c_int32),
        ("x_min", C.c_double), ("x_max", C.c_double), ("y_max", C.c_double),
        ("dt", C.c_double),
        ("bc_field", C.c_int32 * 4),
        ("move_window", C.c_int32),
        ("window_v_x", C.c_double), ("window_start_time", C.c_double),
        ("window_stop_time", C.c_double),
        ("bc_after_move", C.c_int32 * 4),
        ("smooth_currents", C.c_int32), ("smooth_its", C.c_int32),
        ("smooth_comp_its", C.c_int32), ("smooth_stride", C.c_int32),
    ]


class SpeciesDesc(C.Structure):
    _fields_ = [
        ("charge", C.c_double), ("mass", C.c_double),
        ("immobile", C.c_int32),
        ("bc_particle", C.c_int32 * 4),
        ("capacity", C.c_int64),
        ("npart_per_cell", C.c_double),
        ("density_kind", C.c_int32),
        ("density", C.c_double), ("ramp_x0", C.c_double), ("ramp_length", C.c_double),
        ("density_min", C.c_double), ("density_max", C.c_double),
        ("temp", C.c_double * 3),
        ("drift", C.c_double * 3),
    ]


class LaserDesc(C.Structure):
    _fields_ = [
        ("boundary", C.c_int32), ("t_profile", C.c_int32),
        ("amp", C.c_double), ("omega", C.c_double), ("pol_angle", C.c_double),
        ("t_start", C.c_double), ("t_end", C.c_double),
        ("t0", C.c_double), ("tw", C.c_double),
        ("profile", C.POINTER(C.c_double)),
        ("phase", C.POINTER(C.c_double)),
    ]


LaserTimeFn = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double))
LaserOmegaFn = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double))
LaserArrayFn = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double))
InjectFn = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_double, C.c_double, C.POINTER(C.c_double),
                       C.POINTER(C.c_double), C.POINTER(C.c_double))


class DeckFns(C.Structure):
    """cyl_deck_fns: callbacks that evaluate deck expressions while stepping."""
    _fields_ = [
        ("user", C.c_void_p),
        ("laser_time", LaserTimeFn),
        ("laser_omega", LaserOmegaFn),
        ("laser_profile", LaserArrayFn),
        ("laser_phase", LaserArrayFn),
        ("omega_fn_mask", C.c_uint32),
        ("profile_fn_mask", C.c_uint32),
        ("phase_fn_mask", C.c_uint32),
        ("inject", InjectFn),
    ]


IONISE_MULTIPHOTON = 1
IONISE_BSI = 2
ION_NCONST = 15


class IonisationSpecies(C.Structure):
    """cyl_ionisation_species: one species' field-ionisation data."""
    _fields_ = [
        ("ionise", C.c_int32), ("ionise_to", C.c_int32), ("release", C.c_int32),
        ("l", C.c_int32), ("n", C.c_int32), ("energy", C.c_double),
    ]


class RngState(C.Structure):
    _fields_ = [
        ("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32), ("w", C.c_int32),
        ("box_muller_cached", C.c_int32),
        ("cached_random_value", C.c_double),
    ]


class SdfDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("n_mode", C.c_int32),
        ("step", C.c_int32),
        ("time", C.c_double),
        ("xb_min", C.c_double),
        ("dx", C.c_double), ("dy", C.c_double),
        ("restart", C.c_int32),
        ("window_started", C.c_int32),
        ("dt", C.c_double), ("x_grid_min", C.c_double), ("window_shift_fraction", C.c_double),
    ]


class SdfInfo(C.Structure):
    _fields_ = [
        ("step", C.c_int32), ("restart", C.c_int32),
        ("time", C.c_double),
        ("nx", C.c_int32), ("ny", C.c_int32), ("n_mode", C.c_int32),
        ("has_grid", C.c_int32),
        ("grid_x0", C.c_double), ("grid_x1", C.c_double), ("grid_y0", C.c_double), ("grid_y1", C.c_double),
        ("has_dt", C.c_int32), ("has_window_shift_fraction", C.c_int32), ("has_x_grid_min", C.c_int32),
        ("dt", C.c_double), ("window_shift_fraction", C.c_double), ("x_grid_min", C.c_double),
        ("code_name", C.c_char * 33),
    ]


class SdfSpecies(C.Structure):
    _fields_ = [
        ("name", C.c_char_p), ("n", C.c_int64),
        ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)), ("z", C.POINTER(C.c_double)),
        ("px", C.POINTER(C.c_double)), ("py", C.POINTER(C.c_double)), ("pz", C.POINTER(C.c_double)),
        ("w", C.POINTER(C.c_double)), ("id", C.POINTER(C.c_int64)),
    ]


class RunState(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("step", C.c_int64),
        ("x_grid_min", C.c_double), ("xb_min", C.c_double),
        ("x_min", C.c_double), ("x_max", C.c_double),
        ("window_shift_fraction", C.c_double),
        ("window_started", C.c_int32),
        ("bc_field", C.c_int32 * 4),
        ("n_live", C.c_int64 * 8),
        ("n_shifts", C.c_int64),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("kinetic_energy", C.c_double),
        ("field_energy_e", C.c_double),
        ("field_energy_b", C.c_double),
        ("jsum_abs", C.c_double),
        ("n_live", C.c_int64),
        ("device_error", C.c_int32),
    ]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class JobDesc(C.Structure):
    _fields_ = [
        ("grid", GridDesc),
        ("nspecies", C.c_int32),
        ("species", SpeciesDesc * 8),
        ("nlasers", C.c_int32),
        ("lasers", LaserDesc * 8),
        ("nsteps", C.c_int64),
        ("seed", C.c_int32),
        ("rng_mode", C.c_int32),
    ]


class JobResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("error", C.c_int32),
        ("t_submit", C.c_double), ("t_start", C.c_double), ("t_end", C.c_double),
        ("steps_done", C.c_int64),
        ("particle_steps", C.c_double),
        ("device_bytes", C.c_int64),
        ("diag", Diag),
        ("state", RunState),
    ]


class CylError(RuntimeError):
    """Raised when an entry point returns a non-zero status."""

    def __init__(self, func, code):
        super().__init__(f"{func} failed: status {code} ({ERROR_NAMES.get(code, 'unknown')})")
        self.code = code


def check(func, code):
    if code != CYL_OK:
        raise CylError(func, code)
    return code
