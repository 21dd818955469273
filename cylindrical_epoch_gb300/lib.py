"""Loader and ctypes signatures of libcylpic.so (include/cylpic.h).

There is no fallback: if the library is missing the import of ``load()``
raises, and every entry point that needs a GPU returns CYL_ERR_NO_DEVICE on
a machine without one.
"""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcylpic.so")

_lib = None

P = C.POINTER
D = C.c_double
I32 = C.c_int32
I64 = C.c_int64
PD = P(C.c_double)
PI64 = P(C.c_int64)
PI32 = P(C.c_int32)
H = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "cyl_create": (C.c_int, [P(abi.GridDesc), P(abi.SpeciesDesc), I32, P(abi.LaserDesc), I32,
                             P(abi.RngState), P(H)]),
    "cyl_destroy": (C.c_int, [H]),
    "cyl_upload_particles": (C.c_int, [H, I32, PD, PD, PD, PD, PD, PD, PD, PI64, I64]),
    "cyl_load_species_device": (C.c_int, [H, I32, C.c_uint64, I64, PI64]),
    "cyl_set_injection_stream": (C.c_int, [H, I32, C.c_uint64]),
    "cyl_set_merge_e_halves": (C.c_int, [H, I32]),
    "cyl_counter_block": (C.c_int, [C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "cyl_sdf_write": (C.c_int, [C.c_char_p, P(abi.SdfDesc), C.POINTER(PD), P(abi.SdfSpecies), I32]),
    "cyl_write_sdf": (C.c_int, [H, C.c_char_p, I32, C.POINTER(C.c_char_p)]),
    "cyl_sdf_open": (C.c_int, [C.c_char_p, P(H)]),
    "cyl_sdf_close": (C.c_int, [H]),
    "cyl_sdf_get_info": (C.c_int, [H, P(abi.SdfInfo)]),
    "cyl_sdf_read_field": (C.c_int, [H, I32, PD]),
    "cyl_sdf_species_count": (C.c_int, [H, C.c_char_p, PI64]),
    "cyl_sdf_read_particles": (C.c_int, [H, C.c_char_p, PD, PD, PD, PD, PD, PD, PD, PI64, PI64]),
    "cyl_restart_sdf": (C.c_int, [H, C.c_char_p, C.POINTER(C.c_char_p)]),
    "cyl_download_particles": (C.c_int, [H, I32, PD, PD, PD, PD, PD, PD, PD, PI64, PI64]),
    "cyl_upload_field": (C.c_int, [H, I32, PD]),
    "cyl_download_field": (C.c_int, [H, I32, PD]),
    "cyl_initialise": (C.c_int, [H]),
    "cyl_step": (C.c_int, [H, I32]),
    "cyl_step_graph": (C.c_int, [H, I32]),
    "cyl_step_async": (C.c_int, [H, I32]),
    "cyl_step_to_output": (C.c_int, [H, I32]),
    "cyl_diagnostics_async": (C.c_int, [H]),
    "cyl_diagnostics_read": (C.c_int, [H, P(abi.Diag)]),
    "cyl_get_run_state": (C.c_int, [H, P(abi.RunState)]),
    "cyl_diagnostics": (C.c_int, [H, P(abi.Diag)]),
    "cyl_get_rng_state": (C.c_int, [H, P(abi.RngState)]),
    "cyl_debug_record": (C.c_int, [H, P(C.c_float)]),
    "cyl_sort_particles": (C.c_int, [H]),
    "cyl_cell_indices": (C.c_int, [H, I32, PI32, PI32, PI64]),
    "cyl_cell_indices_noalloc": (C.c_int, [H, I32, PI32, PI32, PI64]),
    "cyl_charge_density": (C.c_int, [H, PD]),
    "cyl_number_density": (C.c_int, [H, I32, PD]),
    "cyl_tile_shape": (C.c_int, [I32, PI32, PI32]),
    "cyl_tune_tiles": (C.c_int, [H, I32, PI32]),
    "cyl_push_only": (C.c_int, [H]),
    "cyl_kernel_timing": (C.c_int, [H, PD, PI64]),
    "cyl_get_stream": (C.c_int, [H, P(C.c_void_p)]),
    "cyl_eval_atan2": (C.c_int, [I64, PD, PD, PD]),
    "cyl_set_wait_timeout": (C.c_int, [C.c_double]),
    "cyl_set_deck_fns": (C.c_int, [H, P(abi.DeckFns)]),
    "cyl_set_ionisation": (C.c_int, [H, P(abi.IonisationSpecies), I32, I32, C.c_uint64]),
    "cyl_ionisation_constants": (C.c_int, [P(abi.IonisationSpecies), P(abi.SpeciesDesc), I32, I32, D, PD]),
    "cyl_host_load_species_grid": (C.c_int, [P(abi.GridDesc), P(abi.SpeciesDesc), P(abi.RngState), I64,
                                             PD, PD, PD, PD, PD, PD, PD, PD, PD, PD, PI64, PI64]),
    "cyl_estimate_device_bytes": (C.c_int, [P(abi.GridDesc), P(abi.SpeciesDesc), I32, PI64]),
    "cyl_batch_create": (C.c_int, [I32, P(H)]),
    "cyl_batch_step": (C.c_int, [H, P(H), I32, I32]),
    "cyl_batch_destroy": (C.c_int, [H]),
    "cyl_server_create": (C.c_int, [I64, I32, P(H)]),
    "cyl_server_create_batched": (C.c_int, [I64, I32, I32, P(H)]),
    "cyl_server_submit": (C.c_int, [H, P(abi.JobDesc), PI64]),
    "cyl_server_poll": (C.c_int, [H, I64, P(abi.JobResult)]),
    "cyl_server_wait": (C.c_int, [H, I64, D, P(abi.JobResult)]),
    "cyl_server_stats": (C.c_int, [H, PI32, PI32, PI64]),
    "cyl_server_destroy": (C.c_int, [H]),
    "cyl_rng_init": (None, [P(abi.RngState), I32]),
    "cyl_rng_random": (C.c_double, [P(abi.RngState)]),
    "cyl_rng_box_muller": (C.c_double, [P(abi.RngState), D, D]),
    "cyl_host_load_species": (C.c_int, [P(abi.GridDesc), P(abi.SpeciesDesc), P(abi.RngState), I64,
                                        PD, PD, PD, PD, PD, PD, PD, PI64, PI64]),
}


def load(path=None):
    """Load libcylpic.so (build it first with cylindrical_epoch_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build the CUDA library with "
            "`python -m cylindrical_epoch_gb300.build` (there is no CPU fallback)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
