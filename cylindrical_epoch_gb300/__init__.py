"""GB300-native quasi-3D (x, r, theta-mode) PIC step of cylindrical EPOCH.

The hot path (fused gather / Boris push / charge-conserving per-mode
deposit, per-mode Yee solver with the r = 0 axis rules, laser injection,
particle boundaries, moving window) runs as hand-written sm_103a kernels in
libcylpic.so behind the C ABI of include/cylpic.h.  This package is the
host-side mirror of the reference driver: deck descriptions, the loader and
the run handle.
"""
from . import abi, deck
from .deck import Deck, Laser, Species, thermal_plasma, wakefield, large_wakefield, moving_window_deck, field_ionisation_deck
from .lib import load
from .run import Batch, Particles, Run, SdfFile, host_load, sdf_write_arrays, set_wait_timeout

__all__ = ["abi", "deck", "Deck", "Laser", "Species", "thermal_plasma", "wakefield",
           "large_wakefield", "load", "Particles", "Run", "host_load", "Batch", "sdf_write_arrays", "SdfFile",
           "set_wait_timeout"]
