"""Request loop for parameter scans: Python side of cyl_server_* (cylpic.h).

A Server owns a queue of runs and a pool of worker threads on one GPU.  Runs
are admitted in arrival order against an HBM budget, run concurrently on
their own CUDA streams, and retired when done; each result carries its
submit, start and end times, so completion latency is t_end - t_submit.
"""
import ctypes as C

import numpy as np

from . import abi
from .lib import load


def job_desc(deck, nsteps, seed=None, rng_mode=abi.RNG_KISS):
    """cyl_job_desc for a deck; returns (desc, buffers to keep alive until submitted).
    rng_mode=abi.RNG_COUNTER loads and injects on the device (counter stream
    keyed by the seed) instead of the host KISS stream."""
    d = abi.JobDesc()
    d.grid = deck.grid_desc()
    d.nspecies = len(deck.species)
    for i, s in enumerate(deck.species):
        d.species[i] = s.desc()
    las, keep = deck.laser_descs()
    d.nlasers = len(deck.lasers)
    for i in range(len(deck.lasers)):
        d.lasers[i] = las[i]
    d.nsteps = int(nsteps)
    d.seed = int(deck.seed if seed is None else seed)
    d.rng_mode = int(rng_mode)
    return d, (las, keep)


def estimate_bytes(deck):
    lib = load()
    g = deck.grid_desc()
    sp = deck.species_descs()
    out = C.c_int64(0)
    abi.check("cyl_estimate_device_bytes", lib.cyl_estimate_device_bytes(C.byref(g), sp, len(deck.species),
                                                                         C.byref(out)))
    return out.value


class Server:
    """The request loop.  batched=False: each worker runs its jobs on their
    own streams, start to end.  batched=True: workers only open the small
    mixed-form jobs (at most one push tile per SM); one stepper advances all
    of them with the same mode count together as a batch, and larger or
    FP64-form jobs run as with batched=False (cyl_server_create_batched)."""

    def __init__(self, hbm_budget_bytes=0, workers=4, batched=False, max_batch=16):
        self.lib = load()
        self.h = C.c_void_p()
        if batched:
            abi.check("cyl_server_create_batched",
                      self.lib.cyl_server_create_batched(int(hbm_budget_bytes), int(workers), int(max_batch),
                                                         C.byref(self.h)))
        else:
            abi.check("cyl_server_create", self.lib.cyl_server_create(int(hbm_budget_bytes), int(workers),
                                                                      C.byref(self.h)))

    def submit(self, deck, nsteps, seed=None, rng_mode=abi.RNG_KISS):
        d, keep = job_desc(deck, nsteps, seed, rng_mode)
        jid = C.c_int64(0)
        abi.check("cyl_server_submit", self.lib.cyl_server_submit(self.h, C.byref(d), C.byref(jid)))
        return jid.value

    def poll(self, jid):
        r = abi.JobResult()
        abi.check("cyl_server_poll", self.lib.cyl_server_poll(self.h, jid, C.byref(r)))
        return r

    def wait(self, jid, timeout_s=600.0):
        r = abi.JobResult()
        abi.check("cyl_server_wait", self.lib.cyl_server_wait(self.h, jid, float(timeout_s), C.byref(r)))
        return r

    def stats(self):
        q, run, b = C.c_int32(0), C.c_int32(0), C.c_int64(0)
        abi.check("cyl_server_stats", self.lib.cyl_server_stats(self.h, C.byref(q), C.byref(run), C.byref(b)))
        return q.value, run.value, b.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.cyl_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def latency_stats(results):
    """p50 / p99 completion latency (s) and aggregate particle-steps/s of finished jobs."""
    lat = np.array([r.t_end - r.t_submit for r in results])
    t0 = min(r.t_submit for r in results)
    t1 = max(r.t_end for r in results)
    ps = sum(r.particle_steps for r in results)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "makespan_s": t1 - t0, "particle_steps": ps,
            "aggregate": ps / (t1 - t0)}
