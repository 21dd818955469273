"""Benchmark of the quasi-3D PIC step on one GB300 (and N replicas).

Metric: particle-steps/s = mobile particles pushed x steps / wall time of
the full step (fields + boundaries + push/deposit + moving window), on the
laser-wakefield deck (2048 x 256 cells, modes m = 0..1, 8 particles per cell,
moving window at c).  A step is one iteration of the reference's driver loop
(epoch2d.F90:213-265).  The timed steps are steps [W, W+K) of the deck run
from t = 0 (the default K = 2000 is the whole deck run).

Arms:
  default             this package, CUDA graphs, device-resident state
  --impl reference    the CPU restatement of the reference's step (oracle/)
                      on all host threads, on a bounded sample of the deck

Prints one JSON line (rank 0).
"""
import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_traffic(form, n_mode, ppc):
    """DRAM bytes per particle of the push from the committed ncu summary of
    a workload with the same modes and particles per cell
    (profiles/push_<form>_traffic.json), or None when none was captured."""
    p = os.path.join(ROOT, "profiles", f"push_{form}_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
    except Exception:
        return None
    for e in d.get("entries", [d]):
        if e.get("n_mode") == n_mode and float(e.get("ppc", -1)) == float(ppc):
            return e
    return None


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(deck, parts, rng, seconds=12.0, threads=None):
    """The oracle (CPU restatement of the reference step) on all host threads,
    on a bounded sample of the same deck: as many steps from the loaded state
    as fit in about `seconds`."""
    from oracle.oracle import Oracle, load
    lib = load()
    nt = threads or os.cpu_count() or 1
    lib.orc_set_threads(nt)
    orc = Oracle(deck, particles=parts, rng=rng)
    orc.initialise()
    n0 = sum(p.n for p in parts)
    t0 = time.perf_counter()
    steps = 0
    while True:
        orc.step(1)
        steps += 1
        if time.perf_counter() - t0 >= seconds or steps >= 400:
            break
    dt = time.perf_counter() - t0
    n1 = sum(orc.state().n_live[i] for i in range(len(deck.species)))
    lib.orc_set_threads(1)
    return {"value": 0.5 * (n0 + n1) * steps / dt, "unit": "particle-steps/s", "cores": nt,
            "kind": "port", "sample": f"{steps} oracle steps of the deck from t=0 ({n0} particles), "
                                      f"{dt:.1f} s, {nt} OpenMP threads"}


def build_deck(name, form, modes=None):
    """The named deck; `modes` overrides the wakefield deck's mode count
    (a profiling case of the same grid at m = 0..modes-1)."""
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi
    prec = abi.PREC_MIXED if form == "mixed" else abi.PREC_FP64
    if name == "wakefield":
        return cg.wakefield(precision=prec) if modes is None else cg.wakefield(n_mode=modes, precision=prec)
    if name == "thermal":
        return cg.thermal_plasma(precision=prec)
    if name == "large":
        return cg.large_wakefield(precision=prec)
    raise ValueError(name)


def run_reference(args, rank):
    """The reference arm: the CPU restatement of the reference's step
    (oracle/) on all host threads, with its own loader (the reference's
    load_particles and KISS stream), so that this process maps no library of
    the package.  It runs the same steps as the GPU arm: W untimed steps from
    t = 0, then steps [W, W+K) timed, or the first of them that fit in about
    a minute of host time (the sample is stated)."""
    if rank != 0:
        return 0
    from oracle.oracle import Oracle, load
    form = "fp64"
    deck = build_deck(args.deck, form, args.modes)
    lib = load()
    nt = os.cpu_count() or 1
    lib.orc_set_threads(nt)
    orc = Oracle(deck, load_species=True)
    orc.initialise()
    mobile = [i for i in range(len(deck.species)) if not deck.species[i].immobile]
    orc.step(args.warmup)
    n0 = sum(orc.state().n_live[i] for i in mobile)
    budget = 60.0
    t0 = time.perf_counter()
    steps = 0
    while steps < args.steps:
        orc.step(1)
        steps += 1
        if time.perf_counter() - t0 >= budget:
            break
    dt = time.perf_counter() - t0
    n1 = sum(orc.state().n_live[i] for i in mobile)
    value = 0.5 * (n0 + n1) * steps / dt
    sample = (f"steps [{args.warmup}, {args.warmup + steps}) of the deck from t=0 ({n0} particles), "
              f"{dt:.1f} s, {nt} OpenMP threads, the restatement's own loader")
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value,
        "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / steps, "steps_timed": steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": _config(args, deck, form),
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": nt, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def scan_decks(n, seed=20261204, nzs=(512, 1024, 2048), nrs=(64, 128, 256)):
    """The parameter-scan stream: n wakefield decks with nz in {512, 1024, 2048},
    nr in {64, 128, 256}, modes m = 0..1 or 0..2, a0 ~ U[0.5, 3], density
    log-uniform in [5e23, 5e24] m^-3, 4-16 particles per cell, 500-2000 steps,
    mixed precision (other grid sizes through nzs, nrs)."""
    import numpy as np
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx = int(rng.choice(list(nzs)))
        ny = int(rng.choice(list(nrs)))
        nm = int(rng.choice([2, 3]))
        a0 = float(rng.uniform(0.5, 3.0))
        dens = float(10 ** rng.uniform(math.log10(5e23), math.log10(5e24)))
        ppc = int(rng.integers(4, 17))
        steps = int(rng.integers(500, 2001))
        deck = cg.wakefield(nx=nx, ny=ny, n_mode=nm, ppc=ppc, a0=a0, density=dens, precision=abi.PREC_MIXED)
        deck.seed = 7842432 + k
        out.append((deck, steps))
    return out


def run_serve(args):
    """Serving benchmark: a stream of scan decks with Poisson arrivals through
    the request loop; p50/p99 completion latency and aggregate particle-steps/s,
    beside the plain FP64 form run one deck at a time on a sample of the decks."""
    import numpy as np
    import torch
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi, build, serve
    build.build()
    torch.cuda.set_device(0)
    decks = scan_decks(args.jobs)
    gaps = np.random.default_rng(7).exponential(args.arrival, size=len(decks))
    clocks = ClockSampler(0)
    clocks.start()
    with serve.Server(0, args.workers) as srv:
        ids = []
        t_sub = time.perf_counter()
        for (deck, steps), gap in zip(decks, gaps):
            ids.append(srv.submit(deck, steps))
            time.sleep(float(gap))
        res = [srv.wait(i, 3600.0) for i in ids]
    # the same decks submitted at once: the throughput of the mix when the
    # request loop is never short of work (arrival-bound above)
    with serve.Server(0, args.workers) as srv:
        ids = [srv.submit(deck, steps) for deck, steps in decks]
        res_sat = [srv.wait(i, 3600.0) for i in ids]
    # the same stream and the same burst through the continuous-batching loop
    with serve.Server(0, args.workers, batched=True, max_batch=args.max_batch) as srv:
        ids = []
        for (deck, steps), gap in zip(decks, gaps):
            ids.append(srv.submit(deck, steps))
            time.sleep(float(gap))
        res_b = [srv.wait(i, 3600.0) for i in ids]
    with serve.Server(0, args.workers, batched=True, max_batch=args.max_batch) as srv:
        ids = [srv.submit(deck, steps) for deck, steps in decks]
        res_bsat = [srv.wait(i, 3600.0) for i in ids]
    # the same stream and burst with each job loaded and injected on the
    # device (counter stream) instead of the host KISS load and upload
    with serve.Server(0, args.workers) as srv:
        ids = []
        for (deck, steps), gap in zip(decks, gaps):
            ids.append(srv.submit(deck, steps, rng_mode=abi.RNG_COUNTER))
            time.sleep(float(gap))
        res_c = [srv.wait(i, 3600.0) for i in ids]
    with serve.Server(0, args.workers) as srv:
        ids = [srv.submit(deck, steps, rng_mode=abi.RNG_COUNTER) for deck, steps in decks]
        res_csat = [srv.wait(i, 3600.0) for i in ids]
    # a scan of small decks (at most one push tile per SM: the ones the
    # batched loop steps together), all submitted at once, through both loops
    small = scan_decks(args.jobs, seed=20261205, nzs=(128, 256), nrs=(32, 64))
    small_res = {}
    for mode in ("streams", "batched"):
        with serve.Server(0, args.workers, batched=(mode == "batched"), max_batch=args.max_batch) as srv:
            ids = [srv.submit(deck, steps) for deck, steps in small]
            small_res[mode] = [srv.wait(i, 3600.0) for i in ids]
    clk = clocks.stop()
    bad = [r.error for r in res if r.status != abi.JOB_DONE]
    st = serve.latency_stats(res)
    st_sat = serve.latency_stats(res_sat)
    st_b = serve.latency_stats(res_b)
    st_bsat = serve.latency_stats(res_bsat)
    # plain FP64 form, one deck at a time, on a sample of the decks (bounded steps)
    fp64 = []
    for deck, steps in decks[:args.fp64_sample]:
        d64 = cg.wakefield(nx=deck.nx, ny=deck.ny, n_mode=deck.n_mode, ppc=int(deck.species[0].npart_per_cell),
                           density=deck.species[0].density, precision=abi.PREC_FP64)
        parts, rng = cg.host_load(d64)
        run = cg.Run(d64, particles=parts, rng=rng)
        k = min(steps, args.fp64_steps_max)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run.step(k, graph=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        s = run.state()
        fp64.append(0.5 * (sum(p.n for p in parts) + s.n_live[0]) * k / dt)
        run.close()
    fp64_rate = float(np.mean(fp64)) if fp64 else None
    line = {
        "metric": "scan p50/p99 completion latency and aggregate particle-steps/s",
        "value": st["aggregate"], "unit": "particle-steps/s", "n_gpus": 1,
        "steps": int(sum(s for _, s in decks)), "warmup": 0, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"{len(decks)} wakefield scan decks, Poisson arrivals mean {args.arrival} s, "
                               "nz {512,1024,2048}, nr {64,128,256}, m 0..1|0..2, a0 U[0.5,3], "
                               "n logU[5e23,5e24], 4-16 ppc, 500-2000 steps, mixed form",
                   "workers": args.workers, "hbm_budget": "free memory - 2 GiB"},
        "latency": {"p50_s": st["p50_s"], "p99_s": st["p99_s"], "mean_s": st["mean_s"],
                    "makespan_s": st["makespan_s"]},
        "saturated": {"value": st_sat["aggregate"], "unit": "particle-steps/s",
                      "makespan_s": st_sat["makespan_s"], "p50_s": st_sat["p50_s"], "p99_s": st_sat["p99_s"],
                      "note": "the same decks submitted at once"},
        "batched": {"value": st_b["aggregate"], "unit": "particle-steps/s",
                    "latency": {"p50_s": st_b["p50_s"], "p99_s": st_b["p99_s"], "mean_s": st_b["mean_s"],
                                "makespan_s": st_b["makespan_s"]},
                    "saturated": {"value": st_bsat["aggregate"], "makespan_s": st_bsat["makespan_s"],
                                  "p50_s": st_bsat["p50_s"], "p99_s": st_bsat["p99_s"]},
                    "note": "continuous batching: mixed-form jobs of at most one push tile per SM "
                            "step together (none in this scan: its decks fill the device alone and run "
                            f"on their loader's stream), at most {args.max_batch} open jobs, "
                            f"{args.workers} loader threads"},
        "device_loading": {"value": serve.latency_stats(res_c)["aggregate"], "unit": "particle-steps/s",
                           "latency": {k: serve.latency_stats(res_c)[k] for k in ("p50_s", "p99_s", "mean_s",
                                                                                   "makespan_s")},
                           "saturated": {k: serve.latency_stats(res_csat)[k]
                                         for k in ("aggregate", "makespan_s", "p50_s", "p99_s")},
                           "note": "jobs loaded and window-injected on the device from the counter stream "
                                   "(cyl_load_species_device) instead of the host KISS load and upload"},
        "small_scan": {"workload": f"{len(small)} wakefield decks as above but nz {{128,256}}, nr {{32,64}} "
                                   "(at most 128 tiles of 16x8 cells), all submitted at once",
                       **{mode: {"value": serve.latency_stats(r)["aggregate"], "unit": "particle-steps/s",
                                 "makespan_s": serve.latency_stats(r)["makespan_s"],
                                 "p50_s": serve.latency_stats(r)["p50_s"],
                                 "p99_s": serve.latency_stats(r)["p99_s"]}
                          for mode, r in small_res.items()}},
        "failed_jobs": len(bad) + sum(1 for r in res_sat + res_b + res_bsat + res_c + res_csat
                                      + small_res["streams"] + small_res["batched"] if r.status != abi.JOB_DONE),
        "failed": [{"job": k, "error": int(r.error), "nx": decks[k][0].nx, "ny": decks[k][0].ny,
                    "n_mode": decks[k][0].n_mode, "ppc": decks[k][0].species[0].npart_per_cell,
                    "steps_done": int(r.steps_done)}
                   for k, r in enumerate(res) if r.status != abi.JOB_DONE],
        "particle_steps": st["particle_steps"],
        "fp64_one_at_a_time": {"value": fp64_rate, "unit": "particle-steps/s", "sample": len(fp64),
                               "steps_per_deck_max": args.fp64_steps_max,
                               "estimated_makespan_s": (st["particle_steps"] / fp64_rate) if fp64_rate else None},
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def serving_leg(args):
    """The scan of decks through the request loop (the C5 workload): a seeded
    stream of args.jobs wakefield decks with Poisson arrivals, admitted
    against the HBM budget, each run on its own stream as slots and memory
    free up.  p50 / p99 completion latency (queueing included), the
    aggregate particle-steps/s and its HBM-roofline fraction (each deck's
    mixed-form push bytes, 60 B + (6 8 + 3 16 2) M / ppc B per particle-step,
    summed over its particle-steps, over the makespan), beside the plain FP64
    form run one deck at a time on a sample of the decks."""
    import numpy as np
    import torch
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi, serve
    decks = scan_decks(args.jobs)
    gaps = np.random.default_rng(7).exponential(args.arrival, size=len(decks))

    def serve_all(gaps):
        with serve.Server(0, args.workers) as srv:
            ids = []
            for (deck, steps), gap in zip(decks, gaps):
                ids.append(srv.submit(deck, steps))
                if gap > 0:
                    time.sleep(float(gap))
            return [srv.wait(i, 3600.0) for i in ids]

    def push_bytes(res):
        alg = 0.0
        for (deck, _), r in zip(decks, res):
            if r.status == abi.JOB_DONE:
                alg += r.particle_steps * (60.0 + (6 * 8 + 3 * 16 * 2) * deck.n_mode /
                                           deck.species[0].npart_per_cell)
        return alg

    peak, peak_kind = _peaks()
    # capacity: the same decks submitted at once, so that the makespan is set
    # by the device and not by the arrivals
    sat = serve_all(np.zeros(len(decks)))
    sat_ok = [r for r in sat if r.status == abi.JOB_DONE]
    sat_st = serve.latency_stats(sat_ok) if sat_ok else None
    res = serve_all(gaps)
    ok = [r for r in res if r.status == abi.JOB_DONE]
    st = serve.latency_stats(ok) if ok else None
    alg = push_bytes(res)
    fp64 = []
    for deck, steps in decks[:args.fp64_sample]:
        d64 = cg.wakefield(nx=deck.nx, ny=deck.ny, n_mode=deck.n_mode, ppc=int(deck.species[0].npart_per_cell),
                           density=deck.species[0].density, precision=abi.PREC_FP64)
        parts, rng = cg.host_load(d64)
        run = cg.Run(d64, particles=parts, rng=rng)
        k = min(steps, args.fp64_steps_max)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run.step(k, graph=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        s = run.state()
        fp64.append(0.5 * (sum(p.n for p in parts) + s.n_live[0]) * k / dt)
        run.close()
    fp64_rate = float(np.mean(fp64)) if fp64 else None
    out = {"workload": f"{len(decks)} wakefield scan decks, Poisson arrivals mean {args.arrival} s, "
                       "nz {512,1024,2048}, nr {64,128,256}, m 0..1|0..2, a0 U[0.5,3], n logU[5e23,5e24], "
                       "4-16 ppc, 500-2000 steps, mixed form, host-loaded (the reference's KISS stream)",
           "workers": args.workers, "hbm_budget": "free memory - 2 GiB", "failed_jobs": len(res) - len(ok)}
    if st:
        out.update({"value": st["aggregate"], "unit": "particle-steps/s", "p50_s": st["p50_s"], "p99_s": st["p99_s"],
                    "mean_s": st["mean_s"], "makespan_s": st["makespan_s"], "particle_steps": st["particle_steps"],
                    "roofline": {"bound": "hbm", "achieved": alg / st["makespan_s"] / 1e9, "peak": peak,
                                 "unit": "GB/s", "frac": alg / st["makespan_s"] / 1e9 / peak, "peak_kind": peak_kind,
                                 "note": "push algorithmic bytes of every job over the makespan"}})
    if sat_st:
        sa = push_bytes(sat) / sat_st["makespan_s"] / 1e9
        out["saturated"] = {"value": sat_st["aggregate"], "unit": "particle-steps/s",
                            "makespan_s": sat_st["makespan_s"], "p50_s": sat_st["p50_s"], "p99_s": sat_st["p99_s"],
                            "failed_jobs": len(sat) - len(sat_ok),
                            "note": "the same decks submitted at once: the request loop's capacity",
                            "roofline": {"bound": "hbm", "achieved": sa, "peak": peak, "unit": "GB/s",
                                         "frac": sa / peak, "peak_kind": peak_kind}}
    out["fp64_one_at_a_time"] = {"value": fp64_rate, "unit": "particle-steps/s", "sample": len(fp64),
                                 "steps_per_deck_max": args.fp64_steps_max,
                                 "estimated_makespan_s": (st["particle_steps"] / fp64_rate) if (fp64_rate and st)
                                 else None}
    return out


def _config(args, deck, form):
    return {"workload": f"{deck.name} {deck.nx}x{deck.ny} m=0..{deck.n_mode - 1} "
                        f"{deck.species[0].npart_per_cell:g} ppc, steps [W, W+K) of the deck from t=0",
            "form": form, "nx": deck.nx, "ny": deck.ny, "n_mode": deck.n_mode,
            "ppc": deck.species[0].npart_per_cell, "moving_window": deck.move_window,
            "l2": "state larger than L2 (fields 15 x (nx+10)(ny+10) M complex + particles)",
            "parallelism": f"replicas x{args.gpus}", "rng": getattr(args, "rng", "kiss")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--deck", default="wakefield", choices=["wakefield", "thermal", "large"])
    ap.add_argument("--modes", type=int, default=None, help="wakefield deck with m = 0..modes-1 (profiling)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--eager", action="store_true", help="no CUDA graphs")
    ap.add_argument("--rng", default="kiss", choices=["kiss", "counter"],
                    help="species load and window injection: host KISS stream or device counter stream")
    ap.add_argument("--fp64-steps", type=int, default=-1,
                    help="steps of the plain FP64 form timed beside the mixed form "
                         "(-1: the same K steps, compared with the mixed result; 0: skip)")
    ap.add_argument("--window-start", type=int, default=1100,
                    help="first step of the moving-window-phase leg (0: skip the leg)")
    ap.add_argument("--window-steps", type=int, default=32)
    ap.add_argument("--no-serve-leg", dest="serve_leg", action="store_false",
                    help="skip the scan-serving leg of the default line")
    ap.add_argument("--serve", action="store_true", help="parameter-scan serving benchmark")
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--arrival", type=float, default=0.5, help="mean Poisson arrival gap (s)")
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--max-batch", type=int, default=16)
    ap.add_argument("--fp64-sample", type=int, default=3)
    ap.add_argument("--fp64-steps-max", type=int, default=100)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.serve:
        return run_serve(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi, build
    build.build()
    lib = cg.load()
    form = args.form
    if form == "auto":
        form = "fp64"
        probe = build_deck("thermal", "mixed")
        g = probe.grid_desc()
        sp = probe.species_descs()
        h = C.c_void_p()
        rc = lib.cyl_create(C.byref(g), sp, 1, None, 0, None, C.byref(h))
        if rc == abi.CYL_OK:
            lib.cyl_destroy(h)
            form = "mixed"
    deck = build_deck(args.deck, form, args.modes)
    parts, rng = cg.host_load(deck)
    if args.rng == "counter":
        # species loaded and window columns injected on the device from the
        # counter stream (profiling of the device injector; the e2e and CPU
        # legs keep the host KISS load)
        run = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=deck.seed)
    else:
        run = cg.Run(deck, particles=parts, rng=rng)
    graph = not args.eager
    tile = None
    if form == "mixed":
        tile = run.tune_tiles()  # the push tile shape, timed on the initial state

    run.step(args.warmup, graph=False)
    run.kernel_timing()  # reset counters
    s0 = run.state()
    n_start = sum(s0.n_live[i] for i in range(len(deck.species)) if not deck.species[i].immobile)
    clocks = ClockSampler(local)
    # CUDA events on the handle's own stream bracket the timed steps
    ext = torch.cuda.ExternalStream(run.stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    ev0.record(ext)
    run.step(args.steps, graph=graph)
    ev1.record(ext)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    elapsed = ev0.elapsed_time(ev1) * 1e-3
    wall = t1 - t0
    push_ms, launches = run.kernel_timing()
    s1 = run.state()
    n_end = sum(s1.n_live[i] for i in range(len(deck.species)) if not deck.species[i].immobile)
    psteps = 0.5 * (n_start + n_end) * args.steps
    from cylindrical_epoch_gb300.replicas import reduce_replicas
    elapsed, psteps, value = reduce_replicas(elapsed, psteps, dist, "cuda")

    # roofline of the dominant kernel (push + deposit): algorithmic bytes per
    # particle-step = particle state in + out + amortised field read (6 E/B
    # mode arrays) and current read-modify-write (3 FP64 J mode arrays) per
    # cell.  FP64 form: 7 x 8 B read + 6 x 8 B written, E/B 16 B per complex.
    # Mixed form: 32 B read (int32 cell, FP32 offset, y, z, u(3), w) + 28 B
    # written, E/B 8 B per complex (FP32 storage), J 16 B.
    M = deck.n_mode
    ppc = deck.species[0].npart_per_cell
    if form == "fp64":
        per_particle = 104.0 + (6 * 16 + 3 * 16 * 2) * M / ppc
    else:
        per_particle = 60.0 + (6 * 8 + 3 * 16 * 2) * M / ppc
    nparts = 0.5 * (n_start + n_end)
    peak, peak_kind = _peaks()
    achieved = per_particle * nparts / (push_ms * 1e-3) / 1e9 if push_ms > 0 else None
    prof = _profile_traffic(form, M, ppc)
    traffic = None
    if prof and prof.get("bytes_per_particle"):
        traffic = prof["bytes_per_particle"] * nparts
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "peak_kind": peak_kind, "kernel": "k_push_tiles" if form == "mixed" else "k_push_fp64",
                "kernel_ms": push_ms, "algorithmic_bytes_per_particle_step": per_particle}

    fp64 = None
    accuracy = None
    if form == "mixed" and args.fp64_steps != 0:
        # the plain FP64 form on the same deck, seed and steps; with the whole
        # K steps (the default) its final state is compared with the mixed run
        k64 = args.steps if args.fp64_steps < 0 else args.fp64_steps
        d64 = build_deck(args.deck, "fp64", args.modes)
        r64 = cg.Run(d64, particles=parts, rng=rng)
        r64.step(args.warmup, graph=False)
        s64a = r64.state()
        n64a = sum(s64a.n_live[i] for i in range(len(d64.species)) if not d64.species[i].immobile)
        ext64 = torch.cuda.ExternalStream(r64.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ext64)
        r64.step(k64, graph=graph)
        e1.record(ext64)
        torch.cuda.synchronize()
        dt64 = e0.elapsed_time(e1) * 1e-3
        s64 = r64.state()
        n64 = sum(s64.n_live[i] for i in range(len(d64.species)) if not d64.species[i].immobile)
        fp64 = {"value": 0.5 * (n64a + n64) * k64 / dt64, "steps": k64, "ms_per_step": 1e3 * dt64 / k64,
                "note": "plain FP64 form, the same steps [W, W+K) of the same deck, CUDA events"}
        if k64 == args.steps:
            from cylindrical_epoch_gb300.diagnostics import compare_runs
            accuracy = dict(against="plain FP64 GPU form, same deck, seed and steps (the FP64 form matches "
                                    "the oracle to 1e-10 in tests/)", **compare_runs(run, r64, deck))
        r64.close()

    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(deck, parts, rng, args.steps, graph, tile[0] if tile else None)
        if dist:
            e2e["value"] = reduce_replicas(e2e["seconds"], e2e["psteps"], dist, "cuda")[2]
        if fp64 is not None:
            # the FP64 form end to end as well: the figure at the reference's precision
            e64 = e2e_run(build_deck(args.deck, "fp64", args.modes), parts, rng, fp64["steps"], graph)
            if dist:
                e64["value"] = reduce_replicas(e64["seconds"], e64["psteps"], dist, "cuda")[2]
            fp64["e2e"] = {"value": e64["value"], "unit": "particle-steps/s",
                           "h2d_bytes_per_step": e64["h2d"] / fp64["steps"],
                           "d2h_bytes_per_step": e64["d2h"] / fp64["steps"], "phases_s": e64["phases_s"]}
    window = None
    if form == "mixed" and args.deck == "wakefield" and args.window_start > 0:
        window = window_phase(args, parts, rng, graph, tile[0] if tile else None)
    serving = None
    if rank == 0 and world == 1 and form == "mixed" and args.deck == "wakefield" and args.serve_leg:
        serving = serving_leg(args)
    base = None
    if rank == 0 and world == 1 and not args.no_cpu:
        base = cpu_baseline(build_deck(args.deck, "fp64", args.modes), parts, rng)

    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form == "fp64" else "f32+f64",
            "data": "synthetic", "config": dict(_config(args, deck, form), tile_shape=tile[1] if tile else None),
            "roofline": roofline, "clocks": clk, "gpu_launches": launches,
            "particles": nparts, "host_wall_s": wall, "timing": "CUDA events on the handle's stream",
        }
        if e2e:
            line["e2e"] = {"value": e2e["value"], "unit": "particle-steps/s",
                           "h2d_bytes_per_step": e2e["h2d"] / args.steps,
                           "d2h_bytes_per_step": e2e["d2h"] / args.steps,
                           "phases_s": e2e["phases_s"]}
        if base:
            line["cpu_baseline"] = base
        if fp64:
            line["fp64_form"] = fp64
            line["mixed_over_fp64"] = value / fp64["value"]
        if accuracy:
            line["accuracy"] = accuracy
        if window:
            line["window_phase"] = window
        if serving:
            line["serving"] = serving
        print(json.dumps(line))
    run.close()
    if dist:
        dist.destroy_process_group()
    return 0


def window_phase(args, parts, rng, graph, tile_shape):
    """The moving-window phase of the wakefield deck: both forms stepped
    (untimed) from t = 0 to step S (after the window has started moving:
    injection, removal and field shifts every step or two), then steps
    [S, S + k) timed with CUDA events on each run's stream, and the mixed
    state compared with the FP64 state there."""
    import torch
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300.diagnostics import compare_runs
    S, k = args.window_start, args.window_steps
    out = {"steps": [S, S + k]}
    runs = {}
    for form in ("mixed", "fp64"):
        d = build_deck(args.deck, form, args.modes)
        r = cg.Run(d, particles=parts, rng=rng)
        if form == "mixed" and tile_shape is not None:
            r.tune_tiles(tile_shape)
        r.step(S, graph=graph)
        s0 = r.state()
        mob = [i for i in range(len(d.species)) if not d.species[i].immobile]
        n0 = sum(s0.n_live[i] for i in mob)
        ext = torch.cuda.ExternalStream(r.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        r.kernel_timing()
        torch.cuda.synchronize()
        e0.record(ext)
        r.step(k, graph=graph)
        e1.record(ext)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) * 1e-3
        push_ms, _ = r.kernel_timing()
        s1 = r.state()
        n1 = sum(s1.n_live[i] for i in mob)
        out[form] = {"value": 0.5 * (n0 + n1) * k / dt, "unit": "particle-steps/s", "ms_per_step": 1e3 * dt / k,
                     "push_ms": push_ms, "n_shifts": [int(s0.n_shifts), int(s1.n_shifts)]}
        runs[form] = (r, d)
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    rm, dm = runs["mixed"]
    out["accuracy"] = dict(against="plain FP64 GPU form, same deck, seed and steps", **compare_runs(rm, runs["fp64"][0], dm))
    for r, _ in runs.values():
        r.close()
    return out


def e2e_run(deck, parts, rng, steps, graph, tile_shape=None):
    """The same run through the C ABI with host buffers: the initial state
    is copied from pinned host memory, every 16 steps the diagnostics are
    read back, and the final particles and fields are copied to the host,
    all inside the timed region.  The steps are enqueued without a sync
    (cyl_step_async) and each chunk's diagnostics are read one chunk later
    (cyl_diagnostics_async / _read), so the host's preparation of a chunk
    overlaps the device's work on the one before; every read's device
    error word is checked."""
    import numpy as np
    import torch
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi
    pinned = []
    for p in parts:
        q = cg.Particles(0)
        for k in q.__slots__:
            src = getattr(p, k)
            t = torch.empty(src.shape[0], dtype=torch.float64 if src.dtype == np.float64 else torch.int64,
                            pin_memory=True)
            a = t.numpy()
            a[:] = src
            setattr(q, k, a)
        pinned.append(q)
    h2d = sum(sum(getattr(p, k).nbytes for k in p.__slots__) for p in pinned)
    # pinned destinations of the final download, sized for the capacity
    caps = [int(sd.capacity) for sd in deck.species_descs()]
    outs = []
    for cap in caps:
        q = cg.Particles(0)
        for k in q.__slots__:
            t = torch.empty(max(cap, 1), dtype=torch.int64 if k == "id" else torch.float64, pin_memory=True)
            setattr(q, k, t.numpy())
        outs.append(q)
    shape = (deck.n_mode, deck.ny + 2 * abi.NG, deck.nx + 2 * abi.NG)
    fouts = [torch.empty(shape, dtype=torch.complex128, pin_memory=True).numpy() for _ in range(6)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run = cg.Run(deck, particles=pinned, rng=rng)
    t_up = time.perf_counter()
    if deck.precision == abi.PREC_MIXED:
        # the tile shape this process timed for this deck shape (the request
        # loop likewise times each deck shape once per process), else timed now
        run.tune_tiles(tile_shape)
    t_tune = time.perf_counter()
    d2h = 0
    left = steps
    pending = 0
    while left > 0:
        k = min(16, left)
        if graph:
            run.step_async(k)
        else:
            run.step(k, graph=False)
        if pending:
            assert run.diagnostics_read().device_error == 0
            pending -= 1
        run.diagnostics_async()
        pending += 1
        d2h += 8 * 8 + 4
        left -= k
    while pending:
        assert run.diagnostics_read().device_error == 0
        pending -= 1
    t_steps = time.perf_counter()
    outp = [run.particles(i, out=outs[i]) for i in range(len(deck.species))]
    fields = [run.field(n, out=fouts[j]) for j, n in enumerate(("exm", "erm", "etm", "bxm", "brm", "btm"))]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    s = run.state()
    d2h += sum(sum(getattr(p, k).nbytes for k in p.__slots__) for p in outp)
    d2h += sum(f.nbytes for f in fields)
    n0 = sum(p.n for p in parts)
    n1 = sum(s.n_live[i] for i in range(len(deck.species)))
    run.close()
    # per-step host inputs (step records, laser sources, injected particles)
    # are copied inside cyl_step; count their bytes
    h2d += steps * (512 + 4 * 8 * (deck.ny + 1))
    return {"seconds": t1 - t0, "psteps": 0.5 * (n0 + n1) * steps, "value": 0.5 * (n0 + n1) * steps / (t1 - t0),
            "h2d": h2d, "d2h": d2h,
            "phases_s": {"create_and_upload": t_up - t0, "tune_tiles": t_tune - t_up, "steps": t_steps - t_tune,
                         "download": t1 - t_steps}}


if __name__ == "__main__":
    sys.exit(main())
