"""Benchmark: the batched Life-like ensemble on one GB300 (weak scaling over GPUs).

Workload (per GPU): 4096 independent Life-like lattices (LifelikeCA), each with
a rule drawn uniformly from the 2**18 B/S rules, width and height drawn
uniformly from {64, 128, 256, 512, 1024}, Bernoulli(p ~ U[0.1, 0.6]) cells --
all seeded (``xentica_gb300.batch.ensemble_workload``).  One *step* advances
every lattice by 256 generations: one CUDA-graph launch of the resident
kernel.  Inputs (~645 MB of cells, one byte each) exceed the 129 MB L2, so no
flush is needed between steps.

Reported (one JSON line on rank 0):
  value   cell-updates/s over the K timed steps, device time (CUDA events on
          the launching stream), inputs resident in HBM;
  e2e     the same through ``xk_batch_run`` with pinned host buffers: every
          cell crosses the host link in and out inside the timed region (the
          largest lattices by the copy engines around their launches, the
          others read and written by their kernels), 256 generations between;
  plain   the same lattices with one launch per lattice per generation;
  roofline, cpu_baseline, clocks, gpu_launches as the benchmark contract asks.

  parity  one lattice of each of the 25 size classes, snapshotted before one
          more timed-configuration step (the tuned band, the captured graph)
          and compared with the oracle after it, outside the timed region;
  extras  the other configurations, each with its own value, e2e, roofline,
          cpu_baseline, clocks and parity: Life 512^2 (1000 generations per
          launch), EvoLife 1920x1080 with a rendered frame every generation,
          mass transfer 256^3 with a projection frame and the total checked
          every generation, the serving loop (Poisson arrivals, p50/p99
          latency, a sweep of offered loads), ShiftingSands, GameOfLifeColor
          1920x1080 with a frame every generation, NoiseTV 1920x1080 and
          GraviCowboys 1920x1080 with a frame every generation.
          ``--extras none`` leaves them out.

``--workload life512 | evolife | mass | serve | sands | lifecolor | noise | gravity`` prints one of the extras as
its own line (with the given ``--steps``/``--warmup``).  ``--impl reference``
times the reference's own kernels (its translator's LifelikeCA source compiled
for the CPU, ``oracle/_ref``) on the host cores instead, with the same metric.
"""
import argparse
import json
import multiprocessing
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_ALG = 2.0      # reference-layout bytes per cell-update (read + write one uint8)
METRIC = "cell-updates/s (batched Life-like ensemble)"


def parse():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--generations", type=int, default=256)
    ap.add_argument("--seed", type=int, default=2041)
    ap.add_argument("--plain-generations", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--requests", type=int, default=256, help="serve: requests in the run")
    ap.add_argument("--mass-side", type=int, default=256, help="mass: lattice side (a cube)")
    ap.add_argument("--load", type=float, default=0.7,
                    help="serve: offered load as a fraction of the measured capacity")
    ap.add_argument("--rate", type=float, default=100.0,
                    help="serve: also run at this fixed arrival rate (requests/s; 0: no)")
    ap.add_argument("--quantum", type=int, default=128, help="serve: generations per round")
    ap.add_argument("--sweep", default="", help="serve: extra offered loads after the main run, "
                                                "comma-separated (e.g. 0.3,0.5,0.9)")
    ap.add_argument("--extras", default="life512,evolife,mass,serve,sands,lifecolor,noise,gravity",
                    help="default run: the other configurations measured after the ensemble "
                         "(comma-separated, or 'none')")
    ap.add_argument("--serve-budget-gb", type=int, default=16, help="serve: HBM budget (GiB)")
    ap.add_argument("--workload", choices=("ensemble", "life512", "evolife", "mass", "serve",
                                           "sands", "lifecolor", "noise", "gravity"),
                    default="ensemble",
                    help="ensemble: the batched Life-like ensemble (default); life512: Conway's "
                         "Life 512x512 torus, 1000 generations per step; evolife: EvoLife "
                         "1920x1080 with a render every generation; mass: 3-D sand transfer "
                         "256^3 with the total checked every generation; serve: Poisson "
                         "arrivals of 2-D/3-D requests through the serving loop")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (one process per GPU; barrier + max only, no data path)

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = "nccl" if os.environ.get("XK_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
            if backend == "nccl":
                import torch
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, value):
        if not self.pg:
            return value
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region

class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        loaded = [v for v in sm if v > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------

def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_cell():
    """DRAM bytes per cell per launch of the resident kernel from the committed
    ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "life_resident_traffic.json")
    if os.path.exists(path):
        with open(path) as fh:
            return float(json.load(fh)["dram_bytes_per_cell"])
    return None


def committed_traffic(name):
    """DRAM bytes per launch of a kernel from its committed ncu summary
    (``profiles/<name>_traffic.json``), or None."""
    path = os.path.join(ROOT, "profiles", name + "_traffic.json")
    if os.path.exists(path):
        with open(path) as fh:
            return float(json.load(fh)["dram_bytes_per_launch"])
    return None


def workload(args, rank):
    from xentica_gb300.batch import ensemble_workload
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(min(32, os.cpu_count() or 1)) as pool:
        return ensemble_workload(args.instances, args.seed + 7919 * rank, pool=pool)


def cpu_sample(widths, heights, rules, cells, offsets, seconds, threads):
    """Time the reference's own kernels (oracle/_ref) when built, else the
    oracle port, on one lattice of each size class; returns a dict."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_build
    manifest = ref_build.available()
    seen, picks = set(), []
    for i in range(len(widths)):
        key = (int(widths[i]), int(heights[i]))
        if key not in seen:
            seen.add(key)
            picks.append(i)
    sample_cells = int(sum(int(widths[i]) * int(heights[i]) for i in picks))
    if manifest:
        import ctypes
        kind = "reference"
        libs = {}
        states = []
        for i in picks:
            w, h = int(widths[i]), int(heights[i])
            entry = manifest["lifelike_%dx%d" % (w, h)]
            lib = libs.get((w, h)) or ctypes.CDLL(os.path.join(ref_build.REF_DIR, entry["so"]))
            libs[(w, h)] = lib
            n = w * h
            fld = np.zeros(n * 9 + 1, dtype=np.uint8)
            fld[:n] = cells[offsets[i]:offsets[i] + n]
            col = np.zeros(n * 3, dtype=np.int32)
            states.append((lib, fld, col, n, int(rules[i])))

        def one_generation():
            for lib, fld, col, n, rule in states:
                lib.xkref_emit(ctypes.c_int(threads), ctypes.c_void_p(fld.ctypes.data), ctypes.c_int(n))
                lib.xkref_absorb(ctypes.c_int(threads), ctypes.c_void_p(fld.ctypes.data),
                                 ctypes.c_void_p(col.ctypes.data), ctypes.c_int(rule), ctypes.c_int(n))
    else:
        import oracle as O
        kind = "port"
        states = []
        for i in picks:
            w, h = int(widths[i]), int(heights[i])
            topo = O.Topology((w, h))
            fld = topo.field(cells[offsets[i]:offsets[i] + w * h], np.uint8)
            states.append((topo, fld, np.zeros(w * h * 3, np.int32), int(rules[i])))

        def one_generation():
            for topo, fld, col, rule in states:
                O.life_run(topo, fld, col, 1, born=rule & 511, sustain=rule >> 9, threads=threads)
    one_generation()
    gens, t0 = 0, time.perf_counter()
    while True:
        one_generation()
        gens += 1
        el = time.perf_counter() - t0
        if el >= seconds and gens >= 2:
            break
    rate = sample_cells * gens / el
    return {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": kind, "seconds": el,
            "sample": "%d lattices (one per size class, %d cells) x %d generations, %.1f s, "
                      "%s" % (len(picks), sample_cells, gens, el,
                              "reference LifelikeCA kernels compiled for the CPU (OpenMP)"
                              if kind == "reference" else "oracle port (OpenMP)")}


def run_reference_arm(args, dist):
    if dist.rank != 0:
        return
    # one lattice of every size class of the --instances workload (its first
    # member of the class), cells exactly as the whole workload draws them
    from xentica_gb300.batch import ensemble_seeds
    all_w, all_h, all_r, all_d, all_s = ensemble_seeds(args.instances, args.seed)
    seen, picks = set(), []
    for i in range(args.instances):
        key = (int(all_w[i]), int(all_h[i]))
        if key not in seen:
            seen.add(key)
            picks.append(i)
    widths, heights, rules = all_w[picks], all_h[picks], all_r[picks]
    cells = np.concatenate([
        (np.random.RandomState(int(all_s[i])).random_sample(int(all_w[i]) * int(all_h[i]))
         < all_d[i]).astype(np.uint8) for i in picks])
    offsets = np.concatenate([[0], np.cumsum(widths.astype(np.int64) * heights)[:-1]])
    threads = os.cpu_count()
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_sample(widths, heights, rules, cells, offsets, 0.0, threads)
    results = [cpu_sample(widths, heights, rules, cells, offsets, per_step, threads)
               for _ in range(max(1, args.steps))]
    value = statistics.median(r["value"] for r in results)
    base = dict(results[-1])
    base.pop("seconds")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * statistics.median(r["seconds"] for r in results),
            "ms_per_step_note": "one step is a bounded sample of the workload (one lattice "
                                "of each of its %d size classes for a fixed time, each class "
                                "weighted once rather than by its share of the ensemble), not "
                                "the whole ensemble" % len(picks),
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded)",
            "config": {"workload": "ensemble: LifelikeCA lattices, sides {64..1024}^2, "
                                   "random B/S rules, Bernoulli(p~U[0.1,0.6])",
                       "instances": args.instances, "generations": args.generations},
            "cpu_baseline": dict(base, value=value),
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reference_gpu_sample(ens, cells, generations=2):
    """The reference's own generated LifelikeCA kernels compiled for sm_103a
    (``oracle/ref_gpu.py``), launched as the reference's step() does (emit
    then absorb per lattice per generation, PyCUDA's block and grid) over every
    lattice of the ensemble for ``generations`` generations after one warm-up
    generation; their cells are compared with this library's after the same
    generations.  None when the comparator is not built."""
    import ctypes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu
    path = ref_gpu.available()
    if not path:
        return None
    lib = ctypes.CDLL(path)
    lib.xkrefg_create.restype = ctypes.c_void_p
    lib.xkrefg_create.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
    lib.xkrefg_step.restype = ctypes.c_float
    lib.xkrefg_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.xkrefg_download.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.xkrefg_destroy.argtypes = [ctypes.c_void_p]
    w = np.ascontiguousarray(ens.widths, dtype=np.int32)
    h = np.ascontiguousarray(ens.heights, dtype=np.int32)
    r = np.ascontiguousarray(ens.rules, dtype=np.int32)
    cells = np.ascontiguousarray(cells, dtype=np.uint8)
    handle = lib.xkrefg_create(ens.count, w.ctypes.data, h.ctypes.data, r.ctypes.data,
                               cells.ctypes.data)
    if not handle:
        return {"unavailable": "reference kernels missing for a lattice size, or CUDA failed"}
    lib.xkrefg_step(handle, 1)                       # module load, first launches
    ms = lib.xkrefg_step(handle, generations)
    out = np.empty(ens.total_cells, dtype=np.uint8)
    lib.xkrefg_download(handle, out.ctypes.data)
    lib.xkrefg_destroy(handle)
    if ms <= 0:
        return {"unavailable": "a reference kernel launch failed"}
    ens.upload(cells)
    ens.step(1 + generations)
    exact = bool(np.array_equal(ens.download(), out))
    return {"value": float(ens.total_cells) * generations / (ms / 1000.0), "unit": "cell-updates/s",
            "generations": generations, "launches": 2 * ens.count * generations,
            "bit_exact_vs_ours": exact,
            "kind": "the reference's generated LifelikeCA emit/absorb kernels (translator "
                    "output, nvcc -w for sm_103a), one emit and one absorb launch per lattice "
                    "per generation with PyCUDA's block/grid, launched from a C loop"}


def ensemble_parity(ens, widths, heights, G):
    """One lattice of each size class: snapshot, one more step of G
    generations in the timed configuration, the oracle from the snapshot."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    picks, seen = [], set()
    for i in range(ens.count):
        key = (int(widths[i]), int(heights[i]))
        if key not in seen:
            seen.add(key)
            picks.append(i)
    before = ens.download()
    ens.step(G)
    after = ens.download()
    exact = True
    for i in picks:
        w, h, rule = int(ens.widths[i]), int(ens.heights[i]), int(ens.rules[i])
        topo = O.Topology((w, h))
        fld = topo.field(ens.lattice(before, i).ravel(), np.uint8)
        O.life_run(topo, fld, np.zeros(topo.cells * 3, np.int32), G, born=rule & 511,
                   sustain=rule >> 9)
        exact &= bool(np.array_equal(fld[:topo.cells], ens.lattice(after, i).ravel()))
    return {"lattices": len(picks), "size_classes": len(seen), "generations": G,
            "band": ens.band, "bit_exact": exact,
            "note": "one lattice of every size class, from the state after the timed and the "
                    "end-to-end steps, one more %d-generation step of the timed configuration "
                    "against the oracle" % G}


def run_ours(args, dist):
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    t_host = time.perf_counter()
    widths, heights, rules, dens, cells = workload(args, dist.rank)   # before any GPU call
    host_seed_s = time.perf_counter() - t_host
    xk_build.build()
    nat.set_device(dist.local)
    from xentica_gb300.batch import Ensemble, ensemble_seeds
    ens = Ensemble(widths, heights, rules)
    total = ens.total_cells
    G = args.generations
    # the same cells drawn on the device (MT19937 per lattice), checked bit for bit
    seeds = ensemble_seeds(args.instances, args.seed + 7919 * dist.rank)[4]
    ens.seed_bernoulli(seeds, dens)
    seed_ms = ens.seed_bernoulli(seeds, dens)
    seed_exact = bool(np.array_equal(ens.download(), cells))
    if not seed_exact:
        raise SystemExit("device seeding disagrees with the host draw")
    ens.upload(cells)
    rows_per_band = ens.tune(G)
    ens.upload(cells)
    # self-check of the timed paths on this workload: batched == e2e
    ens.step(G)
    after = ens.download()
    pin_in, pin_out = nat.PinnedBuffer(total), nat.PinnedBuffer(total)
    pin_in.array[:] = cells
    ens.run(pin_in.array, pin_out.array, G)
    if not np.array_equal(pin_out.array, after):
        raise SystemExit("e2e path disagrees with the device path")
    ens.upload(cells)
    for _ in range(args.warmup):
        ens.step(G)
    clocks = Clocks(dist.local)
    time.sleep(0.6)                       # let the sampler start before the timed region
    dist.barrier()
    t_wall = time.perf_counter()
    nat.load().xk_range_push(b"timed")
    step_ms = [ens.step(G) for _ in range(args.steps)]
    nat.load().xk_range_pop()
    wall = time.perf_counter() - t_wall
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    updates = float(total) * G * args.steps
    value = updates * dist.world / dev_s
    # end to end: pinned host in -> device -> 256 generations -> pinned host
    # out, before any CPU-side checking (the oracle's OpenMP threads spin
    # after their work and would compete with the host thread that queues the
    # copies)
    ens.run(pin_in.array, pin_out.array, G)
    dist.barrier()
    e2e_ms = [ens.run(pin_in.array, pin_out.array, G) for _ in range(args.steps)]
    dist.barrier()
    e2e_s = dist.max(sum(e2e_ms) / 1000.0)
    e2e_value = updates * dist.world / e2e_s
    parity = ensemble_parity(ens, widths, heights, G)
    # plain form: one launch per lattice per generation
    ens.upload(cells)
    pg = args.plain_generations
    plain_ms = ens.step_plain(pg)
    plain_value = float(total) * pg / (plain_ms / 1000.0)
    ref_gpu = reference_gpu_sample(ens, cells, pg)
    if ref_gpu and "value" in ref_gpu:
        ref_gpu["batched_over_reference_gpu"] = value / dist.world / ref_gpu["value"]
    launches = ens.launches(G) * args.steps
    peak, peak_kind = measured_peak()
    mean_ms = statistics.mean(step_ms)
    achieved = B_ALG * total * G / (mean_ms / 1000.0) / 1e9
    tpc = traffic_per_cell()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": tpc * total if tpc is not None else None,
                "kernel": "xk_k_life_resident<true> (all instance classes of one graph)",
                "algorithmic_bytes_per_launch": B_ALG * total * G,
                "note": "B_alg = 2 B per cell-update (the reference's uint8 state read and "
                        "written once per generation); the kernel keeps every lattice in "
                        "shared memory for all 256 generations, so frac > 1 is "
                        "reference-format effective, not DRAM traffic",
                # the stricter bit-packed figure: 2 x 1/8 B per cell-update (one bit
                # read and written per cell and generation)
                "bit_packed": {"bytes_per_cell_update": 0.25,
                               "achieved": 0.25 * achieved / B_ALG,
                               "frac": 0.25 * achieved / B_ALG / peak}}
    line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded Bernoulli lattices, random rules)",
            "config": {"workload": "ensemble of %d LifelikeCA lattices x %d generations per step"
                                   % (args.instances, G),
                       "instances": args.instances, "generations_per_step": G,
                       "cells": total, "sides": [64, 128, 256, 512, 1024],
                       "l2": "inputs (%.0f MB) larger than L2, no flush" % (total / 1e6),
                       "rows_per_band": rows_per_band, "parallelism": "replicas x%d" % dist.world},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": total,
                    "d2h_bytes_per_step": total, "ms_per_step": e2e_s * 1000 / args.steps},
            "plain": {"value": plain_value, "unit": "cell-updates/s", "generations": pg,
                      "batched_over_plain": value / dist.world / plain_value},
            "reference_gpu": ref_gpu,
            "seeding": {"device_ms": seed_ms, "host_s": host_seed_s, "bit_exact": seed_exact,
                        "note": "the %d lattices' Bernoulli cells drawn on the device (one "
                                "MT19937 stream per lattice, NumPy's random_sample) against "
                                "the host draw (RandomState per lattice, %d processes)"
                                % (args.instances, min(32, os.cpu_count() or 1))},
            "parity": parity,
            "gpu_launches": launches, "wall_s": wall, "roofline": roofline, "clocks": clk}
    if dist.rank == 0:
        line["cpu_baseline"] = cpu_sample(widths, heights, rules, cells, ens.offsets,
                                          args.cpu_seconds, os.cpu_count())
        line["cpu_baseline"].pop("seconds")
    pin_in.release()
    pin_out.release()
    del ens
    extras = [e.strip() for e in args.extras.split(",") if e.strip() and e.strip() != "none"]
    if extras:
        line["extras"] = {}
        small = argparse.Namespace(**vars(args))
        small.cpu_seconds = 4.0
        for name in extras:
            fn = {"life512": life512_line, "evolife": evolife_line, "mass": mass_line,
                  "serve": serve_line, "sands": sands_line, "lifecolor": lifecolor_line,
                  "noise": noise_line, "gravity": gravity_line}[name]
            steps, warmup = {"life512": (10, 3), "evolife": (100, 3), "mass": (5, 3),
                             "serve": (None, 3), "sands": (10, 3), "lifecolor": (10, 3),
                             "noise": (5, 3), "gravity": (10, 3)}[name]
            small.steps, small.warmup = steps, warmup
            if name == "serve" and not small.sweep:
                small.sweep = "0.3,0.5,0.9"
            sub = fn(small, dist)
            if sub is not None:
                line["extras"][name] = sub
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def c2_experiment():
    """The EvoLife configuration: 1920x1080 torus, every cell seeded with a
    uniform random energy (0..255), genome (0..2^18-1) and random state
    (0..2^16-1) -- PrimordialSoup over the reference's EvoLife
    (examples/evolife.py:20-128) with its default death_speed 15, max_genes 9
    and mutation_prob 0, and CrossbreedingExperiment's MovingAverage fades
    18/3 (examples/evolife.py:137-144)."""
    from xentica_gb300 import core, seeds
    from xentica_gb300.seeds.random import RandInt

    class PrimordialEvoLife(core.Experiment):
        word = "EVOLIFE PRIMORDIAL SOUP 1920X1080"
        size = (1920, 1080)
        zoom = 1
        pos = [0, 0]
        fade_in = 18
        fade_out = 3
        death_speed = 15
        max_genes = 9
        mutation_prob = 0.0
        seed = seeds.patterns.PrimordialSoup(vals={
            "energy": RandInt(0, 255), "rule": RandInt(0, 2 ** 18 - 1),
            "rng": RandInt(0, 2 ** 16 - 1)})
    return PrimordialEvoLife


def evolife_line(args, dist):
    """EvoLife 1920x1080 (c2_experiment): K steps of 100 generations (K = 100
    in the default line: the configuration's 10 000 generations), each
    generation followed by a full-frame render (RendererPlain, zoom 1) into a
    device frame buffer -- the reference's step() + render() pair per frame;
    the step kernel writes that frame itself (one launch per generation).
    e2e: the state and colours loaded from the host, then 100 generations
    with every frame copied to page-locked host memory (min(K, 10) times).
    Parity: the oracle started from the GPU state after the timed steps, two
    more generations (state, colours and both frames compared)."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    from xentica_gb300.core.canonical import EvoLifeProgram
    import torch
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()
    model = EvoLifeProgram(c2_experiment())
    W, H = model.size
    model.set_viewport((W, H))
    n = model.cells_num
    gens = 100
    fb = W * H * 3
    dev_frames = torch.empty(gens * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)

    def step_device():
        return model.gpu.step_frames(gens, W, H, 1, 0, 0, dev_frames.data_ptr(), on_device=True)

    step_device()
    for _ in range(args.warmup):
        step_device()
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    lib.xk_range_push(b"timed")
    step_ms = [step_device() for _ in range(args.steps)]
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    # e2e: host state in, 100 generations, every frame to pinned host memory
    cells = model.gpu.arrays.cells.get()[:n].copy()
    colors = model.gpu.arrays.colors.get()
    host = nat.PinnedBuffer(gens * fb)
    frames = host.array.reshape(gens, fb)
    e2e = []
    e2e_steps = min(args.steps, 10)
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        model.gpu.load(cells, colors)
        model.gpu.step_frames(gens, W, H, 1, 0, 0, frames.reshape(-1))
        e2e.append(time.perf_counter() - t0)
    e2e_s = dist.max(sum(e2e))
    host.release()
    generations_done = gens * (1 + args.warmup + args.steps)
    peak, peak_kind = measured_peak()
    mean_ms = statistics.mean(step_ms)
    bytes_per_update = 8 * 2 + 12 * 2 + 3    # uint64 state r+w, int3 colour r+w, uint8 RGB pixel
    achieved = bytes_per_update * n * gens / (mean_ms / 1000.0) / 1e9
    line = {"metric": "cell-updates/s (EvoLife, frame every generation)", "value": value,
            "unit": "cell-updates/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded PrimordialSoup: uniform random energy, genome, RNG state)",
            "config": {"workload": "EvoLife 1920x1080 torus, uniform random genomes, "
                                   "death_speed 15, max_genes 9, MovingAverage(18, 3), "
                                   "100 generations per step, each followed by a 1920x1080 "
                                   "RendererPlain frame (uint8 RGB)",
                       "timed_generations": gens * args.steps,
                       "step_ms_range": [min(step_ms), max(step_ms)],
                       "first_timed_generation": gens * (1 + args.warmup),
                       "l2": "state + colours (41 MB) fit in L2; frames (622 MB per step) "
                             "stream to HBM"},
            "e2e": {"value": float(n) * gens * e2e_steps * dist.world / e2e_s,
                    "unit": "cell-updates/s", "h2d_bytes_per_step": n * 8 + n * 12,
                    "d2h_bytes_per_step": gens * fb,
                    "note": "state and colours loaded from the host, every frame copied to "
                            "page-locked host memory"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": committed_traffic("evolife"),
                         "kernel": "xk_k_evolife per generation (it also writes the zoom-1 "
                                   "uint8 frame)",
                         "algorithmic_bytes_per_generation": bytes_per_update * n,
                         "note": "B_alg = 43 B per cell-update (8 B state and 12 B colour read "
                                 "and written, 3 B uint8 RGB pixel written); the kernel is bound by "
                                 "integer instruction issue (genome crossover), not by HBM"},
            "gpu_launches": gens * args.steps, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        tpl = model.gpu.template
        info = tpl.color.extra
        topo = O.Topology(model.size)
        fld = topo.field(model.gpu.arrays.cells.get()[:n], np.uint64)
        col = model.gpu.arrays.colors.get()
        smooth = model.constants["SMOOTH_FACTOR"].value \
            if model.is_constant("SMOOTH_FACTOR") else 0
        got = model.step_frames(2)
        gpu_cells = model.gpu.arrays.cells.get()[:n]
        gpu_col = model.gpu.arrays.colors.get()
        exact, el = True, 0.0
        for g in range(2):
            t0 = time.perf_counter()
            O.evolife_run(topo, fld, col, 1, death_speed=15, max_genes=9, mutation_prob=0.0,
                          fade_in=info["fade_in"], fade_out=info["fade_out"],
                          smooth=info["smooth"])
            img = O.render(topo, col, W, H, smooth=smooth).astype(np.uint8)
            el += time.perf_counter() - t0
            exact &= bool(np.array_equal(got[g], img))
        exact &= bool(np.array_equal(gpu_cells, fld[:n])) and bool(np.array_equal(gpu_col, col))
        line["parity"] = {"generations_before": generations_done + gens,
                          "checked_generations": 2, "bit_exact": exact,
                          "note": "oracle started from the GPU state after the timed steps: "
                                  "cells, colours and both frames"}
        line["cpu_baseline"] = {"value": n * 2 / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "2 generations of the full lattice, each with its "
                                          "render, oracle (OpenMP)"}
        return line
    return None


def lifecolor_experiment():
    """GameOfLifeColor (examples/game_of_life.py:112-159) on a 1920x1080
    torus seeded as GOLExperimentColor seeds it (state, red, green, blue
    uniform), with its MovingAverage fades 255 / 10 (examples/game_of_life.py:
    255-276)."""
    from xentica_gb300 import core, seeds
    from xentica_gb300.seeds.random import RandInt

    class LifeColorSoup(core.Experiment):
        word = "LIFE IN COLOR 1920X1080"
        size = (1920, 1080)
        zoom = 1
        pos = [0, 0]
        fade_in = 255
        fade_out = 10
        smooth_factor = 1
        seed = seeds.patterns.PrimordialSoup(vals={
            "state": RandInt(0, 1), "red": RandInt(0, 255), "green": RandInt(0, 255),
            "blue": RandInt(0, 255)})
    return LifeColorSoup


def lifecolor_line(args, dist):
    """GameOfLifeColor 1920x1080: K steps of 100 generations, each generation
    with its zoom-1 frame written by the step kernel into a device buffer; the
    same model on the generic interpreter timed beside it (the path it took
    before it had a kernel of its own); e2e with every frame copied to
    page-locked host memory; parity: the oracle from the GPU state after the
    timed steps, two more generations (cells, colours, frames)."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    from xentica_gb300.core import canonical
    import torch
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()
    exp = lifecolor_experiment()
    model = canonical.LifeColorProgram(exp)
    assert type(model.gpu.template).__name__ == "LifeColorTemplate"
    W, H = model.size
    model.set_viewport((W, H))
    n = model.cells_num
    gens = 100
    fb = W * H * 3
    dev_frames = torch.empty(gens * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)

    def step_device():
        return model.gpu.step_frames(gens, W, H, 1, 0, 0, dev_frames.data_ptr(), on_device=True)

    step_device()
    for _ in range(args.warmup):
        step_device()
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    lib.xk_range_push(b"timed")
    step_ms = [step_device() for _ in range(args.steps)]
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    cells = model.gpu.arrays.cells.get()[:n].copy()
    colors = model.gpu.arrays.colors.get()
    # e2e: host state in, 100 generations, every frame to pinned host memory
    host = nat.PinnedBuffer(gens * fb)
    frames = host.array.reshape(gens, fb)
    e2e = []
    e2e_steps = min(args.steps, 5)
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        model.gpu.load(cells, colors)
        model.gpu.step_frames(gens, W, H, 1, 0, 0, frames.reshape(-1))
        e2e.append(time.perf_counter() - t0)
    e2e_s = dist.max(sum(e2e))
    host.release()
    # the generic interpreter on the same model and state (10 generations,
    # frames rendered by the generic renderer)
    os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
    try:
        vm_model = canonical.LifeColorProgram(exp)
    finally:
        del os.environ["XENTICA_GB300_TEMPLATE"]
    vm_model.set_viewport((W, H))
    vm_model.gpu.load(cells, colors)
    vm_frames = torch.empty(10 * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)
    vm_model.gpu.step_frames(10, W, H, 1, 0, 0, vm_frames.data_ptr(), on_device=True)
    vm_ms = vm_model.gpu.step_frames(10, W, H, 1, 0, 0, vm_frames.data_ptr(), on_device=True)
    del vm_model
    peak, peak_kind = measured_peak()
    mean_ms = statistics.mean(step_ms)
    bytes_per_update = 4 * 2 + 12 * 2 + 3    # uint32 state r+w, int3 colour r+w, uint8 RGB pixel
    achieved = bytes_per_update * n * gens / (mean_ms / 1000.0) / 1e9
    line = {"metric": "cell-updates/s (GameOfLifeColor, frame every generation)", "value": value,
            "unit": "cell-updates/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded PrimordialSoup: uniform state and colour channels)",
            "config": {"workload": "GameOfLifeColor 1920x1080 torus, MovingAverage(255, 10), "
                                   "100 generations per step, each followed by a 1920x1080 "
                                   "RendererPlain frame (uint8 RGB)",
                       "l2": "state + colours (33 MB) fit in L2; frames (622 MB per step) "
                             "stream to HBM"},
            "e2e": {"value": float(n) * gens * e2e_steps * dist.world / e2e_s,
                    "unit": "cell-updates/s", "h2d_bytes_per_step": n * 4 + n * 12,
                    "d2h_bytes_per_step": gens * fb,
                    "note": "state and colours loaded from the host, every frame copied to "
                            "page-locked host memory"},
            "interpreter": {"value": float(n) * 10 / (vm_ms / 1000.0), "unit": "cell-updates/s",
                            "note": "the same model on the generic interpreter (the reference's "
                                    "emit and absorb passes over 8 buffer planes), 10 "
                                    "generations with their frames"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": committed_traffic("lifecolor"),
                         "kernel": "xk_k_lifecolor per generation (it also writes the zoom-1 "
                                   "uint8 frame)",
                         "algorithmic_bytes_per_generation": bytes_per_update * n,
                         "note": "B_alg = 35 B per cell-update (4 B state and 12 B colour read "
                                 "and written, 3 B uint8 RGB pixel written)"},
            "gpu_launches": gens * args.steps, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        topo = O.Topology(model.size)
        fld = topo.field(model.gpu.arrays.cells.get()[:n], np.uint32)
        col = model.gpu.arrays.colors.get()
        got = model.step_frames(2)
        gpu_cells = model.gpu.arrays.cells.get()[:n]
        gpu_col = model.gpu.arrays.colors.get()
        exact, el = True, 0.0
        for g in range(2):
            t0 = time.perf_counter()
            O.lifecolor_run(topo, fld, col, 1, color=O._color(True, 255, 10, 1))
            img = O.render(topo, col, W, H, smooth=1).astype(np.uint8)
            el += time.perf_counter() - t0
            exact &= bool(np.array_equal(got[g], img))
        exact &= bool(np.array_equal(gpu_cells, fld[:n])) and bool(np.array_equal(gpu_col, col))
        line["parity"] = {"checked_generations": 2, "bit_exact": exact,
                          "note": "oracle started from the GPU state after the timed and "
                                  "end-to-end steps: cells, colours and both frames"}
        line["cpu_baseline"] = {"value": n * 2 / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "2 generations of the full lattice, each with its "
                                          "render, oracle (OpenMP)"}
        return line
    return None


def gravity_experiment():
    """GraviCowboys (examples/gravicowboys.py:20-71) on a 1920x1080 torus,
    every cell seeded as GraviCowboysExperiment seeds its patches (energy 0
    or 1, gravity 0), with the reference's MovingAverage fades."""
    from xentica_gb300 import core, seeds
    from xentica_gb300.seeds.random import RandInt

    class GraviSoup(core.Experiment):
        word = "LET IT GROOVE 1920X1080"
        size = (1920, 1080)
        zoom = 1
        pos = [0, 0]
        seed = seeds.patterns.PrimordialSoup(vals={"energy": RandInt(0, 1) * 1, "gravity": 0})
    return GraviSoup


def gravity_line(args, dist):
    """GraviCowboys 1920x1080: K steps of 100 generations, each generation
    with its zoom-1 frame written by the step kernel into a device buffer; the
    same model on the generic interpreter timed beside it; e2e with every
    frame copied to page-locked host memory; parity: the oracle from the GPU
    state after the timed steps, two more generations (cells, colours,
    frames)."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    from xentica_gb300.core import canonical
    import torch
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()
    exp = gravity_experiment()
    model = canonical.GravityProgram(exp)
    assert type(model.gpu.template).__name__ == "GravityTemplate"
    W, H = model.size
    model.set_viewport((W, H))
    n = model.cells_num
    gens = 100
    fb = W * H * 3
    dev_frames = torch.empty(gens * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)

    def step_device():
        return model.gpu.step_frames(gens, W, H, 1, 0, 0, dev_frames.data_ptr(), on_device=True)

    step_device()
    for _ in range(args.warmup):
        step_device()
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    lib.xk_range_push(b"timed")
    step_ms = [step_device() for _ in range(args.steps)]
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    cells = model.gpu.arrays.cells.get()[:n].copy()
    colors = model.gpu.arrays.colors.get()
    host = nat.PinnedBuffer(gens * fb)
    frames = host.array.reshape(gens, fb)
    e2e = []
    e2e_steps = min(args.steps, 5)
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        model.gpu.load(cells, colors)
        model.gpu.step_frames(gens, W, H, 1, 0, 0, frames.reshape(-1))
        e2e.append(time.perf_counter() - t0)
    e2e_s = dist.max(sum(e2e))
    host.release()
    os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
    try:
        vm_model = canonical.GravityProgram(exp)
    finally:
        del os.environ["XENTICA_GB300_TEMPLATE"]
    vm_model.set_viewport((W, H))
    vm_model.gpu.load(cells, colors)
    vm_frames = torch.empty(10 * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)
    vm_model.gpu.step_frames(10, W, H, 1, 0, 0, vm_frames.data_ptr(), on_device=True)
    vm_ms = vm_model.gpu.step_frames(10, W, H, 1, 0, 0, vm_frames.data_ptr(), on_device=True)
    del vm_model
    peak, peak_kind = measured_peak()
    mean_ms = statistics.mean(step_ms)
    bytes_per_update = 8 * 2 + 12 * 2 + 3    # uint64 state r+w, int3 colour r+w, uint8 RGB pixel
    achieved = bytes_per_update * n * gens / (mean_ms / 1000.0) / 1e9
    line = {"metric": "cell-updates/s (GraviCowboys, frame every generation)", "value": value,
            "unit": "cell-updates/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64+f32",
            "data": "synthetic (seeded PrimordialSoup: energy 0 or 1, gravity 0)",
            "config": {"workload": "GraviCowboys 1920x1080 torus, MovingAverage(255, 255), 100 "
                                   "generations per step, each followed by a 1920x1080 "
                                   "RendererPlain frame (uint8 RGB)",
                       "l2": "state + colours (41 MB) fit in L2; frames (622 MB per step) "
                             "stream to HBM"},
            "e2e": {"value": float(n) * gens * e2e_steps * dist.world / e2e_s,
                    "unit": "cell-updates/s", "h2d_bytes_per_step": n * 8 + n * 12,
                    "d2h_bytes_per_step": gens * fb,
                    "note": "state and colours loaded from the host, every frame copied to "
                            "page-locked host memory"},
            "interpreter": {"value": float(n) * 10 / (vm_ms / 1000.0), "unit": "cell-updates/s",
                            "note": "the same model on the generic interpreter (the reference's "
                                    "emit and absorb passes over 8 buffer planes), 10 "
                                    "generations with their frames"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": committed_traffic("gravity"),
                         "kernel": "xk_k_gravity per generation (it also writes the zoom-1 "
                                   "uint8 frame)",
                         "algorithmic_bytes_per_generation": bytes_per_update * n,
                         "note": "B_alg = 43 B per cell-update (8 B state and 12 B colour read "
                                 "and written, 3 B uint8 RGB pixel written)"},
            "gpu_launches": gens * args.steps, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        topo = O.Topology(model.size)
        fld = topo.field(model.gpu.arrays.cells.get()[:n], np.uint64)
        col = model.gpu.arrays.colors.get()
        got = model.step_frames(2)
        gpu_cells = model.gpu.arrays.cells.get()[:n]
        gpu_col = model.gpu.arrays.colors.get()
        exact, el = True, 0.0
        for g in range(2):
            t0 = time.perf_counter()
            O.gravity_run(topo, fld, col, 1, color=O._color(True, 255, 255, 1))
            img = O.render(topo, col, W, H, smooth=1).astype(np.uint8)
            el += time.perf_counter() - t0
            exact &= bool(np.array_equal(got[g], img))
        exact &= bool(np.array_equal(gpu_cells, fld[:n])) and bool(np.array_equal(gpu_col, col))
        line["parity"] = {"checked_generations": 2, "bit_exact": exact,
                          "note": "oracle started from the GPU state after the timed and "
                                  "end-to-end steps: cells, colours and both frames"}
        line["cpu_baseline"] = {"value": n * 2 / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "2 generations of the full lattice, each with its "
                                          "render, oracle (OpenMP)"}
        return line
    return None


def run_gravity(args, dist):
    line = gravity_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def noise_line(args, dist):
    """NoiseTV 1920x1080 (examples/noisetv.py:13-31): K steps of 1000
    generations (cells are independent, so one launch runs up to 1024
    generations of a cell in registers), and the viewer's form, 100
    generations each with its zoom-1 frame; the same model on the generic
    interpreter beside it; parity: the oracle from the GPU state, 1000 more
    generations and two with frames."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    from xentica_gb300 import core, seeds
    from xentica_gb300.core import canonical
    import torch
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()

    class Noise1080(core.Experiment):
        word = "PSHSHSHSH! 1920X1080"
        size = (1920, 1080)
        zoom = 1
        pos = [0, 0]
        seed = seeds.patterns.PrimordialSoup(vals={"rng": seeds.random.RandInt(0, 2 ** 16 - 1)})

    model = canonical.NoiseProgram(Noise1080)
    assert type(model.gpu.template).__name__ == "NoiseTemplate"
    W, H = model.size
    n = model.cells_num
    gens = 1000
    for _ in range(args.warmup):
        model.gpu.step(gens)
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    lib.xk_range_push(b"timed")
    step_ms = []
    for _ in range(args.steps):
        model.gpu.step(gens)
        step_ms.append(lib.xk_last_step_ms())
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    # the viewer's form: 100 generations, each with its frame (one launch each)
    model.set_viewport((W, H))
    fb = W * H * 3
    frames_dev = torch.empty(100 * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)
    model.gpu.step_frames(100, W, H, 1, 0, 0, frames_dev.data_ptr(), on_device=True)
    frame_ms = model.gpu.step_frames(100, W, H, 1, 0, 0, frames_dev.data_ptr(), on_device=True)
    cells = model.gpu.arrays.cells.get()[:n].copy()
    colors = model.gpu.arrays.colors.get()
    os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
    try:
        vm_model = canonical.NoiseProgram(Noise1080)
    finally:
        del os.environ["XENTICA_GB300_TEMPLATE"]
    vm_model.gpu.load(cells, colors)
    vm_model.gpu.step(10)
    vm_model.gpu.step(100)
    vm_ms = lib.xk_last_step_ms()
    del vm_model
    peak, peak_kind = measured_peak()
    bytes_per_update = 2 * 2 + 12 * 2        # uint16 state r+w, int3 colour r+w
    achieved = bytes_per_update * n * gens / (statistics.mean(step_ms) / 1000.0) / 1e9
    line = {"metric": "cell-updates/s (NoiseTV)", "value": value, "unit": "cell-updates/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_s * 1000 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16", "data": "synthetic (seeded PrimordialSoup: uniform "
                                                           "random states)",
            "config": {"workload": "NoiseTV 1920x1080, MovingAverage colours, 1000 generations "
                                   "per step (up to 1024 per launch)",
                       "l2": "state + colours (29 MB) fit in L2"},
            "frames": {"value": float(n) * 100 / (frame_ms / 1000.0), "unit": "cell-updates/s",
                       "note": "100 generations, each with its 1920x1080 uint8 frame written by the "
                               "step kernel (one launch per generation)"},
            "interpreter": {"value": float(n) * 100 / (vm_ms / 1000.0), "unit": "cell-updates/s",
                            "note": "the same model on the generic interpreter, 100 generations"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": committed_traffic("noise"),
                         "kernel": "xk_k_noise, up to 1024 generations per launch",
                         "note": "B_alg = 28 B per cell-update (uint16 state and int3 colour read and "
                                 "written); a launch reads and writes each cell once for up to 1024 "
                                 "generations, so frac > 1 is reference-format effective"},
            "gpu_launches": args.steps * ((gens + 1023) // 1024), "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        topo = O.Topology(model.size)
        fld = topo.field(cells, np.uint16)
        col = colors.copy()
        d = model.gpu.template.descriptor()
        cc = O._color(True, d.fade_in, d.fade_out, d.smooth)
        model.gpu.load(cells, colors)
        model.gpu.step(gens)
        t0 = time.perf_counter()
        O.noise_run(topo, fld, col, gens, color=cc)
        el = time.perf_counter() - t0
        exact = bool(np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])) and \
            bool(np.array_equal(model.gpu.arrays.colors.get(), col))
        got = model.step_frames(2)
        for g in range(2):
            O.noise_run(topo, fld, col, 1, color=cc)
            img = O.render(topo, col, W, H, smooth=d.render_smooth).astype(np.uint8)
            exact &= bool(np.array_equal(got[g], img))
        line["parity"] = {"checked_generations": gens + 2, "bit_exact": exact,
                          "note": "oracle from the GPU state: 1000 generations, then two with "
                                  "frames"}
        line["cpu_baseline"] = {"value": n * gens / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "1000 generations of the full lattice, oracle (OpenMP)"}
        return line
    return None


def run_noise(args, dist):
    line = noise_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def run_lifecolor(args, dist):
    line = lifecolor_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def run_evolife(args, dist):
    line = evolife_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def mass_line(args, dist):
    """Mass transfer ``--mass-side``^3 (256), Poisson(4) masses: K steps of 100
    generations, each generation followed by the z-projection frame
    (RendererPlain over axes 0, 1) into a device frame buffer; the total
    mass of every generation (reduced inside the kernel) checked against the
    initial total after each step.  Parity: the oracle from the GPU state
    after the timed steps, two more generations."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    from xentica_gb300 import core, seeds
    from xentica_gb300.core.canonical import MassTransferProgram
    import torch
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()

    side = args.mass_side

    class SandPiles(core.Experiment):
        word = "SAND PILES 3D"
        size = (side, side, side)
        zoom = 1
        pos = [0, 0]
        seed = seeds.patterns.PrimordialSoup(vals={"mass": seeds.random.RandPoisson(4)})

    model = MassTransferProgram(SandPiles)
    model.set_viewport((side, side))
    n = model.cells_num
    init = model.gpu.arrays.cells.get()[:n].copy()
    total0 = int(init.astype(np.uint64).sum())
    gens = 100
    fb = side * side * 3
    dev_frames = torch.empty(gens * fb, dtype=torch.uint8, device="cuda:%d" % dist.local)

    def step_device():
        return model.gpu.step_frames(gens, side, side, 1, 0, 0, dev_frames.data_ptr(),
                                     on_device=True)

    for _ in range(args.warmup):
        step_device()
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    step_ms = []
    conserved = True
    lib.xk_range_push(b"timed")
    for _ in range(args.steps):
        step_ms.append(step_device())
        totals = model.gpu.mass_totals(gens)
        conserved &= bool((totals == total0).all())
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    # e2e: host masses in, 100 generations, every frame to pinned host memory
    host = nat.PinnedBuffer(gens * fb)
    colors0 = model.gpu.arrays.colors.get()
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        model.gpu.load(init, colors0)
        model.gpu.step_frames(gens, side, side, 1, 0, 0, host.array)
        e2e.append(time.perf_counter() - t0)
    e2e_s = dist.max(sum(e2e))
    host.release()
    bytes_per_update = 4 * 2 + 4           # uint32 mass read + write, projection re-read
    peak, peak_kind = measured_peak()
    achieved = bytes_per_update * n * gens / (statistics.mean(step_ms) / 1000.0) / 1e9
    line = {"metric": "cell-updates/s (mass transfer 3-D, frame every generation)",
            "value": value, "unit": "cell-updates/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded Poisson(4) masses)",
            "config": {"workload": "mass transfer %d^3 von Neumann, StaticBorder wall, "
                                   "100 generations per step, each followed by the %dx%d "
                                   "z-projection frame; total checked every generation"
                                   % (side, side, side),
                       "l2": "state (2 x %.0f MB)%s; no flush" % (
                           4 * n / 2 ** 20, " close to L2 size" if side == 256 else "")},
            "mass_conserved": conserved,
            "e2e": {"value": float(n) * gens * args.steps * dist.world / e2e_s,
                    "unit": "cell-updates/s", "h2d_bytes_per_step": 4 * n,
                    "d2h_bytes_per_step": gens * fb,
                    "note": "masses loaded from the host (load(cells, colors): this model's "
                            "colours are a function of its state, so the library keeps none "
                            "and copies none), every frame copied to page-locked host memory"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": committed_traffic("mass_tma") if side == 256 else None,
                         "kernel": "xk_k_mass_tma per generation (it also sums the column "
                                   "colours and writes the previous generation's frame)",
                         "algorithmic_bytes_per_generation": bytes_per_update * n,
                         "note": "B_alg = 12 B per cell-update (uint32 read + write, and the "
                                 "projection's read of the state, which the step kernel now "
                                 "does on the cells it writes); traffic: DRAM bytes of one "
                                 "mass-transfer launch (one generation)"},
            "gpu_launches": (gens + 1) * args.steps, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        topo = O.Topology(model.size, "von_neumann", border=2 ** 32 - 1)
        fld = topo.field(model.gpu.arrays.cells.get()[:n], np.uint32)
        col = model.gpu.arrays.colors.get()
        model.gpu.step(2)
        t0 = time.perf_counter()
        totals = []
        O.mass_run(topo, fld, col, 2, totals=totals)
        el = time.perf_counter() - t0
        exact = bool(np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]))
        exact &= model.gpu.mass_totals(2).tolist() == totals
        line["parity"] = {"checked_generations": 2, "bit_exact": exact,
                          "note": "oracle started from the GPU state after the timed steps "
                                  "(cells and per-generation totals)"}
        line["cpu_baseline"] = {"value": n * 2 / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "2 generations of the full lattice, oracle (OpenMP)"}
        return line
    return None


def run_mass(args, dist):
    line = mass_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def life512_model():
    """Conway's Life as the reference's examples/game_of_life.py:15-90 writes it,
    on a 512x512 torus seeded Bernoulli(0.5) from a 64-bit integer seed."""
    from xentica_gb300 import core, seeds
    from xentica_gb300.core import color_effects

    class GameOfLife(core.CellularAutomaton):
        state = core.IntegerProperty(max_val=1)

        class Topology:
            dimensions = 2
            lattice = core.OrthogonalLattice()
            neighborhood = core.MooreNeighborhood()
            border = core.TorusBorder()

        def emit(self):
            for buf in self.buffers:
                buf.state = self.main.state

        def absorb(self):
            neighbors_alive = core.IntegerVariable()
            for i in range(len(self.buffers)):
                neighbors_alive += self.neighbors[i].buffer.state
            is_born = (8 >> neighbors_alive) & 1
            is_sustain = (12 >> neighbors_alive) & 1
            self.main.state = is_born | is_sustain & self.main.state

        @color_effects.MovingAverage
        def color(self):
            red = self.main.state * 255
            green = self.main.state * 255
            blue = self.main.state * 255
            return (red, green, blue)

    class Life512(core.Experiment):
        word = 0x5EED0F11FE512A1B
        size = (512, 512)
        zoom = 1
        pos = [0, 0]
        seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})

    return GameOfLife(Life512)


def life512_line(args, dist):
    """Life 512x512: K steps of 1000 generations (one launch each);
    e2e through the public API (load the cells from the host, step 1000,
    read the cells back); also the reference's calling pattern, 1000 calls of
    model.step(); the final state is compared with the oracle."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()
    model = life512_model()
    n = model.cells_num
    init = model.gpu.arrays.cells.get()[:n].copy()
    colors0 = model.gpu.arrays.colors.get()
    gens = 1000
    for _ in range(args.warmup):
        model.gpu.step(gens)
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    step_ms = []
    lib.xk_range_push(b"timed")
    for _ in range(args.steps):
        model.gpu.step(gens)
        step_ms.append(lib.xk_last_step_ms())
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    total_gens = gens * (args.warmup + args.steps)
    final = model.gpu.arrays.cells.get()[:n].copy()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    # end to end: host cells in, 1000 generations, host cells out
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        model.gpu.load(init, colors0)
        model.gpu.step(gens)
        model.gpu.arrays.cells.get()
        e2e.append(time.perf_counter() - t0)
    e2e_s = dist.max(sum(e2e))
    # the reference's calling pattern: one step() per generation
    model.gpu.load(init, colors0)
    t0 = time.perf_counter()
    for _ in range(gens):
        model.step()
    model.gpu.arrays.cells.get()
    api_s = time.perf_counter() - t0
    peak, peak_kind = measured_peak()
    achieved = B_ALG * n * gens / (statistics.mean(step_ms) / 1000.0) / 1e9
    plan = getattr(model.gpu, "plan", None)
    plan_desc = None
    if plan:
        kind = {0: "global", 1: "resident", 2: "cluster", 3: "temporal"}.get(plan[0], str(plan[0]))
        plan_desc = {"kernel_family": kind}
        if kind == "cluster":
            plan_desc.update({"ctas": plan[1], "rows_per_band": plan[2],
                              "sync": {0: "cluster barrier", 1: "neighbour mbarriers",
                                       2: "split cluster barrier",
                                       3: "asynchronous remote stores counted on neighbour "
                                          "mbarriers"}.get(plan[3], plan[3])})
        elif kind == "temporal":
            plan_desc["generations_per_launch"] = plan[3]
        plan_desc["rule_form"] = "B3/S23 compiled in" if nat.load().xk_model_rule_form(
            model.gpu._handle) == 1 else "rule table"
    line = {"metric": "cell-updates/s (Life 512x512)", "value": value, "unit": "cell-updates/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_s * 1000 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded Bernoulli(0.5), 64-bit integer seed)",
            "config": {"workload": "Conway's Life B3/S23 512x512 torus, 1000 generations per step",
                       "l2": "256 KB state, L2 resident; no flush (latency-bound size)",
                       "tuned_plan": plan_desc},
            "e2e": {"value": float(n) * gens * args.steps * dist.world / e2e_s,
                    "unit": "cell-updates/s", "h2d_bytes_per_step": n + 12 * n,
                    "d2h_bytes_per_step": n},
            "api_step_loop": {"value": float(n) * gens / api_s, "unit": "cell-updates/s",
                              "note": "1000 calls of model.step(), one generation each"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": committed_traffic("life_cluster"),
                         "kernel": "xk_k_life_cluster (or the resident kernel, as tuned)",
                         "note": "B_alg = 2 B per cell-update; the lattice stays in the "
                                 "shared memory of one CTA or of a thread-block cluster "
                                 "(whichever the first step's tuning found faster) for all "
                                 "1000 generations, so frac is reference-format effective"},
            "gpu_launches": args.steps, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        topo = O.Topology(model.size)
        fld = topo.field(init, np.uint8)
        col = np.zeros(3 * n, dtype=np.int32)
        t0 = time.perf_counter()
        O.life_run(topo, fld, col, total_gens)
        el = time.perf_counter() - t0
        line["parity"] = {"generations": total_gens,
                          "bit_exact": bool(np.array_equal(fld[:n], final))}
        line["cpu_baseline"] = {"value": n * total_gens / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d generations of the lattice, oracle (OpenMP)"
                                          % total_gens}
        return line
    return None


def sands_model(template=None):
    """ShiftingSands as the reference's examples/shifting_sands.py:15-47
    writes it, on a 1920x1080 torus seeded Bernoulli(0.5); ``template="vm"``
    builds it on the generic interpreter instead of its fused family."""
    from xentica_gb300 import core, seeds
    from xentica_gb300.core import color_effects

    class ShiftingSands(core.CellularAutomaton):
        state = core.IntegerProperty(max_val=1)

        class Topology:
            dimensions = 2
            lattice = core.OrthogonalLattice()
            neighborhood = core.MooreNeighborhood()
            border = core.TorusBorder()

        def emit(self):
            for i, buf in enumerate(self.buffers):
                if i == 0:
                    buf.state = self.main.state
                else:
                    buf.state = 0

        def absorb(self):
            new_val = core.IntegerVariable()
            for i in range(len(self.buffers)):
                new_val += self.neighbors[i].buffer.state
            self.main.state = new_val

        @color_effects.MovingAverage
        def color(self):
            return (self.main.state * 255, self.main.state * 255, self.main.state * 255)

    class Sands(core.Experiment):
        word = "SHIFTING SANDS 1920X1080"
        size = (1920, 1080)
        zoom = 1
        pos = [0, 0]
        seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})

    old = os.environ.get("XENTICA_GB300_TEMPLATE")
    if template:
        os.environ["XENTICA_GB300_TEMPLATE"] = template
    try:
        return ShiftingSands(Sands)
    finally:
        if template:
            if old is None:
                os.environ.pop("XENTICA_GB300_TEMPLATE")
            else:
                os.environ["XENTICA_GB300_TEMPLATE"] = old


def sands_line(args, dist):
    """ShiftingSands 1920x1080 torus: the fused shifting family (K steps of
    1000 generations; on a torus a step is one gather, since every generation
    moves the states by the same offset), its per-generation kernel (the
    form a history-dependent colour forces, 100 generations) and the generic
    interpreter on the same model (100 generations: the reference's two
    passes over N + 1 planes); final states compared with each other and the
    oracle."""
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    xk_build.build()
    nat.set_device(dist.local)
    lib = nat.load()
    fused, vm = sands_model(), sands_model("vm")
    n = fused.cells_num
    init = fused.gpu.arrays.cells.get()[:n].copy()
    colors0 = fused.gpu.arrays.colors.get()
    gens = 1000
    for _ in range(args.warmup):
        fused.gpu.step(gens)
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    dist.barrier()
    lib.xk_range_push(b"timed")
    step_ms = []
    for _ in range(args.steps):
        fused.gpu.step(gens)
        step_ms.append(lib.xk_last_step_ms())
    lib.xk_range_pop()
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(sum(step_ms) / 1000.0)
    value = float(n) * gens * args.steps * dist.world / dev_s
    # per generation: one launch each (reference calling pattern, model.step())
    fused.gpu.load(init, colors0)
    fused.step()
    t0 = time.perf_counter()
    per_gen = 100
    for _ in range(per_gen):
        fused.step()
    fused.gpu.arrays.cells.get()
    api_s = time.perf_counter() - t0
    # the fused kernel one generation per launch (what a history-dependent
    # colour or a static border needs), 100 generations in one call
    os.environ["XK_SHIFT_JUMP"] = "0"
    try:
        fused.gpu.load(init, colors0)
        fused.gpu.step(1)
        fused.gpu.step(per_gen)
        pg_ms = lib.xk_last_step_ms()
    finally:
        del os.environ["XK_SHIFT_JUMP"]
    pg_rate = float(n) * per_gen / (pg_ms / 1000.0)
    # the interpreter, 100 generations in one call
    vm.gpu.load(init, colors0)
    vm.gpu.step(1)
    vm.gpu.step(per_gen)
    vm_ms = lib.xk_last_step_ms()
    fused.gpu.load(init, colors0)
    fused.gpu.step(1 + per_gen)
    same = bool(np.array_equal(fused.gpu.arrays.cells.get()[:n], vm.gpu.arrays.cells.get()[:n]))
    peak, peak_kind = measured_peak()
    vm_rate = float(n) * per_gen / (vm_ms / 1000.0)
    line = {"metric": "cell-updates/s (ShiftingSands 1920x1080)", "value": value,
            "unit": "cell-updates/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded Bernoulli(0.5))",
            "config": {"workload": "ShiftingSands (examples/shifting_sands.py) 1920x1080 torus, "
                                   "1000 generations per step",
                       "l2": "2 MB state, L2 resident; no flush"},
            "api_step_loop": {"value": float(n) * per_gen / api_s, "unit": "cell-updates/s",
                              "note": "100 calls of model.step(), one generation each"},
            "per_generation": {"value": pg_rate, "unit": "cell-updates/s", "generations": per_gen,
                               "achieved_gbs": 2.0 * pg_rate / 1e9,
                               "frac": 2.0 * pg_rate / 1e9 / peak,
                               "note": "xk_k_shift_nd, one launch per generation (XK_SHIFT_JUMP=0)"},
            "interpreter": {"value": vm_rate, "unit": "cell-updates/s", "generations": per_gen,
                            "bytes_per_cell_update": 2 * 9,
                            "achieved_gbs": 18.0 * vm_rate / 1e9,
                            "frac": 18.0 * vm_rate / 1e9 / peak,
                            "fused_over_interpreter": value / dist.world / vm_rate,
                            "per_generation_over_interpreter": pg_rate / vm_rate,
                            "same_cells_as_fused": same,
                            "note": "(N + 1) x 2 x S = 18 B per cell-update: the reference's "
                                    "emit writes 8 buffer planes, absorb reads them and "
                                    "writes the main plane"},
            "roofline": {"bound": "hbm", "achieved": 2.0 * value / dist.world / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": 2.0 * value / dist.world / 1e9 / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "kernel": "xk_k_shift_jump (1000 generations per launch)",
                         "note": "B_alg = 2 B per cell-update (uint8 read + write); a step "
                                 "of 1000 generations reads and writes the state once, so "
                                 "frac is reference-format effective"},
            "gpu_launches": args.steps, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        topo = O.Topology(fused.size)
        fld = topo.field(init, np.uint8)
        col = np.zeros(3 * n, dtype=np.int32)
        lut = [0, 0, 0] + [255 * v for v in range(1, 9) for _ in range(3)]
        t0 = time.perf_counter()
        O.shift_run(topo, fld, col, 1 + per_gen, 8, lut)
        el = time.perf_counter() - t0
        line["parity"] = {"generations": 1 + per_gen,
                          "bit_exact": bool(np.array_equal(fld[:n], fused.gpu.arrays.cells.get()[:n]))}
        line["cpu_baseline"] = {"value": n * (1 + per_gen) / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d generations of the lattice, oracle (OpenMP)"
                                          % (1 + per_gen)}
        return line
    return None


def run_sands(args, dist):
    line = sands_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def run_life512(args, dist):
    line = life512_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def serve_line(args, dist):
    """Serving: ``--requests`` seeded requests (half 2-D Life-like, a quarter
    3-D von Neumann Life-like, a quarter mass transfer) arrive as a Poisson
    process whose rate offers ``--load`` of the capacity measured first with a
    closed batch of the first 48 requests; latency is completion minus
    submission, including admission waits."""
    import threading
    from xentica_gb300 import build as xk_build
    from xentica_gb300 import _native as nat
    from xentica_gb300 import serve
    xk_build.build()
    nat.set_device(dist.local)
    specs = serve.serving_workload(args.requests, seed=args.seed + dist.rank)
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(min(16, os.cpu_count())) as pool:
        cells = pool.map(serve.make_cells, specs, chunksize=2)
    work = [int(np.prod(sp["shape"])) * sp["generations"] for sp in specs]
    srv = serve.Server(args.serve_budget_gb << 30, host_bytes=8 << 30, max_active=1024,
                       quantum=args.quantum)

    def run_batch(idx):
        hs = [srv.submit(specs[i]["kind"], cells[i], specs[i]["rule"], specs[i]["generations"])
              for i in idx]
        for h in hs:
            h.result(timeout=600)

    small = [i for i in range(len(specs)) if work[i] < 5e8][:max(1, args.warmup * 4)]
    run_batch(small)                                   # warm-up: kernels loaded, pools grown
    probe = list(range(min(48, len(specs))))
    t0 = time.perf_counter()
    run_batch(probe)
    capacity = sum(work[i] for i in probe) / (time.perf_counter() - t0)
    mean_work = sum(work) / len(work)

    def open_loop(load, seed, fixed_rate=None):
        """Poisson arrivals offering ``load`` x capacity (or ``fixed_rate``
        requests per second); returns the stats."""
        rate = fixed_rate if fixed_rate else load * capacity / mean_work
        load = rate * mean_work / capacity
        arrivals = serve.poisson_arrivals(rate, len(specs), seed=seed)
        handles = [None] * len(specs)
        launches0 = srv.stats()["launches"]
        dist.barrier()
        start = time.perf_counter()

        def submitter():
            for i in range(len(specs)):
                delay = start + arrivals[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                handles[i] = srv.submit(specs[i]["kind"], cells[i], specs[i]["rule"],
                                        specs[i]["generations"])

        th = threading.Thread(target=submitter)
        th.start()
        infos = []
        for i in range(len(specs)):
            while handles[i] is None:
                time.sleep(0.0005)
            res = handles[i].result(timeout=1800)
            if i in keep:
                keep[i] = res
            infos.append(handles[i].info())
        th.join()
        dist.barrier()
        first = min(inf["submit_s"] for inf in infos)
        last = max(inf["done_s"] for inf in infos)
        span = dist.max(last - first)
        lat = [inf["done_s"] - inf["submit_s"] for inf in infos]
        by_kind = {}
        for k in ("life2d", "life3d", "mass"):
            idx = [i for i in range(len(specs)) if specs[i]["kind"] == k]
            if idx:
                by_kind[k] = {"latency_s": serve.latency_summary([lat[i] for i in idx]),
                              "slowdown": serve.latency_summary(
                                  [lat[i] * capacity / work[i] for i in idx])}
        return {"offered_load": load, "rate_per_s": rate, "by_kind": by_kind,
                "value": sum(work) * dist.world / span, "span_s": span,
                "latency_s": serve.latency_summary(lat),
                "admission_wait_s": serve.latency_summary(
                    [inf["admit_s"] - inf["submit_s"] for inf in infos]),
                # latency over the request's own work at the measured capacity
                "slowdown": serve.latency_summary(
                    [l * capacity / w for l, w in zip(lat, work)]),
                "launches": srv.stats()["launches"] - launches0}

    # parity sample: the two requests of each kind with the least work, their
    # results from the main run compared with the oracle afterwards
    keep = {}
    for kind in ("life2d", "life3d", "mass"):
        idx = sorted((i for i in range(len(specs)) if specs[i]["kind"] == kind),
                     key=lambda i: work[i])[:2]
        keep.update({i: None for i in idx})
    clocks = Clocks(dist.local)
    time.sleep(0.6)
    main_run = open_loop(args.load, args.seed + 17)
    clk = clocks.stop()
    sample = dict(keep)
    keep = {}
    sweep = [open_loop(float(v), args.seed + 17 + k)
             for k, v in enumerate(args.sweep.split(",")) if v.strip()] if args.sweep else []
    fixed = open_loop(None, args.seed + 17, fixed_rate=args.rate) if args.rate > 0 else None
    st = srv.stats()
    srv.close()
    value = main_run["value"]
    h2d = sum(c.nbytes for c in cells)
    # algorithmic bytes of the mix in the reference's format: 2 B per Life-like
    # cell-update (uint8 read + write), 8 B per mass-transfer one (uint32)
    alg_bytes = sum(w * (8 if sp["kind"] == "mass" else 2) for w, sp in zip(work, specs))
    peak, peak_kind = measured_peak()
    achieved = alg_bytes * dist.world / main_run["span_s"] / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                "note": "whole mix over the run's span (arrivals at %.0f %% of capacity, so the "
                        "GPU idles between requests); 2 B per Life-like and 8 B per "
                        "mass-transfer cell-update; many kernels, so no single traffic figure"
                        % (100 * args.load)}
    kinds = {k: sum(1 for sp in specs if sp["kind"] == k) for k in ("life2d", "life3d", "mass")}
    line = {"metric": "cell-updates/s (serving, Poisson arrivals)", "value": value,
            "unit": "cell-updates/s", "n_gpus": dist.world, "steps": len(specs),
            "warmup": len(small), "ms_per_step": main_run["span_s"] * 1000 / len(specs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u32",
            "data": "synthetic (seeded request mix)",
            "config": {"workload": "serving: %d requests %s, 2-D sides log-uniform [32, 4096], "
                                   "3-D sides log-uniform [64, 256], generations uniform "
                                   "[100, 10000], Poisson arrivals" % (len(specs), kinds),
                       "quantum": args.quantum, "budget_gib": args.serve_budget_gb,
                       "l2": "state per request up to 67 MB; no flush"},
            "rate_per_s": main_run["rate_per_s"], "offered_load": args.load,
            "capacity_probe": capacity, "latency_s": main_run["latency_s"],
            "admission_wait_s": main_run["admission_wait_s"], "slowdown": main_run["slowdown"],
            "by_kind": main_run["by_kind"],
            "sweep": [{k: r[k] for k in ("offered_load", "rate_per_s", "value", "latency_s",
                                          "slowdown")} for r in sweep],
            "fixed_rate": ({k: fixed[k] for k in ("offered_load", "rate_per_s", "value", "latency_s",
                                                  "slowdown", "by_kind")} if fixed else None),
            "device_bytes_peak": st["device_bytes_peak"],
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d / len(specs),
                    "d2h_bytes_per_step": h2d / len(specs),
                    "note": "requests enter and leave through host memory"},
            "gpu_launches": main_run["launches"], "roofline": roofline, "clocks": clk}
    if dist.rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        exact, el, updates = True, 0.0, 0
        for i, got in sample.items():
            sp = specs[i]
            shape = tuple(reversed(sp["shape"]))          # (w, h[, d])
            t0 = time.perf_counter()
            if sp["kind"] == "mass":
                topo = O.Topology(shape, "von_neumann", border=2 ** 32 - 1)
                fld = topo.field(cells[i].ravel(), np.uint32)
                O.mass_run(topo, fld, np.zeros(topo.cells * 3, np.int32), sp["generations"])
            else:
                nbr = 8 if sp["kind"] == "life2d" else 6
                topo = O.Topology(shape) if sp["kind"] == "life2d" else \
                    O.Topology(shape, "von_neumann")
                fld = topo.field(cells[i].ravel(), np.uint8)
                O.life_run(topo, fld, np.zeros(topo.cells * 3, np.int32), sp["generations"],
                           born=sp["rule"] & ((1 << (nbr + 1)) - 1), sustain=sp["rule"] >> (nbr + 1))
            el += time.perf_counter() - t0
            updates += work[i]
            exact &= bool(np.array_equal(np.asarray(got).ravel(), fld[:topo.cells]))
        line["parity"] = {"requests": len(sample), "bit_exact": exact,
                          "note": "the two requests of each kind with the least work, results "
                                  "of the main run against the oracle"}
        line["cpu_baseline"] = {"value": updates / el, "unit": "cell-updates/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "the %d parity requests (%.2g cell-updates), oracle "
                                          "(OpenMP)" % (len(sample), updates)}
        return line
    return None


def run_serve(args, dist):
    line = serve_line(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference_arm(args, dist)
        elif args.workload == "evolife":
            run_evolife(args, dist)
        elif args.workload == "life512":
            run_life512(args, dist)
        elif args.workload == "mass":
            run_mass(args, dist)
        elif args.workload == "serve":
            run_serve(args, dist)
        elif args.workload == "sands":
            run_sands(args, dist)
        elif args.workload == "lifecolor":
            run_lifecolor(args, dist)
        elif args.workload == "noise":
            run_noise(args, dist)
        elif args.workload == "gravity":
            run_gravity(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
