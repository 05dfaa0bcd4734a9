"""Benchmark: histories/s of the replicated IMC step on one GB300.

Workload (default): the 50^3 gray hot zone (0.02 cm cells, central 10^3 hot
block at 1 keV in a 0.05 keV surround, sigma_a = 10 T^-3, rho = 1, cV = 0.1,
vacuum boundaries, dt = 0.01 sh) with 1e7 photons per step, seed 777,
synthetic deck generated in-process (no public dataset exists for this
metric).  A step is one full replicated time step on the device: per-cell
energies, sourcing, history transport, census compaction, tally reduce and
temperature update.  The photon bank (~1 GB per step) is far larger than L2,
so no flush is needed between steps.

value     histories transported / device time of K steps (CUDA events on the
          stream the kernels run on), max over ranks
e2e       the same metric through the drop-in call bgs_replicated_transport
          on pinned host buffers, copies in the timed region
roofline  k_transport_history: algorithmic bytes per launch / its CUDA-event
          duration against the measured HBM copy bandwidth.  The bytes are
          96 B per census photon carried in and per census photon left
          (pos 24, dir 24, E 8, E0 8, life 8, cell 4, group 4, counter 8,
          stream 8) plus 104 B per cell (72 B of geometry and coefficients
          read, 32 B of tallies written); photons made this step are
          sourced from (cell, stream) and count 0 input bytes.
roofline_history_bytes  the same kernel against a history-level byte
          model: every history's 96-byte state read once and written once
          (192 B per history) plus 104 B per cell
roofline_issue  the same kernel's live segments/s times ncu's thread
          instructions per segment, against the SM issue peak, and its FP64
          instructions per segment against two FP64 lanes per clock per SM
          (the kernel is integer-ALU / FP64 bound, not HBM bound)
cpu_baseline  the oracle (C restatement, OpenMP on every host core) on a
          bounded sample of the same deck at the same photons per step,
          histories / transport time
marshak, hohlraum  the other two plain decks at their own sizes (100-cell
          Marshak wave at 1e6 photons over its 50 steps; 60^3 30-group
          hohlraum at 5e7 photons over its 5 steps): GPU histories/s and
          segments/s over whole device steps, and the oracle on the same
          steps on the host cores

--impl reference runs the CPU implementation (the oracle port of the
upstream history loop, all host threads) on the same workload, photons per
step and steps, and reports the same metric.
Multi-GPU (torchrun): independent replicas, one per GPU (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "histories/s on 1 GB300 (plain vs batched); adjoint/forward time at 1% tally err"
UNIT = "histories/s"
# algorithmic bytes of k_transport_history per launch: 96 B per census
# photon carried in and per census photon left (pos 24, dir 24, E 8, E0 8,
# life 8, cell 4, group 4, counter 8, stream 8), per cell 72 B of
# coefficients/geometry read and 32 B of tallies written; photons made this
# step are sourced from (cell, stream) and count 0 input bytes
BYTES_PER_CENSUS_PHOTON = 96
BYTES_PER_CELL = 104
# the history-level model beside it: every history's state read and written
BYTES_PER_HISTORY = 192


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="hot_zone", choices=["hot_zone", "marshak", "hohlraum"])
    p.add_argument("--photons", type=float, default=None)
    p.add_argument("--side", type=int, default=None)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-decks", action="store_true", help="skip the Marshak and hohlraum sections")
    p.add_argument("--algorithm", choices=["tuned", "history", "event"], default="tuned",
                   help="transport algorithm of the main section (history/event: no tuning)")
    p.add_argument("--comb", type=int, default=0,
                   help="comb the census to at most this many photons after every step (comb_photons)")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--batch-problems", type=int, default=256)
    p.add_argument("--batch-photon-scale", type=float, default=1.0,
                   help="scale of the ensemble's photon counts (profiling small cases)")
    p.add_argument("--only", choices=["main", "adjoint", "batch", "decks"], default=None,
                   help="run one section alone and print its JSON (profiling)")
    p.add_argument("--adjoint-photons", type=float, default=1e7)
    p.add_argument("--no-fd-check", action="store_true",
                   help="adjoint section: time the forward/backward pair only (profiling)")
    return p.parse_args()


def make_deck(args):
    from branson_gb300 import deck as D
    steps = 10 ** 6  # keep stepping past the deck's own end time
    if args.workload == "hot_zone":
        side = args.side or 50
        photons = int(args.photons or 1e7)
        dk = D.hot_zone(n_per_axis=side, photons=photons, n_steps=10)
        cfg = {"workload": f"hot_zone_{side}^3", "cells": side ** 3, "photons_per_step": photons,
               "dt": 0.01, "groups": 1}
    elif args.workload == "marshak":
        photons = int(args.photons or 1e6)
        dk = D.marshak_wave(n_cells=args.side or 100, photons=photons, n_steps=50)
        cfg = {"workload": f"marshak_{args.side or 100}x1x1", "cells": args.side or 100,
               "photons_per_step": photons, "dt": 0.001, "groups": 1}
    else:
        side = args.side or 60
        photons = int(args.photons or 5e7)
        dk = D.hohlraum(n_per_axis=side, photons=photons, n_steps=5, n_groups=30)
        cfg = {"workload": f"hohlraum_{side}^3_30g", "cells": side ** 3, "photons_per_step": photons,
               "dt": 0.005, "groups": 30}
    dk.t_stop = dk.dt_start * steps
    cfg.update({"seed": dk.seed, "l2": "bank > L2 (no flush needed)", "data": "synthetic deck"})
    return dk, cfg


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampler for the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        import tempfile
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.mkdtemp(prefix="bgs_clocks_"), f"clocks_gpu{index}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() in ("active", "1"):
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def issue_roofline(seg_rate, clk, tpath):
    """Instruction-issue view of the transport kernel: live segments/s times
    the thread instructions per segment that ncu counted on the same kernel
    (profiles/transport_traffic.json), against the SM issue peak (4 warp
    schedulers x 32 lanes per clock per SM) at the SM clock sampled during
    the timed region."""
    if not os.path.exists(tpath):
        return None
    with open(tpath) as fh:
        t = json.load(fh)
    ips = t.get("thread_instructions_per_segment")
    if not ips:
        return None
    import torch
    n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
    if not mhz:
        return None
    achieved = seg_rate * ips / 1e12
    peak = 128.0 * n_sm * mhz * 1e6 / 1e12
    fp64 = t.get("fp64_thread_instructions_per_segment")
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "T thread-instructions/s",
            "frac": achieved / peak, "instructions_per_segment": ips,
            "fp64_per_segment": fp64,
            "fp64_frac": (seg_rate * fp64 / (2.0 * n_sm * mhz * 1e6)) if fp64 else None,
            "note": "instructions per segment from ncu on the 1e6-photon case of the same deck; "
                    "fp64_frac against 2 FP64 lanes per clock per SM"}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_port_rate(dk_gpu, threads: int, steps: int = 1, warmup: int = 0):
    """Oracle (C port of the upstream history loop) on the host cores, timed
    over `steps` steps after `warmup` untimed ones, on the GPU arm's deck
    (same photons per step).  Returns (histories, transport seconds,
    segments, wall seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import copy
    import oracle as O
    orc = O.Oracle(copy.deepcopy(dk_gpu), n_threads=threads)
    for _ in range(warmup):
        orc.step()
    hist = 0
    secs = 0.0
    segs = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        r = orc.step()
        hist += len(r.source)
        secs += r.transport_s
        segs += r.segments
    return hist, secs, segs, time.perf_counter() - t0


def run_reference(args, rank, world):
    """The reference arm: the oracle port of the upstream CPU history path
    (history_cpu_transport_photons over OpenMP, replicated_transport.h:88-92)
    on every host thread, on the GPU arm's deck, photons per step and steps:
    `warmup` untimed steps, then `steps` timed ones; histories / the sum of
    the steps' transport times (the upstream transport timer,
    replicated_transport.h:63-143, which leaves out sourcing)."""
    if rank != 0:
        return
    dk, cfg = make_deck(args)
    threads = os.cpu_count() or 1
    hist, secs, segs, wall = cpu_port_rate(dk, threads, steps=args.steps, warmup=args.warmup)
    v = hist / secs
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(cfg, parallelism=f"replicas{world}"), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"steps {args.warmup + 1}-{args.warmup + args.steps} of the deck at "
                                       f"{dk.photons} photons/step (after {args.warmup} untimed), "
                                       f"{hist} histories, transport time only (replicated_transport timer)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "segments_per_s": segs / secs, "wall_s": wall}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from branson_gb300 import _lib
    from branson_gb300.engine import ReplicatedIMC, records_to_arrays

    dk, cfg = make_deck(args)
    from branson_gb300.replicas import combine, replica_seed
    dk.seed = replica_seed(dk.seed, rank)  # independent replica per rank
    stream = torch.cuda.Stream(device=dev)
    imc = ReplicatedIMC(dk, device=dev, stream=stream.cuda_stream)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # the autotuner picks the transport schedule on this deck's first step
    # (block size, histories per thread, history vs event mode; results are
    # identical under every schedule)
    tuning = None
    if args.algorithm != "tuned":
        imc.algorithm = _lib.HISTORY if args.algorithm == "history" else _lib.EVENT
    elif not args.no_tune:
        from branson_gb300.tune import tune
        res = tune(imc, repeats=2)
        tuning = {"schedule": res.best.label(), "transport_ms": res.best_ms, "algorithm": imc.algorithm,
                  "candidates": {c.label(): ms for c, ms in res.timings}}

    comb_ctr = 0

    def comb(n_census):
        # census population control between steps (census_functions.h:48-93),
        # RNG stream 2^62 (apart from every photon's), its counter carried on
        nonlocal comb_ctr
        if not args.comb:
            return n_census
        kept, comb_ctr = imc.comb_census(args.comb, stream=1 << 62, counter=comb_ctr)
        return kept

    census_in = 0
    for _ in range(args.warmup):
        census_in = comb(imc.step(sync=True).n_census)
    barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    launches0 = imc.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    hist = 0
    segs = 0
    transport_ms = []  # per step: (kernel ms, histories, census in, census out)
    ev0.record(stream)
    for _ in range(args.steps):
        r = imc.step(sync=True)
        hist += r.n_transported
        segs += r.n_segments
        ms, _k = imc.last_transport_ms()
        transport_ms.append((ms, r.n_transported, census_in, r.n_census))
        census_in = comb(r.n_census)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    launches = imc.kernel_launches() - launches0
    clk = clocks.stop()
    elapsed, hist_all = combine(elapsed, hist, device=f"cuda:{dev}")
    value = hist_all / elapsed

    # roofline of the dominant kernel (k_transport_history), live CUDA events
    n_k = len(transport_ms)
    k_ms = sum(t[0] for t in transport_ms) / n_k
    k_hist = sum(t[1] for t in transport_ms) / n_k
    k_census = sum(t[2] + t[3] for t in transport_ms) / n_k  # census photons in + out per launch
    alg_bytes = BYTES_PER_CENSUS_PHOTON * k_census + BYTES_PER_CELL * dk.n_cells
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "transport_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            t = json.load(fh)
        traffic = t.get("bytes_per_history", 0) * k_hist + t.get("bytes_per_cell", 0) * dk.n_cells
    seg_rate = segs / (sum(t[0] for t in transport_ms) * 1e-3)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                "kernel": "k_transport_history", "kernel_ms": k_ms, "segments_per_s": seg_rate,
                "algorithmic_bytes_per_launch": alg_bytes, "census_photons_in_plus_out_per_launch": k_census,
                "note": "96 B per census photon in and out plus 104 B per cell; the kernel is integer-ALU / "
                        "FP64-issue bound, so the HBM fraction is small by construction (roofline_issue "
                        "holds the binding roof); traffic is ncu's DRAM bytes per history on the 1e6-photon "
                        "case of the same deck, scaled to this launch's histories"}
    hist_bytes = BYTES_PER_HISTORY * k_hist + BYTES_PER_CELL * dk.n_cells
    roofline_hist = {"bound": "hbm", "achieved": hist_bytes / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": hist_bytes / (k_ms * 1e-3) / 1e9 / peak, "bytes_per_launch": hist_bytes,
                     "note": "every history's 96-byte state read and written once (192 B per history) plus "
                             "104 B per cell"}
    roofline_issue = issue_roofline(seg_rate, clk, tpath)

    # end to end through the drop-in call on pinned host buffers
    e2e = None
    if not args.no_e2e and rank == 0:
        e2e = e2e_dropin(imc, dk, args)

    cpu = None
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        w = min(args.warmup, 2)
        h, s, sg, _ = cpu_port_rate(dk, threads, steps=2, warmup=w)
        cpu = {"value": h / s, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"steps {w + 1}-{w + 2} (after {w} untimed) of the same deck at {dk.photons} photons/step "
                         f"({h} histories), transport time only; the reference arm runs the GPU arm's own steps"}
    imc.close()
    adjoint = None
    if not args.no_adjoint and rank == 0 and world == 1:
        adjoint = guarded(adjoint_bench, args, dev, clocks_of=dev)
    batched = None
    if not args.no_batch and rank == 0 and world == 1:
        batched = guarded(batch_bench, args, dev, clocks_of=dev)
    decks = None
    if not args.no_decks and rank == 0 and world == 1 and args.workload == "hot_zone":
        decks = guarded(decks_bench, dev)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(cfg, parallelism=f"replicas{world}"), "roofline": roofline,
                "roofline_history_bytes": roofline_hist, "roofline_issue": roofline_issue,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
                "segments_per_s": segs / elapsed * world, "histories_per_step": hist / args.steps,
                "tuning": tuning, "adjoint": adjoint, "batched": batched}
        if decks and "error" not in decks:
            line.update(decks)
        elif decks:
            line["decks"] = decks
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def e2e_dropin(imc, dk, args):
    """Drop-in replicated_transport on pinned host buffers, the host-device
    traffic inside the timed region.  The buffers are page-locked and mapped
    into the device, so by default the kernels read each photon's state at
    pickup and write its end state in place over the host link (NVLink-C2C
    on GB300); the same call with the zero_copy option off copies the bank
    in and the end states out around a pipelined transport, timed beside it."""
    import numpy as np
    from branson_gb300._lib import PhotonArrays
    # inputs: the current step's photon list, made on the device and copied out
    step, dt = imc.step_no, imc.dt
    imc.calculate_photon_energy(step, dt)
    imc.source(step, dt)
    n = imc.bank_size()
    src = imc.photons(0, n)
    work = PhotonArrays(n, pinned=True)
    census = PhotonArrays(n, pinned=True)
    nd = imc.next_dt() if imc.next_dt() > 0 else dt
    k = max(1, min(args.steps, 3))
    rates = {}
    for zero_copy in (1, 0):
        imc.set_option("zero_copy", zero_copy)
        hist, secs = 0, 0.0
        for it in range(k + 1):
            for name in work.arrays:
                np.copyto(work[name], src[name])
            t0 = time.perf_counter()
            abs_E, trk_E, cen, ce, ex = imc.replicated_transport(work, nd, census=census)
            t1 = time.perf_counter()
            if it > 0:  # first call is warm-up
                hist += n
                secs += t1 - t0
        rates[zero_copy] = hist / secs
    imc.set_option("zero_copy", 1)
    in_bytes = sum(a.nbytes for a in src.arrays.values())
    out_bytes = n * (6 * 8 + 8 + 8 + 4 + 4 + 1 + 8) + cen.n * sum(a.itemsize for a in src.arrays.values()) \
        + 2 * 8 * dk.n_cells
    return {"value": rates[1], "unit": UNIT, "h2d_bytes_per_step": int(in_bytes),
            "d2h_bytes_per_step": int(out_bytes), "call": "bgs_replicated_transport", "steps": k,
            "transfer": "photon state read at pickup and end states written in place by the kernels in "
                        "page-locked mapped host memory (over NVLink-C2C); census and tallies copied out",
            "copied_value": rates[0],
            "copied_transfer": "bank copied in and end states out (cudaMemcpyAsync) around a pipelined transport"}


def deck_rate(dk, dev, cfg, cpu_steps=None):
    """One plain deck over all of its steps on the GPU (device time of the
    whole steps, CUDA events on the context's stream, after one untimed
    step of a separate context as warm-up), and the oracle over the same
    steps (or the first `cpu_steps` of them) on every host core."""
    import copy
    import torch
    from branson_gb300.engine import ReplicatedIMC
    n_steps = int(round((dk.t_stop - dk.t_start) / dk.dt_start))
    clocks = Clocks(dev)  # sampled over the GPU part only (warm-up context and the timed steps)
    clocks.start()
    with ReplicatedIMC(copy.deepcopy(dk), device=dev) as w:
        w.step(sync=True)
    stream = torch.cuda.Stream(device=dev)
    hist = segs = 0
    with ReplicatedIMC(copy.deepcopy(dk), device=dev, stream=stream.cuda_stream) as imc:
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        kms = 0.0
        for _ in range(n_steps):
            r = imc.step(sync=True)
            hist += r.n_transported
            segs += r.n_segments
            kms += imc.last_transport_ms()[0]
        ev1.record(stream)
        torch.cuda.synchronize()
        el = ev0.elapsed_time(ev1) / 1e3
    clk = clocks.stop()
    threads = os.cpu_count() or 1
    cs = n_steps if cpu_steps is None else cpu_steps
    h, s, sg, wall = cpu_port_rate(dk, threads, steps=cs, warmup=0)
    return dict(cfg, steps=n_steps, histories=int(hist), segments=int(segs), gpu_s=el, transport_kernel_s=kms / 1e3,
                histories_per_s=hist / el, segments_per_s=segs / el, clocks=clk,
                cpu={"histories_per_s": h / s, "segments_per_s": sg / s, "cores": threads, "kind": "port",
                     "steps": cs, "histories": int(h), "transport_s": s, "wall_s": wall,
                     "sample": "the same deck and photons per step from step 1, transport time only"},
                gpu_over_cpu=(hist / el) / (h / s))


def decks_bench(dev):
    """The other two plain decks at their own sizes: the 100-cell Marshak
    wave at 1e6 photons over its 50 steps, and the 60^3 30-group hohlraum at
    5e7 photons over its 5 steps (the oracle over its first 2)."""
    from branson_gb300 import deck as D
    m = D.marshak_wave(n_cells=100, photons=1_000_000, n_steps=50)
    h = D.hohlraum(n_per_axis=60, photons=50_000_000, n_steps=5, n_groups=30)
    return {"marshak": deck_rate(m, dev, {"workload": "marshak_100x1x1", "cells": 100, "photons_per_step": 1_000_000,
                                          "dt": 0.001, "groups": 1, "seed": m.seed}),
            "hohlraum": deck_rate(h, dev, {"workload": "hohlraum_60^3_30g", "cells": 216000,
                                           "photons_per_step": 50_000_000, "dt": 0.005, "groups": 30,
                                           "seed": h.seed}, cpu_steps=2)}


def batch_adjoint_timing(b):
    """Adjoint of every problem's next step: the forwards (per problem), then
    dL/dsigma_a for all problems from one replay launch, against the same
    backwards called problem by problem (same tapes and weights, equal
    results)."""
    import numpy as np
    from branson_gb300.adjoint import batch_backward, batch_forward
    rng = np.random.default_rng(777)
    t0 = time.perf_counter()
    _, tapes = batch_forward(b)
    fwd = time.perf_counter() - t0
    ws = [rng.uniform(0.0, 1.0, p.n_cells) for p in b.problems]
    batch_backward(b, tapes, ws)  # warm-up (scratch allocation)
    t0 = time.perf_counter()
    grads = batch_backward(b, tapes, ws)
    bwd = time.perf_counter() - t0
    replay_ms = tapes[0].info()["replay_ms"]
    t0 = time.perf_counter()
    same = True
    for p, t, w, g in zip(b.problems, tapes, ws, grads):
        own = np.empty(p.n_cells)
        if b.lib.bgs_adjoint_backward(p.ctx, t.handle, w.ctypes.data, own.ctypes.data) != 0:
            raise RuntimeError("bgs_adjoint_backward failed")
        same &= bool(np.array_equal(own, g))
    seq = time.perf_counter() - t0
    hist = sum(t.info()["n_histories"] for t in tapes)
    for t in tapes:
        t.close()
    return {"histories": int(hist), "forward_s": fwd, "batched_backward_s": bwd,
            "batched_replay_kernel_ms": replay_ms, "sequential_backward_s": seq,
            "batched_backward_over_sequential": seq / bwd, "backward_over_forward": bwd / fwd,
            "equal_to_per_problem": same}


def batch_bench(args, dev, steps: int = 2):
    """Batching workload: 256 independent problems (master seed 777), cubic
    meshes of side U{8..64} on [0,1]^3, photons lognormal (median 1e5)
    clipped to [1e4, 1e6], per-problem sigma_a ~ U(1,200) and source T ~
    U(0.2,1) on x-, T0 = 0.01 keV, steps of 0.005 sh.  Sequential: every
    problem on its own context, one bgs_step after another, each waited for
    (the plain launches).  Batched: the same problems on fresh contexts
    through bgs_batch_step (one persistent transport launch, the step
    recorded as one CUDA graph and launched with one call).  Each arm starts
    from step 1 and times `steps` steps (wall clock around each whole step);
    histories/s = histories of all problems / that time."""
    from branson_gb300 import deck as D
    from branson_gb300.engine import BatchIMC, ReplicatedIMC

    n = args.batch_problems
    k = args.batch_photon_scale
    decks = D.batch_ensemble(n_problems=n, master_seed=777, photon_median=1e5 * k,
                             photon_range=(max(1, int(1e4 * k)), max(1, int(1e6 * k))))
    # warm-up of the batched path (module load, graph machinery) on a small ensemble
    with BatchIMC(D.batch_ensemble(n_problems=4, master_seed=1, side_range=(4, 8), photon_median=2000,
                                   photon_range=(1000, 4000)), device=dev) as w:
        w.step(sync=True)
    seq = {"s": [], "hist": [], "seg": [], "transport_ms": []}
    probs = [ReplicatedIMC(dk, device=dev) for dk in decks]
    try:
        for _ in range(steps):
            reps, kms = [], 0.0
            t0 = time.perf_counter()
            for p in probs:
                reps.append(p.step(sync=True))
                kms += p.last_transport_ms()[0]
            seq["s"].append(time.perf_counter() - t0)
            seq["hist"].append(sum(r.n_transported for r in reps))
            seq["seg"].append(sum(r.n_segments for r in reps))
            seq["transport_ms"].append(kms)
    finally:
        for p in probs:
            p.close()
    bat = {"s": [], "hist": [], "seg": [], "transport_ms": []}
    adj = None
    with BatchIMC(decks, device=dev) as b:
        launches0 = b.last_transport_ms()[1]
        for _ in range(steps):
            t0 = time.perf_counter()
            reps = b.step(sync=True)
            bat["s"].append(time.perf_counter() - t0)
            bat["hist"].append(sum(r.n_transported for r in reps))
            bat["seg"].append(sum(r.n_segments for r in reps))
            bat["transport_ms"].append(b.last_transport_ms()[0])
        launches = b.last_transport_ms()[1] - launches0
        if not args.no_adjoint:
            adj = batch_adjoint_timing(b)
    assert seq["hist"] == bat["hist"] and seq["seg"] == bat["seg"], "batched and sequential runs disagree"
    rate_s = sum(seq["hist"]) / sum(seq["s"])
    rate_b = sum(bat["hist"]) / sum(bat["s"])
    return {"workload": f"batch_ensemble of {n} problems (side U{{8..64}}, photons lognormal median {1e5 * k:g} in "
                        f"[{1e4 * k:g}, {1e6 * k:g}], sigma_a U(1,200), T_source U(0.2,1)), steps from step 1",
            "steps": steps, "histories_per_step": seq["hist"], "segments_per_step": seq["seg"],
            "sequential_hist_per_s": rate_s, "batched_hist_per_s": rate_b, "batched_over_sequential": rate_b / rate_s,
            "sequential_step_s": seq["s"], "batched_step_s": bat["s"],
            "batched_transport_kernel_ms": bat["transport_ms"],
            "sequential_transport_kernel_ms_sum": seq["transport_ms"],
            "batched_segments_per_s": sum(bat["seg"]) / sum(bat["s"]),
            "kernel_launches_per_batched_step": launches // steps,
            "adjoint": adj,
            "timing": "host wall clock around each whole step (sync), same problems and results in both arms"}


_RETRIES = {"fd_forward": 0}


def fd_forward(st, sigma_a, counts):
    """A finite-difference forward at frozen photon counts.  One retry after a
    device check: an FD forward once raised the supplied-counts check in the
    bench (not reproduced since); the retries are counted in the JSON."""
    from branson_gb300._lib import BransonError
    try:
        return st.forward(sigma_a=sigma_a, counts=counts, save=False)[0]
    except BransonError as e:
        _RETRIES["fd_forward"] += 1
        _RETRIES.setdefault("last_error", str(e))
        return st.forward(sigma_a=sigma_a, counts=counts, save=False)[0]


def guarded(fn, *a, clocks_of=None):
    """A bench section whose failure is reported in its own key instead of
    ending the run before the headline line is printed.  With clocks_of (a
    device index) the section's SM clocks and throttle reasons are sampled
    while it runs and returned in its "clocks" key."""
    clk = Clocks(clocks_of) if clocks_of is not None else None
    if clk:
        clk.start()
    try:
        out = fn(*a)
    except Exception as e:  # reported, not hidden: the section's JSON holds the error
        out = {"error": f"{type(e).__name__}: {e}"}
    if clk:
        out["clocks"] = clk.stop()
    return out


def adjoint_bench(args, dev, replicas: int = 6):
    """Differentiation workload: 32^3 cube, one region per cell with sigma_a ~
    lognormal(ln 20, 0.5) from seed 777, T0 = 0.1 keV, 1 keV source on x-,
    one step of 0.01 sh at 1e7 photons; L = sum_c w_c E_abs[c] with w ~ U(0,1).
    Reports the forward and backward call times (host wall, synchronous,
    host arrays in and out) and their ratio.  Checks dL/dsigma_a against
    common-random-number central differences (h = 1e-4 relative, photon
    counts frozen) on 64 random cells among those whose absorbed-energy
    tally has at most 1% relative statistical error.  Both estimates are
    Monte Carlo; each is averaged over `replicas` independent-seed runs of
    the step, and the per-cell difference is given with its standard error
    (z) from the paired replica spread; plus the directional derivative
    along sign(gradient) over the 64 cells."""
    import numpy as np
    from branson_gb300 import deck as D
    from branson_gb300.adjoint import AdjointStep

    photons = int(args.adjoint_photons)
    dk = D.random_opacity_cube(n_per_axis=32, photons=photons, seed=777)
    sig0 = np.array([r.opacA for r in dk.regions])[dk.cell_regions()]
    w = np.random.default_rng(777).uniform(0.0, 1.0, dk.n_cells)
    h = 1e-4
    tallies, grads, tapes_info = [], [], None
    tf, tb, fwd_kernel_ms = [], [], 0.0
    runs = []  # per replica: (context, tape, counts)
    if args.no_fd_check:
        replicas = 1
    for r in range(replicas):
        dk_r = D.random_opacity_cube(n_per_axis=32, photons=photons, seed=777)
        dk_r.seed = 777 + 1000 * r
        st = AdjointStep(dk_r, device=dev)
        a, tape = st.forward(sigma_a=sig0)
        g = st.backward(tape, w)
        if r == 0:  # timing on the first replica, after one warm-up pair
            for _ in range(3):
                t0 = time.perf_counter()
                a, tape = st.forward(sigma_a=sig0, tape=tape)
                tf.append(time.perf_counter() - t0)
                fwd_kernel_ms, _ = st.last_transport_ms()
                t0 = time.perf_counter()
                g = st.backward(tape, w)
                tb.append(time.perf_counter() - t0)
            tapes_info = tape.info()
        tallies.append(a)
        grads.append(g)
        runs.append((st, tape.counts()))
        tape.close()
    if args.no_fd_check:
        for st, _ in runs:
            st.close()
        fwd, bwd = statistics.median(tf), statistics.median(tb)
        return {"histories": int(tapes_info["n_histories"]), "forward_ms": 1e3 * fwd, "backward_ms": 1e3 * bwd,
                "backward_over_forward": bwd / fwd, "backward_replay_kernel_ms": tapes_info["replay_ms"]}
    T = np.array(tallies)
    mean = T.mean(axis=0)
    rel_err = np.where(mean > 0, T.std(axis=0, ddof=1) / np.where(mean > 0, mean, 1.0), np.inf)
    resolved = np.flatnonzero(rel_err <= 0.01)
    rng = np.random.default_rng(4)
    cells = rng.choice(resolved, min(64, len(resolved)), replace=False) if len(resolved) else np.array([], int)
    G = np.array(grads)[:, cells]
    v = np.sign(G.mean(axis=0))
    FD, DIR_FD = [], []
    for st, counts in runs:
        row = []
        for j in cells:
            sp, sm = sig0.copy(), sig0.copy()
            sp[j] *= 1 + h
            sm[j] *= 1 - h
            ap = fd_forward(st, sp, counts)
            am = fd_forward(st, sm, counts)
            row.append(float(np.dot(w, ap - am) / (2 * h * sig0[j])))
        FD.append(row)
        sp, sm = sig0.copy(), sig0.copy()
        sp[cells] *= 1 + h * v
        sm[cells] *= 1 - h * v
        ap = fd_forward(st, sp, counts)
        am = fd_forward(st, sm, counts)
        DIR_FD.append(float(np.dot(w, ap - am) / (2 * h)))
        st.close()
    FD = np.array(FD)
    diff = G - FD
    k = len(runs)
    rel = np.abs(diff.mean(axis=0)) / np.abs(FD.mean(axis=0))
    se = diff.std(axis=0, ddof=1) / math.sqrt(k)
    z = np.abs(diff.mean(axis=0)) / np.where(se > 0, se, np.inf)
    dir_adj = (G * (sig0[cells] * v)).sum(axis=1)
    dir_fd = np.array(DIR_FD)
    dir_diff = dir_adj - dir_fd
    fwd, bwd = statistics.median(tf), statistics.median(tb)
    # the per-replica spread of each cell's difference, and the replicas a
    # median standard error of 0.3% would take at this history count
    sd1 = diff.std(axis=0, ddof=1) / np.abs(FD.mean(axis=0))
    fd_s = 2 * len(cells) + 1  # forwards per replica
    resolved_class = fd_check_resolved(args, dev)
    return {"workload": "random_opacity_cube 32^3, sigma_a ~ lognormal(ln 20, 0.5), 1 keV source on x-, "
                        f"{photons} photons, one step of 0.01 sh",
            "histories": int(tapes_info["n_histories"]), "segments": int(tapes_info["n_segments"]),
            "forward_ms": 1e3 * fwd, "backward_ms": 1e3 * bwd, "backward_over_forward": bwd / fwd,
            "forward_transport_kernel_ms": fwd_kernel_ms, "backward_replay_kernel_ms": tapes_info["replay_ms"],
            "histories_replayed_twice": int(tapes_info["n_long"]),
            "fd_check": {"h_rel": h, "replicas": k, "cells": int(len(cells)),
                         "cells_with_tally_err_le_1pct": int(len(resolved)),
                         "median_rel_diff_of_means": float(np.median(rel)) if len(rel) else None,
                         "frac_within_1pct": float(np.mean(rel <= 0.01)) if len(rel) else None,
                         "frac_within_3pct": float(np.mean(rel <= 0.03)) if len(rel) else None,
                         "frac_z_le_3": float(np.mean(z <= 3.0)) if len(z) else None,
                         "median_rel_stderr": float(np.median(se / np.abs(FD.mean(axis=0)))) if len(se) else None,
                         "directional_rel_diff": float(abs(dir_diff.mean()) / abs(dir_fd.mean())),
                         "directional_rel_stderr": float(dir_diff.std(ddof=1) / math.sqrt(k) / abs(dir_fd.mean())),
                         "median_rel_sd_per_replica": float(np.median(sd1)) if len(sd1) else None,
                         "replicas_for_0.3pct_median_stderr": int(math.ceil((np.median(sd1) / 0.003) ** 2))
                         if len(sd1) else None,
                         "forwards_per_replica": fd_s},
            "fd_check_resolved": resolved_class, "fd_forward_retries": dict(_RETRIES)}


def fd_check_resolved(args, dev, replicas: int = 16):
    """The 1% criterion on a deck class that resolves it: a 4^3 cube (64
    cells of 0.25 cm, every one checked) with the differentiation deck's
    physics and sigma_a ~ lognormal(ln 2, 0.5), a tenth of the 32^3 deck's
    law, so that no history decays to the E/E0 < 0.01 cutoff, whose jump the
    estimator does not differentiate; 1e7 photons per replica, w ~ U(0,1).
    Per cell: the mean over independent-seed replicas of the adjoint gradient
    and of the CRN central difference (h = 1e-4 relative, counts frozen),
    their difference relative to the FD mean, and its standard error."""
    import numpy as np
    from branson_gb300 import deck as D
    from branson_gb300.adjoint import AdjointStep
    n, photons, h = 4, int(args.adjoint_photons), 1e-4
    make = lambda seed: D.random_opacity_cube(n_per_axis=n, photons=photons, seed=777, sigma_median=2.0)
    dk = make(777)
    sig0 = np.array([r.opacA for r in dk.regions])[dk.cell_regions()]
    w = np.random.default_rng(777).uniform(0.0, 1.0, dk.n_cells)
    adj, fd = [], []
    t0 = time.perf_counter()
    for r in range(replicas):
        dk_r = make(777)
        dk_r.seed = 777 + 1000 * r
        with AdjointStep(dk_r, device=dev) as st:
            _, tape = st.forward(sigma_a=sig0)
            counts = tape.counts()
            adj.append(st.backward(tape, w))
            row = []
            for j in range(dk.n_cells):
                sp, sm = sig0.copy(), sig0.copy()
                sp[j] *= 1 + h
                sm[j] *= 1 - h
                ap = fd_forward(st, sp, counts)
                am = fd_forward(st, sm, counts)
                row.append(float(np.dot(w, ap - am) / (2 * h * sig0[j])))
            fd.append(row)
            tape.close()
    adj, fd = np.array(adj), np.array(fd)
    d = adj - fd
    scale = np.abs(fd.mean(axis=0))
    rel = np.abs(d.mean(axis=0)) / scale
    se = d.std(axis=0, ddof=1) / math.sqrt(replicas) / scale
    return {"workload": f"random_opacity_cube {n}^3, sigma_a ~ lognormal(ln 2, 0.5), 1 keV source on x-, "
                        f"{photons} photons, one step of 0.01 sh; all {dk.n_cells} cells",
            "replicas": replicas, "h_rel": h, "seconds": time.perf_counter() - t0,
            "median_rel_stderr": float(np.median(se)), "median_rel_diff": float(np.median(rel)),
            "frac_within_1pct": float(np.mean(rel <= 0.01)),
            "frac_within_1pct_plus_2se": float(np.mean(rel <= 0.01 + 2.0 * se)),
            "max_rel_diff": float(rel.max()), "rel_stderr_at_max": float(se[int(np.argmax(rel))])}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.only in ("adjoint", "batch", "decks"):
        import torch
        torch.cuda.set_device(0)
        fn = {"adjoint": adjoint_bench, "batch": batch_bench, "decks": lambda a, d: decks_bench(d)}[args.only]
        print(json.dumps({"section": args.only, args.only: fn(args, 0)}), flush=True)
        return
    if args.only == "main":
        args.no_adjoint = args.no_batch = args.no_decks = True
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
