"""Parity of the GPU path with the oracle on the benchmark decks at full size.

Cases (the workloads bench.py measures, at their own sizes):
  hot_zone  50^3 gray hot zone, 1e7 photons per step; two warm-up steps on
            the oracle, then one compared step (~1.04e7 histories)
  marshak   100-cell gray Marshak wave, 1e6 photons per step, every one of
            its 50 steps compared
  hohlraum  60^3 box, 30 groups, 5e7 photons; the first step (initial
            census, emission and the source face: ~5.4e7 histories)

Each compared step starts the GPU from the oracle's state (temperatures and
census), so every step is compared on its own ("lockstep"):
  * energies, photon counts and the photons the device sources (their
    sampling bit for bit with the twin, their weights within 1e-13: a
    weight is its cell's energy over the cell's count, and the powers of T
    in the cell energies are rounded by each side's own pow);
  * the drop-in transport (bgs_replicated_transport) of the oracle's photon
    list: every history's end state, the census, the tallies, the census
    and exit energies;
  * the device temperature update that follows (T_e, T_r).

Three CPU runs are the references:
  L  the oracle (oracle/branson_oracle.c, host libm; pinned to upstream);
  G  its twin built with the GPU path's own integer -log/exp/sin/cos
     (make -C oracle gpumath): the same IEEE arithmetic otherwise, so the GPU
     must equal G bit for bit on every history, and a GPU-vs-L difference is
     then the last-bit rounding of those functions and nothing else;
  B  L over 16 interleaved slices of the list: the Monte Carlo variance of
     every cell's tallies, for z-scores.

Against L every history is classified:
  * bit-identical;
  * rounding only: cell, group, descriptor and RNG counter equal, floats
    within 1e-12 (plain relative error; components that are exactly 0 in L
    are measured against the deck's extent);
  * branch flip: cell, group, descriptor or counter differ.  Both CPU builds
    trace the history segment by segment; at the first segment where they
    part, the comparison that decided it is found (which event came first,
    which face was nearest, or the cutoff) and its relative margin measured.
    A flip is a near tie when that margin is at most 1e-9.
Per cell: the tallies of the flipped histories are recomputed alone (GPU
and L); with them taken out both sides must agree within 1e-10 of the cell's
tally on every cell, and the temperatures within 1e-10 on every cell no
flipped history touched.  Where flipped histories deposited, the raw
difference is given as a z-score against the cell's Monte Carlo standard
error.

Run by tests/test_fullsize_gpu.py, or directly on a GPU host:
    python tests/fullsize.py hot_zone [--json report.json]
"""
from __future__ import annotations

import argparse
import copy
import ctypes as C
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

END_RTOL = 1e-12
CELL_RTOL = 1e-10
ENERGY_RTOL = 1e-13
NEAR_TIE = 1e-9
Z_MAX = 5.0
N_SLICES = 16

C_LIGHT = 299.792458
EXIT, PASS, CENSUS, SCATTER, KILLED, BOUND = range(6)


def case_deck(name):
    """(deck, oracle warm-up steps, compared steps) of a case."""
    from branson_gb300 import deck as D
    if name == "hot_zone":
        return D.hot_zone(n_per_axis=50, photons=10_000_000, n_steps=10), 2, 1
    if name == "marshak":
        return D.marshak_wave(n_cells=100, photons=1_000_000, n_steps=50), 0, 50
    if name == "hohlraum":
        return D.hohlraum(n_per_axis=60, photons=50_000_000, n_steps=5, n_groups=30), 0, 1
    if name == "hot_zone_small":  # a quick form of the hot zone (CPU self-check of this module)
        return D.hot_zone(n_per_axis=15, photons=100_000, n_steps=10), 1, 1
    raise ValueError(name)


def extent(dk):
    x, y, z = dk.planes()
    return max(x[-1] - x[0], y[-1] - y[0], z[-1] - z[0], C_LIGHT * dk.dt_start)


# ------------------------------------------------------------- comparisons
def rel_err(a, b, floor):
    """Plain relative error |a-b|/|b|; where b is exactly 0, |a-b|/floor."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    den = np.where(b != 0.0, np.abs(b), floor)
    return np.where(same, 0.0, d / den)


def bitwise_same(a, b):
    """Per record: every field bit-identical (float fields by bit pattern)."""
    same = np.ones(len(a), bool)
    for f in a.dtype.names:
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            x = x.view(np.uint64)
            y = y.view(np.uint64)
        same &= (x == y) if x.ndim == 1 else np.all(x == y, axis=1)
    return same


def int_mismatch(a, b):
    return (a["counter"] != b["counter"]) | (a["cell"] != b["cell"]) | (a["group"] != b["group"]) | \
        (a["descriptor"] != b["descriptor"])


def float_errors(got, ref, ext):
    """Per history and component: plain relative error (0 floors at the
    extent for position and flight, 1 for direction cosines, E0 for E)."""
    out = {}
    for i, a in enumerate("xyz"):
        out[f"pos_{a}"] = rel_err(got["pos"][:, i], ref["pos"][:, i], ext)
        out[f"dir_{a}"] = rel_err(got["dir"][:, i], ref["dir"][:, i], 1.0)
    out["E"] = rel_err(got["E"], ref["E"], ref["E0"])
    out["life_dx"] = rel_err(got["life_dx"], ref["life_dx"], ext)
    return out


def scaled_errors(got, ref, ext):
    """Per history, the largest error against the history's own scales (the
    extent for position and flight, 1 for cosines, E0 for E)."""
    m = np.zeros(len(ref))
    for i in range(3):
        m = np.maximum(m, np.abs(got["pos"][:, i] - ref["pos"][:, i]) / ext)
        m = np.maximum(m, np.abs(got["dir"][:, i] - ref["dir"][:, i]))
    m = np.maximum(m, np.abs(got["E"] - ref["E"]) / np.abs(ref["E0"]))
    m = np.maximum(m, np.abs(got["life_dx"] - ref["life_dx"]) / ext)
    return m


def event_distance(t, desc):
    if desc == SCATTER:
        return t["d_scatter"]
    if desc == CENSUS:
        return t["d_census"]
    return t["d_boundary"]  # BOUND (crossing or reflection) and EXIT


def classify_flip(tl, tg):
    """First segment where the two builds' traces part, and the margin of
    the comparison that decided it.  Returns (segment, kind, margin)."""
    n = min(len(tl), len(tg))
    a, b = tl[:n], tg[:n]
    # the face index matters only where the segment ended on a face
    on_face = (a["descriptor"] == BOUND) | (a["descriptor"] == EXIT)
    diff = np.flatnonzero((a["descriptor"] != b["descriptor"]) | (a["cell"] != b["cell"]) |
                          (on_face & (a["surface"] != b["surface"])) | (a["counter"] != b["counter"]))
    if len(diff) == 0:
        if len(tl) != len(tg):
            j = n - 1
            return j, "history end", float("nan")
        return -1, "none", float("nan")
    j = int(diff[0])
    x, y = a[j], b[j]
    dl, dg = int(x["descriptor"]), int(y["descriptor"])
    if dl == KILLED or dg == KILLED:
        r = x["E"] / x["E0"]
        return j, "cutoff", abs(r - 0.01) / 0.01
    if dl != dg:
        p, q = event_distance(x, dl), event_distance(x, dg)
        return j, "event order", abs(p - q) / max(abs(p), abs(q))
    if x["surface"] != y["surface"] or x["cell"] != y["cell"]:
        fq = np.sort(np.asarray(x["face_q"], np.float64))
        return j, "nearest face", abs(fq[1] - fq[0]) / max(abs(fq[1]), abs(fq[0]))
    return j, "rng counter", float("nan")


# ----------------------------------------------------------------- oracle
def oracle_update(orc, abs_E, trk_E):
    """Mesh::update_temperature on the oracle's cells (copies: the call
    zeroes the tallies); returns (T_e, T_r)."""
    a, t = abs_E.copy(), trk_E.copy()
    ta, pm = C.c_double(), C.c_double()
    import oracle as O
    orc.L.bo_update_temperature(C.byref(orc.mesh), C.byref(orc.cells), orc.dt, O._dptr(a), O._dptr(t),
                                C.byref(ta), C.byref(pm))
    return orc.arr["T_e"].copy(), orc.arr["T_r_diag"].copy()


def oracle_advance(orc, census, nd):
    orc.census = census
    orc.time += orc.dt
    orc.dt = nd
    orc.step_no += 1


def sync_twin(twin, orc):
    for k in orc.arr:
        twin.arr[k][:] = orc.arr[k]
    twin.census = orc.census
    twin.time, twin.dt, twin.step_no = orc.time, orc.dt, orc.step_no


def slice_sigma(orc, photons, nd, n_slices=N_SLICES):
    """Monte Carlo standard error of each cell's tallies from independent
    interleaved slices of the list (each slice's tally is one sample)."""
    A, T = [], []
    for b in range(n_slices):
        part = photons[b::n_slices].copy()
        a, t, *_ = orc.transport(part, nd)
        A.append(a)
        T.append(t)
    A, T = np.array(A), np.array(T)
    k = n_slices
    sa = np.sqrt(k * A.var(axis=0, ddof=1))
    st = np.sqrt(k * T.var(axis=0, ddof=1))
    return sa, st


# --------------------------------------------------------------- one step
def compare_step(gpu, orc, twin, ext, with_source=True, max_traced=5000):
    """One lockstep step; advances the oracle (and the GPU's clock)."""
    import oracle as O
    from branson_gb300.engine import arrays_to_records, records_to_arrays

    rep = {"step": orc.step_no}
    t0 = time.perf_counter()
    step, dt = orc.step_no, orc.dt
    T_e_pre = orc.arr["T_e"].copy()
    census_in = orc.census
    en, photons = orc.source(step)
    nd = orc.next_dt()
    rep["histories"] = int(len(photons))
    sync_twin(twin, orc)
    twin.census = census_in
    twin.arr["T_e"][:] = T_e_pre

    # ---- energies, counts and sourced photons on the device
    gpu.set_field("T_e", T_e_pre)
    if step > 1:
        gpu.set_photons(records_to_arrays(census_in))
    e = gpu.calculate_photon_energy(step, dt)
    ecmp = {}
    for f, key in (("op_a", "op_a"), ("f", "f"), ("emission_E", "emission_E"), ("census_E", "census_E"),
                   ("source_E", "source_E")):
        g = gpu.get_field(f)
        r = orc.arr[key]
        ecmp[f] = {"max_rel": float(np.max(rel_err(g, r, 1e-300))) if len(r) else 0.0,
                   "bit_identical": float(np.mean(g.view(np.uint64) == r.view(np.uint64)))}
    rep["energies"] = ecmp
    rep["counts_equal"] = bool(e["n_new_photons"] + e["n_initial_census"] + (len(census_in) if step > 1 else 0)
                               == len(photons))
    if with_source:
        gpu.source(step, dt)
        bank = np.sort(arrays_to_records(gpu.photons(), O.PHOTON_DTYPE), order="stream", kind="stable")
        _, twin_list = twin.source(step)
        tl = np.sort(twin_list, order="stream", kind="stable")
        ol = np.sort(photons, order="stream", kind="stable")
        src = {"n": int(len(bank)), "twin_mismatches": int(len(bank) != len(tl))}
        if len(bank) == len(tl):
            # sampling bit for bit; the weights follow the cell energies
            # (E = E_cell / count), whose powers of T round independently
            # on each side and are compared above within 1e-13
            sampled = [f for f in bank.dtype.names if f not in ("E", "E0")]
            src["twin_mismatches"] = int((~bitwise_same(bank[sampled], tl[sampled])).sum())
            src["twin_E_max_rel"] = float(max(np.max(rel_err(bank["E"], tl["E"], 1e-300)),
                                              np.max(rel_err(bank["E0"], tl["E0"], 1e-300))))
            ints = int((int_mismatch(bank, ol) | (bank["stream"] != ol["stream"])).sum())
            errs = scaled_errors(bank, ol, ext)
            src.update({"oracle_int_mismatches": ints, "oracle_max_scaled_err": float(errs.max()) if len(errs) else 0.0,
                        "oracle_bit_identical": float(bitwise_same(bank, ol).mean())})
        rep["source"] = src
        del bank, tl, ol, twin_list
    rep["t_source_s"] = time.perf_counter() - t0

    # ---- transport of the oracle's list: GPU drop-in, oracle, twin
    t1 = time.perf_counter()
    for f in ("op_a", "op_s", "f"):
        gpu.set_field(f, orc.arr[f])
    ph = records_to_arrays(photons)
    abs_g, trk_g, census_g, ce_g, ex_g = gpu.replicated_transport(ph, nd)
    end_g = arrays_to_records(ph, O.PHOTON_DTYPE)
    del ph
    census_g = arrays_to_records(census_g, O.PHOTON_DTYPE)
    gpu.update_temperature(dt)
    T_e_g, T_r_g = gpu.get_field("T_e"), gpu.get_field("T_r")
    gpu.advance_time(nd)
    rep["t_gpu_s"] = time.perf_counter() - t1

    t1 = time.perf_counter()
    end_l = photons.copy()
    abs_l, trk_l, census_l, ce_l, ex_l, segs, tl_s = orc.transport(end_l, nd)
    rep["segments"] = int(segs)
    rep["t_oracle_transport_s"] = tl_s
    end_t = photons.copy()
    abs_t, trk_t, census_t, ce_t, ex_t, _, tt_s = twin.transport(end_t, nd)
    rep["t_twin_transport_s"] = tt_s
    T_e_l, T_r_l = oracle_update(orc, abs_l, trk_l)
    T_e_t, T_r_t = oracle_update(twin, abs_t, trk_t)

    # ---- GPU vs the twin: bit for bit on every history
    tw = {"end_state_mismatches": int((~bitwise_same(end_g, end_t)).sum()),
          "census_mismatches": int(len(census_g) != len(census_t))}
    if len(census_g) == len(census_t):
        tw["census_mismatches"] = int((~bitwise_same(census_g, census_t)).sum())
    for name, g, r in (("abs_E", abs_g, abs_t), ("track_E", trk_g, trk_t), ("T_e", T_e_g, T_e_t),
                       ("T_r", T_r_g, T_r_t)):
        tw[f"max_rel_{name}"] = float(np.max(rel_err(g, r, 1e-300)))
    tw["census_exit_max_rel"] = float(np.max(rel_err([ce_g, ex_g], [ce_t, ex_t], 1e-300)))
    rep["gpu_vs_twin"] = tw

    # ---- GPU vs the oracle
    same = bitwise_same(end_g, end_l)
    flips = int_mismatch(end_g, end_l)
    errs = float_errors(end_g, end_l, ext)
    beyond = {k: int((v > END_RTOL).sum()) for k, v in errs.items()}
    any_beyond = np.zeros(len(end_l), bool)
    for v in errs.values():
        any_beyond |= v > END_RTOL
    nonflip = ~flips
    scaled = scaled_errors(end_g[nonflip], end_l[nonflip], ext)
    orep = {"bit_identical": float(same.mean()), "beyond_1e-12_plain": beyond,
            "histories_beyond_1e-12_plain": int(any_beyond.sum()),
            "nonflip_beyond_1e-12_plain": int((any_beyond & nonflip).sum()),
            "nonflip_max_scaled_err": float(scaled.max()) if len(scaled) else 0.0,
            "flips": int(flips.sum())}
    # flipped histories: where the two CPU builds part, and by how much
    idx = np.flatnonzero(flips)
    kinds, margins, firsts = {}, [], []
    for k in idx[:max_traced]:
        trl, _ = orc.trace(photons[k])
        trg, _ = twin.trace(photons[k])
        j, kind, margin = classify_flip(trl, trg)
        kinds[kind] = kinds.get(kind, 0) + 1
        margins.append(margin)
        firsts.append(j)
    margins = np.array(margins)
    fin = margins[np.isfinite(margins)]
    orep["flip_kinds"] = kinds
    orep["flips_traced"] = int(min(len(idx), max_traced))
    orep["flip_max_margin"] = float(fin.max()) if len(fin) else None
    orep["flips_near_tie"] = int((fin <= NEAR_TIE).sum())
    orep["flips_unexplained"] = int(len(margins) - (fin <= NEAR_TIE).sum())
    orep["flip_first_segment_median"] = float(np.median(firsts)) if firsts else None

    # per cell, with the flipped histories' own tallies taken out
    touched = np.zeros(len(abs_l), bool)
    if len(idx):
        sub = photons[idx].copy()
        ph = records_to_arrays(sub)
        abs_gf, trk_gf, _, ce_gf, ex_gf = gpu.replicated_transport(ph, nd)
        abs_lf, trk_lf, _, ce_lf, ex_lf, _, _ = orc.transport(sub.copy(), nd)
        touched = (abs_gf != 0) | (abs_lf != 0) | (trk_gf != 0) | (trk_lf != 0)
    else:
        abs_gf = trk_gf = abs_lf = trk_lf = np.zeros_like(abs_l)
        ce_gf = ex_gf = ce_lf = ex_lf = 0.0
    corr = {}
    for name, g, gf, r, rf in (("abs_E", abs_g, abs_gf, abs_l, abs_lf), ("track_E", trk_g, trk_gf, trk_l, trk_lf)):
        d = np.abs((g - gf) - (r - rf))
        scale = np.abs(r)
        ok = (d == 0) | (d <= CELL_RTOL * scale)
        corr[name] = {"max_rel": float(np.max(np.where(scale > 0, d / np.where(scale > 0, scale, 1), d))),
                      "cells_beyond": int((~ok).sum())}
    dce = abs((ce_g - ce_gf) - (ce_l - ce_lf)) / max(abs(ce_l), 1e-300)
    dex = abs((ex_g - ex_gf) - (ex_l - ex_lf)) / max(abs(ex_l), 1e-300)
    corr["census_exit_max_rel"] = float(max(dce, dex))
    orep["flip_corrected"] = corr
    orep["cells_touched_by_flips"] = int(touched.sum())
    untouched = ~touched
    orep["untouched_max_rel"] = {
        name: float(np.max(rel_err(g[untouched], r[untouched], 1e-300))) if untouched.any() else 0.0
        for name, g, r in (("abs_E", abs_g, abs_l), ("track_E", trk_g, trk_l), ("T_e", T_e_g, T_e_l),
                           ("T_r", T_r_g, T_r_l))}
    if touched.any():
        sa, st = slice_sigma(orc, photons, nd)
        za = np.abs(abs_g - abs_l)[touched] / np.where(sa[touched] > 0, sa[touched], np.inf)
        zt = np.abs(trk_g - trk_l)[touched] / np.where(st[touched] > 0, st[touched], np.inf)
        orep["z_abs_E_max"] = float(za.max())
        orep["z_track_E_max"] = float(zt.max())
        orep["z_abs_E_median"] = float(np.median(za))
        c = np.flatnonzero(touched)[int(np.argmax(za))]
        orep["worst_cell"] = {"cell": int(c), "abs_E_gpu": float(abs_g[c]), "abs_E_oracle": float(abs_l[c]),
                              "rel": float(abs(abs_g[c] - abs_l[c]) / abs(abs_l[c])) if abs_l[c] else None,
                              "sigma": float(sa[c]), "z": float(za.max())}
    # census: the same streams, compared where both have them
    sg, sl = set(census_g["stream"].tolist()), set(census_l["stream"].tolist())
    orep["census_only_in_one"] = len(sg ^ sl)
    both_g = np.isin(census_g["stream"], census_l["stream"])
    both_l = np.isin(census_l["stream"], census_g["stream"])
    cg, cl = census_g[both_g], census_l[both_l]
    orep["census_order_equal"] = bool(np.array_equal(cg["stream"], cl["stream"]))
    cnf = ~int_mismatch(cg, cl)
    orep["census_max_scaled_err"] = float(scaled_errors(cg[cnf], cl[cnf], ext).max()) if cnf.any() else 0.0
    rep["gpu_vs_oracle"] = orep
    rep["t_compare_s"] = time.perf_counter() - t1

    oracle_advance(orc, census_l, nd)
    return rep


def run_case(name, n_threads=None, steps=None, log=None):
    """All compared steps of a case; returns the report."""
    import oracle as O
    from branson_gb300.engine import ReplicatedIMC

    dk, warmup, n_cmp = case_deck(name)
    if steps is not None:
        n_cmp = steps
    n_threads = n_threads or os.cpu_count() or 1
    ext = extent(dk)
    t0 = time.perf_counter()
    orc = O.Oracle(dk, n_threads=n_threads)
    twin = O.Oracle(copy.deepcopy(dk), n_threads=n_threads, math="gpu")
    for _ in range(warmup):
        orc.step()
    report = {"case": name, "cells": int(dk.n_cells), "photons_per_step": int(dk.photons), "groups": dk.n_groups,
              "warmup_steps": warmup, "threads": n_threads, "t_warmup_s": time.perf_counter() - t0, "steps": []}
    with ReplicatedIMC(dk) as gpu:
        gpu.step_no, gpu.time, gpu.dt = orc.step_no, orc.time, orc.dt
        for _ in range(n_cmp):
            r = compare_step(gpu, orc, twin, ext)
            report["steps"].append(r)
            if log:
                log(summary_line(name, r))
    report["t_total_s"] = time.perf_counter() - t0
    return report


def summary_line(name, r):
    o, t = r["gpu_vs_oracle"], r["gpu_vs_twin"]
    return (f"{name} step {r['step']}: {r['histories']} histories, {r['segments']} segments; "
            f"GPU vs twin: {t['end_state_mismatches']} end states differ; GPU vs oracle: "
            f"{100 * o['bit_identical']:.3f}% bit-identical, {o['flips']} flips "
            f"({o['flips_near_tie']} near ties, max margin {o['flip_max_margin']}), "
            f"{o['cells_touched_by_flips']} cells touched, flip-corrected abs_E max rel "
            f"{o['flip_corrected']['abs_E']['max_rel']:.2e}, untouched T_e max rel "
            f"{o['untouched_max_rel']['T_e']:.2e}, z_max {o.get('z_abs_E_max')}")


def check_step(r):
    """The pass criteria of one compared step (raises AssertionError)."""
    name = f"step {r['step']}"
    assert r["counts_equal"], f"{name}: photon counts differ"
    for f, v in r["energies"].items():
        assert v["max_rel"] <= ENERGY_RTOL, f"{name}: {f} differs by {v['max_rel']}"
    if "source" in r:
        s = r["source"]
        assert s["twin_mismatches"] == 0, f"{name}: {s['twin_mismatches']} sourced photons differ from the twin"
        assert s["twin_E_max_rel"] <= ENERGY_RTOL, f"{name}: sourced weights differ by {s['twin_E_max_rel']}"
        assert s["oracle_int_mismatches"] == 0, f"{name}: sourced photons' integers differ from the oracle"
        assert s["oracle_max_scaled_err"] <= END_RTOL, f"{name}: sourced photons differ by {s['oracle_max_scaled_err']}"
    t = r["gpu_vs_twin"]
    assert t["end_state_mismatches"] == 0, f"{name}: {t['end_state_mismatches']} end states differ from the twin"
    assert t["census_mismatches"] == 0, f"{name}: census differs from the twin"
    for k in ("abs_E", "track_E", "T_e", "T_r"):
        assert t[f"max_rel_{k}"] <= CELL_RTOL, f"{name}: {k} differs from the twin by {t[f'max_rel_{k}']}"
    assert t["census_exit_max_rel"] <= CELL_RTOL
    o = r["gpu_vs_oracle"]
    assert o["nonflip_max_scaled_err"] <= END_RTOL, f"{name}: a history without a flip differs by " \
                                                    f"{o['nonflip_max_scaled_err']} of its scale"
    assert o["flips_unexplained"] == 0, f"{name}: {o['flips_unexplained']} flips are not near ties: {o['flip_kinds']}"
    for k in ("abs_E", "track_E"):
        c = o["flip_corrected"][k]
        assert c["cells_beyond"] == 0, f"{name}: {c['cells_beyond']} cells' {k} differ beyond 1e-10 " \
                                       f"with the flipped histories taken out (max {c['max_rel']})"
    assert o["flip_corrected"]["census_exit_max_rel"] <= CELL_RTOL
    for k, v in o["untouched_max_rel"].items():
        assert v <= CELL_RTOL, f"{name}: {k} differs by {v} on a cell no flipped history touched"
    if o["cells_touched_by_flips"]:
        assert o["z_abs_E_max"] <= Z_MAX and o["z_track_E_max"] <= Z_MAX, \
            f"{name}: z-scores {o['z_abs_E_max']}, {o['z_track_E_max']}"
    assert o["census_order_equal"], f"{name}: census order differs"
    assert o["census_max_scaled_err"] <= END_RTOL


def main():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("case", choices=["hot_zone", "marshak", "hohlraum", "hot_zone_small"])
    p.add_argument("--json", default=None, help="write the report here")
    p.add_argument("--steps", type=int, default=None, help="compared steps (default: the case's)")
    a = p.parse_args()
    rep = run_case(a.case, steps=a.steps, log=lambda s: print(s, flush=True))
    if a.json:
        with open(a.json, "w") as fh:
            json.dump(rep, fh, indent=1)
    for r in rep["steps"]:
        check_step(r)
    print(f"{a.case}: all {len(rep['steps'])} compared steps pass ({rep['t_total_s']:.1f} s)")


if __name__ == "__main__":
    main()
