"""Generate the golden vectors in tests/golden/ from the upstream code.

Runs oracle/_ref/ref_harness_g{1,30} -- the upstream Branson headers compiled
unmodified from the reference checkout (make -C oracle ref) -- on three
small synthetic decks and stores, per time step, the photon list before
transport, the end states and census after transport, and the per-cell
energies, tallies and temperatures, as compressed .npz files.  The comb
fixture also holds each step's census after the upstream comb_photons
(census_functions.h:48-93) with RNG(seed, COMB_STREAM) and COMB_MAX.

    python tests/golden/make_golden.py        # needs the reference checkout

The decks are generated by branson_gb300.deck, so the fixtures are
self-describing: each .npz also holds the deck XML it was made from.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
TMP_ROOT = os.path.join(ROOT, "oracle", "_ref")  # scratch for harness output, git-ignored

from branson_gb300 import deck as D  # noqa: E402
import oracle as O  # noqa: E402

CASES = {
    "marshak_g1": (lambda: D.marshak_wave(n_cells=40, photons=1500, n_steps=2), 2),
    "hot_zone_g1": (lambda: D.hot_zone(n_per_axis=5, photons=1500, n_steps=2), 2),
    "hohlraum_g30": (lambda: D.hohlraum(n_per_axis=8, photons=1500, n_steps=2, n_groups=30), 2),
}
COMB_CASE = "comb_marshak_g1"
COMB_MAX, COMB_STREAM = 100, 4242


def comb_fixture():
    dk = D.marshak_wave(n_cells=40, photons=1500, n_steps=2)
    with tempfile.TemporaryDirectory(dir=TMP_ROOT) as tmp:
        O.run_reference_harness(dk, tmp, 2, n_threads=1, comb=(COMB_MAX, COMB_STREAM))
        out = {"deck_xml": np.array(dk.to_xml()), "n_cells": np.array(dk.n_cells), "seed": np.array(dk.seed),
               "comb_max": np.array(COMB_MAX), "comb_stream": np.array(COMB_STREAM), "n_steps": np.array(2)}
        for s in (1, 2):
            h = O.read_harness_step(tmp, s, dk.n_cells)
            out[f"s{s}_census"] = h["census"]
            out[f"s{s}_comb"] = h["comb"]
            out[f"s{s}_comb_draws"] = np.array(int(h["scalars"]["comb_draws"]))
    path = os.path.join(HERE, f"{COMB_CASE}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path)} bytes")


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    for name, (mk, steps) in CASES.items():
        dk = mk()
        with tempfile.TemporaryDirectory(dir=TMP_ROOT) as tmp:
            O.run_reference_harness(dk, tmp, steps, n_threads=1)
            out = {"deck_xml": np.array(dk.to_xml()), "n_groups": np.array(dk.n_groups),
                   "n_steps": np.array(steps)}
            for s in range(1, steps + 1):
                h = O.read_harness_step(tmp, s, dk.n_cells)
                for k in ("source", "end", "census", "cells"):
                    out[f"s{s}_{k}"] = h[k]
                out[f"s{s}_scalars_keys"] = np.array(sorted(h["scalars"]))
                out[f"s{s}_scalars"] = np.array([h["scalars"][k] for k in sorted(h["scalars"])])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {os.path.getsize(path)} bytes")
    comb_fixture()


if __name__ == "__main__":
    main()
