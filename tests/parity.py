"""Comparison helpers shared by the parity tests (GPU path vs the oracle).

Tolerances are the contract's: per-history end states within 1e-12
relative, per-cell tallies and temperatures within 1e-10 relative.
"""
import numpy as np

END_RTOL = 1e-12
CELL_RTOL = 1e-10


def close(a, b, rtol, atol_scale=None, what=""):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    scale = np.maximum(np.abs(b), atol_scale if atol_scale is not None else 0.0)
    bad = np.abs(a - b) > rtol * scale
    bad &= ~((a == b) | (np.isnan(a) & np.isnan(b)))
    if bad.any():
        i = int(np.argmax(bad))
        raise AssertionError(f"{what}: {int(bad.sum())} of {a.size} differ beyond rtol {rtol}; "
                             f"first at {i}: {a.flat[i]!r} vs {b.flat[i]!r}")


def compare_photons(got, ref, extent, what="photons", check_desc=True, rtol=END_RTOL):
    """Record arrays (oracle PHOTON_DTYPE) in the same order."""
    assert len(got) == len(ref), f"{what}: {len(got)} vs {len(ref)} photons"
    if len(ref) == 0:
        return
    for f in ("stream", "cell", "group"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{what}.{f}")
    np.testing.assert_array_equal(got["counter"], ref["counter"], err_msg=f"{what}.counter")
    if check_desc:
        np.testing.assert_array_equal(got["descriptor"], ref["descriptor"], err_msg=f"{what}.descriptor")
    close(got["pos"], ref["pos"], rtol, extent, f"{what}.pos")
    close(got["dir"], ref["dir"], rtol, 1.0, f"{what}.dir")
    # energy weights relative to the history's own scale, its birth weight E0
    close_to_scale(got["E"], ref["E"], rtol, ref["E0"], f"{what}.E")
    close(got["E0"], ref["E0"], rtol, 0.0, f"{what}.E0")
    close(got["life_dx"], ref["life_dx"], rtol, extent, f"{what}.life_dx")


def close_to_scale(a, b, rtol, scale, what=""):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    bad = np.abs(a - b) > rtol * np.maximum(np.abs(b), np.abs(scale))
    if bad.any():
        i = int(np.argmax(bad))
        raise AssertionError(f"{what}: {int(bad.sum())} of {a.size} differ beyond rtol {rtol} of the "
                             f"history scale; first at {i}: {a[i]!r} vs {b[i]!r} (scale {scale[i]!r})")


def bitwise_fraction(got, ref):
    """Share of histories whose whole end state is bit-identical."""
    if len(ref) == 0:
        return 1.0
    same = np.ones(len(ref), bool)
    for f in ("pos", "dir"):
        same &= np.all(got[f] == ref[f], axis=1)
    for f in ("E", "life_dx", "counter", "cell", "group", "descriptor"):
        same &= got[f] == ref[f]
    return float(same.mean())


def by_stream(rec):
    return rec[np.argsort(rec["stream"], kind="stable")]
