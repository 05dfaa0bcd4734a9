"""The oracle's GPU-math twin (make -C oracle gpumath) and the per-segment
trace, on the CPU: the twin differs from the oracle only through the
rounding of -log, exp, sin and cos, so its histories agree with the
oracle's within 1e-12 of their scales unless a branch flipped at a near tie;
the trace reproduces the transport; the flip classifier of the full-size
parity check finds the comparison at which two traces part."""
import numpy as np

import fullsize as F


def _pair(dk, threads=4):
    import copy
    import oracle as O
    orc = O.Oracle(dk, n_threads=threads)
    twin = O.Oracle(copy.deepcopy(dk), n_threads=threads, math="gpu")
    return orc, twin


def test_twin_agrees_up_to_rounding():
    from branson_gb300 import deck as D
    dk = D.hot_zone(n_per_axis=15, photons=200_000, n_steps=3)
    orc, twin = _pair(dk)
    _, photons = orc.source(1)
    _, tw_list = twin.source(1)
    assert len(tw_list) == len(photons)
    nd = orc.next_dt()
    end_l, end_t = photons.copy(), photons.copy()
    a_l, t_l, c_l, *_ = orc.transport(end_l, nd)
    a_t, t_t, c_t, *_ = twin.transport(end_t, nd)
    flips = F.int_mismatch(end_t, end_l)
    ext = F.extent(dk)
    assert F.scaled_errors(end_t[~flips], end_l[~flips], ext).max() <= F.END_RTOL
    same = F.bitwise_same(end_t, end_l).mean()
    assert 0.5 < same < 1.0  # the rounding differs, and mostly not at all
    for k in np.flatnonzero(flips)[:50]:
        j, kind, margin = F.classify_flip(orc.trace(photons[k])[0], twin.trace(photons[k])[0])
        assert j >= 0 and margin <= F.NEAR_TIE, (kind, margin)
    # the sourced photons differ only in the rounding of their directions
    so = np.sort(photons, order="stream")
    st = np.sort(tw_list, order="stream")
    assert not F.int_mismatch(so, st).any()
    assert F.scaled_errors(st, so, ext).max() <= F.END_RTOL


def test_trace_reproduces_transport():
    from branson_gb300 import deck as D
    import oracle as O
    for math in ("libm", "gpu"):
        dk = D.marshak_wave(n_cells=100, photons=20_000, n_steps=2)
        orc = O.Oracle(dk, n_threads=2, math=math)
        _, photons = orc.source(1)
        nd = orc.next_dt()
        end = photons.copy()
        orc.transport(end, nd)
        for k in range(0, len(photons), 997):
            tr, e = orc.trace(photons[k])
            e = np.array([e])
            if e["descriptor"][0] == F.CENSUS:  # post-processing resets the census flight
                e["life_dx"] = F.C_LIGHT * nd
            assert F.bitwise_same(e, end[k:k + 1])[0]
            assert len(tr) >= 1 and tr[-1]["descriptor"] == end[k]["descriptor"]
            assert tr[-1]["counter"] == (int(end[k]["counter"]) & 0xFFFFFFFF)


def test_classify_flip():
    import oracle as O
    t = np.zeros(3, O.TRACE_DTYPE)
    t["descriptor"] = [F.SCATTER, F.BOUND, F.CENSUS]
    t["d_scatter"] = [0.1, 0.5, 0.7]
    t["d_boundary"] = [0.3, 0.2, 0.6]
    t["d_census"] = [1.0, 0.9, 0.4]
    t["E"], t["E0"] = 0.5, 1.0
    u = t.copy()
    assert F.classify_flip(t, u)[:2] == (-1, "none")
    u[1]["descriptor"] = F.SCATTER
    u[1]["d_scatter"] = 0.2 * (1 + 1e-15)
    t[1]["d_scatter"] = 0.2 * (1 + 1e-15)
    j, kind, m = F.classify_flip(t, u)
    assert (j, kind) == (1, "event order") and m < 1e-14
    v = t.copy()
    v[2]["descriptor"] = F.KILLED
    v[2]["E"], t[2]["E"] = 0.01 * (1 - 1e-16), 0.01
    j, kind, m = F.classify_flip(t, v)
    assert (j, kind) == (2, "cutoff") and m < 1e-14
    w = t.copy()
    w[1]["surface"] = 3
    t[1]["face_q"] = [0.2, 0.2 * (1 + 2e-16), 5.0]
    j, kind, m = F.classify_flip(t, w)
    assert (j, kind) == (1, "nearest face") and m < 1e-15
