"""The adjoint estimator's algebra, on the CPU replay in the oracle.

For one step's histories, L at perturbed opacities can be estimated on the
unperturbed paths with causal likelihood ratios (oracle bo_adjoint_reweighted);
that function is smooth, and its derivative at the unperturbed opacities is,
history by history, the adjoint estimator (pathwise weight-decay and Fleck
terms, score-function collision terms, emission weight term).  So its
central difference must reproduce the replayed gradient to finite-difference
precision, cell by cell.  Also: the replay's L equals the forward tally
sum, and the gradient is linear in the tally weights.
"""
import numpy as np
import pytest

import oracle as O
from branson_gb300 import deck as D


def _run(dk, n_threads=2):
    orc = O.Oracle(dk, n_threads=n_threads)
    _, photons = orc.source(1)
    start = photons.copy()
    abs_E, _, _, _, _, segs, _ = orc.transport(photons, orc.next_dt())
    return orc, start, abs_E, segs


def _scattering_cube(n=4, photons=3000, seed=3):
    dk = D.random_opacity_cube(n_per_axis=n, photons=photons, seed=seed)
    rng = np.random.default_rng(seed)
    for r in dk.regions:
        r.opacS = float(rng.uniform(0.0, 5.0))
    dk.n_groups = 3
    return dk


@pytest.mark.parametrize("make", [lambda: D.random_opacity_cube(n_per_axis=4, photons=3000, seed=11),
                                  _scattering_cube],
                         ids=["random_cube", "scattering_3groups"])
def test_replay_matches_reweighted_finite_difference(make):
    dk = make()
    orc, start, abs_E, segs = _run(dk)
    w = np.random.default_rng(5).uniform(0.0, 1.0, orc.n_cells)
    op_a, op_s, f = orc.arr["op_a"].copy(), orc.arr["op_s"].copy(), orc.arr["f"].copy()
    scale, bound = O.adjoint_scale(w, start, op_a, op_s, f, segs)
    grad, dropped = orc.adjoint(start, w, scale, bound)
    assert dropped == 0
    # the replay retraces the forward: its L is the weighted tally
    L0 = orc.reweighted_L(start, w, op_a, f)
    assert abs(L0 - np.dot(w, abs_E)) <= 1e-12 * abs(L0)
    cells = np.argsort(-np.abs(grad))[:6]
    for j in cells:
        d = 1e-5
        opp, opm = op_a.copy(), op_a.copy()
        opp[j] *= 1 + d
        opm[j] *= 1 - d
        Lp = orc.reweighted_L(start, w, opp, orc.fleck(opp, orc.dt))
        Lm = orc.reweighted_L(start, w, opm, orc.fleck(opm, orc.dt))
        fd = (Lp - Lm) / (2 * d * op_a[j])
        # the difference quotient is round-off limited near 1e-6 here
        assert abs(grad[j] - fd) <= 2e-5 * abs(fd) + 1e-12 * abs(L0), (j, grad[j], fd)


def test_gradient_is_linear_in_the_weights():
    dk = D.random_opacity_cube(n_per_axis=4, photons=2000, seed=2)
    orc, start, _, segs = _run(dk)
    rng = np.random.default_rng(1)
    w1, w2 = rng.uniform(0, 1, orc.n_cells), rng.uniform(-1, 1, orc.n_cells)
    op_a, op_s, f = orc.arr["op_a"], orc.arr["op_s"], orc.arr["f"]
    wsum = w1 + w2
    scale, bound = O.adjoint_scale(np.abs(w1) + np.abs(w2), start, op_a, op_s, f, segs)
    g1, _ = orc.adjoint(start, w1, scale, bound)
    g2, _ = orc.adjoint(start, w2, scale, bound)
    g12, _ = orc.adjoint(start, wsum, scale, bound)
    np.testing.assert_allclose(g12, g1 + g2, rtol=1e-9, atol=1e-12 * np.max(np.abs(g12)))


def test_fixed_point_sums_do_not_depend_on_threads():
    dk = D.random_opacity_cube(n_per_axis=4, photons=2000, seed=4)
    orc, start, _, segs = _run(dk)
    w = np.random.default_rng(2).uniform(-1, 1, orc.n_cells)
    scale, bound = O.adjoint_scale(w, start, orc.arr["op_a"], orc.arr["op_s"], orc.arr["f"], segs)
    g1, _ = orc.adjoint(start, w, scale, bound, n_threads=1)
    g4, _ = orc.adjoint(start, w, scale, bound, n_threads=4)
    np.testing.assert_array_equal(g1, g4)


def test_cutoff_jump_is_the_only_bias():
    """The estimator does not differentiate the E/E0 < 0.01 cutoff
    (photon.h:47-49): a history crossing it gives up its last 1% at once, a
    jump of 0.01 E0 in the tally that a pathwise derivative cannot see.  On
    a one-cell pure absorber (T_e = 0, so f = 1 and no effective scattering;
    census photons only, whose counts and weights do not depend on sigma_a)
    every history is one straight flight of length d to a face, killed when
    sigma_a d > ln 100.  The common-random-number central difference of the
    oracle's tally then exceeds the replayed gradient by exactly the counted
    jumps, sum over crossing photons of 0.01 E0 / (2 h sigma_a)."""
    from branson_gb300.deck import Deck, Division, Region, VACUUM
    dk = Deck(t_start=0.0, t_stop=0.01, dt_start=0.01, t_mult=1.0, dt_max=1.0, photons=200000, seed=21,
              x_divisions=[Division(0.0, 1.0, 1)], y_divisions=[Division(0.0, 1.0, 1)],
              z_divisions=[Division(0.0, 1.0, 1)], region_map={(0, 0, 0): 1}, bc=(VACUUM,) * 6, T_source=0.0,
              regions=[Region(1, 0.1, 1.0, 5.0, 0.0, 0.0, 0.0, 0.0, 0.5)])
    orc, start, _, segs = _run(dk, n_threads=4)
    assert orc.arr["f"][0] == 1.0 and np.all(start["source_type"] == 0)
    sig, nd = orc.arr["op_a"][0], orc.dt
    w = np.ones(1)
    scale, bound = O.adjoint_scale(w, start, orc.arr["op_a"], orc.arr["op_s"], orc.arr["f"], segs)
    grad, dropped = orc.adjoint(start, w, scale, bound)
    assert dropped == 0

    def tally(s):
        orc.arr["op_a"][:] = s
        a, *_ = orc.transport(start.copy(), nd)
        orc.arr["op_a"][:] = sig
        return a.sum()

    pos, d = start["pos"], start["dir"]
    flight = np.where(d > 0, (1.0 - pos) / d, -pos / d).min(axis=1)  # to the first face
    for h in (3e-3, 1e-3):
        fd = (tally(sig * (1 + h)) - tally(sig * (1 - h))) / (2 * h * sig)
        cross = (sig * (1 - h) * flight < np.log(100.0)) & (np.log(100.0) < sig * (1 + h) * flight)
        jumps = 0.01 * start["E0"][cross].sum() / (2 * h * sig)
        assert cross.sum() > 50
        assert abs((fd - grad[0]) - jumps) <= 0.01 * jumps, (h, fd, grad[0], jumps)
