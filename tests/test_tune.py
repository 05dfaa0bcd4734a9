"""Autotuner (branson_gb300/tune.py): the candidate set covers block size,
histories per thread and history vs event mode (CPU); on the GPU the tuner
times every candidate, applies the fastest, and the tuned context steps to
exactly the results of an untuned one."""
import numpy as np
import pytest


def test_candidates_cover_the_three_choices():
    from branson_gb300 import _lib
    from branson_gb300.tune import default_candidates
    c = default_candidates()
    assert {s.threads for s in c} == {64, 128, 256}
    assert {s.grid_fraction for s in c if s.algorithm == _lib.HISTORY} == {1.0, 0.5, 0.25}
    assert {s.algorithm for s in c} == {_lib.HISTORY, _lib.EVENT}
    assert len({s.label() for s in c}) == len(c)


@pytest.mark.gpu
def test_tuned_context_steps_to_the_same_results(gpu_lib):
    from branson_gb300 import deck as D
    from branson_gb300.engine import ReplicatedIMC
    from branson_gb300.tune import tune

    dk = D.hot_zone(n_per_axis=10, photons=20000, n_steps=3)
    with ReplicatedIMC(dk) as a, ReplicatedIMC(dk) as b:
        res = tune(a, repeats=1)
        assert len(res.timings) >= 10 and res.best_ms > 0
        assert res.best in [c for c, _ in res.timings]
        print("tuned:", res.best.label(), f"{res.best_ms:.3f} ms;",
              ", ".join(f"{c.label()} {ms:.3f}" for c, ms in res.timings))
        for _ in range(2):
            ra, rb = a.step(), b.step()
            assert (ra.n_transported, ra.n_census, ra.n_segments) == (rb.n_transported, rb.n_census, rb.n_segments)
            for f in ("T_e", "abs_E", "track_E"):
                np.testing.assert_array_equal(a.get_field(f), b.get_field(f))
