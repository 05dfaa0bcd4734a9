"""Batched stepping on the GPU (bgs_batch_step): problems of uneven size,
group count and photon count stepped together through one persistent
transport launch give, problem by problem, exactly the results of stepping
each context on its own -- with the step recorded as a CUDA graph and with
plain launches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ensemble():
    from branson_gb300 import deck as D
    decks = [D.hot_zone(n_per_axis=10, photons=20000, n_steps=3),
             D.marshak_wave(n_cells=100, photons=15000, n_steps=3),
             D.random_opacity_cube(n_per_axis=6, photons=8000, seed=4),
             D.hohlraum(n_per_axis=10, photons=12000, n_steps=3, n_groups=30)]
    decks += D.batch_ensemble(n_problems=5, master_seed=11, side_range=(4, 12), photon_median=5000,
                              photon_range=(1000, 20000))
    for dk in decks:  # several steps for every problem
        dk.t_stop = dk.t_start + 3 * dk.dt_start
    return decks


def _state(imc):
    ph = imc.photons()
    return ({f: imc.get_field(f) for f in ("T_e", "T_r", "abs_E", "track_E")},
            {k: v.copy() for k, v in ph.arrays.items()})


@pytest.mark.parametrize("graph", [1, 0], ids=["graph", "plain"])
def test_batched_steps_equal_single_problem_steps(gpu_lib, graph):
    from branson_gb300.engine import BatchIMC, ReplicatedIMC

    decks = _ensemble()
    with BatchIMC(decks) as batch:
        batch.set_option("graph", graph)
        singles = [ReplicatedIMC(dk) for dk in _ensemble()]
        try:
            for step in range(3):
                reps_b = batch.step(sync=True)
                reps_s = [s.step(sync=True) for s in singles]
                for i, (rb, rs) in enumerate(zip(reps_b, reps_s)):
                    assert (rb.n_transported, rb.n_census, rb.n_segments) == \
                        (rs.n_transported, rs.n_census, rs.n_segments), (step, i)
                    assert (rb.census_E, rb.exit_E, rb.absorbed_E, rb.post_mat_E) == \
                        (rs.census_E, rs.exit_E, rs.absorbed_E, rs.post_mat_E), (step, i)
                    fb, pb = _state(batch.problems[i])
                    fs, ps = _state(singles[i])
                    for k in fb:
                        np.testing.assert_array_equal(fb[k], fs[k], err_msg=f"step {step} problem {i} {k}")
                    for k in pb:
                        np.testing.assert_array_equal(pb[k], ps[k], err_msg=f"step {step} problem {i} bank {k}")
            ms, launches = batch.last_transport_ms()
            assert ms > 0.0 and launches > 0
        finally:
            for s in singles:
                s.close()


def test_batch_rejects_bad_arguments(gpu_lib):
    import ctypes as C
    from branson_gb300 import _lib, deck as D
    from branson_gb300.engine import ReplicatedIMC

    lib = _lib.load()
    imc = ReplicatedIMC(D.marshak_wave(n_cells=10, photons=100, n_steps=1))
    try:
        h = C.c_void_p()
        same = (C.c_void_p * 2)(imc.ctx.value, imc.ctx.value)
        assert lib.bgs_batch_create(C.byref(h), 2, same) == _lib.ERR_INVALID
        assert lib.bgs_batch_create(C.byref(h), 0, same) == _lib.ERR_INVALID
    finally:
        imc.close()


def test_batched_adjoint_equals_per_problem(gpu_lib):
    """One replay launch over every problem's tape gives each problem's
    gradient bit for bit as its own backward does."""
    from branson_gb300 import deck as D
    from branson_gb300.adjoint import batch_backward, batch_forward
    from branson_gb300.engine import BatchIMC

    decks = [D.random_opacity_cube(n_per_axis=n, photons=p, seed=s)
             for n, p, s in ((4, 3000, 1), (6, 12000, 2), (8, 20000, 3))]
    decks += [D.hot_zone(n_per_axis=10, photons=15000, n_steps=2)]
    decks += D.batch_ensemble(n_problems=3, master_seed=5, side_range=(4, 10), photon_median=4000,
                              photon_range=(1000, 9000))
    rng = np.random.default_rng(0)
    with BatchIMC(decks) as batch:
        abs_E, tapes = batch_forward(batch)
        ws = [rng.uniform(-1.0, 1.0, p.n_cells) for p in batch.problems]
        grads = batch_backward(batch, tapes, ws)
        for i, (p, t, w) in enumerate(zip(batch.problems, tapes, ws)):
            own = np.empty(p.n_cells)
            rc = batch.lib.bgs_adjoint_backward(p.ctx, t.handle, w.ctypes.data, own.ctypes.data)
            assert rc == 0, p.lib.bgs_last_error(p.ctx)
            np.testing.assert_array_equal(grads[i], own, err_msg=f"problem {i}")
            assert np.any(own != 0.0)
        for t in tapes:
            t.close()
