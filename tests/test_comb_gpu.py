"""Census comb on the GPU (bgs_comb_census) against the oracle's restatement
of comb_photons (census_functions.h:48-93), which the CPU suite pins to the
upstream code's own output (tests/golden/comb_marshak_g1.npz).

  * after a device step, the combed census equals the oracle's comb of the
    same census list bit for bit (survivors, order, energies, RNG counters)
    and the comb RNG advances one draw per census photon;
  * the census energy is conserved to the rounding of the comb energy, the
    next step starts from the combed census and runs clean;
  * a comb without a census in the bank is refused.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _decks():
    from branson_gb300 import deck as D
    return {
        "marshak": D.marshak_wave(n_cells=100, photons=20000, n_steps=3),
        "hot_zone": D.hot_zone(n_per_axis=10, photons=20000, n_steps=3),
    }


@pytest.mark.parametrize("name", ["marshak", "hot_zone"])
def test_comb_matches_oracle(gpu_lib, name):
    import oracle as O
    from branson_gb300.engine import ReplicatedIMC, arrays_to_records

    dk = _decks()[name]
    with ReplicatedIMC(dk) as gpu:
        counter = 0
        for step in range(2):
            gpu.step()
            census = arrays_to_records(gpu.photons(), O.PHOTON_DTYPE)
            n = len(census)
            assert n > 50, n
            max_census = max(1, n // 3)
            want, want_ctr = O.comb(census, dk.n_cells, max_census, dk.seed, 4242, counter)
            kept, counter = gpu.comb_census(max_census, 4242, counter)
            assert counter == want_ctr and kept == len(want) < n
            got = arrays_to_records(gpu.photons(), O.PHOTON_DTYPE)
            for f in want.dtype.names:
                np.testing.assert_array_equal(got[f], want[f], err_msg=f"{name} step {step + 1} comb {f}")
            np.testing.assert_allclose(got["E"].sum(), census["E"].sum(), rtol=0.0,
                                       atol=1e-12 * census["E"].sum())
            rep = gpu.step()
            assert rep.device_flags == 0 and rep.n_transported >= kept


def test_comb_needs_a_census(gpu_lib):
    from branson_gb300.engine import BransonError, ReplicatedIMC
    dk = _decks()["marshak"]
    with ReplicatedIMC(dk) as gpu:
        assert gpu.comb_census(10, 1) == (0, 0)  # nothing yet: an empty census is left alone
        gpu.step()
        ph = gpu.photons()
        gpu.set_photons(ph)  # a bank to transport, not a census
        with pytest.raises(BransonError):
            gpu.comb_census(10, 1)
        with pytest.raises(BransonError):
            gpu.comb_census(0, 1)
