"""Edge cases of the drop-in transport (bgs_replicated_transport) against the
oracle on the same inputs: an empty photon list, ragged list lengths around
the warp width, and photons that take the rare branches of a segment --
born below the E/E0 cutoff, with no flight left, starting on the face they
move toward, with (nearly) equal distances to two faces (the first face
wins, cell.h:117-132), and with direction cosines outside float's range
(the single-precision face order falls back to three exact divisions).
An exactly zero direction cosine is left out: upstream then picks the face
behind at distance -inf (x/0 with the lower face chosen for a non-positive
cosine), and sampling never produces one (mu = 2u - 1 with u = odd/2^53,
cos and sin of 2 pi u rounded)."""
import numpy as np
import pytest

from parity import CELL_RTOL, close, compare_photons

pytestmark = pytest.mark.gpu


def _setup():
    import oracle as O
    from branson_gb300 import deck as D
    from branson_gb300.engine import ReplicatedIMC
    dk = D.hot_zone(n_per_axis=10, photons=20000, n_steps=2)
    orc = O.Oracle(dk)
    _, photons = orc.source(1)
    gpu = ReplicatedIMC(dk)
    for f in ("op_a", "op_s", "f"):
        gpu.set_field(f, orc.arr[f])
    return dk, orc, gpu, photons, orc.next_dt()


def _run_both(orc, gpu, photons, nd, ext, what):
    import oracle as O
    from branson_gb300.engine import arrays_to_records, records_to_arrays
    ph = records_to_arrays(photons)
    abs_g, trk_g, census_g, ce_g, ex_g = gpu.replicated_transport(ph, nd)
    end_g = arrays_to_records(ph, O.PHOTON_DTYPE)
    mine = photons.copy()
    abs_o, trk_o, census_o, ce_o, ex_o, _, _ = orc.transport(mine, nd)
    compare_photons(end_g, mine, ext, f"{what} end states")
    compare_photons(arrays_to_records(census_g, O.PHOTON_DTYPE), census_o, ext, f"{what} census")
    close(abs_g, abs_o, CELL_RTOL, 0.0, f"{what} abs_E")
    close(trk_g, trk_o, CELL_RTOL, 0.0, f"{what} track_E")
    close([ce_g, ex_g], [ce_o, ex_o], CELL_RTOL, 1e-300, f"{what} census/exit E")
    return end_g


def test_empty_and_ragged_lists(gpu_lib):
    from branson_gb300._lib import PhotonArrays
    dk, orc, gpu, photons, nd = _setup()
    ext = 1.0 + 299.792458 * dk.dt_start
    try:
        abs_g, trk_g, census_g, ce_g, ex_g = gpu.replicated_transport(PhotonArrays(0), nd)
        assert census_g.n == 0 and ce_g == 0.0 and ex_g == 0.0
        assert not np.any(abs_g) and not np.any(trk_g)
        for n in (1, 31, 32, 33, 1031):
            _run_both(orc, gpu, photons[:n], nd, ext, f"{n} photons")
    finally:
        gpu.close()


def test_rare_segment_branches(gpu_lib):
    dk, orc, gpu, photons, nd = _setup()
    ext = 1.0 + 299.792458 * dk.dt_start
    x, y, z = dk.planes()
    p = photons[:64].copy()
    nx, ny = len(x) - 1, len(y) - 1

    def node(i):
        c = int(p["cell"][i])
        a, b, k = c % nx, (c // nx) % ny, c // (nx * ny)
        return (x[a], x[a + 1]), (y[b], y[b + 1]), (z[k], z[k + 1])

    p["E"][0] = 0.005 * p["E0"][0]            # below the cutoff from the start
    p["life_dx"][1] = 0.0                      # no flight left: census at once
    p["dir"][2] = (1e-12, 0.6, 0.8)            # a tiny cosine: a far x face
    p["dir"][3] = (-0.8, 1e-200, -0.6)         # a cosine below float's range
    (x0, _), _, _ = node(4)
    p["pos"][4][0] = x0                        # on the face it moves toward
    p["dir"][4] = (-0.6, 0.64, 0.48)
    (_, x1), (_, y1), _ = node(5)
    d = 0.25 * min(x1 - x[0], y1 - y[0]) / len(x)
    p["pos"][5][0], p["pos"][5][1] = x1 - d, y1 - d  # equal distances to the x+ and y+ faces
    p["dir"][5] = (0.7, 0.7, np.sqrt(1.0 - 0.98))
    p["dir"][6] = (1e-300, -0.6, 0.8)          # another, and a negative one
    try:
        end = _run_both(orc, gpu, p, nd, ext, "rare branches")
        assert end["descriptor"][0] == 4       # KILLED by the cutoff
        assert end["descriptor"][1] == 2       # CENSUS
    finally:
        gpu.close()


@pytest.mark.parametrize("n", [1, 7, 9, 1031, 20928])
def test_pipelined_dropin_equals_whole_bank(gpu_lib, n):
    """The drop-in's pipelined form (copies overlapped with chunked
    transport, used for large history-mode banks) returns what the one-launch
    form returns, bit for bit: end states, census, tallies, energies (the
    threshold is lowered so small lists, including ones that leave some of
    the eight chunks empty, take the pipelined path)."""
    import oracle as O
    from branson_gb300.engine import arrays_to_records, records_to_arrays
    dk, orc, gpu, photons, nd = _setup()
    try:
        outs = []
        for min_n in (0, 1):  # 0: never pipelined; 1: always
            gpu.set_option("pipeline_min_photons", min_n)
            ph = records_to_arrays(photons[:n])
            abs_g, trk_g, census_g, ce_g, ex_g = gpu.replicated_transport(ph, nd)
            outs.append((arrays_to_records(ph, O.PHOTON_DTYPE), abs_g, trk_g,
                         arrays_to_records(census_g, O.PHOTON_DTYPE), ce_g, ex_g))
        (e0, a0, t0, c0, ce0, ex0), (e1, a1, t1, c1, ce1, ex1) = outs
        for f in e0.dtype.names:
            np.testing.assert_array_equal(e1[f], e0[f], err_msg=f"end {f}")
            np.testing.assert_array_equal(c1[f], c0[f], err_msg=f"census {f}")
        np.testing.assert_array_equal(a1, a0)
        np.testing.assert_array_equal(t1, t0)
        assert (ce1, ex1) == (ce0, ex0)
    finally:
        gpu.close()


@pytest.mark.parametrize("n", [1, 33, 20928])
def test_mapped_host_dropin_equals_copied(gpu_lib, n):
    """With every photon array in page-locked, device-mapped host memory, the
    drop-in transports the photons in place there (the kernels read and
    write the caller's arrays; no bulk copies).  Its end states, census,
    tallies and energies equal those of the copying forms bit for bit
    (one launch on the device bank, and the pipelined form), and the
    oracle's within the parity tolerances."""
    import oracle as O
    from branson_gb300.engine import arrays_to_records, records_to_arrays
    dk, orc, gpu, photons, nd = _setup()
    try:
        outs = []
        for zero_copy, min_n in ((1, 0), (0, 0), (0, 1)):
            gpu.set_option("zero_copy", zero_copy)
            gpu.set_option("pipeline_min_photons", min_n)
            ph = records_to_arrays(photons[:n], pinned=True)
            abs_g, trk_g, census_g, ce_g, ex_g = gpu.replicated_transport(ph, nd)
            outs.append((arrays_to_records(ph, O.PHOTON_DTYPE), abs_g.copy(), trk_g.copy(),
                         arrays_to_records(census_g, O.PHOTON_DTYPE), ce_g, ex_g))
        e0, a0, t0, c0, ce0, ex0 = outs[0]
        for e1, a1, t1, c1, ce1, ex1 in outs[1:]:
            for f in e0.dtype.names:
                np.testing.assert_array_equal(e1[f], e0[f], err_msg=f"end {f}")
                np.testing.assert_array_equal(c1[f], c0[f], err_msg=f"census {f}")
            np.testing.assert_array_equal(a1, a0)
            np.testing.assert_array_equal(t1, t0)
            assert (ce1, ex1) == (ce0, ex0)
        mine = photons[:n].copy()
        abs_o, trk_o, census_o, ce_o, ex_o, _, _ = orc.transport(mine, nd)
        ext = max(1.0, 299.792458 * dk.dt_start)
        compare_photons(e0, mine, ext, "mapped end states")
        compare_photons(c0, census_o, ext, "mapped census")
        close(a0, abs_o, CELL_RTOL, 0.0, "mapped abs_E")
        close(t0, trk_o, CELL_RTOL, 0.0, "mapped track_E")
    finally:
        gpu.close()
