"""GPU path vs the oracle (the C restatement pinned to the upstream code).

Two forms, both through the C ABI:
  * drop-in: the oracle makes a step's photon list; bgs_replicated_transport
    transports exactly those photons on host buffers; end states, census
    (order and values), tallies and post-process sums are compared;
  * device-resident staged step: energies, photon counts and the sourced
    photons (matched by RNG stream), tallies and the temperature update.
"""
import numpy as np
import pytest

from parity import CELL_RTOL, END_RTOL, bitwise_fraction, by_stream, close, compare_photons

pytestmark = pytest.mark.gpu

C_LIGHT = 299.792458


def _uniform_deck():
    """Eight identical cells, emission only (T_r = 0, no source face), 8000
    photons: each cell's count n*E/total sits on the integer 1000, inside the
    error window of the tree-summed total, so the step takes the upstream
    serial sum and recounts (source.h:225-245, mesh.h:282-287)."""
    from branson_gb300.deck import Deck, Division, Region, VACUUM
    return Deck(t_start=0.0, t_stop=0.03, dt_start=0.01, t_mult=1.0, dt_max=1.0, photons=8000, seed=11,
                x_divisions=[Division(0.0, 1.0, 2)], y_divisions=[Division(0.0, 1.0, 2)],
                z_divisions=[Division(0.0, 1.0, 2)], region_map={(0, 0, 0): 1}, bc=(VACUUM,) * 6, T_source=0.0,
                regions=[Region(1, 0.1, 1.0, 10.0, 0.0, 0.0, 0.0, 0.5, 0.0)])


def _offset_scatter_deck():
    """Collision-dominated cells on an offset mesh whose z planes straddle 0
    (x in [-7.5, -7.3], y in [2, 2.12], z in [-0.05, 0.05]), physical and
    effective scattering, reflecting and vacuum faces, two groups: long
    runs of collisions inside a cell, ending near its faces, on planes of
    both signs and magnitudes from 0 to 7.5."""
    from branson_gb300.deck import Deck, Division, Region, REFLECT, VACUUM
    return Deck(t_start=0.0, t_stop=0.03, dt_start=0.01, t_mult=1.0, dt_max=1.0, photons=20000, seed=5,
                x_divisions=[Division(-7.5, -7.3, 6)], y_divisions=[Division(2.0, 2.12, 4)],
                z_divisions=[Division(-0.05, 0.05, 5)], region_map={(0, 0, 0): 1},
                bc=(REFLECT, VACUUM, REFLECT, VACUUM, REFLECT, VACUUM), T_source=0.0, n_groups=2,
                regions=[Region(1, 0.1, 1.0, 300.0, 0.0, 0.0, 500.0, 0.3, 0.3)])


def _column_deck():
    """One cell across x (so the cell coordinates divide by ngx = 1), 5 x 7
    cells in y and z, reflecting x faces, a 0.5 keV source on z-."""
    from branson_gb300.deck import Deck, Division, Region, REFLECT, SOURCE, VACUUM
    return Deck(t_start=0.0, t_stop=0.02, dt_start=0.01, t_mult=1.0, dt_max=1.0, photons=20000, seed=9,
                x_divisions=[Division(0.0, 0.3, 1)], y_divisions=[Division(0.0, 0.5, 5)],
                z_divisions=[Division(0.0, 0.7, 7)], region_map={(0, 0, 0): 1},
                bc=(REFLECT, REFLECT, VACUUM, VACUUM, SOURCE, VACUUM), T_source=0.5,
                regions=[Region(1, 0.1, 1.0, 20.0, 0.0, 0.0, 2.0, 0.1, 0.1)])


def _decks():
    from branson_gb300 import deck as D
    return {
        "marshak": D.marshak_wave(n_cells=100, photons=20000, n_steps=3),
        "hot_zone": D.hot_zone(n_per_axis=10, photons=20000, n_steps=3),
        "hohlraum30": D.hohlraum(n_per_axis=10, photons=20000, n_steps=2, n_groups=30),
        "uniform8": _uniform_deck(),
        "offset_scatter": _offset_scatter_deck(),
        "column": _column_deck(),
    }


def _extent(dk):
    x, y, z = dk.planes()
    return max(x[-1] - x[0], y[-1] - y[0], z[-1] - z[0], C_LIGHT * dk.dt_start)


@pytest.mark.parametrize("name", ["marshak", "hot_zone", "hohlraum30", "offset_scatter", "column"])
def test_dropin_transport_matches_oracle(gpu_lib, name):
    import oracle as O
    from branson_gb300.engine import ReplicatedIMC, arrays_to_records, records_to_arrays

    dk = _decks()[name]
    orc = O.Oracle(dk)
    gpu = ReplicatedIMC(dk)
    ext = _extent(dk)
    try:
        for _ in range(2):
            step = orc.step_no
            en, photons = orc.source(step)
            nd = orc.next_dt()
            for f in ("op_a", "op_s", "f"):
                gpu.set_field(f, orc.arr[f])
            ph = records_to_arrays(photons)
            abs_g, trk_g, census_g, ce_g, ex_g = gpu.replicated_transport(ph, nd)
            end_g = arrays_to_records(ph, O.PHOTON_DTYPE)
            abs_o, trk_o, census_o, ce_o, ex_o, segs, _ = orc.transport(photons, nd)
            compare_photons(end_g, photons, ext, f"{name} step {step} end states")
            print(f"{name} step {step}: {len(photons)} histories, "
                  f"{100 * bitwise_fraction(end_g, photons):.2f}% bit-identical end states")
            compare_photons(arrays_to_records(census_g, O.PHOTON_DTYPE), census_o, ext,
                            f"{name} step {step} census")
            close(abs_g, abs_o, CELL_RTOL, 0.0, f"{name} abs_E")
            close(trk_g, trk_o, CELL_RTOL, 0.0, f"{name} track_E")
            close([ce_g, ex_g], [ce_o, ex_o], CELL_RTOL, 1e-300, f"{name} census/exit E")
            # advance the oracle exactly as its driver does
            import ctypes as C
            ta, pm = C.c_double(), C.c_double()
            O.lib().bo_update_temperature(C.byref(orc.mesh), C.byref(orc.cells), orc.dt,
                                          O._dptr(abs_o), O._dptr(trk_o), C.byref(ta), C.byref(pm))
            orc.census = census_o
            orc.time += orc.dt
            orc.dt = nd
            orc.step_no += 1
    finally:
        gpu.close()


@pytest.mark.parametrize("name", ["marshak", "hot_zone", "hohlraum30", "uniform8", "offset_scatter", "column"])
def test_device_step_matches_oracle(gpu_lib, name):
    import oracle as O
    from branson_gb300.engine import ReplicatedIMC, arrays_to_records

    dk = _decks()[name]
    orc = O.Oracle(dk)
    gpu = ReplicatedIMC(dk)
    ext = _extent(dk)
    try:
        for _ in range(2):
            step = orc.step_no
            # keep the material state identical so each step is compared on its own
            gpu.set_field("T_e", orc.arr["T_e"])
            census_in = gpu.bank_size() if step > 1 else 0
            e = gpu.calculate_photon_energy(step, gpu.dt)
            res = orc.step()
            for fname, ref in (("op_a", res.op_a), ("f", res.f), ("emission_E", res.emission_cell_E),
                               ("census_E", res.census_cell_E), ("source_E", res.source_cell_E)):
                close(gpu.get_field(fname), ref, 1e-13, 0.0, f"{name} step {step} {fname}")
            close([e["total_photon_E"], e["pre_mat_E"]], [res.total_photon_E, res.pre_mat_E], 1e-13, 0.0,
                  "totals")
            is_new = res.source["stream"] >= 10000000000000 * step
            assert e["n_new_photons"] == int(is_new.sum())
            gpu.source(step, gpu.dt)
            bank = arrays_to_records(gpu.photons(), O.PHOTON_DTYPE)
            # photons made this step, matched to the oracle by RNG stream
            new_g = by_stream(bank[census_in:])
            new_o = by_stream(res.source[is_new]) if step > 1 else by_stream(res.source)
            compare_photons(new_g, new_o, ext, f"{name} step {step} source", check_desc=False)
            t = gpu.transport(res.next_dt)
            assert t["device_flags"] == 0
            assert t["n_transported"] == len(res.source)
            assert t["n_census"] == len(res.census)
            close(gpu.get_field("abs_E"), res.abs_E, CELL_RTOL, 0.0, f"{name} step {step} abs_E")
            close(gpu.get_field("track_E"), res.track_E, CELL_RTOL, 0.0, f"{name} step {step} track_E")
            close([t["census_E"], t["exit_E"]], [res.census_E, res.exit_E], CELL_RTOL, 1e-300, "census/exit")
            u = gpu.update_temperature(gpu.dt)
            close(gpu.get_field("T_e"), res.T_e, CELL_RTOL, 0.0, f"{name} step {step} T_e")
            close(gpu.get_field("T_r"), res.T_r, CELL_RTOL, 0.0, f"{name} step {step} T_r")
            close([u["absorbed_E"], u["post_mat_E"]], [res.absorbed_E, res.post_mat_E], CELL_RTOL, 0.0,
                  "absorbed/post_mat")
            census_g = by_stream(arrays_to_records(gpu.photons(), O.PHOTON_DTYPE))
            compare_photons(census_g, by_stream(res.census), ext, f"{name} step {step} census")
            gpu.advance_time(res.next_dt)
    finally:
        gpu.close()


@pytest.mark.parametrize("name", ["marshak_g1", "hot_zone_g1", "hohlraum_g30"])
def test_gpu_against_upstream_golden(gpu_lib, name):
    """The GPU drop-in transport on the upstream photon lists (golden vectors
    written by the upstream headers) reproduces the upstream end states,
    census and tallies; the device source reproduces the upstream photons."""
    import os
    import oracle as O
    from branson_gb300 import deck as D
    from branson_gb300.engine import ReplicatedIMC, arrays_to_records, records_to_arrays

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    dk = D.parse_xml(str(g["deck_xml"]), n_groups=int(g["n_groups"]))
    ext = _extent(dk)
    with ReplicatedIMC(dk) as gpu:
        T_e = None
        for s in range(1, int(g["n_steps"]) + 1):
            cells = g[f"s{s}_cells"]
            if T_e is not None:
                gpu.set_field("T_e", T_e)
            gpu.calculate_photon_energy(s, gpu.dt)
            close(gpu.get_field("op_a"), cells[:, 0], 1e-13, 0.0, f"{name} s{s} op_a")
            close(gpu.get_field("emission_E"), cells[:, 2], 1e-13, 0.0, f"{name} s{s} emission_E")
            src = g[f"s{s}_source"]
            if s == 1:
                gpu.source(1, gpu.dt)
                made = by_stream(arrays_to_records(gpu.photons(), O.PHOTON_DTYPE))
                compare_photons(made, by_stream(src), ext, f"{name} s1 sourced", check_desc=False)
            gpu.set_field("op_a", cells[:, 0])
            gpu.set_field("f", cells[:, 1])
            gpu.set_field("op_s", np.zeros(dk.n_cells))
            ph = records_to_arrays(src)
            nd = dk.dt_start
            abs_g, trk_g, census_g, _, _ = gpu.replicated_transport(ph, nd)
            compare_photons(arrays_to_records(ph, O.PHOTON_DTYPE), g[f"s{s}_end"], ext, f"{name} s{s} end")
            compare_photons(arrays_to_records(census_g, O.PHOTON_DTYPE), g[f"s{s}_census"], ext,
                            f"{name} s{s} census")
            close(abs_g, cells[:, 5], CELL_RTOL, 0.0, f"{name} s{s} abs_E")
            close(trk_g, cells[:, 6], CELL_RTOL, 0.0, f"{name} s{s} track_E")
            T_e = cells[:, 7]
            gpu.advance_time(nd)


@pytest.mark.parametrize("name", ["marshak", "hot_zone", "hohlraum30"])
def test_event_mode_reproduces_history_mode(gpu_lib, name):
    """Event-mode stages run the same per-photon arithmetic, so end states,
    census and tallies equal history mode bit for bit, whatever the split
    between event rounds and the history tail."""
    import oracle as O
    from branson_gb300 import _lib
    from branson_gb300.engine import ReplicatedIMC, arrays_to_records, records_to_arrays

    dk = _decks()[name]
    orc = O.Oracle(dk)
    _, photons = orc.source(1)
    nd = orc.next_dt()
    with ReplicatedIMC(dk) as gpu:
        for f in ("op_a", "op_s", "f"):
            gpu.set_field(f, orc.arr[f])
        ph_h = records_to_arrays(photons)
        abs_h, trk_h, cen_h, ce_h, ex_h = gpu.replicated_transport(ph_h, nd, _lib.HISTORY)
        for cap, tail in ((4, 0.0), (1000, 0.0), (8, 0.5)):
            gpu.set_option("event_round_cap", cap)
            gpu.set_option("event_tail_fraction", tail)
            gpu.set_option("event_check_every", 2)
            ph_e = records_to_arrays(photons)
            abs_e, trk_e, cen_e, ce_e, ex_e = gpu.replicated_transport(ph_e, nd, _lib.EVENT)
            for k in ph_h.arrays:
                np.testing.assert_array_equal(ph_e[k], ph_h[k], err_msg=f"{name} cap {cap} {k}")
            np.testing.assert_array_equal(abs_e, abs_h)
            np.testing.assert_array_equal(trk_e, trk_h)
            assert cen_e.n == cen_h.n and ce_e == ce_h and ex_e == ex_h
        # and the event-mode end states are the oracle's
        compare_photons(arrays_to_records(ph_e, O.PHOTON_DTYPE), _oracle_end(orc, photons, nd), _extent(dk),
                        f"{name} event vs oracle")


@pytest.mark.parametrize("name", ["hot_zone", "hohlraum30"])
def test_event_mode_step_counts_every_segment(gpu_lib, name):
    """A whole step in event mode (event rounds, then the history tail)
    reports the segment count and fields of the same step in history mode."""
    from branson_gb300 import _lib
    from branson_gb300.engine import ReplicatedIMC

    dk = _decks()[name]
    with ReplicatedIMC(dk) as h, ReplicatedIMC(dk) as e:
        e.set_option("event_round_cap", 4)
        e.set_option("event_tail_fraction", 0.0)
        rh, re_ = h.step(_lib.HISTORY), e.step(_lib.EVENT)
        assert rh.n_segments > rh.n_transported > 0
        assert (re_.n_transported, re_.n_census, re_.n_segments) == (rh.n_transported, rh.n_census, rh.n_segments)
        for f in ("T_e", "abs_E", "track_E"):
            np.testing.assert_array_equal(e.get_field(f), h.get_field(f))


def _oracle_end(orc, photons, nd):
    ph = photons.copy()
    orc.transport(ph, nd)
    return ph
