"""The C++ drop-in replicated_transport<Census_T>
(include/branson_gb300_transport.hpp) run on the GPU through
tests/dropin/standin_driver.cc, with stand-ins for the upstream types
(tests/dropin/standin/branson_standin.h; the upstream checkout is not on the
GPU host).  Per deck: three steps of the oracle's photon lists, then a list
longer than the first call's device capacity (2n + 4096), in both AoS
(std::vector<Photon>) and SoA (PhotonArray).  Each call's end states
(written back into the caller's container), returned census (input order,
life_dx = c*next_dt), overwritten rank_abs_E / rank_track_E and IMC_State
values (exit_E, post_census_E, census_size, transport runtime) are compared
with the oracle's transport of the same list (replicated_transport.h:33-158,
post_process_functions.h:33-109)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from parity import CELL_RTOL, close, compare_photons

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
C_LIGHT = 299.792458


def _build_driver(out_dir, n_groups):
    from branson_gb300 import build
    lib = build.build()
    exe = os.path.join(out_dir, f"standin_driver_g{n_groups}")
    cmd = ["g++", "-std=c++17", "-O2", f"-DBRANSON_N_GROUPS={n_groups}",
           "-I", os.path.join(ROOT, "tests", "dropin", "standin"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "standin_driver.cc"), lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _advance(orc, abs_o, trk_o, census_o, nd):
    import oracle as O
    ta, pm = C.c_double(), C.c_double()
    orc.L.bo_update_temperature(C.byref(orc.mesh), C.byref(orc.cells), orc.dt, O._dptr(abs_o.copy()),
                                O._dptr(trk_o.copy()), C.byref(ta), C.byref(pm))
    orc.census = census_o
    orc.time += orc.dt
    orc.dt = nd
    orc.step_no += 1


def _prepare(dk, d, small, big):
    """Write the calls; return the oracle's expected results per call."""
    import copy
    import oracle as O
    x, y, z = dk.planes()
    with open(os.path.join(d, "mesh.bin"), "wb") as fh:
        fh.write(np.array(dk.shape, np.uint32).tobytes())
        fh.write(np.array(dk.bc, np.int32).tobytes())
        fh.write(np.array([dk.seed], np.uint32).tobytes())
        fh.write(np.concatenate([x, y, z]).astype(np.float64).tobytes())
    lists = []
    a = copy.deepcopy(dk)
    a.photons = small
    orc = O.Oracle(a)
    for _ in range(3):
        _, photons = orc.source(orc.step_no)
        nd = orc.next_dt()
        cells = np.concatenate([orc.arr["op_a"], orc.arr["op_s"], orc.arr["f"]])
        start = photons.copy()
        res = orc.transport(photons, nd)
        lists.append((start, cells, nd, photons, res))
        _advance(orc, res[0], res[1], res[2], nd)
    b = copy.deepcopy(dk)
    b.photons = big
    orc_b = O.Oracle(b)
    _, photons = orc_b.source(1)
    nd = orc_b.next_dt()
    cells = np.concatenate([orc_b.arr["op_a"], orc_b.arr["op_s"], orc_b.arr["f"]])
    start = photons.copy()
    lists.append((start, cells, nd, photons, orc_b.transport(photons, nd)))
    assert len(lists[-1][0]) > 2 * len(lists[0][0]) + 4096  # outgrows the first call's banks
    with open(os.path.join(d, "calls.txt"), "w") as fh:
        for k, (start, cells, nd, _, _) in enumerate(lists):
            fh.write(f"{len(start)} {nd!r}\n")
            start.tofile(os.path.join(d, f"call{k}_in.bin"))
            cells.astype(np.float64).tofile(os.path.join(d, f"call{k}_cells.bin"))
    return lists


@pytest.mark.parametrize("name", ["marshak", "hot_zone", "hohlraum30"])
def test_cpp_dropin_matches_oracle(gpu_lib, tmp_path, name):
    import oracle as O
    from branson_gb300 import deck as D
    dk = {"marshak": lambda: D.marshak_wave(n_cells=100, photons=4000, n_steps=5),
          "hot_zone": lambda: D.hot_zone(n_per_axis=10, photons=4000, n_steps=5),
          "hohlraum30": lambda: D.hohlraum(n_per_axis=10, photons=4000, n_steps=5, n_groups=30)}[name]()
    exe = _build_driver(str(tmp_path), dk.n_groups)
    calls = _prepare(dk, str(tmp_path), small=4000, big=60000)
    x, y, z = dk.planes()
    ext = max(x[-1] - x[0], y[-1] - y[0], z[-1] - z[0], C_LIGHT * dk.dt_start)
    n_cells = dk.n_cells
    for tag in ("aos", "soa"):
        r = subprocess.run([exe, str(tmp_path), tag], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        for k, (start, _, nd, end_o, (abs_o, trk_o, census_o, ce_o, ex_o, _, _)) in enumerate(calls):
            what = f"{name} {tag} call {k}"
            base = os.path.join(str(tmp_path), f"call{k}")
            end = np.fromfile(f"{base}_end_{tag}.bin", O.PHOTON_DTYPE)
            census = np.fromfile(f"{base}_census_{tag}.bin", O.PHOTON_DTYPE)
            tally = np.fromfile(f"{base}_tally_{tag}.bin", np.float64)
            assert len(end) == len(start)
            np.testing.assert_array_equal(end["stream"], start["stream"], err_msg=what)
            np.testing.assert_array_equal(end["source_type"], start["source_type"], err_msg=what)
            compare_photons(end, end_o, ext, f"{what} end states")
            assert np.all(census["descriptor"] == O.CENSUS)
            compare_photons(census, census_o, ext, f"{what} census")
            np.testing.assert_array_equal(census["life_dx"], np.full(len(census), C_LIGHT * nd))
            close(tally[:n_cells], abs_o, CELL_RTOL, 0.0, f"{what} rank_abs_E")
            close(tally[n_cells:], trk_o, CELL_RTOL, 0.0, f"{what} rank_track_E")
            with open(f"{base}_state_{tag}.txt") as fh:
                exit_E, post_E, n_census, runtime = fh.read().split()
            close([float(exit_E), float(post_E)], [ex_o, ce_o], CELL_RTOL, 1e-300, f"{what} IMC_State energies")
            assert int(n_census) == len(census_o), what
            assert float(runtime) > 0.0, what
