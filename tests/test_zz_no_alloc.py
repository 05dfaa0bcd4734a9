"""bgs_transport_device_noalloc: the transport entry point that allocates
nothing, for callers that own all device memory (pool allocators) or must
not trigger a device allocation between launches.  Its scratch lives in a
static device array of the library; the caller passes device inputs and
outputs.  Checked through the C ABI against the existing entry point
(bgs_replicated_transport) on the same photons, on two calls in a row.

Collected last (test_zz_*) so that a run stopping at the first failure has
run everything else first; it also passes alone in a fresh process.

The results are also checked against the oracle directly, on a mesh of
exactly the 131072 cells the static scratch holds followed by a smaller
mesh (so each call's clearing of its own cells is all the next one needs),
and a mesh one cell beyond the limit is rejected.
"""
import ctypes as C

import numpy as np
import pytest

from parity import CELL_RTOL, close, compare_photons

pytestmark = pytest.mark.gpu

C_LIGHT = 299.792458
FIELDS = ("pos_x", "pos_y", "pos_z", "dir_x", "dir_y", "dir_z", "E", "E0", "life_dx", "cell", "group",
          "descriptor", "source_type", "rng_stream", "rng_counter")


def _to_device(ph):
    """Host SoA photon arrays -> torch device tensors holding the same bits."""
    import torch
    dev = {}
    for name in FIELDS:
        a = ph[name]
        if a.dtype == np.uint32:
            a = a.view(np.int32)
        elif a.dtype == np.uint64:
            a = a.view(np.int64)
        dev[name] = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return dev


def _from_device(dev, like):
    from branson_gb300._lib import PhotonArrays
    out = PhotonArrays(like.n)
    for name in FIELDS:
        host = dev[name].cpu().numpy()
        out[name][:] = host.view(out[name].dtype)
    return out


def _struct(dev):
    from branson_gb300._lib import PhotonsHost
    return PhotonsHost(*[C.c_void_p(dev[name].data_ptr()) for name in FIELDS])


def _noalloc(gpu_lib, dk, photons, cells, nd):
    """One call of bgs_transport_device_noalloc on device copies of the
    oracle-made photon list; returns (end records, abs_E, track_E)."""
    import torch
    import oracle as O
    from branson_gb300._lib import OK
    from branson_gb300.engine import arrays_to_records, records_to_arrays
    nx, ny, nz = dk.shape
    x, y, z = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in dk.planes())
    bc = (C.c_int32 * 6)(*dk.bc)
    ph_in = records_to_arrays(photons)
    dev = _to_device(ph_in)
    op_a, op_s, f = (torch.from_numpy(np.ascontiguousarray(cells[k])).cuda() for k in ("op_a", "op_s", "f"))
    abs_d = torch.full((dk.n_cells,), -1.0, dtype=torch.float64, device="cuda")
    trk_d = torch.full((dk.n_cells,), -1.0, dtype=torch.float64, device="cuda")
    s = _struct(dev)
    torch.cuda.synchronize()
    rc = gpu_lib.bgs_transport_device_noalloc(
        nx, ny, nz, dk.n_groups, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
        bc, C.c_void_p(op_a.data_ptr()), C.c_void_p(op_s.data_ptr()), C.c_void_p(f.data_ptr()), dk.seed,
        len(photons), C.byref(s), nd, C.c_void_p(abs_d.data_ptr()), C.c_void_p(trk_d.data_ptr()), None)
    assert rc == OK, rc
    end = arrays_to_records(_from_device(dev, ph_in), O.PHOTON_DTYPE)
    return end, abs_d.cpu().numpy(), trk_d.cpu().numpy()


def _cap_deck():
    """64 x 64 x 32 = 131072 cells, the no-allocation scratch's limit: a
    warm block in a cold, opaque surround with a source face, so photons
    cross many cells."""
    from branson_gb300.deck import Deck, Division, Region, SOURCE, VACUUM
    return Deck(t_start=0.0, t_stop=0.02, dt_start=0.01, t_mult=1.0, dt_max=1.0, photons=30000, seed=31,
                x_divisions=[Division(0.0, 0.4, 24), Division(0.4, 0.6, 16), Division(0.6, 1.0, 24)],
                y_divisions=[Division(0.0, 1.0, 64)], z_divisions=[Division(0.0, 0.5, 32)],
                region_map={(0, 0, 0): 1, (1, 0, 0): 2, (2, 0, 0): 1},
                bc=(SOURCE, VACUUM, VACUUM, VACUUM, VACUUM, VACUUM), T_source=0.5,
                regions=[Region(1, 0.1, 1.0, 0.0, 2.0, -3.0, 0.0, 0.1, 0.1),
                         Region(2, 0.1, 1.0, 0.0, 2.0, -3.0, 0.0, 0.6, 0.6)])


def test_noalloc_at_the_cell_limit_then_a_smaller_mesh(gpu_lib):
    import oracle as O
    from branson_gb300 import deck as D
    big = _cap_deck()
    assert big.n_cells == 131072
    for dk in (big, D.hot_zone(n_per_axis=10, photons=20000, n_steps=2)):
        orc = O.Oracle(dk, n_threads=4)
        _, photons = orc.source(1)
        nd = orc.next_dt()
        cells = {k: orc.arr[k].copy() for k in ("op_a", "op_s", "f")}
        end, abs_d, trk_d = _noalloc(gpu_lib, dk, photons, cells, nd)
        abs_o, trk_o, _, _, _, _, _ = orc.transport(photons, nd)
        ext = max(1.0, C_LIGHT * dk.dt_start)
        compare_photons(end, photons, ext, f"{dk.n_cells} cells: end states")
        close(abs_d, abs_o, CELL_RTOL, 0.0, f"{dk.n_cells} cells: abs_E vs the oracle")
        close(trk_d, trk_o, CELL_RTOL, 0.0, f"{dk.n_cells} cells: track_E vs the oracle")


def test_noalloc_transport_matches_existing_entry_point(gpu_lib):
    import torch
    import oracle as O
    from branson_gb300 import deck as D
    from branson_gb300._lib import OK
    from branson_gb300.engine import ReplicatedIMC, arrays_to_records, records_to_arrays

    dk = D.hot_zone(n_per_axis=10, photons=20000, n_steps=2)
    nx, ny, nz = dk.shape
    x, y, z = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in dk.planes())
    bc = (C.c_int32 * 6)(*dk.bc)
    orc = O.Oracle(dk)
    gpu = ReplicatedIMC(dk)
    ext = max(1.0, C_LIGHT * dk.dt_start)
    try:
        for call in range(2):  # two calls in a row share the static scratch
            step = orc.step_no
            _, photons = orc.source(step)
            nd = orc.next_dt()
            for fname in ("op_a", "op_s", "f"):
                gpu.set_field(fname, orc.arr[fname])
            # the existing entry point on host buffers
            ph_ref = records_to_arrays(photons)
            abs_ref, trk_ref, _, _, _ = gpu.replicated_transport(ph_ref, nd)
            # the allocation-free entry point on device buffers
            ph_in = records_to_arrays(photons)
            dev = _to_device(ph_in)
            op_a = torch.from_numpy(orc.arr["op_a"].copy()).cuda()
            op_s = torch.from_numpy(orc.arr["op_s"].copy()).cuda()
            f = torch.from_numpy(orc.arr["f"].copy()).cuda()
            abs_d = torch.full((dk.n_cells,), -1.0, dtype=torch.float64, device="cuda")
            trk_d = torch.full((dk.n_cells,), -1.0, dtype=torch.float64, device="cuda")
            s = _struct(dev)
            torch.cuda.synchronize()
            rc = gpu_lib.bgs_transport_device_noalloc(
                nx, ny, nz, dk.n_groups, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                C.c_void_p(z.data_ptr()), bc, C.c_void_p(op_a.data_ptr()), C.c_void_p(op_s.data_ptr()),
                C.c_void_p(f.data_ptr()), dk.seed, len(photons), C.byref(s), nd,
                C.c_void_p(abs_d.data_ptr()), C.c_void_p(trk_d.data_ptr()), None)
            assert rc == OK, rc
            got = arrays_to_records(_from_device(dev, ph_in), O.PHOTON_DTYPE)
            ref = arrays_to_records(ph_ref, O.PHOTON_DTYPE)
            compare_photons(got, ref, ext, f"call {call} end states")
            close(abs_d.cpu().numpy(), abs_ref, CELL_RTOL, 0.0, f"call {call} abs_E")
            close(trk_d.cpu().numpy(), trk_ref, CELL_RTOL, 0.0, f"call {call} track_E")
            # and against the oracle's transport of the same photons
            abs_o, trk_o, census_o, _, _, _, _ = orc.transport(photons, nd)
            compare_photons(got, photons, ext, f"call {call} end states vs the oracle")
            close(abs_d.cpu().numpy(), abs_o, CELL_RTOL, 0.0, f"call {call} abs_E vs the oracle")
            close(trk_d.cpu().numpy(), trk_o, CELL_RTOL, 0.0, f"call {call} track_E vs the oracle")
            # advance the oracle to the next step with the same tallies
            ta, pm = C.c_double(), C.c_double()
            O.lib().bo_update_temperature(C.byref(orc.mesh), C.byref(orc.cells), orc.dt, O._dptr(abs_o),
                                          O._dptr(trk_o), C.byref(ta), C.byref(pm))
            orc.census = census_o
            orc.time += orc.dt
            orc.dt = nd
            orc.step_no += 1
    finally:
        gpu.close()


def test_noalloc_rejects_meshes_beyond_its_scratch(gpu_lib):
    from branson_gb300._lib import ERR_CAPACITY, PhotonsHost
    bc = (C.c_int32 * 6)(1, 1, 1, 1, 1, 1)
    dummy = C.c_void_p(1)
    ph = PhotonsHost(*([dummy] * len(FIELDS)))
    for shape in ((64, 64, 64), (131073, 1, 1)):  # beyond 131072 cells, by far and by one
        rc = gpu_lib.bgs_transport_device_noalloc(*shape, 1, dummy, dummy, dummy, bc, dummy, dummy, dummy,
                                                  777, 0, C.byref(ph), 0.01, dummy, dummy, None)
        assert rc == ERR_CAPACITY, shape
