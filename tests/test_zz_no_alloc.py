"""bgs_transport_device_noalloc: the transport entry point that allocates
nothing, for callers that own all device memory (pool allocators) or must
not trigger a device allocation between launches.  Its scratch lives in a
static device array of the library; the caller passes device inputs and
outputs.  Checked through the C ABI against the existing entry point
(bgs_replicated_transport) on the same photons, on two calls in a row.

Collected last (test_zz_*) so that a run stopping at the first failure has
run everything else first; it also passes alone in a fresh process.
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
            # advance the oracle to the next step with the same tallies
            abs_o, trk_o, census_o, _, _, _, _ = orc.transport(photons, nd)
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
    rc = gpu_lib.bgs_transport_device_noalloc(64, 64, 64, 1, dummy, dummy, dummy, bc, dummy, dummy, dummy,
                                              777, 0, C.byref(ph), 0.01, dummy, dummy, None)
    assert rc == ERR_CAPACITY
