"""Headless field output (the SILO replacement): round trip of the binary
layout, the deck keys that switch it on, and (GPU) the driver loop writing
one file per output step."""
import numpy as np
import pytest

from branson_gb300 import deck as D
from branson_gb300 import fields as F


def test_write_read_round_trip(tmp_path):
    shape = (4, 3, 2)
    n = 24
    rng = np.random.default_rng(0)
    f = {"T_e": rng.random(n), "T_r": rng.random(n), "abs_E": rng.random(n), "region": np.arange(n, dtype=float)}
    p = F.write_fields(str(tmp_path / "output_7.bgsf"), shape, 7, 0.07, f, transport_s=1.5)
    back = F.read_fields(p)
    assert back["shape"] == shape and back["step"] == 7 and back["time"] == 0.07 and back["transport_s"] == 1.5
    for k, v in f.items():
        np.testing.assert_array_equal(back["fields"][k], v)


def test_bad_inputs_raise(tmp_path):
    with pytest.raises(ValueError):
        F.write_fields(str(tmp_path / "x.bgsf"), (2, 2, 1), 1, 0.0, {"T_e": np.zeros(3)})
    (tmp_path / "junk.bgsf").write_bytes(b"not a field file")
    with pytest.raises(ValueError):
        F.read_fields(str(tmp_path / "junk.bgsf"))


def test_deck_output_keys_round_trip():
    dk = D.marshak_wave(n_cells=10, photons=100, n_steps=2)
    dk.write_silo, dk.output_frequency = True, 3
    back = D.parse_xml(dk.to_xml())
    assert back.write_silo and back.output_frequency == 3


@pytest.mark.gpu
def test_driver_writes_every_output_step(gpu_lib, tmp_path):
    from branson_gb300.engine import ReplicatedIMC
    dk = D.marshak_wave(n_cells=20, photons=2000, n_steps=4)
    dk.write_silo, dk.output_frequency = True, 2
    with ReplicatedIMC(dk) as imc:
        reps = F.run(imc, str(tmp_path))
        assert len(reps) == 4
        files = sorted(p.name for p in tmp_path.iterdir())
        assert files == ["output_2.bgsf", "output_4.bgsf"]
        last = F.read_fields(str(tmp_path / "output_4.bgsf"))
        np.testing.assert_array_equal(last["fields"]["T_e"], imc.get_field("T_e"))
