"""Deck model: XML round trip, the upstream parser's rules and error exits,
and the structured-mesh planes (proto_mesh.h:106-218)."""
import os

import numpy as np
import pytest

from branson_gb300 import deck as D

REF = os.environ.get("BRANSON_REFERENCE", "/root/reference")


def test_roundtrip_all_generators():
    for dk in (D.marshak_wave(), D.hot_zone(n_per_axis=10), D.hohlraum(n_per_axis=10),
               D.random_opacity_cube(n_per_axis=4), D.batch_ensemble(n_problems=3)[0]):
        again = D.parse_xml(dk.to_xml(), n_groups=dk.n_groups)
        assert again.shape == dk.shape
        assert again.bc == dk.bc and again.T_source == dk.T_source
        assert [r.opacA for r in again.regions] == [r.opacA for r in dk.regions]
        for a, b in zip(again.planes(), dk.planes()):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(again.cell_regions(), dk.cell_regions())


def test_planes_follow_proto_mesh():
    dk = D.hot_zone(n_per_axis=50)
    x, _, _ = dk.planes()
    assert len(x) == 51
    assert x[20] == 0.4 and x[30] == 0.6          # division ends set exactly
    assert x[1] == 0.0 + 1 * ((0.4 - 0.0) / 20)    # start + i*dx
    assert x[50] == 0.6 + 20 * ((1.0 - 0.6) / 20)  # last plane: start + n*dx


def test_hot_zone_regions():
    dk = D.hot_zone(n_per_axis=5)
    reg = dk.cell_regions().reshape(5, 5, 5)  # (k, j, i)
    hot = [i for i, r in enumerate(dk.regions) if r.T_e == 1.0][0]
    assert reg[2, 2, 2] == hot and (reg == hot).sum() == 1


def test_parser_errors():
    good = D.marshak_wave().to_xml()
    with pytest.raises(D.DeckError):
        D.parse_xml(good.replace("<bc_left>SOURCE</bc_left>", "<bc_left>BOGUS</bc_left>"))
    with pytest.raises(D.DeckError):
        D.parse_xml(good.replace("<regions>", "<nothing>").replace("</regions>", "</nothing>"))
    with pytest.raises(D.DeckError):
        D.parse_xml("<prototype><common>")
    bad_map = good.replace("<region_ID>1</region_ID>", "<region_ID>7</region_ID>")
    with pytest.raises(D.DeckError):
        D.parse_xml(bad_map)


def test_history_forces_large_batch():
    dk = D.parse_xml(D.marshak_wave().to_xml())
    assert dk.batch_size == 100000000  # input.h:488-490


@pytest.mark.skipif(not os.path.isdir(REF), reason="upstream checkout not present")
def test_parses_upstream_decks():
    for rel in ("inputs/marshak_wave_replicated.xml", "inputs/hot_zone_input.xml",
                "src/test/simple_input.xml", "src/test/three_region_mesh_input.xml"):
        dk = D.load(os.path.join(REF, rel))
        assert dk.n_cells > 0 and len(dk.regions) >= 1
