"""Parity at the benchmark decks' full sizes (tests/fullsize.py): the 50^3
hot zone at 1e7 photons per step after two warm-up steps, the 100-cell
Marshak wave at 1e6 photons over all 50 of its steps, and the 60^3 30-group
hohlraum's first step at 5e7 photons.  Every history is compared with the
oracle and with its GPU-math twin (bit for bit), branch flips are traced to
their near tie, and per-cell tallies and temperatures are compared within
1e-10 with the flipped histories taken out, with z-scores where they
deposited."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["marshak", "hot_zone", "hohlraum"])
def test_full_size_parity(gpu_lib, case):
    import fullsize as F
    rep = F.run_case(case, log=print)
    for r in rep["steps"]:
        F.check_step(r)
