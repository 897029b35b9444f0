"""The energy balance restated in the CPU oracle against the reference's energy balance tests
(plugins/energybalance/tests/selfTest.cpp); surface inputs come from the Python mirror."""
import pytest

import scenarios


@pytest.fixture(scope="module")
def run_eb(oracle_mod):
    def _run(model, dt):
        surf, R, To, uu = model.surface_arrays()
        surf["dt"] = dt
        T, out, _ = oracle_mod.energy_balance(surf, R, To)
        model.write_outputs(uu, T, out, surf)
    return _run


@pytest.mark.parametrize("name", scenarios.ENERGY)
def test_energy_balance_known_answers(run_eb, name):
    res = getattr(scenarios, name)(run_eb)
    absn = [r[0] for r in res if r[2] == 0.0]
    assert not scenarios.check(res, abs_tol_names=absn), scenarios.check(res, abs_tol_names=absn)
