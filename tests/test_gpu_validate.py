"""The engine on the reference's physics known answers (src/validate.rs, restated in
validate_scenarios.py): each scenario runs on the engine and on the oracle, both must meet
the reference's thresholds, and the engine's particles must equal the oracle's bit for bit
at the end (matched by id), after hundreds of adaptive substeps (the step length is picked
on the device from the CFL estimate, the host loop is FluidSim::advance_blocking's).
"""
import numpy as np
import pytest

import validate_scenarios as V

pytestmark = pytest.mark.gpu


def by_id(ps):
    return ps[np.argsort(ps["id"], kind="stable")]


@pytest.mark.parametrize("name", list(V.SCENARIOS))
def test_engine_meets_the_known_answers_as_the_oracle(name):
    tank, run = V.SCENARIOS[name]()
    eng = V.Runner(tank, "engine")
    ora = V.Runner(tank, "oracle")
    ce, co = run(eng), run(ora)
    failed = [c for c in ce if not c[2]]
    assert not failed, f"{name} on the engine: {failed} (all: {ce})"
    failed = [c for c in co if not c[2]]
    assert not failed, f"{name} on the oracle: {failed} (all: {co})"
    g, o = by_id(eng.particles()), by_id(ora.particles())
    assert len(g) == len(o) and np.array_equal(g.view(np.uint8), o.view(np.uint8)), f"{name}: particles differ"
    assert eng.stats()[:3] == ora.stats()[:3], f"{name}: solver statistics differ {eng.stats()} vs {ora.stats()}"
