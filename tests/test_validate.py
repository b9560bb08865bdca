"""The oracle against the reference's physics known answers (src/validate.rs), with the
reference's own thresholds: the collapse of a water column against Martin & Moyce's
experiment (validate.rs:177-211), the shallow dam break against Ritter's solution (213-238),
and the analytic decay of viscous shear in a free slab and on a no-slip floor (1120-1199).
These pin the oracle's solver (the pressure projection, the implicit viscosity, the
particle transport) to behaviour the reference itself asserts, beyond the set-up code's
unit-test answers (test_oracle_golden.py). The scenarios that take minutes on the oracle
(the 10 s hydrostatic pool, the sealed tank, the rotating disc) run in
test_gpu_validate.py, where the engine is also compared with the oracle bit for bit.
"""
import pytest

import validate_scenarios as V


@pytest.mark.parametrize("name", ["dam_break", "ritter", "viscosity_free", "viscosity_floor"])
def test_oracle_meets_the_reference_known_answers(name):
    tank, run = V.SCENARIOS[name]()
    checks = run(V.Runner(tank, "oracle"))
    failed = [c for c in checks if not c[2]]
    assert not failed, f"{name}: {failed} (all: {checks})"
