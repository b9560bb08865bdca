"""The workloads of the tests: sprout_gb300.workloads' tank descriptions, built for the engine
(Tank.engine) and for the CPU oracle (oracle_of)."""
from sprout_gb300.workloads import *  # noqa: F401,F403
from sprout_gb300.workloads import Tank


def oracle_of(tank: Tank):
    from oracle import oracle as O
    return O.build_tank(tank)
