"""stats.comp (FluidSim::request_stats / poll_stats): the census of the particle slots, live
particles and per material row its particles and their summed concentration in 1/256 of a
particle. Integer counts, so compared exactly with the same census taken of the oracle's
particles after the same substeps."""
import time

import numpy as np
import pytest

import tanks

pytestmark = pytest.mark.gpu


def census(parts):
    kind = parts["kind"] & 255
    live = kind != 0
    count = np.bincount(kind[live] - 1, minlength=96).astype(np.uint32)
    q = (np.clip(parts["s"][live], np.float32(0.0), np.float32(1.0)) * np.float32(256.0) + np.float32(0.5)).astype(np.uint32)
    conc = np.bincount(kind[live] - 1, weights=q, minlength=96)
    return int(live.sum()), count, (conc / 256.0).astype(np.float32)


def wait_stats(sim):
    for _ in range(2000):
        st = sim.poll_stats()
        if st is not None:
            return st
        time.sleep(0.001)
    raise AssertionError("the census never finished")


@pytest.mark.parametrize("tank", ["families", "currents"])
def test_census_matches_the_oracle(tank):
    t = tanks.families_tank() if tank == "families" else tanks.currents()
    sim, _, _ = t.engine()
    ora, _, _ = tanks.oracle_of(t)
    for _ in range(6):
        sim.step(1, 1 / 240.0)
        ora.step(1, 1 / 240.0)
    sim.request_stats()
    sim.request_stats()   # one in flight: the second request is no new one
    st = wait_stats(sim)
    assert sim.poll_stats() is None
    live, count, conc = census(ora.particles())
    assert st.live == live
    assert np.array_equal(np.array(st.count, np.uint32), count)
    assert np.array_equal(np.array(st.conc, np.float32), conc)
    if tank == "currents":
        assert live < len(t.engine()[1])   # the drain took some
