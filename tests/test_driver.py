"""The caller's time loop (main.cc:1504-1575) on CPU, with a stand-in operator:
the step-size policy (Courant number over the transport speed, re-estimated at
every fifth step from the speed truncated to 3 digits) and the step sequence."""
import math

import numpy as np
import pytest

from oceano_gb300.driver import TimeLoop, truncate_to_n_digits


@pytest.mark.parametrize("x,n,want", [(1.23456, 3, 1.23), (0.0098765, 3, 0.00987),
                                      (-123.45, 3, -123.0), (9.999, 3, 9.99), (7.0, 3, 7.0),
                                      (123456.0, 2, 120000.0), (0.0, 3, 0.0)])
def test_truncate_to_n_digits(x, n, want):
    """Towards zero, n significant digits (deal.II Utilities::truncate_to_n_digits)."""
    assert math.isclose(truncate_to_n_digits(x, n), want, rel_tol=1e-15, abs_tol=0.0)


class FakeOperator:
    """Transport speed that grows with every query; records the steps it takes."""

    def __init__(self):
        self.queries = 0
        self.steps = []

    def compute_cell_transport_speed(self, z, q):
        self.queries += 1
        return 1.23456789 * (1.0 + 0.1 * self.queries)

    def perform_time_step(self, scheme, t, dt, z, q):
        self.steps.append((scheme, t, dt))
        z += dt

    def evaluate_velocity_field(self, z, q, v):
        v[:] = z


def test_step_size_policy_and_sequence():
    op = FakeOperator()
    loop = TimeLoop(op, "ssp33", 0.2)
    z, q, v = np.zeros(4), np.zeros(8), np.zeros(4)
    dts = [loop.advance(z, q, v) for _ in range(12)]
    s0 = 1.23456789 * 1.1  # the first query, not truncated (main.cc:1504-1506)
    assert dts[0] == pytest.approx(0.2 / s0, rel=1e-15)
    assert dts[:4] == [dts[0]] * 4
    # steps 5 and 10 (1-based) re-estimate from the truncated speed, the others keep it
    s5 = truncate_to_n_digits(1.23456789 * 1.2, 3)
    s10 = truncate_to_n_digits(1.23456789 * 1.3, 3)
    assert dts[4] == 0.2 / s5 and dts[5:9] == [dts[4]] * 4
    assert dts[9] == 0.2 / s10 and dts[10:] == [dts[9]] * 2
    assert op.queries == 3
    times = [t for _, t, _ in op.steps]
    assert times == pytest.approx(np.concatenate([[0.0], np.cumsum(dts)[:-1]]), rel=1e-15)
    assert loop.time == pytest.approx(sum(dts), rel=1e-15) and loop.step_number == 12
    assert np.array_equal(v, z) and all(s == "ssp33" for s, _, _ in op.steps)


@pytest.mark.parametrize("speed", [0.0, float("nan")])
def test_non_finite_step_size_stops_the_loop(speed):
    """A still or blown-up state gives no finite step: the loop stops before it."""
    class Bad(FakeOperator):
        def compute_cell_transport_speed(self, z, q):
            return speed

    op = Bad()
    loop = TimeLoop(op, "ssp33", 0.2)
    with pytest.raises(FloatingPointError):
        loop.advance(np.zeros(4), np.zeros(8))
    assert op.steps == []
