"""Time loop of oceano's driver around the GPU operator.

Restates the caller side of the hot path, ``OceanoProblem::run``
(oceano/source/main.cc:1504-1575): the initial step size is the Courant
number over the transport speed, re-estimated every 5 steps from the speed
truncated to 3 significant digits (deal.II ``Utilities::truncate_to_n_digits``),
then each step is one ``perform_time_step`` of the integrator followed by
``evaluate_velocity_field`` (main.cc:1559-1575).  AMR, output and p-adaptation
of the reference loop are not part of this path.
"""
from __future__ import annotations

import math

import numpy as np


def truncate_to_n_digits(x: float, n: int) -> float:
    """x truncated (towards zero) to n significant decimal digits."""
    if x == 0.0 or not math.isfinite(x):
        return x
    order = math.floor(math.log10(abs(x)))
    factor = 10.0 ** (n - order - 1)
    return math.trunc(x * factor) / factor


class TimeLoop:
    """Step size policy and step sequence of main.cc:1504-1575.

    ``speed(z, q)`` returns the transport speed (the operator's
    ``compute_cell_transport_speed``), ``step(scheme, t, dt, z, q)`` advances
    the state in place (``perform_time_step``).  ``velocity`` (optional) is
    refreshed after every step as the reference's postprocess_velocity.
    """

    def __init__(self, op, scheme: str, courant: float, dt_every: int = 5, digits: int = 3):
        self.op = op
        self.scheme = scheme
        self.courant = courant
        self.dt_every = dt_every
        self.digits = digits
        self.time = 0.0
        self.step_number = 0
        self.time_step = None

    def _courant_step(self, speed: float) -> float:
        # C++ semantics: a zero speed gives an infinite step, a NaN speed a NaN one
        return self.courant / speed if speed != 0.0 else math.inf

    def start(self, z, q, time: float = 0.0):
        self.time = time
        self.step_number = 0
        self.time_step = self._courant_step(self.op.compute_cell_transport_speed(z, q))
        return self.time_step

    def next_time_step(self, z, q) -> float:
        """Step size of the next step (main.cc:1550-1555)."""
        if (self.step_number + 1) % self.dt_every == 0:
            s = truncate_to_n_digits(self.op.compute_cell_transport_speed(z, q), self.digits)
            self.time_step = self._courant_step(s)
        return self.time_step

    def advance(self, z, q, velocity=None, dt: float | None = None):
        """One step of the loop; returns the step size used.  A step size that is
        not finite (a blown-up state, main.cc:1526-1529) stops the loop before the
        step."""
        if self.time_step is None:
            self.start(z, q)
        dt = self.next_time_step(z, q) if dt is None else dt
        if not np.isfinite(dt):
            raise FloatingPointError("time step is not finite (the Courant number is too large "
                                     "or the state blew up)")
        self.op.perform_time_step(self.scheme, self.time, dt, z, q)
        if velocity is not None:
            self.op.evaluate_velocity_field(z, q, velocity)
        self.step_number += 1
        self.time += dt
        return dt
