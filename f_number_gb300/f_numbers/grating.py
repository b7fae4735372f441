"""Grating-lobe based F-numbers (``+f_numbers/+grating/**``)."""
from __future__ import annotations

import math

from .. import _lib
from . import f_number


class grating(f_number):
    """``+f_numbers/+grating/grating.m``: lower bound on the first-order grating-lobe angle."""

    def __init__(self, angle_lb_deg: float, F_number_ub: float, distance_deg: float = 10.0):
        a, fu, d = float(angle_lb_deg), float(F_number_ub), float(distance_deg)
        if not (0 <= a <= 90):
            raise _lib.FNumError("MATLAB:validators:mustBeLessThanOrEqual", "angle_lb_deg must be in [0, 90].")
        if not fu >= 0:
            raise _lib.FNumError("MATLAB:validators:mustBeNonnegative", "F_number_ub must be nonnegative.")
        if not d <= 90:
            raise _lib.FNumError("MATLAB:validators:mustBeLessThanOrEqual", "distance_deg must not exceed 90.")
        self.angle_lb_deg, self.F_number_ub, self.distance_deg = a, fu, d
        self.thresh = math.sin(math.radians(a))
        self.lower_bound = 1.0 / (1.0 + self.thresh)
        self.upper_bound = 1.0 / (1.0 / math.sqrt(1.0 + (2.0 * fu) ** 2) + self.thresh)
        self.critical = 1.0 / self.thresh if self.thresh else math.inf


class angle_lb(grating):
    """``+f_numbers/+grating/angle_lb.m``: the frequency-dependent F-number of
    Schiffner & Schmitz (2023)."""

    def c_struct(self):
        return _lib.FNumber(_lib.F_ANGLE_LB, 0, (self.angle_lb_deg, self.F_number_ub, self.distance_deg))

    def spec(self):
        return {"kind": "grating.angle_lb", "angle_lb_deg": self.angle_lb_deg, "F_number_ub": self.F_number_ub,
                "distance_deg": self.distance_deg}

    def string(self):
        s = "angle_lb_deg_%.2f_F_ub_%.2f" % (self.angle_lb_deg, self.F_number_ub)
        if self.distance_deg >= 0:
            s += "_distance_deg_%.2f" % self.distance_deg
        return s
