"""Fixed angular distance F-numbers (``+f_numbers/+distance/**``)."""
from __future__ import annotations

import math

from .. import _lib
from . import f_number


class constant(f_number):
    """``+f_numbers/+distance/constant.m``."""

    def __init__(self, distance_deg: float, F_number_ub: float = math.inf):
        d, fu = float(distance_deg), float(F_number_ub)
        if not (0 <= d <= 90):
            raise _lib.FNumError("MATLAB:validators:mustBeLessThanOrEqual", "distance_deg must be in [0, 90].")
        if not fu > 0:
            raise _lib.FNumError("MATLAB:validators:mustBePositive", "F_number_ub must be positive.")
        self.distance_deg, self.F_number_ub = d, fu
        self.distance_rad = math.radians(d)
        self.sin_distance = math.sin(self.distance_rad)
        self.one_plus_cos_distance = 1.0 + math.cos(self.distance_rad)

    def c_struct(self):
        return _lib.FNumber(_lib.F_DISTANCE_CONSTANT, 0, (self.distance_deg, self.F_number_ub, 0.0))

    def spec(self):
        return {"kind": "distance.constant", "distance_deg": self.distance_deg, "F_number_ub": self.F_number_ub}

    def string(self):
        return "distance_deg_%.2f_F_ub_%.2f" % (self.distance_deg, self.F_number_ub)


class none(constant):
    """``+f_numbers/+distance/none.m``: distance 0, no upper bound."""

    def __init__(self):
        super().__init__(0.0, math.inf)

    def c_struct(self):
        return _lib.FNumber(_lib.F_DISTANCE_NONE, 0, (0.0, 0.0, 0.0))

    def spec(self):
        return {"kind": "distance.none"}
