"""F-number classes (``+f_numbers/**``).  ``compute_values`` runs the
library's native implementation (``fnum_f_number_values``), which is what
the beamformer uses on its band."""
from __future__ import annotations

import math

import numpy as np

from .. import _lib


class f_number:
    """Abstract base (``+f_numbers/f_number.m``)."""

    def c_struct(self) -> "_lib.FNumber":
        raise NotImplementedError

    def spec(self) -> dict:
        raise NotImplementedError

    def compute_values(self, element_pitch_over_lambda):
        """F per normalised element pitch (``f_number.m:50-114``)."""
        p = np.ascontiguousarray(np.asarray(element_pitch_over_lambda, dtype=np.float64).ravel())
        if p.size == 0:
            raise _lib.FNumError("MATLAB:validators:mustBeNonempty", "Value must not be empty.")
        if not np.all(p > 0):
            raise _lib.FNumError("MATLAB:validators:mustBePositive", "Value must be positive.")
        out = np.empty_like(p)
        s = self.c_struct()
        _lib.check(_lib.lib().fnum_f_number_values(s, _lib.dptr(p), p.size, _lib.dptr(out)))
        return out.reshape(np.shape(element_pitch_over_lambda))

    def compute_bounds_main(self, element_pitch_over_lambda):
        """``f_number.m:119-182``."""
        v = self.compute_values(element_pitch_over_lambda)
        return 1.0 / np.sqrt(1.0 + (2.0 * v) ** 2)

    def compute_distances_grating(self, element_pitch_over_lambda):
        """``f_number.m:187-240``."""
        p = np.asarray(element_pitch_over_lambda, dtype=np.float64)
        return 1.0 / p - self.compute_bounds_main(p)

    def compute_depths_of_field(self, element_pitch_over_lambda):
        """``f_number.m:245-298``."""
        p = np.asarray(element_pitch_over_lambda, dtype=np.float64)
        return 6.1434 / p * self.compute_values(p) ** 2

    def __str__(self):
        return self.string()


class constant(f_number):
    """``+f_numbers/constant.m``."""

    def __init__(self, value: float = 1.0):
        value = float(value)
        if not value >= 0:
            raise _lib.FNumError("MATLAB:validators:mustBeNonnegative", "Value must be nonnegative.")
        self.value = value

    def c_struct(self):
        return _lib.FNumber(_lib.F_CONSTANT, 0, (self.value, 0.0, 0.0))

    def spec(self):
        return {"kind": "constant", "value": self.value}

    def string(self):
        return "constant_%.2f" % self.value


from . import distance, grating, directivity  # noqa: E402,F401
