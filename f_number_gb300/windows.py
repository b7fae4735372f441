"""Window functions for the apodization (``+windows/**``).

``compute_samples`` follows the MATLAB classes (``+windows/window.m:48-92``),
evaluated on |position / half-width|; the beamformer itself evaluates the
windows on the device with the MEX semantics (``+cuda/gpu_bf_windows.cu``).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib


class window:
    """Abstract base (``+windows/window.m``)."""

    id: int = -1
    parameter: float = 0.0

    def compute_samples(self, positions_over_halfwidth):
        u = np.abs(np.asarray(positions_over_halfwidth, dtype=np.float64))
        return self._samples(u)

    def string(self) -> str:
        raise NotImplementedError

    def __str__(self):
        return self.string()

    def spec(self):
        return (self.name, float(self.parameter))

    def c_struct(self):
        return _lib.Window(self.id, float(self.parameter))


class boxcar(window):
    """``+windows/boxcar.m``: 1 for |u| < 1."""
    id, name = _lib.WINDOW_BOXCAR, "boxcar"

    def _samples(self, u):
        return (u < 1).astype(np.float64)

    def string(self):
        return "boxcar"


class hann(window):
    """``+windows/hann.m``: (1 + cos(pi u)) / 2 (no cut-off at |u| >= 1, as in MATLAB)."""
    id, name = _lib.WINDOW_HANN, "hann"

    def _samples(self, u):
        return (1.0 + np.cos(math.pi * u)) / 2.0

    def string(self):
        return "hann"


class tukey(window):
    """``+windows/tukey.m``: flat for |u| <= 1 - fraction_cosine, cosine taper to 0 at |u| = 1."""
    id, name = _lib.WINDOW_TUKEY, "tukey"

    def __init__(self, fraction_cosine: float = 0.5):
        fc = float(fraction_cosine)
        if fc <= 0:
            raise _lib.FNumError("tukey:InvalidFractionCosine", "fractions_cosine must be positive!")
        if fc >= 1:
            raise _lib.FNumError("tukey:InvalidFractionCosine", "fractions_cosine must be smaller than one!")
        self.fraction_cosine = fc
        self.fraction_rectangle = 1.0 - fc

    @property
    def parameter(self):
        return self.fraction_cosine

    def _samples(self, u):
        s = (u < 1).astype(np.float64)
        taper = (u < 1) & (u > self.fraction_rectangle)
        s[taper] = (1.0 + np.cos(math.pi * (u[taper] - self.fraction_rectangle) / self.fraction_cosine)) / 2.0
        return s

    def string(self):
        return "tukey_%.2f" % self.fraction_cosine


class triangular(window):
    """``+windows/triangular.m``: 1 - |u| (no cut-off, as in MATLAB)."""
    id, name = _lib.WINDOW_TRIANGULAR, "triangular"

    def _samples(self, u):
        return 1.0 - u

    def string(self):
        return "triangular"
