"""Normalisation of the apodization weights (``+normalizations/**``)."""
from __future__ import annotations

import numpy as np

from . import _lib
from . import windows as _windows


class normalization:
    code = -1

    def apply(self, samples):
        """``+normalizations/normalization.m:48-90`` on [frequencies x elements]."""
        return self._apply(np.asarray(samples, dtype=np.float64))

    def __str__(self):
        return self.string()


class on(normalization):
    """``+normalizations/on.m:60-61``: divide every row by its sum."""
    code = _lib.NORM_ON

    def _apply(self, s):
        return s / s.sum(axis=1, keepdims=True)

    def string(self):
        return "on"


class off(normalization):
    """``+normalizations/off.m``: unchanged."""
    code = _lib.NORM_OFF

    def _apply(self, s):
        return s

    def string(self):
        return "off"


class windowed(on):
    """``+normalizations/windowed.m:69-87``: "on" and a window across the rows.
    The GPU path treats it as "on" (the reference MEX parses the window but
    never applies it, ``+cuda/gpu_bf_das_pw_rf.cu:421-427``)."""
    code = _lib.NORM_WINDOWED

    def __init__(self, window=None):
        if window is None:
            window = _windows.tukey(0.2)
        if not isinstance(window, _windows.window):
            raise _lib.FNumError("windowed:NoWindows", "windows must be windows.window!")
        self.window = window

    def _apply(self, s):
        sn = super()._apply(s)
        n2 = (sn > 0).sum(axis=0) / 2.0
        idx = np.arange(s.shape[0])[:, None]
        return sn * self.window.compute_samples((idx - n2[None, :]) / n2[None, :])

    def string(self):
        return "on_%s" % self.window.string()
