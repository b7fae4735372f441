"""Element-directivity based F-numbers (``+f_numbers/+directivity/**``)."""
from __future__ import annotations

import types

from .. import _lib
from . import f_number


class _obliquity:
    def __str__(self):
        return self.string()


class _rigid_obliquity(_obliquity):
    """``+obliquity/rigid.m``: factor 1."""
    code = _lib.OBLIQUITY_RIGID

    def string(self):
        return "rigid"


class _soft_obliquity(_obliquity):
    """``+obliquity/soft.m``: factor cos(theta)."""
    code = _lib.OBLIQUITY_SOFT

    def string(self):
        return "soft"


obliquity = types.SimpleNamespace(rigid=_rigid_obliquity, soft=_soft_obliquity, obliquity=_obliquity)


class directivity(f_number):
    """``+f_numbers/+directivity/directivity.m``: the angle where the element
    directivity drops by attenuation_dB sets F = 1 / (2 tan(angle))."""

    def __init__(self, width_over_pitch: float, obliquity_factor=None, attenuation_dB: float = 3.0):
        w = float(width_over_pitch)
        if not (0 <= w <= 1):
            raise _lib.FNumError("MATLAB:validators:mustBeLessThanOrEqual", "width_over_pitch must be in [0, 1].")
        if attenuation_dB is None:
            attenuation_dB = 3.0
        if not float(attenuation_dB) > 0:
            raise _lib.FNumError("MATLAB:validators:mustBePositive", "attenuation_dB must be positive.")
        self.width_over_pitch = w
        self.obliquity_factor = obliquity_factor if obliquity_factor is not None else _soft_obliquity()
        self.attenuation_dB = float(attenuation_dB)
        self.thresh = 10.0 ** (-self.attenuation_dB / 20.0)

    def c_struct(self):
        return _lib.FNumber(_lib.F_DIRECTIVITY, self.obliquity_factor.code,
                            (self.width_over_pitch, self.attenuation_dB, 0.0))

    def spec(self):
        return {"kind": "directivity", "width_over_pitch": self.width_over_pitch,
                "obliquity": self.obliquity_factor.string(), "attenuation_dB": self.attenuation_dB}

    def string(self):
        return "directivity_%s_fill_%.2f_att_%.1f_dB" % (self.obliquity_factor.string(),
                                                          self.width_over_pitch * 1e2, self.attenuation_dB)


class rigid(directivity):
    """``rigid.m``: rigid baffle."""

    def __init__(self, width_over_pitch, attenuation_dB=None):
        super().__init__(width_over_pitch, _rigid_obliquity(), attenuation_dB)


class soft(directivity):
    """``soft.m``: soft baffle."""

    def __init__(self, width_over_pitch, attenuation_dB=None):
        super().__init__(width_over_pitch, _soft_obliquity(), attenuation_dB)


class perrot(soft):
    """``perrot.m``: soft baffle, 3 dB."""

    def __init__(self, width_over_pitch):
        super().__init__(width_over_pitch, 3.0)


class szabo(rigid):
    """``szabo.m``: F = (w / lambda) / 1.2."""

    def __init__(self, width_over_pitch):
        super().__init__(width_over_pitch, 6.0)

    def c_struct(self):
        return _lib.FNumber(_lib.F_SZABO, 0, (self.width_over_pitch, 0.0, 0.0))

    def spec(self):
        return {"kind": "directivity.szabo", "width_over_pitch": self.width_over_pitch}
