"""Builds the package's parameter objects from the oracle's spec form
(dicts for F-numbers, (name, parameter) tuples for windows)."""
from f_number_gb300 import f_numbers, normalizations, windows


def window(spec):
    name, par = spec
    if name == "boxcar":
        return windows.boxcar()
    if name == "hann":
        return windows.hann()
    if name == "tukey":
        return windows.tukey(par)
    if name == "triangular":
        return windows.triangular()
    raise ValueError(name)


def f_number(spec):
    if spec is None:
        return None
    k = spec["kind"]
    if k == "constant":
        return f_numbers.constant(spec["value"])
    if k == "grating.angle_lb":
        return f_numbers.grating.angle_lb(spec["angle_lb_deg"], spec["F_number_ub"], spec.get("distance_deg", 10.0))
    if k == "distance.constant":
        return f_numbers.distance.constant(spec["distance_deg"], spec.get("F_number_ub", float("inf")))
    if k == "distance.none":
        return f_numbers.distance.none()
    if k == "directivity":
        obl = f_numbers.directivity.obliquity.soft() if spec.get("obliquity", "soft") == "soft" else \
            f_numbers.directivity.obliquity.rigid()
        return f_numbers.directivity.directivity(spec["width_over_pitch"], obl, spec.get("attenuation_dB", 3.0))
    if k == "directivity.szabo":
        return f_numbers.directivity.szabo(spec["width_over_pitch"])
    raise ValueError(k)


def normalization(name):
    return {"on": normalizations.on(), "off": normalizations.off()}[name]
