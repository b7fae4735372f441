"""Python side of the MEX stand-in (tests/mexshim/mexshim.cpp): builds a gateway
from f_number_gb300/mex linked with the shim and libfnum, and calls its
mexFunction with mxArrays made from numpy arrays and from the parameter
objects' MATLAB class names and properties.

TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "f_number_gb300")
MX_LOGICAL, MX_DOUBLE, MX_SINGLE, MX_OBJECT = 3, 6, 7, 18


class MexError(Exception):
    def __init__(self, ident, msg):
        super().__init__("%s: %s" % (ident, msg))
        self.identifier = ident
        self.message = msg


CALLBACK = C.CFUNCTYPE(C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p))


def build(gateway: str, outdir: str) -> str:
    """Compiles f_number_gb300/mex/<gateway>.cpp with the shim into <outdir>/<gateway>_shim.so."""
    from f_number_gb300 import build as fb
    lib = fb.build()
    gxx = shutil.which("g++")
    if gxx is None:
        raise RuntimeError("no g++")
    out = os.path.join(outdir, gateway + "_shim.so")
    cmd = [gxx, "-std=c++17", "-O1", "-shared", "-fPIC", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", HERE,
           os.path.join(PKG, "mex", gateway + ".cpp"), os.path.join(HERE, "mexshim.cpp"), "-o", out,
           "-L", os.path.dirname(lib), "-lfnum", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return out


class Gateway:
    def __init__(self, path: str):
        L = C.CDLL(path)
        vp = C.c_void_p
        L.shim_numeric.restype = vp
        L.shim_numeric.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_size_t), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
        L.shim_object.restype = vp
        L.shim_object.argtypes = [C.c_char_p, C.c_char_p]
        L.shim_set_property.argtypes = [vp, C.c_char_p, vp]
        L.shim_set_callback.argtypes = [CALLBACK]
        L.shim_class.argtypes = [vp]
        L.shim_is_complex.argtypes = [vp]
        L.shim_ndim.argtypes = [vp]
        L.shim_dims.argtypes = [vp, C.POINTER(C.c_size_t)]
        L.shim_read.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.shim_free.argtypes = [vp]
        L.shim_call.argtypes = [C.c_int, C.POINTER(vp), C.c_int, C.POINTER(vp), C.c_char_p, C.c_int, C.c_char_p,
                                C.c_int]
        self.L = L
        self._cb = None
        self.calls = []

    # ---- building inputs ---------------------------------------------------
    def array(self, a, cls=MX_DOUBLE):
        """numpy array -> mxArray (MATLAB column-major; 1-D becomes a row vector)."""
        a = np.asarray(a)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        if a.ndim == 1:
            a = a.reshape(1, -1)
        dims = (C.c_size_t * a.ndim)(*a.shape)
        re = np.ascontiguousarray(np.real(a).ravel(order="F"), dtype=np.float64)
        im = np.ascontiguousarray(np.imag(a).ravel(order="F"), dtype=np.float64) if np.iscomplexobj(a) else None
        return self.L.shim_numeric(cls, a.ndim, dims, re.ctypes.data_as(C.POINTER(C.c_double)),
                                   im.ctypes.data_as(C.POINTER(C.c_double)) if im is not None else None)

    def empty(self):
        return self.L.shim_numeric(MX_DOUBLE, 2, (C.c_size_t * 2)(0, 0), None, None)

    def obj(self, class_name, supers=(), **props):
        o = self.L.shim_object(class_name.encode(), ",".join(supers).encode())
        for k, v in props.items():
            self.L.shim_set_property(o, k.encode(), self.array(float(v)))
        return o

    def window(self, spec):
        name, par = spec
        if name == "tukey":
            return self.obj("windows.tukey", ("windows.window",), fraction_cosine=float(par))
        return self.obj("windows." + name, ("windows.window",))

    def f_number(self, spec):
        k = spec["kind"]
        base = ("f_numbers.f_number",)
        if k == "constant":
            return self.obj("f_numbers.constant", base, value=float(spec["value"]))
        if k == "grating.angle_lb":
            return self.obj("f_numbers.grating.angle_lb", ("f_numbers.grating.grating",) + base,
                            angle_lb_deg=spec["angle_lb_deg"], F_number_ub=spec["F_number_ub"],
                            distance_deg=spec.get("distance_deg", 10.0))
        if k == "distance.constant":
            return self.obj("f_numbers.distance.constant", base, distance_deg=spec["distance_deg"],
                            F_number_ub=spec.get("F_number_ub", float("inf")))
        if k == "distance.none":
            return self.obj("f_numbers.distance.none", base)
        if k == "directivity":
            obl = self.L.shim_object(("f_numbers.directivity.obliquity." + spec.get("obliquity", "soft")).encode(),
                                     b"f_numbers.directivity.obliquity.obliquity")
            o = self.obj("f_numbers.directivity.perrot", ("f_numbers.directivity.directivity",) + base,
                         width_over_pitch=spec["width_over_pitch"], attenuation_dB=spec.get("attenuation_dB", 3.0))
            self.L.shim_set_property(o, b"obliquity_factor", obl)
            return o
        raise ValueError(k)

    def normalization(self, name):
        return self.obj("normalizations." + name, ("normalizations.normalization",))

    def on_matlab_call(self, fn):
        """fn(name, args: list of mxArray handles) -> numpy array or None (unhandled)."""
        def cb(name, nlhs, plhs, nrhs, prhs):
            self.calls.append(name.decode())
            out = fn(name.decode(), [prhs[i] for i in range(nrhs)])
            if out is None:
                return 1
            plhs[0] = self.array(out)
            return 0
        self._cb = CALLBACK(cb)
        self.L.shim_set_callback(self._cb)

    # ---- reading outputs ---------------------------------------------------
    def read(self, h):
        nd = self.L.shim_ndim(h)
        dims = (C.c_size_t * nd)()
        self.L.shim_dims(h, dims)
        shape = tuple(dims)
        n = int(np.prod(shape))
        re = np.zeros(n)
        im = np.zeros(n)
        self.L.shim_read(h, re.ctypes.data_as(C.POINTER(C.c_double)), im.ctypes.data_as(C.POINTER(C.c_double)))
        v = (re + 1j * im) if self.L.shim_is_complex(h) else re
        return v.reshape(shape, order="F"), self.L.shim_class(h)

    def call(self, nlhs, args):
        plhs = (C.c_void_p * max(nlhs, 1))()
        prhs = (C.c_void_p * max(len(args), 1))(*args)
        ident = C.create_string_buffer(256)
        msg = C.create_string_buffer(1024)
        st = self.L.shim_call(nlhs, plhs, len(args), prhs, ident, 256, msg, 1024)
        for a in args:
            self.L.shim_free(a)
        if st != 0:
            raise MexError(ident.value.decode(), msg.value.decode())
        out = []
        for i in range(nlhs):
            out.append(self.read(plhs[i]))
            self.L.shim_free(plhs[i])
        return out
