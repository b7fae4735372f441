"""GB300-native Fourier-domain delay-and-sum beamformer with frequency-dependent
F-number: the ``das_pw`` / ``das_sa`` GPU path of the f_number toolbox
(plane-wave compounding and synthetic-aperture focusing), behind the
reference's own interface.  The compute runs in libfnum.so (include/fnum.h)."""
from . import f_numbers, normalizations, platforms, windows  # noqa: F401
from ._lib import FNumError, LibraryNotBuilt  # noqa: F401
from .das import (PWPlan, SAPlan, band, das_pw, das_sa, gpu_bf_das_pw_rf,  # noqa: F401
                  gpu_bf_saft_rf)

__all__ = ["das_pw", "das_sa", "gpu_bf_das_pw_rf", "gpu_bf_saft_rf", "PWPlan", "SAPlan", "band", "f_numbers",
           "windows", "normalizations", "platforms", "FNumError", "LibraryNotBuilt"]
