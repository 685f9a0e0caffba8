"""GB300-native (sm_103a) equilibrium line-by-line spectrum synthesis with the
LDM/DIT method, behind the RADIS GPU entry points:

* ``gpuApp``          - the reference's GPU application object (radis/gpu/gpu.py)
* ``SpectrumFactory`` - ``eq_spectrum_gpu`` front end (radis/lbl/factory.py)
* ``calc_spectrum``   - ``mode='gpu'`` one-call front end (radis/lbl/calc.py)
* ``Spectrum``        - output container with ``recalc_gpu`` / ``exit_gpu``

The compute path is the CUDA library ``libradisgb.so`` (C ABI in
include/radis_gb300.h), bound with ctypes in ``radis_gb300._lib``.
"""
__version__ = "0.1.0"

from .factory import SpectrumFactory, calc_spectrum  # noqa: E402,F401
from .gpu import gpuApp  # noqa: E402,F401
from .spectrum import Spectrum  # noqa: E402,F401
