"""adfwi_gb300: GB300-native (sm_103a) propagator hot path of ADFWI.

Drop-in replacements for ADFWI's ``AcousticPropagator`` / ``ElasticPropagator`` whose time
loops and adjoints run as hand-written CUDA kernels behind a C ABI
(``include/adfwi_gb300.h``), plus the model / survey / wavelet classes those propagators
consume. The CUDA library is loaded lazily on the first solve and must have been built
(``python -m adfwi_gb300.build``); there is no CPU implementation.
"""
from .model import AbstractModel, AcousticModel, AnisotropicElasticModel, IsotropicElasticModel  # noqa: F401
from .survey import Receiver, SeismicData, Source, Survey  # noqa: F401
from .utils import wavelet, numpy2tensor, tensor2numpy, gpu2cpu, list2numpy, numpy2list  # noqa: F401
from .boundary import bc_pml, bc_pml_xz, bc_gerjan, bc_sincos  # noqa: F401
from .propagator import AcousticPropagator, ElasticPropagator  # noqa: F401

__version__ = "0.1.0"
