"""GB300-native band detection for PyEBSDIndex (find_bands on sm_103a)."""
from .band_detect import BandDetect, GPUFindBands, getopenclparam, record_dtype  # noqa: F401
from .radon_fast import Radon  # noqa: F401
from .nlpar import NLPAR  # noqa: F401

__version__ = "0.1.0"
