"""GB300-native smart interpolation (random-walk label interpolation of
sparsely pre-segmented volumes), a drop-in for
``biomedisa.interpolation.smart_interpolation``."""
from .interpolation import DEFAULT_RNG_SEED, DeviceJob, smart_interpolation, walk

__all__ = ["smart_interpolation", "walk", "DeviceJob", "DEFAULT_RNG_SEED"]
__version__ = "0.1.0"
