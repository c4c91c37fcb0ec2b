"""GB300-native smart interpolation (random-walk label interpolation of
sparsely pre-segmented volumes), a drop-in for
``biomedisa.interpolation.smart_interpolation``."""
from .batch import smart_interpolation_batch
from .interpolation import DEFAULT_RNG_SEED, DeviceJob, smart_interpolation, walk

__all__ = ["smart_interpolation", "smart_interpolation_batch", "walk", "DeviceJob", "DEFAULT_RNG_SEED"]
__version__ = "0.1.0"
