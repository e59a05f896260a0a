"""GB300-native IC-GN digital image correlation (drop-in for live_dic's
native engines).

The public names follow live_dic/__init__.py (21-41).  All GPU work runs in
libgbdic.so (hand-written sm_103a CUDA) through its C ABI.
"""

from .batch import ICGNBatch
from .engine import PARAMETER_ORDER, ICGNError, ImageInput, ReferenceInfo, RegistrationResult
from .full_pyramid_backend import DEFAULT_FULL_PYRAMID_LEVELS, ICGNWGPUFullPyramid
from .motion import AFFINE_PARAMETER_ORDER, MOTION_MODELS, QUADRATIC_PARAMETER_ORDER
from .native_backend import DEFAULT_IN_FLIGHT_FRAMES, DEFAULT_PYRAMID_LEVELS, ICGNWGPU
from .outlier import OUTLIER_POLICIES
from .pair import BenchmarkResult, EngineInfo, register_pair

SEEDED_SOLVE_API_VERSION = 1
# GB300 names for the same engines (ICGNBatch has no reference counterpart).
ICGNCUDA = ICGNWGPU
ICGNCUDAFullPyramid = ICGNWGPUFullPyramid

__all__ = [
    "AFFINE_PARAMETER_ORDER",
    "BenchmarkResult",
    "DEFAULT_FULL_PYRAMID_LEVELS",
    "DEFAULT_IN_FLIGHT_FRAMES",
    "DEFAULT_PYRAMID_LEVELS",
    "EngineInfo",
    "ICGNBatch",
    "ICGNCUDA",
    "ICGNCUDAFullPyramid",
    "ICGNError",
    "ICGNWGPU",
    "ICGNWGPUFullPyramid",
    "ImageInput",
    "MOTION_MODELS",
    "OUTLIER_POLICIES",
    "PARAMETER_ORDER",
    "QUADRATIC_PARAMETER_ORDER",
    "ReferenceInfo",
    "RegistrationResult",
    "SEEDED_SOLVE_API_VERSION",
    "register_pair",
]
