"""GB300-native bundle adjustment: the Levenberg-Marquardt camera-shared
bundle-adjustment path of hs_sfm, on hand-written sm_103a CUDA kernels behind
a C ABI (include/gba.h, libgba.so)."""
from . import abi  # noqa: F401
