"""GB300-native NSST (nonsubsampled shearlet transform) engine.

The compute path is libnsst.so (hand-written sm_103a kernels behind the C ABI
in include/nsst.h); this package is its Python host side.
"""
from ._lib import NsstError, THRESH_HARD, THRESH_SOFT, PYRAMID_AUTO, PYRAMID_DIRECT, PYRAMID_SPECTRAL  # noqa: F401
from .ops import *  # noqa: F401,F403
from .autograd import NsstDenoiseFn, NsstDenoiser, nsst_denoise_diff, shear_trans_adjoint, inverse_shear_adjoint  # noqa: F401,E402
