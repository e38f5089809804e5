"""GB300-native NSST (nonsubsampled shearlet transform) engine.

The compute path is libnsst.so (hand-written sm_103a kernels behind the C ABI
in include/nsst.h); this package is its Python host side.
"""
from ._lib import NsstError, THRESH_HARD, THRESH_SOFT, PYRAMID_AUTO, PYRAMID_DIRECT, PYRAMID_SPECTRAL  # noqa: F401
from .ops import *  # noqa: F401,F403
from .autograd import NsstDenoiseFn, NsstDenoiser, nsst_denoise_diff, shear_trans_adjoint, inverse_shear_adjoint  # noqa: F401,E402
from .ops3d import (VolumePlan, get_meyer_based_filter, do_pyr_dec, do_pyr_rec, sh_dec, sh_dec_th_rec_cuda,  # noqa: F401,E402
                    nsst_scalars3, denoise3, denoise3_backward, Denoise3Fn, denoise3_diff, DEMO_T,
                    DEMO_NUM_DIRS, V3_NUM_DIRS)
from .separation import MakeONFilter, mrdwt_cuda, mirdwt_cuda, tv_correction_cuda, separate  # noqa: F401,E402
from . import synth  # noqa: F401,E402
