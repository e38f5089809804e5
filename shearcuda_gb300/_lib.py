"""ctypes binding of libnsst.so (the C ABI declared in include/nsst.h).

The library is built in-tree by ``shearcuda_gb300.build``.  There is no
fallback: if the shared library is missing or fails to load, importing the
binding raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libnsst.so')

NSST_OK = 0
STATUS_NAMES = {0: 'NSST_OK', 1: 'NSST_ERR_INVALID_ARG', 2: 'NSST_ERR_UNSUPPORTED_SIZE',
                3: 'NSST_ERR_OUT_OF_MEMORY', 4: 'NSST_ERR_CUDA', 5: 'NSST_ERR_TIMEOUT', 6: 'NSST_ERR_NUMERIC'}
THRESH_HARD, THRESH_SOFT = 0, 1
PYRAMID_AUTO, PYRAMID_DIRECT, PYRAMID_SPECTRAL = 0, 1, 2
DIRECTIONAL_AUTO, DIRECTIONAL_SPLIT, DIRECTIONAL_FUSED = 0, 1, 2
MAX_LEVELS = 8


class NsstConfig(ctypes.Structure):
    _fields_ = [('nlevels', ctypes.c_int), ('dcomp', ctypes.c_int * MAX_LEVELS),
                ('dsize', ctypes.c_int * MAX_LEVELS), ('lpfilt', ctypes.c_char * 16),
                ('pyramid', ctypes.c_int)]


class NsstItem(ctypes.Structure):
    _fields_ = [('x', ctypes.c_void_p), ('out', ctypes.c_void_p), ('sigma', ctypes.c_double), ('plan', ctypes.c_int)]


class Nsst3Config(ctypes.Structure):
    _fields_ = [('nlevels', ctypes.c_int), ('num_dirs', ctypes.c_int * MAX_LEVELS), ('pyr_mode', ctypes.c_double),
                ('grid', ctypes.c_int)]


GRID_FAST, GRID_MARSHAL = 0, 1


class NsstSeparateInfo(ctypes.Structure):
    _fields_ = [('sigma', ctypes.c_double), ('stop', ctypes.c_double), ('buff_shear', ctypes.c_double),
                ('buff_wavelet', ctypes.c_double), ('deltamax', ctypes.c_double), ('lam', ctypes.c_double)]


TUNE_MAX_CANDIDATES = 32


class NsstTuneResult(ctypes.Structure):
    _fields_ = [('n', ctypes.c_int), ('ncand', ctypes.c_int), ('chosen', ctypes.c_int),
                ('name', (ctypes.c_char * 64) * TUNE_MAX_CANDIDATES), ('ms', ctypes.c_float * TUNE_MAX_CANDIDATES),
                ('direct_support', ctypes.c_int * MAX_LEVELS), ('direct_err', ctypes.c_double * MAX_LEVELS),
                ('direct_bound_ms', ctypes.c_float), ('direct_wins', ctypes.c_int)]


class NsstError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__('%s: %s' % (STATUS_NAMES.get(status, status), msg))
        self.status = status


_vp, _ci, _cd, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

# (name, restype, argtypes)
SIGNATURES = [
    ('nsst_last_error', ctypes.c_char_p, []),
    ('nsst_version', ctypes.c_char_p, []),
    ('nsst_plan_create', _ci, [ctypes.POINTER(NsstConfig), _ci, _ci, ctypes.POINTER(_vp)]),
    ('nsst_plan_create_batch', _ci, [ctypes.POINTER(NsstConfig), _ci, _ci, _ci, ctypes.POINTER(_vp)]),
    ('nsst_plan_batch_capacity', _ci, [_vp]),
    ('nsst_filters_save', _ci, [ctypes.c_char_p, ctypes.POINTER(NsstConfig), _ci]),
    ('nsst_filters_load', _ci, [ctypes.c_char_p, _ip, _ip, _ip, _ip, _dp, _dp, _ip]),
    ('nsst_plan_create_from_file', _ci, [ctypes.c_char_p, _ci, _ci, _ci, ctypes.POINTER(_vp)]),
    ('nsst_plan_use_graphs', _ci, [_vp, _ci]),
    ('nsst_plan_set_directional', _ci, [_vp, _ci]),
    ('nsst_plan_directional', _ci, [_vp, _ci]),
    ('nsst_plan_fused_clusters', _ci, [_vp]),
    ('nsst_plan_check_device', _ci, [_vp]),
    ('nsst_plan_autotune', _ci, [_vp, _ci, ctypes.POINTER(NsstTuneResult)]),
    ('nsst_plan_select_directional', _ci, [_vp, _ci, _ci]),
    ('nsst_plan_directional_candidates', _ci, [_vp, ctypes.c_char_p, _sz]),
    ('nsst_direct_support', _ci, [ctypes.POINTER(NsstConfig), _ci, _ci, _cd, _ip, _dp]),
    ('nsst_plan_destroy', _ci, [_vp]),
    ('nsst_plan_num_bands', _ci, [_vp]),
    ('nsst_plan_band_levels', _ci, [_vp, _ip]),
    ('nsst_plan_device_bytes', _sz, [_vp]),
    ('nsst_pyramid_filters', _ci, [ctypes.c_char_p, _ip, _dp]),
    ('nsst_shearing_filters', _ci, [_ci, _ci, _dp]),
    ('nsst_level_spectra', _ci, [_ci, _ci, _ci, _ci, _dp]),
    ('nsst_plan_level_spectra', _ci, [_vp, _ci, _dp]),
    ('nsst_atrousdec', _ci, [_vp, _vp, _vp, _vp]),
    ('nsst_atrousrec', _ci, [_vp, _vp, _vp, _vp]),
    ('nsst_atrousdec_noalloc', _ci, [_vp, _vp, _ci, _ci, _ci, ctypes.c_char_p, _vp]),
    ('nsst_shear_trans', _ci, [_vp, _vp, _vp, _vp]),
    ('nsst_thresh', _ci, [_vp, _vp, _cd, _dp, _dp, _ci, _vp]),
    ('nsst_inverse_shear', _ci, [_vp, _vp, _vp, _vp]),
    ('nsst_denoise', _ci, [_vp, _vp, _vp, _cd, _dp, _dp, _ci, _vp]),
    ('nsst_denoise_batch', _ci, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _ci, _dp, _dp, _dp, _ci, _vp]),
    ('nsst_multi_create', _ci, [ctypes.POINTER(_vp), _ci, ctypes.POINTER(_vp)]),
    ('nsst_multi_denoise', _ci, [_vp, ctypes.POINTER(NsstItem), _ci, _dp, _ci, _vp]),
    ('nsst_multi_destroy', _ci, [_vp]),
    ('nsst_plan_enable_grad', _ci, [_vp]),
    ('nsst_shear_trans_adjoint', _ci, [_vp, _vp, _vp, _vp]),
    ('nsst_inverse_shear_adjoint', _ci, [_vp, _vp, _vp, _vp]),
    ('nsst_denoise_tau_batch', _ci, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _ci, _vp, _ci, _vp]),
    ('nsst_denoise_tau_backward', _ci, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), _ci,
                                        _vp, _vp, _ci, _ci, _vp]),
    ('nsst_denoise_tau_backward_saved', _ci, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _ci, _vp, _vp, _ci, _ci,
                                              _vp]),
    ('nsst_plan_saved_items', _ci, [_vp]),
    ('nsst_thresh_max', _ci, [_vp, _vp, _cd, _dp, _dp, _ci, _dp, _vp]),
    ('nsst_band_norms', _ci, [_vp, _dp]),
    ('nsst_re_weight_band', _ci, [_vp, _vp, _dp, _ci, _vp, _vp]),
    ('nsst_plan_set_scalars', _ci, [_vp, _dp]),
    ('nsst_compute_scalars', _ci, [_vp, ctypes.c_uint64, _dp]),
    ('nsst_timers_enable', _ci, [_vp, _ci]),
    ('nsst_timers_read', _ci, [_vp, ctypes.c_char_p, _sz, ctypes.POINTER(ctypes.c_float), _ci]),
    ('nsst_onfilter', _ci, [ctypes.c_char_p, _ci, _dp, _ip]),
    ('nsst_mrdwt', _ci, [_vp, _ci, _ci, _ci, _dp, _ci, _ci, _vp, _vp, _vp]),
    ('nsst_mirdwt', _ci, [_vp, _vp, _ci, _ci, _ci, _dp, _ci, _ci, _vp, _vp]),
    ('nsst_tv_correction', _ci, [_vp, _ci, _ci, _ci, _cd, _vp, _vp]),
    ('nsst_separate', _ci, [_vp, _vp, _ci, _ci, _ci, _cd, _cd, _dp, _ci, _vp, _vp, ctypes.POINTER(NsstSeparateInfo),
                            _vp]),
    ('nsst_launch_count', ctypes.c_uint64, []),
    ('nsst_debug_fail_next_alloc', None, [_ci]),
    ('nsst3_plan_create', _ci, [ctypes.POINTER(Nsst3Config), _ci, _ci, _ci, _ci, ctypes.POINTER(_vp)]),
    ('nsst3_plan_destroy', _ci, [_vp]),
    ('nsst3_num_bands', _ci, [_vp]),
    ('nsst3_subband_floats', _sz, [_vp]),
    ('nsst3_plan_device_bytes', _sz, [_vp]),
    ('nsst3_level_dims', _ci, [_vp, _ci, _ip, _ip]),
    ('nsst3_band_info', _ci, [_vp, _ci, _ip]),
    ('nsst3_meyer_filters', _ci, [_ci, _ip, _dp]),
    ('nsst3_pyr_dec', _ci, [_vp, _vp, _vp, _ci, _vp]),
    ('nsst3_pyr_rec', _ci, [_vp, _vp, _vp, _ci, _vp]),
    ('nsst3_sh_dec', _ci, [_vp, _vp, _ci, _vp, _ci, _vp]),
    ('nsst3_sh_dec_thresh_rec', _ci, [_vp, _vp, _vp, _ci, _dp, _dp, _dp, _vp]),
    ('nsst3_denoise_batch', _ci, [_vp, _vp, _vp, _ci, _dp, _dp, _dp, _vp]),
    ('nsst3_compute_scalars', _ci, [_vp, ctypes.c_uint64, _dp]),
    ('nsst3_plan_set_scalars', _ci, [_vp, _dp]),
    ('nsst3_plan_enable_grad', _ci, [_vp]),
    ('nsst3_denoise_backward', _ci, [_vp, _vp, _vp, _ci, _vp]),
]

_lib = None


def lib():
    """Load libnsst.so (once).  Raises OSError if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError('libnsst.so is not built (%s); run shearcuda_gb300.build.build()' % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != NSST_OK:
        raise NsstError(status, lib().nsst_last_error().decode())
    return status
