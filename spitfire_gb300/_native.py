"""ctypes binding of the C ABI (include/spitfire_gb300.h) exported by spitfire_gb300/_build/libspitfire_gb300.so.

The library is built in-tree by ``spitfire_gb300.build.build()``. There is no CPU fallback: if the library is
missing, or no CUDA device is present, the product path raises.
"""

import ctypes as C
import os

from ._desc import SfFlameletBatch, SfIntegrateParams, SfMechDesc, SfReactorParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'libspitfire_gb300.so')

_vp = C.c_void_p
_ip = C.c_int
_dp = C.POINTER(C.c_double)
_lib = None


class NativeError(RuntimeError):
    pass


def _declare(L):
    L.sf_last_error.restype = C.c_char_p
    L.sf_version.restype = C.c_char_p
    L.sf_mech_create.argtypes = [C.POINTER(SfMechDesc), C.POINTER(_vp)]
    L.sf_mech_destroy.argtypes = [_vp]
    L.sf_mech_info.argtypes = [_vp, C.POINTER(_ip), C.POINTER(_ip), C.POINTER(_ip)]
    L.sf_mech_set_tuning.argtypes = [_vp, _ip, _ip]
    L.sf_mech_get_tuning.argtypes = [_vp, _ip, C.POINTER(_ip)]
    L.sf_mech_layout.argtypes = [_vp, C.POINTER(_ip), C.POINTER(_ip), C.POINTER(C.c_longlong)]
    L.sf_device_status.argtypes = [_vp, _ip]
    L.sf_thermo_batch.argtypes = [_vp, _ip, _ip, _vp, _vp, _vp, _vp]
    L.sf_chem_workspace_size.argtypes = [_vp, _ip, _ip]
    L.sf_chem_workspace_size.restype = C.c_size_t
    L.sf_production_rates_batch.argtypes = [_vp, _ip, _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_rates_sens_batch.argtypes = [_vp, _ip, _vp, _vp, _vp, _ip, _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_reactor_rhs_batch.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_reactor_jac_batch.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _ip, _vp, _vp, _vp, _vp, _vp,
                                       C.c_size_t, _vp]
    L.sf_reactor_jac_host_workspace_size.argtypes = [_vp, C.POINTER(SfReactorParams), _ip]
    L.sf_reactor_jac_host_workspace_size.restype = C.c_size_t
    L.sf_reactor_jac_host_batch.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _ip, _vp, _vp, _vp, _vp, _ip, _vp,
                                            C.c_size_t, _vp]
    L.sf_reactor_jac_plain_workspace_size.argtypes = [_vp, _ip]
    L.sf_reactor_jac_plain_workspace_size.restype = C.c_size_t
    L.sf_reactor_jac_plain_batch.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _vp, _vp, _vp, _vp, _vp,
                                             C.c_size_t, _vp]
    L.sf_reactor_jac_plain_batch_static.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _vp, _vp, _vp, _vp, _vp]
    L.sf_newton_lu_batch.argtypes = [_ip, _ip, _vp, _vp, _ip, _vp, _vp, _vp, _vp, _vp]
    L.sf_newton_solve_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _ip, _ip, _vp, _vp, _vp]
    L.sf_integrate_workspace_size.argtypes = [_vp, C.POINTER(SfReactorParams), _ip]
    L.sf_integrate_workspace_size.restype = C.c_size_t
    L.sf_integrate_batch.argtypes = [_vp, C.POINTER(SfReactorParams), C.POINTER(SfIntegrateParams), _ip, _vp, _vp,
                                     _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_integrate_plain_workspace_size.argtypes = [_vp, C.POINTER(SfReactorParams), _ip]
    L.sf_integrate_plain_workspace_size.restype = C.c_size_t
    L.sf_integrate_plain_batch.argtypes = [_vp, C.POINTER(SfReactorParams), C.POINTER(SfIntegrateParams), _ip, _vp,
                                           _vp, _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_integrate_record_batch.argtypes = [_vp, C.POINTER(SfReactorParams), C.POINTER(SfIntegrateParams), _ip,
                                            _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp, _ip, _vp]
    L.sf_rate_param_adjoint_batch.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _ip, _vp, _vp, _vp, _vp, _vp]
    L.sf_flamelet_stencils.argtypes = [_vp, _dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    L.sf_flamelet_jac_indices.argtypes = [_vp, _ip, C.POINTER(_ip), C.POINTER(_ip)]
    L.sf_flamelet_rhs_batch.argtypes = [_vp, C.POINTER(SfFlameletBatch), _vp, _vp, _vp]
    L.sf_flamelet_jac_batch.argtypes = [_vp, C.POINTER(SfFlameletBatch), _vp, _ip, _ip, C.c_double, C.c_double,
                                        _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_flamelet_jac_workspace_size.argtypes = [_vp, _ip]
    L.sf_flamelet_jac_workspace_size.restype = C.c_size_t
    L.sf_btddod_factor_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.sf_btddod_solve_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.sf_btddod_matvec_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.sf_btddod_scale_and_add_diagonal_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp, C.c_double, _vp,
                                                         C.c_double, _vp, _vp]
    L.sf_btddod_blockdiag_factor_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp]
    L.sf_btddod_blockdiag_matvec_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp]
    L.sf_btddod_triangle_solve_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _ip, _vp, _vp]
    L.sf_btddod_scale_and_add_block_diagonal_batch.argtypes = [_ip, _ip, _vp, _vp, _vp, _vp, C.c_double, _vp,
                                                               C.c_double, _vp, _vp]
    L.sf_adjoint_workspace_size.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _ip]
    L.sf_adjoint_workspace_size.restype = C.c_size_t
    L.sf_adjoint_batch.argtypes = [_vp, C.POINTER(SfReactorParams), _ip, _vp, _ip, _vp, _vp, _vp, _ip, _vp, _vp, _vp,
                                   _vp, C.c_size_t, _vp]
    L.sf_flamelet_esdirk_workspace_size.argtypes = [_vp, C.POINTER(SfFlameletBatch)]
    L.sf_flamelet_esdirk_workspace_size.restype = C.c_size_t
    L.sf_flamelet_esdirk_attempt_batch.argtypes = [_vp, C.POINTER(SfFlameletBatch), _vp, _vp, _vp, _vp, _ip,
                                                   C.c_double, _ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp, C.c_size_t,
                                                   _vp]
    L.sf_flamelet_steady_workspace_size.argtypes = [_vp, C.POINTER(SfFlameletBatch)]
    L.sf_flamelet_steady_workspace_size.restype = C.c_size_t
    _d = C.c_double
    L.sf_flamelet_steady_newton_batch.argtypes = [_vp, C.POINTER(SfFlameletBatch), _vp, _vp, _d, _ip, _d, _d, _d,
                                                  _ip, _vp, _vp, _vp, C.c_size_t, _vp]
    L.sf_flamelet_steady_psitc_batch.argtypes = [_vp, C.POINTER(SfFlameletBatch), _vp, _vp, _vp, _d, _ip, _d, _d, _d,
                                                 _ip, _d, _d, _d, _d, _d, _ip, _ip, _ip, _vp, _vp, _vp, _vp,
                                                 C.c_size_t, _vp]


# Entry points declared in include/spitfire_gb300.h (the C-ABI test checks the library exports all of them).
EXPORTED = ['sf_last_error', 'sf_version', 'sf_mech_create', 'sf_mech_destroy', 'sf_mech_info', 'sf_device_status',
            'sf_thermo_batch', 'sf_production_rates_batch', 'sf_rates_sens_batch', 'sf_reactor_rhs_batch',
            'sf_reactor_jac_batch', 'sf_reactor_jac_host_workspace_size', 'sf_reactor_jac_host_batch',
            'sf_reactor_jac_plain_workspace_size', 'sf_reactor_jac_plain_batch',
            'sf_reactor_jac_plain_batch_static',
            'sf_newton_lu_batch', 'sf_newton_solve_batch', 'sf_integrate_workspace_size', 'sf_integrate_batch',
            'sf_integrate_plain_workspace_size', 'sf_integrate_plain_batch',
            'sf_flamelet_stencils', 'sf_flamelet_jac_indices', 'sf_flamelet_rhs_batch', 'sf_flamelet_jac_batch',
            'sf_btddod_factor_batch', 'sf_btddod_solve_batch', 'sf_btddod_matvec_batch',
            'sf_btddod_scale_and_add_diagonal_batch', 'sf_integrate_record_batch',
            'sf_rate_param_adjoint_batch', 'sf_mech_set_tuning', 'sf_mech_get_tuning',
            'sf_mech_layout', 'sf_btddod_blockdiag_factor_batch',
            'sf_btddod_blockdiag_matvec_batch', 'sf_btddod_triangle_solve_batch',
            'sf_btddod_scale_and_add_block_diagonal_batch', 'sf_chem_workspace_size',
            'sf_flamelet_jac_workspace_size', 'sf_flamelet_steady_workspace_size',
            'sf_flamelet_steady_newton_batch', 'sf_flamelet_steady_psitc_batch', 'sf_adjoint_workspace_size',
            'sf_adjoint_batch', 'sf_flamelet_esdirk_workspace_size', 'sf_flamelet_esdirk_attempt_batch']


def load(path=None):
    """Load (not build) the native library. Raises NativeError if it is absent."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise NativeError(f'spitfire_gb300 native library not built ({p}); run spitfire_gb300.build.build()')
        L = C.CDLL(p)
        missing = [s for s in EXPORTED if not hasattr(L, s)]
        if missing:
            raise NativeError(f'native library lacks entry points: {missing}')
        _declare(L)
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        msg = load().sf_last_error().decode()
        raise NativeError(f'spitfire_gb300 error {rc}: {msg}')
    return rc


def ptr(t):
    """Device (or host) address of a torch tensor / numpy array, or None."""
    if t is None:
        return None
    if hasattr(t, 'data_ptr'):
        return C.c_void_p(t.data_ptr())
    return C.c_void_p(t.ctypes.data)


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)
