"""GB300-native implementation of LIBIRWLS's training and prediction hot path.

The product is the C-ABI shared library ``libirwls_gb300.so`` built in this
folder (``python -m libirwls_gb300.build``); it exports the reference's C API
(include/*.h). ``load()`` opens it; there is no CPU fallback: if the library
is missing the call raises, and without a CUDA device every training or
prediction call returns NULL with an error message.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libirwls_gb300.so")
_lib = None


def load() -> C.CDLL:
    """Opens libirwls_gb300.so (once) and declares its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libirwls_gb300.so is not built (run `python -m libirwls_gb300.build`); "
            "this package has no CPU fallback")
    lib = _abi.load_library(LIB_PATH)
    PD = C.POINTER(C.c_double)
    PI = C.POINTER(C.c_int)
    extra = {
        "irwls_last_error": (C.c_int, []),
        "irwls_last_error_message": (C.c_char_p, []),
        "irwls_gpu_available": (C.c_int, []),
        "irwls_resident_upload": (C.c_void_p, [_abi.SvmDataset, _abi.Properties, C.c_int]),
        "irwls_resident_free": (None, [C.c_void_p]),
        "irwls_resident_budgeted": (C.c_int, [C.c_void_p, _abi.Properties, PI, PD]),
        "irwls_resident_full": (C.c_int, [C.c_void_p, _abi.Properties, PD]),
        "irwls_dataset_from_dense": (_abi.SvmDataset, [PD, PD, C.c_int, C.c_int]),
        "irwls_dataset_from_dense_with_means": (_abi.SvmDataset, [PD, PD, C.c_int, C.c_int]),
        "irwls_profile_enable": (None, [C.c_int]),
        "irwls_profile_reset": (None, []),
        "irwls_profile_read": (None, [C.c_int, PD, C.POINTER(C.c_longlong)]),
        "irwls_kernel_launches": (C.c_longlong, []),
        "irwls_transfer_bytes": (None, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "irwls_l2_flush": (C.c_int, [C.c_size_t]),
        "irwls_timer_start": (C.c_int, []),
        "irwls_timer_stop": (C.c_double, []),
        "irwls_fp64_peak_tflops": (C.c_double, [C.c_int]),
        "irwls_fp32_peak_tflops": (C.c_double, [C.c_int]),
        "irwls_last_run_info": (None, [C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "irwls_last_gram_flops": (C.c_double, []),
        "irwls_gram_tc_flops": (C.c_double, [C.c_int]),
        "irwls_set_linear_fast_path": (None, [C.c_int]),
        "irwls_get_linear_fast_path": (C.c_int, []),
        "irwls_parse_libsvm": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(_abi.SvmDataset)]),
        "readTrainFileGPU": (_abi.SvmDataset, [C.c_char_p]),
        "irwls_parse_doubles": (C.c_longlong, [C.c_char_p, C.c_size_t, PD, PI, C.c_longlong]),
        "irwls_dmodel_full": (C.c_void_p, [C.c_void_p, _abi.Properties, PD]),
        "irwls_dmodel_budgeted": (C.c_void_p, [C.c_void_p, _abi.Properties, PI, PD]),
        "irwls_dmodel_read": (C.c_void_p, [C.c_char_p]),
        "irwls_dmodel_store": (C.c_int, [C.c_void_p, C.c_char_p]),
        "irwls_dmodel_predict": (PD, [C.c_void_p, _abi.SvmDataset, _abi.PredictProperties, C.c_int]),
        "irwls_dmodel_info": (None, [C.c_void_p, PI, PI, PD]),
        "irwls_dmodel_free": (None, [C.c_void_p]),
        "irwls_full_train_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
        "irwls_budgeted_train_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                 C.c_void_p]),
        "irwls_batch_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
        "irwls_batch_set_workers": (None, [C.c_int]),
        "irwls_rand_sequence": (None, [C.c_uint, C.c_int, C.POINTER(C.c_int)]),
        "irwls_mlp_create": (C.c_void_p, [C.c_uint]),
        "irwls_mlp_free": (None, [C.c_void_p]),
        "irwls_mlp_param_count": (C.c_int, []),
        "irwls_mlp_feature_count": (C.c_int, []),
        "irwls_mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "irwls_mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "irwls_mlp_loss_grad": (C.c_double, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int,
                                             C.POINTER(C.c_float)]),
        "irwls_mlp_predict_host": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float)]),
        "irwls_mlp_train": (C.c_double, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                                         C.c_int, C.c_float, C.c_uint]),
        "irwls_set_sgma_proposer": (None, [C.c_void_p, C.c_int]),
        "irwls_sgma_traces": (C.c_int, [_abi.SvmDataset, _abi.Properties, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float)]),
        "irwls_last_nystrom_residual": (C.c_double, []),
        "irwls_tc_status": (C.c_int, []),
        "irwls_set_precision": (None, [C.c_int]),
        "irwls_get_precision": (C.c_int, []),
        "irwls_dev_sync": (C.c_int, []),
        "storeModel": (None, [C.POINTER(_abi.Model), C.c_void_p]),
        "readModel": (None, [C.POINTER(_abi.Model), C.c_void_p]),
    }
    for name, (res, args) in extra.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    lib = load()
    code = lib.irwls_last_error()
    return "" if code == 0 else "%d: %s" % (code, lib.irwls_last_error_message().decode())


class DeviceError(RuntimeError):
    pass


def check(ptr, what: str):
    """Raises DeviceError when a training/prediction entry point returned NULL."""
    if not ptr:
        raise DeviceError("%s failed: %s" % (what, last_error() or "unknown error"))
    return ptr
