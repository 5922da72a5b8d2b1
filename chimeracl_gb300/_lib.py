"""ctypes binding of the in-tree CUDA library (libchimeracl_gb300.so).

The library is the product's compute path: there is no CPU fallback.  If it
is missing, or no CUDA device is visible, importing the binding raises.
"""
import ctypes as C
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libchimeracl_gb300.so")

CCL_F64 = 0
CCL_F32 = 1


class CCLError(RuntimeError):
    """A C-ABI call returned a non-zero status."""


_vp, _d, _i, _l, _u32, _sz = C.c_void_p, C.c_double, C.c_int, C.c_long, C.c_uint32, C.c_size_t
_pp = C.POINTER(C.c_void_p)

# name -> argtypes (all return int status)
SIGNATURES = {
    "ccl_push_x": [_i, _l, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _vp],
    "ccl_push_x_compensated": [_i, _l] + [_vp] * 10 + [_d, _vp],
    "ccl_index_sort_workspace": [_l, _l, C.POINTER(_sz)],
    "ccl_index_sort": [_i, _l, _vp, _vp, _vp, _i, _d, _d, _i, _d, _d,
                       _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp],
    "ccl_push_x_keys": [_i, _l] + [_vp] * 10 + [_d, _i, _d, _d, _i, _d, _d, _vp, _vp, _vp, _sz,
                                                 _vp],
    "ccl_index_sort_keyed": [_l, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp],
    "ccl_index_sort_noalloc": [_i, _l, _vp, _vp, _vp, _i, _d, _d, _i, _d, _d,
                               _vp, _vp, _vp, _vp, _vp, _vp],
    "ccl_align": [_i, _l, _i, _pp, _pp, _vp, _vp],
    "ccl_iota_u32": [_vp, _l, _vp],
    "ccl_fill_grid": [_i, _l, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp],
    "ccl_dens_profile": [_i, _l, _vp, _vp, _vp, _vp, _vp, _u32, _vp],
    "ccl_gamma_inv": [_i, _l, _vp, _vp, _vp, _vp, _vp],
    "ccl_deposit_scalar": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _d, _d, _i, _d, _d, _pp, _vp],
    "ccl_deposit_vector": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                           _i, _d, _d, _i, _d, _d, _pp, _vp],
    "ccl_deposit_scalar_lo": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _d, _d, _i, _d, _d,
                              _pp, _vp, _vp, _vp, _vp],
    "ccl_deposit_vector_lo": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                              _i, _d, _d, _i, _d, _d, _pp, _vp, _vp, _vp, _vp],
    "ccl_deposit_postproc": [_i, _i, _i, _pp, _i, _i, _vp, _vp],
    "ccl_warp_axis": [_i, _i, _i, _pp, _i, _vp],
    "ccl_gather_push": [_i, _i, _l, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d,
                        _i, _d, _d, _i, _d, _d, _pp, _vp],
    "ccl_gather_push_cells": [_i, _i, _l, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                              _d, _i, _d, _d, _i, _d, _d, _pp, _vp],
    "ccl_gather_push_cells_lo": [_i, _i, _l, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                 _d, _i, _d, _d, _i, _d, _d, _pp, _vp, _vp, _vp, _vp],
    "ccl_phase": [_i, _i, _vp, _vp, _d, _i, _vp],
    "ccl_fft_forward_rows": [_i, _i, _i, _vp, _l, _i, _vp, _vp, _vp, _vp],
    "ccl_fft_backward_rows": [_i, _i, _i, _vp, _vp, _l, _i, _vp, _vp],
    "ccl_damp_rows": [_i, _i, _i, _vp, _vp, _i, _vp, _vp, _vp, _i, _vp],
    "ccl_dht_gemm": [_i, _i, _i, _i, _i, _i, _pp, _pp, _l, _pp, _l, _d, _d, _d, _vp],
    "ccl_fft_forward_batch": [_i, _i, _i, _i, _pp, _vp, _vp, _pp, _vp, _pp, _vp],
    "ccl_fft_backward_batch": [_i, _i, _i, _i, _pp, _pp, _vp, _vp, _vp, _vp],
    "ccl_damp_batch": [_i, _i, _i, _i, _pp, _pp, _vp, _vp, _vp, _vp, _i, _vp],
    "ccl_dht_gemm_batch": [_i, _i, _i, _i, _vp, _i, _pp, _pp, _vp, _pp, _vp, _d, _d, _d, _vp],
    "ccl_psatd_advance": [_i, _l, _d, _vp, _vp, _vp, _pp, _vp],
    "ccl_psatd_advance_split": [_i, _l, _vp, _pp, _vp],
    "ccl_dht_bf16x3_prepare_bytes": [_i, _i, C.POINTER(_sz)],
    "ccl_dht_bf16x3_prepare": [_i, _vp, _i, _i, _vp, _sz, _vp],
    "ccl_dht_bf16x3_gemm_batch": [_i, _i, _i, _vp, _i, _pp, _pp, _vp, _pp, _vp, _d, _d, _d, _vp],
    "ccl_dht_bf16x3_status": [_i],
    "ccl_wait_probe": [_l, _i, _vp, _vp],
    "ccl_sort_status": [_i],
    "ccl_scan_wait_probe": [_l, _i, _vp, _vp, _vp],
    "ccl_get_m1": [_i, _i, _i, _vp, _vp, _vp],
    "ccl_grad_combine": [_i, _i, _i, _i, _vp, _pp, _pp, _pp, _pp, _vp],
    "ccl_rot_combine": [_i, _i, _i, _i, _vp, _pp, _pp, _pp, _pp, _pp, _vp],
    "ccl_set": [_i, _i, _l, _vp, _d, _d, _vp],
    "ccl_set_batch": [_i, _i, C.POINTER(C.c_int), C.POINTER(C.c_long), _pp, _d, _d, _vp],
    "ccl_append_c2c": [_i, _l, _vp, _vp, _vp],
    "ccl_zpaxz": [_i, _l, _vp, _d, _d, _vp, _vp],
    "ccl_axpbyz": [_i, _l, _d, _d, _vp, _d, _d, _vp, _vp, _vp],
    "ccl_mult_elementwise": [_i, _l, _vp, _vp, _vp],
    "ccl_ab_dot_x": [_i, _i, _i, _d, _d, _vp, _vp, _vp, _vp],
    "ccl_cast_c2d": [_i, _l, _vp, _vp, _vp],
    "ccl_profile_edges": [_i, _i, _i, _i, _vp, _vp, _i, _vp],
    "ccl_multiply_by_phase": [_i, _i, _i, _vp, _vp, _vp],
    # adjoint of the step
    "ccl_deposit_adjoint": [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                            _i, _d, _d, _i, _d, _d, _pp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                            _vp, _vp],
    "ccl_gather_push_adjoint": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _i,
                                _d, _d, _i, _d, _d, _pp, _pp, _vp, _vp, _vp, _vp, _vp, _vp,
                                _vp, _vp],
    "ccl_push_x_adjoint": [_i, _l] + [_vp] * 11 + [_d, _vp],
    "ccl_psatd_adjoint": [_i, _l, _vp, _vp, _pp, _vp],
    "ccl_grad_combine_adjoint": [_i, _i, _i, _i, _vp, _pp, _pp, _pp, _pp, _vp],
    "ccl_rot_combine_adjoint": [_i, _i, _i, _i, _vp, _pp, _pp, _pp, _pp, _pp, _vp],
    "ccl_modes_adjoint_accumulate": [_i, _i, _i, _i, _i, _pp, _pp, _pp, _pp, _vp],
    "ccl_add_batch": [_i, _i, _vp, _pp, _pp, _vp],
    "ccl_copy_batch": [_i, _vp, _pp, _pp, _vp],
    "ccl_deposit_postproc_adjoint": [_i, _i, _i, _pp, _i, _i, _vp, _vp],
    "ccl_warp_axis_adjoint": [_i, _i, _i, _pp, _i, _vp],
    "ccl_align_adjoint": [_i, _l, _i, _pp, _pp, _vp, _vp],
    "ccl_dens_profile_adjoint": [_i, _l, _vp, _vp, _vp, _vp, _vp, _vp, _u32, _vp, _vp],
}

_lib = None


def load(path=LIB_PATH):
    """Load the library (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"chimeracl_gb300: {path} is not built; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` "
            "(or `python chimeracl_gb300/build.py`) first")
    lib = C.CDLL(path)
    for name, argt in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = argt
        f.restype = C.c_int
    lib.ccl_version.restype = C.c_int
    lib.ccl_last_error.restype = C.c_char_p
    lib.ccl_launch_count.restype = C.c_ulonglong
    _lib = lib
    return lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("chimeracl_gb300 needs a CUDA device (there is no CPU path)")


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise CCLError(f"{name} failed ({rc}): {lib.ccl_last_error().decode()}")


def P(t, offset=0):
    """Device pointer of a CUDA tensor (+ offset in elements of its dtype)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("chimeracl_gb300 expects CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("chimeracl_gb300 expects contiguous tensors")
    return C.c_void_p(t.data_ptr() + offset * t.element_size())


def PP(tensors):
    """Host array of device pointers."""
    arr = (C.c_void_p * len(tensors))()
    for i, t in enumerate(tensors):
        if t is None:
            arr[i] = None
        elif isinstance(t, int):
            arr[i] = t
        else:
            if not t.is_cuda or not t.is_contiguous():
                raise ValueError("chimeracl_gb300 expects contiguous CUDA tensors")
            arr[i] = t.data_ptr()
    return C.cast(arr, _pp)


def longs(vals):
    """Host array of C longs."""
    return (C.c_long * len(vals))(*vals)


def ints(vals):
    """Host array of C ints."""
    return (C.c_int * len(vals))(*vals)


def launch_count():
    """Kernels launched by the library so far (all threads)."""
    return int(load().ccl_launch_count())


def stream():
    """The current CUDA stream of the current device, as a raw handle."""
    return C.c_void_p(torch._C._cuda_getCurrentRawStream(torch.cuda.current_device()))


def sort_workspace_bytes(np_, ncells):
    out = C.c_size_t(0)
    call("ccl_index_sort_workspace", np_, ncells, C.byref(out))
    return out.value
