"""ctypes binding of ``libcov3d_gb300.so`` (declared in ``include/cov3d_gb300.h``).

The library is built in-tree by ``build.py``.  There is no fallback: if the shared library
is missing or fails to load, every operator raises ``RuntimeError`` with the reason.
"""

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcov3d_gb300.so")

# status codes (cov3d_status)
OK, EINVAL, ENOMEM, ECUDA, ECUFFT, ENONFINITE, EMAXITER, ESTATE = range(8)
# kernels (cov3d_kernel)
KERNEL_ES, KERNEL_LINEAR, KERNEL_NEAREST = 0, 1, 2
# grid orders
GRID_CENTERED, GRID_FFT_NATIVE = 0, 1
# epilogue flags
APPLY_NYQUIST, APPLY_CTF, APPLY_CTF_PARAMS = 1, 2, 4
# CTF parameters per image (pixel size, defocus u, v, astigmatism angle, kV, Cs, amplitude contrast,
# phase shift)
CTF_NPARAMS = 8
# cov3d_plan_reserve flags
RESERVE_POINTS, RESERVE_GRAM_BF16, RESERVE_LS_REG = 1, 2, 4

c_int, c_int64, c_double, c_float, c_void_p = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_float, ctypes.c_void_p


class Opts(ctypes.Structure):
    _fields_ = [("kernel", c_int), ("upsample", c_int), ("width", c_int), ("beta", c_double),
                ("compensated", c_int), ("bin_size", c_int), ("stream", c_void_p)]


class GridLayout(ctypes.Structure):
    _fields_ = [("order", c_int), ("cell_stride", c_int64), ("chan_stride", c_int64)]


class CostArgs(ctypes.Structure):
    _fields_ = [("objective", c_int), ("rank", c_int), ("d_vectors", c_void_p), ("d_log_sqrt", c_void_p),
                ("d_images", c_void_p), ("d_ctf", c_void_p), ("noise_var", c_double), ("reg_scale", c_double),
                ("d_fourier_reg", c_void_p), ("use_grid_correction", c_int), ("d_cost", c_void_p),
                ("gram_bf16", c_int), ("ctf_params", c_int), ("fourier_reg_per_channel", c_int)]


_SIGNATURES = {
    "cov3d_abi_version": (c_int, []),
    "cov3d_last_error": (c_int, [ctypes.c_char_p, c_int]),
    "cov3d_status_string": (ctypes.c_char_p, [c_int]),
    "cov3d_plan_create": (c_int, [c_int, c_int, c_double, ctypes.POINTER(Opts), ctypes.POINTER(c_void_p)]),
    "cov3d_plan_destroy": (c_int, [c_void_p]),
    "cov3d_plan_reserve": (c_int, [c_void_p, c_int64, c_int, c_int, c_int]),
    "cov3d_plan_set_stream": (c_int, [c_void_p, c_void_p]),
    "cov3d_plan_info": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_double)]),
    "cov3d_setpts": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_int64, c_int64, c_int]),
    "cov3d_setrot": (c_int, [c_void_p, c_void_p, c_int64, c_int]),
    "cov3d_interp": (c_int, [c_void_p, c_void_p, ctypes.POINTER(GridLayout), c_int, c_void_p, c_int64, c_int64,
                             c_void_p, c_int, c_float]),
    "cov3d_spread": (c_int, [c_void_p, c_void_p, c_int64, c_int64, c_int, c_void_p, c_int, c_float, c_void_p,
                             ctypes.POINTER(GridLayout), c_int]),
    "cov3d_spread_unaggregated": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int, c_float, c_void_p]),
    "cov3d_execute_type2": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "cov3d_execute_type1": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "cov3d_fine_grid": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "cov3d_project": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int64, c_int64, c_void_p, c_int,
                              c_float]),
    "cov3d_backproject": (c_int, [c_void_p, c_void_p, c_int64, c_int64, c_int, c_void_p, c_int, c_float, c_void_p]),
    "cov3d_grid_correction": (c_int, [c_void_p, c_void_p]),
    "cov3d_ctf_images": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "cov3d_covar_cost_grad": (c_int, [c_void_p, ctypes.POINTER(CostArgs), ctypes.POINTER(c_double), c_void_p,
                                      c_void_p, c_void_p]),
    "cov3d_launch_count": (ctypes.c_longlong, []),
    "cov3d_phase_name": (ctypes.c_char_p, [c_int]),
    "cov3d_plan_timing": (c_int, [c_void_p, c_int]),
    "cov3d_plan_timing_read": (c_int, [c_void_p, ctypes.POINTER(c_double), ctypes.POINTER(c_int), c_int]),
    "cov3d_gram": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_int64, c_int64, c_void_p, c_void_p,
                           c_void_p, c_void_p]),
    "cov3d_cost_solve": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p, c_double,
                                 c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "cov3d_latent_map_noalloc": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_int64, c_int64,
                                         c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_void_p]),
    "cov3d_wpass": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_int64, c_int64, c_void_p, c_void_p,
                            c_void_p, c_void_p, c_int64, c_int64, c_int64]),
    "cov3d_gram_bf16": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_int64, c_int64, c_void_p,
                                c_void_p, c_void_p, c_void_p]),
    "cov3d_mean_accumulate": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]),
    "cov3d_regularize_lhs": (c_int, [c_void_p, c_void_p, c_void_p]),
    "cov3d_mean_init": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "cov3d_circulant_symbol": (c_int, [c_void_p, c_void_p, c_void_p]),
    "cov3d_cg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_double, c_int, c_int, c_void_p,
                               ctypes.POINTER(c_int), ctypes.POINTER(c_double), c_void_p]),
    "cov3d_conv3d_forward": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int,
                                     c_int, c_int, c_void_p]),
    "cov3d_conv3d_backward_data": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int,
                                           c_int, c_void_p, c_void_p]),
    "cov3d_conv3d_backward_weight": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int,
                                             c_int, c_void_p, c_void_p]),
    "cov3d_relu_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    "cov3d_avgpool2": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_int, c_int, c_int, c_void_p]),
    "cov3d_upsample2": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_int, c_int, c_int, c_void_p]),
    "cov3d_resample3d": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols():
    """Names of the entry points this binding expects (one per declaration in the header)."""
    return sorted(_SIGNATURES)


def load(path=LIB_PATH):
    """Load the shared library (once) and attach prototypes.  Raises RuntimeError when absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: the GB300 kernels are not built (run `python -c \"import __graft_entry__ as g; "
                "g.build()\"` or `python 3dcovarestimation_gb300/build.py`); there is no CPU fallback")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.cov3d_abi_version() != 1:
            raise RuntimeError("libcov3d_gb300.so ABI version mismatch")
        _lib = lib
        return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(512)
    lib.cov3d_last_error(buf, 512)
    return buf.value.decode(errors="replace")


class Cov3dError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def check(status):
    """Map a cov3d_status to the exception type the reference raises for the same condition."""
    if status == OK:
        return
    msg = f"cov3d: {load().cov3d_status_string(status).decode()}: {last_error()}"
    if status == EINVAL:
        raise ValueError(msg)
    if status == ENOMEM:
        raise torch.cuda.OutOfMemoryError(msg)
    if status == ENONFINITE:
        raise FloatingPointError(msg)
    raise Cov3dError(status, msg)


def call(name, *args):
    check(getattr(load(), name)(*args))


def ptr(t):
    """Device pointer of a CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("cov3d operators take CUDA tensors; got a tensor on " + str(t.device))
    return c_void_p(t.data_ptr())


NUM_PHASES = 11


def launch_count():
    """Kernels launched by libcov3d_gb300.so since it was loaded."""
    return int(load().cov3d_launch_count())


def phase_names():
    lib = load()
    return [lib.cov3d_phase_name(i).decode() for i in range(NUM_PHASES)]


def stream_ptr(device=None):
    return c_void_p(torch.cuda.current_stream(device).cuda_stream)
