"""Generic methods and the device context (the CUDA counterpart of
chimeraCL/methods/generic_methods_cl.py).

``GenericMethodsCU`` keeps the reference mixin's method names and argument
meaning; ``DataDev`` values are ``torch.Tensor`` on the CUDA device instead of
``pyopencl.array.Array``, and the compute calls go to the C ABI of
``libchimeracl_gb300.so``.
"""
import numpy as np
import torch

from .. import _lib
from .._lib import CCL_F32, CCL_F64, P, PP, call, ints, longs, stream

_NP2TORCH = {
    np.dtype(np.float64): torch.float64,
    np.dtype(np.float32): torch.float32,
    np.dtype(np.complex128): torch.complex128,
    np.dtype(np.complex64): torch.complex64,
    # 32-bit unsigned device integers (keys, offsets, counts) are stored in
    # int32 tensors: same bits, and every value used stays below 2**31.
    np.dtype(np.uint32): torch.int32,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.uint8): torch.uint8,
    np.dtype(np.int8): torch.int8,
    np.dtype(np.bool_): torch.bool,
}


def torch_dtype(dtype):
    if isinstance(dtype, torch.dtype):
        return dtype
    return _NP2TORCH[np.dtype(dtype)]


class LazyScalar:
    """A device scalar read back only when the host asks for its value
    (as an int, or through ``cast``)."""

    def __init__(self, tensor, comm=None, cast=int):
        self.tensor = tensor
        self.comm = comm
        self.cast = cast

    def resolve(self):
        if self.comm is not None:
            self.comm.d2h_bytes += self.tensor.element_size()
        return self.cast(self.tensor.item())


class ArgsDict(dict):
    """``Args`` container: a plain dict, except that values held as
    ``LazyScalar`` (the in-window particle count after a sort, the injector's
    right limit after a window shift) are read from the device the first
    time they are looked up."""

    def __getitem__(self, k):
        v = dict.__getitem__(self, k)
        if isinstance(v, LazyScalar):
            v = v.resolve()
            dict.__setitem__(self, k, v)
        return v

    def get(self, k, default=None):
        return self[k] if k in self else default


class Communicator:
    """Device context (the reference's ``Communicator``,
    generic_methods_cl.py:152-195).

    ``precision='fp64'`` is the plain FP64 drop-in (double particles,
    complex128 fields).  ``precision='fp32'`` runs the same kernels in single
    precision.  ``precision='mixed'`` is FP32 with the radial Hankel and
    derivative GEMMs as BF16x3 split-precision products on the tensor cores
    (FP32 accumulation).  ``seed`` seeds the host generator of the plasma injector's
    random draws.  ``compensated_positions=True`` (FP32 forms) holds each
    coordinate as the sum of its FP32 value and an FP32 low part (``x_lo``,
    ``y_lo``, ``z_lo`` in ``DataDev``): the injector stores the rounding
    residual of its double-precision positions there, the push adds its
    displacements by a two-sum, and the deposits and gather take the shape
    fractions from the full coordinate (a 2^-24 fraction of a cell wherever
    the particle is); the cell sort reads the FP32 value.  It costs 12 bytes
    per particle in each deposit and the gather and 24 per push, and is off
    by default.  The FP64 form ignores it.  Keyword arguments of the reference's OpenCL context choice
    (``answers``, ``interactive``) are accepted and ignored."""

    def __init__(self, precision="fp64", device=0, seed=0, verbose=False,
                 compensated_positions=False, **ctx_kw_args):
        _lib.require_cuda()
        _lib.load()
        if precision not in ("fp64", "fp32", "mixed"):
            raise ValueError(f"precision must be 'fp64', 'fp32' or 'mixed', not {precision!r}")
        self.device = torch.device("cuda", device)
        torch.cuda.set_device(self.device)
        self.ctx = self.device
        self.queue = torch.cuda.current_stream(self.device)
        self.thr = self.queue
        self.dev_type = "GPU"
        self.dev_name = torch.cuda.get_device_name(self.device)
        self.plat_name = "NVIDIA"
        self.ocl_version = None
        self.fft_method = "ccl"
        self.dot_method = "ccl"
        self.precision = precision
        self.seed = seed
        self.real = torch.float64 if precision == "fp64" else torch.float32
        self.cplx = torch.complex128 if precision == "fp64" else torch.complex64
        self.ccl = CCL_F64 if precision == "fp64" else CCL_F32
        self.dht_impl = "bf16x3" if precision == "mixed" else "simt"
        self.compensated = bool(compensated_positions) and precision != "fp64"
        # host<->device traffic issued by the methods (injector draws,
        # profile knots, lazy scalar reads), for end-to-end accounting
        self.h2d_bytes = 0
        self.d2h_bytes = 0
        if verbose:
            print(f"chimeracl_gb300: {self.dev_name} ({precision})")


class GenericMethodsCU:
    """generic_methods_cl.py:19-150 on the CUDA library."""

    def init_generic_methods(self):
        self.set_global_working_group_size()

    def set_global_working_group_size(self):
        self.WGS = 256
        self.block_def_str = "#define BLOCK_SIZE {:d}\n".format(self.WGS)

    def get_wgs(self, Nelem):
        if Nelem <= self.WGS:
            return Nelem, Nelem
        WGS_tot = int(np.ceil(1.0 * Nelem / self.WGS)) * self.WGS
        return self.WGS, WGS_tot

    def import_comm(self, comm):
        self.comm = comm
        self.queue = comm.queue
        self.ctx = comm.ctx
        self.thr = comm.thr
        self.dev_type = comm.dev_type
        self.plat_name = comm.plat_name

    # ------------------------------------------------------------------
    @property
    def _dt(self):
        return self.comm.ccl

    def send_args_to_dev(self):
        """Mirror every int / float / ndarray of ``Args`` on the device
        (generic_methods_cl.py:56-76): ints as 1-element int64 tensors,
        floats as float64, arrays with their own dtype; keys listed in
        ``dont_send`` are skipped, keys in ``dont_keep`` leave ``Args``."""
        for arg in list(self.Args.keys()):
            if arg in self.Args.get("dont_send", []):
                continue
            v = dict.__getitem__(self.Args, arg)
            if type(v) is int:
                self.DataDev[arg] = torch.tensor([v], dtype=torch.int64, device=self.comm.device)
            elif type(v) is float:
                self.DataDev[arg] = torch.tensor([v], dtype=torch.float64, device=self.comm.device)
            elif type(v) is np.ndarray:
                self.DataDev[arg] = self.dev_arr(v, dtype=v.dtype)
            else:
                continue
            if arg in self.Args.get("dont_keep", []):
                self.Args.pop(arg)

    def dev_arr(self, val=None, shape=(1,), dtype=np.double, allocator=None):
        """A device tensor: a copy of an ndarray ``val``, zeros for
        ``val == 0``, else uninitialised (then filled with ``val`` if given)."""
        dev = self.comm.device
        if isinstance(val, np.ndarray):
            a = np.ascontiguousarray(val)
            if a.dtype == np.uint32:
                a = a.astype(np.int32)
            self.comm.h2d_bytes += a.nbytes
            h = torch.from_numpy(a)
            if torch.device(dev).type != "cuda":
                return h.to(dev)
            # through pinned memory: a copy from pageable memory would wait
            # for everything queued on the stream (the injector uploads its
            # grid while the device is still running the steps queued ahead)
            return h.pin_memory().to(dev, non_blocking=True)
        td = torch_dtype(dtype)
        if isinstance(shape, int):
            shape = (shape,)
        if val is not None and np.isscalar(val) and val == 0:
            return torch.zeros(shape, dtype=td, device=dev)
        arr = torch.empty(shape, dtype=td, device=dev)
        if val is not None:
            self.set_to(arr, val)
        return arr

    def _ccl_of(self, t):
        if t.dtype in (torch.float64, torch.complex128):
            return CCL_F64
        if t.dtype in (torch.float32, torch.complex64):
            return CCL_F32
        return None

    def set_to(self, arr, val):
        dt = self._ccl_of(arr)
        if dt is None:
            arr.fill_(val)
            return
        c = complex(val)
        call("ccl_set", dt, int(arr.is_complex()), arr.numel(), P(arr), c.real, c.imag, stream())

    def set_many(self, arrs, val):
        """set_to on several arrays of one dtype in one launch."""
        dt = self._ccl_of(arrs[0])
        if dt is None or len(arrs) > 32:
            for a in arrs:
                self.set_to(a, val)
            return
        c = complex(val)
        call("ccl_set_batch", dt, len(arrs), ints([int(a.is_complex()) for a in arrs]),
             longs([a.numel() for a in arrs]), PP(arrs), c.real, c.imag, stream())

    def cast_array_c2d(self, arr_in, arr_out):
        call("ccl_cast_c2d", self._ccl_of(arr_in), arr_in.numel(), P(arr_in), P(arr_out), stream())

    def append_c2c(self, arr_base, arr_add):
        call("ccl_append_c2c", self._ccl_of(arr_base), arr_base.numel(), P(arr_base), P(arr_add),
             stream())

    def mult_elementwise(self, x, z):
        call("ccl_mult_elementwise", self._ccl_of(z), x.numel(), P(x), P(z), stream())

    def axpbyz(self, a, x, b, y, z):
        a, b = complex(a), complex(b)
        call("ccl_axpbyz", self._ccl_of(z), x.numel(), a.real, a.imag, P(x), b.real, b.imag, P(y),
             P(z), stream())

    def zpaxz(self, z, a, x):
        a = complex(a)
        call("ccl_zpaxz", self._ccl_of(z), x.numel(), P(z), a.real, a.imag, P(x), stream())

    def ab_dot_x(self, a, b, x, z):
        a = complex(a)
        nx = b.numel()
        call("ccl_ab_dot_x", self._ccl_of(z), x.numel() // nx, nx, a.real, a.imag, P(b), P(x),
             P(z), stream())
