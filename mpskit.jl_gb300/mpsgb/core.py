"""Device context and tensors (host side of libmpsgb).

`DeviceTensor` is the analogue of a TensorKit `TensorMap` whose storage lives in GB300
HBM: `from_numpy` / `numpy` exchange data in TensorKit's own layout (column-major,
legs in TensorMap order) and the library converts to its device layout.
"""
import ctypes

import numpy as np

from . import _lib as L

_CTX = {}

_KIND_NAMES = {
    "mps": L.GB_KIND_MPS, "bond": L.GB_KIND_BOND, "ac2": L.GB_KIND_AC2,
    "gl": L.GB_KIND_GL, "gr": L.GB_KIND_GR, "mpo": L.GB_KIND_MPO, "generic": L.GB_KIND_GENERIC,
}


class Context:
    """One device context (stream, solver handles, launch counter)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        L.check(L.lib().gb_ctx_create(device, 0, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def synchronize(self):
        L.check(L.lib().gb_ctx_synchronize(self.handle))

    def kernel_launches(self):
        v = ctypes.c_int64()
        L.check(L.lib().gb_ctx_kernel_launches(self.handle, ctypes.byref(v)))
        return v.value

    def set_precision(self, precision):
        code = L.PRECISIONS[precision]
        L.check(L.lib().gb_ctx_set_precision(self.handle, code))

    def set_gemm_schedule(self, schedule="grouped", tile_n=0):
        """Split-precision GEMM schedule: "grouped" (the default: operators with known U(1)
        sectors run one launch over their charge blocks; other GEMMs as "persistent"),
        "persistent" (tile skipping over the dense embedding), "persistent_dense" or "tile";
        tile_n in (0 = per shape, 128, 256).  Read when an operator is built."""
        code = {"persistent": L.GB_SCHED_PERSISTENT,
                "persistent_dense": L.GB_SCHED_PERSISTENT_DENSE,
                "tile": L.GB_SCHED_TILE,
                "grouped": L.GB_SCHED_GROUPED}[schedule]
        L.check(L.lib().gb_ctx_set_gemm_schedule(self.handle, code, int(tile_n)))

    def set_wait_bound(self, seconds=2.0):
        """Bound on every pipeline wait of the tensor-core kernels (gb_ctx_set_wait_bound)."""
        L.check(L.lib().gb_ctx_set_wait_bound(self.handle, float(seconds)))

    def set_counting(self, on=True):
        """Count the nonzero products of every split GEMM (block-sparse flop accounting)."""
        L.check(L.lib().gb_ctx_set_counting(self.handle, int(bool(on))))

    def read_work(self, reset=True):
        """-> dict(tile_flops, nonzero_flops) accumulated since the last reset."""
        t, z = ctypes.c_double(), ctypes.c_double()
        L.check(L.lib().gb_ctx_read_work(self.handle, ctypes.byref(t), ctypes.byref(z),
                                         int(bool(reset))))
        return {"tile_flops": t.value, "nonzero_flops": z.value}

    def set_svd_method(self, method):
        """'gesvd' (default), 'gesvdp' or 'gram' for gb_svd_trunc."""
        code = {"gesvd": 0, "gesvdp": 1, "gram": 2}[method]
        L.check(L.lib().gb_ctx_set_svd_method(self.handle, code))
        self._svd_method = method

    def set_gauge(self, eig="syevd", lanes=8):
        """Gauge-step options (gb_ctx_set_gauge): the Gram route's eigensolver ('syevd',
        'syevj' or 'syevd32') and the number of host-thread lanes for per-sector
        factorisations."""
        L.check(L.lib().gb_ctx_set_gauge(self.handle, {"syevd": 0, "syevj": 1, "syevd32": 2}[eig],
                                         int(lanes)))

    def set_option(self, name, value):
        """Implementation switches that leave results unchanged (gb_ctx_set_option):
        'staged_mix' (0 direct, 1 by density, 2 staged)."""
        L.check(L.lib().gb_ctx_set_option(self.handle, {"staged_mix": 0}[name], int(value)))

    def profile_begin(self):
        L.check(L.lib().gb_ctx_profile_begin(self.handle))

    def profile_end(self):
        """-> dict(gemm_ms, gemm_launches, gemm_flops, region_ms) of the traced region."""
        ms, fl, rms = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        L.check(L.lib().gb_ctx_profile_end(self.handle, ctypes.byref(ms), ctypes.byref(n),
                                           ctypes.byref(fl), ctypes.byref(rms)))
        out = {"gemm_ms": ms.value, "gemm_launches": n.value, "gemm_flops": fl.value,
               "region_ms": rms.value}
        for name, code in (("persistent", 0), ("grouped", 1)):
            kms, kfl, kn = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
            L.check(L.lib().gb_ctx_profile_kernel(self.handle, code, ctypes.byref(kms),
                                                  ctypes.byref(kn), ctypes.byref(kfl)))
            out[name] = {"ms": kms.value, "launches": kn.value, "flops": kfl.value}
        return out

    def trace_begin(self):
        """Start a launch trace of this context's stream (gb_ctx_trace_begin)."""
        L.check(L.lib().gb_ctx_trace_begin(self.handle))

    def trace_end(self):
        """-> (total_ms, [(site, ms, events)] sorted by ms): the traced span and the time
        charged to each issuing source site (kernel plus the idle gap before it)."""
        n, tot = ctypes.c_int64(), ctypes.c_double()
        L.check(L.lib().gb_ctx_trace_end(self.handle, ctypes.byref(n), ctypes.byref(tot)))
        out = []
        buf = ctypes.create_string_buffer(256)
        for i in range(n.value):
            ms, ev = ctypes.c_double(), ctypes.c_int64()
            L.check(L.lib().gb_ctx_trace_site(self.handle, i, buf, 256, ctypes.byref(ms),
                                              ctypes.byref(ev)))
            out.append((buf.value.decode(), ms.value, ev.value))
        out.sort(key=lambda t: -t[1])
        return tot.value, out

    def device_status(self):
        """Status word of the bounded device waits (0 = clean; GB_ERR_TIMEOUT after a wait
        ran out); cleared on read."""
        v = ctypes.c_int32()
        L.check(L.lib().gb_ctx_device_status(self.handle, ctypes.byref(v)))
        return v.value


def context(device=0):
    """Process-wide default context for `device`."""
    ctx = _CTX.get(device)
    if ctx is None:
        ctx = Context(device)
        _CTX[device] = ctx
    return ctx


def _dtype_code(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.float64:
        return L.GB_F64
    if dtype == np.complex128:
        return L.GB_C128
    raise TypeError(f"unsupported dtype {dtype}; use float64 or complex128")


class DeviceTensor:
    """A dense TensorMap block resident on the GPU.

    `charges` (optional) makes it a U(1)-symmetric tensor: one int32 array of charges per
    leg, in reference leg order, every virtual leg sorted by charge, entries outside the
    charge-conserving blocks exactly zero (see mpsgb.u1)."""

    __slots__ = ("ctx", "handle", "kind", "dtype", "dims", "charges", "__weakref__")

    def __init__(self, ctx, kind, dtype, dims, handle=None, charges=None):
        self.ctx = ctx
        self.charges = charges
        self.kind = _KIND_NAMES[kind] if isinstance(kind, str) else kind
        self.dtype = np.dtype(dtype)
        self.dims = tuple(int(x) for x in dims)
        if handle is None:
            arr = (ctypes.c_int64 * len(self.dims))(*self.dims)
            h = ctypes.c_void_p()
            L.check(L.lib().gb_tensor_create(ctx.handle, self.kind, _dtype_code(self.dtype),
                                             len(self.dims), arr, ctypes.byref(h)))
            handle = h
        self.handle = handle

    @staticmethod
    def wrap(ctx, handle):
        """Adopt a tensor created by the library (e.g. an SVD output)."""
        kind = ctypes.c_int()
        dt = ctypes.c_int()
        nd = ctypes.c_int()
        dims = (ctypes.c_int64 * 6)()
        L.check(L.lib().gb_tensor_shape(handle, ctypes.byref(kind), ctypes.byref(dt),
                                        ctypes.byref(nd), dims))
        dtype = np.float64 if dt.value == L.GB_F64 else np.complex128
        return DeviceTensor(ctx, kind.value, dtype, [dims[i] for i in range(nd.value)], handle)

    @staticmethod
    def from_numpy(ctx, kind, arr, dtype=None):
        arr = np.asarray(arr)
        dtype = np.dtype(dtype or arr.dtype)
        if dtype.kind == "f" and arr.dtype.kind == "c":
            raise TypeError("cannot store complex data in a real tensor")
        t = DeviceTensor(ctx, kind, dtype, arr.shape)
        t.upload(arr)
        return t

    def upload(self, arr):
        a = np.asfortranarray(np.asarray(arr, dtype=self.dtype))
        if a.shape != self.dims:
            raise ValueError(f"shape {a.shape} does not match tensor {self.dims}")
        L.check(L.lib().gb_tensor_upload(self.handle, a.ctypes.data_as(ctypes.c_void_p), a.nbytes))

    def numpy(self):
        out = np.empty(self.dims, dtype=self.dtype, order="F")
        L.check(L.lib().gb_tensor_download(self.handle, out.ctypes.data_as(ctypes.c_void_p),
                                           out.nbytes))
        return out

    def reshape_(self, kind, dims, charges=None):
        """Relabel kind and shape in place over the same device storage (gb_tensor_reshape:
        the new shape reads the storage in its own device order)."""
        kind = _KIND_NAMES[kind] if isinstance(kind, str) else kind
        arr = (ctypes.c_int64 * len(dims))(*[int(x) for x in dims])
        L.check(L.lib().gb_tensor_reshape(self.handle, kind, len(dims), arr))
        self.kind, self.dims, self.charges = kind, tuple(int(x) for x in dims), charges
        return self

    # ------------------------------------------------ VectorInterface-style operations
    def similar(self):
        return DeviceTensor(self.ctx, self.kind, self.dtype, self.dims, charges=self.charges)

    def copy(self):
        t = self.similar()
        L.check(L.lib().gb_tensor_copy(t.handle, self.handle))
        return t

    def scale_(self, a):
        a = complex(a)
        L.check(L.lib().gb_tensor_scale(self.handle, a.real, a.imag))
        return self

    def axpy_(self, a, x):
        a = complex(a)
        L.check(L.lib().gb_tensor_axpy(self.handle, a.real, a.imag, x.handle))
        return self

    def dot(self, other):
        re = ctypes.c_double()
        im = ctypes.c_double()
        L.check(L.lib().gb_tensor_dot(self.handle, other.handle, ctypes.byref(re), ctypes.byref(im)))
        return complex(re.value, im.value) if self.dtype.kind == "c" else re.value

    def norm(self):
        v = ctypes.c_double()
        L.check(L.lib().gb_tensor_norm(self.handle, ctypes.byref(v)))
        return v.value

    def normalize_(self):
        return self.scale_(1.0 / self.norm())

    @property
    def size(self):
        return int(np.prod(self.dims))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and L._lib is not None:
            try:
                L.lib().gb_tensor_free(h)
            except Exception:
                pass
            self.handle = None

    def __repr__(self):
        return f"DeviceTensor(kind={self.kind}, dtype={self.dtype}, dims={self.dims})"


class PackedTensor:
    """A tile-packed copy of a block-sparse device tensor (gb_tensor_pack): only the 64 x 64
    tiles that hold a nonzero stay in HBM; unpack() rebuilds the dense tensor exactly."""

    __slots__ = ("ctx", "handle", "kind", "dtype", "dims", "charges", "__weakref__")

    def __init__(self, t):
        self.ctx, self.kind, self.dtype, self.dims, self.charges = (t.ctx, t.kind, t.dtype,
                                                                     t.dims, t.charges)
        h = ctypes.c_void_p()
        L.check(L.lib().gb_tensor_pack(t.ctx.handle, t.handle, ctypes.byref(h)))
        self.handle = h

    def unpack(self):
        t = DeviceTensor(self.ctx, self.kind, self.dtype, self.dims, charges=self.charges)
        L.check(L.lib().gb_packed_unpack(self.ctx.handle, self.handle, t.handle))
        return t

    def info(self):
        """(tiles kept, tiles total, bytes held)."""
        k, n, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_size_t()
        L.check(L.lib().gb_packed_info(self.handle, ctypes.byref(k), ctypes.byref(n),
                                       ctypes.byref(b)))
        return k.value, n.value, b.value

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and L._lib is not None:
            try:
                L.lib().gb_packed_free(h)
            except Exception:
                pass
            self.handle = None
