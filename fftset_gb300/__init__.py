"""Python binding of the fftset C API on GB300 (libfftset_gb300.so).

Thin ctypes layer over the C ABI declared in include/fftset.h, mirroring the
reference's interface (fftset.h of templeblock/fftset): an FftSet owns plans
(`create_fft`), each plan runs forward / inverse / conv_get_kernel / conv on
buffers of 2*complex_bins floats. Buffers are torch CUDA tensors (used in
place, ordered on torch's current stream) or numpy arrays (host memory,
staged by the library). There is no CPU fallback: importing this module
fails if the CUDA library is missing, and every call goes to the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfftset_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
        "(there is no CPU fallback)")

_lib = C.CDLL(LIB_PATH)

FFTSET_OK, FFTSET_E_INVALID, FFTSET_E_NOMEM, FFTSET_E_CUDA, FFTSET_E_UNSUPPORTED = range(5)

_vp = C.c_void_p
_sz = C.c_size_t
_u = C.c_uint


def _decl(name, res, args):
    f = getattr(_lib, name)
    f.restype = res
    f.argtypes = args
    return f


class _FftsetStruct(C.Structure):
    _fields_ = [("impl", _vp), ("reserved", _vp * 7)]


_P = C.POINTER(_FftsetStruct)
_decl("fftset_init", C.c_int, [_P])
_decl("fftset_destroy", None, [_P])
_decl("fftset_create_fft", _vp, [_P, _vp, _u])
for _n in ("fftset_fft_forward", "fftset_fft_inverse"):
    _decl(_n, None, [_vp, _vp, _vp, _vp])
_decl("fftset_fft_conv_get_kernel", None, [_vp, _vp, _vp])
_decl("fftset_fft_conv", None, [_vp, _vp, _vp, _vp, _vp])
_decl("fftset_recommend_conv_length", _u, [_u, _u])
_decl("fftset_last_error", C.c_int, [_P])
_decl("fftset_clear_error", C.c_int, [_P])
_decl("fftset_cuda_error", C.c_int, [_P])
_decl("fftset_error_string", C.c_char_p, [C.c_int])
_decl("fftset_set_stream", C.c_int, [_P, _vp])
_decl("fftset_get_stream", _vp, [_P])
_decl("fftset_own_stream", _vp, [_P])
_decl("fftset_set_blocking", C.c_int, [_P, C.c_int])
_decl("fftset_set_kernel_layout", C.c_int, [_P, _u])
_decl("fftset_kernel_layout", C.c_int, [_vp, _u, _u, C.POINTER(C.c_int), C.POINTER(_u)])
_decl("fftset_fft_kernel_lanes", _u, [_vp])
_decl("fftset_fft_bins", _u, [_vp])
for _n in ("fftset_fft_forward_batch", "fftset_fft_inverse_batch", "fftset_fft_conv_get_kernel_batch"):
    _decl(_n, C.c_int, [_vp, _vp, _sz, _vp, _sz, _u])
_decl("fftset_fft_conv_batch", C.c_int, [_vp, _vp, _sz, _vp, _sz, _vp, _u])
_decl("fftset_fft_variants", C.c_int, [_vp])
_decl("fftset_fft_variant", C.c_int, [_vp, C.c_int])
_decl("fftset_fft_set_variant", C.c_int, [_vp, C.c_int, C.c_int])
_decl("fftset_fft_autotune", C.c_int, [_vp, C.c_int, _u, C.POINTER(C.c_float)])
_decl("fftset_tuning_save", C.c_int, [_P, C.c_char_p])
_decl("fftset_tuning_load", C.c_int, [_P, C.c_char_p])

OP_FORWARD, OP_INVERSE, OP_GET_KERNEL, OP_CONV, OP_CORR = range(5)

_decl("fftset_ragged_create", _vp, [_P, _vp, C.c_int, _u, C.POINTER(_u), C.POINTER(_sz), C.POINTER(_sz)])
_decl("fftset_ragged_execute", C.c_int, [_vp, _vp, _vp])
_decl("fftset_ragged_set_graph", C.c_int, [_vp, C.c_int])
_decl("fftset_ragged_bytes", C.c_double, [_vp])
_decl("fftset_ragged_persistent_items", _u, [_vp])
_decl("fftset_ragged_destroy", None, [_vp])
_decl("fftset_ragged_autotune", C.c_int, [_vp])
_decl("fftset_fft_conv_overlap_add", C.c_int, [_vp, _vp, _vp, _sz, _vp, _u, _u])
_decl("fftset_fft_conv_adjoint_batch", C.c_int, [_vp, _vp, _sz, _vp, _vp, _sz, _vp, _sz, _vp, _u])

MODULATION_COMPLEX = _vp.in_dll(_lib, "FFTSET_MODULATION_COMPLEX").value
MODULATION_FREQ_OFFSET_REAL = _vp.in_dll(_lib, "FFTSET_MODULATION_FREQ_OFFSET_REAL").value
COMPLEX, FREQ_OFFSET_REAL = 0, 1


def _mod_ptr(modulation):
    if modulation in (FREQ_OFFSET_REAL, "FREQ_OFFSET_REAL", MODULATION_FREQ_OFFSET_REAL):
        return MODULATION_FREQ_OFFSET_REAL
    if modulation in (COMPLEX, "COMPLEX", MODULATION_COMPLEX):
        return MODULATION_COMPLEX
    raise ValueError(f"unknown modulation {modulation!r}")


def library():
    """The loaded ctypes library (for tests that call the C ABI directly)."""
    return _lib


def recommend_conv_length(kernel_length: int, max_block_size: int) -> int:
    return int(_lib.fftset_recommend_conv_length(kernel_length, max_block_size))


def kernel_layout(modulation, complex_bins: int, simd_width: int = 4):
    """(re_offsets list, lanes): float offset of each bin's real part in a
    kernel buffer; the imaginary part follows `lanes` floats later. CPU only."""
    arr = (C.c_int * complex_bins)()
    lanes = _u(0)
    rc = _lib.fftset_kernel_layout(_mod_ptr(modulation), complex_bins, simd_width, arr, C.byref(lanes))
    if rc:
        raise ValueError(f"no kernel layout for {complex_bins} bins")
    return list(arr), int(lanes.value)


def error_string(code: int) -> str:
    return _lib.fftset_error_string(code).decode()


class FftsetError(RuntimeError):
    pass


def _ptr(x):
    """Raw address of a torch tensor or numpy array (no copies)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return x.ctypes.data
    if isinstance(x, int):
        return x
    raise TypeError(f"unsupported buffer type {type(x)}")


def _is_cuda(*xs):
    return any(hasattr(x, "is_cuda") and x.is_cuda for x in xs if x is not None)


class FftSet:
    """Owns a `struct fftset` (plans, twiddles, staging buffers)."""

    def __init__(self, kernel_layout_width: int = 4):
        self._s = _FftsetStruct()
        if _lib.fftset_init(C.byref(self._s)) != 0:
            raise FftsetError("fftset_init failed (no usable CUDA device?)")
        if kernel_layout_width != 4:
            self.set_kernel_layout(kernel_layout_width)
        self._plans = {}
        # ragged batches made from this fftset: fftset_destroy frees the
        # plans they use, so they are destroyed first
        self._ragged = weakref.WeakSet()

    @property
    def handle(self):
        return C.byref(self._s)

    def close(self):
        if self._s.impl:
            for r in list(getattr(self, "_ragged", ())):
                r.close()
            _lib.fftset_destroy(C.byref(self._s))
            self._plans.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_kernel_layout(self, simd_width: int):
        rc = _lib.fftset_set_kernel_layout(C.byref(self._s), simd_width)
        if rc:
            raise FftsetError(error_string(rc))

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream or an int cudaStream_t (0 = CUDA's
        legacy default stream)."""
        s = getattr(stream, "cuda_stream", stream)
        _lib.fftset_set_stream(C.byref(self._s), s if s else None)

    def own_stream(self):
        return _lib.fftset_own_stream(C.byref(self._s))

    def set_blocking(self, blocking: bool):
        _lib.fftset_set_blocking(C.byref(self._s), 1 if blocking else 0)

    def last_error(self) -> int:
        return _lib.fftset_last_error(C.byref(self._s))

    def clear_error(self) -> int:
        return _lib.fftset_clear_error(C.byref(self._s))

    def check(self):
        e = self.clear_error()
        if e:
            cu = _lib.fftset_cuda_error(C.byref(self._s))
            raise FftsetError(f"{error_string(e)} (cuda error {cu})")

    def save_tuning(self, path: str):
        """fftset_tuning_save: the chosen kernels and task schedules of every
        plan, for fftset_tuning_load in another process."""
        rc = _lib.fftset_tuning_save(C.byref(self._s), os.fsencode(path))
        if rc:
            self.clear_error()
            raise FftsetError(error_string(rc))

    def load_tuning(self, path: str):
        """fftset_tuning_load; raises FftsetError (UNSUPPORTED for a file from
        another device model, INVALID for a malformed one)."""
        rc = _lib.fftset_tuning_load(C.byref(self._s), os.fsencode(path))
        if rc:
            self.clear_error()
            raise FftsetError(error_string(rc))

    def create_fft(self, modulation, complex_bins: int):
        h = _lib.fftset_create_fft(C.byref(self._s), _mod_ptr(modulation), complex_bins)
        if not h:
            self.clear_error()
            return None
        return self._plans.setdefault(h, Fft(self, h, _mod_ptr(modulation) == MODULATION_COMPLEX))


class Fft:
    """One plan: a `const struct fftset_fft *`."""

    def __init__(self, owner: FftSet, handle: int, is_complex: bool = False):
        self.owner = owner
        self.handle = handle
        self.is_complex = is_complex
        self.bins = int(_lib.fftset_fft_bins(handle))
        self.kernel_lanes = int(_lib.fftset_fft_kernel_lanes(handle))

    @property
    def variants(self) -> int:
        return int(_lib.fftset_fft_variants(self.handle))

    def variant(self, op: int) -> int:
        return int(_lib.fftset_fft_variant(self.handle, op))

    def set_variant(self, op: int, variant: int):
        rc = _lib.fftset_fft_set_variant(self.handle, op, variant)
        if rc:
            raise FftsetError(error_string(rc))

    def autotune(self, op: int, count: int) -> float:
        """Time every kernel for `op` on `count` blocks; keep the fastest.
        Returns its time in ms."""
        import torch
        self.owner.set_stream(torch.cuda.current_stream())
        ms = C.c_float(0)
        rc = _lib.fftset_fft_autotune(self.handle, op, count, C.byref(ms))
        if rc:
            self.owner.check()
            raise FftsetError(error_string(rc))
        return float(ms.value)

    def _sync_stream(self, *bufs):
        if _is_cuda(*bufs):
            import torch
            self.owner.set_stream(torch.cuda.current_stream())

    def _done(self):
        self.owner.check()

    def forward(self, out, inp, work=None):
        self._sync_stream(out, inp)
        _lib.fftset_fft_forward(self.handle, _ptr(out), _ptr(inp), _ptr(work))
        self._done()
        return out

    def inverse(self, out, inp, work=None):
        self._sync_stream(out, inp)
        _lib.fftset_fft_inverse(self.handle, _ptr(out), _ptr(inp), _ptr(work))
        self._done()
        return out

    def conv_get_kernel(self, out, inp):
        self._sync_stream(out, inp)
        _lib.fftset_fft_conv_get_kernel(self.handle, _ptr(out), _ptr(inp))
        self._done()
        return out

    def conv(self, out, inp, kern, work=None):
        self._sync_stream(out, inp, kern)
        _lib.fftset_fft_conv(self.handle, _ptr(out), _ptr(inp), _ptr(kern), _ptr(work))
        self._done()
        return out

    # batched forms: buffers shaped [count, stride]
    def _batch(self, fn, out, inp, *extra):
        self._sync_stream(out, inp, *extra)
        count = int(inp.shape[0]) if len(inp.shape) > 1 else 1
        in_stride = int(inp.shape[-1])
        out_stride = int(out.shape[-1])
        args = [self.handle, _ptr(out), out_stride, _ptr(inp), in_stride]
        if extra:
            args.append(_ptr(extra[0]))
        rc = fn(*args, count)
        if rc:
            self.owner.check()
            raise FftsetError(error_string(rc))
        return out

    def forward_batch(self, out, inp):
        return self._batch(_lib.fftset_fft_forward_batch, out, inp)

    def inverse_batch(self, out, inp):
        return self._batch(_lib.fftset_fft_inverse_batch, out, inp)

    def conv_get_kernel_batch(self, out, inp):
        return self._batch(_lib.fftset_fft_conv_get_kernel_batch, out, inp)

    def conv_batch(self, out, inp, kern):
        return self._batch(_lib.fftset_fft_conv_batch, out, inp, kern)

    def conv_overlap_add(self, out, inp, kern, kernel_length: int, block_length: int = 0):
        """fftset_fft_conv_overlap_add: out (samples + kernel_length - 1
        samples) = complex_bins x the linear convolution of inp with the
        kernel whose spectrum is kern. Samples are floats (FREQ_OFFSET_REAL)
        or interleaved complex pairs (COMPLEX)."""
        self._sync_stream(out, inp, kern)
        n = int(inp.numel() if hasattr(inp, "numel") else inp.size)
        samples = n // 2 if self.is_complex else n
        rc = _lib.fftset_fft_conv_overlap_add(self.handle, _ptr(out), _ptr(inp), samples, _ptr(kern),
                                              kernel_length, block_length)
        if rc:
            self.owner.check()
            raise FftsetError(error_string(rc))
        return out

    def conv_adjoint_batch(self, grad_input, grad_taps, grad_out, inp, kern):
        """fftset_fft_conv_adjoint_batch: gradients of sum_b <grad_out_b, y_b>
        for y_b = conv(inp_b, kern) with respect to inp ([count, stride],
        may be None) and to the 2L taps that made kern (may be None)."""
        self._sync_stream(grad_out, inp, kern, grad_input, grad_taps)
        count = int(grad_out.shape[0]) if len(grad_out.shape) > 1 else 1
        go = int(grad_out.shape[-1])
        gi = int(grad_input.shape[-1]) if grad_input is not None else 0
        ins = int(inp.shape[-1]) if inp is not None else 0
        rc = _lib.fftset_fft_conv_adjoint_batch(self.handle, _ptr(grad_input), gi, _ptr(grad_taps), _ptr(grad_out),
                                                go, _ptr(inp), ins, _ptr(kern), count)
        if rc:
            self.owner.check()
            raise FftsetError(error_string(rc))
        return grad_input, grad_taps


class Ragged:
    """A ragged batch (fftset_ragged_*): item i has bins[i] complex bins,
    input at in_offsets[i] and output at out_offsets[i] floats from the base
    tensors given to execute()."""

    def __init__(self, owner: FftSet, modulation, op: int, bins, in_offsets, out_offsets):
        n = len(bins)
        self.owner = owner
        b = (_u * n)(*bins)
        io = (_sz * n)(*in_offsets)
        oo = (_sz * n)(*out_offsets)
        self.h = _lib.fftset_ragged_create(owner.handle, _mod_ptr(modulation), op, n, b, io, oo)
        if not self.h:
            owner.check()
            raise FftsetError("fftset_ragged_create failed")
        self.n = n
        owner._ragged.add(self)

    @property
    def bytes(self) -> float:
        return float(_lib.fftset_ragged_bytes(self.h))

    @property
    def persistent_items(self) -> int:
        return int(_lib.fftset_ragged_persistent_items(self.h))

    def set_graph(self, enable: bool):
        _lib.fftset_ragged_set_graph(self.h, 1 if enable else 0)

    def autotune(self):
        """fftset_ragged_autotune: per-size schedules by timing, then a
        rebuilt task list."""
        import torch
        self.owner.set_stream(torch.cuda.current_stream())
        rc = _lib.fftset_ragged_autotune(self.h)
        if rc:
            self.owner.check()
            raise FftsetError(error_string(rc))

    def execute(self, out, inp):
        import torch
        self.owner.set_stream(torch.cuda.current_stream())
        rc = _lib.fftset_ragged_execute(self.h, _ptr(out), _ptr(inp))
        if rc:
            self.owner.check()
            raise FftsetError(error_string(rc))
        return out

    def close(self):
        """fftset_ragged_destroy (before its fftset's destroy: FftSet.close
        calls this for every batch still open)."""
        if getattr(self, "h", None):
            if self.owner._s.impl:
                _lib.fftset_ragged_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
