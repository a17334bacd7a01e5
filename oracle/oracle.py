"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

Checkers for fftset's transform / fast-convolution path. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.

Three checkers live here:

* FP64 mathematical oracle (numpy), the definitions the reference documents
  and tests:
    FREQ_OFFSET_REAL forward  X[k] = sum_n x[n] e^{-j 2 pi n (k+1/2) / N},
                              N = 2L reals -> L bins        (fftset.h:62-73,
                              app_fftset_test/fftset_test.c:110-131)
    inverse                   unnormalised, inverse(forward(x)) = L x
                              (fftset_test.c:142-144, :300-302)
    FREQ_OFFSET_REAL conv     L * negacyclic convolution of length 2L
                              (follows from the half-bin offset; the
                              non-wrapping part is pinned by
                              fftset_test.c:158-222)
    COMPLEX                   plain DFT / unnormalised IDFT / L * cyclic conv
* The C restatement `liboracle.so` (oracle/fftset_oracle.c): the reference's
  own planner, kernel-buffer layout and FP32 algorithm.
* The unmodified reference compiled here against the cop stand-in
  (oracle/_ref/libfftset_ref_vw{1,4,8}.so), available only where the
  reference sources exist; used to generate tests/golden fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MOD_COMPLEX = 0
MOD_FREQ_OFFSET_REAL = 1

_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint)


# --------------------------------------------------------------------------
# FP64 oracle
def _modulation(L: int) -> np.ndarray:
    i = np.arange(L, dtype=np.float64)
    return np.exp(-1j * np.pi * i / (2.0 * L))


def pack_freqoff(x: np.ndarray) -> np.ndarray:
    """c[i] = conj(x[i] + j x[L+i]) e^{-j pi i / (2L)}, the sequence whose
    length-L DFT W gives X[2m] = W[m], X[2m+1] = conj W[L-1-m]
    (src/fftset_mod_freqoffsetreal.c:947-971)."""
    x = np.asarray(x, dtype=np.float64)
    L = x.shape[-1] // 2
    z = x[..., :L] + 1j * x[..., L:]
    return np.conj(z) * _modulation(L)


def split_index(L: int):
    """For output bin m: (index into W, whether conjugated)."""
    m = np.arange(L)
    k = np.where(m % 2 == 0, m // 2, L - 1 - (m - 1) // 2)
    return k, (m % 2 == 1)


def freqoff_forward64(x: np.ndarray) -> np.ndarray:
    """Returns interleaved float64 array [..., 2L]."""
    x = np.asarray(x, dtype=np.float64)
    L = x.shape[-1] // 2
    W = np.fft.fft(pack_freqoff(x), axis=-1)
    k, cj = split_index(L)
    X = W[..., k]
    X = np.where(cj, np.conj(X), X)
    out = np.empty(x.shape[:-1] + (2 * L,), np.float64)
    out[..., 0::2] = X.real
    out[..., 1::2] = X.imag
    return out


def freqoff_direct64(x: np.ndarray) -> np.ndarray:
    """Direct O(N^2) sum of the documented definition (small N only)."""
    x = np.asarray(x, dtype=np.float64)
    N = x.shape[-1]
    L = N // 2
    n = np.arange(N)[:, None]
    k = np.arange(L)[None, :]
    E = np.exp(-2j * np.pi * n * (k + 0.5) / N)
    X = x @ E
    out = np.empty(x.shape[:-1] + (2 * L,), np.float64)
    out[..., 0::2] = X.real
    out[..., 1::2] = X.imag
    return out


def freqoff_inverse64(Xi: np.ndarray) -> np.ndarray:
    """Unnormalised inverse: y[n] = Re sum_k X[k] e^{+j 2 pi n (k+1/2)/N}
    written through W: L z = conj(IDFT_unnorm(W) e^{j pi i/(2L)})."""
    Xi = np.asarray(Xi, dtype=np.float64)
    L = Xi.shape[-1] // 2
    X = Xi[..., 0::2] + 1j * Xi[..., 1::2]
    k, cj = split_index(L)
    W = np.empty_like(X)
    W[..., k] = np.where(cj, np.conj(X), X)
    d = np.fft.ifft(W, axis=-1) * L
    z = np.conj(d * np.conj(_modulation(L)))
    return np.concatenate([z.real, z.imag], axis=-1)


def negacyclic_conv64(x: np.ndarray, h: np.ndarray) -> np.ndarray:
    """y[n] = sum_{m<=n} x[m]h[n-m] - sum_{m>n} x[m]h[n-m+N] via the
    half-bin-offset transform, returned scaled by L like fftset_fft_conv."""
    x = np.asarray(x, dtype=np.float64)
    h = np.asarray(h, dtype=np.float64)
    N = x.shape[-1]
    L = N // 2
    n = np.arange(N)
    tw = np.exp(-1j * np.pi * n / N)
    y = np.fft.ifft(np.fft.fft(x * tw, axis=-1) * np.fft.fft(h * tw, axis=-1), axis=-1) * np.conj(tw)
    return L * y.real


def negacyclic_direct64(x: np.ndarray, h: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    h = np.asarray(h, dtype=np.float64)
    N = x.shape[-1]
    L = N // 2
    y = np.zeros(N)
    for m in range(N):
        for j in range(N):
            t = m + j
            if t < N:
                y[t] += x[m] * h[j]
            else:
                y[t - N] -= x[m] * h[j]
    return L * y


def complex_forward64(xi: np.ndarray) -> np.ndarray:
    xi = np.asarray(xi, dtype=np.float64)
    X = np.fft.fft(xi[..., 0::2] + 1j * xi[..., 1::2], axis=-1)
    out = np.empty(xi.shape, np.float64)
    out[..., 0::2] = X.real
    out[..., 1::2] = X.imag
    return out


def complex_inverse64(Xi: np.ndarray) -> np.ndarray:
    Xi = np.asarray(Xi, dtype=np.float64)
    L = Xi.shape[-1] // 2
    x = np.fft.ifft(Xi[..., 0::2] + 1j * Xi[..., 1::2], axis=-1) * L
    out = np.empty(Xi.shape, np.float64)
    out[..., 0::2] = x.real
    out[..., 1::2] = x.imag
    return out


def complex_conv64(xi: np.ndarray, hi: np.ndarray) -> np.ndarray:
    xi = np.asarray(xi, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    L = xi.shape[-1] // 2
    x = xi[..., 0::2] + 1j * xi[..., 1::2]
    h = hi[..., 0::2] + 1j * hi[..., 1::2]
    y = np.fft.ifft(np.fft.fft(x, axis=-1) * np.fft.fft(h, axis=-1), axis=-1) * L
    out = np.empty(xi.shape, np.float64)
    out[..., 0::2] = y.real
    out[..., 1::2] = y.imag
    return out


def spectrum64(modulation: int, x: np.ndarray) -> np.ndarray:
    """Natural-order length-L DFT W that fftset_fft_conv_get_kernel
    permutes into the kernel buffer (complex128)."""
    x = np.asarray(x, dtype=np.float64)
    if modulation == MOD_FREQ_OFFSET_REAL:
        return np.fft.fft(pack_freqoff(x), axis=-1)
    return np.fft.fft(x[..., 0::2] + 1j * x[..., 1::2], axis=-1)


def forward64(modulation, x):
    return freqoff_forward64(x) if modulation == MOD_FREQ_OFFSET_REAL else complex_forward64(x)


def inverse64(modulation, X):
    return freqoff_inverse64(X) if modulation == MOD_FREQ_OFFSET_REAL else complex_inverse64(X)


def conv64(modulation, x, h):
    return negacyclic_conv64(x, h) if modulation == MOD_FREQ_OFFSET_REAL else complex_conv64(x, h)


def negacyclic_reverse(h: np.ndarray) -> np.ndarray:
    """h'[0] = h[0], h'[k] = -h[N-k]: the negacyclic time reversal, whose
    half-bin-offset spectrum is conj(H). Convolving with h' correlates with
    h, which is how the gradient of a FREQ_OFFSET_REAL convolution is built
    from the reference's own convolution (src/fftset_vec.c:1161-1220)."""
    h = np.asarray(h)
    return np.concatenate([h[..., :1], -h[..., :0:-1]], axis=-1)


def conj_reverse_complex(hi: np.ndarray) -> np.ndarray:
    """h*[k] = conj(h[-k mod L]) for interleaved complex h (spectrum conj(H)):
    the COMPLEX counterpart of negacyclic_reverse."""
    hi = np.asarray(hi)
    h = hi[..., 0::2] + 1j * hi[..., 1::2]
    r = np.conj(np.concatenate([h[..., :1], h[..., :0:-1]], axis=-1))
    out = np.empty(hi.shape, np.float64)
    out[..., 0::2] = r.real
    out[..., 1::2] = r.imag
    return out


def reverse(modulation, h):
    return negacyclic_reverse(h) if modulation == MOD_FREQ_OFFSET_REAL else conj_reverse_complex(h)


def conv_adjoint64(modulation, x, h, g):
    """FP64 adjoint of the batched convolution y_b = conv64(x_b, h) for
    upstream gradients g_b: (dx, dh) with dx_b = conv64(g_b, reverse(h)) and
    dh = sum_b conv64(g_b, reverse(x_b)); for FREQ_OFFSET_REAL the gradients
    of the loss sum_b <g_b, y_b>."""
    x = np.atleast_2d(np.asarray(x, np.float64))
    g = np.atleast_2d(np.asarray(g, np.float64))
    dx = conv64(modulation, g, reverse(modulation, np.asarray(h, np.float64))[None, :])
    dh = conv64(modulation, g, reverse(modulation, x)).sum(axis=0)
    return dx, dh


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def tolerance(N: int) -> float:
    """relL2 bound 2e-6 * log2(N), N = transform length in reals (FREQ_OFFSET
    _REAL: 2L; COMPLEX: L complex points)."""
    return 2e-6 * max(1.0, float(np.log2(max(N, 2))))


def valid_size(L: int) -> bool:
    """2^a 3^b 5^{0,1}, L >= 2 (README.md:3; the planner can place a radix-5
    pass only last, src/fftset_vec.c:949,957,966)."""
    if L < 2:
        return False
    n = L
    for p in (2, 3):
        while n % p == 0:
            n //= p
    if n % 5 == 0:
        n //= 5
    return n == 1


# --------------------------------------------------------------------------
# C restatement
_port = None


def build_port() -> str:
    path = os.path.join(HERE, "_build", "liboracle.so")
    src = os.path.join(HERE, "fftset_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return path


def port():
    global _port
    if _port is None:
        lib = C.CDLL(build_port())
        lib.oracle_plan_chain.restype = C.c_uint
        lib.oracle_plan_chain.argtypes = [C.c_uint, C.c_uint, _UP]
        lib.oracle_lane_width.restype = C.c_uint
        lib.oracle_lane_width.argtypes = [C.c_int, C.c_uint, C.c_uint]
        lib.oracle_kernel_offsets.restype = C.c_uint
        lib.oracle_kernel_offsets.argtypes = [C.c_int, C.c_uint, C.c_uint, _UP]
        lib.oracle_plan_create.restype = C.c_void_p
        lib.oracle_plan_create.argtypes = [C.c_int, C.c_uint, C.c_uint]
        lib.oracle_plan_destroy.argtypes = [C.c_void_p]
        lib.oracle_plan_lanes.restype = C.c_uint
        lib.oracle_plan_lanes.argtypes = [C.c_void_p]
        for name in ("oracle_forward", "oracle_inverse"):
            getattr(lib, name).argtypes = [C.c_void_p, _FP, _FP, _FP]
        lib.oracle_get_kernel.argtypes = [C.c_void_p, _FP, _FP]
        lib.oracle_conv.argtypes = [C.c_void_p, _FP, _FP, _FP, _FP]
        lib.oracle_run_batch.restype = C.c_double
        lib.oracle_run_batch.argtypes = [C.c_void_p, C.c_int, _FP, _FP, _FP, C.c_uint, C.c_size_t, C.c_uint]
        _port = lib
    return _port


def _fp(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_FP)


def plan_chain(length: int, width: int):
    buf = (C.c_uint * 64)()
    n = port().oracle_plan_chain(length, width, buf)
    return [buf[i] for i in range(n)]


def kernel_offsets(modulation: int, L: int, build_vw: int = 4):
    """(re_off[L] indexed by natural bin, lane width V); im at re_off + V."""
    off = np.zeros(L, np.uint32)
    V = port().oracle_kernel_offsets(modulation, L, build_vw, off.ctypes.data_as(_UP))
    if V == 0:
        raise ValueError(f"no plan for L={L}")
    return off.astype(np.int64), int(V)


def kernel_from_spectrum(modulation: int, W: np.ndarray, build_vw: int = 4) -> np.ndarray:
    """Scatter a natural-order spectrum into the reference kernel layout."""
    L = W.shape[-1]
    off, V = kernel_offsets(modulation, L, build_vw)
    K = np.zeros(W.shape[:-1] + (2 * L,), np.float64)
    K[..., off] = W.real
    K[..., off + V] = W.imag
    return K


def spectrum_from_kernel(modulation: int, K: np.ndarray, build_vw: int = 4) -> np.ndarray:
    L = K.shape[-1] // 2
    off, V = kernel_offsets(modulation, L, build_vw)
    return K[..., off] + 1j * K[..., off + V]


class PortPlan:
    """FP32 restatement of one reference plan (modulation, L, SIMD width)."""

    def __init__(self, modulation: int, L: int, build_vw: int = 4):
        self.lib = port()
        self.modulation, self.L, self.build_vw = modulation, L, build_vw
        self.h = self.lib.oracle_plan_create(modulation, L, build_vw)
        if not self.h:
            raise ValueError(f"no plan for L={L}")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_plan_destroy(self.h)
            self.h = None

    def _io(self, x):
        x = np.ascontiguousarray(x, np.float32)
        assert x.shape[-1] == 2 * self.L
        return x

    def forward(self, x):
        x = self._io(x)
        out = np.empty_like(x)
        work = np.empty(2 * self.L, np.float32)
        for o, i in zip(out.reshape(-1, 2 * self.L), x.reshape(-1, 2 * self.L)):
            self.lib.oracle_forward(self.h, _fp(o), _fp(np.ascontiguousarray(i)), _fp(work))
        return out

    def inverse(self, X):
        X = self._io(X)
        out = np.empty_like(X)
        work = np.empty(2 * self.L, np.float32)
        for o, i in zip(out.reshape(-1, 2 * self.L), X.reshape(-1, 2 * self.L)):
            self.lib.oracle_inverse(self.h, _fp(o), _fp(np.ascontiguousarray(i)), _fp(work))
        return out

    def get_kernel(self, h):
        h = self._io(h)
        out = np.empty_like(h)
        self.lib.oracle_get_kernel(self.h, _fp(out), _fp(h))
        return out

    def conv(self, x, K):
        x = self._io(x)
        K = self._io(K)
        out = np.empty_like(x)
        work = np.empty(2 * self.L, np.float32)
        for o, i in zip(out.reshape(-1, 2 * self.L), x.reshape(-1, 2 * self.L)):
            self.lib.oracle_conv(self.h, _fp(o), _fp(np.ascontiguousarray(i)), _fp(K), _fp(work))
        return out

    def run_batch(self, op: str, out, x, K=None, nthreads: int = 1) -> float:
        """Threaded batch over rows of x; returns wall seconds."""
        code = {"conv": 0, "forward": 1, "inverse": 2}[op]
        x = self._io(x).reshape(-1, 2 * self.L)
        assert out.dtype == np.float32 and out.flags["C_CONTIGUOUS"] and out.size == x.size
        kp = _fp(self._io(K)) if K is not None else None
        return self.lib.oracle_run_batch(self.h, code, _fp(out), _fp(x), kp, x.shape[0], 2 * self.L, nthreads)


# --------------------------------------------------------------------------
# The unmodified reference compiled here (only where its sources exist).
# FFTSET_REFERENCE_SRC, the default being where this container mounts them
REF_SOURCES = os.environ.get("FFTSET_REFERENCE_SRC", "/root/reference")


def build_reference() -> bool:
    """Build oracle/_ref when the reference sources are present."""
    if not os.path.isdir(os.path.join(REF_SOURCES, "src")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SOURCES}"], check=True)
    return True


def reference_available(vw: int = 4) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libfftset_ref_vw{vw}.so"))


class Reference:
    """ctypes driver for oracle/_ref/libfftset_ref_vw{vw}.so."""

    def __init__(self, vw: int = 4):
        lib = C.CDLL(os.path.join(HERE, "_ref", f"libfftset_ref_vw{vw}.so"))
        lib.oref_new.restype = C.c_void_p
        lib.oref_free.argtypes = [C.c_void_p]
        lib.oref_modulation.restype = C.c_void_p
        lib.oref_modulation.argtypes = [C.c_int]
        lib.fftset_create_fft.restype = C.c_void_p
        lib.fftset_create_fft.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
        for name in ("fftset_fft_forward", "fftset_fft_inverse"):
            getattr(lib, name).argtypes = [C.c_void_p, _FP, _FP, _FP]
        lib.fftset_fft_conv_get_kernel.argtypes = [C.c_void_p, _FP, _FP]
        lib.fftset_fft_conv.argtypes = [C.c_void_p, _FP, _FP, _FP, _FP]
        lib.fftset_recommend_conv_length.restype = C.c_uint
        lib.fftset_recommend_conv_length.argtypes = [C.c_uint, C.c_uint]
        self.lib = lib
        self.fs = lib.oref_new()

    def __del__(self):
        if getattr(self, "fs", None):
            self.lib.oref_free(self.fs)
            self.fs = None

    def fft(self, modulation: int, L: int):
        f = self.lib.fftset_create_fft(self.fs, self.lib.oref_modulation(modulation), L)
        if not f:
            raise ValueError(f"reference could not create L={L}")
        return f

    @staticmethod
    def _buf(x):
        return np.ascontiguousarray(x, np.float32).copy()

    def forward(self, modulation, L, x):
        f = self.fft(modulation, L)
        x = self._buf(x)
        out = np.zeros_like(x)
        work = np.zeros(2 * L, np.float32)
        for o, i in zip(out.reshape(-1, 2 * L), x.reshape(-1, 2 * L)):
            self.lib.fftset_fft_forward(f, _fp(o), _fp(i), _fp(work))
        return out

    def inverse(self, modulation, L, X, in_place: bool = True):
        """in_place=True mirrors fftset_test.c:142; the width-1 FREQ_OFFSET
        inverse reads its middle bin from output_buf for odd L
        (src/fftset_mod_freqoffsetreal.c:995-998), so only in-place calls are
        defined for it."""
        f = self.fft(modulation, L)
        X = self._buf(X)
        work = np.zeros(2 * L, np.float32)
        if in_place:
            for row in X.reshape(-1, 2 * L):
                self.lib.fftset_fft_inverse(f, _fp(row), _fp(row), _fp(work))
            return X
        out = np.zeros_like(X)
        for o, i in zip(out.reshape(-1, 2 * L), X.reshape(-1, 2 * L)):
            self.lib.fftset_fft_inverse(f, _fp(o), _fp(i), _fp(work))
        return out

    def get_kernel(self, modulation, L, h):
        f = self.fft(modulation, L)
        h = self._buf(h)
        out = np.zeros_like(h)
        self.lib.fftset_fft_conv_get_kernel(f, _fp(out), _fp(h))
        return out

    def conv(self, modulation, L, x, K):
        f = self.fft(modulation, L)
        x = self._buf(x)
        K = self._buf(K)
        out = np.zeros_like(x)
        work = np.zeros(2 * L, np.float32)
        for o, i in zip(out.reshape(-1, 2 * L), x.reshape(-1, 2 * L)):
            self.lib.fftset_fft_conv(f, _fp(o), _fp(i), _fp(K), _fp(work))
        return out

    def recommend_conv_length(self, kernel_length, max_block):
        return self.lib.fftset_recommend_conv_length(kernel_length, max_block)


# --------------------------------------------------------------------------
# Inputs of the reference's own test program (app_fftset_test/fftset_test.c):
# buffers set to 1 at index 0 and at every prime (its table starts with 0,
# fftset_test.c:26-27).
def prime_flags(n: int) -> np.ndarray:
    f = np.zeros(n, bool)
    if n > 0:
        f[0] = True
    sieve = np.ones(max(n, 2), bool)
    sieve[:2] = False
    for p in range(2, int(n ** 0.5) + 1):
        if sieve[p]:
            sieve[p * p::p] = False
    f[2:n] = sieve[2:n]
    return f


def valid_sizes(lo: int, hi: int):
    return [L for L in range(lo, hi + 1) if valid_size(L)]


# sizes of fftset_test.c:327-346
REFERENCE_TEST_LENGTHS = [2, 3, 4, 5, 6, 8, 9, 15, 27, 45, 12, 16, 20, 24, 32, 40,
                          48, 64, 80, 96, 128, 160, 18, 36, 72, 144, 288, 576]
