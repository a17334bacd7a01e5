"""fftset_fft_execute_fixed_scratch through the C ABI.

This entry point is for callers that must not allocate device memory while
they run, such as a real-time audio callback that cannot block in the
driver's allocator. It runs the four-step passes of sizes beyond the
shared-memory limit with their work buffer in a fixed device array. Its
results must equal the regular batched call's (fftset_fft_*_batch) on two
calls in a row, the second one reusing what the first left in the array, and
it must refuse what it cannot run within the array. Each result is also
checked against the FP64 oracle directly (the regular batched forward and
inverse run other kernels, so the comparison between the two GPU paths
alone would pin this one only indirectly). Tolerance: relative L2 <=
2e-6 * log2(N), as in the other parity tests.

This file is named to be collected last, and it makes its own fftset, so it
passes alone in a fresh process as well as after the other tests."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FFTSET_OK, FFTSET_E_INVALID, FFTSET_E_UNSUPPORTED = 0, 1, 4
OPS = {"forward": 0, "inverse": 1, "get_kernel": 2, "conv": 3, "corr": 4}


def _entry(lib):
    fn = lib.library().fftset_fft_execute_fixed_scratch
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_uint]
    return fn


def _tol(mod, L):
    return O.tolerance(2 * L if mod else L)


@pytest.fixture(scope="module")
def fset(fftset_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    s = fftset_lib.FftSet()
    yield s
    s.close()


# 59049 = 243 x 243 and 177147 = 243 x 729: odd factors (a self-mirrored
# middle row or column in the FREQ_OFFSET_REAL pairing); 1048576: four-lane
# tiles of 1024 points
@pytest.mark.parametrize("mod,L,count", [(0, 32768, 4), (1, 36864, 3), (1, 65536, 2), (1, 59049, 2),
                                         (1, 177147, 2), (0, 131072, 2), (1, 1048576, 2)])
def test_fixed_scratch_matches_batched_call(fftset_lib, fset, mod, L, count):
    import torch
    fn = _entry(fftset_lib)
    f = fset.create_fft(mod, L)
    assert f is not None
    fset.set_stream(torch.cuda.current_stream())
    rng = np.random.default_rng(100 + L + mod)
    h_np = rng.standard_normal(2 * L).astype(np.float32)
    h = torch.from_numpy(h_np).cuda()
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, h)
    for call in range(2):
        x_np = rng.standard_normal((count, 2 * L)).astype(np.float32)
        x = torch.from_numpy(x_np).cuda()
        for name, op in OPS.items():
            want = torch.empty_like(x)
            if name == "forward":
                f.forward_batch(want, x)
                want64 = O.forward64(mod, x_np)
            elif name == "inverse":
                f.inverse_batch(want, x)
                want64 = O.inverse64(mod, x_np)
            elif name == "get_kernel":
                f.conv_get_kernel_batch(want, x)
                want64 = np.stack([O.kernel_from_spectrum(mod, O.spectrum64(mod, r), 4) for r in x_np])
            elif name == "conv":
                f.conv_batch(want, x, K)
                want64 = O.conv64(mod, x_np, h_np[None, :])
            else:
                gi = torch.empty_like(x)
                f.conv_adjoint_batch(gi, None, x, x, K)
                want = gi
                want64 = O.conv64(mod, x_np, O.reverse(mod, h_np.astype(np.float64))[None, :])
            got = torch.full_like(x, float("nan"))
            rc = fn(f.handle, op, got.data_ptr(), 2 * L, x.data_ptr(), 2 * L,
                    K.data_ptr() if name in ("conv", "corr") else None, count)
            torch.cuda.synchronize()
            assert rc == FFTSET_OK, (call, name, fftset_lib.error_string(rc))
            g, w = got.cpu().numpy(), want.cpu().numpy()
            assert np.all(np.isfinite(g)), (call, name)
            assert O.rel_l2(g, w) <= _tol(mod, L), (call, name)
            assert O.rel_l2(g, want64) <= _tol(mod, L), (call, name, O.rel_l2(g, want64))
    assert fset.last_error() == 0


def test_fixed_scratch_rejects_what_it_cannot_run(fftset_lib, fset):
    import torch
    fn = _entry(fftset_lib)
    fset.set_stream(torch.cuda.current_stream())
    big = fset.create_fft(0, 65536)
    buf = torch.zeros(2 * 65536, device="cuda")
    # the batch's work would exceed the array: refused before any launch
    limit = 8 << 20
    too_many = limit // (2 * 65536) + 1
    assert fn(big.handle, 0, buf.data_ptr(), 2 * 65536, buf.data_ptr(), 2 * 65536, None, too_many) == FFTSET_E_INVALID
    fset.clear_error()
    # sizes that fit shared memory use no scratch
    small = fset.create_fft(0, 1024)
    assert fn(small.handle, 0, buf.data_ptr(), 2048, buf.data_ptr(), 2048, None, 1) == FFTSET_E_UNSUPPORTED
    fset.clear_error()
    # host buffers would need staging memory
    hbuf = np.zeros(2 * 65536, np.float32)
    assert fn(big.handle, 0, hbuf.ctypes.data, 2 * 65536, hbuf.ctypes.data, 2 * 65536, None, 1) == FFTSET_E_INVALID
    fset.clear_error()
    # a convolution needs its kernel buffer
    assert fn(big.handle, 3, buf.data_ptr(), 2 * 65536, buf.data_ptr(), 2 * 65536, None, 1) == FFTSET_E_INVALID
    fset.clear_error()
    assert fn(big.handle, 0, buf.data_ptr(), 2 * 65536, buf.data_ptr(), 2 * 65536, None, 0) == FFTSET_OK
