"""The call service: blocking single calls on device buffers of resident
sizes are answered by one resident CTA (the compiled variant's service, or
the generic kernel's) instead of a launch each. Its results must be the
batched kernels' bit for bit, it must wait for work already queued on the
fftset's stream, and it must come and go (idle exit, a new launch on the
next call, destroy while it is live) without changing a result."""
import ctypes as C
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _hooks(lib):
    L = lib.library()
    L.fftset__test_set_call_service.restype = C.c_int
    L.fftset__test_set_call_service.argtypes = [lib._P, C.c_uint]
    L.fftset__test_served_calls.restype = C.c_ulonglong
    L.fftset__test_served_calls.argtypes = [lib._P]
    return L


@pytest.mark.parametrize("mod,L", [(0, 1024), (1, 1536), (1, 4096),  # compiled kernels' services
                                   (0, 2048), (1, 45), (0, 27), (1, 19683)])  # the generic kernel's
def test_served_calls_equal_batched_kernels(fftset_lib, mod, L):
    import torch
    H = _hooks(fftset_lib)
    S = fftset_lib.FftSet()
    try:
        f = S.create_fft(mod, L)
        rng = np.random.default_rng(L)
        B = 12
        x = torch.from_numpy(rng.standard_normal((B, 2 * L)).astype(np.float32)).cuda()
        h = rng.standard_normal(2 * L).astype(np.float32)
        K = torch.empty(2 * L, device="cuda")
        f.conv_get_kernel(K, torch.from_numpy(h).cuda())
        ops = ("forward", "inverse", "conv", "conv_get_kernel")
        want = {}
        for op in ops:
            y = torch.empty_like(x)
            if op == "conv":
                f.conv_batch(y, x, K)
            else:
                getattr(f, op + "_batch")(y, x)
            want[op] = y.cpu().numpy()
        n0 = H.fftset__test_served_calls(S.handle)
        for op in ops:
            got = torch.full_like(x, 7.0)
            for b in range(B):  # repeated calls of one kind: the service takes them
                if op == "conv":
                    f.conv(got[b], x[b], K)
                else:
                    getattr(f, op)(got[b], x[b])
            assert np.array_equal(got.cpu().numpy(), want[op]), op
        assert H.fftset__test_served_calls(S.handle) - n0 >= 3 * (B - 2)
        S.check()
    finally:
        S.close()


def test_served_call_waits_for_queued_work(fftset_lib):
    """A non-blocking batched forward queued on the stream, then blocking
    single inverses of its output: each must see the finished forward."""
    import torch
    H = _hooks(fftset_lib)
    S = fftset_lib.FftSet()
    try:
        L, B = 1024, 64
        f = S.create_fft(0, L)
        rng = np.random.default_rng(5)
        x_np = rng.standard_normal((B, 2 * L)).astype(np.float32)
        x = torch.from_numpy(x_np).cuda()
        X = torch.empty_like(x)
        r = torch.empty_like(x)
        f.inverse(r[0], x[0])
        f.inverse(r[0], x[0])  # the service is live from here
        for rep in range(3):
            X.fill_(0.0)
            S.set_blocking(False)
            f.forward_batch(X, x)  # queued, not waited for
            S.set_blocking(True)
            for b in range(B):
                f.inverse(r[b], X[b])
            assert O.rel_l2(r.cpu().numpy() / L, x_np) <= O.tolerance(L), rep
        assert H.fftset__test_served_calls(S.handle) > 0
        S.check()
    finally:
        S.close()


def test_service_idle_exit_and_off(fftset_lib):
    import torch
    H = _hooks(fftset_lib)
    S = fftset_lib.FftSet()
    try:
        L = 1536
        f = S.create_fft(1, L)
        rng = np.random.default_rng(9)
        x = torch.from_numpy(rng.standard_normal((6, 2 * L)).astype(np.float32)).cuda()
        want = torch.empty_like(x)
        f.forward_batch(want, x)
        w = want.cpu().numpy()
        got = torch.empty_like(x)
        for b in range(6):
            f.forward(got[b], x[b])
            time.sleep(0.005)  # far beyond the idle window: the launch exits between calls
        assert np.array_equal(got.cpu().numpy(), w)
        n = H.fftset__test_served_calls(S.handle)
        assert H.fftset__test_set_call_service(S.handle, 0) == 0
        got.fill_(0.0)
        for b in range(6):
            f.forward(got[b], x[b])
        assert np.array_equal(got.cpu().numpy(), w)
        assert H.fftset__test_served_calls(S.handle) == n
        assert H.fftset__test_set_call_service(S.handle, 64) == 0
        for b in range(6):
            f.forward(got[b], x[b])
        assert np.array_equal(got.cpu().numpy(), w)
        assert H.fftset__test_served_calls(S.handle) > n
        S.check()
    finally:
        S.close()


def test_destroy_with_live_service(fftset_lib):
    """fftset_destroy stops a live launch (no wait for its idle exit is
    needed for correctness, and nothing hangs)."""
    import torch
    for _ in range(3):
        S = fftset_lib.FftSet()
        f = S.create_fft(0, 1024)
        x = torch.randn(2 * 1024, device="cuda")
        y = torch.empty_like(x)
        for _ in range(4):
            f.forward(y, x)
        t0 = time.perf_counter()
        S.close()
        assert time.perf_counter() - t0 < 1.0
        torch.cuda.synchronize()
