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


@pytest.mark.parametrize("mod,L", [(1, 1536), (1, 4096), (0, 1024)])
def test_dependent_launch_chain(fftset_lib, mod, L):
    """The compiled kernels, the adjoint kernels and the taps reduction are
    launched as programmatic dependents: each reads what the launches before
    it wrote only after griddepcontrol.wait. A chain of non-blocking calls
    that each consume the previous one's output, with no synchronisation in
    between, must give the FP64 results."""
    import torch
    S = fftset_lib.FftSet()
    try:
        f = S.create_fft(mod, L)
        rng = np.random.default_rng(L + 3)
        B = 64
        x_np = rng.standard_normal((B, 2 * L)).astype(np.float32)
        h_np = rng.standard_normal((B, 2 * L)).astype(np.float32)
        g_np = rng.standard_normal((B, 2 * L)).astype(np.float32)
        x, h, g = (torch.from_numpy(a).cuda() for a in (x_np, h_np, g_np))
        K = torch.empty_like(h)
        y = torch.empty_like(x)
        X = torch.empty_like(x)
        r = torch.empty_like(x)
        dx = torch.empty_like(x)
        dh = torch.empty(2 * L, device="cuda")
        torch.cuda.synchronize()
        S.set_blocking(False)
        for _ in range(3):
            f.conv_get_kernel_batch(K, h)       # K written ...
            f.conv_batch(y, x, K[0])            # ... read by the next launch
            f.forward_batch(X, y)               # y read
            f.inverse_batch(r, X)               # X read
            f.conv_adjoint_batch(dx, dh, r, x, K[0])  # r, K read; kgrad, reduce, inverse
        torch.cuda.synchronize()
        S.set_blocking(True)
        S.check()
        y64 = O.conv64(mod, x_np, h_np[0])
        assert O.rel_l2(y.cpu().numpy(), y64) <= O.tolerance(2 * L if mod else L)
        assert O.rel_l2(r.cpu().numpy() / L, y64) <= 2 * O.tolerance(2 * L if mod else L)
        wx, wh = O.conv_adjoint64(mod, x_np, h_np[0], r.cpu().numpy().astype(np.float64))
        assert O.rel_l2(dx.cpu().numpy(), wx) <= 4 * O.tolerance(2 * L if mod else L)
        assert O.rel_l2(dh.cpu().numpy(), wh) <= 4 * O.tolerance(2 * L if mod else L)
    finally:
        S.close()


@pytest.mark.parametrize("mod,L", [(0, 1024), (1, 1536), (0, 2048), (1, 45)])
def test_served_calls_in_place(fftset_lib, mod, L):
    """Blocking single calls with the output buffer equal to the input (as
    the reference allows) give the batched in-place results bit for bit."""
    import torch
    S = fftset_lib.FftSet()
    try:
        f = S.create_fft(mod, L)
        rng = np.random.default_rng(L + 17)
        B = 10
        x_np = rng.standard_normal((B, 2 * L)).astype(np.float32)
        for op in ("forward", "inverse"):
            want = torch.from_numpy(x_np).cuda()
            getattr(f, op + "_batch")(want, want)
            got = torch.from_numpy(x_np).cuda()
            for b in range(B):
                getattr(f, op)(got[b], got[b])
            assert np.array_equal(got.cpu().numpy(), want.cpu().numpy()), op
        S.check()
    finally:
        S.close()


def test_service_setup_failure_falls_back(fftset_lib):
    """The call service's page cannot be allocated (the allocation wrappers'
    failure hook): blocking calls run the usual way, with the same results,
    no latched error, and nothing left allocated after destroy."""
    import torch
    H = _hooks(fftset_lib)
    L_ = fftset_lib.library()
    L_.fftset__test_fail_allocation.restype = C.c_long
    L_.fftset__test_fail_allocation.argtypes = [C.c_long]
    L_.fftset__test_live_allocations.restype = None
    L_.fftset__test_live_allocations.argtypes = [C.POINTER(C.c_long), C.POINTER(C.c_long)]

    def live():
        h, d = C.c_long(0), C.c_long(0)
        L_.fftset__test_live_allocations(C.byref(h), C.byref(d))
        return h.value, d.value

    L = 1024
    rng = np.random.default_rng(23)
    x = torch.from_numpy(rng.standard_normal((6, 2 * L)).astype(np.float32)).cuda()
    torch.cuda.synchronize()
    base = live()
    S = fftset_lib.FftSet()
    try:
        f = S.create_fft(0, L)
        want = torch.empty_like(x)
        f.forward_batch(want, x)
        got = torch.empty_like(x)
        f.forward(got[0], x[0])  # the first call of its kind: no service yet
        L_.fftset__test_fail_allocation(1)  # the service's page is the next allocation
        try:
            for b in range(1, 6):
                f.forward(got[b], x[b])
        finally:
            L_.fftset__test_fail_allocation(0)
        assert np.array_equal(got.cpu().numpy(), want.cpu().numpy())
        assert H.fftset__test_served_calls(S.handle) == 0
        S.check()
    finally:
        S.close()
    torch.cuda.synchronize()
    assert live() == base
