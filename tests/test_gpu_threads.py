"""Concurrent execution calls on one fftset.

The reference promises that its execution calls are thread-safe as long as
the output and work buffers of concurrent calls are distinct (README.md:38).
Here four host threads call fftset_fft_forward / inverse / conv and their
batched forms through the C ABI at the same time on one fftset, on device
buffers of their own, mixing resident sizes with sizes beyond the
shared-memory limit (65,536 bins: a two-level task split; 131,072 bins: a
three-level one; their convolutions: the two-pass kernels and the fftset's
work buffer), with directions alternating and batch counts changing from
call to call, so that the plans' cached task lists and the work buffer are
built, reused and replaced while other threads launch. Every result is
checked against the FP64 oracle afterwards. Tolerance: relative L2 <=
2e-6 * log2(N), as in the other parity tests."""
import threading

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (modulation, complex bins)
PLANS = [(0, 1024), (1, 1536), (0, 65536), (1, 65536), (1, 131072), (0, 131072)]
OPS = ("forward", "inverse", "conv")


def _tol(mod, L):
    return O.tolerance(2 * L if mod else L)


def _schedule(tid: int, n: int):
    """Thread tid's calls: plans visited in a thread-specific order, the op
    alternating, batch counts 1..3 (count 1 through the reference's own
    single-block calls)."""
    rng = np.random.default_rng(900 + tid)
    out = []
    for i in range(n):
        mod, L = PLANS[(tid + 3 * i) % len(PLANS)]
        op = OPS[(tid + i) % len(OPS)]
        count = int(rng.integers(1, 4))
        out.append((mod, L, op, count, int(rng.integers(1 << 30))))
    return out


def test_concurrent_execution_calls(fftset_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    lib = fftset_lib.library()
    S = fftset_lib.FftSet()
    try:
        plans, kern, taps = {}, {}, {}
        for mod, L in PLANS:
            f = S.create_fft(mod, L)
            assert f is not None
            plans[(mod, L)] = f
            h = np.random.default_rng(L + mod).standard_normal(2 * L).astype(np.float32)
            K = torch.empty(2 * L, device="cuda")
            f.conv_get_kernel(K, torch.from_numpy(h).cuda())
            kern[(mod, L)], taps[(mod, L)] = K, h
        torch.cuda.synchronize()
        S.check()
        maxf = 3 * 2 * max(L for _, L in PLANS)
        nthreads, ncalls = 4, 9
        results, errors = [], []
        lock = threading.Lock()

        def worker(tid):
            try:
                torch.cuda.set_device(0)
                inb = torch.empty(maxf, device="cuda")
                outb = torch.empty(maxf, device="cuda")
                for mod, L, op, count, seed in _schedule(tid, ncalls):
                    f, nf = plans[(mod, L)], 2 * L
                    x = np.random.default_rng(seed).standard_normal((count, nf)).astype(np.float32)
                    inb[:count * nf].copy_(torch.from_numpy(x.ravel()))
                    torch.cuda.synchronize()
                    outb[:count * nf].fill_(float("nan"))
                    torch.cuda.synchronize()
                    ip, op_ = inb.data_ptr(), outb.data_ptr()
                    if count == 1 and op == "forward":
                        lib.fftset_fft_forward(f.handle, op_, ip, None)
                    elif count == 1 and op == "inverse":
                        lib.fftset_fft_inverse(f.handle, op_, ip, None)
                    elif count == 1:
                        lib.fftset_fft_conv(f.handle, op_, ip, kern[(mod, L)].data_ptr(), None)
                    elif op == "forward":
                        assert lib.fftset_fft_forward_batch(f.handle, op_, nf, ip, nf, count) == 0
                    elif op == "inverse":
                        assert lib.fftset_fft_inverse_batch(f.handle, op_, nf, ip, nf, count) == 0
                    else:
                        assert lib.fftset_fft_conv_batch(f.handle, op_, nf, ip, nf,
                                                         kern[(mod, L)].data_ptr(), count) == 0
                    # blocking calls: the results are in place when they return
                    y = outb[:count * nf].cpu().numpy().reshape(count, nf)
                    with lock:
                        results.append((tid, mod, L, op, x, y))
            except Exception as ex:  # reported by the main thread
                with lock:
                    errors.append(repr(ex))

        ts = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        assert not errors, errors
        assert S.last_error() == 0, fftset_lib.error_string(S.last_error())
        assert len(results) == nthreads * ncalls
        seen = set()
        for tid, mod, L, op, x, y in results:
            if op == "forward":
                want = O.forward64(mod, x)
            elif op == "inverse":
                want = O.inverse64(mod, x)
            else:
                want = O.conv64(mod, x, taps[(mod, L)][None, :])
            assert np.all(np.isfinite(y)), (tid, mod, L, op)
            assert O.rel_l2(y, want) <= _tol(mod, L), (tid, mod, L, op, O.rel_l2(y, want))
            seen.add((L > 26244, op))
        # both resident and beyond-shared-memory sizes ran every op
        assert seen == {(b, o) for b in (False, True) for o in OPS}
    finally:
        S.close()
