"""Failure detection without a GPU fault.

- Memory exhaustion, made on the host: a test hook of the library's
  allocation wrappers makes the n-th host or device allocation fail. The
  reference's contract is that fftset_init returns non-zero and
  fftset_create_fft returns NULL when memory runs out (fftset.h:44-47, :78;
  src/fftset.c:84, :112-116); here, in addition, the failure is latched as
  FFTSET_E_NOMEM, an execution call that needed memory reports it, and
  nothing stays allocated once the fftset is destroyed.
- Bounded waits inside a kernel: the ragged task kernel's waits on the
  tiles a tile depends on give up after a number of polls. A test hook
  removes the tiles a wait depends on (a counter nothing increments) with a
  short poll limit; the launch must return, the call must report
  FFTSET_E_TIMEOUT, and the GPU context must stay usable."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FFTSET_OK, FFTSET_E_NOMEM, FFTSET_E_TIMEOUT = 0, 2, 5
TASK_COLS, TASK_PA = 1, 3


def _hooks(lib):
    L = lib.library()
    L.fftset__test_fail_allocation.restype = C.c_long
    L.fftset__test_fail_allocation.argtypes = [C.c_long]
    L.fftset__test_live_allocations.restype = None
    L.fftset__test_live_allocations.argtypes = [C.POINTER(C.c_long), C.POINTER(C.c_long)]
    L.fftset__test_set_spin_limit.restype = C.c_int
    L.fftset__test_set_spin_limit.argtypes = [lib._P, C.c_uint]
    L.fftset__test_ragged_drop_kind.restype = C.c_int
    L.fftset__test_ragged_drop_kind.argtypes = [C.c_void_p, C.c_int]
    return L


def _live(L):
    h, d = C.c_long(0), C.c_long(0)
    L.fftset__test_live_allocations(C.byref(h), C.byref(d))
    return h.value, d.value


def _struct(lib):
    return lib._FftsetStruct()  # a caller-allocated struct fftset


def test_init_reports_exhausted_memory(fftset_lib):
    import torch
    assert torch.cuda.is_available()
    L = _hooks(fftset_lib)
    base = _live(L)
    failed = 0
    for n in range(1, 64):
        s = _struct(fftset_lib)
        L.fftset__test_fail_allocation(n)
        rc = L.fftset_init(C.byref(s))
        left = L.fftset__test_fail_allocation(0)
        if rc == 0:
            assert left > 0, n  # the injected failure lies beyond init
            L.fftset_destroy(C.byref(s))
            assert _live(L) == base
            break
        failed += 1
        assert s.impl is None
        assert _live(L) == base, n
    assert failed >= 2  # init's own allocations (its state, the mapped error flag)


@pytest.mark.parametrize("mod,bins", [(1, 1536), (0, 1920), (1, 65536), (0, 131072)])
def test_create_fft_reports_exhausted_memory(fftset_lib, mod, bins):
    L = _hooks(fftset_lib)
    modp = fftset_lib.MODULATION_FREQ_OFFSET_REAL if mod else fftset_lib.MODULATION_COMPLEX
    base = _live(L)
    failed = 0
    for n in range(1, 200):
        s = _struct(fftset_lib)
        assert L.fftset_init(C.byref(s)) == 0
        L.fftset__test_fail_allocation(n)
        p = L.fftset_create_fft(C.byref(s), modp, bins)
        left = L.fftset__test_fail_allocation(0)
        if p:
            assert left > 0
            L.fftset_destroy(C.byref(s))
            assert _live(L) == base
            break
        failed += 1
        assert L.fftset_last_error(C.byref(s)) == FFTSET_E_NOMEM, n
        # the failed creation left nothing behind, and the next one works
        assert L.fftset_clear_error(C.byref(s)) == FFTSET_E_NOMEM
        assert L.fftset_create_fft(C.byref(s), modp, bins)
        L.fftset_destroy(C.byref(s))
        assert _live(L) == base, n
    assert failed >= 2


@pytest.mark.parametrize("op", ["forward", "conv"])
def test_execution_reports_exhausted_memory(fftset_lib, op):
    """A plan beyond the shared-memory limit allocates on its first batched
    call (its task list, or the convolution's work buffer): every failure
    of those allocations is reported by the call, and a later call works."""
    import torch
    L = _hooks(fftset_lib)
    bins, count, nf = 65536, 3, 2 * 65536
    base = _live(L)
    S = fftset_lib.FftSet()
    try:
        f = S.create_fft(1, bins)
        rng = np.random.default_rng(77)
        h = rng.standard_normal(nf).astype(np.float32)
        K = torch.empty(nf, device="cuda")
        f.conv_get_kernel(K, torch.from_numpy(h).cuda())
        x = rng.standard_normal((count, nf)).astype(np.float32)
        xd = torch.from_numpy(x).cuda()
        y = torch.empty_like(xd)
        failed = 0
        for n in range(1, 100):
            L.fftset__test_fail_allocation(n)
            if op == "forward":
                rc = L.fftset_fft_forward_batch(f.handle, y.data_ptr(), nf, xd.data_ptr(), nf, count)
            else:
                rc = L.fftset_fft_conv_batch(f.handle, y.data_ptr(), nf, xd.data_ptr(), nf, K.data_ptr(), count)
            left = L.fftset__test_fail_allocation(0)
            if rc == FFTSET_OK:
                assert left > 0
                break
            failed += 1
            assert rc == FFTSET_E_NOMEM, (n, rc)
            assert S.clear_error() == FFTSET_E_NOMEM
        assert failed >= 1
        want = O.forward64(1, x) if op == "forward" else O.conv64(1, x, h[None, :])
        torch.cuda.synchronize()
        assert O.rel_l2(y.cpu().numpy(), want) <= O.tolerance(nf)
        assert S.last_error() == 0
    finally:
        S.close()
    assert _live(L) == base


@pytest.mark.parametrize("bins,kind", [(16384, TASK_COLS), (131072, TASK_PA)])
def test_bounded_wait_times_out(fftset_lib, bins, kind):
    """Tiles that wait on tiles which never run give up after the poll
    limit; the call reports FFTSET_E_TIMEOUT and the context stays usable."""
    import torch
    L = _hooks(fftset_lib)
    S = fftset_lib.FftSet()
    try:
        n = 4
        sizes = [bins] * n
        offs = [2 * bins * i for i in range(n)]
        x_np = np.random.default_rng(bins).uniform(-1, 1, 2 * bins * n).astype(np.float32)
        x = torch.from_numpy(x_np).cuda()
        y = torch.zeros_like(x)
        S.set_stream(torch.cuda.current_stream())
        assert L.fftset__test_set_spin_limit(S.handle, 4096) == FFTSET_OK
        rb = fftset_lib.Ragged(S, fftset_lib.COMPLEX, fftset_lib.OP_FORWARD, sizes, offs, offs)
        assert L.fftset__test_ragged_drop_kind(C.c_void_p(rb.h), kind) == FFTSET_OK
        rc = L.fftset_ragged_execute(C.c_void_p(rb.h), C.c_void_p(y.data_ptr()), C.c_void_p(x.data_ptr()))
        assert rc == FFTSET_E_TIMEOUT
        assert S.clear_error() == FFTSET_E_TIMEOUT
        rb.close()
        # the context still works: the same batch, complete, with the default limit
        assert L.fftset__test_set_spin_limit(S.handle, 1 << 22) == FFTSET_OK
        rb = fftset_lib.Ragged(S, fftset_lib.COMPLEX, fftset_lib.OP_FORWARD, sizes, offs, offs)
        rb.execute(y, x)
        torch.cuda.synchronize()
        S.check()
        yh = y.cpu().numpy()
        for o in offs:
            assert O.rel_l2(yh[o:o + 2 * bins], O.complex_forward64(x_np[o:o + 2 * bins])) <= O.tolerance(bins)
        rb.close()
    finally:
        S.close()
