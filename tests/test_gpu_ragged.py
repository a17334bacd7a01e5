"""Ragged batches through the C ABI: many sizes in one submission (persistent
launch for resident sizes, four-step passes for the rest, CUDA graph
replay), every item against FP64."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def draw_sizes(n, seed, lo=60, hi=65536):
    """Log-uniform in [lo, hi], snapped (in log space) to the nearest
    2^a 3^b 5^{0,1} size."""
    valid = np.array(O.valid_sizes(lo, hi))
    rng = np.random.default_rng(seed)
    u = rng.uniform(np.log(lo), np.log(hi), n)
    idx = np.abs(np.log(valid)[None, :] - u[:, None]).argmin(1)
    return valid[idx]


def layout(sizes, gap=2):
    offs, o = [], 0
    for L in sizes:
        offs.append(o)
        o += 2 * int(L) + gap
    return offs, o


@pytest.mark.parametrize("mod", [0, 1])
@pytest.mark.parametrize("graph", [True, False])
def test_ragged_forward_inverse(fftset_lib, gpu_set, mod, graph):
    import torch
    sizes = draw_sizes(240, seed=4 + mod)
    # three-level (beyond 65536), largest two-level, odd two-level, smallest
    sizes[:4] = [393216, 65536, 59049, 60]
    offs, total = layout(sizes)
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, total).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    for op in (fftset_lib.OP_FORWARD, fftset_lib.OP_INVERSE):
        rb = fftset_lib.Ragged(gpu_set, mod, op, [int(s) for s in sizes], offs, offs)
        rb.set_graph(graph)
        y = torch.full_like(xd, 3.0)
        rb.execute(y, xd)
        y1 = y.cpu().numpy()
        rb.execute(y, xd)                       # replay
        torch.cuda.synchronize()
        assert np.array_equal(y.cpu().numpy(), y1)
        assert rb.persistent_items == len(sizes)
        for L, o in zip(sizes, offs):
            L = int(L)
            xi = x[o:o + 2 * L]
            want = O.forward64(mod, xi) if op == fftset_lib.OP_FORWARD else O.inverse64(mod, xi)
            assert O.rel_l2(y1[o:o + 2 * L], want) <= O.tolerance(2 * L if mod else L), (L, op)
            assert np.all(y1[o + 2 * L:o + 2 * L + 2] == 3.0)
        rb.close()


def test_ragged_equals_single_calls(fftset_lib, gpu_set):
    import torch
    sizes = [1024, 60, 4096, 1536, 27000 // 27 * 27 if O.valid_size(27000) else 26244, 32768, 100]
    sizes = [s for s in sizes if O.valid_size(s)]
    offs, total = layout(sizes, gap=0)
    rng = np.random.default_rng(8)
    x = rng.standard_normal(total).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    rb = fftset_lib.Ragged(gpu_set, 0, fftset_lib.OP_FORWARD, sizes, offs, offs)
    y = torch.empty_like(xd)
    rb.execute(y, xd)
    torch.cuda.synchronize()
    for L, o in zip(sizes, offs):
        f = gpu_set.create_fft(0, L)
        one = torch.empty(2 * L, device="cuda")
        f.forward(one, xd[o:o + 2 * L])
        torch.cuda.synchronize()
        assert O.rel_l2(y[o:o + 2 * L].cpu().numpy(), one.cpu().numpy()) <= 1e-6, L
    rb.close()


@pytest.mark.parametrize("mod", [0, 1])
def test_ragged_both_task_shapes(fftset_lib, mod):
    """The list's CTA shape forced either way (narrow 128-thread or wide
    256-thread task CTAs), two-level and three-level items alike: every item
    against FP64, in both directions."""
    import ctypes as C
    import torch
    L_ = fftset_lib.library()
    L_.fftset__test_set_task_shape.restype = C.c_int
    L_.fftset__test_set_task_shape.argtypes = [fftset_lib._P, C.c_int]
    sizes = [int(s) for s in draw_sizes(60, seed=11 + mod)]
    sizes[:3] = [262144, 65536, 19683]
    offs, total = layout(sizes)
    x = np.random.default_rng(12).uniform(-1, 1, total).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    S = fftset_lib.FftSet()
    try:
        for shape in (0, 1):
            assert L_.fftset__test_set_task_shape(S.handle, shape) == 0
            for op in (fftset_lib.OP_FORWARD, fftset_lib.OP_INVERSE):
                rb = fftset_lib.Ragged(S, mod, op, sizes, offs, offs)
                y = torch.full_like(xd, 3.0)
                rb.execute(y, xd)
                torch.cuda.synchronize()
                yh = y.cpu().numpy()
                for L, o in zip(sizes, offs):
                    xi = x[o:o + 2 * L]
                    want = O.forward64(mod, xi) if op == fftset_lib.OP_FORWARD else O.inverse64(mod, xi)
                    assert O.rel_l2(yh[o:o + 2 * L], want) <= O.tolerance(2 * L if mod else L), (shape, L, op)
                rb.close()
        assert L_.fftset__test_set_task_shape(S.handle, 3) != 0
        S.check()
    finally:
        S.close()


@pytest.mark.parametrize("mod", [0, 1])
def test_ragged_single_buffer_shape(fftset_lib, mod):
    """The single-buffer CTA shape (six per SM, one tile buffer) on a list
    whose every chain has two stages (items up to 256 bins, two-level and
    three-level items with such factors): every item against FP64; a list
    with a longer chain is refused on that shape."""
    import ctypes as C
    import torch
    L_ = fftset_lib.library()
    L_.fftset__test_set_task_shape.restype = C.c_int
    L_.fftset__test_set_task_shape.argtypes = [fftset_lib._P, C.c_int]
    sizes = [262144, 65536, 61440, 16384, 256, 240, 128, 96, 60, 64, 200, 256, 16, 12]
    sizes = [s for s in sizes if O.valid_size(s)]
    offs, total = layout(sizes)
    x = np.random.default_rng(31).uniform(-1, 1, total).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    S = fftset_lib.FftSet()
    try:
        assert L_.fftset__test_set_task_shape(S.handle, 2) == 0
        for op in (fftset_lib.OP_FORWARD, fftset_lib.OP_INVERSE):
            rb = fftset_lib.Ragged(S, mod, op, sizes, offs, offs)
            y = torch.full_like(xd, 3.0)
            rb.execute(y, xd)
            torch.cuda.synchronize()
            yh = y.cpu().numpy()
            for L, o in zip(sizes, offs):
                xi = x[o:o + 2 * L]
                want = O.forward64(mod, xi) if op == fftset_lib.OP_FORWARD else O.inverse64(mod, xi)
                assert O.rel_l2(yh[o:o + 2 * L], want) <= O.tolerance(2 * L if mod else L), (L, op)
            rb.close()
        S.check()
        with pytest.raises(fftset_lib.FftsetError):  # 4096 = 16 x 16 x 16: three stages
            fftset_lib.Ragged(S, mod, fftset_lib.OP_FORWARD, [4096, 256], [0, 8192], [0, 8192])
        S.clear_error()
    finally:
        S.close()


def test_ragged_rejects_bad_input(fftset_lib, gpu_set):
    with pytest.raises(fftset_lib.FftsetError):
        fftset_lib.Ragged(gpu_set, 0, fftset_lib.OP_FORWARD, [64, 7], [0, 200], [0, 200])
    with pytest.raises(fftset_lib.FftsetError):
        fftset_lib.Ragged(gpu_set, 0, fftset_lib.OP_FORWARD, [64], [1], [0])



def test_ragged_autotune_keeps_results(fftset_lib):
    """fftset_ragged_autotune picks per-size schedules (radix order, threads
    per item, lanes per tile) by timing and rebuilds the batch: the results
    stay within tolerance of FP64, before and after, graph replay included."""
    import torch
    S = fftset_lib.FftSet()
    try:
        sizes = [60, 96, 243, 1024, 1536, 4096, 6144, 16384, 59049, 65536, 131072]
        sizes = sizes + sizes[::-1][1:]
        offs, total = layout(sizes)
        rng = np.random.default_rng(21)
        x = rng.uniform(-1, 1, total).astype(np.float32)
        xd = torch.from_numpy(x).cuda()
        S.set_stream(torch.cuda.current_stream())
        for mod, op in ((0, fftset_lib.OP_FORWARD), (1, fftset_lib.OP_INVERSE)):
            rb = fftset_lib.Ragged(S, mod, op, sizes, offs, offs)
            y0 = torch.full_like(xd, 3.0)
            rb.execute(y0, xd)
            rb.autotune()
            y1 = torch.full_like(xd, 3.0)
            rb.execute(y1, xd)
            rb.execute(y1, xd)
            torch.cuda.synchronize()
            a, b = y0.cpu().numpy(), y1.cpu().numpy()
            for L, o in zip(sizes, offs):
                xi = x[o:o + 2 * L]
                want = O.forward64(mod, xi) if op == fftset_lib.OP_FORWARD else O.inverse64(mod, xi)
                assert O.rel_l2(a[o:o + 2 * L], want) <= O.tolerance(2 * L if mod else L), (L, "before")
                assert O.rel_l2(b[o:o + 2 * L], want) <= O.tolerance(2 * L if mod else L), (L, "after")
                assert np.all(b[o + 2 * L:o + 2 * L + 2] == 3.0)
            rb.close()
    finally:
        S.close()
