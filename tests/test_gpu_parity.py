"""GPU parity through the C ABI: every execution call against the unmodified
reference's outputs (tests/golden), the FP64 oracle, the reference's own
known-answer tests, and the edge cases of its contract (aliasing, odd sizes,
unsupported sizes, host buffers, batched calls). Tolerance: relative L2 <=
2e-6 * log2(N), N the transform length in reals (FREQ_OFFSET_REAL: 2L) or
complex points (COMPLEX: L)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [(m, L) for m in (0, 1) for L in O.REFERENCE_TEST_LENGTHS] + [(0, 1024), (1, 1536), (1, 4096)]


def tol(mod, L):
    return O.tolerance(2 * L if mod else L)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _g(golden, mod, L, what):
    return golden[f"m{mod}_L{L}_{what}"]


@pytest.mark.parametrize("mod,L", CASES)
def test_forward_matches_reference(gpu_set, golden_outputs, mod, L):
    import torch
    f = gpu_set.create_fft(mod, L)
    x = _g(golden_outputs, mod, L, "x")
    out = torch.empty(2 * L, device="cuda")
    f.forward(out, dev(x))
    y = host(out)
    assert O.rel_l2(y, _g(golden_outputs, mod, L, "fwd")) <= tol(mod, L)
    assert O.rel_l2(y, O.forward64(mod, x)) <= tol(mod, L)


@pytest.mark.parametrize("mod,L", CASES)
def test_inverse_matches_reference(gpu_set, golden_outputs, mod, L):
    import torch
    f = gpu_set.create_fft(mod, L)
    X = _g(golden_outputs, mod, L, "fwd")
    out = torch.empty(2 * L, device="cuda")
    f.inverse(out, dev(X))
    y = host(out)
    assert O.rel_l2(y, _g(golden_outputs, mod, L, "inv")) <= tol(mod, L)
    assert O.rel_l2(y, O.inverse64(mod, X)) <= tol(mod, L)
    # in place, as the reference's own test calls it (fftset_test.c:142)
    buf = dev(X)
    f.inverse(buf, buf)
    assert O.rel_l2(host(buf), y) <= 1e-7


@pytest.mark.parametrize("mod,L", CASES)
def test_get_kernel_matches_reference_layout(gpu_set, golden_outputs, mod, L):
    import torch
    f = gpu_set.create_fft(mod, L)
    h = _g(golden_outputs, mod, L, "h")
    out = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(out, dev(h))
    assert O.rel_l2(host(out), _g(golden_outputs, mod, L, "kern")) <= tol(mod, L)


@pytest.mark.parametrize("mod,L", CASES)
def test_conv_matches_reference(gpu_set, golden_outputs, mod, L):
    """conv with the kernel buffer the REFERENCE prepared (layout interop),
    and with our own; in place (input_buf == output_buf) as the reference
    allows and its test does (fftset_test.c:198)."""
    import torch
    f = gpu_set.create_fft(mod, L)
    x = _g(golden_outputs, mod, L, "x")
    Kref = _g(golden_outputs, mod, L, "kern")
    want = _g(golden_outputs, mod, L, "conv")
    out = torch.empty(2 * L, device="cuda")
    f.conv(out, dev(x), dev(Kref))
    assert O.rel_l2(host(out), want) <= tol(mod, L)
    assert O.rel_l2(host(out), O.conv64(mod, x, _g(golden_outputs, mod, L, "h"))) <= tol(mod, L)
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(_g(golden_outputs, mod, L, "h")))
    buf = dev(x)
    f.conv(buf, buf, K)
    assert O.rel_l2(host(buf), want) <= tol(mod, L)


@pytest.mark.parametrize("L", O.REFERENCE_TEST_LENGTHS)
def test_reference_kats_on_gpu(gpu_set, L):
    """The reference's own known-answer tests (app_fftset_test/fftset_test.c)
    with its RMS thresholds, through the C ABI."""
    import torch
    N = 2 * L
    flags = O.prime_flags(N)
    # FREQ_OFFSET_REAL prime impulse (:70-156)
    f = gpu_set.create_fft(1, L)
    x = flags.astype(np.float32)
    X = torch.empty(N, device="cuda")
    f.forward(X, dev(x))
    Xh = host(X).astype(np.float64)
    err = Xh - O.freqoff_direct64(x)
    assert np.sqrt((err[0::2] ** 2 + err[1::2] ** 2).sum() / L) <= 4e-6
    f.inverse(X, X)
    r = host(X) / L - x
    assert np.sqrt((r ** 2).sum() / L) <= 1e-6
    # convolution (:158-222)
    h = np.where(flags & (np.arange(N) < N // 4), 2.0 / N, 0.0).astype(np.float32)
    s = np.where(flags & (np.arange(N) < 3 * N // 4), 1.0, 0.0).astype(np.float32)
    K = torch.empty(N, device="cuda")
    f.conv_get_kernel(K, dev(h))
    y = dev(s)
    f.conv(y, y, K)
    exp = np.zeros(N)
    for a in np.nonzero(s)[0]:
        for b in np.nonzero(h)[0]:
            exp[a + b] += 1.0
    assert np.sqrt(((exp - host(y)) ** 2).sum() / L) <= 1e-5
    # COMPLEX prime impulse (:224-314), inverse checked on all 2L floats
    g = gpu_set.create_fft(0, L)
    Xc = torch.empty(N, device="cuda")
    g.forward(Xc, dev(x))
    err = host(Xc).astype(np.float64) - O.complex_forward64(x)
    assert np.sqrt((err[0::2] ** 2 + err[1::2] ** 2).sum() / L) <= 4e-6
    g.inverse(Xc, Xc)
    r = host(Xc) / L - x
    assert np.sqrt((r ** 2).sum() / L) <= 1e-6


def _all_sizes():
    return O.valid_sizes(2, 4096)


@pytest.mark.parametrize("mod", [0, 1])
def test_every_size_to_4096_against_fp64(gpu_set, mod):
    """Every supported size 2..4096: forward, inverse, conv vs FP64."""
    import torch
    rng = np.random.default_rng(11 + mod)
    for L in _all_sizes():
        f = gpu_set.create_fft(mod, L)
        assert f is not None, L
        x = rng.standard_normal(2 * L).astype(np.float32)
        h = rng.standard_normal(2 * L).astype(np.float32)
        X = torch.empty(2 * L, device="cuda")
        f.forward(X, dev(x))
        Xh = host(X)
        assert O.rel_l2(Xh, O.forward64(mod, x)) <= tol(mod, L), L
        r = torch.empty(2 * L, device="cuda")
        f.inverse(r, X)
        assert O.rel_l2(host(r), O.inverse64(mod, Xh)) <= tol(mod, L), L
        K = torch.empty(2 * L, device="cuda")
        f.conv_get_kernel(K, dev(h))
        y = torch.empty(2 * L, device="cuda")
        f.conv(y, dev(x), K)
        assert O.rel_l2(host(y), O.conv64(mod, x, h)) <= tol(mod, L), L


@pytest.mark.parametrize("mod,L", [(0, 8192), (1, 8192), (0, 12288), (1, 15360), (0, 16384), (1, 16384),
                                   (1, 20736), (0, 25920), (1, 26244)])
def test_large_resident_sizes_against_fp64(gpu_set, mod, L):
    import torch
    rng = np.random.default_rng(L)
    f = gpu_set.create_fft(mod, L)
    assert f is not None
    x = rng.standard_normal((3, 2 * L)).astype(np.float32)
    h = rng.standard_normal(2 * L).astype(np.float32)
    X = torch.empty(3, 2 * L, device="cuda")
    f.forward_batch(X, dev(x))
    Xh = host(X)
    assert O.rel_l2(Xh, O.forward64(mod, x)) <= tol(mod, L)
    r = torch.empty_like(X)
    f.inverse_batch(r, X)
    assert O.rel_l2(host(r), O.inverse64(mod, Xh)) <= tol(mod, L)
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(h))
    y = torch.empty_like(X)
    f.conv_batch(y, dev(x), K)
    assert O.rel_l2(host(y), O.conv64(mod, x, h)) <= tol(mod, L)


@pytest.mark.parametrize("mod,L", [(1, 1536), (0, 1024), (1, 45), (0, 27), (1, 4096), (0, 60)])
def test_batch_equals_single_calls(gpu_set, mod, L):
    """Batched entry points with padded strides give the single-call result
    block by block, and leave the padding untouched."""
    import torch
    f = gpu_set.create_fft(mod, L)
    rng = np.random.default_rng(3)
    B, pad = 37, 6
    x = rng.standard_normal((B, 2 * L + pad)).astype(np.float32)
    h = rng.standard_normal(2 * L).astype(np.float32)
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(h))
    xd = dev(x)
    for op in ("forward", "inverse", "conv"):
        out = torch.full((B, 2 * L + pad), 7.0, device="cuda")
        if op == "conv":
            f.conv_batch(out, xd, K)
        else:
            getattr(f, op + "_batch")(out, xd)
        ob = host(out)
        assert np.all(ob[:, 2 * L:] == 7.0)
        for b in (0, 1, B // 2, B - 1):
            single = torch.empty(2 * L, device="cuda")
            src = dev(x[b, :2 * L])
            if op == "conv":
                f.conv(single, src, K)
            else:
                getattr(f, op)(single, src)
            assert np.array_equal(host(single), ob[b, :2 * L]), (op, b)


def test_host_buffers_are_staged(gpu_set, golden_outputs):
    """numpy (host) buffers go through the staging path and give the same
    results as device buffers."""
    mod, L = 1, 1536
    f = gpu_set.create_fft(mod, L)
    x = _g(golden_outputs, mod, L, "x").copy()
    K = _g(golden_outputs, mod, L, "kern").copy()
    y = np.empty_like(x)
    f.conv(y, x, K)
    assert O.rel_l2(y, _g(golden_outputs, mod, L, "conv")) <= tol(mod, L)
    X = np.empty_like(x)
    f.forward(X, x)
    assert O.rel_l2(X, _g(golden_outputs, mod, L, "fwd")) <= tol(mod, L)
    f.inverse(X, X)
    assert O.rel_l2(X, O.inverse64(mod, _g(golden_outputs, mod, L, "fwd"))) <= tol(mod, L)


def test_unsupported_sizes_return_null(gpu_set):
    for L in (0, 1, 7, 25, 49, 3 * 7 * 16, 50):
        assert gpu_set.create_fft(1, L) is None
        assert gpu_set.create_fft(0, L) is None


def test_plans_are_shared(gpu_set):
    a = gpu_set.create_fft(1, 1536)
    b = gpu_set.create_fft(1, 1536)
    c = gpu_set.create_fft(0, 1536)
    assert a.handle == b.handle and a.handle != c.handle


@pytest.mark.parametrize("vw", [1, 8])
def test_other_simd_layouts(fftset_lib, golden_layouts, vw):
    """Kernel buffers in the layout of width-1 and width-8 reference builds."""
    import torch
    S = fftset_lib.FftSet(kernel_layout_width=vw)
    rng = np.random.default_rng(vw)
    try:
        for mod, L in ((1, 1536), (1, 576), (0, 1024), (1, 96), (0, 45)):
            f = S.create_fft(mod, L)
            h = rng.standard_normal(2 * L).astype(np.float32)
            K = torch.empty(2 * L, device="cuda")
            f.conv_get_kernel(K, dev(h))
            off = golden_layouts[f"vw{vw}_m{mod}_L{L}"].astype(np.int64)
            V = f.kernel_lanes
            W = O.spectrum64(mod, h)
            want = np.zeros(2 * L)
            want[off] = W.real
            want[off + V] = W.imag
            assert O.rel_l2(host(K), want) <= tol(mod, L)
            x = rng.standard_normal(2 * L).astype(np.float32)
            y = torch.empty(2 * L, device="cuda")
            f.conv(y, dev(x), K)
            assert O.rel_l2(host(y), O.conv64(mod, x, h)) <= tol(mod, L)
    finally:
        S.close()


STATIC = [(1, 1536), (1, 4096), (0, 1024), (0, 1536), (0, 4096)]


@pytest.mark.parametrize("mod,L", STATIC)
@pytest.mark.parametrize("pad", [0, 2])
def test_compiled_size_kernels(fftset_lib, gpu_set, mod, L, pad):
    """Every compile-time kernel variant of the hot sizes (persistent CTAs,
    tables staged in shared memory), on batches large enough to select them:
    forward, inverse and convolution against FP64, with padded strides that
    leave blocks only 8-byte aligned, and in place."""
    import torch
    fs = fftset_lib
    f = gpu_set.create_fft(mod, L)
    assert f.variants >= 1
    rng = np.random.default_rng(L + pad)
    B = 300
    x = rng.standard_normal((B, 2 * L + pad)).astype(np.float32)
    h = rng.standard_normal(2 * L).astype(np.float32)
    xd = dev(x)
    xs = x[:, :2 * L]
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(h))
    want_fwd = O.forward64(mod, xs)
    want_conv = O.conv64(mod, xs, h)
    ran = 0
    defaults = {op: f.variant(op) for op in (fs.OP_FORWARD, fs.OP_INVERSE, fs.OP_CONV)}
    try:
        for v in range(-1, f.variants):
            for op in (fs.OP_FORWARD, fs.OP_INVERSE, fs.OP_CONV):
                try:
                    f.set_variant(op, v)
                except fs.FftsetError:
                    continue
                if op == fs.OP_FORWARD:
                    X = torch.full((B, 2 * L + pad), 5.0, device="cuda")
                    f.forward_batch(X, xd)
                    Xh = host(X)
                    assert np.all(Xh[:, 2 * L:] == 5.0)
                    assert O.rel_l2(Xh[:, :2 * L], want_fwd) <= tol(mod, L), v
                elif op == fs.OP_INVERSE:
                    Xd = dev(np.pad(want_fwd.astype(np.float32), ((0, 0), (0, pad))))
                    r = torch.empty_like(Xd)
                    f.inverse_batch(r, Xd)
                    assert O.rel_l2(host(r)[:, :2 * L], O.inverse64(mod, want_fwd)) <= tol(mod, L), v
                else:
                    y = torch.empty_like(xd)
                    f.conv_batch(y, xd, K)
                    assert O.rel_l2(host(y)[:, :2 * L], want_conv) <= tol(mod, L), v
                    buf = xd.clone()
                    f.conv_batch(buf, buf, K)
                    assert O.rel_l2(host(buf)[:, :2 * L], want_conv) <= tol(mod, L), v
                ran += 1
    finally:
        for op, v in defaults.items():  # the plan is shared with later tests
            f.set_variant(op, v)
    assert ran >= 4


def _supports(f, op, v):
    try:
        f.set_variant(op, v)
        return True
    except Exception:
        return False


def test_autotune_picks_a_working_kernel(fftset_lib, gpu_set):
    import torch
    fs = fftset_lib
    f = gpu_set.create_fft(1, 1536)
    ms = f.autotune(fs.OP_CONV, 2048)
    assert ms > 0
    assert -1 <= f.variant(fs.OP_CONV) < f.variants
    rng = np.random.default_rng(9)
    x = rng.standard_normal((512, 3072)).astype(np.float32)
    h = rng.standard_normal(3072).astype(np.float32)
    K = torch.empty(3072, device="cuda")
    f.conv_get_kernel(K, dev(h))
    y = torch.empty(512, 3072, device="cuda")
    f.conv_batch(y, dev(x), K)
    assert O.rel_l2(host(y), O.conv64(1, x, h)) <= tol(1, 1536)


RADIX9 = [(0, 81), (1, 243), (0, 729), (1, 2187), (0, 3888), (1, 6561), (0, 19683)]


@pytest.mark.parametrize("mod,L", RADIX9)
def test_radix9_chains_against_fp64(gpu_set, mod, L):
    """Resident sizes whose radix chains use the radix-9 codelet (81 = 9 9,
    19683 = 9 9 9 9 3, 3888 = 12 12 9 3): forward, inverse and conv of a
    batch of 3 against FP64."""
    import torch
    f = gpu_set.create_fft(mod, L)
    assert f is not None
    rng = np.random.default_rng(L + 7 * mod)
    x = rng.standard_normal((3, 2 * L)).astype(np.float32)
    X = torch.empty(3, 2 * L, device="cuda")
    f.forward_batch(X, dev(x))
    Xh = host(X)
    assert O.rel_l2(Xh, O.forward64(mod, x)) <= tol(mod, L)
    r = torch.empty_like(X)
    f.inverse_batch(r, X)
    assert O.rel_l2(host(r), O.inverse64(mod, Xh)) <= tol(mod, L)
    h = rng.standard_normal(2 * L).astype(np.float32)
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(h))
    y = torch.empty_like(X)
    f.conv_batch(y, dev(x), K)
    assert O.rel_l2(host(y), O.conv64(mod, x, h)) <= tol(mod, L)


# three-level from 131072 on: n3 groups 4 (131072), 6 (393216), 5 (327680, an
# odd count, so with mirror tiles adjacent the middle group pairs with
# itself) and one (177147 = 27 x 81 x 81: 16 does not divide L3)
FOURSTEP = [32768, 36864, 46656, 59049, 65536, 131072, 393216, 327680, 177147]


@pytest.mark.parametrize("mod", [0, 1])
@pytest.mark.parametrize("L", FOURSTEP)
def test_fourstep_sizes_against_fp64(gpu_set, mod, L):
    """Sizes beyond the shared-memory limit (two HBM passes), including odd
    ones (59049 = 3^10) whose FREQ_OFFSET_REAL mirror pairing has a
    self-mirrored middle row: forward and inverse vs FP64, batched and in
    place."""
    import torch
    f = gpu_set.create_fft(mod, L)
    assert f is not None
    rng = np.random.default_rng(L + mod)
    B = 2
    x = rng.standard_normal((B, 2 * L)).astype(np.float32)
    X = torch.empty(B, 2 * L, device="cuda")
    f.forward_batch(X, dev(x))
    Xh = host(X)
    assert O.rel_l2(Xh, O.forward64(mod, x)) <= tol(mod, L)
    r = torch.empty_like(X)
    f.inverse_batch(r, X)
    assert O.rel_l2(host(r), O.inverse64(mod, Xh)) <= tol(mod, L)
    buf = dev(x[0])
    f.forward(buf, buf)
    assert O.rel_l2(host(buf), Xh[0]) <= 1e-6
    # kernel buffer in the reference layout, and the convolution (in place)
    h = rng.standard_normal(2 * L).astype(np.float32)
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(h))
    want_k = O.kernel_from_spectrum(mod, O.spectrum64(mod, h), 4)
    assert O.rel_l2(host(K), want_k) <= tol(mod, L)
    y = dev(x)
    f.conv_batch(y, y, K)
    assert O.rel_l2(host(y), O.conv64(mod, x, h)) <= tol(mod, L)


@pytest.mark.parametrize("mod,L", [(0, 131072), (1, 327680), (1, 393216), (0, 177147)])
def test_three_level_group_order(fftset_lib, mod, L):
    """Three-level task lists order the A and B tiles by n3 group and the
    later B tiles and the C tiles by k1 group, B tiles waiting for their
    n3 group's A tiles only, C tiles for their k1 group's B tiles. The
    default lists every A tile first; a test hook interleaves the A and B
    passes, the B tiles of a group following the A tiles of the group 1 or
    2 slots later (a distance past the last group is the default). Every
    order must list each tile once and give the same results bit for bit,
    forward and inverse, batched."""
    import ctypes as C
    import torch
    lib = fftset_lib.library()
    lib.fftset__test_set_group_distance.restype = C.c_int
    lib.fftset__test_set_group_distance.argtypes = [fftset_lib._P, C.c_uint]
    rng = np.random.default_rng(L + 7 * mod)
    x = torch.from_numpy(rng.standard_normal((3, 2 * L)).astype(np.float32)).cuda()
    got = []
    for dist in (0, 1, 2, 1000):
        S = fftset_lib.FftSet()
        try:
            assert lib.fftset__test_set_group_distance(S.handle, dist) == 0
            f = S.create_fft(mod, L)
            X = torch.empty_like(x)
            r = torch.empty_like(x)
            f.forward_batch(X, x)
            f.inverse_batch(r, X)
            S.check()
            got.append((X.cpu().numpy(), r.cpu().numpy()))
        finally:
            S.close()
    xh = x.cpu().numpy()
    assert O.rel_l2(got[0][0], O.forward64(mod, xh)) <= tol(mod, L)
    for X, r in got[1:]:
        assert np.array_equal(X, got[0][0]) and np.array_equal(r, got[0][1])


@pytest.mark.parametrize("mod", [0, 1])
def test_beyond_three_levels(gpu_set, mod):
    """2^25 bins has no three-level split (a factor above 256), so the
    two-pass kernels run it: ping-pong tiles, and for the FREQ_OFFSET_REAL
    forward's rows of 8192 points (two tile buffers do not fit) the
    in-place form. Forward against FP64, and the round trip."""
    import torch
    L = 1 << 25
    f = gpu_set.create_fft(mod, L)
    assert f is not None
    rng = np.random.default_rng(25 + mod)
    x = rng.standard_normal((1, 2 * L)).astype(np.float32)
    X = torch.empty(1, 2 * L, device="cuda")
    f.forward_batch(X, dev(x))
    Xh = host(X)
    assert O.rel_l2(Xh, O.forward64(mod, x)) <= tol(mod, L)
    r = torch.empty_like(X)
    f.inverse_batch(r, X)
    assert O.rel_l2(host(r) / L, x) <= 2 * tol(mod, L)
    gpu_set.check()


def test_fourstep_large_single(gpu_set):
    """The 15,728,640-bin FREQ_OFFSET_REAL transform: forward against FP64
    (error per bin band) and the forward/inverse round trip."""
    import torch
    L = 15728640
    f = gpu_set.create_fft(1, L)
    assert f is not None
    rng = np.random.default_rng(6)
    n = np.arange(2 * L)
    freqs = rng.uniform(0, L, 64)
    amps = rng.uniform(0.01, 1, 64)
    phases = rng.uniform(0, 2 * np.pi, 64)
    x = np.zeros(2 * L)
    for fr, a, ph in zip(freqs, amps, phases):
        x += a * np.cos(np.pi * fr * n / L + ph)
    x = (x + rng.normal(0, 1e-3, 2 * L)).astype(np.float32)
    X = torch.empty(2 * L, device="cuda")
    f.forward(X, dev(x))
    Xh = host(X).astype(np.float64)
    want = O.freqoff_forward64(x)
    assert O.rel_l2(Xh, want) <= tol(1, L)
    # every band of L/8 bins within the tolerance itself (measured 1.9-2.6e-7
    # per band, against 5e-5)
    bands = np.array_split(np.arange(L), 8)
    for b in bands:
        sl = np.concatenate([2 * b, 2 * b + 1])
        assert O.rel_l2(Xh[sl], want[sl]) <= tol(1, L)
    r = torch.empty(2 * L, device="cuda")
    f.inverse(r, X)
    assert O.rel_l2(host(r) / L, x) <= tol(1, L)


@pytest.mark.parametrize("mod,L,op", [(1, 1536, "conv"), (0, 1024, "forward"), (1, 4096, "inverse")])
def test_host_buffers_chunk_pipeline(gpu_set, mod, L, op):
    """Host (numpy) buffers large enough for the chunk pipeline (several
    16 MB chunks over three streams), padded rows and in-place: the same
    results as device buffers, every block written."""
    import torch
    f = gpu_set.create_fft(mod, L)
    B, pad = int(40e6 // (8 * L)), 6
    rng = np.random.default_rng(L + 7)
    x = rng.standard_normal((B, 2 * L + pad)).astype(np.float32)
    h = rng.standard_normal(2 * L).astype(np.float32)
    K = np.empty(2 * L, np.float32)
    f.conv_get_kernel(K, h)
    Kd = dev(K)
    want = torch.empty(B, 2 * L, device="cuda")
    xd = dev(x)[:, :2 * L].contiguous()
    got = np.full((B, 2 * L + 2), np.nan, np.float32)
    if op == "conv":
        f.conv_batch(want, xd, Kd)
        f.conv_batch(got, x, K)
    elif op == "forward":
        f.forward_batch(want, xd)
        f.forward_batch(got, x)
    else:
        f.inverse_batch(want, xd)
        f.inverse_batch(got, x)
    w = host(want)
    # staged rows may run a different compiled kernel (alignment): same
    # result to rounding
    assert O.rel_l2(got[:, :2 * L], w) <= 1e-6
    assert np.all(np.isnan(got[:, 2 * L:]))
    # in place on host memory
    y = x.copy()
    if op == "conv":
        f.conv_batch(y, y, K)
    elif op == "forward":
        f.forward_batch(y, y)
    else:
        f.inverse_batch(y, y)
    assert O.rel_l2(y[:, :2 * L], w) <= 1e-6


@pytest.mark.parametrize("mod,L,op", [(1, 1536, "conv"), (0, 1024, "forward"), (1, 4096, "inverse"),
                                      (1, 4096, "conv"), (0, 96, "forward")])
def test_pinned_host_buffers_in_place_access(gpu_set, mod, L, op):
    """Pinned host buffers are read and written by the kernels directly (no
    staging): results equal the device-buffer call's to rounding, the memory
    between padded rows is untouched, in place works."""
    import torch
    f = gpu_set.create_fft(mod, L)
    B, pad = 300, 6
    rng = np.random.default_rng(L + 11)
    x = torch.from_numpy(rng.standard_normal((B, 2 * L + pad)).astype(np.float32)).pin_memory()
    h = rng.standard_normal(2 * L).astype(np.float32)
    K = torch.from_numpy(np.empty(2 * L, np.float32)).pin_memory()
    f.conv_get_kernel(K, torch.from_numpy(h).pin_memory())
    Kd = K.cuda()
    xd = x.cuda()[:, :2 * L].contiguous()
    want = torch.empty(B, 2 * L, device="cuda")
    got = torch.full((B, 2 * L + 2), float("nan")).pin_memory()
    call = {"conv": lambda o, i, k: f.conv_batch(o, i, k), "forward": lambda o, i, k: f.forward_batch(o, i),
            "inverse": lambda o, i, k: f.inverse_batch(o, i)}[op]
    call(want, xd, Kd)
    call(got, x, K)
    w = host(want)
    g = got.numpy()
    assert O.rel_l2(g[:, :2 * L], w) <= 1e-6
    assert np.all(np.isnan(g[:, 2 * L:]))
    y = x.clone().pin_memory()
    call(y, y, K)
    assert O.rel_l2(y.numpy()[:, :2 * L], w) <= 1e-6
    assert np.array_equal(y.numpy()[:, 2 * L:], x.numpy()[:, 2 * L:])


@pytest.mark.parametrize("mod,L,K,blk", [(1, 1536, 401, 0), (1, 1536, 1025, 0), (1, 1536, 1025, 1500),
                                         (1, 1536, 2048, 0), (1, 4096, 900, 1000), (0, 1024, 200, 0),
                                         (1, 768, 1, 0)])
def test_overlap_add_linear_convolution(gpu_set, mod, L, K, blk):
    """fftset_fft_conv_overlap_add: complex_bins times the linear convolution
    of a long signal (several hundred blocks, ragged last block) with a K-tap
    kernel, against FP64 np.convolve. FREQ_OFFSET_REAL at 1536 bins with
    K - 1 <= B runs the fused kernel (blocks read from the signal, results
    added into the output); K = 2048 at 1536 bins (K - 1 > B) and the other
    sizes run split, batched convolution and gather."""
    import torch
    f = gpu_set.create_fft(mod, L)
    N = L if mod == 0 else 2 * L
    rng = np.random.default_rng(L + K)
    n = 97 * N + 13
    if mod == 1:
        x = rng.standard_normal(n).astype(np.float32)
        taps = (rng.standard_normal(K) * np.exp(-np.arange(K) / max(K / 4, 1))).astype(np.float32)
        h = np.zeros(N, np.float32)
        h[:K] = taps
        want = L * np.convolve(x.astype(np.float64), taps.astype(np.float64))
        xin = x
    else:
        xc = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        tc = rng.standard_normal(K) + 1j * rng.standard_normal(K)
        h = np.zeros(2 * N, np.float32)
        h[0:2 * K:2], h[1:2 * K:2] = tc.real, tc.imag
        wc = L * np.convolve(xc.astype(np.complex64).astype(np.complex128), tc.astype(np.complex64).astype(np.complex128))
        want = np.empty(2 * wc.size)
        want[0::2], want[1::2] = wc.real, wc.imag
        xin = np.empty(2 * n, np.float32)
        xin[0::2], xin[1::2] = xc.real, xc.imag
    K_spec = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K_spec, dev(h))
    out = torch.full((want.size + 4,), float("nan"), device="cuda")
    f.conv_overlap_add(out[:want.size], dev(xin), K_spec, K, blk)
    got = host(out)
    assert O.rel_l2(got[:want.size], want) <= tol(mod, L)
    assert np.all(np.isnan(got[want.size:]))
