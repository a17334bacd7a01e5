"""The convolution adjoint (fftset_fft_conv_adjoint_batch) through the C ABI
and a torch.autograd.Function harness (tests/fftset_autograd.py):
  - against the FP64 adjoint (oracle.conv_adjoint64) for both modulations at
    resident, four-step and three-level sizes, with padded strides;
  - against reference gradients built from the reference's own CPU
    convolution with time-reversed kernels (tests/golden/ref_adjoint_vw4.npz);
  - the differentiable batched workload (FREQ_OFFSET_REAL, 4096 bins, batch
    2048, loss sum w*y) against FP64 central finite differences (h = 1e-3, 64
    sampled coordinates of x and of the taps) and against the gradient built
    from the oracle's C restatement of the reference convolution.
Tolerance: relative L2 <= 2e-6 * log2(N) (N = 2L reals for FREQ_OFFSET_REAL,
L points for COMPLEX)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def tol(mod, L):
    return O.tolerance(2 * L if mod else L)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def adjoint(f, g, x, h):
    import torch
    K = torch.empty(h.shape, device="cuda")
    f.conv_get_kernel(K, h)
    dx = torch.full_like(g, float("nan"))
    dh = torch.full((h.shape[-1],), float("nan"), device="cuda")
    f.conv_adjoint_batch(dx, dh, g, x, K)
    return host(dx), host(dh)


# resident (60 .. 16384), four-step (32768, 131072 three-level)
SIZES = [(1, 60), (1, 96), (1, 243), (1, 1536), (1, 4096), (1, 8192), (1, 8748), (1, 16384), (1, 32768), (1, 131072),
         (0, 64), (0, 1024), (0, 4096), (0, 11520), (0, 32768)]


@pytest.mark.parametrize("mod,L", SIZES)
def test_adjoint_against_fp64(gpu_set, mod, L):
    if not O.valid_size(L):
        pytest.skip("not a 2^a 3^b 5^{0,1} size")
    f = gpu_set.create_fft(mod, L)
    assert f is not None
    rng = np.random.default_rng(L * 3 + mod)
    B = 5
    x = rng.standard_normal((B, 2 * L)).astype(np.float32)
    g = rng.standard_normal((B, 2 * L)).astype(np.float32)
    h = rng.standard_normal(2 * L).astype(np.float32)
    dx, dh = adjoint(f, dev(g), dev(x), dev(h))
    wx, wh = O.conv_adjoint64(mod, x, h, g)
    assert O.rel_l2(dx, wx) <= tol(mod, L)
    assert O.rel_l2(dh, wh) <= tol(mod, L)


@pytest.mark.parametrize("L", [1536, 4096])
def test_adjoint_strides_and_single_outputs(gpu_set, L):
    """Padded rows, one output at a time, both at once, count 1 and count 0.
    At 4096 bins the compiled one-pass kernels run (both gradients, or the
    taps gradient alone); at 1536 bins the batched-forward route."""
    import torch
    B, pad = 7, 10
    f = gpu_set.create_fft(1, L)
    rng = np.random.default_rng(11)
    xs = rng.standard_normal((B, 2 * L + pad)).astype(np.float32)
    gs = rng.standard_normal((B, 2 * L + pad)).astype(np.float32)
    h = rng.standard_normal(2 * L).astype(np.float32)
    K = torch.empty(2 * L, device="cuda")
    f.conv_get_kernel(K, dev(h))
    wx, wh = O.conv_adjoint64(1, xs[:, :2 * L], h, gs[:, :2 * L])
    dx = torch.zeros(B, 2 * L + 4, device="cuda")
    f.conv_adjoint_batch(dx, None, dev(gs), dev(xs), K)
    assert O.rel_l2(host(dx)[:, :2 * L], wx) <= tol(1, L)
    assert np.all(host(dx)[:, 2 * L:] == 0)
    dh = torch.empty(2 * L, device="cuda")
    f.conv_adjoint_batch(None, dh, dev(gs), dev(xs), K)
    assert O.rel_l2(host(dh), wh) <= tol(1, L)
    dx2, dh2 = torch.zeros(B, 2 * L + 4, device="cuda"), torch.empty(2 * L, device="cuda")
    f.conv_adjoint_batch(dx2, dh2, dev(gs), dev(xs), K)
    assert O.rel_l2(host(dx2)[:, :2 * L], wx) <= tol(1, L)
    assert np.all(host(dx2)[:, 2 * L:] == 0)
    assert O.rel_l2(host(dh2), wh) <= tol(1, L)
    one_dx, one_dh = torch.empty(2 * L, device="cuda"), torch.empty(2 * L, device="cuda")
    f.conv_adjoint_batch(one_dx, one_dh, dev(gs[0, :2 * L]), dev(xs[0, :2 * L]), K)
    w1x, w1h = O.conv_adjoint64(1, xs[:1, :2 * L], h, gs[:1, :2 * L])
    assert O.rel_l2(host(one_dx), w1x[0]) <= tol(1, L)
    assert O.rel_l2(host(one_dh), w1h) <= tol(1, L)
    z = torch.full((2 * L,), 5.0, device="cuda")
    f.conv_adjoint_batch(None, z, dev(gs[:0]), dev(xs[:0]), K)
    assert np.all(host(z) == 0)


def test_adjoint_rejects_host_buffers(fftset_lib, gpu_set):
    import torch
    f = gpu_set.create_fft(1, 96)
    K = torch.zeros(192, device="cuda")
    g = np.zeros((2, 192), np.float32)
    with pytest.raises(fftset_lib.FftsetError):
        f.conv_adjoint_batch(None, torch.empty(192, device="cuda"), g, torch.zeros(2, 192, device="cuda"), K)


def test_adjoint_matches_reference_gradients(gpu_set):
    """Gradients built from the unmodified reference's CPU convolution with
    time-reversed kernels (tests/golden/make_golden_adjoint.py)."""
    import os
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_adjoint_vw4.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in gold.files})
    assert len(keys) >= 6
    for key in keys:
        mod, L = int(key.split("_")[0][1:]), int(key.split("_")[1][1:])
        f = gpu_set.create_fft(mod, L)
        x, h, g = gold[key + "_x"], gold[key + "_h"], gold[key + "_g"]
        dx, dh = adjoint(f, dev(g), dev(x), dev(h))
        assert O.rel_l2(dx, gold[key + "_dx"]) <= tol(mod, L), key
        assert O.rel_l2(dh, gold[key + "_dh"]) <= tol(mod, L), key


def test_differentiable_conv_4096_x2048(gpu_set):
    """FREQ_OFFSET_REAL conv at 4096 bins, batch 2048, Gaussian input,
    decaying-Gaussian 8192-tap kernel, loss = sum w*y with w ~ N(0,1):
    autograd through the hand-written adjoint."""
    import torch
    from fftset_autograd import ConvFn
    L, B = 4096, 2048
    N = 2 * L
    f = gpu_set.create_fft(1, L)
    x = np.random.default_rng(7).standard_normal((B, N)).astype(np.float32)
    h = (np.random.default_rng(8).standard_normal(N) * np.exp(-np.arange(N) / 1000.0)).astype(np.float32)
    w = np.random.default_rng(9).standard_normal((B, N)).astype(np.float32)
    xt = dev(x).requires_grad_(True)
    ht = dev(h).requires_grad_(True)
    y = ConvFn.apply(xt, ht, f)
    loss = (y * dev(w)).sum()
    loss.backward()
    gx, gh = host(xt.grad), host(ht.grad)

    # FP64 adjoint (exact gradient)
    wx, wh = O.conv_adjoint64(1, x, h, w)
    assert O.rel_l2(gx, wx) <= tol(1, L)
    assert O.rel_l2(gh, wh) <= tol(1, L)

    # FP64 central finite differences, 64 sampled coordinates each
    eps = 1e-3
    rng = np.random.default_rng(10)
    xb, xn = rng.integers(0, B, 64), rng.integers(0, N, 64)
    fd_x = np.empty(64)
    for i, (b, n) in enumerate(zip(xb, xn)):
        xp = x[b].astype(np.float64)
        xm = xp.copy()
        xp[n] += eps
        xm[n] -= eps
        # only block b depends on x_b
        fd_x[i] = (np.dot(w[b], O.conv64(1, xp, h)) - np.dot(w[b], O.conv64(1, xm, h))) / (2 * eps)
    assert O.rel_l2(gx[xb, xn], fd_x) <= tol(1, L)
    # taps: y(h +- eps e_j) = y(h) +- eps conv(x, e_j), conv(x, e_j) = L * (x
    # shifted negacyclically by j); the loss is evaluated in FP64 at both points
    y0 = O.conv64(1, x, h)
    l0 = np.sum(w.astype(np.float64) * y0)
    hj = rng.integers(0, N, 64)
    fd_h = np.empty(64)
    for i, j in enumerate(hj):
        s = np.roll(x.astype(np.float64), j, axis=1)
        s[:, :j] *= -1
        d = L * np.sum(w * s)
        fd_h[i] = ((l0 + eps * d) - (l0 - eps * d)) / (2 * eps)
    assert O.rel_l2(gh[hj], fd_h) <= tol(1, L)

    # gradients built from the oracle's C restatement of the reference conv
    P = O.PortPlan(1, L)
    ref_dx = P.conv(w, P.get_kernel(O.negacyclic_reverse(h).astype(np.float32)))
    assert O.rel_l2(gx, ref_dx) <= tol(1, L)
    xr = O.negacyclic_reverse(x).astype(np.float32)
    ref_dh = np.zeros(N)
    for b in range(B):
        ref_dh += P.conv(w[b], P.get_kernel(xr[b]))
    assert O.rel_l2(gh, ref_dh) <= tol(1, L)
