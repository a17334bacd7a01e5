"""The oracle pinned against the reference: golden outputs of the unmodified
reference (tests/golden, made by tests/golden/make_golden.py), the
reference's own known-answer tests (app_fftset_test/fftset_test.c) and the
FP64 definitions. CPU only."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O

CASES = [(m, L) for m in (0, 1) for L in O.REFERENCE_TEST_LENGTHS] + [(0, 1024), (1, 1536), (1, 4096)]


def _g(golden, mod, L, what):
    return golden[f"m{mod}_L{L}_{what}"]


@pytest.mark.parametrize("mod,L", CASES)
def test_port_matches_reference_outputs(golden_outputs, mod, L):
    g = golden_outputs
    x, h = _g(g, mod, L, "x"), _g(g, mod, L, "h")
    P = O.PortPlan(mod, L, 4)
    K = P.get_kernel(h)
    assert O.rel_l2(K, _g(g, mod, L, "kern")) < 1e-6
    assert O.rel_l2(P.conv(x, _g(g, mod, L, "kern")), _g(g, mod, L, "conv")) < 2e-6
    assert O.rel_l2(P.forward(x), _g(g, mod, L, "fwd")) < 2e-6
    assert O.rel_l2(P.inverse(_g(g, mod, L, "fwd")), _g(g, mod, L, "inv")) < 2e-6


@pytest.mark.parametrize("mod,L", CASES)
def test_fp64_oracle_matches_reference_outputs(golden_outputs, mod, L):
    g = golden_outputs
    x, h = _g(g, mod, L, "x"), _g(g, mod, L, "h")
    tol = O.tolerance(2 * L if mod else L)
    assert O.rel_l2(_g(g, mod, L, "fwd"), O.forward64(mod, x)) < tol
    assert O.rel_l2(_g(g, mod, L, "inv"), O.inverse64(mod, _g(g, mod, L, "fwd"))) < tol
    assert O.rel_l2(_g(g, mod, L, "conv"), O.conv64(mod, x, h)) < tol
    W = O.spectrum_from_kernel(mod, _g(g, mod, L, "kern"), 4)
    assert O.rel_l2(np.concatenate([W.real, W.imag]),
                    np.concatenate([O.spectrum64(mod, h).real, O.spectrum64(mod, h).imag])) < tol


@pytest.mark.parametrize("vw", [1, 4, 8])
def test_oracle_layout_matches_reference(golden_layouts, vw):
    n = 0
    for key in golden_layouts.files:
        if not key.startswith(f"vw{vw}_"):
            continue
        _, m, l = key.split("_")
        mod, L = int(m[1:]), int(l[1:])
        off, V = O.kernel_offsets(mod, L, vw)
        assert np.array_equal(off, golden_layouts[key]), key
        n += 1
    assert n > 100


def test_oracle_layout_hashes_large(golden_layouts):
    g = golden_layouts
    for vw, mod, L, V, sha in zip(g["large_vw"], g["large_mod"], g["large_L"], g["large_V"], g["large_sha256"]):
        off, v = O.kernel_offsets(int(mod), int(L), int(vw))
        assert v == V
        assert hashlib.sha256(np.ascontiguousarray(off, np.int64).tobytes()).hexdigest() == sha, (vw, mod, L)


def test_oracle_layout_hashes_beyond_65536():
    g = np.load(os.path.join(GOLDEN, "ref_layouts_beyond.npz"))
    for vw, mod, L, V, sha in zip(g["vw"], g["mod"], g["L"], g["V"], g["sha256"]):
        off, v = O.kernel_offsets(int(mod), int(L), int(vw))
        assert v == V
        assert hashlib.sha256(np.ascontiguousarray(off, np.int64).tobytes()).hexdigest() == sha, (vw, mod, L)


def test_negacyclic_definition():
    rng = np.random.default_rng(5)
    x, h = rng.standard_normal(24), rng.standard_normal(24)
    assert O.rel_l2(O.negacyclic_conv64(x, h), O.negacyclic_direct64(x, h)) < 1e-12
    assert O.rel_l2(O.freqoff_forward64(x), O.freqoff_direct64(x)) < 1e-12


# --- the reference's own known-answer tests, run on the port (fftset_test.c) ---
@pytest.mark.parametrize("L", O.REFERENCE_TEST_LENGTHS)
def test_reference_kat_freqoff_impulse(L):
    """fftset_test.c:70-156: prime impulse, RMS <= 4e-6 fwd, 1e-6 inverse."""
    N = 2 * L
    x = O.prime_flags(N).astype(np.float32)
    P = O.PortPlan(1, L, 4)
    X = P.forward(x)
    ref = O.freqoff_direct64(x)
    err = X.astype(np.float64) - ref
    assert np.sqrt((err[0::2] ** 2 + err[1::2] ** 2).sum() / L) <= 4e-6
    r = P.inverse(X) / L - x
    assert np.sqrt((r ** 2).sum() / L) <= 1e-6


@pytest.mark.parametrize("L", O.REFERENCE_TEST_LENGTHS)
def test_reference_kat_conv(L):
    """fftset_test.c:158-222: prime trains, pair-count histogram, RMS <= 1e-5."""
    N = 2 * L
    flags = O.prime_flags(N)
    h = np.where(flags & (np.arange(N) < N // 4), 2.0 / N, 0.0).astype(np.float32)
    x = np.where(flags & (np.arange(N) < 3 * N // 4), 1.0, 0.0).astype(np.float32)
    P = O.PortPlan(1, L, 4)
    y = P.conv(x, P.get_kernel(h))
    exp = np.zeros(N)
    pi = np.nonzero(flags & (np.arange(N) < 3 * N // 4))[0]
    pj = np.nonzero(flags & (np.arange(N) < N // 4))[0]
    for a in pi:
        for b in pj:
            exp[a + b] += 1.0
    assert np.sqrt(((exp - y) ** 2).sum() / L) <= 1e-5


@pytest.mark.parametrize("L", O.REFERENCE_TEST_LENGTHS)
def test_reference_kat_complex_impulse(L):
    """fftset_test.c:224-314: primes on re/im slots, RMS <= 4e-6 / 1e-6."""
    x = O.prime_flags(2 * L).astype(np.float32)
    P = O.PortPlan(0, L, 4)
    X = P.forward(x)
    err = X.astype(np.float64) - O.complex_forward64(x)
    assert np.sqrt((err[0::2] ** 2 + err[1::2] ** 2).sum() / L) <= 4e-6
    r = P.inverse(X) / L - x
    assert np.sqrt((r[:L] ** 2).sum() / L) <= 1e-6


def test_recommend_conv_length_reference_values(golden_layouts):
    """Checked against the product implementation in test_abi.py."""
    rec = golden_layouts["recommend"]
    assert rec.shape[1] == 3 and len(rec) > 50


def test_fp64_adjoint_against_finite_differences():
    """oracle.conv_adjoint64 is the gradient of sum_b <g_b, conv64(x_b, h)>
    (both modulations; COMPLEX data as interleaved reals)."""
    rng = np.random.default_rng(3)
    for mod in (0, 1):
        L = 10
        x, g = rng.standard_normal((2, 2 * L)), rng.standard_normal((2, 2 * L))
        h = rng.standard_normal(2 * L)
        dx, dh = O.conv_adjoint64(mod, x, h, g)

        def loss(xx, hh):
            return float(np.sum(g * O.conv64(mod, xx, hh[None, :])))

        eps = 1e-6
        fx = np.zeros_like(x)
        fh = np.zeros_like(h)
        for b in range(2):
            for n in range(2 * L):
                e = np.zeros_like(x)
                e[b, n] = eps
                fx[b, n] = (loss(x + e, h) - loss(x - e, h)) / (2 * eps)
        for n in range(2 * L):
            e = np.zeros_like(h)
            e[n] = eps
            fh[n] = (loss(x, h + e) - loss(x, h - e)) / (2 * eps)
        assert O.rel_l2(dx, fx) <= 1e-7
        assert O.rel_l2(dh, fh) <= 1e-7


def test_fp64_adjoint_against_reference_gradients():
    """The FP64 adjoint against gradients built from the unmodified
    reference's CPU convolution with time-reversed kernels
    (tests/golden/ref_adjoint_vw4.npz)."""
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_adjoint_vw4.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in gold.files})
    for key in keys:
        mod, L = int(key.split("_")[0][1:]), int(key.split("_")[1][1:])
        dx, dh = O.conv_adjoint64(mod, gold[key + "_x"], gold[key + "_h"], gold[key + "_g"])
        assert O.rel_l2(gold[key + "_dx"], dx) <= O.tolerance(2 * L if mod else L), key
        assert O.rel_l2(gold[key + "_dh"], dh) <= O.tolerance(2 * L if mod else L), key
        # and the oracle's C restatement reproduces the reference gradient
        P = O.PortPlan(mod, L, 4)
        rx = P.conv(gold[key + "_g"], P.get_kernel(O.reverse(mod, gold[key + "_h"]).astype(np.float32)))
        assert O.rel_l2(rx, gold[key + "_dx"]) <= O.tolerance(2 * L if mod else L), key
