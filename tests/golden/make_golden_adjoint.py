"""Generate tests/golden/ref_adjoint_vw4.npz: reference gradients of the
batched convolution, built from the UNMODIFIED reference fftset (compiled
here against the cop stand-in, oracle/Makefile `ref` target, SIMD width 4).

    python tests/golden/make_golden_adjoint.py

For y_b = fftset_fft_conv(x_b, get_kernel(h)) and the loss sum_b <g_b, y_b>
the reference itself has no gradient; it is built from the reference's own
convolution with time-reversed kernels (the reversal whose spectrum is the
conjugate: h'[0] = h[0], h'[k] = -h[N-k] for FREQ_OFFSET_REAL,
h*[k] = conj h[-k] for COMPLEX):
    dx_b = conv_ref(g_b, get_kernel_ref(h'))
    dh   = sum_b conv_ref(g_b, get_kernel_ref(x_b'))
Stored per case: x, h, g (seeded float32 Gaussian, the kernel taps decaying
like exp(-t/(N/8))), dx, dh.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

CASES = [(O.MOD_FREQ_OFFSET_REAL, 96, 3), (O.MOD_FREQ_OFFSET_REAL, 1536, 2), (O.MOD_FREQ_OFFSET_REAL, 4096, 2),
         (O.MOD_FREQ_OFFSET_REAL, 243, 2), (O.MOD_COMPLEX, 64, 3), (O.MOD_COMPLEX, 1024, 2)]


def inputs(mod, L, B):
    rng = np.random.default_rng([int(mod), int(L), 77])
    N = 2 * L
    x = rng.standard_normal((B, N)).astype(np.float32)
    h = (rng.standard_normal(N) * np.exp(-np.arange(N) / (N / 8))).astype(np.float32)
    g = rng.standard_normal((B, N)).astype(np.float32)
    return x, h, g


def main():
    assert O.build_reference() or O.reference_available(4), "the reference sources are needed"
    R = O.Reference(4)
    out = {}
    for mod, L, B in CASES:
        x, h, g = inputs(mod, L, B)
        rev = (lambda a: O.reverse(mod, a).astype(np.float32))
        Kh = R.get_kernel(mod, L, rev(h))
        dx = R.conv(mod, L, g, Kh)
        dh = np.zeros(2 * L, np.float64)
        for b in range(B):
            dh += R.conv(mod, L, g[b], R.get_kernel(mod, L, rev(x[b]))).astype(np.float64)
        key = f"m{mod}_L{L}"
        out[key + "_x"], out[key + "_h"], out[key + "_g"] = x, h, g
        out[key + "_dx"], out[key + "_dh"] = dx.astype(np.float32), dh.astype(np.float32)
        dx64, dh64 = O.conv_adjoint64(mod, x, h, g)
        print(key, "B", B, "ref vs fp64: dx", O.rel_l2(dx, dx64), "dh", O.rel_l2(dh, dh64))
    np.savez_compressed(os.path.join(HERE, "ref_adjoint_vw4.npz"), **out)


if __name__ == "__main__":
    main()
