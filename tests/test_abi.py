"""The C-ABI library on the CPU: it loads, exports every entry point the
public header declares, and its host-side logic (kernel-buffer layout,
recommended convolution length, size validation) matches the reference.
No kernel is launched here."""
import ctypes as C
import hashlib
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include"))) if h.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(fftset_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
        for m in re.finditer(r"extern\s+const\s+struct\s+\w+\s*\*\s*(FFTSET_\w+)\s*;", txt):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(fftset_lib):
    lib = fftset_lib.library()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_layout_matches_reference_small(fftset_lib, golden_layouts):
    n = 0
    for key in golden_layouts.files:
        if not key.startswith("vw"):
            continue
        vw, m, l = key.split("_")
        vw, mod, L = int(vw[2:]), int(m[1:]), int(l[1:])
        off, lanes = fftset_lib.kernel_layout(mod, L, vw)
        assert np.array_equal(np.array(off), golden_layouts[key]), key
        n += 1
    assert n > 300


def test_layout_matches_reference_large(fftset_lib, golden_layouts):
    g = golden_layouts
    for vw, mod, L, V, sha in zip(g["large_vw"], g["large_mod"], g["large_L"], g["large_V"], g["large_sha256"]):
        off, lanes = fftset_lib.kernel_layout(int(mod), int(L), int(vw))
        assert lanes == V
        assert hashlib.sha256(np.asarray(off, np.int64).tobytes()).hexdigest() == sha, (vw, mod, L)


def test_layout_matches_reference_beyond_65536(fftset_lib):
    """Sizes of two- and three-level splits (131072, 393216, 15,728,640 bins):
    layouts read off the reference itself (tests/golden/make_golden.py
    --beyond), widths 1, 4 and 8, both modulations."""
    g = np.load(os.path.join(GOLDEN, "ref_layouts_beyond.npz"))
    assert len(g["L"]) == 18
    for vw, mod, L, V, sha in zip(g["vw"], g["mod"], g["L"], g["V"], g["sha256"]):
        off, lanes = fftset_lib.kernel_layout(int(mod), int(L), int(vw))
        assert lanes == V
        assert hashlib.sha256(np.asarray(off, np.int64).tobytes()).hexdigest() == sha, (vw, mod, L)


def test_layout_rejects_unsupported_sizes(fftset_lib):
    for L in (0, 1, 7, 25, 50, 3 * 7 * 16, 2 * 25):
        with pytest.raises(ValueError):
            fftset_lib.kernel_layout(1, L, 4)


def test_recommend_conv_length(fftset_lib, golden_layouts):
    for k, b, want in golden_layouts["recommend"]:
        assert fftset_lib.recommend_conv_length(int(k), int(b)) == int(want), (k, b)


def test_error_strings(fftset_lib):
    for code in range(5):
        assert fftset_lib.error_string(code)


def test_null_handles_are_rejected(fftset_lib):
    lib = fftset_lib.library()
    assert lib.fftset_create_fft(None, fftset_lib.MODULATION_COMPLEX, 16) is None
    assert lib.fftset_fft_bins(None) == 0
    # execution calls on a NULL plan return without touching buffers
    lib.fftset_fft_forward(None, None, None, None)
    assert lib.fftset_fft_forward_batch(None, None, 0, None, 0, 1) != 0


def test_init_without_gpu_fails_cleanly(fftset_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s = fftset_lib._FftsetStruct()
    assert fftset_lib.library().fftset_init(C.byref(s)) != 0
