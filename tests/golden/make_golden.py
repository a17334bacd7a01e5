"""Generate tests/golden fixtures by running the UNMODIFIED reference fftset,
compiled here against the cop stand-in (oracle/Makefile `ref` target).

    python tests/golden/make_golden.py

Writes
  ref_outputs_vw4.npz  seeded inputs and the reference's forward / inverse /
                       get_kernel / conv outputs (SIMD width 4 build) for the
                       sizes of app_fftset_test/fftset_test.c:327-346 plus the
                       headline sizes (COMPLEX 1024, FREQ_OFFSET_REAL 1536 and
                       4096).
  ref_layouts.npz      kernel-buffer layout (float offset of the real part of
                       each bin) for every size in 2..4096 with a plan, both
                       modulations, SIMD widths 1, 4 and 8, plus a sha256 of the
                       layout for every 2^a 3^b 5^{0,1} size in 4097..65536.
  ref_layouts_beyond.npz  the same sha256 for the sizes beyond 65536 bins
                       that the GPU tests run (two- and three-level splits):
                       131072, 393216 and 15,728,640 bins.

    python tests/golden/make_golden.py --beyond   (only ref_layouts_beyond.npz)
The layout is read off the reference itself: a kernel input whose
modulated sequence is a unit impulse at index 1 has spectrum
W[k] = e^{-j 2 pi k / L}, so the phase of each kernel-buffer slot names its bin.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

HEADLINE = [(O.MOD_COMPLEX, 1024), (O.MOD_FREQ_OFFSET_REAL, 1536), (O.MOD_FREQ_OFFSET_REAL, 4096)]


def seeded(mod, L, what):
    rng = np.random.default_rng([int(mod), int(L), {"x": 1, "h": 2}[what]])
    return rng.standard_normal(2 * L).astype(np.float32)


def layout_from_reference(R: O.Reference, mod: int, L: int, V: int) -> np.ndarray:
    h = np.zeros(2 * L, np.float64)
    if mod == O.MOD_COMPLEX:
        h[2] = 1.0                                  # x[1] = 1
    else:
        a = np.pi / (2.0 * L)                       # c[1] = conj(z[1]) e^{-j a} = 1
        h[1] = np.cos(a)
        h[L + 1] = -np.sin(a)
    K = R.get_kernel(mod, L, h.astype(np.float32)).astype(np.float64)
    M = L // V
    off = np.empty(L, np.int64)
    seen = np.zeros(L, bool)
    for s in range(M):
        for lane in range(V):
            re = K[2 * V * s + lane]
            im = K[2 * V * s + V + lane]
            k = int(np.rint(-np.arctan2(im, re) * L / (2 * np.pi))) % L
            assert not seen[k], (mod, L, V, s, lane, k)
            seen[k] = True
            off[k] = 2 * V * s + lane
    assert seen.all()
    return off


def layout_hash(off: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(off, np.int64).tobytes()).hexdigest()


BEYOND = [131072, 393216, 15728640]


def layout_from_reference_fast(R: O.Reference, mod: int, L: int, V: int) -> np.ndarray:
    """layout_from_reference, vectorised for large L: the same impulse, the
    same reading of each slot's phase as its bin, and the same check that
    the slots form a permutation of the bins (at 15,728,640 bins the bins
    are 4e-7 rad apart, well above the float32 phase error of the slots)."""
    h = np.zeros(2 * L, np.float64)
    if mod == O.MOD_COMPLEX:
        h[2] = 1.0
    else:
        a = np.pi / (2.0 * L)
        h[1] = np.cos(a)
        h[L + 1] = -np.sin(a)
    K = R.get_kernel(mod, L, h.astype(np.float32)).astype(np.float64).reshape(L // V, 2, V)
    slot_re = (2 * V * np.arange(L // V)[:, None] + np.arange(V)[None, :]).ravel()
    k = np.rint(-np.arctan2(K[:, 1, :].ravel(), K[:, 0, :].ravel()) * L / (2 * np.pi)).astype(np.int64) % L
    assert np.all(np.bincount(k, minlength=L) == 1), (mod, L, V)
    off = np.empty(L, np.int64)
    off[k] = slot_re
    return off


def beyond(refs):
    rows = []
    for vw in (1, 4, 8):
        for mod in (O.MOD_COMPLEX, O.MOD_FREQ_OFFSET_REAL):
            for L in BEYOND:
                V = O.port().oracle_lane_width(mod, L, vw)
                off = layout_from_reference_fast(refs[vw], mod, L, V)
                rows.append((vw, mod, L, V, layout_hash(off)))
    np.savez_compressed(os.path.join(HERE, "ref_layouts_beyond.npz"),
                        vw=np.array([r[0] for r in rows], np.int64), mod=np.array([r[1] for r in rows], np.int64),
                        L=np.array([r[2] for r in rows], np.int64), V=np.array([r[3] for r in rows], np.int64),
                        sha256=np.array([r[4] for r in rows]))
    print("wrote", len(rows), "layout hashes beyond 65536 bins")


def main():
    if "--beyond" in sys.argv:
        if not O.build_reference():
            raise SystemExit("reference sources not present; fixtures cannot be regenerated here")
        beyond({vw: O.Reference(vw) for vw in (1, 4, 8)})
        return
    if not O.build_reference():
        raise SystemExit("reference sources not present; fixtures cannot be regenerated here")
    refs = {vw: O.Reference(vw) for vw in (1, 4, 8)}

    # ---- outputs (width-4 build) ----
    R = refs[4]
    out = {}
    cases = [(m, L) for m in (O.MOD_COMPLEX, O.MOD_FREQ_OFFSET_REAL) for L in O.REFERENCE_TEST_LENGTHS] + HEADLINE
    for mod, L in cases:
        x = seeded(mod, L, "x")
        h = seeded(mod, L, "h")
        fwd = R.forward(mod, L, x)
        inv = R.inverse(mod, L, fwd, in_place=True)
        K = R.get_kernel(mod, L, h)
        y = R.conv(mod, L, x, K)
        key = f"m{mod}_L{L}"
        out[key + "_x"] = x
        out[key + "_h"] = h
        out[key + "_fwd"] = fwd
        out[key + "_inv"] = inv
        out[key + "_kern"] = K
        out[key + "_conv"] = y
    out["cases"] = np.array(cases, np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_outputs_vw4.npz"), **out)

    # ---- layouts ----
    lay = {}
    small = O.valid_sizes(2, 4096)
    large = O.valid_sizes(4097, 65536)
    hashes = []
    for vw in (1, 4, 8):
        for mod in (O.MOD_COMPLEX, O.MOD_FREQ_OFFSET_REAL):
            for L in small + large:
                V = O.port().oracle_lane_width(mod, L, vw)
                off = layout_from_reference(refs[vw], mod, L, V)
                if L <= 4096:
                    lay[f"vw{vw}_m{mod}_L{L}"] = off.astype(np.int32)
                else:
                    hashes.append((vw, mod, L, V, layout_hash(off)))
    lay["large_vw"] = np.array([h[0] for h in hashes], np.int64)
    lay["large_mod"] = np.array([h[1] for h in hashes], np.int64)
    lay["large_L"] = np.array([h[2] for h in hashes], np.int64)
    lay["large_V"] = np.array([h[3] for h in hashes], np.int64)
    lay["large_sha256"] = np.array([h[4] for h in hashes])
    lay["recommend"] = np.array([[k, b, R.recommend_conv_length(k, b)]
                                 for k in (1, 2, 3, 7, 16, 31, 64, 100, 255, 256, 1000, 3000, 4096)
                                 for b in (0, 1, 64, 100, 512, 4096, 10000)], np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_layouts.npz"), **lay)
    print("wrote", len(out), "output arrays and", len(lay), "layout arrays")


if __name__ == "__main__":
    main()
