"""The GPU planner's host functions (fftset_gb300/csrc/fgk_plan.c) through the
library's exported symbols, on the CPU: radix chains for every supported
size, and the two- and three-level splits that the tile tasks of sizes
beyond the shared-memory limit rely on. No GPU calls."""
import ctypes as C
import math

import pytest

from oracle import oracle as O

CODELETS = {2, 3, 4, 5, 6, 8, 9, 10, 12, 15, 16}
MAX_STAGES = 24
SMEM = 232448 - 1024


@pytest.fixture(scope="module")
def lib(fftset_lib):
    return fftset_lib.library()


def _chain(lib, L):
    rad = (C.c_uint32 * MAX_STAGES)()
    n = C.c_uint32(0)
    rc = lib.fgk_plan_chain(C.c_uint32(L), rad, C.byref(n))
    return rc, [rad[i] for i in range(n.value)]


def test_chains_of_every_size_to_65536(lib):
    sizes = O.valid_sizes(2, 65536)
    assert len(sizes) == 164  # 2^a 3^b 5^{0,1} in [2, 65536]
    for L in sizes:
        rc, rad = _chain(lib, L)
        assert rc == 0, L
        assert 0 < len(rad) <= MAX_STAGES, (L, rad)
        assert math.prod(rad) == L, (L, rad)
        assert set(rad) <= CODELETS, (L, rad)
        assert rad == sorted(rad, reverse=True), (L, rad)  # widest radix first


def test_chains_refuse_unsupported_sizes(lib):
    for L in (7, 11, 25, 49, 75, 14, 2 * 3 * 7):
        rc, _ = _chain(lib, L)
        assert rc != 0, L


def _split(lib, fn, L, *extra):
    buf = (C.c_uint32 * 8192)()  # larger than either plan struct; only the leading fields are read
    rc = fn(buf, C.c_uint32(L), C.c_uint32(1), *extra)
    return rc, list(buf[:3])


@pytest.mark.parametrize("L", [s for s in O.valid_sizes(26245, 65536)])
def test_two_level_splits(lib, L):
    """Sizes above the resident limit up to 65536 bins: L = L1 L2, the most
    balanced split; the tile tasks need both factors <= 256."""
    rc, (L1, L2, _) = _split(lib, lib.fgk_plan_fourstep, L, C.c_uint32(SMEM))
    assert rc == 0
    assert L1 * L2 == L
    assert 2 <= L1 <= 256 and 2 <= L2 <= 256, (L1, L2)


@pytest.mark.parametrize("L", [65536 * 2, 65536 * 3, 393216, 1 << 20, 3 ** 11, 15728640, 1 << 24])
def test_three_level_splits(lib, L):
    """Sizes beyond 65536 bins: L = L1 L2 L3 with L1 in [16, 256] (pass A
    tiles of 16 lanes) and L2, L3 in [2, 256]."""
    if not O.valid_size(L):
        pytest.skip("not a supported size")
    rc, (L1, L2, L3) = _split(lib, lib.fgk_plan_threestep, L)
    assert rc == 0
    assert L1 * L2 * L3 == L
    assert 16 <= L1 <= 256 and 2 <= L2 <= 256 and 2 <= L3 <= 256, (L1, L2, L3)
    for f in (L1, L2, L3):
        rc, rad = _chain(lib, f)
        assert rc == 0 and math.prod(rad) == f
