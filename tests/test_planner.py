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


@pytest.mark.parametrize("mod", [0, 1])
@pytest.mark.parametrize("L", [32768, 59049, 65536, 131072, 177147, 393216, 1 << 20, 15728640, 1 << 24, 1 << 25,
                               3 ** 15])
def test_two_pass_tiles(lib, mod, L):
    """The tiles of the two-pass kernels (get_kernel beyond the resident
    limit, the fixed-scratch entry point, sizes beyond the three-level
    range): ping-pong tiles (emax 0, two buffers) wherever two buffers fit
    the shared memory, else in place (one buffer, emax 16 or 32); lane
    counts of at most 16, at least 2 for the FREQ_OFFSET_REAL passes that
    hold mirror rows (forward pass 2, inverse pass 1), threads a multiple
    of 32 up to 512."""
    if not O.valid_size(L):
        pytest.skip("not a supported size")
    buf = (C.c_uint32 * 8192)()
    assert lib.fgk_plan_fourstep(buf, C.c_uint32(L), C.c_uint32(mod), C.c_uint32(SMEM)) == 0
    L1, L2 = buf[0], buf[1]
    assert L1 * L2 == L
    for Lp, ls, T, slots, emax in ((L1, buf[3], buf[5], buf[7], buf[9]), (L2, buf[4], buf[6], buf[8], buf[10])):
        nl = 1 << ls
        assert ls <= 4 and (mod == 0 or ls >= 1), (Lp, ls)
        assert slots >= Lp * nl + (Lp * nl) // 16 + 1, (Lp, slots)
        assert 32 <= T <= 512 and T % 32 == 0, (Lp, T)
        if emax == 0:
            assert 2 * slots * 8 <= SMEM and slots % 4 == 0, (Lp, slots)
        else:
            assert emax in (16, 32) and slots * 8 <= SMEM, (Lp, emax, slots)
            # in place only where two buffers of the narrowest allowed tile do not fit
            nl_min = 2 if mod else 1
            assert 2 * (Lp * nl_min + (Lp * nl_min) // 16 + 1) * 8 > SMEM, (Lp, emax)
