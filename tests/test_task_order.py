"""The task order of three-level items (fftset_gb300/csrc/fftset_ragged.c,
fsr_list_huge) through a test hook, on the CPU. The task kernel claims
tasks in list order and a tile may wait only for tiles listed before it:
a B tile for the A tiles of its n3 group (all A tiles when 16 does not
divide L3), a C tile for the B tiles of its 16 k1. These tests check, for
the splits the planner makes, that every tile is listed once, that each
wait's tiles come before the waiting tile (no wait can depend on a tile
not yet claimed), and that the counts the kernel waits for (L2 A tiles
per n3 group, min(4, ceil(L1/4) - 4 g) ceil(L3/4) B tiles per k1 group g)
are the tiles listed for that group. No GPU calls."""
import ctypes as C

import pytest

from oracle import oracle as O

PA, PB, PC = 3, 4, 5  # enum fgk_task_kind


class Task(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("ref", C.c_uint32), ("a", C.c_uint32), ("b", C.c_uint32)]


@pytest.fixture(scope="module")
def lib(fftset_lib):
    L_ = fftset_lib.library()
    L_.fftset__test_list_huge.restype = C.c_uint32
    L_.fftset__test_list_huge.argtypes = [C.c_uint32] * 3 + [C.c_int, C.c_int, C.c_uint32, C.c_uint32,
                                                            C.POINTER(Task), C.c_uint32]
    return L_


def _split(lib, L):
    buf = (C.c_uint32 * 8192)()
    assert lib.fgk_plan_threestep(buf, C.c_uint32(L), C.c_uint32(1)) == 0
    return buf[0], buf[1], buf[2]


def _listing(lib, L1, L2, L3, zip_in, zip_out, grid, dist):
    na = (L2 * L3 + 15) // 16
    nb = (L1 + 3) // 4 * ((L3 + 3) // 4)
    nc = (L1 + 15) // 16 * L2
    cap = na + nb + nc
    out = (Task * cap)()
    n = lib.fftset__test_list_huge(L1, L2, L3, zip_in, zip_out, grid, dist, out, cap)
    assert n == cap
    assert lib.fftset__test_list_huge(L1, L2, L3, zip_in, zip_out, grid, dist, out, cap - 1) == 0
    return [(t.kind, t.a) for t in out], na, nb, nc


# 131072 (4 n3 groups), 393216 (6), 327680 (5: an odd count), 1048576 (8),
# 15,728,640 (16), 177147 and 69984 (16 does not divide L3: one group)
SIZES = [131072, 393216, 327680, 1 << 20, 15728640, 3 ** 11, 69984]


@pytest.mark.parametrize("L", SIZES)
@pytest.mark.parametrize("zips", [(0, 0), (1, 0), (0, 1)])
@pytest.mark.parametrize("grid,dist", [(912, 0), (456, 0), (1, 0), (912, 1), (912, 2), (912, 1000)])
def test_three_level_order(lib, L, zips, grid, dist):
    assert O.valid_size(L)
    L1, L2, L3 = _split(lib, L)
    tasks, na, nb, nc = _listing(lib, L1, L2, L3, zips[0], zips[1], grid, dist)
    for kind, n in ((PA, na), (PB, nb), (PC, nc)):
        assert sorted(a for k, a in tasks if k == kind) == list(range(n)), kind
    U = L3 // 16 if L3 % 16 == 0 else 1
    nb3, L1q, nc1 = (L3 + 3) // 4, (L1 + 3) // 4, (L1 + 15) // 16
    pos = {t: i for i, t in enumerate(tasks)}
    # the kernel's group of each tile and the counts it waits for
    last_a, cnt_a = {}, {}
    for t in range(na):
        g = t % U
        last_a[g] = max(last_a.get(g, -1), pos[(PA, t)])
        cnt_a[g] = cnt_a.get(g, 0) + 1
    for g in range(U):
        assert cnt_a[g] == na // U
    last_b, cnt_b = {}, {}
    for t in range(nb):
        k1g, n3b = divmod(t, nb3)
        g = (4 * n3b) >> 4 if U > 1 else 0
        assert pos[(PB, t)] > last_a[g], ("B tile listed before an A tile it waits for", t)
        kg = k1g >> 2
        last_b[kg] = max(last_b.get(kg, -1), pos[(PB, t)])
        cnt_b[kg] = cnt_b.get(kg, 0) + 1
    for kg in range(nc1):
        assert cnt_b[kg] == min(4, L1q - 4 * kg) * nb3
    for t in range(nc):
        kg = t % nc1
        assert pos[(PC, t)] > last_b[kg], ("C tile listed before a B tile it waits for", t)
