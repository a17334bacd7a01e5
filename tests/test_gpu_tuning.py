"""Persistent autotune results (fftset_tuning_save / fftset_tuning_load):
the kernel chosen per op and the ragged task schedules survive a round trip
into a fresh fftset, results stay correct with the loaded choices, and files
from another device model or malformed files are refused."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _records(path):
    with open(path) as fp:
        return sorted(line.strip() for line in fp if line.startswith(("fft ", "ragged ")))


def _ragged_case(fs):
    bins = [60, 96, 243, 1536, 5120, 4096, 19683]
    offs, o = [], 0
    for L in bins:
        offs.append(o)
        o += 2 * L
    return bins, offs, o


def test_tuning_round_trip(fftset_lib, tmp_path):
    import torch
    fs = fftset_lib
    S = fs.FftSet()
    f = S.create_fft(fs.FREQ_OFFSET_REAL, 1536)
    f.set_variant(fs.OP_CONV, 2)
    # the last compiled variant that implements the forward transform (not
    # the default, which is the first)
    v_fwd = None
    for v in range(f.variants - 1, 0, -1):
        try:
            f.set_variant(fs.OP_FORWARD, v)
        except fs.FftsetError:
            continue
        v_fwd = v
        break
    assert v_fwd is not None
    g = S.create_fft(fs.COMPLEX, 1024)
    g.autotune(fs.OP_FORWARD, 512)
    bins, offs, n = _ragged_case(fs)
    rb = fs.Ragged(S, fs.COMPLEX, fs.OP_FORWARD, bins, offs, offs)
    rb.autotune()
    p = str(tmp_path / "tuning.txt")
    S.save_tuning(p)
    recs = _records(p)
    assert any(r.startswith("ragged 0 19683 ") for r in recs)
    assert any(r.startswith("fft 1 1536 ") for r in recs)

    T = fs.FftSet()
    T.load_tuning(p)
    f2 = T.create_fft(fs.FREQ_OFFSET_REAL, 1536)
    assert f2.variant(fs.OP_CONV) == 2 and f2.variant(fs.OP_FORWARD) == v_fwd
    g2 = T.create_fft(fs.COMPLEX, 1024)
    assert g2.variant(fs.OP_FORWARD) == g.variant(fs.OP_FORWARD)
    p2 = str(tmp_path / "again.txt")
    T.save_tuning(p2)
    assert _records(p2) == recs

    # the loaded schedules and kernels compute the same transforms
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    rb2 = fs.Ragged(T, fs.COMPLEX, fs.OP_FORWARD, bins, offs, offs)
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    rb2.execute(y, xd)
    torch.cuda.synchronize()
    T.check()
    yh = y.cpu().numpy()
    for L, o in zip(bins, offs):
        want = O.forward64(0, x[o:o + 2 * L])
        assert O.rel_l2(yh[o:o + 2 * L], want) <= O.tolerance(L)
    xb = rng.standard_normal((300, 3072)).astype(np.float32)
    h = rng.standard_normal(3072).astype(np.float32)
    K = torch.empty(3072, device="cuda")
    f2.conv_get_kernel(K, torch.from_numpy(h).cuda())
    yb = torch.empty(300, 3072, device="cuda")
    f2.conv_batch(yb, torch.from_numpy(xb).cuda(), K)
    torch.cuda.synchronize()
    assert O.rel_l2(yb.cpu().numpy(), O.conv64(1, xb, h)) <= O.tolerance(3072)
    rb.close()
    rb2.close()
    S.close()
    T.close()


def test_tuning_refuses_other_device_and_bad_files(fftset_lib, tmp_path):
    fs = fftset_lib
    S = fs.FftSet()
    f = S.create_fft(fs.FREQ_OFFSET_REAL, 1536)
    f.set_variant(fs.OP_CONV, 1)
    p = tmp_path / "tuning.txt"
    S.save_tuning(str(p))
    lines = p.read_text().splitlines()
    assert lines[0] == "fftset-tuning 1" and lines[1].startswith("device ")

    T = fs.FftSet()
    other = tmp_path / "other.txt"
    other.write_text("\n".join([lines[0], "device 7 Some Other GPU"] + lines[2:]) + "\n")
    with pytest.raises(fs.FftsetError, match="unsupported"):
        T.load_tuning(str(other))
    # nothing was applied: the 1536 plan keeps its default conv kernel
    assert T.create_fft(fs.FREQ_OFFSET_REAL, 1536).variant(fs.OP_CONV) == 0

    bad_cases = [
        "not a tuning file\n",
        lines[0] + "\n",                                           # no device line
        "\n".join(lines[:2] + ["fft 1 1536 -1 -1 -1 99 -1"]) + "\n",  # variant out of range
        "\n".join(lines[:2] + ["fft 3 1536 0 0 0 0 0"]) + "\n",     # unknown modulation
        "\n".join(lines[:2] + ["ragged 0 243 2 9 9 64 0 0"]) + "\n",  # radices do not multiply to L
        "\n".join(lines[:2] + ["ragged 0 243 0 48 0 0"]) + "\n",    # threads not a multiple of 32
        "\n".join(lines[:2] + ["bogus 1 2 3"]) + "\n",
    ]
    for k, text in enumerate(bad_cases):
        q = tmp_path / f"bad{k}.txt"
        q.write_text(text)
        with pytest.raises(fs.FftsetError):
            T.load_tuning(str(q))
    with pytest.raises(fs.FftsetError):
        T.load_tuning(str(tmp_path / "missing.txt"))
    S.close()
    T.close()


def test_ragged_closed_with_its_fftset(fftset_lib):
    """Closing an FftSet first destroys the ragged batches still open on it
    (their plans go with the fftset), so a batch collected afterwards is a
    no-op rather than a use of freed memory."""
    fs = fftset_lib
    S = fs.FftSet()
    rb = fs.Ragged(S, fs.COMPLEX, fs.OP_FORWARD, [64, 5120], [0, 128], [0, 128])
    S.close()
    assert rb.h is None
    rb.close()
    del rb
