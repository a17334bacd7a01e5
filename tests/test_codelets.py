"""The register DFT codelets (fftset_gb300/csrc/fgk_codelets.cuh) on the
host: the header compiles as plain C++, and every radix is checked against
a direct FP64 DFT (tests/native/codelet_check.cpp); the lean-table helpers
(twiddles formed from four table entries, compile-time modulation steps)
against FP64 (tests/native/lean_tables_check.cpp). No GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fftset_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_codelets_match_fp64_dft(tmp_path):
    exe = str(tmp_path / "codelet_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "codelet_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    radices = {int(line.split()[0]): float(line.split()[1]) for line in r.stdout.split("\n") if line.strip()}
    assert sorted(radices) == [2, 3, 4, 5, 6, 8, 9, 10, 12, 15, 16]
    assert r.returncode == 0, r.stdout
    assert max(radices.values()) < 1e-6


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_lean_tables_match_fp64(tmp_path):
    exe = str(tmp_path / "lean_tables_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "lean_tables_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    errs = {line.split()[0]: float(line.split()[1]) for line in r.stdout.split("\n") if line.strip()}
    assert set(errs) == {"powers8", "powers9", "powers12", "powers16", "modstep", "modulation16_1536",
                         "modulation16_4096"}, r.stdout
    assert r.returncode == 0, r.stdout
