"""The C++ facade of the reference's interface (include/senk).

On the CPU: the reference's own driver, Work/main.cpp, compiles unchanged
against the facade and links the library (skipped where the reference tree is
absent), and so does tests/facade_driver.cpp.  On the GPU: the facade driver
solves a generated system through the facade and reaches the tolerance."""
import os
import re
import subprocess

import numpy as np
import pytest

import sagb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "sc23-ad_gb300", "_build")
REF_MAIN = "/root/reference/Work/main.cpp"


def _compile(src, out):
    cmd = ["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include", "senk"), src, "-L", LIBDIR, "-lsagb",
           f"-Wl,-rpath,{LIBDIR}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not os.path.exists(REF_MAIN), reason="reference tree not present")
def test_reference_driver_compiles_against_facade(tmp_path):
    _compile(REF_MAIN, str(tmp_path / "main_gpu"))


def test_facade_driver_compiles(tmp_path):
    _compile(os.path.join(ROOT, "tests", "facade_driver.cpp"), str(tmp_path / "drv"))


def _write_mm(path, r, c, v):
    n = len(r) - 1
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{n} {n} {len(c)}\n")
        rows = np.repeat(np.arange(n), np.diff(r))
        for i, j, x in zip(rows, c, v):
            f.write(f"{int(i) + 1} {int(j) + 1} {float(x)!r}\n")


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [0, 2])
def test_facade_driver_solves(tmp_path, kind):
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, 20)
    r, c, v = A.arrays()
    mm = str(tmp_path / "p3d20.mtx")
    _write_mm(mm, r, c, v)
    exe = str(tmp_path / "drv")
    _compile(os.path.join(ROOT, "tests", "facade_driver.cpp"), exe)
    out = subprocess.run([exe, mm, str(kind), "30"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    it = int(re.search(r"\[Iter\] : (\d+)", out.stdout).group(1))
    res = float(re.search(r"# \[Res\] : (\S+)", out.stdout).group(1))
    # Restarted stops when the inner solver's implicit residual says so, as the
    # reference does; for FGMRESflex that estimate is quantised by F, so the
    # explicit residual of the integer solve can stay above eps (the bench uses
    # the explicit-residual stop instead)
    assert it > 0 and res <= (1e-9 if kind == 0 else 1e-5), out.stdout[-2000:]
    assert "# [1]" in out.stdout and "[Time] :" in out.stdout  # the reference's per-iteration and time lines
