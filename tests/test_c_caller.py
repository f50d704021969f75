"""The relink path of a C caller: a reference-style C program
(tests/c/rod_caller.c) compiled against include/tags_gpu.h and linked with
libtags_gpu.so, as a reference example would be (-ltags_gpu ahead of the
reference's own library)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden


def _build_caller(pkg, tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pkg.build()
    libdir = os.path.dirname(pkg.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("ccaller") / "rod_caller")
    cmd = [cc, "-std=c11", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "rod_caller.c"), "-o", exe, "-L" + libdir, "-ltags_gpu",
           "-Wl,-rpath," + libdir, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    return exe


@pytest.fixture(scope="module")
def caller(pkg, tmp_path_factory):
    return _build_caller(pkg, tmp_path_factory)


def test_c_caller_links_and_runs_host_calls(pkg, caller):
    out = subprocess.run([caller, "host"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    rc, sr, si, er, ei = out.stdout.split()
    sig, epsr = pkg.alipio_soil(1e-3, 2j * np.pi * 1e5, 1.26, 0.54, 12.0)
    assert int(rc) == 0
    assert complex(float(sr), float(si)) == sig and complex(float(er), float(ei)) == epsr


@pytest.mark.gpu
def test_c_caller_rod_impedance_on_gpu(gpu_pkg, caller):
    gd = golden("rod_zf.npz")
    ks = (0, 50, 99)
    out = subprocess.run([caller, "gpu"] + [repr(float(gd["freq"][k])) for k in ks], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    rows = [line.split() for line in out.stdout.strip().splitlines()]
    assert len(rows) == len(ks)
    for k, (f, zr, zi) in zip(ks, rows):
        z = complex(float(zr), float(zi))
        want = gd["sol"][k, 0]
        assert abs(z - want) / abs(want) < 1e-8, (f, z, want)
