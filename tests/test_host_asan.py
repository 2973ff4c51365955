"""Every host code path of the C ABI under AddressSanitizer, without a GPU: the library's CUDA
translation units are linked against a host-only stand-in of the CUDA runtime
(tests/host_asan/fake_cudart.cpp: device memory is host memory, launches do nothing) and driven
through all entry points in both precision forms, 2D and 3D.  Catches host-side memory errors
(use after free, overruns, leaks) that on the GPU machine would surface as crashes."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "trixiparticles.jl_gb300" / "csrc"
INC = ROOT / "include"
HERE = Path(__file__).resolve().parent / "host_asan"
SOURCES = ["tp_api.cu", "tp_fp64.cu", "tp_fp32.cu", "tp_noalloc.cu", "tp_adjoint.cu",
           "tp_batch.cu", "tp_interp.cu"]


def test_host_paths_under_asan(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    objs = []
    procs = []
    for src in SOURCES:
        obj = tmp_path / (Path(src).stem + ".o")
        cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O1", "-g", "-std=c++17",
               "-Xcompiler", "-fsanitize=address,-fno-omit-frame-pointer",
               "--expt-relaxed-constexpr", "-I", str(INC), "-I", str(CSRC), "-c", str(CSRC / src),
               "-o", str(obj)]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE))
        objs.append(str(obj))
    for p in procs:
        out, err = p.communicate()
        assert p.returncode == 0, err.decode()[-2000:]
    exe = tmp_path / "driver"
    cuda_inc = str(Path(nvcc).resolve().parent.parent / "include")
    subprocess.run(["g++", "-g", "-fsanitize=address", "-I", cuda_inc, "-I", str(INC),
                    str(HERE / "fake_cudart.cpp"), str(HERE / "driver.cpp"), *objs, "-o",
                    str(exe)], check=True, capture_output=True)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1")
    res = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr[-4000:]
    assert res.stdout.count("bad=0") == 4, res.stdout
