"""The C++ drop-in header: it compiles on the host without a GPU, and (on a
GPU) a program written against the reference's API gives the oracle's DAG."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import random_codes

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "dropin_main.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def compile_cmd(out):
    return ["g++", "-std=c++17", "-O1", f"-I{REPO}/include", f"-I{CUDA}/include", SRC, "-o", out,
            f"-L{D.LIB_DIR}", "-ldagc", f"-L{CUDA}/lib64", "-lcudart", f"-Wl,-rpath,{D.LIB_DIR}",
            f"-Wl,-rpath,{CUDA}/lib64"]


def test_dropin_header_compiles(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{REPO}/include", f"-I{CUDA}/include", SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("depth,split,seed", [(8, 1, 1), (7, 0, 2)])
def test_dropin_program_matches_oracle(tmp_path, depth, split, seed):
    exe = str(tmp_path / "dropin")
    r = subprocess.run(compile_cmd(exe), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    codes = random_codes(depth, 50_000, seed, cluster=True)
    codes.tofile(tmp_path / "codes.u64")
    r = subprocess.run([exe, str(tmp_path / "codes.u64"), str(depth), str(split), str(tmp_path / "words.u32")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    words = np.fromfile(tmp_path / "words.u32", dtype=np.uint32)
    assert np.array_equal(words, O.final_dag(O.create_dag(codes, depth)))
