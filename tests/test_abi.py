"""CPU tests of the C ABI boundary: the libraries load and export every
function that include/*.h declares (no compute call needs a GPU here)."""
import ctypes
import os
import re

import numpy as np
import pytest

import dag_compression_fast_gb300 as D

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")

# header -> library that must export its functions
HEADERS = {"dagc.h": D.LIBDAGC_PATH, "dagc_gen.h": D.LIBGEN_PATH}


def declared_functions(header):
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dagc_\w+)\s*\(", src)))


@pytest.mark.parametrize("header", sorted(HEADERS))
def test_every_declared_symbol_is_exported(header):
    lib = ctypes.CDLL(HEADERS[header])
    names = declared_functions(header)
    assert names, header
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_lists_every_symbol():
    assert sorted(D.DAGC_SYMBOLS) == declared_functions("dagc.h")
    assert sorted(D.GEN_SYMBOLS) == declared_functions("dagc_gen.h")


def test_status_strings_without_gpu():
    L = D.lib()
    assert L.dagc_version() >= 1
    assert L.dagc_status_string(0) == b"ok"
    assert L.dagc_status_string(4) == b"hash collision"


def test_no_third_party_sort_libraries_in_sources():
    csrc = os.path.join(REPO, "dag_compression_fast_gb300", "csrc")
    for f in os.listdir(csrc):
        text = open(os.path.join(csrc, f)).read()
        code = re.sub(r"//[^\n]*|/\*.*?\*/", "", text, flags=re.S)  # comments may cite the reference
        for banned in ("<cub/", "<thrust/", "moderngpu", "cub::", "thrust::", "mgpu::"):
            assert banned not in code, (f, banned)


def test_dag_file_round_trip(tmp_path):
    from oracle import oracle as O
    from tests.inputs import random_codes
    codes = random_codes(7, 3000, 4, cluster=True)
    words = O.final_dag(O.create_dag(codes, 7))
    path = str(tmp_path / "scene.dag.bin")
    D.write_dag_file(path, words, 7, (-1.0, -2.0, -3.0, 4.0, 5.0, 6.0))
    raw = open(path, "rb").read()
    assert len(raw) == 6 * 8 + 4 + 8 + 4 * words.size  # the reference's layout, no padding
    w, depth, box = D.read_dag_file(path)
    assert depth == 7 and box == (-1.0, -2.0, -3.0, 4.0, 5.0, 6.0)
    assert np.array_equal(w, words)


def test_hash_children_matches_oracle():
    import numpy as np
    from oracle import oracle as O
    rng = np.random.default_rng(3)
    for _ in range(20):
        h = rng.integers(0, 2**64 - 1, 8, dtype=np.uint64)
        assert D.hash_children(h) == O.hash_children(h)
