"""GPU test of dagc_sort_keys_noalloc, the key sort that allocates nothing.

Some callers of this library cannot allocate device memory once they are
running: engines and servers that reserve the whole GPU through their own
allocator at start-up (a cudaMalloc from a library would then fail or carve up
their reservation), and callers that cannot pay for cudaMalloc's implicit
device synchronisation. dagc_sort_keys_noalloc serves them with a fixed
scratch array compiled into the library.

The test calls it through the C ABI twice in a row (the second call reuses the
scratch the first one left behind) and checks each result bit for bit against
numpy's stable sort on the same bit range and against the allocating entry
point dagc_sort_keys. It also checks that a request above the fixed limit is
refused before any memory is touched. This file is collected last so that a
failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

import dag_compression_fast_gb300 as D

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20


def stable_sorted(keys: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """Keys in the order of a stable sort on bits [lo, hi)."""
    u = keys.view(np.uint64)
    digit = u >> np.uint64(lo)
    if hi - lo < 64:
        digit = digit & np.uint64((1 << (hi - lo)) - 1)
    return keys[np.argsort(digit, kind="stable")]


def test_noalloc_sort_matches_allocating_sort_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = D.lib()
    ctx = D.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2024)
    cases = [(MAX_KEYS, 6, 33), (777_777, 0, 64)]  # two calls in a row, different shapes
    for n, lo, hi in cases:
        keys_np = rng.integers(0, 2**63, n, dtype=np.int64)
        keys_np[: n // 4] = keys_np[0]  # a long run of equal keys
        keys = torch.from_numpy(keys_np).cuda()
        expected = ctx.sort_keys(keys, lo, hi)  # the allocating entry point
        out = torch.empty_like(keys)
        st = lib.dagc_sort_keys_noalloc(keys.data_ptr(), out.data_ptr(), n, lo, hi, stream)
        assert st == D.OK, lib.dagc_status_string(st)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), stable_sorted(keys_np, lo, hi))
        assert torch.equal(out, expected)
        assert torch.equal(keys, torch.from_numpy(keys_np).cuda())  # input left intact
    ctx.close()


def test_noalloc_sort_rejects_more_than_its_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = D.lib()
    small = torch.zeros(4, dtype=torch.int64, device="cuda")
    out = torch.empty_like(small)
    st = lib.dagc_sort_keys_noalloc(small.data_ptr(), out.data_ptr(), MAX_KEYS + 1, 0, 64,
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == D.ERR_TOO_LARGE
