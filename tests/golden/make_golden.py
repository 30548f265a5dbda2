"""Regenerates tests/golden/hash_kats.json from the reference's own code.

Runs only where the reference checkout is present: `make -C oracle` compiles
the reference's src/Utils.h into oracle/_ref/libref_hash.so, and this script
records known answers from it:
  * MurmurHash128xN(8 child hashes as 4 x uint128, Size = 4, Seed = 0).Data[0]
    (the hash HashChildrenHashes takes, src/DAGCompression.cu:758-763) for
    edge-case and seeded random child-hash vectors;
  * Utils::ChildOffset(mask, child) for every mask and child;
  * Utils::MurmurHash64 for a few inputs.

Usage: python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402


def vectors():
    m = (1 << 64) - 1
    v = [[0] * 8, [1] + [0] * 7, [0] * 7 + [m], list(range(1, 9)), [m] * 8]
    for c in range(8):
        x = [0] * 8
        x[c] = 0x123456789ABCDEF0
        v.append(x)
    rng = np.random.default_rng(20240613)
    for _ in range(48):
        x = [int(a) for a in rng.integers(0, 2**63, 8, dtype=np.uint64) * 2 + rng.integers(0, 2, 8, dtype=np.uint64)]
        holes = rng.integers(0, 256)
        x = [0 if (holes >> i) & 1 else x[i] for i in range(8)]
        v.append(x)
    return v


def main():
    subprocess_rc = os.system(f"make -s -C {os.path.join(REPO, 'oracle')}")
    assert subprocess_rc == 0
    R = O.ref_lib()
    if R is None:
        raise SystemExit("reference checkout absent: cannot regenerate known answers")
    kats = []
    for x in vectors():
        a = np.array(x, np.uint64)
        raw = int(R.ref_murmur128x4_lo(a.ctypes.data))
        kats.append({"children": [f"{int(c):016x}" for c in x], "murmur128x4_lo": f"{raw:016x}",
                     "node_hash": f"{(raw if raw else 1):016x}"})
    child_offset = [[int(R.ref_child_offset(mask, c)) for c in range(8)] for mask in range(256)]
    m64 = {f"{x:016x}": f"{int(R.ref_murmur64(x)):016x}" for x in [0, 1, 0xFFFFFFFFFFFFFFFF, 0xDEADBEEF]}
    out = {
        "source": "reference src/Utils.h compiled on the host by oracle/Makefile (oracle/ref_hash.cpp)",
        "node_hash_kats": kats,
        "child_offset": child_offset,
        "murmur64": m64,
    }
    with open(os.path.join(HERE, "hash_kats.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(kats)} hash known answers")


if __name__ == "__main__":
    main()
