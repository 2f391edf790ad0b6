"""Generates tests/golden/large_case.json.gz: the oracle's pore and watershed results for a volume
of 2^24 voxels, the size from which the plateau union-find switches to its large-volume form
(pointer jumping, then unions of recorded parent pairs). The oracle needs minutes at this
size, so the GPU test compares against these digests and tables instead of running it.

Run once (CPU only):  python tests/golden/make_large_case.py
The volume is rebuilt by tests/cases.py large_case() (a sphere union: integer and IEEE
arithmetic only, the same on every machine).
"""
import gzip
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from cases import large_case  # noqa: E402
from util import canonical_throats  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    oracle.build()
    vol = large_case()
    o = oracle.full(vol, d3q7=False, geodesic_too=False)
    r = o["pores"]
    out = {
        "shape": list(vol.shape),
        "solid_digest": digest(vol),
        "max_edt2": int(o["max_edt2"]),
        "maximum_balls_count": int(o["maximum_balls_count"]),
        "pores0": [list(p) for p in r.pores0],
        "throats0_lists": sorted([[t[2], t[1]] for t in r.throats0]),
        "throats0": [[t[0], t[1], list(t[2])] for t in r.throats0],
        "labels_initial_canonical": digest(canonical_throats(r.labels_initial)),
        "labels_initial": digest(r.labels_initial),
        "pores": [list(p) for p in r.pores],
        "throats": [[t[0], t[1], list(t[2])] for t in r.throats],
        "labels_canonical": digest(canonical_throats(r.labels)),
        "labels": digest(r.labels),
        "labels_ws": digest(r.labels_ws),
        "pores_ws": [list(p) for p in r.pores_ws],
        "throats_ws": [list(t) for t in r.throats_ws],
    }
    with gzip.open(os.path.join(HERE, "large_case.json.gz"), "wt") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
