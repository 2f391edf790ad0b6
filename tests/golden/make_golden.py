"""Generates the golden fixtures of tests/golden/ from the reference itself.

Run once in a container that holds the reference tree (the first argument, else
$PMA_REFERENCE_DIR, else /root/reference):
    oracle/build_ref.sh && python tests/golden/make_golden.py [reference_dir]

Outputs (small, committed):
  example_solid.npz  packed solid mask of Docs/Example/Images (1196 x 960 x 5);
  example.json       digests of the shipped expected outputs of Docs/Example (produced by the
                     authors' 7-thread run): EDT, containing radii, geodesics, cavity ids,
                     statistics and text tables; plus digests and tables of the reference
                     built here and run with "Number of threads: 1" on the same input;
  ref_cases.json     for seeded synthetic volumes (rebuilt by tests/cases.py), digests of every
                     output field and the text tables of the reference run with 1 thread.
PoreThroatIds_canonical is the digest of PoreThroatIds with shared-type ids renamed by first
appearance (tests/util.py canonical_throats).
A digest is the SHA-256 of the field's bytes in [z][x][y] order (float32 as raw bits).
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import ref_run  # noqa: E402
from cases import CASES, make_case  # noqa: E402
from util import canonical_throats  # noqa: E402
from porousmediaanalysis_gb300 import build as pbuild  # noqa: E402
from porousmediaanalysis_gb300 import capi  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_record(solid, d3q7=False):
    fields, texts = ref_run.run(solid, d3q7=d3q7)
    rec = {"digests": {k: digest(v) for k, v in fields.items()}}
    rec["PoreThroatIds_canonical"] = digest(canonical_throats(fields["PoreThroatIds"]))
    rec["pores"] = ref_run.parse_pores(texts["pores.txt"])
    rec["throats"] = ref_run.parse_throats(texts["sharedPixelTypes.txt"])
    rec["pores_ws"] = ref_run.parse_pores(texts["poresWatershed.txt"])
    rec["throats_ws"] = ref_run.parse_throats(texts["sharedPixelTypesWatershed.txt"])
    rec["cavities"] = ref_run.parse_cavities(texts["cavityDescriptions.txt"])
    st = texts["intermediateStatistics.txt"].split()
    rec["max_edt2"] = int(st[4])
    rec["maximum_balls_count"] = int(st[8])
    rec["hist"] = [int(x) for x in texts["euclideanDistanceSquareCounts.txt"].split("\n")[1:] if x.strip()]
    return rec


def main(ref_dir):
    pbuild.build()
    ex = os.path.join(ref_dir, "Docs", "Example")
    solid = capi.read_tiff_stack(os.path.join(ex, "Images"), 1)
    np.savez_compressed(os.path.join(HERE, "example_solid.npz"),
                        shape=np.array(solid.shape), bits=np.packbits(solid != 0))
    shipped = {}
    exp_all = os.path.join(ex, "Expected results from -all")
    exp_spd = os.path.join(ex, "Expected results from -spd")
    for name in ("EuclideanDistanceSquares", "ContainingBallRadiiSquares"):
        shipped[name] = digest(capi.read_tiff_stack(os.path.join(exp_all, name), 4))
    for name in ("ShortestPathDistances", "CavityIds"):
        shipped[name] = digest(capi.read_tiff_stack(os.path.join(exp_spd, name), 4))
    txt = lambda p: open(p).read().replace("\r\n", "\n")
    st = txt(os.path.join(exp_all, "intermediateStatistics.txt")).split()
    out = {
        "shape": list(solid.shape),
        "shipped": {
            "digests": shipped,
            "max_edt2": int(st[4]),
            "maximum_balls_count_7_threads": int(st[8]),
            "hist": [int(x) for x in txt(os.path.join(exp_all, "euclideanDistanceSquareCounts.txt")).split("\n")[1:] if x.strip()],
            "cavities": ref_run.parse_cavities(txt(os.path.join(exp_spd, "cavityDescriptions.txt"))),
            "pores": ref_run.parse_pores(txt(os.path.join(exp_all, "pores.txt"))),
            "pores_ws": ref_run.parse_pores(txt(os.path.join(exp_all, "poresWatershed.txt"))),
        },
        "reference_1_thread": ref_record(solid),
    }
    with open(os.path.join(HERE, "example.json"), "w") as f:
        json.dump(out, f)
    cases = {}
    for name in CASES:
        vol, d3q7 = make_case(name)
        cases[name] = ref_record(vol, d3q7)
        print(name, vol.shape, len(cases[name]["pores"]), "pores")
    with open(os.path.join(HERE, "ref_cases.json"), "w") as f:
        json.dump(cases, f)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PMA_REFERENCE_DIR", "/root/reference"))
