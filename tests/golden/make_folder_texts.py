"""Generates tests/golden/folder_texts.json: the exact text files the reference writes into a
sample folder for `-all` followed by `-spd` (intermediateStatistics.txt,
euclideanDistanceSquareCounts.txt, pores.txt, sharedPixelTypes.txt, poresWatershed.txt,
sharedPixelTypesWatershed.txt, cavityDescriptions.txt), run with one thread, for the shipped
example and a few seeded cases (tests/cases.py), and for three cases whose configured
resolution makes the reference resample the input stack (then also the digests of the
resampled stack and of every field). The folder-level drop-in test compares the library's
files with these byte for byte.

Run once in a container that holds the reference tree:
    oracle/build_ref.sh && python tests/golden/make_folder_texts.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import ref_run  # noqa: E402
from cases import load_example, make_case, many_pockets  # noqa: E402
from util import digest  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["two_cavities", "pack_small", "union_small_d3q7", "slab_rows"]
RESAMPLED = {"pack_odd_z2": ("pack_odd", "1 1 2"), "pack_odd_xy": ("pack_odd", "2 1.5 1"),
             "union_small_xyz": ("union_small", "1.5 2 1.25")}


def main():
    out = {}
    _, texts = ref_run.run(load_example(HERE))
    out["example"] = texts
    for name in CASES:
        vol, d3q7 = make_case(name)
        out[name] = ref_run.run(vol, d3q7=d3q7)[1]
    out["many_pockets"] = ref_run.run(many_pockets())[1]
    # Resampled inputs (ImageResampler): the stack is resampled before -all and -spd; the
    # record adds digests of every field written and of the resampled Images stack.
    for name, (case, res) in RESAMPLED.items():
        vol, d3q7 = make_case(case)
        fields, texts = ref_run.run(vol, d3q7=d3q7, resolution=res)
        texts["digests"] = {k: digest(v) for k, v in fields.items()}
        texts["shape"] = list(fields["Images"].shape)
        out[name] = texts
    with open(os.path.join(HERE, "folder_texts.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    for k, v in out.items():
        print(k, sorted(v))


if __name__ == "__main__":
    main()
