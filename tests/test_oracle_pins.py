"""The CPU oracle against the reference's own outputs (CPU only).

Fixtures in tests/golden/ were produced by the reference itself (tests/golden/make_golden.py):
the shipped Docs/Example expected results, and the reference built from its sources and run
with one thread on the seeded cases of tests/cases.py.
"""
import os

import numpy as np
import pytest

from cases import QUICK, load_example, make_case
from conftest import GOLDEN
from util import cavity_key, digest, rows, trimmed_hist

FIELD_OF = {
    "EuclideanDistanceSquares": "edt2", "ContainingBallRadiiSquares": "crad2",
    "ContainingBallCoordinatesX": "cx", "ContainingBallCoordinatesY": "cy",
    "ContainingBallCoordinatesZ": "cz", "IsMaximumBall": "mask",
}


def check_against_reference(o, rec):
    r = o["pores"]
    got = {k: digest(o[v]) for k, v in FIELD_OF.items()}
    got["PoreThroatIds"] = digest(r.labels)
    got["PoreThroatIdsWatershed"] = digest(r.labels_ws)
    got["ShortestPathDistances"] = digest(o["dist"])
    got["CavityIds"] = digest(o["cavity"])
    for k, v in rec["digests"].items():
        assert got[k] == v, k
    assert o["max_edt2"] == rec["max_edt2"]
    assert o["maximum_balls_count"] == rec["maximum_balls_count"]
    assert r.pores == rows(rec["pores"])
    assert r.throats == rows(rec["throats"])
    assert r.pores_ws == rows(rec["pores_ws"])
    assert r.throats_ws == rows(rec["throats_ws"])
    assert [cavity_key(c) for c in o["cavities"]] == [cavity_key(c) for c in rows(rec["cavities"])]
    for a, b in zip(o["cavities"], rec["cavities"]):
        assert "%f" % a[4] == "%f" % b[4]


@pytest.mark.parametrize("name", QUICK)
def test_oracle_matches_reference_cases(oracle_mod, ref_cases, name):
    vol, d3q7 = make_case(name)
    o = oracle_mod.full(vol, d3q7=d3q7)
    check_against_reference(o, ref_cases[name])


def test_oracle_histogram_matches_reference(oracle_mod, ref_cases):
    vol, _ = make_case("union_small")
    _, mx, hist = oracle_mod.edt(vol)
    assert trimmed_hist(hist) == ref_cases["union_small"]["hist"]


def test_oracle_matches_shipped_example(oracle_mod, example_golden):
    """Docs/Example: EDT, containing radii, float32 geodesics, cavity ids, statistics and
    the cavity description equal the authors' shipped results bit for bit."""
    solid = load_example(GOLDEN)
    ship = example_golden["shipped"]
    e, mx, hist = oracle_mod.edt(solid)
    assert digest(e) == ship["digests"]["EuclideanDistanceSquares"]
    assert mx == ship["max_edt2"] == 2561
    assert trimmed_hist(hist) == ship["hist"]
    crad2, cx, cy, cz = oracle_mod.containing_balls(e, mx)
    assert digest(crad2) == ship["digests"]["ContainingBallRadiiSquares"]
    d, cav, cavities = oracle_mod.geodesic(solid)
    assert digest(d) == ship["digests"]["ShortestPathDistances"]
    assert digest(cav) == ship["digests"]["CavityIds"]
    assert [cavity_key(c) for c in cavities] == [cavity_key(c) for c in rows(ship["cavities"])]
    assert "%f" % cavities[0][4] == "1.732051"


def test_oracle_matches_reference_example_one_thread(oracle_mod, example_golden):
    solid = load_example(GOLDEN)
    o = oracle_mod.full(solid)
    check_against_reference(o, example_golden["reference_1_thread"])


def test_example_pores_match_shipped_up_to_ids(example_golden):
    """The shipped 7-thread pores differ from the 1-thread run only through thread-order
    tie breaks; the multisets of (radius, boundary flag) of pores agree in size."""
    ship = example_golden["shipped"]
    one = example_golden["reference_1_thread"]
    assert len(ship["pores"]) == len(one["pores"]) == 75
    assert len(ship["pores_ws"]) == len(one["pores_ws"])


REFERENCE = os.environ.get("PMA_REFERENCE_DIR", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "Docs", "Example")),
                    reason="needs the reference tree (fixture-generation container only)")
def test_shipped_coordinates_are_valid_winners(oracle_mod):
    """Where the shipped (7-thread) winning centres differ from the 1-thread rule, both are
    centres of maximal radius covering the voxel, and the oracle's is the smaller in
    (x, y, z) order."""
    from porousmediaanalysis_gb300 import capi
    exp = os.path.join(REFERENCE, "Docs", "Example", "Expected results from -all")
    solid = load_example(GOLDEN)
    e, mx, _ = oracle_mod.edt(solid)
    crad2, cx, cy, cz = oracle_mod.containing_balls(e, mx)
    gx = capi.read_tiff_stack(exp + "/ContainingBallCoordinatesX", 4)
    gy = capi.read_tiff_stack(exp + "/ContainingBallCoordinatesY", 4)
    gz = capi.read_tiff_stack(exp + "/ContainingBallCoordinatesZ", 4)
    void = crad2 > 0
    z, x, y = np.nonzero(void & ((gx != cx) | (gy != cy) | (gz != cz)))
    assert len(z) > 0
    sel = (gz[z, x, y], gx[z, x, y], gy[z, x, y])
    assert (e[sel] == crad2[z, x, y]).all()
    assert ((gx[z, x, y].astype(np.int64) - x) ** 2 + (gy[z, x, y].astype(np.int64) - y) ** 2 +
            (gz[z, x, y].astype(np.int64) - z) ** 2 <= crad2[z, x, y]).all()
    mine = (cx[z, x, y].astype(np.int64), cy[z, x, y].astype(np.int64), cz[z, x, y].astype(np.int64))
    theirs = (gx[z, x, y].astype(np.int64), gy[z, x, y].astype(np.int64), gz[z, x, y].astype(np.int64))
    lex_m = (mine[0] * 10000 + mine[1]) * 10000 + mine[2]
    lex_t = (theirs[0] * 10000 + theirs[1]) * 10000 + theirs[2]
    assert (lex_m < lex_t).all()


def test_large_case_volume_matches_its_fixture():
    """The 2^24-voxel parity volume rebuilt here is the one the fixture was made from."""
    import gzip
    import hashlib
    import json
    import os
    from cases import large_case
    with gzip.open(os.path.join(os.path.dirname(__file__), "golden", "large_case.json.gz"), "rt") as f:
        rec = json.load(f)
    vol = large_case()
    assert list(vol.shape) == rec["shape"]
    assert hashlib.sha256(np.ascontiguousarray(vol).tobytes()).hexdigest() == rec["solid_digest"]
