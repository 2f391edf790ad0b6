"""GPU parity of seeds, pore propagation, empty-pore removal and the watershed, through the
C ABI, against the reference's own outputs (fixture digests and tables) and the oracle.

Exact: pore ids, seeds, radii, boundary flags, volumes, every voxel's label, shared types
with their ids (the reference's depth-first creation order, replayed on the host), and the
whole watershed (labels, pores and shared types with their ids). With the cheaper type
numbering the initial propagation's ids match up to a one-to-one renaming.
"""
import numpy as np
import pytest

from cases import CASES, load_example, make_case
from conftest import GOLDEN
from util import canonical_throats, digest, rows

pytestmark = pytest.mark.gpu


def _gpu_pipeline(ctx, vol, d3q7):
    import torch
    import porousmediaanalysis_gb300 as pma
    st = pma.D3Q7 if d3q7 else pma.D3Q27
    solid = torch.from_numpy(vol).cuda()
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
    labels, table = pma.assign_pore_and_throat_ids(ctx, mask, edt2, crad2, st)
    initial = table.rows()
    labels_initial = labels.cpu().numpy().view(np.uint32).copy()
    pma.remove_empty_pores(ctx, table, labels)
    ws, ws_table = pma.assign_watershed_ids(ctx, table, crad2, mx, st)
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return dict(labels_initial=labels_initial, initial=initial, labels=u32(labels), table=table.rows(),
                ws=u32(ws), ws_table=ws_table.rows())


def _check(g, rec):
    pores, throats = g["table"]
    assert pores == rows(rec["pores"])
    assert throats == rows(rec["throats"])
    assert digest(g["labels"]) == rec["digests"]["PoreThroatIds"]
    assert digest(g["ws"]) == rec["digests"]["PoreThroatIdsWatershed"]
    pws, tws = g["ws_table"]
    assert pws == rows(rec["pores_ws"])
    assert tws == rows(rec["throats_ws"])


@pytest.mark.parametrize("name", list(CASES))
def test_pores_and_watershed_match_reference(ctx, ref_cases, name):
    vol, d3q7 = make_case(name)
    _check(_gpu_pipeline(ctx, vol, d3q7), ref_cases[name])


def test_pores_and_watershed_match_reference_on_example(ctx, example_golden):
    _check(_gpu_pipeline(ctx, load_example(GOLDEN), False), example_golden["reference_1_thread"])


@pytest.mark.parametrize("seed", [31, 32, 33, 34])
def test_pores_and_watershed_match_oracle_random(ctx, oracle_mod, seed):
    """Random packs and fields against the oracle, including the initial propagation's
    tables before removal (types compared up to renaming)."""
    from porousmediaanalysis_gb300 import synth
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(24, 64, 3))
    if seed % 2:
        vol = synth.sphere_pack(shape, rmin=2, rmax=8, solid_fraction=float(rng.uniform(0.3, 0.55)), seed=seed)
    else:
        vol = synth.grf(shape, sigma=float(rng.uniform(1.5, 3.5)), porosity=float(rng.uniform(0.5, 0.8)), seed=seed)
    d3q7 = seed in (32, 33)
    g = _gpu_pipeline(ctx, vol, d3q7)
    o = oracle_mod.full(vol, d3q7=d3q7, geodesic_too=False)
    r = o["pores"]
    p0, t0 = g["initial"]
    assert p0 == r.pores0
    assert t0 == r.throats0
    assert (g["labels_initial"] == r.labels_initial).all()
    assert g["table"] == (r.pores, r.throats)
    assert (g["labels"] == r.labels).all()
    assert (g["ws"] == r.labels_ws).all()
    assert g["ws_table"] == (r.pores_ws, r.throats_ws)


def test_pipeline_host_matches_stage_calls(ctx, ref_cases):
    """The host-buffer pipeline entry point (the e2e path) gives the same fields."""
    import porousmediaanalysis_gb300 as pma
    vol, _ = make_case("union_small")
    res = pma.pipeline_host(ctx, vol, fields=("edt2", "crad2", "maxball_mask", "watershed_labels",
                                              "dist_f32", "cavity"))
    rec = ref_cases["union_small"]
    assert digest(res["edt2"]) == rec["digests"]["EuclideanDistanceSquares"]
    assert digest(res["crad2"]) == rec["digests"]["ContainingBallRadiiSquares"]
    assert digest(res["maxball_mask"]) == rec["digests"]["IsMaximumBall"]
    assert digest(res["watershed_labels"]) == rec["digests"]["PoreThroatIdsWatershed"]
    assert digest(res["dist_f32"]) == rec["digests"]["ShortestPathDistances"]
    assert digest(res["cavity"]) == rec["digests"]["CavityIds"]
    assert res["watershed"].rows() == (rows(rec["pores_ws"]), rows(rec["throats_ws"]))


def test_pipeline_host_with_page_locked_buffers(ctx):
    """Page-locked host buffers move through the streaming copy kernel (16-byte words plus a
    tail of 4 to 13 bytes on this odd-sized volume), a buffer offset by 4 bytes through the copy
    engine: every field equals the run on pageable buffers."""
    import numpy as np
    import torch
    import porousmediaanalysis_gb300 as pma
    vol, _ = make_case("pack_odd")
    fields = ("edt2", "crad2", "cx", "cy", "cz", "maxball_mask", "pore_labels", "watershed_labels",
              "dist_f64", "cavity")
    plain = pma.pipeline_host(ctx, vol, fp64=True, fields=fields)
    kinds = {"maxball_mask": (torch.uint8, np.uint8), "dist_f64": (torch.float64, np.float64)}
    pinned_in = torch.from_numpy(vol).pin_memory()
    keep, outs = [], {}
    for name in fields:
        tdt, ndt = kinds.get(name, (torch.int32, np.uint32))
        if name == "cx":  # a view 4 bytes into its pinned block: alignments differ
            blk = torch.empty(vol.size + 1, dtype=torch.int32).pin_memory()
            arr = blk.numpy()[1:].view(np.uint32).reshape(vol.shape)
        else:
            blk = torch.empty(vol.shape, dtype=tdt).pin_memory()
            arr = blk.numpy().view(ndt)
        keep.append(blk)
        outs[name] = arr
    res = pma.pipeline_host(ctx, pinned_in.numpy(), fp64=True, fields=fields, out_arrays=outs)
    for name in fields:
        assert np.array_equal(res[name], plain[name]), name
    assert res["watershed"].rows() == plain["watershed"].rows()


def test_watershed_accepts_pores_read_back(ctx, ref_cases):
    """Pores built from table rows (as read from pores.txt) drive the watershed."""
    import torch
    import porousmediaanalysis_gb300 as pma
    vol, _ = make_case("pack_small")
    rec = ref_cases["pack_small"]
    solid = torch.from_numpy(vol).cuda()
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    crad2, *_ = pma.set_containing_balls(ctx, edt2, mx)
    table = pma.Table.from_rows([tuple(p) for p in rec["pores"]])
    ws, ws_table = pma.assign_watershed_ids(ctx, table, crad2, mx)
    assert digest(ws.cpu().numpy().view(np.uint32)) == rec["digests"]["PoreThroatIdsWatershed"]
    assert ws_table.rows() == (rows(rec["pores_ws"]), rows(rec["throats_ws"]))


def test_watershed_with_most_voxels_shared(ctx, oracle_mod):
    """Uncorrelated noise (porosity 0.7): nearly every void voxel touches several pores, far
    more shared voxels than the watershed's first guess of records, so the flood is redone
    with more records; the result must still equal the oracle's."""
    rng = np.random.default_rng(12)
    vol = (rng.random((40, 44, 36)) > 0.7).astype(np.uint8)
    g = _gpu_pipeline(ctx, vol, False)
    r = oracle_mod.full(vol, geodesic_too=False)["pores"]
    assert g["table"][0] == r.pores
    assert (g["ws"] == r.labels_ws).all()
    pws, tws = g["ws_table"]
    assert pws == r.pores_ws and tws == r.throats_ws
    assert len(tws) > 0


def test_pores_and_watershed_large_volume_matches_oracle_fixture(ctx):
    """2^24 voxels, where the plateaus are labelled by pointer jumping and unions of recorded
    parent pairs: pores, shared voxels and the whole watershed against the oracle's results
    (tests/golden/large_case.json.gz, made by tests/golden/make_large_case.py; the oracle takes
    minutes at this size)."""
    import gzip
    import json
    import os
    from cases import large_case
    from util import canonical_throats
    with gzip.open(os.path.join(GOLDEN, "large_case.json.gz"), "rt") as f:
        rec = json.load(f)
    vol = large_case()
    assert list(vol.shape) == rec["shape"] and digest(vol) == rec["solid_digest"]
    g = _gpu_pipeline(ctx, vol, False)
    p0, t0 = g["initial"]
    assert p0 == rows(rec["pores0"])
    assert t0 == rows(rec["throats0"])
    assert digest(g["labels_initial"]) == rec["labels_initial"]
    assert g["table"] == (rows(rec["pores"]), rows(rec["throats"]))
    assert digest(g["labels"]) == rec["labels"]
    assert digest(g["ws"]) == rec["labels_ws"]
    assert g["ws_table"] == (rows(rec["pores_ws"]), rows(rec["throats_ws"]))


def _junction(n_seeds, seed):
    """A void box whose centre voxel is touched by `n_seeds` pores seeded on its neighbours:
    containing radii 50 around a centre of radius 1, so that every seed's first generation
    reaches the centre (one claim, n_seeds - 1 extensions: a shared type of n_seeds pores).
    Other voxels get random radii below 50, so the flood also runs over several depths."""
    rng = np.random.default_rng(seed)
    crad = rng.integers(1, 50, (9, 11, 10)).astype(np.uint32)
    c = (4, 5, 5)  # z, x, y
    crad[c[0] - 1:c[0] + 2, c[1] - 1:c[1] + 2, c[2] - 1:c[2] + 2] = 50
    crad[c] = 1
    offs = [(dx, dy, dz) for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)
            if (dx, dy, dz) != (0, 0, 0)]
    pick = rng.permutation(len(offs))[:n_seeds]
    ids = [127 + k for k in range(n_seeds)]
    rng.shuffle(ids)
    rows = [(ids[k], c[1] + offs[i][0], c[2] + offs[i][1], c[0] + offs[i][2], 50, 0, 0)
            for k, i in enumerate(pick)]
    return crad, rows


@pytest.mark.parametrize("n_seeds,seed", [(8, 1), (12, 2), (19, 3), (26, 4)])
def test_watershed_junction_of_many_pores(ctx, oracle_mod, n_seeds, seed):
    """Up to 26 pores meet at one voxel (the reference keys shared types by an unbounded
    pore-id vector): labels and both tables equal the oracle's, including the type of all
    n_seeds pores."""
    import torch
    import porousmediaanalysis_gb300 as pma
    crad, rows_in = _junction(n_seeds, seed)
    o_ws, o_pores, o_throats = oracle_mod.watershed(rows_in, crad, 50)
    assert max(len(t[2]) for t in o_throats) == n_seeds
    table = pma.Table.from_rows(rows_in)
    ws, ws_table = pma.assign_watershed_ids(ctx, table, torch.from_numpy(crad.view(np.int32)).cuda(), 50)
    assert (ws.cpu().numpy().view(np.uint32) == o_ws).all()
    assert ws_table.rows() == (o_pores, o_throats)


def test_cheaper_type_numbering_is_a_renaming(ctx, oracle_mod):
    """With pma_ctx_set_throat_numbering(ctx, 0) the initial propagation's types keep their
    pore lists, volumes and voxels, and only their ids differ from the reference's."""
    vol, d3q7 = make_case("union_small")
    ctx.set_throat_numbering(reference=False)
    try:
        g = _gpu_pipeline(ctx, vol, d3q7)
    finally:
        ctx.set_throat_numbering(reference=True)
    r = oracle_mod.full(vol, d3q7=d3q7, geodesic_too=False)["pores"]
    p0, t0 = g["initial"]
    assert p0 == r.pores0
    assert sorted((t[2], t[1]) for t in t0) == sorted((t[2], t[1]) for t in r.throats0)
    assert (canonical_throats(g["labels_initial"]) == canonical_throats(r.labels_initial)).all()
    assert (g["ws"] == r.labels_ws).all() and g["ws_table"] == (r.pores_ws, r.throats_ws)


def test_watershed_with_radii_beyond_16_bits(ctx, oracle_mod):
    """Containing radii squared of 65536 and more (a void box 900 voxels long in X, split by a
    solid wall with one hole; no solids bound Y or Z) take the watershed's unpacked state path;
    the two pores meet at the hole, and the result equals the oracle's."""
    vol = np.zeros((4, 900, 5), np.uint8)
    vol[:, 450, :] = 1
    vol[2, 450, 2] = 0
    vol[1, 200, 3] = 1
    g = _gpu_pipeline(ctx, vol, False)
    o = oracle_mod.full(vol, geodesic_too=False)
    assert o["max_edt2"] >= 65536
    r = o["pores"]
    assert len(r.throats_ws) >= 2
    assert g["table"] == (r.pores, r.throats)
    assert (g["ws"] == r.labels_ws).all()
    assert g["ws_table"] == (r.pores_ws, r.throats_ws)
