"""GPU parity on the benchmark workloads themselves, through the C ABI.

* 512^3 Gaussian random field (sigma 3, porosity 0.65, seed 2, built in exact arithmetic by
  synth.grf_exact) and the 256-volume sphere-pack batch: every field, statistic and table
  against the oracle's digests (tests/golden/grf512.json.gz and batch256.json.gz, made by
  tests/golden/make_config_fixtures.py; the oracle needs tens of minutes on them).
* 1024^3 leveled-wave spinodal, where the oracle's containing-ball scatter is out of reach:
  size-independent properties of every stage.
"""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from util import digest, rows_digest, trimmed_hist

pytestmark = pytest.mark.gpu

ALL_FIELDS = ("edt2", "crad2", "cx", "cy", "cz", "maxball_mask", "pore_labels", "watershed_labels",
              "dist_f64", "cavity")


def _load(name):
    with gzip.open(os.path.join(GOLDEN, name), "rt") as f:
        return json.load(f)


def _u32(a):
    a = np.asarray(a)
    return a if a.dtype == np.uint8 else a.view(np.uint32)


def test_grf512_matches_oracle_fixture(ctx):
    """The 512^3 workload, stage by stage: every field, statistic and table bit-exact, the
    shared-type ids of the initial propagation included."""
    import torch
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import synth
    rec = _load("grf512.json.gz")
    vol = synth.grf_exact((512, 512, 512), sigma=3.0, porosity=0.65, seed=2)
    assert digest(vol) == rec["solid"], "the exact generator built another volume"
    solid = torch.from_numpy(vol).cuda()
    edt2, mx, hist = pma.compute_euclidean_distances(ctx, solid, hist_cap=1 << 16)
    assert mx == rec["max_edt2"]
    assert rows_digest(trimmed_hist(hist)) == rec["hist"]
    assert digest(_u32(edt2.cpu().numpy())) == rec["edt2"]
    crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
    assert nb == rec["maximum_balls_count"]
    for name, t in (("crad2", crad2), ("cx", cx), ("cy", cy), ("cz", cz), ("mask", mask)):
        assert digest(_u32(t.cpu().numpy())) == rec[name], name
    del cx, cy, cz
    labels, table = pma.assign_pore_and_throat_ids(ctx, mask, edt2, crad2)
    p0, t0 = table.rows()
    assert len(p0) == rec["npores0"] and rows_digest(p0) == rec["pores0"]
    assert len(t0) == rec["nthroats0"] and rows_digest(t0) == rec["throats0"]
    assert digest(_u32(labels.cpu().numpy())) == rec["labels_initial"]
    pma.remove_empty_pores(ctx, table, labels)
    p1, t1 = table.rows()
    assert rows_digest(p1) == rec["pores"] and rows_digest(t1) == rec["throats"]
    assert digest(_u32(labels.cpu().numpy())) == rec["labels"]
    ws, ws_table = pma.assign_watershed_ids(ctx, table, crad2, mx)
    assert digest(_u32(ws.cpu().numpy())) == rec["labels_ws"]
    pw, tw = ws_table.rows()
    assert rows_digest(pw) == rec["pores_ws"] and rows_digest(tw) == rec["throats_ws"]
    del labels, ws, edt2, crad2, mask
    d32, c32, rows32 = pma.compute_shortest_path_distances(ctx, solid)
    assert digest(d32.cpu().numpy()) == rec["dist_f32"]
    assert digest(_u32(c32.cpu().numpy())) == rec["cavity"]
    del d32, c32
    d64, c64, rows64 = pma.compute_shortest_path_distances(ctx, solid, fp64=True)
    assert digest(d64.cpu().numpy()) == rec["dist_f64"]
    assert digest(_u32(c64.cpu().numpy())) == rec["cavity"]
    assert [list(r[:4]) + list(r[5:]) for r in rows64] == [c[:4] + c[5:] for c in rec["cavities"]]
    assert [r[4] for r in rows64] == pytest.approx([c[4] for c in rec["cavities"]], rel=1e-6)


def test_batch256_matches_oracle_fixture(ctx):
    """The 256-volume batch in the batched form (16 lanes): every volume's fields and tables
    equal the oracle run volume by volume."""
    import porousmediaanalysis_gb300 as pma
    import bench
    rec = _load("batch256.json.gz")["volumes"]
    vols = bench.batch_volumes()
    assert len(vols) == len(rec) == 256
    h = lambda a: digest(a)[:32]
    for lo in range(0, 256, 64):  # four calls of 64 volumes bound the host memory of the outputs
        out = pma.pipeline_batch(ctx, vols[lo:lo + 64], fp64=True, fields=ALL_FIELDS, lanes=16)
        for i, res in enumerate(out, lo):
            r = rec[i]
            assert h(vols[i]) == r["solid"], i
            for k, f in (("edt2", "edt2"), ("crad2", "crad2"), ("cx", "cx"), ("cy", "cy"), ("cz", "cz"),
                         ("maxball_mask", "mask"), ("watershed_labels", "labels_ws"),
                         ("dist_f64", "dist_f64"), ("cavity", "cavity")):
                assert h(_u32(res[k]) if k != "dist_f64" else res[k]) == r[f], (i, k)
            assert res["max_edt2"] == r["max_edt2"] and res["maximum_balls_count"] == r["maximum_balls_count"]
            pp, tp = res["pores"].rows()
            assert rows_digest(pp)[:32] == r["pores"], i
            assert rows_digest(tp)[:32] == r["throats"], i
            assert h(_u32(res["pore_labels"])) == r["labels"], i
            pw, tw = res["watershed"].rows()
            assert rows_digest(pw)[:32] == r["pores_ws"] and rows_digest(tw)[:32] == r["throats_ws"], i
            assert [list(c[:4]) + list(c[5:]) for c in res["cavities"]] == \
                [c[:4] + c[5:] for c in r["cavities"]], i
        del out


def test_spinodal1024_properties(ctx):
    """1024^3 leveled-wave spinodal (1.07 G voxels): properties every correct result has.
    EDT: zero exactly on solid, and squared distance to a solid voxel (or the virtual X walls)
    on sampled void voxels by brute force. Containing balls: every void voxel's radius is at
    least its own EDT, its centre lies within that radius and has that EDT. Watershed: every
    void voxel labelled, pore volumes plus shared volumes equal the void count. Geodesics:
    reachability equals the cavity ids, and the distances obey the stencil's triangle bound
    between neighbours."""
    import torch
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import synth
    solid = synth.spinodal((1024, 1024, 1024), seed=3, device="cuda")
    n = solid.numel()
    void = solid == 0
    nvoid = int(void.sum())
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    assert bool(((edt2 == 0) == (solid != 0)).all())
    # brute-force EDT on sampled void voxels (solid positions of a 33^3 window around each)
    g = torch.Generator(device="cuda").manual_seed(1)
    zs, xs, ys = [torch.randint(16, 1008, (64,), generator=g, device="cuda") for _ in range(3)]
    for z, x, y in zip(zs.tolist(), xs.tolist(), ys.tolist()):
        e = int(edt2[z, x, y])
        if e == 0 or e > 256:  # only radii the 33^3 window certainly covers
            continue
        win = solid[z - 16:z + 17, x - 16:x + 17, y - 16:y + 17]
        pz, px, py = torch.nonzero(win, as_tuple=True)
        best = int(((pz - 16) ** 2 + (px - 16) ** 2 + (py - 16) ** 2).min())
        assert e == min(best, (x + 1024) ** 2, (2 * 1024 - 1 - x) ** 2), (z, x, y)
    crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
    assert bool((crad2 >= edt2).all()) and bool(((crad2 == 0) == (solid != 0)).all())
    idx = torch.nonzero(void.view(-1), as_tuple=True)[0][::4099]
    z = idx // (1024 * 1024)
    x = (idx // 1024) % 1024
    y = idx % 1024
    czv, cxv, cyv = cz.view(-1)[idx].long(), cx.view(-1)[idx].long(), cy.view(-1)[idx].long()
    r2 = crad2.view(-1)[idx].long()
    assert bool((((czv - z) ** 2 + (cxv - x) ** 2 + (cyv - y) ** 2) <= r2).all())
    assert bool((edt2[czv, cxv, cyv].long() == r2).all())
    assert bool((mask.view(-1)[(czv * 1024 + cxv) * 1024 + cyv] == 255).all())
    assert nb == int((mask == 255).sum())
    del cx, cy, cz
    labels, table = pma.assign_pore_and_throat_ids(ctx, mask, edt2, crad2)
    del mask
    pma.remove_empty_pores(ctx, table, labels)
    del labels
    ws, ws_table = pma.assign_watershed_ids(ctx, table, crad2, mx)
    assert bool(((ws != 0) == void).all())
    pw, tw = ws_table.rows()
    assert sum(p[6] for p in pw) + sum(t[1] for t in tw) == nvoid
    assert len(pw) == table.counts()[0]
    del ws, edt2, crad2
    d, cav, rows = pma.compute_shortest_path_distances(ctx, solid, fp64=True)
    reached = (d >= 0) & (d < np.finfo(np.float64).max)
    assert bool(((cav.view(torch.int32) != -1) & void).eq(reached).all())
    assert sum(r[5] for r in rows) == int(reached.sum())
    # triangle bound along +y: |d(v) - d(v + e_y)| <= 1 where both are reached
    a, b = d[:, :, :-1], d[:, :, 1:]
    both = reached[:, :, :-1] & reached[:, :, 1:]
    assert float((a - b).abs()[both].max()) <= 1.0 + 1e-12
