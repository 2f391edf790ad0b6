"""GPU parity of the EDT, containing-ball and geodesic stages, through the C ABI.

Bit-exact against the reference's own outputs (fixture digests made by the reference run
with one thread) and against the CPU oracle; at larger sizes against the oracle stages that
finish in seconds and through size-independent properties.
"""
import numpy as np
import pytest

from cases import CASES, load_example, make_case
from conftest import GOLDEN
from util import cavity_key, digest, rows, trimmed_hist

pytestmark = pytest.mark.gpu


def _gpu_stages(ctx, vol, d3q7):
    import torch
    import porousmediaanalysis_gb300 as pma
    solid = torch.from_numpy(vol).cuda()
    edt2, mx, hist = pma.compute_euclidean_distances(ctx, solid, hist_cap=1 << 16)
    crad2, cx, cy, cz, mask, nballs = pma.set_containing_balls(ctx, edt2, mx)
    dist, cav, cavities = pma.compute_shortest_path_distances(ctx, solid, pma.D3Q7 if d3q7 else pma.D3Q27)
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return dict(edt2=u32(edt2), max_edt2=mx, hist=hist, crad2=u32(crad2), cx=u32(cx), cy=u32(cy),
                cz=u32(cz), mask=mask.cpu().numpy(), maximum_balls_count=nballs,
                dist=dist.cpu().numpy(), cavity=u32(cav), cavities=cavities)


def _check_stage_digests(g, rec):
    d = rec["digests"]
    assert digest(g["edt2"]) == d["EuclideanDistanceSquares"]
    assert g["max_edt2"] == rec["max_edt2"]
    assert trimmed_hist(g["hist"]) == rec["hist"]
    assert digest(g["crad2"]) == d["ContainingBallRadiiSquares"]
    assert digest(g["cx"]) == d["ContainingBallCoordinatesX"]
    assert digest(g["cy"]) == d["ContainingBallCoordinatesY"]
    assert digest(g["cz"]) == d["ContainingBallCoordinatesZ"]
    assert digest(g["mask"]) == d["IsMaximumBall"]
    assert g["maximum_balls_count"] == rec["maximum_balls_count"]
    assert digest(g["dist"]) == d["ShortestPathDistances"]
    assert digest(g["cavity"]) == d["CavityIds"]
    assert [cavity_key(c) for c in g["cavities"]] == [cavity_key(c) for c in rows(rec["cavities"])]
    for a, b in zip(g["cavities"], rec["cavities"]):
        assert "%f" % a[4] == "%f" % b[4]


@pytest.mark.parametrize("name", list(CASES))
def test_stages_match_reference(ctx, ref_cases, name):
    vol, d3q7 = make_case(name)
    _check_stage_digests(_gpu_stages(ctx, vol, d3q7), ref_cases[name])


def test_stages_match_reference_on_example(ctx, example_golden):
    vol = load_example(GOLDEN)
    g = _gpu_stages(ctx, vol, False)
    _check_stage_digests(g, example_golden["reference_1_thread"])
    ship = example_golden["shipped"]["digests"]
    assert digest(g["edt2"]) == ship["EuclideanDistanceSquares"]
    assert digest(g["crad2"]) == ship["ContainingBallRadiiSquares"]
    assert digest(g["dist"]) == ship["ShortestPathDistances"]


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_stages_match_oracle_random(ctx, oracle_mod, seed):
    from porousmediaanalysis_gb300 import synth
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(20, 70, 3))
    vol = synth.sphere_pack(shape, rmin=2, rmax=9, solid_fraction=float(rng.uniform(0.3, 0.6)),
                            seed=seed)
    d3q7 = bool(seed % 2)
    g = _gpu_stages(ctx, vol, d3q7)
    e, mx, hist = oracle_mod.edt(vol)
    assert (g["edt2"] == e).all() and g["max_edt2"] == mx
    crad2, cx, cy, cz = oracle_mod.containing_balls(e, mx)
    assert (g["crad2"] == crad2).all()
    assert (g["cx"] == cx).all() and (g["cy"] == cy).all() and (g["cz"] == cz).all()
    mask, nb = oracle_mod.max_ball_mask(cx, cy, cz)
    assert (g["mask"] == mask).all() and g["maximum_balls_count"] == nb
    dist, cav, cavities = oracle_mod.geodesic(vol, d3q7)
    assert (g["dist"].view(np.uint32) == dist.view(np.uint32)).all()
    assert (g["cavity"] == cav).all()


@pytest.mark.parametrize("d3q7", [False, True])
def test_geodesic_f64_matches_fp64_oracle(ctx, oracle_mod, d3q7):
    import torch
    import porousmediaanalysis_gb300 as pma
    vol, _ = make_case("two_cavities")
    solid = torch.from_numpy(vol).cuda()
    d, c, rows64 = pma.compute_shortest_path_distances(ctx, solid, pma.D3Q7 if d3q7 else pma.D3Q27,
                                                       fp64=True)
    od, oc, orows = oracle_mod.geodesic(vol, d3q7, fp64=True)
    assert (d.cpu().numpy().view(np.uint64) == od.view(np.uint64)).all()
    assert (c.cpu().numpy().view(np.uint32) == oc).all()
    assert [cavity_key(r) for r in rows64] == [cavity_key(r) for r in orows]
    # float64 against the float32 reference: same reachability, close values
    d32, c32, _ = oracle_mod.geodesic(vol, d3q7)
    reach = (d32 >= 0) & (d32 < np.finfo(np.float32).max)
    assert ((od >= 0) & (od < np.finfo(np.float64).max) == reach).all()
    rel = np.abs(od[reach] - d32[reach]) / np.maximum(od[reach], 1)
    assert rel.max() < 1e-5


def test_edt_and_geodesic_match_oracle_256(ctx, oracle_mod):
    """256^3 Gaussian random field (the 512^3 workload's structure at a size the oracle
    finishes in seconds)."""
    from porousmediaanalysis_gb300 import synth
    import torch
    import porousmediaanalysis_gb300 as pma
    vol = synth.grf((256, 256, 256), sigma=3.0, porosity=0.65, seed=2)
    solid = torch.from_numpy(vol).cuda()
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    e, omx, _ = oracle_mod.edt(vol)
    assert mx == omx and (edt2.cpu().numpy().view(np.uint32) == e).all()
    dist, cav, cavs = pma.compute_shortest_path_distances(ctx, solid)
    od, oc, ocavs = oracle_mod.geodesic(vol)
    assert (dist.cpu().numpy().view(np.uint32) == od.view(np.uint32)).all()
    assert [cavity_key(r) for r in cavs] == [cavity_key(r) for r in ocavs]


def test_containing_balls_properties_512(ctx):
    """512^3 Gaussian random field: every void voxel's winner is a void centre whose squared
    EDT equals the voxel's containing radius and whose ball covers the voxel; radii are at
    least the voxel's own EDT; solid voxels carry the sentinels; the result is deterministic."""
    import torch
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import synth
    solid = synth.grf((512, 512, 512), seed=2, device="cuda")
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
    void = edt2 != 0
    assert bool((crad2[~void] == 0).all()) and bool((cx[~void] == -1).all())
    e64 = edt2.long()
    c64 = crad2.long()
    assert bool((c64[void] >= e64[void]).all())
    zz, xx, yy = torch.nonzero(void, as_tuple=True)
    sel = torch.arange(0, zz.numel(), 97, device=zz.device)
    z, x, y = zz[sel], xx[sel], yy[sel]
    wx, wy, wz = cx[z, x, y].long(), cy[z, x, y].long(), cz[z, x, y].long()
    assert bool((e64[wz, wx, wy] == c64[z, x, y]).all())
    d2 = (wx - x) ** 2 + (wy - y) ** 2 + (wz - z) ** 2
    assert bool((d2 <= c64[z, x, y]).all())
    assert int((mask == 255).sum()) == nb
    crad2b, cxb, _, _, maskb, nbb = pma.set_containing_balls(ctx, edt2, mx)
    assert bool((crad2b == crad2).all()) and bool((cxb == cx).all()) and nbb == nb


def _balls_vs_oracle(ctx, oracle_mod, vol):
    import torch
    import porousmediaanalysis_gb300 as pma
    solid = torch.from_numpy(np.ascontiguousarray(vol, dtype=np.uint8)).cuda()
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
    e, omx, _ = oracle_mod.edt(vol)
    assert mx == omx
    ocrad, ocx, ocy, ocz = oracle_mod.containing_balls(e, omx)
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    assert (u32(crad2) == ocrad).all()
    assert (u32(cx) == ocx).all() and (u32(cy) == ocy).all() and (u32(cz) == ocz).all()
    omask, onb = oracle_mod.max_ball_mask(ocx, ocy, ocz)
    assert (mask.cpu().numpy() == omask).all() and nb == onb


def test_containing_balls_long_tile_lists(ctx, oracle_mod):
    """96^3 leveled-wave spinodal (wavelength 48): radii up to sqrt(533), tile lists of up to
    several thousand centres, so the gather takes them in several shared-memory chunks."""
    from porousmediaanalysis_gb300 import synth
    vol = synth.spinodal((96, 96, 96), device="cpu").numpy()
    _balls_vs_oracle(ctx, oracle_mod, vol)


def test_containing_balls_wide_radius_span(ctx, oracle_mod):
    """A 44^3 box with two solid voxels: tile lists of up to 40 000 centres (twenty chunks),
    and in two tiles squared radii spanning more than the gather's counting sort (2048), so
    those chunks are scanned in fill order."""
    vol = np.zeros((44, 44, 44), np.uint8)
    vol[0, 0, 0] = 1
    vol[27, 11, 38] = 1
    _balls_vs_oracle(ctx, oracle_mod, vol)


def test_every_cavity_row_is_returned(ctx, oracle_mod):
    """49 cavities, more than the 16 rows of pma_outputs.cavities: the stage call, the
    host-buffer pipeline (through its cavity_rows buffer) and a count-only call all report
    every cavity, with the oracle's rows."""
    import torch
    import porousmediaanalysis_gb300 as pma
    from cases import many_pockets
    vol = many_pockets()
    od, oc, orows = oracle_mod.geodesic(vol)
    assert len(orows) > 40 and not any(r[7] for r in orows)
    solid = torch.from_numpy(vol).cuda()
    d, c, got = pma.compute_shortest_path_distances(ctx, solid)
    assert [cavity_key(r) for r in got] == [cavity_key(r) for r in orows]
    assert (d.cpu().numpy().view(np.uint32) == od.view(np.uint32)).all()
    assert (c.cpu().numpy().view(np.uint32) == oc).all()
    _, _, first, n = pma.shortest_path_with_count(ctx, solid, cavity_cap=5)
    assert n == len(orows) and [cavity_key(r) for r in first] == [cavity_key(r) for r in orows[:5]]
    res = pma.pipeline_host(ctx, vol, run_pores=False, fields=("dist_f32",))
    assert [cavity_key(r) for r in res["cavities"]] == [cavity_key(r) for r in orows]
