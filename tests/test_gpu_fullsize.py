"""Full-size (512^3 Gaussian random field, porosity 0.65, sigma 3) checks through the C ABI.

The oracle takes minutes per stage at this size, so these tests check size-independent
properties that pin each output down exactly:
  * EDT: on sampled void voxels, the squared distance equals the brute-force minimum over
    the solid voxels of a window large enough to hold the nearest one.
  * containing balls: on sampled void voxels, the radius is the largest ball covering the
    voxel and the centre the lexicographically smallest (x, y, z) among those of that radius;
    the maximum-ball mask marks exactly the set of winning centres.
  * pores and watershed: every id's voxel count equals its table volume, and every pore's
    seed voxel carries the pore's id or a shared type listing the pore.
  * float64 geodesics: every reached voxel other than a cavity seed equals
    min over reached neighbours u of fl(d(u) + w), unreached void voxels have no reached
    neighbour (the rounded fixed point the reference's Dijkstra settles on).
  * determinism: a second run gives the same bits.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (512, 512, 512)  # (SZ, SX, SY)
THROAT_MIN = 1 << 31


@pytest.fixture(scope="module")
def run512(ctx):
    import torch
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import synth

    solid = synth.grf(SHAPE, sigma=3.0, porosity=0.65, seed=2, device="cuda")

    def chain():
        edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
        crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
        labels, table = pma.assign_pore_and_throat_ids(ctx, mask, edt2, crad2)
        pma.remove_empty_pores(ctx, table, labels)
        ws, ws_table = pma.assign_watershed_ids(ctx, table, crad2, mx)
        dist, cav, cavities = pma.compute_shortest_path_distances(ctx, solid, fp64=True)
        torch.cuda.synchronize()
        return dict(solid=solid, edt2=edt2, max_edt2=mx, crad2=crad2, cx=cx, cy=cy, cz=cz,
                    mask=mask, nb=nb, labels=labels, table=table.rows(), ws=ws,
                    ws_table=ws_table.rows(), dist=dist, cav=cav, cavities=cavities)

    return chain


def _sample_void(solid, k, seed):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    idx = torch.randint(0, solid.numel(), (4 * k,), generator=g, device="cuda")
    idx = idx[solid.reshape(-1)[idx] == 0][:k]
    sz, sx, sy = solid.shape
    z = idx // (sx * sy)
    x = (idx // sy) % sx
    y = idx % sy
    return [(int(a), int(b), int(c)) for a, b, c in zip(z.tolist(), x.tolist(), y.tolist())]


def _window(shape, z, x, y, r):
    sz, sx, sy = shape
    return (max(z - r, 0), min(z + r + 1, sz)), (max(x - r, 0), min(x + r + 1, sx)), \
        (max(y - r, 0), min(y + r + 1, sy))


def test_full_size_properties(run512):
    import torch
    out = run512()
    solid, edt2, crad2 = out["solid"], out["edt2"], out["crad2"]
    shape = solid.shape
    sz, sx, sy = shape
    mx = out["max_edt2"]
    assert mx > 0
    assert torch.equal(edt2 == 0, solid != 0)

    rmax = int(math.isqrt(mx)) + 1
    for (z, x, y) in _sample_void(solid, 400, 7):
        e = int(edt2[z, x, y])
        # EDT: nearest solid inside a window of radius ceil(sqrt(e)) + 1
        r = int(math.isqrt(e)) + 2
        (z0, z1), (x0, x1), (y0, y1) = _window(shape, z, x, y, r)
        sub = solid[z0:z1, x0:x1, y0:y1] != 0
        dz = (torch.arange(z0, z1, device="cuda") - z).view(-1, 1, 1)
        dx = (torch.arange(x0, x1, device="cuda") - x).view(1, -1, 1)
        dy = (torch.arange(y0, y1, device="cuda") - y).view(1, 1, -1)
        d2 = (dz * dz + dx * dx + dy * dy).expand(sub.shape)
        assert int(d2[sub].min()) == e, (z, x, y)
        # containing ball: every centre within rmax is a candidate
        (z0, z1), (x0, x1), (y0, y1) = _window(shape, z, x, y, rmax)
        ew = edt2[z0:z1, x0:x1, y0:y1].long()
        dz = (torch.arange(z0, z1, device="cuda") - z).view(-1, 1, 1)
        dx = (torch.arange(x0, x1, device="cuda") - x).view(1, -1, 1)
        dy = (torch.arange(y0, y1, device="cuda") - y).view(1, 1, -1)
        d2 = dz * dz + dx * dx + dy * dy
        cover = (ew > 0) & (d2 <= ew)
        best = int(ew[cover].max())
        assert int(crad2[z, x, y]) == best, (z, x, y)
        zz = torch.arange(z0, z1, device="cuda").view(-1, 1, 1).expand(ew.shape)
        xx = torch.arange(x0, x1, device="cuda").view(1, -1, 1).expand(ew.shape)
        yy = torch.arange(y0, y1, device="cuda").view(1, 1, -1).expand(ew.shape)
        win = cover & (ew == best)
        lex = (xx[win] * sy + yy[win]) * sz + zz[win]
        k = int(lex.min())
        wx, wy, wz = k // (sy * sz), (k // sz) % sy, k % sz
        assert (int(out["cx"][z, x, y]), int(out["cy"][z, x, y]), int(out["cz"][z, x, y])) == \
            (wx, wy, wz), (z, x, y)

    # maximum-ball mask = the set of winning centres
    void = solid == 0
    lin = (out["cz"][void].long() * sx + out["cx"][void].long()) * sy + out["cy"][void].long()
    winners = torch.unique(lin)
    assert winners.numel() == out["nb"]
    mask = out["mask"].reshape(-1)
    assert bool((mask[winners] == 255).all())
    assert int((mask == 255).sum()) == out["nb"]
    assert int((mask == 0).sum()) == int((solid != 0).sum())

    # pores and watershed tables against the label images
    for labels, (pores, throats) in ((out["labels"], out["table"]), (out["ws"], out["ws_table"])):
        ids, counts = torch.unique(labels.view(torch.int32).long() & 0xFFFFFFFF, return_counts=True)
        have = dict(zip(ids.tolist(), counts.tolist()))
        want = {p[0]: p[6] for p in pores}
        want.update({t[0]: t[1] for t in throats})
        for i, c in have.items():
            if i != 0:
                assert want.get(i) == c, i
        for i, c in want.items():
            assert have.get(i, 0) == c, i
        # a seed voxel keeps its pore, or becomes a shared type that lists the pore
        lists = {t[0]: t[2] for t in throats}
        for p in pores:
            at = int(labels[p[3], p[1], p[2]]) & 0xFFFFFFFF
            assert at == p[0] or p[0] in lists.get(at, ()), p
        assert all(t[0] >= THROAT_MIN for t in throats)
        assert all(p[0] < THROAT_MIN for p in pores)

    # float64 geodesics: the rounded fixed point
    d = out["dist"]
    reached = (d >= 0) & (d < np.finfo(np.float64).max)
    inf = torch.tensor(float("inf"), dtype=torch.float64, device="cuda")
    best = torch.full(shape, float("inf"), dtype=torch.float64, device="cuda")
    for ddx in (-1, 0, 1):
        for ddy in (-1, 0, 1):
            for ddz in (-1, 0, 1):
                k = abs(ddx) + abs(ddy) + abs(ddz)
                if k == 0:
                    continue
                w = math.sqrt(k)
                dst = (slice(max(ddz, 0), sz + min(ddz, 0)), slice(max(ddx, 0), sx + min(ddx, 0)),
                       slice(max(ddy, 0), sy + min(ddy, 0)))
                src = (slice(max(-ddz, 0), sz + min(-ddz, 0)), slice(max(-ddx, 0), sx + min(-ddx, 0)),
                       slice(max(-ddy, 0), sy + min(-ddy, 0)))
                cand = torch.where(reached[src], d[src] + w, inf)
                best[dst] = torch.minimum(best[dst], cand)
    seeds = torch.zeros(shape, dtype=torch.bool, device="cuda")
    for c in out["cavities"]:
        seeds[c[3], c[1], c[2]] = True
        assert float(d[c[3], c[1], c[2]]) == 0.0
    check = reached & ~seeds
    assert torch.equal(best[check], d[check])
    unreached_void = void & ~reached
    assert bool(torch.isinf(best[unreached_void]).all())
    assert bool((d[solid != 0] == -1).all())


def test_full_size_repeat_is_bitwise_identical(run512):
    import torch
    a = run512()
    b = run512()
    for key in ("edt2", "crad2", "cx", "cy", "cz", "mask", "labels", "ws", "cav"):
        assert torch.equal(a[key], b[key]), key
    assert torch.equal(a["dist"].view(torch.int64), b["dist"].view(torch.int64))
    assert a["table"] == b["table"]
    assert a["ws_table"] == b["ws_table"]
    assert a["cavities"] == b["cavities"]
