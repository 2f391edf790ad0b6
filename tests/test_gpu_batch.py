"""Batched form (pma_pipeline_batch) through the C ABI: every volume of a batch of uneven
sphere packs equals the oracle run volume by volume, from host buffers and from device
buffers, with any number of lanes."""
import numpy as np
import pytest

from util import canonical_throats

pytestmark = pytest.mark.gpu

FIELDS = ("edt2", "crad2", "cx", "cy", "cz", "maxball_mask", "pore_labels", "watershed_labels",
          "dist_f64", "cavity")


def _batch(count, seed):
    from porousmediaanalysis_gb300 import synth
    shapes = synth.batch_shapes(count, lo=12, hi=64, seed=seed)
    return [synth.sphere_pack(s, rmin=2.0, rmax=7.0, solid_fraction=0.4, seed=seed + i)
            for i, s in enumerate(shapes)]


@pytest.fixture(scope="module")
def batch_and_oracle(oracle_mod):
    vols = _batch(24, 40)
    ref = []
    for v in vols:
        o = oracle_mod.full(v, geodesic_too=False)
        o["dist"], o["cavity"], o["cavities"] = oracle_mod.geodesic(v, fp64=True)
        ref.append(o)
    return vols, ref


def _check(res, o):
    as_u32 = lambda a: np.asarray(a).view(np.uint32) if np.asarray(a).dtype != np.uint8 else np.asarray(a)
    for k in ("edt2", "crad2", "cx", "cy", "cz"):
        assert np.array_equal(as_u32(res[k]), o[k]), k
    assert np.array_equal(res["maxball_mask"], o["mask"])
    assert res["max_edt2"] == o["max_edt2"]
    assert res["maximum_balls_count"] == o["maximum_balls_count"]
    r = o["pores"]
    assert res["pores"].rows()[0] == r.pores
    assert (canonical_throats(as_u32(res["pore_labels"])) == canonical_throats(r.labels)).all()
    assert np.array_equal(as_u32(res["watershed_labels"]), r.labels_ws)
    wp, wt = res["watershed"].rows()
    assert wp == r.pores_ws and wt == r.throats_ws
    assert np.array_equal(np.asarray(res["dist_f64"]).view(np.int64), o["dist"].view(np.int64))
    assert np.array_equal(as_u32(res["cavity"]), o["cavity"])
    assert [c[:4] + c[5:] for c in res["cavities"]] == [c[:4] + c[5:] for c in o["cavities"]]


@pytest.mark.parametrize("lanes", [1, 4, 16])
def test_batch_host_buffers_match_oracle(ctx, batch_and_oracle, lanes):
    import porousmediaanalysis_gb300 as pma
    vols, ref = batch_and_oracle
    out = pma.pipeline_batch(ctx, vols, fp64=True, fields=FIELDS, lanes=lanes)
    assert len(out) == len(vols)
    for res, o in zip(out, ref):
        _check(res, o)


def test_batch_device_buffers_match_oracle(ctx, batch_and_oracle):
    import torch
    import porousmediaanalysis_gb300 as pma
    vols, ref = batch_and_oracle
    dvols = [torch.from_numpy(v).cuda() for v in vols]
    out = pma.pipeline_batch(ctx, dvols, fp64=True, fields=FIELDS, resident=True, lanes=6)
    torch.cuda.synchronize()
    for res, o in zip(out, ref):
        host = {k: (v.cpu().numpy() if isinstance(v, torch.Tensor) else v) for k, v in res.items()}
        _check(host, o)


def test_batch_rejects_bad_items_before_running(ctx):
    import ctypes
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import capi
    items = (capi.BatchItem * 1)()
    items[0].solid = None
    items[0].dims = capi.Dims(4, 4, 4)
    outs = capi.Outputs()
    items[0].out = ctypes.pointer(outs)
    status = capi.lib().pma_pipeline_batch(ctx.handle, items, 1, None, 0, 2)
    assert capi.STATUS[status] == "PMA_ERR_ARGUMENT"
    assert "null item" in capi.last_error()
    with pytest.raises(pma.PmaError):
        pma.pipeline_batch(ctx, [np.zeros((0, 4, 4), np.uint8)])
