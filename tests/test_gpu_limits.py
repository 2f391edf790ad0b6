"""Bounded device loops: each bound of pma_limits, set low on a context, makes the call that
reaches it return PMA_ERR_LIMIT instead of looping on, and the same context then computes a
correct result once the bounds are back. The device waits are shown to give up by a wait on a
flag that nothing sets (pma_selftest_bounded_wait). Nothing here faults or hangs the GPU: every
loop stops at its bound and reports it through a status word the host reads."""
import numpy as np
import pytest

from cases import make_case

pytestmark = pytest.mark.gpu


@pytest.fixture
def limited_ctx(ctx):
    saved = ctx.limits
    yield ctx
    ctx.set_limits(**saved)


def _still_correct(ctx, oracle_mod):
    import porousmediaanalysis_gb300 as pma
    vol, _ = make_case("union_small")
    res = pma.pipeline_host(ctx, vol, fields=("watershed_labels", "dist_f32"))
    o = oracle_mod.full(vol)
    assert (res["watershed_labels"] == o["pores"].labels_ws).all()
    assert (res["dist_f32"].view(np.uint32) == o["dist"].view(np.uint32)).all()


def _expect_limit(fn, words):
    import porousmediaanalysis_gb300 as pma
    with pytest.raises(pma.PmaError) as e:
        fn()
    assert e.value.status == 5 and words in str(e.value)


def test_limits_round_trip(limited_ctx):
    ctx = limited_ctx
    d = ctx.limits
    assert d["spin_limit"] == 1 << 20 and d["union_limit"] == 1 << 22
    ctx.set_limits(watershed_generations=7, geodesic_buckets=9)
    assert ctx.limits["watershed_generations"] == 7 and ctx.limits["geodesic_buckets"] == 9


def test_watershed_generation_limit(limited_ctx, oracle_mod):
    import porousmediaanalysis_gb300 as pma
    ctx = limited_ctx
    vol, _ = make_case("union_small")
    ctx.set_limits(watershed_generations=1)
    _expect_limit(lambda: pma.pipeline_host(ctx, vol, run_geodesic=False, fields=("watershed_labels",)),
                  "generation limit")
    ctx.set_limits(watershed_generations=(1 << 23) - 1)
    _still_correct(ctx, oracle_mod)


def _u_plateau():
    """One equal-radius plateau shaped like a U in a 1 x 6 x 5 slice: its two legs start trees
    of their own in the union-find (each leg's smallest voxel has no smaller equal neighbour),
    so the bottom bar must union them. Returns (mask, edt2, crad2) for pma_pores."""
    crad = np.zeros((1, 6, 5), np.uint32)
    crad[0, :5, 0] = 5
    crad[0, :5, 4] = 5
    crad[0, 4, :] = 5
    mask = np.where(crad > 0, 127, 0).astype(np.uint8)
    mask[0, 0, 0] = 255
    return mask, crad.copy(), crad


def test_union_find_limit(limited_ctx, oracle_mod):
    import torch
    import porousmediaanalysis_gb300 as pma
    ctx = limited_ctx
    mask, edt2, crad2 = _u_plateau()
    dev = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()
    ctx.set_limits(union_limit=0)
    _expect_limit(lambda: pma.assign_pore_and_throat_ids(ctx, dev(mask), dev(edt2), dev(crad2)), "union-find")
    ctx.set_limits(union_limit=1 << 22)
    labels, table = pma.assign_pore_and_throat_ids(ctx, dev(mask), dev(edt2), dev(crad2))
    r = oracle_mod.pores_and_watershed(mask, edt2, crad2, 5)
    assert (labels.cpu().numpy().view(np.uint32) == r.labels_initial).all()
    assert table.rows()[0] == r.pores0
    _still_correct(ctx, oracle_mod)


def test_geodesic_bucket_limit(limited_ctx, oracle_mod):
    import porousmediaanalysis_gb300 as pma
    ctx = limited_ctx
    vol = np.zeros((48, 48, 48), np.uint8)  # distances up to ~42: more than 32 buckets
    ctx.set_limits(geodesic_buckets=5)
    _expect_limit(lambda: pma.pipeline_host(ctx, vol, run_pores=False, fields=("dist_f32",)),
                  "bucket sweep")
    ctx.set_limits(geodesic_buckets=0)
    _still_correct(ctx, oracle_mod)


def test_device_wait_gives_up(limited_ctx, oracle_mod):
    import time
    ctx = limited_ctx
    ctx.set_limits(spin_limit=1000)
    assert ctx.selftest_bounded_wait()
    ctx.set_limits(spin_limit=1 << 20)
    t0 = time.perf_counter()
    assert ctx.selftest_bounded_wait()  # the default bound ends the wait within seconds
    assert time.perf_counter() - t0 < 30
    _still_correct(ctx, oracle_mod)
