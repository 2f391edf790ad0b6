"""Serving (pma_server_*) through the C ABI: continuous batching under a device-memory budget.
Each request's result in a mix of concurrent requests equals its result alone, admission
respects the budget, and a request larger than the budget alone is rejected."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("edt2", "crad2", "maxball_mask", "pore_labels", "watershed_labels", "dist_f64", "cavity")


def _requests(count, seed):
    from porousmediaanalysis_gb300 import synth
    rng = np.random.default_rng(seed)
    vols = []
    for i in range(count):
        side = int(rng.choice([16, 24, 32, 48, 64]))
        if i % 2:
            vols.append(synth.grf((side, side, side), sigma=float(rng.uniform(1.5, 3.0)),
                                  porosity=float(rng.uniform(0.5, 0.8)), seed=seed + i))
        else:
            vols.append(synth.sphere_pack((side, side, side), rmin=2.0, rmax=6.0, solid_fraction=0.4,
                                          seed=seed + i))
    return vols


def _same(a, b):
    for k in FIELDS:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        if k == "dist_f64":
            x, y = x.view(np.int64), y.view(np.int64)
        assert np.array_equal(x, y), k
    assert a["pores"].rows() == b["pores"].rows()
    assert a["watershed"].rows() == b["watershed"].rows()
    assert a["cavities"] == b["cavities"]
    assert (a["max_edt2"], a["maximum_balls_count"]) == (b["max_edt2"], b["maximum_balls_count"])


def test_mixed_requests_equal_alone(ctx):
    import porousmediaanalysis_gb300 as pma
    vols = _requests(20, 70)
    alone = [pma.pipeline_host(ctx, v, fp64=True, fields=FIELDS) for v in vols]
    rng = np.random.default_rng(3)
    with pma.Server(ctx, lanes=6, fp64=True) as srv:
        tickets = []
        for v in vols:  # staggered arrivals: later requests join while earlier ones run
            tickets.append(srv.submit(v, fields=FIELDS))
            time.sleep(float(rng.exponential(0.002)))
        got = [srv.wait(t, timeout_ms=120000) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(vols) and st["failed"] == 0 and st["rejected"] == 0
    assert st["max_in_flight"] >= 2
    for (res, latency), ref in zip(got, alone):
        assert latency > 0
        _same(res, ref)


def test_budget_limits_requests_in_flight(ctx):
    import porousmediaanalysis_gb300 as pma
    vols = _requests(8, 90)
    alone = [pma.pipeline_host(ctx, v, fp64=True, fields=FIELDS) for v in vols]
    budget = 400 << 20
    with pma.Server(ctx, lanes=8, memory_budget=budget, fp64=True) as srv:
        tickets = [srv.submit(v, fields=FIELDS) for v in vols]
        got = [srv.wait(t, timeout_ms=120000) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(vols)
    assert st["peak_reserved_bytes"] <= budget
    for (res, _), ref in zip(got, alone):
        _same(res, ref)


def test_request_beyond_budget_is_rejected(ctx):
    import porousmediaanalysis_gb300 as pma
    vols = _requests(1, 7)
    big = np.zeros((96, 96, 96), np.uint8)
    with pma.Server(ctx, lanes=2, memory_budget=80 << 20) as srv:
        t = srv.submit(big)
        with pytest.raises(pma.PmaError, match="budget"):
            srv.wait(t, timeout_ms=60000)
        assert srv.stats()["rejected"] == 1
        with pytest.raises(pma.PmaError):
            srv.wait(t, timeout_ms=0)  # a ticket is waited for once
    del vols
