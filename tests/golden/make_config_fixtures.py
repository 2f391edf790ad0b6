"""Generates the oracle's digests for two benchmark workloads, so that the GPU tests can check
them bit for bit without running the oracle (which needs tens of minutes on them):

  grf512.json.gz     the 512^3 thresholded Gaussian random field (sigma 3, porosity 0.65,
                     seed 2), built by synth.grf_exact (exact arithmetic: the same volume on
                     every machine);
  batch256.json.gz   the 256-volume sphere-pack batch (axes log-uniform in [32, 192], radii
                     U[3, 12], solid fraction 0.40; bench.batch_volumes()).

Each volume's record holds digests of every field (squared EDT, containing radii and centres,
maximum-ball mask, pore labels before and after empty-pore removal, watershed labels, float32
and float64 geodesics, cavity ids), the statistics, and digests of every table (pores and
shared types of the initial propagation, after removal and of the watershed). Initial and
post-removal shared types are stored both exactly (ids in the reference's creation order) and
without ids (canonical label digests, sorted pore lists).

Run once on CPU:  python tests/golden/make_config_fixtures.py [grf512|batch256 ...]
"""
import gzip
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

HERE = os.path.dirname(os.path.abspath(__file__))


def record(vol, short=False):
    """The oracle's full pipeline on one volume, as digests. short=True keeps 32 hex digits."""
    import oracle
    from util import canonical_throats, digest, rows_digest, throat_lists_digest, trimmed_hist
    cut = (lambda s: s[:32]) if short else (lambda s: s)
    dg = lambda a: cut(digest(a))
    o = oracle.full(vol, geodesic_too=False)
    r = o["pores"]
    dist32, cav32, rows32 = oracle.geodesic(vol, fp64=False)
    dist64, cav64, rows64 = oracle.geodesic(vol, fp64=True)
    assert np.array_equal(cav32, cav64)
    return {
        "shape": list(vol.shape),
        "solid": dg(vol),
        "max_edt2": int(o["max_edt2"]),
        "maximum_balls_count": int(o["maximum_balls_count"]),
        "hist": cut(rows_digest(trimmed_hist(o["hist"]))),
        "edt2": dg(o["edt2"]), "crad2": dg(o["crad2"]),
        "cx": dg(o["cx"]), "cy": dg(o["cy"]), "cz": dg(o["cz"]), "mask": dg(o["mask"]),
        "npores0": len(r.pores0), "nthroats0": len(r.throats0),
        "pores0": cut(rows_digest(r.pores0)),
        "throats0": cut(rows_digest(r.throats0)),
        "throats0_lists": cut(throat_lists_digest(r.throats0)),
        "labels_initial": dg(r.labels_initial),
        "labels_initial_canonical": dg(canonical_throats(r.labels_initial)),
        "npores": len(r.pores), "nthroats": len(r.throats),
        "pores": cut(rows_digest(r.pores)),
        "throats": cut(rows_digest(r.throats)),
        "throats_lists": cut(throat_lists_digest(r.throats)),
        "labels": dg(r.labels),
        "labels_canonical": dg(canonical_throats(r.labels)),
        "labels_ws": dg(r.labels_ws),
        "npores_ws": len(r.pores_ws), "nthroats_ws": len(r.throats_ws),
        "pores_ws": cut(rows_digest(r.pores_ws)),
        "throats_ws": cut(rows_digest(r.throats_ws)),
        "dist_f32": dg(dist32), "dist_f64": dg(dist64), "cavity": dg(cav64),
        "cavities": [list(c[:4]) + [float(c[4])] + list(c[5:]) for c in rows64],
    }


def grf512():
    from porousmediaanalysis_gb300 import synth
    vol = synth.grf_exact((512, 512, 512), sigma=3.0, porosity=0.65, seed=2)
    rec = record(vol)
    rec["generator"] = "synth.grf_exact((512, 512, 512), sigma=3.0, porosity=0.65, seed=2)"
    return rec


def _batch_one(i):
    return i, record(_batch_volume(i), short=True)


def _batch_volume(i, count=256, seed=4):
    """Volume i of bench.batch_volumes() (the same shapes and seeds), built alone."""
    from porousmediaanalysis_gb300 import synth
    shape = synth.batch_shapes(count, lo=32, hi=192, seed=seed)[i]
    return synth.sphere_pack(shape, rmin=3.0, rmax=12.0, solid_fraction=0.40, seed=seed * 1000 + i)


def batch256(workers=None):
    import oracle
    oracle.build()
    workers = workers or os.cpu_count() or 1
    out = [None] * 256
    with mp.get_context("spawn").Pool(workers) as pool:
        for i, rec in pool.imap_unordered(_batch_one, range(256)):
            out[i] = rec
    return {"generator": "bench.batch_volumes(): 256 sphere packs", "volumes": out}


def main():
    import oracle
    oracle.build()
    which = sys.argv[1:] or ["grf512", "batch256"]
    for name in which:
        t0 = time.time()
        rec = {"grf512": grf512, "batch256": batch256}[name]()
        with gzip.open(os.path.join(HERE, name + ".json.gz"), "wt") as f:
            json.dump(rec, f, separators=(",", ":"))
        print(name, "done in %.0f s" % (time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
