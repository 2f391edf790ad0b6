"""Helpers shared by the tests: digests and table normalisation."""
import hashlib

import numpy as np


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rows(x):
    """JSON lists of lists -> tuples, so fixture tables compare with Python tuples."""
    out = []
    for r in x:
        out.append(tuple(tuple(v) if isinstance(v, list) else v for v in r))
    return out


def trimmed_hist(hist):
    """The histogram lines euclideanDistanceSquareCounts.txt holds: entries 1 .. last non-zero,
    plus one zero (EuclideanDistanceComputer.cpp:83-110, Serializer.cpp:148-159)."""
    h = [int(v) for v in hist] + [0]
    nz = [i for i, v in enumerate(h) if v]
    return h[1:nz[-1] + 2] if nz else []


def cavity_key(c):
    """Cavity row without the printed float (compared separately at %f precision)."""
    return (c[0], c[1], c[2], c[3], c[5], c[6], c[7])


def canonical_labels(labels):
    """Relabels ids by order of first appearance in scan order (for comparisons up to an
    id permutation)."""
    flat = labels.reshape(-1)
    uniq, first = np.unique(flat, return_index=True)
    order = np.argsort(first)
    remap = np.empty(len(uniq), dtype=np.int64)
    remap[order] = np.arange(len(uniq))
    inv = np.searchsorted(uniq, flat)
    return remap[inv].reshape(labels.shape)


THROAT_MIN = 0x80000000


def canonical_throats(labels):
    """Keeps pore ids and 0, renames shared-type ids (>= 2^31) by order of first appearance
    in [z][x][y] scan order. Two label images that differ only by a one-to-one renaming of
    type ids have the same canonical form."""
    flat = np.ascontiguousarray(labels).reshape(-1).astype(np.uint32)
    out = flat.copy()
    sel = flat >= THROAT_MIN
    if sel.any():
        ids = flat[sel]
        uniq, first = np.unique(ids, return_index=True)
        order = np.argsort(first)
        rank = np.empty(len(uniq), dtype=np.uint32)
        rank[order] = np.arange(len(uniq), dtype=np.uint32)
        out[sel] = THROAT_MIN + rank[np.searchsorted(uniq, ids)]
    return out.reshape(labels.shape)


def rows_digest(x):
    """Digest of a table's rows (tuples or lists of ints and tuples), independent of whether
    they came from JSON lists or Python tuples."""
    import json

    def norm(v):
        if isinstance(v, (list, tuple)):
            return [norm(u) for u in v]
        return int(v)
    return hashlib.sha256(json.dumps(norm(list(x)), separators=(",", ":")).encode()).hexdigest()


def throat_lists_digest(throats):
    """Digest of a shared-type table without its ids: the sorted (pore list, volume) pairs.
    Equal for two tables that differ only by a renaming of the ids."""
    return rows_digest(sorted((tuple(t[2]), t[1]) for t in throats))
