"""Seeded parity volumes shared by the fixture generator and the tests.

Each case is a (SZ, SX, SY) uint8 volume, non-zero = solid, and a stencil flag. The cases
cover the edge cases the reference's behaviour hinges on: all void (virtual X boundary,
one pore), all solid (no pores, no cavity), a single Z slice (five walls), disconnected
cavities (cavity restarts), D3Q7, sphere unions and packs, and the 128^3 benchmark volume.
"""
import numpy as np

from porousmediaanalysis_gb300 import synth


def _two_cavities():
    s = np.ones((24, 30, 28), np.uint8)
    zz, xx, yy = np.ogrid[:24, :30, :28]
    s[(zz - 12) ** 2 + (xx - 15) ** 2 + (yy - 14) ** 2 <= 25] = 0      # pocket around the centre
    s[:, :, :4] = 0                                                    # slab touching 5 walls
    s[(zz - 4) ** 2 + (xx - 25) ** 2 + (yy - 22) ** 2 <= 9] = 0         # isolated pocket
    return s


def _slab_rows():
    s = np.zeros((10, 20, 16), np.uint8)
    s[:, 5, :] = 1      # a full solid X plane
    s[3, :, 7] = 1      # a solid line along X
    return s


CASES = {
    "union_small": lambda: (synth.sphere_union((40, 48, 44), count=40, rmin=3, rmax=7, seed=5), False),
    "union_small_d3q7": lambda: (synth.sphere_union((40, 48, 44), count=40, rmin=3, rmax=7, seed=5), True),
    "pack_small": lambda: (synth.sphere_pack((30, 50, 40), seed=7), False),
    "pack_odd": lambda: (synth.sphere_pack((17, 33, 29), rmin=2, rmax=6, seed=11), False),
    "all_void": lambda: (np.zeros((8, 12, 10), np.uint8), False),
    "all_solid": lambda: (np.ones((6, 7, 8), np.uint8), False),
    "single_slice": lambda: (synth.sphere_union((1, 64, 60), count=30, rmin=2, rmax=6, seed=9), False),
    "two_cavities": lambda: (_two_cavities(), False),
    "slab_rows": lambda: (_slab_rows(), False),
    "union_128": lambda: (synth.sphere_union((128, 128, 128)), False),
}

# Cases light enough for the CPU oracle in the quick suite.
QUICK = [c for c in CASES if c != "union_128"]


def make_case(name):
    vol, d3q7 = CASES[name]()
    return np.ascontiguousarray(vol, dtype=np.uint8), d3q7


def load_example(golden_dir):
    import os
    z = np.load(os.path.join(golden_dir, "example_solid.npz"))
    shape = tuple(int(v) for v in z["shape"])
    n = int(np.prod(shape))
    return np.unpackbits(z["bits"])[:n].reshape(shape).astype(np.uint8)


def large_case():
    """2^24 voxels (256^3): the size from which plateaus are labelled by pointer jumping and
    unions of recorded parent pairs. A union of 6000 spheres, radii U[4, 12]."""
    return synth.sphere_union((256, 256, 256), count=6000, rmin=4.0, rmax=12.0, seed=77)


def many_pockets(count=900, shape=(100, 110, 96), seed=13):
    """A solid block holding `count` small spherical voids, none reaching more than a few
    walls, so that the geodesic stage restarts again and again (49 cavities with the
    defaults; a restart searches shells from one beyond the previous one, so the count is
    bounded by the half-extent of the volume)."""
    rng = np.random.default_rng(seed)
    s = np.ones(shape, np.uint8)
    zz, xx, yy = np.ogrid[:shape[0], :shape[1], :shape[2]]
    for _ in range(count):
        c = rng.uniform(0, 1, 3) * np.array(shape)
        r = rng.uniform(1.0, 2.5)
        s[(zz - c[0]) ** 2 + (xx - c[1]) ** 2 + (yy - c[2]) ** 2 <= r * r] = 0
    return s
