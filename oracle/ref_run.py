"""Runs the reference executable oracle/_ref/pma_ref (built by oracle/build_ref.sh) on a
numpy volume and reads its outputs back.

TEST INFRASTRUCTURE ONLY, for this container: it pins the oracle restatement against the
reference itself and generates the committed fixtures under tests/golden/. Files are in
the private format of oracle/ref_shim/FreeImagePlus.h.
"""
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "pma_ref")

FIELDS = {
    "EuclideanDistanceSquares": np.uint32, "ContainingBallRadiiSquares": np.uint32,
    "ContainingBallCoordinatesX": np.uint32, "ContainingBallCoordinatesY": np.uint32,
    "ContainingBallCoordinatesZ": np.uint32, "IsMaximumBall": np.uint8,
    "PoreThroatIds": np.uint32, "PoreThroatIdsWatershed": np.uint32,
    "ShortestPathDistances": np.float32, "CavityIds": np.uint32,
}


def _write_slice(path, plane):
    h, w = plane.shape
    bpp = plane.dtype.itemsize * 8
    with open(path, "wb") as f:
        f.write(b"PMASHIM1")
        f.write(struct.pack("<3I", w, h, bpp))
        f.write(np.ascontiguousarray(plane).tobytes())


def _read_slice(path, dtype):
    with open(path, "rb") as f:
        assert f.read(8) == b"PMASHIM1", path
        w, h, bpp = struct.unpack("<3I", f.read(12))
        data = f.read()
    assert bpp == np.dtype(dtype).itemsize * 8, (path, bpp)
    return np.frombuffer(data, dtype=dtype).reshape(h, w)


def read_stack(folder, dtype):
    names = sorted(os.listdir(folder), key=lambda n: os.path.splitext(n)[0])
    return np.stack([_read_slice(os.path.join(folder, n), dtype) for n in names])


def run(solid, modes=("-all", "-spd"), threads=1, d3q7=False, keep=None, resolution="1 1 1"):
    """solid: (SZ, SX, SY) array, non-zero = solid. Returns (fields dict, text files dict);
    fields include "Images", the (possibly resampled) input stack after the run."""
    assert os.path.exists(REF_BIN), "build the reference checker with oracle/build_ref.sh"
    root = keep or tempfile.mkdtemp(prefix="pma_ref_")
    sample = os.path.join(root, "sample")
    os.makedirs(os.path.join(sample, "Images"), exist_ok=True)
    sz = solid.shape[0]
    width = len(str(sz))
    for z in range(sz):
        _write_slice(os.path.join(sample, "Images", "%0*d.tif" % (width, z + 1)),
                     np.where(np.asarray(solid[z]) != 0, 255, 0).astype(np.uint8))
    with open(os.path.join(sample, "config.txt"), "w") as f:
        f.write("Resolution of initial images: %s\n"
                "Available memory in megabytes: 200000\n"
                "Max ratio of pore radius to seed radius: 10.0\n"
                "Use D3Q7 stencil: %d\n"
                "Number of threads: %d\n" % (resolution, 1 if d3q7 else 0, threads))
    for m in modes:
        r = subprocess.run([REF_BIN, m], cwd=root, capture_output=True, text=True)
        if r.returncode != 0 or "rror" in r.stdout[-300:]:
            raise RuntimeError("reference failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    fields = {"Images": read_stack(os.path.join(sample, "Images"), np.uint8)}
    for name, dt in FIELDS.items():
        p = os.path.join(sample, name)
        if os.path.isdir(p):
            fields[name] = read_stack(p, dt)
    texts = {}
    for n in os.listdir(sample):
        if n.endswith(".txt") and n != "config.txt":
            texts[n] = open(os.path.join(sample, n)).read()
    if keep is None:
        shutil.rmtree(root)
    return fields, texts


def parse_pores(text):
    rows = []
    for line in text.strip().splitlines()[1:]:
        a = line.split()
        rows.append((int(a[0]), int(a[1]), int(a[2]), int(a[3]), int(a[4]), int(a[5]), int(a[6])))
    return rows


def parse_throats(text):
    rows = []
    for line in text.strip().splitlines()[1:]:
        tid, vol, rest = line.split(";", 2)
        rows.append((int(tid), int(vol), tuple(int(x) for x in rest.split())))
    return rows


def parse_cavities(text):
    rows = []
    for line in text.strip().splitlines()[1:]:
        a = line.split()
        rows.append((int(a[0]), int(a[1]), int(a[2]), int(a[3]), float(a[4]), int(a[5]),
                     int(a[6]), int(a[7])))
    return rows
