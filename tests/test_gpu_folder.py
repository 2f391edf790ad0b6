"""The folder-level drop-in (pma_run_folder and the pma tool) end to end: a sample folder with
config.txt and Images/ is processed like the reference's `-all` and `-spd` modes
(CommandLineDispatcher.cpp:34-72), and every file it writes is compared with the reference
run with one thread on the same volume: text files byte for byte
(tests/golden/folder_texts.json, made by tests/golden/make_folder_texts.py), TIFF folders as
decoded fields against the reference's digests, shared-type ids included.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from cases import load_example, make_case, many_pockets
from conftest import GOLDEN, ROOT
from util import digest

pytestmark = pytest.mark.gpu

EXACT_TEXTS = ("intermediateStatistics.txt", "euclideanDistanceSquareCounts.txt", "pores.txt",
               "sharedPixelTypes.txt", "poresWatershed.txt", "sharedPixelTypesWatershed.txt",
               "cavityDescriptions.txt")
FOLDERS = {"EuclideanDistanceSquares": 4, "ContainingBallRadiiSquares": 4, "ContainingBallCoordinatesX": 4,
           "ContainingBallCoordinatesY": 4, "ContainingBallCoordinatesZ": 4, "IsMaximumBall": 1,
           "PoreThroatIds": 4, "PoreThroatIdsWatershed": 4, "ShortestPathDistances": 4, "CavityIds": 4}


@pytest.fixture(scope="module")
def texts():
    with open(os.path.join(GOLDEN, "folder_texts.json")) as f:
        return json.load(f)


def make_sample(root, vol, d3q7=False, resolution="1 1 1"):
    """A sample folder as the reference expects it: Images/ (255 = solid) and config.txt."""
    from porousmediaanalysis_gb300 import capi
    sample = os.path.join(root, "sample")
    capi.write_tiff_stack(os.path.join(sample, "Images"), np.where(vol != 0, 255, 0).astype(np.uint8))
    with open(os.path.join(sample, "config.txt"), "w") as f:
        f.write("Resolution of initial images: %s\n"
                "Available memory in megabytes: 200000\n"
                "Max ratio of pore radius to seed radius: 10.0\n"
                "Use D3Q7 stencil: %d\n"
                "Number of threads: 1\n" % (resolution, 1 if d3q7 else 0))
    return sample


def check_sample(sample, ref_texts, rec):
    from porousmediaanalysis_gb300 import capi
    for name in EXACT_TEXTS:
        with open(os.path.join(sample, name)) as f:
            assert f.read() == ref_texts[name], name
    for name, bpv in FOLDERS.items():
        a = capi.read_tiff_stack(os.path.join(sample, name), bpv)
        assert digest(a) == rec["digests"][name], name


@pytest.mark.parametrize("name", ["two_cavities", "pack_small", "union_small_d3q7", "slab_rows"])
def test_run_folder_all_then_spd(ctx, tmp_path, texts, ref_cases, name):
    import porousmediaanalysis_gb300 as pma
    vol, d3q7 = make_case(name)
    sample = make_sample(str(tmp_path), vol, d3q7)
    pma.run_folder(ctx, str(tmp_path), pma.MODE_ALL)
    pma.run_folder(ctx, str(tmp_path), pma.MODE_SPD)
    check_sample(sample, texts[name], ref_cases[name])


def test_run_folder_stage_by_stage(ctx, tmp_path, texts, ref_cases):
    """-edt, -rib, -apt, -spd one after another, each reading the folders the previous one
    wrote, give the same files as -all."""
    import porousmediaanalysis_gb300 as pma
    vol, d3q7 = make_case("pack_small")
    sample = make_sample(str(tmp_path), vol, d3q7)
    for mode in (pma.MODE_EDT, pma.MODE_RIB, pma.MODE_APT, pma.MODE_SPD):
        pma.run_folder(ctx, str(tmp_path), mode)
    check_sample(sample, texts["pack_small"], ref_cases["pack_small"])


def test_run_folder_example_with_the_pma_tool(tmp_path, texts, example_golden, pma_lib):
    """The shipped example through the command-line tool (`pma -all`, then `pma -spd`, run in
    the folder above the sample like the reference's executable)."""
    vol = load_example(GOLDEN)
    sample = make_sample(str(tmp_path), vol)
    tool = os.path.join(ROOT, "porousmediaanalysis_gb300", "_build", "pma")
    for mode in ("-all", "-spd"):
        r = subprocess.run([tool, mode], cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "rror" not in r.stdout, r.stdout
    check_sample(sample, texts["example"], example_golden["reference_1_thread"])


def test_run_folder_writes_every_cavity(ctx, tmp_path, texts):
    """49 cavities: cavityDescriptions.txt holds every row, as the reference's does."""
    import porousmediaanalysis_gb300 as pma
    sample = make_sample(str(tmp_path), many_pockets())
    pma.run_folder(ctx, str(tmp_path), pma.MODE_SPD)
    with open(os.path.join(sample, "cavityDescriptions.txt")) as f:
        got = f.read()
    assert got == texts["many_pockets"]["cavityDescriptions.txt"]
    assert got.count("\n") == 50


def test_run_folder_reports_errors(ctx, tmp_path):
    """A malformed config.txt or an empty Images/ folder fails the call with its message."""
    import porousmediaanalysis_gb300 as pma
    sample = tmp_path / "sample"
    (sample / "Images").mkdir(parents=True)
    (sample / "config.txt").write_text("Resolution of initial images: 1 1 1\n")
    with pytest.raises(pma.PmaError):
        pma.run_folder(ctx, str(tmp_path), pma.MODE_ALL)
    (sample / "config.txt").write_text("Resolution of initial images: 1 1 1\nAvailable memory in megabytes: 10\n"
                                       "Max ratio of pore radius to seed radius: 10.0\nUse D3Q7 stencil: 0\n"
                                       "Number of threads: 1\n")
    with pytest.raises(pma.PmaError) as e:
        pma.run_folder(ctx, str(tmp_path), pma.MODE_ALL)
    assert "Images" in str(e.value)


@pytest.mark.parametrize("name,case,resolution", [("pack_odd_z2", "pack_odd", "1 1 2"),
                                                  ("pack_odd_xy", "pack_odd", "2 1.5 1"),
                                                  ("union_small_xyz", "union_small", "1.5 2 1.25")])
def test_run_folder_resamples_the_input_stack(ctx, tmp_path, texts, name, case, resolution):
    """A resolution other than 1 1 1 makes -all and -spd resample Images/ first
    (ImageResampler.cpp:28-67): Original/ keeps the slices, Images/ gets the repeated and
    in-plane upsampled ones, and every later stage runs on those. Compared with the reference
    run (with FreeImage's own resize engine) on the same folder."""
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import capi
    vol, d3q7 = make_case(case)
    sample = make_sample(str(tmp_path), vol, d3q7, resolution)
    pma.run_folder(ctx, str(tmp_path), pma.MODE_ALL)
    pma.run_folder(ctx, str(tmp_path), pma.MODE_SPD)  # Original/ exists: no second resampling
    ref = texts[name]
    images = capi.read_tiff_stack(os.path.join(sample, "Images"), 1)
    assert list(images.shape) == ref["shape"]
    assert digest(images) == ref["digests"]["Images"]
    assert np.array_equal(capi.read_tiff_stack(os.path.join(sample, "Original"), 1),
                          np.where(vol != 0, 255, 0).astype(np.uint8))
    for fname in EXACT_TEXTS:
        with open(os.path.join(sample, fname)) as f:
            assert f.read() == ref[fname], fname
    for fname, bpv in FOLDERS.items():
        assert digest(capi.read_tiff_stack(os.path.join(sample, fname), bpv)) == ref["digests"][fname], fname
