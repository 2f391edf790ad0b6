"""The pore stage's parallel sort of the maximum balls gives std::sort's exact permutation
(ties included), checked by a small C++ program against std::sort on random inputs."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "porousmediaanalysis_gb300", "csrc")


def test_ordered_sort_equals_std_sort(tmp_path):
    exe = str(tmp_path / "ordered_sort_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC,
                        os.path.join(HERE, "ordered_sort_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("build failed:\n" + r.stderr)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
