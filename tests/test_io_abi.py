"""Host-side parts that need no GPU: the C ABI exports, TIFF codec, config parsing and the
folder conventions."""
import ctypes
import os

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(pma_lib):
    from porousmediaanalysis_gb300 import capi
    names = capi.declared_symbols()
    assert len(names) >= 27
    missing = [n for n in names if not hasattr(pma_lib, n)]
    assert not missing, missing


def test_abi_version_and_error_channel(pma_lib):
    from porousmediaanalysis_gb300 import capi
    assert pma_lib.pma_abi_version() == 1
    # A call with a null context fails with PMA_ERR_ARGUMENT and sets the message.
    st = pma_lib.pma_edt(None, None, capi.Dims(1, 1, 1), None, None, None, 0)
    assert st == 1
    assert "context" in capi.last_error()


def test_ctx_create_without_gpu_reports_cuda_error(pma_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from porousmediaanalysis_gb300 import capi
    h = ctypes.c_void_p()
    st = pma_lib.pma_ctx_create(0, ctypes.byref(h))
    assert st == 2  # PMA_ERR_CUDA


@pytest.mark.parametrize("dtype", [np.uint8, np.uint32])
def test_tiff_stack_round_trip(pma_lib, tmp_path, dtype):
    from porousmediaanalysis_gb300 import capi
    rng = np.random.default_rng(0)
    if dtype == np.uint8:
        a = (rng.random((3, 37, 29)) < 0.3).astype(np.uint8) * 255
    else:
        a = rng.integers(0, 2 ** 32, size=(3, 37, 29), dtype=np.uint64).astype(np.uint32)
        a[0, :5] = 0xFFFFFFFF
    capi.write_tiff_stack(str(tmp_path / "s"), a)
    b = capi.read_tiff_stack(str(tmp_path / "s"), a.dtype.itemsize)
    assert b.dtype == a.dtype and b.shape == a.shape
    assert (a == b).all()


def test_tiff_lzw_long_runs_and_table_resets(pma_lib, tmp_path):
    """Sizes that fill the 4094-entry LZW table several times within one strip."""
    from porousmediaanalysis_gb300 import capi
    rng = np.random.default_rng(1)
    a = rng.integers(0, 2 ** 32, size=(2, 300, 257), dtype=np.uint64).astype(np.uint32)
    a[1] = np.arange(300 * 257, dtype=np.uint32).reshape(300, 257) % 7
    capi.write_tiff_stack(str(tmp_path / "t"), a)
    assert (capi.read_tiff_stack(str(tmp_path / "t"), 4) == a).all()


def test_float_field_round_trip_keeps_bits(pma_lib, tmp_path):
    from porousmediaanalysis_gb300 import capi
    d = np.array([-1.0, 0.0, 1.4142135, np.finfo(np.float32).max, 3.7320508], np.float32)
    a = np.resize(d, (2, 4, 5))
    capi.write_tiff_stack(str(tmp_path / "f"), a.view(np.uint32))
    assert (capi.read_tiff_stack(str(tmp_path / "f"), 4).view(np.float32) == a).all()


def test_read_stack_rejects_mismatched_slices(pma_lib, tmp_path):
    from porousmediaanalysis_gb300 import capi
    capi.write_tiff_stack(str(tmp_path / "m"), np.zeros((1, 4, 5), np.uint8))
    os.rename(tmp_path / "m" / "1.tif", tmp_path / "m" / "a.tif")
    capi.write_tiff_stack(str(tmp_path / "m"), np.zeros((1, 6, 5), np.uint8))
    with pytest.raises(capi.PmaError) as e:
        capi.read_tiff_stack(str(tmp_path / "m"), 1)
    assert "size" in str(e.value)


def test_read_stack_rejects_truncated_file(pma_lib, tmp_path):
    from porousmediaanalysis_gb300 import capi
    capi.write_tiff_stack(str(tmp_path / "t"), np.ones((1, 40, 40), np.uint8))
    p = tmp_path / "t" / "1.tif"
    data = p.read_bytes()
    p.write_bytes(data[:20])
    with pytest.raises(capi.PmaError):
        capi.read_tiff_stack(str(tmp_path / "t"), 1)


def test_slices_are_ordered_by_name(pma_lib, tmp_path):
    from porousmediaanalysis_gb300 import capi
    folder = tmp_path / "o"
    for z, name in enumerate(["10", "02", "1"]):
        capi.write_tiff_stack(str(tmp_path / "tmp"), np.full((1, 2, 3), z + 1, np.uint8))
        os.makedirs(folder, exist_ok=True)
        os.rename(tmp_path / "tmp" / "1.tif", folder / (name + ".tif"))
    v = capi.read_tiff_stack(str(folder), 1)
    # lexicographic by name without extension: "02" < "1" < "10"
    assert [int(v[z, 0, 0]) for z in range(3)] == [2, 3, 1]


def test_missing_folder_is_an_io_error(pma_lib, tmp_path):
    from porousmediaanalysis_gb300 import capi
    with pytest.raises(capi.PmaError) as e:
        capi.read_tiff_stack(str(tmp_path / "nothing"), 1)
    assert e.value.status == 3


def test_package_refuses_to_run_without_library(monkeypatch, tmp_path):
    from porousmediaanalysis_gb300 import capi
    monkeypatch.setattr(capi, "_lib", None)
    monkeypatch.setattr(capi, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError):
        capi.lib()


CONFIG = ("Resolution of initial images: {r}\n"
          "Available memory in megabytes: 4000\n"
          "Max ratio of pore radius to seed radius: 2.5\n"
          "Use D3Q7 stencil: {d}\n"
          "Number of threads: 7\n")


def test_config_reads_the_reference_format(pma_lib, tmp_path):
    """Serializer.cpp:40-52: five labelled lines; resolutions normalised by the smallest."""
    from porousmediaanalysis_gb300 import capi
    p = tmp_path / "config.txt"
    p.write_text(CONFIG.format(r="1 1 1", d=0))
    c = capi.read_config(p)
    assert c == {"resolution": (1.0, 1.0, 1.0), "max_pore_radius_ratio": 2.5, "available_memory_mb": 4000,
                 "use_d3q7": 0, "threads": 7}
    p.write_text(CONFIG.format(r="2 3 4", d=1).replace("\n", "\r\n"))  # Windows line ends
    c = capi.read_config(p)
    assert c["resolution"] == (1.0, 1.5, 2.0) and c["use_d3q7"] == 1 and c["threads"] == 7


@pytest.mark.parametrize("text", [
    "",
    "Resolution of initial images: 1 1\nAvailable memory in megabytes: 4000\n",
    CONFIG.format(r="1 1 1", d=0).replace("Available memory", "Memory"),
    CONFIG.format(r="0 1 1", d=0),
    CONFIG.format(r="1 -1 1", d=0),
])
def test_config_rejects_malformed_files(pma_lib, tmp_path, text):
    from porousmediaanalysis_gb300 import capi
    p = tmp_path / "config.txt"
    p.write_text(text)
    with pytest.raises(capi.PmaError) as e:
        capi.read_config(p)
    assert e.value.status == 3  # PMA_ERR_IO
    with pytest.raises(capi.PmaError):
        capi.read_config(tmp_path / "missing.txt")


def test_written_stack_keeps_slice_order(pma_lib, tmp_path):
    """Slices are named with zero padding, so the name order (by which the reference and the
    reader sort) is the slice order beyond nine slices."""
    from porousmediaanalysis_gb300 import capi
    a = np.arange(12 * 3 * 4, dtype=np.uint8).reshape(12, 3, 4)
    capi.write_tiff_stack(str(tmp_path / "s"), a)
    assert sorted(os.listdir(tmp_path / "s"))[:3] == ["01.tif", "02.tif", "03.tif"]
    assert np.array_equal(capi.read_tiff_stack(str(tmp_path / "s"), 1), a)
