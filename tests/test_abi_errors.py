"""Host-side behaviour of the C ABI that needs no GPU: argument checks return PMA_ERR_ARGUMENT
with a message instead of touching the device, tables round-trip through pma_table_create,
and errors never escape as exceptions."""
import ctypes

import numpy as np

from porousmediaanalysis_gb300 import capi

ARG = 1


def _msg(lib):
    buf = ctypes.create_string_buffer(1024)
    lib.pma_last_error(buf, len(buf))
    return buf.value.decode()


def test_null_context_is_an_argument_error(pma_lib):
    d = capi.Dims(4, 4, 4)
    st = capi.EdtStats()
    assert pma_lib.pma_edt(None, None, d, None, ctypes.byref(st), None, 0) == ARG
    assert "null context" in _msg(pma_lib)
    assert pma_lib.pma_pores(None, None, None, None, d, 0, None, ctypes.byref(ctypes.c_void_p())) == ARG
    assert pma_lib.pma_watershed(None, None, None, d, 0, 0, None, ctypes.byref(ctypes.c_void_p())) == ARG
    assert pma_lib.pma_pipeline_host(None, None, d, None, None) == ARG
    assert pma_lib.pma_ctx_trim(None) == ARG
    assert pma_lib.pma_ctx_scratch_bytes(None) == 0


def test_batch_and_server_reject_bad_arguments(pma_lib):
    assert pma_lib.pma_pipeline_batch(None, None, 0, None, 0, 0) == ARG
    assert "null context" in _msg(pma_lib)
    h = ctypes.c_void_p()
    assert pma_lib.pma_server_create(None, None, ctypes.byref(h)) == ARG
    status = ctypes.c_int()
    assert pma_lib.pma_server_wait(None, 1, 0, ctypes.byref(status), None) == ARG
    assert pma_lib.pma_server_get_stats(None, None) == ARG
    assert pma_lib.pma_server_destroy(None) == 0  # destroying nothing is fine


def test_table_round_trip_and_pool_bounds(pma_lib):
    pores = (capi.Pore * 2)()
    pores[0].id, pores[0].volume = 127, 10
    pores[1].id, pores[1].volume = 128, 20
    throats = (capi.Throat * 1)()
    throats[0].id, throats[0].n_pores, throats[0].volume, throats[0].pool_offset = 0xFFFFFFFE, 2, 3, 0
    pool = np.array([127, 128], dtype=np.uint32)
    t = ctypes.c_void_p()
    assert pma_lib.pma_table_create(pores, 2, throats, 1, pool.ctypes.data, 2, ctypes.byref(t)) == 0
    try:
        assert pma_lib.pma_table_npores(t) == 2 and pma_lib.pma_table_nthroats(t) == 1
        assert pma_lib.pma_table_pool_size(t) == 2
        assert pma_lib.pma_table_pores(t)[1].volume == 20
        assert pma_lib.pma_table_throats(t)[0].id == 0xFFFFFFFE
        assert [pma_lib.pma_table_pool(t)[i] for i in range(2)] == [127, 128]
    finally:
        pma_lib.pma_table_free(t)
    throats[0].pool_offset = 1  # pore list would run past the pool
    t2 = ctypes.c_void_p()
    assert pma_lib.pma_table_create(pores, 2, throats, 1, pool.ctypes.data, 2, ctypes.byref(t2)) == ARG
    assert "outside the pool" in _msg(pma_lib)
    assert pma_lib.pma_table_npores(None) == 0 and not pma_lib.pma_table_pores(None)


def test_without_a_device_context_creation_fails_cleanly(pma_lib):
    import torch
    if torch.cuda.is_available():
        return  # this check is for machines without a GPU
    h = ctypes.c_void_p()
    status = pma_lib.pma_ctx_create(0, ctypes.byref(h))
    assert status != 0 and not h.value
    assert _msg(pma_lib)
