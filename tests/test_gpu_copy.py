"""ss_copy_rows_async: the strided row copy that moves a particle sub-range
of the snapshots [n_snap, N, 6] to pinned host memory, by the copy engine
(kind 0) and by SM stores into device-addressable pinned memory (kind 3).
Both must give the same bytes for every alignment class (16-, 4- and 1-byte
units), and kind 3 must refuse a destination that is not pinned."""
import ctypes as C

import pytest
import torch

from streamsculptor_gb300 import _abi

pytestmark = pytest.mark.gpu


def _copy(kind, dst, src, rows, pitch, off, width):
    lib = _abi.load()
    return lib.ss_copy_rows_async(C.c_void_p(dst), C.c_void_p(src), rows, pitch, off, width, kind,
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("rows,pitch,off,width", [(160, 24 * 1000, 24 * 128, 24 * 500),  # 16-byte units
                                                  (7, 1000, 12, 500),                   # 4-byte units
                                                  (5, 1001, 3, 777),                    # bytes
                                                  (1, 1 << 20, 0, 1 << 20)])            # one contiguous row
def test_sm_store_copy_equals_copy_engine(ss, rows, pitch, off, width):
    src = torch.randint(0, 255, (rows * pitch,), dtype=torch.uint8, device="cuda")
    ce = torch.zeros(rows * pitch, dtype=torch.uint8, pin_memory=True)
    sm = torch.zeros(rows * pitch, dtype=torch.uint8, pin_memory=True)
    assert _copy(0, ce.data_ptr(), src.data_ptr(), rows, pitch, off, width) == 0
    assert _copy(3, sm.data_ptr(), src.data_ptr(), rows, pitch, off, width) == 0
    torch.cuda.synchronize()
    assert torch.equal(ce, sm)
    want = torch.zeros(rows, pitch, dtype=torch.uint8)
    want[:, off:off + width] = src.view(rows, pitch)[:, off:off + width].cpu()
    assert torch.equal(sm.view(rows, pitch), want)


def test_sm_store_copy_refuses_pageable_destination(ss):
    src = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    pageable = torch.zeros(4096, dtype=torch.uint8)
    assert not pageable.is_pinned()
    rc = _copy(3, pageable.data_ptr(), src.data_ptr(), 1, 4096, 0, 4096)
    assert rc == _abi.SS_ERR_INVALID_ARGUMENT
    assert b"pinned" in _abi.load().ss_last_error()
