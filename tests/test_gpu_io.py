"""nfem_copy_bytes: SM-driven copies between device memory and pinned host
memory (aligned and unaligned), and its refusal of pageable host memory."""
import numpy as np
import pytest
import torch

from nfempy_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_copy_bytes_device_and_pinned_host(cuda_lib):
    n = (3 << 20) + 7
    d = torch.randint(0, 255, (n,), dtype=torch.uint8, device="cuda")
    h = torch.zeros(n, dtype=torch.uint8).pin_memory()
    _lib.call("nfem_copy_bytes", _lib.ptr(d), _lib.C.c_void_p(h.data_ptr()), n, _lib.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(h, d.cpu())
    # unaligned source and destination, host -> device
    d2 = torch.zeros(n, dtype=torch.uint8, device="cuda")
    _lib.call("nfem_copy_bytes", _lib.C.c_void_p(h.data_ptr() + 3), _lib.C.c_void_p(d2.data_ptr() + 1), n - 5,
              _lib.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(d2[1:n - 4].cpu(), h[3:n - 2])
    assert int(d2[0]) == 0


def test_copy_bytes_refuses_pageable_host(cuda_lib):
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    pageable = np.zeros(64, dtype=np.uint8)
    rc = _lib.lib().nfem_copy_bytes(_lib.ptr(d), _lib.C.c_void_p(pageable.ctypes.data), 64, _lib.stream_ptr())
    assert _lib.STATUS_NAMES[rc] == "NFEM_ERR_INVALID_ARG"
