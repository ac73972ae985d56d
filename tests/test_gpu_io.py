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


@pytest.mark.parametrize("n_points", [1, 2, 3, 7, 1000])
def test_points_split_records(cuda_lib, n_points):
    """Packed fixed-point point records: the header holds a power-of-two
    scale and the bounding-box centre, every coordinate is recovered to
    within the scale, and edge differences come out exact in integers.  The
    sizes cover the single-block fold (fewer than 3 points) and the partial
    boxes of larger sets."""
    rng = np.random.default_rng(n_points)
    pts = rng.uniform(-3.0, 5.0, size=(n_points, 3))
    p = torch.as_tensor(pts, device="cuda")
    out = torch.empty((n_points + 1, 4), dtype=torch.float32, device="cuda")
    _lib.call("nfem_points_split", _lib.ptr(p), n_points, _lib.ptr(out), _lib.stream_ptr())
    torch.cuda.synchronize()
    o = out.cpu()
    scale = float(o[0, 0])
    c = o[0, 1:].double().numpy()
    assert np.log2(scale) == np.round(np.log2(scale))
    np.testing.assert_allclose(c, 0.5 * (pts.min(0) + pts.max(0)), rtol=1e-6, atol=1e-6)
    q = o[1:, :3].contiguous().view(torch.int32).numpy().astype(np.int64)
    assert np.abs(q).max() < 2 ** 30
    rec = q * scale + c[None, :]
    assert np.abs(rec - pts).max() <= 0.5 * scale * (1 + 1e-9)


@pytest.mark.parametrize("n_points", [1, 5, 1000])
def test_points_fixed64_records(cuda_lib, n_points):
    """64-bit fixed-point records of the FP64 kernels: x = q 2^-shift with
    |q| < 2^62; coordinates of a uniform grid and every FP64 coordinate of
    at least 2^-10 max |x| are held exactly, the rest to within 2^-62 max |x|."""
    from fractions import Fraction
    rng = np.random.default_rng(n_points)
    pts = rng.uniform(-3.0, 5.0, size=(n_points, 3))
    pts[0] = [0.0, 1.0 / 64, 1e-9]  # a grid coordinate and a tiny one
    p = torch.as_tensor(pts, device="cuda")
    out = torch.empty((n_points + 1, 4), dtype=torch.int64, device="cuda")
    _lib.call("nfem_points_fixed64", _lib.ptr(p), n_points, _lib.ptr(out), _lib.stream_ptr())
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    shift = int(o[0, 0])
    q = o[1:, :3]
    assert np.abs(q).max() < 2 ** 62 and np.abs(q).max() >= 2 ** 61
    amax = np.abs(pts).max()
    for v in range(n_points):
        for d in range(3):
            err = abs(Fraction(int(q[v, d]), 2 ** shift) - Fraction(pts[v, d]))
            if abs(pts[v, d]) >= amax / 1024:
                assert err == 0, (v, d)
            else:
                assert err <= Fraction(amax) / 2 ** 62
