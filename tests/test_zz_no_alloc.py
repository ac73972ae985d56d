"""The allocation-free scan entry point (nfem_exclusive_scan_noalloc).

Some callers cannot allocate device memory: code running while a CUDA graph
is captured (cudaMalloc cannot be captured) and frameworks that hand out all
device memory from their own pool.  This entry point keeps its scratch in a
fixed array inside the library instead of a caller workspace.  The test
calls it through the C ABI twice in a row, with different sizes and
contents, and compares each result with the workspace-based
nfem_exclusive_scan bit for bit (integer offsets).  It is collected last
(file name) and passes in a fresh process as well as after the other tests.
"""
import pytest
import torch

from nfempy_gb300 import _lib

pytestmark = pytest.mark.gpu


def scan_with_workspace(x):
    n = x.numel()
    out = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    b = _lib.C.c_size_t(0)
    _lib.call("nfem_scan_workspace_bytes", n, _lib.C.byref(b))
    ws = torch.empty(int(b.value), dtype=torch.uint8, device="cuda")
    _lib.call("nfem_exclusive_scan", _lib.ptr(x), n, _lib.ptr(out), _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    return out


def scan_noalloc(x):
    n = x.numel()
    out = torch.full((n + 1,), -7, dtype=torch.int64, device="cuda")
    _lib.call("nfem_exclusive_scan_noalloc", _lib.ptr(x), n, _lib.ptr(out), _lib.stream_ptr())
    return out


def test_noalloc_scan_matches_workspace_scan_twice(cuda_lib):
    g = torch.Generator(device="cpu").manual_seed(11)
    # first call: a large input (many tiles of scratch in use)
    a = torch.randint(0, 1000, (3_000_017,), generator=g, dtype=torch.int32).cuda()
    ra = scan_noalloc(a)
    torch.cuda.synchronize()
    assert torch.equal(ra, scan_with_workspace(a))
    # second call reuses the scratch the first one left: smaller, different data
    b = torch.randint(0, 7, (40_961,), generator=g, dtype=torch.int32).cuda()
    rb = scan_noalloc(b)
    torch.cuda.synchronize()
    assert torch.equal(rb, scan_with_workspace(b))
    ref = torch.zeros(b.numel() + 1, dtype=torch.int64)
    ref[1:] = torch.cumsum(b.cpu().long(), 0)
    assert torch.equal(rb.cpu(), ref)


def test_noalloc_scan_rejects_sizes_beyond_its_scratch(cuda_lib):
    x = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = _lib.lib().nfem_exclusive_scan_noalloc(_lib.ptr(x), 67_108_864 + 1, _lib.ptr(out), _lib.stream_ptr())
    assert rc == 5  # NFEM_ERR_CAPACITY, nothing launched
