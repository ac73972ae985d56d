"""Learned-preconditioner network kernels vs the FP64 oracle (oracle/mlp.py).

Tolerances: FP32-weight forward and gradients within 1e-4 relative to each
tensor's largest entry (FP32 accumulation); BF16-weight forward within 1e-3
against the oracle evaluated with the same BF16-rounded weights."""
import numpy as np
import pytest
import torch

from nfempy_gb300 import _lib
from oracle import mlp as omlp

pytestmark = pytest.mark.gpu
DIMS = (96, 64, 48, 40)


def params_np(rng, dims):
    i, h1, h2, o = dims
    sc = lambda n: 1.0 / np.sqrt(n)
    return [(rng.normal(0, sc(i), (h1, i)), rng.normal(0, 0.1, h1)),
            (rng.normal(0, sc(h1), (h2, h1)), rng.normal(0, 0.1, h2)),
            (rng.normal(0, sc(h2), (o, h2)), rng.normal(0, 0.1, o))]


def flat(params):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in params])


def unflat(v, dims):
    i, h1, h2, o = dims
    out, k = [], 0
    for a, b in ((i, h1), (h1, h2), (h2, o)):
        W = v[k:k + a * b].reshape(b, a); k += a * b
        bb = v[k:k + b]; k += b
        out.append((W, bb))
    return out


def run_forward(dims, P, x, wt=_lib.NFEM_F32, Pf=None):
    B = x.shape[0]
    d = (ctypes_dims := torch.tensor(dims, dtype=torch.int32))
    h1 = torch.empty((B, dims[1]), device="cuda")
    h2 = torch.empty((B, dims[2]), device="cuda")
    y = torch.empty((B, dims[3]), device="cuda")
    _lib.call("nfem_mlp_forward", _lib.C.c_void_p(d.data_ptr()), wt, _lib.ptr(P), _lib.ptr(Pf), B, _lib.ptr(x),
              _lib.ptr(h1), _lib.ptr(h2), _lib.ptr(y), _lib.stream_ptr())
    torch.cuda.synchronize()
    return h1, h2, y


def test_param_count(cuda_lib):
    d = torch.tensor(DIMS, dtype=torch.int32)
    n = _lib.C.c_int64(0)
    _lib.call("nfem_mlp_param_count", _lib.C.c_void_p(d.data_ptr()), _lib.C.byref(n))
    assert n.value == flat(params_np(np.random.default_rng(0), DIMS)).size


@pytest.mark.parametrize("B", [1, 7, 130])
def test_forward_backward_match_oracle(cuda_lib, B):
    rng = np.random.default_rng(B)
    p = params_np(rng, DIMS)
    x = rng.normal(size=(B, DIMS[0]))
    t = rng.normal(size=(B, DIMS[3]))
    yo, _ = omlp.forward(p, x)
    lo, go = omlp.loss_and_grads(p, x, t)
    P = torch.tensor(flat(p), dtype=torch.float32, device="cuda")
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    h1, h2, y = run_forward(DIMS, P, xt)
    yg = y.double().cpu().numpy()
    assert np.abs(yg - yo).max() <= 1e-4 * np.abs(yo).max()
    d = torch.tensor(DIMS, dtype=torch.int32)
    wsb = _lib.C.c_size_t(0)
    _lib.call("nfem_mlp_backward_workspace_bytes", _lib.C.c_void_p(d.data_ptr()), B, _lib.C.byref(wsb))
    ws = torch.empty(int(wsb.value), dtype=torch.uint8, device="cuda")
    G = torch.zeros_like(P)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    _lib.call("nfem_mlp_backward", _lib.C.c_void_p(d.data_ptr()), _lib.NFEM_F32, _lib.ptr(P), B, _lib.ptr(xt),
              _lib.ptr(h1), _lib.ptr(h2), _lib.ptr(y), _lib.ptr(tt), _lib.ptr(G), _lib.ptr(ws), ws.numel(),
              _lib.ptr(loss), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert abs(loss.item() - lo) <= 1e-4 * abs(lo)
    gg = unflat(G.double().cpu().numpy(), DIMS)
    for (gW, gb), (oW, ob) in zip(gg, go):
        assert np.abs(gW - oW).max() <= 1e-4 * max(np.abs(oW).max(), 1e-30)
        assert np.abs(gb - ob).max() <= 1e-4 * max(np.abs(ob).max(), 1e-30)


def test_bf16_forward_and_adam(cuda_lib):
    rng = np.random.default_rng(3)
    p = params_np(rng, DIMS)
    P = torch.tensor(flat(p), dtype=torch.float32, device="cuda")
    Pb = torch.empty(P.numel(), dtype=torch.bfloat16, device="cuda")
    _lib.call("nfem_to_bf16", P.numel(), _lib.ptr(P), _lib.ptr(Pb), _lib.stream_ptr())
    x = rng.normal(size=(33, DIMS[0]))
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    _, _, y = run_forward(DIMS, Pb, xt, _lib.NFEM_BF16, P)
    pr = unflat(Pb.float().double().cpu().numpy(), DIMS)
    pr = [(W, b0) for (W, _), (_, b0) in zip(pr, p)]  # biases from the FP32 copy
    yo, _ = omlp.forward(pr, x)
    assert np.abs(y.double().cpu().numpy() - yo).max() <= 1e-3 * np.abs(yo).max()
    # Adam: three steps vs the oracle
    g = rng.normal(size=P.numel())
    m = torch.zeros_like(P); v = torch.zeros_like(P)
    Gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    po = [(W.copy(), b.copy()) for W, b in p]
    go = unflat(g, DIMS)
    state = [(np.zeros_like(W), np.zeros_like(W), np.zeros_like(b), np.zeros_like(b)) for W, b in p]
    for step in (1, 2, 3):
        _lib.call("nfem_adam_step", P.numel(), _lib.ptr(P), _lib.ptr(Gt), _lib.ptr(m), _lib.ptr(v),
                  _lib.C.c_float(1e-3), _lib.C.c_float(0.9), _lib.C.c_float(0.999), _lib.C.c_float(1e-8), step,
                  _lib.ptr(Pb), _lib.stream_ptr())
        po = omlp.adam(po, go, state, 1e-3, step)
    torch.cuda.synchronize()
    np.testing.assert_allclose(P.double().cpu().numpy(), flat(po), rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(Pb.float().cpu().numpy(), P.cpu().to(torch.bfloat16).float().numpy())


def torch_reference_tc(P32, Pb, dims, x):
    """Plain PyTorch FP32 restatement of nfem_mlp_infer_tc: BF16 weights,
    FP32 biases, the inputs and the layer-1 activations rounded to BF16 (the
    MMA operand type), FP32 accumulation."""
    i, h1, h2, o = dims
    W = Pb.float()
    k = 0
    W1 = W[k:k + h1 * i].view(h1, i); k += h1 * i
    b1 = P32[k:k + h1]; k += h1
    W2 = W[k:k + h2 * h1].view(h2, h1); k += h2 * h1
    b2 = P32[k:k + h2]; k += h2
    W3 = W[k:k + o * h2].view(o, h2); k += o * h2
    b3 = P32[k:k + o]
    xb = x.to(torch.bfloat16).float()
    a1 = torch.relu(xb @ W1.T + b1).to(torch.bfloat16).float()
    a2 = torch.relu(a1 @ W2.T + b2)
    return a2 @ W3.T + b3


@pytest.mark.parametrize("n_in", [8, 13])
@pytest.mark.parametrize("B", [1, 127, 128, 129, 5000, 152 * 128 * 3 + 77])
def test_tensor_core_inference_matches_torch(cuda_lib, n_in, B):
    """The tcgen05 kernel against a PyTorch FP32 reference of the same op.
    Tolerance: 2e-3 of max |y| entrywise (a BF16 rounding of one layer-1
    activation may fall on the other side when the FP32 sums differ in
    order), 1e-4 of max |y| on average."""
    dims = (n_in, 256, 256, 1)
    rng = np.random.default_rng(11 + n_in)
    p = params_np(rng, dims)
    P = torch.tensor(flat(p), dtype=torch.float32, device="cuda")
    Pb = torch.empty(P.numel(), dtype=torch.bfloat16, device="cuda")
    _lib.call("nfem_to_bf16", P.numel(), _lib.ptr(P), _lib.ptr(Pb), _lib.stream_ptr())
    x = torch.tensor(rng.normal(size=(B, n_in)), dtype=torch.float32, device="cuda")
    y = torch.full((B, 1), float("nan"), device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    d = torch.tensor(dims, dtype=torch.int32)
    _lib.call("nfem_mlp_infer_tc", _lib.C.c_void_p(d.data_ptr()), _lib.ptr(Pb), _lib.ptr(P), B, _lib.ptr(x),
              _lib.ptr(y), _lib.ptr(st), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = torch_reference_tc(P, Pb, dims, x)
    err = (y - ref).abs()
    scale = ref.abs().max().item()
    assert torch.isfinite(y).all()
    assert err.max().item() <= 2e-3 * scale, (err.max().item(), scale)
    assert err.mean().item() <= 1e-4 * scale


def test_tensor_core_inference_refuses_other_shapes(cuda_lib):
    P = torch.zeros(10, device="cuda")
    for dims in ((8, 128, 256, 1), (8, 256, 256, 2), (17, 256, 256, 1)):
        d = torch.tensor(dims, dtype=torch.int32)
        rc = _lib.lib().nfem_mlp_infer_tc(_lib.C.c_void_p(d.data_ptr()), _lib.ptr(P), _lib.ptr(P), 4, _lib.ptr(P),
                                          _lib.ptr(P), None, None)
        assert _lib.STATUS_NAMES[rc] == "NFEM_ERR_UNSUPPORTED"
