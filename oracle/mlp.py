"""FP64 reference of the learned-preconditioner network (oracle).

No reference counterpart exists (nfempy has no learned component); this is
the CPU restatement the GPU forward/backward/Adam kernels are checked
against.  Network: x -> relu(W1 x + b1) -> relu(W2 h1 + b2) -> W3 h2 + b3,
weights W_l [out, in] row-major, batch-major activations [B, features].
Loss: 0.5 * mean over the batch of ||y - t||^2.
"""
import numpy as np


def forward(params, x):
    (W1, b1), (W2, b2), (W3, b3) = params
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ W3.T + b3
    return y, (x, z1, h1, z2, h2)


def loss_and_grads(params, x, t):
    (W1, b1), (W2, b2), (W3, b3) = params
    y, (x, z1, h1, z2, h2) = forward(params, x)
    B = x.shape[0]
    d = (y - t) / B
    loss = 0.5 * np.sum((y - t) ** 2) / B
    gW3 = d.T @ h2
    gb3 = d.sum(0)
    dh2 = d @ W3
    dz2 = dh2 * (z2 > 0)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dh1 = dz2 @ W2
    dz1 = dh1 * (z1 > 0)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    return loss, [(gW1, gb1), (gW2, gb2), (gW3, gb3)]


def adam(params, grads, state, lr, t, b1=0.9, b2=0.999, eps=1e-8):
    out = []
    for (W, b), (gW, gb), (mW, vW, mb, vb) in zip(params, grads, state):
        for P, G, M, V in ((W, gW, mW, vW), (b, gb, mb, vb)):
            M[...] = b1 * M + (1 - b1) * G
            V[...] = b2 * V + (1 - b2) * G * G
            mh = M / (1 - b1 ** t)
            vh = V / (1 - b2 ** t)
            P[...] = P - lr * mh / (np.sqrt(vh) + eps)
        out.append((W, b))
    return out
