"""CPU oracle of the learned proposal's network -- TEST INFRASTRUCTURE ONLY.

A numpy FP64 restatement of csrc/fs_mlp_train.cu's forward pass, loss and backward pass
that rounds to BF16 at the same points the kernels do (inputs, weights, post-ReLU
activations, output and hidden gradients), so the GPU gradients can be checked element
by element.  Used by tests/ only.
"""
import numpy as np


def bf16(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def split(params):
    p = np.asarray(params, dtype=np.float64)
    shapes = [(128, 16), (128,), (128, 128), (128,), (128, 128), (128,), (16, 128), (16,)]
    out, o = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(p[o:o + n].reshape(s))
        o += n
    return out


def forward(params, x):
    W1, b1, W2, b2, W3, b3, W4, b4 = split(params)
    q = [bf16(W.astype(np.float32)) for W in (W1, W2, W3, W4)]
    xb = bf16(np.asarray(x, np.float32))
    a1 = bf16(np.maximum(xb @ q[0].T + b1, 0).astype(np.float32))
    a2 = bf16(np.maximum(a1 @ q[1].T + b2, 0).astype(np.float32))
    a3 = bf16(np.maximum(a2 @ q[2].T + b3, 0).astype(np.float32))
    z4 = a3 @ q[3].T + b4
    return xb, q, (a1, a2, a3), z4


def loss_and_grad(params, x, z, dof, inv_batch):
    """Returns (loss sum, flat gradient in the parameter layout)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = split(params)
    xb, q, (a1, a2, a3), z4 = forward(params, x)
    o = z4[:, :dof]
    sr = z4[:, dof:2 * dof]
    th = np.tanh(0.25 * sr)
    s = 4 * th
    e = np.exp(-s)
    df = z[:, :dof] - o
    loss = float(np.sum(0.5 * df * df * e + 0.5 * s))
    g = np.zeros_like(z4)
    g[:, :dof] = -df * e * inv_batch
    g[:, dof:2 * dof] = (0.5 - 0.5 * df * df * e) * (1 - th * th) * inv_batch
    db4 = g.sum(0)
    dz4 = bf16(g.astype(np.float32))
    dW4 = dz4.T @ a3
    dz3f = (dz4 @ q[3]) * (a3 > 0)
    db3 = dz3f.sum(0)
    dz3 = bf16(dz3f.astype(np.float32))
    dW3 = dz3.T @ a2
    dz2f = (dz3 @ q[2]) * (a2 > 0)
    db2 = dz2f.sum(0)
    dz2 = bf16(dz2f.astype(np.float32))
    dW2 = dz2.T @ a1
    dz1f = (dz2 @ q[1]) * (a1 > 0)
    db1 = dz1f.sum(0)
    dz1 = bf16(dz1f.astype(np.float32))
    dW1 = dz1.T @ xb
    grad = np.concatenate([t.ravel() for t in (dW1, db1, dW2, db2, dW3, db3, dW4, db4)])
    return loss, grad
