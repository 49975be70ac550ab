"""CPU reference of the ordering model's training step (the BF16 MLP of the
batched passes' learned ordering): forward and backward in FP32 with the
operands rounded to BF16 exactly where the tensor-core kernel rounds them."""
import numpy as np

SP = 64 * 24 + 64 + 64 * 64 + 64 + 64 + 1


def bf16(a):
    """Round to the nearest BF16 value, ties to even (finite inputs)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(P):
    o = 0
    W1 = P[o:o + 1536].reshape(64, 24); o += 1536
    b1 = P[o:o + 64]; o += 64
    W2 = P[o:o + 4096].reshape(64, 64); o += 4096
    b2 = P[o:o + 64]; o += 64
    w3 = P[o:o + 64]; o += 64
    b3 = P[o]
    return W1, b1, W2, b2, w3, b3


def ref_gradient(P, X, T, batch=128):
    """Gradients of mean((y - t)^2) / 2 over the first `batch` samples."""
    W1, b1, W2, b2, w3, b3 = unpack(P.astype(np.float32))
    x = bf16(X[:batch])
    t = T[:batch].astype(np.float32)
    W1b, W2b = bf16(W1), bf16(W2)
    h1 = bf16(np.maximum(x @ W1b.T + b1, 0.0))
    h2 = bf16(np.maximum(h1 @ W2b.T + b2, 0.0))
    y = h2 @ w3 + b3
    dy = (y - t) / batch
    dw3 = h2.T @ dy
    db3 = dy.sum()
    dz2 = bf16(dy[:, None] * w3[None, :] * (h2 > 0))
    db2 = dz2.sum(0)
    dW2 = dz2.T @ h1
    dz1 = bf16((dz2 @ W2b) * (h1 > 0))
    db1 = dz1.sum(0)
    dW1 = dz1.T @ x
    return np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]]).astype(np.float32)
