"""NumPy restatement of the warm-start MLP (forward, loss, backpropagation).

TEST INFRASTRUCTURE ONLY: the checker of the BF16 tensor-core kernels of
nlm_mlp_*.  With bf16=True every GEMM operand is rounded to bfloat16
(round to nearest even) the way the CUDA kernels round them, products are
accumulated in float64 (the kernels accumulate in float32, so the two agree
to about 1e-6 relative before the next bf16 rounding); with bf16=False the
same network runs in float64, which the finite-difference check uses.

Parameter layout (as nlm_mlp_get_params): per layer W[d_in][d_out]
row-major then b[d_out], padded widths (inputs to 16, hidden to 16, outputs
to 8).
"""
import numpy as np


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def layout(n_in, n_hidden, n_layers, n_out):
    r16 = lambda v: (v + 15) // 16 * 16
    dims = [r16(n_in)] + [r16(n_hidden)] * n_layers + [(n_out + 7) // 8 * 8]
    out, off = [], 0
    for l in range(n_layers + 1):
        di, do = dims[l], dims[l + 1]
        out.append((di, do, off, off + di * do))
        off += di * do + do
    return out, off


def unpack(p, lay):
    Ws, bs = [], []
    for di, do, wo, bo in lay:
        Ws.append(np.asarray(p[wo:wo + di * do], dtype=np.float64).reshape(di, do))
        bs.append(np.asarray(p[bo:bo + do], dtype=np.float64))
    return Ws, bs


def _r(a, on):
    """bf16-rounded copy (on) or the float64 values unchanged."""
    if on:
        return bf16(np.asarray(a, dtype=np.float32)).astype(np.float64)
    return np.asarray(a, dtype=np.float64)


def forward(p, lay, x, n_out, bf16_ops=True):
    """Returns (y, cache); y: rows x n_out."""
    Ws, bs = unpack(p, lay)
    rows = x.shape[0]
    A = np.zeros((rows, lay[0][0]))
    A[:, :x.shape[1]] = x
    A = _r(A, bf16_ops)
    Zs, As = [], [A]
    L = len(Ws)
    for l in range(L):
        W = _r(Ws[l], bf16_ops)
        Z = A @ W + bs[l]
        if bf16_ops:
            Z = Z.astype(np.float32).astype(np.float64)
        Zs.append(Z)
        if l < L - 1:
            A = np.maximum(Z, 0.)
            A = _r(A, bf16_ops)
            As.append(A)
    return Zs[-1][:, :n_out], (Ws, Zs, As)


def loss_grad(p, lay, x, t, n_out, bf16_ops=True):
    """Mean over rows of the summed squared error, and its gradient."""
    y, (Ws, Zs, As) = forward(p, lay, x, n_out, bf16_ops)
    rows = x.shape[0]
    d = y - np.asarray(t, dtype=np.float64)
    loss = float(np.sum(d * d) / rows)
    dZ = np.zeros_like(Zs[-1])
    dZ[:, :n_out] = 2. * d / rows
    if bf16_ops:
        dZ = _r(dZ, True)
    g = np.zeros(lay[-1][3] + lay[-1][1], dtype=np.float64)
    for l in range(len(Ws) - 1, -1, -1):
        di, do, wo, bo = lay[l]
        g[wo:wo + di * do] = (As[l].T @ dZ).ravel()
        g[bo:bo + do] = dZ.sum(axis=0)
        if l == 0:
            break
        W = _r(Ws[l], bf16_ops)
        dA = dZ @ W.T
        dZ = dA * (Zs[l - 1] > 0)
        if bf16_ops:
            dZ = _r(dZ, True)
    return loss, g
