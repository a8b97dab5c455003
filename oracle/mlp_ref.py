"""NumPy oracle of the radiance-cache network (TEST INFRASTRUCTURE).

Restates the forward pass, the relative-L2 loss and its gradient with the
same rounding points as the tensor-core kernels: half-precision inputs and
weights, FP32 accumulation, each hidden activation rounded to half after its
ReLU, output deltas and propagated deltas rounded to half before they feed
the next product.  Used to check kernel outputs and gradients; the reference
has no trained network to compare with (editor/mlp.cuh is an unused FP32
forward pass)."""
import numpy as np

LAYERS = 6


def round_bf16(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def round_half(a, dtype):
    if dtype == "fp32":
        return np.asarray(a, np.float64)
    if dtype == "bf16":
        return round_bf16(a)
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float32)


def to_bits(a, dtype):
    """Half-precision bit patterns (uint16) of a float32 array."""
    a = np.ascontiguousarray(a, np.float32)
    if dtype == "bf16":
        return (round_bf16(a).view(np.uint32) >> 16).astype(np.uint16)
    return a.astype(np.float16).view(np.uint16)


def weights_half(W, dtype):
    Wh = round_half(W, dtype)
    Wh[LAYERS - 1][:, 3:] = 0.0
    return Wh


def forward(W, x, dtype):
    """W: (6, 64, 64) [layer][in][out] FP32 masters; x: (n, 64) already
    half-representable.  Returns (output (n, 3), activations list)."""
    Wh = weights_half(W, dtype)
    ft = np.float64 if dtype == "fp32" else np.float32
    acts = [np.asarray(x, ft)]
    a = acts[0]
    for l in range(LAYERS - 1):
        z = a.astype(ft) @ Wh[l]
        a = round_half(np.maximum(z, 0.0), dtype)
        acts.append(a)
    y = (a @ Wh[LAYERS - 1][:, :16])[:, :3]
    return y.astype(ft), acts


def loss_and_grad(W, x, t, dtype):
    n = len(x)
    y, acts = forward(W, x, dtype)
    den = y * y + 0.01
    diff = y - t[:, :3]
    loss = float(np.sum(diff * diff / den))
    d = np.zeros((n, 16), np.float64 if dtype == "fp32" else np.float32)
    d[:, :3] = round_half(2.0 * diff / den / n, dtype)
    Wh = weights_half(W, dtype)
    grad = np.zeros_like(W)
    ncols = 16
    for l in range(LAYERS - 1, -1, -1):
        grad[l][:, :ncols] = acts[l].T.astype(np.float64) @ d[:, :ncols].astype(np.float64)
        if l == 0:
            break
        prop = d[:, :ncols] @ Wh[l][:, :ncols].T
        d = round_half(np.where(acts[l] > 0, prop, 0.0), dtype)
        ncols = 64
    return loss, grad


def encode_inputs(rng, n, dtype):
    x = rng.uniform(-1, 1, (n, 64)).astype(np.float32)
    return round_half(x, dtype)
