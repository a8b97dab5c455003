"""Radiance-cache network on the tensor cores against the NumPy oracle with
the same half-precision rounding points (oracle/mlp_ref.py): forward outputs,
gradients of the relative L2 loss, and that training lowers the loss.
Tolerances: forward 2e-2 relative (BF16) / 2e-3 (FP16) of the output scale;
gradients within 5e-2 of each layer's gradient norm (accumulation order
differs: FP32 atomics versus float64)."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import mlp_ref

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def half_tensor(x, dtype):
    bits = mlp_ref.to_bits(x, dtype)
    return torch.from_numpy(bits.view(np.int16)).cuda()


@pytest.mark.parametrize("dtype,tol", [("bf16", 2e-2), ("fp16", 2e-3)])
def test_forward_matches_oracle(dtype, tol):
    net = kgr.Mlp(dtype, seed=3)
    net.set_inference("mma")
    W = net.weights()
    rng = np.random.default_rng(0)
    n = 5000  # not a multiple of the 128-row tile
    x = mlp_ref.encode_inputs(rng, n, dtype)
    xd = half_tensor(x, dtype)
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    net.forward(xd.data_ptr(), n, out.data_ptr())
    torch.cuda.synchronize()
    y = out.cpu().numpy()[:, :3]
    ref, _ = mlp_ref.forward(W, x, dtype)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() <= tol * scale + 1e-6
    assert np.all(out.cpu().numpy()[:, 3] == 0)


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
def test_gradients_match_oracle(dtype):
    net = kgr.Mlp(dtype, seed=5)
    net.set_training("mma")  # the tcgen05 kernel is tested in test_gpu_mlp_tc.py
    W = net.weights()
    rng = np.random.default_rng(1)
    n = 4096 + 77
    x = mlp_ref.encode_inputs(rng, n, dtype)
    t = np.zeros((n, 4), np.float32)
    t[:, :3] = rng.uniform(0, 2, (n, 3))
    # keep the device tensors alive for the call (a temporary's memory can be
    # handed to the next temporary by the caching allocator)
    xd, td = half_tensor(x, dtype), torch.from_numpy(t).cuda()
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), n)
    rl, rg = mlp_ref.loss_and_grad(W, x, t, dtype)
    assert abs(loss - rl) <= 2e-2 * abs(rl)
    for l in range(6):
        cols = 3 if l == 5 else 64
        a, b = g[l][:, :cols], rg[l][:, :cols]
        assert np.linalg.norm(a - b) <= 5e-2 * np.linalg.norm(b) + 1e-9, l
    assert np.all(g[5][:, 3:] == 0)


def test_training_lowers_loss():
    net = kgr.Mlp("bf16", seed=7)
    net.set_training("mma")
    rng = np.random.default_rng(2)
    n = 1 << 14
    x = mlp_ref.encode_inputs(rng, n, "bf16")
    t = np.zeros((n, 4), np.float32)
    t[:, 0] = 0.5 + 0.4 * np.sin(3 * x[:, 0])
    t[:, 1] = 0.5 + 0.4 * x[:, 1] * x[:, 2]
    t[:, 2] = np.abs(x[:, 3])
    xd, td = half_tensor(x, "bf16"), torch.from_numpy(t).cuda()
    first, _ = net.gradients(xd.data_ptr(), td.data_ptr(), n)
    for _ in range(300):
        net.train_step(xd.data_ptr(), td.data_ptr(), n, lr=1e-3)
    last, _ = net.gradients(xd.data_ptr(), td.data_ptr(), n)
    print(f"relative L2 loss {first / n:.4f} -> {last / n:.4f}")
    assert last < 0.2 * first
