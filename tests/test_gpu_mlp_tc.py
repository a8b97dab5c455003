"""Radiance-cache network inference on the fifth-generation tensor cores
(tcgen05.mma, accumulators in tensor memory) against the NumPy oracle with
the same half-precision rounding points, and against the mma.sync kernel of
the same network.  Tolerances as for the mma.sync forward: 2e-2 (BF16) and
2e-3 (FP16) of the output scale; the two kernels differ only in the order of
FP32 summation, which can move a half-precision rounding of an activation by
one step."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import mlp_ref

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def half_tensor(x, dtype):
    return torch.from_numpy(mlp_ref.to_bits(x, dtype).view(np.int16)).cuda()


@pytest.mark.parametrize("dtype,tol", [("bf16", 2e-2), ("fp16", 2e-3)])
def test_tcgen05_forward_matches_oracle_and_mma(dtype, tol):
    net = kgr.Mlp(dtype, seed=3)
    W = net.weights()
    rng = np.random.default_rng(0)
    for n in (5000, 3 * 128, 77):  # ragged, whole tiles, less than one tile
        x = mlp_ref.encode_inputs(rng, n, dtype)
        xd = half_tensor(x, dtype)
        outs = {}
        for kernel in ("mma", "tcgen05", "tcgen05"):  # the second tcgen05 call reuses freed TMEM
            net.set_inference(kernel)
            out = torch.full((n, 4), -7.0, dtype=torch.float32, device="cuda")
            net.forward(xd.data_ptr(), n, out.data_ptr())
            net.check()
            outs.setdefault(kernel, []).append(out.cpu().numpy())
        ref, _ = mlp_ref.forward(W, x, dtype)
        scale = np.abs(ref).max()
        for y in outs["tcgen05"]:
            assert np.all(y[:, 3] == 0)
            assert np.abs(y[:, :3] - ref).max() <= tol * scale + 1e-6, n
            assert np.abs(y[:, :3] - outs["mma"][0][:, :3]).max() <= tol * scale + 1e-6, n
        np.testing.assert_array_equal(outs["tcgen05"][0], outs["tcgen05"][1])


def test_tcgen05_inference_speed_beside_mma():
    """Both kernels over 2M rows of the radiance cache's query size (printed;
    the assertion only checks that both ran)."""
    net = kgr.Mlp("bf16", seed=1)
    n = 1920 * 1080
    x = torch.randint(-2000, 2000, (n, 64), dtype=torch.int16, device="cuda")  # finite BF16 bit patterns
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    times = {}
    for kernel in ("mma", "tcgen05"):
        net.set_inference(kernel)
        for _ in range(3):
            net.forward(x.data_ptr(), n, out.data_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            net.forward(x.data_ptr(), n, out.data_ptr())
        e1.record()
        e1.synchronize()
        net.check()
        times[kernel] = e0.elapsed_time(e1) / 10
    flops = 2.0 * (5 * 64 * 64 + 64 * 16) * n
    print({k: f"{v:.3f} ms, {flops / v / 1e9:.1f} TFLOP/s" for k, v in times.items()})
    assert all(v > 0 for v in times.values())


def test_tcgen05_wait_timeout_is_reported_and_the_network_recovers():
    """A launch whose tile loads are withheld: every block's wait on its first
    load runs out (65,536 polls), the error word is set and kgr_mlp_check
    raises; the blocks free their tensor memory, nothing is written, and the
    next ordinary inference is correct."""
    net = kgr.Mlp("bf16", seed=5)
    W = net.weights()
    rng = np.random.default_rng(1)
    n = 3000
    x = mlp_ref.encode_inputs(rng, n, "bf16")
    xd = half_tensor(x, "bf16")
    out = torch.full((n, 4), -7.0, dtype=torch.float32, device="cuda")
    net.set_inference("tcgen05")
    net.test_wait_timeout(xd.data_ptr(), n, out.data_ptr())
    with pytest.raises(kgr.KgrError, match="iteration limit"):
        net.check()
    assert torch.all(out == -7.0)
    net.check()  # the flag was cleared
    net.forward(xd.data_ptr(), n, out.data_ptr())
    net.check()
    ref, _ = mlp_ref.forward(W, x, "bf16")
    assert np.abs(out.cpu().numpy()[:, :3] - ref).max() <= 2e-2 * np.abs(ref).max() + 1e-6


def gradients(net, kernel, xd, td, n):
    net.set_training(kernel)
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), n)
    net.check()
    return loss, g


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
def test_tcgen05_gradients_match_oracle_and_mma(dtype):
    """Training on tcgen05 (forward and input deltas at M = 128, weight
    gradients at M = 64 accumulated in tensor memory) against the NumPy
    oracle -- within 5e-2 of each layer's gradient norm, the tolerance of the
    mma.sync kernel's test -- and against the mma.sync kernel within 1e-2
    (same rounding points, different FP32 summation order).  Row counts:
    ragged, whole 128-row tiles, less than one tile."""
    net = kgr.Mlp(dtype, seed=5)
    W = net.weights()
    rng = np.random.default_rng(1)
    for n in (4096 + 77, 2 * 128, 51):
        x = mlp_ref.encode_inputs(rng, n, dtype)
        t = np.zeros((n, 4), np.float32)
        t[:, :3] = rng.uniform(0, 2, (n, 3))
        xd, td = half_tensor(x, dtype), torch.from_numpy(t).cuda()
        loss_tc, g_tc = gradients(net, "tcgen05", xd, td, n)
        loss_mma, g_mma = gradients(net, "mma", xd, td, n)
        rl, rg = mlp_ref.loss_and_grad(W, x, t, dtype)
        assert abs(loss_tc - rl) <= 2e-2 * abs(rl)
        assert abs(loss_tc - loss_mma) <= 1e-3 * abs(loss_mma)
        for l in range(6):
            cols = 3 if l == 5 else 64
            a, b, c = g_tc[l][:, :cols], rg[l][:, :cols], g_mma[l][:, :cols]
            print(f"{dtype} n={n} layer {l}: |tc - oracle| / |oracle| = "
                  f"{np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30):.2e}, "
                  f"|tc - mma| / |mma| = {np.linalg.norm(a - c) / (np.linalg.norm(c) + 1e-30):.2e}")
            assert np.linalg.norm(a - b) <= 5e-2 * np.linalg.norm(b) + 1e-9, l
            assert np.linalg.norm(a - c) <= 1e-2 * np.linalg.norm(c) + 1e-9, l
        assert np.all(g_tc[5][:, 3:] == 0)


def test_tcgen05_training_lowers_loss_and_times_both_kernels():
    """300 Adam steps with the tcgen05 gradients lower the loss as the
    mma.sync ones do; the gradient pass of each kernel over 2^16 rows is
    timed (CUDA events, 20 passes after 3)."""
    n = 1 << 16
    rng = np.random.default_rng(2)
    x = mlp_ref.encode_inputs(rng, n, "bf16")
    t = np.zeros((n, 4), np.float32)
    t[:, 0] = 0.5 + 0.4 * np.sin(3 * x[:, 0])
    t[:, 1] = 0.5 + 0.4 * x[:, 1] * x[:, 2]
    t[:, 2] = np.abs(x[:, 3])
    xd, td = half_tensor(x, "bf16"), torch.from_numpy(t).cuda()
    net = kgr.Mlp("bf16", seed=7)
    net.set_training("tcgen05")
    first, _ = net.gradients(xd.data_ptr(), td.data_ptr(), n)
    for _ in range(300):
        net.train_step(xd.data_ptr(), td.data_ptr(), n, lr=1e-3)
    last, _ = net.gradients(xd.data_ptr(), td.data_ptr(), n)
    net.check()
    print(f"tcgen05 training: relative L2 loss {first / n:.4f} -> {last / n:.4f}")
    assert last < 0.2 * first
    times = {}
    for kernel in ("mma", "tcgen05"):
        net.set_training(kernel)
        for _ in range(3):
            net.train_step(xd.data_ptr(), td.data_ptr(), n, lr=0.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(20):
            net.train_step(xd.data_ptr(), td.data_ptr(), n, lr=0.0)
        e1.record()
        torch.cuda.synchronize()
        times[kernel] = e0.elapsed_time(e1) / 20
    net.check()
    print(f"gradient pass + Adam over 2^16 rows: mma.sync {times['mma'] * 1e3:.1f} us, "
          f"tcgen05 {times['tcgen05'] * 1e3:.1f} us")
