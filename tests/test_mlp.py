"""The learned proposal's network on the tensor cores (tcgen05): the matrix-product kernel against a
torch FP32 product of the same BF16 operands, the forward pass and the gradients against the FP64
oracle (oracle/mlp_oracle.py), and Adam training reducing the loss."""
import numpy as np
import pytest

import ntg

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


@pytest.mark.parametrize("m,n,k", [(128, 256, 48), (200, 16, 256), (256, 48, 1024), (1000, 256, 256), (64, 64, 16)])
def test_gemm_matches_torch(m, n, k):
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(m * 7 + n + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(n, k, generator=g).to(torch.bfloat16).cuda()
    c = ntg.gemm_bf16(a, b)
    ref = a.float() @ b.float().T
    torch.cuda.synchronize()
    err = (c - ref).abs().max().item()
    assert err <= 1e-3 * max(1.0, ref.abs().max().item()), err


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 48), dtype=np.float32)
    t = np.concatenate([rng.random((n, 5)), rng.random((n, 1)) * 4, np.zeros((n, 2))], axis=1).astype(np.float32)
    return x, t


def test_forward_matches_oracle():
    torch = _torch()
    import mlp_oracle
    net = ntg.MLP(seed=11)
    try:
        x, _ = _data(512, 1)
        y = net.infer_unfused(torch.from_numpy(x).cuda()).cpu().numpy()
        ref, _ = mlp_oracle.forward(net.get_params(), x)
        assert np.all(y[:, 8:] == 0)
        assert np.max(np.abs(y[:, :8] - ref)) < 2e-3 * max(1.0, np.abs(ref).max())
    finally:
        net.close()


@pytest.mark.parametrize("rows", [1, 127, 128, 5000, 40000])
def test_fused_inference_matches_unfused(rows):
    """The persistent fused kernel (weights in shared memory, layers chained through TMEM) against
    the three-product path the training uses."""
    torch = _torch()
    net = ntg.MLP(seed=rows)
    try:
        x, _ = _data(rows, rows + 1)
        dx = torch.from_numpy(x).cuda()
        a = net.infer(dx).cpu().numpy()
        b = net.infer_unfused(dx).cpu().numpy()
        assert np.max(np.abs(a - b)) < 1e-3 * max(1.0, np.abs(b).max())
    finally:
        net.close()


@pytest.mark.parametrize("batch", [256, 1024])
def test_gradients_match_oracle(batch):
    torch = _torch()
    import mlp_oracle
    net = ntg.MLP(seed=5 + batch)
    try:
        x, t = _data(batch, batch)
        g, loss = net.gradients(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
        g = g.cpu().numpy().astype(np.float64)
        ref, ref_loss = mlp_oracle.gradients(net.get_params(), x, t)
        assert abs(loss - ref_loss) <= 1e-3 * ref_loss
        # per parameter block: relative L2 error of the gradient
        offs = np.cumsum([0, 256 * 48, 256, 256 * 256, 256, 8 * 256, 8])
        for a, b in zip(offs[:-1], offs[1:]):
            num = np.linalg.norm(g[a:b] - ref[a:b])
            den = max(np.linalg.norm(ref[a:b]), 1e-12)
            assert num / den < 2e-2, (a, b, num / den)
    finally:
        net.close()


def test_training_reduces_loss():
    torch = _torch()
    net = ntg.MLP(seed=3)
    try:
        x, t = _data(8192, 77)
        # a learnable target: per-block channel minima and maxima, and a log spread
        xt = x.reshape(-1, 16, 3)
        t[:, 0:3] = xt.min(axis=1)
        t[:, 3:5] = xt.max(axis=1)[:, :2]
        t[:, 5] = np.log1p(((xt - xt.mean(axis=1, keepdims=True)) ** 2).sum(axis=(1, 2)) * 255.0)
        dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        _, loss0 = net.gradients(dx, dt)
        lossbuf = torch.zeros(1, dtype=torch.float32, device="cuda")
        for _ in range(300):
            net.train_step(dx, dt, lr=1e-3, loss_out=lossbuf)
        net.status()
        _, loss1 = net.gradients(dx, dt)
        assert loss1 < 0.2 * loss0, (loss0, loss1)
    finally:
        net.close()


def test_bounded_waits_run_out_without_a_fault():
    """A wait limit of zero polls makes every tensor-core wait give up at once: the kernels record the
    timeout (the status reports it, the gradient call returns the error), drain their issued MMAs, free
    TMEM and return. With the default limit back, the same network gives the results it gave before."""
    torch = _torch()
    net = ntg.MLP(seed=21)
    try:
        x, t = _data(1000, 9)
        dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        before = net.infer(dx).cpu().numpy()
        grads_before, _ = net.gradients(dx, dt)
        net.set_wait_limit(0)
        net.infer(dx)          # the fused kernel's first wait gives up
        with pytest.raises(ntg.NtgError) as e:
            net.status()
        assert e.value.code == ntg.NTG_ERROR_CUDA and "timed out" in str(e.value)
        with pytest.raises(ntg.NtgError):
            net.gradients(dx, dt)  # the product kernels' waits give up too
        net.set_wait_limit(-1)     # default limit, status cleared
        net.status()
        after = net.infer(dx).cpu().numpy()
        grads_after, _ = net.gradients(dx, dt)
        net.status()
        assert np.array_equal(before, after)
        assert torch.equal(torch.isfinite(grads_after), torch.isfinite(grads_before))
        assert torch.allclose(grads_after, grads_before, rtol=1e-4, atol=1e-6)
    finally:
        net.close()
