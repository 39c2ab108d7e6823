"""The learned shader's MLP on tcgen05 tensor cores against a CPU reference.

The reference rounds exactly where the kernel does (BF16 inputs, weights and
hidden activations; FP32 accumulation), so the only differences come from
the order of the FP32 sums; tolerance 2e-2 absolute on outputs of order 1.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(x):
    import torch
    return torch.as_tensor(x, dtype=torch.float32).to(torch.bfloat16).to(torch.float32)


def random_mlp(seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    w1 = torch.zeros(64, 32); w1[:, :24] = torch.randn(64, 24, generator=g) * (2 / 24) ** 0.5
    w2 = torch.randn(64, 64, generator=g) * (2 / 64) ** 0.5
    w3 = torch.randn(64, 64, generator=g) * (2 / 64) ** 0.5
    w4 = torch.zeros(16, 64); w4[:3] = torch.randn(3, 64, generator=g) * (1 / 64) ** 0.5
    b = [torch.randn(64, generator=g) * 0.1 for _ in range(3)]
    b4 = torch.zeros(16); b4[:3] = torch.randn(3, generator=g) * 0.1
    return dict(w1=w1, w2=w2, w3=w3, w4=w4, b1=b[0], b2=b[1], b3=b[2], b4=b4)


def reference(p, x):
    import torch
    h = bf16(x)
    for k in ("1", "2", "3"):
        h = torch.relu(h @ bf16(p["w" + k]).T + p["b" + k])
        h = bf16(h)
    return (h @ bf16(p["w4"]).T + p["b4"])[:, :3]


@pytest.mark.parametrize("n", [128, 1000, 70000])
def test_mlp_forward_matches_reference(built, n):
    import torch
    from rsr_gb300.gpu import GPU
    p = random_mlp(7)
    g = torch.Generator().manual_seed(n)
    x = torch.zeros(n, 32)
    x[:, :24] = torch.rand(n, 24, generator=g) * 2 - 1
    want = reference(p, x)
    dev = {k: (v.to(torch.bfloat16) if k.startswith("w") else v).cuda().contiguous() for k, v in p.items()}
    feat = x.to(torch.bfloat16).cuda().contiguous()
    out = torch.zeros(n, 3, device="cuda")
    gpu = GPU(0)
    try:
        gpu.mlp_forward(dev, feat, out)
    finally:
        gpu.close()
    got = out.cpu()
    err = (got - want).abs().max().item()
    assert err < 2e-2, "max abs error %g (reference scale %g)" % (err, want.abs().max().item())


def reference_grads(p, x, tgt):
    """FP32 CPU backward with the kernel's BF16 rounding points (the oracle for
    the training kernel's gradients)."""
    import torch
    B = x.shape[0]
    h = [bf16(x)]
    for k in ("1", "2", "3"):
        h.append(bf16(torch.relu(h[-1] @ bf16(p["w" + k]).T + p["b" + k])))
    y = (h[3] @ bf16(p["w4"]).T + p["b4"])[:, :3]
    e = y - tgt
    loss = (e * e).sum()
    dy = torch.zeros(B, 16)
    dy[:, :3] = bf16(2.0 * e / (3 * B))
    g = {"w4": dy.T @ h[3], "b4": dy.sum(0)}
    dz = dy
    for k, hk, hprev in (("3", h[3], h[2]), ("2", h[2], h[1]), ("1", h[1], h[0])):
        wnext = bf16(p[{"3": "w4", "2": "w3", "1": "w2"}[k]])
        da = dz @ wnext
        dz = bf16(da * (hk > 0))
        g["w" + k] = dz.T @ hprev
        g["b" + k] = dz.sum(0)
    return g, loss


def test_mlp_gradients_match_cpu_reference(built):
    import torch
    from rsr_gb300.gpu import GPU
    p = random_mlp(11)
    n, batch = 4000, 1000
    g = torch.Generator().manual_seed(5)
    x = torch.zeros(n, 32)
    x[:, :24] = torch.rand(n, 24, generator=g) * 2 - 1
    tgt = torch.rand(n, 3, generator=g)
    idx = torch.randperm(n, generator=g)[:batch].to(torch.int32)
    want, want_loss = reference_grads(p, x[idx.long()], tgt[idx.long()])
    dev = {k: (v.to(torch.bfloat16) if k.startswith("w") else v).cuda().contiguous() for k, v in p.items()}
    grad = torch.zeros(11472, device="cuda")
    loss = torch.zeros(1, device="cuda")
    gpu = GPU(0)
    try:
        gpu.mlp_grad(dev, x.to(torch.bfloat16).cuda(), tgt.cuda(), idx.cuda(), grad, loss)
    finally:
        gpu.close()
    gr = grad.cpu()
    off = {"w1": (0, (64, 32)), "w2": (2048, (64, 64)), "w3": (6144, (64, 64)), "w4": (10240, (16, 64)),
           "b1": (11264, (64,)), "b2": (11328, (64,)), "b3": (11392, (64,)), "b4": (11456, (16,))}
    for k, (o, shape) in off.items():
        got = gr[o:o + int(np.prod(shape))].reshape(shape)
        w = want[k]
        if k == "w1":
            got, w = got[:, :24], w[:, :24]
        scale = w.abs().max().item() + 1e-12
        err = (got - w).abs().max().item()
        assert err <= 0.03 * scale, "%s: max error %g vs scale %g" % (k, err, scale)
    assert abs(loss.item() - want_loss.item()) <= 1e-3 * want_loss.item()


def test_mlp_training_reduces_loss(built):
    """A few hundred Adam steps on a smooth target function fit it."""
    import torch
    from rsr_gb300.gpu import GPU
    g = torch.Generator().manual_seed(3)
    n = 32768
    x = torch.zeros(n, 32)
    x[:, :24] = torch.rand(n, 24, generator=g) * 2 - 1
    tgt = torch.stack([0.5 + 0.3 * torch.sin(2 * x[:, 0]) * x[:, 1], x[:, 2] * x[:, 3] * 0.5 + 0.5,
                       0.4 + 0.4 * torch.relu(x[:, 4] + x[:, 5]) - 0.2 * x[:, 6]], 1)
    p = random_mlp(1)
    params = torch.cat([p[k].reshape(-1) for k in ("w1", "w2", "w3", "w4", "b1", "b2", "b3", "b4")]).cuda()
    wbf = params[:11264].to(torch.bfloat16).contiguous()
    bias = params[11264:].clone()
    views = {"w1": wbf[0:2048], "w2": wbf[2048:6144], "w3": wbf[6144:10240], "w4": wbf[10240:11264],
             "b1": bias[0:64], "b2": bias[64:128], "b3": bias[128:192], "b4": bias[192:208]}
    m, v = torch.zeros_like(params), torch.zeros_like(params)
    grad = torch.zeros_like(params)
    loss = torch.zeros(1, device="cuda")
    feat, t = x.to(torch.bfloat16).cuda(), tgt.cuda()
    gpu = GPU(0)
    losses = []
    try:
        for step in range(1, 301):
            idx = torch.randint(0, n, (4096,), generator=g).to(torch.int32).cuda()
            gpu.mlp_grad(views, feat, t, idx, grad, loss)
            gpu.mlp_adam(params, grad, m, v, step, 3e-3, wbf, bias)
            losses.append(loss.item() / (3 * 4096))
    finally:
        gpu.close()
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    # better than predicting the mean: explained variance above one half
    assert losses[-1] < 0.5 * tgt.var(0).mean().item(), (losses[-1], tgt.var(0).mean().item())
