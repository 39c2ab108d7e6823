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
