"""Post-processing on the device (include/rsrgpu.h rsrgpu_kawase_blur,
rsrgpu_kawase_chain, rsrgpu_glow) against rsr's KawaseBlurFilter
(src/rgl/rglr/rglr_kawase.cxx:22-84), the $kawase node's chain
(src/viewer/node/kawase.cxx:79-117) and the $glow node's
Filter<GlowShader> (src/rgl/rglr/rglr_algorithm.hxx:107-144,
src/viewer/node/glow.cxx:24-36).

Bar: the blur bit-exact; the glow bit-exact with the linear packing and
within 1/255 with sRGB (the library's sRGB8 encoder differs from rsr's table
encoder, as in every TrueColor store).  The oracle is pinned to rsr by golden
digests of rsr's own output (tests/golden/postfx.json).  The whole chain --
a frame stored as full-size quads and a half-size float canvas, blurred,
then glowed -- is compared end to end.
"""
import json
import os
import sys

import numpy as np
import pytest

from rsr_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

with open(os.path.join(HERE, "golden", "postfx.json")) as _f:
    GOLDEN = json.load(_f)


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def test_golden_covers_every_case():
    assert set(GOLDEN) == set(make_golden.POSTFX_CASES)


@pytest.mark.parametrize("name", sorted(make_golden.POSTFX_CASES))
def test_oracle_matches_reference_golden(name, orc):
    out = make_golden.run_postfx(orc, name)
    assert make_golden.digest(np.ascontiguousarray(out).view(np.uint32).tobytes()) == GOLDEN[name]


def test_kawase_properties(orc):
    """A constant canvas stays constant (16 equal terms / 16); the blur is
    linear in exact arithmetic, so scaling by a power of two commutes."""
    c = np.full((20, 30, 4), 0.375, np.float32)
    assert (orc.kawase(c, 2) == np.float32(0.375)).all()
    x = make_golden.postfx_inputs("kawase", 30, 20, 9)[0]
    assert np.array_equal(orc.kawase(x * np.float32(4.0), 1), orc.kawase(x, 1) * np.float32(4.0))


def _chain(orc, src, intensity):
    out = src
    for d in range(intensity):
        out = orc.kawase(out, d)
    return out


def _channels(c):
    c = c.view(np.uint32)
    return np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1).astype(np.int32)


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(2, 2, 0), (61, 37, 1), (160, 90, 3), (96, 54, 30), (960, 540, 2)],
                         ids=lambda c: "%dx%d_d%d" % c)
def test_gpu_kawase_matches_oracle(case, gpu, orc):
    import torch
    w, h, d = case
    src = make_golden.postfx_inputs("kawase", w, h, w + d)[0]
    want = orc.kawase(src, d)
    s = torch.from_numpy(src.reshape(-1)).cuda()
    o = torch.full((w * h * 4,), float("nan"), dtype=torch.float32, device="cuda")
    gpu.kawase_blur(s, o, w, h, d)
    torch.cuda.synchronize()
    assert np.array_equal(o.cpu().numpy().view(np.uint32), want.reshape(-1).view(np.uint32))


@pytest.mark.gpu
def test_gpu_kawase_chain_matches_oracle(gpu, orc):
    import torch
    w, h = 240, 136
    src = make_golden.postfx_inputs("kawase", w, h, 17)[0]
    s = torch.from_numpy(src.reshape(-1)).cuda()
    for intensity in range(0, 6):
        a = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
        b = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
        res = gpu.kawase_chain(s, a, b, w, h, intensity)
        torch.cuda.synchronize()
        want = _chain(orc, src, intensity)
        assert res is (s if intensity == 0 else (a if intensity % 2 else b))
        assert np.array_equal(res.cpu().numpy().view(np.uint32), want.reshape(-1).view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("srgb", [0, 1])
def test_gpu_glow_matches_oracle(srgb, gpu, orc):
    import torch
    w, h = 320, 180
    q, bl = make_golden.postfx_inputs("glow", w, h, 6)
    want = orc.glow(q, bl, w, h, srgb)
    out = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    gpu.glow(torch.from_numpy(q.reshape(-1)).cuda(), torch.from_numpy(bl.reshape(-1)).cuda(), out, w, h, srgb=bool(srgb))
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    if srgb:
        assert np.abs(_channels(got) - _channels(want)).max() <= 1
    else:
        assert np.array_equal(got, want)


@pytest.mark.gpu
def test_gpu_canvas_checks(gpu):
    import torch
    from rsr_gb300.gpu import RsrGpuError
    t = torch.zeros(64 * 64 * 4, dtype=torch.float32, device="cuda")
    with pytest.raises(RsrGpuError):
        gpu.kawase_blur(t, t, 64, 64, 1)                    # source and destination overlap
    with pytest.raises(RsrGpuError):
        gpu.kawase_blur(t, t[64 * 4 * 8:], 64, 32, 1)       # overlap at an offset
    u = torch.zeros(64 * 64 * 4, dtype=torch.float32, device="cuda")
    with pytest.raises(RsrGpuError):
        gpu.kawase_blur(t, u, 64, 64, -1)                   # negative distance


@pytest.mark.gpu
def test_gpu_glow_frame_end_to_end(gpu, orc):
    """The glow chain of rsr's viewer: a frame stored with StoreColor(QFloat4Canvas*)
    and StoreColor(FloatingPointCanvas*, downsample), the half-size canvas
    blurred by three Kawase passes, then Filter<GlowShader, sRGB>."""
    import torch
    sc = scenes.textured_sphere(seed=4, divs=5, width=640, height=360, tile_blocks=(4, 4), tex_dim=256)
    w, h = sc.width, sc.height
    # oracle
    quads = np.zeros((h // 2) * (w // 2) * 16, np.float32)
    half = np.zeros((h // 2) * (w // 2) * 4, np.float32)
    gl = sc.record(gamma=False)
    gl.StoreColorQuads(quads, w, h)
    gl.StoreColorFP(half, w // 2, h // 2, downsample=True)
    orc.render_gl(gl, w, h, sc.tile_blocks)
    blurred = _chain(orc, half.reshape(h // 2, w // 2, 4), 3)
    want_lin = orc.glow(quads.reshape(h // 2, w // 2, 16), blurred, w, h, 0)
    want_srgb = orc.glow(quads.reshape(h // 2, w // 2, 16), blurred, w, h, 1)
    # device
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    dep = torch.zeros(w * h, dtype=torch.float32, device="cuda")
    dq = torch.zeros(quads.size, dtype=torch.float32, device="cuda")
    dh = torch.zeros(half.size, dtype=torch.float32, device="cuda")
    ta = torch.zeros(half.size, dtype=torch.float32, device="cuda")
    tb = torch.zeros(half.size, dtype=torch.float32, device="cuda")
    out = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    gl.StoreColorQuads(dq, w, h)
    gl.StoreColorFP(dh, w // 2, h // 2, downsample=True)
    stream = torch.cuda.current_stream().cuda_stream
    gpu.Reset(w, h, sc.tile_blocks)
    gpu.Run(gl, stream=stream)
    res = gpu.kawase_chain(dh, ta, tb, w // 2, h // 2, 3, stream=stream)
    gpu.glow(dq, res, out, w, h, srgb=False, stream=stream)
    gpu.Wait()
    torch.cuda.synchronize()
    assert np.array_equal(res.cpu().numpy().view(np.uint32), blurred.reshape(-1).view(np.uint32))
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want_lin)
    gpu.glow(dq, res, out, w, h, srgb=True, stream=stream)
    torch.cuda.synchronize()
    assert np.abs(_channels(out.cpu().numpy()) - _channels(want_srgb)).max() <= 1
