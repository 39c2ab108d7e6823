"""Deferred path (G-buffer pass + 64-light plain shader).

rsr has no deferred or multi-light shading, so the plain shader's oracle is
this repository's C restatement (parity to rsr unpinned for the shading).
The G-buffer pass runs on rsr's rasteriser path, so its depth is pinned to
rsr: the same geometry drawn through rsr with the Gouraud test program gives
the same depth buffer (golden digest from tests/golden/make_golden.py).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from rsr_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def test_gbuffer_depth_pinned_to_reference(orc):
    with open(os.path.join(HERE, "golden", "frames.json")) as f:
        golden = json.load(f)["deferred_gouraud_640/gamma0"]
    g = orc.render_gbuffer(scenes.deferred_scene(nobj=20000, width=640, height=360))
    assert hashlib.sha256(g["depth"].view(np.uint32).tobytes()).hexdigest() == golden["depth"]
    assert int((g["depth"] < 1).sum()) == golden["covered"]
    assert ((g["albedo"] != 0) == (g["depth"] < 1)).all()


def test_plain_shader_basic_properties(orc):
    sc = scenes.deferred_scene(nobj=4000, width=320, height=180, tile_blocks=(2, 2))
    g = orc.render_gbuffer(sc)
    img = orc.shade_plain(g, sc.width, sc.height, sc.ivp, sc.eye, sc.lights, (0.25, 0.5, 0.75))
    bg = g["albedo"] == 0
    assert np.all(img[bg] == np.array([0.25, 0.5, 0.75], np.float32))
    assert np.all(img[~bg] >= 0) and np.isfinite(img).all()
    # no lights: ambient term only
    dark = orc.shade_plain(g, sc.width, sc.height, sc.ivp, sc.eye, sc.lights[:0])
    alb = g["albedo"][~bg]
    want_r = np.float32(0.03) * ((alb & 255).astype(np.float32) / np.float32(255.0))
    assert np.array_equal(dark[~bg, 0], want_r)


@pytest.mark.gpu
def test_gpu_gbuffer_and_plain_shading_match_oracle(orc):
    import torch
    from rsr_gb300.gpu import GPU, render_gbuffer
    sc = scenes.deferred_scene(nobj=30000, width=640, height=360, tile_blocks=(4, 4))
    og = orc.render_gbuffer(sc)
    otiles = orc.tiles()
    gpu = GPU(0)
    try:
        gpu.InstallDefaults()
        gg, _ = render_gbuffer(gpu, sc)
        torch.cuda.synchronize()
        for k in ("depth", "nx", "ny", "nz", "albedo"):
            a = gg[k].cpu().numpy().view(og[k].dtype)
            assert np.array_equal(a.view(np.uint8), og[k].view(np.uint8)), k
        assert gpu.tiles() == otiles
        lights = torch.from_numpy(sc.lights).cuda()
        n = sc.width * sc.height
        lin = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
        srgb = torch.zeros(n, dtype=torch.int32, device="cuda")
        gpu.shade_plain(gg, sc.width, sc.height, sc.ivp, sc.eye, lights, (0.1, 0.2, 0.3), srgb, lin)
        torch.cuda.synchronize()
        oimg = orc.shade_plain(og, sc.width, sc.height, sc.ivp, sc.eye, sc.lights, (0.1, 0.2, 0.3))
        assert np.array_equal(lin.cpu().numpy().view(np.uint32), oimg.reshape(-1).view(np.uint32))
        c = srgb.cpu().numpy().view(np.uint32)
        ch = np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1).astype(np.int32)
        enc = np.clip(oimg, 0, 1)
        enc = np.where(enc <= 0.0031308, 12.92 * enc, 1.055 * enc ** (1 / 2.4) - 0.055)
        assert np.abs(ch - np.round(enc * 255)).max() <= 1
    finally:
        gpu.close()


@pytest.mark.gpu
def test_gpu_benchmarked_deferred_frame_matches_oracle():
    """The deferred frame the benchmark measures (1920x1080, 2 M objects,
    seed 100, 64 lights): every G-buffer plane bit-exact with the oracle,
    and the plain shader's linear colour bit-exact with its restatement."""
    import torch
    import oracle
    from rsr_gb300.gpu import GPU, render_gbuffer
    sc = scenes.deferred_scene(seed=100, width=1920, height=1080, nobj=2_000_000)
    orc = oracle.CpuRenderer("oracle", threads=os.cpu_count())
    og = orc.render_gbuffer(sc)
    gpu = GPU(0)
    try:
        gpu.InstallDefaults()
        gg, _ = render_gbuffer(gpu, sc)
        torch.cuda.synchronize()
        for k in ("depth", "nx", "ny", "nz", "albedo"):
            a = gg[k].cpu().numpy().view(og[k].dtype)
            assert np.array_equal(a.view(np.uint8), og[k].view(np.uint8)), k
        lights = torch.from_numpy(sc.lights).cuda()
        lin = torch.zeros(sc.width * sc.height * 3, dtype=torch.float32, device="cuda")
        gpu.shade_plain(gg, sc.width, sc.height, sc.ivp, sc.eye, lights, out_linear=lin)
        torch.cuda.synchronize()
        oimg = orc.shade_plain(og, sc.width, sc.height, sc.ivp, sc.eye, sc.lights)
        assert np.array_equal(lin.cpu().numpy().view(np.uint32), oimg.reshape(-1).view(np.uint32))
    finally:
        gpu.close()
