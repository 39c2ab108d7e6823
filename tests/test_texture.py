"""Texture upload and mip chain on the device (include/rsrgpu.h
rsrgpu_texture_from_rgba8, rsrgpu_texture_mipmap) against rsr's image-loader
path: PNGToTexture's per-pixel conversion (src/rgl/rglr/rglr_texture_load.cxx:
40-63, sRGB through ryg::srgb8_to_float) and Texture::maybe_make_mipmap
(src/rgl/rglr/rglr_texture.cxx:33-80).

Bar: bit-exact.  The oracle is pinned to rsr by golden digests of rsr's own
output (tests/golden/textures.json, tests/golden/srgb8_to_float.bin); the
GPU is compared with the oracle on the same seeded pixels, including the
render-to-texture flow (a frame stored as float, then its chain built).
"""
import json
import os
import sys

import numpy as np
import pytest

from rsr_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

with open(os.path.join(HERE, "golden", "textures.json")) as _f:
    GOLDEN = json.load(_f)


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def test_device_decode_table_is_the_reference_decoder():
    """The library's constant table (rsr_gb300/csrc/srgb_decode_table.inc)
    equals ryg::srgb8_to_float's output run from the reference build."""
    with open(os.path.join(REPO, "rsr_gb300", "csrc", "srgb_decode_table.inc")) as f:
        table = np.array([int(x.rstrip("u,"), 16) for x in f.read().split()], np.uint32)
    golden = np.fromfile(os.path.join(HERE, "golden", "srgb8_to_float.bin"), np.uint32)
    assert len(table) == 256 and np.array_equal(table, golden)


def test_golden_covers_every_case():
    assert set(GOLDEN) == set(make_golden.TEXTURE_CASES)


@pytest.mark.parametrize("name", sorted(make_golden.TEXTURE_CASES))
def test_oracle_matches_reference_golden(name, orc):
    w, h, pm, seed = make_golden.TEXTURE_CASES[name]
    texels, power = orc.texture_from_rgba8(make_golden.texture_bytes(w, h, seed), w, h, pm)
    assert make_golden.texture_digest(texels, power) == GOLDEN[name]


def test_chain_layout_properties(orc):
    """Each level-k texel is the row-major sum of its 2x2 parents over 4, the
    levels sit in rsr's stacked rows, and every other texel past level 0 is 0."""
    w = 64
    texels, power = orc.texture_from_rgba8(make_golden.texture_bytes(w, w, 9), w, w, 0)
    assert power == 6 and texels.shape == (2 * w * w, 4)
    img = texels.reshape(2 * w, w, 4)
    covered = np.zeros((2 * w, w), bool)
    covered[:w] = True
    prev, row = img[:w, :w], w
    for k in range(1, power + 1):
        e = w >> k
        lvl = img[row:row + e, :e]
        want = (((prev[0::2, 0::2] + prev[0::2, 1::2]) + prev[1::2, 0::2]) + prev[1::2, 1::2]) / np.float32(4.0)
        assert np.array_equal(lvl, want)
        covered[row:row + e, :e] = True
        prev, row = lvl, row + e
    assert row == 2 * w - 1
    assert (img[~covered] == 0).all()


def test_live_reference_matches_oracle_on_a_1024_chain(orc):
    import oracle
    if not oracle.ref_available():
        pytest.skip("rsr not built on this host")
    ref = oracle.CpuRenderer("ref")
    px = make_golden.texture_bytes(1024, 1024, 11)
    a, pa = ref.texture_from_rgba8(px, 1024, 1024, 1)
    b, pb = orc.texture_from_rgba8(px, 1024, 1024, 1)
    assert pa == pb == 10 and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


GPU_CASES = [(1, 1, 0), (2, 2, 1), (16, 16, 0), (32, 32, 1), (64, 64, 0), (128, 128, 1), (1024, 1024, 0),
             (4096, 4096, 1), (96, 64, 0), (100, 100, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", GPU_CASES, ids=lambda c: "%dx%d_pm%d" % c)
def test_gpu_texture_from_rgba8_matches_oracle(case, gpu, orc):
    import torch
    w, h, pm = case
    px = make_golden.texture_bytes(w, h, w + h + pm)
    want, wpow = orc.texture_from_rgba8(px, w, h, pm)
    dpx = torch.from_numpy(px).cuda()
    # poisoned output: every texel of the result must be written
    out = torch.full((want.shape[0] * 4,), float("nan"), dtype=torch.float32, device="cuda")
    power = gpu.texture_from_rgba8(dpx, w, h, out, premultiply=bool(pm))
    torch.cuda.synchronize()
    assert power == wpow
    got = out.cpu().numpy().reshape(-1, 4)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_gpu_texture_mipmap_on_float_texels(gpu, orc):
    import torch
    w = 256
    level0 = np.random.default_rng(5).random((w * w, 4), dtype=np.float32)
    want, power = orc.texture_mipmap(level0, w, w)
    t = torch.full((2 * w * w * 4,), float("nan"), dtype=torch.float32, device="cuda")
    t[:w * w * 4] = torch.from_numpy(level0.reshape(-1)).cuda()
    assert gpu.texture_mipmap(t, w, w) == power == 8
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy().reshape(-1, 4).view(np.uint32), want.view(np.uint32))
    # no chain for other sizes: nothing written
    u = torch.zeros(60 * 60 * 4, dtype=torch.float32, device="cuda")
    assert gpu.texture_mipmap(u, 60, 60) == -1


@pytest.mark.gpu
def test_gpu_texture_capacity_is_checked(gpu):
    import torch
    from rsr_gb300.gpu import RsrGpuError
    px = torch.zeros(64 * 64 * 4, dtype=torch.uint8, device="cuda")
    out = torch.zeros(64 * 64 * 4, dtype=torch.float32, device="cuda")   # room for level 0 only
    with pytest.raises(RsrGpuError):
        gpu.texture_from_rgba8(px, 64, 64, out)


@pytest.mark.gpu
def test_gpu_render_to_texture(gpu, orc):
    """rsr's renderToTexture node: StoreColor(FloatingPointCanvas*) of a
    square frame, then Texture::maybe_make_mipmap on it."""
    import torch
    w = 256
    sc = scenes.plain_raster(seed=12, ntris=3000, width=w, height=w, tile_blocks=(4, 4), spread=0.4)
    tex = np.zeros(2 * w * w * 4, np.float32)
    gl = sc.record(gamma=False)
    gl.StoreColorFP(tex, w, w)
    orc.render_gl(gl, w, w, sc.tile_blocks)
    want, power = orc.texture_mipmap(tex.reshape(-1, 4), w, w)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(w * w, dtype=torch.int32, device="cuda")
    dep = torch.zeros(w * w, dtype=torch.float32, device="cuda")
    dtex = torch.full((2 * w * w * 4,), float("nan"), dtype=torch.float32, device="cuda")
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    gl.StoreColorFP(dtex, w, w)
    stream = torch.cuda.current_stream().cuda_stream
    gpu.Reset(w, w, sc.tile_blocks)
    gpu.Run(gl, stream=stream)
    assert gpu.texture_mipmap(dtex, w, w, stream=stream) == power
    gpu.Wait()
    torch.cuda.synchronize()
    assert np.array_equal(dtex.cpu().numpy().reshape(-1, 4).view(np.uint32), want.view(np.uint32))
