"""rsr's float colour stores: StoreColor(FloatingPointCanvas*, downsample) and
StoreColor(QFloat4Canvas*) (src/rgl/rglv/rglv_gl.cxx:64-77), i.e. the tile
interpreter's CMD_STORE_COLOR_FULL_LINEAR_FP, CMD_STORE_COLOR_HALF_LINEAR_FP
and CMD_STORE_COLOR_FULL_QUADS_FP (src/rgl/rglv/rglv_gpu.cxx:345-383).

Bar: every float output bit-exact with the oracle, which is pinned to rsr by
golden digests of rsr's own outputs (tests/golden/frames.json); the sRGB8
TrueColor store of the same frames within 1/255, linear TrueColor and depth
bit-exact; tile streams bit-exact.  Frames store between draws (sequential
walk) and after the last draw (visibility by keys), with an RB_RGBF32 colour
buffer and with RB_COLOR_DEPTH (depth in the colour's w).
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

with open(os.path.join(HERE, "golden", "frames.json")) as _f:
    GOLDEN = {k: v for k, v in json.load(_f).items() if k.split("/")[0] in make_golden.FLOAT_STORE_SCENES}


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def test_golden_has_every_float_store_scene():
    assert len(GOLDEN) == 2 * len(make_golden.FLOAT_STORE_SCENES)


@pytest.mark.parametrize("key", sorted(GOLDEN))
def test_oracle_float_stores_match_reference_golden(key, orc):
    name, g = key.split("/")
    sc = scenes.float_store_frame(**make_golden.FLOAT_STORE_SCENES[name])
    assert make_golden.render_float_store(orc, sc, g == "gamma1") == GOLDEN[key]


def test_float_store_layouts(orc):
    """Size-independent properties of the oracle's float stores: the half
    store is the quad mean of the full store, the quads store holds the full
    store's pixels lane by lane, w is 1 (RB_RGBF32) or the depth
    (RB_COLOR_DEPTH), alpha of the linear stores is 0."""
    for cd in (False, True):
        sc = scenes.float_store_frame(color_depth=cd, ntris=2000, width=160, height=96)
        make_golden.render_float_store(orc, sc, False)
        w, h = sc.width, sc.height
        full = sc.outputs["full"].reshape(h, w, 4)
        half = sc.outputs["half"].reshape(h // 2, w // 2, 4)
        quads = sc.outputs["quads"].reshape(h // 2, w // 2, 4, 4)   # [qy][qx][component][lane]
        assert (full[..., 3] == 0).all() and (half[..., 3] == 0).all()
        lanes = [full[0::2, 0::2], full[0::2, 1::2], full[1::2, 0::2], full[1::2, 1::2]]
        mean = (((lanes[0] + lanes[1]) + lanes[2]) + lanes[3]) * np.float32(0.25)
        assert np.array_equal(half[..., :3], mean[..., :3])
        for l in range(4):
            assert np.array_equal(quads[:, :, :3, l], lanes[l][..., :3])
        if cd:
            assert ((quads[:, :, 3, :] < 1.0).mean() > 0.3)   # covered pixels carry their depth
        else:
            assert (quads[:, :, 3, :] == 1.0).all()


def _channels(c):
    c = c.view(np.uint32)
    return np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1).astype(np.int32)


def _check_outputs(got, want, gamma):
    for k in want:
        if k == "tc" and gamma:
            diff = np.abs(_channels(got[k]) - _channels(want[k])).max()
            assert diff <= 1, "sRGB8 colour differs by %d/255" % diff
        else:
            assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), "%s differs" % k


def _oracle_outputs(orc, sc, gamma):
    for v in sc.outputs.values():
        v[:] = 0
    orc.render_gl(sc.record(gamma=gamma), sc.width, sc.height, sc.tile_blocks)
    return {k: v.copy() for k, v in sc.outputs.items()}, orc.tiles()


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(make_golden.FLOAT_STORE_SCENES))
def test_gpu_float_stores_match_oracle(name, gpu, orc):
    """Host (pageable) buffers: mirrors and copies."""
    sc = scenes.float_store_frame(**make_golden.FLOAT_STORE_SCENES[name])
    for gamma in (False, True):
        want, otiles = _oracle_outputs(orc, sc, gamma)
        for v in sc.outputs.values():
            v[:] = 0
        bufs = list(sc.arrays.values()) + list(sc.outputs.values())
        for a in bufs:
            gpu.register_host_buffer(a)
        try:
            gpu.Reset(sc.width, sc.height, sc.tile_blocks)
            gpu.Run(sc.record(gamma=gamma))
            gpu.Wait()
        finally:
            for a in bufs:
                gpu.unregister_host_buffer(a)
        _check_outputs(sc.outputs, want, gamma)
        assert gpu.tiles() == otiles


@pytest.mark.gpu
def test_gpu_float_stores_device_resident(gpu, orc):
    """Device inputs and outputs used in place."""
    import torch
    sc = scenes.float_store_frame(color_depth=True, mid=True, seed=22)
    want, _ = _oracle_outputs(orc, sc, False)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    out = {k: torch.zeros(v.size, dtype=torch.float32 if v.dtype == np.float32 else torch.int32, device="cuda")
           for k, v in sc.outputs.items()}
    gpu.Reset(sc.width, sc.height, sc.tile_blocks)
    gpu.Run(sc.record(ref=dev.__getitem__, outputs=out, gamma=False), stream=torch.cuda.current_stream().cuda_stream)
    gpu.Wait()
    torch.cuda.synchronize()
    _check_outputs({k: v.cpu().numpy() for k, v in out.items()}, want, False)


def _sphere_with_float_stores(sc, ref, color, depth, full, half, quads):
    gl = sc.record(ref=ref, color=color, depth=depth, gamma=False)
    gl.StoreColorFP(full, sc.width, sc.height)
    gl.StoreColorFP(half, sc.width // 2, sc.height // 2, downsample=True)
    gl.StoreColorQuads(quads, sc.width, sc.height)
    return gl


@pytest.mark.gpu
def test_gpu_float_stores_pinned_split_pass(gpu, orc):
    """Pinned host buffers with a texture: the raster pass of this opaque
    frame runs as two launches (visibility while the texture is copied, then
    shading and the colour stores); the float stores are written in place
    into the host buffers by the second launch."""
    import torch
    sc = scenes.textured_sphere(seed=2, divs=4, width=640, height=360, tile_blocks=(4, 4), tex_dim=256)
    w, h = sc.width, sc.height
    sizes = {"color": w * h, "depth": w * h, "full": w * h * 4, "half": (w // 2) * (h // 2) * 4,
             "quads": (w // 2) * (h // 2) * 16}
    want = {k: np.zeros(n, np.uint32 if k == "color" else np.float32) for k, n in sizes.items()}
    orc.render_gl(_sphere_with_float_stores(sc, None, want["color"], want["depth"], want["full"], want["half"],
                                            want["quads"]), w, h, sc.tile_blocks)
    host = {k: torch.from_numpy(v.copy()).pin_memory() for k, v in sc.arrays.items()}
    out = {k: torch.zeros(n, dtype=torch.int32 if k == "color" else torch.float32).pin_memory()
           for k, n in sizes.items()}
    bufs = list(host.values()) + list(out.values())
    for t in bufs:
        gpu.register_host_buffer(t)
    try:
        gpu.Reset(w, h, sc.tile_blocks)
        gpu.submit(_sphere_with_float_stores(sc, host.__getitem__, out["color"], out["depth"], out["full"],
                                             out["half"], out["quads"]))
        gpu.run()
        gpu.Wait()
        launches = gpu.stats()["gpu_launches"]
    finally:
        for t in bufs:
            gpu.unregister_host_buffer(t)
    assert launches == 6   # gather, counters, setup, bin, raster (visibility), raster (shading and stores)
    _check_outputs({k: v.numpy() for k, v in out.items()}, want, False)
