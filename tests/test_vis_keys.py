"""Visibility by (depth, order) keys in the raster pass.

Frames whose draws are all opaque with depth test and write on and one depth
function (LESS or LEQUAL) resolve visibility with shared-memory 64-bit
atomicMin over (depth rank, drawing order) instead of drawing the triangles
one after another.  These frames stress what the keys must reproduce exactly:
  * ties: every triangle is drawn twice, by two draws with the same geometry
    and different colours -- LESS keeps the first draw's fragment, LEQUAL the
    second's;
  * the drawing order across draws and passes: with a perspective camera many
    triangles are clipped, so each draw has inline triangles and clipped fans
    (a draw's fans come after its inline triangles, before the next draw);
  * depth exactly zero, whose sign the key does not keep: the owner's depth
    is evaluated again.
Each frame must equal the oracle bit for bit (colour with gamma off, depth).
"""
import numpy as np
import pytest

from rsr_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def twice_drawn(func, seed=21, ntris=1500, width=640, height=360, tile_blocks=(4, 4), zero=False):
    nverts = 3 * ntris
    u = scenes.uniform01(seed, nverts * 9).reshape(ntris, 3, 9)
    pos = scenes.lerp(-4.0, 4.0, u[:, :, 0:3]).reshape(nverts, 3)
    if zero:
        # flat triangles at z = 0 in NDC, w = 1 (the second draw's z negated: -0)
        pos = scenes.lerp(-1.2, 1.2, u[:, :, 0:3]).reshape(nverts, 3)
        pos[:, 2] = 0.0
    rgb_a = scenes.lerp(0.0, 1.0, u[:, :, 3:6]).reshape(nverts, 3)
    rgb_b = scenes.lerp(0.0, 1.0, u[:, :, 6:9]).reshape(nverts, 3)
    arrays = {
        "px": scenes.pad4(pos[:, 0]), "py": scenes.pad4(pos[:, 1]), "pz": scenes.pad4(pos[:, 2]),
        "pzb": scenes.pad4(-pos[:, 2] if zero else pos[:, 2]),
        "ar": scenes.pad4(rgb_a[:, 0]), "ag": scenes.pad4(rgb_a[:, 1]), "ab": scenes.pad4(rgb_a[:, 2]),
        "br": scenes.pad4(rgb_b[:, 0]), "bg": scenes.pad4(rgb_b[:, 1]), "bb": scenes.pad4(rgb_b[:, 2]),
        "idx": np.arange(nverts, dtype=np.uint16),
    }
    proj = None if zero else scenes.perspective(90.0, width / height, 0.5, 50.0)

    def record(gl, ref):
        scenes._begin_frame(gl)
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        gl.DepthFunc(func)
        if proj is not None:
            gl.ProjectionMatrix(proj)
        for z, c in (("pz", ("ar", "ag", "ab")), ("pzb", ("br", "bg", "bb"))):
            gl.UseBuffer(0, (ref("px"), ref("py"), ref(z)))
            gl.UseBuffer(3, tuple(ref(k) for k in c))
            gl.DrawElements(nverts, ref("idx"), 0)

    return scenes.Scene("twice_drawn", width, height, tile_blocks, arrays, record, 2 * ntris)


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.mark.parametrize("func", [abi.GL_LESS, abi.GL_LEQUAL])
@pytest.mark.parametrize("zero", [False, True])
def test_keys_match_oracle(gpu, func, zero):
    import oracle
    import torch
    from rsr_gb300.gpu import render_scene
    sc = twice_drawn(func, zero=zero)
    oc, od = oracle.CpuRenderer("oracle").render(sc, False)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    render_scene(gpu, sc, gamma=False, device_inputs=dev, color=col, depth=dep)
    torch.cuda.synchronize()
    gc, gd = col.cpu().numpy().view(np.uint32), dep.cpu().numpy().view(np.uint32)
    assert np.array_equal(gd, od.view(np.uint32)), "depth differs at %d pixels" % int((gd != od.view(np.uint32)).sum())
    assert np.array_equal(gc, oc.view(np.uint32)), "colour differs at %d pixels" % int((gc != oc.view(np.uint32)).sum())
    covered = od.view(np.uint32) != np.float32(1.0).view(np.uint32)
    assert covered.mean() > 0.05
    if zero:
        # depth exactly zero: the key keeps the rank of zero, not its sign, so
        # the owner's depth is evaluated again (owner_depth)
        assert (od.view(np.uint32)[covered] & 0x7fffffff == 0).mean() > 0.5
    else:
        gpu.tiles()
        assert gpu.stats()["total_clipped_records"] > 0


def test_nan_cleared_depth_walks_the_list(gpu):
    """A NaN cleared depth: no fragment passes, and the tiles cannot use keys
    (the clear key would not order).  With this frame's few raster blocks
    the visibility launch shares each block's list among several CTAs, so
    the first of them walks the whole list alone and the others leave it:
    colour is the clear colour and depth the NaN, as in the oracle."""
    import oracle
    import torch
    from rsr_gb300.gpu import render_scene
    base = twice_drawn(abi.GL_LESS)

    def record(gl, ref):
        gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_RGBF32)
        gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_F32)
        gl.ClearColor((0.25, 0.5, 0.75))
        gl.ClearDepth(float("nan"))
        gl.Clear(abi.GL_COLOR_BUFFER_BIT | abi.GL_DEPTH_BUFFER_BIT)
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        gl.UseBuffer(0, (ref("px"), ref("py"), ref("pz")))
        gl.UseBuffer(3, (ref("ar"), ref("ag"), ref("ab")))
        gl.DrawElements(len(base.arrays["idx"]), ref("idx"), 0)

    sc = scenes.Scene("nan_clear", base.width, base.height, base.tile_blocks, base.arrays, record, base.ntris // 2)
    oc, od = oracle.CpuRenderer("oracle").render(sc, False)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    render_scene(gpu, sc, gamma=False, device_inputs=dev, color=col, depth=dep)
    torch.cuda.synchronize()
    gc, gd = col.cpu().numpy().view(np.uint32), dep.cpu().numpy().view(np.uint32)
    assert np.array_equal(gd, od.view(np.uint32))
    assert np.array_equal(gc, oc.view(np.uint32))
    assert np.isnan(dep.cpu().numpy()).all()
