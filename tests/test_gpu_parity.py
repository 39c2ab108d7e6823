"""GPU parity against the oracle (rsr_oracle.c, itself pinned bit-exact to rsr).

Bar (same seeded inputs on both sides):
  * depth buffer           bit-exact
  * colour, gamma off      bit-exact (to_tc_basic truncation of the linear colour)
  * colour, gamma on       within 1/255 per channel (sRGB8 encoders differ)
  * tile streams           bit-exact canonical bin lists (order, back-face bits,
                           clipped-triangle records)
  * clipped vertices       bit-exact coordinates and varyings
All calls go through the C ABI (librsrgpu.so) via rsr_gb300.gpu.
"""
import numpy as np
import pytest

from rsr_gb300 import scenes
from rsr_gb300.gpu import GPU, render_scene

pytestmark = pytest.mark.gpu

SCENES = {
    "plain_640_t64": lambda: scenes.plain_raster(),
    "plain_320_t8": lambda: scenes.plain_raster(seed=7, ntris=2000, width=320, height=180, tile_blocks=(1, 1)),
    "plain_1080_t128": lambda: scenes.plain_raster(seed=8, ntris=500, width=1920, height=1080, tile_blocks=(16, 16)),
    "plain_640_t16x32": lambda: scenes.plain_raster(seed=9, ntris=3000, width=640, height=360, tile_blocks=(2, 4)),
    "sphere_1080_t32": lambda: scenes.textured_sphere(divs=6),
    # the benchmarked frame (bench.py's workload): 327 680 triangles
    "sphere_1080_t32_d7": lambda: scenes.textured_sphere(seed=1, divs=7, width=1920, height=1080, tile_blocks=(4, 4),
                                                         tex_dim=1024),
    "clip_640_t64": lambda: scenes.clip_stress(),
    "clip_2160_t32": lambda: scenes.clip_stress(seed=5, width=3840, height=2160, tile_blocks=(4, 4), extent=3.0),
    "mixed_640_t32": lambda: scenes.mixed_states(),
    "mixed_640_t8": lambda: scenes.mixed_states(seed=14, tile_blocks=(1, 1)),
    # scissor-enabled draws (odd rectangle edges, off screen, whole screen,
    # empty, clipped triangles), both attachment layouts, partial tiles
    "scissor_640_t32": lambda: scenes.scissor_scene(),
    "scissor_640_t8_color_depth": lambda: scenes.scissor_scene(seed=62, tile_blocks=(1, 1), color_depth=True),
    "scissor_360_t64": lambda: scenes.scissor_scene(seed=63, width=360, height=202, tile_blocks=(8, 8)),
    # a scissor rectangle past the right and bottom edges: rsr bins outside its
    # tile grid there; the oracle and the device keep to the grid (no rsr digest)
    "scissor_640_t32_past_edges": lambda: scenes.scissor_scene(seed=64, past_edges=True),
    # 1250 chunks of 32 large triangles, nearly all overlapping every 8x8 tile:
    # binning takes its windows of 1024 chunks; four draws
    "plain_320_t8_windows": lambda: scenes.plain_raster(seed=31, ntris=40000, width=320, height=180, tile_blocks=(1, 1)),
    # instanced draws (ManyProgram with per-instance matrices, clipped
    # instances, and an instanced Gouraud draw)
    "instanced_640_t32": lambda: scenes.instanced_scene(),
    "instanced_320_t8_nocull": lambda: scenes.instanced_scene(cull=False, seed=42, ninst=500, width=320, height=180,
                                                              tile_blocks=(1, 1)),
    "instanced_720_t64": lambda: scenes.instanced_scene(seed=43, ninst=3000, width=1280, height=720, tile_blocks=(8, 8)),
}


@pytest.fixture(scope="module")
def gpu(built):
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.fixture(scope="module")
def cpu(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def _channels(c):
    return np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1).astype(np.int32)


@pytest.mark.parametrize("name", list(SCENES))
def test_frame_parity(name, gpu, cpu):
    sc = SCENES[name]()
    for gamma in (False, True):
        oc, od = cpu.render(sc, gamma)
        otiles = cpu.tiles()
        oclip = cpu.clipped()
        gc, gd = render_scene(gpu, sc, gamma)
        assert np.array_equal(gd.view(np.uint32), od.view(np.uint32)), "depth differs"
        if gamma:
            diff = np.abs(_channels(gc) - _channels(oc)).max()
            assert diff <= 1, "sRGB8 colour differs by %d/255" % diff
        else:
            assert np.array_equal(gc, oc), "linear colour differs"
        gtiles = gpu.tiles()
        assert len(gtiles) == len(otiles)
        bad = [i for i in range(len(otiles)) if gtiles[i] != otiles[i]]
        assert not bad, "tile streams differ in %d tiles, first %d" % (len(bad), bad[0])
        gclip = gpu.clipped()
        assert gclip.shape == oclip.shape
        assert np.array_equal(gclip.view(np.uint32), oclip.view(np.uint32)), "clipped vertices differ"


def test_device_resident_inputs(gpu, cpu):
    """Inputs and outputs in device memory are used in place (no staging)."""
    torch = pytest.importorskip("torch")
    sc = scenes.plain_raster(seed=11, ntris=4000)
    oc, od = cpu.render(sc, False)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    gpu.Reset(sc.width, sc.height, sc.tile_blocks)
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    gpu.Run(gl, stream=torch.cuda.current_stream().cuda_stream)
    gpu.Wait()
    torch.cuda.synchronize()
    assert np.array_equal(col.cpu().numpy().view(np.uint32), oc)
    assert np.array_equal(dep.cpu().numpy().view(np.uint32), od.view(np.uint32))


def test_run_timings(gpu):
    """rsrgpu_last_timings: the raster pass (from the end of binning) lies
    within the frame (from its start), on the first run and on graph replays."""
    torch = pytest.importorskip("torch")
    sc = scenes.plain_raster(seed=12, ntris=4000)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    gpu.Reset(sc.width, sc.height, sc.tile_blocks)
    gpu.Run(sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False), stream=stream)
    gpu.Wait()
    for _ in range(3):
        total, raster = gpu.timings()
        assert 0.0 < raster <= total
        gpu.run(stream)
        gpu.Wait()


def test_repeat_determinism(gpu):
    sc = scenes.textured_sphere(divs=5, width=640, height=360, tile_blocks=(4, 4))
    a = render_scene(gpu, sc, True)
    b = render_scene(gpu, sc, True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


def test_unregistered_host_pointer_is_an_error(gpu):
    from rsr_gb300.gpu import RsrGpuError
    sc = scenes.plain_raster(seed=1, ntris=10)
    gpu.Reset(sc.width, sc.height, sc.tile_blocks)
    gl = sc.record(color=np.zeros(sc.width * sc.height, np.uint32), depth=np.zeros(sc.width * sc.height, np.float32))
    with pytest.raises(RsrGpuError):
        gpu.submit(gl)


def test_missing_dispatch_is_an_error(built):
    from rsr_gb300.gpu import RsrGpuError
    g = GPU(0)
    try:
        sc = scenes.plain_raster(seed=1, ntris=10)
        with pytest.raises(RsrGpuError):
            render_scene(g, sc, False)   # nothing installed: GPU::BinImpl would exit(1)
        with pytest.raises(RsrGpuError):
            g.Install(3, 0, 2)           # IQPostProgram has no device implementation
    finally:
        g.close()
