"""Frames submitted again and again (rsr's GPUNode::Main records and submits
every frame, src/viewer/node/gpu.cxx:107-146), and the perf harness
rsrgpu_perf_frames (src/viewer/perf.cxx:200-244) over the C ABI.

A submission with the structure of the captured one keeps its CUDA graph and
uploads only the tables; every frame must still equal the oracle's render of
that frame (depth and linear colour bit-exact).
"""
import numpy as np
import pytest

from rsr_gb300 import scenes
from rsr_gb300.gpu import GPU
from rsr_gb300.recorder import ScriptGL

pytestmark = pytest.mark.gpu


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


def _device(sc):
    import torch
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    return dev, col, dep


def _check(sc, col, dep, cpu):
    oc, od = cpu.render(sc, False)
    assert np.array_equal(dep.cpu().numpy().view(np.uint32), od.view(np.uint32)), "depth differs"
    assert np.array_equal(col.cpu().numpy().view(np.uint32), oc), "linear colour differs"


def test_same_structure_keeps_the_graph_and_renders_each_frame(gpu, cpu):
    """Three frames with the same triangle count and states but other vertex
    data, outputs and clear colour: one graph capture, a table upload each,
    every frame equal to the oracle; a frame with another triangle count
    captures anew."""
    import torch
    frames = [scenes.plain_raster(seed=s, ntris=3000, width=320, height=180, tile_blocks=(4, 4), clear_rgb=c)
              for s, c in ((1, (0.0, 0.0, 0.0)), (2, (0.0, 0.0, 0.0)), (3, (0.25, 0.5, 0.75)))]
    made = [_device(sc) for sc in frames]
    gpu.Reset(320, 180, (4, 4))
    before = gpu.stats()
    for sc, (dev, col, dep) in zip(frames, made):
        gpu.Reset(320, 180, (4, 4))
        gpu.submit(sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False))
        gpu.run()
        gpu.Wait()
        torch.cuda.synchronize()
        _check(sc, col, dep, cpu)
    st = gpu.stats()
    assert st["graph_captures"] - before["graph_captures"] == 1
    assert st["table_uploads"] - before["table_uploads"] == 3
    # the same frame again uploads nothing
    sc, (dev, col, dep) = frames[0], made[0]
    gpu.submit(sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False))
    gpu.submit(sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False))
    gpu.run()
    gpu.Wait()
    assert gpu.stats()["table_uploads"] - st["table_uploads"] == 1
    # another triangle count: a new capture
    other = scenes.plain_raster(seed=4, ntris=2000, width=320, height=180, tile_blocks=(4, 4))
    dev, col, dep = _device(other)
    gpu.submit(other.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False))
    gpu.run()
    gpu.Wait()
    torch.cuda.synchronize()
    _check(other, col, dep, cpu)
    assert gpu.stats()["graph_captures"] - st["graph_captures"] == 1


def test_perf_harness_renders_the_frame(gpu, cpu):
    """rsrgpu_perf_frames: every frame reset, recorded natively from the call
    script, submitted, run and waited for; the output is the oracle's."""
    import torch
    sc = scenes.textured_sphere(divs=5, width=640, height=360, tile_blocks=(4, 4), tex_dim=256)
    dev, col, dep = _device(sc)
    script = ScriptGL()
    orig = scenes.GL
    scenes.GL = lambda: script
    try:
        sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    finally:
        scenes.GL = orig
    before = gpu.stats()
    ms = gpu.perf_frames(script, sc.width, sc.height, sc.tile_blocks, frames=5, priming=2)
    torch.cuda.synchronize()
    assert len(ms) == 5 and all(t > 0 for t in ms)
    _check(sc, col, dep, cpu)
    st = gpu.stats()
    assert st["graph_captures"] - before["graph_captures"] <= 1
    assert st["table_uploads"] - before["table_uploads"] <= 1


def test_perf_harness_with_pinned_host_buffers(gpu, cpu):
    """The end-to-end route: inputs and outputs in pinned host memory,
    gathered and written in place inside every frame."""
    import torch
    sc = scenes.textured_sphere(divs=5, width=640, height=360, tile_blocks=(4, 4), tex_dim=256)
    host = {k: torch.from_numpy(v).pin_memory() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32).pin_memory()
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32).pin_memory()
    for t in list(host.values()) + [col, dep]:
        gpu.register_host_buffer(t)
    try:
        script = ScriptGL()
        orig = scenes.GL
        scenes.GL = lambda: script
        try:
            sc.record(ref=host.__getitem__, color=col, depth=dep, gamma=False)
        finally:
            scenes.GL = orig
        gpu.perf_frames(script, sc.width, sc.height, sc.tile_blocks, frames=3, priming=1)
        _check(sc, col, dep, cpu)
        # inputs are read in every frame: moved vertices show up
        for k in [k for k in sc.arrays if k.startswith("px")]:
            sc.arrays[k] *= np.float32(0.75)
            host[k].copy_(torch.from_numpy(sc.arrays[k]))
        gpu.perf_frames(script, sc.width, sc.height, sc.tile_blocks, frames=1)
        _check(sc, col, dep, cpu)
    finally:
        for t in list(host.values()) + [col, dep]:
            gpu.unregister_host_buffer(t)


def test_perf_harness_reports_a_failing_call(gpu):
    from rsr_gb300.gpu import RsrGpuError
    script = ScriptGL()
    script.UseBuffer(16, None)
    with pytest.raises(RsrGpuError):
        gpu.perf_frames(script, 320, 180, (4, 4), frames=1)
