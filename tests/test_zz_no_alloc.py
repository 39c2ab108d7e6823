"""rsrgpu_render_static(): rendering with no device allocation.

Callers such as a host framework that hands out all device memory from its
own pool, or a real-time loop that may never call cudaMalloc (it blocks the
device and its latency is unbounded), use this entry point: all frame
scratch lives in a fixed array inside the library.  These tests call it
through the C ABI twice in a row and compare each frame with the same frame
rendered through the context-based entry points (rsrgpu_submit/run/wait),
using the tolerances of the other parity tests: depth bit-exact, colour
bit-exact without sRGB and within 1/255 with it.  The file sorts last so a
run that stops at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

from rsr_gb300 import abi, scenes
from rsr_gb300.gpu import GPU

pytestmark = pytest.mark.gpu


def _render_with_context(gpu, sc, dev, col, dep, gamma):
    gpu.Reset(sc.width, sc.height, sc.tile_blocks)
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=gamma)
    gpu.Run(gl)
    gpu.Wait()


def _render_static(lib, sc, dev, col, dep, gamma, stream, gl=None):
    gl = gl or sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=gamma)
    cmds = gl.stream()
    buf = ctypes.create_string_buffer(cmds, len(cmds))
    states = gl.c_states()
    err = ctypes.create_string_buffer(512)
    rc = lib.rsrgpu_render_static(ctypes.cast(buf, ctypes.c_void_p), len(cmds), states, len(gl.states),
                                  sc.width, sc.height, sc.tile_blocks[0], sc.tile_blocks[1],
                                  ctypes.c_void_p(stream), err, 512)
    assert rc == 0, err.value.decode()


def _channels(c):
    return np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1).astype(np.int32)


def test_static_entry_point_matches_context_path(built):
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    gpu = GPU(0)
    gpu.InstallDefaults()
    stream = torch.cuda.current_stream().cuda_stream
    frames = [
        (scenes.plain_raster(seed=21, ntris=6000), False),
        (scenes.clip_stress(seed=22, ntris=2000, tile_blocks=(4, 4)), True),
    ]
    try:
        for sc, gamma in frames:   # two calls in a row, different frames
            dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
            n = sc.width * sc.height
            want_c = torch.zeros(n, dtype=torch.int32, device="cuda")
            want_d = torch.zeros(n, dtype=torch.float32, device="cuda")
            got_c = torch.full((n,), 7, dtype=torch.int32, device="cuda")
            got_d = torch.full((n,), 7.0, dtype=torch.float32, device="cuda")
            _render_with_context(gpu, sc, dev, want_c, want_d, gamma)
            _render_static(lib, sc, dev, got_c, got_d, gamma, stream)
            torch.cuda.synchronize()
            wc, wd = want_c.cpu().numpy().view(np.uint32), want_d.cpu().numpy()
            gc, gd = got_c.cpu().numpy().view(np.uint32), got_d.cpu().numpy()
            assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32))
            if gamma:
                assert np.abs(_channels(gc) - _channels(wc)).max() <= 1
            else:
                assert np.array_equal(gc, wc)
    finally:
        gpu.close()


def test_static_entry_point_float_stores_and_no_device_allocation(built):
    """A frame with rsr's float colour stores (the extended raster
    instantiation) matches the context path bit for bit, and repeated calls
    leave the device's free memory unchanged: the entry point allocates
    nothing (the set-up and the kernels' modules are loaded by a first,
    untimed call)."""
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    gpu = GPU(0)
    gpu.InstallDefaults()
    stream = torch.cuda.current_stream().cuda_stream
    sc = scenes.float_store_frame(seed=23, mid=True)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}

    def outputs(fill):
        return {k: torch.full((v.size,), fill, dtype=torch.float32 if v.dtype == np.float32 else torch.int32,
                              device="cuda") for k, v in sc.outputs.items()}

    try:
        want = outputs(0)
        gpu.Reset(sc.width, sc.height, sc.tile_blocks)
        gpu.Run(sc.record(ref=dev.__getitem__, outputs=want, gamma=False))
        gpu.Wait()
        got = outputs(7)
        gl = sc.record(ref=dev.__getitem__, outputs=got, gamma=False)
        _render_static(lib, sc, dev, None, None, False, stream, gl=gl)
        torch.cuda.synchronize()
        for k in want:
            assert np.array_equal(got[k].cpu().numpy().view(np.uint32), want[k].cpu().numpy().view(np.uint32)), k
        # the opaque plain frame takes the keys path; repeated calls allocate nothing
        pl = scenes.plain_raster(seed=24, ntris=8000)
        pdev = {k: torch.from_numpy(v).cuda() for k, v in pl.arrays.items()}
        pc = torch.zeros(pl.width * pl.height, dtype=torch.int32, device="cuda")
        pd = torch.zeros(pl.width * pl.height, dtype=torch.float32, device="cuda")
        _render_static(lib, pl, pdev, pc, pd, False, stream)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(5):
            _render_static(lib, pl, pdev, pc, pd, False, stream)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 >= free0
        wc = torch.zeros_like(pc)
        wd = torch.zeros_like(pd)
        _render_with_context(gpu, pl, pdev, wc, wd, False)
        torch.cuda.synchronize()
        assert torch.equal(pc, wc) and torch.equal(pd.view(torch.int32), wd.view(torch.int32))
    finally:
        gpu.close()


def test_static_entry_point_rejects_oversized_frames(built):
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    sc = scenes.textured_sphere(divs=6, width=640, height=360, tile_blocks=(4, 4))   # 81 920 triangles
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep)
    cmds = gl.stream()
    buf = ctypes.create_string_buffer(cmds, len(cmds))
    err = ctypes.create_string_buffer(512)
    rc = lib.rsrgpu_render_static(ctypes.cast(buf, ctypes.c_void_p), len(cmds), gl.c_states(), len(gl.states),
                                  sc.width, sc.height, 4, 4, None, err, 512)
    assert rc == -4 and b"triangles" in err.value
