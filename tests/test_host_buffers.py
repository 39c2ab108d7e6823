"""Frames whose inputs and outputs are registered host buffers
(include/rsrgpu.h rsrgpu_register_host_buffer).

Pageable host memory goes through device mirrors: inputs copied in before
the run, outputs copied back after it.  Pinned, mapped host memory takes the
other route: the inputs triangle setup reads arrive by one gather kernel,
textures by a copy on a second stream while setup, binning and (for opaque
frames) the visibility half of the raster pass run, and the raster pass writes
colour and depth straight into the host buffers.  Every route must give the
frame the device-resident inputs give, bit for bit.
"""
import numpy as np
import pytest

from rsr_gb300 import scenes


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


def _device_render(gpu, sc):
    import torch
    from rsr_gb300.gpu import render_scene
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    render_scene(gpu, sc, gamma=True, device_inputs=dev, color=col, depth=dep)
    torch.cuda.synchronize()
    return col.cpu().numpy().view(np.uint32), dep.cpu().numpy().view(np.uint32)


def _pinned_render(gpu, sc, runs=1, mutate=None):
    import torch
    host = {k: torch.from_numpy(v.copy()).pin_memory() for k, v in sc.arrays.items()}
    hcol = torch.zeros(sc.width * sc.height, dtype=torch.int32).pin_memory()
    hdep = torch.zeros(sc.width * sc.height, dtype=torch.float32).pin_memory()
    bufs = list(host.values()) + [hcol, hdep]
    for t in bufs:
        gpu.register_host_buffer(t)
    try:
        gpu.Reset(sc.width, sc.height, sc.tile_blocks)
        gl = sc.record(ref=host.__getitem__, color=hcol, depth=hdep, gamma=True)
        gpu.submit(gl)
        outs = []
        for i in range(runs):
            if mutate is not None and i > 0:
                mutate(host)
            gpu.run()
            gpu.Wait()
            outs.append((hcol.numpy().view(np.uint32).copy(), hdep.numpy().view(np.uint32).copy()))
        launches = gpu.stats()["gpu_launches"]
    finally:
        for t in bufs:
            gpu.unregister_host_buffer(t)
    return outs, launches


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["sphere", "plain"])
def test_pinned_and_pageable_host_buffers_match_device_inputs(gpu, which):
    from rsr_gb300.gpu import render_scene
    if which == "sphere":
        sc = scenes.textured_sphere(seed=2, divs=4, width=640, height=360, tile_blocks=(4, 4), tex_dim=256)
    else:
        sc = scenes.plain_raster(seed=4, ntris=5000, width=640, height=360, tile_blocks=(2, 2))
    want_c, want_d = _device_render(gpu, sc)
    pc, pd = render_scene(gpu, sc, gamma=True)          # pageable: mirrors and copies
    assert np.array_equal(pd.view(np.uint32), want_d) and np.array_equal(pc.view(np.uint32), want_c)
    (outs, launches) = _pinned_render(gpu, sc)
    c, d = outs[0]
    assert np.array_equal(d, want_d) and np.array_equal(c, want_c)
    # gather, the frame's counters, setup, bin, and the raster pass of these
    # opaque frames as two launches (visibility, then shading; the texture of
    # the sphere arrives during the first)
    assert launches == 6


@pytest.mark.gpu
def test_pinned_inputs_are_read_at_every_run(gpu):
    """A second run of the same submission reads the host inputs as they are
    then (vertex positions moved between the runs)."""
    sc = scenes.textured_sphere(seed=3, divs=3, width=320, height=180, tile_blocks=(2, 2), tex_dim=64)
    keys = [k for k in sc.arrays if k.startswith("px")]

    def shrink(host):
        for k in keys:
            host[k].mul_(0.5)

    outs, _ = _pinned_render(gpu, sc, runs=2, mutate=shrink)
    first, second = outs
    assert not np.array_equal(first[1], second[1])
    moved = scenes.textured_sphere(seed=3, divs=3, width=320, height=180, tile_blocks=(2, 2), tex_dim=64)
    for k in keys:
        moved.arrays[k] = moved.arrays[k] * np.float32(0.5)
    want_c, want_d = _device_render(gpu, moved)
    assert np.array_equal(second[1], want_d) and np.array_equal(second[0], want_c)
