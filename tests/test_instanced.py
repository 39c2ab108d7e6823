"""Instanced draws: GL::DrawElementsInstanced / DrawArraysInstanced
(src/rgl/rglv/rglv_gl.cxx:23-55), binned by BinTriangles1P/2P<INSTANCED>
(src/rgl/rglv/rglv_gpu_impl.hxx:315-675: the draw's triangles once per
instance, each tile record (iid, i0|bf, i1, i2) under
CMD_DRAW_INLINE_INSTANCED), drawn with ManyProgram (src/viewer/shaders.hxx:
482-585: per-instance matrix from buffer 15, colour (u, v, magic)).

Parity: the oracle is pinned to rsr by golden digests (tests/golden/
frames.json, instanced_* scenes, checked in tests/test_oracle.py) and the
GPU is checked against the oracle bit-exact on colour, depth, tile streams
and clipped vertices in tests/test_gpu_parity.py.  This file holds the
recorder bytes, the oracle's instance semantics, and the device routes and
rejections.
"""
import struct

import numpy as np
import pytest

from rsr_gb300 import abi, scenes
from rsr_gb300.gl import GL


def test_recorder_bytes_of_instanced_draws():
    gl = GL()
    idx = np.arange(6, dtype=np.uint16)
    gl.DrawElementsInstanced(6, idx, 7)
    gl.DrawArraysInstanced(9, 3)
    b = gl.stream()
    # a fresh recorder has no pending state change (MaybeUpdateState), so the draws come first
    body = b[17:] if b[0] == abi.CMD_STATE else b
    op, flags, count, ptr, ninst = struct.unpack_from("<BBiQi", body, 0)
    assert (op, flags, count, ptr, ninst) == (abi.CMD_DRAW_ELEMENTS_INSTANCED, 0x14, 6, idx.ctypes.data, 7)
    assert struct.unpack_from("<Bii", body, 18) == (abi.CMD_DRAW_ARRAYS_INSTANCED, 9, 3)
    assert len(body) == 18 + 9


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def _records(tile):
    """(iid, i0|bf, i1, i2) records of every CMD_DRAW_INLINE_INSTANCED in a canonical tile stream."""
    out, p = [], 0
    while p < len(tile):
        op = tile[p]; p += 1
        if op == abi.CMD_EOF:
            break
        if op == abi.CMD_STATE:
            p += 4
        elif op in (abi.CMD_CLEAR, abi.CMD_STORE_COLOR_FULL_LINEAR_TC):
            p += 1
        elif op in (abi.CMD_DRAW_INLINE, abi.CMD_DRAW_INLINE_INSTANCED):
            words = 4 if op == abi.CMD_DRAW_INLINE_INSTANCED else 3
            while True:
                (w,) = struct.unpack_from("<H", tile, p)
                if w == 0xffff:
                    p += 2
                    break
                rec = struct.unpack_from("<%dH" % words, tile, p)
                p += 2 * words
                if op == abi.CMD_DRAW_INLINE_INSTANCED:
                    out.append(rec)
        elif op == abi.CMD_CLIPPED_TRI:
            p += 6
    return out


def test_instance_records_in_instance_order(orc):
    """Within a tile the records of one draw come instance by instance, and an
    instanced copy of a program without instance data repeats the triangles."""
    sc = scenes.instanced_scene(ninst=300, width=320, height=180, tile_blocks=(4, 4))
    orc.render(sc, False)
    tiles = orc.tiles()
    seen_many = seen_copies = False
    for t in tiles:
        recs = _records(t)
        iids = [r[0] for r in recs]
        # two draws per tile at most: iids never decrease within one draw
        breaks = sum(1 for a, b in zip(iids, iids[1:]) if b < a)
        assert breaks <= 1
        seen_many |= len(set(iids)) > 3
        # the Gouraud draw: the same triangle in instances 0, 1, 2
        tri = {}
        for r in recs:
            tri.setdefault(r[1:], []).append(r[0])
        seen_copies |= any(v == [0, 1, 2] for v in tri.values())
    assert seen_many and seen_copies


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.mark.gpu
def test_gpu_instanced_device_and_pinned_routes(gpu, orc):
    """Device-resident inputs and pinned host buffers (instance matrices
    gathered with the vertices) give the oracle's frame bit for bit."""
    import torch
    from rsr_gb300.gpu import render_scene
    sc = scenes.instanced_scene(seed=44, ninst=1500)
    oc, od = orc.render(sc, False)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    render_scene(gpu, sc, gamma=False, device_inputs=dev, color=col, depth=dep)
    torch.cuda.synchronize()
    assert np.array_equal(col.cpu().numpy().view(np.uint32), oc)
    assert np.array_equal(dep.cpu().numpy().view(np.uint32), od.view(np.uint32))
    host = {k: torch.from_numpy(v.copy()).pin_memory() for k, v in sc.arrays.items()}
    hcol = torch.zeros(sc.width * sc.height, dtype=torch.int32).pin_memory()
    hdep = torch.zeros(sc.width * sc.height, dtype=torch.float32).pin_memory()
    bufs = list(host.values()) + [hcol, hdep]
    for t in bufs:
        gpu.register_host_buffer(t)
    try:
        gpu.Reset(sc.width, sc.height, sc.tile_blocks)
        gpu.submit(sc.record(ref=host.__getitem__, color=hcol, depth=hdep, gamma=False))
        gpu.run()
        gpu.Wait()
    finally:
        for t in bufs:
            gpu.unregister_host_buffer(t)
    assert np.array_equal(hcol.numpy().view(np.uint32), oc)
    assert np.array_equal(hdep.numpy().view(np.uint32), od.view(np.uint32))


@pytest.mark.gpu
def test_gpu_instanced_rejections(gpu, built):
    """ManyProgram without instancing, and instanced frames in the
    allocation-free entry: RSRGPU_EUNSUPPORTED with a message.  (Batches take
    instanced frames: tests/test_batch_ext.py.)"""
    import ctypes
    import torch
    from rsr_gb300.gpu import RsrGpuError
    sc = scenes.instanced_scene(ninst=10, width=320, height=180)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    # ManyProgram with a plain DrawElements
    gl = GL()
    gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_RGBF32)
    gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_F32)
    gl.Clear(abi.GL_COLOR_BUFFER_BIT | abi.GL_DEPTH_BUFFER_BIT)
    gl.UseProgram(abi.PROGRAM_MANY)
    gl.UseBuffer(0, (dev["cx"], dev["cy"], dev["cz"]))
    gl.UseBuffer(15, dev["imat"])
    gl.DrawElements(36, dev["cidx"], 0)
    gpu.Reset(sc.width, sc.height, sc.tile_blocks)
    with pytest.raises(RsrGpuError) as e:
        gpu.submit(gl)
    assert e.value.code == -6
    gl2 = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    # the allocation-free entry
    lib = abi.load_library()
    cmds = gl2.stream()
    buf = ctypes.create_string_buffer(cmds, len(cmds))
    err = ctypes.create_string_buffer(256)
    rc = lib.rsrgpu_render_static(ctypes.cast(buf, ctypes.c_void_p), len(cmds), gl2.c_states(), len(gl2.states),
                                  sc.width, sc.height, 4, 4, None, err, 256)
    assert rc == -6 and b"instanced" in err.value
