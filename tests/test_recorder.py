"""The native command recorder (include/rsrgpu.h rsrgpu_recorder_* /
rsrgpu_gl_*, rglv::GL's calling surface) against the Python recorder
(rsr_gb300/gl.py, whose bytes tests/test_abi.py pins to rglv_gl.cxx).

Every scene the parity tests use is recorded through both with the same
calls: the command streams must be equal byte for byte (canvas and G-buffer
pointers compared by the descriptors they point to) and the state snapshots
equal field for field.  Runs without a GPU (the recorder makes no CUDA call).
"""
import ctypes
import struct

import numpy as np
import pytest

from rsr_gb300 import abi, scenes
from rsr_gb300.recorder import NativeGL


def _canonical(stream):
    """The stream with every descriptor pointer replaced by the descriptor's bytes."""
    out, p = bytearray(), 0
    while p < len(stream):
        op = stream[p]
        out.append(op)
        p += 1
        if op == abi.CMD_STATE:
            out += stream[p:p + 8]; p += 8
        elif op == abi.CMD_CLEAR:
            out += stream[p:p + 1]; p += 1
        elif op == abi.CMD_DRAW_ELEMENTS:
            out += stream[p:p + 14]; p += 14
        elif op == abi.CMD_DRAW_ARRAYS:
            out += stream[p:p + 4]; p += 4
        elif op == abi.CMD_DRAW_ELEMENTS_INSTANCED:
            out += stream[p:p + 17]; p += 17
        elif op == abi.CMD_DRAW_ARRAYS_INSTANCED:
            out += stream[p:p + 8]; p += 8
        elif op == abi.CMD_STORE_COLOR_FULL_LINEAR_TC:
            out += stream[p:p + 1]
            (ptr,) = struct.unpack_from("<Q", stream, p + 1)
            out += ctypes.string_at(ptr, ctypes.sizeof(abi.TrueColorCanvasC)); p += 9
        elif op in (abi.CMD_STORE_COLOR_FULL_LINEAR_FP, abi.CMD_STORE_COLOR_HALF_LINEAR_FP,
                    abi.CMD_STORE_COLOR_FULL_QUADS_FP):
            (ptr,) = struct.unpack_from("<Q", stream, p)
            out += ctypes.string_at(ptr, ctypes.sizeof(abi.FloatCanvasC)); p += 8
        elif op == abi.CMD_STORE_GBUFFER:
            (ptr,) = struct.unpack_from("<Q", stream, p)
            out += ctypes.string_at(ptr, ctypes.sizeof(abi.GBufferC)); p += 8
        elif op == abi.CMD_STORE_DEPTH_FULL_LINEAR_FP:
            out += stream[p:p + 8]; p += 8
        else:
            raise AssertionError("unexpected opcode %d" % op)
    return bytes(out)


SCENES = {
    "plain": lambda: scenes.plain_raster(ntris=3000),
    "plain_multi_draw": lambda: scenes.plain_raster(seed=31, ntris=25000, width=320, height=180, tile_blocks=(1, 1)),
    "sphere": lambda: scenes.textured_sphere(divs=4, width=640, height=360, tex_dim=64),
    "clip": lambda: scenes.clip_stress(),
    "mixed": lambda: scenes.mixed_states(),
    "instanced": lambda: scenes.instanced_scene(ninst=50, width=320, height=180),
    "obj1": lambda: scenes.obj1_scene(nspheres=4, divs=2),
    "float_stores": lambda: scenes.float_store_frame(ntris=500, mid=True),
    "gbuffer": lambda: scenes.deferred_scene(nobj=300, width=320, height=180, tile_blocks=(2, 2)),
}


@pytest.fixture(scope="module")
def lib(built):
    return abi.load_library()


@pytest.mark.parametrize("name", list(SCENES))
def test_native_recorder_matches_python_recorder(name, lib, monkeypatch):
    sc = SCENES[name]()
    py = sc.record()
    monkeypatch.setattr(scenes, "GL", lambda: NativeGL(lib))
    nat = sc.record()
    monkeypatch.undo()
    assert isinstance(nat, NativeGL)
    assert _canonical(nat.stream()) == _canonical(py.stream())
    assert len(nat.states) == len(py.states)
    a, b = nat.c_states(), py.c_states()
    assert ctypes.string_at(a, ctypes.sizeof(a)) == ctypes.string_at(b, ctypes.sizeof(b))
    nat.close()


@pytest.mark.parametrize("name", list(SCENES))
def test_call_script_plays_like_native_calls(name, lib, monkeypatch):
    """A frame's calls written as a script (ScriptGL) and played on a native
    recorder by rsrgpu_gl_play give the stream and snapshots of the same
    calls made one by one."""
    from rsr_gb300.recorder import ScriptGL
    sc = SCENES[name]()
    monkeypatch.setattr(scenes, "GL", lambda: NativeGL(lib))
    nat = sc.record()
    monkeypatch.setattr(scenes, "GL", ScriptGL)
    script = sc.record()
    monkeypatch.undo()
    played = NativeGL(lib)
    assert lib.rsrgpu_gl_play(played.h, script.array(), len(script.calls)) == 0
    assert _canonical(played.stream()) == _canonical(nat.stream())
    a, b = played.c_states(), nat.c_states()
    assert ctypes.string_at(a, ctypes.sizeof(a)) == ctypes.string_at(b, ctypes.sizeof(b))
    bad = ScriptGL()
    bad.UseBuffer(16, None)
    assert lib.rsrgpu_gl_play(played.h, bad.array(), 1) != 0
    played.close()
    nat.close()


def test_recorder_reset_and_errors(lib):
    g = NativeGL(lib)
    g.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_RGBF32)
    g.Clear(3)
    assert len(g.stream()) == 9 + 2 and len(g.states) == 1
    assert lib.rsrgpu_recorder_reset(g.h) == 0
    assert g.stream() == b"" and len(g.states) == 0
    # the state is back to the defaults: the next snapshot equals a fresh recorder's
    g.ResetX()
    g.Clear(3)
    ref = NativeGL(lib)
    ref.ResetX()
    ref.Clear(3)
    a, b = g.c_states(), ref.c_states()
    assert ctypes.string_at(a, ctypes.sizeof(a)) == ctypes.string_at(b, ctypes.sizeof(b))
    with pytest.raises(ValueError):
        g.Enable(99)
    with pytest.raises(ValueError):
        g.UseBuffer(16, None)
    with pytest.raises(ValueError):
        g.UseUniforms(np.zeros(33, np.float32))
    g.close()
    ref.close()


def test_reset_snapshots_the_defaults(lib):
    """GL::Reset leaves the state marked changed (rglv_gl.cxx:92-97): a Clear
    right after it, with no state setter, is preceded by CMD_STATE and a
    snapshot of the default state -- in both recorders."""
    from rsr_gb300.gl import GL
    fresh = NativeGL(lib)
    fresh.ResetX()
    fresh.Clear(3)
    for g in (NativeGL(lib), GL()):
        g.DepthFunc(abi.GL_LEQUAL)
        g.Clear(3)
        g.Reset()
        assert g.stream() == b""
        g.Clear(3)
        s = g.stream()
        assert s[0] == abi.CMD_STATE and struct.unpack_from("<Q", s, 1)[0] == 0
        assert s[9] == abi.CMD_CLEAR and len(s) == 11
        assert len(g.states) == 1
        a, b = g.c_states(), fresh.c_states()
        assert ctypes.string_at(a, ctypes.sizeof(a)) == ctypes.string_at(b, ctypes.sizeof(b))
        if isinstance(g, NativeGL):
            g.close()
    fresh.close()


@pytest.mark.gpu
def test_gpu_renders_a_natively_recorded_frame(built, monkeypatch):
    """A frame recorded by the native recorder renders like the oracle's
    (the recorder owns the canvas descriptors the stream points to)."""
    import oracle
    from rsr_gb300.gpu import GPU, render_scene
    sc = scenes.mixed_states()
    cpu = oracle.CpuRenderer("oracle")
    oc, od = cpu.render(sc, False)
    g = GPU(0)
    try:
        g.InstallDefaults()
        lib = abi.load_library()
        monkeypatch.setattr(scenes, "GL", lambda: NativeGL(lib))
        gc, gd = render_scene(g, sc, False)
    finally:
        g.close()
    assert np.array_equal(gd.view(np.uint32), od.view(np.uint32))
    assert np.array_equal(gc, oc)
