"""The C++ shim of include/rsrgpu_rglv.hpp (rglv::GPU's surface over the C
ABI) compiled against rsr's own headers, with rsr's own rglv::GL recording
the frame (x86-64 hosts with the reference checkout; skipped elsewhere).

tests/shim/rsr_translate plays a GL call script on rsr's recorder and
translates the stream with TranslateFrame(); the result must equal, byte for
byte (canvas descriptors compared by content), the stream and state
snapshots this library's native recorder makes from the same calls -- whose
bytes tests/test_recorder.py ties to the Python recorder and
tests/test_abi.py to rglv_gl.cxx.  No GPU is used.
"""
import ctypes
import os
import subprocess

import pytest

from rsr_gb300 import abi, scenes
from rsr_gb300.recorder import NativeGL, ScriptGL

from test_recorder import SCENES, _canonical

# rsr has no G-buffer store (a command of this library only)
SHIM_SCENES = [n for n in SCENES if n != "gbuffer"]


@pytest.fixture(scope="module")
def translator(built):
    from rsr_gb300 import build
    try:
        exe = build.build_shim_test()
    except RuntimeError as e:
        pytest.fail("the shim test program does not build:\n%s" % e)
    if exe is None:
        pytest.skip("needs the reference checkout on an x86-64 host")
    return exe


@pytest.mark.parametrize("name", SHIM_SCENES)
def test_translated_rsr_stream_equals_native_recording(name, translator, tmp_path, monkeypatch):
    lib = abi.load_library()
    sc = SCENES[name]()
    monkeypatch.setattr(scenes, "GL", ScriptGL)
    script = sc.record()
    monkeypatch.undo()
    calls = script.array()
    src = tmp_path / "script.bin"
    src.write_bytes(ctypes.string_at(calls, ctypes.sizeof(abi.GLCallC) * len(script.calls)))
    out = tmp_path / "out.bin"
    r = subprocess.run([translator, str(src), str(out)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    blob = out.read_bytes()
    n = int.from_bytes(blob[:8], "little")
    stream = blob[8:8 + n]
    m = int.from_bytes(blob[8 + n:16 + n], "little")
    states = blob[16 + n:]
    assert len(states) == m * ctypes.sizeof(abi.GLStateC)
    nat = NativeGL(lib)
    assert lib.rsrgpu_recorder_reset(nat.h) == 0
    assert lib.rsrgpu_gl_play(nat.h, calls, len(script.calls)) == 0
    assert stream == _canonical(nat.stream())
    a = nat.c_states()
    assert m == len(nat.states)
    assert states == ctypes.string_at(a, ctypes.sizeof(abi.GLStateC) * m)
    nat.close()
