"""The C ABI library loads and exports every entry point include/rsrgpu.h
declares (no CUDA calls: runs without a GPU)."""
import ctypes
import os
import re
import struct

import numpy as np

from rsr_gb300 import abi
from rsr_gb300.gl import GL

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(REPO, "include", "rsrgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*int\s+(rsrgpu_\w+)\s*\(", text, re.M)))


def test_header_declares_the_runtime_surface():
    names = declared_functions()
    for n in ("rsrgpu_create", "rsrgpu_reset", "rsrgpu_submit", "rsrgpu_run", "rsrgpu_wait", "rsrgpu_install"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(abi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing
    assert set(declared_functions()) == set(abi.SYMBOLS)


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors agree with the C compiler on sizes and field offsets."""
    import subprocess
    structs = {"rsrgpu_texture_state": abi.TextureState, "rsrgpu_glstate": abi.GLStateC,
               "rsrgpu_truecolor_canvas": abi.TrueColorCanvasC, "rsrgpu_fp_canvas": abi.FloatCanvasC,
               "rsrgpu_qfloat4_canvas": abi.FloatCanvasC,
               "rsrgpu_clipped_vertex": abi.ClippedVertexC, "rsrgpu_stats": abi.StatsC}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rsrgpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        for fname, _ in py._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, fname))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout.split()]
    want = []
    for py in structs.values():
        want.append(ctypes.sizeof(py))
        want += [getattr(py, f).offset for f, _ in py._fields_]
    assert got == want


def test_gl_recorder_protocol_bytes():
    """Byte layout of rglv::GL commands (rglv_gl.cxx:34-89, MaybeUpdateState :100-106)."""
    gl = GL()
    idx = np.arange(6, dtype=np.uint16)
    gl.UseProgram(abi.PROGRAM_GOURAUD)
    gl.DrawElements(6, idx, abi.RGL_HINT_DENSE)
    gl.Clear(abi.GL_COLOR_BUFFER_BIT)          # no state change: no new CMD_STATE
    gl.DepthFunc(abi.GL_LEQUAL)
    gl.DrawArrays(3)
    s = gl.stream()
    assert s[0] == abi.CMD_STATE and struct.unpack_from("<Q", s, 1)[0] == 0
    assert s[9] == abi.CMD_DRAW_ELEMENTS and s[10] == 0x14 and s[11] == abi.RGL_HINT_DENSE
    assert struct.unpack_from("<iQ", s, 12) == (6, idx.ctypes.data)
    assert s[24] == abi.CMD_CLEAR and s[25] == 1
    assert s[26] == abi.CMD_STATE and struct.unpack_from("<Q", s, 27)[0] == 1
    assert s[35] == abi.CMD_DRAW_ARRAYS and struct.unpack_from("<i", s, 36)[0] == 3
    assert len(gl.states) == 2 and gl.states[1].depth_func == abi.GL_LEQUAL


def test_splitmix64_known_values():
    from rsr_gb300.scenes import splitmix64
    # splitmix64 with seed 0: the published first outputs
    assert [hex(int(v)) for v in splitmix64(0, 3)] == [
        "0xe220a8397b1dcdaf", "0x6e789e6aa1b965f4", "0x6c45d188009454f"]
