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
               "rsrgpu_clipped_vertex": abi.ClippedVertexC, "rsrgpu_stats": abi.StatsC,
               "rsrgpu_gl_call": abi.GLCallC, "rsrgpu_perf_target": abi.PerfTargetC}
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


def test_c_caller_links_and_records(built, tmp_path):
    """A C99 program includes include/rsrgpu.h, links librsrgpu.so and records
    a frame with the native recorder (no CUDA call); its stream equals the
    Python recorder's for the same calls, up to the canvas pointer."""
    import subprocess
    src = tmp_path / "caller.c"
    src.write_text(r'''
#include <stdio.h>
#include "rsrgpu.h"
int main(void) {
    static float x[4], y[4], z[4], r[4], g[4], b[4];
    static uint16_t idx[3] = { 0, 1, 2 };
    static uint32_t color[64 * 32];
    rsrgpu_recorder* rec;
    if (rsrgpu_recorder_create(&rec)) return 1;
    rsrgpu_gl_state_int(rec, RSRGPU_GLSTATE_COLOR_ATTACHMENT, RSRGPU_RB_RGBF32);
    rsrgpu_gl_state_int(rec, RSRGPU_GLSTATE_DEPTH_ATTACHMENT, RSRGPU_RB_F32);
    rsrgpu_gl_clear(rec, RSRGPU_GL_COLOR_BUFFER_BIT | RSRGPU_GL_DEPTH_BUFFER_BIT);
    rsrgpu_gl_state_int(rec, RSRGPU_GLSTATE_PROGRAM, RSRGPU_PROGRAM_GOURAUD);
    const float* bufs[6] = { x, y, z, r, g, b };
    for (int i = 0; i < 6; ++i) rsrgpu_gl_use_buffer(rec, i, bufs[i]);
    rsrgpu_gl_draw_elements(rec, 3, idx, 0);
    rsrgpu_gl_state_int(rec, RSRGPU_GLSTATE_PROGRAM, RSRGPU_PROGRAM_DEFAULT_POST);
    rsrgpu_gl_store_color_tc(rec, color, 64, 32, 0, 1);
    const uint8_t* cmds; size_t n; const rsrgpu_glstate* states; int ns;
    if (rsrgpu_recorder_frame(rec, &cmds, &n, &states, &ns)) return 2;
    printf("%d %lu %lu %lu\n", ns, (unsigned long)(uintptr_t)idx, (unsigned long)(uintptr_t)x, (unsigned long)n);
    for (size_t i = 0; i < n; ++i) printf("%02x", cmds[i]);
    printf("\n");
    rsrgpu_recorder_destroy(rec);
    return 0;
}
''')
    exe = tmp_path / "caller"
    libdir = os.path.dirname(abi.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lrsrgpu", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout.split("\n")
    ns, idx_addr, x_addr, n = (int(v) for v in out[0].split())
    got = bytes.fromhex(out[1])
    assert ns == 3 and len(got) == n
    gl = GL()
    gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_RGBF32)
    gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_F32)
    gl.Clear(3)
    gl.UseProgram(abi.PROGRAM_GOURAUD)
    gl.UseBuffer(0, (x_addr, x_addr + 16, x_addr + 32))
    gl.DrawElements(3, idx_addr, 0)
    gl.UseProgram(abi.PROGRAM_DEFAULT_POST)
    gl.StoreColor(np.zeros(64 * 32, np.uint32), 64, 32, True)
    want = gl.stream()
    # equal up to the last 8 bytes: the TrueColor canvas descriptor's address
    assert len(got) == len(want) and got[:-8] == want[:-8]
