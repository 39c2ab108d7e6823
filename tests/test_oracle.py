"""The oracle against rsr's own known answers (CPU only).

* the rasteriser known-answer test of src/rgl/rglv/rglv_triangle.t.cxx:208-235
  (DirectX top-left fill rule, 8x8 mask),
* golden digests of rsr's own frames (tests/golden/frames.json, generated by
  tests/golden/make_golden.py from oracle/_ref) for colour with and without
  sRGB, depth, per-tile command streams and clipped vertices,
* where this host can run rsr itself (x86-64 with oracle/_ref built), a live
  comparison on a fresh seed,
* on x86-64 hosts, the rcpps table against the CPU instruction.
"""
import ctypes
import json
import os
import platform

import numpy as np
import pytest

from rsr_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))

# rglv_triangle.t.cxx:213-228
KAT_POINTS = [(2.0, 4.0), (6.0, 2.0), (1.0, 1.0)]
KAT_EXPECTED = [
    "........",
    ".XX.....",
    ".XXXX...",
    "..X.....",
    "........",
    "........",
    "........",
    "........",
]


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


def test_top_left_fill_rule_kat(orc):
    lib = orc.lib
    pts = (ctypes.c_float * 6)(*[c for p in KAT_POINTS for c in p])
    mask = (ctypes.c_uint8 * 64)()
    assert lib.rsroracle_kat_top_left(pts, 8, 8, mask) == 0
    got = ["".join("X" if mask[y * 8 + x] else "." for x in range(8)) for y in range(8)]
    assert got == KAT_EXPECTED


def _golden():
    # frames of the scenes this test renders (the float-store frames have
    # their own test, tests/test_float_stores.py)
    with open(os.path.join(HERE, "golden", "frames.json")) as f:
        return {k: v for k, v in json.load(f).items() if not k.startswith("float_store")}


GOLDEN = _golden()


@pytest.mark.parametrize("key", sorted(GOLDEN))
def test_oracle_matches_reference_golden(key, orc):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    name, g = key.split("/")
    gamma = g == "gamma1"
    sc = make_golden.make_scene(name)
    c, d = orc.render(sc, gamma)
    nvary = make_golden.GOLDEN_SCENES[name][2]
    got = make_golden.frame_digests(c, d, orc.tiles(), orc.clipped(), nvary)
    assert got == GOLDEN[key]


def test_golden_covers_clipping_and_all_tile_sizes():
    keys = {k.split("/")[0] for k in GOLDEN}
    assert any(GOLDEN[k]["nclipped"] > 0 for k in GOLDEN)
    assert {"plain_320_t8", "plain_1080_t128", "clip_2160_t32", "sphere_1080_t32"} <= keys


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="rsr is SSE code")
def test_live_reference_vs_oracle(orc):
    import oracle
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built on this host")
    ref = oracle.CpuRenderer("ref")
    sc = scenes.clip_stress(seed=42, ntris=1500, width=320, height=180, tile_blocks=(2, 2), extent=4.0)
    for gamma in (False, True):
        c1, d1 = ref.render(sc, gamma)
        t1, v1 = ref.tiles(), ref.clipped()
        c2, d2 = orc.render(sc, gamma)
        t2, v2 = orc.tiles(), orc.clipped()
        assert np.array_equal(c1, c2)
        assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))
        assert t1 == t2
        assert np.array_equal(v1[:, :7].view(np.uint32), v2[:, :7].view(np.uint32))


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="RCPPS is an x86 instruction")
def test_rcpps_table_matches_this_cpu():
    """The committed table reproduces _mm_rcp_ss on this host (sampled; the
    generator checks all 2^32 inputs)."""
    import subprocess
    import tempfile
    src = os.path.join(os.path.dirname(HERE), "rsr_gb300", "csrc", "gen_rcpps_table.c")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "gen")
        subprocess.run(["gcc", "-O2", "-msse2", src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout
    with open(os.path.join(os.path.dirname(HERE), "rsr_gb300", "csrc", "rcpps_table.inc")) as f:
        assert f.read() == out


def test_candidate_fragment_count(orc):
    """The oracle's candidate-fragment count (pixels the coverage test
    accepts, per triangle, before depth): two triangles tiling the screen
    give each pixel once (the top-left rule assigns the shared edge to one
    of them); the same quad drawn twice gives each pixel twice."""
    w, h = 320, 180
    # two triangles of the square [-1, 1]^2, z = 0.5, drawn twice
    quad = np.array([[-1, -1], [1, -1], [1, 1], [-1, -1], [1, 1], [-1, 1]], np.float32)
    pos = np.concatenate([quad, quad])
    arrays = {"px": scenes.pad4(pos[:, 0]), "py": scenes.pad4(pos[:, 1]),
              "pz": scenes.pad4(np.full(len(pos), 0.5, np.float32)),
              "cr": scenes.pad4(np.ones(len(pos), np.float32)), "cg": scenes.pad4(np.zeros(len(pos), np.float32)),
              "cb": scenes.pad4(np.zeros(len(pos), np.float32)), "idx": np.arange(len(pos), dtype=np.uint16)}

    def record(gl, ref, n):
        gl.RenderbufferType(2, 1)   # GL_COLOR_ATTACHMENT0, RB_RGBF32
        gl.RenderbufferType(0, 3)   # GL_DEPTH_ATTACHMENT, RB_F32
        gl.ClearColor((0.0, 0.0, 0.0))
        gl.ClearDepth(1.0)
        gl.Clear(3)
        gl.UseProgram(90)
        gl.UseBuffer(0, (ref("px"), ref("py"), ref("pz")))
        gl.UseBuffer(3, (ref("cr"), ref("cg"), ref("cb")))
        gl.DrawElements(n, ref("idx"), 0)

    for n, want in ((6, w * h), (12, 2 * w * h)):
        sc = scenes.Scene("quad", w, h, (2, 2), arrays, lambda gl, ref, n=n: record(gl, ref, n), n // 3)
        orc.render(sc, False)
        assert orc.candidate_fragments() == want
