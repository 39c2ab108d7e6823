"""OBJ1Program (src/viewer/shaders.hxx:586-699): Gouraud colour lit per vertex
in view space by a point light at the eye -- sqrt, RSQRTPS (rmlv::normalize)
and a divide per vertex.

Parity chain:
  * the oracle is pinned to rsr by golden digests of rsr's own frames
    (tests/golden/frames.json, obj1_* scenes: colour, depth, tile streams,
    clipped vertices), checked in tests/test_oracle.py;
  * RSQRTPS is reproduced by a table measured on the host
    (rsr_gb300/csrc/gen_rsqrtps_table.c checks its model on all 2^32 inputs);
  * the device's shading source (rsr_gb300/csrc/rsrgpu_obj1.h, the function
    the setup kernel calls) is compiled for the host here and compared with
    the oracle bit for bit on random and edge-case vertices;
  * on the GPU, frames are compared with the oracle bit-exact (depth, linear
    colour, tile streams, clipped vertices; sRGB8 within 1/255).
"""
import ctypes
import os
import platform
import subprocess

import numpy as np
import pytest

from rsr_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rsr_gb300", "csrc")


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="RSQRTPS is an x86 instruction")
def test_rsqrtps_table_matches_this_cpu(tmp_path):
    """The committed table reproduces _mm_rsqrt_ss on this host (the generator
    checks its model on all 2^32 inputs before printing)."""
    exe = tmp_path / "gen"
    subprocess.run(["gcc", "-O2", "-msse2", os.path.join(CSRC, "gen_rsqrtps_table.c"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout
    with open(os.path.join(CSRC, "rsqrtps_table.inc")) as f:
        assert f.read() == out


def _host_shading_lib(tmp_path):
    """rsrgpu_obj1.h built for the host (no contraction, like the device build's -fmad=false)."""
    src = tmp_path / "obj1_host.cpp"
    src.write_text(
        '#include "rsrgpu_obj1.h"\n'
        'static const uint32_t T[4096] = {\n#include "rsqrtps_table.inc"\n};\n'
        'extern "C" int obj1_host(const float* vm, const float* vpm, const float* p, const float* n, const float* kd,\n'
        '                         int count, float* pos, float* kd_out) {\n'
        '  for (int i = 0; i < count; ++i)\n'
        '    rsrgpu::obj1_shade(vm, vpm, T, p + 3 * i, n + 3 * i, kd + 3 * i, pos + 4 * i, kd_out + 3 * i);\n'
        '  return 0; }\n')
    so = tmp_path / "libobj1host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                    "-I", CSRC, str(src), "-o", str(so)], check=True)
    return ctypes.CDLL(str(so))


def _vertices(n, seed):
    u = scenes.uniform01(seed, n * 9).reshape(n, 9)
    p = (u[:, 0:3] * np.float32(600.0) - np.float32(300.0)).astype(np.float32)
    nrm = (u[:, 3:6] * np.float32(2.0) - np.float32(1.0)).astype(np.float32)
    kd = u[:, 6:9].astype(np.float32)
    # edge cases: the eye itself (distance 0), points on the near side, tiny
    # and huge coordinates, a zero normal, negative zero
    p[:8] = [[0, 0, 0], [0, 0, -1e-30], [1e-20, 0, 0], [0, 0, 1], [3e18, 0, 0], [-0.0, -0.0, -0.0],
             [0.5, 0.25, -1.0], [1e-38, 1e-38, 1e-38]]
    nrm[:3] = [[0, 0, 0], [-0.0, 0, 0], [0, 1, 0]]
    return p, nrm, kd


def test_device_shading_source_matches_oracle(orc, tmp_path):
    import oracle
    lib = _host_shading_lib(tmp_path)
    olib = oracle.load_oracle()
    rng_views = [scenes.look_at((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0)),
                 scenes.look_at((3.0, 40.0, 25.0), (0.0, -5.0, -80.0), (0.0, 1.0, 0.0))]
    proj = scenes.perspective(60.0, 16 / 9, 1.0, 1000.0)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    n = 200000
    for k, view in enumerate(rng_views):
        vm = np.ascontiguousarray(view, np.float32).reshape(16)
        vpm = np.ascontiguousarray(np.asarray(proj, np.float64).reshape(4, 4).T @ np.asarray(view, np.float64).reshape(4, 4).T,
                                   np.float32).T.reshape(16)
        p, nrm, kd = _vertices(n, 300 + k)
        got = (np.zeros((n, 4), np.float32), np.zeros((n, 3), np.float32))
        want = (np.zeros((n, 4), np.float32), np.zeros((n, 3), np.float32))
        lib.obj1_host(vp(vm), vp(vpm), vp(p), vp(nrm), vp(kd), n, vp(got[0]), vp(got[1]))
        olib.rsroracle_obj1_vertices(vp(vm), vp(vpm), vp(p), vp(nrm), vp(kd), n, vp(want[0]), vp(want[1]))
        for g, w in zip(got, want):
            assert np.array_equal(g.view(np.uint32), w.view(np.uint32))
        if k == 0:
            # at the eye, rsr's qfloat4 operator- leaves d = (0, 0, 0, 1): distance 1,
            # L = (0, 0, 0, 1), diffuse = max(mvn.w = 0, 0.1) * 100
            assert np.array_equal(want[1][0], kd[0] * (np.float32(0.1) * np.float32(100.0)))


def test_obj1_lighting_properties(orc):
    """Lit colours stay below 1 for most of the scene (the comparison is not
    saturated) and the near sphere is clipped."""
    sc = scenes.obj1_scene()
    c, d = orc.render(sc, False)
    ch = np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1)
    covered = d < 1
    assert covered.mean() > 0.2
    assert (ch[covered] == 255).mean() < 0.35   # the near sphere saturates, the far ones do not
    assert len(orc.clipped()) > 0


OBJ1_SCENES = {
    "obj1_640_t32": lambda: scenes.obj1_scene(),
    "obj1_320_t8_2p": lambda: scenes.obj1_scene(dense_hint=True, seed=52, width=320, height=180, tile_blocks=(1, 1)),
    "obj1_720_t64": lambda: scenes.obj1_scene(seed=53, nspheres=60, width=1280, height=720, tile_blocks=(8, 8)),
}


def _channels(c):
    return np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1).astype(np.int32)


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(OBJ1_SCENES))
def test_gpu_obj1_matches_oracle(name, gpu, orc):
    from rsr_gb300.gpu import render_scene
    sc = OBJ1_SCENES[name]()
    for gamma in (False, True):
        oc, od = orc.render(sc, gamma)
        otiles, oclip = orc.tiles(), orc.clipped()
        gc, gd = render_scene(gpu, sc, gamma)
        assert np.array_equal(gd.view(np.uint32), od.view(np.uint32)), "depth differs"
        if gamma:
            assert np.abs(_channels(gc) - _channels(oc)).max() <= 1
        else:
            assert np.array_equal(gc, oc), "linear colour differs"
        assert gpu.tiles() == otiles
        gclip = gpu.clipped()
        assert gclip.shape == oclip.shape
        assert np.array_equal(gclip[:, :7].view(np.uint32), oclip[:, :7].view(np.uint32)), "clipped vertices differ"


@pytest.mark.gpu
def test_gpu_obj1_float_colour(gpu, orc):
    """The lit colour itself, through the full-size float store: bit-exact."""
    import torch
    sc = scenes.obj1_scene(seed=54, nspheres=12)
    w, h = sc.width, sc.height
    want = np.zeros(w * h * 4, np.float32)
    gl = sc.record(gamma=False)
    gl.StoreColorFP(want, w, h)
    orc.render_gl(gl, w, h, sc.tile_blocks)
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    dep = torch.zeros(w * h, dtype=torch.float32, device="cuda")
    fp = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    gl.StoreColorFP(fp, w, h)
    gpu.Reset(w, h, sc.tile_blocks)
    gpu.Run(gl, stream=torch.cuda.current_stream().cuda_stream)
    gpu.Wait()
    torch.cuda.synchronize()
    assert np.array_equal(fp.cpu().numpy().view(np.uint32), want.view(np.uint32))
