"""Oracle for the rasteriser path -- test infrastructure, not product code.

Two CPU implementations live here, both driven by the same (command stream,
state snapshots) input that rsrgpu_submit() takes:

  * oracle/rsr_oracle.c  -- a plain-C restatement of rsr's binner, clipper,
    tile rasteriser, fragment programs and resolve (each function cites the
    reference lines it follows).  Portable (x86-64 and aarch64), built into
    oracle/librsroracle.so.  Runs on every machine, including the GPU machine,
    and is the CPU baseline there.
  * oracle/_ref/librsrref.so -- rsr's own sources compiled by
    oracle/ref/Makefile (x86-64 only, SSE4.1), used to pin the restatement.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may load
this package.
"""
import atexit
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "librsrref.so")
ORACLE_LIB = os.path.join(HERE, "librsroracle.so")
SRGB_LUT = os.path.join(os.path.dirname(HERE), "tests", "golden", "srgb8_lut.bin")
SRGB_DECODE = os.path.join(os.path.dirname(HERE), "tests", "golden", "srgb8_to_float.bin")

_ref = None
_oracle = None


def _declare(lib, prefix):
    from rsr_gb300 import abi
    getattr(lib, prefix + "_init").argtypes = [ctypes.c_int]
    getattr(lib, prefix + "_render").argtypes = [
        ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(abi.GLStateC), ctypes.c_int,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    getattr(lib, prefix + "_dump_tiles").argtypes = [
        ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    getattr(lib, prefix + "_dump_clipped").argtypes = [
        ctypes.POINTER(abi.ClippedVertexC), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]


def ref_available():
    return os.path.exists(REF_LIB)


def load_ref(threads=None):
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_LIB)
        _declare(_ref, "rsrref")
        _ref.rsrref_init(threads or os.cpu_count())
        atexit.register(_ref.rsrref_shutdown)
    return _ref


def load_oracle(threads=None):
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError("oracle not built: %s" % ORACLE_LIB)
        _oracle = ctypes.CDLL(ORACLE_LIB)
        _declare(_oracle, "rsroracle")
        _oracle.rsroracle_init(threads or os.cpu_count())
        lut = np.fromfile(SRGB_LUT, np.uint8)
        _oracle.rsroracle_set_srgb_lut(lut.ctypes.data_as(ctypes.c_void_p), len(lut))
    return _oracle


class CpuRenderer:
    """Renders scenes through one of the CPU implementations."""

    def __init__(self, which="oracle", threads=None):
        self.which = which
        self.lib = load_ref(threads) if which == "ref" else load_oracle(threads)
        self.prefix = "rsrref" if which == "ref" else "rsroracle"

    def render_gl(self, gl, width, height, tile_blocks):
        cmds = gl.stream()
        states = gl.c_states()
        buf = ctypes.create_string_buffer(cmds, len(cmds))
        rc = getattr(self.lib, self.prefix + "_render")(
            ctypes.cast(buf, ctypes.c_void_p), len(cmds), states, len(gl.states),
            width, height, tile_blocks[0], tile_blocks[1])
        if rc != 0:
            raise RuntimeError("%s render failed: %d" % (self.which, rc))

    def candidate_fragments(self):
        """Candidate fragments of the last frame (the oracle only): the
        (pixel, triangle) pairs the coverage test accepts, before depth."""
        if self.which == "ref":
            raise RuntimeError("rsr does not count candidate fragments")
        n = ctypes.c_uint64(0)
        if self.lib.rsroracle_candidate_fragments(ctypes.byref(n)) != 0:
            raise RuntimeError("rsroracle_candidate_fragments failed")
        return int(n.value)

    def render(self, scene, gamma=True):
        gl = scene.record(gamma=gamma)
        self.render_gl(gl, scene.width, scene.height, scene.tile_blocks)
        return scene.color.copy(), scene.depth.copy()

    def render_gbuffer(self, scene):
        """Renders a scenes.DeferredScene and returns copies of its G-buffer planes."""
        gl = scene.record()
        self.render_gl(gl, scene.width, scene.height, scene.tile_blocks)
        return {k: v.copy() for k, v in scene.gbuf.items()}

    def shade_plain(self, gbuf, width, height, ivp, eye, lights, background=(0.0, 0.0, 0.0)):
        """The deferred plain shader (oracle restatement); linear RGB float32 (H*W, 3)."""
        from rsr_gb300 import abi
        if self.which != "oracle":
            raise RuntimeError("rsr has no deferred shader; only the oracle implements it")
        g = abi.GBufferC(gbuf["depth"].ctypes.data, gbuf["nx"].ctypes.data, gbuf["ny"].ctypes.data,
                         gbuf["nz"].ctypes.data, gbuf["albedo"].ctypes.data, width, height)
        out = np.zeros((width * height, 3), np.float32)
        lights = np.ascontiguousarray(lights, np.float32)
        f16 = lambda a: (ctypes.c_float * len(a))(*[float(x) for x in a])
        self.lib.rsroracle_shade_plain(ctypes.byref(g), f16(ivp), f16(eye), lights.ctypes.data_as(ctypes.c_void_p),
                                       len(lights), f16(background), out.ctypes.data_as(ctypes.c_void_p))
        return out

    def learned_features(self, gbuf, width, height, ivp, eye, lights, targets=True):
        """The learned shader's per-pixel inputs (oracle restatement): dict with
        'bf16' (H*W, 32) uint16, 'f32' (H*W, 24), 'targets' (H*W, 3) or None
        (sqrt(plain) - base), 'base' (H*W, 3), 'candidates' (tiles, 8) int32 and
        'reach' (H*W,) the candidate lights reaching each pixel."""
        from rsr_gb300 import abi
        if self.which != "oracle":
            raise RuntimeError("only the oracle implements the learned shader's inputs")
        g = abi.GBufferC(gbuf["depth"].ctypes.data, gbuf["nx"].ctypes.data, gbuf["ny"].ctypes.data,
                         gbuf["nz"].ctypes.data, gbuf["albedo"].ctypes.data, width, height)
        npx = width * height
        tiles = ((width + 31) // 32) * ((height + 31) // 32)
        out = {"bf16": np.zeros((npx, 32), np.uint16), "f32": np.zeros((npx, 24), np.float32),
               "targets": np.zeros((npx, 3), np.float32) if targets else None,
               "base": np.zeros((npx, 3), np.float32), "candidates": np.zeros((tiles, 8), np.int32),
               "reach": np.zeros(npx, np.uint8)}
        lights = np.ascontiguousarray(lights, np.float32)
        fa = lambda a: (ctypes.c_float * len(a))(*[float(x) for x in a])
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
        rc = self.lib.rsroracle_learned_features(ctypes.byref(g), fa(ivp), fa(eye), vp(lights), len(lights),
                                                 vp(out["bf16"]), vp(out["f32"]), vp(out["targets"]),
                                                 vp(out["base"]), vp(out["candidates"]), vp(out["reach"]))
        if rc != 0:
            raise RuntimeError("oracle learned_features failed: %d" % rc)
        return out

    def texture_from_rgba8(self, rgba8, width, height, premultiply=False):
        """PNGToTexture's conversion + Texture::maybe_make_mipmap; returns
        (texels float32 (n, 4), power).  The oracle decodes with the reference
        decoder's golden table (tests/golden/srgb8_to_float.bin)."""
        rgba8 = np.ascontiguousarray(rgba8, np.uint8)
        n = width * height
        out = np.zeros((2 * n, 4), np.float32)
        power = ctypes.c_int(0)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        if self.which == "ref":
            rc = self.lib.rsrref_texture_from_rgba8(vp(rgba8), width, height, int(premultiply), vp(out),
                                                    ctypes.c_size_t(2 * n), ctypes.byref(power))
        else:
            lut = np.fromfile(SRGB_DECODE, np.float32)
            rc = self.lib.rsroracle_texture_from_rgba8(vp(rgba8), width, height, int(premultiply), vp(lut), vp(out),
                                                       ctypes.c_size_t(2 * n), ctypes.byref(power))
        if rc != 0:
            raise RuntimeError("%s texture build failed: %d" % (self.which, rc))
        return out[:2 * n if power.value >= 0 else n].copy(), power.value

    def texture_mipmap(self, texels, width, height):
        """Texture::maybe_make_mipmap on float texels (level 0 in the first
        width*height rows of texels (n, 4)); returns (texels, power)."""
        n = width * height
        out = np.zeros((2 * n, 4), np.float32)
        out[:n] = texels[:n]
        power = ctypes.c_int(0)
        fn = getattr(self.lib, self.prefix + "_texture_mipmap")
        rc = fn(out.ctypes.data_as(ctypes.c_void_p), width, height, ctypes.c_size_t(2 * n), ctypes.byref(power))
        if rc != 0:
            raise RuntimeError("%s mipmap failed: %d" % (self.which, rc))
        return out[:2 * n if power.value >= 0 else n].copy(), power.value

    def kawase(self, src, d, out=None):
        """KawaseBlurFilter over a whole RGBA float canvas src (h, w, 4);
        returns the blurred canvas (same size)."""
        src = np.ascontiguousarray(src, np.float32)
        h, w = src.shape[:2]
        dst = np.zeros_like(src) if out is None else out
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        rc = getattr(self.lib, self.prefix + "_kawase")(vp(src), w, h, w, vp(dst), w, h, w, int(d))
        if rc != 0:
            raise RuntimeError("%s kawase failed: %d" % (self.which, rc))
        return dst

    def glow(self, quads, blur, width, height, srgb):
        """Filter<GlowShader> of a full-size quads canvas ((h/2, w/2, 16)
        floats) and a half-size RGBA blur canvas ((h/2, w/2, 4)); returns the
        0x00RRGGBB pixels (h*w,) uint32."""
        quads = np.ascontiguousarray(quads, np.float32)
        blur = np.ascontiguousarray(blur, np.float32)
        out = np.zeros(width * height, np.uint32)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        bh, bw = blur.shape[:2]
        if self.which == "ref":
            rc = self.lib.rsrref_glow(vp(quads), width // 2, vp(blur), bw, bh, bw, vp(out), width, width, height,
                                      int(srgb))
        else:
            rc = self.lib.rsroracle_glow(vp(quads), width // 2, vp(blur), bw, vp(out), width, width, height, int(srgb))
        if rc != 0:
            raise RuntimeError("%s glow failed: %d" % (self.which, rc))
        return out

    def tiles(self):
        need = ctypes.c_size_t(0)
        fn = getattr(self.lib, self.prefix + "_dump_tiles")
        fn(None, 0, ctypes.byref(need))
        out = (ctypes.c_uint8 * max(1, need.value))()
        fn(out, need.value, ctypes.byref(need))
        return split_tiles(bytes(out)[:need.value])

    def clipped(self):
        from rsr_gb300 import abi
        n = ctypes.c_int(0)
        fn = getattr(self.lib, self.prefix + "_dump_clipped")
        fn(None, 0, ctypes.byref(n))
        out = (abi.ClippedVertexC * max(1, n.value))()
        fn(out, n.value, ctypes.byref(n))
        return np.ctypeslib.as_array(ctypes.cast(out, ctypes.POINTER(ctypes.c_float)),
                                     shape=(max(1, n.value) * 20,))[:n.value * 20].reshape(n.value, 20).copy()


def split_tiles(blob):
    """Splits a canonical tile dump (u32 length + bytes per tile) into a list."""
    out = []
    p = 0
    while p < len(blob):
        n = int.from_bytes(blob[p:p + 4], "little")
        out.append(blob[p + 4:p + 4 + n])
        p += 4 + n
    return out
