"""rglv::GPU over the C ABI of librsrgpu.so.

Mirrors src/rgl/rglv/rglv_gpu.hxx:97-277: Install(programId, stateKey, ...),
Reset(size, tileBlocks), IC() -> GL recorder, Run().  Run() submits the
recorded stream and enqueues the frame; Wait() blocks until the outputs have
landed.  Failures raise RsrGpuError carrying the library's message (the
reference calls std::exit(1) on the same conditions).
"""
import ctypes

import numpy as np

from . import abi
from .gl import GL


class RsrGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rsrgpu error %d: %s" % (code, msg))
        self.code = code


# The fragment state keys rsr's viewer installs (src/viewer/shaders.cxx:49-53,
# 71-126) plus LEQUAL and the no-depth-write variant of the RGB f32 layout.
# Each is installed with and without the scissor test (key bit 0).
DRAW_STATE_KEYS = tuple(k | scissor for k in (0x6E2, 0x6E6, 0x6F2, 0x6C2, 0x62, 0x72) for scissor in (0, 1))


class GPU:
    def __init__(self, device=0):
        self.lib = abi.load_library()
        h = ctypes.c_void_p()
        rc = self.lib.rsrgpu_create(int(device), ctypes.byref(h))
        if rc != 0:
            raise RsrGpuError(rc, "rsrgpu_create failed")
        self.ctx = h
        self._gl = GL()
        self._keep = None
        self.width = self.height = 0
        self.tile_blocks = (8, 8)

    def close(self):
        if self.ctx:
            self.lib.rsrgpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            buf = ctypes.create_string_buffer(512)
            self.lib.rsrgpu_last_error(self.ctx, buf, 512)
            raise RsrGpuError(rc, buf.value.decode(errors="replace"))

    # ---- rglv::GPU surface ----
    def Install(self, program_id, state_key, kind):
        self._check(self.lib.rsrgpu_install(self.ctx, int(program_id), int(state_key), int(kind)))

    def InstallDefaults(self):
        """The device counterpart of rqv::Install (src/viewer/shaders.cxx:54-126)
        for the programs this library implements."""
        for pid in (abi.PROGRAM_GOURAUD, abi.PROGRAM_AMY, abi.PROGRAM_GBUFFER, abi.PROGRAM_MANY, abi.PROGRAM_OBJ1):
            self.Install(pid, 0, abi.KIND_BIN)
            for key in DRAW_STATE_KEYS:
                self.Install(pid, key, abi.KIND_DRAW)
        for pid in (abi.PROGRAM_DEFAULT_POST, abi.PROGRAM_EXPOSURE_POST, abi.PROGRAM_GOURAUD):
            self.Install(pid, 0, abi.KIND_BLT)

    def Reset(self, width, height, tile_blocks=(8, 8)):
        self._check(self.lib.rsrgpu_reset(self.ctx, int(width), int(height),
                                          int(tile_blocks[0]), int(tile_blocks[1])))
        self.width, self.height, self.tile_blocks = width, height, tuple(tile_blocks)
        self._gl = GL()

    def IC(self):
        return self._gl

    def register_host_buffer(self, arr):
        nbytes = arr.nbytes if isinstance(arr, np.ndarray) else arr.numel() * arr.element_size()
        ptr = arr.ctypes.data if isinstance(arr, np.ndarray) else arr.data_ptr()
        self._check(self.lib.rsrgpu_register_host_buffer(self.ctx, ctypes.c_void_p(ptr), nbytes))

    def unregister_host_buffer(self, arr):
        ptr = arr.ctypes.data if isinstance(arr, np.ndarray) else arr.data_ptr()
        self._check(self.lib.rsrgpu_unregister_host_buffer(self.ctx, ctypes.c_void_p(ptr)))

    def submit(self, gl=None):
        gl = gl or self._gl
        cmds = gl.stream()
        states = gl.c_states()
        buf = ctypes.create_string_buffer(cmds, max(1, len(cmds)))
        self._keep = (buf, states, gl)
        self._check(self.lib.rsrgpu_submit(self.ctx, ctypes.cast(buf, ctypes.c_void_p), len(cmds),
                                           states, len(gl.states)))

    def Run(self, gl=None, stream=None):
        """Submit the recorded frame and enqueue it (GPU::Run)."""
        self.submit(gl)
        self.run(stream)

    def run(self, stream=None):
        self._check(self.lib.rsrgpu_run(self.ctx, ctypes.c_void_p(stream) if stream else None))

    def Wait(self, timeout_ms=-1):
        self._check(self.lib.rsrgpu_wait(self.ctx, int(timeout_ms)))

    def perf_frames(self, script, width, height, tile_blocks, frames, priming=0, stream=None):
        """rsr's perf loop through the C ABI (rsrgpu_perf_frames): per frame
        Reset, the script's GL calls on a native recorder, submit, run, wait.
        `script`: a recorder.ScriptGL.  Returns the timed frames' host times
        in milliseconds."""
        from .recorder import NativeGL
        rec = NativeGL(self.lib)
        try:
            calls = script.array()
            target = abi.PerfTargetC(int(width), int(height), int(tile_blocks[0]), int(tile_blocks[1]))
            out = (ctypes.c_double * max(1, frames))()
            self._check(self.lib.rsrgpu_perf_frames(self.ctx, rec.h, ctypes.byref(target), calls, len(script.calls),
                                                    int(priming), int(frames),
                                                    ctypes.c_void_p(stream) if stream else None, out))
            self.width, self.height, self.tile_blocks = width, height, tuple(tile_blocks)
            return list(out)[:frames]
        finally:
            rec.close()

    # ---- inspection ----
    def tiles(self):
        need = ctypes.c_size_t(0)
        self._check(self.lib.rsrgpu_dump_tiles(self.ctx, None, 0, ctypes.byref(need)))
        out = (ctypes.c_uint8 * max(1, need.value))()
        self._check(self.lib.rsrgpu_dump_tiles(self.ctx, out, need.value, ctypes.byref(need)))
        blob = bytes(out)[:need.value]
        res, p = [], 0
        while p < len(blob):
            n = int.from_bytes(blob[p:p + 4], "little")
            res.append(blob[p + 4:p + 4 + n])
            p += 4 + n
        return res

    def clipped(self):
        n = ctypes.c_int(0)
        self._check(self.lib.rsrgpu_dump_clipped(self.ctx, None, 0, ctypes.byref(n)))
        out = (abi.ClippedVertexC * max(1, n.value))()
        self._check(self.lib.rsrgpu_dump_clipped(self.ctx, out, n.value, ctypes.byref(n)))
        flat = np.ctypeslib.as_array(ctypes.cast(out, ctypes.POINTER(ctypes.c_float)),
                                     shape=(max(1, n.value) * 20,))
        return flat[:n.value * 20].reshape(n.value, 20).copy()

    def texture_from_rgba8(self, rgba8, width, height, texels, premultiply=False, stream=None):
        """rsrgpu_texture_from_rgba8: device RGBA8 pixels -> device float texels
        (with rsr's mip chain when square, a power of two and at most 4096);
        returns Texture::pow.  texels: a device tensor of float32."""
        p = ctypes.c_int(0)
        self._check(self.lib.rsrgpu_texture_from_rgba8(self.ctx, ctypes.c_void_p(rgba8.data_ptr()), int(width),
                                                       int(height), 1 if premultiply else 0,
                                                       ctypes.c_void_p(texels.data_ptr()), texels.numel() // 4,
                                                       ctypes.byref(p), ctypes.c_void_p(stream) if stream else None))
        return p.value

    def texture_mipmap(self, texels, width, height, stream=None):
        """rsrgpu_texture_mipmap on a device float texture; returns Texture::pow."""
        p = ctypes.c_int(0)
        self._check(self.lib.rsrgpu_texture_mipmap(self.ctx, ctypes.c_void_p(texels.data_ptr()), int(width), int(height),
                                                   texels.numel() // 4, ctypes.byref(p),
                                                   ctypes.c_void_p(stream) if stream else None))
        return p.value

    @staticmethod
    def _canvas(t, width, height, stride=None):
        return abi.FloatCanvasC(t.data_ptr(), int(width), int(height), int(stride or width), 0)

    def kawase_blur(self, src, dst, width, height, dist, stream=None):
        """rsrgpu_kawase_blur: one KawaseBlurFilter pass between two device RGBA
        float canvases (tensors of width*height*4 float32)."""
        a, b = self._canvas(src, width, height), self._canvas(dst, width, height)
        self._check(self.lib.rsrgpu_kawase_blur(self.ctx, ctypes.byref(a), ctypes.byref(b), int(dist),
                                                ctypes.c_void_p(stream) if stream else None))

    def kawase_chain(self, src, tmp_a, tmp_b, width, height, intensity, stream=None):
        """rsrgpu_kawase_chain (the $kawase node); returns the tensor holding the result."""
        cs = [self._canvas(t, width, height) for t in (src, tmp_a, tmp_b)]
        r = ctypes.c_int(-1)
        self._check(self.lib.rsrgpu_kawase_chain(self.ctx, ctypes.byref(cs[0]), ctypes.byref(cs[1]), ctypes.byref(cs[2]),
                                                 int(intensity), ctypes.byref(r),
                                                 ctypes.c_void_p(stream) if stream else None))
        return (src, tmp_a, tmp_b)[r.value]

    def glow(self, quads, blur, out, width, height, srgb=True, blur_size=None, stream=None):
        """rsrgpu_glow: full-size quads canvas + half-size blur canvas -> 0x00RRGGBB
        (device tensors; blur_size (w, h) defaults to half the image)."""
        bw, bh = blur_size or (width // 2, height // 2)
        q = self._canvas(quads, width, height, width // 2)
        b = self._canvas(blur, bw, bh)
        o = abi.TrueColorCanvasC(out.data_ptr(), int(width), int(height), int(width), 0)
        self._check(self.lib.rsrgpu_glow(self.ctx, ctypes.byref(q), ctypes.byref(b), ctypes.byref(o), 1 if srgb else 0,
                                         ctypes.c_void_p(stream) if stream else None))

    def shade_plain(self, gbuf, width, height, ivp, eye, lights, background=(0.0, 0.0, 0.0),
                    out_srgb=None, out_linear=None, stream=None):
        """Deferred plain shading (include/rsrgpu.h rsrgpu_shade_plain); device tensors."""
        g = abi.GBufferC(gbuf["depth"].data_ptr(), gbuf["nx"].data_ptr(), gbuf["ny"].data_ptr(),
                         gbuf["nz"].data_ptr(), gbuf["albedo"].data_ptr(), width, height)
        fa = lambda a: (ctypes.c_float * len(a))(*[float(x) for x in a])
        self._check(self.lib.rsrgpu_shade_plain(
            self.ctx, ctypes.byref(g), fa(ivp), fa(eye), ctypes.c_void_p(lights.data_ptr()), lights.shape[0],
            fa(background), ctypes.c_void_p(out_srgb.data_ptr() if out_srgb is not None else None),
            ctypes.c_void_p(out_linear.data_ptr() if out_linear is not None else None),
            ctypes.c_void_p(stream) if stream else None))

    def mlp_forward(self, weights, features, out, stream=None):
        """rsrgpu_mlp_forward: features (n, 32) bf16 device tensor -> out (n, 3) fp32."""
        m = abi.MlpC(*[weights[k].data_ptr() for k in ("w1", "w2", "w3", "w4", "b1", "b2", "b3", "b4")])
        self._check(self.lib.rsrgpu_mlp_forward(self.ctx, ctypes.byref(m), ctypes.c_void_p(features.data_ptr()),
                                                features.shape[0], ctypes.c_void_p(out.data_ptr()),
                                                ctypes.c_void_p(stream) if stream else None))

    def mlp_grad(self, weights, features, targets, index, grad, loss, stream=None):
        m = abi.MlpC(*[weights[k].data_ptr() for k in ("w1", "w2", "w3", "w4", "b1", "b2", "b3", "b4")])
        vp = lambda t: ctypes.c_void_p(t.data_ptr())
        self._check(self.lib.rsrgpu_mlp_grad(self.ctx, ctypes.byref(m), vp(features), vp(targets), features.shape[0],
                                             vp(index), index.shape[0], vp(grad), vp(loss),
                                             ctypes.c_void_p(stream) if stream else None))

    def mlp_adam(self, params, grad, m, v, step, lr, wbf16, biases, stream=None):
        vp = lambda t: ctypes.c_void_p(t.data_ptr())
        self._check(self.lib.rsrgpu_mlp_adam(self.ctx, vp(params), vp(grad), vp(m), vp(v), int(step), float(lr),
                                             vp(wbf16), vp(biases), ctypes.c_void_p(stream) if stream else None))

    @staticmethod
    def _mlp_c(weights):
        return abi.MlpC(*[weights[k].data_ptr() for k in ("w1", "w2", "w3", "w4", "b1", "b2", "b3", "b4")])

    @staticmethod
    def _gbuffer_c(gbuf, width, height):
        return abi.GBufferC(gbuf["depth"].data_ptr(), gbuf["nx"].data_ptr(), gbuf["ny"].data_ptr(),
                            gbuf["nz"].data_ptr(), gbuf["albedo"].data_ptr(), width, height)

    def shade_learned(self, weights, gbuf, width, height, ivp, eye, lights, background=(0.0, 0.0, 0.0),
                      max_tile_mse=6.5025, out_srgb=None, out_linear=None, tile_status=None, tile_mse=None,
                      stream=None):
        """Fused learned deferred shading (rsrgpu_shade_learned); device tensors.
        Enqueues only: call shade_learned_check() (or synchronise) before reading."""
        fa = lambda a: (ctypes.c_float * len(a))(*[float(x) for x in a])
        vp = lambda t: ctypes.c_void_p(t.data_ptr() if t is not None else None)
        m, g = self._mlp_c(weights), self._gbuffer_c(gbuf, width, height)
        self._check(self.lib.rsrgpu_shade_learned(
            self.ctx, ctypes.byref(m), ctypes.byref(g), fa(ivp), fa(eye), vp(lights), lights.shape[0], fa(background),
            float(max_tile_mse), vp(out_srgb), vp(out_linear), vp(tile_status), vp(tile_mse),
            ctypes.c_void_p(stream) if stream else None))

    def shade_learned_check(self):
        self._check(self.lib.rsrgpu_shade_learned_check(self.ctx))

    def set_debug(self, knob, value):
        """rsrgpu_set_debug: test hooks for failure paths (abi.DEBUG_*)."""
        self._check(self.lib.rsrgpu_set_debug(self.ctx, int(knob), int(value)))

    def learned_features(self, gbuf, width, height, ivp, eye, lights, features, targets=None, candidates=None,
                         stream=None):
        """rsrgpu_learned_features: dense BF16 features (H*W, 32), optional targets and candidates."""
        fa = lambda a: (ctypes.c_float * len(a))(*[float(x) for x in a])
        vp = lambda t: ctypes.c_void_p(t.data_ptr() if t is not None else None)
        g = self._gbuffer_c(gbuf, width, height)
        self._check(self.lib.rsrgpu_learned_features(
            self.ctx, ctypes.byref(g), fa(ivp), fa(eye), vp(lights), lights.shape[0], vp(features), vp(targets),
            vp(candidates), ctypes.c_void_p(stream) if stream else None))

    def stats(self):
        s = abi.StatsC()
        self._check(self.lib.rsrgpu_get_stats(self.ctx, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.StatsC._fields_}

    def timings(self):
        t, r = ctypes.c_float(), ctypes.c_float()
        self._check(self.lib.rsrgpu_last_timings(self.ctx, ctypes.byref(t), ctypes.byref(r)))
        return t.value, r.value


class FrameContext(GPU):
    """A batch frame's context (rsrgpu_batch_frame): the inspection calls of
    GPU (tiles, clipped, stats) on one frame of a batch; owned by the batch."""

    def __init__(self, lib, handle):
        self.lib = lib
        self.ctx = handle
        self._keep = None

    def close(self):
        self.ctx = None


class Batch:
    """Batched frames (include/rsrgpu.h rsrgpu_batch_*): many independent
    frames, each rsr's byte stream with its own target size and tiling,
    rendered by one captured kernel chain.  Frames are GL recordings whose
    pointers are device tensors."""

    def __init__(self, device=0):
        self.lib = abi.load_library()
        h = ctypes.c_void_p()
        rc = self.lib.rsrgpu_batch_create(int(device), ctypes.byref(h))
        if rc != 0:
            raise RsrGpuError(rc, "rsrgpu_batch_create failed")
        self.h = h
        self._keep = None

    def close(self):
        if self.h:
            self.lib.rsrgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            buf = ctypes.create_string_buffer(512)
            self.lib.rsrgpu_batch_last_error(self.h, buf, 512)
            raise RsrGpuError(rc, buf.value.decode(errors="replace"))

    def Install(self, program_id, state_key, kind):
        self._check(self.lib.rsrgpu_batch_install(self.h, int(program_id), int(state_key), int(kind)))

    def InstallDefaults(self):
        for pid in (abi.PROGRAM_GOURAUD, abi.PROGRAM_AMY, abi.PROGRAM_GBUFFER, abi.PROGRAM_MANY, abi.PROGRAM_OBJ1):
            self.Install(pid, 0, abi.KIND_BIN)
            for key in DRAW_STATE_KEYS:
                self.Install(pid, key, abi.KIND_DRAW)
        for pid in (abi.PROGRAM_DEFAULT_POST, abi.PROGRAM_EXPOSURE_POST, abi.PROGRAM_GOURAUD):
            self.Install(pid, 0, abi.KIND_BLT)

    def _descs(self, frames):
        """frames: [(gl, width, height, tile_px, region_px, bin_capacity)]"""
        arr = (abi.FrameDescC * len(frames))()
        keep = []
        for i, (gl, w, h, tile, region, cap) in enumerate(frames):
            cmds = gl.stream()
            buf = ctypes.create_string_buffer(cmds, max(1, len(cmds)))
            states = gl.c_states()
            keep += [buf, states, gl]
            arr[i] = abi.FrameDescC(ctypes.cast(buf, ctypes.c_void_p), len(cmds), ctypes.cast(states, ctypes.c_void_p),
                                    len(gl.states), w, h, tile, region, cap)
        return arr, keep

    def tune(self, frames, reps=3):
        """Autotuner (rsrgpu_batch_tune): returns [(tile_px, region_px, bin_capacity)] per frame."""
        arr, keep = self._descs([(gl, w, h, 8, 0, 0) for gl, w, h in frames])
        self._check(self.lib.rsrgpu_batch_tune(self.h, arr, len(frames), int(reps)))
        return [(arr[i].tile_px, arr[i].region_px, arr[i].bin_capacity) for i in range(len(frames))]

    def submit(self, frames):
        arr, keep = self._descs(frames)
        self._keep = (arr, keep)
        self._check(self.lib.rsrgpu_batch_submit(self.h, arr, len(frames)))

    def run(self, stream=None):
        self._check(self.lib.rsrgpu_batch_run(self.h, ctypes.c_void_p(stream) if stream else None))

    def wait(self, timeout_ms=-1):
        self._check(self.lib.rsrgpu_batch_wait(self.h, int(timeout_ms)))

    def last_ms(self):
        ms = ctypes.c_float(0)
        self._check(self.lib.rsrgpu_batch_last_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def frame(self, i):
        h = ctypes.c_void_p()
        self._check(self.lib.rsrgpu_batch_frame(self.h, int(i), ctypes.byref(h)))
        return FrameContext(self.lib, h)


def render_scene(gpu, scene, gamma=True, device_inputs=None, color=None, depth=None):
    """Render a scenes.Scene.  With device_inputs (name -> device tensor) the
    inputs are used in place; otherwise the scene's host arrays are
    registered and copied inside the run.  Returns (color, depth) on the
    host."""
    gpu.Reset(scene.width, scene.height, scene.tile_blocks)
    if device_inputs is None:
        for arr in scene.arrays.values():
            gpu.register_host_buffer(arr)
        if color is None:
            gpu.register_host_buffer(scene.color)
            gpu.register_host_buffer(scene.depth)
        ref = None
    else:
        ref = device_inputs.__getitem__
    gl = scene.record(ref=ref, color=color, depth=depth, gamma=gamma)
    try:
        gpu.Run(gl)
        gpu.Wait()
    finally:
        if device_inputs is None:
            for arr in scene.arrays.values():
                gpu.unregister_host_buffer(arr)
            if color is None:
                gpu.unregister_host_buffer(scene.color)
                gpu.unregister_host_buffer(scene.depth)
    if color is None:
        return scene.color.copy(), scene.depth.copy()
    return color, depth


def render_gbuffer(gpu, scene, dev=None, gbuf=None, stream=None):
    """Renders a scenes.DeferredScene with device-resident inputs and G-buffer.
    dev: name -> device tensor copies of scene.arrays (made here if None)."""
    import torch
    if dev is None:
        dev = {k: torch.from_numpy(v).cuda() for k, v in scene.arrays.items()}
    n = scene.width * scene.height
    if gbuf is None:
        gbuf = {"depth": torch.zeros(n, dtype=torch.float32, device="cuda"),
                "nx": torch.zeros(n, dtype=torch.int16, device="cuda"),
                "ny": torch.zeros(n, dtype=torch.int16, device="cuda"),
                "nz": torch.zeros(n, dtype=torch.int16, device="cuda"),
                "albedo": torch.zeros(n, dtype=torch.int32, device="cuda")}
    gpu.Reset(scene.width, scene.height, scene.tile_blocks)
    gl = scene.record(ref=lambda k, off=0: dev[k][off:], gbuffer=gbuf)
    gpu.Run(gl, stream=stream)
    gpu.Wait()
    return gbuf, dev
