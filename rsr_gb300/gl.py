"""GL command recorder with the calling surface of rglv::GL.

Mirrors src/rgl/rglv/rglv_gl.hxx:182-345 and rglv_gl.cxx:13-106: state
setters mark the state dirty; the next command snapshots the full state
(MaybeUpdateState, rglv_gl.cxx:100-106) and emits CMD_STATE followed by the
snapshot's index.  Commands are written in the reference's byte protocol
(rglv_gpu_protocol.hxx) so the stream can be handed to rsrgpu_submit(), to
the oracle, or replayed into the reference itself.
"""
import ctypes
import struct

import numpy as np

from . import abi

UNIFORM_BUFFER_SIZE = 32


def _identity():
    m = np.zeros(16, np.float32)
    m[0] = m[5] = m[10] = m[15] = 1.0
    return m


class GLState:
    """Python-side GLState with the defaults of GLState::reset (rglv_gl.hxx:152-179)."""

    def __init__(self):
        self.reset()

    def reset(self):
        self.clear_color = (0.0, 0.0, 0.0, 1.0)
        self.clear_depth = 1.0
        self.culling_enabled = False
        self.cull_face = abi.GL_BACK
        self.scissor_enabled = False
        self.scissor_origin = (0, 0)
        self.scissor_size = (0, 0)
        self.viewport_origin = (0, 0)
        self.viewport_size = None
        self.blending_enabled = False
        self.color_write_mask = True
        self.depth_write_mask = True
        self.depth_test_enabled = True
        self.depth_func = abi.GL_LESS
        self.program_id = 0
        self.uniforms = None
        self.color0_attachment_type = abi.RB_COLOR_DEPTH
        self.depth_attachment_type = abi.RB_COLOR_DEPTH
        self.buffers = [None] * 16
        self.tus = [(None, 8, 8, 8, abi.GL_NEAREST_MIPMAP_NEAREST)] * 2
        self.tu3 = (None, 256)
        self.view_matrix = _identity()
        self.normal_matrix = _identity()
        self.projection_matrix = _identity()

    def copy(self):
        c = GLState.__new__(GLState)
        c.__dict__ = dict(self.__dict__)
        c.buffers = list(self.buffers)
        c.tus = list(self.tus)
        return c

    def to_c(self):
        s = abi.GLStateC()
        s.clear_color[:] = list(self.clear_color)
        s.clear_depth = self.clear_depth
        s.culling_enabled = int(self.culling_enabled)
        s.cull_face = self.cull_face
        s.scissor_enabled = int(self.scissor_enabled)
        s.scissor_origin[:] = list(self.scissor_origin)
        s.scissor_size[:] = list(self.scissor_size)
        s.viewport_origin[:] = list(self.viewport_origin)
        s.viewport_size[:] = list(self.viewport_size or (0, 0))
        s.blending_enabled = int(self.blending_enabled)
        s.color_write_mask = int(self.color_write_mask)
        s.depth_write_mask = int(self.depth_write_mask)
        s.depth_test_enabled = int(self.depth_test_enabled)
        s.depth_func = self.depth_func
        s.program_id = self.program_id
        if self.uniforms is not None:
            s.uniforms_ofs = 0
            u = np.zeros(UNIFORM_BUFFER_SIZE, np.float32)
            u[:len(self.uniforms)] = self.uniforms
            s.uniforms[:] = u.tolist()
        else:
            s.uniforms_ofs = -1
        s.color0_attachment_type = self.color0_attachment_type
        s.depth_attachment_type = self.depth_attachment_type
        for i, b in enumerate(self.buffers):
            s.buffers[i] = _addr(b)
        for u, (ptr, w, h, stride, filt) in enumerate(self.tus):
            s.tus[u].ptr = _addr(ptr)
            s.tus[u].width, s.tus[u].height, s.tus[u].stride = w, h, stride
            s.tus[u].filter = filt
        s.tu3ptr = _addr(self.tu3[0])
        s.tu3dim = self.tu3[1]
        s.view_matrix[:] = [float(x) for x in self.view_matrix]
        s.normal_matrix[:] = [float(x) for x in self.normal_matrix]
        s.projection_matrix[:] = [float(x) for x in self.projection_matrix]
        return s


def _addr(obj):
    """Address of a numpy array, a torch tensor, an int address, or None."""
    if obj is None:
        return None
    if isinstance(obj, int):
        return obj
    if isinstance(obj, np.ndarray):
        return obj.ctypes.data
    if hasattr(obj, "data_ptr"):
        return obj.data_ptr()
    raise TypeError("unsupported buffer type %r" % type(obj))


class GL:
    """Records one frame.  Buffers passed in are referenced, not copied."""

    def __init__(self):
        self.commands = bytearray()
        self.states = []
        self._cs = GLState()
        self._dirty = False
        self._keep = []  # canvases and other objects the stream points into

    # ---- state (rglv_gl.hxx:186-312) ----
    def Enable(self, v):
        self._dirty = True
        if v == abi.GL_CULL_FACE:
            self._cs.culling_enabled = True
        elif v == abi.GL_SCISSOR_TEST:
            self._cs.scissor_enabled = True
        elif v == abi.GL_BLEND:
            self._cs.blending_enabled = True
        elif v == abi.GL_DEPTH_TEST:
            self._cs.depth_test_enabled = True
        else:
            raise ValueError("unknown glEnable value")

    def Disable(self, v):
        self._dirty = True
        if v == abi.GL_CULL_FACE:
            self._cs.culling_enabled = False
        elif v == abi.GL_SCISSOR_TEST:
            self._cs.scissor_enabled = False
        elif v == abi.GL_BLEND:
            self._cs.blending_enabled = False
        elif v == abi.GL_DEPTH_TEST:
            self._cs.depth_test_enabled = False
        else:
            raise ValueError("unknown glEnable value")

    def DepthFunc(self, v):
        self._dirty = True
        self._cs.depth_func = v

    def DepthWriteMask(self, v):
        self._dirty = True
        self._cs.depth_write_mask = bool(v)

    def ColorWriteMask(self, v):
        self._dirty = True
        self._cs.color_write_mask = bool(v)

    def CullFace(self, v):
        self._dirty = True
        self._cs.cull_face = v

    def Scissor(self, x, y, w, h):
        self._dirty = True
        self._cs.scissor_origin = (x, y)
        self._cs.scissor_size = (w, h)

    def Viewport(self, x, y, w, h):
        self._dirty = True
        self._cs.viewport_origin = (x, y)
        self._cs.viewport_size = (w, h)

    def UseProgram(self, v):
        self._dirty = True
        self._cs.program_id = v

    def UseUniforms(self, values):
        self._dirty = True
        self._cs.uniforms = np.asarray(values, np.float32).copy()

    def RenderbufferType(self, attachment, rbtype):
        self._dirty = True
        if attachment == abi.GL_DEPTH_ATTACHMENT:
            self._cs.depth_attachment_type = rbtype
        elif attachment == abi.GL_COLOR_ATTACHMENT0:
            self._cs.color0_attachment_type = rbtype

    def BindTexture(self, unit, ptr, width, height, stride, mode):
        self._dirty = True
        self._cs.tus = list(self._cs.tus)
        self._cs.tus[unit] = (ptr, width, height, stride, mode)

    def UseBuffer(self, idx, ptr):
        """UseBuffer(idx, float*) or UseBuffer(idx, (x, y, z)) for a Float3Array."""
        self._dirty = True
        if isinstance(ptr, (tuple, list)):
            for k, p in enumerate(ptr):
                self._cs.buffers[idx + k] = p
        else:
            self._cs.buffers[idx] = ptr

    def ClearColor(self, rgb):
        self._dirty = True
        self._cs.clear_color = (float(rgb[0]), float(rgb[1]), float(rgb[2]), 1.0)

    def ClearDepth(self, v):
        self._dirty = True
        self._cs.clear_depth = float(v)

    def ViewMatrix(self, m):
        self._dirty = True
        self._cs.view_matrix = np.asarray(m, np.float32).reshape(16).copy()

    def ProjectionMatrix(self, m):
        self._dirty = True
        self._cs.projection_matrix = np.asarray(m, np.float32).reshape(16).copy()

    def NormalMatrix(self, m):
        self._dirty = True
        self._cs.normal_matrix = np.asarray(m, np.float32).reshape(16).copy()

    def ResetX(self):
        self._dirty = True
        self._cs.reset()

    def Reset(self):
        """GL::Reset (rglv_gl.cxx:92-97): an empty frame, the default state,
        marked changed so the next command snapshots it."""
        self.commands = bytearray()
        self.states = []
        self._keep = []
        self._cs.reset()
        self._dirty = True

    # ---- commands (rglv_gl.cxx:13-89) ----
    def _maybe_update_state(self):
        if not self._dirty:
            return
        self.states.append(self._cs.copy())
        self.commands += struct.pack("<BQ", abi.CMD_STATE, len(self.states) - 1)
        self._dirty = False

    def DrawElements(self, count, indices, hint=0):
        self._maybe_update_state()
        self.commands += struct.pack("<BBBiQ", abi.CMD_DRAW_ELEMENTS, 0x14, hint,
                                     int(count), _addr(indices))

    def DrawArrays(self, count):
        self._maybe_update_state()
        self.commands += struct.pack("<Bi", abi.CMD_DRAW_ARRAYS, int(count))

    def DrawElementsInstanced(self, count, indices, instances):
        """GL::DrawElementsInstanced (rglv_gl.cxx:46-55): no hint byte."""
        self._maybe_update_state()
        self.commands += struct.pack("<BBiQi", abi.CMD_DRAW_ELEMENTS_INSTANCED, 0x14, int(count),
                                     _addr(indices), int(instances))

    def DrawArraysInstanced(self, count, instances):
        """GL::DrawArraysInstanced (rglv_gl.cxx:23-31)."""
        self._maybe_update_state()
        self.commands += struct.pack("<Bii", abi.CMD_DRAW_ARRAYS_INSTANCED, int(count), int(instances))

    def Clear(self, bits):
        self._maybe_update_state()
        self.commands += struct.pack("<BB", abi.CMD_CLEAR, bits)

    def StoreColor(self, data, width, height, gamma=True, stride=None):
        """StoreColor(TrueColorCanvas*, enableGammaCorrection)."""
        self._maybe_update_state()
        c = abi.TrueColorCanvasC(_addr(data), width, height, stride or width, 0)
        self._keep.append(c)
        self.commands += struct.pack("<BBQ", abi.CMD_STORE_COLOR_FULL_LINEAR_TC,
                                     1 if gamma else 0, ctypes.addressof(c))

    def StoreColorFP(self, data, width, height, downsample=False, stride=None):
        """StoreColor(FloatingPointCanvas*, downsample) (rglv_gl.cxx:64-70):
        RGBA float pixels, the full target (width x height) or, downsampled,
        one pixel per 2x2 quad (width/2 x height/2 -- pass the canvas size)."""
        self._maybe_update_state()
        c = abi.FloatCanvasC(_addr(data), width, height, stride or width, 0)
        self._keep.append(c)
        op = abi.CMD_STORE_COLOR_HALF_LINEAR_FP if downsample else abi.CMD_STORE_COLOR_FULL_LINEAR_FP
        self.commands += struct.pack("<BQ", op, ctypes.addressof(c))

    def StoreColorQuads(self, data, width, height, stride=None):
        """StoreColor(QFloat4Canvas*) (rglv_gl.cxx:73-77): one 64-byte qfloat4
        per 2x2 quad, stride in quads (default width/2)."""
        self._maybe_update_state()
        c = abi.FloatCanvasC(_addr(data), width, height, stride or width // 2, 0)
        self._keep.append(c)
        self.commands += struct.pack("<BQ", abi.CMD_STORE_COLOR_FULL_QUADS_FP, ctypes.addressof(c))

    def StoreDepth(self, data):
        self._maybe_update_state()
        self.commands += struct.pack("<BQ", abi.CMD_STORE_DEPTH_FULL_LINEAR_FP, _addr(data))

    def StoreGBuffer(self, depth, normal_x, normal_y, normal_z, albedo, width, height):
        """RSRGPU_CMD_STORE_GBUFFER (this library's extension): depth, fp16
        normal planes and RGBA8 albedo of the pixels drawn with the G-buffer
        program."""
        self._maybe_update_state()
        g = abi.GBufferC(_addr(depth), _addr(normal_x), _addr(normal_y), _addr(normal_z), _addr(albedo),
                         width, height)
        self._keep.append(g)
        self.commands += struct.pack("<BQ", abi.CMD_STORE_GBUFFER, ctypes.addressof(g))

    # ---- hand-off ----
    def c_states(self):
        arr = (abi.GLStateC * max(1, len(self.states)))()
        for i, s in enumerate(self.states):
            arr[i] = s.to_c()
        return arr

    def stream(self):
        return bytes(self.commands)
