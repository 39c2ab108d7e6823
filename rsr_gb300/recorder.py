"""NativeGL: the library's own command recorder (include/rsrgpu.h
rsrgpu_recorder_* / rsrgpu_gl_*) behind the method names of rsr_gb300.gl.GL
(rglv::GL's calling surface), so a frame recorded natively can be handed to
GPU.submit() / Batch.submit() like one recorded in Python."""
import ctypes

import numpy as np

from . import abi
from .gl import _addr

_STATE = {"CullFace": 1, "DepthFunc": 2, "DepthWriteMask": 3, "ColorWriteMask": 4, "UseProgram": 5}


class NativeGL:
    def __init__(self, lib=None):
        self.lib = lib or abi.load_library()
        h = ctypes.c_void_p()
        rc = self.lib.rsrgpu_recorder_create(ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("rsrgpu_recorder_create failed: %d" % rc)
        self.h = h
        self._keep = []

    def close(self):
        if self.h:
            self.lib.rsrgpu_recorder_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc):
        if rc != 0:
            raise ValueError("rsrgpu recorder call failed: %d" % rc)

    # ---- state ----
    def Enable(self, v):
        self._ok(self.lib.rsrgpu_gl_enable(self.h, int(v)))

    def Disable(self, v):
        self._ok(self.lib.rsrgpu_gl_disable(self.h, int(v)))

    def _int(self, what, v):
        self._ok(self.lib.rsrgpu_gl_state_int(self.h, what, int(v)))

    def CullFace(self, v):
        self._int(1, v)

    def DepthFunc(self, v):
        self._int(2, v)

    def DepthWriteMask(self, v):
        self._int(3, bool(v))

    def ColorWriteMask(self, v):
        self._int(4, bool(v))

    def UseProgram(self, v):
        self._int(5, v)

    def RenderbufferType(self, attachment, rbtype):
        self._int(6 if attachment == abi.GL_COLOR_ATTACHMENT0 else 7, rbtype)

    def Scissor(self, x, y, w, h):
        self._ok(self.lib.rsrgpu_gl_scissor(self.h, x, y, w, h))

    def Viewport(self, x, y, w, h):
        self._ok(self.lib.rsrgpu_gl_viewport(self.h, x, y, w, h))

    def UseUniforms(self, values):
        v = np.ascontiguousarray(values, np.float32)
        self._ok(self.lib.rsrgpu_gl_use_uniforms(self.h, v.ctypes.data_as(ctypes.c_void_p), len(v)))

    def BindTexture(self, unit, ptr, width, height, stride, mode):
        self._ok(self.lib.rsrgpu_gl_bind_texture(self.h, unit, _addr(ptr), width, height, stride, mode))

    def UseBuffer(self, idx, ptr):
        if isinstance(ptr, (tuple, list)):
            for k, p in enumerate(ptr):
                self._ok(self.lib.rsrgpu_gl_use_buffer(self.h, idx + k, _addr(p)))
        else:
            self._ok(self.lib.rsrgpu_gl_use_buffer(self.h, idx, _addr(ptr)))

    def ClearColor(self, rgb):
        self._ok(self.lib.rsrgpu_gl_clear_color(self.h, float(rgb[0]), float(rgb[1]), float(rgb[2])))

    def ClearDepth(self, v):
        self._ok(self.lib.rsrgpu_gl_clear_depth(self.h, float(v)))

    def _matrix(self, which, m):
        a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
        self._ok(self.lib.rsrgpu_gl_matrix(self.h, which, a.ctypes.data_as(ctypes.c_void_p)))

    def ViewMatrix(self, m):
        self._matrix(0, m)

    def ProjectionMatrix(self, m):
        self._matrix(1, m)

    def NormalMatrix(self, m):
        self._matrix(2, m)

    def ResetX(self):
        self._ok(self.lib.rsrgpu_gl_reset_state(self.h))

    def Reset(self):
        """GL::Reset: an empty frame and the default state, snapshotted by
        the next command."""
        self._ok(self.lib.rsrgpu_recorder_reset(self.h))
        self._keep = []

    # ---- commands ----
    def Clear(self, bits):
        self._ok(self.lib.rsrgpu_gl_clear(self.h, int(bits)))

    def DrawElements(self, count, indices, hint=0):
        self._ok(self.lib.rsrgpu_gl_draw_elements(self.h, int(count), _addr(indices), int(hint)))

    def DrawArrays(self, count):
        self._ok(self.lib.rsrgpu_gl_draw_arrays(self.h, int(count)))

    def DrawElementsInstanced(self, count, indices, instances):
        self._ok(self.lib.rsrgpu_gl_draw_elements_instanced(self.h, int(count), _addr(indices), int(instances)))

    def DrawArraysInstanced(self, count, instances):
        self._ok(self.lib.rsrgpu_gl_draw_arrays_instanced(self.h, int(count), int(instances)))

    def StoreColor(self, data, width, height, gamma=True, stride=None):
        self._ok(self.lib.rsrgpu_gl_store_color_tc(self.h, _addr(data), width, height, stride or 0, 1 if gamma else 0))

    def StoreColorFP(self, data, width, height, downsample=False, stride=None):
        self._ok(self.lib.rsrgpu_gl_store_color_fp(self.h, _addr(data), width, height, stride or 0, 1 if downsample else 0))

    def StoreColorQuads(self, data, width, height, stride=None):
        self._ok(self.lib.rsrgpu_gl_store_color_quads(self.h, _addr(data), width, height, stride or 0))

    def StoreDepth(self, data):
        self._ok(self.lib.rsrgpu_gl_store_depth(self.h, _addr(data)))

    def StoreGBuffer(self, depth, normal_x, normal_y, normal_z, albedo, width, height):
        g = abi.GBufferC(_addr(depth), _addr(normal_x), _addr(normal_y), _addr(normal_z), _addr(albedo), width, height)
        self._ok(self.lib.rsrgpu_gl_store_gbuffer(self.h, ctypes.byref(g)))

    # ---- hand-off (the interface GPU.submit / Batch use) ----
    def _frame(self):
        cmds, n = ctypes.c_void_p(), ctypes.c_size_t()
        states, ns = ctypes.c_void_p(), ctypes.c_int()
        self._ok(self.lib.rsrgpu_recorder_frame(self.h, ctypes.byref(cmds), ctypes.byref(n), ctypes.byref(states),
                                                ctypes.byref(ns)))
        return cmds, n.value, states, ns.value

    def stream(self):
        cmds, n, _, _ = self._frame()
        return ctypes.string_at(cmds, n) if n else b""

    @property
    def states(self):
        return [None] * self._frame()[3]

    def c_states(self):
        _, _, states, ns = self._frame()
        arr = (abi.GLStateC * max(1, ns))()
        if ns:
            ctypes.memmove(arr, states, ctypes.sizeof(abi.GLStateC) * ns)
        return arr


class ScriptGL:
    """rglv::GL's calling surface that writes each call into a call script
    (include/rsrgpu.h rsrgpu_gl_call) instead of making it.  The script is
    played on a native recorder by rsrgpu_gl_play(), or every frame by the
    perf harness rsrgpu_perf_frames(), so the calls are made natively, as a
    C++ caller makes them, without one Python call each."""

    def __init__(self):
        self.calls = []
        self._keep = []

    def _add(self, fn, i=(), p=None, f=()):
        c = abi.GLCallC()
        c.fn = fn
        for k, v in enumerate(i):
            c.i[k] = int(v)
        c.p = _addr(p) or 0
        for k, v in enumerate(f):
            c.f[k] = float(v)
        self.calls.append(c)

    def array(self):
        """The script as a ctypes array of rsrgpu_gl_call."""
        arr = (abi.GLCallC * max(1, len(self.calls)))()
        for k, c in enumerate(self.calls):
            arr[k] = c
        return arr

    # ---- state ----
    def Enable(self, v):
        self._add(abi.CALL_ENABLE, (v,))

    def Disable(self, v):
        self._add(abi.CALL_DISABLE, (v,))

    def _int(self, what, v):
        self._add(abi.CALL_STATE_INT, (what, int(v)))

    def CullFace(self, v):
        self._int(1, v)

    def DepthFunc(self, v):
        self._int(2, v)

    def DepthWriteMask(self, v):
        self._int(3, bool(v))

    def ColorWriteMask(self, v):
        self._int(4, bool(v))

    def UseProgram(self, v):
        self._int(5, v)

    def RenderbufferType(self, attachment, rbtype):
        self._int(6 if attachment == abi.GL_COLOR_ATTACHMENT0 else 7, rbtype)

    def Scissor(self, x, y, w, h):
        self._add(abi.CALL_SCISSOR, (x, y, w, h))

    def Viewport(self, x, y, w, h):
        self._add(abi.CALL_VIEWPORT, (x, y, w, h))

    def UseUniforms(self, values):
        v = np.ascontiguousarray(values, np.float32).reshape(-1)
        if len(v) > 32:
            raise ValueError("at most 32 uniforms")
        self._add(abi.CALL_USE_UNIFORMS, (len(v),), f=v)

    def BindTexture(self, unit, ptr, width, height, stride, mode):
        self._add(abi.CALL_BIND_TEXTURE, (unit, width, height, stride, mode), p=ptr)

    def UseBuffer(self, idx, ptr):
        if isinstance(ptr, (tuple, list)):
            for k, q in enumerate(ptr):
                self._add(abi.CALL_USE_BUFFER, (idx + k,), p=q)
        else:
            self._add(abi.CALL_USE_BUFFER, (idx,), p=ptr)

    def ClearColor(self, rgb):
        self._add(abi.CALL_CLEAR_COLOR, f=rgb[:3])

    def ClearDepth(self, v):
        self._add(abi.CALL_CLEAR_DEPTH, f=(v,))

    def _matrix(self, which, m):
        self._add(abi.CALL_MATRIX, (which,), f=np.asarray(m, np.float32).reshape(16))

    def ViewMatrix(self, m):
        self._matrix(0, m)

    def ProjectionMatrix(self, m):
        self._matrix(1, m)

    def NormalMatrix(self, m):
        self._matrix(2, m)

    def ResetX(self):
        self._add(abi.CALL_RESET_STATE)

    # ---- commands ----
    def Clear(self, bits):
        self._add(abi.CALL_CLEAR, (bits,))

    def DrawElements(self, count, indices, hint=0):
        self._add(abi.CALL_DRAW_ELEMENTS, (count, hint), p=indices)

    def DrawArrays(self, count):
        self._add(abi.CALL_DRAW_ARRAYS, (count,))

    def DrawElementsInstanced(self, count, indices, instances):
        self._add(abi.CALL_DRAW_ELEMENTS_INSTANCED, (count, instances), p=indices)

    def DrawArraysInstanced(self, count, instances):
        self._add(abi.CALL_DRAW_ARRAYS_INSTANCED, (count, instances))

    def StoreColor(self, data, width, height, gamma=True, stride=None):
        self._add(abi.CALL_STORE_COLOR_TC, (width, height, stride or 0, 1 if gamma else 0), p=data)

    def StoreColorFP(self, data, width, height, downsample=False, stride=None):
        self._add(abi.CALL_STORE_COLOR_FP, (width, height, stride or 0, 1 if downsample else 0), p=data)

    def StoreColorQuads(self, data, width, height, stride=None):
        self._add(abi.CALL_STORE_COLOR_QUADS, (width, height, stride or 0), p=data)

    def StoreDepth(self, data):
        self._add(abi.CALL_STORE_DEPTH, p=data)

    def StoreGBuffer(self, depth, normal_x, normal_y, normal_z, albedo, width, height):
        g = abi.GBufferC(_addr(depth), _addr(normal_x), _addr(normal_y), _addr(normal_z), _addr(albedo), width, height)
        self._keep.append(g)
        self._add(abi.CALL_STORE_GBUFFER, p=ctypes.addressof(g))
