"""ctypes mirror of include/rsrgpu.h (structs, constants) and the library loader.

The product library is rsr_gb300/librsrgpu.so, built in-tree by
rsr_gb300/build.py.  Loading it never falls back to anything else: if the
shared object is missing the import of the GPU entry points fails loudly.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librsrgpu.so")

# protocol (src/rgl/rglv/rglv_gpu_protocol.hxx:7-56)
CMD_EOF = 0x8D
CMD_STATE = 1
CMD_CLEAR = 10
CMD_DRAW_ELEMENTS = 11
CMD_DRAW_ARRAYS = 12
CMD_DRAW_ELEMENTS_INSTANCED = 13
CMD_DRAW_ARRAYS_INSTANCED = 14
CMD_DRAW_INLINE = 15
CMD_DRAW_INLINE_INSTANCED = 16
CMD_STORE_COLOR_FULL_LINEAR_FP = 20
CMD_STORE_COLOR_HALF_LINEAR_FP = 21
CMD_STORE_COLOR_FULL_LINEAR_TC = 22
CMD_STORE_COLOR_FULL_QUADS_FP = 23
CMD_STORE_DEPTH_FULL_LINEAR_FP = 25
CMD_CLIPPED_TRI = 100
CMD_STORE_GBUFFER = 40

# GL enums (src/rgl/rglv/rglv_gl.hxx:20-62)
GL_CULL_FACE = 1
GL_SCISSOR_TEST = 2
GL_BLEND = 3
GL_DEPTH_TEST = 4
GL_FRONT = 1
GL_BACK = 2
GL_LESS = 0
GL_LEQUAL = 1
GL_EQUAL = 2
GL_COLOR_BUFFER_BIT = 1
GL_DEPTH_BUFFER_BIT = 2
GL_DEPTH_ATTACHMENT = 0
GL_COLOR_ATTACHMENT0 = 2
RGL_HINT_READ4 = 1
RGL_HINT_DENSE = 2
RB_COLOR_DEPTH = 0
RB_RGBF32 = 1
RB_RGBAF32 = 2
RB_F32 = 3
GL_NEAREST_MIPMAP_NEAREST = 0
GL_LINEAR_MIPMAP_NEAREST = 1

PROGRAM_DEFAULT_POST = 1
PROGRAM_EXPOSURE_POST = 2
PROGRAM_AMY = 4
PROGRAM_MANY = 6
PROGRAM_OBJ1 = 7
PROGRAM_GOURAUD = 90
PROGRAM_GBUFFER = 91

KIND_BIN, KIND_DRAW, KIND_BLT = 0, 1, 2

DEBUG_LEARNED_STALL = 1

RSRGPU_OK = 0


class TextureState(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("stride", ctypes.c_int32),
                ("filter", ctypes.c_int32)]


class GLStateC(ctypes.Structure):
    """rsrgpu_glstate, mirrors rglv::GLState (rglv_gl.hxx:80-179)."""
    _fields_ = [
        ("clear_color", ctypes.c_float * 4),
        ("clear_depth", ctypes.c_float),
        ("clear_stencil", ctypes.c_int32),
        ("culling_enabled", ctypes.c_int32),
        ("cull_face", ctypes.c_int32),
        ("scissor_enabled", ctypes.c_int32),
        ("scissor_origin", ctypes.c_int32 * 2),
        ("scissor_size", ctypes.c_int32 * 2),
        ("viewport_origin", ctypes.c_int32 * 2),
        ("viewport_size", ctypes.c_int32 * 2),
        ("blending_enabled", ctypes.c_int32),
        ("color_write_mask", ctypes.c_int32),
        ("depth_write_mask", ctypes.c_int32),
        ("depth_test_enabled", ctypes.c_int32),
        ("depth_func", ctypes.c_int32),
        ("program_id", ctypes.c_int32),
        ("uniforms_ofs", ctypes.c_int32),
        ("color0_attachment_type", ctypes.c_int32),
        ("depth_attachment_type", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("uniforms", ctypes.c_float * 32),
        ("buffers", ctypes.c_void_p * 16),
        ("tus", TextureState * 2),
        ("tu3ptr", ctypes.c_void_p),
        ("tu3dim", ctypes.c_int32),
        ("reserved1", ctypes.c_int32),
        ("view_matrix", ctypes.c_float * 16),
        ("normal_matrix", ctypes.c_float * 16),
        ("projection_matrix", ctypes.c_float * 16),
    ]


class TrueColorCanvasC(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("stride", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class FloatCanvasC(ctypes.Structure):
    """rsrgpu_fp_canvas and rsrgpu_qfloat4_canvas (same layout)."""
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("stride", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class ClippedVertexC(ctypes.Structure):
    _fields_ = [("coord", ctypes.c_float * 4), ("data", ctypes.c_float * 16)]


class GBufferC(ctypes.Structure):
    _fields_ = [("depth", ctypes.c_void_p), ("normal_x", ctypes.c_void_p), ("normal_y", ctypes.c_void_p),
                ("normal_z", ctypes.c_void_p), ("albedo", ctypes.c_void_p), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32)]


class LightC(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("radius", ctypes.c_float),
                ("color", ctypes.c_float * 3), ("reserved", ctypes.c_float)]


class MlpC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("w1", "w2", "w3", "w4", "b1", "b2", "b3", "b4")]


class FrameDescC(ctypes.Structure):
    _fields_ = [("commands", ctypes.c_void_p), ("nbytes", ctypes.c_size_t), ("states", ctypes.c_void_p),
                ("nstates", ctypes.c_int32), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("tile_px", ctypes.c_int32), ("region_px", ctypes.c_int32), ("bin_capacity", ctypes.c_uint32)]


class StatsC(ctypes.Structure):
    _fields_ = [("total_tiles", ctypes.c_int64),
                ("total_tile_records", ctypes.c_int64),
                ("total_clipped_records", ctypes.c_int64),
                ("max_tile_records", ctypes.c_int64),
                ("primitives_submitted", ctypes.c_int64),
                ("primitives_clipped", ctypes.c_int64),
                ("gpu_launches", ctypes.c_int64),
                ("graph_captures", ctypes.c_int64),
                ("table_uploads", ctypes.c_int64)]


class GLCallC(ctypes.Structure):
    """rsrgpu_gl_call: one rglv::GL call of a call script."""
    _fields_ = [("fn", ctypes.c_int32), ("i", ctypes.c_int32 * 7), ("p", ctypes.c_uint64),
                ("f", ctypes.c_float * 32)]


class PerfTargetC(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("tile_blocks_x", ctypes.c_int),
                ("tile_blocks_y", ctypes.c_int)]


# rsrgpu_gl_call.fn
(CALL_ENABLE, CALL_DISABLE, CALL_STATE_INT, CALL_SCISSOR, CALL_VIEWPORT, CALL_USE_UNIFORMS, CALL_BIND_TEXTURE,
 CALL_USE_BUFFER, CALL_CLEAR_COLOR, CALL_CLEAR_DEPTH, CALL_MATRIX, CALL_RESET_STATE, CALL_CLEAR, CALL_DRAW_ELEMENTS,
 CALL_DRAW_ARRAYS, CALL_DRAW_ELEMENTS_INSTANCED, CALL_DRAW_ARRAYS_INSTANCED, CALL_STORE_COLOR_TC, CALL_STORE_COLOR_FP,
 CALL_STORE_COLOR_QUADS, CALL_STORE_DEPTH, CALL_STORE_GBUFFER) = range(1, 23)


_LIB = None

SYMBOLS = {
    "rsrgpu_create": ([ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rsrgpu_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_install": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_int], ctypes.c_int),
    "rsrgpu_reset": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_register_host_buffer": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t], ctypes.c_int),
    "rsrgpu_unregister_host_buffer": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_submit": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(GLStateC), ctypes.c_int], ctypes.c_int),
    "rsrgpu_run": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_wait": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_dump_tiles": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "rsrgpu_dump_clipped": ([ctypes.c_void_p, ctypes.POINTER(ClippedVertexC), ctypes.c_int, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "rsrgpu_get_stats": ([ctypes.c_void_p, ctypes.POINTER(StatsC)], ctypes.c_int),
    "rsrgpu_last_timings": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "rsrgpu_last_error": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "rsrgpu_shade_plain": ([ctypes.c_void_p, ctypes.POINTER(GBufferC), ctypes.POINTER(ctypes.c_float),
                            ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                           ctypes.c_int),
    "rsrgpu_texture_from_rgba8": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p],
                                  ctypes.c_int),
    "rsrgpu_texture_mipmap": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                               ctypes.POINTER(ctypes.c_int), ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_kawase_blur": ([ctypes.c_void_p, ctypes.POINTER(FloatCanvasC), ctypes.POINTER(FloatCanvasC), ctypes.c_int,
                            ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_kawase_chain": ([ctypes.c_void_p, ctypes.POINTER(FloatCanvasC), ctypes.POINTER(FloatCanvasC),
                             ctypes.POINTER(FloatCanvasC), ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p],
                            ctypes.c_int),
    "rsrgpu_glow": ([ctypes.c_void_p, ctypes.POINTER(FloatCanvasC), ctypes.POINTER(FloatCanvasC),
                     ctypes.POINTER(TrueColorCanvasC), ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_mlp_forward": ([ctypes.c_void_p, ctypes.POINTER(MlpC), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                            ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_mlp_grad": ([ctypes.c_void_p, ctypes.POINTER(MlpC), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_mlp_adam": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                         ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_shade_learned": ([ctypes.c_void_p, ctypes.POINTER(MlpC), ctypes.POINTER(GBufferC),
                              ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_void_p,
                              ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_shade_learned_check": ([ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_set_debug": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_learned_features": ([ctypes.c_void_p, ctypes.POINTER(GBufferC), ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_batch_create": ([ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rsrgpu_batch_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_batch_install": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_int], ctypes.c_int),
    "rsrgpu_batch_submit": ([ctypes.c_void_p, ctypes.POINTER(FrameDescC), ctypes.c_int], ctypes.c_int),
    "rsrgpu_batch_run": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_batch_wait": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_batch_last_ms": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "rsrgpu_batch_frame": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rsrgpu_batch_tune": ([ctypes.c_void_p, ctypes.POINTER(FrameDescC), ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_batch_last_error": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "rsrgpu_recorder_create": ([ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rsrgpu_recorder_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_recorder_reset": ([ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_recorder_frame": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t),
                               ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "rsrgpu_gl_enable": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_disable": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_state_int": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_scissor": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_viewport": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_use_uniforms": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_bind_texture": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_use_buffer": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_gl_clear_color": ([ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float], ctypes.c_int),
    "rsrgpu_gl_clear_depth": ([ctypes.c_void_p, ctypes.c_float], ctypes.c_int),
    "rsrgpu_gl_matrix": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_gl_reset_state": ([ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_gl_clear": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_draw_elements": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_draw_arrays": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_draw_elements_instanced": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_draw_arrays_instanced": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_store_color_tc": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
                                 ctypes.c_int),
    "rsrgpu_gl_store_color_fp": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
                                 ctypes.c_int),
    "rsrgpu_gl_store_color_quads": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rsrgpu_gl_store_depth": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rsrgpu_gl_store_gbuffer": ([ctypes.c_void_p, ctypes.POINTER(GBufferC)], ctypes.c_int),
    "rsrgpu_gl_play": ([ctypes.c_void_p, ctypes.POINTER(GLCallC), ctypes.c_int], ctypes.c_int),
    "rsrgpu_perf_frames": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(PerfTargetC), ctypes.POINTER(GLCallC),
                            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)],
                           ctypes.c_int),
    "rsrgpu_render_static": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(GLStateC), ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                              ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
}


def load_library(path=LIB_PATH):
    """Loads librsrgpu.so and declares every entry point of include/rsrgpu.h."""
    global _LIB
    if _LIB is not None and path == LIB_PATH:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(
            "librsrgpu.so is not built (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (argtypes, restype) in SYMBOLS.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = restype
    if path == LIB_PATH:
        _LIB = lib
    return lib
