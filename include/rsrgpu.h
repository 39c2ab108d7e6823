/*
 * rsrgpu.h -- C ABI of the GB300 rasteriser (tile binning, per-tile coverage,
 * depth test, fragment shading, sRGB8 resolve) that replaces the rglv
 * virtual GPU of rsr.
 *
 * The calling surface mirrors rglv::GPU (src/rgl/rglv/rglv_gpu.hxx:97-277)
 * and the command protocol recorded by rglv::GL (src/rgl/rglv/rglv_gl.hxx:
 * 182-345, src/rgl/rglv/rglv_gpu_protocol.hxx:7-56).  Everything crosses the
 * boundary as plain pointers and sizes; no C++ or torch types appear here.
 *
 * Command stream
 * --------------
 * A frame is a byte stream in rsr's own protocol (same opcodes, same field
 * order and widths as rglv::GL writes them), with one difference: the 8-byte
 * field after CMD_STATE carries the index of the state snapshot in the
 * `states` array passed to rsrgpu_submit(), instead of a GLState address.
 * Every other pointer field is an address supplied by the caller:
 *   CMD_DRAW_ELEMENTS   op u8, 0x14 u8, hint u8, count i32, indices u16*
 *   CMD_DRAW_ARRAYS     op u8, count i32
 *   CMD_DRAW_ELEMENTS_INSTANCED  op u8, 0x14 u8, count i32, indices u16*, instances i32
 *   CMD_DRAW_ARRAYS_INSTANCED    op u8, count i32, instances i32
 *     (the draw's triangles once per instance, instance ids 0 .. instances-1,
 *     at most 65536; ManyProgram reads instance i's column-major mat4 from
 *     buffer 15 at floats [16i, 16i+16) and is drawn only this way; frames with
 *     instanced draws are not taken by rsrgpu_render_static)
 *   CMD_CLEAR           op u8, bits u8
 *   CMD_STORE_COLOR_FULL_LINEAR_TC  op u8, gamma u8, rsrgpu_truecolor_canvas*
 *   CMD_STORE_DEPTH_FULL_LINEAR_FP  op u8, float* (width*height, row-major)
 *   CMD_STORE_COLOR_FULL_LINEAR_FP  op u8, rsrgpu_fp_canvas* (width x height)
 *   CMD_STORE_COLOR_HALF_LINEAR_FP  op u8, rsrgpu_fp_canvas* (width/2 x height/2)
 *   CMD_STORE_COLOR_FULL_QUADS_FP   op u8, rsrgpu_qfloat4_canvas* (width x height)
 *   CMD_EOF (optional; the stream may simply end)
 *
 * Memory
 * ------
 * Pointers in the stream and in the state snapshots may be device pointers
 * (used in place) or host pointers previously declared with
 * rsrgpu_register_host_buffer().  Host inputs reach the device and host
 * outputs come back inside every rsrgpu_run(), so the caller's buffers keep
 * the reference's meaning of "read when the frame runs".  Pageable memory
 * goes through device mirrors and copies.  Pinned, mapped memory
 * (cudaHostAlloc) is read by a gather kernel, textures are copied while
 * setup and binning run, and outputs are written in place by the kernels.
 *
 * Errors
 * ------
 * Every entry point returns 0 on success and a negative RSRGPU_E* code
 * otherwise; rsrgpu_last_error() gives the message.  The reference
 * terminates the process on the same conditions (std::exit(1) at
 * src/rgl/rglv/rglv_gpu.cxx:202-242,301-431).
 */
#ifndef RSRGPU_H
#define RSRGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- protocol constants (src/rgl/rglv/rglv_gpu_protocol.hxx:7-56) ---- */
#define RSRGPU_CMD_EOF                        0x8d
#define RSRGPU_CMD_STATE                      1
#define RSRGPU_CMD_CLEAR                      10
#define RSRGPU_CMD_DRAW_ELEMENTS              11
#define RSRGPU_CMD_DRAW_ARRAYS                12
#define RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED    13
#define RSRGPU_CMD_DRAW_ARRAYS_INSTANCED      14
#define RSRGPU_CMD_DRAW_INLINE                15
#define RSRGPU_CMD_DRAW_INLINE_INSTANCED      16
#define RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP 20
#define RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP 21
#define RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC 22
#define RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP  23
#define RSRGPU_CMD_STORE_DEPTH_FULL_QUADS_FP  24
#define RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP 25
#define RSRGPU_CMD_CLIPPED_TRI                100
/* Extension of this library (rsr has no deferred path): op u8,
 * rsrgpu_gbuffer*.  Stores the depth buffer and, for pixels whose visible
 * fragment comes from RSRGPU_PROGRAM_GBUFFER, its interpolated normal and
 * albedo; other pixels get normal 0 and albedo 0.  The frame's draws must
 * all use RSRGPU_PROGRAM_GBUFFER without blending and the store must follow
 * them with no other store in between. */
#define RSRGPU_CMD_STORE_GBUFFER              40

/* ---- GL enums (src/rgl/rglv/rglv_gl.hxx:20-62) ---- */
#define RSRGPU_GL_CULL_FACE        1
#define RSRGPU_GL_SCISSOR_TEST     2
#define RSRGPU_GL_BLEND            3
#define RSRGPU_GL_DEPTH_TEST       4
#define RSRGPU_GL_NEAREST_MIPMAP_NEAREST 0
#define RSRGPU_GL_LINEAR_MIPMAP_NEAREST  1
#define RSRGPU_GL_FRONT            1
#define RSRGPU_GL_BACK             2
#define RSRGPU_GL_LESS             0
#define RSRGPU_GL_LEQUAL           1
#define RSRGPU_GL_EQUAL            2
#define RSRGPU_GL_COLOR_BUFFER_BIT 1
#define RSRGPU_GL_DEPTH_BUFFER_BIT 2
#define RSRGPU_HINT_READ4          1
#define RSRGPU_HINT_DENSE          2
#define RSRGPU_RB_COLOR_DEPTH      0
#define RSRGPU_RB_RGBF32           1
#define RSRGPU_RB_RGBAF32          2
#define RSRGPU_RB_F32              3

/* ---- program ids (src/viewer/shaders.hxx, rglv_gpu_shaders.hxx) ---- */
#define RSRGPU_PROGRAM_DEFAULT_POST  1   /* DefaultPostProgram, shaders.hxx:32 */
#define RSRGPU_PROGRAM_EXPOSURE_POST 2   /* ExposurePostProgram, shaders.hxx:40 */
#define RSRGPU_PROGRAM_AMY           4   /* AmyProgram (textured), shaders.hxx:69 */
#define RSRGPU_PROGRAM_MANY          6   /* ManyProgram (instanced: per-instance matrix in buffer 15,
                                            position 0-2, uv 9-10; colour (u, v, uniform 0)),
                                            shaders.hxx:482-585 */
#define RSRGPU_PROGRAM_OBJ1          7   /* OBJ1Program (Gouraud kd lit per vertex by a light at the eye;
                                            position 0-2, normal 3-5, kd 6-8), shaders.hxx:586-699 */
#define RSRGPU_PROGRAM_GOURAUD       90  /* test program: per-vertex rgb, no lighting */
#define RSRGPU_PROGRAM_GBUFFER       91  /* G-buffer program: position 0-2, normal 3-5,
                                            RGBA8 albedo bits (as float) in 6 */

/* ---- error codes ---- */
#define RSRGPU_OK            0
#define RSRGPU_EINVAL       -1   /* bad argument / malformed stream */
#define RSRGPU_ENODISPATCH  -2   /* no program installed for a state key */
#define RSRGPU_ECUDA        -3   /* CUDA runtime error */
#define RSRGPU_ECAPACITY    -4   /* a device capacity was exceeded and could not be grown */
#define RSRGPU_ETIMEOUT     -5   /* rsrgpu_wait() timed out */
#define RSRGPU_EUNSUPPORTED -6   /* a protocol feature this library does not implement */

/* Texture unit binding, mirrors rglv::TextureState (rglv_gl.hxx:64-77).
 * ptr: RGBA float32 pixels (PixelToaster::FloatingPointPixel).  For square
 * power-of-two textures the buffer holds the stacked mip chain built as in
 * rglr::Texture::maybe_make_mipmap (rglr_texture.cxx:33-80): 2*width*width
 * pixels. */
typedef struct rsrgpu_texture_state {
    const float* ptr;
    int32_t width;
    int32_t height;
    int32_t stride;
    int32_t filter;   /* 0 = nearest, 1 = bilinear (GL_LINEAR_MIPMAP_NEAREST) */
} rsrgpu_texture_state;

/* State snapshot, mirrors rglv::GLState (rglv_gl.hxx:80-179).  Matrices are
 * column-major exactly as rmlm::mat4::ff. */
typedef struct rsrgpu_glstate {
    float clear_color[4];
    float clear_depth;
    int32_t clear_stencil;
    int32_t culling_enabled;
    int32_t cull_face;
    int32_t scissor_enabled;
    int32_t scissor_origin[2];
    int32_t scissor_size[2];
    int32_t viewport_origin[2];
    int32_t viewport_size[2];      /* {0,0}: unset (std::nullopt) */
    int32_t blending_enabled;
    int32_t color_write_mask;
    int32_t depth_write_mask;
    int32_t depth_test_enabled;
    int32_t depth_func;
    int32_t program_id;
    int32_t uniforms_ofs;          /* -1: no uniform block */
    int32_t color0_attachment_type;
    int32_t depth_attachment_type;
    int32_t reserved0;
    float uniforms[32];            /* the 32-float uniform block (UNIFORM_BUFFER_SIZE) */
    const float* buffers[16];      /* SoA vertex attribute arrays */
    rsrgpu_texture_state tus[2];
    const float* tu3ptr;
    int32_t tu3dim;
    int32_t reserved1;
    float view_matrix[16];
    float normal_matrix[16];
    float projection_matrix[16];
} rsrgpu_glstate;

/* Output target of CMD_STORE_COLOR_FULL_LINEAR_TC, mirrors
 * rglr::TrueColorCanvas: 0x00RRGGBB pixels, row-major. */
typedef struct rsrgpu_truecolor_canvas {
    uint32_t* data;
    int32_t width;
    int32_t height;
    int32_t stride;   /* in pixels */
    int32_t reserved;
} rsrgpu_truecolor_canvas;

/* Target of CMD_STORE_COLOR_FULL_LINEAR_FP and CMD_STORE_COLOR_HALF_LINEAR_FP,
 * mirrors rglr::FloatingPointCanvas (src/rgl/rglr/rglr_canvas.hxx:488-529):
 * RGBA float pixels (PixelToaster::FloatingPointPixel), row-major, stride in
 * pixels.  The full store writes (r, g, b, 0) per pixel as
 * Copy(QFloat3Canvas|QFloat4Canvas -> FloatingPointCanvas) does
 * (src/rgl/rglr/rglr_algorithm.cxx:192-225,247-280); the half store writes
 * one pixel per 2x2 quad, (((p0 + p1) + p2) + p3) * 0.25 per channel, as
 * Downsample does (rglr_algorithm.cxx:118-168).  The tile interpreter's
 * cases are src/rgl/rglv/rglv_gpu.cxx:345-383.  For the full store the
 * canvas is width x height, for the half store width/2 x height/2; data must
 * be 16-byte aligned. */
typedef struct rsrgpu_fp_canvas {
    float* data;      /* 4 floats per pixel */
    int32_t width;
    int32_t height;
    int32_t stride;   /* in pixels */
    int32_t reserved;
} rsrgpu_fp_canvas;

/* Target of CMD_STORE_COLOR_FULL_QUADS_FP, mirrors rglr::QFloat4Canvas
 * (src/rgl/rglr/rglr_canvas.hxx:228-320): one 64-byte qfloat4 per 2x2 quad,
 * laid out x[4] y[4] z[4] w[4] over the quad's lanes (x,y) (x+1,y) (x,y+1)
 * (x+1,y+1); quads row-major, stride in quads.  x, y, z are the colour; w is
 * 1 for an RB_RGBF32 colour buffer and the depth for RB_COLOR_DEPTH, as
 * Copy(QFloat3Canvas|QFloat4Canvas -> QFloat4Canvas) writes them
 * (src/rgl/rglr/rglr_algorithm.cxx:320-372).  width x height in pixels
 * (the target's size); data must be 16-byte aligned. */
typedef struct rsrgpu_qfloat4_canvas {
    float* data;      /* 16 floats per quad */
    int32_t width;
    int32_t height;
    int32_t stride;   /* in quads */
    int32_t reserved;
} rsrgpu_qfloat4_canvas;

/* G-buffer written by RSRGPU_CMD_STORE_GBUFFER: fp32 NDC depth, the normal
 * as three fp16 planes (IEEE binary16 bits, round to nearest even), and
 * RGBA8 albedo (R in the low byte); all row-major width*height. */
typedef struct rsrgpu_gbuffer {
    float* depth;
    uint16_t* normal_x;
    uint16_t* normal_y;
    uint16_t* normal_z;
    uint32_t* albedo;
    int32_t width;
    int32_t height;
} rsrgpu_gbuffer;

/* Point light of the deferred shader. */
typedef struct rsrgpu_light {
    float position[3];
    float radius;
    float color[3];
    float reserved;
} rsrgpu_light;

/* One clipped vertex as stored by the clipper, mirrors rglv::ClippedVertex
 * (rglv_gpu.hxx:38-40): device coordinate + the program's VertexOutputSD. */
typedef struct rsrgpu_clipped_vertex {
    float coord[4];
    float data[16];
} rsrgpu_clipped_vertex;

/* Per-frame statistics, mirrors rglv::GPUStats (rglv_gpu.hxx:51-62). */
typedef struct rsrgpu_stats {
    int64_t total_tiles;
    int64_t total_tile_records;      /* triangle records over all tile lists */
    int64_t total_clipped_records;
    int64_t max_tile_records;
    int64_t primitives_submitted;
    int64_t primitives_clipped;
    int64_t gpu_launches;            /* kernels launched by the last run */
    int64_t graph_captures;          /* runs captured into a new CUDA graph, since rsrgpu_create */
    int64_t table_uploads;           /* frame-table uploads, since rsrgpu_create */
} rsrgpu_stats;

typedef struct rsrgpu_ctx rsrgpu_ctx;

/* GPU::GPU(concurrency, guid) -- rglv_gpu.cxx:18-24.  device: CUDA ordinal. */
int rsrgpu_create(int device, rsrgpu_ctx** out);
int rsrgpu_destroy(rsrgpu_ctx* ctx);

/* GPU::Install(programId, stateKey, ptrs) -- rglv_gpu.cxx:26-47.  kind:
 * 0 = bin (vertex) program, 1 = draw (fragment) program, 2 = blt program.
 * Fails with RSRGPU_ENODISPATCH when this library has no device implementation
 * of the program for that state key. */
int rsrgpu_install(rsrgpu_ctx* ctx, int program_id, uint32_t state_key, int kind);

/* GPU::Reset(sizeInPixels, tileSizeInBlocks) -- rglv_gpu.cxx:50-56.  Tiles are
 * tile_blocks_x*8 by tile_blocks_y*8 pixels (kBlockDimensionsInPixels,
 * rglv_gpu.hxx:27); width must be a multiple of 4 and height of 2, and tiles
 * at most 128 pixels on a side (the reference's quad stride). */
int rsrgpu_reset(rsrgpu_ctx* ctx, int width, int height, int tile_blocks_x, int tile_blocks_y);

/* Declare a host buffer the stream or a state may point to. */
int rsrgpu_register_host_buffer(rsrgpu_ctx* ctx, const void* host_ptr, size_t bytes);
int rsrgpu_unregister_host_buffer(rsrgpu_ctx* ctx, const void* host_ptr);

/* Hand over one frame's commands (GL::commands_ plus its state deque):
 * GPU::BinImpl's interpretation of the stream (rglv_gpu.cxx:119-260), done on
 * the host.  The decoded tables (states, draws, ops) are uploaded by the next
 * rsrgpu_run(), unless they equal the ones already on the device.  Submit
 * after the previous run has been waited for. */
int rsrgpu_submit(rsrgpu_ctx* ctx, const uint8_t* commands, size_t nbytes,
                  const rsrgpu_glstate* states, int nstates);

/* GPU::Run() -- rglv_gpu.hxx:167, rglv_gpu.cxx:90-116.  Enqueues the frame on
 * `stream` (a cudaStream_t; NULL = the context's own stream).  A run
 * captures its work into a CUDA graph and later runs replay it (inputs are
 * still read when each run executes).  A new submission keeps the graph when
 * the frame has the structure of the one captured -- the same target and
 * tiling, triangle count, table sizes, kernel choices and host-buffer
 * routes -- so a frame re-recorded every time (GPUNode::Main) costs its
 * decode, a table upload when states changed, and a graph launch.  Other
 * submissions, host-buffer (un)registration and capacity growth drop it.
 * A run on a stream the caller is capturing, or one that copies pageable
 * host memory, is enqueued directly. */
int rsrgpu_run(rsrgpu_ctx* ctx, void* stream);

/* Wait for the last run; timeout_ms < 0 waits without limit. */
int rsrgpu_wait(rsrgpu_ctx* ctx, int timeout_ms);

/* Debug/parity access to the bins of the last run.  Tile streams are written
 * in the canonical form shared with the oracle: for each tile (row-major) a
 * u32 byte length followed by the tile's command bytes with every pointer
 * field removed and CMD_STATE carrying a u32 state ordinal.  *needed receives
 * the full size. */
int rsrgpu_dump_tiles(rsrgpu_ctx* ctx, uint8_t* out, size_t capacity, size_t* needed);
int rsrgpu_dump_clipped(rsrgpu_ctx* ctx, rsrgpu_clipped_vertex* out, int capacity, int* count);
int rsrgpu_get_stats(rsrgpu_ctx* ctx, rsrgpu_stats* out);

/* Device timing of the last run (CUDA events in the run's work): total_ms from
 * the frame's start (after any input gather) to the end of the raster pass,
 * raster_ms from the end of binning to the end of the raster pass.  The start
 * marks are recorded on a branch that waits for the run stream's work before
 * them, so no kernel waits for them. */
int rsrgpu_last_timings(rsrgpu_ctx* ctx, float* total_ms, float* raster_ms);

int rsrgpu_last_error(rsrgpu_ctx* ctx, char* buf, size_t len);

/* ---- recording a frame (the producer side) ----
 * A native recorder with rglv::GL's calling surface (src/rgl/rglv/
 * rglv_gl.hxx:182-345, rglv_gl.cxx:13-106), for callers that produce frames
 * without rsr.  State setters change the current state; the next command
 * appends a snapshot of it and emits CMD_STATE with the snapshot's index
 * (GL::MaybeUpdateState, rglv_gl.cxx:100-106), then the command in rsr's byte
 * protocol.  The state starts (and rsrgpu_gl_reset_state() returns to) the
 * defaults of GLState::reset (rglv_gl.hxx:152-179) with RB_COLOR_DEPTH
 * attachments and identity matrices.  rsrgpu_recorder_frame() gives the
 * stream and the snapshots for rsrgpu_submit() or an rsrgpu_frame_desc; the
 * recorder owns them and the canvas / G-buffer descriptors the stream points
 * to (copies of the arguments), valid until the next command,
 * rsrgpu_recorder_reset() or rsrgpu_recorder_destroy().  Buffers, indices
 * and canvas data are the caller's and are referenced, not copied.  No CUDA
 * call is made. */
typedef struct rsrgpu_recorder rsrgpu_recorder;
int rsrgpu_recorder_create(rsrgpu_recorder** out);
int rsrgpu_recorder_destroy(rsrgpu_recorder* rec);
/* GL::Reset: an empty frame and the default state, marked changed, so the
 * next command records a snapshot of the defaults first (rglv_gl.cxx:92-97) */
int rsrgpu_recorder_reset(rsrgpu_recorder* rec);
int rsrgpu_recorder_frame(rsrgpu_recorder* rec, const uint8_t** commands, size_t* nbytes,
                          const rsrgpu_glstate** states, int* nstates);
/* GL::Enable / Disable: RSRGPU_GL_CULL_FACE, _SCISSOR_TEST, _BLEND, _DEPTH_TEST */
int rsrgpu_gl_enable(rsrgpu_recorder* rec, int cap);
int rsrgpu_gl_disable(rsrgpu_recorder* rec, int cap);
/* GL::CullFace, DepthFunc, DepthWriteMask, ColorWriteMask, UseProgram,
 * RenderbufferType(GL_COLOR_ATTACHMENT0 / GL_DEPTH_ATTACHMENT, type) */
#define RSRGPU_GLSTATE_CULL_FACE        1
#define RSRGPU_GLSTATE_DEPTH_FUNC       2
#define RSRGPU_GLSTATE_DEPTH_WRITE_MASK 3
#define RSRGPU_GLSTATE_COLOR_WRITE_MASK 4
#define RSRGPU_GLSTATE_PROGRAM          5
#define RSRGPU_GLSTATE_COLOR_ATTACHMENT 6
#define RSRGPU_GLSTATE_DEPTH_ATTACHMENT 7
int rsrgpu_gl_state_int(rsrgpu_recorder* rec, int what, int value);
int rsrgpu_gl_scissor(rsrgpu_recorder* rec, int x, int y, int width, int height);
int rsrgpu_gl_viewport(rsrgpu_recorder* rec, int x, int y, int width, int height);
/* the state's uniform block: up to 32 floats (the rest zero) */
int rsrgpu_gl_use_uniforms(rsrgpu_recorder* rec, const float* values, int n);
int rsrgpu_gl_bind_texture(rsrgpu_recorder* rec, int unit, const float* texels, int width, int height, int stride,
                           int filter);
/* GL::UseBuffer(slot, float*): slots 0..15 (a Float3Array is three slots) */
int rsrgpu_gl_use_buffer(rsrgpu_recorder* rec, int slot, const float* data);
int rsrgpu_gl_clear_color(rsrgpu_recorder* rec, float red, float green, float blue);
int rsrgpu_gl_clear_depth(rsrgpu_recorder* rec, float depth);
/* GL::ViewMatrix, ProjectionMatrix, NormalMatrix: column-major mat4 */
#define RSRGPU_GLMATRIX_VIEW       0
#define RSRGPU_GLMATRIX_PROJECTION 1
#define RSRGPU_GLMATRIX_NORMAL     2
int rsrgpu_gl_matrix(rsrgpu_recorder* rec, int which, const float m[16]);
/* GL::ResetX */
int rsrgpu_gl_reset_state(rsrgpu_recorder* rec);
/* commands (rglv_gl.cxx:13-89); stride 0 = width (quads: width / 2) */
int rsrgpu_gl_clear(rsrgpu_recorder* rec, int bits);
int rsrgpu_gl_draw_elements(rsrgpu_recorder* rec, int count, const uint16_t* indices, int hint);
int rsrgpu_gl_draw_arrays(rsrgpu_recorder* rec, int count);
int rsrgpu_gl_draw_elements_instanced(rsrgpu_recorder* rec, int count, const uint16_t* indices, int instances);
int rsrgpu_gl_draw_arrays_instanced(rsrgpu_recorder* rec, int count, int instances);
int rsrgpu_gl_store_color_tc(rsrgpu_recorder* rec, uint32_t* data, int width, int height, int stride, int gamma);
int rsrgpu_gl_store_color_fp(rsrgpu_recorder* rec, float* data, int width, int height, int stride, int downsample);
int rsrgpu_gl_store_color_quads(rsrgpu_recorder* rec, float* data, int width, int height, int stride);
int rsrgpu_gl_store_depth(rsrgpu_recorder* rec, float* data);
int rsrgpu_gl_store_gbuffer(rsrgpu_recorder* rec, const rsrgpu_gbuffer* gbuffer);

/* ---- GL call scripts and the perf harness ----
 * A frame's rglv::GL calls as data: one rsrgpu_gl_call per rsrgpu_gl_* call,
 * with that call's arguments (integers in i[], the pointer in p, floats --
 * colours, depth, matrix, uniforms -- in f[]):
 *   ENABLE/DISABLE i0=cap; STATE_INT i0=what i1=value; SCISSOR/VIEWPORT
 *   i0..i3; USE_UNIFORMS i0=n f; BIND_TEXTURE i0=unit p i1=width i2=height
 *   i3=stride i4=filter; USE_BUFFER i0=slot p; CLEAR_COLOR f0..f2;
 *   CLEAR_DEPTH f0; MATRIX i0=which f0..f15; RESET_STATE; CLEAR i0=bits;
 *   DRAW_ELEMENTS i0=count p i1=hint; DRAW_ARRAYS i0=count;
 *   DRAW_ELEMENTS_INSTANCED i0=count p i1=instances; DRAW_ARRAYS_INSTANCED
 *   i0=count i1=instances; STORE_COLOR_TC p i0=width i1=height i2=stride
 *   i3=gamma; STORE_COLOR_FP p i0..i2 i3=downsample; STORE_COLOR_QUADS p
 *   i0..i2; STORE_DEPTH p; STORE_GBUFFER p=rsrgpu_gbuffer*.
 * rsrgpu_gl_play() makes the calls on a recorder, in order, and stops at the
 * first that fails (its status is returned). */
#define RSRGPU_CALL_ENABLE                  1
#define RSRGPU_CALL_DISABLE                 2
#define RSRGPU_CALL_STATE_INT               3
#define RSRGPU_CALL_SCISSOR                 4
#define RSRGPU_CALL_VIEWPORT                5
#define RSRGPU_CALL_USE_UNIFORMS            6
#define RSRGPU_CALL_BIND_TEXTURE            7
#define RSRGPU_CALL_USE_BUFFER              8
#define RSRGPU_CALL_CLEAR_COLOR             9
#define RSRGPU_CALL_CLEAR_DEPTH             10
#define RSRGPU_CALL_MATRIX                  11
#define RSRGPU_CALL_RESET_STATE             12
#define RSRGPU_CALL_CLEAR                   13
#define RSRGPU_CALL_DRAW_ELEMENTS           14
#define RSRGPU_CALL_DRAW_ARRAYS             15
#define RSRGPU_CALL_DRAW_ELEMENTS_INSTANCED 16
#define RSRGPU_CALL_DRAW_ARRAYS_INSTANCED   17
#define RSRGPU_CALL_STORE_COLOR_TC          18
#define RSRGPU_CALL_STORE_COLOR_FP          19
#define RSRGPU_CALL_STORE_COLOR_QUADS       20
#define RSRGPU_CALL_STORE_DEPTH             21
#define RSRGPU_CALL_STORE_GBUFFER           22
typedef struct rsrgpu_gl_call {
    int32_t fn;
    int32_t i[7];
    uint64_t p;
    float f[32];
} rsrgpu_gl_call;
int rsrgpu_gl_play(rsrgpu_recorder* rec, const rsrgpu_gl_call* calls, int ncalls);

/* rsr's perf harness (src/viewer/perf.cxx:200-244: priming frames, then
 * timed frames, each GPUNode::Main's work, src/viewer/node/gpu.cxx:107-146)
 * through this library: per frame rsrgpu_reset(target), rsrgpu_recorder_reset,
 * rsrgpu_gl_play(calls), rsrgpu_submit, rsrgpu_run(stream), rsrgpu_wait.
 * frame_ms[k] receives the host's steady-clock time of timed frame k, from
 * the reset to the end of the wait.  The first failing call ends the loop
 * and its status is returned. */
typedef struct rsrgpu_perf_target {
    int width, height, tile_blocks_x, tile_blocks_y;
} rsrgpu_perf_target;
int rsrgpu_perf_frames(rsrgpu_ctx* ctx, rsrgpu_recorder* rec, const rsrgpu_perf_target* target,
                       const rsrgpu_gl_call* calls, int ncalls, int priming, int frames, void* stream,
                       double* frame_ms);

/* ---- texture upload and mip chain on the device ----
 * rglr::Texture's layout (src/rgl/rglr/rglr_texture.hxx:10-33): RGBA float
 * texels (16 bytes, PixelToaster::FloatingPointPixel), row-major with stride
 * width.  A square power-of-two texture of edge w <= 4096 gets the mip chain
 * Texture::maybe_make_mipmap builds (src/rgl/rglr/rglr_texture.cxx:33-80):
 * w*w*2 texels, level k (edge w >> k) in rows [2w - 2(w >> k), 2w - (w >> k))
 * and columns [0, w >> k), every other texel of rows [w, 2w) zero; a level-k
 * texel is (((a + b) + c) + d) / 4 of its 2x2 parents in level k-1, in
 * row-major order.  Other sizes get no chain (power -1), as in the
 * reference.  All pointers are device pointers; the work is enqueued on
 * `stream` (NULL = the context's stream) and the call returns without
 * waiting. */
#define RSRGPU_TEXTURE_MAX_EDGE 4096

/* PNGToTexture's conversion of decoded RGBA8 pixels
 * (src/rgl/rglr/rglr_texture_load.cxx:40-63): r, g, b through
 * ryg::srgb8_to_float, alpha / 255, rgb multiplied by alpha when
 * `premultiply`; then the mip chain above.  rgba8: width*height*4 bytes,
 * 4-byte aligned.  texels: 16-byte aligned, room for 2*width*height texels
 * when a chain is built, else width*height.  *power (may be NULL) receives
 * Texture::pow: log2(width), or -1 without a chain. */
int rsrgpu_texture_from_rgba8(rsrgpu_ctx* ctx, const uint8_t* rgba8, int width, int height, int premultiply,
                              float* texels, size_t texel_capacity, int* power, void* stream);

/* Texture::maybe_make_mipmap on a float texture already on the device (level
 * 0 in texels[0 .. width*height)), for example a frame stored there by
 * CMD_STORE_COLOR_FULL_LINEAR_FP as rsr's render-to-texture node does
 * (src/viewer/node/rendertotexture.cxx:64-95).  Without a chain (power -1)
 * nothing is written. */
int rsrgpu_texture_mipmap(rsrgpu_ctx* ctx, float* texels, int width, int height, size_t texel_capacity,
                          int* power, void* stream);

/* ---- post-processing of float canvases (rsr's $kawase and $glow nodes) ----
 * Device pointers; enqueued on `stream` (NULL = the context's stream).
 *
 * KawaseBlurFilter (src/rgl/rglr/rglr_kawase.cxx:22-84) over the whole
 * canvas: dst(x, y) = (((+0 + S(x-d-1, y-d-1)) + S(x+d, y-d-1)) + S(x-d-1, y+d))
 * + S(x+d, y+d), times 1/16, per channel (RGBA), where S(u, v) is the box sum
 * ((p(u,v) + p(u+1,v)) + p(u,v+1)) + p(u+1,v+1) of source pixels with
 * coordinates clamped to the source.  src and dst are float canvases of the
 * same size (16-byte aligned, stride >= width) that do not overlap. */
int rsrgpu_kawase_blur(rsrgpu_ctx* ctx, const rsrgpu_fp_canvas* src, const rsrgpu_fp_canvas* dst, int dist,
                       void* stream);

/* The $kawase node's chain (src/viewer/node/kawase.cxx:79-117): `intensity`
 * passes with distances 0, 1, ..., the first from src into tmp_a, then
 * alternating tmp_a -> tmp_b -> tmp_a ...  *result (may be NULL) names the
 * canvas holding the result: 0 src (intensity 0), 1 tmp_a, 2 tmp_b. */
int rsrgpu_kawase_chain(rsrgpu_ctx* ctx, const rsrgpu_fp_canvas* src, const rsrgpu_fp_canvas* tmp_a,
                        const rsrgpu_fp_canvas* tmp_b, int intensity, int* result, void* stream);

/* The $glow node's resolve, rglr::Filter<GlowShader, sRGB|LinearColor>
 * (src/rgl/rglr/rglr_algorithm.hxx:107-144, shader src/viewer/node/
 * glow.cxx:24-36): per output pixel (image + blur * 0.7) * 0.5 per channel,
 * image the pixel's lane of the full-size quads canvas (x, y, z), blur the
 * half-size canvas pixel under its quad; packed to 0x00RRGGBB with the
 * sRGB8 encoder of the TrueColor stores (srgb != 0: within 1/255 of rsr's
 * table encoder) or to_tc_basic's truncation (srgb == 0: bit-exact).  The
 * image is width x height (width a multiple of 4, height of 2), the blur
 * canvas at least width/2 x height/2, the output width x height with an
 * even stride. */
int rsrgpu_glow(rsrgpu_ctx* ctx, const rsrgpu_qfloat4_canvas* image, const rsrgpu_fp_canvas* blur,
                const rsrgpu_truecolor_canvas* out, int srgb, void* stream);

/* ---- deferred shading (extension; no counterpart in rsr) ----
 * Plain multi-light Blinn-Phong over a G-buffer: for each pixel with albedo
 * != 0, world position from depth through inv_view_proj (column-major), then
 * for every light closer than its radius: att = (1 - d/r)^2, diffuse
 * max(N.L, 0) * albedo, specular max(N.H, 0)^32, summed and packed to sRGB8
 * (0x00RRGGBB) into out_srgb and/or as linear RGB float triples into
 * out_linear (either may be NULL).  Pixels with albedo 0 get
 * `background` (linear RGB).  All pointers are device pointers; the call is
 * enqueued on `stream`. */
int rsrgpu_shade_plain(rsrgpu_ctx* ctx, const rsrgpu_gbuffer* gbuffer, const float inv_view_proj[16],
                       const float eye[3], const rsrgpu_light* lights, int nlights,
                       const float background[3], uint32_t* out_srgb, float* out_linear, void* stream);

/* ---- learned deferred shader (extension; no counterpart in rsr) ----
 * MLP 24 -> 64 -> 64 -> 64 -> 3 with ReLU, BF16 weights and activations,
 * FP32 accumulation, run on tcgen05 tensor cores.  Weights are row-major
 * [out][in] BF16 with the input padded to 32 columns and the output layer to
 * 16 rows (padding must be zero); biases FP32.  Device pointers. */
typedef struct rsrgpu_mlp {
    const uint16_t* w1;   /* [64][32] */
    const uint16_t* w2;   /* [64][64] */
    const uint16_t* w3;   /* [64][64] */
    const uint16_t* w4;   /* [16][64] */
    const float* b1;      /* [64] */
    const float* b2;      /* [64] */
    const float* b3;      /* [64] */
    const float* b4;      /* [16] */
} rsrgpu_mlp;

/* out[n][3] = MLP(features[n][32]) with BF16 features (columns 24..31 zero). */
int rsrgpu_mlp_forward(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp, const uint16_t* features, int n,
                       float* out, void* stream);

/* Gradient of the mean squared error of one batch.  Sample rows
 * index[0..batch) of features[.][32] (BF16) against targets[.][3] (FP32).
 * grad receives RSRGPU_MLP_PARAMS floats laid out w1 | w2 | w3 | w4 | b1 |
 * b2 | b3 | b4 (row-major [out][in], padded shapes as in rsrgpu_mlp); loss
 * receives the batch's sum of squared errors.  Both are zeroed here.  The
 * forward and backward GEMMs run on tcgen05 tensor cores. */
#define RSRGPU_MLP_WEIGHTS 11264
#define RSRGPU_MLP_PARAMS  11472
int rsrgpu_mlp_grad(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp, const uint16_t* features, const float* targets,
                    int nsamples, const int32_t* index, int batch, float* grad, float* loss, void* stream);

/* Adam step on FP32 master parameters (same layout as the gradient); writes
 * the BF16 weights (RSRGPU_MLP_WEIGHTS values, the layout rsrgpu_mlp points
 * into) and the FP32 biases. */
int rsrgpu_mlp_adam(rsrgpu_ctx* ctx, float* params, const float* grad, float* m, float* v, int step,
                    float lr, uint16_t* weights_bf16, float* biases, void* stream);

/* ---- learned deferred shading, fused (extension; no counterpart in rsr) ----
 * The G-buffer is shaded in 32x32-pixel tiles.  Per tile: the 8 candidate
 * lights with the largest bound on their contribution to the tile's
 * world-space box; per covered pixel (albedo != 0) 24 features: unit normal,
 * unit view vector, albedo, eye distance / 50, and a summary of the candidate
 * lights reaching the pixel (sum of colour * att, sum of w L, the six
 * entries of sum w L L^T, sum of w max(N.L, 0), mean d/r weighted by w, with
 * att = (1 - d/r)^2 and w the colour sum of colour * att).  The output is
 * rgb = max(MLP(features) + base, 0)^2 per channel, where base is the square
 * root of an analytic estimate from the same features (Blinn-Phong of one
 * virtual light with direction sum w L and colour sum colour * att, plus
 * ambient); with a zero output layer the shader is that estimate.  The gate shades min(16, covered) sample
 * pixels of the tile (its 4x4 grid of pixels (8i+4, 8j+4) first) with the
 * plain shader; if the mean squared difference of learned and plain sRGB8
 * values over the samples exceeds max_tile_mse (8-bit units squared; 6.5 is
 * 40 dB), the tile is shaded by the plain shader, bit-exact with
 * rsrgpu_shade_plain.  A negative max_tile_mse shades every tile plain,
 * INFINITY none.  tile_status (optional, one byte per tile in row-major
 * order): 0 learned, 1 plain, 2 nothing covered; tile_mse (optional) the
 * gate's estimate.  All pointers are device pointers; the call is enqueued
 * on `stream` and returns without waiting (it may be captured into a CUDA
 * graph).  A tensor-core stall is reported by the next
 * rsrgpu_shade_learned_check(); after graph replays, synchronise their
 * stream before that check. */
#define RSRGPU_SHADE_TILE 32
int rsrgpu_shade_learned(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp, const rsrgpu_gbuffer* gbuffer,
                         const float inv_view_proj[16], const float eye[3], const rsrgpu_light* lights, int nlights,
                         const float background[3], float max_tile_mse, uint32_t* out_srgb, float* out_linear,
                         uint8_t* tile_status, float* tile_mse, void* stream);

/* Waits for the work rsrgpu_shade_learned() enqueued and returns
 * RSRGPU_ETIMEOUT if a tensor-core wait expired in any call since the last
 * check (the affected tiles were left unwritten), else 0. */
int rsrgpu_shade_learned_check(rsrgpu_ctx* ctx);

/* Test hooks for the failure paths that a healthy GPU never takes.
 * RSRGPU_DEBUG_LEARNED_STALL, value = polls > 0: in the following
 * rsrgpu_shade_learned() calls the tensor-core kernel's producer threads
 * issue no copy (so no MMA either), and every pipeline wait gives up after
 * `value` polls; the kernel then raises its error flag, frees its tensor
 * memory and returns, and rsrgpu_shade_learned_check() reports
 * RSRGPU_ETIMEOUT.  value 0 restores normal operation.  No fault, trap or
 * endless wait is involved. */
#define RSRGPU_DEBUG_LEARNED_STALL 1
int rsrgpu_set_debug(rsrgpu_ctx* ctx, int knob, int value);

/* The learned shader's inputs and training targets for every pixel:
 * features[W*H][32] BF16 (columns 24..31 and uncovered rows zero), targets
 * (optional) [W*H][3] = sqrt(max(plain linear RGB, 0)) - base, the network's
 * training target (zero rows where uncovered), candidates (optional) [tiles][8] light indices (-1 pads).
 * Device pointers; synchronous. */
int rsrgpu_learned_features(rsrgpu_ctx* ctx, const rsrgpu_gbuffer* gbuffer, const float inv_view_proj[16],
                            const float eye[3], const rsrgpu_light* lights, int nlights, uint16_t* features,
                            float* targets, int32_t* candidates, void* stream);

/* ---- batched frames (extension; no counterpart in rsr) ----
 * Many independent frames rendered by one kernel chain: one launch of the
 * setup kernel, one of the binning kernel and one raster launch per CTA
 * shape cover every frame of the batch; the chain, with one upload of all
 * frames' decoded tables and one read-back of their counters, is captured
 * once in a CUDA graph and replayed by rsrgpu_batch_run().  Each frame is
 * rsr's byte stream as for rsrgpu_submit() with its own target size and
 * tiling (float colour stores, instanced and OBJ1Program draws included);
 * every pointer it holds must be a device pointer.  A frame's results equal
 * those of rsrgpu_submit()/rsrgpu_run() on a context reset to the same size
 * and tiling.  Each raster launch is a persistent grid taking the blocks of
 * all its frames from one device work queue, heaviest tiles first. */
#define RSRGPU_MAX_BATCH 64
typedef struct rsrgpu_batch rsrgpu_batch;
typedef struct rsrgpu_frame_desc {
    const uint8_t* commands;
    size_t nbytes;
    const rsrgpu_glstate* states;
    int nstates;
    int width, height;
    int tile_px;           /* tile edge in pixels: 8, 16, ..., 128 (a multiple of 8) */
    int region_px;         /* raster CTA region edge: 8, 16 or 32 (0: min(tile, 32)) */
    uint32_t bin_capacity; /* tile-list entries to reserve (0: default; grows on overflow) */
} rsrgpu_frame_desc;

int rsrgpu_batch_create(int device, rsrgpu_batch** out);
int rsrgpu_batch_destroy(rsrgpu_batch* batch);
/* as rsrgpu_install(), for every frame of the batch */
int rsrgpu_batch_install(rsrgpu_batch* batch, int program_id, uint32_t state_key, int kind);
/* decodes up to RSRGPU_MAX_BATCH frames, sizes their scratch and captures the
 * graph; a frame with a float colour store (CMD_STORE_COLOR_*_FP) fails with
 * RSRGPU_EUNSUPPORTED (render it with rsrgpu_run) */
int rsrgpu_batch_submit(rsrgpu_batch* batch, const rsrgpu_frame_desc* frames, int nframes);
/* replays the captured graph on `stream` (NULL: the batch's own stream) */
int rsrgpu_batch_run(rsrgpu_batch* batch, void* stream);
/* waits for the run; a frame whose clip staging or tile lists overflowed is
 * regrown and the batch re-captured and run again (as rsrgpu_wait) */
int rsrgpu_batch_wait(rsrgpu_batch* batch, int timeout_ms);
/* device time of the last run (CUDA events around the graph launch) */
int rsrgpu_batch_last_ms(rsrgpu_batch* batch, float* ms);
/* the context holding frame i after a run: rsrgpu_get_stats(),
 * rsrgpu_dump_tiles() and rsrgpu_dump_clipped() read that frame */
int rsrgpu_batch_frame(rsrgpu_batch* batch, int i, rsrgpu_ctx** ctx);
/* Autotuner: for each frame, renders it alone with every candidate tiling
 * (tile 8/16/32/64 px, raster region 8/16/32 px; tilings whose tile lists
 * exceed the device capacity are skipped) `reps` times, keeps the
 * fastest median device time, and sizes its tile-list capacity from the
 * entries the frame used (plus a quarter).  Frames of the same size whose
 * triangle counts fall in the same power of two reuse a measured tiling
 * (one run of the frame then sizes its capacity).  These choices start a
 * search on the whole batch's time (a small frame timed alone is mostly
 * launch latency, which the batch shares): the default 32/32 tiling
 * everywhere, then, one resolution class at a time, every candidate tiling
 * for all frames of the class, each kept when the batch runs faster; the
 * capacities come from a run of the final tilings.
 * Writes tile_px, region_px and bin_capacity into frames[] (the commands
 * are rendered, so their outputs are written too). */
int rsrgpu_batch_tune(rsrgpu_batch* batch, rsrgpu_frame_desc* frames, int nframes, int reps);
int rsrgpu_batch_last_error(rsrgpu_batch* batch, char* buf, size_t len);

/* ---- rendering without any device allocation ----
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc (for example a host framework that owns all
 * device memory through its own pool, or a real-time loop that must never
 * allocate): it renders one frame through the same kernels as rsrgpu_run()
 * but keeps all frame scratch in one fixed file-scope device array of
 * RSRGPU_STATIC_SCRATCH_BYTES (about 7 MiB) that every GPU loading this
 * library holds until the process exits.  Inputs and outputs must be device
 * pointers; there is no context and no host staging.  The first call on a
 * device sets the array up (symbol address lookup and two synchronous table
 * uploads, under a lock, so first calls from several host threads are safe),
 * so make it before any stream capture; the address it caches does not
 * survive cudaDeviceReset().  Calls share the array
 * (the counters that must start at zero are cleared on every call), so
 * calls that overlap on the GPU race: serialise them.  The call returns once
 * the frame has finished on `stream` (a cudaStream_t, NULL = legacy stream);
 * frames larger than the limits below fail with RSRGPU_ECAPACITY and the
 * reason in errbuf (may be NULL). */
#define RSRGPU_STATIC_MAX_TRIANGLES    32768
#define RSRGPU_STATIC_MAX_TILES        8192
#define RSRGPU_STATIC_MAX_TILE_ENTRIES 524288
#define RSRGPU_STATIC_MAX_CLIP_VERTS   16384
#define RSRGPU_STATIC_MAX_STATES       64
#define RSRGPU_STATIC_MAX_DRAWS        256
#define RSRGPU_STATIC_MAX_OPS          1024
#define RSRGPU_STATIC_SCRATCH_BYTES    7374592
int rsrgpu_render_static(const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates,
                         int width, int height, int tile_blocks_x, int tile_blocks_y, void* stream,
                         char* errbuf, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* RSRGPU_H */
