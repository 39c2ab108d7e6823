// rsrgpu_internal.h -- device-side data layout shared by the host runtime
// (rsrgpu_host.cu) and the kernels (rsrgpu_kernels.cu).
//
// One frame in HBM:
//   DevState[nstates]   decoded GLState snapshots (matrices premultiplied on
//                       the host in the reference's float order)
//   DevDraw[ndraws]     draws in submission order; triangles are numbered
//                       globally g = draw.first_tri + t
//   TriRecord[ntris]    per-triangle setup (fixed-point device coords, z/w,
//                       varyings) in the reference's post-swap vertex order
//   bin_rect[ntris]     u16x4 tile rectangle used for binning (union of the
//                       inline rectangle and the clipped fans' rectangles)
//   chunk/super rects   hierarchy over 32 / 1024 consecutive triangles
//   ClipPoly/ClipVert   clipped polygons (staging order) for clip-source tris
//   tile lists          per tile: ordered inline triangle ids and ordered
//                       clipped fan-triangle ids
#pragma once
#include <cstdint>
#include <vector>

namespace rsrgpu {

constexpr int kMaxVary = 4;
constexpr int kChunk = 32;        // triangles per chunk (one warp)
constexpr int kSuper = 1024;      // triangles per super-chunk
constexpr int kSetupBlock = 256;
constexpr int kMaxClipVerts = 8;  // 3 + one per clipping plane (5 planes)
constexpr int kRegionPx = 32;     // default raster region: a CTA covers at most 32x32 px of one tile
constexpr int kBinBlock = 256;    // bin CTA: one tile, eight warps
constexpr int kMaxBatch = 64;     // frames per batched launch
constexpr int kRasterBatch = 256; // triangles set up per shared-memory batch
constexpr int kOpCache = 64;      // frame ops a raster CTA keeps in shared memory

enum ProgramId : int32_t {
    kProgDefaultPost = 1,
    kProgExposurePost = 2,
    kProgAmy = 4,
    kProgMany = 6,        // ManyProgram (src/viewer/shaders.hxx:482-585): per-instance matrix, uv, magic
    kProgOBJ1 = 7,
    kProgGouraud = 90,
    kProgGBuffer = 91,
};

struct DevTexture {
    const float* buf;
    int32_t kind;   // 0 nearest-mip, 1 linear-mip, 2 non-pow2 nearest
    int32_t power;
    int32_t width, height, stride;
    int32_t texels;   // RGBA texels addressable from buf
};

struct DevState {
    float vpm[16];
    float DS[2], DO[2];
    float guard;
    int32_t scissor[4];   // left, top, right, bottom (GPU::ScissorRect; the whole target when the test is off)
    int32_t scissor_test; // GL_SCISSOR_TEST: draws are cut to scissor[] in the raster pass
    int32_t program;
    int32_t nvary;
    int32_t keep_backs, keep_fronts;
    int32_t cull_enabled, cull_face;
    int32_t depth_test, depth_func, depth_write, color_write, blend;
    int32_t color_type, depth_type;
    float clear_color[4];
    float clear_depth;
    const float* buffers[16];
    int32_t buffer_len[16];   // floats readable from each buffer pointer
    DevTexture tu0;
    float uniforms[32];
};

struct DevDraw {
    int32_t state;
    int32_t first_tri;
    int32_t ntris;
    int32_t is_arrays;
    const uint16_t* indices;
};

// Every kind from kOpStoreTC on is a store; all but kOpStoreDepth read colour.
// The FP stores: rsr's CMD_STORE_COLOR_FULL_LINEAR_FP (kOpStoreFP),
// CMD_STORE_COLOR_HALF_LINEAR_FP (kOpStoreHalfFP) and
// CMD_STORE_COLOR_FULL_QUADS_FP (kOpStoreQuadsFP).
// Per draw of a frame that needs the extended setup (setup_ext_kernel):
// instanced draws (CMD_DRAW_*_INSTANCED), whose triangles are numbered
// instance by instance, g = first_tri + iid * per_inst + t, and OBJ1Program
// draws, which light vertices in view space.
struct DevDrawExt {
    const float* matrices;   // buffers[15]: one column-major mat4 per instance (ManyProgram)
    int32_t per_inst;        // triangles per instance; 0: not instanced
    int32_t ninst;
    float vm[16];            // the draw state's view matrix (OBJ1Program)
};

enum OpKind : int32_t { kOpState = 0, kOpClear = 1, kOpDraw = 2, kOpStoreTC = 3, kOpStoreDepth = 4, kOpStoreGBuffer = 5,
                        kOpStoreFP = 6, kOpStoreHalfFP = 7, kOpStoreQuadsFP = 8 };
__host__ __device__ inline bool op_is_store(int32_t kind) { return kind >= kOpStoreTC; }

// device addresses of one G-buffer target (RSRGPU_CMD_STORE_GBUFFER)
struct GBufferDesc {
    float* depth;
    uint16_t* nx;
    uint16_t* ny;
    uint16_t* nz;
    uint32_t* albedo;
};

struct FrameOp {
    int32_t kind;
    int32_t arg;      // state index / clear bits / draw index / gamma
    int32_t ordinal;  // state ordinal for the canonical dump
    int32_t pad;
    void* ptr;        // output base (device address)
    int32_t width, height, stride, pad2;
    // What the raster pass needs of the op without another load (filled by
    // the host decode): kOpState info[0] program, info[1] kFrag* flags;
    // kOpClear val = clear colour rgb and depth, info[2] 1 for RB_COLOR_DEPTH;
    // kOpDraw info[0] first triangle, info[1] triangles, info[2] state.
    int32_t info[4];
    float val[4];
};
// kOpState info[1]: the fragment stage's switches
constexpr int32_t kFragDepthTest = 1, kFragDepthFuncShift = 1, kFragDepthWrite = 8, kFragColorWrite = 16,
                  kFragBlend = 32, kFragScissor = 64;

struct TriRecord {        // 96 bytes, 16-byte aligned
    int32_t fx[3], fy[3];
    float z[3], w[3];
    float vary[3][kMaxVary];
};

struct ClipVert {         // clipped vertex: device coord + varyings
    float coord[4];
    float vary[kMaxVary];
};

struct ClipInfo {         // per source triangle (valid when nverts > 0)
    int32_t vbase;        // staging index of the polygon's first vertex
    int32_t nverts;       // polygon vertex count (0: not clipped or culled away)
    int32_t backfacing;
    int32_t pad;
};

// frame-global counters, cleared at the start of every run
// Tiles go to the raster pass heaviest first (rsr sorts its tile jobs by
// stream length, rglv_gpu.cxx:100-104): binning files each tile's raster
// blocks in the bucket of its list length's power of two, the raster CTAs
// take work items from a counter, highest bucket first.  In a batch the
// items of a raster launch run frame by frame, each frame's heaviest first.
constexpr int kCostBuckets = 16;

struct FrameCounters {
    uint32_t clip_verts;      // staging vertices allocated
    uint32_t bin_used;        // tile-list entries allocated
    uint32_t overflow;        // bit 0: clip staging, bit 1: bin pool, bit 2: vertex index out of range
    uint32_t next_item;       // raster work items taken (the frame's, or in a batch the launch's)
    uint32_t bucket[kCostBuckets];   // the frame's raster blocks filed per cost bucket
};

struct TileBin {
    uint32_t inl_off, inl_cnt;
    uint32_t clip_off, clip_cnt;
};

struct FrameView {
    const DevState* states;
    const DevDraw* draws;
    int32_t ndraws;
    int32_t ntris;
    const FrameOp* ops;
    int32_t nops;
    const GBufferDesc* gbufs;
    int32_t width, height;
    int32_t tile_w, tile_h, tiles_x, tiles_y, ntiles;
    int32_t nchunks, nsupers;
    TriRecord* tris;
    uint64_t* bin_rect;       // tx0 | ty0<<16 | tx1<<32 | ty1<<48; empty when tx0 > tx1
    uint32_t* rec16;          // 2 words per tri: (i0|bf) | i1<<16, i2
    int4* chunk_rect;
    int4* super_rect;         // (minx, miny, -maxx, -maxy), atomically reduced
    ClipInfo* clip_info;
    ClipVert* clip_verts;
    int32_t* clip_poly;       // per staging vertex: polygon base
    int32_t* clip_src;        // per staging vertex: source triangle (valid at the base)
    uint64_t* clip_fan_rect;  // per staging vertex v (fan apex index), tile rect of fan (base, v, v+1)
    uint32_t clip_cap;
    TileBin* bins;
    uint32_t* bin_pool;
    uint32_t bin_cap;
    FrameCounters* counters;
    const uint32_t* rcp_table;
    const uint8_t* srgb_lut;
    int32_t region_px;        // raster CTA region edge (8, 16 or 32 px; at most the tile)
    int32_t vis_keys;         // 0, or 1 + the depth function (LESS / LEQUAL) of a frame whose draws
                              // are all opaque with depth test and write on (see raster_body)
    int32_t raster_phase;     // 0 the whole raster pass; for vis_keys frames split in two launches:
                              // 1 visibility (owners and depths into vis_own / vis_dep), 2 the rest
    uint32_t* vis_own;        // [height * width] per pixel, phases 1 and 2
    float* vis_dep;
    int32_t ext;              // float colour stores or ManyProgram draws: raster_ext_kernel runs the frame
    int32_t any_scissor;      // a draw of the frame has the scissor test on
    int32_t keys_resume_op;   // vis_keys frames: the first op after the last draw (0: not given)
    int32_t keys_resume_state_op; // the last state op before it
    FrameCounters* host_counters; // pinned host copy of *counters, written by the raster pass (or null)
    uint32_t* tile_queue;     // [kCostBuckets][queue_cap] the frame's raster blocks by cost bucket
                              // (counts in counters->bucket); null: CTA b draws block b
    uint32_t queue_cap;       // the frame's raster blocks
    FrameCounters* taken;     // next_item of the raster launch: the frame's counters, or its batch launch's
    int32_t slices;           // visibility launch: CTAs sharing each raster block's tile list (1: one)
    unsigned long long* slice_keys;   // slices > 1: the blocks' merged (depth, order) keys, one per pixel
    uint32_t* slice_done;     // slices > 1: per raster block, the slices that have merged their keys
    const DevDrawExt* dext;   // per draw, for frames with instanced or OBJ1Program draws (setup_ext_kernel); else null
};

// Copies of up to kMaxGather byte ranges in one launch (inputs from pinned,
// mapped host memory into their device mirrors).
constexpr int kMaxGather = 64;
// Copies of gather_kernel: range r is rows[r] rows (0 counts as 1) of
// bytes[r] bytes, pitch[r] bytes apart in both source and destination
// (rows > 1: 16-byte aligned ends and pitch).
struct GatherList {
    int n;
    const uint8_t* src[kMaxGather];
    uint8_t* dst[kMaxGather];
    size_t bytes[kMaxGather];
    uint32_t rows[kMaxGather];
    uint32_t pitch[kMaxGather];
};

// One launch of a stage over many frames: block b belongs to frame f when
// start[f] <= b < start[f + 1]; passed as a __grid_constant__ parameter.
struct BatchLaunch {
    int32_t nframes;
    int32_t start[kMaxBatch + 1];
    FrameView fv[kMaxBatch];
};

// the sRGB8 encode table the raster pass stores through (26 624 entries; the
// context path and rsrgpu_render_static upload the same table)
void build_srgb_lut(std::vector<uint8_t>& lut);

}  // namespace rsrgpu
