// rsrgpu_host.cu -- host runtime behind include/rsrgpu.h.
//
// Replaces the host half of rglv::GPU (src/rgl/rglv/rglv_gpu.cxx): program
// installation, Reset/Retile, the command interpreter of BinImpl (here it only
// decodes the stream into device tables: states, draws and the frame's op
// list, since state/clear/store commands are identical for every tile), and
// RunImpl, which becomes a fixed sequence of stream-ordered device work:
//   H2D of host inputs -> memset(counters) -> setup -> bin -> raster -> D2H.
// Errors are reported as status codes instead of std::exit(1).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_internal.h"

namespace rsrgpu {
cudaError_t launch_frame_init(const FrameView& fv, cudaStream_t st);
cudaError_t launch_setup(const FrameView& fv, cudaStream_t st, bool after_init = false);
cudaError_t launch_bin(const FrameView& fv, cudaStream_t st);
cudaError_t launch_raster(const FrameView& fv, cudaStream_t st, int phase = 0);
cudaError_t launch_gather(const GatherList& g, cudaStream_t st);
cudaError_t launch_setup_batch(const BatchLaunch& b, int blocks, cudaStream_t st);
cudaError_t launch_bin_batch(const BatchLaunch& b, int blocks, cudaStream_t st);
cudaError_t launch_raster_batch(const BatchLaunch& b, int blocks, int threads, cudaStream_t st, bool vis);
int pixel_blocks(const FrameView& fv);
int vis_slots(const FrameView& fv);
cudaError_t launch_shade_pixels_batch(const BatchLaunch& b, int blocks, cudaStream_t st);
int setup_blocks(const FrameView& fv);
int bin_blocks(const FrameView& fv);
int raster_blocks(const FrameView& fv);
int raster_threads(const FrameView& fv);
cudaError_t launch_mlp_forward(const rsrgpu_mlp& w, const uint16_t* feat, int n, float* out, int* error,
                               int num_sms, cudaStream_t st);
cudaError_t launch_mlp_train(const rsrgpu_mlp& w, const uint16_t* feat, const float* target, const int32_t* index,
                             int batch, float* grad, float* loss, int* error, int num_sms, cudaStream_t st);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int n, int nw, float lr, float b1, float b2,
                        float eps, int step, uint16_t* wbf16, float* bias_out, cudaStream_t st);
cudaError_t launch_shade_plain(const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                               const rsrgpu_light* lights, int nlights, const float background[3],
                               uint32_t* out_srgb, float* out_linear, const uint8_t* srgb_lut, cudaStream_t st);
cudaError_t launch_learned_features(const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                                    const rsrgpu_light* lights, int nlights, uint16_t* features, float* targets,
                                    int32_t* candidates, int num_sms, cudaStream_t st);
cudaError_t launch_shade_learned(const rsrgpu_mlp& w, const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                                 const rsrgpu_light* lights, int nlights, const float background[3], float max_tile_mse,
                                 uint32_t* out_srgb, float* out_linear, uint8_t* tile_status, float* tile_mse,
                                 const uint8_t* srgb_lut, int* error, int* counters, void* scratch,
                                 int num_sms, int stall_polls, cudaStream_t st);
size_t learned_scratch_bytes(int tiles);
int texture_power(int width, int height);
struct FloatCanvasView {
    float4* data;
    int width, height, stride;
};
cudaError_t launch_kawase(const FloatCanvasView& src, const FloatCanvasView& dst, int dist, cudaStream_t st);
cudaError_t launch_glow(const FloatCanvasView& image, const FloatCanvasView& blur, uint32_t* out, int ostride,
                        int width, int height, const uint8_t* srgb_lut, cudaStream_t st);
cudaError_t launch_texture_chain(float* tex, const uint8_t* rgba8, int w, int premultiply, cudaStream_t st);
cudaError_t launch_rgba8_to_float(const uint8_t* rgba8, float* out, size_t n, int premultiply, int num_sms,
                                  cudaStream_t st);

static const uint32_t kRcpTable[2048] = {
#include "rcpps_table.inc"
};
}  // namespace rsrgpu

using namespace rsrgpu;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t n = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) cap = n;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// The part of a texture's mip chain the samplers address: level 0 (rows
// [0, w), w texels each) and the mip levels (rows [w, 2w), the first w/2
// texels of each); rsr's Texture leaves the rest of those rows zero.
struct TexRegion { size_t offset; int32_t edge; };   // bytes from the buffer start; edge 0: the whole rest

struct HostBuffer {
    const uint8_t* host = nullptr;
    size_t bytes = 0;
    std::vector<TexRegion> tex;   // this frame's textures in the buffer (late inputs)
    void* dev = nullptr;          // device mirror
    void* mapped = nullptr;       // device address of the host memory itself (pinned and mapped), else null
    bool in = false, out = false; // this frame reads it through the mirror / writes the mirror
    bool early = false;           // read by triangle setup (vertices, indices): copied first
    bool late = false;            // read only by the raster pass (textures): copied while setup and binning run
    bool direct = false;          // written by this frame straight into host memory (no mirror, no copy back)
};

// How a frame uses a caller pointer (resolve): kProbe maps without recording
// a use (entry points that take device pointers only check what they get).
enum Use { kProbe, kEarlyInput, kLateInput, kOutput };

struct Copy { void* dst; const void* src; size_t bytes; };

}  // namespace

struct rsrgpu_ctx {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t run_stream = nullptr;
    std::string err;
    // render target (GPU::Reset)
    int width = 0, height = 0, tile_w = 64, tile_h = 64, tiles_x = 0, tiles_y = 0, ntiles = 0;
    std::set<uint64_t> installed;   // (kind << 56) | (program << 24) | key
    std::map<const uint8_t*, HostBuffer> host;
    // frame tables
    std::vector<DevState> states;
    std::vector<int32_t> state_ordinal;
    std::vector<DevDraw> draws;
    std::vector<FrameOp> ops;
    std::vector<GBufferDesc> gbufs;
    std::vector<DevDrawExt> dext;   // per draw; uploaded when a draw is instanced or uses OBJ1Program
    bool any_inst = false;          // an instanced draw
    bool any_dext = false;          // the frame needs the extended setup (instanced or OBJ1Program draws)
    int ntris = 0;
    bool submitted = false;
    bool ran = false;
    // The submission's tables packed as they go to the device: states, draws,
    // ops, G-buffer descriptors, draw extensions (offsets in `tab_ofs`).
    // `packed_dev` is what the device tables hold; a submission whose packed
    // tables equal it uploads nothing.
    std::vector<uint8_t> packed, packed_dev;
    size_t tab_ofs[5] = {0, 0, 0, 0, 0};
    uint8_t* h_tables = nullptr;    // pinned staging of the table upload
    size_t h_tables_cap = 0;
    cudaEvent_t ev_tables = nullptr;  // the last upload from h_tables
    bool ev_tables_live = false;
    // what the captured graph depends on besides the tables' contents
    // (sizes, kernel choices, host-buffer routes): a submission with the same
    // signature keeps the graph
    std::vector<uint8_t> graph_sig;
    // device memory
    DevBuf d_tables, d_tris, d_bin_rect, d_rec16, d_chunk, d_super, d_clip_info,
        d_clip_verts, d_clip_poly, d_clip_src, d_clip_fan, d_bins, d_pool, d_counters, d_rcp, d_srgb,
        d_mlp_err, d_learn_err, d_learn_status, d_learn_tiles;
    std::map<cudaStream_t, cudaEvent_t> learn_events;   // last learned-shader launch per stream
    int num_sms = 0;
    int* h_mlp_err = nullptr;   // pinned
    uint32_t clip_cap = 1u << 18;
    uint32_t bin_cap = 1u << 22;
    int region_px = kRegionPx;      // raster CTA region (the autotuner may pick 16)
    int debug_learned_stall = 0;    // RSRGPU_DEBUG_LEARNED_STALL (rsrgpu_set_debug)
    int vis_keys = 0;               // FrameView::vis_keys of the submitted frame
    DevBuf d_vis;                   // owners and depths between the two launches of a split raster pass
    DevBuf d_queue;                 // the raster work queue: tiles by cost bucket
    DevBuf d_slice_keys;            // sliced visibility: merged keys per pixel
    DevBuf d_slice_done;            // sliced visibility: slices merged per raster block
    // the run's work captured once per submission and replayed by every run
    // (one launch instead of a dozen API calls); dropped when anything it
    // holds changes (submit, reset, host buffers, capacity growth)
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    bool tables_uploaded = false;   // states, draws, ops and G-buffer tables of this submission
    cudaGraphExec_t gexec = nullptr;
    FrameCounters* h_counters = nullptr;   // pinned, mapped: the raster pass writes it
    FrameCounters* h_counters_dev = nullptr;   // its device address
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    cudaEvent_t ev_done = nullptr;   // ev2 or ev3: the last event of a run (not owned)
    // textures from host buffers are copied on `side` while setup and binning run
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_late = nullptr;
    // the timing marks ev0 and ev1 are recorded on `marks`, a branch the
    // kernels do not wait for
    cudaStream_t marks = nullptr;
    cudaEvent_t ev_mark_fork = nullptr, ev_mark_join = nullptr;
    FrameView fv{};
    rsrgpu_stats stats{};
};

namespace {

int fail(rsrgpu_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

int cuda_fail(rsrgpu_ctx* c, cudaError_t e, const char* what) {
    return fail(c, RSRGPU_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what) do { cudaError_t e_ = (expr); if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); } while (0)

// float op order of rmlm::operator*(mat4, mat4) (rmlm_mat4.hxx:196-207); the
// host compiler runs with -ffp-contract=off so each product and sum rounds
void mat4_mul(const float* l, const float* r, float* out) {
    for (int row = 0; row < 4; ++row) {
        for (int col = 0; col < 4; ++col) {
            float ax = l[0 * 4 + row] * r[col * 4 + 0];
            ax = ax + l[1 * 4 + row] * r[col * 4 + 1];
            ax = ax + l[2 * 4 + row] * r[col * 4 + 2];
            ax = ax + l[3 * 4 + row] * r[col * 4 + 3];
            out[col * 4 + row] = ax;
        }
    }
}

int ilog2u(unsigned x) { int p = 0; while (x) { x >>= 1; ++p; } return p - 1; }

uint32_t fragment_state_key(const rsrgpu_glstate& s) {   // GLState::FragmentStateKey (rglv_gl.hxx:136-146)
    uint32_t key = uint32_t(s.program_id) << 24;
    key |= uint32_t(s.scissor_enabled != 0);
    key |= uint32_t(s.depth_test_enabled != 0) << 1;
    if (s.depth_test_enabled) key |= uint32_t(s.depth_func) << 2;
    key |= uint32_t(s.blending_enabled != 0) << 4;
    key |= uint32_t(s.depth_write_mask != 0) << 5;
    key |= uint32_t(s.color_write_mask != 0) << 6;
    key |= uint32_t(s.color0_attachment_type) << 7;
    key |= uint32_t(s.depth_attachment_type) << 9;
    return key;
}

bool draw_program_supported(int pid) {
    return pid == kProgGouraud || pid == kProgAmy || pid == kProgGBuffer || pid == kProgMany || pid == kProgOBJ1;
}
bool blt_program_supported(int pid) { return pid == kProgDefaultPost || pid == kProgExposurePost || pid == kProgGouraud; }

// the fragment state keys this device implementation covers: scissor test on
// or off, depth test on with LESS/LEQUAL/EQUAL, RGB f32 colour with f32 depth,
// or colour and depth packed in RGBA (RB_COLOR_DEPTH)
bool draw_key_supported(uint32_t key) {
    key &= 0xffffffu;   // bit 0, the scissor test, is taken with every state
    if (!(key & 2u)) return false;
    if (((key >> 2) & 3u) > 2u) return false;
    const uint32_t ct = (key >> 7) & 3u, dt = (key >> 9) & 3u;
    if (ct == RSRGPU_RB_RGBF32 && dt == RSRGPU_RB_F32) return true;
    if (ct == RSRGPU_RB_COLOR_DEPTH && dt == RSRGPU_RB_COLOR_DEPTH) return true;
    return false;
}

}  // namespace

// sRGB8 encode table of this library: for each of the 13*2048 float classes
// the clamped input falls into (exponent and top 11 mantissa bits), the
// correctly rounded 8-bit sRGB value of the class midpoint.
void rsrgpu::build_srgb_lut(std::vector<uint8_t>& lut) {
    lut.resize(26624);
    for (uint32_t k = 0; k < 26624; ++k) {
        const uint32_t bits = ((k + ((127u - 13u) << 11)) << 12) | 0x800u;
        float f;
        std::memcpy(&f, &bits, 4);
        const double x = f;
        const double s = x <= 0.0031308 ? 12.92 * x : 1.055 * std::pow(x, 1.0 / 2.4) - 0.055;
        double v = std::floor(s * 255.0 + 0.5);
        lut[k] = uint8_t(v < 0 ? 0 : (v > 255 ? 255 : v));
    }
}

namespace {

// Maps a caller pointer to a device address and the number of bytes that
// are valid from it (to the end of the registered host buffer, or of the
// device allocation containing it).  For a registered host buffer the use
// decides the address: outputs of pinned, mapped host memory are written in
// place by the kernels (the transfer overlaps the raster pass instead of
// following it); other uses go through the device mirror, copied in before
// the pass that reads it or out after the frame.
int resolve(rsrgpu_ctx* ctx, const void* p, Use use, void** out, const char* what, size_t* avail = nullptr,
            HostBuffer** owner = nullptr) {
    *out = nullptr;
    if (owner) *owner = nullptr;
    if (avail) *avail = 0;
    if (p == nullptr) return 0;
    const uint8_t* bp = static_cast<const uint8_t*>(p);
    auto it = ctx->host.upper_bound(bp);
    if (it != ctx->host.begin()) {
        --it;
        HostBuffer& hb = it->second;
        if (bp >= hb.host && bp < hb.host + hb.bytes) {
            void* base = hb.dev;
            if (use == kOutput) {
                if (hb.mapped != nullptr && !hb.in) { hb.direct = true; base = hb.mapped; }
                else hb.out = true;
            } else if (use != kProbe) {
                if (hb.direct) {
                    base = hb.mapped;   // this frame writes it in place: read it there too
                } else {
                    hb.in = true;
                    if (use == kLateInput) hb.late = true; else hb.early = true;
                }
            }
            *out = static_cast<uint8_t*>(base) + (bp - hb.host);
            if (avail) *avail = hb.bytes - size_t(bp - hb.host);
            if (owner) *owner = &hb;
            return 0;
        }
    }
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e == cudaSuccess && (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)) {
        // cuMemGetAddressRange through the runtime's driver entry point, so the
        // library itself does not link libcuda (it loads on machines without a GPU)
        using RangeFn = CUresult (*)(CUdeviceptr*, size_t*, CUdeviceptr);
        static RangeFn range_fn = nullptr;
        if (range_fn == nullptr) {
            void* fn = nullptr;
            cudaDriverEntryPointQueryResult q{};
            if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                range_fn = reinterpret_cast<RangeFn>(fn);
        }
        CUdeviceptr base = 0;
        size_t size = 0;
        if (range_fn == nullptr || range_fn(&base, &size, CUdeviceptr(uintptr_t(p))) != CUDA_SUCCESS)
            return fail(ctx, RSRGPU_EINVAL, "%s pointer %p: allocation range unknown", what, p);
        *out = const_cast<void*>(p);
        if (avail) *avail = size_t(base + size - CUdeviceptr(uintptr_t(p)));
        return 0;
    }
    cudaGetLastError();
    return fail(ctx, RSRGPU_EINVAL, "%s pointer %p is neither device memory nor a registered host buffer", what, p);
}

template <typename T>
bool rd(const uint8_t*& p, const uint8_t* end, T& v) {
    if (p + sizeof(T) > end) return false;
    std::memcpy(&v, p, sizeof(T));
    p += sizeof(T);
    return true;
}

int decode_state(rsrgpu_ctx* ctx, const rsrgpu_glstate& s, DevState& d) {
    std::memset(&d, 0, sizeof(d));
    mat4_mul(s.projection_matrix, s.view_matrix, d.vpm);   // MakeMatrices: vpm = P * V
    int vx = ctx->width, vy = ctx->height;                 // GPU::DSDO (rglv_gpu.hxx:265-270)
    if (s.viewport_size[0] != 0 || s.viewport_size[1] != 0) { vx = s.viewport_size[0]; vy = s.viewport_size[1]; }
    d.DS[0] = float(vx / 2);
    d.DS[1] = float(-vy / 2);
    d.DO[0] = float(vx / 2 + s.viewport_origin[0]);
    d.DO[1] = float(ctx->height - (vy / 2 + s.viewport_origin[1]));
    {   // CalcGuardBandFactor (rglv_view_frustum.hxx:36-39)
        const int longSide = std::max(ctx->width, ctx->height);
        const int half = longSide / 2;
        d.guard = (2048.0f - float(half)) / float(half);
    }
    if (!s.scissor_enabled) {   // GPU::ScissorRect (rglv_gpu.hxx:272-276)
        d.scissor[0] = 0; d.scissor[1] = 0; d.scissor[2] = ctx->width; d.scissor[3] = ctx->height;
    } else {
        const int left = s.scissor_origin[0], right = left + s.scissor_size[0];
        const int bottom = ctx->height - s.scissor_origin[1] - 1, top = bottom - s.scissor_size[1];
        d.scissor[0] = left; d.scissor[1] = top; d.scissor[2] = right; d.scissor[3] = bottom;
    }
    d.scissor_test = s.scissor_enabled != 0;
    d.program = s.program_id;
    d.nvary = (s.program_id == kProgGouraud || s.program_id == kProgOBJ1) ? 3
            : (s.program_id == kProgAmy || s.program_id == kProgMany) ? 2 : (s.program_id == kProgGBuffer ? 4 : 0);
    d.keep_backs = !(s.culling_enabled && s.cull_face == RSRGPU_GL_BACK);
    d.keep_fronts = !(s.culling_enabled && s.cull_face == RSRGPU_GL_FRONT);
    d.cull_enabled = s.culling_enabled != 0;
    d.cull_face = s.cull_face;
    d.depth_test = s.depth_test_enabled != 0;
    d.depth_func = s.depth_func;
    d.depth_write = s.depth_write_mask != 0;
    d.color_write = s.color_write_mask != 0;
    d.blend = s.blending_enabled != 0;
    d.color_type = s.color0_attachment_type;
    d.depth_type = s.depth_attachment_type;
    std::memcpy(d.clear_color, s.clear_color, sizeof(d.clear_color));
    d.clear_depth = s.clear_depth;
    std::memcpy(d.uniforms, s.uniforms, sizeof(d.uniforms));
    for (int i = 0; i < 16; ++i) {
        void* dp = nullptr;
        size_t avail = 0;
        int rc = resolve(ctx, s.buffers[i], kEarlyInput, &dp, "vertex buffer", &avail);
        if (rc) return rc;
        d.buffers[i] = static_cast<const float*>(dp);
        d.buffer_len[i] = int32_t(std::min<size_t>(avail / sizeof(float), size_t(INT32_MAX)));
    }
    // MakeTextureUnit (rglr_texture_sampler.cxx:314-363)
    const rsrgpu_texture_state& t = s.tus[0];
    d.tu0.width = t.width; d.tu0.height = t.height; d.tu0.stride = t.stride;
    d.tu0.power = ilog2u(unsigned(t.width));
    const bool pow2 = t.width > 0 && (1 << d.tu0.power) == t.width && t.width == t.height && t.stride == t.width;
    d.tu0.kind = pow2 ? (t.filter ? 1 : 0) : 2;
    if (s.program_id == kProgAmy) {
        if (t.ptr == nullptr) return fail(ctx, RSRGPU_EINVAL, "AmyProgram draw without a texture on unit 0");
        if (pow2 && (t.width < 4 || t.width > 1024))
            return fail(ctx, RSRGPU_EUNSUPPORTED, "can't make TextureUnit for pow2 size %d", t.width);
        void* dp = nullptr;
        size_t avail = 0;
        HostBuffer* hb = nullptr;
        int rc = resolve(ctx, t.ptr, kLateInput, &dp, "texture", &avail, &hb);
        if (rc) return rc;
        if (hb != nullptr && hb->late) {   // each texture once, however many states bind it
            const TexRegion reg{ size_t(static_cast<const uint8_t*>(static_cast<const void*>(t.ptr)) - hb->host),
                                 pow2 ? t.width : 0 };
            bool seen = false;
            for (const TexRegion& r : hb->tex) seen = seen || (r.offset == reg.offset && r.edge == reg.edge);
            if (!seen) hb->tex.push_back(reg);
        }
        // the mip chain of a square power-of-two texture (2*W*W texels), else H rows of stride texels
        const size_t need = pow2 ? size_t(2) * size_t(t.width) * size_t(t.width) * 16u
                                 : size_t(std::max(t.height, 1)) * size_t(std::max(t.stride, 1)) * 16u;
        if (t.width <= 0 || t.height <= 0 || t.stride < t.width || avail < need)
            return fail(ctx, RSRGPU_EINVAL, "texture buffer holds %zu bytes, its %dx%d (stride %d) layout needs %zu",
                        avail, t.width, t.height, t.stride, need);
        d.tu0.buf = static_cast<const float*>(dp);
        d.tu0.texels = int32_t(std::min<size_t>(avail / 16u, size_t(INT32_MAX)));
    }
    return 0;
}

}  // namespace

extern "C" {

namespace {
void drop_graph(rsrgpu_ctx* ctx) {
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    if (ctx->graph) { cudaGraphDestroy(ctx->graph); ctx->graph = nullptr; }
}
}  // namespace

int rsrgpu_create(int device, rsrgpu_ctx** out) {
    if (out == nullptr) return RSRGPU_EINVAL;
    *out = nullptr;
    rsrgpu_ctx* ctx = new rsrgpu_ctx;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete ctx; return RSRGPU_ECUDA; }
    if (cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->cap, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->marks, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_mark_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_mark_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_late, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_tables, cudaEventDisableTiming) != cudaSuccess ||
        cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_counters), sizeof(FrameCounters), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->h_counters_dev), ctx->h_counters, 0) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->ev2) != cudaSuccess || cudaEventCreate(&ctx->ev3) != cudaSuccess) {
        rsrgpu_destroy(ctx);
        return RSRGPU_ECUDA;
    }
    std::vector<uint8_t> lut;
    build_srgb_lut(lut);
    if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        rsrgpu_destroy(ctx);
        return RSRGPU_ECUDA;
    }
    if (ctx->d_rcp.ensure(sizeof(kRcpTable)) != cudaSuccess || ctx->d_srgb.ensure(lut.size()) != cudaSuccess ||
        cudaMemcpy(ctx->d_rcp.p, kRcpTable, sizeof(kRcpTable), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(ctx->d_srgb.p, lut.data(), lut.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        rsrgpu_destroy(ctx);
        return RSRGPU_ECUDA;
    }
    std::memset(ctx->h_counters, 0, sizeof(FrameCounters));
    *out = ctx;
    return 0;
}

int rsrgpu_destroy(rsrgpu_ctx* ctx) {
    if (ctx == nullptr) return 0;
    if (ctx->own) cudaStreamSynchronize(ctx->own);
    for (auto& kv : ctx->host) if (kv.second.dev) cudaFree(kv.second.dev);
    if (ctx->h_mlp_err) cudaFreeHost(ctx->h_mlp_err);
    for (auto& kv : ctx->learn_events) { cudaEventSynchronize(kv.second); cudaEventDestroy(kv.second); }
    DevBuf* bufs[] = { &ctx->d_slice_keys, &ctx->d_slice_done, &ctx->d_queue, &ctx->d_vis, &ctx->d_mlp_err, &ctx->d_learn_err, &ctx->d_learn_status, &ctx->d_learn_tiles, &ctx->d_tables, &ctx->d_tris, &ctx->d_bin_rect, &ctx->d_rec16,
                       &ctx->d_chunk, &ctx->d_super, &ctx->d_clip_info, &ctx->d_clip_verts, &ctx->d_clip_poly,
                       &ctx->d_clip_src, &ctx->d_clip_fan, &ctx->d_bins, &ctx->d_pool, &ctx->d_counters,
                       &ctx->d_rcp, &ctx->d_srgb };
    for (DevBuf* b : bufs) b->release();
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->ev_tables_live) cudaEventSynchronize(ctx->ev_tables);
    if (ctx->h_tables) cudaFreeHost(ctx->h_tables);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->marks) cudaStreamSynchronize(ctx->marks);
    drop_graph(ctx);
    if (ctx->cap) cudaStreamDestroy(ctx->cap);
    cudaEvent_t evs[] = { ctx->ev0, ctx->ev1, ctx->ev2, ctx->ev3, ctx->ev_fork, ctx->ev_late, ctx->ev_tables,
                          ctx->ev_mark_fork, ctx->ev_mark_join };
    for (cudaEvent_t ev : evs) if (ev) cudaEventDestroy(ev);
    if (ctx->marks) cudaStreamDestroy(ctx->marks);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
    return 0;
}

int rsrgpu_install(rsrgpu_ctx* ctx, int program_id, uint32_t state_key, int kind) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (kind == 0) {
        if (!draw_program_supported(program_id))
            return fail(ctx, RSRGPU_ENODISPATCH, "no device vertex program for pid(%d)", program_id);
    } else if (kind == 1) {
        if (!draw_program_supported(program_id) || !draw_key_supported(state_key))
            return fail(ctx, RSRGPU_ENODISPATCH, "no device fragment program for pid(%d) state(0x%x)", program_id, state_key);
    } else if (kind == 2) {
        if (!blt_program_supported(program_id))
            return fail(ctx, RSRGPU_ENODISPATCH, "no device blt program for pid(%d)", program_id);
    } else {
        return fail(ctx, RSRGPU_EINVAL, "unknown program kind %d", kind);
    }
    ctx->installed.insert((uint64_t(kind) << 56) | (uint64_t(uint32_t(program_id) & 0xff) << 24) | (state_key & 0xffffffu));
    return 0;
}

int rsrgpu_reset(rsrgpu_ctx* ctx, int width, int height, int tile_blocks_x, int tile_blocks_y) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (width <= 0 || height <= 0 || (width & 3) || (height & 1))
        return fail(ctx, RSRGPU_EINVAL, "target %dx%d: width must be a multiple of 4 and height of 2", width, height);
    if (tile_blocks_x <= 0 || tile_blocks_y <= 0 || tile_blocks_x > 16 || tile_blocks_y > 16)
        return fail(ctx, RSRGPU_EINVAL, "tile size in blocks must be 1..16");
    ctx->width = width;
    ctx->height = height;
    ctx->tile_w = tile_blocks_x * 8;   // kBlockDimensionsInPixels (rglv_gpu.hxx:27)
    ctx->tile_h = tile_blocks_y * 8;
    ctx->tiles_x = (width + ctx->tile_w - 1) / ctx->tile_w;   // GPU::Retile (rglv_gpu.cxx:67-87)
    ctx->tiles_y = (height + ctx->tile_h - 1) / ctx->tile_h;
    ctx->ntiles = ctx->tiles_x * ctx->tiles_y;
    if (ctx->tiles_x > 32767 || ctx->tiles_y > 32767) return fail(ctx, RSRGPU_EINVAL, "too many tiles");
    ctx->submitted = false;   // the captured run stays: a submission of the same structure and size replays it
    return 0;
}

int rsrgpu_register_host_buffer(rsrgpu_ctx* ctx, const void* host_ptr, size_t bytes) {
    if (ctx != nullptr) drop_graph(ctx);
    if (ctx == nullptr || host_ptr == nullptr || bytes == 0) return RSRGPU_EINVAL;
    const uint8_t* p = static_cast<const uint8_t*>(host_ptr);
    auto it = ctx->host.find(p);
    if (it != ctx->host.end()) {
        if (it->second.bytes >= bytes) return 0;
        cudaFree(it->second.dev);
        ctx->host.erase(it);
    }
    // drop registrations the new range overlaps (their memory was reused)
    for (auto jt = ctx->host.begin(); jt != ctx->host.end();) {
        if (jt->second.host < p + bytes && p < jt->second.host + jt->second.bytes) {
            cudaStreamSynchronize(ctx->own);
            cudaFree(jt->second.dev);
            jt = ctx->host.erase(jt);
        } else {
            ++jt;
        }
    }
    HostBuffer hb;
    hb.host = p;
    hb.bytes = bytes;
    CK(cudaMalloc(&hb.dev, bytes), "cudaMalloc(host mirror)");
    // texture mirrors take only the texels the samplers address (the rest of
    // the mip rows is zero in rsr's layout): start from zeros
    CK(cudaMemset(hb.dev, 0, bytes), "clear host mirror");
    // pinned host memory the device can address (cudaHostAlloc, or registered as mapped)
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer != nullptr)
        hb.mapped = a.devicePointer;
    else
        cudaGetLastError();
    ctx->host[p] = hb;
    return 0;
}

int rsrgpu_unregister_host_buffer(rsrgpu_ctx* ctx, const void* host_ptr) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    drop_graph(ctx);
    auto it = ctx->host.find(static_cast<const uint8_t*>(host_ptr));
    if (it == ctx->host.end()) return fail(ctx, RSRGPU_EINVAL, "buffer %p is not registered", host_ptr);
    cudaStreamSynchronize(ctx->own);
    cudaFree(it->second.dev);
    ctx->host.erase(it);
    return 0;
}

namespace {

// GPU::BinImpl's command interpretation (rglv_gpu.cxx:119-260), on the host:
// the frame's states, draws and op list, and how it uses every caller buffer.
int decode_frame(rsrgpu_ctx* ctx, const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates) {
    for (auto& kv : ctx->host) {
        kv.second.in = kv.second.out = kv.second.early = kv.second.late = kv.second.direct = false;
        kv.second.tex.clear();
    }
    ctx->states.assign(size_t(nstates), DevState{});
    ctx->state_ordinal.assign(size_t(nstates), -1);
    ctx->draws.clear();
    ctx->ops.clear();
    ctx->gbufs.clear();
    ctx->dext.clear();
    ctx->any_inst = false;
    ctx->any_dext = false;
    ctx->ntris = 0;
    bool gbuffer_frame = false, other_op_since_draw = false, any_draw = false;
    std::vector<bool> decoded(size_t(nstates), false);
    int ordinals = 0;
    int cur = -1;
    const uint8_t* p = commands;
    const uint8_t* end = commands + nbytes;
    while (p < end) {
        uint8_t op = 0;
        rd(p, end, op);
        if (op == RSRGPU_CMD_EOF) break;
        FrameOp fo{};
        switch (op) {
        case RSRGPU_CMD_STATE: {
            uint64_t idx;
            if (!rd(p, end, idx) || idx >= uint64_t(nstates)) return fail(ctx, RSRGPU_EINVAL, "CMD_STATE index out of range");
            if (!decoded[idx]) {
                int rc = decode_state(ctx, states[idx], ctx->states[idx]);
                if (rc) return rc;
                decoded[idx] = true;
            }
            if (ctx->state_ordinal[idx] < 0) ctx->state_ordinal[idx] = ordinals++;
            cur = int(idx);
            fo.kind = kOpState;
            fo.arg = int(idx);
            fo.ordinal = ctx->state_ordinal[idx];
            ctx->ops.push_back(fo);
        } break;
        case RSRGPU_CMD_CLEAR: {
            uint8_t bits;
            if (!rd(p, end, bits)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_CLEAR");
            if (cur < 0) return fail(ctx, RSRGPU_EINVAL, "CMD_CLEAR before any state");
            if (bits & 4) return fail(ctx, RSRGPU_EUNSUPPORTED, "CLEAR on STENCIL not implemented");
            const auto& s = states[cur];
            if (s.color0_attachment_type == RSRGPU_RB_COLOR_DEPTH && bits != 3)
                return fail(ctx, RSRGPU_EINVAL, "must clear color and depth when using RB_COLOR_DEPTH");
            fo.kind = kOpClear;
            fo.arg = bits;
            ctx->ops.push_back(fo);
            other_op_since_draw = true;
        } break;
        case RSRGPU_CMD_DRAW_ELEMENTS:
        case RSRGPU_CMD_DRAW_ARRAYS:
        case RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED:
        case RSRGPU_CMD_DRAW_ARRAYS_INSTANCED: {
            int32_t count = 0, ninst = 1;
            uint64_t iptr = 0;
            const bool instanced = op == RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED || op == RSRGPU_CMD_DRAW_ARRAYS_INSTANCED;
            if (op == RSRGPU_CMD_DRAW_ELEMENTS) {
                uint8_t flags, hint;
                if (!rd(p, end, flags) || !rd(p, end, hint) || !rd(p, end, count) || !rd(p, end, iptr))
                    return fail(ctx, RSRGPU_EINVAL, "truncated CMD_DRAW_ELEMENTS");
                if (flags != 0x14) return fail(ctx, RSRGPU_EINVAL, "CMD_DRAW_ELEMENTS flags must be 0x14");
            } else if (op == RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED) {
                // GL::DrawElementsInstanced (rglv_gl.cxx:46-55): no hint byte
                uint8_t flags;
                if (!rd(p, end, flags) || !rd(p, end, count) || !rd(p, end, iptr) || !rd(p, end, ninst))
                    return fail(ctx, RSRGPU_EINVAL, "truncated CMD_DRAW_ELEMENTS_INSTANCED");
                if (flags != 0x14) return fail(ctx, RSRGPU_EINVAL, "CMD_DRAW_ELEMENTS_INSTANCED flags must be 0x14");
            } else if (op == RSRGPU_CMD_DRAW_ARRAYS_INSTANCED) {
                if (!rd(p, end, count) || !rd(p, end, ninst)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_DRAW_ARRAYS_INSTANCED");
            } else {
                if (!rd(p, end, count)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_DRAW_ARRAYS");
            }
            // the tile records carry the instance id as a u16 (rglv_gpu_impl.hxx:490,657)
            if (ninst < 0 || ninst > 65536) return fail(ctx, RSRGPU_EINVAL, "instance count %d: 0 .. 65536", ninst);
            if (cur < 0) return fail(ctx, RSRGPU_EINVAL, "draw before any state");
            const auto& s = states[cur];
            const uint32_t vkey = (uint32_t(s.program_id) & 0xff) << 24;
            if (!ctx->installed.count((uint64_t(0) << 56) | vkey))
                return fail(ctx, RSRGPU_ENODISPATCH, "BIN:DRAW no dispatch entry for 0x%x", vkey);
            const uint32_t fkey = fragment_state_key(s) & 0xffffffu;
            if (!ctx->installed.count((uint64_t(1) << 56) | vkey | fkey))
                return fail(ctx, RSRGPU_ENODISPATCH, "no dispatch entry for 0x%x found for CMD_DRAW_INLINE", vkey | fkey);
            if (count < 0) return fail(ctx, RSRGPU_EINVAL, "negative draw count");
            if (s.program_id == kProgGouraud && (!s.buffers[0] || !s.buffers[3] || !s.buffers[4] || !s.buffers[5]))
                return fail(ctx, RSRGPU_EINVAL, "Gouraud program needs buffers 0-5");
            if (s.program_id == kProgGBuffer && (!s.buffers[0] || !s.buffers[3] || !s.buffers[4] || !s.buffers[5] || !s.buffers[6]))
                return fail(ctx, RSRGPU_EINVAL, "G-buffer program needs buffers 0-6");
            if (s.program_id == kProgGBuffer && s.blending_enabled)
                return fail(ctx, RSRGPU_EUNSUPPORTED, "the G-buffer program does not blend");
            if (s.program_id == kProgMany && !instanced)
                return fail(ctx, RSRGPU_EUNSUPPORTED, "ManyProgram draws take instance matrices: use an instanced draw");
            if (s.program_id == kProgMany && s.blending_enabled)
                return fail(ctx, RSRGPU_EUNSUPPORTED, "ManyProgram is not drawn with blending on the device");
            if (s.program_id == kProgMany && ninst > 0 &&
                (ctx->states[size_t(cur)].buffers[15] == nullptr ||
                 int64_t(ctx->states[size_t(cur)].buffer_len[15]) < int64_t(ninst) * 16))
                return fail(ctx, RSRGPU_EINVAL, "ManyProgram: buffer 15 must hold %d instance matrices", ninst);
            any_draw = true;
            other_op_since_draw = false;
            DevDraw dd{};
            dd.state = cur;
            dd.first_tri = ctx->ntris;
            dd.ntris = count / 3;
            dd.is_arrays = op == RSRGPU_CMD_DRAW_ARRAYS || op == RSRGPU_CMD_DRAW_ARRAYS_INSTANCED;
            DevDrawExt di{};
            std::memcpy(di.vm, s.view_matrix, sizeof(di.vm));
            if (s.program_id == kProgOBJ1) ctx->any_dext = true;
            if (instanced) {
                di.per_inst = dd.ntris;
                di.ninst = ninst;
                di.matrices = s.program_id == kProgMany ? ctx->states[size_t(cur)].buffers[15] : nullptr;
                if (int64_t(dd.ntris) * ninst > (int64_t(1) << 30)) return fail(ctx, RSRGPU_ECAPACITY, "too many triangles");
                dd.ntris *= ninst;
                ctx->any_inst = true;
                ctx->any_dext = true;
            }
            if (!dd.is_arrays) {
                // the indices of one instance (every instance reads the same ones)
                const size_t tris = size_t(instanced ? di.per_inst : dd.ntris);
                void* dp = nullptr;
                size_t avail = 0;
                int rc = resolve(ctx, reinterpret_cast<const void*>(uintptr_t(iptr)), kEarlyInput, &dp, "index", &avail);
                if (rc) return rc;
                if (dp == nullptr || avail < tris * 3u * sizeof(uint16_t))
                    return fail(ctx, RSRGPU_EINVAL, "index buffer holds %zu bytes, draw needs %zu", avail, tris * 6u);
                dd.indices = static_cast<const uint16_t*>(dp);
            }
            if (int64_t(ctx->ntris) + dd.ntris > (int64_t(1) << 30)) return fail(ctx, RSRGPU_ECAPACITY, "too many triangles");
            ctx->ntris += dd.ntris;
            fo.kind = kOpDraw;
            fo.arg = int(ctx->draws.size());
            ctx->draws.push_back(dd);
            ctx->dext.push_back(di);
            ctx->ops.push_back(fo);
        } break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC: {
            uint8_t gamma;
            uint64_t cp;
            if (!rd(p, end, gamma) || !rd(p, end, cp)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_STORE_COLOR_FULL_LINEAR_TC");
            if (cur < 0) return fail(ctx, RSRGPU_EINVAL, "store before any state");
            const auto& s = states[cur];
            const uint32_t bkey = (uint32_t(s.program_id) & 0xff) << 24;
            if (!ctx->installed.count((uint64_t(2) << 56) | bkey))
                return fail(ctx, RSRGPU_ENODISPATCH, "no dispatch entry for %x found for CMD_STORE_COLOR_FULL_LINEAR_TC", bkey);
            const auto* cv = reinterpret_cast<const rsrgpu_truecolor_canvas*>(uintptr_t(cp));
            if (cv == nullptr || cv->width != ctx->width || cv->height != ctx->height || cv->stride < cv->width || (cv->stride & 1))
                return fail(ctx, RSRGPU_EINVAL, "TrueColor canvas must match the %dx%d target (even stride)", ctx->width, ctx->height);
            void* dp = nullptr;
            size_t avail = 0;
            int rc = resolve(ctx, cv->data, kOutput, &dp, "color output", &avail);
            if (rc) return rc;
            if (dp == nullptr || avail < size_t(cv->stride) * size_t(cv->height) * 4u)
                return fail(ctx, RSRGPU_EINVAL, "color output holds %zu bytes, needs %zu", avail, size_t(cv->stride) * size_t(cv->height) * 4u);
            if (reinterpret_cast<uintptr_t>(dp) & 7) return fail(ctx, RSRGPU_EINVAL, "color output must be 8-byte aligned");
            other_op_since_draw = true;
            fo.kind = kOpStoreTC;
            fo.arg = gamma ? 1 : 0;
            fo.ptr = dp;
            fo.width = cv->width; fo.height = cv->height; fo.stride = cv->stride;
            ctx->ops.push_back(fo);
        } break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP: {
            // rglv_gpu.cxx:345-383: Copy / Downsample of the tile's colour
            // buffer into a float canvas (RB_RGBF32 or RB_COLOR_DEPTH)
            uint64_t cp;
            if (!rd(p, end, cp)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_STORE_COLOR_*_FP");
            if (cur < 0) return fail(ctx, RSRGPU_EINVAL, "store before any state");
            const int ct = states[cur].color0_attachment_type;
            if (ct != RSRGPU_RB_RGBF32 && ct != RSRGPU_RB_COLOR_DEPTH)
                return fail(ctx, RSRGPU_EUNSUPPORTED, "CMD_STORE_COLOR_*_FP not implemented for attachment type %d", ct);
            const bool half = op == RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP;
            const bool quads = op == RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP;
            // both canvas mirrors share the layout {data, width, height, stride}
            const auto* cv = reinterpret_cast<const rsrgpu_fp_canvas*>(uintptr_t(cp));
            const int want_w = half ? ctx->width / 2 : ctx->width;
            const int want_h = half ? ctx->height / 2 : ctx->height;
            const int min_stride = quads ? ctx->width / 2 : want_w;
            if (cv == nullptr || cv->width != want_w || cv->height != want_h || cv->stride < min_stride)
                return fail(ctx, RSRGPU_EINVAL, "float canvas must be %dx%d with stride >= %d", want_w, want_h, min_stride);
            // bytes from the canvas base to the end of its last written row
            const size_t rows = quads ? size_t(ctx->height / 2) : size_t(want_h);
            const size_t unit = quads ? 64u : 16u;
            const size_t need = ((rows - 1) * size_t(cv->stride) + size_t(min_stride)) * unit;
            void* dp = nullptr;
            size_t avail = 0;
            int rc = resolve(ctx, cv->data, kOutput, &dp, "float color output", &avail);
            if (rc) return rc;
            if (dp == nullptr || avail < need)
                return fail(ctx, RSRGPU_EINVAL, "float color output holds %zu bytes, needs %zu", avail, need);
            if (reinterpret_cast<uintptr_t>(dp) & 15) return fail(ctx, RSRGPU_EINVAL, "float color output must be 16-byte aligned");
            other_op_since_draw = true;
            fo.kind = half ? kOpStoreHalfFP : quads ? kOpStoreQuadsFP : kOpStoreFP;
            fo.ptr = dp;
            fo.width = cv->width; fo.height = cv->height; fo.stride = cv->stride;
            ctx->ops.push_back(fo);
        } break;
        case RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP: {
            uint64_t dp64;
            if (!rd(p, end, dp64)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_STORE_DEPTH_FULL_LINEAR_FP");
            if (cur < 0) return fail(ctx, RSRGPU_EINVAL, "store before any state");
            if (states[cur].depth_attachment_type != RSRGPU_RB_F32)
                return fail(ctx, RSRGPU_EUNSUPPORTED, "STORE_DEPTH_FULL_LINEAR_FP not implemented for attachment type %d", states[cur].depth_attachment_type);
            void* dp = nullptr;
            size_t avail = 0;
            int rc = resolve(ctx, reinterpret_cast<const void*>(uintptr_t(dp64)), kOutput, &dp, "depth output", &avail);
            if (rc) return rc;
            if (dp == nullptr || avail < size_t(ctx->width) * size_t(ctx->height) * 4u)
                return fail(ctx, RSRGPU_EINVAL, "depth output holds %zu bytes, needs %zu", avail, size_t(ctx->width) * size_t(ctx->height) * 4u);
            if (reinterpret_cast<uintptr_t>(dp) & 7) return fail(ctx, RSRGPU_EINVAL, "depth output must be 8-byte aligned");
            other_op_since_draw = true;
            fo.kind = kOpStoreDepth;
            fo.ptr = dp;
            fo.width = ctx->width; fo.height = ctx->height; fo.stride = ctx->width;
            ctx->ops.push_back(fo);
        } break;
        case RSRGPU_CMD_STORE_GBUFFER: {
            uint64_t gp;
            if (!rd(p, end, gp)) return fail(ctx, RSRGPU_EINVAL, "truncated CMD_STORE_GBUFFER");
            if (cur < 0) return fail(ctx, RSRGPU_EINVAL, "store before any state");
            if (other_op_since_draw && any_draw)
                return fail(ctx, RSRGPU_EINVAL, "CMD_STORE_GBUFFER must directly follow the G-buffer draws");
            const auto* g = reinterpret_cast<const rsrgpu_gbuffer*>(uintptr_t(gp));
            if (g == nullptr || g->width != ctx->width || g->height != ctx->height)
                return fail(ctx, RSRGPU_EINVAL, "G-buffer must match the %dx%d target", ctx->width, ctx->height);
            const size_t npx = size_t(ctx->width) * size_t(ctx->height);
            GBufferDesc gd{};
            void* dp = nullptr;
            size_t avail = 0;
            const void* srcs[5] = { g->depth, g->normal_x, g->normal_y, g->normal_z, g->albedo };
            const size_t need[5] = { npx * 4, npx * 2, npx * 2, npx * 2, npx * 4 };
            void** dsts[5] = { reinterpret_cast<void**>(&gd.depth), reinterpret_cast<void**>(&gd.nx),
                               reinterpret_cast<void**>(&gd.ny), reinterpret_cast<void**>(&gd.nz),
                               reinterpret_cast<void**>(&gd.albedo) };
            for (int k = 0; k < 5; ++k) {
                int rc = resolve(ctx, srcs[k], kOutput, &dp, "G-buffer", &avail);
                if (rc) return rc;
                if (dp == nullptr || avail < need[k] || (reinterpret_cast<uintptr_t>(dp) & 7))
                    return fail(ctx, RSRGPU_EINVAL, "G-buffer plane %d: need %zu bytes, 8-byte aligned", k, need[k]);
                *dsts[k] = dp;
            }
            gbuffer_frame = true;
            other_op_since_draw = true;
            fo.kind = kOpStoreGBuffer;
            fo.arg = int(ctx->gbufs.size());
            fo.width = ctx->width; fo.height = ctx->height; fo.stride = ctx->width;
            ctx->gbufs.push_back(gd);
            ctx->ops.push_back(fo);
        } break;
        default:
            return fail(ctx, RSRGPU_EUNSUPPORTED, "command 0x%02x is not supported", op);
        }
    }
    if (gbuffer_frame) {
        for (const DevDraw& d : ctx->draws)
            if (ctx->states[size_t(d.state)].program != kProgGBuffer)
                return fail(ctx, RSRGPU_EINVAL, "a frame with CMD_STORE_GBUFFER draws only with the G-buffer program");
    }
    if (nstates == 0) ctx->states.assign(1, DevState{});
    // visibility by (depth, order) keys in the raster pass: every draw opaque
    // with depth test and write on and one depth function (LESS or LEQUAL),
    // clears before the first draw, stores after the last, at most 4096 draws
    {
        int func = -1;
        bool ok = !ctx->draws.empty() && ctx->draws.size() <= 4096, drawn = false, stored = false;
        for (const FrameOp& o : ctx->ops) {
            if (o.kind == kOpClear && drawn) ok = false;
            if (op_is_store(o.kind)) stored = true;
            if (o.kind != kOpDraw) continue;
            if (stored) ok = false;
            drawn = true;
            const DevState& st = ctx->states[size_t(ctx->draws[size_t(o.arg)].state)];
            if (st.blend || !st.depth_test || !st.depth_write || !st.color_write || st.depth_func < 0 || st.depth_func > 1 ||
                (func >= 0 && st.depth_func != func) || st.scissor_test)
                ok = false;
            func = st.depth_func;
        }
        ctx->vis_keys = ok ? 1 + func : 0;
    }
    // what the raster pass reads of each op, inline (no state or draw load)
    int st = -1;
    for (FrameOp& o : ctx->ops) {
        if (o.kind == kOpState) {
            st = o.arg;
            const DevState& d = ctx->states[size_t(st)];
            o.info[0] = d.program;
            o.info[1] = (d.depth_test ? kFragDepthTest : 0) | (d.depth_func << kFragDepthFuncShift) |
                        (d.depth_write ? kFragDepthWrite : 0) | (d.color_write ? kFragColorWrite : 0) |
                        (d.blend ? kFragBlend : 0) | (d.scissor_test ? kFragScissor : 0);
        } else if (o.kind == kOpClear && st >= 0) {
            const DevState& d = ctx->states[size_t(st)];
            for (int k = 0; k < 3; ++k) o.val[k] = d.clear_color[k];
            o.val[3] = d.clear_depth;
            o.info[2] = d.color_type == RSRGPU_RB_COLOR_DEPTH ? 1 : 0;
        } else if (o.kind == kOpDraw) {
            const DevDraw& dd = ctx->draws[size_t(o.arg)];
            o.info[0] = dd.first_tri;
            o.info[1] = dd.ntris;
            o.info[2] = dd.state;
        }
    }
    return 0;
}

bool frame_is_ext(const rsrgpu_ctx* ctx) {
    for (const FrameOp& o : ctx->ops)
        if (o.kind >= kOpStoreFP) return true;
    for (const DevDraw& d : ctx->draws)
        if (ctx->states[size_t(d.state)].program == kProgMany) return true;
    return false;
}

void put_raw(std::vector<uint8_t>& v, const void* x, size_t n) {
    const auto* b = static_cast<const uint8_t*>(x);
    v.insert(v.end(), b, b + n);
}
#define put_bytes(v, x) put_raw((v), &(x), sizeof(x))

// The submission's tables in one block, each part 256-byte aligned.
void pack_tables(rsrgpu_ctx* ctx) {
    const size_t sizes[5] = { sizeof(DevState) * ctx->states.size(), sizeof(DevDraw) * ctx->draws.size(),
                              sizeof(FrameOp) * ctx->ops.size(), sizeof(GBufferDesc) * ctx->gbufs.size(),
                              ctx->any_dext ? sizeof(DevDrawExt) * ctx->dext.size() : 0 };
    const void* srcs[5] = { ctx->states.data(), ctx->draws.data(), ctx->ops.data(), ctx->gbufs.data(), ctx->dext.data() };
    size_t at = 0;
    for (int k = 0; k < 5; ++k) {
        ctx->tab_ofs[k] = at;
        at += (std::max<size_t>(sizes[k], 1) + 255) & ~size_t(255);
    }
    ctx->packed.assign(at, 0);
    for (int k = 0; k < 5; ++k)
        if (sizes[k]) std::memcpy(ctx->packed.data() + ctx->tab_ofs[k], srcs[k], sizes[k]);
}

// Everything the captured run depends on other than the tables' contents.
std::vector<uint8_t> graph_signature(const rsrgpu_ctx* ctx) {
    std::vector<uint8_t> sig;
    const int dims[4] = { ctx->width, ctx->height, ctx->tile_w, ctx->tile_h };
    put_bytes(sig, dims);
    put_bytes(sig, ctx->ntris);
    const size_t packed_size = ctx->packed.size();
    put_bytes(sig, packed_size);
    for (size_t o : ctx->tab_ofs) put_bytes(sig, o);
    put_bytes(sig, ctx->vis_keys);
    put_bytes(sig, ctx->region_px);
    const uint8_t flags = uint8_t(ctx->any_dext) | uint8_t(ctx->any_inst) << 1 | uint8_t(frame_is_ext(ctx)) << 2;
    put_bytes(sig, flags);
    for (const auto& kv : ctx->host) {
        const HostBuffer& hb = kv.second;
        put_bytes(sig, kv.first);
        const uint8_t f = uint8_t(hb.in) | uint8_t(hb.out) << 1 | uint8_t(hb.early) << 2 | uint8_t(hb.late) << 3 |
                          uint8_t(hb.direct) << 4;
        put_bytes(sig, f);
        for (const TexRegion& r : hb.tex) { put_bytes(sig, r.offset); put_bytes(sig, r.edge); }
    }
    return sig;
}
#undef put_bytes

}  // namespace

int rsrgpu_submit(rsrgpu_ctx* ctx, const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates) {
    if (ctx == nullptr || (commands == nullptr && nbytes) || nstates < 0) return RSRGPU_EINVAL;
    if (ctx->ntiles == 0) return fail(ctx, RSRGPU_EINVAL, "rsrgpu_reset() has not been called");
    ctx->submitted = false;
    const int rc = decode_frame(ctx, commands, nbytes, states, nstates);
    if (rc) {
        drop_graph(ctx);
        ctx->graph_sig.clear();
        ctx->packed_dev.clear();
        return rc;
    }
    pack_tables(ctx);
    // A frame with the structure of the last one (the same sizes, kernels and
    // host-buffer routes) replays the captured graph; only tables that
    // changed are uploaded before it.
    std::vector<uint8_t> sig = graph_signature(ctx);
    if (ctx->gexec == nullptr || sig != ctx->graph_sig) {
        drop_graph(ctx);
        ctx->graph_sig.swap(sig);
    }
    ctx->tables_uploaded = ctx->packed == ctx->packed_dev;
    ctx->submitted = true;
    return 0;
}

namespace {

// Device tables a batch provides for one of its frames (packed for all frames).
struct ViewTables {
    DevState* states;
    DevDraw* draws;
    FrameOp* ops;
    GBufferDesc* gbufs;
    FrameCounters* counters;
    int4* super_rect;
    DevDrawExt* dext;         // per draw, for frames with instanced or OBJ1Program draws
};

// Allocates the frame's scratch and fills ctx->fv; `tables` (batches) points
// the frame's tables, counters and super-chunk rectangles elsewhere.
bool late_inputs(const rsrgpu_ctx* ctx);
int prepare_view(rsrgpu_ctx* ctx, const ViewTables* tables = nullptr) {
    const int ntris = ctx->ntris;
    const int nchunks = (ntris + kChunk - 1) / kChunk;
    const int nsupers = (ntris + kSuper - 1) / kSuper;
    const size_t nt = size_t(std::max(ntris, 1));
    uint8_t* tab = nullptr;
    if (tables == nullptr) {
        const size_t before = ctx->d_tables.cap;
        CK(ctx->d_tables.ensure(ctx->packed.size()), "alloc frame tables");
        if (ctx->d_tables.cap != before) ctx->packed_dev.clear();   // a new allocation holds nothing yet
        tab = ctx->d_tables.as<uint8_t>();
        CK(ctx->d_super.ensure(sizeof(int4) * std::max(nsupers, 1)), "alloc super rects");
        CK(ctx->d_counters.ensure(sizeof(FrameCounters)), "alloc counters");
    }
    CK(ctx->d_tris.ensure(sizeof(TriRecord) * nt), "alloc tris");
    CK(ctx->d_bin_rect.ensure(sizeof(uint64_t) * nt), "alloc bin_rect");
    CK(ctx->d_rec16.ensure(sizeof(uint32_t) * 2 * nt), "alloc rec16");
    CK(ctx->d_chunk.ensure(sizeof(int4) * std::max(nchunks, 1)), "alloc chunk rects");
    CK(ctx->d_clip_info.ensure(sizeof(ClipInfo) * nt), "alloc clip info");
    CK(ctx->d_clip_verts.ensure(sizeof(ClipVert) * size_t(ctx->clip_cap)), "alloc clip verts");
    CK(ctx->d_clip_poly.ensure(sizeof(int32_t) * size_t(ctx->clip_cap)), "alloc clip poly");
    CK(ctx->d_clip_src.ensure(sizeof(int32_t) * size_t(ctx->clip_cap)), "alloc clip src");
    CK(ctx->d_clip_fan.ensure(sizeof(uint64_t) * size_t(ctx->clip_cap)), "alloc clip fans");
    CK(ctx->d_bins.ensure(sizeof(TileBin) * size_t(ctx->ntiles)), "alloc bins");
    CK(ctx->d_pool.ensure(sizeof(uint32_t) * size_t(ctx->bin_cap)), "alloc bin pool");
    FrameView& fv = ctx->fv;
    fv.states = tables ? tables->states : reinterpret_cast<DevState*>(tab + ctx->tab_ofs[0]);
    fv.draws = tables ? tables->draws : reinterpret_cast<DevDraw*>(tab + ctx->tab_ofs[1]);
    fv.ndraws = int(ctx->draws.size());
    fv.ntris = ntris;
    fv.ops = tables ? tables->ops : reinterpret_cast<FrameOp*>(tab + ctx->tab_ofs[2]);
    fv.nops = int(ctx->ops.size());
    fv.gbufs = tables ? tables->gbufs : reinterpret_cast<GBufferDesc*>(tab + ctx->tab_ofs[3]);
    fv.width = ctx->width; fv.height = ctx->height;
    fv.tile_w = ctx->tile_w; fv.tile_h = ctx->tile_h;
    fv.tiles_x = ctx->tiles_x; fv.tiles_y = ctx->tiles_y; fv.ntiles = ctx->ntiles;
    fv.nchunks = nchunks; fv.nsupers = nsupers;
    fv.tris = ctx->d_tris.as<TriRecord>();
    fv.bin_rect = ctx->d_bin_rect.as<uint64_t>();
    fv.rec16 = ctx->d_rec16.as<uint32_t>();
    fv.chunk_rect = ctx->d_chunk.as<int4>();
    fv.super_rect = tables ? tables->super_rect : ctx->d_super.as<int4>();
    fv.clip_info = ctx->d_clip_info.as<ClipInfo>();
    fv.clip_verts = ctx->d_clip_verts.as<ClipVert>();
    fv.clip_poly = ctx->d_clip_poly.as<int32_t>();
    fv.clip_src = ctx->d_clip_src.as<int32_t>();
    fv.clip_fan_rect = ctx->d_clip_fan.as<uint64_t>();
    fv.clip_cap = ctx->clip_cap;
    fv.bins = ctx->d_bins.as<TileBin>();
    fv.bin_pool = ctx->d_pool.as<uint32_t>();
    fv.bin_cap = ctx->bin_cap;
    fv.counters = tables ? tables->counters : ctx->d_counters.as<FrameCounters>();
    fv.rcp_table = ctx->d_rcp.as<uint32_t>();
    fv.srgb_lut = ctx->d_srgb.as<uint8_t>();
    fv.region_px = std::min(ctx->region_px, std::min(ctx->tile_w, ctx->tile_h));
    if (tables == nullptr && fv.region_px > 16 && ctx->num_sms > 0) {
        // few, large tiles (config 1: 60 tiles of 64 px): raster CTAs of
        // 16x16-pixel regions, so every SM gets several (the region changes
        // which CTA draws a pixel, not what it draws)
        const int subs = ((ctx->tile_w + fv.region_px - 1) / fv.region_px) * ((ctx->tile_h + fv.region_px - 1) / fv.region_px);
        if (int64_t(ctx->ntiles) * subs < 2 * int64_t(ctx->num_sms)) fv.region_px = 16;
    }
    fv.vis_keys = ctx->vis_keys;
    fv.keys_resume_op = 0;
    fv.keys_resume_state_op = 0;
    fv.host_counters = tables == nullptr ? ctx->h_counters_dev : nullptr;
    fv.tile_queue = nullptr;   // a batch places its frames' queues (build_batch)
    fv.queue_cap = uint32_t(raster_blocks(fv));
    fv.taken = fv.counters;
    fv.slices = 1;
    fv.slice_keys = nullptr;
    fv.slice_done = nullptr;
    if (fv.vis_keys) {   // the raster pass jumps from the first draw to the op after the last
        int last_draw = -1, st_at = 0;
        for (int i = 0; i < int(ctx->ops.size()); ++i)
            if (ctx->ops[size_t(i)].kind == kOpDraw) last_draw = i;
        for (int i = 0; i <= last_draw; ++i)
            if (ctx->ops[size_t(i)].kind == kOpState) st_at = i;
        fv.keys_resume_op = last_draw + 1;
        fv.keys_resume_state_op = st_at;
    }
    fv.raster_phase = 0;
    fv.vis_own = nullptr;
    fv.vis_dep = nullptr;
    fv.ext = frame_is_ext(ctx) ? 1 : 0;
    fv.any_scissor = 0;
    for (const DevState& st : ctx->states) fv.any_scissor |= st.scissor_test;
    fv.dext = !ctx->any_dext ? nullptr : tables ? tables->dext : reinterpret_cast<DevDrawExt*>(tab + ctx->tab_ofs[4]);
    if (tables == nullptr) {
        // A frame with too few raster blocks to fill the GPU's visibility
        // slots (an opaque frame split in two launches, textures resident)
        // has each block's tile list swept by several CTAs, about two work
        // items per slot, at most eight per block.
        if (fv.vis_keys != 0 && !fv.ext && !fv.any_scissor && !late_inputs(ctx)) {
            const int blocks = std::max(1, raster_blocks(fv));
            fv.slices = std::min(8, std::max(1, (2 * vis_slots(fv) + blocks - 1) / blocks));
        }
        fv.queue_cap = uint32_t(raster_blocks(fv) * fv.slices);
        // the raster pass's work queue: raster blocks by cost bucket
        CK(ctx->d_queue.ensure(sizeof(uint32_t) * size_t(kCostBuckets) * size_t(fv.queue_cap)), "alloc tile queue");
        fv.tile_queue = ctx->d_queue.as<uint32_t>();
        if (fv.slices > 1) {
            CK(ctx->d_slice_keys.ensure(sizeof(unsigned long long) * size_t(fv.width) * size_t(fv.height)), "alloc slice keys");
            CK(ctx->d_slice_done.ensure(sizeof(uint32_t) * size_t(raster_blocks(fv))), "alloc slice counters");
            fv.slice_keys = ctx->d_slice_keys.as<unsigned long long>();
            fv.slice_done = ctx->d_slice_done.as<uint32_t>();
        }
    }
    return 0;
}

// whether the prepared frame's raster pass runs as the compiled split with
// per-pixel shading: opaque (vis_keys), no float stores, ManyProgram draws
// or scissor, and only state changes and TrueColor / depth stores after the
// last draw
bool pixel_split(const rsrgpu_ctx* ctx) {
    const FrameView& fv = ctx->fv;
    if (fv.vis_keys == 0 || fv.ext || fv.any_scissor) return false;
    for (size_t k = size_t(fv.keys_resume_op); k < ctx->ops.size(); ++k) {
        const int32_t kind = ctx->ops[k].kind;
        if (kind != kOpState && kind != kOpStoreTC && kind != kOpStoreDepth) return false;
    }
    return true;
}

// whether a registered host buffer only the raster pass reads comes with the run
bool late_inputs(const rsrgpu_ctx* ctx) {
    for (const auto& kv : ctx->host)
        if (kv.second.in && !kv.second.early) return true;
    return false;
}

// The frame's packed tables to the device, on `st` ahead of the run: one
// copy from pinned staging, which is refilled only after the previous copy
// from it has completed.  `capturing`: `st` is being captured by the caller.
int upload_tables(rsrgpu_ctx* ctx, cudaStream_t st, bool capturing) {
    if (ctx->tables_uploaded) return 0;
    const size_t n = ctx->packed.size();
    if (ctx->ev_tables_live) {
        CK(cudaEventSynchronize(ctx->ev_tables), "table staging");
        ctx->ev_tables_live = false;
    }
    if (n > ctx->h_tables_cap) {
        if (ctx->h_tables) cudaFreeHost(ctx->h_tables);
        ctx->h_tables = nullptr;
        ctx->h_tables_cap = 0;
        const size_t cap = std::max<size_t>(n, 64u << 10);
        CK(cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_tables), cap, cudaHostAllocDefault), "pinned table staging");
        ctx->h_tables_cap = cap;
    }
    std::memcpy(ctx->h_tables, ctx->packed.data(), n);
    ++ctx->stats.table_uploads;
    CK(cudaMemcpyAsync(ctx->d_tables.p, ctx->h_tables, n, cudaMemcpyHostToDevice, st), "H2D frame tables");
    if (!capturing) {
        CK(cudaEventRecord(ctx->ev_tables, st), "event");
        ctx->ev_tables_live = true;
        ctx->packed_dev = ctx->packed;
    } else {
        ctx->packed_dev.clear();   // the caller's graph copies them when it runs
    }
    ctx->tables_uploaded = true;
    return 0;
}

// allocations of a run, and the frame's tables (before the run's own stream
// work, which may be captured)
int prepare_run(rsrgpu_ctx* ctx, cudaStream_t st, bool capturing) {
    int rc = prepare_view(ctx);
    if (rc) return rc;
    rc = upload_tables(ctx, st, capturing);
    if (rc) return rc;
    if (ctx->fv.vis_keys != 0 && (late_inputs(ctx) || (!ctx->fv.ext && !ctx->fv.any_scissor)))
        CK(ctx->d_vis.ensure(size_t(ctx->fv.width) * size_t(ctx->fv.height) * 8u), "alloc visibility hand-over");
    return 0;
}

// the stream work of a run; `captured`: into a graph, whose timing and
// completion events must then be recorded as external event nodes
int record_run(rsrgpu_ctx* ctx, cudaStream_t st, bool captured) {
    const FrameView& fv = ctx->fv;
    const unsigned evflags = captured ? cudaEventRecordExternal : cudaEventRecordDefault;
    // Inputs that live in registered host buffers travel with every run.  The
    // ones triangle setup reads come first: from pinned, mapped memory in one
    // gather kernel (many small arrays cost one launch rather than a copy
    // each), others by copies.  Textures, which only the raster pass reads,
    // follow on the side stream while setup, binning and the visibility half
    // of a split raster pass run.
    GatherList gl{};
    bool any_late = false;
    for (auto& kv : ctx->host) {
        HostBuffer& hb = kv.second;
        if (!hb.in) continue;
        if (!hb.early) { any_late = true; continue; }
        if (hb.mapped != nullptr && gl.n < kMaxGather) {
            gl.src[gl.n] = static_cast<const uint8_t*>(hb.mapped);
            gl.dst[gl.n] = static_cast<uint8_t*>(hb.dev);
            gl.bytes[gl.n] = hb.bytes;
            gl.rows[gl.n] = 1;
            ++gl.n;
        } else {
            CK(cudaMemcpyAsync(hb.dev, hb.host, hb.bytes, cudaMemcpyHostToDevice, st), "H2D input");
        }
    }
    // the vertex data first (setup waits for it), then the textures on the
    // side stream (the link is shared: the gather goes first)
    if (gl.n > 0) CK(launch_gather(gl, st), "gather_kernel");
    if (any_late) {
        CK(cudaEventRecord(ctx->ev_fork, st), "event");
        CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0), "stream wait");
        for (auto& kv : ctx->host) {
            const HostBuffer& hb = kv.second;
            if (!hb.in || hb.early) continue;
            // the whole buffer unless every texture in it is a mip chain of
            // pinned, mapped memory (pageable memory goes by plain copies)
            bool whole = hb.tex.empty() || hb.mapped == nullptr || hb.tex.size() > size_t(kMaxGather);
            for (const TexRegion& r : hb.tex) whole = whole || r.edge < 4;
            if (whole) {
                CK(cudaMemcpyAsync(hb.dev, hb.host, hb.bytes, cudaMemcpyHostToDevice, ctx->side), "H2D texture");
                continue;
            }
            // square power-of-two textures: level 0 (one copy), then the used
            // half of each mip row, read from mapped memory by gather_kernel
            GatherList tg{};
            for (const TexRegion& r : hb.tex) {
                const size_t row = size_t(r.edge) * 16u;
                uint8_t* d = static_cast<uint8_t*>(hb.dev) + r.offset;
                const uint8_t* h = hb.host + r.offset;
                CK(cudaMemcpyAsync(d, h, row * size_t(r.edge), cudaMemcpyHostToDevice, ctx->side), "H2D texture level 0");
                if (tg.n < kMaxGather && r.edge >= 4) {
                    tg.src[tg.n] = static_cast<const uint8_t*>(hb.mapped) + r.offset + row * size_t(r.edge);
                    tg.dst[tg.n] = d + row * size_t(r.edge);
                    tg.bytes[tg.n] = row / 2;
                    tg.rows[tg.n] = uint32_t(r.edge);
                    tg.pitch[tg.n] = uint32_t(row);
                    ++tg.n;
                }
            }
            if (tg.n > 0) CK(launch_gather(tg, ctx->side), "gather_kernel (texture mip rows)");
        }
        CK(cudaEventRecord(ctx->ev_late, ctx->side), "event");
    }
    // Timing marks branch off st: ev0 (the frame's start) and ev1 (the raster
    // pass's start) are recorded on `marks` once st reaches them, and st
    // rejoins the branch before ev2, so no kernel waits on an event node.
    auto mark = [&](cudaEvent_t ev) {
        cudaError_t e = cudaEventRecord(ctx->ev_mark_fork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->marks, ctx->ev_mark_fork, 0);
        if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev, ctx->marks, evflags);
        return e;
    };
    CK(mark(ctx->ev0), "timing mark");
    // counters, super-chunk rectangles and slice keys, then setup launched
    // programmatically dependent on that launch (nothing may come between the
    // two on st)
    CK(launch_frame_init(fv, st), "frame_init_kernel");
    CK(launch_setup(fv, st, true), "setup_kernel");
    CK(launch_bin(fv, st), "bin_kernel");
    // A frame whose visibility is resolved by keys rasterises in two
    // launches: visibility (owners and depths handed over through d_vis),
    // then shading and stores.  Without float stores, ManyProgram draws or
    // scissor, the two are kernels compiled for their half (the visibility
    // kernel fits three CTAs per SM), the first taking its tiles from the
    // work queue; otherwise both are the frame's raster kernel, split only
    // to let textures still on their way arrive during the visibility launch.
    const bool compiled_split = fv.vis_keys != 0 && !fv.ext && !fv.any_scissor;
    const bool split = fv.vis_keys != 0 && (any_late || compiled_split);
    CK(mark(ctx->ev1), "timing mark");
    if (split) {
        FrameView f = fv;
        f.vis_own = ctx->d_vis.as<uint32_t>();
        f.vis_dep = reinterpret_cast<float*>(f.vis_own + size_t(fv.width) * size_t(fv.height));
        f.raster_phase = 1;
        // With textures on their way the visibility launch runs one CTA per
        // block (CTAs retire and leave SMs to the texture gather); the
        // shading launch always does.
        if (!compiled_split || any_late) f.tile_queue = nullptr;
        CK(launch_raster(f, st, compiled_split ? 1 : 0), "raster_kernel (visibility)");
        if (any_late) CK(cudaStreamWaitEvent(st, ctx->ev_late, 0), "stream wait");
        f.raster_phase = 2;
        f.tile_queue = nullptr;
        // A frame whose ops after the last draw are state changes and
        // TrueColor / depth stores is shaded one thread per pixel, launched
        // programmatically dependent on the visibility launch; with textures
        // arriving during the frame the quad kernel shades (measured faster
        // there: 0.253 against 0.295 ms per end-to-end headline frame).
        const int shade = any_late ? (compiled_split ? 2 : 0) : pixel_split(ctx) ? 4 : compiled_split ? 2 : 0;
        CK(launch_raster(f, st, shade), "raster_kernel (shading)");
    } else {
        if (any_late) CK(cudaStreamWaitEvent(st, ctx->ev_late, 0), "stream wait");
        CK(launch_raster(fv, st), "raster_kernel");
    }
    CK(cudaEventRecord(ctx->ev_mark_join, ctx->marks), "event");
    CK(cudaStreamWaitEvent(st, ctx->ev_mark_join, 0), "stream wait");
    CK(cudaEventRecordWithFlags(ctx->ev2, st, evflags), "event");
    // outputs written in place need no copy back
    bool copies = false;
    for (auto& kv : ctx->host)
        if (kv.second.out) {
            CK(cudaMemcpyAsync(const_cast<uint8_t*>(kv.second.host), kv.second.dev, kv.second.bytes, cudaMemcpyDeviceToHost, st), "D2H output");
            copies = true;
        }
    // the run's completion: after the output copies, or the end of the raster
    // pass (the counters reach h_counters from the raster pass,
    // FrameView::host_counters)
    if (copies) CK(cudaEventRecordWithFlags(ctx->ev3, st, evflags), "event");
    ctx->ev_done = copies ? ctx->ev3 : ctx->ev2;
    ctx->stats.gpu_launches = 4 + (gl.n > 0 ? 1 : 0) + (split ? 1 : 0);
    return 0;
}

}  // namespace

namespace {
// One run on ctx->run_stream.  Unless the stream is being captured by the
// caller, or pageable host memory has to be copied, the work is captured
// once into a CUDA graph and replayed.
int run_frame(rsrgpu_ctx* ctx) {
    cudaStream_t st = ctx->run_stream;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cs), "stream capture status");
    bool graph = cs == cudaStreamCaptureStatusNone;
    for (const auto& kv : ctx->host)
        if ((kv.second.in || kv.second.out) && kv.second.mapped == nullptr) graph = false;
    if (!graph) {
        int rc = prepare_run(ctx, st, cs != cudaStreamCaptureStatusNone);
        return rc ? rc : record_run(ctx, st, false);
    }
    if (ctx->gexec == nullptr) {
        int rc = prepare_run(ctx, st, false);
        if (rc) return rc;
        CK(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
        ++ctx->stats.graph_captures;
        rc = record_run(ctx, ctx->cap, true);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->cap, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        CK(e, "end capture");
        ctx->graph = g;
        const cudaError_t ie = cudaGraphInstantiate(&ctx->gexec, g, 0);
        if (ie != cudaSuccess) { drop_graph(ctx); return cuda_fail(ctx, ie, "graph instantiate"); }
    } else {
        int rc = upload_tables(ctx, st, false);   // a resubmitted frame of the same structure
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(ctx->gexec, st), "graph launch");
    return 0;
}
}  // namespace

int rsrgpu_run(rsrgpu_ctx* ctx, void* stream) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (!ctx->submitted) return fail(ctx, RSRGPU_EINVAL, "nothing submitted");
    ctx->run_stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    int rc = run_frame(ctx);
    if (rc) return rc;
    ctx->ran = true;
    return 0;
}

int rsrgpu_wait(rsrgpu_ctx* ctx, int timeout_ms) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (!ctx->ran) return 0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        const auto t0 = std::chrono::steady_clock::now();
        while (true) {
            cudaError_t q = cudaEventQuery(ctx->ev_done);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return cuda_fail(ctx, q, "run");
            if (timeout_ms >= 0) {
                const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
                if (ms > timeout_ms) return fail(ctx, RSRGPU_ETIMEOUT, "rsrgpu_wait timed out after %d ms", timeout_ms);
            }
            std::this_thread::yield();
        }
        const FrameCounters c = *ctx->h_counters;
        if (c.overflow == 0) return 0;
        if (c.overflow & 4u) return fail(ctx, RSRGPU_EINVAL, "a vertex index lies outside its attribute buffer");
        // a capacity was too small: grow from the counts the frame requested and run again
        if (c.overflow & 1u) ctx->clip_cap = std::max<uint32_t>(ctx->clip_cap * 2, c.clip_verts + c.clip_verts / 4 + 1024);
        if (c.overflow & 2u) ctx->bin_cap = std::max<uint32_t>(ctx->bin_cap * 2, c.bin_used + c.bin_used / 4 + 4096);
        if (ctx->clip_cap > (1u << 28) || ctx->bin_cap > (1u << 30))
            return fail(ctx, RSRGPU_ECAPACITY, "frame needs %u clipped vertices and %u tile entries", c.clip_verts, c.bin_used);
        drop_graph(ctx);   // its scratch pointers and capacities change
        int rc = run_frame(ctx);
        if (rc) return rc;
    }
    return fail(ctx, RSRGPU_ECAPACITY, "capacity growth did not converge");
}

int rsrgpu_last_timings(rsrgpu_ctx* ctx, float* total_ms, float* raster_ms) {
    if (ctx == nullptr || !ctx->ran) return RSRGPU_EINVAL;
    float t = 0, r = 0;
    CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev2), "elapsed");
    CK(cudaEventElapsedTime(&r, ctx->ev1, ctx->ev2), "elapsed");
    if (total_ms) *total_ms = t;
    if (raster_ms) *raster_ms = r;
    return 0;
}

int rsrgpu_get_stats(rsrgpu_ctx* ctx, rsrgpu_stats* out) {
    if (ctx == nullptr || out == nullptr) return RSRGPU_EINVAL;
    *out = ctx->stats;
    out->total_tiles = ctx->ntiles;
    out->primitives_submitted = ctx->ntris;
    return 0;
}

int rsrgpu_dump_tiles(rsrgpu_ctx* ctx, uint8_t* out, size_t capacity, size_t* needed) {
    if (ctx == nullptr || needed == nullptr || !ctx->ran) return RSRGPU_EINVAL;
    CK(cudaStreamSynchronize(ctx->run_stream), "sync");
    const int nt = ctx->ntris, ntiles = ctx->ntiles;
    std::vector<TileBin> bins(static_cast<size_t>(ntiles));
    std::vector<uint32_t> rec16(static_cast<size_t>(2) * size_t(std::max(nt, 1)));
    std::vector<ClipInfo> ci(static_cast<size_t>(std::max(nt, 1)));
    const FrameCounters c = *ctx->h_counters;
    std::vector<uint32_t> pool(static_cast<size_t>(c.bin_used));
    std::vector<int32_t> poly(size_t(c.clip_verts) + 1), src(size_t(c.clip_verts) + 1);
    CK(cudaMemcpy(bins.data(), ctx->d_bins.p, sizeof(TileBin) * bins.size(), cudaMemcpyDeviceToHost), "D2H bins");
    if (nt) {
        CK(cudaMemcpy(rec16.data(), ctx->d_rec16.p, sizeof(uint32_t) * 2 * size_t(nt), cudaMemcpyDeviceToHost), "D2H rec16");
        CK(cudaMemcpy(ci.data(), ctx->d_clip_info.p, sizeof(ClipInfo) * size_t(nt), cudaMemcpyDeviceToHost), "D2H clip info");
    }
    if (c.bin_used) CK(cudaMemcpy(pool.data(), ctx->d_pool.p, sizeof(uint32_t) * pool.size(), cudaMemcpyDeviceToHost), "D2H pool");
    if (c.clip_verts) {
        CK(cudaMemcpy(poly.data(), ctx->d_clip_poly.p, sizeof(int32_t) * c.clip_verts, cudaMemcpyDeviceToHost), "D2H clip poly");
        CK(cudaMemcpy(src.data(), ctx->d_clip_src.p, sizeof(int32_t) * c.clip_verts, cudaMemcpyDeviceToHost), "D2H clip src");
    }
    // canonical clipped-vertex numbering: polygons in source-triangle order
    std::vector<int32_t> canon(size_t(std::max(nt, 1)), 0);
    int32_t running = 0;
    for (int g = 0; g < nt; ++g) if (ci[g].nverts > 0) { canon[g] = running; running += ci[g].nverts; }
    std::vector<uint8_t> all;
    auto put8 = [&](std::vector<uint8_t>& v, uint8_t x) { v.push_back(x); };
    auto put16 = [&](std::vector<uint8_t>& v, uint16_t x) { v.push_back(x & 0xff); v.push_back(x >> 8); };
    auto put32 = [&](std::vector<uint8_t>& v, uint32_t x) { for (int i = 0; i < 4; ++i) v.push_back((x >> (8 * i)) & 0xff); };
    int64_t total_rec = 0, total_clip = 0, max_rec = 0;
    for (int t = 0; t < ntiles; ++t) {
        std::vector<uint8_t> one;
        const TileBin b = bins[t];
        total_rec += b.inl_cnt; total_clip += b.clip_cnt; max_rec = std::max<int64_t>(max_rec, b.inl_cnt + b.clip_cnt);
        uint32_t ic = 0, cc = 0;
        for (const FrameOp& o : ctx->ops) {
            if (o.kind == kOpState) { put8(one, RSRGPU_CMD_STATE); put32(one, uint32_t(o.ordinal)); }
            else if (o.kind == kOpClear) { put8(one, RSRGPU_CMD_CLEAR); put8(one, uint8_t(o.arg)); }
            else if (o.kind == kOpStoreTC) { put8(one, RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC); put8(one, uint8_t(o.arg)); }
            else if (o.kind == kOpStoreDepth) { put8(one, RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP); }
            else if (o.kind == kOpStoreGBuffer) { put8(one, RSRGPU_CMD_STORE_GBUFFER); }
            else if (o.kind == kOpStoreFP) { put8(one, RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP); }
            else if (o.kind == kOpStoreHalfFP) { put8(one, RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP); }
            else if (o.kind == kOpStoreQuadsFP) { put8(one, RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP); }
            else if (o.kind == kOpDraw) {
                const DevDraw& d = ctx->draws[size_t(o.arg)];
                const DevDrawExt& di = ctx->dext[size_t(o.arg)];
                const uint32_t endg = uint32_t(d.first_tri + d.ntris);
                bool opened = false;
                while (ic < b.inl_cnt && pool[b.inl_off + ic] < endg) {
                    const uint32_t g = pool[b.inl_off + ic++];
                    if (!opened) {
                        put8(one, di.per_inst > 0 ? RSRGPU_CMD_DRAW_INLINE_INSTANCED : RSRGPU_CMD_DRAW_INLINE);
                        opened = true;
                    }
                    // an instanced record starts with its instance id (rglv_gpu_impl.hxx:488-494)
                    if (di.per_inst > 0) put16(one, uint16_t((g - uint32_t(d.first_tri)) / uint32_t(di.per_inst)));
                    put16(one, uint16_t(rec16[2 * g] & 0xffff));
                    put16(one, uint16_t(rec16[2 * g] >> 16));
                    put16(one, uint16_t(rec16[2 * g + 1]));
                }
                if (opened) put16(one, 0xffff);
                while (cc < b.clip_cnt) {
                    const uint32_t e = pool[b.clip_off + cc];
                    const int32_t pb = poly[e];
                    const int32_t g = src[pb];
                    if (uint32_t(g) >= endg) break;
                    ++cc;
                    const int32_t bi = canon[g];
                    const int32_t vi = int32_t(e) - pb;
                    put8(one, RSRGPU_CMD_CLIPPED_TRI);
                    put16(one, uint16_t((bi + 0) | (ci[g].backfacing ? 0x8000 : 0)));
                    put16(one, uint16_t(bi + vi));
                    put16(one, uint16_t(bi + vi + 1));
                }
            }
        }
        put8(one, RSRGPU_CMD_EOF);
        put32(all, uint32_t(one.size()));
        all.insert(all.end(), one.begin(), one.end());
    }
    ctx->stats.total_tile_records = total_rec;
    ctx->stats.total_clipped_records = total_clip;
    ctx->stats.max_tile_records = max_rec;
    *needed = all.size();
    if (out && capacity >= all.size()) std::memcpy(out, all.data(), all.size());
    return 0;
}

int rsrgpu_dump_clipped(rsrgpu_ctx* ctx, rsrgpu_clipped_vertex* out, int capacity, int* count) {
    if (ctx == nullptr || count == nullptr || !ctx->ran) return RSRGPU_EINVAL;
    CK(cudaStreamSynchronize(ctx->run_stream), "sync");
    const int nt = ctx->ntris;
    std::vector<ClipInfo> ci(static_cast<size_t>(std::max(nt, 1)));
    if (nt) CK(cudaMemcpy(ci.data(), ctx->d_clip_info.p, sizeof(ClipInfo) * size_t(nt), cudaMemcpyDeviceToHost), "D2H clip info");
    const FrameCounters c = *ctx->h_counters;
    std::vector<ClipVert> verts(size_t(c.clip_verts) + 1);
    if (c.clip_verts) CK(cudaMemcpy(verts.data(), ctx->d_clip_verts.p, sizeof(ClipVert) * c.clip_verts, cudaMemcpyDeviceToHost), "D2H clip verts");
    int n = 0;
    size_t d = 0;
    for (int g = 0; g < nt; ++g) {
        if (ci[g].nverts <= 0) continue;
        while (d + 1 < ctx->draws.size() && ctx->draws[d + 1].first_tri <= g) ++d;
        const int nvary = ctx->states[size_t(ctx->draws[d].state)].nvary;
        for (int i = 0; i < ci[g].nverts; ++i, ++n) {
            if (out && n < capacity) {
                std::memset(&out[n], 0, sizeof(out[n]));
                const ClipVert& v = verts[size_t(ci[g].vbase + i)];
                std::memcpy(out[n].coord, v.coord, 16);
                for (int k = 0; k < nvary && k < kMaxVary; ++k) out[n].data[k] = v.vary[k];
            }
        }
    }
    *count = n;
    return 0;
}

int rsrgpu_shade_plain(rsrgpu_ctx* ctx, const rsrgpu_gbuffer* gbuffer, const float inv_view_proj[16],
                       const float eye[3], const rsrgpu_light* lights, int nlights,
                       const float background[3], uint32_t* out_srgb, float* out_linear, void* stream) {
    if (ctx == nullptr || gbuffer == nullptr || inv_view_proj == nullptr || eye == nullptr || background == nullptr)
        return RSRGPU_EINVAL;
    if (nlights < 0 || nlights > 256) return fail(ctx, RSRGPU_EINVAL, "1..256 lights");
    if (gbuffer->width <= 0 || gbuffer->height <= 0) return fail(ctx, RSRGPU_EINVAL, "empty G-buffer");
    const size_t npx = size_t(gbuffer->width) * size_t(gbuffer->height);
    const void* ins[6] = { gbuffer->depth, gbuffer->normal_x, gbuffer->normal_y, gbuffer->normal_z, gbuffer->albedo, lights };
    const size_t need[6] = { npx * 4, npx * 2, npx * 2, npx * 2, npx * 4, size_t(nlights) * sizeof(rsrgpu_light) };
    rsrgpu_gbuffer g = *gbuffer;
    void* dp = nullptr;
    size_t avail = 0;
    for (int k = 0; k < 6; ++k) {
        if (need[k] == 0) continue;
        int rc = resolve(ctx, ins[k], kProbe, &dp, "deferred input", &avail);
        if (rc) return rc;
        if (dp == nullptr || avail < need[k]) return fail(ctx, RSRGPU_EINVAL, "deferred input %d holds %zu bytes, needs %zu", k, avail, need[k]);
        if (dp != ins[k]) return fail(ctx, RSRGPU_EINVAL, "rsrgpu_shade_plain takes device pointers");
    }
    const void* outs[2] = { out_srgb, out_linear };
    const size_t oneed[2] = { npx * 4, npx * 12 };
    for (int k = 0; k < 2; ++k) {
        if (outs[k] == nullptr) continue;
        int rc = resolve(ctx, outs[k], kProbe, &dp, "deferred output", &avail);
        if (rc) return rc;
        if (dp != outs[k] || avail < oneed[k]) return fail(ctx, RSRGPU_EINVAL, "deferred output %d: device pointer with %zu bytes needed", k, oneed[k]);
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_shade_plain(g, inv_view_proj, eye, lights, nlights, background, out_srgb, out_linear,
                          ctx->d_srgb.as<uint8_t>(), st), "shade_plain_kernel");
    return 0;
}

namespace {
int check_device_input(rsrgpu_ctx* ctx, const void* p, size_t need, size_t align, const char* what) {
    void* dp = nullptr;
    size_t avail = 0;
    int rc = resolve(ctx, p, kProbe, &dp, what, &avail);
    if (rc) return rc;
    if (dp == nullptr || dp != p || avail < need || (reinterpret_cast<uintptr_t>(p) % align))
        return fail(ctx, RSRGPU_EINVAL, "%s: device pointer with %zu bytes, %zu-byte aligned, needed", what, need, align);
    return 0;
}
}  // namespace

int rsrgpu_texture_from_rgba8(rsrgpu_ctx* ctx, const uint8_t* rgba8, int width, int height, int premultiply,
                              float* texels, size_t texel_capacity, int* power, void* stream) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (width <= 0 || height <= 0) return fail(ctx, RSRGPU_EINVAL, "texture of %dx%d pixels", width, height);
    const int p = texture_power(width, height);
    const size_t npx = size_t(width) * size_t(height);
    const size_t need = p >= 0 ? 2 * npx : npx;
    if (texel_capacity < need) return fail(ctx, RSRGPU_EINVAL, "texture needs %zu texels, room for %zu", need, texel_capacity);
    int rc = check_device_input(ctx, rgba8, npx * 4, 4, "RGBA8 pixels");
    if (rc == 0) rc = check_device_input(ctx, texels, need * 16, 16, "texels");
    if (rc) return rc;
    if (ctx->num_sms == 0)
        CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    if (p >= 0) CK(launch_texture_chain(texels, rgba8, width, premultiply, st), "mip_block_kernel");
    else CK(launch_rgba8_to_float(rgba8, texels, npx, premultiply, ctx->num_sms, st), "rgba8_to_float_kernel");
    if (power) *power = p;
    return 0;
}

int rsrgpu_texture_mipmap(rsrgpu_ctx* ctx, float* texels, int width, int height, size_t texel_capacity,
                          int* power, void* stream) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (width <= 0 || height <= 0) return fail(ctx, RSRGPU_EINVAL, "texture of %dx%d pixels", width, height);
    const int p = texture_power(width, height);
    if (power) *power = p;
    if (p < 0) return 0;   // no chain: the texture stays as it is
    const size_t need = 2 * size_t(width) * size_t(height);
    if (texel_capacity < need) return fail(ctx, RSRGPU_EINVAL, "the mip chain needs %zu texels, room for %zu", need, texel_capacity);
    int rc = check_device_input(ctx, texels, need * 16, 16, "texels");
    if (rc) return rc;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_texture_chain(texels, nullptr, width, 0, st), "mip_block_kernel");
    return 0;
}

namespace {
// a float canvas of device memory: width x height pixels of `unit` bytes,
// stride >= width, 16-byte aligned
int float_canvas(rsrgpu_ctx* ctx, const rsrgpu_fp_canvas* c, size_t unit, const char* what, FloatCanvasView& v) {
    if (c == nullptr || c->data == nullptr || c->width <= 0 || c->height <= 0 || c->stride < c->width)
        return fail(ctx, RSRGPU_EINVAL, "%s: canvas needs data, a positive size and stride >= width", what);
    const size_t bytes = ((size_t(c->height) - 1) * size_t(c->stride) + size_t(c->width)) * unit;
    int rc = check_device_input(ctx, c->data, bytes, 16, what);
    if (rc) return rc;
    v.data = reinterpret_cast<float4*>(c->data);
    v.width = c->width; v.height = c->height; v.stride = c->stride;
    return 0;
}
size_t canvas_end(const FloatCanvasView& v, size_t unit) {
    return reinterpret_cast<uintptr_t>(v.data) + ((size_t(v.height) - 1) * size_t(v.stride) + size_t(v.width)) * unit;
}
bool canvases_overlap(const FloatCanvasView& a, const FloatCanvasView& b) {
    return reinterpret_cast<uintptr_t>(a.data) < canvas_end(b, 16) && reinterpret_cast<uintptr_t>(b.data) < canvas_end(a, 16);
}
}  // namespace

int rsrgpu_kawase_blur(rsrgpu_ctx* ctx, const rsrgpu_fp_canvas* src, const rsrgpu_fp_canvas* dst, int dist, void* stream) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (dist < 0 || dist > (1 << 20)) return fail(ctx, RSRGPU_EINVAL, "kawase distance %d: 0 .. 2^20", dist);
    FloatCanvasView s{}, d{};
    int rc = float_canvas(ctx, src, 16, "kawase source", s);
    if (rc == 0) rc = float_canvas(ctx, dst, 16, "kawase destination", d);
    if (rc) return rc;
    if (s.width != d.width || s.height != d.height)
        return fail(ctx, RSRGPU_EINVAL, "kawase canvases differ in size (%dx%d, %dx%d)", s.width, s.height, d.width, d.height);
    if (canvases_overlap(s, d)) return fail(ctx, RSRGPU_EINVAL, "kawase source and destination overlap");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_kawase(s, d, dist, st), "kawase_kernel");
    return 0;
}

int rsrgpu_kawase_chain(rsrgpu_ctx* ctx, const rsrgpu_fp_canvas* src, const rsrgpu_fp_canvas* tmp_a,
                        const rsrgpu_fp_canvas* tmp_b, int intensity, int* result, void* stream) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (intensity < 0 || intensity > 64) return fail(ctx, RSRGPU_EINVAL, "kawase intensity %d: 0 .. 64", intensity);
    if (result) *result = 0;
    if (intensity == 0) return 0;
    // pass k blurs with distance k: src -> a, a -> b, b -> a, ...
    const rsrgpu_fp_canvas* from = src;
    const rsrgpu_fp_canvas* to = tmp_a;
    for (int k = 0; k < intensity; ++k) {
        int rc = rsrgpu_kawase_blur(ctx, from, to, k, stream);
        if (rc) return rc;
        from = to;
        to = (to == tmp_a) ? tmp_b : tmp_a;
    }
    if (result) *result = (from == tmp_a) ? 1 : 2;
    return 0;
}

int rsrgpu_glow(rsrgpu_ctx* ctx, const rsrgpu_qfloat4_canvas* image, const rsrgpu_fp_canvas* blur,
                const rsrgpu_truecolor_canvas* out, int srgb, void* stream) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (image == nullptr || out == nullptr) return fail(ctx, RSRGPU_EINVAL, "glow needs an image and an output");
    const int w = image->width, h = image->height;
    if (w <= 0 || h <= 0 || (w & 3) || (h & 1))
        return fail(ctx, RSRGPU_EINVAL, "glow image %dx%d: width a multiple of 4, height of 2", w, h);
    // the quads canvas: (h/2) rows of (w/2) 64-byte quads
    rsrgpu_fp_canvas iq{ image->data, w / 2, h / 2, image->stride, 0 };
    FloatCanvasView iv{}, bv{};
    int rc = float_canvas(ctx, &iq, 64, "glow image", iv);
    if (rc == 0) rc = float_canvas(ctx, blur, 16, "glow blur", bv);
    if (rc) return rc;
    if (bv.width < w / 2 || bv.height < h / 2)
        return fail(ctx, RSRGPU_EINVAL, "glow blur canvas %dx%d is smaller than %dx%d", bv.width, bv.height, w / 2, h / 2);
    if (out->width != w || out->height != h || out->stride < w || (out->stride & 1))
        return fail(ctx, RSRGPU_EINVAL, "glow output must be %dx%d with an even stride >= width", w, h);
    const size_t obytes = ((size_t(h) - 1) * size_t(out->stride) + size_t(w)) * 4;
    rc = check_device_input(ctx, out->data, obytes, 8, "glow output");
    if (rc) return rc;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_glow(iv, bv, out->data, out->stride, w, h, srgb ? ctx->d_srgb.as<uint8_t>() : nullptr, st), "glow_kernel");
    return 0;
}

int rsrgpu_mlp_forward(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp, const uint16_t* features, int n,
                       float* out, void* stream) {
    if (ctx == nullptr || mlp == nullptr || n < 0) return RSRGPU_EINVAL;
    if (n == 0) return 0;
    struct { const void* p; size_t bytes; size_t align; const char* what; } ins[] = {
        { mlp->w1, 64 * 32 * 2, 16, "w1" }, { mlp->w2, 64 * 64 * 2, 16, "w2" }, { mlp->w3, 64 * 64 * 2, 16, "w3" },
        { mlp->w4, 16 * 64 * 2, 16, "w4" }, { mlp->b1, 64 * 4, 4, "b1" }, { mlp->b2, 64 * 4, 4, "b2" },
        { mlp->b3, 64 * 4, 4, "b3" }, { mlp->b4, 16 * 4, 4, "b4" },
        { features, size_t(n) * 64, 16, "features" }, { out, size_t(n) * 12, 4, "mlp output" } };
    for (const auto& in : ins) {
        int rc = check_device_input(ctx, in.p, in.bytes, in.align, in.what);
        if (rc) return rc;
    }
    if (ctx->num_sms == 0)
        CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
    if (ctx->h_mlp_err == nullptr) {
        CK(ctx->d_mlp_err.ensure(sizeof(int)), "alloc mlp error flag");
        CK(cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_mlp_err), sizeof(int), cudaHostAllocDefault), "alloc pinned flag");
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(cudaMemsetAsync(ctx->d_mlp_err.p, 0, sizeof(int), st), "memset mlp error");
    CK(launch_mlp_forward(*mlp, features, n, out, ctx->d_mlp_err.as<int>(), ctx->num_sms, st), "mlp_forward_kernel");
    CK(cudaMemcpyAsync(ctx->h_mlp_err, ctx->d_mlp_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H mlp error");
    CK(cudaStreamSynchronize(st), "mlp sync");
    if (*ctx->h_mlp_err) return fail(ctx, RSRGPU_ETIMEOUT, "tensor-core MMA did not complete (bounded wait expired)");
    return 0;
}

namespace {
int check_mlp(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp) {
    struct { const void* p; size_t bytes; size_t align; const char* what; } ins[] = {
        { mlp->w1, 64 * 32 * 2, 16, "w1" }, { mlp->w2, 64 * 64 * 2, 16, "w2" }, { mlp->w3, 64 * 64 * 2, 16, "w3" },
        { mlp->w4, 16 * 64 * 2, 16, "w4" }, { mlp->b1, 64 * 4, 4, "b1" }, { mlp->b2, 64 * 4, 4, "b2" },
        { mlp->b3, 64 * 4, 4, "b3" }, { mlp->b4, 16 * 4, 4, "b4" } };
    for (const auto& in : ins) {
        int rc = check_device_input(ctx, in.p, in.bytes, in.align, in.what);
        if (rc) return rc;
    }
    if (ctx->num_sms == 0)
        CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
    if (ctx->h_mlp_err == nullptr) {
        CK(ctx->d_mlp_err.ensure(sizeof(int)), "alloc mlp error flag");
        CK(cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_mlp_err), sizeof(int), cudaHostAllocDefault), "alloc pinned flag");
    }
    return 0;
}
}  // namespace

int rsrgpu_mlp_grad(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp, const uint16_t* features, const float* targets,
                    int nsamples, const int32_t* index, int batch, float* grad, float* loss, void* stream) {
    if (ctx == nullptr || mlp == nullptr || nsamples <= 0 || batch <= 0) return RSRGPU_EINVAL;
    int rc = check_mlp(ctx, mlp);
    if (rc) return rc;
    struct { const void* p; size_t bytes; size_t align; const char* what; } ins[] = {
        { features, size_t(nsamples) * 64, 16, "features" }, { targets, size_t(nsamples) * 12, 4, "targets" },
        { index, size_t(batch) * 4, 4, "batch index" }, { grad, RSRGPU_MLP_PARAMS * 4, 4, "gradient" },
        { loss, 4, 4, "loss" } };
    for (const auto& in : ins) {
        rc = check_device_input(ctx, in.p, in.bytes, in.align, in.what);
        if (rc) return rc;
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(cudaMemsetAsync(grad, 0, RSRGPU_MLP_PARAMS * 4, st), "memset grad");
    CK(cudaMemsetAsync(loss, 0, 4, st), "memset loss");
    CK(cudaMemsetAsync(ctx->d_mlp_err.p, 0, sizeof(int), st), "memset mlp error");
    CK(launch_mlp_train(*mlp, features, targets, index, batch, grad, loss, ctx->d_mlp_err.as<int>(), ctx->num_sms, st), "mlp_train_kernel");
    CK(cudaMemcpyAsync(ctx->h_mlp_err, ctx->d_mlp_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H mlp error");
    CK(cudaStreamSynchronize(st), "mlp sync");
    if (*ctx->h_mlp_err) return fail(ctx, RSRGPU_ETIMEOUT, "tensor-core MMA did not complete (bounded wait expired)");
    return 0;
}

int rsrgpu_mlp_adam(rsrgpu_ctx* ctx, float* params, const float* grad, float* m, float* v, int step,
                    float lr, uint16_t* weights_bf16, float* biases, void* stream) {
    if (ctx == nullptr || step < 1) return RSRGPU_EINVAL;
    struct { const void* p; size_t bytes; const char* what; } ins[] = {
        { params, RSRGPU_MLP_PARAMS * 4, "params" }, { grad, RSRGPU_MLP_PARAMS * 4, "grad" },
        { m, RSRGPU_MLP_PARAMS * 4, "adam m" }, { v, RSRGPU_MLP_PARAMS * 4, "adam v" },
        { weights_bf16, RSRGPU_MLP_WEIGHTS * 2, "bf16 weights" },
        { biases, (RSRGPU_MLP_PARAMS - RSRGPU_MLP_WEIGHTS) * 4, "biases" } };
    for (const auto& in : ins) {
        int rc = check_device_input(ctx, in.p, in.bytes, 4, in.what);
        if (rc) return rc;
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_adam(params, grad, m, v, RSRGPU_MLP_PARAMS, RSRGPU_MLP_WEIGHTS, lr, 0.9f, 0.999f, 1e-8f, step,
                   weights_bf16, biases, st), "adam_kernel");
    return 0;
}

namespace {
// device G-buffer planes and lights of a deferred call, checked for size
int check_gbuffer(rsrgpu_ctx* ctx, const rsrgpu_gbuffer* gb, const rsrgpu_light* lights, int nlights) {
    if (nlights < 0 || nlights > 256) return fail(ctx, RSRGPU_EINVAL, "0..256 lights");
    if (gb->width <= 0 || gb->height <= 0) return fail(ctx, RSRGPU_EINVAL, "empty G-buffer");
    const size_t npx = size_t(gb->width) * size_t(gb->height);
    struct { const void* p; size_t bytes; size_t align; const char* what; } ins[] = {
        { gb->depth, npx * 4, 4, "G-buffer depth" }, { gb->normal_x, npx * 2, 2, "G-buffer normal x" },
        { gb->normal_y, npx * 2, 2, "G-buffer normal y" }, { gb->normal_z, npx * 2, 2, "G-buffer normal z" },
        { gb->albedo, npx * 4, 4, "G-buffer albedo" }, { lights, size_t(nlights) * sizeof(rsrgpu_light), 4, "lights" } };
    for (const auto& in : ins) {
        if (in.bytes == 0) continue;
        int rc = check_device_input(ctx, in.p, in.bytes, in.align, in.what);
        if (rc) return rc;
    }
    return 0;
}
int check_device_output(rsrgpu_ctx* ctx, void* p, size_t need, size_t align, const char* what) {
    if (p == nullptr) return 0;
    void* dp = nullptr;
    size_t avail = 0;
    int rc = resolve(ctx, p, kProbe, &dp, what, &avail);
    if (rc) return rc;
    if (dp != p || avail < need || (reinterpret_cast<uintptr_t>(p) % align))
        return fail(ctx, RSRGPU_EINVAL, "%s: device pointer with %zu bytes, %zu-byte aligned, needed", what, need, align);
    return 0;
}
}  // namespace

int rsrgpu_shade_learned(rsrgpu_ctx* ctx, const rsrgpu_mlp* mlp, const rsrgpu_gbuffer* gbuffer,
                         const float inv_view_proj[16], const float eye[3], const rsrgpu_light* lights, int nlights,
                         const float background[3], float max_tile_mse, uint32_t* out_srgb, float* out_linear,
                         uint8_t* tile_status, float* tile_mse, void* stream) {
    if (ctx == nullptr || mlp == nullptr || gbuffer == nullptr || inv_view_proj == nullptr || eye == nullptr ||
        background == nullptr)
        return RSRGPU_EINVAL;
    if (max_tile_mse != max_tile_mse) return fail(ctx, RSRGPU_EINVAL, "max_tile_mse is NaN");
    int rc = check_mlp(ctx, mlp);
    if (rc) return rc;
    rc = check_gbuffer(ctx, gbuffer, lights, nlights);
    if (rc) return rc;
    const size_t npx = size_t(gbuffer->width) * size_t(gbuffer->height);
    const size_t tiles = size_t((gbuffer->width + RSRGPU_SHADE_TILE - 1) / RSRGPU_SHADE_TILE) *
                         size_t((gbuffer->height + RSRGPU_SHADE_TILE - 1) / RSRGPU_SHADE_TILE);
    if ((rc = check_device_output(ctx, out_srgb, npx * 4, 4, "sRGB output")) ||
        (rc = check_device_output(ctx, out_linear, npx * 12, 4, "linear output")) ||
        (rc = check_device_output(ctx, tile_status, tiles, 1, "tile status")) ||
        (rc = check_device_output(ctx, tile_mse, tiles * 4, 4, "tile mse")))
        return rc;
    if (ctx->d_learn_err.p == nullptr) {   // [0] error flag, [1..3] work counters
        CK(ctx->d_learn_err.ensure(4 * sizeof(int)), "alloc learned-shader flags");
        CK(cudaMemset(ctx->d_learn_err.p, 0, 4 * sizeof(int)), "clear learned-shader flags");
    }
    if (tile_status == nullptr) {   // the fallback pass reads the gate's decisions
        CK(ctx->d_learn_status.ensure(tiles), "alloc tile status");
        tile_status = ctx->d_learn_status.as<uint8_t>();
    }
    CK(ctx->d_learn_tiles.ensure(learned_scratch_bytes(int(tiles))), "alloc learned-shader blocks");
    if (ctx->num_sms == 0)
        CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_shade_learned(*mlp, *gbuffer, inv_view_proj, eye, lights, nlights, background, max_tile_mse, out_srgb,
                            out_linear, tile_status, tile_mse, ctx->d_srgb.as<uint8_t>(), ctx->d_learn_err.as<int>(),
                            ctx->d_learn_err.as<int>() + 1, ctx->d_learn_tiles.p, ctx->num_sms, ctx->debug_learned_stall, st),
       "shade_learned_kernel");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cap), "stream capture status");
    if (cap == cudaStreamCaptureStatusNone) {   // a captured call is checked after its replays are synchronised
        cudaEvent_t& ev = ctx->learn_events[st];
        if (ev == nullptr) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "learned-shader event");
        CK(cudaEventRecord(ev, st), "learned-shader event record");
    }
    return 0;
}

int rsrgpu_shade_learned_check(rsrgpu_ctx* ctx) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (ctx->d_learn_err.p == nullptr) return 0;
    for (auto& kv : ctx->learn_events) CK(cudaEventSynchronize(kv.second), "learned shader sync");
    int flag = 0;
    CK(cudaMemcpy(&flag, ctx->d_learn_err.p, sizeof(int), cudaMemcpyDeviceToHost), "D2H learned-shader error");
    if (flag == 0) return 0;
    CK(cudaMemset(ctx->d_learn_err.p, 0, sizeof(int)), "clear learned-shader error flag");
    return fail(ctx, RSRGPU_ETIMEOUT, "a bounded wait of the learned shader's tensor-core kernel expired");
}

int rsrgpu_set_debug(rsrgpu_ctx* ctx, int knob, int value) {
    if (ctx == nullptr) return RSRGPU_EINVAL;
    if (knob == RSRGPU_DEBUG_LEARNED_STALL) {
        if (value < 0) return fail(ctx, RSRGPU_EINVAL, "RSRGPU_DEBUG_LEARNED_STALL: polls >= 0");
        ctx->debug_learned_stall = value;
        return 0;
    }
    return fail(ctx, RSRGPU_EINVAL, "unknown debug knob %d", knob);
}

int rsrgpu_learned_features(rsrgpu_ctx* ctx, const rsrgpu_gbuffer* gbuffer, const float inv_view_proj[16],
                            const float eye[3], const rsrgpu_light* lights, int nlights, uint16_t* features,
                            float* targets, int32_t* candidates, void* stream) {
    if (ctx == nullptr || gbuffer == nullptr || inv_view_proj == nullptr || eye == nullptr || features == nullptr)
        return RSRGPU_EINVAL;
    int rc = check_gbuffer(ctx, gbuffer, lights, nlights);
    if (rc) return rc;
    const size_t npx = size_t(gbuffer->width) * size_t(gbuffer->height);
    const size_t tiles = size_t((gbuffer->width + RSRGPU_SHADE_TILE - 1) / RSRGPU_SHADE_TILE) *
                         size_t((gbuffer->height + RSRGPU_SHADE_TILE - 1) / RSRGPU_SHADE_TILE);
    if ((rc = check_device_output(ctx, features, npx * 64, 16, "features")) ||
        (rc = check_device_output(ctx, targets, npx * 12, 4, "targets")) ||
        (rc = check_device_output(ctx, candidates, tiles * 32, 4, "candidates")))
        return rc;
    if (ctx->num_sms == 0)
        CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    CK(launch_learned_features(*gbuffer, inv_view_proj, eye, lights, nlights, features, targets, candidates,
                               ctx->num_sms, st), "learned_features_kernel");
    CK(cudaStreamSynchronize(st), "learned features sync");
    return 0;
}

// ---------------------------------------------------------------------------
// batched frames
// ---------------------------------------------------------------------------
}  // extern "C"

struct rsrgpu_batch {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t run_stream = nullptr;
    std::string err;
    std::vector<std::tuple<int, uint32_t, int>> installs;
    std::vector<rsrgpu_ctx*> frames;      // one context per frame slot, reused across submits
    int nframes = 0;
    // all frames' tables in one device buffer, staged in pinned memory
    DevBuf d_tables, d_counters, d_super;
    DevBuf d_queue;                       // the raster launches' work queues
    DevBuf d_vis;                         // owners and depths of every frame (split pass)
    uint8_t* h_tables = nullptr;
    size_t h_tables_cap = 0, tables_bytes = 0, super_count = 0;
    FrameCounters* h_counters = nullptr;  // pinned, kMaxBatch entries
    std::vector<size_t> off_states, off_draws, off_ops, off_gbufs, off_dext, off_super;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // raster launches of different CTA shapes run as parallel graph branches
    static constexpr int kBranches = 4;
    cudaStream_t aux[kBranches] = {};
    cudaEvent_t fork = nullptr, join[kBranches] = {};
    bool ran = false;
    std::map<uint64_t, rsrgpu_frame_desc> tuned;   // (w, h, log2 ntris) -> choice
};

namespace {

int bfail(rsrgpu_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    b->err = buf;
    return code;
}

#define BCK(call, what)                                                                 \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return bfail(b, RSRGPU_ECUDA, "%s: %s", what, cudaGetErrorString(e_));      \
    } while (0)

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int frame_ctx(rsrgpu_batch* b, int i, rsrgpu_ctx** out) {
    while (int(b->frames.size()) <= i) {
        rsrgpu_ctx* c = nullptr;
        int rc = rsrgpu_create(b->device, &c);
        if (rc) return bfail(b, rc, "frame context: create failed");
        for (auto& in : b->installs) {
            rc = rsrgpu_install(c, std::get<0>(in), std::get<1>(in), std::get<2>(in));
            if (rc) { b->err = c->err; rsrgpu_destroy(c); return rc; }
        }
        b->frames.push_back(c);
    }
    *out = b->frames[size_t(i)];
    return 0;
}

// decodes one frame into context c with the tiling of d
int decode_into(rsrgpu_batch* b, rsrgpu_ctx* c, const rsrgpu_frame_desc& d) {
    if (d.tile_px < 8 || d.tile_px > 128 || (d.tile_px & 7))
        return bfail(b, RSRGPU_EINVAL, "tile_px %d: 8..128, a multiple of 8", d.tile_px);
    if (d.region_px != 0 && d.region_px != 8 && d.region_px != 16 && d.region_px != 32)
        return bfail(b, RSRGPU_EINVAL, "region_px %d: 0, 8, 16 or 32", d.region_px);
    int rc = rsrgpu_reset(c, d.width, d.height, d.tile_px / 8, d.tile_px / 8);
    if (rc == 0) rc = rsrgpu_submit(c, d.commands, d.nbytes, d.states, d.nstates);
    if (rc) { b->err = c->err; return rc; }
    if (!c->host.empty()) return bfail(b, RSRGPU_EINVAL, "batched frames take device pointers only");
    c->region_px = d.region_px ? d.region_px : std::min(d.tile_px, kRegionPx);
    if (d.bin_capacity) c->bin_cap = std::max<uint32_t>(d.bin_capacity, 1024u);
    return 0;
}

// packs the frames' tables, sizes their scratch and captures the kernel chain
int build_batch(rsrgpu_batch* b) {
    const int n = b->nframes;
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    b->off_states.assign(size_t(n), 0); b->off_draws.assign(size_t(n), 0); b->off_ops.assign(size_t(n), 0);
    b->off_gbufs.assign(size_t(n), 0); b->off_dext.assign(size_t(n), 0); b->off_super.assign(size_t(n), 0);
    size_t bytes = 0, supers = 0;
    for (int i = 0; i < n; ++i) {
        rsrgpu_ctx* c = b->frames[size_t(i)];
        b->off_states[size_t(i)] = bytes; bytes = align256(bytes + sizeof(DevState) * c->states.size());
        b->off_draws[size_t(i)] = bytes; bytes = align256(bytes + sizeof(DevDraw) * c->draws.size());
        b->off_ops[size_t(i)] = bytes; bytes = align256(bytes + sizeof(FrameOp) * c->ops.size());
        b->off_gbufs[size_t(i)] = bytes; bytes = align256(bytes + sizeof(GBufferDesc) * c->gbufs.size());
        b->off_dext[size_t(i)] = bytes; bytes = align256(bytes + (c->any_dext ? sizeof(DevDrawExt) * c->dext.size() : 0));
        b->off_super[size_t(i)] = supers; supers += size_t((c->ntris + kSuper - 1) / kSuper);
    }
    b->tables_bytes = std::max<size_t>(bytes, 256);
    b->super_count = std::max<size_t>(supers, 1);
    if (b->h_tables_cap < b->tables_bytes) {
        if (b->h_tables) cudaFreeHost(b->h_tables);
        b->h_tables = nullptr;
        b->h_tables_cap = 0;
        BCK(cudaHostAlloc(reinterpret_cast<void**>(&b->h_tables), b->tables_bytes, cudaHostAllocDefault), "alloc staging");
        b->h_tables_cap = b->tables_bytes;
    }
    BCK(b->d_tables.ensure(b->tables_bytes), "alloc batch tables");
    BCK(b->d_super.ensure(sizeof(int4) * b->super_count), "alloc batch super rects");
    uint8_t* dt = b->d_tables.as<uint8_t>();
    std::vector<BatchLaunch> setup(1), bin(1);
    setup[0].nframes = bin[0].nframes = n;
    int sblocks = 0, bblocks = 0;
    std::map<int, BatchLaunch> raster;      // by CTA size
    std::map<int, int> rblocks;
    // Each raster launch (one per CTA size) takes its frames' blocks from one
    // counter, the slot after the frames' own counters (n + the launch's place
    // among the CTA sizes); each frame's queue, [kCostBuckets][its blocks], is
    // at kCostBuckets x its first block in the launch's part of d_queue.
    std::map<int, int> group_blocks, group_index;
    for (int i = 0; i < n; ++i) {
        rsrgpu_ctx* c = b->frames[size_t(i)];
        FrameView probe{};
        probe.tile_w = c->tile_w; probe.tile_h = c->tile_h; probe.ntiles = c->ntiles;
        probe.region_px = std::min(c->region_px, std::min(c->tile_w, c->tile_h));
        group_blocks[raster_threads(probe)] += raster_blocks(probe);
    }
    size_t queue_entries = 0;
    std::map<int, size_t> group_queue;
    for (auto& kv : group_blocks) {
        group_index[kv.first] = int(group_index.size());
        group_queue[kv.first] = queue_entries;
        queue_entries += size_t(kCostBuckets) * size_t(kv.second);
    }
    BCK(b->d_queue.ensure(sizeof(uint32_t) * std::max<size_t>(queue_entries, 1)), "alloc batch work queues");
    const int ngroups = int(group_blocks.size());
    BCK(b->d_counters.ensure(sizeof(FrameCounters) * size_t(n + ngroups)), "alloc batch counters");
    // the split pass (visibility, then per-pixel shading) when every frame
    // takes it; owners and depths of frame i at vis_at[i] in d_vis
    std::vector<size_t> vis_at(size_t(n), 0);
    size_t vis_px = 0;
    bool split = true;
    std::map<int, std::vector<int>> group_frames;   // the frames of each raster launch, in launch order
    for (int i = 0; i < n; ++i) {
        vis_at[size_t(i)] = vis_px;
        vis_px += size_t(b->frames[size_t(i)]->width) * size_t(b->frames[size_t(i)]->height);
    }
    for (int i = 0; i < n; ++i) {
        rsrgpu_ctx* c = b->frames[size_t(i)];
        std::memcpy(b->h_tables + b->off_states[size_t(i)], c->states.data(), sizeof(DevState) * c->states.size());
        if (!c->draws.empty()) std::memcpy(b->h_tables + b->off_draws[size_t(i)], c->draws.data(), sizeof(DevDraw) * c->draws.size());
        if (!c->ops.empty()) std::memcpy(b->h_tables + b->off_ops[size_t(i)], c->ops.data(), sizeof(FrameOp) * c->ops.size());
        if (!c->gbufs.empty()) std::memcpy(b->h_tables + b->off_gbufs[size_t(i)], c->gbufs.data(), sizeof(GBufferDesc) * c->gbufs.size());
        if (c->any_dext) std::memcpy(b->h_tables + b->off_dext[size_t(i)], c->dext.data(), sizeof(DevDrawExt) * c->dext.size());
        ViewTables vt{ reinterpret_cast<DevState*>(dt + b->off_states[size_t(i)]),
                       reinterpret_cast<DevDraw*>(dt + b->off_draws[size_t(i)]),
                       reinterpret_cast<FrameOp*>(dt + b->off_ops[size_t(i)]),
                       reinterpret_cast<GBufferDesc*>(dt + b->off_gbufs[size_t(i)]),
                       b->d_counters.as<FrameCounters>() + i,
                       b->d_super.as<int4>() + b->off_super[size_t(i)],
                       reinterpret_cast<DevDrawExt*>(dt + b->off_dext[size_t(i)]) };
        int rc = prepare_view(c, &vt);
        if (rc) { b->err = c->err; return rc; }
        split = split && pixel_split(c);
        FrameView& fv = c->fv;
        const int th = raster_threads(fv);
        BatchLaunch& rl = raster[th];
        int& rb = rblocks[th];
        fv.tile_queue = b->d_queue.as<uint32_t>() + group_queue[th] + size_t(kCostBuckets) * size_t(rb);
        fv.taken = b->d_counters.as<FrameCounters>() + n + group_index[th];
        setup[0].start[i] = sblocks; setup[0].fv[i] = fv; sblocks += setup_blocks(fv);
        bin[0].start[i] = bblocks; bin[0].fv[i] = fv; bblocks += bin_blocks(fv);
        rl.start[rl.nframes] = rb;
        rl.fv[rl.nframes] = fv;
        rl.nframes++;
        group_frames[th].push_back(i);
        rb += raster_blocks(fv);
        c->stats.gpu_launches = 0;
    }
    setup[0].start[n] = sblocks;
    bin[0].start[n] = bblocks;
    for (auto& kv : raster) kv.second.start[kv.second.nframes] = rblocks[kv.first];
    BatchLaunch shade;
    int pblocks = 0;
    if (split) {
        BCK(b->d_vis.ensure(std::max<size_t>(vis_px, 1) * 8u), "alloc batch visibility hand-over");
        shade.nframes = n;
        auto place = [&](FrameView& f, int i) {
            f.vis_own = b->d_vis.as<uint32_t>() + vis_at[size_t(i)];
            f.vis_dep = reinterpret_cast<float*>(b->d_vis.as<uint32_t>() + vis_px) + vis_at[size_t(i)];
        };
        for (auto& kv : raster)
            for (int k = 0; k < kv.second.nframes; ++k) {
                place(kv.second.fv[k], group_frames[kv.first][size_t(k)]);
                kv.second.fv[k].raster_phase = 1;
            }
        for (int i = 0; i < n; ++i) {
            shade.fv[i] = b->frames[size_t(i)]->fv;
            place(shade.fv[i], i);
            shade.fv[i].raster_phase = 2;
            shade.start[i] = pblocks;
            pblocks += pixel_blocks(shade.fv[i]);
        }
        shade.start[n] = pblocks;
    }
    cudaStream_t st = b->own;
    BCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    int rc = 0;
    auto step = [&](cudaError_t e, const char* what) {
        if (rc == 0 && e != cudaSuccess) rc = bfail(b, RSRGPU_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    };
    step(cudaMemcpyAsync(b->d_tables.p, b->h_tables, b->tables_bytes, cudaMemcpyHostToDevice, st), "H2D tables");
    step(cudaMemsetAsync(b->d_counters.p, 0, sizeof(FrameCounters) * size_t(n + ngroups), st), "memset counters");
    step(cudaMemsetAsync(b->d_super.p, 0x7f, sizeof(int4) * b->super_count, st), "memset super rects");
    step(launch_setup_batch(setup[0], sblocks, st), "setup_batch_kernel");
    step(launch_bin_batch(bin[0], bblocks, st), "bin_batch_kernel");
    // one branch per CTA shape (the largest on the capture stream), joined before the read-back
    int branch = 0;
    if (raster.size() > 1) step(cudaEventRecord(b->fork, st), "fork");
    for (auto it = raster.rbegin(); it != raster.rend(); ++it, ++branch) {
        cudaStream_t rs = branch == 0 ? st : b->aux[(branch - 1) % rsrgpu_batch::kBranches];
        if (branch > 0) step(cudaStreamWaitEvent(rs, b->fork, 0), "fork wait");
        step(launch_raster_batch(it->second, rblocks[it->first], it->first, rs, split), "raster_batch_kernel");
        if (branch > 0) step(cudaEventRecord(b->join[(branch - 1) % rsrgpu_batch::kBranches], rs), "join");
    }
    for (int k = 0; k + 1 < branch && k < rsrgpu_batch::kBranches; ++k)
        step(cudaStreamWaitEvent(st, b->join[k], 0), "join wait");
    if (split) step(launch_shade_pixels_batch(shade, pblocks, st), "shade_pixels_batch_kernel");
    step(cudaMemcpyAsync(b->h_counters, b->d_counters.p, sizeof(FrameCounters) * size_t(n), cudaMemcpyDeviceToHost, st), "D2H counters");
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    BCK(e, "end capture");
    b->graph = g;
    BCK(cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate graph");
    const int launches = 2 + int(raster.size()) + (split ? 1 : 0);
    for (int i = 0; i < n; ++i) b->frames[size_t(i)]->stats.gpu_launches = launches;
    return 0;
}

uint64_t tune_key(const rsrgpu_frame_desc& d, int ntris) {
    return (uint64_t(uint32_t(d.width)) << 40) | (uint64_t(uint32_t(d.height)) << 16) | uint64_t(ilog2u(unsigned(ntris) | 1u));
}

}  // namespace

extern "C" {

int rsrgpu_batch_create(int device, rsrgpu_batch** out) {
    if (out == nullptr) return RSRGPU_EINVAL;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return RSRGPU_ECUDA;
    rsrgpu_batch* b = new rsrgpu_batch();
    b->device = device;
    if (cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaHostAlloc(reinterpret_cast<void**>(&b->h_counters), sizeof(FrameCounters) * kMaxBatch, cudaHostAllocDefault) != cudaSuccess ||
        b->d_counters.ensure(sizeof(FrameCounters) * kMaxBatch) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
        rsrgpu_batch_destroy(b);
        return RSRGPU_ECUDA;
    }
    for (int k = 0; k < rsrgpu_batch::kBranches; ++k)
        if (cudaStreamCreateWithFlags(&b->aux[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming) != cudaSuccess) {
            rsrgpu_batch_destroy(b);
            return RSRGPU_ECUDA;
        }
    *out = b;
    return 0;
}

int rsrgpu_batch_destroy(rsrgpu_batch* b) {
    if (b == nullptr) return 0;
    if (b->own) cudaStreamSynchronize(b->own);
    if (b->run_stream && b->run_stream != b->own) cudaStreamSynchronize(b->run_stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (rsrgpu_ctx* c : b->frames) rsrgpu_destroy(c);
    if (b->h_tables) cudaFreeHost(b->h_tables);
    if (b->h_counters) cudaFreeHost(b->h_counters);
    b->d_tables.release(); b->d_counters.release(); b->d_super.release(); b->d_queue.release(); b->d_vis.release();
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->fork) cudaEventDestroy(b->fork);
    for (int k = 0; k < rsrgpu_batch::kBranches; ++k) {
        if (b->join[k]) cudaEventDestroy(b->join[k]);
        if (b->aux[k]) cudaStreamDestroy(b->aux[k]);
    }
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return 0;
}

int rsrgpu_batch_install(rsrgpu_batch* b, int program_id, uint32_t state_key, int kind) {
    if (b == nullptr) return RSRGPU_EINVAL;
    for (rsrgpu_ctx* c : b->frames) {
        int rc = rsrgpu_install(c, program_id, state_key, kind);
        if (rc) { b->err = c->err; return rc; }
    }
    b->installs.emplace_back(program_id, state_key, kind);
    return 0;
}

int rsrgpu_batch_submit(rsrgpu_batch* b, const rsrgpu_frame_desc* frames, int nframes) {
    if (b == nullptr || frames == nullptr) return RSRGPU_EINVAL;
    if (nframes < 1 || nframes > kMaxBatch) return bfail(b, RSRGPU_EINVAL, "1..%d frames per batch", kMaxBatch);
    BCK(cudaSetDevice(b->device), "set device");
    b->nframes = 0;
    b->ran = false;
    for (int i = 0; i < nframes; ++i) {
        rsrgpu_ctx* c = nullptr;
        int rc = frame_ctx(b, i, &c);
        if (rc == 0) rc = decode_into(b, c, frames[i]);
        if (rc) {
            std::string m = b->err;
            return bfail(b, rc, "frame %d: %s", i, m.c_str());
        }
    }
    b->nframes = nframes;
    return build_batch(b);
}

int rsrgpu_batch_run(rsrgpu_batch* b, void* stream) {
    if (b == nullptr) return RSRGPU_EINVAL;
    if (b->exec == nullptr) return bfail(b, RSRGPU_EINVAL, "nothing submitted");
    b->run_stream = stream ? static_cast<cudaStream_t>(stream) : b->own;
    BCK(cudaEventRecord(b->ev0, b->run_stream), "event");
    BCK(cudaGraphLaunch(b->exec, b->run_stream), "graph launch");
    BCK(cudaEventRecord(b->ev1, b->run_stream), "event");
    b->ran = true;
    for (int i = 0; i < b->nframes; ++i) {
        b->frames[size_t(i)]->ran = true;
        b->frames[size_t(i)]->run_stream = b->run_stream;
    }
    return 0;
}

int rsrgpu_batch_wait(rsrgpu_batch* b, int timeout_ms) {
    if (b == nullptr) return RSRGPU_EINVAL;
    if (!b->ran) return 0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        const auto t0 = std::chrono::steady_clock::now();
        while (true) {
            cudaError_t q = cudaEventQuery(b->ev1);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return bfail(b, RSRGPU_ECUDA, "batch run: %s", cudaGetErrorString(q));
            if (timeout_ms >= 0) {
                const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
                if (ms > timeout_ms) return bfail(b, RSRGPU_ETIMEOUT, "rsrgpu_batch_wait timed out after %d ms", timeout_ms);
            }
            std::this_thread::yield();
        }
        bool again = false;
        for (int i = 0; i < b->nframes; ++i) {
            const FrameCounters c = b->h_counters[i];
            rsrgpu_ctx* x = b->frames[size_t(i)];
            *x->h_counters = c;
            if (c.overflow == 0) continue;
            if (c.overflow & 4u) return bfail(b, RSRGPU_EINVAL, "frame %d: a vertex index lies outside its attribute buffer", i);
            if (c.overflow & 1u) x->clip_cap = std::max<uint32_t>(x->clip_cap * 2, c.clip_verts + c.clip_verts / 4 + 1024);
            if (c.overflow & 2u) x->bin_cap = std::max<uint32_t>(x->bin_cap * 2, c.bin_used + c.bin_used / 4 + 4096);
            if (x->clip_cap > (1u << 28) || x->bin_cap > (1u << 30))
                return bfail(b, RSRGPU_ECAPACITY, "frame %d needs %u clipped vertices and %u tile entries", i, c.clip_verts, c.bin_used);
            again = true;
        }
        if (!again) return 0;
        int rc = build_batch(b);
        if (rc == 0) rc = rsrgpu_batch_run(b, b->run_stream);
        if (rc) return rc;
    }
    return bfail(b, RSRGPU_ECAPACITY, "capacity growth did not converge");
}

int rsrgpu_batch_last_ms(rsrgpu_batch* b, float* ms) {
    if (b == nullptr || ms == nullptr || !b->ran) return RSRGPU_EINVAL;
    BCK(cudaEventSynchronize(b->ev1), "sync");
    BCK(cudaEventElapsedTime(ms, b->ev0, b->ev1), "elapsed");
    return 0;
}

int rsrgpu_batch_frame(rsrgpu_batch* b, int i, rsrgpu_ctx** ctx) {
    if (b == nullptr || ctx == nullptr || i < 0 || i >= b->nframes) return RSRGPU_EINVAL;
    *ctx = b->frames[size_t(i)];
    return 0;
}

namespace {
// median device time of the batch over `reps` runs after one warm-up run
int time_batch(rsrgpu_batch* b, const rsrgpu_frame_desc* frames, int nframes, int reps, float* ms) {
    int rc = rsrgpu_batch_submit(b, frames, nframes);
    if (rc) return rc;
    std::vector<float> t;
    for (int r = 0; r <= reps; ++r) {
        rc = rsrgpu_batch_run(b, nullptr);
        if (rc == 0) rc = rsrgpu_batch_wait(b, -1);
        if (rc) return rc;
        float x = 0.f;
        rc = rsrgpu_batch_last_ms(b, &x);
        if (rc) return rc;
        if (r > 0) t.push_back(x);
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return 0;
}
}  // namespace

int rsrgpu_batch_tune(rsrgpu_batch* b, rsrgpu_frame_desc* frames, int nframes, int reps) {
    if (b == nullptr || frames == nullptr || nframes < 0) return RSRGPU_EINVAL;
    if (reps < 1) reps = 1;
    BCK(cudaSetDevice(b->device), "set device");
    static const int kCandidates[][2] = { { 8, 8 }, { 16, 16 }, { 16, 8 }, { 32, 32 }, { 32, 16 }, { 64, 32 } };
    static const int kTuneDefault[2] = { 32, 32 };
    rsrgpu_ctx* c = nullptr;
    int rc = frame_ctx(b, 0, &c);   // scratch context: frame slot 0 is re-decoded by the next submit
    if (rc) return rc;
    for (int i = 0; i < nframes; ++i) {
        rsrgpu_frame_desc d = frames[i];
        d.tile_px = 8; d.region_px = 8; d.bin_capacity = 0;
        rc = decode_into(b, c, d);
        if (rc) { std::string m = b->err; return bfail(b, rc, "frame %d: %s", i, m.c_str()); }
        const uint64_t key = tune_key(d, c->ntris);
        auto hit = b->tuned.find(key);
        if (hit != b->tuned.end()) {
            // same size class: keep the measured tiling, size the capacity from one run of this frame
            d.tile_px = hit->second.tile_px;
            d.region_px = hit->second.region_px;
            rc = decode_into(b, c, d);
            if (rc == 0) rc = rsrgpu_run(c, b->own);
            if (rc == 0) rc = rsrgpu_wait(c, -1);
            if (rc) { b->err = c->err; return rc; }
            const uint32_t used = c->h_counters->bin_used;
            frames[i].tile_px = d.tile_px;
            frames[i].region_px = d.region_px;
            frames[i].bin_capacity = used + used / 4 + 1024;
            continue;
        }
        float best = 1e30f, base = 1e30f;
        rsrgpu_frame_desc choice = d, base_choice = d;
        for (const auto& cand : kCandidates) {
            d.tile_px = cand[0]; d.region_px = cand[1];
            rc = decode_into(b, c, d);
            if (rc) { std::string m = b->err; return bfail(b, rc, "frame %d: %s", i, m.c_str()); }
            std::vector<float> t;
            uint32_t used = 0;
            bool fits = true;
            for (int r = 0; r <= reps && fits; ++r) {
                rc = rsrgpu_run(c, b->own);
                if (rc == 0) rc = rsrgpu_wait(c, -1);
                if (rc == RSRGPU_ECAPACITY) { fits = false; break; }   // this tiling's lists cannot be held
                if (rc) { b->err = c->err; return rc; }
                float ms = 0.f;
                BCK(cudaEventElapsedTime(&ms, c->ev0, c->ev2), "elapsed");
                if (r > 0) t.push_back(ms);   // the first run warms the scratch up
                used = c->h_counters->bin_used;
            }
            if (!fits || t.empty()) continue;
            std::sort(t.begin(), t.end());
            const float med = t[t.size() / 2];
            if (med < best) {
                best = med;
                choice = d;
                choice.bin_capacity = used + used / 4 + 1024;
            }
            if (cand[0] == kTuneDefault[0] && cand[1] == kTuneDefault[1]) {
                base = med;
                base_choice = d;
                base_choice.bin_capacity = used + used / 4 + 1024;
            }
        }
        if (best >= 1e30f) return bfail(b, RSRGPU_ECAPACITY, "frame %d: no candidate tiling holds its tile lists", i);
        (void)base;
        (void)base_choice;
        b->tuned[key] = choice;
        frames[i].tile_px = choice.tile_px;
        frames[i].region_px = choice.region_px;
        frames[i].bin_capacity = choice.bin_capacity;
    }
    // Timed alone, a small frame is mostly launch latency, while in the batch
    // it shares the launches (and another region size adds a raster launch).
    // So the per-frame choices are only the start of a search on the batch's
    // own time: the default tiling everywhere is tried, then, for each
    // resolution class in turn, every candidate tiling for all of the class's
    // frames, the rest held; a change is kept when the batch runs faster.
    if (nframes > 1) {
        std::vector<rsrgpu_frame_desc> cur(frames, frames + nframes);
        float t_cur = 0.f;
        rc = time_batch(b, cur.data(), nframes, reps, &t_cur);
        if (rc) return rc;
        auto try_set = [&](const std::vector<rsrgpu_frame_desc>& trial) -> int {
            float t = 0.f;
            const int r = time_batch(b, trial.data(), nframes, reps, &t);
            if (r == RSRGPU_ECAPACITY) return 0;   // this tiling's lists cannot be held
            if (r) return r;
            if (t < t_cur) { t_cur = t; cur = trial; }
            return 0;
        };
        std::vector<rsrgpu_frame_desc> deflt = cur;
        for (auto& f : deflt) { f.tile_px = kTuneDefault[0]; f.region_px = kTuneDefault[1]; f.bin_capacity = 0; }
        rc = try_set(deflt);
        if (rc) return rc;
        std::vector<std::pair<int, int>> classes;
        for (int i = 0; i < nframes; ++i) {
            const std::pair<int, int> wh(frames[i].width, frames[i].height);
            if (std::find(classes.begin(), classes.end(), wh) == classes.end()) classes.push_back(wh);
        }
        for (const auto& wh : classes) {
            for (const auto& cand : kCandidates) {
                std::vector<rsrgpu_frame_desc> trial = cur;
                bool changed = false;
                for (auto& f : trial) {
                    if (f.width != wh.first || f.height != wh.second) continue;
                    if (f.tile_px == cand[0] && f.region_px == cand[1]) continue;
                    f.tile_px = cand[0]; f.region_px = cand[1]; f.bin_capacity = 0;
                    changed = true;
                }
                if (!changed) continue;
                rc = try_set(trial);
                if (rc) return rc;
            }
        }
        // capacities from the entries each frame uses with the chosen tilings
        float t = 0.f;
        rc = time_batch(b, cur.data(), nframes, reps, &t);
        if (rc) return rc;
        for (int i = 0; i < nframes; ++i) {
            const uint32_t used = b->frames[size_t(i)]->h_counters->bin_used;
            frames[i] = cur[size_t(i)];
            frames[i].bin_capacity = used + used / 4 + 1024;
        }
    }
    return 0;
}

int rsrgpu_batch_last_error(rsrgpu_batch* b, char* buf, size_t len) {
    if (b == nullptr || buf == nullptr || len == 0) return RSRGPU_EINVAL;
    std::snprintf(buf, len, "%s", b->err.c_str());
    return 0;
}

int rsrgpu_last_error(rsrgpu_ctx* ctx, char* buf, size_t len) {
    if (ctx == nullptr || buf == nullptr || len == 0) return RSRGPU_EINVAL;
    std::snprintf(buf, len, "%s", ctx->err.c_str());
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Frame decode for callers without a context (rsrgpu_static.cu): runs the
// same stream parser as rsrgpu_submit() on a temporary context that owns no
// device memory, with every program this library implements installed.
// Pointers must therefore be device pointers.
// ---------------------------------------------------------------------------
namespace rsrgpu {
int decode_frame_without_context(int width, int height, int tile_blocks_x, int tile_blocks_y,
                                 const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates,
                                 std::vector<DevState>& out_states, std::vector<DevDraw>& out_draws,
                                 std::vector<FrameOp>& out_ops, int& ntris, int& ntiles, int& vis_keys,
                                 std::string& err) {
    rsrgpu_ctx tmp;
    int rc = rsrgpu_reset(&tmp, width, height, tile_blocks_x, tile_blocks_y);
    const int programs[] = { kProgGouraud, kProgAmy, kProgMany };
    const uint32_t keys[] = { 0x6e2, 0x6e6, 0x6ea, 0x6f2, 0x6f6, 0x6c2, 0x6c6, 0x62, 0x66, 0x72, 0x42, 0x6a };
    for (int pid : programs) {
        if (rc == 0) rc = rsrgpu_install(&tmp, pid, 0, 0);
        for (uint32_t k : keys)
            for (uint32_t scissor = 0; scissor < 2; ++scissor)
                if (rc == 0 && draw_key_supported(k | scissor)) rc = rsrgpu_install(&tmp, pid, k | scissor, 1);
    }
    const int blts[] = { kProgDefaultPost, kProgExposurePost, kProgGouraud };
    for (int pid : blts)
        if (rc == 0) rc = rsrgpu_install(&tmp, pid, 0, 2);
    if (rc == 0) rc = rsrgpu_submit(&tmp, commands, nbytes, states, nstates);
    if (rc != 0) {
        err = tmp.err;
        return rc;
    }
    if (!tmp.gbufs.empty()) {
        err = "CMD_STORE_GBUFFER is not available without a context";
        return RSRGPU_EUNSUPPORTED;
    }
    if (tmp.any_inst) {
        err = "instanced draws are not available without a context";
        return RSRGPU_EUNSUPPORTED;
    }
    out_states = std::move(tmp.states);
    out_draws = std::move(tmp.draws);
    out_ops = std::move(tmp.ops);
    ntris = tmp.ntris;
    ntiles = tmp.ntiles;
    vis_keys = tmp.vis_keys;
    return 0;
}
}  // namespace rsrgpu
