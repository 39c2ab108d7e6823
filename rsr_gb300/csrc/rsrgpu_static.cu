// rsrgpu_static.cu -- rsrgpu_render_static(): one frame with no device
// allocation at all.
//
// Some callers cannot call cudaMalloc: a host framework that owns every byte
// of device memory through its own pool, a real-time loop that must not
// allocate (cudaMalloc synchronises the device and can take milliseconds), or
// code that is already inside a region where allocation is not allowed.  For
// them this entry point renders through the same setup, bin and raster
// kernels as rsrgpu_run(), but all frame scratch (state tables, triangle
// records, tile lists, clipped vertices, counters and the rcpps / sRGB
// tables) lives in one file-scope __device__ array of fixed size that every
// GPU loading this library holds until the process exits.
//
// Rules of use:
//  * Inputs and outputs are device pointers supplied by the caller; there is
//    no host staging.
//  * The first call on a device does the set-up (looks up the array's device
//    address with cudaGetSymbolAddress and uploads the rcpps and sRGB tables
//    with synchronous copies); make that first call before any stream capture.
//    The set-up runs under a lock, so first calls from several host threads
//    are safe.  The address is cached per device for the life of the process:
//    after cudaDeviceReset() the cache is stale.
//  * Every call shares the array and it keeps the last call's contents; the
//    counters and rectangles that must start at zero are cleared each call.
//    Calls that overlap on the GPU (concurrent streams or threads) race on
//    the array: serialise them.
//  * The call returns when the frame has finished on `stream`, so it can
//    report capacity overflow and out-of-range vertex indices.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_internal.h"

namespace rsrgpu {
cudaError_t launch_setup(const FrameView& fv, cudaStream_t st, bool after_init = false);
cudaError_t launch_bin(const FrameView& fv, cudaStream_t st);
cudaError_t launch_raster(const FrameView& fv, cudaStream_t st, int phase = 0);
int decode_frame_without_context(int width, int height, int tile_blocks_x, int tile_blocks_y,
                                 const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates,
                                 std::vector<DevState>& out_states, std::vector<DevDraw>& out_draws,
                                 std::vector<FrameOp>& out_ops, int& ntris, int& ntiles, int& vis_keys,
                                 std::string& err);
static const uint32_t kStaticRcpTable[2048] = {
#include "rcpps_table.inc"
};
}  // namespace rsrgpu

using namespace rsrgpu;

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// region layout of the scratch array
constexpr size_t kMaxTris = RSRGPU_STATIC_MAX_TRIANGLES;
constexpr size_t kOffStates = 0;
constexpr size_t kOffDraws = kOffStates + align256(sizeof(DevState) * RSRGPU_STATIC_MAX_STATES);
constexpr size_t kOffOps = kOffDraws + align256(sizeof(DevDraw) * RSRGPU_STATIC_MAX_DRAWS);
constexpr size_t kOffTris = kOffOps + align256(sizeof(FrameOp) * RSRGPU_STATIC_MAX_OPS);
constexpr size_t kOffBinRect = kOffTris + align256(sizeof(TriRecord) * kMaxTris);
constexpr size_t kOffRec16 = kOffBinRect + align256(sizeof(uint64_t) * kMaxTris);
constexpr size_t kOffChunk = kOffRec16 + align256(sizeof(uint32_t) * 2 * kMaxTris);
constexpr size_t kOffSuper = kOffChunk + align256(sizeof(int4) * (kMaxTris / kChunk));
constexpr size_t kOffClipInfo = kOffSuper + align256(sizeof(int4) * (kMaxTris / kSuper));
constexpr size_t kOffClipVerts = kOffClipInfo + align256(sizeof(ClipInfo) * kMaxTris);
constexpr size_t kOffClipPoly = kOffClipVerts + align256(sizeof(ClipVert) * RSRGPU_STATIC_MAX_CLIP_VERTS);
constexpr size_t kOffClipSrc = kOffClipPoly + align256(sizeof(int32_t) * RSRGPU_STATIC_MAX_CLIP_VERTS);
constexpr size_t kOffClipFan = kOffClipSrc + align256(sizeof(int32_t) * RSRGPU_STATIC_MAX_CLIP_VERTS);
constexpr size_t kOffBins = kOffClipFan + align256(sizeof(uint64_t) * RSRGPU_STATIC_MAX_CLIP_VERTS);
constexpr size_t kOffPool = kOffBins + align256(sizeof(TileBin) * RSRGPU_STATIC_MAX_TILES);
constexpr size_t kOffCounters = kOffPool + align256(sizeof(uint32_t) * RSRGPU_STATIC_MAX_TILE_ENTRIES);
constexpr size_t kOffRcp = kOffCounters + align256(sizeof(FrameCounters));
constexpr size_t kOffSrgb = kOffRcp + align256(sizeof(uint32_t) * 2048);
constexpr size_t kScratchBytes = kOffSrgb + align256(26624);
static_assert(kScratchBytes == RSRGPU_STATIC_SCRATCH_BYTES, "scratch size in rsrgpu.h is out of date");

// the frame scratch: one fixed array, resident on every device that loads the library
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::atomic<unsigned char*> g_base[kMaxDevices];   // device address of g_scratch, per device (set up once)
std::mutex g_setup_mu;                             // serialises the set-up of first calls

int set_up_device(int dev, unsigned char** base, std::string& err) {
    if (dev < 0 || dev >= kMaxDevices) { err = "device ordinal out of range"; return RSRGPU_EINVAL; }
    if ((*base = g_base[dev].load(std::memory_order_acquire)) != nullptr) return 0;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if ((*base = g_base[dev].load(std::memory_order_acquire)) != nullptr) return 0;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) { err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e); return RSRGPU_ECUDA; }
    unsigned char* b = static_cast<unsigned char*>(p);
    std::vector<uint8_t> lut;
    build_srgb_lut(lut);
    e = cudaMemcpy(b + kOffRcp, kStaticRcpTable, sizeof(kStaticRcpTable), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b + kOffSrgb, lut.data(), lut.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { err = std::string("table upload: ") + cudaGetErrorString(e); return RSRGPU_ECUDA; }
    g_base[dev].store(b, std::memory_order_release);
    *base = b;
    return 0;
}

thread_local std::string g_static_err;

int render_static(const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates,
                  int width, int height, int tile_blocks_x, int tile_blocks_y, void* stream);

int fail_static(int code, const std::string& msg) {
    g_static_err = msg;
    return code;
}

}  // namespace

extern "C" {

int rsrgpu_render_static(const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates,
                         int width, int height, int tile_blocks_x, int tile_blocks_y, void* stream,
                         char* errbuf, size_t errlen) {
    if (errbuf != nullptr && errlen > 0) errbuf[0] = '\0';
    int rc = render_static(commands, nbytes, states, nstates, width, height, tile_blocks_x, tile_blocks_y, stream);
    if (rc != 0 && errbuf != nullptr && errlen > 0) std::snprintf(errbuf, errlen, "%s", g_static_err.c_str());
    return rc;
}

}  // extern "C"

namespace {

int render_static(const uint8_t* commands, size_t nbytes, const rsrgpu_glstate* states, int nstates,
                  int width, int height, int tile_blocks_x, int tile_blocks_y, void* stream) {
    std::vector<DevState> st;
    std::vector<DevDraw> dr;
    std::vector<FrameOp> ops;
    int ntris = 0, ntiles = 0, vis_keys = 0;
    std::string err;
    int rc = decode_frame_without_context(width, height, tile_blocks_x, tile_blocks_y, commands, nbytes, states,
                                          nstates, st, dr, ops, ntris, ntiles, vis_keys, err);
    if (rc != 0) return fail_static(rc, err);
    char msg[256];
    if (st.size() > RSRGPU_STATIC_MAX_STATES || dr.size() > RSRGPU_STATIC_MAX_DRAWS || ops.size() > RSRGPU_STATIC_MAX_OPS ||
        size_t(ntris) > kMaxTris || ntiles > RSRGPU_STATIC_MAX_TILES) {
        std::snprintf(msg, sizeof(msg),
                      "frame exceeds the static scratch: %zu states (max %d), %zu draws (max %d), %zu ops (max %d), "
                      "%d triangles (max %d), %d tiles (max %d)",
                      st.size(), RSRGPU_STATIC_MAX_STATES, dr.size(), RSRGPU_STATIC_MAX_DRAWS, ops.size(),
                      RSRGPU_STATIC_MAX_OPS, ntris, RSRGPU_STATIC_MAX_TRIANGLES, ntiles, RSRGPU_STATIC_MAX_TILES);
        return fail_static(RSRGPU_ECAPACITY, msg);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_static(RSRGPU_ECUDA, cudaGetErrorString(e));
    unsigned char* base = nullptr;
    rc = set_up_device(dev, &base, err);
    if (rc != 0) return fail_static(rc, err);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    FrameView fv{};
    fv.slices = 1;
    fv.states = reinterpret_cast<const DevState*>(base + kOffStates);
    fv.draws = reinterpret_cast<const DevDraw*>(base + kOffDraws);
    fv.ndraws = int(dr.size());
    fv.ntris = ntris;
    fv.ops = reinterpret_cast<const FrameOp*>(base + kOffOps);
    fv.nops = int(ops.size());
    fv.width = width; fv.height = height;
    fv.tile_w = tile_blocks_x * 8; fv.tile_h = tile_blocks_y * 8;
    fv.tiles_x = (width + fv.tile_w - 1) / fv.tile_w;
    fv.tiles_y = (height + fv.tile_h - 1) / fv.tile_h;
    fv.ntiles = ntiles;
    fv.nchunks = (ntris + kChunk - 1) / kChunk;
    fv.nsupers = (ntris + kSuper - 1) / kSuper;
    fv.tris = reinterpret_cast<TriRecord*>(base + kOffTris);
    fv.bin_rect = reinterpret_cast<uint64_t*>(base + kOffBinRect);
    fv.rec16 = reinterpret_cast<uint32_t*>(base + kOffRec16);
    fv.chunk_rect = reinterpret_cast<int4*>(base + kOffChunk);
    fv.super_rect = reinterpret_cast<int4*>(base + kOffSuper);
    fv.clip_info = reinterpret_cast<ClipInfo*>(base + kOffClipInfo);
    fv.clip_verts = reinterpret_cast<ClipVert*>(base + kOffClipVerts);
    fv.clip_poly = reinterpret_cast<int32_t*>(base + kOffClipPoly);
    fv.clip_src = reinterpret_cast<int32_t*>(base + kOffClipSrc);
    fv.clip_fan_rect = reinterpret_cast<uint64_t*>(base + kOffClipFan);
    fv.clip_cap = RSRGPU_STATIC_MAX_CLIP_VERTS;
    fv.bins = reinterpret_cast<TileBin*>(base + kOffBins);
    fv.bin_pool = reinterpret_cast<uint32_t*>(base + kOffPool);
    fv.bin_cap = RSRGPU_STATIC_MAX_TILE_ENTRIES;
    fv.counters = reinterpret_cast<FrameCounters*>(base + kOffCounters);
    fv.rcp_table = reinterpret_cast<const uint32_t*>(base + kOffRcp);
    fv.srgb_lut = reinterpret_cast<const uint8_t*>(base + kOffSrgb);
    fv.region_px = kRegionPx;
    fv.vis_keys = vis_keys;   // visibility by (depth, order) keys where the frame allows it, as rsrgpu_run
    for (const DevState& d : st) fv.any_scissor |= d.scissor_test;
    for (const FrameOp& o : ops)
        if (o.kind >= kOpStoreFP) fv.ext = 1;

#define CKS(expr) do { cudaError_t e_ = (expr); if (e_ != cudaSuccess) return fail_static(RSRGPU_ECUDA, cudaGetErrorString(e_)); } while (0)
    CKS(cudaMemcpyAsync(base + kOffStates, st.data(), sizeof(DevState) * st.size(), cudaMemcpyHostToDevice, s));
    if (!dr.empty()) CKS(cudaMemcpyAsync(base + kOffDraws, dr.data(), sizeof(DevDraw) * dr.size(), cudaMemcpyHostToDevice, s));
    if (!ops.empty()) CKS(cudaMemcpyAsync(base + kOffOps, ops.data(), sizeof(FrameOp) * ops.size(), cudaMemcpyHostToDevice, s));
    // state that must start at zero each call: counters; super-chunk rectangles start "empty"
    CKS(cudaMemsetAsync(base + kOffCounters, 0, sizeof(FrameCounters), s));
    if (fv.nsupers > 0) CKS(cudaMemsetAsync(base + kOffSuper, 0x7f, sizeof(int4) * size_t(fv.nsupers), s));
    CKS(launch_setup(fv, s));
    CKS(launch_bin(fv, s));
    CKS(launch_raster(fv, s));
    FrameCounters c{};
    CKS(cudaMemcpyAsync(&c, base + kOffCounters, sizeof(c), cudaMemcpyDeviceToHost, s));
    CKS(cudaStreamSynchronize(s));
#undef CKS
    if (c.overflow & 4u) return fail_static(RSRGPU_EINVAL, "a vertex index lies outside its attribute buffer");
    if (c.overflow & 1u) {
        std::snprintf(msg, sizeof(msg), "frame needs %u clipped vertices, the static scratch holds %d",
                      c.clip_verts, RSRGPU_STATIC_MAX_CLIP_VERTS);
        return fail_static(RSRGPU_ECAPACITY, msg);
    }
    if (c.overflow & 2u) {
        std::snprintf(msg, sizeof(msg), "frame needs %u tile-list entries, the static scratch holds %d",
                      c.bin_used, RSRGPU_STATIC_MAX_TILE_ENTRIES);
        return fail_static(RSRGPU_ECAPACITY, msg);
    }
    return 0;
}

}  // namespace
