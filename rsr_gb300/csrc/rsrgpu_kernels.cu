// rsrgpu_kernels.cu -- sm_103a kernels of the rasteriser path.
//
//   setup_kernel   one thread per triangle: vertex program, frustum flags,
//                  rcpps-based perspective divide, viewport, fixed point,
//                  area/cull, tile rectangle; clip-source triangles run the
//                  Sutherland-Hodgman clipper in place.  Replaces
//                  GPUBinImpl::BinTriangles1P/2P + ClipTriangles
//                  (src/rgl/rglv/rglv_gpu_impl.hxx:315-793).
//   bin_kernel     one warp per tile: walks the triangle stream in submission
//                  order through a 1024/32-triangle rectangle hierarchy and
//                  compacts the triangles touching the tile with ballot +
//                  popc, so every tile list comes out in the reference's
//                  append order without sorting or atomics on list slots.
//   raster_kernel  one CTA per (tile, 32x32 px region): the region's colour
//                  and depth live in registers (one 2x2 quad per thread);
//                  triangles are set up per tile in shared memory in batches
//                  and walked in list order; coverage, depth test, fragment
//                  program, blend and the sRGB8/fp32 stores follow
//                  GPU::DrawImpl, VTriangleRasterizer/TriangleRasterizer and
//                  TriangleProgram::Render (rglv_gpu.cxx:263-432,
//                  rglv_triangle.hxx:79-304, rglv_gpu_impl.hxx:166-222).
//
// Built with -fmad=false: every float expression keeps the reference's
// separate multiply and add roundings and its evaluation order.
#include <cstdint>
#include <climits>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "rsrgpu_internal.h"
#include "rsrgpu_obj1.h"

namespace rsrgpu {

#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// SSE lane semantics (src/rml/rmlv/rmlv_mvec4.hxx)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t f2u(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }

// _mm_rcp_ps through the table measured on the reference's host
__device__ __forceinline__ float rcpps(const uint32_t* __restrict__ T, float x) {
    const uint32_t b = f2u(x), s = b & 0x80000000u, e = (b >> 23) & 255u, m = b & 0x7fffffu;
    if (e == 255u) return u2f(m ? (b | 0x00400000u) : s);
    if (e == 0u) return u2f(s | 0x7f800000u);
    const uint32_t t = __ldg(T + (m >> 12));
    const int er = int((t >> 23) & 255u) - (int(e) - 127);
    if (er <= 0) return u2f(s);
    return u2f(s | (uint32_t(er) << 23) | (t & 0x7fffffu));
}

// rmlv::oneover (rmlv_mvec4.hxx:631-651)
__device__ __forceinline__ float oneover(const uint32_t* __restrict__ T, float a) {
    const float r = rcpps(T, a);
    const float muls = __fmul_rn(a, __fmul_rn(r, r));
    return __fsub_rn(__fadd_rn(r, r), muls);
}

// _mm_cvttps_epi32: truncation, INT_MIN when out of range or NaN
__device__ __forceinline__ int32_t ftoi(float f) {
    return (f >= -2147483648.0f && f < 2147483648.0f) ? __float2int_rz(f) : INT_MIN;
}
__device__ __forceinline__ float itof(int32_t i) { return __int2float_rn(i); }
__device__ __forceinline__ float sse_min(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float sse_max(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return int32_t(uint32_t(a) - uint32_t(b)); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return int32_t(uint32_t(a) * uint32_t(b)); }
__device__ __forceinline__ float fract(float a) { return a - itof(ftoi(a)); }

// ---------------------------------------------------------------------------
// vertex programs
// ---------------------------------------------------------------------------
// SHADER::ShadeVertex: gl_Position = vpm * (position, 1) (qmat4 * qfloat4,
// rmlm_soa.hxx:59-65) and the program's VertexOutputSD.
// Attribute fetch with a bounds check: an index past the end of a buffer
// raises the frame's error bit and reads 0 instead of faulting.
__device__ __forceinline__ float fetch(const DevState& s, int b, int idx, FrameCounters* ctr) {
    if (idx >= s.buffer_len[b]) {
        atomicOr(&ctr->overflow, 4u);
        return 0.f;
    }
    return __ldg(s.buffers[b] + idx);
}

__device__ __forceinline__ void shade_vertex(const DevState& s, int idx, float pos[4], float vary[kMaxVary],
                                             FrameCounters* ctr) {
    float x = 0.f, y = 0.f, z = 0.f;
    if (s.buffers[0] != nullptr && s.buffers[1] != nullptr && s.buffers[2] != nullptr) {
        x = fetch(s, 0, idx, ctr);
        y = fetch(s, 1, idx, ctr);
        z = fetch(s, 2, idx, ctr);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
        pos[r] = ((s.vpm[r] * x + s.vpm[4 + r] * y) + s.vpm[8 + r] * z) + s.vpm[12 + r] * 1.0f;
#pragma unroll
    for (int k = 0; k < kMaxVary; ++k) vary[k] = 0.f;
    if (s.program == kProgGouraud) {
        vary[0] = fetch(s, 3, idx, ctr);
        vary[1] = fetch(s, 4, idx, ctr);
        vary[2] = fetch(s, 5, idx, ctr);
    } else if (s.program == kProgAmy) {
        vary[0] = s.buffers[9] ? fetch(s, 9, idx, ctr) : 0.f;
        vary[1] = s.buffers[10] ? fetch(s, 10, idx, ctr) : 0.f;
    } else if (s.program == kProgGBuffer) {
        // normal (interpolated) and the packed RGB albedo (flat)
        vary[0] = fetch(s, 3, idx, ctr);
        vary[1] = fetch(s, 4, idx, ctr);
        vary[2] = fetch(s, 5, idx, ctr);
        vary[3] = fetch(s, 6, idx, ctr);
    }
}

// OBJ1Program's vertex inputs (its Loader::LoadLane, shaders.hxx:623-636:
// missing position 0, normal (0,0,1), kd (1,1,1)) and its lighting
// (rsrgpu_obj1.h), with RSRGPU's measured RSQRTPS table
__device__ const uint32_t kRsqrtTable[4096] = {
#include "rsqrtps_table.inc"
};
__device__ __forceinline__ void shade_vertex_obj1(const DevState& s, const float* __restrict__ vm, int idx,
                                                  float pos[4], float vary[kMaxVary], FrameCounters* ctr) {
    float p[3] = { 0.f, 0.f, 0.f }, n[3] = { 0.f, 0.f, 1.f }, kd[3] = { 1.f, 1.f, 1.f };
    if (s.buffers[0] != nullptr) { p[0] = fetch(s, 0, idx, ctr); p[1] = fetch(s, 1, idx, ctr); p[2] = fetch(s, 2, idx, ctr); }
    if (s.buffers[3] != nullptr) { n[0] = fetch(s, 3, idx, ctr); n[1] = fetch(s, 4, idx, ctr); n[2] = fetch(s, 5, idx, ctr); }
    if (s.buffers[6] != nullptr) { kd[0] = fetch(s, 6, idx, ctr); kd[1] = fetch(s, 7, idx, ctr); kd[2] = fetch(s, 8, idx, ctr); }
    float m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = __ldg(vm + i);
    float out[3];
    obj1_shade(m, s.vpm, kRsqrtTable, p, n, kd, pos, out);
#pragma unroll
    for (int k = 0; k < kMaxVary; ++k) vary[k] = 0.f;
    vary[0] = out[0];
    vary[1] = out[1];
    vary[2] = out[2];
}

// ManyProgram::ShadeVertex (src/viewer/shaders.hxx:555-562): the instance's
// matrix times (position, 1), then vpm times that; uv from buffers 9-10 (its
// Loader, :500-535: missing position or uv buffers read as 0)
__device__ __forceinline__ void shade_vertex_many(const DevState& s, const float* __restrict__ imat, int idx,
                                                  float pos[4], float vary[kMaxVary], FrameCounters* ctr) {
    float x = 0.f, y = 0.f, z = 0.f;
    if (s.buffers[0] != nullptr && s.buffers[1] != nullptr && s.buffers[2] != nullptr) {
        x = fetch(s, 0, idx, ctr);
        y = fetch(s, 1, idx, ctr);
        z = fetch(s, 2, idx, ctr);
    }
    float m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = __ldg(imat + i);
    float p1[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) p1[r] = ((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * 1.0f;
#pragma unroll
    for (int r = 0; r < 4; ++r)
        pos[r] = ((s.vpm[r] * p1[0] + s.vpm[4 + r] * p1[1]) + s.vpm[8 + r] * p1[2]) + s.vpm[12 + r] * p1[3];
#pragma unroll
    for (int k = 0; k < kMaxVary; ++k) vary[k] = 0.f;
    vary[0] = s.buffers[9] ? fetch(s, 9, idx, ctr) : 0.f;
    vary[1] = s.buffers[10] ? fetch(s, 10, idx, ctr) : 0.f;
}

// ViewFrustum::Test, SIMD version (rglv_view_frustum.hxx:60-73)
__device__ __forceinline__ uint32_t frustum_test(float factor, const float p[4]) {
    const float w = p[3] * factor;
    const uint32_t left = (w + p[0]) <= 0.f;
    const uint32_t bottom = (w + p[1]) <= 0.f;
    const uint32_t nearp = (p[3] + p[2]) <= 0.f;
    const uint32_t right = (w - p[0]) <= 0.f;
    const uint32_t top = (w - p[1]) <= 0.f;
    return left | (bottom << 1) | (nearp << 2) | (right << 3) | (top << 4);
}

constexpr uint64_t kEmptyRect = 0x0000'0000'ffff'ffffull;   // tx0=ty0=0xffff > tx1=ty1=0
// a rectangle whose far corner lies before its near corner covers no tile (the
// reference's tile loops run zero times)
__device__ __forceinline__ uint64_t pack_rect(int tx0, int ty0, int tx1, int ty1) {
    if (tx1 < tx0 || ty1 < ty0) return kEmptyRect;
    return uint64_t(uint16_t(tx0)) | (uint64_t(uint16_t(ty0)) << 16) | (uint64_t(uint16_t(tx1)) << 32) |
           (uint64_t(uint16_t(ty1) & 0x7fffu) << 48);
}
__device__ __forceinline__ bool rect_has(uint64_t r, int tx, int ty) {
    const int x0 = int(r & 0xffff), y0 = int((r >> 16) & 0xffff);
    const int x1 = int((r >> 32) & 0xffff), y1 = int((r >> 48) & 0x7fff);
    return x0 <= tx && tx <= x1 && y0 <= ty && ty <= y1;
}

// v / d (C's truncating division) for a tile size d > 0: by a shift when d is
// a power of two (every frame's d is uniform, so the test is a uniform branch
// and a runtime division is left only for other sizes)
__device__ __forceinline__ int div_tile(int v, int d) {
    if ((d & (d - 1)) == 0) return (v + ((v >> 31) & (d - 1))) >> (__ffs(d) - 1);
    return v / d;
}

// raster blocks (CTA regions) per tile
__device__ __forceinline__ int raster_subs(const FrameView& fv) {
    return ((fv.tile_w + fv.region_px - 1) / fv.region_px) * ((fv.tile_h + fv.region_px - 1) / fv.region_px);
}

// files a binned tile's raster blocks in the raster pass's work queue
// (bucket: the power of two of the tile's list length); one thread
__device__ __forceinline__ void enqueue_tile(const FrameView& fv, int tile, uint32_t cost) {
    if (fv.tile_queue == nullptr) return;
    const int b = min(kCostBuckets - 1, 32 - __clz(int(cost)));
    const int subs = raster_subs(fv) * fv.slices;   // items: (block, slice), slice fastest
    const uint32_t pos = atomicAdd(&fv.counters->bucket[b], uint32_t(subs));
    uint32_t* row = fv.tile_queue + size_t(b) * size_t(fv.queue_cap) + pos;
    for (int k = 0; k < subs; ++k) row[k] = uint32_t(tile * subs + k);
}

__device__ __forceinline__ int find_draw(const DevDraw* __restrict__ draws, int ndraws, int g) {
    int lo = 0, hi = ndraws - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&draws[mid].first_tri) <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// clipping: GPUBinImpl::ClipTriangles for one triangle (rglv_gpu_impl.hxx:678-793)
// ---------------------------------------------------------------------------
struct CV { float c[4]; float d[kMaxVary]; };

__device__ __forceinline__ bool is_inside(int plane, const float* p) {
    switch (plane) {
    case 0: return p[3] + p[0] >= 0.f;   // left
    case 1: return p[3] + p[1] >= 0.f;   // bottom
    case 2: return p[3] + p[2] >= 0.f;   // near
    case 3: return p[3] - p[0] >= 0.f;   // right
    default: return p[3] - p[1] >= 0.f;  // top
    }
}
__device__ __forceinline__ float plane_distance(int plane, const float* a, const float* b) {
    switch (plane) {
    case 0: return (a[3] + a[0]) / ((a[3] + a[0]) - (b[3] + b[0]));
    case 1: return (a[3] + a[1]) / ((a[3] + a[1]) - (b[3] + b[1]));
    case 2: return (a[3] + a[2]) / ((a[3] + a[2]) - (b[3] + b[2]));
    case 3: return (a[3] - a[0]) / ((a[3] - a[0]) - (b[3] - b[0]));
    default: return (a[3] - a[1]) / ((a[3] - a[1]) - (b[3] - b[1]));
    }
}

// ForEachCoveredTile's rectangle (rglv_gpu_impl.hxx:796-808)
__device__ __forceinline__ uint64_t fan_rect(const FrameView& fv, const int sc[4], const float* a, const float* b, const float* c) {
    const int x0 = __float2int_rz(a[0]), y0 = __float2int_rz(a[1]);
    const int x1 = __float2int_rz(b[0]), y1 = __float2int_rz(b[1]);
    const int x2 = __float2int_rz(c[0]), y2 = __float2int_rz(c[1]);
    const int vminx = max(min(x0, min(x1, x2)), sc[0]);
    const int vminy = max(min(y0, min(y1, y2)), sc[1]);
    const int vmaxx = min(max(x0, max(x1, x2)) + 1, sc[2] - 1);
    const int vmaxy = min(max(y0, max(y1, y2)) + 1, sc[3] - 1);
    return pack_rect(div_tile(vminx, fv.tile_w), div_tile(vminy, fv.tile_h), div_tile(vmaxx, fv.tile_w), div_tile(vmaxy, fv.tile_h));
}

// The three transformed vertices of a triangle, passed by value to the
// clipper: the setup keeps them in registers (a pointer would put them in
// local memory for every triangle, clipped or not).
struct TriVerts {
    float pos[3][4];
    float vary[3][kMaxVary];
};

// Returns the tile rectangle of the triangle's fans (bit 63 set), or rect_union
// when no fan survives.
__device__ __noinline__ uint64_t clip_triangle(const FrameView& fv, const DevState& s, int g, const TriVerts tv,
                                               uint64_t rect_union) {
    CV A[kMaxClipVerts + 1], B[kMaxClipVerts + 1];
    int na = 3;
    for (int i = 0; i < 3; ++i) {
        for (int k = 0; k < 4; ++k) A[i].c[k] = tv.pos[i][k];
        for (int k = 0; k < kMaxVary; ++k) A[i].d[k] = tv.vary[i][k];
    }
    const int nv = s.nvary;
    for (int plane = 0; plane < 5 && na > 0; ++plane) {   // clipping_panes order L,B,N,R,T
        bool hereIsInside = is_inside(plane, A[0].c);
        int nb = 0;
        for (int h = 0; h < na; ++h) {
            const int n = (h + 1) % na;
            const bool nextIsInside = is_inside(plane, A[n].c);
            if (hereIsInside && nb <= kMaxClipVerts) B[nb++] = A[h];
            if (hereIsInside != nextIsInside) {
                const CV& from = hereIsInside ? A[h] : A[n];
                const CV& to = hereIsInside ? A[n] : A[h];
                const float d = plane_distance(plane, from.c, to.c);
                CV o;
                for (int k = 0; k < 4; ++k) o.c[k] = (1.0f - d) * from.c[k] + d * to.c[k];
                for (int k = 0; k < kMaxVary; ++k) o.d[k] = k < nv ? (1.0f - d) * from.d[k] + d * to.d[k] : 0.f;
                if (s.program == kProgGBuffer) o.d[3] = from.d[3];   // the albedo is flat
                if (nb <= kMaxClipVerts) B[nb++] = o;
                hereIsInside = !hereIsInside;
            }
        }
        for (int i = 0; i < nb; ++i) A[i] = B[i];
        na = nb > kMaxClipVerts ? kMaxClipVerts : nb;
    }
    ClipInfo info{0, 0, 0, 0};
    if (na >= 3) {
        for (int i = 0; i < na; ++i) {
            const float iw = oneover(fv.rcp_table, A[i].c[3]);   // pdiv (rglv_math.hxx:143-152)
            A[i].c[0] = A[i].c[0] * iw; A[i].c[1] = A[i].c[1] * iw; A[i].c[2] = A[i].c[2] * iw; A[i].c[3] = iw;
            A[i].c[0] = A[i].c[0] * s.DS[0] + s.DO[0];
            A[i].c[1] = A[i].c[1] * s.DS[1] + s.DO[1];
        }
        const float d31x = A[2].c[0] - A[0].c[0], d31y = A[2].c[1] - A[0].c[1];
        const float d21x = A[1].c[0] - A[0].c[0], d21y = A[1].c[1] - A[0].c[1];
        const bool backfacing = (d31x * d21y - d31y * d21x) < 0.f;
        bool willCull = true;
        if (backfacing) { if (!s.cull_enabled || (s.cull_face & 2) == 0) willCull = false; }
        else { if (!s.cull_enabled || (s.cull_face & 1) == 0) willCull = false; }
        if (!willCull) {
            if (backfacing) {
                for (int i = 0; i < na / 2; ++i) { CV t = A[i]; A[i] = A[na - 1 - i]; A[na - 1 - i] = t; }
            }
            const uint32_t vbase = atomicAdd(&fv.counters->clip_verts, uint32_t(na));
            if (vbase + uint32_t(na) > fv.clip_cap) {
                atomicOr(&fv.counters->overflow, 1u);
            } else {
                for (int i = 0; i < na; ++i) {
                    ClipVert cvx;
                    for (int k = 0; k < 4; ++k) cvx.coord[k] = A[i].c[k];
                    for (int k = 0; k < kMaxVary; ++k) cvx.vary[k] = A[i].d[k];
                    fv.clip_verts[vbase + i] = cvx;
                    fv.clip_poly[vbase + i] = int32_t(vbase);
                }
                fv.clip_src[vbase] = g;
                int sc[4] = { s.scissor[0], s.scissor[1], s.scissor[2], s.scissor[3] };
                int ux0 = INT_MAX, uy0 = INT_MAX, ux1 = INT_MIN, uy1 = INT_MIN;
                for (int vi = 1; vi < na - 1; ++vi) {
                    const uint64_t r = fan_rect(fv, sc, A[0].c, A[vi].c, A[vi + 1].c);
                    fv.clip_fan_rect[vbase + vi] = r;
                    const int x0 = int(r & 0xffff), y0 = int((r >> 16) & 0xffff);
                    const int x1 = int((r >> 32) & 0xffff), y1 = int((r >> 48) & 0x7fff);
                    if (x0 <= x1 && y0 <= y1) {
                        ux0 = min(ux0, x0); uy0 = min(uy0, y0); ux1 = max(ux1, x1); uy1 = max(uy1, y1);
                    }
                }
                info.vbase = int32_t(vbase);
                info.nverts = na;
                info.backfacing = backfacing ? 1 : 0;
                if (ux0 <= ux1) rect_union = pack_rect(ux0, uy0, ux1, uy1) | (1ull << 63);
            }
        }
    }
    fv.clip_info[g] = info;
    return rect_union;
}

// ---------------------------------------------------------------------------
// setup
// ---------------------------------------------------------------------------
// kExt: the frame has instanced or OBJ1Program draws (fv.dext): a draw's
// triangles are its instances' triangles in instance order (BinTriangles1P/2P's
// instance loop, rglv_gpu_impl.hxx:364,554), ManyProgram vertices take their
// instance's matrix, OBJ1Program vertices are lit with the draw's view matrix.
template <bool kExt>
__device__ __forceinline__ void setup_body(const FrameView& fv, int block) {
    const int g = block * kSetupBlock + threadIdx.x;
    uint64_t rect = kEmptyRect;
    if (g < fv.ntris) {
        const int d = find_draw(fv.draws, fv.ndraws, g);
        const DevDraw dr = fv.draws[d];
        const DevState& s = fv.states[dr.state];
        int t = g - dr.first_tri;
        const float* imat = nullptr;
        const float* vm = nullptr;
        if (kExt) {
            const DevDrawExt& de = fv.dext[d];
            const int per_inst = de.per_inst;
            if (per_inst > 0) {
                const int iid = t / per_inst;
                t -= iid * per_inst;
                if (s.program == kProgMany) imat = de.matrices + size_t(iid) * 16;
            }
            if (s.program == kProgOBJ1) vm = de.vm;
        }
        int idx[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) idx[k] = dr.is_arrays ? 3 * t + k : int(__ldg(dr.indices + 3 * t + k));
        TriVerts tv;
        float dx[3], dy[3], zz[3], ww[3];
        uint32_t cf[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (kExt && imat != nullptr) shade_vertex_many(s, imat, idx[k], tv.pos[k], tv.vary[k], fv.counters);
            else if (kExt && vm != nullptr) shade_vertex_obj1(s, vm, idx[k], tv.pos[k], tv.vary[k], fv.counters);
            else shade_vertex(s, idx[k], tv.pos[k], tv.vary[k], fv.counters);
            cf[k] = frustum_test(s.guard, tv.pos[k]);
            const float iw = oneover(fv.rcp_table, tv.pos[k][3]);
            dx[k] = (tv.pos[k][0] * iw) * s.DS[0] + s.DO[0];
            dy[k] = (tv.pos[k][1] * iw) * s.DS[1] + s.DO[1];
            zz[k] = tv.pos[k][2] * iw;
            ww[k] = iw;
        }
        // BinTriangles1P (rglv_gpu_impl.hxx:605-661)
        const bool pointsOutside = int32_t(cf[0] | cf[1] | cf[2]) > 0;
        const bool primsOutside = int32_t(cf[0] & cf[1] & cf[2]) > 0;
        const bool needClip = !primsOutside && pointsOutside;
        const float d31x = dx[2] - dx[0], d31y = dy[2] - dy[0];
        const float d21x = dx[1] - dx[0], d21y = dy[1] - dy[0];
        const bool front = (d31x * d21y - d31y * d21x) > 0.f;
        const int32_t ix0 = ftoi(dx[0]), iy0 = ftoi(dy[0]);
        const int32_t ix1 = ftoi(dx[1]), iy1 = ftoi(dy[1]);
        const int32_t ix2 = ftoi(dx[2]), iy2 = ftoi(dy[2]);
        const int32_t vminx = max(min(ix0, min(ix1, ix2)), s.scissor[0]);
        const int32_t vminy = max(min(iy0, min(iy1, iy2)), s.scissor[1]);
        const int32_t vmaxx = min(wadd(max(ix0, max(ix1, ix2)), 1), s.scissor[2] - 1);
        const int32_t vmaxy = min(wadd(max(iy0, max(iy1, iy2)), 1), s.scissor[3] - 1);
        bool notCulled = (!front && s.keep_backs) || (front && s.keep_fronts);
        notCulled = notCulled && !pointsOutside;
        const bool accept = notCulled && vmaxx > vminx && vmaxy > vminy;
        if (accept) {
            // vertices in record order: back faces swap the first and last
            // (by selects: a variable index would put the arrays in local memory)
            auto sel = [front](float a0, float a2) { return front ? a0 : a2; };
            const float x0 = sel(dx[0], dx[2]), x2 = sel(dx[2], dx[0]);
            const float y0 = sel(dy[0], dy[2]), y2 = sel(dy[2], dy[0]);
            float4 q[6];   // TriRecord: fx[3], fy[3], z[3], w[3], vary[3][4]
            q[0] = make_float4(__int_as_float(ftoi(16.0f * x0)), __int_as_float(ftoi(16.0f * dx[1])),
                               __int_as_float(ftoi(16.0f * x2)), __int_as_float(ftoi(16.0f * y0)));
            q[1] = make_float4(__int_as_float(ftoi(16.0f * dy[1])), __int_as_float(ftoi(16.0f * y2)),
                               sel(zz[0], zz[2]), zz[1]);
            q[2] = make_float4(sel(zz[2], zz[0]), sel(ww[0], ww[2]), ww[1], sel(ww[2], ww[0]));
            q[3] = make_float4(sel(tv.vary[0][0], tv.vary[2][0]), sel(tv.vary[0][1], tv.vary[2][1]),
                               sel(tv.vary[0][2], tv.vary[2][2]), sel(tv.vary[0][3], tv.vary[2][3]));
            q[4] = make_float4(tv.vary[1][0], tv.vary[1][1], tv.vary[1][2], tv.vary[1][3]);
            q[5] = make_float4(sel(tv.vary[2][0], tv.vary[0][0]), sel(tv.vary[2][1], tv.vary[0][1]),
                               sel(tv.vary[2][2], tv.vary[0][2]), sel(tv.vary[2][3], tv.vary[0][3]));
            float4* dst = reinterpret_cast<float4*>(fv.tris + g);
#pragma unroll
            for (int k = 0; k < 6; ++k) dst[k] = q[k];
            const int i0 = front ? idx[0] : idx[2], i2 = front ? idx[2] : idx[0];
            const uint32_t ni0 = uint32_t(uint16_t(i0)) | (front ? 0u : 0x8000u);
            fv.rec16[2 * g] = (ni0 & 0xffffu) | (uint32_t(uint16_t(idx[1])) << 16);
            fv.rec16[2 * g + 1] = uint32_t(uint16_t(i2));
            rect = pack_rect(div_tile(vminx, fv.tile_w), div_tile(vminy, fv.tile_h), div_tile(vmaxx, fv.tile_w), div_tile(vmaxy, fv.tile_h));
        }
        if (needClip) {
            rect = clip_triangle(fv, s, g, tv, rect);
        } else {
            fv.clip_info[g] = ClipInfo{0, 0, 0, 0};
        }
        fv.bin_rect[g] = rect;
    }
    // chunk and super-chunk rectangles
    const bool nonempty = (rect & 0xffff) <= ((rect >> 32) & 0xffff) && ((rect >> 16) & 0xffff) <= ((rect >> 48) & 0x7fff);
    int x0 = nonempty ? int(rect & 0xffff) : INT_MAX;
    int y0 = nonempty ? int((rect >> 16) & 0xffff) : INT_MAX;
    int x1 = nonempty ? int((rect >> 32) & 0xffff) : INT_MIN;
    int y1 = nonempty ? int((rect >> 48) & 0x7fff) : INT_MIN;
    x0 = __reduce_min_sync(FULL_MASK, x0);
    y0 = __reduce_min_sync(FULL_MASK, y0);
    x1 = __reduce_max_sync(FULL_MASK, x1);
    y1 = __reduce_max_sync(FULL_MASK, y1);
    const int chunk = (block * kSetupBlock + threadIdx.x) >> 5;
    if ((threadIdx.x & 31) == 0 && chunk < fv.nchunks) {
        fv.chunk_rect[chunk] = make_int4(x0, y0, x1, y1);
        if (x0 <= x1) {
            int4* sr = fv.super_rect + (chunk >> 5);
            atomicMin(&sr->x, x0);
            atomicMin(&sr->y, y0);
            atomicMin(&sr->z, -x1);
            atomicMin(&sr->w, -y1);
        }
    }
}

// ---------------------------------------------------------------------------
// binning
// ---------------------------------------------------------------------------

// ---- binning: one CTA of kBinBlock threads per tile ----
// The tile's overlapping chunks are listed in triangle order (super-chunk
// masks, then chunk masks of the overlapping super-chunks, then a prefix),
// the warps count the chunks' entries in parallel (chunk k: warp k % 8), a
// prefix over the counts gives every chunk its place, and the warps write.
// Chunks are taken in windows of up to kBinChunks (consecutive overlapping
// super-chunks), and super-chunks 1024 at a time, counted in one pass and
// written in a second.  The lists are those of walking the chunks in order
// (order within a chunk: lane order; clipped fans: lane order, then fan
// order).
constexpr int kBinWarps = kBinBlock / 32;
constexpr int kBinChunks = 1024;
struct BinShared {
    uint32_t gm[32];                 // overlap masks of super-chunk groups
    uint32_t cm[1024];               // overlap masks of the chunks of the listed super-chunks
    int32_t sup[1024];               // overlapping super-chunks, in order
    int32_t pre[1024];               // exclusive prefix of their overlapping chunks
    int32_t chunk[kBinChunks];       // the window's overlapping chunks, in order
    uint32_t imask[kBinChunks];      // per chunk: lanes with an inline entry
    int32_t ninl[kBinChunks];        // per chunk: inline entries, then their prefix
    int32_t ncl[kBinChunks];         // per chunk: clipped fan entries, then their prefix
    int32_t wsum[kBinWarps];
    int nsup;
    uint32_t base;
};

// Exclusive prefix of v[0 .. n) in place (n <= 4 * kBinBlock), total returned
// (all threads of the CTA call it).  For n <= 128 one warp scans and the
// total is also left in v[n], which nothing else reads.
__device__ __forceinline__ int bin_scan(int32_t* v, int n, BinShared& S) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (n <= 128) {   // one warp scans (four values a lane): one barrier instead of two
        if (warp == 0) {
            int x[4], sum = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) { const int i = 4 * lane + k; x[k] = i < n ? v[i] : 0; sum += x[k]; }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL_MASK, incl, o);
                if (lane >= o) incl += y;
            }
            int before = incl - sum;
#pragma unroll
            for (int k = 0; k < 4; ++k) { const int i = 4 * lane + k; if (i < n) v[i] = before; before += x[k]; }
            if (lane == 31) v[n] = incl;   // the total, past the prefix (every array scanned here has room)
        }
        __syncthreads();
        return v[n];
    }
    int x[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { const int i = 4 * t + k; x[k] = i < n ? v[i] : 0; sum += x[k]; }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) S.wsum[warp] = incl;
    __syncthreads();
    int before = incl - sum, total = 0;
    for (int w = 0; w < kBinWarps; ++w) {
        if (w < warp) before += S.wsum[w];
        total += S.wsum[w];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) { const int i = 4 * t + k; if (i < n) v[i] = before; before += x[k]; }
    __syncthreads();
    return total;
}

// Entries of chunk c (32 triangles) for tile (tx, ty): the inline lanes, and
// this lane's clipped fan entries.
__device__ __forceinline__ void chunk_entries(const FrameView& fv, int c, int tx, int ty, int lane, bool& inl, int& fans) {
    const int g = c * 32 + lane;
    inl = false;
    fans = 0;
    if (g >= fv.ntris) return;
    const uint64_t br = fv.bin_rect[g];
    if (!rect_has(br, tx, ty)) return;
    if ((br >> 63) == 0) { inl = true; return; }
    const ClipInfo ci = fv.clip_info[g];
    for (int vi = 1; vi < ci.nverts - 1; ++vi) fans += rect_has(fv.clip_fan_rect[ci.vbase + vi], tx, ty) ? 1 : 0;
}

// The window of overlapping super-chunks from k0: up to kBinChunks chunks
// (a super-chunk has at most 32, so a window holds at least one).
__device__ __forceinline__ int bin_window_end(const BinShared& S, int k0, int nsup) {
    int lo = k0 + 1, hi = nsup;   // the last k1 in [k0 + 1, nsup] with pre[k1] - pre[k0] <= kBinChunks
    const int limit = S.pre[k0] + kBinChunks;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int pm = mid < nsup ? S.pre[mid] : S.pre[nsup - 1] + __popc(S.cm[nsup - 1]);
        if (pm <= limit) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The window's chunks into S.chunk, counted into S.imask / S.ninl / S.ncl;
// returns how many.
__device__ __forceinline__ int bin_window_count(const FrameView& fv, BinShared& S, int k0, int k1, int tx, int ty) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int p0 = S.pre[k0];
    for (int k = k0 + t; k < k1; k += kBinBlock) {
        int at = S.pre[k] - p0;
        for (uint32_t mm = S.cm[k]; mm; mm &= mm - 1) S.chunk[at++] = S.sup[k] * 32 + __ffs(mm) - 1;
    }
    __syncthreads();
    const int nc = (k1 < S.nsup ? S.pre[k1] : S.pre[S.nsup - 1] + __popc(S.cm[S.nsup - 1])) - p0;
    for (int k = warp; k < nc; k += kBinWarps) {
        bool inl;
        int fans;
        chunk_entries(fv, S.chunk[k], tx, ty, lane, inl, fans);
        const uint32_t mi = __ballot_sync(FULL_MASK, inl);
        const int tf = __reduce_add_sync(FULL_MASK, fans);
        if (lane == 0) { S.imask[k] = mi; S.ninl[k] = __popc(mi); S.ncl[k] = tf; }
    }
    __syncthreads();
    return nc;
}

// Lists the super-chunks of groups g0 .. g0 + gn - 1 (gn <= 32, 1024
// super-chunks) that overlap tile (tx, ty), in order, into S.sup / S.nsup,
// with their chunk masks in S.cm and the exclusive prefix of their
// overlapping chunks in S.pre (all threads of the CTA call it).
__device__ __forceinline__ void bin_list_supers(const FrameView& fv, BinShared& S, int g0, int gn, int tx, int ty) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // super-chunk group masks: group g by warp g % 8
    for (int g = warp; g < gn; g += kBinWarps) {
        const int sidx = (g0 + g) * 32 + lane;
        bool hs = false;
        if (sidx < fv.nsupers) {
            const int4 r = fv.super_rect[sidx];
            hs = r.x <= tx && tx <= -r.z && r.y <= ty && ty <= -r.w;
        }
        const uint32_t m = __ballot_sync(FULL_MASK, hs);
        if (lane == 0) S.gm[g] = m;
    }
    __syncthreads();
    // the overlapping super-chunks in order (warp 0: lane g lists group g)
    if (warp == 0) {
        const uint32_t m = lane < gn ? S.gm[lane] : 0u;
        const int c = __popc(m);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= o) incl += y;
        }
        int at = incl - c;
        for (uint32_t mm = m; mm; mm &= mm - 1) S.sup[at++] = (g0 + lane) * 32 + __ffs(mm) - 1;
        if (lane == 31) S.nsup = incl;
    }
    __syncthreads();
    const int nsup = S.nsup;
    // their chunk masks: super-chunk k by warp k % 8, and the prefix of their counts
    for (int k = warp; k < nsup; k += kBinWarps) {
        const int c = S.sup[k] * 32 + lane;
        bool hc = false;
        if (c < fv.nchunks) {
            const int4 r = fv.chunk_rect[c];
            hc = r.x <= tx && tx <= r.z && r.y <= ty && ty <= r.w;
        }
        const uint32_t m = __ballot_sync(FULL_MASK, hc);
        if (lane == 0) { S.cm[k] = m; S.pre[k] = __popc(m); }
    }
    __syncthreads();
    bin_scan(S.pre, nsup, S);
}

// One tile's lists: the overlapping super-chunks are taken 1024 at a time
// (super windows), their overlapping chunks up to kBinChunks at a time
// (chunk windows); the counts of all windows size the tile's lists, then
// the windows are visited again to write them.
__device__ __forceinline__ void bin_body(const FrameView& fv, int tile, BinShared& S) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (tile >= fv.ntiles) return;
    if (fv.counters->overflow & 1u) {
        if (t == 0) { fv.bins[tile] = TileBin{0, 0, 0, 0}; enqueue_tile(fv, tile, 0); }
        return;
    }
    const int tx = tile % fv.tiles_x, ty = tile / fv.tiles_x;
    const int ngroups = (fv.nsupers + 31) / 32;
    const int nsw = (ngroups + 31) / 32;
    // count, window by window
    int tinl = 0, tcl = 0;
    for (int sw = 0; sw < nsw; ++sw) {
        bin_list_supers(fv, S, sw * 32, min(32, ngroups - sw * 32), tx, ty);
        const int nsup = S.nsup;
        for (int k0 = 0; k0 < nsup;) {
            const int k1 = bin_window_end(S, k0, nsup);
            const int nc = bin_window_count(fv, S, k0, k1, tx, ty);
            tinl += bin_scan(S.ninl, nc, S);
            tcl += bin_scan(S.ncl, nc, S);
            k0 = k1;
        }
    }
    if (t == 0) {
        uint32_t off = 0;
        if (tinl + tcl > 0) off = atomicAdd(&fv.counters->bin_used, uint32_t(tinl + tcl));
        if (off + uint32_t(tinl + tcl) > fv.bin_cap) {
            atomicOr(&fv.counters->overflow, 2u);
            fv.bins[tile] = TileBin{0, 0, 0, 0};
            off = 0xffffffffu;
        } else {
            fv.bins[tile] = TileBin{off, uint32_t(tinl), off + uint32_t(tinl), uint32_t(tcl)};
        }
        enqueue_tile(fv, tile, uint32_t(tinl + tcl));
        S.base = off;
    }
    __syncthreads();
    const uint32_t base = S.base;
    if (base == 0xffffffffu) return;
    uint32_t* inl_out = fv.bin_pool + base;
    uint32_t* clip_out = fv.bin_pool + base + tinl;
    const uint32_t lt = (1u << lane) - 1u;
    // write, window by window (the first chunk window's counts are recounted
    // unless it was the only window)
    int winl = 0, wcl = 0;
    for (int sw = 0; sw < nsw; ++sw) {
        if (nsw > 1) bin_list_supers(fv, S, sw * 32, min(32, ngroups - sw * 32), tx, ty);
        const int nsup = S.nsup;
        for (int k0 = 0; k0 < nsup;) {
            const int k1 = bin_window_end(S, k0, nsup);
            int nc;
            if (nsw == 1 && k0 == 0 && k1 == nsup) {
                nc = S.pre[nsup - 1] + __popc(S.cm[nsup - 1]);   // still in place from the count
            } else {
                nc = bin_window_count(fv, S, k0, k1, tx, ty);
                bin_scan(S.ninl, nc, S);
                bin_scan(S.ncl, nc, S);
            }
            for (int k = warp; k < nc; k += kBinWarps) {
                const int c = S.chunk[k];
                const uint32_t mi = S.imask[k];
                if (mi & (1u << lane)) inl_out[winl + S.ninl[k] + __popc(mi & lt)] = uint32_t(c * 32 + lane);
                bool inl;
                int fans;
                const bool has_fans = k + 1 < nc ? S.ncl[k + 1] != S.ncl[k] : true;
                if (!has_fans) continue;
                chunk_entries(fv, c, tx, ty, lane, inl, fans);
                if (!__any_sync(FULL_MASK, fans != 0)) continue;
                int incl = fans;
    #pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL_MASK, incl, o);
                    if (lane >= o) incl += y;
                }
                if (fans) {
                    const ClipInfo ci = fv.clip_info[c * 32 + lane];
                    uint32_t pos = uint32_t(wcl + S.ncl[k] + incl - fans);
                    for (int vi = 1; vi < ci.nverts - 1; ++vi)
                        if (rect_has(fv.clip_fan_rect[ci.vbase + vi], tx, ty)) clip_out[pos++] = uint32_t(ci.vbase + vi);
                }
            }
            // the window's totals (from the last chunk's prefix and count)
            if (nc > 0) {
                winl += S.ninl[nc - 1] + __popc(S.imask[nc - 1]);
                // clip total: recount the last chunk's fans (cheap; rarely any)
                bool inl;
                int fans;
                chunk_entries(fv, S.chunk[nc - 1], tx, ty, lane, inl, fans);
                wcl += S.ncl[nc - 1] + __reduce_add_sync(FULL_MASK, fans);
            }
            __syncthreads();
            k0 = k1;
        }
    }
}

// ---------------------------------------------------------------------------
// raster
// ---------------------------------------------------------------------------
// per-(triangle, tile) rasteriser setup: the bounding box clamped to the tile
// and aligned to quads, the three edge values at its first quad and their
// steps, and 1 / (c1 + c2 + c3)
struct TriSetup {
    int32_t minx, miny, maxx, maxy;
    int32_t c1, c2, c3;
    int32_t dy12, dx12, dy23, dx23, dy31, dx31;
    float scale;
};

// structure of arrays in shared memory, one batch of triangles
template <int N>
struct RasterSmem {
    int32_t minx[N], miny[N], maxx[N], maxy[N];
    int32_t c1[N], c2[N], c3[N];
    int32_t dy12[N], dx12[N], dy23[N], dx23[N];
    int32_t dy31[N], dx31[N];
    float scale[N];
    float z[3][N], w[3][N];
    float vary[3][kMaxVary][N];
    uint32_t code[N];   // fragment owner: triangle id, or clipped fan id | bit 31
    uint32_t order[N];  // visibility by keys: the entry's drawing order (see frag_key)
    FrameOp ops[kOpCache];         // the frame's ops, when they fit
    int32_t dfirst[kOpCache];      // the draws' first triangles, when they fit
    uint8_t big[N];     // visibility by keys: the triangle covers many quads of the region
    uint32_t zr[N];     // visibility by keys: a depth rank no covered pixel of the triangle goes below
                                   // (0 where no such bound is known)
    int qsum;                      // visibility by keys: the batch's boxes, in quads of the region
    const FrameOp* ops_of;         // the frame whose ops and draw starts are in ops / dfirst (a CTA
                                   // taking several blocks of one frame loads them once)
};

// VTriangleRasterizer setup for one lane (rglv_triangle.hxx:209-240), int32 wrap
__device__ __forceinline__ void setup_vector(TriSetup& t, const int rect[4],
                                             int32_t x1, int32_t x2, int32_t x3, int32_t y1, int32_t y2, int32_t y3) {
    int32_t vminx = max(min(min(x1, x2), x3) >> 4, rect[0]);
    const int32_t vmaxx = min(wadd(max(max(x1, x2), x3), 15) >> 4, rect[2]);
    int32_t vminy = max(min(min(y1, y2), y3) >> 4, rect[1]);
    const int32_t vmaxy = min(wadd(max(max(y1, y2), y3), 15) >> 4, rect[3]);
    vminx &= ~1; vminy &= ~1;
    const int32_t dx12 = wsub(x1, x2), dy12 = wsub(y2, y1);
    const int32_t dx23 = wsub(x2, x3), dy23 = wsub(y3, y2);
    const int32_t dx31 = wsub(x3, x1), dy31 = wsub(y1, y3);
    const int32_t sx = wadd(int32_t(uint32_t(vminx) << 4), 8);
    const int32_t sy = wadd(int32_t(uint32_t(vminy) << 4), 8);
    int32_t c1 = wadd(wmul(dy12, wsub(sx, x1)), wmul(dx12, wsub(sy, y1)));
    int32_t c2 = wadd(wmul(dy23, wsub(sx, x2)), wmul(dx23, wsub(sy, y2)));
    int32_t c3 = wadd(wmul(dy31, wsub(sx, x3)), wmul(dx31, wsub(sy, y3)));
    const int tl12 = dy12 > 0 || (dy12 == 0 && dx12 > 0);
    const int tl23 = dy23 > 0 || (dy23 == 0 && dx23 > 0);
    const int tl31 = dy31 > 0 || (dy31 == 0 && dx31 > 0);
    c1 = wsub(wadd(c1, tl12), 1) >> 4;
    c2 = wsub(wadd(c2, tl23), 1) >> 4;
    c3 = wsub(wadd(c3, tl31), 1) >> 4;
    t.minx = vminx; t.miny = vminy; t.maxx = vmaxx; t.maxy = vmaxy;
    t.c1 = c1; t.c2 = c2; t.c3 = c3;
    t.dy12 = dy12; t.dx12 = dx12; t.dy23 = dy23; t.dx23 = dx23; t.dy31 = dy31; t.dx31 = dx31;
    t.scale = __fdiv_rn(1.0f, itof(wadd(wadd(c1, c2), c3)));
}

// TriangleRasterizer setup (rglv_triangle.hxx:79-131), int64
__device__ __forceinline__ void setup_scalar(TriSetup& t, const int rect[4],
                                             int x1, int x2, int x3, int y1, int y2, int y3) {
    int minx = max(min(x1, min(x2, x3)) >> 4, rect[0]);
    const int endx = min((max(x1, max(x2, x3)) + 15) >> 4, rect[2]);
    int miny = max(min(y1, min(y2, y3)) >> 4, rect[1]);
    const int endy = min((max(y1, max(y2, y3)) + 15) >> 4, rect[3]);
    minx &= ~1; miny &= ~1;
    const int64_t dx12 = x1 - x2, dy12 = y2 - y1;
    const int64_t dx23 = x2 - x3, dy23 = y3 - y2;
    const int64_t dx31 = x3 - x1, dy31 = y1 - y3;
    const int64_t sx = (minx << 4) + 8, sy = (miny << 4) + 8;
    int64_t c1 = dy12 * (sx - x1) + dx12 * (sy - y1);
    int64_t c2 = dy23 * (sx - x2) + dx23 * (sy - y2);
    int64_t c3 = dy31 * (sx - x3) + dx31 * (sy - y3);
    if (dy12 > 0 || (dy12 == 0 && dx12 > 0)) c1++;
    --c1;
    if (dy23 > 0 || (dy23 == 0 && dx23 > 0)) c2++;
    --c2;
    if (dy31 > 0 || (dy31 == 0 && dx31 > 0)) c3++;
    --c3;
    c1 >>= 4; c2 >>= 4; c3 >>= 4;
    t.minx = minx; t.miny = miny; t.maxx = endx; t.maxy = endy;
    t.c1 = int32_t(c1); t.c2 = int32_t(c2); t.c3 = int32_t(c3);
    t.dy12 = int32_t(dy12); t.dx12 = int32_t(dx12);
    t.dy23 = int32_t(dy23); t.dx23 = int32_t(dx23);
    t.dy31 = int32_t(dy31); t.dx31 = int32_t(dx31);
    t.scale = __fdiv_rn(1.0f, __ll2float_rn(c1 + c2 + c3));
}

template <int N>
__device__ __forceinline__ void put_setup(RasterSmem<N>& S, int i, const TriSetup& t) {
    S.minx[i] = t.minx; S.miny[i] = t.miny; S.maxx[i] = t.maxx; S.maxy[i] = t.maxy;
    S.c1[i] = t.c1; S.c2[i] = t.c2; S.c3[i] = t.c3;
    S.dy12[i] = t.dy12; S.dx12[i] = t.dx12; S.dy23[i] = t.dy23; S.dx23[i] = t.dx23;
    S.dy31[i] = t.dy31; S.dx31[i] = t.dx31;
    S.scale[i] = t.scale;
}

// Edge values of one lane of quad (qx, qy): the quad walk adds 2*dy per quad
// column and 2*dx per quad row to the first quad's values, lane l adds dy for
// x+1 and dx for y+1 -- all wrapping 32-bit sums, so the direct form is equal.
__device__ __forceinline__ void lane_edges(const TriSetup& t, int qx, int qy, int l, int32_t& e1, int32_t& e2, int32_t& e3) {
    const int32_t kx = qx - t.minx + (l & 1), ky = qy - t.miny + (l >> 1);
    e1 = wadd(wadd(t.c1, wmul(kx, t.dy12)), wmul(ky, t.dx12));
    e2 = wadd(wadd(t.c2, wmul(kx, t.dy23)), wmul(ky, t.dx23));
    e3 = wadd(wadd(t.c3, wmul(kx, t.dy31)), wmul(ky, t.dx31));
}

// Texel fetch for the nearest samplers: their offsets come from fract() of
// the coordinate, which is negative for coordinates below -10 (-100 for the
// non-power-of-two unit), where the reference reads outside the texture;
// here such texels read as zero.
__device__ __forceinline__ float4 texel(const DevTexture& tu, int32_t ofs4) {
    const int32_t t = ofs4 >> 2;
    if (t < 0 || t >= tu.texels) return make_float4(0.f, 0.f, 0.f, 0.f);
    return __ldg(reinterpret_cast<const float4*>(tu.buf) + t);
}

// texture units (src/rgl/rglr/rglr_texture_sampler.cxx)
__device__ __forceinline__ void tex_sample(const DevTexture& tu, const float u[4], const float v[4], float out[4][4]) {
    const float almostone = u2f(0x3f7fffffu);
    if (tu.kind == 2) {   // NM_ONEMAP_WRAP_NEAREST (:289-311)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int32_t pu = ftoi(fract(u[l] + 100.0f) * float(tu.width));
            const int32_t pv = ftoi((almostone - fract(v[l] + 100.0f)) * float(tu.height));
            const float4 px = texel(tu, wmul(wadd(wmul(pv, tu.stride), pu), 4));
            out[l][0] = px.x; out[l][1] = px.y; out[l][2] = px.z; out[l][3] = px.w;
        }
        return;
    }
    const int P = tu.power;
    const float baseDim = float(1 << P);
    // LevelOfDetail (:25-42), coarse: lanes 1 - 0
    const float dux = u[1] * baseDim - u[0] * baseDim;
    const float dvx = v[1] * baseDim - v[0] * baseDim;
    const float sqd = dux * dux + dvx * dvx;
    int lod = (int32_t(f2u(sqd)) - (127 << 23)) >> 24;
    lod = lod < 0 ? 0 : (lod > P ? P : lod);
    if (tu.kind == 0) {   // P2_MIPMAP_WRAP_NEAREST (:63-109)
        const float levelDim = float(1 << (P - lod));
        const int32_t levelBeginRow = int32_t((0xfffffffeu << (P - lod)) & ((1u << (P + 1)) - 1u));
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int32_t lx = ftoi(fract(u[l] + 10.0f) * levelDim);
            const int32_t ly = ftoi((almostone - fract(v[l] + 10.0f)) * levelDim);
            const float4 px = texel(tu, wmul(wadd(int32_t(uint32_t(wadd(levelBeginRow, ly)) << P), lx), 4));
            out[l][0] = px.x; out[l][1] = px.y; out[l][2] = px.z; out[l][3] = px.w;
        }
        return;
    }
    // P2_MIPMAP_WRAP_LINEAR (:172-286)
    const int levelDim = 1 << (P - lod);
    const int32_t wrapMask = levelDim - 1;
    const int32_t levelLastRow = int32_t(((0xffffffffu << (P - lod)) & ((1u << (P + 1)) - 1u)) - 1u);
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const float levelX = u[l] * float(levelDim);
        const float levelY = v[l] * float(levelDim);
        int32_t tx0 = ftoi(levelX - 0.5f), ty0 = ftoi(levelY - 0.5f);
        int32_t tx1 = wadd(tx0, 1), ty1 = wadd(ty0, 1);
        const float fx = (levelX - itof(tx0)) - 0.5f;
        const float fy = (levelY - itof(ty0)) - 0.5f;
        const float fx1 = 1.0f - fx, fy1 = 1.0f - fy;
        const float w00 = fx1 * fy1, w10 = fx * fy1, w01 = fx1 * fy, w11 = fx * fy;
        tx0 &= wrapMask; ty0 &= wrapMask; tx1 &= wrapMask; ty1 &= wrapMask;
        const int32_t y0 = wsub(levelLastRow, ty0), y1 = wsub(levelLastRow, ty1);
        const float4 p00 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y0) << P), tx0));
        const float4 p10 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y0) << P), tx1));
        const float4 p01 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y1) << P), tx0));
        const float4 p11 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y1) << P), tx1));
        out[l][0] = ((p00.x * w00 + p10.x * w10) + p01.x * w01) + p11.x * w11;
        out[l][1] = ((p00.y * w00 + p10.y * w10) + p01.y * w01) + p11.y * w11;
        out[l][2] = ((p00.z * w00 + p10.z * w10) + p01.z * w01) + p11.z * w11;
        out[l][3] = ((p00.w * w00 + p10.w * w10) + p01.w * w01) + p11.w * w11;
    }
}

// LINEAR mip sampler for one lane, with the quad's coarse LoD taken from
// lanes 0 and 1 (u0,v0), (u1,v1) exactly as the four-lane sampler does
__device__ __forceinline__ void tex_sample_lane(const DevTexture& tu, float u0, float v0, float u1, float v1,
                                                float ul, float vl, float out[4]) {
    float u[4] = { u0, u1, ul, ul }, v[4] = { v0, v1, vl, vl };
    float o[4][4];
    if (tu.kind == 1) {
        // only the LoD needs lanes 0 and 1; sample lane l alone
        const int P = tu.power;
        const float baseDim = float(1 << P);
        const float dux = u1 * baseDim - u0 * baseDim;
        const float dvx = v1 * baseDim - v0 * baseDim;
        const float sqd = dux * dux + dvx * dvx;
        int lod = (int32_t(f2u(sqd)) - (127 << 23)) >> 24;
        lod = lod < 0 ? 0 : (lod > P ? P : lod);
        const int levelDim = 1 << (P - lod);
        const int32_t wrapMask = levelDim - 1;
        const int32_t levelLastRow = int32_t(((0xffffffffu << (P - lod)) & ((1u << (P + 1)) - 1u)) - 1u);
        const float levelX = ul * float(levelDim);
        const float levelY = vl * float(levelDim);
        int32_t tx0 = ftoi(levelX - 0.5f), ty0 = ftoi(levelY - 0.5f);
        int32_t tx1 = wadd(tx0, 1), ty1 = wadd(ty0, 1);
        const float fx = (levelX - itof(tx0)) - 0.5f;
        const float fy = (levelY - itof(ty0)) - 0.5f;
        const float fx1 = 1.0f - fx, fy1 = 1.0f - fy;
        const float w00 = fx1 * fy1, w10 = fx * fy1, w01 = fx1 * fy, w11 = fx * fy;
        tx0 &= wrapMask; ty0 &= wrapMask; tx1 &= wrapMask; ty1 &= wrapMask;
        const int32_t y0 = wsub(levelLastRow, ty0), y1 = wsub(levelLastRow, ty1);
        const float4 p00 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y0) << P), tx0));
        const float4 p10 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y0) << P), tx1));
        const float4 p01 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y1) << P), tx0));
        const float4 p11 = __ldg(reinterpret_cast<const float4*>(tu.buf) + wadd(int32_t(uint32_t(y1) << P), tx1));
        out[0] = ((p00.x * w00 + p10.x * w10) + p01.x * w01) + p11.x * w11;
        out[1] = ((p00.y * w00 + p10.y * w10) + p01.y * w01) + p11.y * w11;
        out[2] = ((p00.z * w00 + p10.z * w10) + p01.z * w01) + p11.z * w11;
        out[3] = ((p00.w * w00 + p10.w * w10) + p01.w * w01) + p11.w * w11;
        return;
    }
    tex_sample(tu, u, v, o);
    out[0] = o[2][0]; out[1] = o[2][1]; out[2] = o[2][2]; out[3] = o[2][3];
}

// fragment-stage constants of the current state, held in registers
struct FragState {
    int program, nvary;
    int depth_test, depth_func, depth_write, color_write, blend, scissor;
    DevTexture tu0;
};

// from a kOpState op (its switches are inline); the texture unit only for
// blended draws, which shade as they draw
__device__ __forceinline__ void load_frag_state(const FrameView& fv, const FrameOp& o, FragState& f) {
    const int32_t fl = o.info[1];
    f.program = o.info[0];
    f.depth_test = (fl & kFragDepthTest) != 0; f.depth_func = (fl >> kFragDepthFuncShift) & 3;
    f.depth_write = (fl & kFragDepthWrite) != 0; f.color_write = (fl & kFragColorWrite) != 0;
    f.blend = (fl & kFragBlend) != 0; f.scissor = (fl & kFragScissor) != 0;
    if (f.blend) f.tu0 = fv.states[o.arg].tu0;
}

// The rectangle a draw rasterises in: the tile, cut to the scissor rectangle
// when the state's scissor test is on (GPUTileImpl::DrawTriangles /
// DrawClipped: Intersect(rect, scissor), rglv_gpu_impl.hxx:848-849,953-954).
// The quad walk starts at even coordinates, so a quad can reach one pixel
// past an odd edge of it; the reference masks those lanes (ScissorFlags,
// rglv_triangle.hxx:23-28,268-292), which is the same as leaving out pixels
// outside the rectangle.
__device__ __forceinline__ void draw_rect(const DevState& s, const int tile[4], int out[4]) {
    if (s.scissor_test) {
        out[0] = max(tile[0], s.scissor[0]); out[1] = max(tile[1], s.scissor[1]);
        out[2] = min(tile[2], s.scissor[2]); out[3] = min(tile[3], s.scissor[3]);
    } else {
        out[0] = tile[0]; out[1] = tile[1]; out[2] = tile[2]; out[3] = tile[3];
    }
}

// sRGB8 encode with this library's own table (see rsrgpu_host.cu)
__device__ __forceinline__ uint32_t srgb8(const uint8_t* __restrict__ lut, float v) {
    const float c = sse_min(sse_max(v, u2f((127u - 13u) << 23)), u2f(0x3f7fffffu));
    return __ldg(lut + ((f2u(c) >> 12) - ((127u - 13u) << 11)));
}
__device__ __forceinline__ uint32_t basic8(float v) {   // to_tc_basic (rglr_canvas_util.hxx:22-31)
    return uint32_t(ftoi(sse_max(sse_min(v, 1.0f), 0.0f) * 255.0f));
}

__device__ __forceinline__ bool depth_pass(int func, float frag, float dest) {
    return func == 0 ? (frag < dest) : (func == 1 ? (frag <= dest) : (frag == dest));
}

constexpr uint32_t kNoOwner = 0xffffffffu;
constexpr uint32_t kClippedBit = 0x80000000u;
constexpr uint32_t kKeyPosBits = 19;   // the list-position bits of a key's order (see frag_key)

// Per-(triangle, tile) setup and vertex data of one list entry, for the
// resolve pass: the triangle that last wrote a pixel is set up again exactly
// as when it was rasterised.
// first_s / state_s (or null): the draws' first triangles and states in
// shared memory, for the draw search
template <bool kScissor>
__device__ __forceinline__ void owner_setup_inline(const FrameView& fv, uint32_t code, const int tile[4], TriSetup& t,
                                                   float w[3], float vary[3][kMaxVary], int& state,
                                                   const int* first_s = nullptr, const int* state_s = nullptr) {
    const int g = (code & kClippedBit) ? fv.clip_src[fv.clip_poly[code & ~kClippedBit]] : int(code);
    int rect[4] = { tile[0], tile[1], tile[2], tile[3] };
    if (kScissor && fv.any_scissor) {   // the draw's rectangle depends on its state
        state = fv.draws[find_draw(fv.draws, fv.ndraws, g)].state;
        draw_rect(fv.states[state], tile, rect);
    }
    if (code & kClippedBit) {
        const uint32_t e = code & ~kClippedBit;
        const int pbase = fv.clip_poly[e];
        const ClipVert v0 = fv.clip_verts[pbase], v1 = fv.clip_verts[e], v2 = fv.clip_verts[e + 1];
        setup_scalar(t, rect,
                     __float2int_rz(v0.coord[0] * 16.0f), __float2int_rz(v1.coord[0] * 16.0f), __float2int_rz(v2.coord[0] * 16.0f),
                     __float2int_rz(v0.coord[1] * 16.0f), __float2int_rz(v1.coord[1] * 16.0f), __float2int_rz(v2.coord[1] * 16.0f));
        w[0] = v0.coord[3]; w[1] = v1.coord[3]; w[2] = v2.coord[3];
        for (int q = 0; q < kMaxVary; ++q) { vary[0][q] = v0.vary[q]; vary[1][q] = v1.vary[q]; vary[2][q] = v2.vary[q]; }
    } else {
        const float4* rp = reinterpret_cast<const float4*>(fv.tris + g);
        TriRecord r;
        float4* rr = reinterpret_cast<float4*>(&r);
        for (int q = 0; q < 6; ++q) rr[q] = __ldg(rp + q);
        setup_vector(t, rect, r.fx[0], r.fx[1], r.fx[2], r.fy[0], r.fy[1], r.fy[2]);
        for (int k = 0; k < 3; ++k) {
            w[k] = r.w[k];
            for (int q = 0; q < kMaxVary; ++q) vary[k][q] = r.vary[k][q];
        }
    }
    if (!(kScissor && fv.any_scissor)) {
        if (first_s != nullptr) {
            int lo = 0, hi = fv.ndraws - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (first_s[mid] <= g) lo = mid; else hi = mid - 1;
            }
            state = state_s[lo];
        } else {
            state = fv.draws[find_draw(fv.draws, fv.ndraws, g)].state;
        }
    }
}
// the raster kernels call it out of line (their register budget)
template <bool kScissor>
__device__ __noinline__ void owner_setup(const FrameView& fv, uint32_t code, const int tile[4], TriSetup& t,
                                         float w[3], float vary[3][kMaxVary], int& state) {
    owner_setup_inline<kScissor>(fv, code, tile, t, w, vary, state);
}

// perspective-correct barycentrics of one lane (TriangleProgram::Render,
// rglv_gpu_impl.hxx:187-191)
__device__ __forceinline__ void lane_bary(const FrameView& fv, const TriSetup& t, const float w[3], int qx, int qy, int l,
                                          float& px, float& py, float& pz) {
    int32_t e1, e2, e3;
    lane_edges(t, qx, qy, l, e1, e2, e3);
    const float bx = itof(e2) * t.scale;
    const float bz = itof(e1) * t.scale;
    const float by = (1.0f - bx) - bz;
    const float fragW = oneover(fv.rcp_table, (bx * w[0] + by * w[1]) + bz * w[2]);
    px = (w[0] * bx) * fragW;
    pz = (w[2] * bz) * fragW;
    py = (1.0f - px) - pz;
}

// Shades every pixel of the quad whose last visible fragment is still
// pending, with the owning triangle's program, and writes the colour.
// Element l of a four-lane quad array, with constant indices only: the loops
// over the quad's lanes below stay rolled (their bodies are large), and an
// array indexed by a variable would live in local memory for the whole kernel.
template <typename T>
__device__ __forceinline__ T quad_get(const T a[4], int l) {
    return l == 0 ? a[0] : l == 1 ? a[1] : l == 2 ? a[2] : a[3];
}
__device__ __forceinline__ void quad_put_rgb(float col[4][3], int l, float r, float g, float b) {
    if (l == 0) { col[0][0] = r; col[0][1] = g; col[0][2] = b; }
    else if (l == 1) { col[1][0] = r; col[1][1] = g; col[1][2] = b; }
    else if (l == 2) { col[2][0] = r; col[2][1] = g; col[2][2] = b; }
    else { col[3][0] = r; col[3][1] = g; col[3][2] = b; }
}

// The colour of lane l of the quad at (qx, qy), shaded by its owning
// triangle (set up by owner_setup) with the owner's program.
template <bool kExt>
__device__ __forceinline__ void owner_color(const FrameView& fv, const TriSetup& t, const float w[3],
                                            const float vary[3][kMaxVary], int state, int qx, int qy, int l, float c[3]) {
    const DevState& s = fv.states[state];
    if (s.program == kProgAmy) {
        // the LoD's lanes 0 and 1, and this lane's coordinates (a lane of the
        // quad's top row is one of those two)
        float b0x, b0y, b0z, b1x, b1y, b1z;
        lane_bary(fv, t, w, qx, qy, 0, b0x, b0y, b0z);
        lane_bary(fv, t, w, qx, qy, 1, b1x, b1y, b1z);
        const float u0 = (b0x * vary[0][0] + b0y * vary[1][0]) + b0z * vary[2][0];
        const float v0 = (b0x * vary[0][1] + b0y * vary[1][1]) + b0z * vary[2][1];
        const float u1 = (b1x * vary[0][0] + b1y * vary[1][0]) + b1z * vary[2][0];
        const float v1 = (b1x * vary[0][1] + b1y * vary[1][1]) + b1z * vary[2][1];
        float ul, vl;
        if (l == 0) {
            ul = u0; vl = v0;
        } else if (l == 1) {
            ul = u1; vl = v1;
        } else {
            float bpx, bpy, bpz;
            lane_bary(fv, t, w, qx, qy, l, bpx, bpy, bpz);
            ul = (bpx * vary[0][0] + bpy * vary[1][0]) + bpz * vary[2][0];
            vl = (bpx * vary[0][1] + bpy * vary[1][1]) + bpz * vary[2][1];
        }
        float o[4];
        const DevTexture tu = s.tu0;
        tex_sample_lane(tu, u0, v0, u1, v1, ul, vl, o);
        c[0] = o[0]; c[1] = o[1]; c[2] = o[2];
    } else {
        float bpx, bpy, bpz;
        lane_bary(fv, t, w, qx, qy, l, bpx, bpy, bpz);
#pragma unroll
        for (int q = 0; q < 3; ++q) c[q] = (bpx * vary[0][q] + bpy * vary[1][q]) + bpz * vary[2][q];
        // ManyProgram::ShadeFragment (shaders.hxx:567-582): (u, v, magic, 1)
        if (kExt && s.program == kProgMany) c[2] = s.uniforms[0];
    }
}

template <bool kExt, bool kScissor>
__device__ __forceinline__ void resolve_quad(const FrameView& fv, const int rect[4], int qx, int qy,
                                             uint32_t own[4], float col[4][3]) {
    uint32_t cur = kNoOwner;
    TriSetup t;
    float w[3], vary[3][kMaxVary];
    int state = 0;
#pragma unroll 1
    for (int l = 0; l < 4; ++l) {
        const uint32_t ol = quad_get(own, l);
        if (ol == kNoOwner) continue;
        if (ol != cur) {
            cur = ol;
            owner_setup<kScissor>(fv, cur, rect, t, w, vary, state);
        }
        float c[3];
        owner_color<kExt>(fv, t, w, vary, state, qx, qy, l, c);
        quad_put_rgb(col, l, c[0], c[1], c[2]);
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) own[l] = kNoOwner;
}

// ---- visibility by (depth, order) keys ----
// In a frame whose draws are all opaque (no blending) with depth test and
// depth write on and one depth function, LESS or LEQUAL, and whose clears
// all come before its first draw and stores after its last, the fragment
// that ends up owning a pixel is the one with the least depth, ties going to
// the earliest (LESS) or latest (LEQUAL) in drawing order, among those that
// pass against the cleared depth.  That is a minimum over 64-bit keys
// (depth rank, order rank), so the fragments of a batch can be taken in any
// order -- one triangle per lane -- with shared-memory atomicMin, and the
// owners and depths are those of drawing them one after another.
//   depth rank: an order-preserving map of the float bits (-0 ranks with +0,
//     as the comparison treats them; NaN depths never pass and are skipped);
//   order rank: draw index (12 bits), inline / clipped pass (1 bit),
//     position in the tile's list (19 bits) -- the drawing order within a tile.
constexpr int kKeySmallQuads = 16;  // triangles covering at most this many quads of the region go one per lane,
constexpr int kKeyTinyQuads = 2;    // or this many where the batch's boxes cover the region more than
constexpr int kKeyCrowded = 6;      // kKeyCrowded times over

__device__ __forceinline__ uint32_t depth_rank(float z) {
    uint32_t b = __float_as_uint(z);
    if ((b & 0x7fffffffu) == 0u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float rank_depth(uint32_t r) {   // inverse of depth_rank (+0 for the zero rank)
    return __uint_as_float((r & 0x80000000u) ? (r & 0x7fffffffu) : ~r);
}
__device__ __forceinline__ unsigned long long frag_key(float z, uint32_t order, bool leq) {
    return (static_cast<unsigned long long>(depth_rank(z)) << 32) | (leq ? 0xfffffffeu - order : order + 1u);
}
__device__ __forceinline__ unsigned long long clear_key(float z, bool leq) {
    return (static_cast<unsigned long long>(depth_rank(z)) << 32) | (leq ? 0xffffffffu : 0u);
}

// A lower bound of the depth rank of every fragment the triangle covers in
// the tile, or 0 (no bound) where none is known.  Inside the triangle the
// barycentric weights bx = l2 * scale, bz = l1 * scale, by = (1 - bx) - bz are
// within a few float roundings of [0, 1] and sum to 1 within a few ulps, as
// long as the edge values keep their exact integer values there (no 32-bit
// wrap in the tile: |c| + |dy| (tile width + 2) + |dx| (tile height + 2) below
// 2^31 for every edge), so every fragment depth
// (bx z0 + by z1) + bz z2 is at least min(z) - 2^-18 max|z|.
template <int N>
__device__ __forceinline__ uint32_t tri_min_rank(const RasterSmem<N>& S, int i, int tw, int th) {
    const float scale = S.scale[i];
    if (!(scale > 0.0f && scale <= 3.4e38f)) return 0u;
    const float z0 = S.z[0][i], z1 = S.z[1][i], z2 = S.z[2][i];
    const float zabs = fmaxf(fmaxf(fabsf(z0), fabsf(z1)), fabsf(z2));
    if (!(zabs <= 3.4e38f)) return 0u;   // an infinite or NaN vertex depth
    const long long W = tw + 2, H = th + 2;
    const long long lim = 1ll << 31;
    if (llabs(S.c1[i]) + llabs(S.dy12[i]) * W + llabs(S.dx12[i]) * H >= lim ||
        llabs(S.c2[i]) + llabs(S.dy23[i]) * W + llabs(S.dx23[i]) * H >= lim ||
        llabs(S.c3[i]) + llabs(S.dy31[i]) * W + llabs(S.dx31[i]) * H >= lim)
        return 0u;
    const float lo = fminf(fminf(z0, z1), z2) - (zabs * 0x1p-18f + 0x1p-126f);
    return depth_rank(lo);
}

// Whether edge (c, dy, dx) is negative at every pixel of [x0, x1) x [y0, y1):
// its exact value at the rectangle's corners (int64) is below zero and not
// below -2^31, so the 32-bit lane values, which wrap, equal the exact ones
// there and all lanes of the rectangle are outside the triangle.
__device__ __forceinline__ bool edge_outside(int32_t c, int32_t dy, int32_t dx, int32_t kx0, int32_t ky0, int32_t kx1,
                                             int32_t ky1) {
    const long long hi = (long long)c + (long long)dy * (dy > 0 ? kx1 : kx0) + (long long)dx * (dx > 0 ? ky1 : ky0);
    const long long lo = (long long)c + (long long)dy * (dy > 0 ? kx0 : kx1) + (long long)dx * (dx > 0 ? ky0 : ky1);
    return hi < 0 && lo >= -(1ll << 31);
}
// Batch triangle i covers no pixel of [x0, x1) x [y0, y1) (pixel coordinates).
template <int N>
__device__ __forceinline__ bool footprint_outside(const RasterSmem<N>& S, int i, int x0, int y0, int x1, int y1) {
    const int32_t kx0 = x0 - S.minx[i], kx1 = x1 - 1 - S.minx[i];
    const int32_t ky0 = y0 - S.miny[i], ky1 = y1 - 1 - S.miny[i];
    return edge_outside(S.c1[i], S.dy12[i], S.dx12[i], kx0, ky0, kx1, ky1) ||
           edge_outside(S.c2[i], S.dy23[i], S.dx23[i], kx0, ky0, kx1, ky1) ||
           edge_outside(S.c3[i], S.dy31[i], S.dx31[i], kx0, ky0, kx1, ky1);
}

// The largest depth rank among the keys of the warp's quads: a fragment of
// greater rank changes none of them (keys only decrease).
__device__ __forceinline__ uint32_t warp_max_rank(const unsigned long long kq[4], bool active) {
    uint32_t r = 0u;
    if (active) {
#pragma unroll
        for (int l = 0; l < 4; ++l) r = max(r, uint32_t(kq[l] >> 32));
    }
    return __reduce_max_sync(FULL_MASK, r);
}

// Quads of the region [rx0, rx1) x [ry0, ry1) in batch triangle i's box.
template <int N>
__device__ __forceinline__ int region_quads(const RasterSmem<N>& S, int i, int rx0, int ry0, int rx1, int ry1) {
    const int x0 = max(S.minx[i], rx0), x1 = min(S.maxx[i], rx1);
    const int y0 = max(S.miny[i], ry0), y1 = min(S.maxy[i], ry1);
    return x0 < x1 && y0 < y1 ? ((x1 - x0 + 1) >> 1) * ((y1 - y0 + 1) >> 1) : 0;
}

// Coverage and depth of the pixels of quad (qx, qy) for batch triangle i,
// with the arithmetic of the lockstep loop in raster_body; false (and no
// depths) when the triangle covers none of them.
template <int N>
__device__ __forceinline__ bool batch_quad(const RasterSmem<N>& S, int i, int qx, int qy, bool inside[4], float fz[4]) {
    const int32_t kx = qx - S.minx[i], ky = qy - S.miny[i];
    const int32_t dy12 = S.dy12[i], dx12 = S.dx12[i];
    const int32_t dy23 = S.dy23[i], dx23 = S.dx23[i];
    const int32_t dy31 = S.dy31[i], dx31 = S.dx31[i];
    const int32_t e1 = wadd(wadd(S.c1[i], wmul(kx, dy12)), wmul(ky, dx12));
    const int32_t e2 = wadd(wadd(S.c2[i], wmul(kx, dy23)), wmul(ky, dx23));
    const int32_t e3 = wadd(wadd(S.c3[i], wmul(kx, dy31)), wmul(ky, dx31));
    int32_t l1[4], l2[4], l3[4];
    l1[0] = e1; l1[1] = wadd(e1, dy12); l1[2] = wadd(e1, dx12); l1[3] = wadd(wadd(e1, dx12), dy12);
    l2[0] = e2; l2[1] = wadd(e2, dy23); l2[2] = wadd(e2, dx23); l2[3] = wadd(wadd(e2, dx23), dy23);
    l3[0] = e3; l3[1] = wadd(e3, dy31); l3[2] = wadd(e3, dx31); l3[3] = wadd(wadd(e3, dx31), dy31);
    bool any = false;
#pragma unroll
    for (int l = 0; l < 4; ++l) { inside[l] = (l1[l] | l2[l] | l3[l]) >= 0; any |= inside[l]; }
    if (!any) return false;
    const float scale = S.scale[i];
    const float z0 = S.z[0][i], z1 = S.z[1][i], z2 = S.z[2][i];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const float bx = itof(l2[l]) * scale;
        const float bz = itof(l1[l]) * scale;
        const float by = (1.0f - bx) - bz;
        fz[l] = (bx * z0 + by * z1) + bz * z2;
    }
    return true;
}

// The keys of quad (qx, qy) for batch triangle i, by atomicMin: other lanes
// may update the same pixels.
template <int N>
__device__ __forceinline__ void key_quad(const RasterSmem<N>& S, unsigned long long* keys, int rx0, int ry0, int rw,
                                         int i, int qx, int qy, uint32_t order, bool leq) {
    bool inside[4];
    float fz[4];
    if (!batch_quad(S, i, qx, qy, inside, fz)) return;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        if (!inside[l] || fz[l] != fz[l]) continue;
        unsigned long long* k = keys + (qy - ry0 + (l >> 1)) * rw + (qx - rx0 + (l & 1));
        const unsigned long long key = frag_key(fz[l], order, leq);
        if (key < *k) atomicMin(k, key);
    }
}

// The same for the lane's own quad, whose keys it holds in registers.
template <int N>
__device__ __forceinline__ void key_quad_own(const RasterSmem<N>& S, unsigned long long kq[4], int i, int qx, int qy,
                                             uint32_t order, bool leq) {
    bool inside[4];
    float fz[4];
    if (!batch_quad(S, i, qx, qy, inside, fz)) return;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        if (!inside[l] || fz[l] != fz[l]) continue;
        const unsigned long long key = frag_key(fz[l], order, leq);
        kq[l] = key < kq[l] ? key : kq[l];
    }
}

// The depth the owner of pixel l of quad (qx, qy) gave it (for owners whose
// depth rank is that of zero, whose sign the key does not keep).
__device__ __noinline__ float owner_depth(const FrameView& fv, uint32_t code, const int rect[4], int qx, int qy, int l) {
    TriSetup t;
    float z[3];
    if (code & kClippedBit) {
        const uint32_t e = code & ~kClippedBit;
        const int pbase = fv.clip_poly[e];
        const ClipVert v0 = fv.clip_verts[pbase], v1 = fv.clip_verts[e], v2 = fv.clip_verts[e + 1];
        setup_scalar(t, rect,
                     __float2int_rz(v0.coord[0] * 16.0f), __float2int_rz(v1.coord[0] * 16.0f), __float2int_rz(v2.coord[0] * 16.0f),
                     __float2int_rz(v0.coord[1] * 16.0f), __float2int_rz(v1.coord[1] * 16.0f), __float2int_rz(v2.coord[1] * 16.0f));
        z[0] = v0.coord[2]; z[1] = v1.coord[2]; z[2] = v2.coord[2];
    } else {
        const TriRecord& r = fv.tris[code];
        setup_vector(t, rect, r.fx[0], r.fx[1], r.fx[2], r.fy[0], r.fy[1], r.fy[2]);
        z[0] = r.z[0]; z[1] = r.z[1]; z[2] = r.z[2];
    }
    int32_t e1, e2, e3;
    lane_edges(t, qx, qy, l, e1, e2, e3);
    const float bx = itof(e2) * t.scale;
    const float bz = itof(e1) * t.scale;
    const float by = (1.0f - bx) - bz;
    return (bx * z[0] + by * z[1]) + bz * z[2];
}

// kExt: the frame has float colour stores (rsr's CMD_STORE_COLOR_*_FP) or
// ManyProgram draws; frames without them run the instantiation that has no
// code for them.  kScissor: the instantiation for frames with scissored
// draws (the others keep the draw rectangle, the tile, out of registers).
// kPhase 0: the pass of FrameView::raster_phase (0 whole, 1 or 2 a split
// pass's launch); kPhase 1 / 2: compiled for one launch of a split pass of an
// opaque frame (visibility only, or shading and stores only), whose smaller
// register demand lets more CTAs share an SM.
// slice: with fv.slices > 1 (visibility launches of opaque frames), this
// CTA's share of the block's tile list (see the key merge below).
template <bool kExt, bool kScissor, int kPhase = 0, int N>
__device__ __forceinline__ void raster_body(const FrameView& fv, int block, RasterSmem<N>& S, int slice = 0) {
    if (fv.counters->overflow != 0u) return;

    const int region = fv.region_px;
    const int sub_x = (fv.tile_w + region - 1) / region;
    const int sub_y = (fv.tile_h + region - 1) / region;
    const int subs = sub_x * sub_y;
    const int tile = block / subs;
    const int sub = block % subs;
    const int ttx = tile % fv.tiles_x, tty = tile / fv.tiles_x;
    int rect[4];   // the tile rectangle (GPU::TileRect, rglv_gpu.hxx:292-299)
    rect[0] = ttx * fv.tile_w; rect[1] = tty * fv.tile_h;
    rect[2] = min(rect[0] + fv.tile_w, fv.width); rect[3] = min(rect[1] + fv.tile_h, fv.height);
    const int rx0 = rect[0] + (sub % sub_x) * region, ry0 = rect[1] + (sub / sub_x) * region;
    const int rx1 = min(rx0 + region, rect[2]), ry1 = min(ry0 + region, rect[3]);
    if (rx0 >= rx1 || ry0 >= ry1) return;
    const int qw = (rx1 - rx0) >> 1, qh = (ry1 - ry0) >> 1;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const bool active = tid < qw * qh;
    const int qx = rx0 + 2 * (active ? tid % qw : 0);
    const int qy = ry0 + 2 * (active ? tid / qw : 0);
    // the warp's quad footprint, for whole-warp triangle rejection
    const int wx0 = __reduce_min_sync(FULL_MASK, active ? qx : INT_MAX);
    const int wy0 = __reduce_min_sync(FULL_MASK, active ? qy : INT_MAX);
    const int wx1 = __reduce_max_sync(FULL_MASK, active ? qx : INT_MIN);
    const int wy1 = __reduce_max_sync(FULL_MASK, active ? qy : INT_MIN);

    const TileBin bin = fv.bins[tile];
    float col[4][3], dep[4];
    uint32_t own[4];   // pending last visible fragment of each pixel (visibility mode)
#pragma unroll
    for (int l = 0; l < 4; ++l) { col[l][0] = col[l][1] = col[l][2] = 0.f; dep[l] = 1.f; own[l] = kNoOwner; }
    bool pending = false;
    uint32_t inl_cur = 0, clip_cur = 0;
    int cur_state = 0;
    FragState fs{};   // every frame starts with a state op
    // visibility by keys (see frag_key): decided at the first draw, resolved
    // into own / dep before the first store
    __shared__ unsigned long long keys[4 * N];   // one per pixel of the region (a quad per thread)
    const int rw = rx1 - rx0;
    const bool leq = fv.vis_keys == 2;
    int key_state = 0;   // 0 not decided, 1 keys in use, 2 not used, 3 resolved
    bool phase_pending = true;   // second launch of a split pass: the hand-over is still to take

    // the op list is read by every thread at every step: one load into shared memory
    const bool ops_cached = fv.nops <= kOpCache;
    const bool draws_cached = fv.ndraws <= kOpCache;
    if (S.ops_of != fv.ops) {   // the same for every thread (set below, after a barrier)
        if (ops_cached)
            for (int i = tid; i < fv.nops; i += blockDim.x) S.ops[i] = fv.ops[i];
        if (draws_cached)
            for (int i = tid; i < fv.ndraws; i += blockDim.x) S.dfirst[i] = fv.draws[i].first_tri;
        __syncthreads();
        if (tid == 0) S.ops_of = fv.ops;
    }
    for (int op = 0; op < fv.nops; ++op) {
        const FrameOp o = ops_cached ? S.ops[op] : fv.ops[op];
        if (o.kind == kOpState) {
            cur_state = o.arg;
            load_frag_state(fv, o, fs);
            continue;
        }
        if (kPhase != 2 && key_state == 1 && o.kind != kOpDraw && o.kind != kOpState) {
            // owners and depths from the keys
            __syncthreads();
            if (kPhase == 1 && fv.slices > 1) {
                // The block's slices each swept a part of the list: their keys
                // merge by minimum in slice_keys, and the last slice to merge
                // (counted in slice_done; no CTA waits for another) goes on
                // with the merged keys.  The minimum is that of one sweep.
                __shared__ int last_slice;
                if (active) {
#pragma unroll
                    for (int l = 0; l < 4; ++l) {
                        const int px = qx + (l & 1), py = qy + (l >> 1);
                        atomicMin(fv.slice_keys + size_t(py) * size_t(fv.width) + size_t(px),
                                  keys[(py - ry0) * rw + (px - rx0)]);
                    }
                }
                __threadfence();
                __syncthreads();
                if (tid == 0) last_slice = atomicAdd(fv.slice_done + block, 1u) == uint32_t(fv.slices - 1);
                __syncthreads();
                if (!last_slice) return;
                __threadfence();
                if (active) {
#pragma unroll
                    for (int l = 0; l < 4; ++l) {
                        const int px = qx + (l & 1), py = qy + (l >> 1);
                        keys[(py - ry0) * rw + (px - rx0)] = __ldcg(fv.slice_keys + size_t(py) * size_t(fv.width) + size_t(px));
                    }
                }
            }
            if (active) {
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    const unsigned long long k = keys[(qy - ry0 + (l >> 1)) * rw + (qx - rx0 + (l & 1))];
                    const uint32_t low = uint32_t(k), rank = uint32_t(k >> 32);
                    if (low == (leq ? 0xffffffffu : 0u)) continue;   // no fragment passed
                    const uint32_t order = leq ? 0xfffffffeu - low : low - 1u;
                    const uint32_t pos = order & ((1u << kKeyPosBits) - 1u);
                    const uint32_t code = ((order >> kKeyPosBits) & 1u) ? (fv.bin_pool[bin.clip_off + pos] | kClippedBit)
                                                                        : fv.bin_pool[bin.inl_off + pos];
                    own[l] = code;
                    dep[l] = rank == depth_rank(0.0f) ? owner_depth(fv, code, rect, qx, qy, l) : rank_depth(rank);
                }
            }
            key_state = 3;
        }
        // A pass split in two launches (raster_phase): the first draws, stores
        // depth and hands over the owners and depths at its end; the second
        // replays states and clears, skips the draws and depth stores, takes
        // the owners and depths at the first store and shades.
        if ((kPhase != 0 || fv.raster_phase != 0) && op_is_store(o.kind)) {
            if ((kPhase == 1 || fv.raster_phase == 1) && o.kind != kOpStoreDepth) continue;
            if (kPhase == 2 || fv.raster_phase == 2) {
                if (phase_pending) {
                    if (active) {
#pragma unroll
                        for (int l = 0; l < 4; ++l) {
                            const size_t i = size_t(qy + (l >> 1)) * size_t(fv.width) + size_t(qx + (l & 1));
                            own[l] = fv.vis_own[i];
                            dep[l] = fv.vis_dep[i];
                        }
                    }
                    phase_pending = false;
                }
                if (o.kind == kOpStoreDepth) continue;
            }
        }
        // Without blending the colour of a pixel is that of the last fragment
        // that passed the depth test, so draws without blending only track
        // that fragment's owner and shade it once; anything that reads or
        // replaces colour first resolves the pending pixels.
        const bool visibility = o.kind == kOpDraw && !fs.blend;
        if (kPhase != 1 && !visibility && o.kind != kOpStoreGBuffer && pending && fv.raster_phase != 1) {
            if (active) resolve_quad<kExt, kScissor>(fv, rect, qx, qy, own, col);
            pending = false;
        }
        if (o.kind == kOpClear) {
            const bool packed = o.info[2] != 0;   // RB_COLOR_DEPTH clears both
            if (packed || (o.arg & 1)) {
#pragma unroll
                for (int l = 0; l < 4; ++l) { col[l][0] = o.val[0]; col[l][1] = o.val[1]; col[l][2] = o.val[2]; }
            }
            if (packed || (o.arg & 2)) {
#pragma unroll
                for (int l = 0; l < 4; ++l) dep[l] = o.val[3];
            }
        } else if (o.kind == kOpDraw) {
            int end_tri = o.info[0] + o.info[1];
            int drect[4] = { rect[0], rect[1], rect[2], rect[3] };   // the tile, or its part inside the scissor rectangle
            if (kScissor && fv.any_scissor) draw_rect(fv.states[o.info[2]], rect, drect);
            if (visibility) pending = true;
            if (kPhase == 2 || fv.raster_phase == 2) {   // drawn by the first launch
                // the frame's draws are all opaque: none needs a visit, so
                // jump to the op after the last, in the state it leaves
                if (fv.keys_resume_op > op) {
                    op = fv.keys_resume_op - 1;
                    const FrameOp so = ops_cached ? S.ops[fv.keys_resume_state_op] : fv.ops[fv.keys_resume_state_op];
                    cur_state = so.arg;
                    load_frag_state(fv, so, fs);
                }
                continue;
            }
            if (key_state == 0) {
                bool ok = fv.vis_keys != 0 && bin.inl_cnt < (1u << kKeyPosBits) && bin.clip_cnt < (1u << kKeyPosBits);
                if (active) {
#pragma unroll
                    for (int l = 0; l < 4; ++l) if (dep[l] != dep[l]) ok = false;   // a NaN clear depth: nothing passes
                }
                key_state = __syncthreads_and(ok) ? 1 : 2;
                if (kPhase == 1 && key_state == 2 && slice > 0) return;   // slice 0 walks the whole list
                if (key_state == 1 && active) {
#pragma unroll
                    for (int l = 0; l < 4; ++l) keys[(qy - ry0 + (l >> 1)) * rw + (qx - rx0 + (l & 1))] = clear_key(dep[l], leq);
                }
            } else if (key_state == 1) {
                continue;   // the first draw took the whole list
            }
            // With keys, a fragment's drawing order is part of its key, so the
            // first draw sweeps the tile's whole list -- every draw's
            // triangles, then every draw's fans -- in full batches; each entry
            // carries the order of its own draw.
            const bool sweep = key_state == 1;
            if (sweep) end_tri = INT_MAX;
            // inline triangles of this draw, then its clipped fans (rglv_gpu_impl.hxx:506-508)
            for (int pass = 0; pass < 2; ++pass) {
                const uint32_t base = pass == 0 ? bin.inl_off : bin.clip_off;
                uint32_t cnt = pass == 0 ? bin.inl_cnt : bin.clip_cnt;
                uint32_t& cur = pass == 0 ? inl_cur : clip_cur;
                if (kPhase == 1 && sweep && fv.slices > 1) {   // this slice's share of the list
                    const uint32_t all = cnt;
                    cur = uint32_t((uint64_t(all) * uint32_t(slice)) / uint32_t(fv.slices));
                    cnt = uint32_t((uint64_t(all) * uint32_t(slice + 1)) / uint32_t(fv.slices));
                }
                if (cur >= cnt) continue;   // nothing left in this list (the same for every thread)
                while (true) {
                    __syncthreads();
                    if (tid == 0) S.qsum = 0;
                    bool valid = false;
                    uint32_t e = 0;
                    if (cur + uint32_t(tid) < cnt) {
                        e = fv.bin_pool[base + cur + tid];
                        const int src = pass == 0 ? int(e) : fv.clip_src[fv.clip_poly[e]];
                        valid = src < end_tri;
                        if (sweep) {
                            // Without clipped fans the list position alone orders the
                            // tile's fragments (the list is in drawing order): the
                            // draw field stays zero.
                            int d = 0;
                            if (bin.clip_cnt == 0) {
                            } else if (draws_cached) {   // the last draw starting at or before src
                                int lo = 0, hi = fv.ndraws - 1;
                                while (lo < hi) {
                                    const int mid = (lo + hi + 1) >> 1;
                                    if (S.dfirst[mid] <= src) lo = mid; else hi = mid - 1;
                                }
                                d = lo;
                            } else {
                                d = find_draw(fv.draws, fv.ndraws, src);
                            }
                            S.order[tid] = (uint32_t(d) << (kKeyPosBits + 1)) | (uint32_t(pass) << kKeyPosBits) | (cur + uint32_t(tid));
                        }
                    }
                    const int n = __syncthreads_count(valid);
                    if (n == 0) break;
                    if (valid) {
                        TriSetup t;
                        if (pass == 0) {
                            // the visibility launch reads positions and depths only
                            // (the record's first 36 bytes); w and varyings are for shading
                            const float4* rp = reinterpret_cast<const float4*>(fv.tris + e);
                            TriRecord r;
                            float4* rr = reinterpret_cast<float4*>(&r);
                            constexpr int kParts = kPhase == 1 ? 3 : 6;
#pragma unroll
                            for (int q = 0; q < kParts; ++q) rr[q] = __ldg(rp + q);
                            setup_vector(t, drect, r.fx[0], r.fx[1], r.fx[2], r.fy[0], r.fy[1], r.fy[2]);
#pragma unroll
                            for (int k = 0; k < 3; ++k) {
                                S.z[k][tid] = r.z[k];
                                if (kPhase != 1) {
                                    S.w[k][tid] = r.w[k];
#pragma unroll
                                    for (int q = 0; q < kMaxVary; ++q) S.vary[k][q][tid] = r.vary[k][q];
                                }
                            }
                            S.code[tid] = e;
                        } else {
                            const int pbase = fv.clip_poly[e];
                            const ClipVert v0 = fv.clip_verts[pbase], v1 = fv.clip_verts[e], v2 = fv.clip_verts[e + 1];
                            // DrawClipped: int(dev.x * FP_MUL) (rglv_gpu_impl.hxx:997-998)
                            setup_scalar(t, drect,
                                         __float2int_rz(v0.coord[0] * 16.0f), __float2int_rz(v1.coord[0] * 16.0f), __float2int_rz(v2.coord[0] * 16.0f),
                                         __float2int_rz(v0.coord[1] * 16.0f), __float2int_rz(v1.coord[1] * 16.0f), __float2int_rz(v2.coord[1] * 16.0f));
                            S.z[0][tid] = v0.coord[2]; S.z[1][tid] = v1.coord[2]; S.z[2][tid] = v2.coord[2];
                            if (kPhase != 1) {
                                S.w[0][tid] = v0.coord[3]; S.w[1][tid] = v1.coord[3]; S.w[2][tid] = v2.coord[3];
#pragma unroll
                                for (int q = 0; q < kMaxVary; ++q) {
                                    S.vary[0][q][tid] = v0.vary[q]; S.vary[1][q][tid] = v1.vary[q]; S.vary[2][q][tid] = v2.vary[q];
                                }
                            }
                            S.code[tid] = e | kClippedBit;
                        }
                        put_setup(S, tid, t);
                        if (key_state == 1) atomicAdd(&S.qsum, region_quads(S, tid, rx0, ry0, rx1, ry1));
                    }
                    __syncthreads();
                    if (key_state == 1) {
                        // small triangles: one per lane, over its quads in the region.
                        // Where the batch covers the region many times over, lanes
                        // would contend for the same keys: then only the smallest go
                        // one per lane.
                        const int small_max = S.qsum > kKeyCrowded * qw * qh ? kKeyTinyQuads : kKeySmallQuads;
                        bool big = false;
                        if (tid < n) {
                            const int x0 = max(S.minx[tid], rx0), x1 = min(S.maxx[tid], rx1);
                            const int y0 = max(S.miny[tid], ry0), y1 = min(S.maxy[tid], ry1);
                            const int nq = x0 < x1 && y0 < y1 ? ((x1 - x0 + 1) >> 1) * ((y1 - y0 + 1) >> 1) : 0;
                            big = nq > small_max;
                            if (big) S.zr[tid] = tri_min_rank(S, tid, fv.tile_w, fv.tile_h);
                            if (!big) {
                                for (int qyy = y0; qyy < y1; qyy += 2)
                                    for (int qxx = x0; qxx < x1; qxx += 2)
                                        key_quad(S, keys, rx0, ry0, rw, tid, qxx, qyy, S.order[tid], leq);
                            }
                        }
                        // larger ones: every lane its own quad, a triangle at a time,
                        // with the quad's keys in registers (after the small ones:
                        // each pixel then has one writer)
                        S.big[tid] = big ? 1 : 0;
                        if (!__syncthreads_or(big)) {
                            cur += uint32_t(n);
                            if (n < int(blockDim.x)) break;
                            continue;
                        }
                        unsigned long long kq[4];
                        if (active) {
#pragma unroll
                            for (int l = 0; l < 4; ++l) kq[l] = keys[(qy - ry0 + (l >> 1)) * rw + (qx - rx0 + (l & 1))];
                        }
                        // the warp skips triangles that cannot change any of its keys:
                        // no fragment of theirs goes below the warp's largest depth
                        // rank, or an edge excludes every pixel of its quads
                        uint32_t wmax = warp_max_rank(kq, active);
                        for (int b0 = 0; b0 < n; b0 += 32) {
                            bool hit = false;
                            if (b0 + lane < n && S.big[b0 + lane]) {
                                const int j = b0 + lane;
                                hit = !(S.maxx[j] <= wx0 || S.minx[j] > wx1 || S.maxy[j] <= wy0 || S.miny[j] > wy1) &&
                                      S.zr[j] <= wmax && !footprint_outside(S, j, wx0, wy0, wx1 + 2, wy1 + 2);
                            }
                            uint32_t m = __ballot_sync(FULL_MASK, hit);
                            const bool drawn = m != 0u;
                            while (m) {
                                const int i = b0 + __ffs(m) - 1;
                                m &= m - 1;
                                if (!active || qx < S.minx[i] || qx >= S.maxx[i] || qy < S.miny[i] || qy >= S.maxy[i]) continue;
                                key_quad_own(S, kq, i, qx, qy, S.order[i], leq);
                            }
                            if (drawn) wmax = warp_max_rank(kq, active);
                        }
                        if (active) {
#pragma unroll
                            for (int l = 0; l < 4; ++l) keys[(qy - ry0 + (l >> 1)) * rw + (qx - rx0 + (l & 1))] = kq[l];
                        }
                        cur += uint32_t(n);
                        if (n < int(blockDim.x)) break;
                        continue;
                    }
                    // triangles of the batch in list order; a warp visits only
                    // those whose box meets its quads (ballot over 32 at a time)
                    for (int b0 = 0; b0 < n; b0 += 32) {
                        bool hit = false;
                        if (b0 + lane < n) {
                            const int j = b0 + lane;
                            hit = !(S.maxx[j] <= wx0 || S.minx[j] > wx1 || S.maxy[j] <= wy0 || S.miny[j] > wy1);
                        }
                        uint32_t m = __ballot_sync(FULL_MASK, hit);
                        while (m) {
                            const int i = b0 + __ffs(m) - 1;
                            m &= m - 1;
                            if (!active || qx < S.minx[i] || qx >= S.maxx[i] || qy < S.miny[i] || qy >= S.maxy[i]) continue;
                            const int32_t kx = qx - S.minx[i], ky = qy - S.miny[i];
                            const int32_t dy12 = S.dy12[i], dx12 = S.dx12[i];
                            const int32_t dy23 = S.dy23[i], dx23 = S.dx23[i];
                            const int32_t dy31 = S.dy31[i], dx31 = S.dx31[i];
                            const int32_t e1 = wadd(wadd(S.c1[i], wmul(kx, dy12)), wmul(ky, dx12));
                            const int32_t e2 = wadd(wadd(S.c2[i], wmul(kx, dy23)), wmul(ky, dx23));
                            const int32_t e3 = wadd(wadd(S.c3[i], wmul(kx, dy31)), wmul(ky, dx31));
                            int32_t l1[4], l2[4], l3[4];
                            l1[0] = e1; l1[1] = wadd(e1, dy12); l1[2] = wadd(e1, dx12); l1[3] = wadd(wadd(e1, dx12), dy12);
                            l2[0] = e2; l2[1] = wadd(e2, dy23); l2[2] = wadd(e2, dx23); l2[3] = wadd(wadd(e2, dx23), dy23);
                            l3[0] = e3; l3[1] = wadd(e3, dy31); l3[2] = wadd(e3, dx31); l3[3] = wadd(wadd(e3, dx31), dy31);
                            bool inside[4];
                            bool anyin = false;
#pragma unroll
                            for (int l = 0; l < 4; ++l) {
                                inside[l] = (l1[l] | l2[l] | l3[l]) >= 0;
                                if (kScissor && fs.scissor) {
                                    const int px = qx + (l & 1), py = qy + (l >> 1);
                                    inside[l] = inside[l] && px >= drect[0] && px < drect[2] && py >= drect[1] && py < drect[3];
                                }
                                anyin |= inside[l];
                            }
                            if (!anyin) continue;
                            const float scale = S.scale[i];
                            const float z0 = S.z[0][i], z1 = S.z[1][i], z2 = S.z[2][i];
                            float bx[4], by[4], bz[4], fz[4];
                            bool mask[4];
                            bool any = false;
#pragma unroll
                            for (int l = 0; l < 4; ++l) {
                                bx[l] = itof(l2[l]) * scale;
                                bz[l] = itof(l1[l]) * scale;
                                by[l] = (1.0f - bx[l]) - bz[l];
                                fz[l] = (bx[l] * z0 + by[l] * z1) + bz[l] * z2;
                                const bool pass = fs.depth_test ? depth_pass(fs.depth_func, fz[l], dep[l]) : true;
                                mask[l] = inside[l] && pass;
                                any |= mask[l];
                            }
                            if (!any) continue;
                            if (fs.depth_write) {
#pragma unroll
                                for (int l = 0; l < 4; ++l) if (mask[l]) dep[l] = fz[l];
                            }
                            if (!fs.color_write) continue;
                            if (visibility) {
                                const uint32_t code = S.code[i];
#pragma unroll
                                for (int l = 0; l < 4; ++l) if (mask[l]) own[l] = code;
                                continue;
                            }
                            if (kPhase == 1) continue;   // split passes are of opaque frames: never reached
                            // immediate shading (blending draws)
                            const float w0 = S.w[0][i], w1 = S.w[1][i], w2 = S.w[2][i];
                            float bpx[4], bpy[4], bpz[4];
#pragma unroll
                            for (int l = 0; l < 4; ++l) {
                                const float fragW = oneover(fv.rcp_table, (bx[l] * w0 + by[l] * w1) + bz[l] * w2);
                                bpx[l] = (w0 * bx[l]) * fragW;
                                bpz[l] = (w2 * bz[l]) * fragW;
                                bpy[l] = (1.0f - bpx[l]) - bpz[l];
                            }
                            float frag[4][4];
                            if (fs.program == kProgAmy) {
                                float uu[4], vv[4];
                                const float u0 = S.vary[0][0][i], u1 = S.vary[1][0][i], u2 = S.vary[2][0][i];
                                const float v0 = S.vary[0][1][i], v1 = S.vary[1][1][i], v2 = S.vary[2][1][i];
#pragma unroll
                                for (int l = 0; l < 4; ++l) {
                                    uu[l] = (bpx[l] * u0 + bpy[l] * u1) + bpz[l] * u2;
                                    vv[l] = (bpx[l] * v0 + bpy[l] * v1) + bpz[l] * v2;
                                }
                                tex_sample(fs.tu0, uu, vv, frag);
                            } else {
#pragma unroll
                                for (int q = 0; q < 3; ++q) {
                                    const float a0 = S.vary[0][q][i], a1 = S.vary[1][q][i], a2 = S.vary[2][q][i];
#pragma unroll
                                    for (int l = 0; l < 4; ++l) frag[l][q] = (bpx[l] * a0 + bpy[l] * a1) + bpz[l] * a2;
                                }
#pragma unroll
                                for (int l = 0; l < 4; ++l) frag[l][3] = 1.0f;
                            }
#pragma unroll
                            for (int l = 0; l < 4; ++l) {
                                if (!mask[l]) continue;
                                // BlendAlpha (rglv_gpu_impl.hxx:80-84)
                                const float a = frag[l][3], oma = 1.0f - a;
#pragma unroll
                                for (int c = 0; c < 3; ++c) col[l][c] = frag[l][c] * a + col[l][c] * oma;
                            }
                        }
                    }
                    cur += uint32_t(n);
                    if (n < int(blockDim.x)) break;
                }
            }
            if (sweep && fv.keys_resume_op > op) {
                // the later draws and the states between them have nothing
                // left to do: go on at the op after the last draw
                op = fv.keys_resume_op - 1;
                const FrameOp so = ops_cached ? S.ops[fv.keys_resume_state_op] : fv.ops[fv.keys_resume_state_op];
                cur_state = so.arg;
                load_frag_state(fv, so, fs);
            }
        } else if (o.kind == kOpStoreTC) {
            // GPUBltImpl::StoreTrueColor -> FilterTile (rglr_algorithm.hxx:31-104)
            if (active) {
                const DevState& s = fv.states[cur_state];
                const float ex = s.program == kProgExposurePost ? s.uniforms[0] : 1.0f;
                uint32_t px[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    float c3[3] = { col[l][0], col[l][1], col[l][2] };
                    if (s.program == kProgExposurePost) { c3[0] = c3[0] * ex; c3[1] = c3[1] * ex; c3[2] = c3[2] * ex; }
                    if (o.arg) px[l] = (srgb8(fv.srgb_lut, c3[0]) << 16) | (srgb8(fv.srgb_lut, c3[1]) << 8) | srgb8(fv.srgb_lut, c3[2]);
                    else px[l] = (basic8(c3[0]) << 16) | (basic8(c3[1]) << 8) | basic8(c3[2]);
                }
                uint32_t* dst = static_cast<uint32_t*>(o.ptr);
                *reinterpret_cast<uint2*>(dst + size_t(qy) * o.stride + qx) = make_uint2(px[0], px[1]);
                *reinterpret_cast<uint2*>(dst + size_t(qy + 1) * o.stride + qx) = make_uint2(px[2], px[3]);
            }
        } else if (o.kind == kOpStoreGBuffer) {
            if (active) {
                const GBufferDesc gb = fv.gbufs[o.arg];
                // per lane l: normal x/y/z (fp16 bits) and albedo, packed by
                // constant index (see quad_get)
                uint32_t nxy[4] = { 0u, 0u, 0u, 0u }, nzl[4] = { 0u, 0u, 0u, 0u }, alb[4] = { 0u, 0u, 0u, 0u };
#pragma unroll 1
                for (int l = 0; l < 4; ++l) {
                    const uint32_t ol = quad_get(own, l);
                    if (ol == kNoOwner) continue;
                    TriSetup t;
                    float w[3], vary[3][kMaxVary];
                    int state;
                    owner_setup<kScissor>(fv, ol, rect, t, w, vary, state);
                    if (fv.states[state].program != kProgGBuffer) continue;
                    float bpx, bpy, bpz;
                    lane_bary(fv, t, w, qx, qy, l, bpx, bpy, bpz);
                    const uint32_t hx = __half_as_ushort(__float2half_rn((bpx * vary[0][0] + bpy * vary[1][0]) + bpz * vary[2][0]));
                    const uint32_t hy = __half_as_ushort(__float2half_rn((bpx * vary[0][1] + bpy * vary[1][1]) + bpz * vary[2][1]));
                    const uint32_t hz = __half_as_ushort(__float2half_rn((bpx * vary[0][2] + bpy * vary[1][2]) + bpz * vary[2][2]));
                    const uint32_t al = uint32_t(vary[0][3]) | 0xff000000u;
                    const uint32_t xy = hx | (hy << 16);
                    if (l == 0) { nxy[0] = xy; nzl[0] = hz; alb[0] = al; }
                    else if (l == 1) { nxy[1] = xy; nzl[1] = hz; alb[1] = al; }
                    else if (l == 2) { nxy[2] = xy; nzl[2] = hz; alb[2] = al; }
                    else { nxy[3] = xy; nzl[3] = hz; alb[3] = al; }
                }
                uint16_t nx[4], ny[4], nz[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) { nx[l] = uint16_t(nxy[l] & 0xffffu); ny[l] = uint16_t(nxy[l] >> 16); nz[l] = uint16_t(nzl[l]); }
                const size_t r0 = size_t(qy) * o.stride + qx, r1 = r0 + o.stride;
                *reinterpret_cast<float2*>(gb.depth + r0) = make_float2(dep[0], dep[1]);
                *reinterpret_cast<float2*>(gb.depth + r1) = make_float2(dep[2], dep[3]);
                *reinterpret_cast<uint32_t*>(gb.nx + r0) = uint32_t(nx[0]) | (uint32_t(nx[1]) << 16);
                *reinterpret_cast<uint32_t*>(gb.nx + r1) = uint32_t(nx[2]) | (uint32_t(nx[3]) << 16);
                *reinterpret_cast<uint32_t*>(gb.ny + r0) = uint32_t(ny[0]) | (uint32_t(ny[1]) << 16);
                *reinterpret_cast<uint32_t*>(gb.ny + r1) = uint32_t(ny[2]) | (uint32_t(ny[3]) << 16);
                *reinterpret_cast<uint32_t*>(gb.nz + r0) = uint32_t(nz[0]) | (uint32_t(nz[1]) << 16);
                *reinterpret_cast<uint32_t*>(gb.nz + r1) = uint32_t(nz[2]) | (uint32_t(nz[3]) << 16);
                *reinterpret_cast<uint2*>(gb.albedo + r0) = make_uint2(alb[0], alb[1]);
                *reinterpret_cast<uint2*>(gb.albedo + r1) = make_uint2(alb[2], alb[3]);
            }
        } else if (o.kind == kOpStoreDepth) {
            // Copy(QFloatCanvas -> FloatCanvas) (rglr_algorithm.cxx:227-244)
            if (active) {
                float* dst = static_cast<float*>(o.ptr);
                *reinterpret_cast<float2*>(dst + size_t(qy) * o.stride + qx) = make_float2(dep[0], dep[1]);
                *reinterpret_cast<float2*>(dst + size_t(qy + 1) * o.stride + qx) = make_float2(dep[2], dep[3]);
            }
        } else if (kExt && o.kind >= kOpStoreFP) {
            // rsr's CMD_STORE_COLOR_{FULL_LINEAR,HALF_LINEAR,FULL_QUADS}_FP
            // (rglv_gpu.cxx:345-383); four float4 writes at most
            if (active) {
                float4* base = static_cast<float4*>(o.ptr);
                const size_t qoff = size_t(qy >> 1) * o.stride + (qx >> 1);
                if (o.kind == kOpStoreHalfFP) {
                    // Downsample (rglr_algorithm.cxx:118-168): the quad's four
                    // pixels (r, g, b, 0) summed in lane order, times 0.25
                    base[qoff] = make_float4((((col[0][0] + col[1][0]) + col[2][0]) + col[3][0]) * 0.25f,
                                             (((col[0][1] + col[1][1]) + col[2][1]) + col[3][1]) * 0.25f,
                                             (((col[0][2] + col[1][2]) + col[2][2]) + col[3][2]) * 0.25f, 0.0f);
                } else if (o.kind == kOpStoreFP) {
                    // Copy(QFloat3Canvas|QFloat4Canvas -> FloatingPointCanvas)
                    // (rglr_algorithm.cxx:192-225,247-280): (r, g, b, 0) per pixel
                    float4* p0 = base + size_t(qy) * o.stride + qx;
#pragma unroll
                    for (int l = 0; l < 4; ++l)
                        p0[(l >> 1) * o.stride + (l & 1)] = make_float4(col[l][0], col[l][1], col[l][2], 0.0f);
                } else {
                    // Copy(QFloat3Canvas|QFloat4Canvas -> QFloat4Canvas)
                    // (rglr_algorithm.cxx:320-372): x, y, z the colour lanes, w 1
                    // for RB_RGBF32 and the packed depth for RB_COLOR_DEPTH
                    float4* q = base + qoff * 4;
#pragma unroll
                    for (int c = 0; c < 3; ++c) q[c] = make_float4(col[0][c], col[1][c], col[2][c], col[3][c]);
                    const bool packed = fv.states[cur_state].color_type == 0;
                    q[3] = packed ? make_float4(dep[0], dep[1], dep[2], dep[3]) : make_float4(1.0f, 1.0f, 1.0f, 1.0f);
                }
            }
        }
    }
    if ((kPhase == 1 || fv.raster_phase == 1) && active) {   // the hand-over to the second launch
        const bool pairs = (fv.width & 1) == 0 && ((reinterpret_cast<uintptr_t>(fv.vis_own) |
                                                    reinterpret_cast<uintptr_t>(fv.vis_dep)) & 7u) == 0;
        if (pairs) {   // the quad's rows as 8-byte stores
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const size_t i = size_t(qy + r) * size_t(fv.width) + size_t(qx);
                *reinterpret_cast<uint2*>(fv.vis_own + i) = make_uint2(own[2 * r], own[2 * r + 1]);
                *reinterpret_cast<float2*>(fv.vis_dep + i) = make_float2(dep[2 * r], dep[2 * r + 1]);
            }
        } else {
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const size_t i = size_t(qy + (l >> 1)) * size_t(fv.width) + size_t(qx + (l & 1));
                fv.vis_own[i] = own[l];
                fv.vis_dep[i] = dep[l];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// kernels: one frame, and a batch of frames in one launch per stage
// ---------------------------------------------------------------------------
// A frame starts from zeroed counters and empty super-chunk rectangles
// (0x7f7f7f7f: setup's atomicMin lands below), and, where the visibility
// launch slices tile lists, merged keys above every key and no slice merged;
// one small launch writes them and lets setup launch at once (setup waits
// for it before its first access).
__global__ void __launch_bounds__(256) frame_init_kernel(const __grid_constant__ FrameView fv, int nblocks) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    static_assert(sizeof(FrameCounters) % 4 == 0, "counters as words");
    constexpr int kWords = int(sizeof(FrameCounters) / 4);
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x, step = size_t(gridDim.x) * blockDim.x;
    if (i < size_t(kWords)) reinterpret_cast<uint32_t*>(fv.counters)[i] = 0u;
    for (size_t k = i; k < size_t(fv.nsupers); k += step)
        fv.super_rect[k] = make_int4(0x7f7f7f7f, 0x7f7f7f7f, 0x7f7f7f7f, 0x7f7f7f7f);
    if (fv.slices > 1) {
        const size_t nkeys = size_t(fv.width) * size_t(fv.height);
        for (size_t k = i; k < nkeys; k += step) fv.slice_keys[k] = ~0ull;
        for (size_t k = i; k < size_t(nblocks); k += step) fv.slice_done[k] = 0u;
    }
}
// The binning launch is programmatically dependent on setup (launched while
// setup's CTAs drain; it waits for their results before it reads them), and
// setup on frame_init_kernel where that runs (without a prerequisite launch
// the wait returns at once).
__global__ void __launch_bounds__(kSetupBlock, 5) setup_kernel(const __grid_constant__ FrameView fv) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    setup_body<false>(fv, blockIdx.x);
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__global__ void __launch_bounds__(kSetupBlock) setup_ext_kernel(const __grid_constant__ FrameView fv) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    setup_body<true>(fv, blockIdx.x);
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__global__ void __launch_bounds__(kBinBlock, 6) bin_kernel(const __grid_constant__ FrameView fv) {
    __shared__ BinShared S;
    asm volatile("griddepcontrol.wait;" ::: "memory");
    bin_body(fv, blockIdx.x, S);
}
// The frame's counters, final once setup and binning are done, go to the
// caller-visible pinned copy from the raster pass (no copy after the frame).
__device__ __forceinline__ void publish_counters(const FrameView& fv) {
    if (fv.host_counters != nullptr && blockIdx.x == 0 && threadIdx.x == 0) *fv.host_counters = *fv.counters;
}
// A frame's work queue, read by thread 0 of a raster CTA: bucket_end[b] is
// the number of entries in the buckets from the heaviest down to b, and the
// k-th item is the k-th entry in that order (-1 past the filed entries: a
// tile that was never filed draws nothing).
__device__ __forceinline__ void load_bucket_ends(const FrameView& fv, int* bucket_end) {
    int sum = 0;
    for (int b = kCostBuckets - 1; b >= 0; --b) bucket_end[b] = (sum += int(fv.counters->bucket[b]));
}
__device__ __forceinline__ int queue_entry(const FrameView& fv, const int* bucket_end, int k) {
    int b = kCostBuckets - 1;
    while (b > 0 && k >= bucket_end[b]) --b;
    if (k >= bucket_end[b]) return -1;
    const int first = b == kCostBuckets - 1 ? 0 : bucket_end[b + 1];
    return int(fv.tile_queue[size_t(b) * size_t(fv.queue_cap) + size_t(k - first)]);
}
// The raster blocks of a frame: a persistent grid takes them from the work
// queue, heaviest tiles first, until it is empty; without a queue, CTA b
// draws block b.
template <bool kExt, bool kScissor, int kPhase = 0, int N>
__device__ __forceinline__ void raster_items(const FrameView& fv, RasterSmem<N>& S) {
    if (threadIdx.x == 0) S.ops_of = nullptr;   // no frame's ops loaded yet
    __syncthreads();
    if (fv.tile_queue == nullptr) {
        const int sl = kPhase == 1 ? fv.slices : 1;
        raster_body<kExt, kScissor, kPhase>(fv, int(blockIdx.x) / sl, S, int(blockIdx.x) % sl);
        return;
    }
    __shared__ int item;
    __shared__ int bucket_end[kCostBuckets];
    if (threadIdx.x == 0) load_bucket_ends(fv, bucket_end);
    while (true) {
        __syncthreads();   // the previous item is done with the shared state
        if (threadIdx.x == 0) {
            const int i = int(atomicAdd(&fv.taken->next_item, 1u));
            item = i < int(fv.queue_cap) ? queue_entry(fv, bucket_end, i) : -2;   // -2: empty
        }
        __syncthreads();
        const int e = item;
        if (e == -2) return;
        const int sl = kPhase == 1 ? fv.slices : 1;
        if (e >= 0) raster_body<kExt, kScissor, kPhase>(fv, e / sl, S, e % sl);
    }
}
// Raster kernels are compiled for CTAs of N threads (one 2x2 quad each): 256
// for 32 px regions, 64 for 16 and 8 px regions, with shared memory for
// batches of N triangles, so that small CTAs are not held to the large ones'
// shared-memory share of an SM.  kRasterCtas: CTAs per SM the launch bounds
// allow (registers).
template <int N> constexpr int raster_ctas(int per256) { return N == 256 ? per256 : per256 * 4; }

// The split pass of an opaque frame without float stores, ManyProgram draws or
// scissor: visibility (80 registers), then shading.
// The shading launch is programmatically dependent on this one: it is
// scheduled as these CTAs finish their last items and waits for the whole
// grid's results.
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(3)) raster_vis_kernel(const __grid_constant__ FrameView fv) {
    __shared__ RasterSmem<N> S;
    raster_items<false, false, 1>(fv, S);
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_shade_kernel(const __grid_constant__ FrameView fv) {
    __shared__ RasterSmem<N> S;
    publish_counters(fv);
    raster_items<false, false, 2>(fv, S);
}
// The shading launch of a split pass, one thread per pixel, for an opaque
// frame whose ops after its last draw are state changes and TrueColor and
// depth stores (no float stores, ManyProgram draws or scissor): the pixel's
// colour is the clear colour or its owner's (as resolve_quad shades it), then
// the stores run in op order.  32x8 pixels per CTA: a warp stores 128
// contiguous bytes of a row (outputs may be mapped host memory).
constexpr int kPixelW = 32, kPixelH = 8;
// What every pixel of a CTA reads: the clear colour (the last colour clear
// before the first draw) and, for frames of up to kOpCache draws, the draws'
// first triangles and states.
struct PixelShared {
    float clear[3];
    int first[kOpCache];
    int state[kOpCache];
};
__device__ __forceinline__ void pixel_shared_load(const FrameView& fv, PixelShared& P) {
    if (fv.ndraws <= kOpCache)
        for (int i = threadIdx.x; i < fv.ndraws; i += blockDim.x) { P.first[i] = fv.draws[i].first_tri; P.state[i] = fv.draws[i].state; }
    if (threadIdx.x == 0) {
        float c[3] = { 0.0f, 0.0f, 0.0f };
        for (int op = 0; op < fv.nops; ++op) {
            const FrameOp o = fv.ops[op];
            if (o.kind == kOpDraw) break;
            if (o.kind == kOpClear && (o.info[2] != 0 || (o.arg & 1))) { c[0] = o.val[0]; c[1] = o.val[1]; c[2] = o.val[2]; }
        }
        P.clear[0] = c[0]; P.clear[1] = c[1]; P.clear[2] = c[2];
    }
    __syncthreads();
}
__device__ __forceinline__ void shade_pixel(const FrameView& fv, int x, int y, const PixelShared& P) {
    if (fv.counters->overflow != 0u) return;
    if (x >= (fv.width & ~1) || y >= (fv.height & ~1)) return;   // the pixels of whole quads, as the raster pass
    const size_t i = size_t(y) * size_t(fv.width) + size_t(x);
    const uint32_t own = fv.vis_own[i];
    const float dep = fv.vis_dep[i];
    // the colour: the clear colour, or the owner's
    float c[3] = { P.clear[0], P.clear[1], P.clear[2] };
    if (own != kNoOwner) {
        const int tx = div_tile(x, fv.tile_w), ty = div_tile(y, fv.tile_h);
        const int rect[4] = { tx * fv.tile_w, ty * fv.tile_h, min(tx * fv.tile_w + fv.tile_w, fv.width),
                              min(ty * fv.tile_h + fv.tile_h, fv.height) };
        TriSetup t;
        float w[3], vary[3][kMaxVary];
        int state = 0;
        const bool cached = fv.ndraws <= kOpCache;
        owner_setup_inline<false>(fv, own, rect, t, w, vary, state, cached ? P.first : nullptr, cached ? P.state : nullptr);
        owner_color<false>(fv, t, w, vary, state, x & ~1, y & ~1, (x & 1) | ((y & 1) << 1), c);
    }
    int cur_state = fv.ops[fv.keys_resume_state_op].arg;
    for (int op = fv.keys_resume_op; op < fv.nops; ++op) {
        const FrameOp o = fv.ops[op];
        if (o.kind == kOpState) {
            cur_state = o.arg;
        } else if (o.kind == kOpStoreTC) {
            // GPUBltImpl::StoreTrueColor -> FilterTile (rglr_algorithm.hxx:31-104), as raster_body
            const DevState& s = fv.states[cur_state];
            float c3[3] = { c[0], c[1], c[2] };
            if (s.program == kProgExposurePost) {
                const float ex = s.uniforms[0];
                c3[0] = c3[0] * ex; c3[1] = c3[1] * ex; c3[2] = c3[2] * ex;
            }
            const uint32_t px = o.arg ? (srgb8(fv.srgb_lut, c3[0]) << 16) | (srgb8(fv.srgb_lut, c3[1]) << 8) | srgb8(fv.srgb_lut, c3[2])
                                      : (basic8(c3[0]) << 16) | (basic8(c3[1]) << 8) | basic8(c3[2]);
            static_cast<uint32_t*>(o.ptr)[size_t(y) * o.stride + x] = px;
        } else if (o.kind == kOpStoreDepth) {
            static_cast<float*>(o.ptr)[size_t(y) * o.stride + x] = dep;
        }
    }
}
// A persistent grid: each CTA reads the draw table once and takes pixel
// blocks (32x8) in grid-stride order.
__global__ void __launch_bounds__(kPixelW * kPixelH) shade_pixels_kernel(const __grid_constant__ FrameView fv) {
    __shared__ PixelShared P;
    asm volatile("griddepcontrol.wait;" ::: "memory");   // the visibility launch's owners and depths
    publish_counters(fv);
    pixel_shared_load(fv, P);
    const int bx = (fv.width + kPixelW - 1) / kPixelW;
    const int nblocks = bx * ((fv.height + kPixelH - 1) / kPixelH);
    // block b = by * bx + bxi, stepped by the grid size without a division
    // per block
    const int step = int(gridDim.x), step_x = step % bx, step_y = step / bx;
    int bxi = int(blockIdx.x) % bx, by = int(blockIdx.x) / bx;
    const int px = threadIdx.x % kPixelW, py = threadIdx.x / kPixelW;
    for (int b = blockIdx.x; b < nblocks; b += step) {
        shade_pixel(fv, bxi * kPixelW + px, by * kPixelH + py, P);
        bxi += step_x;
        by += step_y;
        if (bxi >= bx) { bxi -= bx; ++by; }
    }
}
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_kernel(const __grid_constant__ FrameView fv) {
    __shared__ RasterSmem<N> S;
    publish_counters(fv);
    raster_items<false, false>(fv, S);
}
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_scissor_kernel(const __grid_constant__ FrameView fv) {
    __shared__ RasterSmem<N> S;
    publish_counters(fv);
    raster_items<false, true>(fv, S);
}
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_ext_kernel(const __grid_constant__ FrameView fv) {
    __shared__ RasterSmem<N> S;
    publish_counters(fv);
    raster_items<true, true>(fv, S);
}

// frame of a block: the last f with start[f] <= block (start[] ascending)
__device__ __forceinline__ int batch_frame(const BatchLaunch& b, int block) {
    int lo = 0, hi = b.nframes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b.start[mid] <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__global__ void __launch_bounds__(kSetupBlock) setup_batch_kernel(const __grid_constant__ BatchLaunch b) {
    const int f = batch_frame(b, blockIdx.x);
    setup_body<false>(b.fv[f], blockIdx.x - b.start[f]);
}
// batches with a frame of instanced or OBJ1Program draws: the extended setup
// for those frames, the plain one for the others
__global__ void __launch_bounds__(kSetupBlock) setup_batch_ext_kernel(const __grid_constant__ BatchLaunch b) {
    const int f = batch_frame(b, blockIdx.x);
    if (b.fv[f].dext != nullptr) setup_body<true>(b.fv[f], blockIdx.x - b.start[f]);
    else setup_body<false>(b.fv[f], blockIdx.x - b.start[f]);
}
__global__ void __launch_bounds__(kBinBlock) bin_batch_kernel(const __grid_constant__ BatchLaunch b) {
    __shared__ BinShared S;
    const int f = batch_frame(b, blockIdx.x);
    bin_body(b.fv[f], blockIdx.x - b.start[f], S);
}
// The raster blocks of a batch launch's frames: a persistent grid takes the
// launch's items from one counter, frame after frame in launch order (a
// frame's triangle records and tile lists stay in L2 while its tiles are
// drawn), each frame's tiles heaviest first; without queues, CTA b draws
// block b.
template <bool kExt, bool kScissor, int kPhase = 0, int N>
__device__ __forceinline__ void raster_batch_items(const BatchLaunch& b, RasterSmem<N>& S) {
    if (threadIdx.x == 0) S.ops_of = nullptr;   // no frame's ops loaded yet
    __syncthreads();
    if (b.fv[0].tile_queue == nullptr) {
        const int f = batch_frame(b, blockIdx.x);
        raster_body<kExt, kScissor, kPhase>(b.fv[f], blockIdx.x - b.start[f], S);
        return;
    }
    __shared__ int item, item_frame, cached_frame;
    __shared__ int bucket_end[kCostBuckets];   // of cached_frame
    if (threadIdx.x == 0) cached_frame = -1;
    while (true) {
        __syncthreads();   // the previous item is done with the shared state
        if (threadIdx.x == 0) {
            const int i = int(atomicAdd(&b.fv[0].taken->next_item, 1u));
            int e = -2, f = 0;   // -2: empty
            if (i < b.start[b.nframes]) {
                f = batch_frame(b, i);
                if (f != cached_frame) {
                    load_bucket_ends(b.fv[f], bucket_end);
                    cached_frame = f;
                }
                e = queue_entry(b.fv[f], bucket_end, i - b.start[f]);
            }
            item = e;
            item_frame = f;
        }
        __syncthreads();
        const int e = item;
        if (e == -2) return;
        if (e >= 0) raster_body<kExt, kScissor, kPhase>(b.fv[item_frame], e, S);
    }
}
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_batch_kernel(const __grid_constant__ BatchLaunch b) {
    __shared__ RasterSmem<N> S;
    raster_batch_items<false, false>(b, S);
}
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_batch_scissor_kernel(const __grid_constant__ BatchLaunch b) {
    __shared__ RasterSmem<N> S;
    raster_batch_items<false, true>(b, S);
}
// The split pass of a batch of opaque frames (as raster_vis_kernel and
// shade_pixels_kernel): visibility per CTA shape, then one launch shading
// every frame's pixels (block b of frame f: start[f] <= b < start[f + 1], in
// rows of ceil(width / kPixelW) blocks).
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(3)) raster_batch_vis_kernel(const __grid_constant__ BatchLaunch b) {
    __shared__ RasterSmem<N> S;
    raster_batch_items<false, false, 1>(b, S);
}
__global__ void __launch_bounds__(kPixelW * kPixelH) shade_pixels_batch_kernel(const __grid_constant__ BatchLaunch b) {
    __shared__ PixelShared P;
    __shared__ int blk[2];   // the block's column and row in its frame (divided once per CTA)
    const int f = batch_frame(b, blockIdx.x);
    const FrameView& fv = b.fv[f];
    if (threadIdx.x == 0) {
        const int k = blockIdx.x - b.start[f], bx = (fv.width + kPixelW - 1) / kPixelW;
        blk[0] = k % bx;
        blk[1] = k / bx;
    }
    pixel_shared_load(fv, P);   // ends with a barrier
    shade_pixel(fv, blk[0] * kPixelW + (threadIdx.x % kPixelW), blk[1] * kPixelH + (threadIdx.x / kPixelW), P);
}
// launches with a frame of float colour stores or ManyProgram draws (the
// code of raster_ext_kernel, which renders the other frames alike)
template <int N>
__global__ void __launch_bounds__(N, raster_ctas<N>(2)) raster_batch_ext_kernel(const __grid_constant__ BatchLaunch b) {
    __shared__ RasterSmem<N> S;
    raster_batch_items<true, true>(b, S);
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
int raster_blocks(const FrameView& fv);

cudaError_t launch_frame_init(const FrameView& fv, cudaStream_t st) {
    const int nblocks = raster_blocks(fv);
    size_t n = sizeof(FrameCounters) / 4;
    if (size_t(fv.nsupers) > n) n = size_t(fv.nsupers);
    if (fv.slices > 1 && size_t(fv.width) * size_t(fv.height) / 4 > n) n = size_t(fv.width) * size_t(fv.height) / 4;
    const size_t blocks = (n + 255) / 256 < 152 ? (n + 255) / 256 : 152;
    frame_init_kernel<<<unsigned(blocks), 256, 0, st>>>(fv, nblocks);
    return cudaGetLastError();
}

// after_init: launched programmatically dependent on frame_init_kernel, the
// launch just before it on st
cudaError_t launch_setup(const FrameView& fv, cudaStream_t st, bool after_init) {
    const int blocks = (fv.ntris + kSetupBlock - 1) / kSetupBlock;
    if (blocks == 0) return cudaSuccess;
    if (!after_init) {
        if (fv.dext != nullptr) setup_ext_kernel<<<blocks, kSetupBlock, 0, st>>>(fv);
        else setup_kernel<<<blocks, kSetupBlock, 0, st>>>(fv);
        return cudaGetLastError();
    }
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(blocks));
    cfg.blockDim = dim3(kSetupBlock);
    cfg.stream = st;
    cfg.attrs = pdl;
    cfg.numAttrs = 1;
    if (fv.dext != nullptr) return cudaLaunchKernelEx(&cfg, setup_ext_kernel, fv);
    return cudaLaunchKernelEx(&cfg, setup_kernel, fv);
}

int setup_blocks(const FrameView& fv) { return (fv.ntris + kSetupBlock - 1) / kSetupBlock; }
int bin_blocks(const FrameView& fv) { return fv.ntiles; }
// One CTA row per range: 16-byte loads and stores where both ends are aligned, bytes otherwise.
__global__ void __launch_bounds__(256) gather_kernel(const __grid_constant__ GatherList g) {
    const int r = blockIdx.y;
    const uint8_t* __restrict__ src = g.src[r];
    uint8_t* __restrict__ dst = g.dst[r];
    const size_t n = g.bytes[r];
    const size_t first = size_t(blockIdx.x) * blockDim.x + threadIdx.x, step = size_t(gridDim.x) * blockDim.x;
    // Reads from host memory have a long latency: each thread keeps four
    // 16-byte loads in flight before it stores them.
    if (g.rows[r] > 1) {   // a block of rows (16-byte units; checked by the host)
        const uint32_t per = uint32_t(n / 16), pitch16 = g.pitch[r] / 16;
        const size_t total = size_t(per) * g.rows[r];
        for (size_t i0 = first; i0 < total; i0 += 4 * step) {
            uint4 v[4];
            size_t at[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const size_t i = i0 + size_t(k) * step;
                at[k] = ~size_t(0);
                if (i < total) {
                    const size_t row = i / per;
                    at[k] = row * pitch16 + (i - row * per);
                    v[k] = reinterpret_cast<const uint4*>(src)[at[k]];
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (at[k] != ~size_t(0)) reinterpret_cast<uint4*>(dst)[at[k]] = v[k];
        }
        return;
    }
    size_t done = 0;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
        const size_t n16 = n / 16;
        for (size_t i0 = first; i0 < n16; i0 += 4 * step) {
            uint4 v[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (i0 + size_t(k) * step < n16) v[k] = reinterpret_cast<const uint4*>(src)[i0 + size_t(k) * step];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (i0 + size_t(k) * step < n16) reinterpret_cast<uint4*>(dst)[i0 + size_t(k) * step] = v[k];
        }
        done = n16 * 16;
    }
    for (size_t i = done + first; i < n; i += step) dst[i] = src[i];
}

cudaError_t launch_gather(const GatherList& g, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    gather_kernel<<<dim3(128, unsigned(g.n)), 256, 0, st>>>(g);
    return cudaGetLastError();
}

int raster_blocks(const FrameView& fv) {
    const int sub_x = (fv.tile_w + fv.region_px - 1) / fv.region_px;
    const int sub_y = (fv.tile_h + fv.region_px - 1) / fv.region_px;
    return fv.ntiles * sub_x * sub_y;
}
// threads of a raster CTA: one per 2x2 quad of a region, in whole warps
int raster_threads(const FrameView& fv) {
    const int qx = (fv.tile_w < fv.region_px ? fv.tile_w : fv.region_px) / 2;
    const int qy = (fv.tile_h < fv.region_px ? fv.tile_h : fv.region_px) / 2;
    return ((qx * qy + 31) / 32) * 32;
}

cudaError_t launch_bin(const FrameView& fv, cudaStream_t st) {
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(bin_blocks(fv));
    cfg.blockDim = dim3(kBinBlock);
    cfg.stream = st;
    cfg.attrs = pdl;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, bin_kernel, fv);
}

// a persistent grid for a work queue: every CTA slot of the GPU, at most one per block
static int persistent_blocks(const void* kernel, int threads, int blocks) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    const int slots = sms * (per > 0 ? per : 1);
    return blocks < slots ? blocks : slots;
}

template <int N>
static cudaError_t launch_raster_n(const FrameView& fv, cudaStream_t st, int phase) {
    int blocks = raster_blocks(fv) * (phase == 1 ? fv.slices : 1);
    const int threads = raster_threads(fv);
    const void* k = phase == 1 ? reinterpret_cast<const void*>(raster_vis_kernel<N>)
                  : phase == 2 ? reinterpret_cast<const void*>(raster_shade_kernel<N>)
                  : fv.ext ? reinterpret_cast<const void*>(raster_ext_kernel<N>)
                  : fv.any_scissor ? reinterpret_cast<const void*>(raster_scissor_kernel<N>)
                                   : reinterpret_cast<const void*>(raster_kernel<N>);
    if (fv.tile_queue != nullptr) blocks = persistent_blocks(k, threads, blocks);
    if (phase == 1) raster_vis_kernel<N><<<blocks, threads, 0, st>>>(fv);
    else if (phase == 2) raster_shade_kernel<N><<<blocks, threads, 0, st>>>(fv);
    else if (fv.ext) raster_ext_kernel<N><<<blocks, threads, 0, st>>>(fv);
    else if (fv.any_scissor) raster_scissor_kernel<N><<<blocks, threads, 0, st>>>(fv);
    else raster_kernel<N><<<blocks, threads, 0, st>>>(fv);
    return cudaGetLastError();
}
// CTAs of the visibility kernel the GPU holds at once for this frame's CTA size
int vis_slots(const FrameView& fv) {
    const int threads = raster_threads(fv);
    const void* k = threads <= 64 ? reinterpret_cast<const void*>(raster_vis_kernel<64>)
                                  : reinterpret_cast<const void*>(raster_vis_kernel<kRasterBatch>);
    return persistent_blocks(k, threads, 1 << 30);
}
// phase 1 / 2: the launches of a split pass compiled for it (a frame with
// vis_keys and neither ext nor any_scissor); 3: its shading launch per pixel
// (shade_pixels_kernel), 4: the same launched programmatically dependent on
// the visibility launch just before it; 0: raster_phase decides.  CTAs of up to 64 threads
// (16 and 8 px regions) run the 64-thread instantiation.
cudaError_t launch_raster(const FrameView& fv, cudaStream_t st, int phase) {
    if (phase == 3 || phase == 4) {   // 4: launched programmatically dependent on the visibility launch
        cudaLaunchAttribute pdl[1];
        pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        pdl[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg = {};
        const int nblocks = ((fv.width + kPixelW - 1) / kPixelW) * ((fv.height + kPixelH - 1) / kPixelH);
        cfg.gridDim = dim3(unsigned(persistent_blocks(reinterpret_cast<const void*>(shade_pixels_kernel),
                                                      kPixelW * kPixelH, nblocks)));
        cfg.blockDim = dim3(kPixelW * kPixelH);
        cfg.stream = st;
        cfg.attrs = pdl;
        cfg.numAttrs = phase == 4 ? 1 : 0;
        return cudaLaunchKernelEx(&cfg, shade_pixels_kernel, fv);
    }
    return raster_threads(fv) <= 64 ? launch_raster_n<64>(fv, st, phase) : launch_raster_n<kRasterBatch>(fv, st, phase);
}

cudaError_t launch_setup_batch(const BatchLaunch& b, int blocks, cudaStream_t st) {
    if (blocks == 0) return cudaSuccess;
    bool ext = false;
    for (int f = 0; f < b.nframes; ++f) ext = ext || b.fv[f].dext != nullptr;
    if (ext) setup_batch_ext_kernel<<<blocks, kSetupBlock, 0, st>>>(b);
    else setup_batch_kernel<<<blocks, kSetupBlock, 0, st>>>(b);
    return cudaGetLastError();
}
cudaError_t launch_bin_batch(const BatchLaunch& b, int blocks, cudaStream_t st) {
    if (blocks == 0) return cudaSuccess;
    bin_batch_kernel<<<blocks, kBinBlock, 0, st>>>(b);
    return cudaGetLastError();
}
template <int N>
static cudaError_t launch_raster_batch_n(const BatchLaunch& b, int blocks, int threads, cudaStream_t st, bool vis) {
    if (vis) {
        if (b.fv[0].tile_queue != nullptr)
            blocks = persistent_blocks(reinterpret_cast<const void*>(raster_batch_vis_kernel<N>), threads, blocks);
        raster_batch_vis_kernel<N><<<blocks, threads, 0, st>>>(b);
        return cudaGetLastError();
    }
    bool scissor = false, ext = false;
    for (int f = 0; f < b.nframes; ++f) {
        scissor = scissor || b.fv[f].any_scissor;
        ext = ext || b.fv[f].ext;
    }
    const void* k = ext ? reinterpret_cast<const void*>(raster_batch_ext_kernel<N>)
                  : scissor ? reinterpret_cast<const void*>(raster_batch_scissor_kernel<N>)
                            : reinterpret_cast<const void*>(raster_batch_kernel<N>);
    if (b.fv[0].tile_queue != nullptr) blocks = persistent_blocks(k, threads, blocks);
    if (ext) raster_batch_ext_kernel<N><<<blocks, threads, 0, st>>>(b);
    else if (scissor) raster_batch_scissor_kernel<N><<<blocks, threads, 0, st>>>(b);
    else raster_batch_kernel<N><<<blocks, threads, 0, st>>>(b);
    return cudaGetLastError();
}
// vis: the visibility launch of a split pass (every frame of the launch is
// opaque, without float stores, ManyProgram draws or scissor)
cudaError_t launch_raster_batch(const BatchLaunch& b, int blocks, int threads, cudaStream_t st, bool vis) {
    if (blocks == 0) return cudaSuccess;
    return threads <= 64 ? launch_raster_batch_n<64>(b, blocks, threads, st, vis)
                         : launch_raster_batch_n<kRasterBatch>(b, blocks, threads, st, vis);
}
// the shading launch of a batch's split pass: start[] counts pixel blocks
int pixel_blocks(const FrameView& fv) {
    return ((fv.width + kPixelW - 1) / kPixelW) * ((fv.height + kPixelH - 1) / kPixelH);
}
cudaError_t launch_shade_pixels_batch(const BatchLaunch& b, int blocks, cudaStream_t st) {
    if (blocks == 0) return cudaSuccess;
    shade_pixels_batch_kernel<<<blocks, kPixelW * kPixelH, 0, st>>>(b);
    return cudaGetLastError();
}

}  // namespace rsrgpu
