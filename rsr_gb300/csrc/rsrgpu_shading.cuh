// rsrgpu_shading.cuh -- per-pixel deferred shading math shared by the plain
// multi-light shader, the learned shader's feature builder and its per-tile
// fallback.  rsr has no deferred or multi-light path; these functions are
// this library's definition, restated on the CPU in oracle/rsr_oracle.c.
// Every file including this header is built with -fmad=false, so each
// expression rounds once per operation in the written order and the GPU
// matches the CPU restatement bit for bit.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>

#include "../../include/rsrgpu.h"

namespace rsrgpu {

constexpr int kMaxLights = 256;
constexpr int kShadeTile = 32;     // learned shader: light-candidate and gate tile (pixels)
constexpr int kCandidates = 8;     // candidate lights per shading tile
constexpr int kFeatures = 24;      // learned-shader input features per pixel

struct PlainParams {
    const float* depth;
    const uint16_t* nx;
    const uint16_t* ny;
    const uint16_t* nz;
    const uint32_t* albedo;
    int width, height;
    float ivp[16];
    float eye[3];
    float background[3];
    const rsrgpu_light* lights;
    int nlights;
    uint32_t* out_srgb;
    float* out_linear;
    const uint8_t* srgb_lut;
};

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return (ax * bx + ay * by) + az * bz;
}
__device__ __forceinline__ float pos0(float x) { return x > 0.0f ? x : 0.0f; }
__device__ __forceinline__ uint32_t srgb8_lut(const uint8_t* __restrict__ lut, float v) {
    const float lo = __uint_as_float((127u - 13u) << 23), hi = __uint_as_float(0x3f7fffffu);
    float c = v > lo ? v : lo;
    c = c < hi ? c : hi;
    return __ldg(lut + ((__float_as_uint(c) >> 12) - ((127u - 13u) << 11)));
}
__device__ __forceinline__ uint32_t pack_srgb(const uint8_t* lut, const float rgb[3]) {
    return (srgb8_lut(lut, rgb[0]) << 16) | (srgb8_lut(lut, rgb[1]) << 8) | srgb8_lut(lut, rgb[2]);
}

// pixel centre -> NDC -> world through the column-major inverse view-projection
__device__ __forceinline__ void world_pos(const PlainParams& p, int x, int y, float z, float P[3]) {
    const float ndcx = (2.0f * (float(x) + 0.5f)) / float(p.width) - 1.0f;
    const float ndcy = 1.0f - (2.0f * (float(y) + 0.5f)) / float(p.height);
    const float* m = p.ivp;
    const float cx = ((m[0] * ndcx + m[4] * ndcy) + m[8] * z) + m[12];
    const float cy = ((m[1] * ndcx + m[5] * ndcy) + m[9] * z) + m[13];
    const float cz = ((m[2] * ndcx + m[6] * ndcy) + m[10] * z) + m[14];
    const float cw = ((m[3] * ndcx + m[7] * ndcy) + m[11] * z) + m[15];
    P[0] = cx / cw; P[1] = cy / cw; P[2] = cz / cw;
}

// unit normal from the fp16 planes, unit view vector and its length
__device__ __forceinline__ void surface(const PlainParams& p, const float P[3], uint16_t hx, uint16_t hy, uint16_t hz,
                                        float n[3], float v[3], float& vlen) {
    n[0] = __half2float(__ushort_as_half(hx)); n[1] = __half2float(__ushort_as_half(hy)); n[2] = __half2float(__ushort_as_half(hz));
    const float nlen = sqrtf(dot3(n[0], n[1], n[2], n[0], n[1], n[2]));
    n[0] = n[0] / nlen; n[1] = n[1] / nlen; n[2] = n[2] / nlen;
    v[0] = p.eye[0] - P[0]; v[1] = p.eye[1] - P[1]; v[2] = p.eye[2] - P[2];
    vlen = sqrtf(dot3(v[0], v[1], v[2], v[0], v[1], v[2]));
    v[0] = v[0] / vlen; v[1] = v[1] / vlen; v[2] = v[2] / vlen;
}

__device__ __forceinline__ void albedo_rgb(uint32_t alb, float a[3]) {
    a[0] = float(alb & 255u) / 255.0f; a[1] = float((alb >> 8) & 255u) / 255.0f; a[2] = float((alb >> 16) & 255u) / 255.0f;
}

// A squared distance at or beyond which a light of radius r is out of reach
// for certain: for d2 >= reach_bound(r), sqrtf(d2) >= r (the bound is above r^2
// by far more than the rounding of r * r, sqrtf is correctly rounded and
// monotonic) and also d2 * rsqrtf(d2) >= r (the approximate reciprocal square
// root is off by far less than 2^-17).  Radii below 1e-18, whose square would
// lose precision, and NaN give infinity: such lights are never skipped early.
__device__ __forceinline__ float reach_bound(float r) {
    if (!(r >= 1e-18f)) return INFINITY;
    return (r * r) * 1.0000152587890625f;   // 1 + 2^-16; an overflow gives infinity
}

// Copies the lights into shared memory with reach_bound(radius) in the
// reserved field, which the loops below test before any square root.
__device__ __forceinline__ void load_lights(rsrgpu_light* L, const rsrgpu_light* __restrict__ src, int nl) {
    for (int i = threadIdx.x; i < nl; i += blockDim.x) {
        rsrgpu_light l = src[i];
        l.reserved = reach_bound(l.radius);
        L[i] = l;
    }
}

// The Blinn-Phong term of one light at P: att = (1 - d/r)^2, diffuse
// max(N.L,0)*albedo, specular max(N.H,0)^32, times the light's colour; false
// (and no term) when the light does not reach P.  l is a load_lights() copy: a
// light with d^2 >= its bound is rejected without the square root (sqrtf(d^2)
// < r would be false), so the outcome is that of testing it with sqrtf.
__device__ __forceinline__ bool plain_term(const rsrgpu_light& l, const float P[3], const float n[3],
                                           const float v[3], const float a[3], float term[3]) {
    float lx = l.position[0] - P[0], ly = l.position[1] - P[1], lz = l.position[2] - P[2];
    const float d2 = dot3(lx, ly, lz, lx, ly, lz);
    if (d2 >= l.reserved) return false;
    const float d = sqrtf(d2);
    const float r = l.radius;
    if (!(d < r)) return false;
    lx = lx / d; ly = ly / d; lz = lz / d;
    const float t = 1.0f - d / r;
    const float att = t * t;
    const float ndl = pos0(dot3(n[0], n[1], n[2], lx, ly, lz));
    float hx = lx + v[0], hy = ly + v[1], hz = lz + v[2];
    const float hlen = sqrtf(dot3(hx, hy, hz, hx, hy, hz));
    hx = hx / hlen; hy = hy / hlen; hz = hz / hlen;
    float sp = pos0(dot3(n[0], n[1], n[2], hx, hy, hz));
    sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp;   // ^32
    term[0] = (l.color[0] * att) * (a[0] * ndl + sp);
    term[1] = (l.color[1] * att) * (a[1] * ndl + sp);
    term[2] = (l.color[2] * att) * (a[2] * ndl + sp);
    return true;
}

// Blinn-Phong sum over lights first, first+step, ... < nl, added in light
// order (L: load_lights() copies)
__device__ __forceinline__ void plain_sum(const rsrgpu_light* L, int first, int step, int nl, const float P[3],
                                          const float n[3], const float v[3], const float a[3], float s[3]) {
    for (int i = first; i < nl; i += step) {
        float term[3];
        if (!plain_term(L[i], P, n, v, a, term)) continue;
        s[0] = s[0] + term[0];
        s[1] = s[1] + term[1];
        s[2] = s[2] + term[2];
    }
}

// Multi-light Blinn-Phong for one pixel plus ambient 0.03 * albedo; linear RGB.
__device__ __forceinline__ void plain_pixel(const PlainParams& p, const rsrgpu_light* L, int nl, int x, int y,
                                            float z, uint16_t hx, uint16_t hy, uint16_t hz, uint32_t alb,
                                            float rgb[3]) {
    float P[3], n[3], v[3], vlen, a[3];
    world_pos(p, x, y, z, P);
    surface(p, P, hx, hy, hz, n, v, vlen);
    albedo_rgb(alb, a);
    float s[3] = { 0.0f, 0.0f, 0.0f };
    plain_sum(L, 0, 1, nl, P, n, v, a, s);
    rgb[0] = s[0] + 0.03f * a[0];
    rgb[1] = s[1] + 0.03f * a[1];
    rgb[2] = s[2] + 0.03f * a[2];
}

// ---- the plain shader over a block of pixels ----
// kPlainBlock x kPlainBlock pixels, one per thread of a 256-thread CTA.  The
// lights that can reach the world-space box of the block's covered pixels
// are gathered once, in light order, and every pixel sums only those.  A
// light is dropped only if its squared distance to the box is at least
// (1 + 2^-12) times its reach bound: the distance to the box is a lower
// bound of the distance to every pixel of the block, and the few ulps by
// which the two computed values can disagree are far below that margin, so
// every dropped light fails plain_term for every pixel of the block and the
// sum is that of plain_sum over all lights, bit for bit.
constexpr int kPlainBlock = 16;
constexpr int kPlainThreads = kPlainBlock * kPlainBlock;

struct PlainBlockShared {
    float lo[kPlainThreads / 32][3], hi[kPlainThreads / 32][3];
    int count[kPlainThreads / 32];
    uint16_t keep[kMaxLights];
};

// The block's lights (all threads of the CTA call it; L: load_lights()
// copies, nl <= kMaxLights); returns how many were kept, in S.keep.
__device__ __forceinline__ int plain_block_lights(const rsrgpu_light* L, int nl, bool live, const float P[3],
                                                  PlainBlockShared& S) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = live ? P[k] : INFINITY;
        hi[k] = live ? P[k] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        if (lane == 0) { S.lo[warp][k] = lo[k]; S.hi[warp][k] = hi[k]; }
    }
    __syncthreads();
    for (int k = 0; k < 3; ++k) {
        lo[k] = S.lo[0][k]; hi[k] = S.hi[0][k];
        for (int w = 1; w < kPlainThreads / 32; ++w) { lo[k] = fminf(lo[k], S.lo[w][k]); hi[k] = fmaxf(hi[k], S.hi[w][k]); }
    }
    bool keep = false;
    if (t < nl) {
        const rsrgpu_light& l = L[t];
        float e[3];
        for (int k = 0; k < 3; ++k) e[k] = l.position[k] - fminf(fmaxf(l.position[k], lo[k]), hi[k]);
        keep = dot3(e[0], e[1], e[2], e[0], e[1], e[2]) < l.reserved * 1.000244140625f;
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) S.count[warp] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kPlainThreads / 32; ++w) {
        if (w == warp) before = total;
        total += S.count[w];
    }
    if (keep) S.keep[before + __popc(bal & ((1u << lane) - 1u))] = uint16_t(t);
    __syncthreads();
    return total;
}

// Blinn-Phong sum over the kept lights, in light order, plus ambient.
__device__ __forceinline__ void plain_block_pixel(const rsrgpu_light* L, const uint16_t* keep, int nkeep, const float P[3],
                                                  const float n[3], const float v[3], const float a[3], float rgb[3]) {
    float s[3] = { 0.0f, 0.0f, 0.0f };
    for (int k = 0; k < nkeep; ++k) {
        float term[3];
        if (!plain_term(L[keep[k]], P, n, v, a, term)) continue;
        s[0] = s[0] + term[0];
        s[1] = s[1] + term[1];
        s[2] = s[2] + term[2];
    }
    rgb[0] = s[0] + 0.03f * a[0];
    rgb[1] = s[1] + 0.03f * a[1];
    rgb[2] = s[2] + 0.03f * a[2];
}

// ---- learned shader inputs ----
// Candidate score of a light for a shading tile whose covered pixels span the
// world-space box [b0, b1]: (1 - d/r)^2 * (r + g + b) at the box point nearest
// the light, or -1 when the light cannot reach the box.
__device__ __forceinline__ float light_score(const rsrgpu_light& l, const float b0[3], const float b1[3]) {
    float e[3];
    for (int k = 0; k < 3; ++k) {
        const float c = fminf(fmaxf(l.position[k], b0[k]), b1[k]);
        e[k] = l.position[k] - c;
    }
    const float d = sqrtf(dot3(e[0], e[1], e[2], e[0], e[1], e[2]));
    if (!(d < l.radius)) return -1.0f;
    const float t = 1.0f - d / l.radius;
    return (t * t) * ((l.color[0] + l.color[1]) + l.color[2]);
}

// Warp-wide choice of the tile's candidates: up to kCandidates lights in
// descending score (ties to the lower index), only scores > 0; -1 pads.
// score(i) is evaluated for i < nl by the calling warp; `scratch` holds nl
// floats of shared memory.  Each light's slot is its rank: the number of
// lights with a higher score, or an equal one and a lower index.
template <typename Score>
__device__ __forceinline__ void select_candidates(int nl, Score score, int* cand, float* scratch) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < nl; i += 32) scratch[i] = score(i);
    if (lane < kCandidates) cand[lane] = -1;
    __syncwarp();
    for (int i = lane; i < nl; i += 32) {
        const float si = scratch[i];
        if (!(si > 0.0f)) continue;
        // every light is compared (no early exit), eight loads in flight at a time
        int rank = 0;
#pragma unroll 8
        for (int j = 0; j < nl; ++j) {
            const float sj = scratch[j];
            rank += (sj > si || (sj == si && j < i)) ? 1 : 0;
        }
        if (rank < kCandidates) cand[rank] = i;
    }
    __syncwarp();
}

// ---- the learned shader's inputs ----
// The 24 input features of one covered pixel:
//   0-2 unit normal, 3-5 unit view vector, 6-8 albedo, 9 eye distance / 50,
//   and a summary of the tile's candidate lights that reach the pixel, each
//   with colour c * att (att = (1 - d/r)^2), weight w = c.r + c.g + c.b (of
//   c * att) and unit direction L:
//   10-12 sum c*att, 13-15 sum w L, 16-21 sum w L L^T (xx xy xz yy yz zz),
//   22 sum w max(N.L, 0), 23 sum w (d/r) / sum w (0 without lights).
// The analytic base: one virtual light with direction sum w L (normalised)
// and colour sum c * att, Blinn-Phong (exponent 32) plus ambient 0.03 *
// albedo; base = its square root per channel.  The network adds its output
// to base, so it learns the residual sqrt(plain) - base.
// The oracle restates these exactly (oracle/rsr_oracle.c).  The kernels
// evaluate them with the SFU's approximate reciprocal and reciprocal square
// root (about one ulp each) and reciprocals multiplied in; the training data
// and the inference kernels use the same functions, so both see the same
// inputs, within a few ulps of the exact definitions.
__device__ __forceinline__ float frcp(float x) { return __fdividef(1.0f, x); }

__device__ __forceinline__ void world_pos_fast(const PlainParams& p, int x, int y, float z, float P[3]) {
    const float ndcx = (2.0f * (float(x) + 0.5f)) * frcp(float(p.width)) - 1.0f;
    const float ndcy = 1.0f - (2.0f * (float(y) + 0.5f)) * frcp(float(p.height));
    const float* m = p.ivp;
    const float cx = ((m[0] * ndcx + m[4] * ndcy) + m[8] * z) + m[12];
    const float cy = ((m[1] * ndcx + m[5] * ndcy) + m[9] * z) + m[13];
    const float cz = ((m[2] * ndcx + m[6] * ndcy) + m[10] * z) + m[14];
    const float cw = ((m[3] * ndcx + m[7] * ndcy) + m[11] * z) + m[15];
    const float iw = frcp(cw);
    P[0] = cx * iw; P[1] = cy * iw; P[2] = cz * iw;
}

// plain_sum with the SFU's approximate reciprocal square root and reciprocal
// (for estimates such as the learned shader's gate; the plain shader itself
// uses plain_sum)
__device__ __forceinline__ void plain_sum_fast(const rsrgpu_light* L, int first, int step, int nl, const float P[3],
                                               const float n[3], const float v[3], const float a[3], float s[3]) {
    for (int i = first; i < nl; i += step) {
        float lx = L[i].position[0] - P[0], ly = L[i].position[1] - P[1], lz = L[i].position[2] - P[2];
        const float d2 = dot3(lx, ly, lz, lx, ly, lz);
        if (d2 >= L[i].reserved) continue;
        const float id = rsqrtf(d2);
        const float d = d2 * id;
        const float r = L[i].radius;
        if (!(d < r)) continue;
        lx *= id; ly *= id; lz *= id;
        const float t = 1.0f - d * frcp(r);
        const float att = t * t;
        const float ndl = pos0(dot3(n[0], n[1], n[2], lx, ly, lz));
        float hx = lx + v[0], hy = ly + v[1], hz = lz + v[2];
        const float ih = rsqrtf(dot3(hx, hy, hz, hx, hy, hz));
        hx *= ih; hy *= ih; hz *= ih;
        float sp = pos0(dot3(n[0], n[1], n[2], hx, hy, hz));
        sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp;   // ^32
        s[0] = s[0] + (L[i].color[0] * att) * (a[0] * ndl + sp);
        s[1] = s[1] + (L[i].color[1] * att) * (a[1] * ndl + sp);
        s[2] = s[2] + (L[i].color[2] * att) * (a[2] * ndl + sp);
    }
}

// unit normal, unit view vector (fast arithmetic)
__device__ __forceinline__ void surface_fast(const PlainParams& p, const float P[3], uint16_t hx, uint16_t hy, uint16_t hz,
                                             float n[3], float v[3]) {
    n[0] = __half2float(__ushort_as_half(hx)); n[1] = __half2float(__ushort_as_half(hy)); n[2] = __half2float(__ushort_as_half(hz));
    const float in = rsqrtf(dot3(n[0], n[1], n[2], n[0], n[1], n[2]));
    n[0] *= in; n[1] *= in; n[2] *= in;
    v[0] = p.eye[0] - P[0]; v[1] = p.eye[1] - P[1]; v[2] = p.eye[2] - P[2];
    const float iv = rsqrtf(dot3(v[0], v[1], v[2], v[0], v[1], v[2]));
    v[0] *= iv; v[1] *= iv; v[2] *= iv;
}

// features f[24] and the virtual-light base[3] of one covered pixel; returns
// the number of candidate lights reaching it (with at most one the base is
// the pixel's Blinn-Phong shading itself)
__device__ __forceinline__ int pixel_features_fast(const PlainParams& p, const rsrgpu_light* L, const int* cand,
                                                   const float P[3], uint16_t hx, uint16_t hy, uint16_t hz,
                                                   uint32_t alb, float f[kFeatures], float base[3]) {
    float n[3] = { __half2float(__ushort_as_half(hx)), __half2float(__ushort_as_half(hy)), __half2float(__ushort_as_half(hz)) };
    const float in = rsqrtf(dot3(n[0], n[1], n[2], n[0], n[1], n[2]));
    n[0] = n[0] * in; n[1] = n[1] * in; n[2] = n[2] * in;
    float v[3] = { p.eye[0] - P[0], p.eye[1] - P[1], p.eye[2] - P[2] };
    const float v2 = dot3(v[0], v[1], v[2], v[0], v[1], v[2]);
    const float iv = rsqrtf(v2);
    v[0] = v[0] * iv; v[1] = v[1] * iv; v[2] = v[2] * iv;
    const float k255 = 1.0f / 255.0f;
    const float a[3] = { float(alb & 255u) * k255, float((alb >> 8) & 255u) * k255, float((alb >> 16) & 255u) * k255 };
    for (int k = 0; k < 3; ++k) { f[k] = n[k]; f[3 + k] = v[k]; f[6 + k] = a[k]; }
    f[9] = (v2 * iv) * 0.02f;
    for (int k = 10; k < kFeatures; ++k) f[k] = 0.0f;
    float wsum = 0.0f;
    int reach = 0;
    // the candidates within their reach bound first, then the full terms for
    // those alone (in candidate order): a warp runs the loop body as often as
    // its busiest pixel needs, not once per candidate
    uint32_t near = 0u;
    for (int c = 0; c < kCandidates; ++c) {
        const int li = cand[c];
        if (li < 0) break;
        const rsrgpu_light& l = L[li];
        const float lx = l.position[0] - P[0], ly = l.position[1] - P[1], lz = l.position[2] - P[2];
        if (dot3(lx, ly, lz, lx, ly, lz) < l.reserved) near |= 1u << c;
    }
    while (near != 0u) {
        const int c = __ffs(near) - 1;
        near &= near - 1u;
        const rsrgpu_light& l = L[cand[c]];
        const float lx = l.position[0] - P[0], ly = l.position[1] - P[1], lz = l.position[2] - P[2];
        const float d2 = dot3(lx, ly, lz, lx, ly, lz);
        const float id = rsqrtf(d2);
        const float d = d2 * id;
        if (!(d < l.radius)) continue;
        ++reach;
        const float q = d * frcp(l.radius);
        const float t = 1.0f - q;
        const float att = t * t;
        const float cr = l.color[0] * att, cg = l.color[1] * att, cb = l.color[2] * att;
        const float w = (cr + cg) + cb;
        const float ux = lx * id, uy = ly * id, uz = lz * id;
        const float wx = w * ux, wy = w * uy, wz = w * uz;
        f[10] += cr; f[11] += cg; f[12] += cb;
        f[13] += wx; f[14] += wy; f[15] += wz;
        f[16] += wx * ux; f[17] += wx * uy; f[18] += wx * uz;
        f[19] += wy * uy; f[20] += wy * uz; f[21] += wz * uz;
        f[22] += w * pos0(dot3(n[0], n[1], n[2], ux, uy, uz));
        f[23] += w * q;
        wsum += w;
    }
    f[23] = wsum > 0.0f ? f[23] * frcp(wsum) : 0.0f;
    // virtual light: direction sum w L, colour sum c * att
    const float D2 = dot3(f[13], f[14], f[15], f[13], f[14], f[15]);
    float l[3] = { 0.0f, 0.0f, 0.0f };
    if (D2 > 0.0f) { const float iD = rsqrtf(D2); l[0] = f[13] * iD; l[1] = f[14] * iD; l[2] = f[15] * iD; }
    float h[3] = { l[0] + v[0], l[1] + v[1], l[2] + v[2] };
    const float h2 = dot3(h[0], h[1], h[2], h[0], h[1], h[2]);
    if (h2 > 0.0f) { const float ih = rsqrtf(h2); h[0] *= ih; h[1] *= ih; h[2] *= ih; }
    const float ndl = pos0(dot3(n[0], n[1], n[2], l[0], l[1], l[2]));
    float sp = pos0(dot3(n[0], n[1], n[2], h[0], h[1], h[2]));
    sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp;   // ^32
    for (int c = 0; c < 3; ++c) {
        const float x = pos0(f[10 + c] * (a[c] * ndl + sp) + 0.03f * a[c]);
        base[c] = x > 0.0f ? x * rsqrtf(x) : 0.0f;
    }
    return reach;
}

}  // namespace rsrgpu
