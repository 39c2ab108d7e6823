// rsrgpu_deferred.cu -- deferred shading over the G-buffer written by
// RSRGPU_CMD_STORE_GBUFFER.  rsr has no deferred or multi-light path; the
// plain shader here is this library's definition (its CPU restatement in
// oracle/rsr_oracle.c is the oracle).  Built with -fmad=false like the
// rasteriser, so every expression rounds once per operation in the written
// order and the GPU matches the oracle bit for bit.
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_internal.h"

namespace rsrgpu {

constexpr int kMaxLights = 256;

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

// Multi-light Blinn-Phong for one pixel; returns linear RGB.
__device__ __forceinline__ void plain_pixel(const PlainParams& p, const rsrgpu_light* L, int nl, int x, int y,
                                            float z, uint16_t hx, uint16_t hy, uint16_t hz, uint32_t alb,
                                            float rgb[3]) {
    const float ndcx = (2.0f * (float(x) + 0.5f)) / float(p.width) - 1.0f;
    const float ndcy = 1.0f - (2.0f * (float(y) + 0.5f)) / float(p.height);
    const float* m = p.ivp;
    const float cx = ((m[0] * ndcx + m[4] * ndcy) + m[8] * z) + m[12];
    const float cy = ((m[1] * ndcx + m[5] * ndcy) + m[9] * z) + m[13];
    const float cz = ((m[2] * ndcx + m[6] * ndcy) + m[10] * z) + m[14];
    const float cw = ((m[3] * ndcx + m[7] * ndcy) + m[11] * z) + m[15];
    const float px = cx / cw, py = cy / cw, pz = cz / cw;
    float nx = __half2float(__ushort_as_half(hx)), ny = __half2float(__ushort_as_half(hy)), nz = __half2float(__ushort_as_half(hz));
    const float nlen = sqrtf(dot3(nx, ny, nz, nx, ny, nz));
    nx = nx / nlen; ny = ny / nlen; nz = nz / nlen;
    float vx = p.eye[0] - px, vy = p.eye[1] - py, vz = p.eye[2] - pz;
    const float vlen = sqrtf(dot3(vx, vy, vz, vx, vy, vz));
    vx = vx / vlen; vy = vy / vlen; vz = vz / vlen;
    const float ar = float(alb & 255u) / 255.0f, ag = float((alb >> 8) & 255u) / 255.0f, ab = float((alb >> 16) & 255u) / 255.0f;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f;
    for (int i = 0; i < nl; ++i) {
        float lx = L[i].position[0] - px, ly = L[i].position[1] - py, lz = L[i].position[2] - pz;
        const float d = sqrtf(dot3(lx, ly, lz, lx, ly, lz));
        const float r = L[i].radius;
        if (!(d < r)) continue;
        lx = lx / d; ly = ly / d; lz = lz / d;
        const float t = 1.0f - d / r;
        const float att = t * t;
        const float ndl = pos0(dot3(nx, ny, nz, lx, ly, lz));
        float hx2 = lx + vx, hy2 = ly + vy, hz2 = lz + vz;
        const float hlen = sqrtf(dot3(hx2, hy2, hz2, hx2, hy2, hz2));
        hx2 = hx2 / hlen; hy2 = hy2 / hlen; hz2 = hz2 / hlen;
        float s = pos0(dot3(nx, ny, nz, hx2, hy2, hz2));
        s = s * s; s = s * s; s = s * s; s = s * s; s = s * s;   // ^32
        sr = sr + (L[i].color[0] * att) * (ar * ndl + s);
        sg = sg + (L[i].color[1] * att) * (ag * ndl + s);
        sb = sb + (L[i].color[2] * att) * (ab * ndl + s);
    }
    rgb[0] = sr + 0.03f * ar;
    rgb[1] = sg + 0.03f * ag;
    rgb[2] = sb + 0.03f * ab;
}

__global__ void __launch_bounds__(256) shade_plain_kernel(PlainParams p) {
    __shared__ rsrgpu_light L[kMaxLights];
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    for (int i = threadIdx.x; i < nl; i += blockDim.x) L[i] = p.lights[i];
    __syncthreads();
    const int n = p.width * p.height;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int x = i % p.width, y = i / p.width;
        const uint32_t alb = p.albedo[i];
        float rgb[3];
        if (alb == 0u) {
            rgb[0] = p.background[0]; rgb[1] = p.background[1]; rgb[2] = p.background[2];
        } else {
            plain_pixel(p, L, nl, x, y, p.depth[i], p.nx[i], p.ny[i], p.nz[i], alb, rgb);
        }
        if (p.out_linear) { p.out_linear[3 * i] = rgb[0]; p.out_linear[3 * i + 1] = rgb[1]; p.out_linear[3 * i + 2] = rgb[2]; }
        if (p.out_srgb)
            p.out_srgb[i] = (srgb8_lut(p.srgb_lut, rgb[0]) << 16) | (srgb8_lut(p.srgb_lut, rgb[1]) << 8) | srgb8_lut(p.srgb_lut, rgb[2]);
    }
}

cudaError_t launch_shade_plain(const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                               const rsrgpu_light* lights, int nlights, const float background[3],
                               uint32_t* out_srgb, float* out_linear, const uint8_t* srgb_lut, cudaStream_t st) {
    PlainParams p{};
    p.depth = gb.depth; p.nx = gb.normal_x; p.ny = gb.normal_y; p.nz = gb.normal_z; p.albedo = gb.albedo;
    p.width = gb.width; p.height = gb.height;
    for (int i = 0; i < 16; ++i) p.ivp[i] = ivp[i];
    for (int i = 0; i < 3; ++i) { p.eye[i] = eye[i]; p.background[i] = background[i]; }
    p.lights = lights; p.nlights = nlights; p.out_srgb = out_srgb; p.out_linear = out_linear; p.srgb_lut = srgb_lut;
    const int n = gb.width * gb.height;
    int blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    shade_plain_kernel<<<blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace rsrgpu
