// rsrgpu_postfx.cu -- rsr's post-processing of float canvases on the device:
// the Kawase blur pass (KawaseBlurFilter, src/rgl/rglr/rglr_kawase.cxx:22-84,
// chained by the $kawase node, src/viewer/node/kawase.cxx:79-117) and the
// glow resolve (rglr::Filter<GlowShader, sRGB|LinearColor>,
// src/rgl/rglr/rglr_algorithm.hxx:107-144, with the $glow node's shader,
// src/viewer/node/glow.cxx:24-36).
//
// Canvases are rsr's: RGBA float pixels (FloatingPointCanvas), quads of
// x[4] y[4] z[4] w[4] (QFloat4Canvas) and 0x00RRGGBB pixels
// (TrueColorCanvas).  Both kernels are bandwidth work on canvases that stay
// in the 129 MB L2 between the passes of a chain (a 960x540 float canvas is
// 8.3 MB).
//
// kawase_kernel: one thread per output pixel; the sixteen source pixels of
// its four 2x2 boxes come through the read-only cache (neighbouring threads
// share most of them).  The sums keep the reference's order: each box
// ((p(x,y) + p(x+1,y)) + p(x,y+1)) + p(x+1,y+1), the boxes added one by one
// onto +0 in offset order, then times 1/16.  Coordinates are clamped to the
// source, which gives the reference's values on its fast interior path and
// its clamped border path alike.
//
// glow_kernel: one thread per 2x2 quad of the output: the quad's image lanes
// (x, y, z of its qfloat4) and the half-size blur pixel under it,
// (image + blur * 0.7) * 0.5 per channel, packed to sRGB8 or linear 8-bit.
#include <cstdint>

#include <cuda_runtime.h>

namespace rsrgpu {

struct FloatCanvasView {      // rsrgpu_fp_canvas / rsrgpu_qfloat4_canvas on the device
    float4* data;
    int width, height, stride;
};

constexpr int kPostThreads = 256;

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

__global__ void __launch_bounds__(kPostThreads) kawase_kernel(const float4* __restrict__ src, int sw, int sh, int sstride,
                                                              float4* __restrict__ dst, int dw, int dh, int dstride, int d) {
    const int x = int(blockIdx.x) * 32 + int(threadIdx.x & 31);
    const int y = int(blockIdx.y) * (kPostThreads / 32) + int(threadIdx.x >> 5);
    if (x >= dw || y >= dh) return;
    const int ox[4] = { -d - 1, d, -d - 1, d };
    const int oy[4] = { -d - 1, -d - 1, d, d };
    float4 ax = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        // sample_safe / sample_fast (rglr_kawase.cxx:37-49): the 2x2 box at
        // (x + ox, y + oy), coordinates clamped to the source
        const int bx = x + ox[k], by = y + oy[k];
        const int x0 = min(max(bx, 0), sw - 1), x1 = min(max(bx + 1, 0), sw - 1);
        const int y0 = min(max(by, 0), sh - 1), y1 = min(max(by + 1, 0), sh - 1);
        const float4* r0 = src + size_t(y0) * sstride;
        const float4* r1 = src + size_t(y1) * sstride;
        const float4 s = add4(add4(add4(__ldg(r0 + x0), __ldg(r0 + x1)), __ldg(r1 + x0)), __ldg(r1 + x1));
        ax = add4(ax, s);
    }
    const float k16 = 1.0f / 16.0f;
    dst[size_t(y) * dstride + x] = make_float4(ax.x * k16, ax.y * k16, ax.z * k16, ax.w * k16);
}

// to_tc_basic's channel (rglr_canvas_util.hxx:39-49): minps with 1, maxps
// with 0, times 255, truncated
__device__ __forceinline__ uint32_t basic8_post(float v) {
    float r = v < 1.0f ? v : 1.0f;
    r = r > 0.0f ? r : 0.0f;
    return uint32_t(__float2int_rz(r * 255.0f));
}
// the sRGB8 encoder of the TrueColor stores (correctly rounded sRGB curve,
// a table over the top 20 bits of the clamped value)
__device__ __forceinline__ uint32_t srgb8_post(const uint8_t* __restrict__ lut, float v) {
    const float lo = __uint_as_float((127u - 13u) << 23), hi = __uint_as_float(0x3f7fffffu);
    float c = v > lo ? v : lo;
    c = c < hi ? c : hi;
    return __ldg(lut + ((__float_as_uint(c) >> 12) - ((127u - 13u) << 11)));
}

__global__ void __launch_bounds__(kPostThreads) glow_kernel(const float4* __restrict__ image, int istride,
                                                            const float4* __restrict__ blur, int bstride,
                                                            uint32_t* __restrict__ out, int ostride, int qw, int qh,
                                                            const uint8_t* __restrict__ srgb_lut) {
    const int q = int(blockIdx.x) * kPostThreads + int(threadIdx.x);
    if (q >= qw * qh) return;
    const int qx = q % qw, qy = q / qw;
    const float4* iq = image + (size_t(qy) * istride + qx) * 4;
    const float4 r = __ldg(iq), g = __ldg(iq + 1), b = __ldg(iq + 2);
    const float4 bl = __ldg(blur + size_t(qy) * bstride + qx);
    const float blur_amt = 0.700f, brightness = 0.5f;
    // GlowShader::ShadeCanvas (glow.cxx:25-36): (image + blur * blurAmt) * brightness
    const float br = bl.x * blur_amt, bg = bl.y * blur_amt, bb = bl.z * blur_amt;
    const float rl[4] = { r.x, r.y, r.z, r.w }, gl[4] = { g.x, g.y, g.z, g.w }, bll[4] = { b.x, b.y, b.z, b.w };
    uint32_t px[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const float cr = (rl[l] + br) * brightness, cg = (gl[l] + bg) * brightness, cb = (bll[l] + bb) * brightness;
        px[l] = srgb_lut ? (srgb8_post(srgb_lut, cr) << 16) | (srgb8_post(srgb_lut, cg) << 8) | srgb8_post(srgb_lut, cb)
                         : (basic8_post(cr) << 16) | (basic8_post(cg) << 8) | basic8_post(cb);
    }
    uint32_t* o = out + size_t(2 * qy) * ostride + 2 * qx;
    *reinterpret_cast<uint2*>(o) = make_uint2(px[0], px[1]);
    *reinterpret_cast<uint2*>(o + ostride) = make_uint2(px[2], px[3]);
}

cudaError_t launch_kawase(const FloatCanvasView& src, const FloatCanvasView& dst, int dist, cudaStream_t st) {
    const dim3 grid((dst.width + 31) / 32, (dst.height + kPostThreads / 32 - 1) / (kPostThreads / 32));
    kawase_kernel<<<grid, kPostThreads, 0, st>>>(src.data, src.width, src.height, src.stride, dst.data, dst.width,
                                                 dst.height, dst.stride, dist);
    return cudaGetLastError();
}

cudaError_t launch_glow(const FloatCanvasView& image, const FloatCanvasView& blur, uint32_t* out, int ostride,
                        int width, int height, const uint8_t* srgb_lut, cudaStream_t st) {
    const int qw = width / 2, qh = height / 2;
    const int blocks = (qw * qh + kPostThreads - 1) / kPostThreads;
    glow_kernel<<<blocks, kPostThreads, 0, st>>>(image.data, image.stride, blur.data, blur.stride, out, ostride, qw, qh,
                                                 srgb_lut);
    return cudaGetLastError();
}

}  // namespace rsrgpu
