// rsrgpu_texture.cu -- texture upload and mip-chain build on the device.
//
// rsr builds its textures on the host: PNGToTexture converts decoded RGBA8
// pixels to linear float (src/rgl/rglr/rglr_texture_load.cxx:40-63) and
// Texture::maybe_make_mipmap appends the mip chain (src/rgl/rglr/
// rglr_texture.cxx:33-80).  Here both run as one pass over HBM.
//
// Layout (rsr's): RGBA float texels (PixelToaster::FloatingPointPixel),
// row stride = the texture's width.  A square power-of-two texture of edge
// w = 2^p (p <= 12) holds w*w*2 texels: level 0 in rows [0, w); level k
// (edge w >> k) in rows [2w - 2(w >> k), 2w - (w >> k)), columns
// [0, w >> k); every other texel of rows [w, 2w) is zero (the reference's
// buffer is value-initialised when it grows to w*w*2).
//
// mip_block_kernel: one CTA per 32x32 block of a source level (the whole
// level when it is smaller).  It reads the block once -- RGBA8 through the
// decode table in shared memory (writing level 0), or float -- and reduces it
// in shared memory through up to five levels, writing each.  Levels above
// the fifth take another launch over the fifth level (L2-resident).  The
// first launch also carries CTAs that zero the texels of rows [w, 2w) that
// no level covers, so every byte of the chain is written exactly once.
#include <cstdint>

#include <cuda_runtime.h>

namespace rsrgpu {

// ryg::srgb8_to_float (3rdparty/ryg-srgb/ryg-srgb.h:33-56) for every byte,
// generated by gen_srgb_decode_table.c
__device__ const uint32_t kSrgbDecode[256] = {
#include "srgb_decode_table.inc"
};

constexpr int kMipBlock = 32;       // source block edge of one CTA
constexpr int kMipThreads = 256;
constexpr int kZeroPerCta = 4096;   // zeroed texels per zero-fill CTA

struct MipArgs {
    float4* tex;            // texture base, row stride w
    const uchar4* rgba8;    // level-0 bytes, w x w (conversion launch)
    int w;                  // level-0 edge, 2^p
    int src_level;          // level the block CTAs read
    int levels;             // levels written below it (0..5)
    int premultiply;
    int block_ctas;         // CTAs that reduce blocks; the rest zero-fill
};

// first row of level k >= 1: 2w - 2(w >> k)
__device__ __forceinline__ int level_row(int w, int k) { return k == 0 ? 0 : 2 * w - 2 * (w >> k); }

// edge of the level owning row r of [w, 2w): the power of two s with
// s < 2w - r <= 2s; 0 for the last row, which no level uses
__device__ __forceinline__ int row_level_edge(int w, int r) {
    const int d = 2 * w - r;
    return d <= 1 ? 0 : 1 << (31 - __clz(d - 1));
}

// Texture::maybe_make_mipmap's texel: the 2x2 parents added in row-major
// order, then divided by 4 (rglr_texture.cxx:60-66)
__device__ __forceinline__ float4 mip_texel(float4 a, float4 b, float4 c, float4 d) {
    float4 v;
    v.x = (((a.x + b.x) + c.x) + d.x) / 4.0f;
    v.y = (((a.y + b.y) + c.y) + d.y) / 4.0f;
    v.z = (((a.z + b.z) + c.z) + d.z) / 4.0f;
    v.w = (((a.w + b.w) + c.w) + d.w) / 4.0f;
    return v;
}

// PNGToTexture's texel (rglr_texture_load.cxx:52-60): rgb through the sRGB
// table, alpha / 255, optionally premultiplied
__device__ __forceinline__ float4 decode_texel(uchar4 c, const float* lut, bool premultiply) {
    float4 v;
    v.x = lut[c.x];
    v.y = lut[c.y];
    v.z = lut[c.z];
    v.w = float(c.w) / 255.0f;
    if (premultiply) {
        v.x = v.x * v.w;
        v.y = v.y * v.w;
        v.z = v.z * v.w;
    }
    return v;
}

template <bool kFromRGBA8>
__global__ void __launch_bounds__(kMipThreads) mip_block_kernel(const MipArgs a) {
    __shared__ float4 s0[kMipBlock * kMipBlock];
    __shared__ float4 s1[(kMipBlock / 2) * (kMipBlock / 2)];
    __shared__ float lut[256];
    const int tid = threadIdx.x;
    if (int(blockIdx.x) >= a.block_ctas) {
        // zero-fill: texels of rows [w, 2w) that hold no level
        const size_t region = size_t(a.w) * size_t(a.w);
        const size_t t0 = size_t(int(blockIdx.x) - a.block_ctas) * kZeroPerCta;
        for (size_t t = t0 + tid; t < t0 + kZeroPerCta && t < region; t += kMipThreads) {
            const int r = a.w + int(t / size_t(a.w)), c = int(t % size_t(a.w));
            if (c >= row_level_edge(a.w, r)) a.tex[size_t(r) * a.w + c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        return;
    }
    if (kFromRGBA8) {
        for (int i = tid; i < 256; i += kMipThreads) lut[i] = __uint_as_float(kSrgbDecode[i]);
        __syncthreads();
    }
    const int src_edge = a.w >> a.src_level;
    const int B = src_edge < kMipBlock ? src_edge : kMipBlock;
    const int nbx = src_edge / B;
    const int bx = int(blockIdx.x) % nbx, by = int(blockIdx.x) / nbx;
    const int row0 = level_row(a.w, a.src_level);
    for (int i = tid; i < B * B; i += kMipThreads) {
        const int x = bx * B + i % B, y = by * B + i / B;
        float4 v;
        if (kFromRGBA8) {
            v = decode_texel(a.rgba8[size_t(y) * a.w + x], lut, a.premultiply != 0);
            a.tex[size_t(y) * a.w + x] = v;
        } else {
            v = a.tex[size_t(row0 + y) * a.w + x];
        }
        s0[i] = v;
    }
    float4* src = s0;
    float4* dst = s1;
    int e = B;
    for (int j = 1; j <= a.levels; ++j) {
        __syncthreads();
        const int h = e >> 1;
        const int rowl = level_row(a.w, a.src_level + j);
        for (int i = tid; i < h * h; i += kMipThreads) {
            const int x = i % h, y = i / h;
            const float4* p = src + (2 * y) * e + 2 * x;
            const float4 v = mip_texel(p[0], p[1], p[e], p[e + 1]);
            dst[i] = v;
            a.tex[size_t(rowl + by * h + y) * a.w + bx * h + x] = v;
        }
        float4* t = src; src = dst; dst = t;
        e = h;
    }
}

// Conversion only (textures without a mip chain): one texel per thread.
__global__ void __launch_bounds__(kMipThreads) rgba8_to_float_kernel(const uchar4* __restrict__ in, float4* __restrict__ out,
                                                                     size_t n, int premultiply) {
    __shared__ float lut[256];
    for (int i = threadIdx.x; i < 256; i += kMipThreads) lut[i] = __uint_as_float(kSrgbDecode[i]);
    __syncthreads();
    for (size_t i = size_t(blockIdx.x) * kMipThreads + threadIdx.x; i < n; i += size_t(gridDim.x) * kMipThreads)
        out[i] = decode_texel(in[i], lut, premultiply != 0);
}

static int ilog2(int w) { int p = 0; while ((1 << p) < w) ++p; return p; }

// Texture::maybe_make_mipmap's test (rglr_texture.cxx:35-50): the power of
// a square power-of-two edge of at most 4096, else -1 (no chain)
int texture_power(int width, int height) {
    if (width != height || width <= 0 || (width & (width - 1)) != 0) return -1;
    const int p = ilog2(width);
    return p > 12 ? -1 : p;
}

// Launches the chain of a texture of edge w = 2^p whose level 0 is in tex
// (from_rgba8: converted from rgba8 by the first launch).
cudaError_t launch_texture_chain(float* tex, const uint8_t* rgba8, int w, int premultiply, cudaStream_t st) {
    const int p = ilog2(w);
    MipArgs a{};
    a.tex = reinterpret_cast<float4*>(tex);
    a.rgba8 = reinterpret_cast<const uchar4*>(rgba8);
    a.w = w;
    a.premultiply = premultiply;
    a.src_level = 0;
    bool first = true;
    while (first || a.src_level < p) {
        const int src_edge = w >> a.src_level;
        const int B = src_edge < kMipBlock ? src_edge : kMipBlock;
        a.levels = ilog2(B);
        a.block_ctas = (src_edge / B) * (src_edge / B);
        int ctas = a.block_ctas;
        if (first) ctas += int((size_t(w) * size_t(w) + kZeroPerCta - 1) / kZeroPerCta);
        if (first && rgba8 != nullptr) mip_block_kernel<true><<<ctas, kMipThreads, 0, st>>>(a);
        else mip_block_kernel<false><<<ctas, kMipThreads, 0, st>>>(a);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        first = false;
        a.src_level += a.levels;
    }
    return cudaSuccess;
}

cudaError_t launch_rgba8_to_float(const uint8_t* rgba8, float* out, size_t n, int premultiply, int num_sms,
                                  cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    size_t blocks = (n + kMipThreads - 1) / kMipThreads;
    const size_t cap = size_t(num_sms) * 8;
    if (blocks > cap) blocks = cap;
    rgba8_to_float_kernel<<<unsigned(blocks), kMipThreads, 0, st>>>(reinterpret_cast<const uchar4*>(rgba8),
                                                                     reinterpret_cast<float4*>(out), n, premultiply);
    return cudaGetLastError();
}

}  // namespace rsrgpu
