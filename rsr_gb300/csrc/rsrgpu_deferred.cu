// rsrgpu_deferred.cu -- deferred shading over the G-buffer written by
// RSRGPU_CMD_STORE_GBUFFER: the plain multi-light shader and the learned
// shader's dense feature/target builder (training data).  The per-pixel math
// lives in rsrgpu_shading.cuh.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_shading.cuh"

namespace rsrgpu {

// One CTA per 16x16-pixel block: the block's lights are culled against its
// world-space box once (plain_block_lights), then each pixel sums those.
__global__ void __launch_bounds__(kPlainThreads) shade_plain_kernel(PlainParams p) {
    __shared__ rsrgpu_light L[kMaxLights];
    __shared__ PlainBlockShared S;
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    load_lights(L, p.lights, nl);
    const int bx = (p.width + kPlainBlock - 1) / kPlainBlock;
    const int x = (int(blockIdx.x) % bx) * kPlainBlock + int(threadIdx.x) % kPlainBlock;
    const int y = (int(blockIdx.x) / bx) * kPlainBlock + int(threadIdx.x) / kPlainBlock;
    const bool inside = x < p.width && y < p.height;
    const int i = y * p.width + x;
    const uint32_t alb = inside ? p.albedo[i] : 0u;
    const bool live = alb != 0u;
    float P[3] = { 0.0f, 0.0f, 0.0f }, n[3], v[3], vlen, a[3];
    if (live) {
        world_pos(p, x, y, p.depth[i], P);
        surface(p, P, p.nx[i], p.ny[i], p.nz[i], n, v, vlen);
        albedo_rgb(alb, a);
    }
    __syncthreads();   // the lights are in shared memory
    const int nkeep = plain_block_lights(L, nl, live, P, S);
    if (!inside) return;
    float rgb[3];
    if (live) {
        plain_block_pixel(L, S.keep, nkeep, P, n, v, a, rgb);
    } else {
        rgb[0] = p.background[0]; rgb[1] = p.background[1]; rgb[2] = p.background[2];
    }
    if (p.out_linear) { p.out_linear[3 * i] = rgb[0]; p.out_linear[3 * i + 1] = rgb[1]; p.out_linear[3 * i + 2] = rgb[2]; }
    if (p.out_srgb)
        p.out_srgb[i] = pack_srgb(p.srgb_lut, rgb);
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
    const int blocks = ((gb.width + kPlainBlock - 1) / kPlainBlock) * ((gb.height + kPlainBlock - 1) / kPlainBlock);
    shade_plain_kernel<<<blocks, kPlainThreads, 0, st>>>(p);
    return cudaGetLastError();
}

// ---- learned shader: dense features and training targets ----
// One CTA of 128 threads per 32x32 shading tile (grid-stride over tiles).
// Pass 1: the world-space box of the tile's covered pixels; warp 0 picks the
// tile's candidate lights; pass 2: features (BF16, 32 columns,
// 24..31 zero) and the network's targets sqrt(max(plain, 0)) - base per pixel
// (base: the analytic virtual-light estimate, see rsrgpu_shading.cuh).  Uncovered pixels
// (albedo 0) get zero rows.
struct FeatParams {
    PlainParams pl;
    uint16_t* features;    // [W*H][32] bf16
    float* targets;        // [W*H][3] or null
    int32_t* candidates;   // [tiles][8] or null
};

__global__ void __launch_bounds__(128) learned_features_kernel(FeatParams F) {
    __shared__ rsrgpu_light lights[kMaxLights];
    __shared__ float box[2][4][3];
    __shared__ int cand[kCandidates];
    __shared__ float scores[kMaxLights];
    const PlainParams& p = F.pl;
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    load_lights(lights, p.lights, nl);
    const int tiles_x = (p.width + kShadeTile - 1) / kShadeTile, tiles_y = (p.height + kShadeTile - 1) / kShadeTile;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int tile = blockIdx.x; tile < tiles_x * tiles_y; tile += gridDim.x) {
        const int x0 = (tile % tiles_x) * kShadeTile, y0 = (tile / tiles_x) * kShadeTile;
        // thread t: row t / 4, columns (t % 4) * 8 .. + 7
        const int y = y0 + t / 4, xb = x0 + (t % 4) * 8;
        float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int x = xb + j;
            if (x < p.width && y < p.height && p.albedo[y * p.width + x] != 0u) {
                float P[3];
                world_pos(p, x, y, p.depth[y * p.width + x], P);
                for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], P[k]); hi[k] = fmaxf(hi[k], P[k]); }
            }
        }
        for (int k = 0; k < 3; ++k) {
            for (int o = 16; o > 0; o >>= 1) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
            }
            if (lane == 0) { box[0][warp][k] = lo[k]; box[1][warp][k] = hi[k]; }
        }
        __syncthreads();
        if (warp == 0) {
            float b0[3], b1[3];
            for (int k = 0; k < 3; ++k) {
                b0[k] = fminf(fminf(box[0][0][k], box[0][1][k]), fminf(box[0][2][k], box[0][3][k]));
                b1[k] = fmaxf(fmaxf(box[1][0][k], box[1][1][k]), fmaxf(box[1][2][k], box[1][3][k]));
            }
            const bool empty = !(b0[0] <= b1[0]);
            select_candidates(empty ? 0 : nl, [&](int i) { return light_score(lights[i], b0, b1); }, cand, scores);
            if (lane == 0 && F.candidates)
                for (int c = 0; c < kCandidates; ++c) F.candidates[tile * kCandidates + c] = cand[c];
        }
        __syncthreads();
#pragma unroll 1
        for (int j = 0; j < 8; ++j) {
            const int x = xb + j;
            if (x >= p.width || y >= p.height) continue;
            const int pi = y * p.width + x;
            const uint32_t alb = p.albedo[pi];
            uint4* dst = reinterpret_cast<uint4*>(F.features + size_t(pi) * 32);
            if (alb == 0u) {
                for (int q = 0; q < 4; ++q) dst[q] = make_uint4(0, 0, 0, 0);
                if (F.targets) { F.targets[3 * size_t(pi)] = 0.f; F.targets[3 * size_t(pi) + 1] = 0.f; F.targets[3 * size_t(pi) + 2] = 0.f; }
                continue;
            }
            float P[3], f[32], base[3];
            world_pos_fast(p, x, y, p.depth[pi], P);
            pixel_features_fast(p, lights, cand, P, p.nx[pi], p.ny[pi], p.nz[pi], alb, f, base);
            for (int q = kFeatures; q < 32; ++q) f[q] = 0.0f;
            uint32_t w[16];
            for (int q = 0; q < 16; ++q)
                w[q] = uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(f[2 * q]))) |
                       (uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(f[2 * q + 1]))) << 16);
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
            if (F.targets) {
                float rgb[3];
                plain_pixel(p, lights, nl, x, y, p.depth[pi], p.nx[pi], p.ny[pi], p.nz[pi], alb, rgb);
                for (int c = 0; c < 3; ++c) F.targets[3 * size_t(pi) + c] = sqrtf(pos0(rgb[c])) - base[c];
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_learned_features(const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                                    const rsrgpu_light* lights, int nlights, uint16_t* features, float* targets,
                                    int32_t* candidates, int num_sms, cudaStream_t st) {
    FeatParams F{};
    PlainParams& p = F.pl;
    p.depth = gb.depth; p.nx = gb.normal_x; p.ny = gb.normal_y; p.nz = gb.normal_z; p.albedo = gb.albedo;
    p.width = gb.width; p.height = gb.height;
    for (int i = 0; i < 16; ++i) p.ivp[i] = ivp[i];
    for (int i = 0; i < 3; ++i) p.eye[i] = eye[i];
    p.lights = lights; p.nlights = nlights;
    F.features = features; F.targets = targets; F.candidates = candidates;
    const int tiles = ((gb.width + kShadeTile - 1) / kShadeTile) * ((gb.height + kShadeTile - 1) / kShadeTile);
    int grid = num_sms * 8;
    if (grid > tiles) grid = tiles;
    learned_features_kernel<<<grid, 128, 0, st>>>(F);
    return cudaGetLastError();
}

}  // namespace rsrgpu
