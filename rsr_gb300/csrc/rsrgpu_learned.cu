// rsrgpu_learned.cu -- the learned deferred shader as one fused kernel.
//
// Persistent CTAs of four warps take 32x32 shading tiles from a counter:
//   1. coverage of the tile's pixels, compacted into a list (the tile's 4x4
//      grid of gate sample pixels first) and the world-space box of the
//      covered pixels; background pixels are written at once
//   2. warp 0 picks the tile's candidate lights (rsrgpu_shading.cuh)
//   3. the gate's reference: the plain shader at the first min(16, covered)
//      listed pixels, each split over eight threads
//   4. for each 128 covered pixels: 24 features per pixel into a BF16 A tile
//      and the analytic base (virtual_light_base, FP32), the MLP's four
//      layers on tcgen05, output rgb = max(y + base, 0)^2 (the network
//      predicts the residual of square roots of linear RGB); after the first
//      128 the gate compares the learned and plain sRGB8 values of the samples
//      and, when their mean squared error exceeds the threshold, the tile is
//      shaded by the plain shader instead (bit-exact with rsrgpu_shade_plain),
//      skipping the remaining MLP work
//
// The biases ride in the MMAs: every A tile carries two columns of ones and
// every weight tile the bias split into a BF16 high part and a BF16 low part
// (b - hi), so D = A W^T already holds W a + b to about 2^-16 relative; the
// epilogue is one cvt.rn.relu.bf16x2 per two activations.  One shared-memory
// A buffer serves all layers: layer 1 reads it as 128 x 32 (features, ones
// at 24 and 25), the hidden layers as 128 x 80 (activations, ones at 64 and
// 65); each MMA group has completed before the epilogue overwrites it.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_mlp.cuh"
#include "rsrgpu_shading.cuh"

namespace rsrgpu {

constexpr int kTilePx = kShadeTile * kShadeTile;   // 1024
constexpr int kGateSamples = 16;
constexpr int kK1 = 32;          // layer-1 K: 24 features, ones at 24/25, zeros
constexpr int kKH = 80;          // hidden-layer K: 64 activations, ones at 64/65, zeros

struct LearnSmem {
    alignas(128) uint8_t w1[kHid * kK1 * 2];      // 64 x 32
    alignas(128) uint8_t w2[kHid * kKH * 2];      // 64 x 80
    alignas(128) uint8_t w3[kHid * kKH * 2];
    alignas(128) uint8_t w4[kOut * kKH * 2];      // 16 x 80
    alignas(128) uint8_t act[kRows * kKH * 2];    // A operand of every layer
    uint16_t list[kTilePx];                       // covered pixels (tile-local index y * 32 + x)
    float box[2][4][3];
    int scan[4];
    int cand[kCandidates];
    float gate_plain[kGateSamples][3];
    int gate_sum;
    int tile;
    uint64_t mbar;
    uint32_t tmem;
    alignas(16) rsrgpu_light lights[1];           // nlights entries (dynamic shared memory)
};

struct LearnParams {
    PlainParams pl;
    rsrgpu_mlp w;
    float max_tile_mse;       // in 8-bit sRGB units squared
    uint8_t* tile_status;     // [tiles] or null: 0 learned, 1 plain fallback, 2 nothing covered
    float* tile_mse;          // [tiles] or null: the gate's estimate
    int* error;
    int* tile_counter;        // zero at launch
};

__device__ __forceinline__ void store_pixel(const PlainParams& p, int pi, const float rgb[3]) {
    if (p.out_linear) { p.out_linear[3 * size_t(pi)] = rgb[0]; p.out_linear[3 * size_t(pi) + 1] = rgb[1]; p.out_linear[3 * size_t(pi) + 2] = rgb[2]; }
    if (p.out_srgb) p.out_srgb[pi] = pack_srgb(p.srgb_lut, rgb);
}

__device__ __forceinline__ uint16_t bf16_rn(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }

// W (the first KSRC columns of a row-major [rows][LD] bf16 matrix) plus the
// bias as columns KSRC (high) and KSRC+1 (low), zeros to KDIM, into a K-major
// tile of K = KDIM; 16-byte chunks (8 columns of one row) per thread
template <int KSRC, int LD, int KDIM>
__device__ __forceinline__ void load_weights_bias(uint8_t* dst, const uint16_t* __restrict__ W, int rows,
                                                  const float* __restrict__ bias) {
    constexpr int kChunks = KDIM / 8, kSrcChunks = KSRC / 8;
    for (int c = threadIdx.x; c < rows * kChunks; c += blockDim.x) {
        const int r = c / kChunks, j = c % kChunks;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (j < kSrcChunks) {
            v = __ldg(reinterpret_cast<const uint4*>(W + r * LD + j * 8));
        } else if (j == kSrcChunks) {
            const float b = __ldg(bias + r);
            const uint16_t hi = bf16_rn(b);
            const uint16_t lo = bf16_rn(b - __bfloat162float(__ushort_as_bfloat16(hi)));
            v.x = uint32_t(hi) | (uint32_t(lo) << 16);
        }
        *reinterpret_cast<uint4*>(dst + tc::kmajor_offset(r, j * 8, KDIM)) = v;
    }
}

// MMAs of one layer: D[128 x n] = act (128 x kdim) * W (n x kdim)^T, committed to mbar
__device__ __forceinline__ void issue(uint32_t d, const uint8_t* a, const uint8_t* w, int kdim, int n, uint64_t* mbar) {
    tc::fence_after_sync();
    const uint32_t sa = tc::smem_addr(a), sw = tc::smem_addr(w);
    const uint32_t sbo = uint32_t(kdim / 8) * 128u;
    for (int ks = 0; ks < kdim / 16; ++ks)
        tc::mma_bf16(d, tc::smem_desc(sa + ks * 256u, 128u, sbo), tc::smem_desc(sw + ks * 256u, 128u, sbo),
                     tc::idesc_bf16(kRows, n), ks > 0 ? 1u : 0u);
    tc::mma_commit(mbar);
}

// TMEM row (64 fp32 columns) -> ReLU -> BF16 activations of row t (K = 80 layout)
__device__ __forceinline__ void relu_epilogue(uint32_t trow, uint8_t* act, int t) {
    uint32_t r[64];
    tc::tmem_ld32_nowait(trow, r);
    tc::tmem_ld32_nowait(trow + 32, r + 32);
    tc::tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < 64; c += 8) {
        uint4 pk;
        pk.x = tc::relu_bf16x2(r[c], r[c + 1]); pk.y = tc::relu_bf16x2(r[c + 2], r[c + 3]);
        pk.z = tc::relu_bf16x2(r[c + 4], r[c + 5]); pk.w = tc::relu_bf16x2(r[c + 6], r[c + 7]);
        *reinterpret_cast<uint4*>(act + tc::kmajor_offset(t, c, kKH)) = pk;
    }
}

__global__ void __launch_bounds__(128, 4) shade_learned_kernel(LearnParams A) {
    extern __shared__ uint8_t smem_raw[];
    LearnSmem& S = *reinterpret_cast<LearnSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const PlainParams& p = A.pl;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    load_weights_bias<kFeatures, kIn, kK1>(S.w1, A.w.w1, kHid, A.w.b1);
    load_weights_bias<kHid, kHid, kKH>(S.w2, A.w.w2, kHid, A.w.b2);
    load_weights_bias<kHid, kHid, kKH>(S.w3, A.w.w3, kHid, A.w.b3);
    load_weights_bias<kHid, kHid, kKH>(S.w4, A.w.w4, kOut, A.w.b4);
    for (int i = t; i < nl; i += blockDim.x) S.lights[i] = p.lights[i];
    if (t == 0) tc::mbar_init(&S.mbar, 1);
    if (warp == 0) { tc::tmem_alloc(&S.tmem, 64); tc::tmem_relinquish(); }
    tc::fence_smem_for_mma();
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem;
    const uint32_t trow = tmem + (uint32_t(warp * 32) << 16);
    uint32_t phase = 0;
    bool aborted = false;
    // columns 64..79 of a hidden-layer A row: ones at 64 and 65 (the bias columns)
    const uint32_t one2 = uint32_t(bf16_rn(1.0f)) | (uint32_t(bf16_rn(1.0f)) << 16);
    const uint4 ones_row = make_uint4(one2, 0u, 0u, 0u);

    const int tiles_x = (p.width + kShadeTile - 1) / kShadeTile, tiles_y = (p.height + kShadeTile - 1) / kShadeTile;
    const int ntiles = tiles_x * tiles_y;
    for (;;) {
        if (t == 0) S.tile = atomicAdd(A.tile_counter, 1);
        __syncthreads();
        const int tile = S.tile;
        if (tile >= ntiles) break;
        const int x0 = (tile % tiles_x) * kShadeTile, y0 = (tile / tiles_x) * kShadeTile;
        // ---- 1. coverage, compaction, box ----
        const int ly = t / 4, lx0 = (t % 4) * 8;
        const int y = y0 + ly;
        uint32_t cov = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int x = x0 + lx0 + j;
            if (x >= p.width || y >= p.height) continue;
            const int pi = y * p.width + x;
            if (p.albedo[pi] != 0u) cov |= 1u << j;
            else store_pixel(p, pi, p.background);
        }
        // the gate samples are the pixels (8i + 4, 8j + 4): j == 4 of rows with ly % 8 == 4
        const uint32_t smp = ((ly & 7) == 4) ? (cov & 0x10u) : 0u;
        const uint32_t oth = cov & ~smp;
        const int mine = (__popc(smp) << 16) | __popc(oth);
        int incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) S.scan[warp] = incl;
        if (t == 0) S.gate_sum = 0;
        __syncthreads();
        int before = incl - mine;
        for (int w = 0; w < warp; ++w) before += S.scan[w];
        const int total = (S.scan[0] + S.scan[1]) + (S.scan[2] + S.scan[3]);
        const int nsmp = total >> 16, ncov = nsmp + (total & 0xffff);
        int sp = before >> 16, op = nsmp + (before & 0xffff);
        float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (!((cov >> j) & 1u)) continue;
            const int slot = ((smp >> j) & 1u) ? sp++ : op++;
            const int x = x0 + lx0 + j;
            S.list[slot] = uint16_t(ly * kShadeTile + lx0 + j);
            float P[3];
            world_pos(p, x, y, p.depth[y * p.width + x], P);
            for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], P[k]); hi[k] = fmaxf(hi[k], P[k]); }
        }
        for (int k = 0; k < 3; ++k) {
            for (int o = 16; o > 0; o >>= 1) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
            }
            if (lane == 0) { S.box[0][warp][k] = lo[k]; S.box[1][warp][k] = hi[k]; }
        }
        __syncthreads();
        if (ncov == 0) {
            if (t == 0) {
                if (A.tile_status) A.tile_status[tile] = 2;
                if (A.tile_mse) A.tile_mse[tile] = 0.0f;
            }
            continue;   // every thread has read this tile's shared state
        }
        // ---- 2. candidate lights ----
        if (warp == 0) {
            float b0[3], b1[3];
            for (int k = 0; k < 3; ++k) {
                b0[k] = fminf(fminf(S.box[0][0][k], S.box[0][1][k]), fminf(S.box[0][2][k], S.box[0][3][k]));
                b1[k] = fmaxf(fmaxf(S.box[1][0][k], S.box[1][1][k]), fmaxf(S.box[1][2][k], S.box[1][3][k]));
            }
            select_candidates(nl, [&](int i) { return light_score(S.lights[i], b0, b1); }, S.cand);
        }
        // ---- 3. plain shading of the gate samples, 8 threads per sample ----
        const int ngate = ncov < kGateSamples ? ncov : kGateSamples;
        {
            const int sj = t >> 3, g = t & 7;
            float s[3] = { 0.0f, 0.0f, 0.0f }, a[3] = { 0.0f, 0.0f, 0.0f };
            if (sj < ngate) {
                const int li = S.list[sj];
                const int x = x0 + li % kShadeTile, yy = y0 + li / kShadeTile;
                const int pi = yy * p.width + x;
                float P[3], n[3], v[3], vlen;
                world_pos(p, x, yy, p.depth[pi], P);
                surface(p, P, p.nx[pi], p.ny[pi], p.nz[pi], n, v, vlen);
                albedo_rgb(p.albedo[pi], a);
                plain_sum(S.lights, g, 8, nl, P, n, v, a, s);
            }
            for (int o = 1; o < 8; o <<= 1)
                for (int c = 0; c < 3; ++c) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
            if (sj < ngate && g == 0)
                for (int c = 0; c < 3; ++c) S.gate_plain[sj][c] = s[c] + 0.03f * a[c];
        }
        __syncthreads();
        // ---- 4. MLP over the covered pixels, 128 at a time ----
        const int nbatch = (ncov + kRows - 1) / kRows;
        bool fallback = false;
        float tile_mse = 0.0f;
        for (int b = 0; b < nbatch; ++b) {
            const int r = b * kRows + t;
            int pi = -1;
            float base[3] = { 0.0f, 0.0f, 0.0f };
            {
                float f[kFeatures];
                uint32_t w[16];
                if (r < ncov) {
                    const int li = S.list[r];
                    const int x = x0 + li % kShadeTile, yy = y0 + li / kShadeTile;
                    pi = yy * p.width + x;
                    float P[3];
                    world_pos(p, x, yy, p.depth[pi], P);
                    pixel_features(p, S.lights, S.cand, P, p.nx[pi], p.ny[pi], p.nz[pi], p.albedo[pi], f);
                    virtual_light_base(f, base);
#pragma unroll
                    for (int q = 0; q < 12; ++q) w[q] = pack_bf16x2(f[2 * q], f[2 * q + 1]);
                    w[12] = one2;
                } else {
#pragma unroll
                    for (int q = 0; q < 13; ++q) w[q] = 0u;
                }
                w[13] = w[14] = w[15] = 0u;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    *reinterpret_cast<uint4*>(S.act + tc::kmajor_offset(t, 8 * j, kK1)) =
                        make_uint4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
            }
            float rgb[3] = { 0.0f, 0.0f, 0.0f };
            for (int layer = 0; layer < 4; ++layer) {
                tc::fence_smem_for_mma();
                tc::fence_before_sync();
                __syncthreads();
                if (t == 0) {
                    if (layer == 0) issue(tmem, S.act, S.w1, kK1, kHid, &S.mbar);
                    else issue(tmem, S.act, layer == 1 ? S.w2 : layer == 2 ? S.w3 : S.w4, kKH,
                               layer == 3 ? kOut : kHid, &S.mbar);
                }
                const bool ok = tc::mbar_wait(&S.mbar, phase);
                phase ^= 1u;
                if (__syncthreads_or(!ok)) { aborted = true; break; }
                tc::fence_after_sync();
                if (layer < 3) {
                    relu_epilogue(trow, S.act, t);
                    if (layer == 0) {
                        *reinterpret_cast<uint4*>(S.act + tc::kmajor_offset(t, 64, kKH)) = ones_row;
                        *reinterpret_cast<uint4*>(S.act + tc::kmajor_offset(t, 72, kKH)) = make_uint4(0u, 0u, 0u, 0u);
                    }
                } else {
                    uint32_t v[32];
                    tc::tmem_ld32_nowait(trow, v);
                    tc::tmem_wait_ld();
                    for (int c = 0; c < 3; ++c) {
                        const float q = pos0(__uint_as_float(v[c]) + base[c]);
                        rgb[c] = q * q;
                    }
                }
            }
            if (aborted) break;
            if (b == 0) {
                if (t < ngate) {
                    int e = 0;
                    for (int c = 0; c < 3; ++c) {
                        const int d = int(srgb8_lut(p.srgb_lut, rgb[c])) - int(srgb8_lut(p.srgb_lut, S.gate_plain[t][c]));
                        e += d * d;
                    }
                    atomicAdd(&S.gate_sum, e);
                }
                __syncthreads();
                tile_mse = float(S.gate_sum) / float(3 * ngate);
                if (tile_mse > A.max_tile_mse) { fallback = true; break; }
            }
            if (pi >= 0) store_pixel(p, pi, rgb);
        }
        if (aborted) break;
        if (fallback) {
            for (int r = t; r < ncov; r += blockDim.x) {
                const int li = S.list[r];
                const int x = x0 + li % kShadeTile, yy = y0 + li / kShadeTile;
                const int pi = yy * p.width + x;
                float rgb[3];
                plain_pixel(p, S.lights, nl, x, yy, p.depth[pi], p.nx[pi], p.ny[pi], p.nz[pi], p.albedo[pi], rgb);
                store_pixel(p, pi, rgb);
            }
        }
        if (t == 0) {
            if (A.tile_status) A.tile_status[tile] = fallback ? 1 : 0;
            if (A.tile_mse) A.tile_mse[tile] = tile_mse;
        }
        __syncthreads();
    }
    if (aborted && t == 0) atomicExch(A.error, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) { tc::fence_after_sync(); tc::tmem_dealloc(tmem, 64); }
}

size_t learned_smem_bytes(int nlights) {
    return sizeof(LearnSmem) + sizeof(rsrgpu_light) * size_t(nlights > 1 ? nlights - 1 : 0) + 128;
}

cudaError_t launch_shade_learned(const rsrgpu_mlp& w, const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                                 const rsrgpu_light* lights, int nlights, const float background[3], float max_tile_mse,
                                 uint32_t* out_srgb, float* out_linear, uint8_t* tile_status, float* tile_mse,
                                 const uint8_t* srgb_lut, int* error, int* tile_counter, int num_sms, cudaStream_t st) {
    LearnParams A{};
    PlainParams& p = A.pl;
    p.depth = gb.depth; p.nx = gb.normal_x; p.ny = gb.normal_y; p.nz = gb.normal_z; p.albedo = gb.albedo;
    p.width = gb.width; p.height = gb.height;
    for (int i = 0; i < 16; ++i) p.ivp[i] = ivp[i];
    for (int i = 0; i < 3; ++i) { p.eye[i] = eye[i]; p.background[i] = background[i]; }
    p.lights = lights; p.nlights = nlights; p.out_srgb = out_srgb; p.out_linear = out_linear; p.srgb_lut = srgb_lut;
    A.w = w; A.max_tile_mse = max_tile_mse; A.tile_status = tile_status; A.tile_mse = tile_mse; A.error = error;
    A.tile_counter = tile_counter;
    const size_t smem = learned_smem_bytes(nlights);
    cudaError_t e = cudaFuncSetAttribute(shade_learned_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(tile_counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    const int tiles = ((gb.width + kShadeTile - 1) / kShadeTile) * ((gb.height + kShadeTile - 1) / kShadeTile);
    // CTAs per SM: shared memory (227 KB per SM) and TMEM (512 columns, 64 per CTA)
    int per_sm = int((227u * 1024u) / (smem + 1024u));
    if (per_sm > 8) per_sm = 8;
    if (per_sm < 1) per_sm = 1;
    int grid = num_sms * per_sm;
    if (grid > tiles) grid = tiles;
    shade_learned_kernel<<<grid, 128, smem, st>>>(A);
    return cudaGetLastError();
}

}  // namespace rsrgpu
