// rsrgpu_learned.cu -- the learned deferred shader as one fused kernel.
//
// A persistent CTA of four warps takes one 32x32 shading tile at a time:
//   1. coverage of the tile's pixels, compacted into a list (the tile's 4x4
//      grid of gate sample pixels first), world positions of the covered
//      pixels and their box; background pixels are written at once
//   2. warp 0 picks the tile's candidate lights (rsrgpu_shading.cuh)
//   3. the gate's reference: the plain shader at the first min(16, covered)
//      listed pixels, each split over eight threads
//   4. for each 128 covered pixels: 24 features per pixel into a BF16 A tile
//      and the analytic base (virtual_light_base, FP32), the MLP's four
//      layers on tcgen05 (rsrgpu_mlp.cuh), output rgb = max(y + base, 0)^2
//      (the network predicts the residual of square roots of linear RGB);
//      after the first 128 the gate compares the learned and plain sRGB8
//      values of the samples and, when their mean squared error exceeds the
//      threshold, the tile is shaded by the plain shader instead (bit-exact
//      with rsrgpu_shade_plain), skipping the remaining MLP work
// Weights, biases and lights stay in shared memory for the CTA's lifetime.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_mlp.cuh"
#include "rsrgpu_shading.cuh"

namespace rsrgpu {

constexpr int kTilePx = kShadeTile * kShadeTile;   // 1024
constexpr int kGateSamples = 16;

struct LearnSmem {
    alignas(1024) uint8_t w1[kHid * kIn * 2];
    alignas(1024) uint8_t w2[kHid * kHid * 2];
    alignas(1024) uint8_t w3[kHid * kHid * 2];
    alignas(1024) uint8_t w4[kOut * kHid * 2];
    alignas(1024) uint8_t a0[kRows * kIn * 2];
    alignas(1024) uint8_t ah[kRows * kHid * 2];
    float b1[kHid], b2[kHid], b3[kHid], b4[kOut];
    rsrgpu_light lights[kMaxLights];
    float pos[kTilePx][3];           // world position of list entry i
    uint16_t list[kTilePx];          // covered pixels (tile-local index y * 32 + x)
    float box[2][4][3];
    int scan[4];
    int cand[kCandidates];
    float gate_plain[kGateSamples][3];
    int gate_sum;
    uint64_t mbar;
    uint32_t tmem;
};

struct LearnParams {
    PlainParams pl;
    rsrgpu_mlp w;
    float max_tile_mse;       // in 8-bit sRGB units squared
    uint8_t* tile_status;     // [tiles] or null: 0 learned, 1 plain fallback, 2 nothing covered
    float* tile_mse;          // [tiles] or null: the gate's estimate
    int* error;
};

__device__ __forceinline__ void store_pixel(const PlainParams& p, int pi, const float rgb[3]) {
    if (p.out_linear) { p.out_linear[3 * size_t(pi)] = rgb[0]; p.out_linear[3 * size_t(pi) + 1] = rgb[1]; p.out_linear[3 * size_t(pi) + 2] = rgb[2]; }
    if (p.out_srgb) p.out_srgb[pi] = pack_srgb(p.srgb_lut, rgb);
}

__global__ void __launch_bounds__(128) shade_learned_kernel(LearnParams A) {
    extern __shared__ uint8_t smem_raw[];
    LearnSmem& S = *reinterpret_cast<LearnSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const PlainParams& p = A.pl;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    load_kmajor(S.w1, A.w.w1, kHid, kIn);
    load_kmajor(S.w2, A.w.w2, kHid, kHid);
    load_kmajor(S.w3, A.w.w3, kHid, kHid);
    load_kmajor(S.w4, A.w.w4, kOut, kHid);
    for (int i = t; i < kHid; i += blockDim.x) { S.b1[i] = A.w.b1[i]; S.b2[i] = A.w.b2[i]; S.b3[i] = A.w.b3[i]; }
    if (t < kOut) S.b4[t] = A.w.b4[t];
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

    const int tiles_x = (p.width + kShadeTile - 1) / kShadeTile, tiles_y = (p.height + kShadeTile - 1) / kShadeTile;
    for (int tile = blockIdx.x; tile < tiles_x * tiles_y && !aborted; tile += gridDim.x) {
        const int x0 = (tile % tiles_x) * kShadeTile, y0 = (tile / tiles_x) * kShadeTile;
        // ---- 1. coverage, compaction, world positions ----
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
            S.pos[slot][0] = P[0]; S.pos[slot][1] = P[1]; S.pos[slot][2] = P[2];
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
            continue;   // no shared state of this tile is read after this point
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
                const int pi = (y0 + li / kShadeTile) * p.width + x0 + li % kShadeTile;
                float n[3], v[3], vlen;
                surface(p, S.pos[sj], p.nx[pi], p.ny[pi], p.nz[pi], n, v, vlen);
                albedo_rgb(p.albedo[pi], a);
                plain_sum(S.lights, g, 8, nl, S.pos[sj], n, v, a, s);
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
                float f[32];
                if (r < ncov) {
                    const int li = S.list[r];
                    pi = (y0 + li / kShadeTile) * p.width + x0 + li % kShadeTile;
                    pixel_features(p, S.lights, S.cand, S.pos[r], p.nx[pi], p.ny[pi], p.nz[pi], p.albedo[pi], f);
                    virtual_light_base(f, base);
                    for (int q = kFeatures; q < 32; ++q) f[q] = 0.0f;
                } else {
                    for (int q = 0; q < 32; ++q) f[q] = 0.0f;
                }
#pragma unroll
                for (int j = 0; j < kIn; j += 8) {
                    uint4 pk;
                    pk.x = pack_bf16x2(f[j], f[j + 1]); pk.y = pack_bf16x2(f[j + 2], f[j + 3]);
                    pk.z = pack_bf16x2(f[j + 4], f[j + 5]); pk.w = pack_bf16x2(f[j + 6], f[j + 7]);
                    *reinterpret_cast<uint4*>(S.a0 + tc::kmajor_offset(t, j, kIn)) = pk;
                }
            }
            const uint8_t* a_in = S.a0;
            int k_in = kIn;
            const uint8_t* wl[4] = { S.w1, S.w2, S.w3, S.w4 };
            const float* bl[3] = { S.b1, S.b2, S.b3 };
            float rgb[3] = { 0.0f, 0.0f, 0.0f };
            for (int layer = 0; layer < 4; ++layer) {
                tc::fence_smem_for_mma();
                tc::fence_before_sync();
                __syncthreads();
                if (t == 0) issue_layer(tmem, a_in, wl[layer], k_in, layer == 3 ? kOut : kHid, &S.mbar);
                const bool ok = tc::mbar_wait(&S.mbar, phase);
                phase ^= 1u;
                if (__syncthreads_or(!ok)) { aborted = true; break; }
                tc::fence_after_sync();
                if (layer < 3) {
                    hidden_epilogue(trow, bl[layer], S.ah, t);
                    a_in = S.ah;
                    k_in = kHid;
                } else {
                    float v[16];
                    tc::tmem_ld16(trow, v);
                    for (int c = 0; c < 3; ++c) {
                        const float q = pos0((v[c] + S.b4[c]) + base[c]);
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

size_t learned_smem_bytes() { return sizeof(LearnSmem) + 1024; }

cudaError_t launch_shade_learned(const rsrgpu_mlp& w, const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                                 const rsrgpu_light* lights, int nlights, const float background[3], float max_tile_mse,
                                 uint32_t* out_srgb, float* out_linear, uint8_t* tile_status, float* tile_mse,
                                 const uint8_t* srgb_lut, int* error, int num_sms, cudaStream_t st) {
    LearnParams A{};
    PlainParams& p = A.pl;
    p.depth = gb.depth; p.nx = gb.normal_x; p.ny = gb.normal_y; p.nz = gb.normal_z; p.albedo = gb.albedo;
    p.width = gb.width; p.height = gb.height;
    for (int i = 0; i < 16; ++i) p.ivp[i] = ivp[i];
    for (int i = 0; i < 3; ++i) { p.eye[i] = eye[i]; p.background[i] = background[i]; }
    p.lights = lights; p.nlights = nlights; p.out_srgb = out_srgb; p.out_linear = out_linear; p.srgb_lut = srgb_lut;
    A.w = w; A.max_tile_mse = max_tile_mse; A.tile_status = tile_status; A.tile_mse = tile_mse; A.error = error;
    const size_t smem = learned_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(shade_learned_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const int tiles = ((gb.width + kShadeTile - 1) / kShadeTile) * ((gb.height + kShadeTile - 1) / kShadeTile);
    int per_sm = int((227u * 1024u) / smem);
    if (per_sm < 1) per_sm = 1;
    int grid = num_sms * per_sm;
    if (grid > tiles) grid = tiles;
    shade_learned_kernel<<<grid, 128, smem, st>>>(A);
    return cudaGetLastError();
}

}  // namespace rsrgpu
