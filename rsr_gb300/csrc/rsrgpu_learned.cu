// rsrgpu_learned.cu -- the learned deferred shader: a per-tile SIMT pre-pass,
// a persistent tensor-core kernel fed by bulk copies, and a fallback pass.
//
// The shader's output is rgb = max(y + base, 0)^2 per channel, base the
// square root of the analytic virtual-light estimate and y the network's
// residual.  A pixel reached by at most one of its tile's candidate lights
// needs no network: its virtual light is that light, so base is its
// Blinn-Phong shading; only pixels reached by two or more go through the MLP.
//
// learned_prep_kernel (four CTAs of 256 threads per SM, so that their latency
// chains overlap, each taking 32x32 shading tiles in turn): coverage and
// compaction (the tile's 4x4 grid of gate samples first), the world-space box
// of the covered pixels, the candidate lights, the plain shader at the gate
// samples (8 threads per sample), background pixels; then, list entry
// i * 256 + t per pass, the features and base of every covered pixel: pixels
// on the exact path are written at once, the others are compacted (ballot,
// list order) into the tile's blocks of 128 rows -- an 8 KB A tile per block
// (24 BF16 features and two ones columns per row, in the chunked layout
// below) and a PipeMeta record (base, pixel index, gate samples) -- and the
// tile's blocks are appended to a block list.
//
// shade_learned_kernel (one CTA per SM): two lanes, each a producer thread
//   and a consumer warpgroup joined by three pipelines.  The producer takes
//   its lane's share of the block list (every 2 * gridDim.x-th entry) and,
//   for each block, waits for the next pipeline's slot
//   to be free and issues two bulk copies (cp.async.bulk) of the block's A
//   tile and record into it, completed on the pipeline's full barrier by
//   transaction count.  The consumer visits its pipelines in turn and
//   advances each by one step: issue layer 1 from a full slot (the block's
//   record goes to registers), or, when the pipeline's MMAs have completed,
//   run the epilogue (TMEM -> ReLU -> BF16 into the pipeline's activation
//   tile) and issue the next layer -- after layer 1 the slot goes back to the
//   producer, whose copy of the next block overlaps layers 2-4 -- or after
//   layer 4 write rgb; while one pipeline's MMAs run the warpgroup serves the
//   other two.
// The gate: the mean squared difference of learned and plain sRGB8 values
// over the tile's samples -- those on the exact path are scored in the
// pre-pass (which decides alone when all are), the others after layer 4 of
// the tile's first block.  Rejected tiles go to a list; shade_fallback_kernel
// shades them with the plain shader afterwards (bit-exact with
// rsrgpu_shade_plain).  The three kernels are chained by programmatic
// dependent launch.
//
// A tiles use a chunked K-major layout: chunk j (8 columns) of all 128 rows
// is 2 KB, row r at j * 2048 + (r / 8) * 128 + (r % 8) * 16 (descriptor LBO
// 2048, SBO 128).  Layer 1 reads the 8 KB slot (features, ones at columns
// 24-25), the hidden layers the pipeline's 20 KB activation tile
// (activations, ones at 64-65, zeros); the biases ride in the weights as a
// BF16 high/low pair, so the epilogue is one cvt.rn.relu.bf16x2 per two
// activations.  Six pipelines x 64 TMEM columns.  Every wait is bounded; on
// expiry the kernel raises the error flag and winds down.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_mlp.cuh"
#include "rsrgpu_shading.cuh"

namespace rsrgpu {

constexpr int kTilePx = kShadeTile * kShadeTile;   // 1024
constexpr int kGateSamples = 16;
constexpr int kK1 = 32;                 // layer-1 K: 24 features, ones at 24/25, zeros
constexpr int kKH = 80;                 // hidden-layer K: 64 activations, ones at 64/65, zeros
constexpr int kLanes = 2;               // producer/consumer pairs per CTA
constexpr int kPipes = 3;               // pipelines per lane
constexpr int kChunk = kRows * 16;      // one 8-column chunk of a 128-row tile
constexpr int kTileBytes = kChunk * (kKH / 8);
constexpr int kFeatBytes = kChunk * (kK1 / 8);     // the A tile of layer 1: 8 KB
constexpr int kBlocksPerTile = kTilePx / kRows;    // 8
constexpr int kThreads = 320;           // 2 consumer warpgroups + 2 producer warps

struct PipeMeta {
    float base[kRows][3];
    int32_t pix[kRows];                 // pixel index, -1: row unused
    uint32_t gate_plain[kGateSamples];  // plain shader at the gate samples among the rows, packed sRGB8
    int32_t tile;                       // -1: no more work
    int32_t first;                      // the tile's first block (its first rows are gate samples)
    int32_t ngate;                      // gate samples among this block's rows
    int32_t ngate_total;                // the tile's gate samples
    int32_t gate_err;                   // squared sRGB8 error of the samples shaded in the pre-pass
    int32_t pad[3];
};
static_assert(sizeof(PipeMeta) % 16 == 0, "bulk copies move multiples of 16 bytes");

// tile t's blocks live at t * 8 .. t * 8 + 7 of the block arrays; the
// pre-pass appends the index of every block it fills to a block list

struct LearnSmem {
    alignas(128) uint8_t act[kLanes * kPipes][kTileBytes];     // hidden-layer A tiles
    alignas(128) uint8_t feat[kLanes * kPipes][kFeatBytes];    // layer-1 A tiles (bulk-copied)
    alignas(128) uint8_t w1[kHid * kK1 * 2];
    alignas(128) uint8_t w2[kHid * kKH * 2];
    alignas(128) uint8_t w3[kHid * kKH * 2];
    alignas(128) uint8_t w4[kOut * kKH * 2];
    alignas(16) PipeMeta meta[kLanes * kPipes];
    uint64_t full[kLanes * kPipes], empty[kLanes * kPipes], mma[kLanes * kPipes];
    int gate_sum[kLanes];
    uint32_t tmem;
    int abort;
};

struct LearnParams {
    PlainParams pl;
    rsrgpu_mlp w;
    float max_tile_mse;       // in 8-bit sRGB units squared
    uint8_t* tile_status;     // [tiles]: 0 learned, 1 plain fallback, 2 nothing covered
    float* tile_mse;          // [tiles] or null: the gate's estimate
    int* error;
    int* counters;            // [0] tiles taken by the pre-pass, [1] blocks listed, [2] tiles
                              // rejected by the gate; zero at launch
    int32_t* blocks;          // [tiles * 8] the filled blocks
    int32_t* rejected;        // [tiles] tiles for the fallback pass
    uint8_t* feat;            // [tiles * 8][8 KB] A tiles
    PipeMeta* metas;          // [tiles * 8]
    uint32_t poll_limit;      // polls of a pipeline wait before it gives up
    int32_t stall;            // test hook: the producers issue nothing, so the waits run out
};

__device__ __forceinline__ void store_pixel(const PlainParams& p, int pi, const float rgb[3]) {
    if (p.out_linear) { p.out_linear[3 * size_t(pi)] = rgb[0]; p.out_linear[3 * size_t(pi) + 1] = rgb[1]; p.out_linear[3 * size_t(pi) + 2] = rgb[2]; }
    if (p.out_srgb) p.out_srgb[pi] = pack_srgb(p.srgb_lut, rgb);
}

__device__ __forceinline__ uint16_t bf16_rn(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }

// row r, columns 8j..8j+7 of a chunked 128-row tile
__device__ __forceinline__ uint4* chunk_row(uint8_t* tile, int j, int r) {
    return reinterpret_cast<uint4*>(tile + j * kChunk + (r >> 3) * 128 + (r & 7) * 16);
}

// ---------------------------------------------------------------- pre-pass
constexpr int kPrepThreads = 256;   // per 32x32 tile: four pixels of a row per thread
constexpr int kPrepWarps = kPrepThreads / 32;
constexpr int kPrepPx = kTilePx / kPrepThreads;
static_assert(kPrepPx == 4, "the coverage loads move four pixels as one vector");

__global__ void __launch_bounds__(kPrepThreads, 4) learned_prep_kernel(LearnParams A) {
    extern __shared__ rsrgpu_light L[];
    __shared__ uint16_t list[kTilePx];
    __shared__ float box[2][kPrepWarps][3];
    __shared__ int scan[kPrepWarps];
    __shared__ int cand[kCandidates];
    __shared__ float scores[kMaxLights];
    __shared__ uint32_t gate_plain[kGateSamples];
    __shared__ int gate_err, netsamples;
    __shared__ int wcount[2][kPrepWarps];
    const PlainParams& p = A.pl;
    const int t = threadIdx.x, wl = t & 31, warp = t >> 5;
    // the tensor-core kernel may take the SMs this grid's CTAs leave: once
    // every CTA of this grid has started, its prologue overlaps their work
    // (it reads nothing of theirs before its griddepcontrol.wait)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    load_lights(L, p.lights, nl);
    const int tiles_x = (p.width + kShadeTile - 1) / kShadeTile;
    const int ntiles = tiles_x * ((p.height + kShadeTile - 1) / kShadeTile);
    __shared__ int next_tile;
    // tiles in turn from a counter: no CTA launch per tile, and the tiles
    // with nothing covered cost little
    for (;;) {
        if (t == 0) next_tile = atomicAdd(A.counters, 1);
        __syncthreads();   // also: the previous tile's shared state is no longer read
        const int tile = next_tile;
        if (tile >= ntiles) break;
        const int x0 = (tile % tiles_x) * kShadeTile, y0 = (tile / tiles_x) * kShadeTile;
        // ---- coverage, compaction (gate samples first), box ----
        const int ly = t / (kShadeTile / kPrepPx), lx0 = (t % (kShadeTile / kPrepPx)) * kPrepPx;
        const int y = y0 + ly;
        const uint32_t bg = pack_srgb(p.srgb_lut, p.background);
        uint32_t cov = 0;
        float zd[kPrepPx];
        uint32_t alb[kPrepPx];
        // every load of the thread's four pixels before any is used: one round
        // trip to memory (a branch on each albedo would make it four)
        const int row = y * p.width + x0 + lx0;
        const bool full = y < p.height && x0 + lx0 + kPrepPx <= p.width && (row % 4) == 0 &&
                          ((reinterpret_cast<uintptr_t>(p.depth) | reinterpret_cast<uintptr_t>(p.albedo)) & 15u) == 0;
        if (full) {
            const float4 z4 = *reinterpret_cast<const float4*>(p.depth + row);
            const uint4 a4 = *reinterpret_cast<const uint4*>(p.albedo + row);
            zd[0] = z4.x; zd[1] = z4.y; zd[2] = z4.z; zd[3] = z4.w;
            alb[0] = a4.x; alb[1] = a4.y; alb[2] = a4.z; alb[3] = a4.w;
        } else {
#pragma unroll
            for (int j = 0; j < kPrepPx; ++j) {
                const bool in = y < p.height && x0 + lx0 + j < p.width;
                zd[j] = in ? p.depth[row + j] : 1.0f;
                alb[j] = in ? p.albedo[row + j] : 0u;
            }
        }
#pragma unroll
        for (int j = 0; j < kPrepPx; ++j) {
            if (y >= p.height || x0 + lx0 + j >= p.width) continue;
            if (alb[j] != 0u) {
                cov |= 1u << j;
            } else {
                const int pi = row + j;
                if (p.out_srgb) p.out_srgb[pi] = bg;
                if (p.out_linear) { p.out_linear[3 * size_t(pi)] = p.background[0]; p.out_linear[3 * size_t(pi) + 1] = p.background[1]; p.out_linear[3 * size_t(pi) + 2] = p.background[2]; }
            }
        }
        // gate samples: the pixels (8i + 4, 8j + 4), here the first of every other thread's four
        const uint32_t smp = ((ly & 7) == 4 && (lx0 & 7) == 4) ? (cov & 1u) : 0u;
        const int mine = (__popc(smp) << 16) | __popc(cov & ~smp);
        int incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (wl >= o) incl += v;
        }
        if (wl == 31) scan[warp] = incl;
        __syncthreads();
        int before = incl - mine;
        int total = 0;
        for (int w = 0; w < kPrepWarps; ++w) {
            if (w == warp) before += total;
            total += scan[w];
        }
        const int nsmp = total >> 16, ncov = nsmp + (total & 0xffff);
        int sp = before >> 16, op = nsmp + (before & 0xffff);
        float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
#pragma unroll
        for (int j = 0; j < kPrepPx; ++j) {
            if (!((cov >> j) & 1u)) continue;
            const int slot = ((smp >> j) & 1u) ? sp++ : op++;
            const int x = x0 + lx0 + j;
            list[slot] = uint16_t(ly * kShadeTile + lx0 + j);
            float Q[3];
            world_pos(p, x, y, zd[j], Q);
            for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], Q[k]); hi[k] = fmaxf(hi[k], Q[k]); }
        }
        for (int k = 0; k < 3; ++k) {
            for (int o = 16; o > 0; o >>= 1) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
            }
            if (wl == 0) { box[0][warp][k] = lo[k]; box[1][warp][k] = hi[k]; }
        }
        __syncthreads();
        if (ncov == 0) {
            if (t == 0) {
                A.tile_status[tile] = 2;
                if (A.tile_mse) A.tile_mse[tile] = 0.0f;
            }
            continue;
        }
        // ---- candidate lights (warp 0), gate samples (8 threads each) ----
        if (warp == 0) {
            float b0[3], b1[3];
            for (int k = 0; k < 3; ++k) {
                b0[k] = box[0][0][k]; b1[k] = box[1][0][k];
                for (int w = 1; w < kPrepWarps; ++w) { b0[k] = fminf(b0[k], box[0][w][k]); b1[k] = fmaxf(b1[k], box[1][w][k]); }
            }
            select_candidates(nl, [&](int i) { return light_score(L[i], b0, b1); }, cand, scores);
        }
        const int ngate = ncov < kGateSamples ? ncov : kGateSamples;
        if (t >= 32 && t < 32 + 8 * kGateSamples) {   // warps 1-4, beside warp 0's choice
            const int sj = (t - 32) >> 3, g = t & 7;
            float s[3] = { 0.0f, 0.0f, 0.0f }, a[3] = { 0.0f, 0.0f, 0.0f };
            if (sj < ngate) {
                const int li = list[sj];
                const int x = x0 + li % kShadeTile, yy = y0 + li / kShadeTile;
                const int pi = yy * p.width + x;
                float Q[3], n[3], v[3];
                world_pos_fast(p, x, yy, p.depth[pi], Q);
                surface_fast(p, Q, p.nx[pi], p.ny[pi], p.nz[pi], n, v);
                albedo_rgb(p.albedo[pi], a);
                plain_sum_fast(L, g, 8, nl, Q, n, v, a, s);
            }
            for (int o = 1; o < 8; o <<= 1)
                for (int c = 0; c < 3; ++c) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
            if (sj < ngate && g == 0) {
                const float rgb[3] = { s[0] + 0.03f * a[0], s[1] + 0.03f * a[1], s[2] + 0.03f * a[2] };
                gate_plain[sj] = pack_srgb(p.srgb_lut, rgb);
            }
        }
        __syncthreads();
        // ---- features; pixels reached by two or more candidate lights become the
        // network's rows (in list order, so the gate samples come first), the
        // others take the analytic base, which is then their Blinn-Phong shading.
        // Entry i * 256 + t per pass: consecutive threads, consecutive pixels. ----
        if (t == 0) { gate_err = 0; netsamples = 0; }
        const uint32_t one2 = uint32_t(bf16_rn(1.0f)) | (uint32_t(bf16_rn(1.0f)) << 16);
        const uint32_t lt = (1u << wl) - 1u;
        int nrows = 0;
        __syncthreads();
        // G-buffer values of this thread's next list entry, fetched a pass ahead
        struct Px { int pi; float z; uint16_t hx, hy, hz; uint32_t alb; };
        auto fetch = [&](int r, Px& q) {
            if (r >= ncov) return;
            const int li = list[r];
            q.pi = (y0 + li / kShadeTile) * p.width + x0 + li % kShadeTile;
            q.z = p.depth[q.pi]; q.hx = p.nx[q.pi]; q.hy = p.ny[q.pi]; q.hz = p.nz[q.pi]; q.alb = p.albedo[q.pi];
        };
        Px nxt{ 0, 0.0f, 0, 0, 0, 0u };
        fetch(t, nxt);
        for (int i = 0; i * kPrepThreads < ncov; ++i) {
            const int r = i * kPrepThreads + t;
            const Px cur = nxt;
            fetch(r + kPrepThreads, nxt);
            bool net = false;
            const int pi = cur.pi;
            float f[kFeatures], base[3];
            if (r < ncov) {
                const int x = pi % p.width, yy = pi / p.width;
                float Q[3];
                world_pos_fast(p, x, yy, cur.z, Q);
                net = pixel_features_fast(p, L, cand, Q, cur.hx, cur.hy, cur.hz, cur.alb, f, base) >= 2;
                if (!net) {
                    const float rgb[3] = { base[0] * base[0], base[1] * base[1], base[2] * base[2] };
                    store_pixel(p, pi, rgb);
                    if (r < ngate) {
                        int err = 0;
                        for (int c = 0; c < 3; ++c) {
                            const int d = int(srgb8_lut(p.srgb_lut, rgb[c])) - int((gate_plain[r] >> (16 - 8 * c)) & 255u);
                            err += d * d;
                        }
                        atomicAdd(&gate_err, err);
                    }
                }
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, net);
            if (wl == 0) wcount[i & 1][warp] = __popc(bal);
            __syncthreads();
            int slot = nrows + __popc(bal & lt);
            for (int w = 0; w < kPrepWarps; ++w) {
                if (w < warp) slot += wcount[i & 1][w];
                nrows += wcount[i & 1][w];
            }
            if (net) {
                const int blk = tile * kBlocksPerTile + slot / kRows, row = slot % kRows;
                uint8_t* ftile = A.feat + size_t(blk) * kFeatBytes;
                PipeMeta& M = A.metas[blk];
                uint32_t w[16];
#pragma unroll
                for (int q = 0; q < 12; ++q) w[q] = pack_bf16x2(f[2 * q], f[2 * q + 1]);
                w[12] = one2;
                w[13] = w[14] = w[15] = 0u;
#pragma unroll
                for (int j = 0; j < 4; ++j) *chunk_row(ftile, j, row) = make_uint4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
                M.base[row][0] = base[0]; M.base[row][1] = base[1]; M.base[row][2] = base[2];
                M.pix[row] = pi;
                if (r < ngate) { M.gate_plain[slot] = gate_plain[r]; atomicAdd(&netsamples, 1); }
            }
        }
        const int nblocks = (nrows + kRows - 1) / kRows;
        // rows of the last block past the network's pixels
        for (int sidx = nrows + t; sidx < nblocks * kRows; sidx += blockDim.x) {
            const int blk = tile * kBlocksPerTile + sidx / kRows, row = sidx % kRows;
            uint8_t* ftile = A.feat + size_t(blk) * kFeatBytes;
#pragma unroll
            for (int j = 0; j < 4; ++j) *chunk_row(ftile, j, row) = make_uint4(0u, 0u, 0u, 0u);
            PipeMeta& M = A.metas[blk];
            M.base[row][0] = M.base[row][1] = M.base[row][2] = 0.0f;
            M.pix[row] = -1;
        }
        __syncthreads();
        if (t < nblocks) {
            PipeMeta& M = A.metas[tile * kBlocksPerTile + t];
            M.tile = tile;
            M.first = t == 0;
            M.ngate = t == 0 ? netsamples : 0;
            M.ngate_total = ngate;
            M.gate_err = gate_err;
            M.pad[0] = M.pad[1] = M.pad[2] = 0;
        }
        if (t == 0) {
            if (nblocks == 0) {   // every sample on the exact path: the gate decides here
                const float mse = float(gate_err) / float(3 * ngate);
                const int fb = mse > A.max_tile_mse ? 1 : 0;
                A.tile_status[tile] = uint8_t(fb);
                if (A.tile_mse) A.tile_mse[tile] = mse;
                if (fb) A.rejected[atomicAdd(A.counters + 2, 1)] = tile;
            } else {
                const int at = atomicAdd(A.counters + 1, nblocks);
                for (int b = 0; b < nblocks; ++b) A.blocks[at + b] = tile * kBlocksPerTile + b;
            }
        }
    }
}

// ---------------------------------------------------------------- tensor-core kernel
// Chunk c (16 bytes) of the four weight matrices, in order w1 | w2 | w3 | w4,
// each in the row-wise K-major layout (LBO 128, SBO KDIM/8 * 128): columns
// 8j..8j+7 of W (the first KSRC columns of a row-major [rows][LD] bf16
// matrix), the bias as columns KSRC (high) and KSRC+1 (low), zeros to KDIM.
// Returns the chunk and sets its shared-memory destination.
__device__ __forceinline__ uint4 weight_chunk(const rsrgpu_mlp& w, uint8_t* w1, uint8_t* w2, uint8_t* w3, uint8_t* w4,
                                              int c, uint8_t*& dst) {
    constexpr int c1 = kHid * (kK1 / 8), c2 = kHid * (kKH / 8);
    const uint16_t* W;
    const float* B;
    int kdim, ksrc, ld;
    if (c < c1) { W = w.w1; B = w.b1; dst = w1; kdim = kK1; ksrc = kFeatures; ld = kIn; }
    else if (c < c1 + c2) { c -= c1; W = w.w2; B = w.b2; dst = w2; kdim = kKH; ksrc = kHid; ld = kHid; }
    else if (c < c1 + 2 * c2) { c -= c1 + c2; W = w.w3; B = w.b3; dst = w3; kdim = kKH; ksrc = kHid; ld = kHid; }
    else { c -= c1 + 2 * c2; W = w.w4; B = w.b4; dst = w4; kdim = kKH; ksrc = kHid; ld = kHid; }
    const int r = c / (kdim / 8), j = c % (kdim / 8);
    dst += tc::kmajor_offset(r, j * 8, kdim);
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (j < ksrc / 8) {
        v = __ldg(reinterpret_cast<const uint4*>(W + r * ld + j * 8));
    } else if (j == ksrc / 8) {
        const float b = __ldg(B + r);
        const uint16_t hi = bf16_rn(b);
        const uint16_t lo = bf16_rn(b - __bfloat162float(__ushort_as_bfloat16(hi)));
        v.x = uint32_t(hi) | (uint32_t(lo) << 16);
    }
    return v;
}

// All four weight matrices into shared memory: every thread issues its loads
// (at most kPer chunks) before it stores any, so the prologue waits for one
// round trip to memory rather than one per chunk.
__device__ __forceinline__ void load_weights(const rsrgpu_mlp& w, uint8_t* w1, uint8_t* w2, uint8_t* w3, uint8_t* w4) {
    constexpr int total = kHid * (kK1 / 8) + 2 * kHid * (kKH / 8) + kOut * (kKH / 8);
    constexpr int kPer = (total + kThreads - 1) / kThreads;
    uint4 v[kPer];
    uint8_t* dst[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int c = int(threadIdx.x) + k * kThreads;
        dst[k] = nullptr;
        if (c < total) v[k] = weight_chunk(w, w1, w2, w3, w4, c, dst[k]);
    }
#pragma unroll
    for (int k = 0; k < kPer; ++k)
        if (dst[k] != nullptr) *reinterpret_cast<uint4*>(dst[k]) = v[k];
}

// D[128 x n] = A (chunked, K = kdim) * W (n x kdim, row-wise K-major)^T, committed to mbar
__device__ __forceinline__ void issue(uint32_t d, const uint8_t* a, const uint8_t* w, int kdim, int n, uint64_t* mbar) {
    tc::fence_after_sync();
    const uint32_t sa = tc::smem_addr(a), sw = tc::smem_addr(w);
    const uint32_t wsbo = uint32_t(kdim / 8) * 128u;
    for (int ks = 0; ks < kdim / 16; ++ks)
        tc::mma_bf16(d, tc::smem_desc(sa + ks * 2u * kChunk, kChunk, 128u), tc::smem_desc(sw + ks * 256u, 128u, wsbo),
                     tc::idesc_bf16(kRows, n), ks > 0 ? 1u : 0u);
    tc::mma_commit(mbar);
}

// bounded wait that also gives up when the CTA is winding down
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        if (tc::mbar_try_wait(bar, parity)) return true;
        if ((i & 255u) == 255u && *abort) return false;
        if (i > 64) __nanosleep(32);
    }
    *abort = 1;
    return false;
}

// one thread per lane: blocks from the list into the lane's pipelines.  Lane
// l of CTA c takes list entries c * kLanes + l, + gridDim.x * kLanes, ...: an
// equal share for every lane, also for CTAs that start late (on SMs the
// pre-pass still held), where taking blocks first-come would leave them none.
__device__ void produce(LearnSmem& S, const LearnParams& A, int lane) {
    volatile int* abort = &S.abort;
    if (A.stall) return;   // nothing issued: the consumers' waits run out with no copy or MMA in flight
    uint32_t eparity = 0xfu;   // per pipeline: the parity to wait for on its empty barrier (fresh: passes)
    int pipe = 0;
    const int nblocks = *reinterpret_cast<volatile int*>(A.counters + 1);
    const int stride = int(gridDim.x) * kLanes;
    for (int k = int(blockIdx.x) * kLanes + lane; k < nblocks && !*abort; k += stride) {
        const int blk = A.blocks[k];
        const int pp = lane * kPipes + pipe;
        if (!wait_or_abort(&S.empty[pp], (eparity >> pipe) & 1u, abort, A.poll_limit)) break;
        eparity ^= 1u << pipe;
        tc::mbar_arrive_expect_tx(&S.full[pp], uint32_t(kFeatBytes + sizeof(PipeMeta)));
        tc::bulk_g2s(S.feat[pp], A.feat + size_t(blk) * kFeatBytes, kFeatBytes, &S.full[pp]);
        tc::bulk_g2s(&S.meta[pp], A.metas + blk, uint32_t(sizeof(PipeMeta)), &S.full[pp]);
        pipe = (pipe + 1) % kPipes;
    }
    // end of work: one sentinel per pipeline
    for (int k = 0; k < kPipes && !*abort; ++k) {
        const int pp = lane * kPipes + pipe;
        if (!wait_or_abort(&S.empty[pp], (eparity >> pipe) & 1u, abort, A.poll_limit)) break;
        eparity ^= 1u << pipe;
        S.meta[pp].tile = -1;
        tc::mbar_arrive(&S.full[pp]);
        pipe = (pipe + 1) % kPipes;
    }
}

// Per pipeline: wait for a full slot, keep the block's record in registers
// and issue layer 1 from the slot; when layer 1 has completed the slot is
// handed back to the producer (it refills it while layers 2-4 run) and the
// epilogues pass the activations through the pipeline's own A tile.
struct BlockRegs {
    int stage;          // 0 wait for a full slot, 1..4 layer in flight, 5 finished
    int pix, tile, first, ngate, ngate_total, gate_err;
    float base[3];
    uint32_t gate;      // thread t < 16: the plain value of sample t
};

__device__ __forceinline__ void consume_step(LearnSmem& S, const LearnParams& A, int lane, int pipe, BlockRegs& B,
                                             uint32_t& fparity, uint32_t& mparity, int& done) {
    const PlainParams& p = A.pl;
    const int t = threadIdx.x & 127, warp = (threadIdx.x >> 5) & 3;
    const int bar = 1 + lane;
    volatile int* abort = &S.abort;
    const int pp = lane * kPipes + pipe;
    const uint32_t dcol = S.tmem + uint32_t(64 * pp);
    const uint32_t trow = dcol + (uint32_t(warp * 32) << 16);
    uint8_t* tileb = S.act[pp];
    if (B.stage == 0) {
        if (!wait_or_abort(&S.full[pp], (fparity >> pipe) & 1u, abort, A.poll_limit)) return;
        fparity ^= 1u << pipe;
        const PipeMeta& M = S.meta[pp];
        B.tile = M.tile;
        if (B.tile < 0) { B.stage = 5; ++done; return; }
        B.pix = M.pix[t];
        B.base[0] = M.base[t][0]; B.base[1] = M.base[t][1]; B.base[2] = M.base[t][2];
        B.first = M.first; B.ngate = M.ngate; B.ngate_total = M.ngate_total; B.gate_err = M.gate_err;
        B.gate = t < kGateSamples ? M.gate_plain[t] : 0u;
        if (t == 0) issue(dcol, S.feat[pp], S.w1, kK1, kHid, &S.mma[pp]);
        B.stage = 1;
        return;
    }
    if (!wait_or_abort(&S.mma[pp], (mparity >> pipe) & 1u, abort, A.poll_limit)) return;
    mparity ^= 1u << pipe;
    tc::fence_after_sync();
    if (B.stage < 4) {
        uint32_t r[64];
        tc::tmem_ld32_nowait(trow, r);
        tc::tmem_ld32_nowait(trow + 32, r + 32);
        tc::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j)
            *chunk_row(tileb, j, t) = make_uint4(tc::relu_bf16x2(r[8 * j], r[8 * j + 1]), tc::relu_bf16x2(r[8 * j + 2], r[8 * j + 3]),
                                                 tc::relu_bf16x2(r[8 * j + 4], r[8 * j + 5]), tc::relu_bf16x2(r[8 * j + 6], r[8 * j + 7]));
        tc::fence_smem_for_mma();
        tc::fence_before_sync();
        tc::wg_sync(bar);
        if (t == 0) {
            // layer 1 has read the slot and every thread has its record: the producer may refill it
            if (B.stage == 1) tc::mbar_arrive(&S.empty[pp]);
            issue(dcol, tileb, B.stage == 1 ? S.w2 : B.stage == 2 ? S.w3 : S.w4, kKH, B.stage == 3 ? kOut : kHid, &S.mma[pp]);
        }
        B.stage += 1;
        return;
    }
    // ---- layer 4 done: output ----
    uint32_t v[32];
    tc::tmem_ld32_nowait(trow, v);
    tc::tmem_wait_ld();
    float rgb[3];
    for (int c = 0; c < 3; ++c) {
        const float q = pos0(__uint_as_float(v[c]) + B.base[c]);
        rgb[c] = q * q;
    }
    if (B.first) {
        if (t == 0) S.gate_sum[lane] = B.gate_err;   // the samples shaded in the pre-pass
        tc::wg_sync(bar);
        if (t < B.ngate) {
            int e = 0;
            for (int c = 0; c < 3; ++c) {
                const int d = int(srgb8_lut(p.srgb_lut, rgb[c])) - int((B.gate >> (16 - 8 * c)) & 255u);
                e += d * d;
            }
            atomicAdd(&S.gate_sum[lane], e);
        }
        tc::wg_sync(bar);
        const float mse = float(S.gate_sum[lane]) / float(3 * B.ngate_total);
        const int fb = mse > A.max_tile_mse ? 1 : 0;
        if (t == 0) {
            A.tile_status[B.tile] = uint8_t(fb);
            if (A.tile_mse) A.tile_mse[B.tile] = mse;
            if (fb) A.rejected[atomicAdd(A.counters + 2, 1)] = B.tile;
        }
    }
    // pixels of tiles the gate rejects are overwritten by the fallback pass
    if (B.pix >= 0) store_pixel(p, B.pix, rgb);
    // every thread's TMEM reads precede the next block's layer 1 in these columns
    tc::fence_before_sync();
    tc::wg_sync(bar);
    B.stage = 0;
}

__device__ void consume(LearnSmem& S, const LearnParams& A, int lane) {
    BlockRegs B[kPipes];
#pragma unroll
    for (int k = 0; k < kPipes; ++k) B[k].stage = 0;
    uint32_t fparity = 0, mparity = 0;
    int done = 0;
    volatile int* abort = &S.abort;
    while (done < kPipes && !*abort) {
#pragma unroll
        for (int k = 0; k < kPipes; ++k)
            if (B[k].stage != 5 && !*abort) consume_step(S, A, lane, k, B[k], fparity, mparity, done);
    }
    // winding down after an expired wait: let issued MMAs finish before TMEM is released
    if (*abort) {
#pragma unroll
        for (int k = 0; k < kPipes; ++k)
            if (B[k].stage >= 1 && B[k].stage <= 4)
                tc::mbar_wait(&S.mma[lane * kPipes + k], (mparity >> k) & 1u, 1u << 20);
    }
}

__global__ void __launch_bounds__(kThreads, 1) shade_learned_kernel(LearnParams A) {
    extern __shared__ uint8_t smem_raw[];
    LearnSmem& S = *reinterpret_cast<LearnSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const PlainParams& p = A.pl;
    const int t = threadIdx.x, warp = t >> 5;
    load_weights(A.w, S.w1, S.w2, S.w3, S.w4);
    // the constant chunks 8 (ones at columns 64, 65) and 9 (zeros) of every pipeline tile
    const uint32_t one2 = uint32_t(bf16_rn(1.0f)) | (uint32_t(bf16_rn(1.0f)) << 16);
    for (int i = t; i < kLanes * kPipes * kRows; i += blockDim.x) {
        uint8_t* tileb = S.act[i / kRows];
        *chunk_row(tileb, 8, i % kRows) = make_uint4(one2, 0u, 0u, 0u);
        *chunk_row(tileb, 9, i % kRows) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (t == 0) {
        for (int i = 0; i < kLanes * kPipes; ++i) {
            tc::mbar_init(&S.full[i], 1);
            tc::mbar_init(&S.empty[i], 1);
            tc::mbar_init(&S.mma[i], 1);
        }
        S.abort = 0;
    }
    if (warp == 0) { tc::tmem_alloc(&S.tmem, 512); tc::tmem_relinquish(); }
    tc::fence_smem_for_mma();
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // the prologue above overlaps the pre-pass's tail; its results are read from here on
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (warp < 4 * kLanes) consume(S, A, warp / 4);
    else if ((t & 31) == 0) produce(S, A, warp - 4 * kLanes);
    if (t == 0 && S.abort) atomicExch(A.error, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) { tc::fence_after_sync(); tc::tmem_dealloc(S.tmem, 512); }
}

// Plain shading of the tiles the gates rejected, bit-exact with the plain
// shader: work items of 16x16 pixels (four per tile), each culling the lights
// against its box and summing the rest (plain_block_lights / _pixel), one
// thread per pixel.  The CTAs are small enough to sit beside the tensor-core
// kernel's CTA on an SM, so one per SM is resident and waiting when it ends.
constexpr int kFbItems = (kShadeTile / kPlainBlock) * (kShadeTile / kPlainBlock);   // per tile
__global__ void __launch_bounds__(kPlainThreads, 6) shade_fallback_kernel(PlainParams p, const int32_t* __restrict__ rejected,
                                                                       const int* __restrict__ count) {
    __shared__ rsrgpu_light L[kMaxLights];
    __shared__ PlainBlockShared S;
    asm volatile("griddepcontrol.wait;" ::: "memory");   // the gates' decisions are complete
    const int items = kFbItems * *count;
    if (int(blockIdx.x) >= items) return;
    const int nl = p.nlights < kMaxLights ? p.nlights : kMaxLights;
    load_lights(L, p.lights, nl);
    const int tiles_x = (p.width + kShadeTile - 1) / kShadeTile;
    constexpr int per_row = kShadeTile / kPlainBlock;
    for (int k = blockIdx.x; k < items; k += gridDim.x) {
        const int tile = rejected[k / kFbItems], b = k % kFbItems;
        const int x = (tile % tiles_x) * kShadeTile + (b % per_row) * kPlainBlock + int(threadIdx.x) % kPlainBlock;
        const int y = (tile / tiles_x) * kShadeTile + (b / per_row) * kPlainBlock + int(threadIdx.x) / kPlainBlock;
        const int pi = y * p.width + x;
        const bool live = x < p.width && y < p.height && p.albedo[pi] != 0u;
        float P[3] = { 0.0f, 0.0f, 0.0f }, n[3], v[3], vlen, a[3];
        if (live) {
            world_pos(p, x, y, p.depth[pi], P);
            surface(p, P, p.nx[pi], p.ny[pi], p.nz[pi], n, v, vlen);
            albedo_rgb(p.albedo[pi], a);
        }
        __syncthreads();   // lights loaded; the previous item's light list read
        const int nkeep = plain_block_lights(L, nl, live, P, S);
        if (live) {
            float rgb[3];
            plain_block_pixel(L, S.keep, nkeep, P, n, v, a, rgb);
            store_pixel(p, pi, rgb);
        }
    }
}

size_t learned_scratch_bytes(int tiles) {
    return 512 + sizeof(int32_t) * size_t(tiles) * (kBlocksPerTile + 1) +
           size_t(tiles) * kBlocksPerTile * (size_t(kFeatBytes) + sizeof(PipeMeta));
}

cudaError_t launch_shade_learned(const rsrgpu_mlp& w, const rsrgpu_gbuffer& gb, const float ivp[16], const float eye[3],
                                 const rsrgpu_light* lights, int nlights, const float background[3], float max_tile_mse,
                                 uint32_t* out_srgb, float* out_linear, uint8_t* tile_status, float* tile_mse,
                                 const uint8_t* srgb_lut, int* error, int* counters, void* scratch,
                                 int num_sms, int stall_polls, cudaStream_t st) {
    LearnParams A{};
    A.poll_limit = stall_polls > 0 ? uint32_t(stall_polls) : (1u << 22);
    A.stall = stall_polls > 0 ? 1 : 0;
    PlainParams& p = A.pl;
    p.depth = gb.depth; p.nx = gb.normal_x; p.ny = gb.normal_y; p.nz = gb.normal_z; p.albedo = gb.albedo;
    p.width = gb.width; p.height = gb.height;
    for (int i = 0; i < 16; ++i) p.ivp[i] = ivp[i];
    for (int i = 0; i < 3; ++i) { p.eye[i] = eye[i]; p.background[i] = background[i]; }
    p.lights = lights; p.nlights = nlights; p.out_srgb = out_srgb; p.out_linear = out_linear; p.srgb_lut = srgb_lut;
    const int tiles = ((gb.width + kShadeTile - 1) / kShadeTile) * ((gb.height + kShadeTile - 1) / kShadeTile);
    A.w = w; A.max_tile_mse = max_tile_mse; A.tile_status = tile_status; A.tile_mse = tile_mse; A.error = error;
    A.counters = counters;
    uint8_t* base = static_cast<uint8_t*>(scratch);
    A.blocks = reinterpret_cast<int32_t*>(base);
    A.rejected = A.blocks + size_t(tiles) * kBlocksPerTile;
    A.feat = base + ((sizeof(int32_t) * size_t(tiles) * (kBlocksPerTile + 1) + 255) & ~size_t(255));
    A.metas = reinterpret_cast<PipeMeta*>(A.feat + size_t(tiles) * kBlocksPerTile * kFeatBytes);
    const size_t smem = sizeof(LearnSmem) + 128;
    static int smem_set = -1;   // the attribute is per device function: set it once per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (smem_set != dev) {
        e = cudaFuncSetAttribute(shade_learned_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        smem_set = dev;
    }
    e = cudaMemsetAsync(counters, 0, 3 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const size_t light_bytes = sizeof(rsrgpu_light) * size_t(nlights > 0 ? nlights : 1);
    int pgrid = num_sms * 4;
    if (pgrid > tiles) pgrid = tiles;
    learned_prep_kernel<<<pgrid, kPrepThreads, light_bytes, st>>>(A);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int grid = num_sms;
    if (grid > (tiles + 1) / 2) grid = (tiles + 1) / 2;
    if (grid < 1) grid = 1;
    // the tensor-core kernel and the fallback pass start while their predecessor
    // drains (programmatic dependent launch); each waits for its inputs
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = pdl;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, shade_learned_kernel, A);
    if (e != cudaSuccess) return e;
    int fgrid = num_sms * 4;
    if (fgrid > tiles * kFbItems) fgrid = tiles * kFbItems;
    cfg.gridDim = dim3(fgrid);
    cfg.blockDim = dim3(kPlainThreads);
    cfg.dynamicSmemBytes = 0;
    const int32_t* rej = A.rejected;
    const int* cnt = counters + 2;
    return cudaLaunchKernelEx(&cfg, shade_fallback_kernel, p, rej, cnt);
}

}  // namespace rsrgpu
