// rsrgpu_mlp.cu -- the learned deferred shader's MLP on tcgen05 tensor cores.
//
// Network: 24 -> 64 -> 64 -> 64 -> 3, ReLU, BF16 weights and activations,
// FP32 accumulation (inputs padded to 32, outputs to 16 columns).  One CTA of
// four warps processes 128 pixels at a time: the pixel rows are the MMA's M
// dimension, so thread t owns TMEM lane t, reads its layer output with
// tcgen05.ld, adds the bias, applies ReLU, rounds to BF16 and writes the next
// layer's A tile.  Weights stay resident in shared memory for the CTA's
// whole persistent loop.  See rsrgpu_tc.cuh for the operand layout.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/rsrgpu.h"
#include "rsrgpu_mlp.cuh"

namespace rsrgpu {

struct MlpSmem {
    alignas(1024) uint8_t w1[kHid * kIn * 2];     // 64 x 32, K-major core layout
    alignas(1024) uint8_t w2[kHid * kHid * 2];    // 64 x 64
    alignas(1024) uint8_t w3[kHid * kHid * 2];
    alignas(1024) uint8_t w4[kOut * kHid * 2];    // 16 x 64
    alignas(1024) uint8_t a0[kRows * kIn * 2];    // input features 128 x 32
    alignas(1024) uint8_t ah[kRows * kHid * 2];   // hidden activations 128 x 64
    float b1[kHid], b2[kHid], b3[kHid], b4[kOut];
    uint64_t mbar;
    uint32_t tmem;
    int abort_flag;
};

__global__ void __launch_bounds__(128) mlp_forward_kernel(rsrgpu_mlp w, const uint16_t* __restrict__ feat, int n,
                                                          float* __restrict__ out, int* __restrict__ error) {
    extern __shared__ uint8_t smem_raw[];
    MlpSmem& S = *reinterpret_cast<MlpSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int t = threadIdx.x;
    const int warp = t >> 5;
    load_kmajor(S.w1, w.w1, kHid, kIn);
    load_kmajor(S.w2, w.w2, kHid, kHid);
    load_kmajor(S.w3, w.w3, kHid, kHid);
    load_kmajor(S.w4, w.w4, kOut, kHid);
    for (int i = t; i < kHid; i += blockDim.x) { S.b1[i] = w.b1[i]; S.b2[i] = w.b2[i]; S.b3[i] = w.b3[i]; }
    if (t < kOut) S.b4[t] = w.b4[t];
    if (t == 0) { tc::mbar_init(&S.mbar, 1); S.abort_flag = 0; }
    if (warp == 0) { tc::tmem_alloc(&S.tmem, 64); tc::tmem_relinquish(); }
    tc::fence_smem_for_mma();
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem;
    const uint32_t row = tmem + (uint32_t(warp * 32) << 16);
    uint32_t phase = 0;
    const int ntiles = (n + kRows - 1) / kRows;
    bool aborted = false;
    for (int tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
        const int p = tile * kRows + t;
        // features: 32 bf16 per pixel, 4 x 16 bytes
#pragma unroll
        for (int j = 0; j < kIn; j += 8) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (p < n) v = __ldg(reinterpret_cast<const uint4*>(feat + size_t(p) * kIn + j));
            *reinterpret_cast<uint4*>(S.a0 + tc::kmajor_offset(t, j, kIn)) = v;
        }
        const uint8_t* a_in = S.a0;
        int k_in = kIn;
        const uint8_t* wl[4] = { S.w1, S.w2, S.w3, S.w4 };
        const float* bl[3] = { S.b1, S.b2, S.b3 };
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
                hidden_epilogue(row, bl[layer], S.ah, t);
                a_in = S.ah;
                k_in = kHid;
            } else {
                float v[16];
                tc::tmem_ld16(row, v);
                if (p < n) {
                    out[size_t(p) * 3 + 0] = v[0] + S.b4[0];
                    out[size_t(p) * 3 + 1] = v[1] + S.b4[1];
                    out[size_t(p) * 3 + 2] = v[2] + S.b4[2];
                }
            }
        }
    }
    if (aborted && t == 0) atomicExch(error, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) { tc::fence_after_sync(); tc::tmem_dealloc(tmem, 64); }
}

size_t mlp_smem_bytes() { return sizeof(MlpSmem) + 1024; }

cudaError_t launch_mlp_forward(const rsrgpu_mlp& w, const uint16_t* feat, int n, float* out, int* error,
                               int num_sms, cudaStream_t st) {
    const size_t smem = mlp_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const int ntiles = (n + kRows - 1) / kRows;
    int grid = num_sms * 4;
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    mlp_forward_kernel<<<grid, kRows, smem, st>>>(w, feat, n, out, error);
    return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// training step: forward + backward over a batch, gradients summed into FP32
// ---------------------------------------------------------------------------
// TMEM columns: [0,64) layer scratch, [64,128) dW1^T, [128,192) dW2^T,
// [192,256) dW3^T, [256,272) dW4^T.  Each dW^T accumulator holds input
// feature i in lane i and output unit o in column o; lane 64 holds the bias
// gradient (the transposed activation tile carries a row of ones there).
constexpr uint32_t kColScratch = 0, kColW1 = 64, kColW2 = 128, kColW3 = 192, kColW4 = 256;
constexpr int kPix = 128;          // pixels per tile = K of the weight-gradient MMAs

struct TrainSmem {
    alignas(1024) uint8_t w1[kHid * kIn * 2];     // forward B operands
    alignas(1024) uint8_t w2[kHid * kHid * 2];
    alignas(1024) uint8_t w3[kHid * kHid * 2];
    alignas(1024) uint8_t w4[kOut * kHid * 2];
    alignas(1024) uint8_t w2t[kHid * kHid * 2];   // backward B operands: W^T (in x out)
    alignas(1024) uint8_t w3t[kHid * kHid * 2];
    alignas(1024) uint8_t w4t[kHid * kOut * 2];   // 64 x 16
    alignas(1024) uint8_t a0[kRows * kIn * 2];
    alignas(1024) uint8_t a1[kRows * kHid * 2];
    alignas(1024) uint8_t a2[kRows * kHid * 2];
    alignas(1024) uint8_t a3[kRows * kHid * 2];
    alignas(1024) uint8_t at[128 * kPix * 2];     // A^T of one layer, rows 64.. = ones row + zeros
    alignas(1024) uint8_t dz[kRows * kHid * 2];   // dZ (A operand), K = 16 or 64
    alignas(1024) uint8_t dzt[kHid * kPix * 2];   // dZ^T (B operand), N = 16 or 64
    float b1[kHid], b2[kHid], b3[kHid], b4[kOut];
    float loss[4];
    uint64_t mbar;
    uint32_t tmem;
};

__device__ __forceinline__ uint16_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

// loads W (rows x k, row-major) transposed into a K-major (k x rows)... i.e. tile (n = k_in, K = rows)
__device__ __forceinline__ void load_transposed(uint8_t* dst, const uint16_t* src, int rows, int k) {
    for (int e = threadIdx.x; e < rows * k; e += blockDim.x) {
        const int o = e / k, i = e % k;   // src[o][i] -> dst row i, column o (tile K = rows)
        *reinterpret_cast<uint16_t*>(dst + tc::kmajor_offset(i, o, rows)) = __ldg(src + e);
    }
}

// one MMA group: D (+)= A (128 x k, K-major, kdim) * B (n x k)^T
__device__ __forceinline__ void mma_group(uint32_t d, const uint8_t* a, int akdim, const uint8_t* b, int bkdim,
                                          int k, int n, bool accumulate) {
    const uint32_t sa = tc::smem_addr(a), sb = tc::smem_addr(b);
    for (int ks = 0; ks < k / 16; ++ks) {
        const uint64_t ad = tc::smem_desc(sa + ks * 256u, 128u, uint32_t(akdim / 8) * 128u);
        const uint64_t bd = tc::smem_desc(sb + ks * 256u, 128u, uint32_t(bkdim / 8) * 128u);
        tc::mma_bf16(d, ad, bd, tc::idesc_bf16(kRows, n), (accumulate || ks > 0) ? 1u : 0u);
    }
}

struct TrainArgs {
    rsrgpu_mlp w;
    const uint16_t* feat;      // [nsamples][32] bf16
    const float* target;       // [nsamples][3]
    const int32_t* index;      // [batch] sample rows
    int batch;
    float inv_count;           // 1 / (3 * batch): mean-squared-error scale
    float* grad;               // fp32: w1 64x32, w2 64x64, w3 64x64, w4 16x64, b1 64, b2 64, b3 64, b4 16
    float* loss;               // sum of squared errors
    int* error;
};

__global__ void __launch_bounds__(128) mlp_train_kernel(TrainArgs A) {
    extern __shared__ uint8_t smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int t = threadIdx.x, warp = t >> 5;
    load_kmajor(S.w1, A.w.w1, kHid, kIn);
    load_kmajor(S.w2, A.w.w2, kHid, kHid);
    load_kmajor(S.w3, A.w.w3, kHid, kHid);
    load_kmajor(S.w4, A.w.w4, kOut, kHid);
    load_transposed(S.w2t, A.w.w2, kHid, kHid);
    load_transposed(S.w3t, A.w.w3, kHid, kHid);
    load_transposed(S.w4t, A.w.w4, kOut, kHid);
    for (int i = t; i < kHid; i += blockDim.x) { S.b1[i] = A.w.b1[i]; S.b2[i] = A.w.b2[i]; S.b3[i] = A.w.b3[i]; }
    if (t < kOut) S.b4[t] = A.w.b4[t];
    // A^T rows 64..127: a row of ones (bias gradient), zeros below
    for (int e = t; e < 64 * kPix; e += blockDim.x) {
        const int r = 64 + e / kPix, c = e % kPix;
        *reinterpret_cast<uint16_t*>(S.at + tc::kmajor_offset(r, c, kPix)) = r == 64 ? bf16_bits(1.0f) : 0;
    }
    if (t == 0) { tc::mbar_init(&S.mbar, 1); }
    if (t < 4) S.loss[t] = 0.f;
    if (warp == 0) { tc::tmem_alloc(&S.tmem, 512); tc::tmem_relinquish(); }
    tc::fence_smem_for_mma();
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem;
    const uint32_t lane_base = uint32_t(warp * 32) << 16;
    uint32_t phase = 0;
    bool aborted = false, first = true;
    float sq = 0.f;
    const int ntiles = (A.batch + kPix - 1) / kPix;

    // waits for the committed MMAs; false on timeout (all threads agree)
    auto sync_mma = [&](bool issue_commit) -> bool {
        if (issue_commit && t == 0) tc::mma_commit(&S.mbar);
        const bool ok = tc::mbar_wait(&S.mbar, phase);
        phase ^= 1u;
        const bool bad = __syncthreads_or(!ok);
        tc::fence_after_sync();
        return !bad;
    };
    auto before_issue = [&]() {
        tc::fence_smem_for_mma();
        tc::fence_before_sync();
        __syncthreads();
        if (t == 0) tc::fence_after_sync();
    };

    for (int tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
        const int r = tile * kPix + t;
        const bool valid = r < A.batch;
        const int sidx = valid ? A.index[r] : 0;
        // ---- forward ----
#pragma unroll
        for (int j = 0; j < kIn; j += 8) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (valid) v = __ldg(reinterpret_cast<const uint4*>(A.feat + size_t(sidx) * kIn + j));
            *reinterpret_cast<uint4*>(S.a0 + tc::kmajor_offset(t, j, kIn)) = v;
        }
        before_issue();
        if (t == 0) mma_group(tmem + kColScratch, S.a0, kIn, S.w1, kIn, kIn, kHid, false);
        if (!sync_mma(true)) { aborted = true; break; }
        hidden_epilogue(tmem + lane_base, S.b1, S.a1, t);
        before_issue();
        if (t == 0) mma_group(tmem + kColScratch, S.a1, kHid, S.w2, kHid, kHid, kHid, false);
        if (!sync_mma(true)) { aborted = true; break; }
        hidden_epilogue(tmem + lane_base, S.b2, S.a2, t);
        before_issue();
        if (t == 0) mma_group(tmem + kColScratch, S.a2, kHid, S.w3, kHid, kHid, kHid, false);
        if (!sync_mma(true)) { aborted = true; break; }
        hidden_epilogue(tmem + lane_base, S.b3, S.a3, t);
        before_issue();
        if (t == 0) mma_group(tmem + kColScratch, S.a3, kHid, S.w4, kHid, kHid, kOut, false);
        if (!sync_mma(true)) { aborted = true; break; }
        // ---- loss and dY ----
        {
            float v[16];
            tc::tmem_ld16(tmem + lane_base + kColScratch, v);
            uint16_t dy[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) dy[c] = 0;
            if (valid) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float y = v[c] + S.b4[c];
                    const float e = y - __ldg(A.target + size_t(sidx) * 3 + c);
                    sq += e * e;
                    dy[c] = bf16_bits(2.0f * e * A.inv_count);
                }
            }
            // dY as the A operand (128 x 16) and dY^T as the B operand (16 x 128)
#pragma unroll
            for (int j = 0; j < 16; j += 8) {
                uint4 pk;
                pk.x = dy[j] | (uint32_t(dy[j + 1]) << 16); pk.y = dy[j + 2] | (uint32_t(dy[j + 3]) << 16);
                pk.z = dy[j + 4] | (uint32_t(dy[j + 5]) << 16); pk.w = dy[j + 6] | (uint32_t(dy[j + 7]) << 16);
                *reinterpret_cast<uint4*>(S.dz + tc::kmajor_offset(t, j, 16)) = pk;
            }
#pragma unroll
            for (int c = 0; c < 16; ++c) *reinterpret_cast<uint16_t*>(S.dzt + tc::kmajor_offset(c, t, kPix)) = dy[c];
            // A3^T
#pragma unroll 8
            for (int f = 0; f < kHid; ++f)
                *reinterpret_cast<uint16_t*>(S.at + tc::kmajor_offset(f, t, kPix)) =
                    *reinterpret_cast<const uint16_t*>(S.a3 + tc::kmajor_offset(t, f, kHid));
        }
        // ---- backward, layer 4: dW4^T += A3^T dY ; dA3 = dY W4 ----
        before_issue();
        if (t == 0) {
            mma_group(tmem + kColW4, S.at, kPix, S.dzt, kPix, kPix, kOut, !first);
            mma_group(tmem + kColScratch, S.dz, 16, S.w4t, 16, 16, kHid, false);
        }
        if (!sync_mma(true)) { aborted = true; break; }
        // ---- layers 3, 2, 1 ----
        const uint8_t* act[3] = { S.a3, S.a2, S.a1 };     // mask source for dZ
        const uint8_t* prev[3] = { S.a2, S.a1, S.a0 };    // A^T source for dW
        const int prevk[3] = { kHid, kHid, kIn };
        const uint32_t wcol[3] = { kColW3, kColW2, kColW1 };
        const uint8_t* wt[3] = { S.w3t, S.w2t, nullptr };
        bool ok = true;
        for (int l = 0; l < 3 && ok; ++l) {
            // dZ = dA * (act > 0), written as A operand (128 x 64) and B operand (64 x 128)
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float v[16];
                tc::tmem_ld16(tmem + lane_base + kColScratch + c0, v);
#pragma unroll
                for (int j = 0; j < 16; j += 8) {
                    uint16_t z[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const uint16_t a = *reinterpret_cast<const uint16_t*>(act[l] + tc::kmajor_offset(t, c0 + j + q, kHid));
                        z[q] = (bf16_val(a) > 0.f && valid) ? bf16_bits(v[j + q]) : uint16_t(0);
                        *reinterpret_cast<uint16_t*>(S.dzt + tc::kmajor_offset(c0 + j + q, t, kPix)) = z[q];
                    }
                    uint4 pk;
                    pk.x = z[0] | (uint32_t(z[1]) << 16); pk.y = z[2] | (uint32_t(z[3]) << 16);
                    pk.z = z[4] | (uint32_t(z[5]) << 16); pk.w = z[6] | (uint32_t(z[7]) << 16);
                    *reinterpret_cast<uint4*>(S.dz + tc::kmajor_offset(t, c0 + j, kHid)) = pk;
                }
            }
            // previous layer's activation, transposed (rows >= its width are zero)
            for (int f = 0; f < kHid; ++f) {
                const uint16_t a = f < prevk[l] ? *reinterpret_cast<const uint16_t*>(prev[l] + tc::kmajor_offset(t, f, prevk[l])) : uint16_t(0);
                *reinterpret_cast<uint16_t*>(S.at + tc::kmajor_offset(f, t, kPix)) = a;
            }
            before_issue();
            if (t == 0) {
                mma_group(tmem + wcol[l], S.at, kPix, S.dzt, kPix, kPix, kHid, !first);
                if (wt[l] != nullptr) mma_group(tmem + kColScratch, S.dz, kHid, wt[l], kHid, kHid, kHid, false);
            }
            ok = sync_mma(true);
        }
        if (!ok) { aborted = true; break; }
        first = false;
    }
    // ---- gradients out: lane i holds input i (bias in lane 64) ----
    if (!aborted && !first) {
        const int i = t;
        const uint32_t base = tmem + lane_base;
        const int fin[4] = { 24, kHid, kHid, kHid };
        const uint32_t cols[4] = { kColW1, kColW2, kColW3, kColW4 };
        const int nout[4] = { kHid, kHid, kHid, kOut };
        const int woff[4] = { 0, 64 * 32, 64 * 32 + 64 * 64, 64 * 32 + 2 * 64 * 64 };
        const int boff = 64 * 32 + 2 * 64 * 64 + 16 * 64;
        const int bstart[4] = { boff, boff + 64, boff + 128, boff + 192 };
        const int kin[4] = { kIn, kHid, kHid, kHid };
        for (int l = 0; l < 4; ++l) {
            for (int c0 = 0; c0 < nout[l]; c0 += 16) {
                float v[16];
                tc::tmem_ld16(base + cols[l] + c0, v);
                for (int q = 0; q < 16; ++q) {
                    const int o = c0 + q;
                    if (i < fin[l]) atomicAdd(A.grad + woff[l] + o * kin[l] + i, v[q]);
                    else if (i == 64) atomicAdd(A.grad + bstart[l] + o, v[q]);
                }
            }
        }
    }
    // loss
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
    if ((t & 31) == 0) S.loss[warp] = sq;
    __syncthreads();
    if (t == 0) {
        atomicAdd(A.loss, (S.loss[0] + S.loss[1]) + (S.loss[2] + S.loss[3]));
        if (aborted) atomicExch(A.error, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) { tc::fence_after_sync(); tc::tmem_dealloc(tmem, 512); }
}

size_t mlp_train_smem_bytes() { return sizeof(TrainSmem) + 1024; }

cudaError_t launch_mlp_train(const rsrgpu_mlp& w, const uint16_t* feat, const float* target, const int32_t* index,
                             int batch, float* grad, float* loss, int* error, int num_sms, cudaStream_t st) {
    const size_t smem = mlp_train_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    TrainArgs a;
    a.w = w; a.feat = feat; a.target = target; a.index = index; a.batch = batch;
    a.inv_count = 1.0f / (3.0f * float(batch));
    a.grad = grad; a.loss = loss; a.error = error;
    const int ntiles = (batch + kPix - 1) / kPix;
    int grid = num_sms;
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    mlp_train_kernel<<<grid, kRows, smem, st>>>(a);
    return cudaGetLastError();
}

// Adam on FP32 master parameters; writes the BF16 weights the kernels read.
// Layout of params/grads/m/v: w1 64x32, w2 64x64, w3 64x64, w4 16x64, b1 64, b2 64, b3 64, b4 16.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            int n, int nw, float lr, float b1, float b2, float eps, float c1, float c2,
                            uint16_t* __restrict__ wbf16, float* __restrict__ bias_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (i < nw) wbf16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(pi));
    else bias_out[i - nw] = pi;
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int n, int nw, float lr, float b1, float b2,
                        float eps, int step, uint16_t* wbf16, float* bias_out, cudaStream_t st) {
    const float c1 = 1.0f - powf(b1, float(step)), c2 = 1.0f - powf(b2, float(step));
    adam_kernel<<<(n + 255) / 256, 256, 0, st>>>(p, g, m, v, n, nw, lr, b1, b2, eps, c1, c2, wbf16, bias_out);
    return cudaGetLastError();
}

}  // namespace rsrgpu
