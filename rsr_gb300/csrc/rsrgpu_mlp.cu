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
#include "rsrgpu_tc.cuh"

namespace rsrgpu {

constexpr int kIn = 32, kHid = 64, kOut = 16, kRows = 128;

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

// copies a row-major bf16 [rows][k] matrix into the K-major core layout
__device__ __forceinline__ void load_kmajor(uint8_t* dst, const uint16_t* src, int rows, int k) {
    const int chunks = rows * (k / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (k / 8), j = c % (k / 8);
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + r * k + j * 8));
        *reinterpret_cast<uint4*>(dst + tc::kmajor_offset(r, j * 8, k)) = v;
    }
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat16 lo = __float2bfloat16_rn(a), hi = __float2bfloat16_rn(b);
    return uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
}

// D (TMEM lane = thread) columns [0, 64) -> bias + ReLU -> bf16 row `t` of the hidden A tile
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem_row, const float* bias, uint8_t* ah, int t) {
#pragma unroll
    for (int c0 = 0; c0 < kHid; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem_row + c0, v);
#pragma unroll
        for (int j = 0; j < 16; j += 8) {
            uint4 pk;
            float x[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { const float y = v[j + q] + bias[c0 + j + q]; x[q] = y > 0.f ? y : 0.f; }
            pk.x = pack_bf16x2(x[0], x[1]); pk.y = pack_bf16x2(x[2], x[3]);
            pk.z = pack_bf16x2(x[4], x[5]); pk.w = pack_bf16x2(x[6], x[7]);
            *reinterpret_cast<uint4*>(ah + tc::kmajor_offset(t, c0 + j, kHid)) = pk;
        }
    }
}

// issue D = A * B^T for a K-major A (128 x k) and B (n x k), then commit
__device__ __forceinline__ void issue_layer(uint32_t d, const uint8_t* a, const uint8_t* b, int k, int n, uint64_t* mbar) {
    tc::fence_after_sync();
    const uint32_t sa = tc::smem_addr(a), sb = tc::smem_addr(b);
    const uint32_t sbo = uint32_t(k / 8) * 128u;
    for (int ks = 0; ks < k / 16; ++ks) {
        const uint64_t ad = tc::smem_desc(sa + ks * 256u, 128u, sbo);
        const uint64_t bd = tc::smem_desc(sb + ks * 256u, 128u, sbo);
        tc::mma_bf16(d, ad, bd, tc::idesc_bf16(kRows, n), ks > 0 ? 1u : 0u);
    }
    tc::mma_commit(mbar);
}

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

}  // namespace rsrgpu
