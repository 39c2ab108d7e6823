// rsrgpu_mlp.cuh -- layer building blocks of the learned shader's MLP
// (24 -> 64 -> 64 -> 64 -> 3, BF16 weights/activations, FP32 accumulation on
// tcgen05), shared by the stand-alone MLP kernels and the fused learned
// shading kernel.  One CTA of four warps runs 128 pixel rows at a time: the
// rows are the MMA's M dimension, thread t owns TMEM lane t.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

#include "rsrgpu_tc.cuh"

namespace rsrgpu {

constexpr int kIn = 32, kHid = 64, kOut = 16, kRows = 128;

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

}  // namespace rsrgpu
