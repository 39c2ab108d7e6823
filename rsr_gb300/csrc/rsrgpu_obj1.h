// rsrgpu_obj1.h -- OBJ1Program's vertex shading (src/viewer/shaders.hxx:586-699),
// shared by the device setup kernel and a host build of the same source that
// the tests compare with the oracle.
//
// The program lights each vertex in view space with a point light at the eye
// and passes the lit colour on to Gouraud interpolation:
//   mvv = vm * (position, 1)            mvn = vm * (normal, 0)
//   d   = (0,0,0,1) - mvv               (rmlv's qfloat4 operator- takes the w
//                                        component as 1 - mvv.z, rmlv_soa.hxx:163)
//   distance = sqrt(dot(d, d))          lightVector = d * rsqrtps(dot(d, d))
//   diffuse  = max(dot(mvn, lightVector), 0.1) * (100 / distance)
//   kd_out   = kd * diffuse             gl_Position = vpm * (position, 1)
// with rsr's operation order everywhere (dot products and matrix rows summed
// left to right, no fused multiply-add) and RSQRTPS reproduced by the measured
// table of gen_rsqrtps_table.c.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#ifdef __CUDACC__
#define RSRGPU_HD __host__ __device__ __forceinline__
#else
#define RSRGPU_HD inline
#endif

namespace rsrgpu {

RSRGPU_HD uint32_t obj1_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
RSRGPU_HD float obj1_float(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

// _mm_rsqrt_ps by the model of gen_rsqrtps_table.c (T: 4096 entries)
RSRGPU_HD float rsqrtps_model(const uint32_t* T, float xf) {
    const uint32_t x = obj1_bits(xf);
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 255u, m = x & 0x7fffffu;
    if (e == 255u) {
        if (m) return obj1_float(x | 0x00400000u);
        return obj1_float(s ? 0xffc00000u : 0u);
    }
    if (e == 0u) return obj1_float(s | 0x7f800000u);
    if (s) return obj1_float(0xffc00000u);
    const int k = int(e) - 127, p = k & 1;
    const uint32_t t = T[uint32_t(p) * 2048u + (m >> 12)];
    const int er = int((t >> 23) & 255u) - (k - p) / 2;
    return obj1_float((uint32_t(er) << 23) | (t & 0x7fffffu));
}

// _mm_max_ps(a, b): a > b ? a : b
RSRGPU_HD float obj1_maxps(float a, float b) { return a > b ? a : b; }

RSRGPU_HD float obj1_sqrt(float x) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}

// qmat4 * qfloat4 (rmlm_soa.hxx:59-65), one lane
RSRGPU_HD void obj1_mat_vec(const float* m, float x, float y, float z, float w, float out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = ((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w;
}

// OBJ1Program::ShadeVertex for one vertex (shaders.hxx:656-676)
RSRGPU_HD void obj1_shade(const float* vm, const float* vpm, const uint32_t* rsqrt_table, const float p[3],
                          const float n[3], const float kd[3], float pos[4], float out_kd[3]) {
    float mvv[4], mvn[4];
    obj1_mat_vec(vm, p[0], p[1], p[2], 1.0f, mvv);
    obj1_mat_vec(vm, n[0], n[1], n[2], 0.0f, mvn);
    const float dx = 0.0f - mvv[0], dy = 0.0f - mvv[1], dz = 0.0f - mvv[2], dw = 1.0f - mvv[2];
    const float dd = ((dx * dx + dy * dy) + dz * dz) + dw * dw;
    const float distance = obj1_sqrt(dd);
    const float scale = rsqrtps_model(rsqrt_table, dd);
    const float lx = dx * scale, ly = dy * scale, lz = dz * scale, lw = dw * scale;
    float diffuse = obj1_maxps(((mvn[0] * lx + mvn[1] * ly) + mvn[2] * lz) + mvn[3] * lw, 0.1f);
    diffuse = diffuse * (100.0f / distance);
    out_kd[0] = kd[0] * diffuse;
    out_kd[1] = kd[1] * diffuse;
    out_kd[2] = kd[2] * diffuse;
    obj1_mat_vec(vpm, p[0], p[1], p[2], 1.0f, pos);
}

}  // namespace rsrgpu
