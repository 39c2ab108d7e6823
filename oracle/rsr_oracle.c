/*
 * rsr_oracle.c -- ORACLE (test infrastructure only; never linked into the
 * GPU library).  A portable plain-C restatement of rsr's CPU rasteriser
 * path: command interpretation and tile binning (GPU::BinImpl,
 * GPUBinImpl::BinTriangles1P/2P), Sutherland-Hodgman clipping
 * (GPUBinImpl::ClipTriangles), the per-tile interpreter (GPU::DrawImpl),
 * the vector and scalar triangle rasterisers (rglv_triangle.hxx), the
 * per-quad fragment pipeline (TriangleProgram::Render), the Gouraud test
 * program and AmyProgram with rsr's texture samplers, and the TrueColor /
 * depth stores (FilterTile, Copy).
 *
 * Parity is pinned against rsr itself: tests compare this file's output with
 * oracle/_ref/librsrref.so (the reference sources compiled by
 * oracle/ref/Makefile) on the same seeded scenes, bit-exact for colour
 * (gamma off and on), depth, tile streams and clipped vertices.  The sRGB8
 * pack uses tests/golden/srgb8_lut.bin, the reference encoder's output
 * table generated by oracle/ref/gen_srgb_lut.cxx.  RCPPS is reproduced with
 * rsr_gb300/csrc/rcpps_table.inc (measured by gen_rcpps_table.c).
 *
 * Arithmetic follows the reference's SSE semantics lane by lane: IEEE binary32
 * with no contraction (build with -ffp-contract=off), truncating and
 * round-to-nearest-even float->int conversions that return INT32_MIN out of
 * range, wrapping 32-bit integer products, and x86 min/max operand order.
 * Citations are to the reference's files (path within the rsr project).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rsrgpu.h"

/* ======================================================================
 * SIMD lane semantics (src/rml/rmlv/rmlv_mvec4.hxx)
 * ====================================================================== */
static const uint32_t RCPPS_TABLE[2048] = {
#include "../rsr_gb300/csrc/rcpps_table.inc"
};

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* _mm_rcp_ps, modelled by the measured table (see gen_rcpps_table.c) */
static float rcpps(float x) {
    uint32_t b = f2u(x), s = b & 0x80000000u, e = (b >> 23) & 255u, m = b & 0x7fffffu;
    if (e == 255u) return u2f(m ? (b | 0x00400000u) : s);
    if (e == 0u) return u2f(s | 0x7f800000u);
    uint32_t t = RCPPS_TABLE[m >> 12];
    int er = (int)((t >> 23) & 255u) - ((int)e - 127);
    if (er <= 0) return u2f(s);
    return u2f(s | ((uint32_t)er << 23) | (t & 0x7fffffu));
}

/* _mm_rsqrt_ps, modelled by the measured table (see gen_rsqrtps_table.c):
   the parity of the exponent and the top 11 mantissa bits index it */
static const uint32_t RSQRTPS_TABLE[4096] = {
#include "../rsr_gb300/csrc/rsqrtps_table.inc"
};
static float rsqrtps(float x) {
    uint32_t b = f2u(x), s = b & 0x80000000u, e = (b >> 23) & 255u, m = b & 0x7fffffu;
    if (e == 255u) return u2f(m ? (b | 0x00400000u) : (s ? 0xffc00000u : 0u));
    if (e == 0u) return u2f(s | 0x7f800000u);
    if (s) return u2f(0xffc00000u);
    int k = (int)e - 127, p = k & 1;
    uint32_t t = RSQRTPS_TABLE[(uint32_t)p * 2048u + (m >> 12)];
    int er = (int)((t >> 23) & 255u) - (k - p) / 2;
    return u2f(((uint32_t)er << 23) | (t & 0x7fffffu));
}

/* rmlv::oneover: rcpps + one Newton step (rmlv_mvec4.hxx:631-651) */
static float oneover(float a) {
    float r = rcpps(a);
    float muls = a * (r * r);
    return (r + r) - muls;
}

/* rmlv::ftoi = _mm_cvttps_epi32 (rmlv_mvec4.hxx:552) */
static inline int32_t ftoi(float f) {
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int32_t)f;
}
static inline float itof(int32_t i) { return (float)i; }
static inline float sse_min(float a, float b) { return a < b ? a : b; }   /* minps */
static inline float sse_max(float a, float b) { return a > b ? a : b; }   /* maxps */
static inline int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }
static inline int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
/* rmlv::fract (rmlv_mvec4.hxx:576-582): a - itof(ftoi(a)) */
static inline float fract(float a) { return a - itof(ftoi(a)); }

/* ======================================================================
 * matrices (src/rml/rmlm/rmlm_mat4.hxx, rmlm_soa.hxx)
 * ====================================================================== */
/* rmlm::operator*(mat4, mat4) (rmlm_mat4.hxx:196-207); cr[col][row] = ff[col*4+row] */
static void mat4_mul(const float* l, const float* r, float* out) {
    for (int row = 0; row < 4; ++row) {
        for (int col = 0; col < 4; ++col) {
            float ax;
            ax = l[0 * 4 + row] * r[col * 4 + 0];
            ax += l[1 * 4 + row] * r[col * 4 + 1];
            ax += l[2 * 4 + row] * r[col * 4 + 2];
            ax += l[3 * 4 + row] * r[col * 4 + 3];
            out[col * 4 + row] = ax;
        }
    }
}

/* qmat4 * qfloat4 (rmlm_soa.hxx:59-65), one lane */
static void qmat_mul(const float* f, const float v[4], float out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = ((f[r] * v[0] + f[4 + r] * v[1]) + f[8 + r] * v[2]) + f[12 + r] * v[3];
}

/* ======================================================================
 * shader programs (src/viewer/shaders.hxx; Gouraud test program)
 * ====================================================================== */
#define MAX_VARY 4

static int program_nvary(int pid) {
    switch (pid) {
    case RSRGPU_PROGRAM_GOURAUD: return 3;
    case RSRGPU_PROGRAM_AMY: return 2;
    case RSRGPU_PROGRAM_MANY: return 2;
    case RSRGPU_PROGRAM_OBJ1: return 3;
    case RSRGPU_PROGRAM_GBUFFER: return 4;
    default: return -1;
    }
}

/* SHADER::ShadeVertex for one vertex: gl_Position = vpm * (pos, 1) and the
 * VertexOutputSD (GouraudProgram: rgb from buffers 3-5; AmyProgram
 * shaders.hxx:127-135: uv from buffers 9-10, zero when unbound). */
/* OBJ1Program::ShadeVertex (src/viewer/shaders.hxx:656-676) for one vertex:
 * view-space point light at the eye,
 *   mvv = vm*(p,1), mvn = vm*(n,0), d = (0,0,0,1) - mvv with rmlv's qfloat4
 *   operator- taking w as 1 - mvv.z (src/rml/rmlv/rmlv_soa.hxx:163),
 *   distance = sqrt(dot(d,d)) (rmlv::length, :220-223),
 *   L = d * rsqrtps(dot(d,d)) (rmlv::normalize, :242-248),
 *   diffuse = maxps(dot(mvn, L), 0.1) * (100 / distance),
 *   kd_out = kd * diffuse, gl_Position = vpm*(p,1). */
static void obj1_vertex(const float* vm, const float* vpm, const float p[3], const float n[3], const float kd[3],
                        float pos[4], float kd_out[3]) {
    const float in[4] = { p[0], p[1], p[2], 1.0f }, nrm[4] = { n[0], n[1], n[2], 0.0f };
    float mvv[4], mvn[4];
    qmat_mul(vm, in, mvv);
    qmat_mul(vm, nrm, mvn);
    const float d[4] = { 0.0f - mvv[0], 0.0f - mvv[1], 0.0f - mvv[2], 1.0f - mvv[2] };
    const float dd = ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + d[3] * d[3];
    const float distance = sqrtf(dd);
    const float sc = rsqrtps(dd);
    const float L[4] = { d[0] * sc, d[1] * sc, d[2] * sc, d[3] * sc };
    float diffuse = sse_max(((mvn[0] * L[0] + mvn[1] * L[1]) + mvn[2] * L[2]) + mvn[3] * L[3], 0.1f);
    diffuse = diffuse * (100.0f / distance);
    for (int c = 0; c < 3; ++c) kd_out[c] = kd[c] * diffuse;
    qmat_mul(vpm, in, pos);
}

/* exported for the check of the device shading source (tests/test_obj1.py) */
int rsroracle_obj1_vertices(const float* vm, const float* vpm, const float* p, const float* n, const float* kd, int count,
                            float* pos, float* kd_out) {
    for (int i = 0; i < count; ++i) obj1_vertex(vm, vpm, p + 3 * i, n + 3 * i, kd + 3 * i, pos + 4 * i, kd_out + 3 * i);
    return 0;
}

static void shade_vertex_inst(const rsrgpu_glstate* s, const float* vpm, int iid, int idx, float pos[4],
                              float vary[MAX_VARY]) {
    float in[4];
    if (s->buffers[0]) { in[0] = s->buffers[0][idx]; in[1] = s->buffers[1][idx]; in[2] = s->buffers[2][idx]; }
    else { in[0] = in[1] = in[2] = 0.0f; }
    in[3] = 1.0f;
    if (s->program_id == RSRGPU_PROGRAM_OBJ1) {
        /* OBJ1Program's Loader::LoadLane (shaders.hxx:623-636): position 0,
           normal (0,0,1), kd (1,1,1) when unbound */
        float nrm[3] = { 0.0f, 0.0f, 1.0f }, kd[3] = { 1.0f, 1.0f, 1.0f };
        if (s->buffers[3]) { nrm[0] = s->buffers[3][idx]; nrm[1] = s->buffers[4][idx]; nrm[2] = s->buffers[5][idx]; }
        if (s->buffers[6]) { kd[0] = s->buffers[6][idx]; kd[1] = s->buffers[7][idx]; kd[2] = s->buffers[8][idx]; }
        memset(vary, 0, sizeof(float) * MAX_VARY);
        obj1_vertex(s->view_matrix, vpm, in, nrm, kd, pos, vary);
        return;
    }
    if (s->program_id == RSRGPU_PROGRAM_MANY) {
        /* ManyProgram::ShadeVertex (shaders.hxx:555-562): p1 = imat * (pos, 1),
           gl_Position = vpm * p1; imat = instance iid's mat4 from buffer 15
           (Loader::LoadInstance, :505-506) */
        float p1[4];
        qmat_mul(s->buffers[15] + (size_t)iid * 16, in, p1);
        qmat_mul(vpm, p1, pos);
    } else {
        qmat_mul(vpm, in, pos);
    }
    memset(vary, 0, sizeof(float) * MAX_VARY);
    if (s->program_id == RSRGPU_PROGRAM_GOURAUD) {
        vary[0] = s->buffers[3][idx]; vary[1] = s->buffers[4][idx]; vary[2] = s->buffers[5][idx];
    } else if (s->program_id == RSRGPU_PROGRAM_AMY || s->program_id == RSRGPU_PROGRAM_MANY) {
        vary[0] = s->buffers[9] ? s->buffers[9][idx] : 0.0f;
        vary[1] = s->buffers[10] ? s->buffers[10][idx] : 0.0f;
    } else if (s->program_id == RSRGPU_PROGRAM_GBUFFER) {
        /* G-buffer program (this library's extension): interpolated normal, flat packed-RGB albedo */
        vary[0] = s->buffers[3][idx]; vary[1] = s->buffers[4][idx]; vary[2] = s->buffers[5][idx];
        vary[3] = s->buffers[6][idx];
    }
}

static void shade_vertex(const rsrgpu_glstate* s, const float* vpm, int idx, float pos[4], float vary[MAX_VARY]) {
    shade_vertex_inst(s, vpm, 0, idx, pos, vary);
}

/* ---- texture units (src/rgl/rglr/rglr_texture_sampler.cxx) ---- */
typedef struct TexUnit {
    int kind;           /* 0 nearest-mip, 1 linear-mip, 2 non-pow2 nearest */
    int power;
    const float* buf;
    int width, height, stride;
} TexUnit;

static int ilog2u(unsigned x) { int p = 0; while (x) { x >>= 1; ++p; } return p - 1; }  /* rmlg_pow2.hxx:13-18 */

/* MakeTextureUnit (rglr_texture_sampler.cxx:314-363) */
static int make_texture_unit(const rsrgpu_texture_state* t, TexUnit* u) {
    int power = ilog2u((unsigned)t->width);
    int isp2 = ((1 << power) == t->width) && t->width == t->height && t->stride == t->width;
    u->buf = t->ptr; u->width = t->width; u->height = t->height; u->stride = t->stride; u->power = power;
    if (!isp2) { u->kind = 2; return 0; }
    if (t->width < 4 || t->width > 1024) return -1;
    u->kind = t->filter ? 1 : 0;
    return 0;
}

/* LevelOfDetail (rglr_texture_sampler.cxx:25-42): coarse, lanes 1 - 0 */
static int level_of_detail(const float upx[4], const float vpx[4]) {
    float dux = upx[1] - upx[0];
    float dvx = vpx[1] - vpx[0];
    float sqd = dux * dux + dvx * dvx;
    return ((int32_t)f2u(sqd) - (127 << 23)) >> 24;
}

static inline int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* TextureUnit*::sample for a quad: uv[lane][2] -> rgba[lane][4] */
static void tex_sample(const TexUnit* tu, const float uv[4][2], float out[4][4]) {
    const float almostone = u2f(0x3f7fffffu);
    if (tu->kind == 2) {  /* NM_ONEMAP_WRAP_NEAREST (:289-311) */
        for (int l = 0; l < 4; ++l) {
            int32_t pu = ftoi(fract(uv[l][0] + 100.0f) * (float)tu->width);
            int32_t pv = ftoi((almostone - fract(uv[l][1] + 100.0f)) * (float)tu->height);
            int32_t ofs = wmul(wadd(wmul(pv, tu->stride), pu), 4);
            memcpy(out[l], tu->buf + ofs, 16);
        }
        return;
    }
    const int P = tu->power;
    const float baseDim = (float)(1 << P);
    float upx[4], vpx[4];
    for (int l = 0; l < 4; ++l) { upx[l] = uv[l][0] * baseDim; vpx[l] = uv[l][1] * baseDim; }
    const int lod = iclamp(level_of_detail(upx, vpx), 0, P);
    if (tu->kind == 0) {  /* P2_MIPMAP_WRAP_NEAREST (:63-109) */
        const float levelDim = (float)(1 << (P - lod));
        const int32_t levelBeginRow = (int32_t)((0xfffffffeu << (P - lod)) & ((1u << (P + 1)) - 1u));
        for (int l = 0; l < 4; ++l) {
            int32_t lx = ftoi(fract(uv[l][0] + 10.0f) * levelDim);
            int32_t ly = ftoi((almostone - fract(uv[l][1] + 10.0f)) * levelDim);
            int32_t by = wadd(levelBeginRow, ly);
            int32_t ofs = wmul(wadd((int32_t)((uint32_t)by << P), lx), 4);
            memcpy(out[l], tu->buf + ofs, 16);
        }
        return;
    }
    /* P2_MIPMAP_WRAP_LINEAR (:172-286) */
    const int levelDim = 1 << (P - lod);
    const int32_t wrapMask = levelDim - 1;
    const int32_t levelLastRow = (int32_t)(((0xffffffffu << (P - lod)) & ((1u << (P + 1)) - 1u)) - 1u);
    for (int l = 0; l < 4; ++l) {
        float levelX = uv[l][0] * (float)levelDim;
        float levelY = uv[l][1] * (float)levelDim;
        int32_t tx0 = ftoi(levelX - 0.5f), ty0 = ftoi(levelY - 0.5f);
        int32_t tx1 = wadd(tx0, 1), ty1 = wadd(ty0, 1);
        float fx = (levelX - itof(tx0)) - 0.5f;
        float fy = (levelY - itof(ty0)) - 0.5f;
        float fx1 = 1.0f - fx, fy1 = 1.0f - fy;
        float w00 = fx1 * fy1, w10 = fx * fy1, w01 = fx1 * fy, w11 = fx * fy;
        tx0 &= wrapMask; ty0 &= wrapMask; tx1 &= wrapMask; ty1 &= wrapMask;
        int32_t y0 = wsub(levelLastRow, ty0), y1 = wsub(levelLastRow, ty1);
        const float* p00 = tu->buf + (int64_t)wadd((int32_t)((uint32_t)y0 << P), tx0) * 4;
        const float* p10 = tu->buf + (int64_t)wadd((int32_t)((uint32_t)y0 << P), tx1) * 4;
        const float* p01 = tu->buf + (int64_t)wadd((int32_t)((uint32_t)y1 << P), tx0) * 4;
        const float* p11 = tu->buf + (int64_t)wadd((int32_t)((uint32_t)y1 << P), tx1) * 4;
        for (int c = 0; c < 4; ++c) {
            float ax = p00[c] * w00;
            ax = ax + p10[c] * w10;
            ax = ax + p01[c] * w01;
            ax = ax + p11[c] * w11;
            out[l][c] = ax;
        }
    }
}

/* ======================================================================
 * frame and tile streams
 * ====================================================================== */
typedef struct ByteBuf { uint8_t* p; size_t n, cap; } ByteBuf;

static int bb_reserve(ByteBuf* b, size_t extra) {
    if (b->n + extra <= b->cap) return 0;
    size_t nc = b->cap ? b->cap * 2 : 256;
    while (nc < b->n + extra) nc *= 2;
    uint8_t* np = (uint8_t*)realloc(b->p, nc);
    if (!np) return -1;
    b->p = np; b->cap = nc;
    return 0;
}
static void bb_put(ByteBuf* b, const void* src, size_t n) {
    if (bb_reserve(b, n) != 0) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    memcpy(b->p + b->n, src, n);
    b->n += n;
}
static void bb_u8(ByteBuf* b, uint8_t v) { bb_put(b, &v, 1); }
static void bb_u16(ByteBuf* b, uint16_t v) { bb_put(b, &v, 2); }
static void bb_u64(ByteBuf* b, uint64_t v) { bb_put(b, &v, 8); }

typedef struct Frame {
    int width, height;
    int tile_w, tile_h, tiles_x, tiles_y, ntiles;
    const rsrgpu_glstate* states;
    int nstates;
    ByteBuf* tiles;          /* per-tile streams: reference byte layout, pointer fields hold
                                state indices / host addresses */
    size_t* mark;            /* Mark()/Touched() (rglv_gpu.hxx:230-236) */
    rsrgpu_clipped_vertex* clipped;
    int nclipped, capclipped;
    const uint8_t* srgb_lut;
    uint64_t frags;          /* candidate fragments of the frame, all tiles */
} Frame;

typedef struct Session {
    int threads;
    Frame f;
    uint8_t* srgb_lut;
} Session;

static Session g_session;

/* ViewFrustum (src/rgl/rglv/rglv_view_frustum.hxx:36-94) */
static float guard_band_factor(int w, int h) {
    int longSide = w > h ? w : h;
    int half = longSide / 2;
    return (2048.0f - (float)half) / (float)half;
}
static uint32_t frustum_test(float factor, const float p[4]) {  /* SIMD Test, :60-73 */
    float w = p[3] * factor;
    uint32_t left = (w + p[0]) <= 0.0f;
    uint32_t bottom = (w + p[1]) <= 0.0f;
    uint32_t near = (p[3] + p[2]) <= 0.0f;
    uint32_t right = (w - p[0]) <= 0.0f;
    uint32_t top = (w - p[1]) <= 0.0f;
    return left | (bottom << 1) | (near << 2) | (right << 3) | (top << 4);
}
enum { PL_LEFT, PL_BOTTOM, PL_NEAR, PL_RIGHT, PL_TOP };
static const int CLIP_PLANES[5] = { PL_LEFT, PL_BOTTOM, PL_NEAR, PL_RIGHT, PL_TOP };  /* clipping_panes :24-30 */
static int is_inside(int plane, const float* p) {
    switch (plane) {
    case PL_LEFT: return p[3] + p[0] >= 0;
    case PL_RIGHT: return p[3] - p[0] >= 0;
    case PL_BOTTOM: return p[3] + p[1] >= 0;
    case PL_TOP: return p[3] - p[1] >= 0;
    default: return p[3] + p[2] >= 0;
    }
}
static float plane_distance(int plane, const float* a, const float* b) {
    switch (plane) {
    case PL_LEFT: return (a[3] + a[0]) / ((a[3] + a[0]) - (b[3] + b[0]));
    case PL_RIGHT: return (a[3] - a[0]) / ((a[3] - a[0]) - (b[3] - b[0]));
    case PL_BOTTOM: return (a[3] + a[1]) / ((a[3] + a[1]) - (b[3] + b[1]));
    case PL_TOP: return (a[3] - a[1]) / ((a[3] - a[1]) - (b[3] - b[1]));
    default: return (a[3] + a[2]) / ((a[3] + a[2]) - (b[3] + b[2]));
    }
}

/* GPU::DSDO (rglv_gpu.hxx:265-270) */
static void dsdo(const Frame* f, const rsrgpu_glstate* s, float DS[2], float DO[2]) {
    int vx = f->width, vy = f->height;
    if (s->viewport_size[0] != 0 || s->viewport_size[1] != 0) { vx = s->viewport_size[0]; vy = s->viewport_size[1]; }
    DS[0] = (float)(vx / 2);
    DS[1] = (float)(-vy / 2);
    DO[0] = (float)(vx / 2 + s->viewport_origin[0]);
    DO[1] = (float)(f->height - (vy / 2 + s->viewport_origin[1]));
}

/* The tile range a triangle is binned to, kept inside the tile grid.  rsr
 * indexes tilesHead_[ty * stride + tx] unchecked (rglv_gpu_impl.hxx:490-496,
 * 808-815): a scissor rectangle reaching past the right or bottom edge of the
 * target gives tx = tiles_x (the next row's first tile) or ty = tiles_y (past
 * the array).  Without such a rectangle the range is inside the grid and
 * this changes nothing. */
static void clamp_to_grid(const Frame* f, int* tx0, int* ty0, int* tx1, int* ty1) {
    if (*tx0 < 0) *tx0 = 0;
    if (*ty0 < 0) *ty0 = 0;
    if (*tx1 > f->tiles_x - 1) *tx1 = f->tiles_x - 1;
    if (*ty1 > f->tiles_y - 1) *ty1 = f->tiles_y - 1;
}

/* GPU::ScissorRect (rglv_gpu.hxx:272-276): left, top, right, bottom */
static void scissor_rect(const Frame* f, const rsrgpu_glstate* s, int r[4]) {
    if (!s->scissor_enabled) { r[0] = 0; r[1] = 0; r[2] = f->width; r[3] = f->height; return; }
    int left = s->scissor_origin[0], right = left + s->scissor_size[0];
    int bottom = f->height - s->scissor_origin[1] - 1, top = bottom - s->scissor_size[1];
    r[0] = left; r[1] = top; r[2] = right; r[3] = bottom;
}

static void make_vpm(const rsrgpu_glstate* s, float vpm[16]) {  /* MakeMatrices (rglv_gpu_impl.hxx:44-51) */
    mat4_mul(s->projection_matrix, s->view_matrix, vpm);
}

/* ======================================================================
 * binning: GPUBinImpl::BinTriangles1P/2P (rglv_gpu_impl.hxx:315-675)
 * ====================================================================== */
typedef struct ClipEntry { int iid, i0, i1, i2; } ClipEntry;

static int clip_triangles(Frame* f, const rsrgpu_glstate* s, const ClipEntry* q, int nq);

/* BinTriangles1P/2P (rglv_gpu_impl.hxx:315-675) for `ninst` instances
 * (instanced: CMD_DRAW_INLINE_INSTANCED records start with the instance id) */
static int bin_draw(Frame* f, int state_idx, int count, const uint16_t* indices, int cmd_is_arrays, int ninst,
                    int instanced) {
    const rsrgpu_glstate* s = &f->states[state_idx];
    if (program_nvary(s->program_id) < 0) return RSRGPU_ENODISPATCH;
    /* ManyProgram's vertex input includes the instance matrix, which only
       instanced draws load (rglv_gpu_impl.hxx:364-366,561-564) */
    if (s->program_id == RSRGPU_PROGRAM_MANY && (!instanced || !s->buffers[15])) return RSRGPU_EUNSUPPORTED;
    float vpm[16];
    make_vpm(s, vpm);
    const float factor = guard_band_factor(f->width, f->height);
    int sc[4];
    scissor_rect(f, s, sc);
    float DS[2], DO[2];
    dsdo(f, s, DS, DO);
    const int32_t tlx = sc[0], tly = sc[1], brx = sc[2] - 1, bry = sc[3] - 1;
    const int keepBacks = !(s->culling_enabled && s->cull_face == RSRGPU_GL_BACK);
    const int keepFronts = !(s->culling_enabled && s->cull_face == RSRGPU_GL_FRONT);

    /* per-vertex transform over [0, maxidx] (the 2P path; the 1P path computes the
       same values per corner) */
    int maxidx = 0;
    for (int i = 0; i < count; ++i) {
        int v = cmd_is_arrays ? i : indices[i];
        if (v > maxidx) maxidx = v;
    }
    const int nv = maxidx + 1;
    uint32_t* cf = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nv);
    float* dx = (float*)malloc(sizeof(float) * (size_t)nv);
    float* dy = (float*)malloc(sizeof(float) * (size_t)nv);
    ClipEntry* q = (ClipEntry*)malloc(sizeof(ClipEntry) * ((size_t)(count / 3) * (size_t)(ninst > 0 ? ninst : 1) + 1));
    int nq = 0;
    if (!cf || !dx || !dy || !q) { free(cf); free(dx); free(dy); free(q); return RSRGPU_EINVAL; }
    for (int t = 0; t < f->ntiles; ++t) {
        bb_u8(&f->tiles[t], instanced ? RSRGPU_CMD_DRAW_INLINE_INSTANCED : RSRGPU_CMD_DRAW_INLINE);
        f->mark[t] = f->tiles[t].n;
    }
    for (int iid = 0; iid < ninst; ++iid) {
    for (int v = 0; v < nv; ++v) {
        float pos[4], vary[MAX_VARY];
        shade_vertex_inst(s, vpm, iid, v, pos, vary);
        cf[v] = frustum_test(factor, pos);
        float iw = oneover(pos[3]);                       /* pdiv (rglv_math.hxx:19-23) */
        dx[v] = (pos[0] * iw) * DS[0] + DO[0];
        dy[v] = (pos[1] * iw) * DS[1] + DO[1];
    }
    const int numPrims = count / 3;
    for (int pi = 0; pi < numPrims; ++pi) {
        int i0 = (uint16_t)(cmd_is_arrays ? 3 * pi : indices[3 * pi]);
        int i1 = (uint16_t)(cmd_is_arrays ? 3 * pi + 1 : indices[3 * pi + 1]);
        int i2 = (uint16_t)(cmd_is_arrays ? 3 * pi + 2 : indices[3 * pi + 2]);
        uint32_t c0 = cf[i0], c1 = cf[i1], c2 = cf[i2];
        int pointsOutside = (int32_t)(c0 | c1 | c2) > 0;
        int primsOutside = (int32_t)(c0 & c1 & c2) > 0;
        if (!primsOutside && pointsOutside) { q[nq].iid = iid; q[nq].i0 = i0; q[nq].i1 = i1; q[nq].i2 = i2; ++nq; }
        /* rmlg::Area (rmlg_triangle.hxx:17-21) */
        float d31x = dx[i2] - dx[i0], d31y = dy[i2] - dy[i0];
        float d21x = dx[i1] - dx[i0], d21y = dy[i1] - dy[i0];
        float area = d31x * d21y - d31y * d21x;
        int front = area > 0.0f;
        int32_t ix0 = ftoi(dx[i0]), iy0 = ftoi(dy[i0]);
        int32_t ix1 = ftoi(dx[i1]), iy1 = ftoi(dy[i1]);
        int32_t ix2 = ftoi(dx[i2]), iy2 = ftoi(dy[i2]);
        int32_t vminx = imax(imin(ix0, imin(ix1, ix2)), tlx);
        int32_t vminy = imax(imin(iy0, imin(iy1, iy2)), tly);
        int32_t vmaxx = imin(wadd(imax(ix0, imax(ix1, ix2)), 1), brx);
        int32_t vmaxy = imin(wadd(imax(iy0, imax(iy1, iy2)), 1), bry);
        int notCulled = (!front && keepBacks) || (front && keepFronts);
        notCulled = notCulled && !pointsOutside;
        int accept = notCulled && (vmaxx > vminx) && (vmaxy > vminy);
        if (!accept) continue;
        int ni0 = front ? i0 : i2, ni1 = i1, ni2 = front ? i2 : i0;
        if (!front) ni0 |= 0x8000;
        int tx0 = vminx / f->tile_w, ty0 = vminy / f->tile_h;
        int tx1 = vmaxx / f->tile_w, ty1 = vmaxy / f->tile_h;
        clamp_to_grid(f, &tx0, &ty0, &tx1, &ty1);
        for (int ty = ty0; ty <= ty1; ++ty) {
            for (int tx = tx0; tx <= tx1; ++tx) {
                ByteBuf* b = &f->tiles[ty * f->tiles_x + tx];
                if (instanced) bb_u16(b, (uint16_t)iid);
                bb_u16(b, (uint16_t)ni0); bb_u16(b, (uint16_t)ni1); bb_u16(b, (uint16_t)ni2);
            }
        }
    }
    }   /* instance loop */
    for (int t = 0; t < f->ntiles; ++t) {
        if (f->tiles[t].n != f->mark[t]) bb_u16(&f->tiles[t], 0xffff);
        else f->tiles[t].n -= 1;   /* Unappend the opcode (rglv_gpu_impl.hxx:665-671) */
    }
    int rc = 0;
    if (nq) rc = clip_triangles(f, s, q, nq);
    free(cf); free(dx); free(dy); free(q);
    return rc;
}

/* ClipTriangles (rglv_gpu_impl.hxx:678-793) */
typedef struct CV { float c[4]; float d[MAX_VARY]; } CV;

static CV cv_mix(const CV* a, const CV* b, float t, int nvary, int program) {  /* CVMix, rmlv::mix (rmlv_math.hxx:87-90) */
    CV o;
    memset(&o, 0, sizeof(o));
    for (int k = 0; k < 4; ++k) o.c[k] = (1.0f - t) * a->c[k] + t * b->c[k];
    for (int k = 0; k < nvary; ++k) o.d[k] = (1.0f - t) * a->d[k] + t * b->d[k];
    if (program == RSRGPU_PROGRAM_GBUFFER) o.d[3] = a->d[3];   /* flat albedo */
    return o;
}

static int clip_triangles(Frame* f, const rsrgpu_glstate* s, const ClipEntry* q, int nq) {
    const int nvary = program_nvary(s->program_id);
    float vpm[16];
    make_vpm(s, vpm);
    float DS[2], DO[2];
    dsdo(f, s, DS, DO);
    int sc[4];
    scissor_rect(f, s, sc);
    CV A[16], B[16];
    for (int e = 0; e < nq; ++e) {
        int na = 0;
        const int idx[3] = { q[e].i0, q[e].i1, q[e].i2 };
        for (int i = 0; i < 3; ++i) {
            memset(&A[na], 0, sizeof(CV));
            shade_vertex_inst(s, vpm, q[e].iid, idx[i], A[na].c, A[na].d);
            ++na;
        }
        for (int pl = 0; pl < 5 && na > 0; ++pl) {
            const int plane = CLIP_PLANES[pl];
            int hereIsInside = is_inside(plane, A[0].c);
            int nb = 0;
            for (int h = 0; h < na; ++h) {
                const int n = (h + 1) % na;
                const int nextIsInside = is_inside(plane, A[n].c);
                if (hereIsInside) B[nb++] = A[h];
                if (hereIsInside != nextIsInside) {
                    const CV* from = hereIsInside ? &A[h] : &A[n];
                    const CV* to = hereIsInside ? &A[n] : &A[h];
                    float d = plane_distance(plane, from->c, to->c);
                    B[nb++] = cv_mix(from, to, d, nvary, s->program_id);
                    hereIsInside = !hereIsInside;
                }
            }
            memcpy(A, B, sizeof(CV) * (size_t)nb);
            na = nb;
        }
        if (na == 0) continue;
        for (int i = 0; i < na; ++i) {
            float iw = oneover(A[i].c[3]);               /* pdiv (rglv_math.hxx:143-152) */
            A[i].c[0] = A[i].c[0] * iw; A[i].c[1] = A[i].c[1] * iw; A[i].c[2] = A[i].c[2] * iw; A[i].c[3] = iw;
            A[i].c[0] = A[i].c[0] * DS[0] + DO[0];
            A[i].c[1] = A[i].c[1] * DS[1] + DO[1];
        }
        float d31x = A[2].c[0] - A[0].c[0], d31y = A[2].c[1] - A[0].c[1];
        float d21x = A[1].c[0] - A[0].c[0], d21y = A[1].c[1] - A[0].c[1];
        int backfacing = (d31x * d21y - d31y * d21x) < 0.0f;
        int willCull = 1;
        if (backfacing) { if (!s->culling_enabled || (s->cull_face & RSRGPU_GL_BACK) == 0) willCull = 0; }
        else { if (!s->culling_enabled || (s->cull_face & RSRGPU_GL_FRONT) == 0) willCull = 0; }
        if (willCull) continue;
        if (backfacing) {
            for (int i = 0; i < na / 2; ++i) { CV t = A[i]; A[i] = A[na - 1 - i]; A[na - 1 - i] = t; }
        }
        const int bi = f->nclipped;
        if (f->nclipped + na > f->capclipped) {
            int nc = f->capclipped ? f->capclipped * 2 : 256;
            while (nc < f->nclipped + na) nc *= 2;
            rsrgpu_clipped_vertex* np = (rsrgpu_clipped_vertex*)realloc(f->clipped, sizeof(*np) * (size_t)nc);
            if (!np) return RSRGPU_EINVAL;
            f->clipped = np; f->capclipped = nc;
        }
        for (int i = 0; i < na; ++i) {
            rsrgpu_clipped_vertex* o = &f->clipped[f->nclipped++];
            memset(o, 0, sizeof(*o));
            memcpy(o->coord, A[i].c, 16);
            memcpy(o->data, A[i].d, sizeof(float) * (size_t)nvary);
        }
        for (int vi = 1; vi < na - 1; ++vi) {
            const CV* p0 = &A[0]; const CV* p1 = &A[vi]; const CV* p2 = &A[vi + 1];
            /* ForEachCoveredTile (rglv_gpu_impl.hxx:796-817) */
            int32_t x0 = (int32_t)p0->c[0], y0 = (int32_t)p0->c[1];
            int32_t x1 = (int32_t)p1->c[0], y1 = (int32_t)p1->c[1];
            int32_t x2 = (int32_t)p2->c[0], y2 = (int32_t)p2->c[1];
            int vminx = imax(imin(x0, imin(x1, x2)), sc[0]);
            int vminy = imax(imin(y0, imin(y1, y2)), sc[1]);
            int vmaxx = imin(imax(x0, imax(x1, x2)) + 1, sc[2] - 1);
            int vmaxy = imin(imax(y0, imax(y1, y2)) + 1, sc[3] - 1);
            int tx0 = vminx / f->tile_w, ty0 = vminy / f->tile_h, tx1 = vmaxx / f->tile_w, ty1 = vmaxy / f->tile_h;
            clamp_to_grid(f, &tx0, &ty0, &tx1, &ty1);
            for (int ty = ty0; ty <= ty1; ++ty) {
                for (int tx = tx0; tx <= tx1; ++tx) {
                    ByteBuf* b = &f->tiles[ty * f->tiles_x + tx];
                    bb_u8(b, RSRGPU_CMD_CLIPPED_TRI);
                    bb_u16(b, (uint16_t)((bi + 0) | (backfacing ? 0x8000 : 0)));
                    bb_u16(b, (uint16_t)(bi + vi));
                    bb_u16(b, (uint16_t)(bi + vi + 1));
                }
            }
        }
    }
    return 0;
}

/* GPU::BinImpl (rglv_gpu.cxx:119-260) */
static int bin_frame(Frame* f, const uint8_t* cmds, size_t n) {
    const uint8_t* p = cmds;
    const uint8_t* end = cmds + n;
    int state = -1;
    int rc = 0;
#define RD(T, var) T var; if (p + sizeof(T) > end) return RSRGPU_EINVAL; memcpy(&var, p, sizeof(T)); p += sizeof(T)
    while (1) {
        uint8_t op = RSRGPU_CMD_EOF;
        if (p < end) { op = *p++; }
        switch (op) {
        case RSRGPU_CMD_EOF:
            for (int t = 0; t < f->ntiles; ++t) bb_u8(&f->tiles[t], RSRGPU_CMD_EOF);
            return 0;
        case RSRGPU_CMD_STATE: {
            RD(uint64_t, idx);
            if (idx >= (uint64_t)f->nstates) return RSRGPU_EINVAL;
            state = (int)idx;
            for (int t = 0; t < f->ntiles; ++t) { bb_u8(&f->tiles[t], op); bb_u64(&f->tiles[t], idx); bb_u64(&f->tiles[t], 0); }
        } break;
        case RSRGPU_CMD_CLEAR: {
            RD(uint8_t, bits);
            for (int t = 0; t < f->ntiles; ++t) { bb_u8(&f->tiles[t], op); bb_u8(&f->tiles[t], bits); }
        } break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC: {
            RD(uint8_t, gamma);
            RD(uint64_t, ptr);
            for (int t = 0; t < f->ntiles; ++t) { bb_u8(&f->tiles[t], op); bb_u8(&f->tiles[t], gamma); bb_u64(&f->tiles[t], ptr); }
        } break;
        case RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP:   /* GPU::BinImpl, rglv_gpu.cxx:156-176 */
        case RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP:
        case RSRGPU_CMD_STORE_GBUFFER: {
            RD(uint64_t, ptr);
            for (int t = 0; t < f->ntiles; ++t) { bb_u8(&f->tiles[t], op); bb_u64(&f->tiles[t], ptr); }
        } break;
        case RSRGPU_CMD_DRAW_ELEMENTS: {
            RD(uint8_t, flags); (void)flags;
            RD(uint8_t, hint); (void)hint;
            RD(int32_t, count);
            RD(uint64_t, ptr);
            if (state < 0) return RSRGPU_EINVAL;
            rc = bin_draw(f, state, count, (const uint16_t*)(uintptr_t)ptr, 0, 1, 0);
            if (rc) return rc;
        } break;
        case RSRGPU_CMD_DRAW_ARRAYS: {
            RD(int32_t, count);
            if (state < 0) return RSRGPU_EINVAL;
            rc = bin_draw(f, state, count, NULL, 1, 1, 0);
            if (rc) return rc;
        } break;
        case RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED: {   /* GPU::BinImpl, rglv_gpu.cxx:230-242 */
            RD(uint8_t, flags); (void)flags;
            RD(int32_t, count);
            RD(uint64_t, ptr);
            RD(int32_t, ninst);
            if (state < 0 || ninst < 0 || ninst > 65536) return RSRGPU_EINVAL;
            rc = bin_draw(f, state, count, (const uint16_t*)(uintptr_t)ptr, 0, ninst, 1);
            if (rc) return rc;
        } break;
        case RSRGPU_CMD_DRAW_ARRAYS_INSTANCED: {     /* rglv_gpu.cxx:204-215 */
            RD(int32_t, count);
            RD(int32_t, ninst);
            if (state < 0 || ninst < 0 || ninst > 65536) return RSRGPU_EINVAL;
            rc = bin_draw(f, state, count, NULL, 1, ninst, 1);
            if (rc) return rc;
        } break;
        default:
            return RSRGPU_EUNSUPPORTED;
        }
    }
#undef RD
}

/* ======================================================================
 * tile drawing: GPU::DrawImpl (rglv_gpu.cxx:263-432)
 * ====================================================================== */
typedef struct TileCtx {
    const Frame* f;
    int rect[4];                 /* the tile: left, top, right, bottom */
    int drect[4];                /* the draw's rectangle: the tile, cut to the scissor rectangle when
                                    the state's scissor test is on (GPUTileImpl::DrawTriangles/DrawClipped,
                                    rglv_gpu_impl.hxx:848-849,953-954) */
    int scissor;                 /* the state's scissor test is on */
    float* color;                /* tile-local rgba, row-major, tile_w*tile_h */
    float* depth;
    uint8_t* gbflag;             /* pixel's colour written by the G-buffer program */
    const rsrgpu_glstate* s;
    float vpm[16];
    float DS[2], DO[2];
    TexUnit tu0;
    int nvary;
    uint64_t frags;              /* candidate fragments: pixels inside a drawn triangle */
} TileCtx;

/* installed (program, FragmentStateKey) combinations -- the same table the
 * reference harness installs (oracle/ref/ref_harness.cxx InstallDrawStates) */
static uint32_t fragment_state_key(const rsrgpu_glstate* s) {  /* rglv_gl.hxx:136-146 */
    uint32_t key = (uint32_t)s->program_id << 24;
    key |= (uint32_t)(s->scissor_enabled != 0);
    key |= (uint32_t)(s->depth_test_enabled != 0) << 1;
    if (s->depth_test_enabled) key |= (uint32_t)s->depth_func << 2;
    key |= (uint32_t)(s->blending_enabled != 0) << 4;
    key |= (uint32_t)(s->depth_write_mask != 0) << 5;
    key |= (uint32_t)(s->color_write_mask != 0) << 6;
    key |= (uint32_t)s->color0_attachment_type << 7;
    key |= (uint32_t)s->depth_attachment_type << 9;
    return key;
}
static int draw_dispatch_ok(const rsrgpu_glstate* s) {
    if (program_nvary(s->program_id) < 0) return 0;
    if (s->program_id == RSRGPU_PROGRAM_GBUFFER && s->blending_enabled) return 0;
    uint32_t k = fragment_state_key(s) & 0xffffffu;
    k &= ~1u;   /* each state is installed with and without the scissor test */
    return k == 0x6e2 || k == 0x6e6 || k == 0x6f2 || k == 0x6c2 || k == 0x62 || k == 0x72;
}

/* TriangleProgram::Render (rglv_gpu_impl.hxx:166-222) for one quad. */
typedef struct TriSetup {
    float w[3], z[3];
    float vary[3][MAX_VARY];
} TriSetup;

static void render_quad(TileCtx* tc, const TriSetup* tri, int qx, int qy, const int32_t tri_mask[4],
                        const float bs[3][4]) {
    const rsrgpu_glstate* s = tc->s;
    const int tw = tc->f->tile_w;
    int lx[4], ly[4];
    for (int l = 0; l < 4; ++l) { lx[l] = qx + (l & 1) - tc->rect[0]; ly[l] = qy + (l >> 1) - tc->rect[1]; }
    float fragDepth[4], destDepth[4];
    int fragMask[4];
    for (int l = 0; l < 4; ++l) {
        fragDepth[l] = (bs[0][l] * tri->z[0] + bs[1][l] * tri->z[1]) + bs[2][l] * tri->z[2];
        destDepth[l] = tc->depth[ly[l] * tw + lx[l]];
    }
    /* early-Z (all installed programs have earlyZ = true, rglv_gpu_shaders.hxx:23) */
    int any = 0;
    for (int l = 0; l < 4; ++l) {
        int pass;
        if (s->depth_func == RSRGPU_GL_LESS) pass = fragDepth[l] < destDepth[l];
        else if (s->depth_func == RSRGPU_GL_LEQUAL) pass = fragDepth[l] <= destDepth[l];
        else pass = fragDepth[l] == destDepth[l];
        fragMask[l] = (tri_mask[l] == 0) && pass;
        any |= fragMask[l];
    }
    if (!any) return;
    if (s->depth_write_mask) {
        for (int l = 0; l < 4; ++l) if (fragMask[l]) tc->depth[ly[l] * tw + lx[l]] = fragDepth[l];
    }
    float bp[3][4];
    for (int l = 0; l < 4; ++l) {
        float fragW = oneover((bs[0][l] * tri->w[0] + bs[1][l] * tri->w[1]) + bs[2][l] * tri->w[2]);
        bp[0][l] = (tri->w[0] * bs[0][l]) * fragW;
        bp[2][l] = (tri->w[2] * bs[2][l]) * fragW;
        bp[1][l] = (1.0f - bp[0][l]) - bp[2][l];
    }
    float attr[4][MAX_VARY];
    for (int l = 0; l < 4; ++l)
        for (int k = 0; k < tc->nvary; ++k)
            attr[l][k] = (bp[0][l] * tri->vary[0][k] + bp[1][l] * tri->vary[1][k]) + bp[2][l] * tri->vary[2][k];
    float frag[4][4];
    if (s->program_id == RSRGPU_PROGRAM_AMY) {
        float uv[4][2];
        for (int l = 0; l < 4; ++l) { uv[l][0] = attr[l][0]; uv[l][1] = attr[l][1]; }
        tex_sample(&tc->tu0, uv, frag);
    } else if (s->program_id == RSRGPU_PROGRAM_MANY) {
        /* ManyProgram::ShadeFragment (shaders.hxx:567-582): (u, v, magic, 1) */
        for (int l = 0; l < 4; ++l) { frag[l][0] = attr[l][0]; frag[l][1] = attr[l][1]; frag[l][2] = s->uniforms[0]; frag[l][3] = 1.0f; }
    } else if (s->program_id == RSRGPU_PROGRAM_GBUFFER) {
        /* colour = interpolated normal, alpha = flat albedo of the record's first vertex */
        for (int l = 0; l < 4; ++l) { frag[l][0] = attr[l][0]; frag[l][1] = attr[l][1]; frag[l][2] = attr[l][2]; frag[l][3] = tri->vary[0][3]; }
    } else {
        for (int l = 0; l < 4; ++l) { frag[l][0] = attr[l][0]; frag[l][1] = attr[l][1]; frag[l][2] = attr[l][2]; frag[l][3] = 1.0f; }
    }
    if (s->color_write_mask) {
        for (int l = 0; l < 4; ++l) {
            if (!fragMask[l]) continue;
            float* dst = &tc->color[(ly[l] * tw + lx[l]) * 4];
            if (s->blending_enabled) {  /* BlendAlpha (:80-84) */
                float a = frag[l][3], oma = 1.0f - a;
                for (int c = 0; c < 3; ++c) dst[c] = frag[l][c] * a + dst[c] * oma;
            } else {
                for (int c = 0; c < 3; ++c) dst[c] = frag[l][c];
            }
            if (s->program_id == RSRGPU_PROGRAM_GBUFFER) { dst[3] = frag[l][3]; tc->gbflag[ly[l] * tw + lx[l]] = 1; }
            else tc->gbflag[ly[l] * tw + lx[l]] = 0;
        }
    }
}

/* quad walk shared by both rasterisers: cb* are the start-corner edge values
 * of lanes 0..3, stepping 2*dy per quad column and 2*dx per quad row */
static void walk_quads(TileCtx* tc, const TriSetup* tri, int minx, int miny, int endx, int endy,
                       const int32_t cb1s[4], const int32_t cb2s[4], const int32_t cb3s[4],
                       int32_t dy12, int32_t dx12, int32_t dy23, int32_t dx23, int32_t dy31, int32_t dx31,
                       float scale) {
    int32_t cb1[4], cb2[4], cb3[4];
    memcpy(cb1, cb1s, 16); memcpy(cb2, cb2s, 16); memcpy(cb3, cb3s, 16);
    const int32_t s1x = wmul(dy12, 2), s1y = wmul(dx12, 2);
    const int32_t s2x = wmul(dy23, 2), s2y = wmul(dx23, 2);
    const int32_t s3x = wmul(dy31, 2), s3y = wmul(dx31, 2);
    /* ScissorFlags (rglv_triangle.hxx:23-28) of the draw rectangle: with the
     * scissor test on, the lanes of quads cut by an odd edge of the rectangle
     * are masked (rglv_triangle.hxx:268-292) */
    const int* r = tc->drect;
    const int fTop = (r[1] & 1) != 0, fBot = (r[3] & 1) != 0, fLeft = (r[0] & 1) != 0, fRight = (r[2] & 1) != 0;
    for (int y = miny; y < endy; y += 2) {
        int32_t cx1[4], cx2[4], cx3[4];
        memcpy(cx1, cb1, 16); memcpy(cx2, cb2, 16); memcpy(cx3, cb3, 16);
        int32_t sTop = 0, sBot = 0;
        if (tc->scissor) {
            if (y == (r[1] & ~1) && fTop) sTop = -1;
            if (y >= (r[3] & ~1) && fBot) sBot = -1;
        }
        for (int x = minx; x < endx; x += 2) {
            int32_t edges[4];
            int allout = 1;
            for (int l = 0; l < 4; ++l) { edges[l] = cx1[l] | cx2[l] | cx3[l]; allout &= edges[l] < 0; }
            if (!allout) {
                int32_t trimask[4];
                float bs[3][4];
                int32_t sLeft = 0, sRight = 0;
                if (tc->scissor) {
                    if (x == (r[0] & ~1) && fLeft) sLeft = -1;
                    if (x >= (r[2] & ~1) && fRight) sRight = -1;
                }
                const int32_t smask[4] = { sLeft | sTop, sRight | sTop, sLeft | sBot, sRight | sBot };
                for (int l = 0; l < 4; ++l) {
                    trimask[l] = (edges[l] >> 31) | smask[l];
                    tc->frags += trimask[l] == 0;
                    bs[0][l] = itof(cx2[l]) * scale;
                    bs[2][l] = itof(cx1[l]) * scale;
                    bs[1][l] = (1.0f - bs[0][l]) - bs[2][l];
                }
                render_quad(tc, tri, x, y, trimask, bs);
            }
            for (int l = 0; l < 4; ++l) { cx1[l] = wadd(cx1[l], s1x); cx2[l] = wadd(cx2[l], s2x); cx3[l] = wadd(cx3[l], s3x); }
        }
        for (int l = 0; l < 4; ++l) { cb1[l] = wadd(cb1[l], s1y); cb2[l] = wadd(cb2[l], s2y); cb3[l] = wadd(cb3[l], s3y); }
    }
}

/* VTriangleRasterizer::Draw for one lane (rglv_triangle.hxx:193-304), int32 wrap */
static void raster_vector(TileCtx* tc, const TriSetup* tri, int32_t x1, int32_t x2, int32_t x3,
                          int32_t y1, int32_t y2, int32_t y3) {
    const int32_t* r = tc->drect;
    int32_t vminx = imax(imin(imin(x1, x2), x3) >> 4, r[0]);
    int32_t vmaxx = imin(wadd(imax(imax(x1, x2), x3), 15) >> 4, r[2]);
    int32_t vminy = imax(imin(imin(y1, y2), y3) >> 4, r[1]);
    int32_t vmaxy = imin(wadd(imax(imax(y1, y2), y3), 15) >> 4, r[3]);
    vminx &= ~1; vminy &= ~1;
    int32_t dx12 = wsub(x1, x2), dy12 = wsub(y2, y1);
    int32_t dx23 = wsub(x2, x3), dy23 = wsub(y3, y2);
    int32_t dx31 = wsub(x3, x1), dy31 = wsub(y1, y3);
    int32_t sx = wadd((int32_t)((uint32_t)vminx << 4), 8);
    int32_t sy = wadd((int32_t)((uint32_t)vminy << 4), 8);
    int32_t c1 = wadd(wmul(dy12, wsub(sx, x1)), wmul(dx12, wsub(sy, y1)));
    int32_t c2 = wadd(wmul(dy23, wsub(sx, x2)), wmul(dx23, wsub(sy, y2)));
    int32_t c3 = wadd(wmul(dy31, wsub(sx, x3)), wmul(dx31, wsub(sy, y3)));
    int tl12 = dy12 > 0 || (dy12 == 0 && dx12 > 0);
    int tl23 = dy23 > 0 || (dy23 == 0 && dx23 > 0);
    int tl31 = dy31 > 0 || (dy31 == 0 && dx31 > 0);
    c1 = wsub(wadd(c1, tl12), 1) >> 4;
    c2 = wsub(wadd(c2, tl23), 1) >> 4;
    c3 = wsub(wadd(c3, tl31), 1) >> 4;
    float scale = 1.0f / itof(wadd(wadd(c1, c2), c3));
    int32_t cb1[4] = { c1, wadd(c1, dy12), wadd(c1, dx12), wadd(wadd(c1, dx12), dy12) };
    int32_t cb2[4] = { c2, wadd(c2, dy23), wadd(c2, dx23), wadd(wadd(c2, dx23), dy23) };
    int32_t cb3[4] = { c3, wadd(c3, dy31), wadd(c3, dx31), wadd(wadd(c3, dx31), dy31) };
    walk_quads(tc, tri, vminx, vminy, vmaxx, vmaxy, cb1, cb2, cb3, dy12, dx12, dy23, dx23, dy31, dx31, scale);
}

/* TriangleRasterizer::Draw (rglv_triangle.hxx:79-167), int64 setup */
static void raster_scalar(TileCtx* tc, const TriSetup* tri, int x1, int x2, int x3, int y1, int y2, int y3) {
    const int32_t* r = tc->drect;
    int minx = imax(imin(x1, imin(x2, x3)) >> 4, r[0]);
    int endx = imin((imax(x1, imax(x2, x3)) + 15) >> 4, r[2]);
    int miny = imax(imin(y1, imin(y2, y3)) >> 4, r[1]);
    int endy = imin((imax(y1, imax(y2, y3)) + 15) >> 4, r[3]);
    minx &= ~1; miny &= ~1;
    int64_t dx12 = x1 - x2, dy12 = y2 - y1;
    int64_t dx23 = x2 - x3, dy23 = y3 - y2;
    int64_t dx31 = x3 - x1, dy31 = y1 - y3;
    int64_t sx = (minx << 4) + 8, sy = (miny << 4) + 8;
    int64_t c1 = dy12 * (sx - x1) + dx12 * (sy - y1);
    int64_t c2 = dy23 * (sx - x2) + dx23 * (sy - y2);
    int64_t c3 = dy31 * (sx - x3) + dx31 * (sy - y3);
    if (dy12 > 0 || (dy12 == 0 && dx12 > 0)) c1++;
    --c1;
    if (dy23 > 0 || (dy23 == 0 && dx23 > 0)) c2++;
    --c2;
    if (dy31 > 0 || (dy31 == 0 && dx31 > 0)) c3++;
    --c3;
    c1 >>= 4; c2 >>= 4; c3 >>= 4;
    int32_t cb1[4] = { (int32_t)c1, (int32_t)(c1 + dy12), (int32_t)(c1 + dx12), (int32_t)(c1 + dx12 + dy12) };
    int32_t cb2[4] = { (int32_t)c2, (int32_t)(c2 + dy23), (int32_t)(c2 + dx23), (int32_t)(c2 + dx23 + dy23) };
    int32_t cb3[4] = { (int32_t)c3, (int32_t)(c3 + dy31), (int32_t)(c3 + dx31), (int32_t)(c3 + dx31 + dy31) };
    float scale = 1.0f / (float)(c1 + c2 + c3);
    walk_quads(tc, tri, minx, miny, endx, endy, cb1, cb2, cb3, (int32_t)dy12, (int32_t)dx12,
               (int32_t)dy23, (int32_t)dx23, (int32_t)dy31, (int32_t)dx31, scale);
}

static const uint8_t* rd_u16(const uint8_t* p, uint16_t* v) { memcpy(v, p, 2); return p + 2; }

/* GPUTileImpl::DrawTriangles<INSTANCED> (rglv_gpu_impl.hxx:841-947): an
 * instanced record is (iid, i0|bf, i1, i2) and is shaded with its instance */
static const uint8_t* draw_inline(TileCtx* tc, const uint8_t* p, int instanced) {
    while (1) {
        uint16_t w0, i1, i2, iid = 0;
        p = rd_u16(p, &w0);
        if (w0 == 0xffff) break;
        if (instanced) { iid = w0; p = rd_u16(p, &w0); }
        p = rd_u16(p, &i1);
        p = rd_u16(p, &i2);
        const int idx[3] = { w0 & 0x7fff, i1, i2 };
        TriSetup tri;
        int32_t fx[3], fy[3];
        for (int i = 0; i < 3; ++i) {
            float pos[4];
            shade_vertex_inst(tc->s, tc->vpm, iid, idx[i], pos, tri.vary[i]);
            float iw = oneover(pos[3]);
            float dvx = pos[0] * iw, dvy = pos[1] * iw;
            tri.z[i] = pos[2] * iw;
            tri.w[i] = iw;
            fx[i] = ftoi(16.0f * (dvx * tc->DS[0] + tc->DO[0]));
            fy[i] = ftoi(16.0f * (dvy * tc->DS[1] + tc->DO[1]));
        }
        raster_vector(tc, &tri, fx[0], fx[1], fx[2], fy[0], fy[1], fy[2]);
    }
    return p;
}

/* GPUTileImpl::DrawClipped (rglv_gpu_impl.hxx:949-998) */
static const uint8_t* draw_clipped(TileCtx* tc, const uint8_t* p) {
    uint16_t w0, i1, i2;
    p = rd_u16(p, &w0); p = rd_u16(p, &i1); p = rd_u16(p, &i2);
    const int idx[3] = { w0 & 0x7fff, i1, i2 };
    TriSetup tri;
    int xs[3], ys[3];
    for (int i = 0; i < 3; ++i) {
        const rsrgpu_clipped_vertex* v = &tc->f->clipped[idx[i]];
        tri.w[i] = v->coord[3];
        tri.z[i] = v->coord[2];
        memcpy(tri.vary[i], v->data, sizeof(float) * MAX_VARY);
        xs[i] = (int)(v->coord[0] * 16.0f);
        ys[i] = (int)(v->coord[1] * 16.0f);
    }
    raster_scalar(tc, &tri, xs[0], xs[1], xs[2], ys[0], ys[1], ys[2]);
    return p;
}

/* IEEE binary32 -> binary16, round to nearest even (finite inputs) */
static uint16_t f32_to_f16(float f) {
    const uint32_t x = f2u(f);
    const uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
    const uint32_t e = (x >> 23) & 255u;
    uint32_t m = x & 0x7fffffu;
    if (e == 255u) return (uint16_t)(sign | 0x7c00u | (m ? 0x200u : 0u));
    const int exp = (int)e - 127 + 15;
    if (exp >= 31) return (uint16_t)(sign | 0x7c00u);
    if (exp <= 0) {
        if (exp < -10) return sign;
        m |= 0x800000u;
        const int shift = 14 - exp;
        uint32_t hm = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (hm & 1u))) ++hm;
        return (uint16_t)(sign | hm);
    }
    uint32_t h = ((uint32_t)exp << 10) | (m >> 13);
    const uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

static float f16_to_f32(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 31u, m = h & 0x3ffu;
    if (e == 0) {
        if (m == 0) return u2f(sign);
        int k = 0;
        while (!(m & 0x400u)) { m <<= 1; ++k; }
        m &= 0x3ffu;
        return u2f(sign | ((uint32_t)(113 - k) << 23) | (m << 13));
    }
    if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

static uint8_t srgb8(const uint8_t* lut, float v) {
    /* float_to_srgb8_var2_SSE2 (ryg-srgb.h:183-219) reproduced through the
       golden output table: clamp with maxps/minps then index by bits >> 12 */
    float c = sse_min(sse_max(v, u2f((127u - 13u) << 23)), u2f(0x3f7fffffu));
    return lut[(f2u(c) >> 12) - ((127u - 13u) << 11)];
}
static int32_t basic8(float v) {   /* to_tc_basic (rglr_canvas_util.hxx:22-31) */
    return ftoi(sse_max(sse_min(v, 1.0f), 0.0f) * 255.0f);
}

static int draw_tile(const Frame* f, int tile, float* color, float* depth, uint8_t* gbflag, uint64_t* frags) {
    TileCtx tc;
    memset(&tc, 0, sizeof(tc));
    tc.f = f;
    tc.gbflag = gbflag;
    const int tx = tile % f->tiles_x, ty = tile / f->tiles_x;
    tc.rect[0] = tx * f->tile_w; tc.rect[1] = ty * f->tile_h;
    tc.rect[2] = imin(tc.rect[0] + f->tile_w, f->width);
    tc.rect[3] = imin(tc.rect[1] + f->tile_h, f->height);
    tc.color = color; tc.depth = depth;
    const uint8_t* p = f->tiles[tile].p;
    while (1) {
        uint8_t op = *p++;
        switch (op) {
        case RSRGPU_CMD_EOF:
            *frags = tc.frags;
            return 0;
        case RSRGPU_CMD_STATE: {
            uint64_t idx;
            memcpy(&idx, p, 8); p += 16;
            tc.s = &f->states[idx];
            const int c0 = tc.s->color0_attachment_type, dt = tc.s->depth_attachment_type;
            if (!(c0 == RSRGPU_RB_COLOR_DEPTH || c0 == RSRGPU_RB_RGBAF32 || c0 == RSRGPU_RB_RGBF32)) return RSRGPU_EINVAL;
            if (!(dt == RSRGPU_RB_F32 || (dt == RSRGPU_RB_COLOR_DEPTH && c0 == RSRGPU_RB_COLOR_DEPTH))) return RSRGPU_EINVAL;
            make_vpm(tc.s, tc.vpm);
            dsdo(f, tc.s, tc.DS, tc.DO);
            memcpy(tc.drect, tc.rect, sizeof(tc.drect));
            tc.scissor = tc.s->scissor_enabled != 0;
            if (tc.scissor) {   /* Intersect(rect, gl_offset_and_size_to_irect(...)) (rmlg_irect.hxx:47-50) */
                int sc[4];
                scissor_rect(f, tc.s, sc);
                tc.drect[0] = imax(tc.rect[0], sc[0]); tc.drect[1] = imax(tc.rect[1], sc[1]);
                tc.drect[2] = imin(tc.rect[2], sc[2]); tc.drect[3] = imin(tc.rect[3], sc[3]);
            }
            tc.nvary = program_nvary(tc.s->program_id);
            if (tc.s->program_id == RSRGPU_PROGRAM_AMY && make_texture_unit(&tc.s->tus[0], &tc.tu0) != 0) return RSRGPU_EUNSUPPORTED;
        } break;
        case RSRGPU_CMD_CLEAR: {
            const uint8_t bits = *p++;
            const int n = f->tile_w * f->tile_h;
            const rsrgpu_glstate* s = tc.s;
            if (s->color0_attachment_type == RSRGPU_RB_COLOR_DEPTH) {
                if (bits != (RSRGPU_GL_COLOR_BUFFER_BIT | RSRGPU_GL_DEPTH_BUFFER_BIT)) return RSRGPU_EINVAL;
                for (int i = 0; i < n; ++i) { memcpy(&color[i * 4], s->clear_color, 12); color[i * 4 + 3] = s->clear_depth; depth[i] = s->clear_depth; gbflag[i] = 0; }
            } else {
                if (bits & RSRGPU_GL_COLOR_BUFFER_BIT) for (int i = 0; i < n; ++i) { memcpy(&color[i * 4], s->clear_color, 16); gbflag[i] = 0; }
                if (bits & RSRGPU_GL_DEPTH_BUFFER_BIT) for (int i = 0; i < n; ++i) depth[i] = s->clear_depth;
            }
        } break;
        case RSRGPU_CMD_DRAW_INLINE:
        case RSRGPU_CMD_DRAW_INLINE_INSTANCED:
            if (!draw_dispatch_ok(tc.s)) return RSRGPU_ENODISPATCH;
            p = draw_inline(&tc, p, op == RSRGPU_CMD_DRAW_INLINE_INSTANCED);
            break;
        case RSRGPU_CMD_CLIPPED_TRI:
            if (!draw_dispatch_ok(tc.s)) return RSRGPU_ENODISPATCH;
            p = draw_clipped(&tc, p);
            break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC: {
            /* GPUBltImpl::StoreTrueColor -> FilterTile (rglr_algorithm.hxx:31-104) */
            const uint8_t gamma = *p++;
            uint64_t cp;
            memcpy(&cp, p, 8); p += 8;
            const int pid = tc.s->program_id;
            if (!(pid == RSRGPU_PROGRAM_DEFAULT_POST || pid == RSRGPU_PROGRAM_EXPOSURE_POST || pid == RSRGPU_PROGRAM_GOURAUD))
                return RSRGPU_ENODISPATCH;
            if (gamma && !f->srgb_lut) return RSRGPU_EINVAL;
            const rsrgpu_truecolor_canvas* cv = (const rsrgpu_truecolor_canvas*)(uintptr_t)cp;
            const float ex = (pid == RSRGPU_PROGRAM_EXPOSURE_POST) ? tc.s->uniforms[0] : 1.0f;
            for (int y = tc.rect[1]; y < tc.rect[3]; ++y) {
                for (int x = tc.rect[0]; x < tc.rect[2]; ++x) {
                    const float* src = &color[((y - tc.rect[1]) * f->tile_w + (x - tc.rect[0])) * 4];
                    float rgb[3] = { src[0], src[1], src[2] };
                    if (pid == RSRGPU_PROGRAM_EXPOSURE_POST) for (int c = 0; c < 3; ++c) rgb[c] = rgb[c] * ex;
                    uint32_t px;
                    if (gamma) px = ((uint32_t)srgb8(f->srgb_lut, rgb[0]) << 16) | ((uint32_t)srgb8(f->srgb_lut, rgb[1]) << 8) | srgb8(f->srgb_lut, rgb[2]);
                    else px = ((uint32_t)basic8(rgb[0]) << 16) | ((uint32_t)basic8(rgb[1]) << 8) | (uint32_t)basic8(rgb[2]);
                    cv->data[(size_t)y * cv->stride + x] = px;
                }
            }
        } break;
        case RSRGPU_CMD_STORE_GBUFFER: {
            uint64_t gp;
            memcpy(&gp, p, 8); p += 8;
            const rsrgpu_gbuffer* gb = (const rsrgpu_gbuffer*)(uintptr_t)gp;
            for (int y = tc.rect[1]; y < tc.rect[3]; ++y) {
                for (int x = tc.rect[0]; x < tc.rect[2]; ++x) {
                    const int li = (y - tc.rect[1]) * f->tile_w + (x - tc.rect[0]);
                    const size_t o = (size_t)y * f->width + x;
                    gb->depth[o] = depth[li];
                    if (gbflag[li]) {
                        gb->normal_x[o] = f32_to_f16(color[li * 4 + 0]);
                        gb->normal_y[o] = f32_to_f16(color[li * 4 + 1]);
                        gb->normal_z[o] = f32_to_f16(color[li * 4 + 2]);
                        gb->albedo[o] = (uint32_t)color[li * 4 + 3] | 0xff000000u;
                    } else {
                        gb->normal_x[o] = gb->normal_y[o] = gb->normal_z[o] = 0;
                        gb->albedo[o] = 0;
                    }
                }
            }
        } break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP: {
            /* GPU::DrawImpl, rglv_gpu.cxx:345-383: the tile's RGB colour
               (an RB_RGBF32 QFloat3 buffer or the rgb of RB_COLOR_DEPTH's
               QFloat4 buffer, whose w is the depth) copied out as float */
            uint64_t cp;
            memcpy(&cp, p, 8); p += 8;
            const int c0 = tc.s->color0_attachment_type;
            if (c0 != RSRGPU_RB_RGBF32 && c0 != RSRGPU_RB_COLOR_DEPTH) return RSRGPU_EUNSUPPORTED;
            const rsrgpu_fp_canvas* cv = (const rsrgpu_fp_canvas*)(uintptr_t)cp;
            for (int y = tc.rect[1]; y < tc.rect[3]; y += 2) {
                for (int x = tc.rect[0]; x < tc.rect[2]; x += 2) {
                    /* the quad's lanes: (x,y) (x+1,y) (x,y+1) (x+1,y+1) */
                    const float* px[4];
                    float dq[4];
                    for (int l = 0; l < 4; ++l) {
                        const int li = (y + (l >> 1) - tc.rect[1]) * f->tile_w + (x + (l & 1) - tc.rect[0]);
                        px[l] = &color[li * 4];
                        dq[l] = depth[li];
                    }
                    if (op == RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP) {
                        /* Copy(QFloat3Canvas|QFloat4Canvas -> FloatingPointCanvas),
                           rglr_algorithm.cxx:192-225,247-280: the transpose of
                           (r, g, b, zero) quads gives (r, g, b, 0) pixels */
                        for (int l = 0; l < 4; ++l) {
                            float* d = cv->data + ((size_t)(y + (l >> 1)) * cv->stride + (x + (l & 1))) * 4;
                            d[0] = px[l][0]; d[1] = px[l][1]; d[2] = px[l][2]; d[3] = 0.0f;
                        }
                    } else if (op == RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP) {
                        /* Downsample, rglr_algorithm.cxx:118-168: the four
                           (r, g, b, 0) pixels added in lane order, times 0.25 */
                        float* d = cv->data + ((size_t)(y / 2) * cv->stride + x / 2) * 4;
                        for (int c = 0; c < 3; ++c) d[c] = (((px[0][c] + px[1][c]) + px[2][c]) + px[3][c]) * 0.25f;
                        d[3] = (((0.0f + 0.0f) + 0.0f) + 0.0f) * 0.25f;
                    } else {
                        /* Copy(QFloat3Canvas -> QFloat4Canvas) sets w to 1,
                           Copy(QFloat4Canvas -> QFloat4Canvas) keeps it (the
                           depth of RB_COLOR_DEPTH), rglr_algorithm.cxx:320-372 */
                        float* q = cv->data + ((size_t)(y / 2) * cv->stride + x / 2) * 16;
                        for (int l = 0; l < 4; ++l) {
                            q[l] = px[l][0]; q[4 + l] = px[l][1]; q[8 + l] = px[l][2];
                            q[12 + l] = c0 == RSRGPU_RB_COLOR_DEPTH ? dq[l] : 1.0f;
                        }
                    }
                }
            }
        } break;
        case RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP: {
            uint64_t dp;
            memcpy(&dp, p, 8); p += 8;
            if (tc.s->depth_attachment_type != RSRGPU_RB_F32) return RSRGPU_EUNSUPPORTED;
            float* dst = (float*)(uintptr_t)dp;
            for (int y = tc.rect[1]; y < tc.rect[3]; ++y)
                for (int x = tc.rect[0]; x < tc.rect[2]; ++x)
                    dst[(size_t)y * f->width + x] = depth[(y - tc.rect[1]) * f->tile_w + (x - tc.rect[0])];
        } break;
        default:
            return RSRGPU_EINVAL;
        }
    }
}

/* ---- tile jobs over a thread pool (replaces the jobsys Draw jobs) ---- */
typedef struct Pool {
    const Frame* f;
    int next;
    int rc;
    uint64_t frags;
    pthread_mutex_t mu;
} Pool;

static void* tile_worker(void* arg) {
    Pool* pool = (Pool*)arg;
    const Frame* f = pool->f;
    float* color = (float*)malloc(sizeof(float) * 4 * (size_t)f->tile_w * (size_t)f->tile_h);
    float* depth = (float*)malloc(sizeof(float) * (size_t)f->tile_w * (size_t)f->tile_h);
    uint8_t* gbflag = (uint8_t*)calloc((size_t)f->tile_w * (size_t)f->tile_h, 1);
    while (1) {
        pthread_mutex_lock(&pool->mu);
        int t = pool->next++;
        pthread_mutex_unlock(&pool->mu);
        if (t >= f->ntiles) break;
        uint64_t frags = 0;
        int rc = draw_tile(f, t, color, depth, gbflag, &frags);
        pthread_mutex_lock(&pool->mu);
        pool->frags += frags;
        pthread_mutex_unlock(&pool->mu);
        if (rc) { pthread_mutex_lock(&pool->mu); pool->rc = rc; pthread_mutex_unlock(&pool->mu); }
    }
    free(color); free(depth); free(gbflag);
    return NULL;
}

/* ======================================================================
 * C entry points (same shape as oracle/ref/ref_harness.cxx)
 * ====================================================================== */
int rsroracle_init(int threads) {
    g_session.threads = threads > 0 ? threads : 1;
    return 0;
}

int rsroracle_set_srgb_lut(const uint8_t* lut, int n) {
    if (n != 26624) return RSRGPU_EINVAL;
    free(g_session.srgb_lut);
    g_session.srgb_lut = (uint8_t*)malloc((size_t)n);
    memcpy(g_session.srgb_lut, lut, (size_t)n);
    return 0;
}

static void frame_free(Frame* f) {
    if (f->tiles) for (int t = 0; t < f->ntiles; ++t) free(f->tiles[t].p);
    free(f->tiles); free(f->mark); free(f->clipped);
    memset(f, 0, sizeof(*f));
}

int rsroracle_render(const uint8_t* cmds, size_t n, const rsrgpu_glstate* states, int nstates,
                     int width, int height, int tile_blocks_x, int tile_blocks_y) {
    Frame* f = &g_session.f;
    frame_free(f);
    if (width <= 0 || height <= 0 || tile_blocks_x <= 0 || tile_blocks_y <= 0) return RSRGPU_EINVAL;
    f->width = width; f->height = height;
    f->tile_w = tile_blocks_x * 8; f->tile_h = tile_blocks_y * 8;
    if (f->tile_w > 128 || f->tile_h > 128) return RSRGPU_EINVAL;
    f->tiles_x = (width + f->tile_w - 1) / f->tile_w;
    f->tiles_y = (height + f->tile_h - 1) / f->tile_h;
    f->ntiles = f->tiles_x * f->tiles_y;
    f->states = states; f->nstates = nstates;
    f->srgb_lut = g_session.srgb_lut;
    f->tiles = (ByteBuf*)calloc((size_t)f->ntiles, sizeof(ByteBuf));
    f->mark = (size_t*)calloc((size_t)f->ntiles, sizeof(size_t));
    if (!f->tiles || !f->mark) return RSRGPU_EINVAL;
    int rc = bin_frame(f, cmds, n);
    if (rc) return rc;
    Pool pool;
    pool.f = f; pool.next = 0; pool.rc = 0; pool.frags = 0;
    pthread_mutex_init(&pool.mu, NULL);
    int nt = g_session.threads;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    for (int i = 1; i < nt; ++i) pthread_create(&th[i], NULL, tile_worker, &pool);
    tile_worker(&pool);
    for (int i = 1; i < nt; ++i) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&pool.mu);
    f->frags = pool.frags;
    return pool.rc;
}

/* candidate fragments of the last frame: (pixel, triangle) pairs whose pixel
 * centre the rasteriser's coverage test accepts, before the depth test */
int rsroracle_candidate_fragments(uint64_t* out) {
    if (out == NULL) return RSRGPU_EINVAL;
    *out = g_session.f.frags;
    return 0;
}

/* canonical tile streams (same layout as rsrgpu_dump_tiles / rsrref_dump_tiles) */
int rsroracle_dump_tiles(uint8_t* out, size_t capacity, size_t* needed) {
    const Frame* f = &g_session.f;
    ByteBuf all = { 0 };
    ByteBuf one = { 0 };
    uint32_t ord_of[4096];
    int nord = 0;
    uint64_t ord_key[4096];
    for (int t = 0; t < f->ntiles; ++t) {
        one.n = 0;
        const uint8_t* p = f->tiles[t].p;
        int done = 0;
        while (!done) {
            uint8_t op = *p++;
            bb_u8(&one, op);
            switch (op) {
            case RSRGPU_CMD_EOF: done = 1; break;
            case RSRGPU_CMD_STATE: {
                uint64_t idx; memcpy(&idx, p, 8); p += 16;
                int k;
                for (k = 0; k < nord; ++k) if (ord_key[k] == idx) break;
                if (k == nord && nord < 4096) { ord_key[nord] = idx; ord_of[nord] = (uint32_t)nord; ++nord; }
                uint32_t o = ord_of[k];
                bb_put(&one, &o, 4);
            } break;
            case RSRGPU_CMD_CLEAR: bb_u8(&one, *p++); break;
            case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC: bb_u8(&one, *p++); p += 8; break;
            case RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP: p += 8; break;
            case RSRGPU_CMD_STORE_GBUFFER: p += 8; break;
            case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP:
            case RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP:
            case RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP: p += 8; break;
            case RSRGPU_CMD_DRAW_INLINE:
            case RSRGPU_CMD_DRAW_INLINE_INSTANCED:
                while (1) {
                    uint16_t w; p = rd_u16(p, &w); bb_u16(&one, w);
                    if (w == 0xffff) break;
                    if (op == RSRGPU_CMD_DRAW_INLINE_INSTANCED) { p = rd_u16(p, &w); bb_u16(&one, w); }
                    p = rd_u16(p, &w); bb_u16(&one, w);
                    p = rd_u16(p, &w); bb_u16(&one, w);
                }
                break;
            case RSRGPU_CMD_CLIPPED_TRI:
                for (int k = 0; k < 3; ++k) { uint16_t w; p = rd_u16(p, &w); bb_u16(&one, w); }
                break;
            default: done = 1; break;
            }
        }
        uint32_t len = (uint32_t)one.n;
        bb_put(&all, &len, 4);
        bb_put(&all, one.p, one.n);
    }
    *needed = all.n;
    if (out && capacity >= all.n) memcpy(out, all.p, all.n);
    free(all.p); free(one.p);
    return 0;
}

int rsroracle_dump_clipped(rsrgpu_clipped_vertex* out, int capacity, int* count) {
    const Frame* f = &g_session.f;
    *count = f->nclipped;
    for (int i = 0; i < f->nclipped && i < capacity; ++i) out[i] = f->clipped[i];
    return 0;
}

/* The rasteriser known-answer test of rglv_triangle.t.cxx:208-288: the scalar
 * rasteriser on an 8x8 target with a program that writes BS.x where the
 * cmple depth test passes; returns the "X where BS.x > 0" mask. */
int rsroracle_kat_top_left(const float pts[6], int w, int h, uint8_t* mask) {
    if (w > 128 || h > 128) return RSRGPU_EINVAL;
    int xs[3], ys[3];
    for (int i = 0; i < 3; ++i) { xs[i] = (int)(16.0f * pts[2 * i]); ys[i] = (int)(16.0f * pts[2 * i + 1]); }
    int minx = imax(imin(xs[0], imin(xs[1], xs[2])) >> 4, 0);
    int endx = imin((imax(xs[0], imax(xs[1], xs[2])) + 15) >> 4, w);
    int miny = imax(imin(ys[0], imin(ys[1], ys[2])) >> 4, 0);
    int endy = imin((imax(ys[0], imax(ys[1], ys[2])) + 15) >> 4, h);
    minx &= ~1; miny &= ~1;
    int64_t dx12 = xs[0] - xs[1], dy12 = ys[1] - ys[0];
    int64_t dx23 = xs[1] - xs[2], dy23 = ys[2] - ys[1];
    int64_t dx31 = xs[2] - xs[0], dy31 = ys[0] - ys[2];
    int64_t sx = (minx << 4) + 8, sy = (miny << 4) + 8;
    int64_t c1 = dy12 * (sx - xs[0]) + dx12 * (sy - ys[0]);
    int64_t c2 = dy23 * (sx - xs[1]) + dx23 * (sy - ys[1]);
    int64_t c3 = dy31 * (sx - xs[2]) + dx31 * (sy - ys[2]);
    if (dy12 > 0 || (dy12 == 0 && dx12 > 0)) c1++;
    --c1;
    if (dy23 > 0 || (dy23 == 0 && dx23 > 0)) c2++;
    --c2;
    if (dy31 > 0 || (dy31 == 0 && dx31 > 0)) c3++;
    --c3;
    c1 >>= 4; c2 >>= 4; c3 >>= 4;
    float scale = 1.0f / (float)(c1 + c2 + c3);
    memset(mask, 0, (size_t)(w * h));
    for (int y = miny; y < endy; y += 2) {
        for (int x = minx; x < endx; x += 2) {
            for (int l = 0; l < 4; ++l) {
                int64_t e1 = c1 + (x - minx + (l & 1)) * dy12 + (y - miny + (l >> 1)) * dx12;
                int64_t e2 = c2 + (x - minx + (l & 1)) * dy23 + (y - miny + (l >> 1)) * dx23;
                int64_t e3 = c3 + (x - minx + (l & 1)) * dy31 + (y - miny + (l >> 1)) * dx31;
                int32_t edges = (int32_t)e1 | (int32_t)e2 | (int32_t)e3;
                if (edges < 0) continue;
                float bsx = itof((int32_t)e2) * scale;
                int px = x + (l & 1), py = y + (l >> 1);
                if (px < w && py < h && bsx > 0.0f) mask[py * w + px] = 1;
            }
        }
    }
    return 0;
}


/* ======================================================================
 * deferred plain shading (this library's extension; no rsr counterpart)
 * Same definition and operation order as shade_plain_kernel in
 * rsr_gb300/csrc/rsrgpu_deferred.cu.
 * ====================================================================== */
static float dot3(float ax, float ay, float az, float bx, float by, float bz) { return (ax * bx + ay * by) + az * bz; }
static float pos0(float x) { return x > 0.0f ? x : 0.0f; }

typedef struct PlainJob {
    const rsrgpu_gbuffer* gb;
    const float* ivp; const float* eye; const rsrgpu_light* lights; int nlights;
    const float* bg; float* out_linear; int next; pthread_mutex_t mu;
} PlainJob;

static void plain_row(const PlainJob* j, int y) {
    const rsrgpu_gbuffer* g = j->gb;
    const float* m = j->ivp;
    for (int x = 0; x < g->width; ++x) {
        const size_t i = (size_t)y * g->width + x;
        float* o = j->out_linear + 3 * i;
        const uint32_t alb = g->albedo[i];
        if (alb == 0) { o[0] = j->bg[0]; o[1] = j->bg[1]; o[2] = j->bg[2]; continue; }
        const float z = g->depth[i];
        const float ndcx = (2.0f * ((float)x + 0.5f)) / (float)g->width - 1.0f;
        const float ndcy = 1.0f - (2.0f * ((float)y + 0.5f)) / (float)g->height;
        const float cx = ((m[0] * ndcx + m[4] * ndcy) + m[8] * z) + m[12];
        const float cy = ((m[1] * ndcx + m[5] * ndcy) + m[9] * z) + m[13];
        const float cz = ((m[2] * ndcx + m[6] * ndcy) + m[10] * z) + m[14];
        const float cw = ((m[3] * ndcx + m[7] * ndcy) + m[11] * z) + m[15];
        const float px = cx / cw, py = cy / cw, pz = cz / cw;
        float nx = f16_to_f32(g->normal_x[i]), ny = f16_to_f32(g->normal_y[i]), nz = f16_to_f32(g->normal_z[i]);
        const float nlen = sqrtf(dot3(nx, ny, nz, nx, ny, nz));
        nx = nx / nlen; ny = ny / nlen; nz = nz / nlen;
        float vx = j->eye[0] - px, vy = j->eye[1] - py, vz = j->eye[2] - pz;
        const float vlen = sqrtf(dot3(vx, vy, vz, vx, vy, vz));
        vx = vx / vlen; vy = vy / vlen; vz = vz / vlen;
        const float ar = (float)(alb & 255u) / 255.0f, ag = (float)((alb >> 8) & 255u) / 255.0f, ab = (float)((alb >> 16) & 255u) / 255.0f;
        float sr = 0.0f, sg = 0.0f, sb = 0.0f;
        for (int k = 0; k < j->nlights; ++k) {
            const rsrgpu_light* L = &j->lights[k];
            float lx = L->position[0] - px, ly = L->position[1] - py, lz = L->position[2] - pz;
            const float d = sqrtf(dot3(lx, ly, lz, lx, ly, lz));
            if (!(d < L->radius)) continue;
            lx = lx / d; ly = ly / d; lz = lz / d;
            const float t = 1.0f - d / L->radius;
            const float att = t * t;
            const float ndl = pos0(dot3(nx, ny, nz, lx, ly, lz));
            float hx = lx + vx, hy = ly + vy, hz = lz + vz;
            const float hlen = sqrtf(dot3(hx, hy, hz, hx, hy, hz));
            hx = hx / hlen; hy = hy / hlen; hz = hz / hlen;
            float sp = pos0(dot3(nx, ny, nz, hx, hy, hz));
            sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp;
            sr = sr + (L->color[0] * att) * (ar * ndl + sp);
            sg = sg + (L->color[1] * att) * (ag * ndl + sp);
            sb = sb + (L->color[2] * att) * (ab * ndl + sp);
        }
        o[0] = sr + 0.03f * ar; o[1] = sg + 0.03f * ag; o[2] = sb + 0.03f * ab;
    }
}

static void* plain_worker(void* arg) {
    PlainJob* j = (PlainJob*)arg;
    while (1) {
        pthread_mutex_lock(&j->mu);
        int y = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (y >= j->gb->height) break;
        plain_row(j, y);
    }
    return NULL;
}

int rsroracle_shade_plain(const rsrgpu_gbuffer* gb, const float ivp[16], const float eye[3],
                          const rsrgpu_light* lights, int nlights, const float background[3], float* out_linear) {
    PlainJob j;
    j.gb = gb; j.ivp = ivp; j.eye = eye; j.lights = lights; j.nlights = nlights; j.bg = background;
    j.out_linear = out_linear; j.next = 0;
    pthread_mutex_init(&j.mu, NULL);
    int nt = g_session.threads;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    for (int i = 1; i < nt; ++i) pthread_create(&th[i], NULL, plain_worker, &j);
    plain_worker(&j);
    for (int i = 1; i < nt; ++i) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return 0;
}

/* ---- learned deferred shader: inputs (the CUDA feature builder's restatement) ----
 * Shading tiles of 32x32 pixels.  Per tile: the world-space box of its covered
 * pixels, each light's score (1 - d/r)^2 * (r + g + b) at the box point nearest
 * the light (or -1 when d >= r), and up to 8 candidates in descending score,
 * ties to the lower index, scores > 0 only.  Per covered pixel 24 features:
 * unit normal, unit view vector, albedo, eye distance / 50, then over the
 * candidates reaching the pixel (att = (1 - d/r)^2, c = colour * att,
 * w = c.r + c.g + c.b, L unit direction to the light): sum c, sum w L,
 * sum w L L^T (xx xy xz yy yz zz), sum w max(N.L, 0), sum w (d/r) / sum w. */
#define SHADE_TILE 32
#define NCAND 8

static void world_pos(const rsrgpu_gbuffer* g, const float* m, int x, int y, float P[3]) {
    const float z = g->depth[(size_t)y * g->width + x];
    const float ndcx = (2.0f * ((float)x + 0.5f)) / (float)g->width - 1.0f;
    const float ndcy = 1.0f - (2.0f * ((float)y + 0.5f)) / (float)g->height;
    const float cx = ((m[0] * ndcx + m[4] * ndcy) + m[8] * z) + m[12];
    const float cy = ((m[1] * ndcx + m[5] * ndcy) + m[9] * z) + m[13];
    const float cz = ((m[2] * ndcx + m[6] * ndcy) + m[10] * z) + m[14];
    const float cw = ((m[3] * ndcx + m[7] * ndcy) + m[11] * z) + m[15];
    P[0] = cx / cw; P[1] = cy / cw; P[2] = cz / cw;
}

static float light_score(const rsrgpu_light* l, const float b0[3], const float b1[3]) {
    float e[3];
    for (int k = 0; k < 3; ++k) {
        const float c = fminf(fmaxf(l->position[k], b0[k]), b1[k]);
        e[k] = l->position[k] - c;
    }
    const float d = sqrtf(dot3(e[0], e[1], e[2], e[0], e[1], e[2]));
    if (!(d < l->radius)) return -1.0f;
    const float t = 1.0f - d / l->radius;
    return (t * t) * ((l->color[0] + l->color[1]) + l->color[2]);
}

static uint16_t bf16_rne(float x) {
    uint32_t u = f2u(x);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

int rsroracle_learned_candidates(const rsrgpu_gbuffer* g, const float ivp[16], const rsrgpu_light* lights,
                                 int nlights, int tile, int32_t cand[NCAND]) {
    const int tiles_x = (g->width + SHADE_TILE - 1) / SHADE_TILE;
    const int x0 = (tile % tiles_x) * SHADE_TILE, y0 = (tile / tiles_x) * SHADE_TILE;
    float b0[3] = { INFINITY, INFINITY, INFINITY }, b1[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (int y = y0; y < y0 + SHADE_TILE && y < g->height; ++y)
        for (int x = x0; x < x0 + SHADE_TILE && x < g->width; ++x) {
            if (g->albedo[(size_t)y * g->width + x] == 0) continue;
            float P[3];
            world_pos(g, ivp, x, y, P);
            for (int k = 0; k < 3; ++k) { b0[k] = fminf(b0[k], P[k]); b1[k] = fmaxf(b1[k], P[k]); }
        }
    float score[256];
    const int empty = !(b0[0] <= b1[0]);
    for (int i = 0; i < nlights && i < 256; ++i) score[i] = empty ? -1.0f : light_score(&lights[i], b0, b1);
    for (int c = 0; c < NCAND; ++c) {
        int best = -1;
        float bs = 0.0f;
        for (int i = 0; i < nlights && i < 256; ++i)
            if (score[i] > bs) { bs = score[i]; best = i; }
        cand[c] = best;
        if (best >= 0) score[best] = -1.0f;
    }
    return 0;
}

/* returns the number of candidate lights reaching the pixel */
static int pixel_features(const rsrgpu_gbuffer* g, const float* ivp, const float* eye, const rsrgpu_light* lights,
                          const int32_t* cand, int x, int y, float f[24]) {
    const size_t i = (size_t)y * g->width + x;
    float P[3];
    world_pos(g, ivp, x, y, P);
    float nx = f16_to_f32(g->normal_x[i]), ny = f16_to_f32(g->normal_y[i]), nz = f16_to_f32(g->normal_z[i]);
    const float nlen = sqrtf(dot3(nx, ny, nz, nx, ny, nz));
    nx = nx / nlen; ny = ny / nlen; nz = nz / nlen;
    float vx = eye[0] - P[0], vy = eye[1] - P[1], vz = eye[2] - P[2];
    const float vlen = sqrtf(dot3(vx, vy, vz, vx, vy, vz));
    vx = vx / vlen; vy = vy / vlen; vz = vz / vlen;
    const uint32_t alb = g->albedo[i];
    f[0] = nx; f[1] = ny; f[2] = nz; f[3] = vx; f[4] = vy; f[5] = vz;
    f[6] = (float)(alb & 255u) / 255.0f; f[7] = (float)((alb >> 8) & 255u) / 255.0f; f[8] = (float)((alb >> 16) & 255u) / 255.0f;
    f[9] = vlen / 50.0f;
    for (int k = 10; k < 24; ++k) f[k] = 0.0f;
    float wsum = 0.0f;
    int reach = 0;
    for (int c = 0; c < NCAND; ++c) {
        if (cand[c] < 0) break;
        const rsrgpu_light* l = &lights[cand[c]];
        float lx = l->position[0] - P[0], ly = l->position[1] - P[1], lz = l->position[2] - P[2];
        const float d = sqrtf(dot3(lx, ly, lz, lx, ly, lz));
        if (!(d < l->radius)) continue;
        ++reach;
        const float q = d / l->radius;
        const float t = 1.0f - q;
        const float att = t * t;
        const float cr = l->color[0] * att, cg = l->color[1] * att, cb = l->color[2] * att;
        const float w = (cr + cg) + cb;
        lx = lx / d; ly = ly / d; lz = lz / d;
        const float wx = w * lx, wy = w * ly, wz = w * lz;
        f[10] = f[10] + cr; f[11] = f[11] + cg; f[12] = f[12] + cb;
        f[13] = f[13] + wx; f[14] = f[14] + wy; f[15] = f[15] + wz;
        f[16] = f[16] + wx * lx; f[17] = f[17] + wx * ly; f[18] = f[18] + wx * lz;
        f[19] = f[19] + wy * ly; f[20] = f[20] + wy * lz; f[21] = f[21] + wz * lz;
        f[22] = f[22] + w * pos0(dot3(nx, ny, nz, lx, ly, lz));
        f[23] = f[23] + w * q;
        wsum = wsum + w;
    }
    f[23] = wsum > 0.0f ? f[23] / wsum : 0.0f;
    return reach;
}

/* The analytic base the network's output is added to: one virtual light with
 * direction sum w L (normalised) and colour sum c, Blinn-Phong exponent 32 plus
 * ambient 0.03 * albedo, square root per channel. */
static void virtual_light_base(const float* f, float base[3]) {
    const float dlen = sqrtf(dot3(f[13], f[14], f[15], f[13], f[14], f[15]));
    float l[3] = { 0.0f, 0.0f, 0.0f };
    if (dlen > 0.0f) { l[0] = f[13] / dlen; l[1] = f[14] / dlen; l[2] = f[15] / dlen; }
    float h[3] = { l[0] + f[3], l[1] + f[4], l[2] + f[5] };
    const float hlen = sqrtf(dot3(h[0], h[1], h[2], h[0], h[1], h[2]));
    if (hlen > 0.0f) { h[0] = h[0] / hlen; h[1] = h[1] / hlen; h[2] = h[2] / hlen; }
    const float ndl = pos0(dot3(f[0], f[1], f[2], l[0], l[1], l[2]));
    float sp = pos0(dot3(f[0], f[1], f[2], h[0], h[1], h[2]));
    sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp; sp = sp * sp;
    for (int c = 0; c < 3; ++c) base[c] = sqrtf(pos0(f[10 + c] * (f[6 + c] * ndl + sp) + 0.03f * f[6 + c]));
}

/* features (bf16 [W*H][32]), features_f32 ([W*H][24], optional), targets
 * ([W*H][3] sqrt(max(plain, 0)) - base, optional), base ([W*H][3], optional),
 * candidates ([tiles][8], optional), reach ([W*H], optional: candidate lights
 * reaching the pixel); uncovered pixels give zero rows */
int rsroracle_learned_features(const rsrgpu_gbuffer* g, const float ivp[16], const float eye[3],
                               const rsrgpu_light* lights, int nlights, uint16_t* features, float* features_f32,
                               float* targets, float* base, int32_t* candidates, uint8_t* reach) {
    const int tiles_x = (g->width + SHADE_TILE - 1) / SHADE_TILE, tiles_y = (g->height + SHADE_TILE - 1) / SHADE_TILE;
    const size_t npx = (size_t)g->width * g->height;
    float* plain = NULL;
    if (targets) {
        static const float bg[3] = { 0.0f, 0.0f, 0.0f };
        plain = (float*)malloc(npx * 12);
        if (!plain) return -1;
        rsroracle_shade_plain(g, ivp, eye, lights, nlights, bg, plain);
    }
    for (int tile = 0; tile < tiles_x * tiles_y; ++tile) {
        int32_t cand[NCAND];
        rsroracle_learned_candidates(g, ivp, lights, nlights, tile, cand);
        if (candidates) memcpy(candidates + (size_t)tile * NCAND, cand, sizeof(cand));
        const int x0 = (tile % tiles_x) * SHADE_TILE, y0 = (tile / tiles_x) * SHADE_TILE;
        for (int y = y0; y < y0 + SHADE_TILE && y < g->height; ++y)
            for (int x = x0; x < x0 + SHADE_TILE && x < g->width; ++x) {
                const size_t i = (size_t)y * g->width + x;
                float f[24];
                const int covered = g->albedo[i] != 0;
                int nr = 0;
                if (covered) nr = pixel_features(g, ivp, eye, lights, cand, x, y, f);
                else for (int k = 0; k < 24; ++k) f[k] = 0.0f;
                if (reach) reach[i] = (uint8_t)nr;
                for (int k = 0; k < 32; ++k) features[i * 32 + k] = k < 24 ? bf16_rne(f[k]) : 0;
                if (features_f32) memcpy(features_f32 + i * 24, f, sizeof(f));
                float b[3] = { 0.0f, 0.0f, 0.0f };
                if (covered) virtual_light_base(f, b);
                if (base) memcpy(base + i * 3, b, sizeof(b));
                if (targets)
                    for (int c = 0; c < 3; ++c) targets[i * 3 + c] = covered ? sqrtf(pos0(plain[i * 3 + c])) - b[c] : 0.0f;
            }
    }
    free(plain);
    return 0;
}


/* ======================================================================
 * texture upload and mip chain (test infrastructure: the oracle of
 * rsrgpu_texture_from_rgba8 / rsrgpu_texture_mipmap)
 * ====================================================================== */

/* Texture::maybe_make_mipmap's size test (src/rgl/rglr/rglr_texture.cxx:35-50) */
static int texture_power(int w, int h) {
    if (w != h || w <= 0 || (w & (w - 1)) != 0) return -1;
    const int p = ilog2u((unsigned)w);
    return p > 12 ? -1 : p;
}

/* Texture::maybe_make_mipmap (rglr_texture.cxx:33-80): the buffer grows to
   w*w*2 zeroed texels past level 0, then each level is written below the
   previous one with the level-0 row stride, texel = (((a + b) + c) + d) / 4 */
static void make_mipmap(float* buf, int w, int p) {
    memset(buf + (size_t)w * w * 4, 0, sizeof(float) * 4 * (size_t)w * w);
    int src_size = w;
    size_t src = 0, dst = (size_t)w * w;
    for (int level = p - 1; level >= 0; --level) {
        for (int sy = 0; sy < src_size; sy += 2) {
            size_t drow = dst;
            for (int sx = 0; sx < src_size; sx += 2) {
                const float* a = buf + (src + (size_t)sy * w + sx) * 4;
                const float* c = buf + (src + (size_t)(sy + 1) * w + sx) * 4;
                float* d = buf + drow * 4;
                for (int k = 0; k < 4; ++k) d[k] = (((a[k] + a[4 + k]) + c[k]) + c[4 + k]) / 4.0f;
                ++drow;
            }
            dst += (size_t)w;
        }
        src += (size_t)src_size * w;
        src_size >>= 1;
    }
}

/* PNGToTexture's per-pixel conversion (src/rgl/rglr/rglr_texture_load.cxx:
   40-63) with the reference decoder's table (lut: ryg::srgb8_to_float of
   every byte), then the chain.  Returns 0, or -1 if cap (texels) is short. */
int rsroracle_texture_from_rgba8(const uint8_t* rgba8, int w, int h, int premultiply, const float* lut,
                                 float* out, size_t cap, int* power) {
    const int p = texture_power(w, h);
    const size_t n = (size_t)w * h;
    if (cap < (p >= 0 ? 2 * n : n)) return -1;
    for (size_t i = 0; i < n; ++i) {
        const uint8_t* c = rgba8 + 4 * i;
        float* d = out + 4 * i;
        d[0] = lut[c[0]];
        d[1] = lut[c[1]];
        d[2] = lut[c[2]];
        d[3] = (float)c[3] / 255.0f;
        if (premultiply) { d[0] *= d[3]; d[1] *= d[3]; d[2] *= d[3]; }
    }
    if (p >= 0) make_mipmap(out, w, p);
    if (power) *power = p;
    return 0;
}

int rsroracle_texture_mipmap(float* texels, int w, int h, size_t cap, int* power) {
    const int p = texture_power(w, h);
    if (power) *power = p;
    if (p < 0) return 0;
    if (cap < 2 * (size_t)w * h) return -1;
    make_mipmap(texels, w, p);
    return 0;
}


/* ======================================================================
 * post-processing of float canvases (test infrastructure: the oracle of
 * rsrgpu_kawase_blur / rsrgpu_glow)
 * ====================================================================== */

/* KawaseBlurFilter (src/rgl/rglr/rglr_kawase.cxx:22-84): per output pixel the
   four 2x2 boxes at offsets (-d-1,-d-1) (d,-d-1) (-d-1,d) (d,d), each summed
   ((p00 + p10) + p01) + p11 with clamped coordinates, added in that order onto
   a zero accumulator, times 1/16.  Canvases are RGBA float, strides in pixels. */
int rsroracle_kawase(const float* src, int sw, int sh, int sstride, float* dst, int dw, int dh, int dstride, int d) {
    const int ox[4] = { -d - 1, d, -d - 1, d };
    const int oy[4] = { -d - 1, -d - 1, d, d };
    for (int y = 0; y < dh; ++y) {
        for (int x = 0; x < dw; ++x) {
            float ax[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
            for (int k = 0; k < 4; ++k) {
                const int bx = x + ox[k], by = y + oy[k];
                const int x0 = iclamp(bx, 0, sw - 1), x1 = iclamp(bx + 1, 0, sw - 1);
                const int y0 = iclamp(by, 0, sh - 1), y1 = iclamp(by + 1, 0, sh - 1);
                const float* p00 = src + ((size_t)y0 * sstride + x0) * 4;
                const float* p10 = src + ((size_t)y0 * sstride + x1) * 4;
                const float* p01 = src + ((size_t)y1 * sstride + x0) * 4;
                const float* p11 = src + ((size_t)y1 * sstride + x1) * 4;
                for (int c = 0; c < 4; ++c) ax[c] = ax[c] + (((p00[c] + p10[c]) + p01[c]) + p11[c]);
            }
            float* o = dst + ((size_t)y * dstride + x) * 4;
            for (int c = 0; c < 4; ++c) o[c] = ax[c] * (1.0f / 16.0f);
        }
    }
    return 0;
}

/* rglr::Filter<GlowShader, sRGB|LinearColor> (src/rgl/rglr/rglr_algorithm.hxx:
   107-144) with the $glow node's shader (src/viewer/node/glow.cxx:24-36):
   (image + blur * 0.7) * 0.5 per channel; image = the pixel's lane of the
   full-size quads canvas (16 floats per quad: x[4] y[4] z[4] w[4]), blur = the
   half-size RGBA pixel under the quad; packed like the TrueColor store
   (srgb: the reference encoder's golden table, else to_tc_basic). */
int rsroracle_glow(const float* image, int istride, const float* blur, int bstride, uint32_t* out, int ostride,
                   int w, int h, int srgb) {
    if (srgb && !g_session.srgb_lut) return RSRGPU_EINVAL;
    for (int y = 0; y < h; y += 2) {
        for (int x = 0; x < w; x += 2) {
            const float* q = image + ((size_t)(y / 2) * istride + x / 2) * 16;
            const float* b = blur + ((size_t)(y / 2) * bstride + x / 2) * 4;
            for (int l = 0; l < 4; ++l) {
                float c[3];
                for (int k = 0; k < 3; ++k) c[k] = (q[4 * k + l] + b[k] * 0.700f) * 0.5f;
                uint32_t px;
                if (srgb) px = ((uint32_t)srgb8(g_session.srgb_lut, c[0]) << 16) | ((uint32_t)srgb8(g_session.srgb_lut, c[1]) << 8) | srgb8(g_session.srgb_lut, c[2]);
                else px = ((uint32_t)basic8(c[0]) << 16) | ((uint32_t)basic8(c[1]) << 8) | (uint32_t)basic8(c[2]);
                out[(size_t)(y + (l >> 1)) * ostride + x + (l & 1)] = px;
            }
        }
    }
    return 0;
}
