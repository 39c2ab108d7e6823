// rsrgpu_recorder.cu -- a native recorder of rsr's command stream, for C and
// C++ callers that produce frames themselves (the producer side of the ABI).
//
// It has rglv::GL's calling surface (src/rgl/rglv/rglv_gl.hxx:182-345,
// rglv_gl.cxx:13-106): state setters mark the current state dirty; the next
// command appends a snapshot of the full state and emits CMD_STATE with the
// snapshot's index (MaybeUpdateState, rglv_gl.cxx:100-106).  Commands are
// written in the reference's byte protocol with the ABI's canvas descriptors,
// so a recorded frame goes straight to rsrgpu_submit() or into an
// rsrgpu_frame_desc of a batch.  Canvas and G-buffer descriptors are copied
// into the recorder, whose memory holds them (and the snapshots) until the
// next rsrgpu_recorder_reset() or rsrgpu_recorder_destroy().  Host code only:
// no CUDA call is made.
#include <cstring>
#include <deque>
#include <vector>

#include "../../include/rsrgpu.h"

struct rsrgpu_recorder {
    std::vector<uint8_t> cmds;
    std::vector<rsrgpu_glstate> states;     // the snapshots, indexed by CMD_STATE
    rsrgpu_glstate cur{};
    bool dirty = false;
    // descriptors the stream points to: a deque keeps their addresses stable
    std::deque<rsrgpu_truecolor_canvas> tc;
    std::deque<rsrgpu_fp_canvas> fp;
    std::deque<rsrgpu_gbuffer> gb;
};

namespace {

void identity(float* m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

// GLState::reset (rglv_gl.hxx:152-179) and the defaults of the members it
// leaves alone: both attachments RB_COLOR_DEPTH, identity matrices, texture
// units unbound (8x8, nearest), no uniforms
void default_state(rsrgpu_glstate& s) {
    std::memset(&s, 0, sizeof(s));
    s.clear_color[3] = 1.0f;
    s.clear_depth = 1.0f;
    s.cull_face = RSRGPU_GL_BACK;
    s.color_write_mask = 1;
    s.depth_write_mask = 1;
    s.depth_test_enabled = 1;
    s.depth_func = RSRGPU_GL_LESS;
    s.uniforms_ofs = -1;
    s.color0_attachment_type = RSRGPU_RB_COLOR_DEPTH;
    s.depth_attachment_type = RSRGPU_RB_COLOR_DEPTH;
    for (auto& t : s.tus) { t.width = t.height = t.stride = 8; t.filter = RSRGPU_GL_NEAREST_MIPMAP_NEAREST; }
    s.tu3dim = 256;
    identity(s.view_matrix);
    identity(s.normal_matrix);
    identity(s.projection_matrix);
}

template <typename T>
void put(rsrgpu_recorder* r, const T& v) {
    const auto* b = reinterpret_cast<const uint8_t*>(&v);
    r->cmds.insert(r->cmds.end(), b, b + sizeof(T));
}

// MaybeUpdateState (rglv_gl.cxx:100-106)
void maybe_update_state(rsrgpu_recorder* r) {
    if (!r->dirty) return;
    r->states.push_back(r->cur);
    put<uint8_t>(r, RSRGPU_CMD_STATE);
    put<uint64_t>(r, uint64_t(r->states.size() - 1));
    r->dirty = false;
}

int set_cap(rsrgpu_recorder* r, int cap, int32_t on) {
    if (r == nullptr) return RSRGPU_EINVAL;
    int32_t* f = cap == RSRGPU_GL_CULL_FACE ? &r->cur.culling_enabled
               : cap == RSRGPU_GL_SCISSOR_TEST ? &r->cur.scissor_enabled
               : cap == RSRGPU_GL_BLEND ? &r->cur.blending_enabled
               : cap == RSRGPU_GL_DEPTH_TEST ? &r->cur.depth_test_enabled : nullptr;
    if (f == nullptr) return RSRGPU_EINVAL;
    *f = on;
    r->dirty = true;
    return 0;
}

}  // namespace

extern "C" {

int rsrgpu_recorder_create(rsrgpu_recorder** out) {
    if (out == nullptr) return RSRGPU_EINVAL;
    auto* r = new rsrgpu_recorder;
    default_state(r->cur);
    *out = r;
    return 0;
}

int rsrgpu_recorder_destroy(rsrgpu_recorder* r) {
    delete r;
    return 0;
}

int rsrgpu_recorder_reset(rsrgpu_recorder* r) {
    if (r == nullptr) return RSRGPU_EINVAL;
    r->cmds.clear();
    r->states.clear();
    r->tc.clear();
    r->fp.clear();
    r->gb.clear();
    default_state(r->cur);
    // GL::Reset (rglv_gl.cxx:92-97) leaves the state dirty: the first command
    // after a reset snapshots the default state
    r->dirty = true;
    return 0;
}

int rsrgpu_recorder_frame(rsrgpu_recorder* r, const uint8_t** commands, size_t* nbytes,
                          const rsrgpu_glstate** states, int* nstates) {
    if (r == nullptr || commands == nullptr || nbytes == nullptr || states == nullptr || nstates == nullptr)
        return RSRGPU_EINVAL;
    *commands = r->cmds.data();
    *nbytes = r->cmds.size();
    *states = r->states.data();
    *nstates = int(r->states.size());
    return 0;
}

// ---- state (rglv_gl.hxx:186-312) ----
int rsrgpu_gl_enable(rsrgpu_recorder* r, int cap) { return set_cap(r, cap, 1); }
int rsrgpu_gl_disable(rsrgpu_recorder* r, int cap) { return set_cap(r, cap, 0); }

int rsrgpu_gl_state_int(rsrgpu_recorder* r, int what, int value) {
    if (r == nullptr) return RSRGPU_EINVAL;
    switch (what) {
    case RSRGPU_GLSTATE_CULL_FACE: r->cur.cull_face = value; break;
    case RSRGPU_GLSTATE_DEPTH_FUNC: r->cur.depth_func = value; break;
    case RSRGPU_GLSTATE_DEPTH_WRITE_MASK: r->cur.depth_write_mask = value != 0; break;
    case RSRGPU_GLSTATE_COLOR_WRITE_MASK: r->cur.color_write_mask = value != 0; break;
    case RSRGPU_GLSTATE_PROGRAM: r->cur.program_id = value; break;
    case RSRGPU_GLSTATE_COLOR_ATTACHMENT: r->cur.color0_attachment_type = value; break;
    case RSRGPU_GLSTATE_DEPTH_ATTACHMENT: r->cur.depth_attachment_type = value; break;
    default: return RSRGPU_EINVAL;
    }
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_scissor(rsrgpu_recorder* r, int x, int y, int w, int h) {
    if (r == nullptr) return RSRGPU_EINVAL;
    r->cur.scissor_origin[0] = x; r->cur.scissor_origin[1] = y;
    r->cur.scissor_size[0] = w; r->cur.scissor_size[1] = h;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_viewport(rsrgpu_recorder* r, int x, int y, int w, int h) {
    if (r == nullptr) return RSRGPU_EINVAL;
    r->cur.viewport_origin[0] = x; r->cur.viewport_origin[1] = y;
    r->cur.viewport_size[0] = w; r->cur.viewport_size[1] = h;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_use_uniforms(rsrgpu_recorder* r, const float* values, int n) {
    if (r == nullptr || n < 0 || n > 32 || (n > 0 && values == nullptr)) return RSRGPU_EINVAL;
    std::memset(r->cur.uniforms, 0, sizeof(r->cur.uniforms));
    if (n > 0) std::memcpy(r->cur.uniforms, values, sizeof(float) * size_t(n));
    r->cur.uniforms_ofs = 0;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_bind_texture(rsrgpu_recorder* r, int unit, const float* texels, int width, int height, int stride,
                           int filter) {
    if (r == nullptr || unit < 0 || unit > 1) return RSRGPU_EINVAL;
    rsrgpu_texture_state& t = r->cur.tus[unit];
    t.ptr = texels;
    t.width = width; t.height = height; t.stride = stride; t.filter = filter;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_use_buffer(rsrgpu_recorder* r, int slot, const float* data) {
    if (r == nullptr || slot < 0 || slot > 15) return RSRGPU_EINVAL;
    r->cur.buffers[slot] = data;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_clear_color(rsrgpu_recorder* r, float red, float green, float blue) {
    if (r == nullptr) return RSRGPU_EINVAL;
    r->cur.clear_color[0] = red; r->cur.clear_color[1] = green; r->cur.clear_color[2] = blue;
    r->cur.clear_color[3] = 1.0f;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_clear_depth(rsrgpu_recorder* r, float depth) {
    if (r == nullptr) return RSRGPU_EINVAL;
    r->cur.clear_depth = depth;
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_matrix(rsrgpu_recorder* r, int which, const float m[16]) {
    if (r == nullptr || m == nullptr) return RSRGPU_EINVAL;
    float* dst = which == RSRGPU_GLMATRIX_VIEW ? r->cur.view_matrix
               : which == RSRGPU_GLMATRIX_PROJECTION ? r->cur.projection_matrix
               : which == RSRGPU_GLMATRIX_NORMAL ? r->cur.normal_matrix : nullptr;
    if (dst == nullptr) return RSRGPU_EINVAL;
    std::memcpy(dst, m, sizeof(float) * 16);
    r->dirty = true;
    return 0;
}

int rsrgpu_gl_reset_state(rsrgpu_recorder* r) {   // GL::ResetX
    if (r == nullptr) return RSRGPU_EINVAL;
    default_state(r->cur);
    r->dirty = true;
    return 0;
}

// ---- commands (rglv_gl.cxx:13-89) ----
int rsrgpu_gl_clear(rsrgpu_recorder* r, int bits) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    put<uint8_t>(r, RSRGPU_CMD_CLEAR);
    put<uint8_t>(r, uint8_t(bits));
    return 0;
}

int rsrgpu_gl_draw_elements(rsrgpu_recorder* r, int count, const uint16_t* indices, int hint) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    put<uint8_t>(r, RSRGPU_CMD_DRAW_ELEMENTS);
    put<uint8_t>(r, 0x14);
    put<uint8_t>(r, uint8_t(hint));
    put<int32_t>(r, count);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(indices)));
    return 0;
}

int rsrgpu_gl_draw_arrays(rsrgpu_recorder* r, int count) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    put<uint8_t>(r, RSRGPU_CMD_DRAW_ARRAYS);
    put<int32_t>(r, count);
    return 0;
}

int rsrgpu_gl_draw_elements_instanced(rsrgpu_recorder* r, int count, const uint16_t* indices, int instances) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    put<uint8_t>(r, RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED);
    put<uint8_t>(r, 0x14);
    put<int32_t>(r, count);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(indices)));
    put<int32_t>(r, instances);
    return 0;
}

int rsrgpu_gl_draw_arrays_instanced(rsrgpu_recorder* r, int count, int instances) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    put<uint8_t>(r, RSRGPU_CMD_DRAW_ARRAYS_INSTANCED);
    put<int32_t>(r, count);
    put<int32_t>(r, instances);
    return 0;
}

int rsrgpu_gl_store_color_tc(rsrgpu_recorder* r, uint32_t* data, int width, int height, int stride, int gamma) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    r->tc.push_back(rsrgpu_truecolor_canvas{ data, width, height, stride ? stride : width, 0 });
    put<uint8_t>(r, RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC);
    put<uint8_t>(r, gamma ? 1 : 0);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(&r->tc.back())));
    return 0;
}

int rsrgpu_gl_store_color_fp(rsrgpu_recorder* r, float* data, int width, int height, int stride, int downsample) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    r->fp.push_back(rsrgpu_fp_canvas{ data, width, height, stride ? stride : width, 0 });
    put<uint8_t>(r, downsample ? RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP : RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(&r->fp.back())));
    return 0;
}

int rsrgpu_gl_store_color_quads(rsrgpu_recorder* r, float* data, int width, int height, int stride) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    // rsrgpu_qfloat4_canvas has rsrgpu_fp_canvas's layout
    r->fp.push_back(rsrgpu_fp_canvas{ data, width, height, stride ? stride : width / 2, 0 });
    put<uint8_t>(r, RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(&r->fp.back())));
    return 0;
}

int rsrgpu_gl_store_depth(rsrgpu_recorder* r, float* data) {
    if (r == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    put<uint8_t>(r, RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(data)));
    return 0;
}

int rsrgpu_gl_store_gbuffer(rsrgpu_recorder* r, const rsrgpu_gbuffer* g) {
    if (r == nullptr || g == nullptr) return RSRGPU_EINVAL;
    maybe_update_state(r);
    r->gb.push_back(*g);
    put<uint8_t>(r, RSRGPU_CMD_STORE_GBUFFER);
    put<uint64_t>(r, uint64_t(reinterpret_cast<uintptr_t>(&r->gb.back())));
    return 0;
}

}  // extern "C"
