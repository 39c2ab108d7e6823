// rsr's perf harness over the C ABI: frames recorded, submitted, run and
// waited for one after another, each timed on the host's steady clock.
//
// rsr's `perf` tool (src/viewer/perf.cxx:200-244) renders priming frames,
// then N timed frames, each one GPUNode::Main's work (src/viewer/node/
// gpu.cxx:107-146): GPU::Reset, the layers record their GL calls, GPU::Run,
// wait.  rsrgpu_perf_frames() does the same through this library's entry
// points: rsrgpu_reset, the native recorder (rsrgpu_recorder_reset and the
// rsrgpu_gl_* calls of a call script), rsrgpu_submit, rsrgpu_run and
// rsrgpu_wait.  The call script is what the layers would call; it lets a
// caller in another language hand the frame's calls over once and time the
// loop without its own per-call overhead.

#include <chrono>
#include <cstring>

#include "rsrgpu.h"

namespace {

int play_one(rsrgpu_recorder* r, const rsrgpu_gl_call& c) {
    const int* i = c.i;
    void* p = reinterpret_cast<void*>(uintptr_t(c.p));
    switch (c.fn) {
    case RSRGPU_CALL_ENABLE: return rsrgpu_gl_enable(r, i[0]);
    case RSRGPU_CALL_DISABLE: return rsrgpu_gl_disable(r, i[0]);
    case RSRGPU_CALL_STATE_INT: return rsrgpu_gl_state_int(r, i[0], i[1]);
    case RSRGPU_CALL_SCISSOR: return rsrgpu_gl_scissor(r, i[0], i[1], i[2], i[3]);
    case RSRGPU_CALL_VIEWPORT: return rsrgpu_gl_viewport(r, i[0], i[1], i[2], i[3]);
    case RSRGPU_CALL_USE_UNIFORMS: return rsrgpu_gl_use_uniforms(r, c.f, i[0]);
    case RSRGPU_CALL_BIND_TEXTURE:
        return rsrgpu_gl_bind_texture(r, i[0], static_cast<const float*>(p), i[1], i[2], i[3], i[4]);
    case RSRGPU_CALL_USE_BUFFER: return rsrgpu_gl_use_buffer(r, i[0], static_cast<const float*>(p));
    case RSRGPU_CALL_CLEAR_COLOR: return rsrgpu_gl_clear_color(r, c.f[0], c.f[1], c.f[2]);
    case RSRGPU_CALL_CLEAR_DEPTH: return rsrgpu_gl_clear_depth(r, c.f[0]);
    case RSRGPU_CALL_MATRIX: return rsrgpu_gl_matrix(r, i[0], c.f);
    case RSRGPU_CALL_RESET_STATE: return rsrgpu_gl_reset_state(r);
    case RSRGPU_CALL_CLEAR: return rsrgpu_gl_clear(r, i[0]);
    case RSRGPU_CALL_DRAW_ELEMENTS: return rsrgpu_gl_draw_elements(r, i[0], static_cast<const uint16_t*>(p), i[1]);
    case RSRGPU_CALL_DRAW_ARRAYS: return rsrgpu_gl_draw_arrays(r, i[0]);
    case RSRGPU_CALL_DRAW_ELEMENTS_INSTANCED:
        return rsrgpu_gl_draw_elements_instanced(r, i[0], static_cast<const uint16_t*>(p), i[1]);
    case RSRGPU_CALL_DRAW_ARRAYS_INSTANCED: return rsrgpu_gl_draw_arrays_instanced(r, i[0], i[1]);
    case RSRGPU_CALL_STORE_COLOR_TC:
        return rsrgpu_gl_store_color_tc(r, static_cast<uint32_t*>(p), i[0], i[1], i[2], i[3]);
    case RSRGPU_CALL_STORE_COLOR_FP:
        return rsrgpu_gl_store_color_fp(r, static_cast<float*>(p), i[0], i[1], i[2], i[3]);
    case RSRGPU_CALL_STORE_COLOR_QUADS: return rsrgpu_gl_store_color_quads(r, static_cast<float*>(p), i[0], i[1], i[2]);
    case RSRGPU_CALL_STORE_DEPTH: return rsrgpu_gl_store_depth(r, static_cast<float*>(p));
    case RSRGPU_CALL_STORE_GBUFFER: return rsrgpu_gl_store_gbuffer(r, static_cast<const rsrgpu_gbuffer*>(p));
    default: return RSRGPU_EINVAL;
    }
}

}  // namespace

extern "C" {

int rsrgpu_gl_play(rsrgpu_recorder* rec, const rsrgpu_gl_call* calls, int ncalls) {
    if (rec == nullptr || ncalls < 0 || (ncalls > 0 && calls == nullptr)) return RSRGPU_EINVAL;
    for (int k = 0; k < ncalls; ++k) {
        const int rc = play_one(rec, calls[k]);
        if (rc) return rc;
    }
    return 0;
}

int rsrgpu_perf_frames(rsrgpu_ctx* ctx, rsrgpu_recorder* rec, const rsrgpu_perf_target* target,
                       const rsrgpu_gl_call* calls, int ncalls, int priming, int frames, void* stream,
                       double* frame_ms) {
    if (ctx == nullptr || rec == nullptr || target == nullptr || priming < 0 || frames < 0 ||
        (frames > 0 && frame_ms == nullptr))
        return RSRGPU_EINVAL;
    for (int n = 0; n < priming + frames; ++n) {
        const auto t0 = std::chrono::steady_clock::now();
        // GPUNode::Main: GPU::Reset (which resets the recorder), the layers' calls, GPU::Run, wait
        int rc = rsrgpu_reset(ctx, target->width, target->height, target->tile_blocks_x, target->tile_blocks_y);
        if (rc == 0) rc = rsrgpu_recorder_reset(rec);
        if (rc == 0) rc = rsrgpu_gl_play(rec, calls, ncalls);
        const uint8_t* cmds = nullptr;
        size_t nbytes = 0;
        const rsrgpu_glstate* states = nullptr;
        int nstates = 0;
        if (rc == 0) rc = rsrgpu_recorder_frame(rec, &cmds, &nbytes, &states, &nstates);
        if (rc == 0) rc = rsrgpu_submit(ctx, cmds, nbytes, states, nstates);
        if (rc == 0) rc = rsrgpu_run(ctx, stream);
        if (rc == 0) rc = rsrgpu_wait(ctx, -1);
        if (rc) return rc;
        const auto t1 = std::chrono::steady_clock::now();
        if (n >= priming) frame_ms[n - priming] = std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
    return 0;
}

}  // extern "C"
