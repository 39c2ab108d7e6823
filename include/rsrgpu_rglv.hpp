/*
 * rsrgpu_rglv.hpp -- the C++ shim that puts this library behind rsr's own
 * rglv::GPU calling surface (src/rgl/rglv/rglv_gpu.hxx:97-277), for code in
 * rsr's tree (it includes rsr's headers, with rsr's checkout on the include
 * path).  C callers use rsrgpu.h alone.
 *
 *   ToDevice(GLState, uniforms)  a GLState snapshot (rglv_gl.hxx:80-179) as the
 *                                ABI's rsrgpu_glstate, its uniform block copied
 *   TranslateFrame(GL&, frame)   rsr's recorded command stream (GL::commands_,
 *                                written by rglv_gl.cxx:13-106) as the ABI's
 *                                stream: CMD_STATE's GLState* becomes the
 *                                snapshot's index, canvas pointers become ABI
 *                                canvas descriptors held by the frame
 *   DeviceGPU                    rglv::GPU's members (Install, Reset, IC, Run)
 *                                over a device context; Run() returns a jobsys
 *                                job that waits for the frame, as
 *                                GPU::Run() does (rglv_gpu.cxx:90-116)
 */
#ifndef RSRGPU_RGLV_HPP
#define RSRGPU_RGLV_HPP

#include <cstdint>
#include <cstring>
#include <deque>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "rsrgpu.h"
#include "src/rcl/rclmt/rclmt_jobsys.hxx"
#include "src/rgl/rglr/rglr_canvas.hxx"
#include "src/rgl/rglv/rglv_gl.hxx"
#include "src/rgl/rglv/rglv_gpu_protocol.hxx"

namespace rqdq {
namespace rglv {

inline rsrgpu_glstate ToDevice(const GLState& s, const void* uniforms) {
    rsrgpu_glstate d{};
    const float cc[4] = { s.clearColor.x, s.clearColor.y, s.clearColor.z, s.clearColor.w };
    std::memcpy(d.clear_color, cc, sizeof(cc));
    d.clear_depth = s.clearDepth;
    d.clear_stencil = s.clearStencil;
    d.culling_enabled = s.cullingEnabled;
    d.cull_face = s.cullFace;
    d.scissor_enabled = s.scissorEnabled;
    d.scissor_origin[0] = s.scissorOrigin.x; d.scissor_origin[1] = s.scissorOrigin.y;
    d.scissor_size[0] = s.scissorSize.x; d.scissor_size[1] = s.scissorSize.y;
    d.viewport_origin[0] = s.viewportOrigin.x; d.viewport_origin[1] = s.viewportOrigin.y;
    if (s.viewportSize) { d.viewport_size[0] = s.viewportSize->x; d.viewport_size[1] = s.viewportSize->y; }
    d.blending_enabled = s.blendingEnabled;
    d.color_write_mask = s.colorWriteMask;
    d.depth_write_mask = s.depthWriteMask;
    d.depth_test_enabled = s.depthTestEnabled;
    d.depth_func = s.depthFunc;
    d.program_id = s.programId;
    d.uniforms_ofs = uniforms != nullptr ? 0 : -1;
    if (uniforms != nullptr) std::memcpy(d.uniforms, uniforms, sizeof(d.uniforms));   // UNIFORM_BUFFER_SIZE floats
    d.color0_attachment_type = s.color0AttachmentType;
    d.depth_attachment_type = s.depthAttachmentType;
    for (int i = 0; i < 16; ++i) d.buffers[i] = s.buffers[size_t(i)];
    for (int u = 0; u < 2; ++u) {
        const TextureState& t = s.tus[size_t(u)];
        d.tus[u].ptr = reinterpret_cast<const float*>(t.ptr);
        d.tus[u].width = t.width; d.tus[u].height = t.height; d.tus[u].stride = t.stride;
        d.tus[u].filter = t.filter;
    }
    d.tu3ptr = s.tu3ptr;
    d.tu3dim = s.tu3dim;
    std::memcpy(d.view_matrix, s.viewMatrix.ff.data(), sizeof(d.view_matrix));
    std::memcpy(d.normal_matrix, s.normalMatrix.ff.data(), sizeof(d.normal_matrix));
    std::memcpy(d.projection_matrix, s.projectionMatrix.ff.data(), sizeof(d.projection_matrix));
    return d;
}

// A frame in the ABI's form; the canvas descriptors the stream points to
// live in the deques (their addresses stay put as they grow).
struct DeviceFrame {
    std::vector<uint8_t> cmds;
    std::vector<rsrgpu_glstate> states;
    std::deque<rsrgpu_truecolor_canvas> tc;
    std::deque<rsrgpu_fp_canvas> fp;
    void clear() { cmds.clear(); states.clear(); tc.clear(); fp.clear(); }
};

// Reads the recorder's stream to its end, as GPU::BinImpl does
// (rglv_gpu.cxx:119-260: an EOF is appended, then the commands are consumed).
// Returns false at a command the ABI does not know.
inline bool TranslateFrame(GL& ic, DeviceFrame& f) {
    f.clear();
    std::unordered_map<const GLState*, uint64_t> index;
    auto& cs = ic.commands_;
    cs.appendByte(CMD_EOF);
    auto put = [&](const void* p, size_t n) {
        const auto* b = static_cast<const uint8_t*>(p);
        f.cmds.insert(f.cmds.end(), b, b + n);
    };
    while (true) {
        const uint8_t op = cs.consumeByte();
        switch (op) {
        case CMD_EOF:
            return true;
        case CMD_STATE: {
            const auto* s = static_cast<const GLState*>(cs.consumePtr());
            const auto found = index.emplace(s, uint64_t(f.states.size()));
            if (found.second) f.states.push_back(ToDevice(*s, ic.GetUniformBufferAddr(s->uniformsOfs)));
            f.cmds.push_back(op);
            put(&found.first->second, 8);
        } break;
        case CMD_CLEAR: {
            const uint8_t bits = cs.consumeByte();
            f.cmds.push_back(op); put(&bits, 1);
        } break;
        case CMD_DRAW_ELEMENTS: {
            const uint8_t flags = cs.consumeByte(), hint = cs.consumeByte();
            const int32_t count = cs.consumeInt();
            const void* p = cs.consumePtr();
            f.cmds.push_back(op); put(&flags, 1); put(&hint, 1); put(&count, 4); put(&p, 8);
        } break;
        case CMD_DRAW_ARRAYS: {
            const int32_t count = cs.consumeInt();
            f.cmds.push_back(op); put(&count, 4);
        } break;
        case CMD_DRAW_ELEMENTS_INSTANCED: {
            const uint8_t flags = cs.consumeByte();
            const int32_t count = cs.consumeInt();
            const void* p = cs.consumePtr();
            const int32_t n = cs.consumeInt();
            f.cmds.push_back(op); put(&flags, 1); put(&count, 4); put(&p, 8); put(&n, 4);
        } break;
        case CMD_DRAW_ARRAYS_INSTANCED: {
            const int32_t count = cs.consumeInt(), n = cs.consumeInt();
            f.cmds.push_back(op); put(&count, 4); put(&n, 4);
        } break;
        case CMD_STORE_COLOR_FULL_LINEAR_TC: {
            const uint8_t gamma = cs.consumeByte();
            auto* c = static_cast<rglr::TrueColorCanvas*>(cs.consumePtr());
            f.tc.push_back(rsrgpu_truecolor_canvas{ reinterpret_cast<uint32_t*>(c->data()), c->width(), c->height(),
                                                    c->stride(), 0 });
            const void* p = &f.tc.back();
            f.cmds.push_back(op); put(&gamma, 1); put(&p, 8);
        } break;
        case CMD_STORE_COLOR_FULL_LINEAR_FP:
        case CMD_STORE_COLOR_HALF_LINEAR_FP: {
            auto* c = static_cast<rglr::FloatingPointCanvas*>(cs.consumePtr());
            f.fp.push_back(rsrgpu_fp_canvas{ reinterpret_cast<float*>(c->data()), c->width(), c->height(), c->stride(), 0 });
            const void* p = &f.fp.back();
            f.cmds.push_back(op); put(&p, 8);
        } break;
        case CMD_STORE_COLOR_FULL_QUADS_FP: {   // rsrgpu_qfloat4_canvas has rsrgpu_fp_canvas's layout
            auto* c = static_cast<rglr::QFloat4Canvas*>(cs.consumePtr());
            f.fp.push_back(rsrgpu_fp_canvas{ reinterpret_cast<float*>(c->data()), c->width(), c->height(), c->stride(), 0 });
            const void* p = &f.fp.back();
            f.cmds.push_back(op); put(&p, 8);
        } break;
        case CMD_STORE_DEPTH_FULL_LINEAR_FP: {
            const void* p = cs.consumePtr();
            f.cmds.push_back(op); put(&p, 8);
        } break;
        default:
            return false;
        }
    }
}

// rglv::GPU's public surface over a device context.  The host arrays rsr
// keeps (VAOs, index lists, textures, canvases) are declared once with
// Register(); rsr's frame loop (GPUNode::Main, src/viewer/node/gpu.cxx:
// 107-146) then stays as it is.
class DeviceGPU {
public:
    explicit DeviceGPU(int device) { status_ = rsrgpu_create(device, &ctx_); }
    ~DeviceGPU() { rsrgpu_destroy(ctx_); }
    DeviceGPU(const DeviceGPU&) = delete;
    DeviceGPU& operator=(const DeviceGPU&) = delete;
    int Install(int programId, uint32_t stateKey, int kind) { return rsrgpu_install(ctx_, programId, stateKey, kind); }
    int Register(const void* p, size_t bytes) { return rsrgpu_register_host_buffer(ctx_, p, bytes); }
    auto IC() -> GL& { return ic_; }
    void Reset(rmlv::ivec2 size, rmlv::ivec2 tileBlocks) {
        status_ = rsrgpu_reset(ctx_, size.x, size.y, tileBlocks.x, tileBlocks.y);
        ic_.Reset();
    }
    // GPU::Run: the frame goes to the device now; the returned job waits for it
    auto Run() -> rclmt::jobsys::Job* {
        status_ = TranslateFrame(ic_, frame_) ? 0 : RSRGPU_EUNSUPPORTED;
        if (status_ == 0)
            status_ = rsrgpu_submit(ctx_, frame_.cmds.data(), frame_.cmds.size(), frame_.states.data(),
                                    int(frame_.states.size()));
        if (status_ == 0) status_ = rsrgpu_run(ctx_, nullptr);
        return rclmt::jobsys::make_job(DeviceGPU::WaitJmp, std::tuple{ this });
    }
    // 0, or the first failing call's status (rsrgpu_last_error has the message)
    int Status() const { return status_; }
    rsrgpu_ctx* Context() const { return ctx_; }

private:
    static void WaitJmp(rclmt::jobsys::Job*, unsigned, std::tuple<DeviceGPU*>* data) {
        DeviceGPU* self = std::get<0>(*data);
        if (self->status_ == 0) self->status_ = rsrgpu_wait(self->ctx_, -1);
    }
    rsrgpu_ctx* ctx_{ nullptr };
    GL ic_{};
    DeviceFrame frame_;
    int status_{ 0 };
};

}  // namespace rglv
}  // namespace rqdq

#endif  // RSRGPU_RGLV_HPP
