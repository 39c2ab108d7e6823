// Test program for include/rsrgpu_rglv.hpp: plays a GL call script (an array
// of rsrgpu_gl_call, include/rsrgpu.h) on rsr's own rglv::GL recorder,
// translates the recorded stream with TranslateFrame(), and writes the
// result with every canvas pointer replaced by the descriptor it points to:
//   u64 n, n bytes of stream; u64 m, m rsrgpu_glstate snapshots.
// tests/test_rglv_shim.py compares that with the library's native recorder
// playing the same script.
//   rsr_translate script.bin out.bin
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "rsrgpu_rglv.hpp"

using namespace rqdq;

namespace {

struct Canvases {
    std::vector<std::unique_ptr<rglr::TrueColorCanvas>> tc;
    std::vector<std::unique_ptr<rglr::FloatingPointCanvas>> fp;
    std::vector<std::unique_ptr<rglr::QFloat4Canvas>> quads;
};

rmlm::mat4 Mat(const float* f) {
    rmlm::mat4 m;
    std::memcpy(m.ff.data(), f, 64);
    return m;
}

bool Play(rglv::GL& gl, const rsrgpu_gl_call& c, Canvases& cv) {
    using namespace rglv;
    const int* i = c.i;
    void* p = reinterpret_cast<void*>(uintptr_t(c.p));
    switch (c.fn) {
    case RSRGPU_CALL_ENABLE: gl.Enable(i[0]); return true;
    case RSRGPU_CALL_DISABLE: gl.Disable(i[0]); return true;
    case RSRGPU_CALL_STATE_INT:
        switch (i[0]) {
        case RSRGPU_GLSTATE_CULL_FACE: gl.CullFace(i[1]); return true;
        case RSRGPU_GLSTATE_DEPTH_FUNC: gl.DepthFunc(i[1]); return true;
        case RSRGPU_GLSTATE_DEPTH_WRITE_MASK: gl.DepthWriteMask(i[1] != 0); return true;
        case RSRGPU_GLSTATE_COLOR_WRITE_MASK: gl.ColorWriteMask(i[1] != 0); return true;
        case RSRGPU_GLSTATE_PROGRAM: gl.UseProgram(i[1]); return true;
        case RSRGPU_GLSTATE_COLOR_ATTACHMENT: gl.RenderbufferType(GL_COLOR_ATTACHMENT0, i[1]); return true;
        case RSRGPU_GLSTATE_DEPTH_ATTACHMENT: gl.RenderbufferType(GL_DEPTH_ATTACHMENT, i[1]); return true;
        default: return false;
        }
    case RSRGPU_CALL_SCISSOR: gl.Scissor(i[0], i[1], i[2], i[3]); return true;
    case RSRGPU_CALL_VIEWPORT: gl.Viewport(i[0], i[1], i[2], i[3]); return true;
    case RSRGPU_CALL_USE_UNIFORMS: {
        auto block = gl.AllocUniformBuffer();
        std::memcpy(block.second, c.f, sizeof(float) * size_t(i[0]));
        gl.UseUniforms(block.first);
        return true;
    }
    case RSRGPU_CALL_BIND_TEXTURE:
        gl.BindTexture(i[0], static_cast<const PixelToaster::FloatingPointPixel*>(p), i[1], i[2], i[3],
                       i[4] ? GL_LINEAR_MIPMAP_NEAREST : GL_NEAREST_MIPMAP_NEAREST);
        return true;
    case RSRGPU_CALL_USE_BUFFER: gl.UseBuffer(i[0], static_cast<const float*>(p)); return true;
    case RSRGPU_CALL_CLEAR_COLOR: gl.ClearColor(rmlv::vec3{ c.f[0], c.f[1], c.f[2] }); return true;
    case RSRGPU_CALL_CLEAR_DEPTH: gl.ClearDepth(c.f[0]); return true;
    case RSRGPU_CALL_MATRIX:
        if (i[0] == RSRGPU_GLMATRIX_VIEW) gl.ViewMatrix(Mat(c.f));
        else if (i[0] == RSRGPU_GLMATRIX_PROJECTION) gl.ProjectionMatrix(Mat(c.f));
        else gl.NormalMatrix(Mat(c.f));
        return true;
    case RSRGPU_CALL_RESET_STATE: gl.ResetX(); return true;
    case RSRGPU_CALL_CLEAR: gl.Clear(uint8_t(i[0])); return true;
    case RSRGPU_CALL_DRAW_ELEMENTS:
        gl.DrawElements(GL_TRIANGLES, i[0], GL_UNSIGNED_SHORT, static_cast<const uint16_t*>(p), uint8_t(i[1]));
        return true;
    case RSRGPU_CALL_DRAW_ARRAYS: gl.DrawArrays(GL_TRIANGLES, 0, i[0]); return true;
    case RSRGPU_CALL_DRAW_ELEMENTS_INSTANCED:
        gl.DrawElementsInstanced(GL_TRIANGLES, i[0], GL_UNSIGNED_SHORT, static_cast<const uint16_t*>(p), i[1]);
        return true;
    case RSRGPU_CALL_DRAW_ARRAYS_INSTANCED: gl.DrawArraysInstanced(GL_TRIANGLES, 0, i[0], i[1]); return true;
    case RSRGPU_CALL_STORE_COLOR_TC:
        cv.tc.emplace_back(std::make_unique<rglr::TrueColorCanvas>(static_cast<PixelToaster::TrueColorPixel*>(p), i[0],
                                                                    i[1], i[2]));
        gl.StoreColor(cv.tc.back().get(), i[3] != 0);
        return true;
    case RSRGPU_CALL_STORE_COLOR_FP:
        cv.fp.emplace_back(std::make_unique<rglr::FloatingPointCanvas>(static_cast<PixelToaster::FloatingPointPixel*>(p),
                                                                        i[0], i[1], i[2]));
        gl.StoreColor(cv.fp.back().get(), i[3] != 0);
        return true;
    case RSRGPU_CALL_STORE_COLOR_QUADS:
        cv.quads.emplace_back(i[2] ? std::make_unique<rglr::QFloat4Canvas>(i[0], i[1], static_cast<rmlv::qfloat4*>(p), i[2])
                                   : std::make_unique<rglr::QFloat4Canvas>(i[0], i[1], static_cast<rmlv::qfloat4*>(p)));
        gl.StoreColor(cv.quads.back().get());
        return true;
    case RSRGPU_CALL_STORE_DEPTH: gl.StoreDepth(static_cast<float*>(p)); return true;
    default: return false;   // no G-buffer store in rsr
    }
}

// the stream with each canvas pointer replaced by its descriptor's bytes
std::vector<uint8_t> Canonical(const std::vector<uint8_t>& s) {
    std::vector<uint8_t> out;
    size_t p = 0;
    auto copy = [&](size_t n) { out.insert(out.end(), s.begin() + long(p), s.begin() + long(p + n)); p += n; };
    auto deref = [&](size_t n) {
        uint64_t a;
        std::memcpy(&a, s.data() + p, 8);
        const auto* b = reinterpret_cast<const uint8_t*>(uintptr_t(a));
        out.insert(out.end(), b, b + n);
        p += 8;
    };
    while (p < s.size()) {
        const uint8_t op = s[p];
        copy(1);
        switch (op) {
        case RSRGPU_CMD_STATE: copy(8); break;
        case RSRGPU_CMD_CLEAR: copy(1); break;
        case RSRGPU_CMD_DRAW_ELEMENTS: copy(14); break;
        case RSRGPU_CMD_DRAW_ARRAYS: copy(4); break;
        case RSRGPU_CMD_DRAW_ELEMENTS_INSTANCED: copy(17); break;
        case RSRGPU_CMD_DRAW_ARRAYS_INSTANCED: copy(8); break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_TC: copy(1); deref(sizeof(rsrgpu_truecolor_canvas)); break;
        case RSRGPU_CMD_STORE_COLOR_FULL_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_HALF_LINEAR_FP:
        case RSRGPU_CMD_STORE_COLOR_FULL_QUADS_FP: deref(sizeof(rsrgpu_fp_canvas)); break;
        case RSRGPU_CMD_STORE_DEPTH_FULL_LINEAR_FP: copy(8); break;
        default: return {};
        }
    }
    return out;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: rsr_translate script.bin out.bin\n"); return 2; }
    std::FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    std::vector<rsrgpu_gl_call> calls;
    rsrgpu_gl_call c;
    while (std::fread(&c, sizeof(c), 1, in) == 1) calls.push_back(c);
    std::fclose(in);
    // a fresh recorder in the native recorder's starting state: GL::Reset,
    // both attachments RB_COLOR_DEPTH, identity matrices
    rglv::GL gl{};
    gl.Reset();
    gl.RenderbufferType(rglv::GL_COLOR_ATTACHMENT0, rglv::RB_COLOR_DEPTH);
    gl.RenderbufferType(rglv::GL_DEPTH_ATTACHMENT, rglv::RB_COLOR_DEPTH);
    const float id[16] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1 };
    gl.ViewMatrix(Mat(id));
    gl.NormalMatrix(Mat(id));
    gl.ProjectionMatrix(Mat(id));
    Canvases cv;
    for (const auto& call : calls)
        if (!Play(gl, call, cv)) { std::fprintf(stderr, "unplayable call %d\n", call.fn); return 1; }
    rglv::DeviceFrame frame;
    if (!rglv::TranslateFrame(gl, frame)) { std::fprintf(stderr, "untranslatable stream\n"); return 1; }
    const std::vector<uint8_t> canon = Canonical(frame.cmds);
    std::FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    const uint64_t n = canon.size(), m = frame.states.size();
    std::fwrite(&n, 8, 1, out);
    std::fwrite(canon.data(), 1, canon.size(), out);
    std::fwrite(&m, 8, 1, out);
    std::fwrite(frame.states.data(), sizeof(rsrgpu_glstate), frame.states.size(), out);
    std::fclose(out);
    if (argc > 99) {   // never taken: DeviceGPU's members are compiled and linked too
        rglv::DeviceGPU g(0);
        g.Install(4, 0x6e2, 1);
        g.Reset(rmlv::ivec2{ 64, 64 }, rmlv::ivec2{ 4, 4 });
        rclmt::jobsys::Job* j = g.Run();
        (void)j;
        return g.Status();
    }
    return 0;
}
