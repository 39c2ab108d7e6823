// ref_harness.cxx -- drives rsr's own CPU rasteriser (rglv::GPU and the
// GPUBinImpl / GPUTileImpl / GPUBltImpl templates) headless, for use as the
// oracle's pin and as the CPU baseline.  Test infrastructure only: it is
// compiled against the reference sources by oracle/ref/Makefile into
// oracle/_ref/librsrref.so and is loaded by tests and by bench.py's
// reference arm, never by the GPU library.
//
// Input is the same (command stream, state snapshots) pair that
// rsrgpu_submit() takes (include/rsrgpu.h); the harness replays it through
// the reference's rglv::GL recorder API (src/rgl/rglv/rglv_gl.hxx:186-331) so
// the reference records its own stream, then runs GPU::Run() on the jobsys
// thread pool (src/rcl/rclmt/rclmt_jobsys.cxx) with doubleBuffer=false
// (src/rgl/rglv/rglv_gpu.cxx:16,96-98).
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "src/rcl/rclmt/rclmt_jobsys.hxx"
#include "src/rgl/rglr/rglr_canvas.hxx"
#include "src/rgl/rglr/rglr_fragmentcursor.hxx"
#include "src/rgl/rglr/rglr_texture.hxx"
#include "src/rgl/rglr/rglr_algorithm.hxx"
#include "src/rgl/rglr/rglr_canvas_util.hxx"
#include "src/rgl/rglr/rglr_kawase.hxx"
#include "src/rgl/rglv/rglv_gl.hxx"
#include "src/rgl/rglv/rglv_gpu.hxx"
#include "src/rgl/rglv/rglv_gpu_impl.hxx"
#include "src/rgl/rglv/rglv_gpu_shaders.hxx"
#include "src/viewer/shaders.hxx"

#include "include/rsrgpu.h"
#include "3rdparty/ryg-srgb/ryg-srgb.h"

namespace rqdq {
namespace harness {

// Gouraud test program: per-vertex rgb interpolated perspective-correct, no
// lighting.  It is OBJ1Program (src/viewer/shaders.hxx:586-699) without its
// lighting term, written against rglv::BaseProgram the way
// src/rgl/rglv/rglv_triangle.t.cxx:134-202 writes its test programs.
// Attribute slots: position 0-2, colour 3-5.
struct GouraudProgram final : public rglv::BaseProgram {
	static constexpr int id = RSRGPU_PROGRAM_GOURAUD;

	struct VertexInput {
		rmlv::qfloat3 position;
		rmlv::qfloat3 color; };

	struct Loader {
		const std::array<const float*, 16> ptrs_;
		Loader(const std::array<const float*, 16>& buffers) : ptrs_(buffers) {}
		void LoadInstance(int, VertexInput&) {}
		void LoadMD(int idx, VertexInput& vi) {
			vi.position.x = _mm_load_ps(&ptrs_[0][idx]);
			vi.position.y = _mm_load_ps(&ptrs_[1][idx]);
			vi.position.z = _mm_load_ps(&ptrs_[2][idx]);
			vi.color.x = _mm_load_ps(&ptrs_[3][idx]);
			vi.color.y = _mm_load_ps(&ptrs_[4][idx]);
			vi.color.z = _mm_load_ps(&ptrs_[5][idx]); }
		void LoadLane(int idx, int li, VertexInput& vi) {
			vi.position.setLane(li, rmlv::vec3{ ptrs_[0][idx], ptrs_[1][idx], ptrs_[2][idx] });
			vi.color.setLane(li, rmlv::vec3{ ptrs_[3][idx], ptrs_[4][idx], ptrs_[5][idx] }); }};

	struct VertexOutputSD {
		rmlv::vec3 color;
		static VertexOutputSD Mix(VertexOutputSD a, VertexOutputSD b, float t) {
			return { mix(a.color, b.color, t) }; }};

	struct VertexOutputMD {
		rmlv::qfloat3 color;
		VertexOutputSD Lane(const int li) const {
			return VertexOutputSD{ color.lane(li) }; }};

	struct Interpolants {
		Interpolants() = default;
		Interpolants(VertexOutputSD d0, VertexOutputSD d1, VertexOutputSD d2) :
			color({ d0.color, d1.color, d2.color }) {}
		VertexOutputMD Interpolate(rglv::BaryCoord BS [[maybe_unused]], rglv::BaryCoord BP) const {
			return { rglv::Interpolate(BP, color) }; }
		rglv::VertexFloat3 color; };

	static void ShadeVertex(const rglv::Matrices& mats, const UniformsMD& u [[maybe_unused]],
	                        const VertexInput& v, rmlv::qfloat4& gl_Position, VertexOutputMD& outs) {
		outs.color = v.color;
		gl_Position = mats.vpm * rmlv::qfloat4{ v.position, 1.0F }; }

	template <typename TU0, typename TU1, typename TU3>
	static void ShadeFragment(const rglv::Matrices&, const UniformsMD&, const TU0, const TU1, const TU3&,
	                          const rglv::BaryCoord&, const rglv::BaryCoord&, const VertexOutputMD& outs,
	                          const rmlv::qfloat2&, const rmlv::qfloat&, rmlv::qfloat4& gl_FragColor,
	                          rmlv::mvec4i&) {
		gl_FragColor = { outs.color, 1.0F }; }

	static rmlv::qfloat3 ShadeCanvas(const UniformsMD&, const rmlv::qfloat2, const rmlv::qfloat3 source) {
		return source; } };


// The $glow node's shader (src/viewer/node/glow.cxx:24-36), which rsr keeps
// in an unnamed namespace of the viewer: (image + blur * 0.7) * 0.5.
struct GlowShader {
	static rmlv::qfloat3 ShadeCanvas(rmlv::qfloat2, rmlv::qfloat3 c1, rmlv::qfloat3 c2) {
		auto& image = c1;
		auto& blur = c2;
		const rmlv::qfloat blurAmt{ 0.700F };
		const rmlv::qfloat brightness{ 0.5F };
		rmlv::qfloat3 out;
		out = (image + blur*blurAmt) * brightness;
		return out; } };


// Subclass that exposes the protected tile streams and clipped vertices of
// rglv::GPU (rglv_gpu.hxx:106-150) for bin-list parity checks.
class InspectableGPU : public rglv::GPU {
public:
	using rglv::GPU::GPU;
	int NumTiles() const { return static_cast<int>(tilesHead_.size()); }
	const uint8_t* TileStream(int t) const { return ReadRange(t).first; }
	const rcls::vector<rglv::ClippedVertex>& Clipped() const { return clippedVertexBuffer1_; }
	rglv::GPUStats Stats() const { return stats1_; } };


template <typename PGM>
void InstallDrawStates(rglv::GPU& gpu) {
	using namespace rglv;
	using namespace rglr;
	const int id = PGM::id;
	gpu.Install(id, 0, GPUBinImpl<PGM>::MakeBinProgramPtrs());
	// RB_RGBF32 colour + RB_F32 depth
	gpu.Install(id, 0x6e2, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, false, true, DepthLT, true, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x6e6, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, false, true, DepthLE, true, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x6f2, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, false, true, DepthLT, true, true, BlendAlpha>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x6c2, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, false, true, DepthLT, false, true, BlendOff>::MakeDrawProgramPtrs());
	// RB_COLOR_DEPTH (colour rgb + depth in alpha)
	gpu.Install(id, 0x62, GPUTileImpl<QFloat4RGBFragmentCursor, QFloat4AFragmentCursor, PGM, false, true, DepthLT, true, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x72, GPUTileImpl<QFloat4RGBFragmentCursor, QFloat4AFragmentCursor, PGM, false, true, DepthLT, true, true, BlendAlpha>::MakeDrawProgramPtrs());
	// the same states with the scissor test on (SCISSOR_ENABLED = true, key bit 0)
	gpu.Install(id, 0x6e3, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, true, true, DepthLT, true, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x6e7, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, true, true, DepthLE, true, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x6f3, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, true, true, DepthLT, true, true, BlendAlpha>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x6c3, GPUTileImpl<QFloat3FragmentCursor, QFloatFragmentCursor, PGM, true, true, DepthLT, false, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x63, GPUTileImpl<QFloat4RGBFragmentCursor, QFloat4AFragmentCursor, PGM, true, true, DepthLT, true, true, BlendOff>::MakeDrawProgramPtrs());
	gpu.Install(id, 0x73, GPUTileImpl<QFloat4RGBFragmentCursor, QFloat4AFragmentCursor, PGM, true, true, DepthLT, true, true, BlendAlpha>::MakeDrawProgramPtrs()); }


struct Session {
	std::unique_ptr<InspectableGPU> gpu;
	int threads{0}; };

Session* g_session = nullptr;


void ApplyState(rglv::GL& gl, const rsrgpu_glstate& s) {
	using namespace rglv;
	gl.ResetX();
	gl.RenderbufferType(GL_COLOR_ATTACHMENT0, s.color0_attachment_type);
	gl.RenderbufferType(GL_DEPTH_ATTACHMENT, s.depth_attachment_type);
	gl.ClearColor(rmlv::vec3{ s.clear_color[0], s.clear_color[1], s.clear_color[2] });
	gl.ClearDepth(s.clear_depth);
	if (s.culling_enabled) gl.Enable(GL_CULL_FACE); else gl.Disable(GL_CULL_FACE);
	gl.CullFace(s.cull_face);
	if (s.scissor_enabled) gl.Enable(GL_SCISSOR_TEST); else gl.Disable(GL_SCISSOR_TEST);
	gl.Scissor(s.scissor_origin[0], s.scissor_origin[1], s.scissor_size[0], s.scissor_size[1]);
	if (s.viewport_size[0] != 0 || s.viewport_size[1] != 0) {
		gl.Viewport(s.viewport_origin[0], s.viewport_origin[1], s.viewport_size[0], s.viewport_size[1]); }
	if (s.blending_enabled) gl.Enable(GL_BLEND); else gl.Disable(GL_BLEND);
	if (s.depth_test_enabled) gl.Enable(GL_DEPTH_TEST); else gl.Disable(GL_DEPTH_TEST);
	gl.DepthFunc(s.depth_func);
	gl.DepthWriteMask(s.depth_write_mask != 0);
	gl.ColorWriteMask(s.color_write_mask != 0);
	gl.UseProgram(s.program_id);
	if (s.uniforms_ofs >= 0) {
		auto [idx, ptr] = gl.AllocUniformBuffer();
		std::memcpy(ptr, s.uniforms, sizeof(s.uniforms));
		gl.UseUniforms(idx); }
	for (int i = 0; i < 16; ++i) {
		gl.UseBuffer(i, s.buffers[i]); }
	for (int u = 0; u < 2; ++u) {
		const auto& t = s.tus[u];
		gl.BindTexture(u, reinterpret_cast<const PixelToaster::FloatingPointPixel*>(t.ptr),
		               t.width, t.height, t.stride, t.filter ? GL_LINEAR_MIPMAP_NEAREST : GL_NEAREST_MIPMAP_NEAREST); }
	gl.BindTexture3(s.tu3ptr, s.tu3dim);
	rmlm::mat4 vm, nm, pm;
	std::memcpy(vm.ff.data(), s.view_matrix, 64);
	std::memcpy(nm.ff.data(), s.normal_matrix, 64);
	std::memcpy(pm.ff.data(), s.projection_matrix, 64);
	gl.ViewMatrix(vm);
	gl.NormalMatrix(nm);
	gl.ProjectionMatrix(pm); }


template <typename T>
T Read(const uint8_t*& p) {
	T v; std::memcpy(&v, p, sizeof(T)); p += sizeof(T); return v; }


// Output canvases of one frame, created per store command and kept alive
// until the frame completes.
struct Canvases {
	std::vector<std::unique_ptr<rglr::TrueColorCanvas>> tc;
	std::vector<std::unique_ptr<rglr::FloatingPointCanvas>> fp;
	std::vector<std::unique_ptr<rglr::QFloat4Canvas>> quads; };


// Replays the caller's stream into the reference's GL recorder.
int Replay(rglv::GL& gl, const uint8_t* cmds, size_t n, const rsrgpu_glstate* states, int nstates,
           Canvases& canvases) {
	using namespace rglv;
	const uint8_t* p = cmds;
	const uint8_t* end = cmds + n;
	while (p < end) {
		const uint8_t op = Read<uint8_t>(p);
		switch (op) {
		case CMD_EOF:
			return 0;
		case CMD_STATE: {
			auto idx = Read<uint64_t>(p);
			if (idx >= uint64_t(nstates)) return -1;
			ApplyState(gl, states[idx]); }
			break;
		case CMD_CLEAR:
			gl.Clear(Read<uint8_t>(p));
			break;
		case CMD_DRAW_ELEMENTS: {
			Read<uint8_t>(p);  // 0x14
			auto hint = Read<uint8_t>(p);
			auto count = Read<int32_t>(p);
			auto ptr = Read<const uint16_t*>(p);
			gl.DrawElements(GL_TRIANGLES, count, GL_UNSIGNED_SHORT, ptr, hint); }
			break;
		case CMD_DRAW_ARRAYS: {
			auto count = Read<int32_t>(p);
			gl.DrawArrays(GL_TRIANGLES, 0, count); }
			break;
		case CMD_DRAW_ELEMENTS_INSTANCED: {
			Read<uint8_t>(p);  // 0x14
			auto count = Read<int32_t>(p);
			auto ptr = Read<const uint16_t*>(p);
			auto ninst = Read<int32_t>(p);
			gl.DrawElementsInstanced(GL_TRIANGLES, count, GL_UNSIGNED_SHORT, ptr, ninst); }
			break;
		case CMD_DRAW_ARRAYS_INSTANCED: {
			auto count = Read<int32_t>(p);
			auto ninst = Read<int32_t>(p);
			gl.DrawArraysInstanced(GL_TRIANGLES, 0, count, ninst); }
			break;
		case CMD_STORE_COLOR_FULL_LINEAR_TC: {
			auto gamma = Read<uint8_t>(p);
			auto* c = Read<const rsrgpu_truecolor_canvas*>(p);
			canvases.tc.emplace_back(std::make_unique<rglr::TrueColorCanvas>(
				reinterpret_cast<PixelToaster::TrueColorPixel*>(c->data), c->width, c->height, c->stride));
			gl.StoreColor(canvases.tc.back().get(), gamma != 0); }
			break;
		case CMD_STORE_COLOR_FULL_LINEAR_FP:
		case CMD_STORE_COLOR_HALF_LINEAR_FP: {
			auto* c = Read<const rsrgpu_fp_canvas*>(p);
			canvases.fp.emplace_back(std::make_unique<rglr::FloatingPointCanvas>(
				reinterpret_cast<PixelToaster::FloatingPointPixel*>(c->data), c->width, c->height, c->stride));
			gl.StoreColor(canvases.fp.back().get(), op == CMD_STORE_COLOR_HALF_LINEAR_FP); }
			break;
		case CMD_STORE_COLOR_FULL_QUADS_FP: {
			auto* c = Read<const rsrgpu_qfloat4_canvas*>(p);
			canvases.quads.emplace_back(std::make_unique<rglr::QFloat4Canvas>(
				c->width, c->height, reinterpret_cast<rmlv::qfloat4*>(c->data), c->stride));
			gl.StoreColor(canvases.quads.back().get()); }
			break;
		case CMD_STORE_DEPTH_FULL_LINEAR_FP:
			gl.StoreDepth(Read<float*>(p));
			break;
		default:
			return -1; }}
	return 0; }


// Canonical tile stream (shared with the oracle and the GPU library): the
// reference's bytes with pointer fields removed and CMD_STATE carrying the
// ordinal of the state in order of first appearance.
void Canonical(const uint8_t* s, std::map<const void*, uint32_t>& ordinals, std::vector<uint8_t>& out) {
	using namespace rglv;
	auto put8 = [&](uint8_t v) { out.push_back(v); };
	auto put16 = [&](uint16_t v) { out.push_back(v & 0xff); out.push_back(v >> 8); };
	auto put32 = [&](uint32_t v) { for (int i = 0; i < 4; ++i) out.push_back((v >> (8*i)) & 0xff); };
	const uint8_t* p = s;
	while (true) {
		const uint8_t op = Read<uint8_t>(p);
		put8(op);
		switch (op) {
		case CMD_EOF:
			return;
		case CMD_STATE: {
			auto sp = Read<const void*>(p);
			Read<const void*>(p);  // uniforms
			auto it = ordinals.find(sp);
			uint32_t ord;
			if (it == ordinals.end()) { ord = uint32_t(ordinals.size()); ordinals[sp] = ord; }
			else { ord = it->second; }
			put32(ord); }
			break;
		case CMD_CLEAR:
			put8(Read<uint8_t>(p));
			break;
		case CMD_STORE_COLOR_FULL_LINEAR_TC:
			put8(Read<uint8_t>(p));
			Read<const void*>(p);
			break;
		case CMD_STORE_DEPTH_FULL_LINEAR_FP:
		case CMD_STORE_COLOR_FULL_LINEAR_FP:
		case CMD_STORE_COLOR_HALF_LINEAR_FP:
		case CMD_STORE_COLOR_FULL_QUADS_FP:
			Read<const void*>(p);
			break;
		case CMD_DRAW_INLINE:
		case CMD_DRAW_INLINE_INSTANCED:
			while (true) {
				auto w = Read<uint16_t>(p);
				put16(w);
				if (w == 0xffff) break;
				if (op == CMD_DRAW_INLINE_INSTANCED) put16(Read<uint16_t>(p));
				put16(Read<uint16_t>(p));
				put16(Read<uint16_t>(p)); }
			break;
		case CMD_CLIPPED_TRI:
			put16(Read<uint16_t>(p));
			put16(Read<uint16_t>(p));
			put16(Read<uint16_t>(p));
			break;
		default:
			return; }}}

}  // namespace harness
}  // namespace rqdq


using namespace rqdq;

extern "C" {

// Starts the jobsys pool (threads includes the calling thread).
int rsrref_init(int threads) {
	if (harness::g_session != nullptr) return 0;
	rclmt::jobsys::telemetryEnabled = false;
	rclmt::jobsys::init(threads);
	rclmt::jobsys::work_start();
	auto* s = new harness::Session;
	s->threads = threads;
	s->gpu = std::make_unique<harness::InspectableGPU>(threads, "oracle");
	auto& gpu = *s->gpu;
	harness::InstallDrawStates<harness::GouraudProgram>(gpu);
	harness::InstallDrawStates<rqv::AmyProgram>(gpu);
	harness::InstallDrawStates<rqv::OBJ1Program>(gpu);
	harness::InstallDrawStates<rqv::ManyProgram>(gpu);
	gpu.Install(harness::GouraudProgram::id, 0, rglv::GPUBltImpl<harness::GouraudProgram>::MakeBltProgramPtrs());
	gpu.Install(rqv::DefaultPostProgram::id, 0, rglv::GPUBltImpl<rqv::DefaultPostProgram>::MakeBltProgramPtrs());
	gpu.Install(rqv::ExposurePostProgram::id, 0, rglv::GPUBltImpl<rqv::ExposurePostProgram>::MakeBltProgramPtrs());
	rglv::doubleBuffer = false;
	harness::g_session = s;
	return 0; }

// Renders one frame.  Outputs land in the buffers the stream points to.
int rsrref_render(const uint8_t* cmds, size_t n, const rsrgpu_glstate* states, int nstates,
                  int width, int height, int tile_blocks_x, int tile_blocks_y) {
	auto* s = harness::g_session;
	if (s == nullptr) return -1;
	namespace jobsys = rclmt::jobsys;
	auto& gpu = *s->gpu;
	jobsys::reset();
	gpu.Reset(rmlv::ivec2{ width, height }, rmlv::ivec2{ tile_blocks_x, tile_blocks_y });
	harness::Canvases canvases;
	if (harness::Replay(gpu.IC(), cmds, n, states, nstates, canvases) != 0) return -1;
	auto* done = jobsys::make_job(jobsys::noop);
	auto* run = gpu.Run();
	jobsys::add_link(run, done);
	jobsys::run(run);
	jobsys::wait(done);
	return 0; }

// Canonical tile streams of the last frame, same layout as rsrgpu_dump_tiles.
int rsrref_dump_tiles(uint8_t* out, size_t capacity, size_t* needed) {
	auto* s = harness::g_session;
	if (s == nullptr) return -1;
	std::map<const void*, uint32_t> ordinals;
	std::vector<uint8_t> all;
	for (int t = 0; t < s->gpu->NumTiles(); ++t) {
		std::vector<uint8_t> one;
		harness::Canonical(s->gpu->TileStream(t), ordinals, one);
		uint32_t len = uint32_t(one.size());
		for (int i = 0; i < 4; ++i) all.push_back((len >> (8*i)) & 0xff);
		all.insert(all.end(), one.begin(), one.end()); }
	*needed = all.size();
	if (out != nullptr && capacity >= all.size()) {
		std::memcpy(out, all.data(), all.size()); }
	return 0; }

int rsrref_dump_clipped(rsrgpu_clipped_vertex* out, int capacity, int* count) {
	auto* s = harness::g_session;
	if (s == nullptr) return -1;
	const auto& cv = s->gpu->Clipped();
	*count = int(cv.size());
	for (int i = 0; i < int(cv.size()) && i < capacity; ++i) {
		std::memset(&out[i], 0, sizeof(out[i]));
		out[i].coord[0] = cv[i].coord.x; out[i].coord[1] = cv[i].coord.y;
		out[i].coord[2] = cv[i].coord.z; out[i].coord[3] = cv[i].coord.w;
		std::memcpy(out[i].data, cv[i].data, sizeof(out[i].data)); }
	return 0; }

// A texture built the way rsr's image loader builds one: PNGToTexture's
// per-pixel conversion with the reference's ryg::srgb8_to_float
// (src/rgl/rglr/rglr_texture_load.cxx:40-63; the loop is restated here, it
// sits in an unnamed namespace behind the PNG decoder), then the reference's
// own rglr::Texture::maybe_make_mipmap (src/rgl/rglr/rglr_texture.cxx:33-80).
// out receives buf (texels * 4 floats); returns -1 if cap (texels) is short.
int rsrref_texture_from_rgba8(const uint8_t* rgba8, int w, int h, int premultiply, float* out, size_t cap,
                              int* power) {
	rcls::vector<PixelToaster::FloatingPointPixel> pc(size_t(w) * size_t(h));
	const uint8_t* ic = rgba8;
	for (auto& dst : pc) {
		dst.r = ryg::srgb8_to_float(*(ic++));
		dst.g = ryg::srgb8_to_float(*(ic++));
		dst.b = ryg::srgb8_to_float(*(ic++));
		dst.a = *(ic++) / 255.0F;
		if (premultiply) {
			dst.r *= dst.a;
			dst.g *= dst.a;
			dst.b *= dst.a; }}
	rglr::Texture tex{ pc, w, h, w, "oracle", -1, false };
	tex.maybe_make_mipmap();
	if (cap < tex.buf.size()) return -1;
	std::memcpy(out, tex.buf.data(), tex.buf.size() * sizeof(PixelToaster::FloatingPointPixel));
	*power = tex.pow;
	return 0; }

// rglr::Texture::maybe_make_mipmap on float texels (level 0 in texels).
int rsrref_texture_mipmap(float* texels, int w, int h, size_t cap, int* power) {
	rcls::vector<PixelToaster::FloatingPointPixel> pc(size_t(w) * size_t(h));
	std::memcpy(pc.data(), texels, pc.size() * sizeof(PixelToaster::FloatingPointPixel));
	rglr::Texture tex{ pc, w, h, w, "oracle", -1, false };
	tex.maybe_make_mipmap();
	*power = tex.pow;
	if (!tex.mipmap) return 0;
	if (cap < tex.buf.size()) return -1;
	std::memcpy(texels, tex.buf.data(), tex.buf.size() * sizeof(PixelToaster::FloatingPointPixel));
	return 0; }

// rsr's own KawaseBlurFilter over the whole destination (one job's rows).
int rsrref_kawase(const float* src, int sw, int sh, int sstride, float* dst, int dw, int dh, int dstride, int d) {
	using PT = PixelToaster::FloatingPointPixel;
	const rglr::FloatingPointCanvas s(reinterpret_cast<PT*>(const_cast<float*>(src)), sw, sh, sstride);
	rglr::FloatingPointCanvas o(reinterpret_cast<PT*>(dst), dw, dh, dstride);
	rglr::KawaseBlurFilter(s, o, d, 0, dh);
	return 0; }

// rsr's own rglr::Filter template with the $glow node's shader (restated as
// harness::GlowShader; the node's copy sits in an unnamed namespace).
int rsrref_glow(const float* image, int istride, const float* blur, int bw, int bh, int bstride, uint32_t* out,
                int ostride, int w, int h, int srgb) {
	using PT = PixelToaster::FloatingPointPixel;
	const rglr::QFloat4Canvas src1(w, h, reinterpret_cast<rmlv::qfloat4*>(const_cast<float*>(image)), istride);
	const rglr::FloatingPointCanvas src2(reinterpret_cast<PT*>(const_cast<float*>(blur)), bw, bh, bstride);
	rglr::TrueColorCanvas dst(reinterpret_cast<PixelToaster::TrueColorPixel*>(out), w, h, ostride);
	const rmlg::irect rect{ { 0, 0 }, { w, h } };
	if (srgb) rglr::Filter<harness::GlowShader, rglr::sRGB>(src1, src2, dst, rect);
	else rglr::Filter<harness::GlowShader, rglr::LinearColor>(src1, src2, dst, rect);
	return 0; }

}  // extern "C"

extern "C" int rsrref_shutdown() {
	if (rqdq::harness::g_session == nullptr) return 0;
	rqdq::rclmt::jobsys::work_end();
	rqdq::rclmt::jobsys::stop();
	rqdq::rclmt::jobsys::join();
	delete rqdq::harness::g_session;
	rqdq::harness::g_session = nullptr;
	return 0; }
