// gen_srgb_lut.cxx -- golden output table of the reference's sRGB8 encoder.
//
// rsr packs colour with ryg::float_to_srgb8_var2_SSE2
// (3rdparty/ryg-srgb/ryg-srgb.h:183-219, called from
// src/rgl/rglr/rglr_canvas_util.hxx:15-19).  After clamping to
// [2^-13, 1-eps] its result depends only on the top 20 bits of the float
// (exponent and 11 mantissa bits).  This program runs the reference function
// on every such input, checks the property on random low bits, and writes
// the 26 624 outputs (index = (bits >> 12) - ((127-13) << 11)) to stdout as
// raw bytes.  The oracle loads this golden vector to reproduce the
// reference's quantisation; it is generated from the reference build:
//   make -C oracle/ref golden
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include "3rdparty/ryg-srgb/ryg-srgb.h"

static uint8_t enc(uint32_t bits) {
	float f; std::memcpy(&f, &bits, 4);
	__m128i r = ryg::float_to_srgb8_var2_SSE2(_mm_set1_ps(f));
	return uint8_t(_mm_cvtsi128_si32(r)); }

int main() {
	const uint32_t lo = (127u - 13u) << 23, hi = 0x3f7fffffu;
	std::mt19937 rng(1234);
	std::vector<uint8_t> lut;
	for (uint32_t k = lo >> 12; k <= (hi >> 12); ++k) {
		uint8_t v = enc(k << 12);
		for (int j = 0; j < 8; ++j) {
			uint32_t b = (k << 12) | (rng() & 0xfffu);
			if (b > hi) b = hi;
			if (enc(b) != v) { std::fprintf(stderr, "low bits matter at %08x\n", b); return 1; }}
		lut.push_back(v); }
	// clamp behaviour below/above the range and for NaN
	if (enc(0) != lut.front() || enc(0x7fc00000u) != lut.front() || enc(0x3f800000u) != lut.back()) {
		std::fprintf(stderr, "unexpected clamp\n"); return 1; }
	std::fwrite(lut.data(), 1, lut.size(), stdout);
	return 0; }
