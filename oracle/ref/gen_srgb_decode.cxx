// gen_srgb_decode.cxx -- golden output table of the reference's sRGB8 decoder.
//
// rsr converts texture bytes to linear float with ryg::srgb8_to_float
// (3rdparty/ryg-srgb/ryg-srgb.h:33-56; src/rgl/rglr/rglr_texture_load.cxx:
// 52-54).  This program runs the reference function on all 256 inputs and
// writes the float results to stdout as raw little-endian bytes.  The oracle's
// texture upload uses this golden vector and tests check the library's
// constant table against it:
//   make -C oracle/ref golden-decode
#include <cstdint>
#include <cstdio>
#include "3rdparty/ryg-srgb/ryg-srgb.h"

int main() {
	for (int i = 0; i < 256; ++i) {
		const float v = ryg::srgb8_to_float(static_cast<uint8_t>(i));
		std::fwrite(&v, 4, 1, stdout); }
	return 0; }
