// shim2.h -- declares an rmlv overload that rglr_texture_sampler.cxx names in
// a template that is never instantiated for it (MSVC accepts the unresolved
// name; GCC's two-phase lookup does not).
#pragma once
#include "src/rml/rmlv/rmlv_mvec4.hxx"
namespace rqdq { namespace rmlv {
void load_interleaved_lut(const uint32_t*, mvec4i, mvec4i&);
}}
