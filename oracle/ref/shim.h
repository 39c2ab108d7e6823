// shim.h -- force-included when compiling rsr's MSVC/clang-cl sources with
// g++ for the oracle build.  Maps the few Microsoft-specific names the
// rasteriser path uses onto GCC equivalents; it changes no arithmetic.
#pragma once
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <iostream>
#include <optional>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <deque>
#undef M_PI  // rmlv_math.hxx declares its own constexpr M_PI
#define _aligned_malloc(size, align) std::aligned_alloc((align), ((((size_t)(size)) + (align) - 1) / (align)) * (align))
#define _aligned_free(p) std::free(p)
static inline unsigned char _BitScanForward(unsigned long* idx, unsigned long mask) {
	if (mask == 0) return 0;
	*idx = (unsigned long)__builtin_ctzl(mask);
	return 1; }
#define __declspec(x) __rsr_declspec_##x
#define __rsr_declspec_align(n) __attribute__((aligned(n)))
#define __forceinline inline __attribute__((always_inline))
