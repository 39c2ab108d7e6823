// intrin.h -- stands in for the MSVC header of the same name.
#pragma once
#include <x86intrin.h>
