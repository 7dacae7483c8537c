/* Stand-in for MSVC's <intrin.h> when the reference sources are compiled with
 * gcc for the oracle: the x86 intrinsics come from the gcc headers. */
#pragma once
#include <immintrin.h>
