// Host-side internals shared by the library's translation units.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "albba.h"

namespace alb {

// Thread-local last-error message (alb_last_error).
void set_error(const char *fmt, ...);
alb_status fail(alb_status code, const char *fmt, ...);

// Host fault injection for device allocations (alb_debug_fail_alloc_after).
bool injected_alloc_failure();

// SplitMix64 finaliser (Steele, Lea, Flood 2014; Vigna's splitmix64.c):
// a bijective 64-bit mix used for every counter-based random draw.
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform double in [0, 1) from the top 53 bits.
inline double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace alb
