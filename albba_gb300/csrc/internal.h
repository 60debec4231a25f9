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

// Limits and test hooks of the bounded device-side waits
// (alb_debug_device_waits): the given defaults unless a test shortened them.
struct DeviceWaits {
    uint64_t barrier_ns;     // grid barrier of the persistent kernels
    uint64_t bulk_ns;        // bulk copy into shared memory
    int32_t withhold_level;  // level at which one block skips its barrier arrival (-1: none)
    int32_t withhold_block;
    int32_t short_bulk;      // the staged pull expects 16 bytes its copy never delivers
};
DeviceWaits device_waits(uint64_t barrier_ns, uint64_t bulk_ns);

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
