// Status reporting and host-side fault injection for the C ABI.
//
// The reference reports nothing and exits the process on allocation failure
// (bfs/src/utils.c:102-109); every entry point here returns an alb_status and
// leaves a thread-local message instead.
#include <atomic>
#include <cstdarg>
#include <cstdio>

#include "internal.h"

namespace alb {

static thread_local char g_msg[512] = "";
static std::atomic<int32_t> g_fail_after{0};
static std::atomic<int32_t> g_dbg_level{-1}, g_dbg_block{0}, g_dbg_short_bulk{0};
static std::atomic<int64_t> g_dbg_timeout_us{0};

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

alb_status fail(alb_status code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    return code;
}

bool injected_alloc_failure() {
    int32_t k = g_fail_after.load();
    while (k > 0) {
        if (g_fail_after.compare_exchange_weak(k, k - 1)) return k == 1;
    }
    return false;
}

DeviceWaits device_waits(uint64_t barrier_ns, uint64_t bulk_ns) {
    DeviceWaits w;
    const int64_t us = g_dbg_timeout_us.load();
    w.barrier_ns = us > 0 ? (uint64_t)us * 1000u : barrier_ns;
    w.bulk_ns = us > 0 ? (uint64_t)us * 1000u : bulk_ns;
    w.withhold_level = g_dbg_level.load();
    w.withhold_block = g_dbg_block.load();
    w.short_bulk = g_dbg_short_bulk.load();
    return w;
}

}  // namespace alb

extern "C" {

const char *alb_last_error(void) { return alb::g_msg; }

const char *alb_version(void) { return "albba_gb300 0.1 (sm_103a)"; }

void alb_debug_fail_alloc_after(int32_t k) { alb::g_fail_after.store(k > 0 ? k : 0); }

void alb_debug_device_waits(int32_t withhold_level, int32_t withhold_block, int32_t short_bulk,
                            int64_t timeout_us) {
    alb::g_dbg_level.store(withhold_level);
    alb::g_dbg_block.store(withhold_block > 0 ? withhold_block : 0);
    alb::g_dbg_short_bulk.store(short_bulk ? 1 : 0);
    alb::g_dbg_timeout_us.store(timeout_us > 0 ? timeout_us : 0);
}

}  // extern "C"
