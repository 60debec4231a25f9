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

}  // namespace alb

extern "C" {

const char *alb_last_error(void) { return alb::g_msg; }

const char *alb_version(void) { return "albba_gb300 0.1 (sm_103a)"; }

void alb_debug_fail_alloc_after(int32_t k) { alb::g_fail_after.store(k > 0 ? k : 0); }

}  // extern "C"
