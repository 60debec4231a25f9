// Selector parameter storage (device + host copies) and its C ABI.
// Training kernels live in selector_train.cu.
#include <cstring>
#include <mutex>

#include "graph.h"
#include "selector.cuh"

namespace alb {

// Two parameter blocks (0: single-root BFS, 1: 64-root batched BFS); the
// element after the parameters is 1.0f once weights are loaded. Fixed
// addresses, so cached CUDA graphs may hold the pointer.
// 16-byte aligned rows (1444 floats each): mlp_select_warp reads them as float4
__device__ __align__(16) float g_selector[2][kMlpParams + 1];

static std::mutex g_sel_mu;
static float g_sel_host[2][kMlpParams];
static bool g_sel_loaded[2] = {false, false};

const float *selector_device_params(int which) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_selector) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (const float *)p + (size_t)which * (kMlpParams + 1);
}

bool selector_host_params(int which, float *out) {
    std::lock_guard<std::mutex> lk(g_sel_mu);
    if (!g_sel_loaded[which]) return false;
    std::memcpy(out, g_sel_host[which], sizeof(float) * kMlpParams);
    return true;
}

}  // namespace alb

using namespace alb;

extern "C" {

alb_status alb_selector_load(int32_t which, const float *params) {
    if (which < 0 || which > 1 || !params) return fail(ALB_ERR_INVALID, "alb_selector_load: bad arguments");
    float buf[kMlpParams + 1];
    std::memcpy(buf, params, sizeof(float) * kMlpParams);
    buf[kMlpParams] = 1.0f;
    ALB_CK(cudaMemcpyToSymbol(g_selector, buf, sizeof(buf), sizeof(buf) * (size_t)which));
    std::lock_guard<std::mutex> lk(g_sel_mu);
    std::memcpy(g_sel_host[which], params, sizeof(float) * kMlpParams);
    g_sel_loaded[which] = true;
    return ALB_OK;
}

alb_status alb_selector_clear(int32_t which) {
    if (which < 0 || which > 1) return fail(ALB_ERR_INVALID, "alb_selector_clear: bad selector id");
    float zero = 0.0f;
    ALB_CK(cudaMemcpyToSymbol(g_selector, &zero, sizeof(float),
                              sizeof(float) * ((size_t)which * (kMlpParams + 1) + kMlpParams)));
    std::lock_guard<std::mutex> lk(g_sel_mu);
    g_sel_loaded[which] = false;
    return ALB_OK;
}

}  // extern "C"
