// ABI-wide entry points: version, thread-local error message, and the
// strategy-name selector (impl_selector, src/tools/impl_selector.hpp:31-49).
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "common.cuh"

namespace bkma {
namespace {
// The last error message of the calling thread: a fixed buffer, so that
// recording an error never allocates and never throws.
thread_local char g_last_error[1024];

void store(const char *msg, size_t n) noexcept {
    n = std::min(n, sizeof(g_last_error) - 1);
    std::memcpy(g_last_error, msg, n);
    g_last_error[n] = 0;
}
}  // namespace
void set_error(const std::string &msg) noexcept { store(msg.data(), msg.size()); }
bkma_status fail(bkma_status s, const std::string &msg) noexcept {
    store(msg.data(), msg.size());
    return s;
}
bkma_status cuda_fail(cudaError_t e, const char *what) noexcept {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s)", what, cudaGetErrorName(e),
                  cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return BKMA_ERR_NO_DEVICE;
    return BKMA_ERR_CUDA;
}
bkma_status host_fail(const char *fn) noexcept {
    const char *why = "unknown C++ exception";
    try {
        throw;
    } catch (const std::bad_alloc &) {
        why = "out of host memory";
    } catch (const std::exception &e) {
        why = e.what();
    } catch (...) {
    }
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", fn, why);
    return BKMA_ERR_HOST;
}
}  // namespace bkma

extern "C" {

int32_t bkma_abi_version(void) { return BKMA_ABI_VERSION; }

const char *bkma_last_error(void) { return bkma::g_last_error; }

bkma_status bkma_impl_from_name(const char *name, int32_t *impl, int32_t *inplace) try {
    if (!name || !impl || !inplace)
        return bkma::fail(BKMA_ERR_INVALID_ARG, "bkma_impl_from_name: null argument");
    std::string s(name);
    std::string low = s;
    std::transform(low.begin(), low.end(), low.begin(),
                   [](unsigned char c) { return (char)std::tolower(c); });
    if (low == "ndrange" || low == "adaptivewg" || low == "staged" || low == "gb300" ||
        low == "cuda") {
        *impl = BKMA_ADV_STAGED;
        *inplace = 1;
    } else if (low == "basicrange") {
        *impl = BKMA_ADV_STAGED;
        *inplace = 0;
    } else if (low == "plain") {
        *impl = BKMA_ADV_PLAIN;
        *inplace = 1;
    } else {
        return bkma::fail(BKMA_ERR_UNSUPPORTED,
                          s + " is not a valid implementation name.\n"
                              "Should be: {BasicRange, NDRange, AdaptiveWg}");
    }
    bkma::set_error("");
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_impl_from_name")

}  // extern "C"
