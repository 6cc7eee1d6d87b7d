// ABI-wide entry points: version, thread-local error message, and the
// strategy-name selector (impl_selector, src/tools/impl_selector.hpp:31-49).
#include <algorithm>
#include <cctype>
#include <string>

#include "common.cuh"

namespace bkma {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string &msg) { g_last_error = msg; }
bkma_status fail(bkma_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}
bkma_status cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                   cudaGetErrorString(e) + ")";
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return BKMA_ERR_NO_DEVICE;
    return BKMA_ERR_CUDA;
}
}  // namespace bkma

extern "C" {

int32_t bkma_abi_version(void) { return BKMA_ABI_VERSION; }

const char *bkma_last_error(void) { return bkma::g_last_error.c_str(); }

bkma_status bkma_impl_from_name(const char *name, int32_t *impl, int32_t *inplace) {
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
}

}  // extern "C"
