// Allocation-free entry point for the in-place BF16 tensor-core conv1d.
//
// Some callers cannot call cudaMalloc while they run: runtimes that hand all
// device memory to their own pool at start-up and forbid further driver
// allocations, and latency-critical loops where an allocation (and the
// implicit device synchronization that cudaFree brings) is not allowed. The
// plan-based bkma_conv_run needs plan-owned scratch (the halo snapshot and
// the packed weights), which bkma_conv_plan_create allocates. This entry
// point instead uses one file-scope device array, reserved when the library
// is loaded and held by every GPU that loads it until the process exits.
//
// The array's name is only a host-side stand-in in host code; its device
// address is looked up once per device (cudaGetSymbolAddress, with that device
// current) on the first call, which should therefore happen before any stream
// capture. All calls share the array: it keeps the last call's contents, the
// status word is cleared at every call, and calls that overlap on the GPU
// (different streams, or different host threads on the same device) race on it.
// bkma_conv1d_noalloc_status reads the status word of the last call.
#include <array>
#include <mutex>
#include <string>

#include "conv.cuh"

// File-scope scratch of the allocation-free entry point (16 MiB per device).
static __device__ __align__(256) unsigned char g_conv_noalloc_scratch[16u << 20];

namespace bkma {
namespace {

constexpr size_t kNoAllocScratchBytes = sizeof(g_conv_noalloc_scratch);
constexpr size_t kStatusOff = 0;                      // int status word
constexpr size_t kWpackOff = 256;                     // packed weights
constexpr size_t kWpackMax = 512u << 10;
constexpr size_t kHaloOff = kWpackOff + kWpackMax;    // halo snapshot
constexpr size_t kHaloMax = kNoAllocScratchBytes - kHaloOff;

std::mutex g_addr_mu;
std::array<unsigned char *, 128> g_addr{};  // device address of the array, per device

bkma_status scratch_address(unsigned char **out) {
    int dev = 0;
    BKMA_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= (int)g_addr.size())
        return fail(BKMA_ERR_UNSUPPORTED, "allocation-free conv1d: device index out of range");
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[(size_t)dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_conv_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_conv_noalloc_scratch)");
        g_addr[(size_t)dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[(size_t)dev];
    return BKMA_OK;
}

}  // namespace
}  // namespace bkma

using namespace bkma;

extern "C" bkma_status bkma_conv1d_bf16_inplace_noalloc(void *data, const void *weight,
                                                        const void *bias, int64_t batch,
                                                        int64_t channels, int64_t length,
                                                        int64_t ksize, void *stream) try {
    BKMA_CHECK_ARG(data && weight, "bkma_conv1d_bf16_inplace_noalloc: null data or weight");
    bkma_conv_desc d{};
    d.batch = batch;
    d.cin = channels;
    d.cout = channels;
    d.length = length;
    d.ksize = ksize;
    d.n2 = 1;
    d.dtype = BKMA_BF16;
    d.semantics = BKMA_CONV_TORCH;
    d.impl = BKMA_CONV_TENSOR;
    d.inplace = 1;
    bkma_status s = conv_check_desc(d);  // the same bounds as bkma_conv_plan_create
    if (s != BKMA_OK) return s;
    size_t halo_bytes = 0, wpack_bytes = 0;
    s = conv_tc_scratch_need(d, &halo_bytes, &wpack_bytes);
    if (s != BKMA_OK) return s;
    if (halo_bytes > kHaloMax || wpack_bytes > kWpackMax)
        return fail(BKMA_ERR_INVALID_ARG,
                    "bkma_conv1d_bf16_inplace_noalloc: this shape needs " +
                        std::to_string(halo_bytes) + " bytes of halo scratch and " +
                        std::to_string(wpack_bytes) + " of packed weights; the fixed device array "
                        "holds at most " + std::to_string(kHaloMax) + " and " +
                        std::to_string(kWpackMax) +
                        " (halo <= 3840 * channels * 2 * max(8, round_up(ksize-1, 8)) bytes); "
                        "use bkma_conv_run");
    unsigned char *base = nullptr;
    s = scratch_address(&base);
    if (s != BKMA_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    int *status = reinterpret_cast<int *>(base + kStatusOff);
    BKMA_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    return conv_tc_run_into(d, data, weight, bias, base + kHaloOff, base + kWpackOff, status, st);
} BKMA_ABI_CATCH("bkma_conv1d_bf16_inplace_noalloc")

extern "C" bkma_status bkma_conv1d_noalloc_status(void *stream) try {
    unsigned char *base = nullptr;
    bkma_status s = scratch_address(&base);
    if (s != BKMA_OK) return s;
    BKMA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    int *status = reinterpret_cast<int *>(base + kStatusOff);
    int v = 0;
    BKMA_CUDA_TRY(cudaMemcpy(&v, status, sizeof(int), cudaMemcpyDeviceToHost));
    BKMA_CUDA_TRY(cudaMemset(status, 0, sizeof(int)));
    if (v != 0)
        return fail((bkma_status)v,
                    "bkma_conv1d_bf16_inplace_noalloc: a bounded device wait timed out");
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_conv1d_noalloc_status")
