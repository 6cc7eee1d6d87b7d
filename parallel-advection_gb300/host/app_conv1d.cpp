// conv1d [file.ini]: the reference's conv1d driver (src/conv1d.cpp:13-111)
// over the C ABI, FP64 with ConvSolver semantics (bit-identical to the
// reference), the reference's constant fills (data 7.3, warm-up data 1.0,
// weight 1.5, bias 1.0; src/tools/init.hpp:50-72), three warm-up runs, one
// timed run, and the same printed checks (normalized sums before/after,
// equality across batches, PERF_DIAGS).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ConfigMap.hpp"
#include "Params.hpp"
#include "bkma_gb300.h"

using namespace bkma_host;

static void check(bkma_status s) {
    if (s == BKMA_OK) return;
    if (s == BKMA_ERR_INVALID_ARG) throw std::invalid_argument(bkma_last_error());
    throw std::runtime_error(bkma_last_error());
}

static void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

int main(int argc, char **argv) {
    try {
        const std::string input_file = argc > 1 ? argv[1] : "conv1d.ini";
        ConfigMap cm(input_file);
        Conv1dParams p;
        p.setup(cm);
        cudaDeviceProp prop{};
        cuda_check(cudaGetDeviceProperties(&prop, 0), "cudaGetDeviceProperties");
        std::cout << "Using device: " << prop.name << "\n";
        p.print();

        const size_t n0 = p.n0, n1 = p.n1, n2 = p.n2, k = p.k, cin = p.channel_in;
        const size_t cells = n0 * n1 * n2;
        const size_t nweight = k * cin * cin;
        double *data = nullptr, *warm = nullptr, *weight = nullptr, *bias = nullptr;
        cuda_check(cudaMalloc(&data, cells * 8), "cudaMalloc");
        cuda_check(cudaMalloc(&warm, cells * 8), "cudaMalloc");
        cuda_check(cudaMalloc(&weight, nweight * 8), "cudaMalloc");
        cuda_check(cudaMalloc(&bias, cin * 8), "cudaMalloc");
        // fill_buffer_conv1d (src/tools/init.hpp:50-72), on the device
        check(bkma_fill(data, (int64_t)cells, BKMA_F64, 7.3, nullptr));
        check(bkma_fill(warm, (int64_t)cells, BKMA_F64, 1.0, nullptr));
        check(bkma_fill(weight, (int64_t)nweight, BKMA_F64, 1.5, nullptr));
        check(bkma_fill(bias, (int64_t)cin, BKMA_F64, 1.0, nullptr));

        bkma_conv_desc d{};
        d.batch = (int64_t)n0;
        d.cin = (int64_t)cin;
        d.cout = (int64_t)cin;
        d.length = (int64_t)p.length;
        d.ksize = (int64_t)k;
        d.n2 = (int64_t)n2;
        d.dtype = BKMA_F64;
        d.semantics = BKMA_CONV_REFERENCE;
        d.impl = BKMA_CONV_PLAIN;
        d.inplace = 1;
        bkma_conv_plan *plan = nullptr;
        check(bkma_conv_plan_create(&d, &plan));

        // sum_and_normalize_conv1d + validate_conv1d (src/tools/validation.hpp:
        // 84-156) as one device pass
        double mean = 0;
        int32_t equal = 0;
        check(bkma_conv_check(data, BKMA_F64, (int64_t)n0, (int64_t)n1, (int64_t)n2,
                              (int64_t)n1, &mean, &equal, nullptr));
        std::cout << std::endl << "Normalized Array before: " << mean << std::endl;
        for (int i = 0; i < 3; ++i) {  // warm-up
            check(bkma_conv_run(plan, warm, nullptr, weight, bias, nullptr));
            cuda_check(cudaDeviceSynchronize(), "warm-up");
        }
        const auto start = std::chrono::high_resolution_clock::now();
        check(bkma_conv_run(plan, data, nullptr, weight, bias, nullptr));
        cuda_check(cudaDeviceSynchronize(), "run");
        const auto end = std::chrono::high_resolution_clock::now();
        const double elapsed = std::chrono::duration<double>(end - start).count();

        check(bkma_conv_check(data, BKMA_F64, (int64_t)n0, (int64_t)n1, (int64_t)n2,
                              (int64_t)p.n_write, &mean, &equal, nullptr));
        std::cout << "Normalized Array after: " << mean << std::endl << std::endl;
        if (!equal)
            std::cout << "WARNING: Values at same position i1 are not equivalent throught the "
                         "batchs. Check implementation."
                      << std::endl;
        else
            std::cout << "All values data[:,i1,:] are equal." << std::endl;

        std::cout << "PERF_DIAGS:" << std::endl;
        std::cout << "elapsed_time: " << elapsed << " s\n";
        const double gcells = ((double)cells / elapsed) / 1e9;
        std::cout << "upd_cells_per_sec: " << gcells << " Gcell/sec\n";
        std::cout << "estimated_throughput: " << gcells * 8 * 2 << " GB/s" << std::endl;

        bkma_conv_plan_destroy(plan);
        cudaFree(data);
        cudaFree(warm);
        cudaFree(weight);
        cudaFree(bias);
        return 0;
    } catch (const std::exception &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
}
