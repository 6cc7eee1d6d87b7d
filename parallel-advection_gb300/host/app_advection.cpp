// advection [file.ini] [--fp32] [--fused K] [--hi-lo]: the reference's advection driver
// (src/advection.cpp:14-71) over the C ABI. Same .ini keys, same printed
// blocks (runtime parameters, RESULTS_VALIDATION, PERF_DIAGS).
//
// kernelImpl selects the strategy like impl_selector: NDRange / AdaptiveWg /
// GB300 run in place, BasicRange out of place into a second buffer (the
// reference's global scratch), Plain runs the per-cell FP64 reference math.
// The field is FP64 like the reference unless --fp32 is given (FP64 steps run
// in FP32-pair arithmetic, within 2e-13 max|f| per step of FP64 arithmetic).
// --fused K runs K time steps per kernel launch on shared-memory strips (FP32:
// the same bits; FP64: FP64 arithmetic; one call for all maxIter steps
// instead of a wait after each); --hi-lo (FP32,
// with --fused) keeps each cell as an FP32 hi + lo pair between the steps of
// a launch, rounding to FP32 once per launch.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>

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
        std::string input_file = "advection.ini";
        bool fp32 = false, hi_lo = false;
        int fused = 1;
        for (int i = 1; i < argc; ++i) {
            if (std::strcmp(argv[i], "--fp32") == 0) fp32 = true;
            else if (std::strcmp(argv[i], "--hi-lo") == 0) hi_lo = true;
            else if (std::strcmp(argv[i], "--fused") == 0 && i + 1 < argc) fused = std::atoi(argv[++i]);
            else input_file = argv[i];
        }
        if (fused < 1) throw std::invalid_argument("--fused needs K >= 1");
        ConfigMap cm(input_file);
        AdvParams p;
        p.setup(cm);
        int impl = 0, inplace = 1;
        check(bkma_impl_from_name(p.kernelImpl.c_str(), &impl, &inplace));

        cudaDeviceProp prop{};
        cuda_check(cudaGetDeviceProperties(&prop, 0), "cudaGetDeviceProperties");
        std::cout << "Using device: " << prop.name << "\n";
        p.print();

        const size_t cells = p.n0 * p.n1 * p.n2;
        const size_t es = fp32 ? 4 : 8;
        void *data = nullptr, *scratch = nullptr;
        cuda_check(cudaMalloc(&data, cells * es), "cudaMalloc");
        if (!inplace) cuda_check(cudaMalloc(&scratch, cells * es), "cudaMalloc");

        bkma_adv_desc d{};
        d.n0 = (int64_t)p.n0;
        d.n1 = (int64_t)p.n1;
        d.n2 = (int64_t)p.n2;
        d.dtype = fp32 ? BKMA_F32 : BKMA_F64;
        d.degree = 5;
        d.weights = BKMA_W_REFERENCE;
        d.impl = impl;
        d.inplace = inplace;
        d.dt = p.dt;
        d.minX = p.minRealX;
        d.maxX = p.maxRealX;
        d.minVx = p.minRealVx;
        d.maxVx = p.maxRealVx;
        bkma_adv_plan *plan = nullptr;
        check(bkma_adv_plan_create(&d, &plan));
        if (hi_lo) check(bkma_adv_plan_set_fused_state(plan, BKMA_FUSED_F32X2));
        if (fused > 1) check(bkma_adv_plan_set_fusion(plan, fused));
        check(bkma_adv_fill(plan, data, 0, 0.0, 0, nullptr));  // fill_buffer_adv
        cuda_check(cudaDeviceSynchronize(), "fill");

        const auto start = std::chrono::high_resolution_clock::now();
        if (fused > 1) {  // every step in one call, K per launch
            check(bkma_adv_step(plan, data, inplace ? nullptr : scratch, (int32_t)p.maxIter, nullptr));
            if (!inplace && p.maxIter > 0) std::swap(data, scratch);
            cuda_check(cudaDeviceSynchronize(), "steps");
        }
        for (size_t t = 0; fused == 1 && t < p.maxIter; ++t) {
            if (inplace) {
                check(bkma_adv_step(plan, data, nullptr, 1, nullptr));
            } else {
                check(bkma_adv_step(plan, data, scratch, 1, nullptr));
                std::swap(data, scratch);
            }
            cuda_check(cudaDeviceSynchronize(), "step");  // Q.wait() per step
        }
        const auto end = std::chrono::high_resolution_clock::now();
        const double elapsed = std::chrono::duration<double>(end - start).count();

        double hi = 0, lo = 0;
        check(bkma_adv_validate(plan, data, (int64_t)p.maxIter, &hi, &lo, nullptr));
        std::cout << "\nRESULTS_VALIDATION:" << std::endl;
        std::cout << "Highest L1 error found: " << hi << " (lowest is " << lo << ")\n" << std::endl;

        const double gcells = ((double)cells * (double)p.maxIter / elapsed) / 1e9;
        std::cout << "PERF_DIAGS:" << std::endl;
        std::cout << "elapsed_time: " << elapsed << " s\n";
        std::cout << "upd_cells_per_sec: " << gcells << " Gcell/sec\n";
        std::cout << "estimated_throughput: " << gcells * (double)es * 2 << " GB/s" << std::endl;

        bkma_adv_plan_destroy(plan);
        cudaFree(data);
        cudaFree(scratch);
        return 0;
    } catch (const std::exception &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
}
