// Runtime parameters of the two drivers, with the reference's keys, defaults
// and derived quantities:
//  - ADVParams / ADVParamsNonCopyable::setup, update_deltas
//    (src/config/AdvectionParams.hpp:10-74, AdvectionParams.cpp:64-103);
//  - Conv1dParams / Conv1dParamsNonCopyable::setup, compute_output_size
//    (src/config/Conv1dParams.hpp:10-49, Conv1dParams.cpp:44-76).
#pragma once
#include <cstddef>
#include <string>

#include "ConfigMap.hpp"

namespace bkma_host {

struct AdvParams {
    // values of a default-constructed ADVParams (AdvectionParams.hpp:14-53)
    bool gpu = false;
    bool outputSolution = false;
    size_t maxIter = 100;
    size_t n1 = 1024, n0 = 32, n2 = 32;
    size_t pref_wg_size = 128;
    size_t seq_size0 = 0, seq_size2 = 0;
    double dt = 0.0001;
    double dx = 0, dvx = 0, inv_dx = 0;
    double minRealX = 0, maxRealX = 1, realWidthX = 1;
    double minRealVx = 0, maxRealVx = 1;
    // ADVParamsNonCopyable extras
    std::string kernelImpl;
    bool inplace = false;

    AdvParams() { update_deltas(); }
    // ADVParamsNonCopyable::setup (AdvectionParams.cpp:64-92)
    void setup(const ConfigMap &cm);
    // ADVParams::update_deltas (AdvectionParams.cpp:96-103)
    void update_deltas();
    void print() const;
};

struct Conv1dParams {
    size_t length = 1024;
    unsigned short channel_in = 3, channel_out = 3, k = 3;
    size_t total_batch_size = 262144, batch_size_n2 = 512;
    size_t n0 = 0, n1 = 0, n2 = 0, n_write = 0;
    bool gpu = true;
    unsigned short pref_wg_size = 512;
    size_t seq_size0 = 1, seq_size2 = 1;
    bool inplace = true;
    std::string kernelImpl;

    // Conv1dParamsNonCopyable::setup (Conv1dParams.cpp:44-68)
    void setup(const ConfigMap &cm);
    // Conv1dParams::compute_output_size (Conv1dParams.cpp:72-76)
    static size_t compute_output_size(size_t Lin, unsigned short kernel_size) {
        return Lin - (kernel_size - 1);
    }
    void print() const;
};

}  // namespace bkma_host
