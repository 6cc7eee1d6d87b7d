#include "Params.hpp"

#include <iostream>

namespace bkma_host {

void AdvParams::setup(const ConfigMap &cm) {
    n1 = (size_t)cm.getInteger("problem", "n1", 1024);
    n0 = (size_t)cm.getInteger("problem", "n0", 1024);
    n2 = (size_t)cm.getInteger("problem", "n2", 1024);
    maxIter = (size_t)cm.getInteger("problem", "maxIter", 50);

    dt = cm.getFloat("problem", "dt", 0.0001f);
    minRealX = cm.getFloat("problem", "minRealX", 0.0f);
    maxRealX = cm.getFloat("problem", "maxRealX", 1.0f);
    minRealVx = cm.getFloat("problem", "minRealVx", -1.0f);
    maxRealVx = cm.getFloat("problem", "maxRealVx", 1.0f);

    kernelImpl = cm.getString("impl", "kernelImpl", "AdaptiveWg");
    inplace = cm.getBool("impl", "inplace", true);

    gpu = cm.getBool("optimization", "gpu", true);
    pref_wg_size = (size_t)cm.getInteger("optimization", "pref_wg_size", 512);
    seq_size0 = (size_t)cm.getInteger("optimization", "seq_size0", 1);
    seq_size2 = (size_t)cm.getInteger("optimization", "seq_size2", 1);

    outputSolution = cm.getBool("io", "outputSolution", false);
    update_deltas();
}

void AdvParams::update_deltas() {
    realWidthX = maxRealX - minRealX;
    dx = realWidthX / (double)n1;
    dvx = (maxRealVx - minRealVx) / (double)n0;
    inv_dx = 1 / dx;
}

void AdvParams::print() const {
    std::cout << "##########################\n"
              << "Runtime parameters:\n"
              << "##########################\n"
              << "kernelImpl  : " << kernelImpl << "\n"
              << "inplace     : " << inplace << "\n"
              << "gpu         : " << gpu << "\n"
              << "maxIter     : " << maxIter << "\n"
              << "n0 (nvx)    : " << n0 << "\n"
              << "n1 (nx)     : " << n1 << "\n"
              << "n2          : " << n2 << "\n"
              << "pref_wg_size: " << pref_wg_size << "\n"
              << "seq_size0   : " << seq_size0 << "\n"
              << "seq_size2   : " << seq_size2 << "\n"
              << "dt          : " << dt << "\n"
              << "dx          : " << dx << "\n"
              << "dvx         : " << dvx << "\n"
              << "minRealX    : " << minRealX << "\n"
              << "maxRealX    : " << maxRealX << "\n"
              << "minRealVx   : " << minRealVx << "\n"
              << "maxRealVx   : " << maxRealVx << "\n"
              << std::endl;
}

void Conv1dParams::setup(const ConfigMap &cm) {
    length = (size_t)cm.getInteger("problem", "length", 1024);
    channel_in = (unsigned short)cm.getInteger("problem", "channel_in", 3);
    channel_out = channel_in;  // constraint (Conv1dParams.cpp:48)
    k = (unsigned short)cm.getInteger("problem", "k", 3);
    total_batch_size = (size_t)cm.getInteger("problem", "total_batch_size", 262144);
    batch_size_n2 = (size_t)cm.getInteger("problem", "batch_size_n2", 512);
    n0 = total_batch_size / batch_size_n2;
    n1 = length * channel_out;
    n2 = batch_size_n2;
    n_write = compute_output_size(length, k);

    kernelImpl = cm.getString("impl", "kernelImpl", "AdaptiveWg");
    inplace = cm.getBool("impl", "inplace", true);

    gpu = cm.getBool("optimization", "gpu", true);
    pref_wg_size = (unsigned short)cm.getInteger("optimization", "pref_wg_size", 512);
    seq_size0 = (size_t)cm.getInteger("optimization", "seq_size0", 1);
    seq_size2 = (size_t)cm.getInteger("optimization", "seq_size2", 1);
}

void Conv1dParams::print() const {
    std::cout << "##########################\n"
              << "Runtime parameters:\n"
              << "##########################\n"
              << "kernelImpl   : " << kernelImpl << "\n"
              << "inplace      : " << inplace << "\n"
              << "gpu          : " << gpu << "\n"
              << "n0           : " << n0 << "\n"
              << "n1           : " << n1 << "\n"
              << "n2           : " << n2 << "\n"
              << "pref_wg_size : " << pref_wg_size << "\n"
              << "seq_size0    : " << seq_size0 << "\n"
              << "seq_size2    : " << seq_size2 << "\n"
              << "batch_size   : " << total_batch_size << "\n"
              << "length       : " << length << "\n"
              << "channels(i/o): " << channel_in << "\n"
              << "k            : " << k << "\n"
              << "batch_n2     : " << batch_size_n2 << "\n"
              << "n_write      : " << n_write << "\n"
              << std::endl;
}

}  // namespace bkma_host
