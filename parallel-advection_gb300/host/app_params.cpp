// bkma_params adv|conv <file.ini>: parse an .ini the way the reference's
// drivers do and print the resulting parameters as one JSON object (used to
// check the parser against the reference's own parsing).
#include <cstdio>
#include <string>

#include "ConfigMap.hpp"
#include "Params.hpp"

using namespace bkma_host;

static void print_str(const char *k, const std::string &v, bool last = false) {
    std::printf("\"%s\": \"", k);
    for (char c : v) {
        if (c == '"' || c == '\\') std::printf("\\%c", c);
        else std::printf("%c", c);
    }
    std::printf("\"%s", last ? "" : ", ");
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s adv|conv file.ini\n", argv[0]);
        return 2;
    }
    ConfigMap cm(argv[2]);
    if (cm.parseError() < 0) {
        std::fprintf(stderr, "cannot open %s\n", argv[2]);
        return 1;
    }
    const std::string kind = argv[1];
    if (kind == "adv") {
        AdvParams p;
        p.setup(cm);
        std::printf("{\"n0\": %zu, \"n1\": %zu, \"n2\": %zu, \"max_iter\": %zu, ", p.n0, p.n1, p.n2,
                    p.maxIter);
        std::printf("\"dt\": %.17g, \"minX\": %.17g, \"maxX\": %.17g, \"minVx\": %.17g, "
                    "\"maxVx\": %.17g, \"width\": %.17g, \"dx\": %.17g, \"dvx\": %.17g, "
                    "\"inv_dx\": %.17g, ",
                    p.dt, p.minRealX, p.maxRealX, p.minRealVx, p.maxRealVx, p.realWidthX, p.dx,
                    p.dvx, p.inv_dx);
        std::printf("\"inplace\": %d, \"gpu\": %d, \"pref_wg_size\": %zu, \"seq_size0\": %zu, "
                    "\"seq_size2\": %zu, ",
                    (int)p.inplace, (int)p.gpu, p.pref_wg_size, p.seq_size0, p.seq_size2);
        print_str("kernel_impl", p.kernelImpl, true);
        std::printf("}\n");
        return 0;
    }
    if (kind == "conv") {
        Conv1dParams p;
        p.setup(cm);
        std::printf("{\"length\": %zu, \"channel_in\": %u, \"channel_out\": %u, \"k\": %u, "
                    "\"total_batch_size\": %zu, \"batch_size_n2\": %zu, \"n0\": %zu, \"n1\": %zu, "
                    "\"n2\": %zu, \"n_write\": %zu, \"inplace\": %d, \"gpu\": %d, "
                    "\"pref_wg_size\": %u, \"seq_size0\": %zu, \"seq_size2\": %zu, ",
                    p.length, p.channel_in, p.channel_out, p.k, p.total_batch_size, p.batch_size_n2,
                    p.n0, p.n1, p.n2, p.n_write, (int)p.inplace, (int)p.gpu, p.pref_wg_size,
                    p.seq_size0, p.seq_size2);
        print_str("kernel_impl", p.kernelImpl, true);
        std::printf("}\n");
        return 0;
    }
    std::fprintf(stderr, "unknown kind %s\n", argv[1]);
    return 2;
}
