// psim_gb300 command line: the drop-in for `psim a.json [b.json ...]` (psim/src/main.cpp:10-31).
// Each model file is read, run on the GPU and written to ss_<name>.txt or per_<name>.txt next
// to it.  Options (before the files): --seed N, --fp64.  The messages are the reference's; the
// exit status is 1 when any file could not be read, run or written (the reference exits 0).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "psim_gb300.h"

int main(int argc, char** argv) {
    std::uint64_t seed = 1;
    std::int32_t precision = PSIM_PRECISION_FP32;
    std::vector<std::string> files;
    for (int i = 1; i < argc; ++i) {
        if (std::strcmp(argv[i], "--seed") == 0 && i + 1 < argc) {
            seed = std::strtoull(argv[++i], nullptr, 10);
        } else if (std::strcmp(argv[i], "--fp64") == 0) {
            precision = PSIM_PRECISION_FP64;
        } else {
            files.emplace_back(argv[i]);
        }
    }
    if (files.empty()) {
        std::printf("Need filenames\ndone\n");
        return 0;
    }
    int status = 0;
    for (const auto& f : files) {
        psim_model* m = nullptr;
        if (psim_model_load_json(f.c_str(), &m) != PSIM_OK) {
            std::fprintf(stderr, "%s\nThere was an error reading the data from the file at \"%s\"\n", psim_last_error(), f.c_str());
            status = 1;
            continue;
        }
        psim_model_set_options(m, seed, precision, nullptr);
        const auto t0 = std::chrono::steady_clock::now();
        if (psim_model_run(m) != PSIM_OK) {
            std::fprintf(stderr, "run failed for %s: %s\n", f.c_str(), psim_last_error());
            psim_model_destroy(m);
            status = 1;
            continue;
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("Time Taken: %g[s]\n", secs);
        if (psim_model_export(m, f.c_str(), secs) != PSIM_OK) {
            std::fprintf(stderr, "export failed for %s: %s\n", f.c_str(), psim_last_error());
            status = 1;
        }
        psim_model_destroy(m);
    }
    std::printf("done\n");
    return status;
}
