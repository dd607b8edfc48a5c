// Command-line front end of the CPU oracle (oracle/psim_oracle.cpp): runs a psim
// model file and prints one JSON line with the phonon-step count and wall time.
// Used as the timed CPU baseline; it is test infrastructure, not the product.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" {
int oracle_run(const char* json_path, unsigned seed, int threads, int* n_sensors, int* n_recorded, double* stats,
    long long* energy, double* flux, unsigned long long* counters, double* seconds);
const char* oracle_last_error(void);
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: psim_oracle model.json [seed] [threads]\n");
        return 2;
    }
    const unsigned seed = argc > 2 ? static_cast<unsigned>(std::strtoul(argv[2], nullptr, 10)) : 5489U;
    const int threads = argc > 3 ? std::atoi(argv[3]) : 1;
    int ns = 0;
    int nk = 0;
    unsigned long long counters[4] = { 0, 0, 0, 0 };
    double secs = 0.;
    if (oracle_run(argv[1], seed, threads, &ns, &nk, nullptr, nullptr, nullptr, counters, &secs) != 0) {
        std::fprintf(stderr, "oracle error: %s\n", oracle_last_error());
        return 1;
    }
    std::printf("{\"sensors\": %d, \"recorded_steps\": %d, \"phonons\": %llu, \"phonon_steps\": %llu, "
                "\"seconds\": %.6f, \"threads\": %d, \"rate\": %.6e}\n",
        ns, nk, counters[1], counters[2], secs, threads, static_cast<double>(counters[2]) / secs);
    return 0;
}
