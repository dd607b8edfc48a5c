// Forced-include shim for building the reference psim sources as a test oracle.
//
// The reference draws every random number from Utils::urand(), a thread_local
// std::mt19937 seeded from std::random_device (psim/include/psim/utils.h:16-21),
// and shuffles phonons with a std::random_device (psim/src/modelSimulator.cpp:239).
// This header is passed with `-include` so it is read before any reference
// header.  It includes the reference utils.h with its urand renamed out of the
// way, then supplies a urand() seeded from the PSIM_SEED environment variable
// and redirects the shuffle's std::random_device to a seeded engine.  No
// reference file is modified.
#pragma once
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <random>

#define urand psim_reference_unseeded_urand
#include <psim/utils.h>
#undef urand

namespace psim_oracle_seed {
inline std::uint32_t seed() noexcept {
    const char* s = std::getenv("PSIM_SEED");
    return s != nullptr ? static_cast<std::uint32_t>(std::strtoull(s, nullptr, 10)) : 5489U;
}
inline std::mt19937& shuffle_engine() noexcept {
    static std::mt19937 engine(seed() ^ 0x9E3779B9U);
    return engine;
}
}// namespace psim_oracle_seed

namespace Utils {
inline double urand() noexcept {
    thread_local std::mt19937 generator(psim_oracle_seed::seed());
    std::uniform_real_distribution dist(0., std::nextafter(1., 2.));
    return dist(generator);
}
}// namespace Utils

// Uniform random bit generator with std::random_device's interface and range,
// drawing from the seeded shuffle engine.
struct psim_oracle_seeded_device {
    using result_type = unsigned int;
    static constexpr result_type min() { return 0U; }
    static constexpr result_type max() { return UINT_MAX; }
    result_type operator()() { return static_cast<result_type>(psim_oracle_seed::shuffle_engine()()); }
};
namespace std {
using psim_oracle_seeded_device_alias = ::psim_oracle_seeded_device;
}
#define random_device psim_oracle_seeded_device_alias
