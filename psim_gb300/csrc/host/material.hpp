// Material dispersion, density-of-states and per-temperature cumulative tables (FP64, host).
//
// Built once per run on the host and uploaded to the GPU.  The arithmetic follows
// psim/src/material.cpp (constructor :20-51, phononDist :184-204, buildCumulDist
// :170-179, cumulDistEmit/Scatter :140-168, initializeTables :101-123, rates
// :207-239, getTempIndex :241-246) operation for operation, so the tables are
// bit-identical to the reference's when built with the same libm.
#pragma once

#include <array>
#include <cstddef>
#include <string>
#include <vector>

namespace psim {

constexpr std::size_t kBins = 1000;
constexpr double kHbar = 1.054517e-34;
constexpr double kBoltz = 1.38065e-23;
constexpr float kTempInterval = .1F;// temperature grid step of the tables (psim/src/model.cpp:25)
// Most grid temperatures one material's tables may hold: a 5000 K span at kTempInterval, about
// 2.4 GB of host tables (three cumulative tables of 1000 (probability, LA fraction) pairs each).
constexpr std::size_t kMaxTableTemps = 50001;

enum Polar : int { kLA = 0, kTA = 1 };

// One cumulative table: cumulative probability and LA fraction per bin, and the sum of
// the unnormalised distribution (energy / heat capacity, emitted energy or scatter weight).
struct CumTable {
    std::array<double, kBins> cum{};
    std::array<double, kBins> la_frac{};
    double sum{ 0. };
};

struct MaterialSpec {
    std::string name;
    std::array<double, 3> la{}, ta{};// w = c0 k^2 + c1 k + c2
    double w_max_la{ 0. }, w_max_ta{ 0. };
    double b_l{ 0. }, b_tn{ 0. }, b_tu{ 0. }, b_i{ 0. }, w{ 0. };
};

class MaterialTables {
public:
    MaterialTables() = default;
    MaterialTables(const MaterialSpec& spec, bool full_simulation);

    const MaterialSpec& spec() const noexcept { return spec_; }
    bool full() const noexcept { return full_; }
    double width() const noexcept { return width_; }
    const std::array<double, kBins>& freq() const noexcept { return freq_; }
    const std::array<double, kBins>& vel(int pol) const noexcept { return pol == kLA ? vel_la_ : vel_ta_; }
    const std::array<double, kBins>& dens(int pol) const noexcept { return pol == kLA ? dens_la_ : dens_ta_; }

    // Relaxation rates [N, U, I] at temperature T for frequency f.
    std::array<double, 3> rates(double T, double f, int pol) const;

    // Temperature grid [lo, hi] in kTempInterval steps plus hi, and the three tables per grid point.
    void build_tables(double lo, double hi);
    const std::vector<double>& temps() const noexcept { return temps_; }
    std::size_t temp_index(double T) const noexcept;
    const CumTable& base(std::size_t i) const { return base_[i]; }
    const CumTable& emit(std::size_t i) const { return emit_[i]; }
    const CumTable& scatter(std::size_t i) const { return scatter_[i]; }

private:
    MaterialSpec spec_;
    bool full_{ false };
    double width_{ 0. };
    std::array<double, kBins> freq_{}, vel_la_{}, vel_ta_{}, dens_la_{}, dens_ta_{};
    std::vector<double> temps_;
    std::vector<CumTable> base_, emit_, scatter_;

    std::array<double, kBins> distribution(double T, int pol) const;
};

}// namespace psim
