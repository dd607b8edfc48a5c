#include "material.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "geom64.hpp"

namespace psim {
namespace {

// Wave number of a quadratic dispersion branch: the smaller root of c0 k^2 + c1 k + c2 = f
// (Material::getK, psim/src/material.cpp:86-92).
double wave_number(double f, const std::array<double, 3>& c) {
    const double d = std::pow(c[1], 2) - 4. * c[0] * (c[2] - f);
    const double a = (-c[1] - std::sqrt(d)) / (2. * c[0]);
    const double b = (-c[1] + std::sqrt(d)) / (2. * c[0]);
    return (a < b) ? a : b;
}

// Group velocity dw/dk at that root (Material::getGv, material.cpp:93-95).
double group_velocity(double f, const std::array<double, 3>& c) { return 2. * c[0] * wave_number(f, c) + c[1]; }

double left_sum(const std::array<double, kBins>& a) {
    double s = 0.;
    for (double v : a) { s += v; }
    return s;
}

CumTable cumulate(const std::array<double, kBins>& t1, const std::array<double, kBins>& t2) {
    CumTable t;
    const double total = left_sum(t1) + left_sum(t2);
    t.cum[0] = (t1[0] + t2[0]) / total;
    t.la_frac[0] = t1[0] / (t1[0] + t2[0]);
    for (std::size_t i = 1; i < kBins; ++i) {
        t.cum[i] = t.cum[i - 1] + (t1[i] + t2[i]) / total;
        t.la_frac[i] = t1[i] / (t1[i] + t2[i]);
    }
    t.sum = total;
    return t;
}

}// namespace

MaterialTables::MaterialTables(const MaterialSpec& spec, bool full_simulation)
    : spec_{ spec }
    , full_{ full_simulation }
    , width_{ std::max(spec.w_max_la, spec.w_max_ta) / kBins } {
    for (std::size_t i = 0; i < kBins; ++i) {
        freq_[i] = static_cast<double>(static_cast<int>(2 * i + 1)) * width_ / 2.;
    }
    for (std::size_t i = 0; i < kBins; ++i) {
        const double f = freq_[i];
        const double la_gv = group_velocity(f, spec_.la);
        vel_la_[i] = la_gv;
        dens_la_[i] = std::pow(wave_number(f, spec_.la), 2) / 2. / std::pow(kPi, 2) / la_gv;
        const double ta_gv = group_velocity(f, spec_.ta);
        if (!std::isnan(ta_gv)) {// TA states end at the TA branch maximum; beyond it the arrays stay 0
            vel_ta_[i] = ta_gv;
            dens_ta_[i] = std::pow(wave_number(f, spec_.ta), 2) / std::pow(kPi, 2) / ta_gv;// doubly degenerate
        }
    }
}

std::array<double, 3> MaterialTables::rates(double T, double f, int pol) const {
    double n = 0.;
    double u = 0.;
    if (pol == kLA) {
        n = spec_.b_l * f * f * std::pow(T, 3);
        u = spec_.b_l * f * f * std::pow(T, 3);
    } else {
        n = (f < spec_.w) ? spec_.b_tn * f * std::pow(T, 4) : 0.;
        u = (f >= spec_.w) ? spec_.b_tu * f * f / std::sinh(kHbar * f / (T * kBoltz)) : 0.;
    }
    return { n, u, spec_.b_i * std::pow(f, 4) };
}

// Energy (full simulation) or heat capacity (deviational, Bose-Einstein derivative) per bin.
std::array<double, kBins> MaterialTables::distribution(double T, int pol) const {
    std::array<double, kBins> out{};
    const auto& dens = (pol == kLA) ? dens_la_ : dens_ta_;
    const double k = kHbar / (kBoltz * T);
    for (std::size_t i = 0; i < kBins; ++i) {
        const double f = freq_[i];
        double d = f * kHbar / std::expm1(k * f) * width_ * dens[i];
        if (!full_) { d *= k * f * std::exp(k * f) / (std::expm1(k * f) * T); }
        out[i] = d;
    }
    return out;
}

void MaterialTables::build_tables(double lo, double hi) {
    const double span = (hi - lo) / static_cast<double>(kTempInterval);
    if (!(span >= 0.) || !std::isfinite(span)) { throw std::invalid_argument("invalid temperature bounds for the material tables"); }
    if (span >= static_cast<double>(kMaxTableTemps - 1)) {
        throw std::length_error("the model's temperatures span more than "
                                + std::to_string(static_cast<int>((kMaxTableTemps - 1) * static_cast<double>(kTempInterval)))
                                + " K: its material tables (one per 0.1 K) would not fit in host memory");
    }
    const auto n = static_cast<std::size_t>(span);
    temps_.assign(n, 0.);
    double step = -1.;
    for (auto& t : temps_) { t = lo + static_cast<double>(kTempInterval) * (step += 1); }
    temps_.push_back(hi);
    base_.clear();
    emit_.clear();
    scatter_.clear();
    base_.reserve(temps_.size());
    emit_.reserve(temps_.size());
    scatter_.reserve(temps_.size());
    for (const double T : temps_) {
        const auto la = distribution(T, kLA);
        const auto ta = distribution(T, kTA);
        base_.push_back(cumulate(la, ta));
        std::array<double, kBins> la_e{};
        std::array<double, kBins> ta_e{};
        std::array<double, kBins> la_s{};
        std::array<double, kBins> ta_s{};
        for (std::size_t i = 0; i < kBins; ++i) {
            la_e[i] = la[i] * vel_la_[i];
            ta_e[i] = ta[i] * vel_ta_[i];
            const auto rl = rates(T, freq_[i], kLA);
            la_s[i] = la[i] * (((0. + rl[0]) + rl[1]) + rl[2]);
            const auto rt = rates(T, freq_[i], kTA);
            ta_s[i] = ta[i] * (((0. + rt[0]) + rt[1]) + rt[2]);
        }
        emit_.push_back(cumulate(la_e, ta_e));
        scatter_.push_back(cumulate(la_s, ta_s));
    }
}

std::size_t MaterialTables::temp_index(double T) const noexcept {
    const auto idx = static_cast<std::size_t>(std::lower_bound(temps_.begin(), temps_.end(), T) - temps_.begin());
    return std::min(idx, temps_.size() - 1);
}

}// namespace psim
