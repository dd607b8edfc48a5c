// Steady-state detection on the recorded tallies.  psim has no detector (the user fixes the
// simulated time); its README proposes stopping "when the flux across each cell is constant
// within some margin of error for a certain amount of time" (README.md, Steady-State Detection).
// This is that criterion, made statistical:
//   - each sensor's per-step energy count and flux components are cut into windows of W steps,
//     each window into B batches of W/B steps;
//   - a window's mean is the mean of its batch means, and its standard error the spread of the
//     batch means over sqrt(B) (batch means: a phonon stays in a sensor's cells for several
//     steps, so per-step tallies are correlated and their own spread would understate the
//     error);
//   - window c "agrees" with window j when, for every quantity, the means differ by at most
//     z combined standard errors: |m_c - m_j| <= z sqrt(se_c^2 + se_j^2);
//   - a sensor is steady from window j when each of the M windows after it agrees with window j
//     itself (the anchor: a drift too slow to show between neighbouring windows still has to stay
//     within the tolerance over all M of them); a window that disagrees becomes the next anchor;
//     the onset is step j*W;
//   - with a trend tolerance zd > 0, the M + 1 windows from the anchor must also show no linear
//     trend: the least-squares slope of each quantity's window means over the window index
//     (weighted equally, its variance from the windows' standard errors) must lie within zd of its
//     standard error; a trend makes the latest window the next anchor, like a disagreement.  A
//     relaxation slow enough to stay within z standard errors of the anchor for M windows still
//     shows as a consistent slope;
//   - the model is steady at the largest onset over its sensors, and not steady while any
//     sensor has none.
// The statistics are computed in FP64 from the exact integer tallies (flux in fixed point), in a
// fixed order, with sums taken about the previous window's mean (no cancellation when the
// spread is small next to the mean).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.hpp"

namespace psim::gpu {

namespace {

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) { throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e)); }
}

struct WindowStats {
    double mean[3];
    double se[3];
};

// One warp per sensor: lanes split each batch's steps, then reduce.
__global__ void steady_kernel(const TallySlot* tally, std::uint32_t S, std::uint64_t k_used, std::uint32_t W, std::uint32_t B,
                              double z, std::uint32_t M, double zd, long long* onset) {
    const std::uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31U;
    if (warp >= S) { return; }
    const std::uint32_t s = warp;
    const std::uint32_t L = W / B;// steps per batch
    const std::uint64_t nw = k_used / W;
    WindowStats prev{};
    WindowStats anchor{};
    std::uint64_t anchor_w = 0;
    std::uint32_t streak = 0;
    // sums over the windows from the anchor (index i = 0, 1, ...) for the trend test: sum i,
    // sum i^2, and per quantity sum d, sum i d (d: window mean minus the anchor's) and sum se^2,
    // sum i se^2, sum i^2 se^2
    double n_w = 0., s_i = 0., s_ii = 0.;
    double s_d[3] = { 0., 0., 0. }, s_id[3] = { 0., 0., 0. };
    double v0[3] = { 0., 0., 0. }, v1[3] = { 0., 0., 0. }, v2[3] = { 0., 0., 0. };
    long long result = -1;
    for (std::uint64_t w = 0; w < nw && result < 0; ++w) {
        double bsum[3] = { 0., 0., 0. };// batch means about 'shift'
        double bsq[3] = { 0., 0., 0. };
        const double shift[3] = { prev.mean[0], prev.mean[1], prev.mean[2] };
        for (std::uint32_t b = 0; b < B; ++b) {
            double sum[3] = { 0., 0., 0. };
            const std::uint64_t k0 = w * W + static_cast<std::uint64_t>(b) * L;
            for (std::uint64_t k = k0 + lane; k < k0 + L; k += 32) {
                const TallySlot t = tally[k * S + s];
                sum[0] += static_cast<double>(t.count) - shift[0];
                sum[1] += static_cast<double>(t.fx) - shift[1];
                sum[2] += static_cast<double>(t.fy) - shift[2];
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) { sum[q] += __shfl_xor_sync(0xFFFFFFFFU, sum[q], o); }
                const double bm = sum[q] / static_cast<double>(L);
                bsum[q] += bm;
                bsq[q] += bm * bm;
            }
        }
        WindowStats cur{};
        const double n = static_cast<double>(B);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double d = bsum[q] / n;// window mean minus shift
            const double var = fmax(0., (bsq[q] - n * d * d) / (n - 1.));
            cur.mean[q] = shift[q] + d;
            cur.se[q] = sqrt(var / n);
        }
        bool agree = w > 0;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double tol = z * sqrt(cur.se[q] * cur.se[q] + anchor.se[q] * anchor.se[q]);
            agree = agree && fabs(cur.mean[q] - anchor.mean[q]) <= tol;
        }
        bool reset = !agree;
        if (agree) {
            ++streak;
            const double i = static_cast<double>(streak);
            n_w += 1.;
            s_i += i;
            s_ii += i * i;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const double d = cur.mean[q] - anchor.mean[q];
                const double v = cur.se[q] * cur.se[q];
                s_d[q] += d;
                s_id[q] += i * d;
                v0[q] += v;
                v1[q] += i * v;
                v2[q] += i * i * v;
            }
            if (streak >= M) {
                bool flat = true;
                if (zd > 0.) {
                    const double ib = s_i / n_w;
                    const double sxx = s_ii - n_w * ib * ib;
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const double slope = (s_id[q] - ib * s_d[q]) / sxx;
                        const double var = fmax(0., v2[q] - 2. * ib * v1[q] + ib * ib * v0[q]) / (sxx * sxx);
                        flat = flat && fabs(slope) <= zd * sqrt(var);
                    }
                }
                if (flat) {
                    result = static_cast<long long>(anchor_w * W);
                } else {
                    reset = true;
                }
            }
        }
        if (reset) {
            anchor = cur;
            anchor_w = w;
            streak = 0;
            n_w = 1.;
            s_i = 0.;
            s_ii = 0.;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                s_d[q] = 0.;
                s_id[q] = 0.;
                v0[q] = cur.se[q] * cur.se[q];
                v1[q] = 0.;
                v2[q] = 0.;
            }
        }
        prev = cur;
    }
    if (lane == 0) { onset[s] = result; }
}

// Largest onset over the sensors, or -1 when some sensor has none.
long long model_onset(const std::vector<long long>& per_sensor) {
    long long m = -1;
    for (long long v : per_sensor) {
        if (v < 0) { return -1; }
        m = std::max(m, v);
    }
    return m;
}

struct DevMem {
    void* p{ nullptr };
    explicit DevMem(std::size_t bytes) { check(cudaMalloc(&p, bytes > 0 ? bytes : 16), "cudaMalloc"); }
    ~DevMem() { cudaFree(p); }
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
};

}// namespace

void validate_steady(const SteadyCriterion& c) {
    if (c.batches < 2) { throw std::invalid_argument("steady-state windows need at least 2 batches"); }
    if (c.window < c.batches || c.window % c.batches != 0) {
        throw std::invalid_argument("steady-state window must be a positive multiple of its batch count");
    }
    if (!(c.z > 0.)) { throw std::invalid_argument("steady-state tolerance must be positive"); }
    if (c.patience < 1) { throw std::invalid_argument("steady-state patience must be at least 1 window"); }
    if (!(c.drift_z >= 0.) || !std::isfinite(c.drift_z)) { throw std::invalid_argument("steady-state trend tolerance must be finite and not negative"); }
}

long long steady_onset_device(const void* tally, std::uint32_t S, std::uint64_t k_used, const SteadyCriterion& c,
                              long long* per_sensor, void* stream_handle) {
    validate_steady(c);
    auto stream = static_cast<cudaStream_t>(stream_handle);
    std::vector<long long> onset(S, -1);
    if (S > 0) {
        DevMem d_onset(S * sizeof(long long));
        const unsigned threads = 256;
        const unsigned blocks = static_cast<unsigned>((static_cast<std::uint64_t>(S) * 32 + threads - 1) / threads);
        steady_kernel<<<blocks, threads, 0, stream>>>(static_cast<const TallySlot*>(tally), S, k_used, c.window, c.batches,
                                                      c.z, c.patience, c.drift_z, static_cast<long long*>(d_onset.p));
        check(cudaGetLastError(), "steady-state kernel");
        check(cudaMemcpyAsync(onset.data(), d_onset.p, S * sizeof(long long), cudaMemcpyDeviceToHost, stream), "copy onsets");
        check(cudaStreamSynchronize(stream), "steady-state sync");
    }
    if (per_sensor != nullptr) { std::copy(onset.begin(), onset.end(), per_sensor); }
    return model_onset(onset);
}

long long steady_onset_host(const std::int64_t* energy, const double* flux, std::uint32_t S, std::uint64_t K,
                            const SteadyCriterion& c, long long* per_sensor) {
    validate_steady(c);
    // [S][K] host arrays -> the tallies' [K][S] layout with flux in fixed point
    std::vector<TallySlot> t(static_cast<std::size_t>(S) * K);
    for (std::uint32_t s = 0; s < S; ++s) {
        for (std::uint64_t k = 0; k < K; ++k) {
            TallySlot& v = t[k * S + s];
            v.count = energy[s * K + k];
            v.fx = std::llrint(flux[(s * K + k) * 2] * static_cast<double>(kFluxScale));
            v.fy = std::llrint(flux[(s * K + k) * 2 + 1] * static_cast<double>(kFluxScale));
        }
    }
    DevMem d(t.size() * sizeof(TallySlot));
    if (!t.empty()) { check(cudaMemcpy(d.p, t.data(), t.size() * sizeof(TallySlot), cudaMemcpyHostToDevice), "upload tallies"); }
    return steady_onset_device(d.p, S, K, c, per_sensor, nullptr);
}

}// namespace psim::gpu
