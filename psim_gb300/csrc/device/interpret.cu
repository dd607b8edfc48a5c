// Energy-to-temperature inversion and per-sensor statistics on the GPU in FP64
// (SensorInterpreter, psim/src/sensorInterpreter.cpp:19-111), plus the FP64 geometry
// check kernels.  Compiled with -fmad=false: every result is bit-identical to the
// reference's host arithmetic on the same tallies.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../host/geom64.hpp"
#include "common.cuh"
#include "engine.hpp"

namespace psim::gpu {

namespace {

constexpr double kInvEps = .0001;            // EPS (psim/src/sensorInterpreter.cpp:9)
constexpr unsigned kInvMaxIters = 40;        // MAX_ITERS (psim/src/sensorInterpreter.cpp:10)

struct InterpDev {
    std::uint32_t S;
    std::uint64_t K;
    double t_eq, eff, lb, ub;
    const double* area;
    const double* heat;
    const double* init_temp;
    const std::uint32_t* material;
    const std::uint64_t* mtb;
    const double* temps;
    const double* energies;
};

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) { throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e)); }
}

// Material::theoreticalEnergy -> baseData(T).second: the base table sum at the first grid
// temperature not below T (getTempIndex, psim/src/material.cpp:241-246).
__device__ double tabulated_energy(const InterpDev& d, std::uint32_t mat, double T) {
    const std::uint64_t lo = d.mtb[mat];
    const std::uint64_t n = d.mtb[mat + 1] - lo;
    std::uint64_t first = 0;
    std::uint64_t count = n;
    while (count > 0) {
        const std::uint64_t step = count / 2;
        if (d.temps[lo + first + step] < T) {
            first += step + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    if (first > n - 1) { first = n - 1; }
    return d.energies[lo + first];
}

// findTemperature for one tally (psim/src/sensorInterpreter.cpp:80-111).
__device__ double temperature(const InterpDev& d, std::uint32_t s, long long units) {
    const double energy = d.eff * static_cast<double>(units);
    if (d.t_eq != 0.) { return energy / (d.area[s] * d.heat[s]) + d.t_eq; }
    double temp = 0.;
    double ub = d.ub;
    double lb = d.lb;
    unsigned iter = 0;
    while ((ub - lb >= kInvEps) && (++iter != kInvMaxIters)) {
        temp = (ub + lb) / 2.;
        const double de = (tabulated_energy(d, d.material[s], temp) * d.area[s]) - energy;
        if (de < 0.) {
            lb = temp;
        } else {
            ub = temp;
        }
    }
    return temp;
}

__global__ void temps_kernel(InterpDev d, const long long* energy, std::uint64_t start, double* out) {
    const std::uint64_t n = static_cast<std::uint64_t>(d.S) * (d.K - start);
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x) {
        const std::uint32_t s = static_cast<std::uint32_t>(i / (d.K - start));
        const std::uint64_t k = start + i % (d.K - start);
        out[i] = temperature(d, s, energy[s * d.K + k]);
    }
}

// getFinalTemp (psim/src/sensorInterpreter.cpp:68-74): sequential sum over the steps.
__global__ void final_kernel(InterpDev d, const double* temps, std::uint64_t start, double* out) {
    const std::uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) { return; }
    if (d.area[s] == 0.) {
        out[s] = 0.;
        return;
    }
    const std::uint64_t n = d.K - start;
    double sum = 0.;
    for (std::uint64_t k = 0; k < n; ++k) { sum += temps[s * n + k]; }
    out[s] = sum / static_cast<double>(n);
}

// std::reduce / std::transform_reduce order of libstdc++ for random-access ranges, which
// psim's avgAndStdError uses with execution::seq: groups of four, then a sequential tail.
template<typename F> __device__ double grouped_sum(std::uint64_t n, F f) {
    double init = 0.;
    std::uint64_t i = 0;
    while (n - i >= 4) {
        const double v1 = f(i) + f(i + 1);
        const double v2 = f(i + 2) + f(i + 3);
        const double v3 = v1 + v2;
        init = init + v3;
        i += 4;
    }
    for (; i < n; ++i) { init = init + f(i); }
    return init;
}

template<typename F> __device__ void mean_se(std::uint64_t n, F f, double* avg, double* se) {
    const double size = static_cast<double>(n);
    const double a = grouped_sum(n, f) / size;
    const double sd = sqrt(grouped_sum(n, [&](std::uint64_t i) {
                                const double x = f(i);
                                return (a - x) * (a - x);
                            })
                           / size);
    *avg = a;
    *se = sd / sqrt(size);
}

// scaleHeatParams (psim/src/sensorInterpreter.cpp:19-66) for one sensor per thread.
__global__ void scale_kernel(InterpDev d, double* temps, const double* flux, double* fluxes, double* stats) {
    const std::uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.S) { return; }
    const std::uint64_t K = d.K;
    double* t = temps + s * K;
    if (K > 0) { t[0] = d.init_temp[s]; }
    const double f = d.eff / d.area[s];
    const double* fl = flux + s * K * 2;
    double* out = fluxes + s * K * 2;
    for (std::uint64_t k = 0; k < K; ++k) {
        out[2 * k] = fl[2 * k] * f;
        out[2 * k + 1] = fl[2 * k + 1] * f;
    }
    double* st = stats + s * 6;
    mean_se(K, [&](std::uint64_t i) { return t[i]; }, st + 0, st + 1);
    mean_se(K, [&](std::uint64_t i) { return out[2 * i]; }, st + 2, st + 3);
    mean_se(K, [&](std::uint64_t i) { return out[2 * i + 1]; }, st + 4, st + 5);
}

// ---------------------------------------------------------------- device buffers for interpretations
// A buffer that only grows: reused across calls, so an engine's repeated interpretations do not
// allocate (a cudaFree would wait for every stream of the device, runs of other models too).
struct DevBuf {
    void* p{ nullptr };
    std::size_t cap{ 0 };
    DevBuf() = default;
    explicit DevBuf(std::size_t bytes) { reserve(bytes); }
    ~DevBuf() {
        if (p != nullptr) { cudaFree(p); }
    }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    void reserve(std::size_t bytes) {
        bytes = std::max<std::size_t>(bytes, 16);
        if (bytes <= cap) { return; }
        if (p != nullptr) { cudaFree(p); }
        p = nullptr;
        cap = 0;
        check(cudaMalloc(&p, bytes), "cudaMalloc");
        cap = bytes;
    }
    template<typename T> T* as() const { return static_cast<T*>(p); }
};

template<typename T> void upload(DevBuf& b, const std::vector<T>& v, cudaStream_t stream) {
    b.reserve(v.size() * sizeof(T));
    if (!v.empty()) { check(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream), "upload"); }
}

}// namespace

// The interpreter's device buffers of one engine (or of one stand-alone call).
struct InterpCache {
    DevBuf area, heat, init, mat, mtb, temps, energies;// the description's tables
    DevBuf out_temps, out_fluxes, out_stats, out_final;
};

InterpCache* interp_cache_create() { return new InterpCache(); }
void interp_cache_destroy(InterpCache* c) noexcept { delete c; }

namespace {

InterpDev upload_interp(const InterpDesc& d, InterpCache& c, cudaStream_t stream) {
    upload(c.area, d.area, stream);
    upload(c.heat, d.heat_capacity, stream);
    upload(c.init, d.init_temp, stream);
    upload(c.mat, d.material, stream);
    upload(c.mtb, d.mat_temp_begin, stream);
    upload(c.temps, d.temps, stream);
    upload(c.energies, d.energies, stream);
    return InterpDev{ d.n_sensors, d.recorded, d.t_eq, d.eff_energy, d.lb, d.ub, c.area.as<double>(), c.heat.as<double>(),
        c.init.as<double>(), c.mat.as<std::uint32_t>(), c.mtb.as<std::uint64_t>(), c.temps.as<double>(), c.energies.as<double>() };
}

int blocks_for(std::uint64_t n, int block) { return static_cast<int>(std::min<std::uint64_t>((n + block - 1) / block, 65535ULL * 16ULL)); }

}// namespace

// Interpretation with the tallies already on the device (energy [S][K], flux [S][K][2]).
void interpret_device(const InterpDesc& d, const long long* energy, const double* flux, double* temps_h, double* fluxes_h,
                      double* stats_h, cudaStream_t stream, InterpCache* cache) {
    InterpCache local;
    InterpCache& c = cache != nullptr ? *cache : local;
    const InterpDev dev = upload_interp(d, c, stream);
    const std::uint64_t SK = static_cast<std::uint64_t>(d.n_sensors) * d.recorded;
    DevBuf& temps = c.out_temps;
    DevBuf& fluxes = c.out_fluxes;
    DevBuf& stats = c.out_stats;
    temps.reserve(SK * sizeof(double));
    fluxes.reserve(SK * 2 * sizeof(double));
    stats.reserve(static_cast<std::size_t>(d.n_sensors) * 6 * sizeof(double));
    if (SK > 0) { temps_kernel<<<std::max(1, blocks_for(SK, 256)), 256, 0, stream>>>(dev, energy, 0, temps.as<double>()); }
    scale_kernel<<<std::max(1U, (d.n_sensors + 127) / 128), 128, 0, stream>>>(dev, temps.as<double>(), flux,
                                                                               fluxes.as<double>(), stats.as<double>());
    check(cudaGetLastError(), "interpret kernels");
    if (temps_h != nullptr) { check(cudaMemcpyAsync(temps_h, temps.p, SK * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy temps"); }
    if (fluxes_h != nullptr) { check(cudaMemcpyAsync(fluxes_h, fluxes.p, SK * 2 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy fluxes"); }
    if (stats_h != nullptr) { check(cudaMemcpyAsync(stats_h, stats.p, d.n_sensors * 6 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy stats"); }
    check(cudaStreamSynchronize(stream), "interpret sync");
}

void final_temps_device(const InterpDesc& d, const long long* energy, std::uint64_t start, double* out_h, cudaStream_t stream,
                        InterpCache* cache) {
    if (start > d.recorded) { throw std::invalid_argument("start step beyond the recorded steps"); }
    InterpCache local;
    InterpCache& c = cache != nullptr ? *cache : local;
    const InterpDev dev = upload_interp(d, c, stream);
    const std::uint64_t n = static_cast<std::uint64_t>(d.n_sensors) * (d.recorded - start);
    DevBuf& temps = c.out_temps;
    DevBuf& out = c.out_final;
    temps.reserve(n * sizeof(double));
    out.reserve(static_cast<std::size_t>(d.n_sensors) * sizeof(double));
    if (n > 0) { temps_kernel<<<std::max(1, blocks_for(n, 256)), 256, 0, stream>>>(dev, energy, start, temps.as<double>()); }
    final_kernel<<<std::max(1U, (d.n_sensors + 127) / 128), 128, 0, stream>>>(dev, temps.as<double>(), start, out.as<double>());
    check(cudaGetLastError(), "final temps kernels");
    check(cudaMemcpyAsync(out_h, out.p, d.n_sensors * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy final temps");
    check(cudaStreamSynchronize(stream), "final temps sync");
}

void interpret_host(const InterpDesc& d, const std::int64_t* energy, const double* flux, double* temps, double* fluxes,
                    double* stats) {
    const std::uint64_t SK = static_cast<std::uint64_t>(d.n_sensors) * d.recorded;
    DevBuf e(SK * sizeof(long long));
    DevBuf f(SK * 2 * sizeof(double));
    check(cudaMemcpy(e.p, energy, SK * sizeof(long long), cudaMemcpyHostToDevice), "upload energy");
    check(cudaMemcpy(f.p, flux, SK * 2 * sizeof(double), cudaMemcpyHostToDevice), "upload flux");
    interpret_device(d, e.as<long long>(), f.as<double>(), temps, fluxes, stats, nullptr, nullptr);
}

void final_temps_host(const InterpDesc& d, const std::int64_t* energy, std::uint64_t start, double* out) {
    const std::uint64_t SK = static_cast<std::uint64_t>(d.n_sensors) * d.recorded;
    DevBuf e(SK * sizeof(long long));
    check(cudaMemcpy(e.p, energy, SK * sizeof(long long), cudaMemcpyHostToDevice), "upload energy");
    final_temps_device(d, e.as<long long>(), start, out, nullptr, nullptr);
}

// ---------------------------------------------------------------- final temperatures without allocation
// The same two kernels as final_temps_device, with every intermediate buffer carved out of
// one fixed, module-scope device array instead of cudaMalloc.  It serves callers that must
// not allocate device memory during a call: a host that keeps all device memory in its own
// pool, or that runs under a hard device-memory quota.
namespace {

// Holds, each aligned to 256 bytes: sensor areas, heat capacities and materials, the material
// offsets, the temperature grid and tabulated energies, then S x (K - start) temperatures.
// Nothing in it has to start at zero: every byte a call reads, the same call writes first.
static __device__ __align__(256) unsigned char g_final_temps_scratch[kFinalTempsScratchBytes];

constexpr int kMaxScratchDevices = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[kMaxScratchDevices] = {};

// Device address of the scratch on the current device, looked up on the first call per device
// (which may load this module onto that device).
unsigned char* scratch_for_current_device() {
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxScratchDevices) { throw std::invalid_argument("device ordinal beyond the scratch table"); }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_ptr[dev] == nullptr) {
        void* p = nullptr;
        check(cudaGetSymbolAddress(&p, g_final_temps_scratch), "cudaGetSymbolAddress(final temps scratch)");
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_ptr[dev];
}

constexpr std::size_t round256(std::size_t n) { return (n + 255) & ~std::size_t{ 255 }; }

// Validates the view and returns its table sizes; throws std::invalid_argument.
std::uint64_t checked_grid_size(const InterpView& d, std::uint64_t start) {
    if (start > d.recorded) { throw std::invalid_argument("start step beyond the recorded steps"); }
    if (d.n_sensors == 0) { return 0; }
    if (d.area == nullptr || d.heat_capacity == nullptr || d.material == nullptr || d.mat_temp_begin == nullptr) {
        throw std::invalid_argument("missing sensor or material array");
    }
    if (d.n_materials == 0) { throw std::invalid_argument("no materials"); }
    for (std::uint32_t m = 0; m < d.n_materials; ++m) {
        if (d.mat_temp_begin[m + 1] < d.mat_temp_begin[m]) { throw std::invalid_argument("mat_temp_begin decreases"); }
    }
    for (std::uint32_t s = 0; s < d.n_sensors; ++s) {
        const std::uint32_t m = d.material[s];
        if (m >= d.n_materials) { throw std::invalid_argument("sensor material out of range"); }
        if (d.mat_temp_begin[m + 1] <= d.mat_temp_begin[m]) { throw std::invalid_argument("material has an empty temperature grid"); }
    }
    const std::uint64_t nt = d.mat_temp_begin[d.n_materials];
    if (nt > 0 && (d.temps == nullptr || d.energies == nullptr)) { throw std::invalid_argument("missing temperature grid"); }
    return nt;
}

}// namespace

std::size_t final_temps_scratch_bytes(const InterpView& d, std::uint64_t start) {
    const std::uint64_t nt = checked_grid_size(d, start);
    const std::uint64_t S = d.n_sensors;
    const std::uint64_t steps = d.recorded - start;
    const std::uint64_t cap = kFinalTempsScratchBytes;
    // every term is bounded before it is multiplied, so nothing wraps
    if (nt > cap || (S > 0 && steps > cap / (S * sizeof(double)))) { return SIZE_MAX; }
    return 2 * round256(S * sizeof(double)) + round256(S * sizeof(std::uint32_t))
           + round256((static_cast<std::size_t>(d.n_materials) + 1) * sizeof(std::uint64_t)) + 2 * round256(nt * sizeof(double))
           + round256(S * steps * sizeof(double));
}

void final_temps_noalloc(const InterpView& d, const std::int64_t* energy_dev, std::uint64_t start, double* out_dev,
                         void* stream_handle) {
    const std::size_t need = final_temps_scratch_bytes(d, start);
    if (need > kFinalTempsScratchBytes) {
        throw std::length_error("final temperatures need more than the fixed " + std::to_string(kFinalTempsScratchBytes >> 20)
                                + " MiB device scratch (tables plus sensors x steps x 8 bytes)");
    }
    if (d.n_sensors == 0) { return; }
    if (out_dev == nullptr || (d.recorded > start && energy_dev == nullptr)) { throw std::invalid_argument("null device buffer"); }
    auto stream = static_cast<cudaStream_t>(stream_handle);
    unsigned char* base = scratch_for_current_device();
    const std::uint64_t S = d.n_sensors;
    const std::uint64_t nt = d.mat_temp_begin[d.n_materials];
    std::size_t off = 0;
    auto place = [&](const void* src, std::size_t bytes) {
        unsigned char* dst = base + off;
        off += round256(bytes);
        if (bytes > 0) { check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream), "copy interpreter tables"); }
        return dst;
    };
    InterpDev dev{};
    dev.S = d.n_sensors;
    dev.K = d.recorded;
    dev.t_eq = d.t_eq;
    dev.eff = d.eff_energy;
    dev.lb = d.lb;
    dev.ub = d.ub;
    dev.area = reinterpret_cast<const double*>(place(d.area, S * sizeof(double)));
    dev.heat = reinterpret_cast<const double*>(place(d.heat_capacity, S * sizeof(double)));
    dev.init_temp = nullptr;
    dev.material = reinterpret_cast<const std::uint32_t*>(place(d.material, S * sizeof(std::uint32_t)));
    dev.mtb = reinterpret_cast<const std::uint64_t*>(
        place(d.mat_temp_begin, (static_cast<std::size_t>(d.n_materials) + 1) * sizeof(std::uint64_t)));
    dev.temps = reinterpret_cast<const double*>(place(d.temps, nt * sizeof(double)));
    dev.energies = reinterpret_cast<const double*>(place(d.energies, nt * sizeof(double)));
    double* tvals = reinterpret_cast<double*>(base + off);
    const std::uint64_t n = S * (d.recorded - start);
    if (n > 0) {
        temps_kernel<<<std::max(1, blocks_for(n, 256)), 256, 0, stream>>>(dev, reinterpret_cast<const long long*>(energy_dev),
                                                                           start, tvals);
    }
    final_kernel<<<std::max(1U, (d.n_sensors + 127) / 128), 128, 0, stream>>>(dev, tvals, start, out_dev);
    check(cudaGetLastError(), "final temps kernels");
}

// ---------------------------------------------------------------- FP64 geometry check kernels
namespace {

__global__ void intersect_kernel(std::int64_t n, const double* a, const double* b, double* poi, std::int32_t* has) {
    const std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) { return; }
    bool va = false;
    bool vb = false;
    const psim::Seg64 sa = psim::make_seg(psim::P2{ a[4 * i], a[4 * i + 1] }, psim::P2{ a[4 * i + 2], a[4 * i + 3] }, &va);
    const psim::Seg64 sb = psim::make_seg(psim::P2{ b[4 * i], b[4 * i + 1] }, psim::P2{ b[4 * i + 2], b[4 * i + 3] }, &vb);
    if (!va || !vb) {
        has[i] = -1;
        poi[2 * i] = 0.;
        poi[2 * i + 1] = 0.;
        return;
    }
    psim::P2 p{ 0., 0. };
    const bool h = psim::intersection(sa, sb, &p);
    has[i] = h ? 1 : 0;
    poi[2 * i] = h ? p.x : 0.;
    poi[2 * i + 1] = h ? p.y : 0.;
}

__global__ void on_line_kernel(std::int64_t n, const double* l, const double* p, std::int32_t* out) {
    const std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) { return; }
    bool valid = false;
    const psim::Seg64 s = psim::make_seg(psim::P2{ l[4 * i], l[4 * i + 1] }, psim::P2{ l[4 * i + 2], l[4 * i + 3] }, &valid);
    out[i] = valid ? (psim::on_line(s, psim::P2{ p[2 * i], p[2 * i + 1] }) ? 1 : 0) : -1;
}

__global__ void tri_contains_kernel(std::int64_t n, const double* t, const double* p, std::int32_t* out) {
    const std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) { return; }
    const double* v = t + 6 * i;
    out[i] = psim::tri_contains(psim::P2{ v[0], v[1] }, psim::P2{ v[2], v[3] }, psim::P2{ v[4], v[5] },
                                psim::P2{ p[2 * i], p[2 * i + 1] })
                 ? 1
                 : 0;
}

// Cell::handleSurfaceCollision: first edge (p1p2, p2p3, p3p1) whose line contains the point.
__global__ void edge_index_kernel(std::int64_t n, const double* t, const double* p, std::int32_t* out) {
    const std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) { return; }
    const double* v = t + 6 * i;
    const psim::P2 q{ p[2 * i], p[2 * i + 1] };
    int found = -1;
    for (int e = 0; e < 3 && found < 0; ++e) {
        const int f = (e + 1) % 3;
        const psim::Seg64 s = psim::make_seg(psim::P2{ v[2 * e], v[2 * e + 1] }, psim::P2{ v[2 * f], v[2 * f + 1] }, nullptr);
        if (psim::on_line(s, q)) { found = e; }
    }
    out[i] = found;
}

template<typename Launch> void run_geom(std::int64_t n, std::size_t in_a, std::size_t in_b, const double* a, const double* b,
                                        std::size_t out_d, double* od, std::int32_t* oi, Launch launch) {
    if (n <= 0) { return; }
    DevBuf da(in_a * n * sizeof(double));
    DevBuf db(in_b * n * sizeof(double));
    DevBuf dd(std::max<std::size_t>(out_d, 1) * n * sizeof(double));
    DevBuf di(n * sizeof(std::int32_t));
    check(cudaMemcpy(da.p, a, in_a * n * sizeof(double), cudaMemcpyHostToDevice), "geom upload");
    check(cudaMemcpy(db.p, b, in_b * n * sizeof(double), cudaMemcpyHostToDevice), "geom upload");
    launch(static_cast<int>((n + 255) / 256), da.as<double>(), db.as<double>(), dd.as<double>(), di.as<std::int32_t>());
    check(cudaGetLastError(), "geom kernel");
    check(cudaDeviceSynchronize(), "geom sync");
    if (out_d > 0) { check(cudaMemcpy(od, dd.p, out_d * n * sizeof(double), cudaMemcpyDeviceToHost), "geom download"); }
    check(cudaMemcpy(oi, di.p, n * sizeof(std::int32_t), cudaMemcpyDeviceToHost), "geom download");
}

}// namespace

void geom_intersect(std::int64_t n, const double* a, const double* b, double* poi, std::int32_t* has) {
    run_geom(n, 4, 4, a, b, 2, poi, has, [n](int g, const double* x, const double* y, double* od, std::int32_t* oi) {
        intersect_kernel<<<g, 256>>>(n, x, y, od, oi);
    });
}
void geom_on_line(std::int64_t n, const double* lines, const double* pts, std::int32_t* out) {
    run_geom(n, 4, 2, lines, pts, 0, nullptr, out, [n](int g, const double* x, const double* y, double*, std::int32_t* oi) {
        on_line_kernel<<<g, 256>>>(n, x, y, oi);
    });
}
void geom_tri_contains(std::int64_t n, const double* tris, const double* pts, std::int32_t* out) {
    run_geom(n, 6, 2, tris, pts, 0, nullptr, out, [n](int g, const double* x, const double* y, double*, std::int32_t* oi) {
        tri_contains_kernel<<<g, 256>>>(n, x, y, oi);
    });
}
void geom_edge_index(std::int64_t n, const double* tris, const double* pts, std::int32_t* out) {
    run_geom(n, 6, 2, tris, pts, 0, nullptr, out, [n](int g, const double* x, const double* y, double*, std::int32_t* oi) {
        edge_index_kernel<<<g, 256>>>(n, x, y, oi);
    });
}

}// namespace psim::gpu
