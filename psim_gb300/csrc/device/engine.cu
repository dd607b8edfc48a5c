// GPU engine: device model construction, phonon births, the per-step launch sequence
// (captured as one CUDA graph per run) and tally read-out.
#include "engine.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../host/geom64.hpp"
#include "cells.hpp"
#include "common.cuh"
#include "transport.cuh"

namespace psim::gpu {

void launch_step_f32(const StepParams& P, int grid, int block, std::size_t smem, cudaStream_t stream);
void launch_batch_f32(const BatchLaunch& B, int grid, std::size_t smem, cudaStream_t stream);
void launch_gather_counts(const std::uint32_t* const* ptrs, std::uint32_t n, std::uint32_t* out, cudaStream_t stream);
int occupancy_batch_f32(std::size_t smem);
std::size_t batch_static_smem();
void launch_population_max(const std::uint32_t* population, std::uint32_t n, unsigned long long* counters, cudaStream_t stream);
void launch_step_f64(const StepParams& P, int grid, std::size_t smem, cudaStream_t stream);
void launch_rates32(const MaterialDev& m, const SensorDev* s, const float* w, const int* pol, int n, double* out, cudaStream_t stream);
void launch_rates64(const MaterialDev& m, const double* T, const double* f, const int* pol, int n, double* out, cudaStream_t stream);
int occupancy_f32(unsigned stage_mask, int block, std::size_t smem);
int occupancy_f64(std::size_t smem);
void interpret_device(const InterpDesc& d, const long long* energy, const double* flux, double* temps_h, double* fluxes_h,
                      double* stats_h, cudaStream_t stream, InterpCache* cache);
void final_temps_device(const InterpDesc& d, const long long* energy, std::uint64_t start, double* out_h, cudaStream_t stream,
                        InterpCache* cache);

namespace {

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) { throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e)); }
}

struct Buf {
    void* p{ nullptr };
    std::size_t bytes{ 0 };
    Buf() = default;
    ~Buf() { release(); }
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    void alloc(std::size_t n) {
        release();
        bytes = n > 0 ? n : 16;
        check(cudaMalloc(&p, bytes), "cudaMalloc");
    }
    void release() {
        if (p != nullptr) { cudaFree(p); }
        p = nullptr;
        bytes = 0;
    }
    template<typename T> void upload(const std::vector<T>& v) {
        alloc(v.size() * sizeof(T));
        if (!v.empty()) { check(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload"); }
    }
    template<typename T> T* as() const { return static_cast<T*>(p); }
    // Takes over o's allocation (releasing its own).
    void take(Buf& o) {
        release();
        p = o.p;
        bytes = o.bytes;
        o.p = nullptr;
        o.bytes = 0;
    }
};

// Phonon state of a run whose phonons all fit in this many bytes (two buffers) is sized for
// every phonon of the run, and the run is one CUDA graph; larger runs are sized near their peak
// population and grow between chunks of launches (Engine::run).
constexpr std::uint64_t kWholeRunStateBytes = std::uint64_t{ 512 } << 20;
// Transport launches per chunk of a chunked run.
constexpr std::uint64_t kLaunchesPerChunk = 16;
// A warp of the FP32 kernel takes new work items once this many of its lanes are free: the start of
// new phonons (a global work counter, state loads) then runs on several lanes at once.  Kinked
// benchmark model, 2000 steps: 1 lane 1.818e10, 2: 1.852e10, 4: 1.886e10, 8: 1.860e10, 16: 1.739e10
// phonon-steps/s (identical tallies).
constexpr std::uint32_t kFetchLanes = 4;
// Work items a warp of the FP32 kernel takes from the work counter at a time (0: as many as it has
// free lanes).  A pool of 32 with L2 prefetch of its state records: kinked benchmark model 1.904e10
// against 1.896e10 without; the 10-cell bar of 2e5 phonons per step 7.69e9 against 8.75e9.
constexpr std::uint32_t kWarpPool = 0;
// 1: the FP32 kernel's loop tail overlaps the output counter's atomic with the tallies.  Kinked
// benchmark model, 2000 steps: 1.896e10 against 1.861e10 phonon-steps/s; the 10-cell bar 8.75e9
// against 8.55e9 (identical tallies).
constexpr std::uint32_t kTailOrder = 1;

Line64 line64(psim::P2 a, psim::P2 b) {
    const psim::Seg64 s = psim::make_seg(a, b, nullptr);
    return Line64{ s.a.x, s.a.y, s.b.x, s.b.y, s.m, s.c, s.lo.x, s.lo.y, s.hi.x, s.hi.y };
}

psim::Seg64 seg_from(const double* l) { return psim::make_seg(psim::P2{ l[0], l[1] }, psim::P2{ l[2], l[3] }, nullptr); }

// Walker alias table (Vose's construction) over the (bin, polarization) outcomes that
// Material::freqIndex (psim/src/material.cpp:64-75) produces from a cumulative table: the
// bisection returns bin h with probability cum[h] - cum[h-1] (bin 1 also takes bin 0's mass,
// bin 999 everything above cum[998]) and LA with probability la_frac[h] (TA when it is NaN).
std::vector<std::uint32_t> alias_table(const double* tab) {
    std::vector<double> p(kAliasCols, 0.);
    for (int h = 1; h < kBins; ++h) {
        const double cum_h = tab[2 * h];
        const double prev = (h == 1) ? 0. : tab[2 * (h - 1)];
        double ph = (h == kBins - 1) ? 1. - prev : cum_h - prev;
        if (!(ph > 0.)) { ph = 0.; }
        double la = tab[2 * h + 1];
        if (std::isnan(la)) { la = 0.; }
        la = std::min(std::max(la, 0.), 1.);
        p[2 * h] = ph * la;
        p[2 * h + 1] = ph * (1. - la);
    }
    double total = 0.;
    for (double v : p) { total += v; }
    if (!(total > 0.)) { throw std::invalid_argument("frequency table has no probability mass"); }
    std::vector<double> q(kAliasCols);
    std::vector<int> small;
    std::vector<int> large;
    for (int i = 0; i < kAliasCols; ++i) {
        q[i] = p[i] / total * kAliasCols;
        (q[i] < 1. ? small : large).push_back(i);
    }
    std::vector<std::uint32_t> out(kAliasCols);
    constexpr double kOne = 2097152.;// 2^21
    while (!small.empty() && !large.empty()) {
        const int l = small.back();
        small.pop_back();
        const int g = large.back();
        large.pop_back();
        const auto thr = static_cast<std::uint32_t>(std::min(std::floor(q[l] * kOne + 0.5), kOne - 1.));
        out[l] = (thr << 11) | static_cast<std::uint32_t>(g);
        q[g] = (q[g] + q[l]) - 1.;
        (q[g] < 1. ? small : large).push_back(g);
    }
    // Rounding leftovers: columns of real outcomes keep themselves; a column without
    // probability (padding, or an impossible outcome) always takes the most probable outcome.
    const int best = static_cast<int>(std::max_element(p.begin(), p.end()) - p.begin());
    for (int i : large) { out[i] = (0x1FFFFFU << 11) | static_cast<std::uint32_t>(i); }
    for (int i : small) {
        out[i] = p[i] > 0. ? ((0x1FFFFFU << 11) | static_cast<std::uint32_t>(i)) : static_cast<std::uint32_t>(best);
    }
    for (int i = 2 * kBins; i < kAliasCols; ++i) {// padding columns must never be accepted
        if ((out[i] >> 11) != 0U || (out[i] & 0x7FFU) >= static_cast<std::uint32_t>(2 * kBins)) { out[i] = static_cast<std::uint32_t>(best); }
    }
    return out;
}

__global__ void unpack_kernel(const TallySlot* t, std::uint32_t S, std::uint64_t K, long long* energy, double* flux) {
    const std::uint64_t n = static_cast<std::uint64_t>(S) * K;
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x) {
        const std::uint64_t k = i / S;
        const std::uint32_t s = static_cast<std::uint32_t>(i % S);
        const TallySlot v = t[i];
        energy[s * K + k] = v.count;
        flux[(s * K + k) * 2] = static_cast<double>(v.fx) * kFluxScaleInv;
        flux[(s * K + k) * 2 + 1] = static_cast<double>(v.fy) * kFluxScaleInv;
    }
}

}// namespace

std::vector<std::uint32_t> alias_table_of(const double* tab) { return alias_table(tab); }

MaterialDev material_dev(const double* pr) {
    MaterialDev md{};
    md.b_l = pr[0];
    md.b_tn = pr[1];
    md.b_tu = pr[2];
    md.b_i = pr[3];
    md.w = pr[4];
    md.width64 = pr[5];
    md.w_max_la64 = pr[6];
    md.w_max_ta64 = pr[7];
    md.cL = static_cast<float>(pr[0] * 1e26);
    md.cTN = static_cast<float>(pr[1] * 1e13);
    md.cTU = static_cast<float>(pr[2] * 1e26);
    md.cI = static_cast<float>(pr[3] * 1e52);
    md.w_cut = static_cast<float>(pr[4] / 1e13);
    md.width = static_cast<float>(pr[5] / 1e13);
    md.w_max_la = static_cast<float>(pr[6] / 1e13);
    md.w_max_ta = static_cast<float>(pr[7] / 1e13);
    return md;
}

void sensor_rate_factors(double T, SensorDev& sd) {
    constexpr double kHbar = 1.054517e-34;// psim/src/material.cpp:13-14
    constexpr double kBoltz = 1.38065e-23;
    sd.T = T;
    sd.T3 = static_cast<float>(T * T * T);
    sd.T4 = static_cast<float>(T * T * T * T);
    sd.xk = static_cast<float>(kHbar * 1e13 / (kBoltz * T));
}

void rates_probe(const double* mat_params, std::int64_t n, const double* T, const double* f, const std::int32_t* pol,
                 int precision, double* out) {
    if (n <= 0) { return; }
    if (n > (std::int64_t{ 1 } << 24)) { throw std::invalid_argument("at most 2^24 rate cases per call"); }
    const MaterialDev m = material_dev(mat_params);
    const auto cnt = static_cast<std::size_t>(n);
    Buf pol_d;
    Buf out_d;
    pol_d.upload(std::vector<std::int32_t>(pol, pol + cnt));
    out_d.alloc(cnt * 3 * sizeof(double));
    if (precision == 0) {// the FP32 kernel's inputs: per-sensor factors of T, frequency in 1e13 rad/s
        std::vector<SensorDev> s(cnt);
        std::vector<float> w(cnt);
        for (std::size_t i = 0; i < cnt; ++i) {
            sensor_rate_factors(T[i], s[i]);
            w[i] = static_cast<float>(f[i] / 1e13);
        }
        Buf s_d;
        Buf w_d;
        s_d.upload(s);
        w_d.upload(w);
        launch_rates32(m, s_d.as<SensorDev>(), w_d.as<float>(), pol_d.as<int>(), static_cast<int>(n), out_d.as<double>(), nullptr);
    } else {
        Buf t_d;
        Buf f_d;
        t_d.upload(std::vector<double>(T, T + cnt));
        f_d.upload(std::vector<double>(f, f + cnt));
        launch_rates64(m, t_d.as<double>(), f_d.as<double>(), pol_d.as<int>(), static_cast<int>(n), out_d.as<double>(), nullptr);
    }
    check(cudaGetLastError(), "rates kernel");
    check(cudaMemcpy(out, out_d.p, cnt * 3 * sizeof(double), cudaMemcpyDeviceToHost), "rates copy");
}

// Device cell records from the flattened description: the FP32 cell-local form (outward
// normals, offsets, edge links, neighbour entry edges) and the FP64 reference form.
void build_cells(const SimDesc& d, std::vector<CellF32>& c32, std::vector<CellF64>& c64, std::vector<Sub64>& subs) {
    const std::uint32_t C = d.n_cells;
    c32.assign(C, CellF32{});
    c64.assign(C, CellF64{});
    subs.assign(d.sub_kind.size(), Sub64{});
    auto vtx = [&](std::uint32_t c, int i) {
        return psim::P2{ d.cell_vertices[6 * c + 2 * i], d.cell_vertices[6 * c + 2 * i + 1] };
    };
    std::vector<int> cell_sign(C);
    for (std::uint32_t c = 0; c < C; ++c) {
        cell_sign[c] = psim::tri_clockwise(vtx(c, 0), vtx(c, 1), vtx(c, 2)) ? 1 : -1;
    }
    for (std::uint32_t c = 0; c < C; ++c) {
        CellF32& f = c32[c];
        CellF64& g = c64[c];
        std::memset(&f, 0, sizeof f);
        std::memset(&g, 0, sizeof g);
        const psim::P2 o = vtx(c, 0);
        const std::uint32_t sensor = d.cell_sensor[c];
        if (sensor >= d.n_sensors) { throw std::invalid_argument("cell sensor index out of range"); }
        f.sensor = g.sensor = sensor;
        f.material = g.material = d.sensor_material[sensor];
        const double spec = std::min(std::max(d.cell_spec[c], 0.), 1.);
        f.spec = static_cast<float>(spec);
        g.spec = spec;
        f.rev = 0;
        for (int e = 0; e < 3; ++e) {
            const psim::P2 a = vtx(c, e);
            const psim::P2 b = vtx(c, (e + 1) % 3);
            const float2 local = make_float2(static_cast<float>(a.x - o.x), static_cast<float>(a.y - o.y));
            if (e == 1) { f.v1 = local; }
            if (e == 2) { f.v2 = local; }
            g.vx[e] = a.x;
            g.vy[e] = a.y;
            g.edge[e] = line64(a, b);
            const psim::P2 n_in = psim::seg_normal(a, b, cell_sign[c]);
            g.nx[e] = n_in.x;
            g.ny[e] = n_in.y;
            const double h = -(n_in.x * (a.x - o.x) + n_in.y * (a.y - o.y));
            f.edge[e] = make_float4(static_cast<float>(-n_in.x), static_cast<float>(-n_in.y), static_cast<float>(h), 0.f);// w: link, below
            const std::uint32_t sb = d.edge_sub_begin[3 * c + e];
            const std::uint32_t se = d.edge_sub_begin[3 * c + e + 1];
            g.sub_begin[e] = sb;
            if (e == 2) { g.sub_begin[3] = se; }
            int link = -1;
            std::uint32_t rev = kNoEdge;
            bool flip = false;
            for (std::uint32_t k = sb; k < se && link == -1; ++k) {
                if (d.sub_kind[k] != 0) { continue; }
                const std::uint32_t n = d.sub_target[k];
                if (n >= C) { throw std::invalid_argument("transition target out of range"); }
                link = static_cast<int>(n);
                const psim::P2 on = vtx(n, 0);
                f.offset[e] = make_float2(static_cast<float>(o.x - on.x), static_cast<float>(o.y - on.y));
                const psim::Seg64 sl = seg_from(&d.sub_line[4 * k]);
                const psim::P2 mid{ (sl.a.x + sl.b.x) / 2., (sl.a.y + sl.b.y) / 2. };
                for (int e2 = 0; e2 < 3 && rev == kNoEdge; ++e2) {
                    const psim::Seg64 ne = psim::make_seg(vtx(n, e2), vtx(n, (e2 + 1) % 3), nullptr);
                    if (psim::on_line(ne, mid) && psim::on_line(ne, sl.a) && psim::on_line(ne, sl.b)) { rev = static_cast<std::uint32_t>(e2); }
                }
                const psim::P2 sn = psim::seg_normal(sl.a, sl.b, cell_sign[c]);
                flip = (sn.x * n_in.x + sn.y * n_in.y) < 0.;
            }
            for (std::uint32_t k = sb; k < se && link == -1; ++k) {
                if (d.sub_kind[k] != 1) { continue; }
                if (d.sub_target[k] >= d.n_emitters) { throw std::invalid_argument("emitter index out of range"); }
                link = -static_cast<int>(d.sub_target[k]) - 2;
            }
            std::memcpy(&f.edge[e].w, &link, sizeof link);// the edge's link, as int bits
            f.rev |= (rev & 3U) << (2 * e);
            if (flip) { f.rev |= 1U << (8 + e); }
            for (std::uint32_t k = sb; k < se; ++k) {
                Sub64& s = subs[k];
                const double* l = &d.sub_line[4 * k];
                s.line = line64(psim::P2{ l[0], l[1] }, psim::P2{ l[2], l[3] });
                const psim::P2 sn = (d.sub_kind[k] == 0) ? psim::seg_normal(psim::P2{ l[0], l[1] }, psim::P2{ l[2], l[3] }, cell_sign[c]) : n_in;
                s.nx = sn.x;
                s.ny = sn.y;
                s.kind = d.sub_kind[k];
                s.target = d.sub_target[k];
            }
        }
    }
}

struct Engine::Impl {
    Buf cells32, cells64, subs64, sensors, materials, emitters, alias, centre32, vel32, centre64, vel64;
    InterpCache* interp{ nullptr };// the interpreter's buffers, reused by every read-out
    std::vector<EmitterDev> emit_host;
    std::vector<BirthGroup> groups;
    std::vector<std::uint32_t> group_begin;// [N+1]
    std::vector<std::uint32_t> n_new;      // [N]
    std::vector<std::uint32_t> id_base;    // [N]
    Buf d_groups;
    Buf state[2];
    std::uint64_t capacity{ 0 };
    Buf counts;  // u32: survivor counters [0, 3), work counters [4, 7), back-group survivor counters [8, 11)
    Buf counters;// 8 x u64: phonon-steps, relocations, overflow, max population, event-limit hits
    Buf tally;   // [K][S]
    Buf population;// [N] u32
    Buf unpacked_energy, unpacked_flux;
    std::uint64_t total{ 0 };
    std::uint32_t key0{ 0 }, key1{ 0 };
    bool builders_ready{ false };
    cudaEvent_t ev0{ nullptr }, ev1{ nullptr };
    cudaStream_t own{ nullptr };
    int sms{ 0 };

    Impl() = default;
    Impl(const Impl&) = delete;
    Impl& operator=(const Impl&) = delete;
    ~Impl() {// also when the engine's constructor throws part-way
        if (ev0 != nullptr) { cudaEventDestroy(ev0); }
        if (ev1 != nullptr) { cudaEventDestroy(ev1); }
        if (own != nullptr) { cudaStreamDestroy(own); }
        interp_cache_destroy(interp);
    }
};

void* create_stream() {
    cudaStream_t s = nullptr;
    check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    return s;
}

void destroy_stream(void* stream) noexcept {
    if (stream != nullptr) { cudaStreamDestroy(static_cast<cudaStream_t>(stream)); }
}

int sm_count() {
    int dev = 0;
    int sms = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    return sms;
}

int device_count() noexcept {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

namespace {

// The inputs of the scattering rates (Material::relaxRates, psim/src/material.cpp:54-62).  The
// kernels' event loops end only when every rate is finite and non-negative: a negative or NaN
// rate sum gives a negative or NaN time to the next scattering event, and the step boundary is
// then never reached.  So the relaxation coefficients must be finite and non-negative and the
// sensor temperatures positive and finite; both are checked before any device work.
void check_rate_inputs(const SimDesc& d) {
    if (d.mat_params.size() < static_cast<std::size_t>(d.n_materials) * 8 || d.sensor_temp.size() < d.n_sensors) {
        throw std::invalid_argument("missing material parameters or sensor temperatures");
    }
    for (std::uint32_t m = 0; m < d.n_materials; ++m) {
        const double* pr = &d.mat_params[8 * static_cast<std::size_t>(m)];
        for (int k = 0; k < 4; ++k) {// b_l, b_tn, b_tu, b_i
            if (!std::isfinite(pr[k]) || pr[k] < 0.) {
                throw std::invalid_argument("relaxation coefficients must be finite and non-negative (material "
                                            + std::to_string(m) + ")");
            }
        }
        if (!std::isfinite(pr[4])) { throw std::invalid_argument("the relaxation cut-off frequency w must be finite"); }
    }
    for (std::uint32_t s = 0; s < d.n_sensors; ++s) {
        const double T = d.sensor_temp[s];
        if (!(T > 0.) || !std::isfinite(T)) {
            throw std::invalid_argument("sensor temperatures must be positive and finite (sensor " + std::to_string(s) + ")");
        }
    }
}

// The run's time line: a positive simulated time, and emitting windows inside it
// (Model::setEmitSurface's rule, psim/src/model.cpp:125-133), so that birth steps are in range.
void check_time_line(const SimDesc& d) {
    if (!(d.sim_time > 0.) || !std::isfinite(d.sim_time)) { throw std::invalid_argument("simulation time must be positive and finite"); }
    if (d.emit_start.size() < d.n_emitters || d.emit_duration.size() < d.n_emitters) {
        throw std::invalid_argument("missing emitter start times or durations");
    }
    for (std::uint32_t e = 0; e < d.n_emitters; ++e) {
        const double start = d.emit_start[e];
        const double dur = d.emit_duration[e];
        if (!(start >= 0.) || !(start < d.sim_time) || !(dur >= 0.) || !(dur <= d.sim_time - start)) {
            throw std::invalid_argument("emitter start time or duration outside the simulated time (emitter " + std::to_string(e) + ")");
        }
    }
}

}// namespace

Engine::Engine(const SimDesc& d)
    : desc_{ d }
    , impl_{ std::make_unique<Impl>() } {
    if (d.n_cells == 0 || d.n_sensors == 0 || d.n_materials == 0 || d.steps == 0) { throw std::invalid_argument("empty model"); }
    if (d.n_materials > kMaxMaterials) { throw std::invalid_argument("at most 16 materials are supported"); }
    if (d.n_cells >= (1U << 24)) { throw std::invalid_argument("at most 2^24 - 1 cells are supported"); }
    if (d.steps >= 0xFFFFFFFFULL) { throw std::invalid_argument("too many measurement steps"); }
    check_rate_inputs(d);
    check_time_line(d);
    if (device_count() <= 0) { throw std::runtime_error("no CUDA device is available"); }
    Impl& I = *impl_;
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&I.sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    check(cudaStreamCreateWithFlags(&I.own, cudaStreamNonBlocking), "stream");
    I.interp = interp_cache_create();
    stream_ = I.own;
    check(cudaEventCreate(&I.ev0), "event");
    check(cudaEventCreate(&I.ev1), "event");

    std::vector<CellF32> c32;
    std::vector<CellF64> c64;
    std::vector<Sub64> subs;
    build_cells(d, c32, c64, subs);
    const std::uint32_t C = d.n_cells;
    auto vtx = [&](std::uint32_t c, int i) {
        return psim::P2{ d.cell_vertices[6 * c + 2 * i], d.cell_vertices[6 * c + 2 * i + 1] };
    };
    I.cells32.upload(c32);
    I.cells64.upload(c64);
    I.subs64.upload(subs);

    // ---- materials
    std::vector<MaterialDev> mats(d.n_materials);
    std::vector<float> centre32(static_cast<std::size_t>(d.n_materials) * kBins);
    std::vector<float> vel32(static_cast<std::size_t>(d.n_materials) * 2 * kBins);
    for (std::uint32_t m = 0; m < d.n_materials; ++m) {
        mats[m] = material_dev(&d.mat_params[8 * m]);
        for (int b = 0; b < kBins; ++b) {
            centre32[m * kBins + b] = static_cast<float>(d.mat_freq[m * kBins + b] / 1e13);
            vel32[(m * 2) * kBins + b] = static_cast<float>(d.mat_vel[(m * 2) * kBins + b]);
            vel32[(m * 2 + 1) * kBins + b] = static_cast<float>(d.mat_vel[(m * 2 + 1) * kBins + b]);
        }
    }
    I.materials.upload(mats);
    I.centre32.upload(centre32);
    I.vel32.upload(vel32);
    I.centre64.upload(d.mat_freq);
    I.vel64.upload(d.mat_vel);

    // ---- alias tables
    std::vector<std::uint32_t> alias(static_cast<std::size_t>(d.n_tables) * kAliasCols);
    for (std::uint32_t t = 0; t < d.n_tables; ++t) {
        const auto a = alias_table(&d.tables[static_cast<std::size_t>(t) * kBins * 2]);
        std::copy(a.begin(), a.end(), alias.begin() + static_cast<std::ptrdiff_t>(t) * kAliasCols);
    }
    I.alias.upload(alias);

    // ---- sensors
    std::vector<SensorDev> sens(d.n_sensors);
    for (std::uint32_t s = 0; s < d.n_sensors; ++s) {
        SensorDev& sd = sens[s];
        sensor_rate_factors(d.sensor_temp[s], sd);
        sd.material = d.sensor_material[s];
        if (sd.material >= d.n_materials) { throw std::invalid_argument("sensor material out of range"); }
        sd.base_table = d.sensor_base_table[s];
        sd.scatter_table = d.sensor_scatter_table[s];
        if (sd.base_table >= d.n_tables || sd.scatter_table >= d.n_tables) { throw std::invalid_argument("sensor table out of range"); }
    }
    I.sensors.upload(sens);

    // ---- emitters
    const double dt = d.sim_time / static_cast<double>(d.steps);
    I.emit_host.resize(d.n_emitters);
    for (std::uint32_t e = 0; e < d.n_emitters; ++e) {
        EmitterDev& em = I.emit_host[e];
        std::memset(&em, 0, sizeof em);
        const std::uint32_t c = d.emit_cell[e];
        const int edge = static_cast<int>(d.emit_edge[e]);
        if (c >= C || edge > 2) { throw std::invalid_argument("emitter cell/edge out of range"); }
        const psim::P2 o = vtx(c, 0);
        const double* l = &d.emit_line[4 * e];
        em.ax = l[0];
        em.ay = l[1];
        em.bx = l[2];
        em.by = l[3];
        em.a = make_float2(static_cast<float>(l[0] - o.x), static_cast<float>(l[1] - o.y));
        em.b = make_float2(static_cast<float>(l[2] - o.x), static_cast<float>(l[3] - o.y));
        em.nx64 = c64[c].nx[edge];
        em.ny64 = c64[c].ny[edge];
        em.nx = static_cast<float>(em.nx64);
        em.ny = static_cast<float>(em.ny64);
        em.cell = c;
        em.edge = static_cast<std::uint32_t>(edge);
        em.table = d.emit_table[e];
        if (em.table >= d.n_tables) { throw std::invalid_argument("emit table out of range"); }
        em.spec = c64[c].spec;
        // EmitSurface::handlePhonon absorbs when the phonon's step time s*dt is inside
        // [start, start + duration - dt] (psim/src/surface.cpp:61-65), evaluated exactly.
        em.absorb_lo = 1U;
        em.absorb_hi = 0U;
        bool any = false;
        for (std::uint64_t s = 0; s < d.steps; ++s) {
            const double pt = static_cast<double>(s) * dt;
            const bool absorb = !(pt < d.emit_start[e] || pt + dt > d.emit_start[e] + d.emit_duration[e]);
            if (absorb) {
                if (!any) { em.absorb_lo = static_cast<std::uint32_t>(s); }
                em.absorb_hi = static_cast<std::uint32_t>(s);
                any = true;
            }
        }
    }
    I.emitters.upload(I.emit_host);

    model_bytes_ = I.cells32.bytes + I.cells64.bytes + I.subs64.bytes + I.materials.bytes + I.centre32.bytes + I.vel32.bytes
                   + I.centre64.bytes + I.vel64.bytes + I.alias.bytes + I.sensors.bytes + I.emitters.bytes;
    // ---- run buffers
    I.counts.alloc(16 * sizeof(std::uint32_t));// 3 survivor counters, 3 work counters, 3 back-group counters
    I.counters.alloc(8 * sizeof(unsigned long long));
    I.tally.alloc(static_cast<std::size_t>(d.recorded) * d.n_sensors * sizeof(TallySlot));
    I.population.alloc(static_cast<std::size_t>(d.steps) * sizeof(std::uint32_t));
    check(cudaMemset(I.population.p, 0, I.population.bytes), "memset population");
    check(cudaMemset(I.tally.p, 0, I.tally.bytes), "memset tally");
}

Engine::~Engine() = default;

std::uint64_t Engine::init_builders(double t_eq, double eff_energy, const double* cell_energy, const double* emit_energy,
                                    const double* sensor_init_temp, std::uint64_t seed) {
    Impl& I = *impl_;
    const SimDesc& d = desc_;
    const std::uint64_t N = d.steps;
    std::mt19937_64 rng(seed ^ 0x5DEECE66DULL);
    std::uniform_real_distribution<double> uni(0., 1.);
    // floor(E / eff) plus one with probability equal to the fraction (modelSimulator.cpp:44-49)
    auto count = [&](double energy) -> std::uint64_t {
        if (!(energy > 0.) || !(eff_energy > 0.)) { return 0; }
        double whole = 0.;
        const double frac = std::modf(energy / eff_energy, &whole);
        if (!(whole < 4294967295.)) { throw std::length_error("more than 2^32 - 1 phonons in one run"); }
        auto n = static_cast<std::uint64_t>(whole);
        return (uni(rng) < frac) ? n + 1 : n;
    };
    std::vector<std::vector<BirthGroup>> per_step(N);
    std::uint64_t total = 0;
    std::uint32_t first0 = 0;
    for (std::uint32_t c = 0; c < d.n_cells; ++c) {
        const std::uint64_t n = count(cell_energy[c]);
        if (n == 0) { continue; }
        BirthGroup g{};
        g.first = first0;
        g.source = static_cast<std::int32_t>(c);
        g.sign = (sensor_init_temp[d.cell_sensor[c]] > t_eq) ? 1 : -1;
        per_step[0].push_back(g);
        total += n;
        if (total >= 0xFFFFFFFFULL) { throw std::length_error("more than 2^32 - 1 phonons in one run"); }
        first0 += static_cast<std::uint32_t>(n);
    }
    std::vector<std::uint64_t> step_total(N, 0);
    step_total[0] = first0;
    const double dt = d.sim_time / static_cast<double>(N);
    for (std::uint32_t e = 0; e < d.n_emitters; ++e) {
        std::uint64_t n = count(emit_energy[e]);
        if (n == 0) { continue; }
        total += n;
        if (total >= 0xFFFFFFFFULL) { throw std::length_error("more than 2^32 - 1 phonons in one run"); }
        // Birth times are uniform over [start, start + duration] (EmitSurface::getPhononTime,
        // psim/src/surface.cpp:67-69); the number born in each step is multinomial.
        const double start = d.emit_start[e];
        const double end = start + d.emit_duration[e];
        const auto s_first = static_cast<std::uint64_t>(std::min<double>(std::floor(start / dt), static_cast<double>(N - 1)));
        const auto s_last = static_cast<std::uint64_t>(std::min<double>(std::floor(end / dt), static_cast<double>(N - 1)));
        double mass = end - start;
        const int sign = (d.emit_temp[e] > t_eq) ? 1 : -1;
        for (std::uint64_t s = s_first; s <= s_last && n > 0; ++s) {
            const double lo = std::max(start, static_cast<double>(s) * dt);
            const double hi = (s == s_last) ? end : std::min(end, static_cast<double>(s + 1) * dt);
            const double len = std::max(hi - lo, 0.);
            std::uint64_t m = n;
            if (s != s_last) {
                const double p = mass > 0. ? std::min(std::max(len / mass, 0.), 1.) : 1.;
                std::binomial_distribution<std::uint64_t> bin(n, p);
                m = bin(rng);
            }
            mass -= len;
            n -= m;
            if (m == 0) { continue; }
            BirthGroup g{};
            g.first = static_cast<std::uint32_t>(step_total[s]);
            g.source = -static_cast<std::int32_t>(e) - 1;
            g.t0_64 = lo - static_cast<double>(s) * dt;
            g.span64 = len;
            g.t0 = static_cast<float>(g.t0_64);
            g.span = static_cast<float>(g.span64);
            g.sign = sign;
            per_step[s].push_back(g);
            step_total[s] += m;
        }
    }
    I.groups.clear();
    I.group_begin.assign(N + 1, 0);
    I.n_new.assign(N, 0);
    I.id_base.assign(N, 0);
    std::uint64_t ids = 0;
    for (std::uint64_t s = 0; s < N; ++s) {
        I.group_begin[s] = static_cast<std::uint32_t>(I.groups.size());
        for (const auto& g : per_step[s]) { I.groups.push_back(g); }
        I.n_new[s] = static_cast<std::uint32_t>(step_total[s]);
        I.id_base[s] = static_cast<std::uint32_t>(ids);
        ids += step_total[s];
    }
    I.group_begin[N] = static_cast<std::uint32_t>(I.groups.size());
    I.d_groups.upload(I.groups);
    counters_.h2d_bytes += I.groups.size() * sizeof(BirthGroup);
    I.total = total;
    I.key0 = static_cast<std::uint32_t>(seed) ^ 0x243F6A88U;
    I.key1 = static_cast<std::uint32_t>(seed >> 32) ^ 0x85A308D3U;
    I.builders_ready = true;
    counters_.phonons = total;
    return total;
}

// Room for at least 'need' phonons of rec_bytes each; the records of state buffer 'cur' are kept:
// its first live_front slots and its last live_back slots (the two groups of survivors).
// grow_ahead allocates a quarter more than asked (and at least half again the current capacity),
// for runs that grow their buffers between chunks of launches.
void Engine::ensure_capacity(std::uint64_t need, std::uint64_t live_front, std::uint64_t live_back, int cur, std::size_t rec_bytes,
                             bool grow_ahead, void* stream_ptr) {
    Impl& I = *impl_;
    auto stream = static_cast<cudaStream_t>(stream_ptr);
    if (need <= I.capacity) { return; }
    if (need > 0xFFFFFFFFULL) { throw std::length_error("more than 2^32 - 1 phonons in flight"); }
    std::size_t free_b = 0;
    std::size_t total_b = 0;
    check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    const std::uint64_t held = I.capacity * 2 * rec_bytes;
    const std::uint64_t limit = static_cast<std::uint64_t>((free_b + held) * 0.8) / (2 * rec_bytes);
    std::uint64_t cap = grow_ahead ? std::max(need + need / 4, I.capacity + I.capacity / 2) : need;
    cap = std::min<std::uint64_t>(std::min(cap, limit), 0xFFFFFFFFULL);
    if (cap < need) {
        throw std::length_error("phonon buffers: " + std::to_string(need) + " phonons in flight do not fit in device memory");
    }
    Buf a;
    Buf b;
    a.alloc(cap * rec_bytes);
    b.alloc(cap * rec_bytes);
    if (live_front + live_back > 0) {// records are SoA: one 16-byte word per phonon per segment of 'capacity' words
        for (std::size_t k = 0; k < rec_bytes / 16; ++k) {
            const char* src = static_cast<const char*>(I.state[cur].p) + k * I.capacity * 16;
            char* dst = static_cast<char*>(a.p) + k * cap * 16;
            if (live_front > 0) { check(cudaMemcpyAsync(dst, src, live_front * 16, cudaMemcpyDeviceToDevice, stream), "state copy"); }
            if (live_back > 0) {
                check(cudaMemcpyAsync(dst + (cap - live_back) * 16, src + (I.capacity - live_back) * 16, live_back * 16,
                                      cudaMemcpyDeviceToDevice, stream),
                      "state copy");
            }
        }
        check(cudaStreamSynchronize(stream), "state copy");
    }
    I.state[cur].take(a);
    I.state[1 - cur].take(b);
    I.capacity = cap;
}

// The launch parameters that do not change between a run's launches.
void Engine::base_params(StepParams& P) const {
    const Impl& I = *impl_;
    const SimDesc& d = desc_;
    P = StepParams{};
    P.cells32 = I.cells32.as<CellF32>();
    P.cells64 = I.cells64.as<CellF64>();
    P.subs64 = I.subs64.as<Sub64>();
    P.sensors = I.sensors.as<SensorDev>();
    P.materials = I.materials.as<MaterialDev>();
    P.emitters = I.emitters.as<EmitterDev>();
    P.alias = I.alias.as<std::uint32_t>();
    P.centre32 = I.centre32.as<float>();
    P.vel32 = I.vel32.as<float>();
    P.centre64 = I.centre64.as<double>();
    P.vel64 = I.vel64.as<double>();
    P.n_sensors = d.n_sensors;
    P.groups = I.d_groups.as<BirthGroup>();
    P.capacity = static_cast<std::uint32_t>(std::min<std::uint64_t>(I.capacity, 0xFFFFFFFFULL));
    P.n_steps = static_cast<std::uint32_t>(d.steps);
    P.step_adj = static_cast<std::uint32_t>(d.step_adj);
    P.n_recorded = static_cast<std::uint32_t>(d.recorded);
    P.dt64 = d.sim_time / static_cast<double>(d.steps);
    P.dt = static_cast<float>(P.dt64);
    P.phasor_sim = d.phasor ? 1 : 0;
    P.full_sim = d.full ? 1 : 0;
    P.key0 = I.key0;
    P.key1 = I.key1;
    P.tally = I.tally.as<TallySlot>();
    P.counters = I.counters.as<unsigned long long>();
    P.population = I.population.as<std::uint32_t>();
    P.n_cells = d.n_cells;
    P.n_tables = d.n_tables;
    P.n_materials = d.n_materials;
    P.n_emitters = d.n_emitters;
}

// Launch w of the run: steps [s0, s0 + tw), its state buffers and counters (cycling with w) and
// the births of each of its steps.
void Engine::window_params(StepParams& P, std::uint64_t w, std::uint64_t s0, std::uint32_t tw) const {
    const Impl& I = *impl_;
    auto* counts = I.counts.as<std::uint32_t>();
    P.capacity = static_cast<std::uint32_t>(I.capacity);
    P.step = static_cast<std::uint32_t>(s0);
    P.n_fused = tw;
    P.in = I.state[w % 2].p;
    P.out = I.state[(w + 1) % 2].p;
    P.count_in = counts + (w % 3);
    P.count_out = counts + ((w + 1) % 3);
    P.count_clear = counts + ((w + 2) % 3);
    P.work = counts + 4 + (w % 3);
    P.work_clear = counts + 4 + ((w + 2) % 3);
    P.back_in = counts + 8 + (w % 3);
    P.back_out = counts + 8 + ((w + 1) % 3);
    P.back_clear = counts + 8 + ((w + 2) % 3);
    P.group_begin = I.group_begin[s0];
    P.group_end = I.group_begin[s0 + 1];
    P.n_new = I.n_new[s0];
    P.id_base = I.id_base[s0];
    P.new_begin[0] = 0U;
    for (std::uint32_t j = 0; j < tw; ++j) {
        P.new_begin[j + 1] = P.new_begin[j] + I.n_new[s0 + j];
        P.id_base_f[j] = I.id_base[s0 + j];
        P.group_begin_f[j] = I.group_begin[s0 + j];
    }
    P.group_begin_f[tw] = I.group_begin[s0 + tw];
}

// Steps of launches covering [s0, s0 + cap) whose work items all number in 32 bits.
std::uint32_t Engine::window_steps(std::uint64_t s0, std::uint32_t cap, std::uint64_t capacity) const {
    const Impl& I = *impl_;
    std::uint32_t tw = static_cast<std::uint32_t>(std::min<std::uint64_t>(cap, desc_.steps - s0));
    auto items = [&](std::uint32_t n) {
        std::uint64_t t = capacity;
        for (std::uint32_t j = 0; j < n; ++j) { t += I.n_new[s0 + j]; }
        return t;
    };
    while (tw > 1 && items(tw) > 0xFFFFFFFFULL) { --tw; }
    if (items(tw) > 0xFFFFFFFFULL) { throw std::length_error("too many phonons in one step for 32-bit work indices"); }
    return tw;
}

// Reads the run's device counters into the run counters.
void Engine::finish_run(double ms, std::uint64_t launches, std::uint64_t transport_launches, std::uint32_t fused) {
    Impl& I = *impl_;
    unsigned long long c[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    check(cudaMemcpy(c, I.counters.p, sizeof c, cudaMemcpyDeviceToHost), "counters");
    counters_.phonon_steps += c[0];
    counters_.relocations += c[1];
    counters_.event_limits += c[4];
    counters_.backscatters += c[6];
    counters_.state_bytes = I.state[0].bytes + I.state[1].bytes;
    I.builders_ready = false;
    if (c[5] != 0) { throw std::runtime_error("CUDA staging of the model tables into shared memory timed out"); }
    counters_.overflow += c[2];
    counters_.max_population = std::max<std::uint64_t>(counters_.max_population, c[3]);
    counters_.kernel_ms += ms;
    counters_.d2h_bytes += sizeof c;
    counters_.kernel_launches += launches;
    counters_.transport_launches += transport_launches;
    counters_.steps_per_launch = fused;
    last_fused_ = fused;
    if (c[2] != 0) { throw std::length_error("phonon buffer overflow: the device ran out of memory for the population"); }
}

void Engine::run(int precision, void* stream_ptr) {
    Impl& I = *impl_;
    const SimDesc& d = desc_;
    if (!I.builders_ready) { throw std::logic_error("init_builders must be called before run"); }
    cudaStream_t stream = stream_ptr != nullptr ? static_cast<cudaStream_t>(stream_ptr) : I.own;
    const bool fp64 = precision != 0;
    const std::size_t rec_bytes = fp64 ? 64 : 32;
    // State buffers.  The population never exceeds the phonons created in the run, so a run whose
    // phonons all fit in kWholeRunStateBytes gets room for every one of them and runs as one CUDA
    // graph.  A larger run is chunked instead: before each chunk of launches the host reads the
    // population entering it and grows the buffers when that population plus the chunk's newborns
    // would not fit, so the buffers follow the peak population and no phonon is ever dropped.
    const std::uint64_t whole = std::max<std::uint64_t>(I.total + 1024, 4096);
    bool chunked = stop_on_ || whole * 2 * rec_bytes > kWholeRunStateBytes;
    if (const char* ch = std::getenv("PSIM_GB300_CHUNKED"); ch != nullptr) {// test and measurement switch
        chunked = std::atoi(ch) != 0 || stop_on_;
    }
    if (I.state[0].bytes != I.capacity * rec_bytes) {// first run, or the other precision's records
        I.state[0].release();
        I.state[1].release();
        I.capacity = 0;
    }
    if (!chunked) { ensure_capacity(whole, 0, 0, 0, rec_bytes, false, stream); }
    check(cudaMemsetAsync(I.counts.p, 0, I.counts.bytes, stream), "memset counts");
    check(cudaMemsetAsync(I.counters.p, 0, I.counters.bytes, stream), "memset counters");
    check(cudaMemsetAsync(I.population.p, 0, I.population.bytes, stream), "memset population");

    StepParams P{};
    base_params(P);
    auto* counts = I.counts.as<std::uint32_t>();
    // Launch shape and shared memory.  The FP32 kernel stages the cell records and the
    // alias / velocity / bin-centre tables into shared memory (TMA bulk copies) when they fit
    // next to the block's tally, and then runs one 1024-thread block per SM.  An FP32 launch
    // covers as many steps (up to kMaxFused) as tally slots fit in the shared memory left.
    std::uint32_t fuse_cap = kMaxFused;
    if (const char* f = std::getenv("PSIM_GB300_FUSE"); f != nullptr && std::atoi(f) > 0) {
        fuse_cap = std::min<std::uint32_t>(kMaxFused, static_cast<std::uint32_t>(std::atoi(f)));
    }
    std::uint32_t fused = 1;
    P.coast_lanes = coast_lanes_;
    P.tail_order = kTailOrder;
    if (const char* to = std::getenv("PSIM_GB300_TAIL"); to != nullptr) { P.tail_order = std::atoi(to) != 0 ? 1U : 0U; }
    P.pool = kWarpPool;
    if (const char* pl = std::getenv("PSIM_GB300_POOL"); pl != nullptr) { P.pool = static_cast<std::uint32_t>(std::max(0, std::atoi(pl))); }
    P.fetch_lanes = kFetchLanes;
    if (const char* fl = std::getenv("PSIM_GB300_FETCH"); fl != nullptr && std::atoi(fl) > 0) {
        P.fetch_lanes = static_cast<std::uint32_t>(std::min(32, std::atoi(fl)));
    }
    P.sort_mode = 0U;
    if (const char* so = std::getenv("PSIM_GB300_SORT"); so != nullptr && !fp64) {// "mode:value", value in steps or m/s
        const int mode = std::atoi(so);
        const char* colon = std::strchr(so, ':');
        const double v = colon != nullptr ? std::atof(colon + 1) : 0.;
        if (mode == 1) {
            P.sort_mode = 1U;
            P.sort_after = static_cast<float>(v * P.dt64);
        } else if (mode == 2) {
            P.sort_mode = 2U;
            P.sort_after = static_cast<float>(v);
        }
    }
    if (const char* c = std::getenv("PSIM_GB300_COAST"); c != nullptr) { P.coast_lanes = static_cast<std::uint32_t>(std::max(0, std::atoi(c))); }
    std::size_t tally_b = tally_smem_bytes(d.n_sensors, 1);
    P.stage_mask = 0U;
    P.off_tally = 0U;
    std::size_t smem = tally_b;
    int block = 256;
    bool stage = stage_tables_;
    bool tables_only = false;// stage the tables but not the cell records even where both fit
    if (const char* st = std::getenv("PSIM_GB300_STAGE"); st != nullptr) {
        stage = stage && std::atoi(st) != 0;
        tables_only = std::atoi(st) == 2;
    }
    if (!fp64 && stage) {
        int dev = 0;
        int optin = 0;
        check(cudaGetDevice(&dev), "cudaGetDevice");
        check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device attribute");
        const std::size_t budget = static_cast<std::size_t>(optin) - 1024;// static shared memory and slack
        const std::size_t cells_b = static_cast<std::size_t>(d.n_cells) * sizeof(CellF32);
        const std::size_t alias_b = static_cast<std::size_t>(d.n_tables) * kAliasCols * 4;
        const std::size_t vel_b = static_cast<std::size_t>(d.n_materials) * 2 * kBins * 4;
        const std::size_t centre_b = static_cast<std::size_t>(d.n_materials) * kBins * 4;
        const std::size_t sens_b = static_cast<std::size_t>(d.n_sensors) * sizeof(SensorDev);
        const std::size_t mat_b = static_cast<std::size_t>(d.n_materials) * sizeof(MaterialDev);
        const std::size_t emit_b = static_cast<std::size_t>(d.n_emitters) * sizeof(EmitterDev);
        const std::size_t tables_b = alias_b + vel_b + centre_b + sens_b + mat_b + emit_b;
        // Everything when it fits next to the tally, else the tables without the cell records
        // (large models: cells and, above kSharedSensors sensors, tallies in global memory).
        const bool all = !tables_only && cells_b + tables_b + tally_b <= budget;
        if (all || tables_b + tally_b <= budget) {
            const std::size_t cb = all ? cells_b : 0;
            const std::size_t used = cb + tables_b;
            while (fused < fuse_cap && used + tally_smem_bytes(d.n_sensors, fused + 1) <= budget) { ++fused; }
            tally_b = tally_smem_bytes(d.n_sensors, fused);
            P.off_cells = 0U;
            P.off_alias = static_cast<std::uint32_t>(cb);
            P.off_vel = static_cast<std::uint32_t>(cb + alias_b);
            P.off_centre = static_cast<std::uint32_t>(cb + alias_b + vel_b);
            P.off_sensors = static_cast<std::uint32_t>(cb + alias_b + vel_b + centre_b);
            P.off_materials = static_cast<std::uint32_t>(P.off_sensors + sens_b);
            P.off_emitters = static_cast<std::uint32_t>(P.off_materials + mat_b);
            P.off_tally = static_cast<std::uint32_t>(used);
            P.stage_mask = all ? 7U : 6U;
            smem = used + tally_b;
            block = 1024;
        }
    }
    // global tables: tally slots up to 32 KB per 256-thread block
    auto unstaged_fuse = [&]() {
        fused = 1;
        while (fused < fuse_cap && tally_smem_bytes(d.n_sensors, fused + 1) <= 32 * 1024) { ++fused; }
        tally_b = tally_smem_bytes(d.n_sensors, fused);
        smem = tally_b;
    };
    if (!fp64 && P.stage_mask == 0U) { unstaged_fuse(); }
    int occ = fp64 ? occupancy_f64(smem) : occupancy_f32(P.stage_mask, block, smem);
    if (occ <= 0 && !fp64 && P.stage_mask != 0U) {// cannot launch staged: fall back to global tables
        P.stage_mask = 0U;
        P.off_tally = 0U;
        block = 256;
        unstaged_fuse();
        occ = occupancy_f32(0U, block, smem);
    }
    if (fp64) { fused = 1; }
    occ = std::max(1, occ);
    int grid = grid_override_ > 0 ? grid_override_ : I.sms * occ;
    last_stage_mask_ = P.stage_mask;
    if (const char* g = std::getenv("PSIM_GB300_GRID"); g != nullptr && std::atoi(g) > 0) { grid = std::atoi(g); }// launch-shape override

    // FP32: launch w covers steps [s0, s0 + tw); FP64: one step per launch.  Steps [from, to) are
    // enqueued; the launch index w (which buffer and counter each launch uses) runs on across calls.
    std::uint64_t launches = 0;
    std::uint64_t w = 0;
    auto enqueue = [&](std::uint64_t from, std::uint64_t to) {
        for (std::uint64_t s0 = from; s0 < to; ++w) {
            std::uint32_t tw = window_steps(s0, static_cast<std::uint32_t>(std::min<std::uint64_t>(fused, to - s0)), I.capacity);
            window_params(P, w, s0, tw);
            if (fp64) {
                launch_step_f64(P, grid, smem, stream);
            } else {
                launch_step_f32(P, grid, block, smem, stream);
            }
            ++launches;
            s0 += tw;
        }
    };
    auto finish = [&](std::uint64_t steps_done) {
        if (!fp64) {
            launch_population_max(P.population, static_cast<std::uint32_t>(steps_done), P.counters, stream);
            ++launches;
        }
    };
    std::uint64_t checks = 0;
    steps_run_ = d.steps;

    check(cudaEventRecord(I.ev0, stream), "event record");
    if (chunked) {// launches in chunks: buffers grown between chunks, steady-state checks where asked
        if (stop_on_ && (d.step_adj != 0 || d.recorded != d.steps)) {
            throw std::invalid_argument("stopping at steady state needs every step recorded (periodic or transient runs)");
        }
        const std::uint64_t min_steps = static_cast<std::uint64_t>(stop_crit_.patience + 1) * stop_crit_.window;
        const std::uint64_t every = stop_check_ > 0 ? stop_check_ : min_steps;
        std::vector<std::uint64_t> born(d.steps + 1, 0);// newborns of steps [0, s)
        for (std::uint64_t s = 0; s < d.steps; ++s) { born[s + 1] = born[s] + I.n_new[s]; }
        std::uint64_t done = 0;
        // steady checks at the multiples of 'every' from min_steps on
        std::uint64_t next_check = stop_on_ ? std::max<std::uint64_t>(1, (min_steps + every - 1) / every) * every : d.steps;
        while (done < d.steps) {
            std::uint64_t to = std::min<std::uint64_t>(d.steps, done + kLaunchesPerChunk * fused);
            if (stop_on_) { to = std::min(to, next_check); }
            // the phonons entering step 'done' (the next launch's input count) plus the chunk's newborns
            std::uint32_t live[2] = { 0U, 0U };// the front and back groups of survivors
            if (done > 0) {
                check(cudaMemcpyAsync(&live[0], counts + (w % 3), sizeof(std::uint32_t), cudaMemcpyDeviceToHost, stream), "count read");
                check(cudaMemcpyAsync(&live[1], counts + 8 + (w % 3), sizeof(std::uint32_t), cudaMemcpyDeviceToHost, stream), "count read");
                check(cudaStreamSynchronize(stream), "count read");
            }
            ensure_capacity(static_cast<std::uint64_t>(live[0]) + live[1] + (born[to] - born[done]) + 1024, live[0], live[1],
                            static_cast<int>(w % 2), rec_bytes, true, stream);
            enqueue(done, to);
            check(cudaGetLastError(), "step launch");
            done = to;
            if (stop_on_ && done == next_check && done < d.steps) {
                next_check = std::min<std::uint64_t>(d.steps, done + every);
                ++checks;
                if (steady_onset_device(I.tally.p, d.n_sensors, done, stop_crit_, nullptr, stream) >= 0) { break; }
            }
        }
        steps_run_ = done;
        finish(done);
        check(cudaGetLastError(), "step launch");
        check(cudaEventRecord(I.ev1, stream), "event record");
        check(cudaStreamSynchronize(stream), "run sync");
    } else if (use_graph_) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        enqueue(0, d.steps);
        finish(d.steps);
        check(cudaStreamEndCapture(stream, &graph), "end capture");
        check(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
        check(cudaGraphLaunch(exec, stream), "graph launch");
        check(cudaEventRecord(I.ev1, stream), "event record");
        check(cudaStreamSynchronize(stream), "run sync");
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
    } else {
        enqueue(0, d.steps);
        finish(d.steps);
        check(cudaGetLastError(), "step launch");
        check(cudaEventRecord(I.ev1, stream), "event record");
        check(cudaStreamSynchronize(stream), "run sync");
    }
    float ms = 0.f;
    check(cudaEventElapsedTime(&ms, I.ev0, I.ev1), "event time");
    finish_run(ms, launches + checks, fp64 ? launches : launches - 1, fused);// FP32 adds one population pass
}

bool Engine::run_batched(const std::vector<Engine*>& engines, void* stream_ptr, std::uint32_t per_thread) {
    if (engines.empty()) { return true; }
    auto stream = static_cast<cudaStream_t>(stream_ptr);
    const std::uint64_t steps = engines.front()->desc_.steps;
    int dev = 0;
    int optin = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device attribute");
    const std::size_t budget = static_cast<std::size_t>(optin) - batch_static_smem() - 256;
    std::uint32_t fuse_cap = kMaxFused;
    if (const char* f = std::getenv("PSIM_GB300_FUSE"); f != nullptr && std::atoi(f) > 0) {
        fuse_cap = std::min<std::uint32_t>(kMaxFused, static_cast<std::uint32_t>(std::atoi(f)));
    }
    // every model's tables and a shared tally of `fused` slots in one block's shared memory
    struct Layout {
        std::size_t cells, alias, vel, centre, sens, mat, emit;
        std::size_t tables() const { return cells + alias + vel + centre + sens + mat + emit; }
    };
    std::vector<Layout> lay(engines.size());
    std::uint32_t fused = fuse_cap;
    for (std::size_t e = 0; e < engines.size(); ++e) {
        const Engine& E = *engines[e];
        const SimDesc& d = E.desc_;
        if (!E.impl_->builders_ready || d.steps != steps || E.stop_on_ || d.n_sensors > static_cast<std::uint32_t>(kSharedSensors)) {
            return false;
        }
        Layout& L = lay[e];
        L.cells = static_cast<std::size_t>(d.n_cells) * sizeof(CellF32);
        L.alias = static_cast<std::size_t>(d.n_tables) * kAliasCols * 4;
        L.vel = static_cast<std::size_t>(d.n_materials) * 2 * kBins * 4;
        L.centre = static_cast<std::size_t>(d.n_materials) * kBins * 4;
        L.sens = static_cast<std::size_t>(d.n_sensors) * sizeof(SensorDev);
        L.mat = static_cast<std::size_t>(d.n_materials) * sizeof(MaterialDev);
        L.emit = static_cast<std::size_t>(d.n_emitters) * sizeof(EmitterDev);
        while (fused > 1 && L.tables() + tally_smem_bytes(d.n_sensors, fused) > budget) { --fused; }
        if (L.tables() + tally_smem_bytes(d.n_sensors, fused) > budget) { return false; }
    }
    std::size_t smem = 0;
    for (std::size_t e = 0; e < engines.size(); ++e) {
        smem = std::max(smem, lay[e].tables() + tally_smem_bytes(engines[e]->desc_.n_sensors, fused));
    }
    const int occ = occupancy_batch_f32(smem);
    if (occ <= 0) { return false; }
    const int grid = engines.front()->impl_->sms * occ;

    // state buffers that grow with each run's population (as a chunked single run's), cleared counters
    const std::size_t M = engines.size();
    std::vector<std::vector<std::uint64_t>> born(M);// newborns of steps [0, s) per model
    for (std::size_t m = 0; m < M; ++m) {
        Engine& E = *engines[m];
        Impl& I = *E.impl_;
        if (I.state[0].bytes != I.capacity * 32) {
            I.state[0].release();
            I.state[1].release();
            I.capacity = 0;
        }
        born[m].assign(steps + 1, 0);
        for (std::uint64_t k = 0; k < steps; ++k) { born[m][k + 1] = born[m][k] + I.n_new[k]; }
        check(cudaMemsetAsync(I.counts.p, 0, I.counts.bytes, stream), "memset counts");
        check(cudaMemsetAsync(I.counters.p, 0, I.counters.bytes, stream), "memset counters");
        check(cudaMemsetAsync(I.population.p, 0, I.population.bytes, stream), "memset population");
    }
    std::vector<std::uint64_t> starts;
    for (std::uint64_t s0 = 0; s0 < steps; s0 += fused) { starts.push_back(s0); }
    // each model's launch parameters that stay the same (tables, layout of its staged tables)
    std::vector<StepParams> base(M);
    for (std::size_t m = 0; m < M; ++m) {
        const Layout& L = lay[m];
        StepParams& P = base[m];
        engines[m]->base_params(P);
        P.coast_lanes = 0U;
        P.fetch_lanes = kFetchLanes;
        P.pool = kWarpPool;
        P.tail_order = kTailOrder;
        P.sort_mode = 0U;
        P.stage_mask = 7U;
        P.off_cells = 0U;
        P.off_alias = static_cast<std::uint32_t>(L.cells);
        P.off_vel = static_cast<std::uint32_t>(L.cells + L.alias);
        P.off_centre = static_cast<std::uint32_t>(L.cells + L.alias + L.vel);
        P.off_sensors = static_cast<std::uint32_t>(L.cells + L.alias + L.vel + L.centre);
        P.off_materials = static_cast<std::uint32_t>(P.off_sensors + L.sens);
        P.off_emitters = static_cast<std::uint32_t>(P.off_materials + L.mat);
        P.off_tally = static_cast<std::uint32_t>(L.tables());
    }
    // Launches in chunks: before each chunk every model's buffers are grown, where needed, to hold
    // its survivors entering the chunk plus the chunk's newborns (one gathered read of the counts).
    constexpr std::size_t kChunk = kLaunchesPerChunk;
    Buf d_params;
    Buf d_items;
    Buf d_live;// [M][2] survivors entering the next chunk: front and back groups
    d_params.alloc(std::min(kChunk, starts.size()) * M * sizeof(StepParams));
    d_items.alloc((M + 2) * sizeof(std::uint32_t));
    Buf d_status;
    d_status.alloc(8 * sizeof(std::uint32_t));
    check(cudaMemsetAsync(d_status.p, 0, d_status.bytes, stream), "memset status");
    std::uint32_t status[8] = {};
    const bool debug = std::getenv("PSIM_GB300_BATCH_DEBUG") != nullptr;
    // The batch's status: fail with what the kernels recorded when they gave up.
    auto check_status = [&](const char* where) {
        check(cudaMemcpyAsync(status, d_status.p, sizeof status, cudaMemcpyDeviceToHost, stream), "batch status");
        check(cudaStreamSynchronize(stream), "batch status");
        if (debug) {
            std::fprintf(stderr, "batch %s: abort %u, staging timeouts %u, items %u, stagings %u\n", where, status[0], status[1], status[2],
                         status[3]);
        }
        if (status[0] != 0U) {
            throw std::runtime_error(std::string("batched launches stopped (") + where + "): "
                                     + (status[0] == 1U ? "a CUDA staging of model tables into shared memory timed out"
                                                        : "a model's event-limit hits ran past the batch bound")
                                     + ", " + std::to_string(status[2]) + " work items run, " + std::to_string(status[3]) + " stagings");
        }
    };
    d_live.alloc(M * 2 * sizeof(std::uint32_t));
    std::vector<const std::uint32_t*> count_ptrs(2 * M);
    Buf d_count_ptrs;
    std::vector<std::uint32_t> live(2 * M, 0U);
    std::vector<StepParams> params(std::min(kChunk, starts.size()) * M);
    BatchLaunch B{};
    B.item_begin = d_items.as<std::uint32_t>();
    B.item_next = d_items.as<std::uint32_t>() + M + 1;
    B.status = d_status.as<std::uint32_t>();
    B.n_models = static_cast<std::uint32_t>(M);
    B.chunk = std::max<std::uint32_t>(1U, per_thread) * 1024U;
    cudaEvent_t ev0 = nullptr;
    cudaEvent_t ev1 = nullptr;
    check(cudaEventCreate(&ev0), "event");
    check(cudaEventCreate(&ev1), "event");
    float ms = 0.f;
    std::uint64_t launches = 0;
    try {
        check(cudaEventRecord(ev0, stream), "event record");
        for (std::size_t c0 = 0; c0 < starts.size(); c0 += kChunk) {
            const std::size_t c1 = std::min(starts.size(), c0 + kChunk);
            const std::uint64_t s_from = starts[c0];
            const std::uint64_t s_to = c1 < starts.size() ? starts[c1] : steps;
            if (c0 > 0) {
                for (std::size_t m = 0; m < M; ++m) {
                    const auto* counts = engines[m]->impl_->counts.as<std::uint32_t>();
                    count_ptrs[2 * m] = counts + (c0 % 3);
                    count_ptrs[2 * m + 1] = counts + 8 + (c0 % 3);
                }
                d_count_ptrs.upload(count_ptrs);
                launch_gather_counts(d_count_ptrs.as<const std::uint32_t*>(), static_cast<std::uint32_t>(2 * M), d_live.as<std::uint32_t>(),
                                     stream);
                check(cudaMemcpyAsync(live.data(), d_live.p, 2 * M * sizeof(std::uint32_t), cudaMemcpyDeviceToHost, stream), "count read");
                check(cudaStreamSynchronize(stream), "count read");
                check_status("between chunks");
            }
            for (std::size_t m = 0; m < M; ++m) {
                Engine& E = *engines[m];
                E.ensure_capacity(static_cast<std::uint64_t>(live[2 * m]) + live[2 * m + 1] + (born[m][s_to] - born[m][s_from]) + 1024,
                                  live[2 * m], live[2 * m + 1], static_cast<int>(c0 % 2), 32, true, stream);
                for (std::size_t w = c0; w < c1; ++w) {
                    StepParams P = base[m];
                    const auto tw = static_cast<std::uint32_t>(std::min<std::uint64_t>(fused, steps - starts[w]));
                    if (E.window_steps(starts[w], tw, E.impl_->capacity) != tw) {
                        throw std::length_error("too many phonons in one step for 32-bit work indices");
                    }
                    E.window_params(P, w, starts[w], tw);
                    params[(w - c0) * M + m] = P;
                }
            }
            check(cudaMemcpyAsync(d_params.p, params.data(), (c1 - c0) * M * sizeof(StepParams), cudaMemcpyHostToDevice, stream),
                  "batch parameters");
            for (std::size_t w = c0; w < c1; ++w) {
                B.params = d_params.as<StepParams>() + (w - c0) * M;
                launch_batch_f32(B, grid, smem, stream);
                launches += 2;
            }
            check(cudaGetLastError(), "batched launch");
            // the parameter buffer is rewritten for the next chunk: its launches must have read it
            if (c1 < starts.size()) { check(cudaStreamSynchronize(stream), "batch chunk"); }
        }
        for (Engine* E : engines) {
            Impl& I = *E->impl_;
            launch_population_max(I.population.as<std::uint32_t>(), static_cast<std::uint32_t>(steps), I.counters.as<unsigned long long>(),
                                  stream);
        }
        check(cudaEventRecord(ev1, stream), "event record");
        check(cudaStreamSynchronize(stream), "batch sync");
        check(cudaEventElapsedTime(&ms, ev0, ev1), "event time");
        check_status("at the end");
    } catch (...) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        throw;
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    // each run's counters; the batch's device time split by phonon-steps
    std::vector<unsigned long long> st(M, 0ULL);
    unsigned long long all = 0;
    for (std::size_t m = 0; m < M; ++m) {
        check(cudaMemcpy(&st[m], engines[m]->impl_->counters.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost), "counters");
        all += st[m];
    }
    for (std::size_t m = 0; m < M; ++m) {
        const double share = all > 0 ? static_cast<double>(st[m]) / static_cast<double>(all) : 1. / static_cast<double>(M);
        engines[m]->steps_run_ = steps;
        engines[m]->last_stage_mask_ = 7U;
        engines[m]->finish_run(ms * share, launches + 1, starts.size(), fused);
    }
    return true;
}

void Engine::set_steady_stop(bool on, const SteadyCriterion& c, std::uint64_t check_every) {
    if (on) { validate_steady(c); }
    stop_on_ = on;
    stop_crit_ = c;
    stop_check_ = check_every;
}

void Engine::reset() {
    Impl& I = *impl_;
    check(cudaMemset(I.tally.p, 0, I.tally.bytes), "memset tally");
    counters_ = RunCounters{};
    I.builders_ready = false;
    I.total = 0;
}

namespace {
// The first K recorded steps of the tallies, [K][S] records -> energy[S][K], flux[S][K][2].
void unpack(const Engine& eng, Buf& e, Buf& f, cudaStream_t stream, const void* tally, std::uint64_t K) {
    const SimDesc& d = eng.desc();
    if (K > d.recorded) { throw std::invalid_argument("more steps asked for than recorded"); }
    const std::uint64_t SK = static_cast<std::uint64_t>(d.n_sensors) * K;
    if (e.bytes < SK * sizeof(long long) || e.p == nullptr) { e.alloc(SK * sizeof(long long)); }
    if (f.bytes < SK * 2 * sizeof(double) || f.p == nullptr) { f.alloc(SK * 2 * sizeof(double)); }
    if (SK > 0) {
        const int blocks = static_cast<int>(std::min<std::uint64_t>((SK + 255) / 256, 8192));
        unpack_kernel<<<blocks, 256, 0, stream>>>(static_cast<const TallySlot*>(tally), d.n_sensors, K, e.as<long long>(),
                                                 f.as<double>());
        check(cudaGetLastError(), "unpack kernel");
    }
}
}// namespace

void Engine::population(std::uint32_t* out) const {
    Impl& I = *impl_;
    check(cudaMemcpy(out, I.population.p, desc_.steps * sizeof(std::uint32_t), cudaMemcpyDeviceToHost), "copy population");
    counters_.d2h_bytes += desc_.steps * sizeof(std::uint32_t);
}

void Engine::tallies(std::int64_t* energy, double* flux, std::uint64_t K) const {
    Impl& I = *impl_;
    K = std::min<std::uint64_t>(K, desc_.recorded);
    unpack(*this, I.unpacked_energy, I.unpacked_flux, I.own, I.tally.p, K);
    const std::uint64_t SK = static_cast<std::uint64_t>(desc_.n_sensors) * K;
    if (energy != nullptr) {
        check(cudaMemcpyAsync(energy, I.unpacked_energy.p, SK * sizeof(long long), cudaMemcpyDeviceToHost, I.own), "copy energy");
        counters_.d2h_bytes += SK * sizeof(long long);
    }
    if (flux != nullptr) {
        check(cudaMemcpyAsync(flux, I.unpacked_flux.p, SK * 2 * sizeof(double), cudaMemcpyDeviceToHost, I.own), "copy flux");
        counters_.d2h_bytes += SK * 2 * sizeof(double);
    }
    check(cudaStreamSynchronize(I.own), "tallies sync");
}

void Engine::interpret(const InterpDesc& d, double* temps, double* fluxes, double* stats) const {
    Impl& I = *impl_;
    unpack(*this, I.unpacked_energy, I.unpacked_flux, I.own, I.tally.p, d.recorded);
    interpret_device(d, I.unpacked_energy.as<long long>(), I.unpacked_flux.as<double>(), temps, fluxes, stats, I.own,
                     I.interp);
    const std::uint64_t SK = static_cast<std::uint64_t>(d.n_sensors) * d.recorded;
    counters_.h2d_bytes += (d.area.size() + d.heat_capacity.size() + d.init_temp.size() + d.temps.size() + d.energies.size()) * sizeof(double)
                           + d.material.size() * 4 + d.mat_temp_begin.size() * 8;
    counters_.d2h_bytes += (temps != nullptr ? SK * 8 : 0) + (fluxes != nullptr ? SK * 16 : 0) + (stats != nullptr ? d.n_sensors * 48ULL : 0);
}

long long Engine::steady_onset(const SteadyCriterion& c, long long* per_sensor) const {
    Impl& I = *impl_;
    const long long onset = steady_onset_device(I.tally.p, desc_.n_sensors, std::min<std::uint64_t>(desc_.recorded, steps_run_), c,
                                                per_sensor, I.own);
    counters_.d2h_bytes += desc_.n_sensors * 8ULL;
    return onset;
}

void Engine::final_temps(const InterpDesc& d, std::uint64_t start, double* out) const {
    Impl& I = *impl_;
    unpack(*this, I.unpacked_energy, I.unpacked_flux, I.own, I.tally.p, d.recorded);
    final_temps_device(d, I.unpacked_energy.as<long long>(), start, out, I.own, I.interp);
    counters_.h2d_bytes += (d.area.size() + d.heat_capacity.size() + d.init_temp.size() + d.temps.size() + d.energies.size()) * sizeof(double)
                           + d.material.size() * 4 + d.mat_temp_begin.size() * 8;
    counters_.d2h_bytes += d.n_sensors * 8ULL;
}

}// namespace psim::gpu
