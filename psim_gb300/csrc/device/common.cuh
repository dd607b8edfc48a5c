// Device-side data layout shared by the phonon transport kernels.
//
// Phonon state lives in HBM as structure-of-arrays records read and written with
// 128-bit accesses:
//   FP32 kernel: two 16-byte words per phonon (32 B)
//     pos_dir  = float4 {px, py, dx, dy}    position relative to the cell's first vertex (nm),
//                                            direction (|d| <= 1, the 2-D projection of a 3-D unit vector)
//     meta     = uint4  {cell|flags, bin|jitter, tts bits, id}
//   FP64 kernel: four 16-byte words per phonon (64 B)
//     pos = double2 {px, py} (global nm), dir = double2 {dx, dy}, tw = double2 {tts, omega},
//     meta = uint4 {cell|flags, bin, pad, id}
// Every random number comes from Philox4x32-10 keyed by the run seed with the
// counter (draw block, step, phonon id, stream tag), so a phonon's trajectory does
// not depend on where it sits in the buffer or which thread runs it.
#pragma once

#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

namespace psim::gpu {

constexpr int kBins = 1000;
constexpr int kAliasCols = 2048;             // 2 * kBins outcomes (bin, polarization) padded to 2^11
constexpr std::uint32_t kNoEdge = 3U;
constexpr int kMaxCollisions = 100;          // ModelSimulator MAX_COLLISIONS (psim/src/modelSimulator.cpp:25)
constexpr unsigned kMaxEventsPerStep = 1U << 16; // hard bound on one phonon's events in one step
constexpr float kFluxScale = 1048576.0f;     // flux tallies are fixed point: 2^20 units per m/s
constexpr double kFluxScaleInv = 1.0 / 1048576.0;

// ---------------------------------------------------------------- meta word 0 (FP32 and FP64)
//   bits  0..23 cell index, 24..25 entry edge (3 = none), 26 TA polarization, 27 negative sign,
//   28 phasor phonon (fixed velocity 1000 m/s, frequency 1 rad/s)
__host__ __device__ __forceinline__ std::uint32_t meta_cell(std::uint32_t w) { return w & 0xFFFFFFU; }
__host__ __device__ __forceinline__ std::uint32_t meta_edge(std::uint32_t w) { return (w >> 24) & 3U; }
__host__ __device__ __forceinline__ int meta_pol(std::uint32_t w) { return static_cast<int>((w >> 26) & 1U); }
__host__ __device__ __forceinline__ int meta_sign(std::uint32_t w) { return ((w >> 27) & 1U) ? -1 : 1; }
__host__ __device__ __forceinline__ bool meta_phasor(std::uint32_t w) { return ((w >> 28) & 1U) != 0U; }
__host__ __device__ __forceinline__ std::uint32_t make_meta(std::uint32_t cell, std::uint32_t edge, int pol, int sign,
                                                            bool phasor) {
    return (cell & 0xFFFFFFU) | ((edge & 3U) << 24) | (static_cast<std::uint32_t>(pol & 1) << 26)
           | ((sign < 0 ? 1U : 0U) << 27) | ((phasor ? 1U : 0U) << 28);
}
__host__ __device__ __forceinline__ std::uint32_t meta_with_cell_edge(std::uint32_t w, std::uint32_t cell,
                                                                      std::uint32_t edge) {
    return (w & ~0x3FFFFFFU) | (cell & 0xFFFFFFU) | ((edge & 3U) << 24);
}
__host__ __device__ __forceinline__ std::uint32_t meta_with_pol(std::uint32_t w, int pol) {
    return (w & ~(1U << 26)) | (static_cast<std::uint32_t>(pol & 1) << 26);
}
// meta word 1: bits 0..9 frequency bin, 10..13 material whose dispersion the bin refers to
// (the material the phonon was last sampled in; it keeps its frequency and velocity when it
// crosses into another material), 14..31 position of the frequency inside the bin (18 bits, FP32)
__host__ __device__ __forceinline__ std::uint32_t bin_of(std::uint32_t w) { return w & 0x3FFU; }
__host__ __device__ __forceinline__ std::uint32_t smat_of(std::uint32_t w) { return (w >> 10) & 0xFU; }
__host__ __device__ __forceinline__ std::uint32_t jitter_of(std::uint32_t w) { return w >> 14; }
__host__ __device__ __forceinline__ std::uint32_t make_binw(std::uint32_t bin, std::uint32_t smat, std::uint32_t jit) {
    return (bin & 0x3FFU) | ((smat & 0xFU) << 10) | (jit << 14);
}
constexpr std::uint32_t kMaxMaterials = 16;

// ---------------------------------------------------------------- Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11).
struct U4 {
    std::uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, std::uint32_t k0, std::uint32_t k1) {
    constexpr std::uint32_t M0 = 0xD2511F53U;
    constexpr std::uint32_t M1 = 0xCD9E8D57U;
    constexpr std::uint32_t W0 = 0x9E3779B9U;
    constexpr std::uint32_t W1 = 0xBB67AE85U;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const std::uint32_t lo0 = M0 * c.x;
        const std::uint32_t hi0 = __umulhi(M0, c.x);
        const std::uint32_t lo1 = M1 * c.z;
        const std::uint32_t hi1 = __umulhi(M1, c.z);
        c = U4{ hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0 };
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// One Philox block for (block, step, id) of a stream.  Not inlined: the transport kernels draw at
// a dozen places, and one shared copy of the rounds keeps their code small.
static __device__ __noinline__ U4 philox_block(std::uint32_t block, std::uint32_t step, std::uint32_t id, std::uint32_t k0,
                                               std::uint32_t k1) {
    return philox4x32_10(U4{ block, step, id, 0x7073696DU }, k0, k1);
}

// Per-phonon stream for one step: four 32-bit words per Philox call, refilled on demand.  The
// words shift through registers (no indexed array, so nothing spills to local memory).
struct Stream {
    std::uint32_t k0, k1;
    std::uint32_t step, id;
    std::uint32_t block;
    std::uint32_t b0, b1, b2, b3;
    int left;

    __device__ __forceinline__ void init(std::uint32_t key0, std::uint32_t key1, std::uint32_t s, std::uint32_t pid) {
        k0 = key0;
        k1 = key1;
        step = s;
        id = pid;
        block = 0;
        left = 0;
    }
    // Compute the next block of four words now (used where many lanes start a step together).
    __device__ __forceinline__ void prefill() {
        const U4 r = philox_block(block, step, id, k0, k1);
        b0 = r.x;
        b1 = r.y;
        b2 = r.z;
        b3 = r.w;
        ++block;
        left = 4;
    }
    __device__ __forceinline__ std::uint32_t next() {
        if (left == 0) {
            const U4 r = philox_block(block, step, id, k0, k1);
            b0 = r.x;
            b1 = r.y;
            b2 = r.z;
            b3 = r.w;
            ++block;
            left = 4;
        }
        const std::uint32_t out = b0;
        b0 = b1;
        b1 = b2;
        b2 = b3;
        --left;
        return out;
    }
    // Uniform in the open interval (0, 1), 24-bit resolution.
    __device__ __forceinline__ float uf() { return (static_cast<float>(next() >> 8) + 0.5f) * 5.9604644775390625e-8f; }
    // The same draw at 32-bit resolution in double: (x + 0.5) / 2^32.
    __device__ __forceinline__ double ud() { return (static_cast<double>(next()) + 0.5) * 2.3283064365386963e-10; }
};

// ---------------------------------------------------------------- device model
// FP32 cell record, 128 bytes (one cache line).  Local frame: origin at the cell's first
// vertex.  For edge e (vertices e -> e+1): outward unit normal (nx, ny) and offset h, so a
// point p is inside the edge's half-plane when nx*px + ny*py < h.
// 112 bytes = 28 words: successive records start 4 banks apart, so the lanes of a warp reading
// the same field of different cells from shared memory spread over 8 bank groups (a 128-byte
// record would put every cell's field in the same banks).
struct alignas(16) CellF32 {
    float4 edge[3];      // nx, ny, h; w: the edge's link as int bits (>= 0 neighbour cell, -1 boundary,
                         // <= -2 emitter -(link+2))
    float2 v1, v2;       // local vertices 1 and 2 (vertex 0 is the origin)
    float2 offset[3];    // add to a local position when crossing edge e into the neighbour
    std::uint32_t rev;   // neighbour's entry edge per edge (2 bits each); bit 8+e: flip backscatter normal
    std::uint32_t sensor;
    float spec;
    std::uint32_t material;
};
static_assert(sizeof(CellF32) == 112, "CellF32 is 112 bytes (28 words)");
__host__ __device__ __forceinline__ int edge_link(const float4& e) {
    int v;
    std::memcpy(&v, &e.w, sizeof v);
    return v;
}

// FP64 cell record: the three edge lines in the reference's Line form and the triangle.
struct Line64 {
    double ax, ay, bx, by;// end points
    double m, c;          // slope, intercept
    double lox, loy, hix, hiy;
};
struct CellF64 {
    Line64 edge[3];
    double vx[3], vy[3];  // triangle vertices (global)
    double nx[3], ny[3];  // inward (reference) normal per edge
    std::uint32_t sub_begin[4];
    std::uint32_t sensor;
    std::uint32_t material;
    double spec;
};
// One sub-surface of an edge (transition or emitting surface), reference order.
struct Sub64 {
    Line64 line;
    double nx, ny;     // normal of the sub-surface (used for a transition backscatter)
    int kind;          // 0 transition, 1 emit
    std::uint32_t target;
};

struct SensorDev {
    float T3, T4, xk;          // T^3, T^4 and hbar*1e13/(k*T): FP32 rate factors
    std::uint32_t material;
    double T;                  // temperature for the FP64 rates
    std::uint32_t base_table;  // alias table index, cell-origin phonons
    std::uint32_t scatter_table;
};

struct MaterialDev {
    // FP32 rate coefficients with frequencies in units of 1e13 rad/s
    float cL, cTN, cTU, cI, w_cut;        // b_l*1e26, b_tn*1e13, b_tu*1e26, b_i*1e52, w/1e13
    float width;                          // bin width / 1e13
    float w_max_la, w_max_ta;             // / 1e13
    // FP64 originals
    double b_l, b_tn, b_tu, b_i, w, width64, w_max_la64, w_max_ta64;
};

struct EmitterDev {
    float2 a, b;            // local end points in the owning cell's frame (FP32 kernel)
    double ax, ay, bx, by;  // global end points (FP64 kernel)
    float nx, ny;           // inward normal (FP32)
    double nx64, ny64;
    std::uint32_t cell, edge;
    std::uint32_t table;    // emit alias table
    int sign;               // +1 if hotter than t_eq
    std::uint32_t absorb_lo, absorb_hi; // steps s with s*dt >= start and s*dt + dt <= start + duration
    double spec;
    double pad;
};
// Records staged into shared memory by 1-D bulk copies: sizes must be multiples of 16 bytes.
static_assert(sizeof(SensorDev) % 16 == 0, "SensorDev size");
static_assert(sizeof(MaterialDev) % 16 == 0, "MaterialDev size");
static_assert(sizeof(EmitterDev) % 16 == 0, "EmitterDev size");

// A group of phonons born in one step: all from one cell (step 0) or one emitter.
struct BirthGroup {
    std::uint32_t first;     // index of the group's first phonon among the step's newborns
    std::int32_t source;     // >= 0 cell, < 0 emitter -(source+1)
    float t0, span;          // birth time window inside the step (ns from the step start)
    double t0_64, span64;
    int sign;                // phonon sign: +1 when the source is hotter than t_eq
    std::uint32_t pad;
};

// Tally slot for (recorded step, sensor): count of phonon signs and fixed-point flux sums.
struct alignas(8) TallySlot {
    long long count;
    long long fx;
    long long fy;
};

// Measurement steps one FP32 launch may cover (the shared-memory tally holds one slot per step).
constexpr std::uint32_t kMaxFused = 16;

struct StepParams {
    // model
    const CellF32* cells32;
    const CellF64* cells64;
    const Sub64* subs64;
    const SensorDev* sensors;
    const MaterialDev* materials;
    const EmitterDev* emitters;
    const std::uint32_t* alias;       // [tables][kAliasCols]: threshold (21 bits) << 11 | alias column
    const float* centre32;            // [materials][kBins] bin centres / 1e13
    const float* vel32;               // [materials][2][kBins] m/s
    const double* centre64;           // [materials][kBins] rad/s
    const double* vel64;              // [materials][2][kBins]
    std::uint32_t n_sensors;
    // births of this step
    const BirthGroup* groups;
    std::uint32_t group_begin, group_end;
    std::uint32_t n_new;
    std::uint32_t id_base;
    // FP32 launches cover steps [step, step + n_fused).  Work items are the survivors entering
    // 'step', then the newborns of each covered step j at [new_begin[j], new_begin[j+1]) after
    // them, with ids from id_base_f[j] and birth groups [group_begin_f[j], group_begin_f[j+1]).
    std::uint32_t n_fused;
    // Plain step boundaries (no edge impact and no scattering before the boundary) are crossed in
    // a warp-uniform loop while at least this many lanes of the warp can cross one (0: never)
    std::uint32_t coast_lanes;
    // A warp takes new work items once at least this many of its lanes are free (1: as soon as
    // one is), so that the start of new phonons runs on more lanes at once
    std::uint32_t fetch_lanes;
    // Work items a warp takes from the work counter at a time into a pool of its own (0: as many as
    // it has free lanes)
    std::uint32_t pool;
    // 1: the loop tail issues the output counter's atomic before the tallies and the next step's
    // set-up and reads it after them
    std::uint32_t tail_order;
    std::uint32_t new_begin[kMaxFused + 1];
    std::uint32_t id_base_f[kMaxFused];
    std::uint32_t group_begin_f[kMaxFused + 1];
    // state buffers
    const void* in;
    void* out;
    std::uint32_t capacity;
    const std::uint32_t* count_in;
    std::uint32_t* count_out;
    std::uint32_t* count_clear;
    // FP32 survivors may be written in two groups: the front group from slot 0 up (count_*), the
    // back group from slot capacity - 1 down (back_*), by the key sort_mode picks (0: front only;
    // 1: back when the time to the next scattering event is below sort_after ns; 2: back when
    // the group velocity is at least sort_after m/s), so that the next launch hands its lanes
    // runs of phonons alike.  Work item i < *count_in is slot i, the others are the back group.
    const std::uint32_t* back_in;
    std::uint32_t* back_out;
    std::uint32_t* back_clear;
    std::uint32_t sort_mode;
    float sort_after;
    std::uint32_t* work;              // this step's work counter (phonons handed to lanes)
    std::uint32_t* work_clear;        // the counter of two steps ahead, cleared by this step
    std::uint32_t* population;        // [n_steps] phonons in flight per step (FP32: accumulated, zeroed per run)
    // Shared-memory staging of read-only tables (FP32 kernel): bit 0 cells, 1 alias tables,
    // 2 velocities + bin centres; byte offsets of each staged segment and of the tallies.
    std::uint32_t stage_mask;
    std::uint32_t off_cells, off_alias, off_vel, off_centre, off_tally;
    std::uint32_t off_sensors, off_materials, off_emitters, n_emitters;
    std::uint32_t n_cells, n_tables, n_materials;
    // step
    std::uint32_t step;               // 0-based (first) step; phonons alive at its end reach boundary step+1
    std::uint32_t n_steps;
    std::uint32_t step_adj;           // first tallied boundary
    std::uint32_t n_recorded;
    float dt;                         // ns
    double dt64;
    int phasor_sim;
    int full_sim;
    std::uint32_t key0, key1;
    TallySlot* tally;                 // [n_recorded][n_sensors]
    unsigned long long* counters;     // [0] phonon-steps, [1] collision-limit relocations, [2] overflow,
                                      // [3] max population, [4] event-limit hits, [5] staging timeouts,
                                      // [6] backscatters at interfaces between materials
};

// One launch of the batched FP32 kernel: the same window of measurement steps for every model of
// a batch.  params[m] is model m's StepParams for this launch (its tables, buffers, counters and
// births, and the shared-memory layout of its staged tables).  The plan kernel cuts each model's
// work items (survivors, then newborns) into runs of 'chunk' items and numbers them: model m owns
// items [item_begin[m], item_begin[m + 1]).  Each block of the batch kernel takes the next item
// from item_next, stages its model's tables when they are not the ones it holds, and runs it.
struct BatchLaunch {
    const StepParams* params;
    std::uint32_t* item_begin;   // [n_models + 1], written by the plan kernel
    std::uint32_t* item_next;    // items handed out, cleared by the plan kernel
    // [0] abort (1: a table staging timed out, 2: a model's event-limit hits ran past
    // kBatchEventLimitAbort), [1] staging timeouts, [2] work items run, [3] stagings; once set, the
    // abort ends every later item and launch at once and the host reports it
    std::uint32_t* status;
    std::uint32_t n_models;
    std::uint32_t chunk;
};
constexpr unsigned long long kBatchEventLimitAbort = 4096;

}// namespace psim::gpu
