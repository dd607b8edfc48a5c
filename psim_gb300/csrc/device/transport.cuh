// Pieces shared by the FP32 and FP64 transport kernels: alias sampling, births,
// warp-aggregated tallies and stream compaction.
#pragma once

#include "common.cuh"

namespace psim::gpu {

constexpr int kBlock = 256;
constexpr int kSharedSensors = 2048;   // sensors tallied in shared memory; larger models use global atomics

// Walker alias table over the 2000 (bin, polarization) outcomes, one 32-bit word per column:
// a 21-bit acceptance threshold and an 11-bit alias column.  One 32-bit random word picks the
// column (top 11 bits) and decides acceptance (low 21 bits).
__device__ __forceinline__ std::uint32_t alias_draw(const std::uint32_t* table, std::uint32_t x) {
    const std::uint32_t col = x >> 21;
    const std::uint32_t e = table[col];
    const std::uint32_t o = ((x & 0x1FFFFFU) < (e >> 11)) ? col : (e & 0x7FFU);
    return min(o, static_cast<std::uint32_t>(2 * kBins - 1));// columns >= 2000 carry no probability
}

// Newborn j of a step -> its birth group among groups [lo, hi) of that step (sorted by 'first').
__device__ __forceinline__ std::uint32_t find_group(const StepParams& P, std::uint32_t lo, std::uint32_t hi, std::uint32_t j) {
    // invariant: groups[lo].first <= j < groups[hi].first (hi exclusive)
    while (hi - lo > 1) {
        const std::uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&P.groups[mid].first) <= j) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    return lo;
}

// Shared-memory tally of one block: one slot of S sensors per boundary the launch ends steps on
// (slot j: the boundary after step P.step + j), plus the phonons crossing each boundary alive.
// Layout from 'base': fx[n], fy[n] (8-byte aligned), count[n], cross[kMaxFused], n = slots x S.
struct BlockTally {
    unsigned char* base;
    std::uint32_t n;
    bool shared;
    __device__ __forceinline__ long long* fx() const { return reinterpret_cast<long long*>(base); }
    __device__ __forceinline__ long long* fy() const { return fx() + n; }
    __device__ __forceinline__ int* count() const { return reinterpret_cast<int*>(fy() + n); }
    __device__ __forceinline__ unsigned* cross() const { return reinterpret_cast<unsigned*>(count() + n); }
};

__device__ __forceinline__ void tally_add(const StepParams& P, BlockTally& bt, bool tallied, std::uint32_t sensor,
                                          int sign, long long fx, long long fy, std::uint32_t slot) {
    const unsigned full = 0xFFFFFFFFU;
    const int key = tallied ? static_cast<int>(sensor) : -1;
    const unsigned peers = __match_any_sync(full, key);
    if (key < 0) { return; }
    const int lane = static_cast<int>(threadIdx.x & 31U);
    const int leader = __ffs(static_cast<int>(peers)) - 1;
    const int c = __reduce_add_sync(peers, sign);
    if (bt.shared) {
        if (lane == leader) { atomicAdd(bt.count() + sensor, c); }
        atomicAdd(reinterpret_cast<unsigned long long*>(bt.fx() + sensor), static_cast<unsigned long long>(fx));
        atomicAdd(reinterpret_cast<unsigned long long*>(bt.fy() + sensor), static_cast<unsigned long long>(fy));
    } else {
        TallySlot* t = P.tally + static_cast<std::size_t>(slot) * P.n_sensors + sensor;
        if (lane == leader) { atomicAdd(reinterpret_cast<unsigned long long*>(&t->count), static_cast<unsigned long long>(static_cast<long long>(c))); }
        atomicAdd(reinterpret_cast<unsigned long long*>(&t->fx), static_cast<unsigned long long>(fx));
        atomicAdd(reinterpret_cast<unsigned long long*>(&t->fy), static_cast<unsigned long long>(fy));
    }
}

// ---------------------------------------------------------------- TMA bulk copies into shared memory
__device__ __forceinline__ std::uint32_t smem_u32(const void* p) { return static_cast<std::uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(std::uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(std::uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// One 1-D bulk copy global -> shared by the TMA engine, completing on the mbarrier.
// Both addresses must be 16-byte aligned and the size a multiple of 16.
__device__ __forceinline__ void bulk_to_shared(void* dst, const void* src, unsigned bytes, std::uint64_t* bar) {
    std::uint64_t gsrc;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(std::uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0U;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase of the staging barrier with the given parity (0 for its first use);
// false after the iteration limit or 200 ms, whichever comes first.
__device__ __forceinline__ bool mbar_wait_bounded(std::uint64_t* bar, unsigned parity = 0U) {
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0; it < (1U << 22); ++it) {
        if (mbar_try_wait(bar, parity)) { return true; }
        if ((it & 63U) == 63U && global_ns() - t0 > 200000000ULL) { return false; }
    }
    return false;
}

// The tally of an FP32 launch (one slot per covered step), rebuilt from the parameters where it
// is used so that no pointer to it stays live in registers.
__device__ __forceinline__ BlockTally window_tally(const StepParams& P, unsigned char* smem) {
    const bool shared = P.n_sensors <= static_cast<std::uint32_t>(kSharedSensors);
    return BlockTally{ smem + P.off_tally, shared ? P.n_fused * P.n_sensors : 0U, shared };
}

// FP32 launch over several steps: a phonon ending step P.step + j at its boundary.  'crossing'
// phonons go on into the next step (they count towards its population); 'tallied' ones (the
// boundary is recorded) add their sign and flux to sensor 'sensor' of slot j.  Each lane adds its
// own: at a few crossings per warp and iteration spread over the sensors, plain shared-memory
// atomics cost less than grouping the lanes first (__match_any_sync every iteration).
// 'smem' is the kernel's dynamic shared memory; the tally sits at P.off_tally in it.
__device__ __forceinline__ void window_add(const StepParams& P, unsigned char* smem, bool crossing, bool tallied, std::uint32_t j,
                                           std::uint32_t sensor, int sign, long long fx, long long fy) {
    if (!crossing) { return; }
    const BlockTally bt = window_tally(P, smem);
    if (bt.shared) {
        const std::uint32_t i = j * P.n_sensors + sensor;
        atomicAdd(bt.cross() + j, 1U);
        if (tallied) {
            atomicAdd(bt.count() + i, sign);
            atomicAdd(reinterpret_cast<unsigned long long*>(bt.fx() + i), static_cast<unsigned long long>(fx));
            atomicAdd(reinterpret_cast<unsigned long long*>(bt.fy() + i), static_cast<unsigned long long>(fy));
        }
    } else {// tallies straight to global memory; the crossings are still counted per block
        atomicAdd(bt.cross() + j, 1U);
        if (tallied) {
            TallySlot* t = P.tally + static_cast<std::size_t>(P.step + j + 1U - P.step_adj) * P.n_sensors + sensor;
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->count), static_cast<unsigned long long>(static_cast<long long>(sign)));
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->fx), static_cast<unsigned long long>(fx));
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->fy), static_cast<unsigned long long>(fy));
        }
    }
}

// Adds a block's window tally to the run's tallies (recorded boundaries only) and its crossing
// counts to the population of the steps they enter.
__device__ __forceinline__ void window_flush(const StepParams& P, unsigned char* smem) {
    const BlockTally bt = window_tally(P, smem);
    __syncthreads();
    const std::uint32_t n = bt.shared ? P.n_fused * P.n_sensors : 0U;
    for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const std::uint32_t j = i / P.n_sensors;
        const std::uint32_t s = i - j * P.n_sensors;
        const std::uint32_t boundary = P.step + j + 1U;
        if (boundary < P.step_adj || boundary - P.step_adj >= P.n_recorded) { continue; }
        const int c = bt.count()[i];
        const long long fx = bt.fx()[i];
        const long long fy = bt.fy()[i];
        if (c != 0 || fx != 0 || fy != 0) {
            TallySlot* t = P.tally + static_cast<std::size_t>(boundary - P.step_adj) * P.n_sensors + s;
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->count), static_cast<unsigned long long>(static_cast<long long>(c)));
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->fx), static_cast<unsigned long long>(fx));
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->fy), static_cast<unsigned long long>(fy));
        }
    }
    if (threadIdx.x < P.n_fused && P.step + threadIdx.x + 1U < P.n_steps && bt.cross()[threadIdx.x] != 0U) {
        atomicAdd(P.population + P.step + threadIdx.x + 1U, bt.cross()[threadIdx.x]);
    }
}

__device__ __forceinline__ void tally_flush(const StepParams& P, BlockTally& bt, std::uint32_t slot) {
    if (!bt.shared) { return; }
    __syncthreads();
    for (std::uint32_t s = threadIdx.x; s < P.n_sensors; s += blockDim.x) {
        const int c = bt.count()[s];
        const long long fx = bt.fx()[s];
        const long long fy = bt.fy()[s];
        if (c != 0 || fx != 0 || fy != 0) {
            TallySlot* t = P.tally + static_cast<std::size_t>(slot) * P.n_sensors + s;
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->count), static_cast<unsigned long long>(static_cast<long long>(c)));
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->fx), static_cast<unsigned long long>(fx));
            atomicAdd(reinterpret_cast<unsigned long long*>(&t->fy), static_cast<unsigned long long>(fy));
        }
    }
}

__device__ __forceinline__ void tally_init(const StepParams& P, BlockTally& bt, unsigned char* smem, std::uint32_t slots) {
    // layout: fx[slots*S], fy[slots*S] (8-byte aligned), count[slots*S], cross[kMaxFused] with
    // S <= kSharedSensors; cross[kMaxFused] alone for larger S (tallies in global memory)
    bt.shared = P.n_sensors <= static_cast<std::uint32_t>(kSharedSensors);
    const std::uint32_t n = bt.shared ? slots * P.n_sensors : 0U;
    bt.base = smem + P.off_tally;
    bt.n = n;
    for (std::uint32_t s = threadIdx.x; s < n; s += blockDim.x) {
        bt.fx()[s] = 0;
        bt.fy()[s] = 0;
        bt.count()[s] = 0;
    }
    if (threadIdx.x < kMaxFused) { bt.cross()[threadIdx.x] = 0U; }
    __syncthreads();
}

// Shared bytes of a block's tally with 'slots' boundary slots of S sensors, 16-aligned.  Above
// kSharedSensors sensors the tallies go straight to global memory and only the per-boundary
// crossing counts stay in shared memory.
inline std::size_t tally_smem_bytes(std::uint32_t S, std::uint32_t slots = 1) {
    if (S > static_cast<std::uint32_t>(kSharedSensors)) { return kMaxFused * 4; }
    return ((static_cast<std::size_t>(S) * slots * 20 + kMaxFused * 4 + 15) / 16) * 16;
}

// Warp-aggregated slot reservation in the output buffer, in the front group (from slot 0 up) or,
// with 'back', the back group (from the last slot down); returns the slot or UINT32_MAX.
__device__ __forceinline__ std::uint32_t reserve_slot(const StepParams& P, bool alive, bool back = false) {
    const unsigned full = 0xFFFFFFFFU;
    if (P.sort_mode == 0U) {// one group: front only
        const unsigned mask = __ballot_sync(full, alive);
        const int lane = static_cast<int>(threadIdx.x & 31U);
        std::uint32_t base = 0;
        if (lane == 0 && mask != 0U) { base = atomicAdd(P.count_out, static_cast<std::uint32_t>(__popc(mask))); }
        base = __shfl_sync(full, base, 0);
        if (!alive) { return 0xFFFFFFFFU; }
        const std::uint32_t slot = base + static_cast<std::uint32_t>(__popc(mask & ((1U << lane) - 1U)));
        if (slot >= P.capacity) {
            atomicAdd(P.counters + 2, 1ULL);
            return 0xFFFFFFFFU;
        }
        return slot;
    }
    const unsigned front_mask = __ballot_sync(full, alive && !back);
    const unsigned back_mask = __ballot_sync(full, alive && back);
    const int lane = static_cast<int>(threadIdx.x & 31U);
    std::uint32_t base = 0;
    std::uint32_t base_back = 0;
    if (lane == 0) {
        if (front_mask != 0U) { base = atomicAdd(P.count_out, static_cast<std::uint32_t>(__popc(front_mask))); }
        if (back_mask != 0U) { base_back = atomicAdd(P.back_out, static_cast<std::uint32_t>(__popc(back_mask))); }
    }
    base = __shfl_sync(full, base, 0);
    base_back = __shfl_sync(full, base_back, 0);
    if (!alive) { return 0xFFFFFFFFU; }
    const unsigned below = (1U << lane) - 1U;
    const std::uint32_t idx = back ? base_back + static_cast<std::uint32_t>(__popc(back_mask & below))
                                   : base + static_cast<std::uint32_t>(__popc(front_mask & below));
    if (idx >= P.capacity) {
        atomicAdd(P.counters + 2, 1ULL);
        return 0xFFFFFFFFU;
    }
    return back ? P.capacity - 1U - idx : idx;
}

// Survivors entering a launch (both groups; beyond the buffer they were dropped and counted).
__device__ __forceinline__ std::uint32_t alive_in(const StepParams& P) { return min(*P.count_in + *P.back_in, P.capacity); }


__device__ __forceinline__ void block_count_add(unsigned long long* target, unsigned long long v) {
    const unsigned full = 0xFFFFFFFFU;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { v += __shfl_down_sync(full, v, o); }
    if ((threadIdx.x & 31U) == 0U && v != 0ULL) { atomicAdd(target, v); }
}

}// namespace psim::gpu
