// FP32 cell-local phonon transport: one launch advances every phonon across up to kMaxFused
// measurement steps (ModelSimulator::simulatePhonon, psim/src/modelSimulator.cpp:139-198,
// reorganised step by step instead of phonon by phonon).
//
// Per phonon: load 32 B of state (or create the phonon in the step it is born in), run events
// until a step boundary or absorption, and tally at the boundary.  A phonon that crosses a
// boundary inside the launch's steps goes on in registers, with the next step's random
// stream; one that crosses the launch's last boundary is written, 32 B, to the compacted
// output buffer.  Results do not depend on how many steps a launch covers.
//
// Geometry: positions are relative to the cell's first vertex.  The exit time through
// edge e is (h_e - n_e.p) / (n_e.w) for edges the phonon moves towards (n_e.w > 0), the
// edge it entered through excluded; for a triangle this is the first boundary the
// straight path meets, the impact the reference finds with Line::getIntersection
// (psim/src/modelSimulator.cpp:87-122).  What happens at the impact follows the
// reference: Cell::handleSurfaceCollision -> CompositeSurface::handlePhonon
// (psim/src/cell.cpp:103-108, psim/src/compositeSurface.cpp:47-66) resolves each edge
// to its first transition surface, else its first emitting surface, else the boundary.
#include <algorithm>

#include "transport.cuh"

namespace psim::gpu {
namespace {

extern __shared__ __align__(16) unsigned char g_smem[];

// Read-only tables: the shared-memory copies where the kernel's staging mask M says so, else
// global memory.  M is a compile-time copy of StepParams::stage_mask: bit 0 cell records, bits 1-2
// the alias tables with the velocity and bin-centre tables (with them the sensor, material and
// emitter records).  Each variant reads its tables with direct shared or global loads.
constexpr unsigned kStageCells = 1U;
constexpr unsigned kStageTables = 6U;
template<unsigned M> __device__ __forceinline__ const CellF32* cells_of(const StepParams& P) {
    if constexpr ((M & kStageCells) != 0U) {
        return reinterpret_cast<const CellF32*>(g_smem + P.off_cells);
    } else {
        return P.cells32;
    }
}
template<unsigned M> __device__ __forceinline__ const std::uint32_t* alias_of(const StepParams& P) {
    if constexpr ((M & kStageTables) != 0U) {
        return reinterpret_cast<const std::uint32_t*>(g_smem + P.off_alias);
    } else {
        return P.alias;
    }
}
template<unsigned M> __device__ __forceinline__ const float* vel_of(const StepParams& P) {
    if constexpr ((M & kStageTables) != 0U) {
        return reinterpret_cast<const float*>(g_smem + P.off_vel);
    } else {
        return P.vel32;
    }
}
template<unsigned M> __device__ __forceinline__ const SensorDev* sensors_of(const StepParams& P) {
    if constexpr ((M & kStageTables) != 0U) {
        return reinterpret_cast<const SensorDev*>(g_smem + P.off_sensors);
    } else {
        return P.sensors;
    }
}
template<unsigned M> __device__ __forceinline__ const MaterialDev* materials_of(const StepParams& P) {
    if constexpr ((M & kStageTables) != 0U) {
        return reinterpret_cast<const MaterialDev*>(g_smem + P.off_materials);
    } else {
        return P.materials;
    }
}
template<unsigned M> __device__ __forceinline__ const EmitterDev* emitters_of(const StepParams& P) {
    if constexpr ((M & kStageTables) != 0U) {
        return reinterpret_cast<const EmitterDev*>(g_smem + P.off_emitters);
    } else {
        return P.emitters;
    }
}
template<unsigned M> __device__ __forceinline__ const float* centre_of(const StepParams& P) {
    if constexpr ((M & kStageTables) != 0U) {
        return reinterpret_cast<const float*>(g_smem + P.off_centre);
    } else {
        return P.centre32;
    }
}

struct Ph32 {
    float px, py, dx, dy;
    std::uint32_t meta, binw;
    float tts;
    std::uint32_t id;
};

// Group velocity of the phonon's bin (Material::getVel, psim/src/material.cpp:82-84).
template<unsigned S> __device__ __forceinline__ float vel32(const StepParams& P, std::uint32_t binw, int pol, bool phasor) {
    return phasor ? 1000.f : vel_of<S>(P)[(smat_of(binw) * 2U + static_cast<std::uint32_t>(pol)) * kBins + bin_of(binw)];
}

// Frequency in units of 1e13 rad/s (Material::getFreq, psim/src/material.cpp:77-80): bin
// centre plus the stored uniform offset inside the bin in a deviational simulation.
template<unsigned S> __device__ __forceinline__ float omega32(const StepParams& P, std::uint32_t binw, bool phasor) {
    if (phasor) { return 1e-13f; }
    const std::uint32_t sm = smat_of(binw);
    const float c = centre_of<S>(P)[sm * kBins + bin_of(binw)];
    if (P.full_sim) { return c; }
    const float u = (static_cast<float>(jitter_of(binw)) + 0.5f) * (1.0f / 262144.0f);
    return c + (2.f * u - 1.f) * (materials_of<S>(P)[sm].width * 0.5f);
}

// Relaxation rates [N, U, I] (Material::tauNInv/tauUInv/tauIInv, psim/src/material.cpp:207-239),
// frequency w in 1e13 rad/s, coefficients pre-scaled so every factor stays in FP32 range.
__device__ __forceinline__ float3 rates32(const MaterialDev& m, const SensorDev& s, float w, int pol) {
    const float w2 = w * w;
    float n;
    float u;
    if (pol == 0) {
        n = m.cL * w2 * s.T3;
        u = n;
    } else {
        n = (w < m.w_cut) ? m.cTN * w * s.T4 : 0.f;
        if (w >= m.w_cut) {// 1 / sinh(x) = 2 e^-x / (1 - e^-2x) with x = hbar w / kT > 0: no overflow at any T
            const float em = __expf(-w * s.xk);
            u = __fdividef(2.f * m.cTU * w2 * em, 1.f - em * em);// cTU w^2 / sinh(x)
        } else {
            u = 0.f;
        }
    }
    return make_float3(n, u, m.cI * w2 * w2);
}

// Phonon::setRandDirection (psim/src/phonon.cpp:28-31): dx = 2u-1, dy = sqrt(1-dx^2) cos(2 pi u').
__device__ __forceinline__ void iso_dir(Ph32& p, Stream& rs) {
    const float dx = 2.f * rs.uf() - 1.f;
    p.dx = dx;
    p.dy = sqrtf(fmaxf(0.f, 1.f - dx * dx)) * __cosf(6.2831853071795865f * rs.uf());
}

// Surface::redirectPhonon (psim/src/surface.cpp:23-30): Lambertian about the inward normal n.
__device__ __forceinline__ void diffuse_dir(Ph32& p, Stream& rs, float nx, float ny) {
    const float u = rs.uf();
    const float a = sqrtf(u);
    const float b = sqrtf(1.f - u) * __cosf(6.2831853071795865f * rs.uf());
    p.dx = nx * a - ny * b;
    p.dy = ny * a + nx * b;
}

// Surface::boundaryHandlePhonon (psim/src/surface.cpp:32-44): specular with probability spec.
__device__ __forceinline__ void reflect(Ph32& p, Stream& rs, float spec, float4 e) {
    if (spec >= 1.f || (spec > 0.f && rs.uf() < spec)) {
        const float dn = p.dx * e.x + p.dy * e.y;
        p.dx -= 2.f * dn * e.x;
        p.dy -= 2.f * dn * e.y;
    } else {
        diffuse_dir(p, rs, -e.x, -e.y);
    }
}

// Material::freqIndex + getFreq (psim/src/material.cpp:64-80) from an alias table of the
// material 'mat'.
template<unsigned S> __device__ __forceinline__ void sample_freq(const StepParams& P, Ph32& p, Stream& rs, std::uint32_t table,
                                            std::uint32_t mat) {
    const std::uint32_t o = alias_draw(alias_of<S>(P) + static_cast<std::size_t>(table) * kAliasCols, rs.next());
    const std::uint32_t jit = P.full_sim ? 0U : (rs.next() >> 14);
    p.binw = make_binw(o >> 1, mat, jit);
    p.meta = meta_with_pol(p.meta, static_cast<int>(o & 1U));
}

// Create newborn j of the launch's step jf (CellOriginBuilder / SurfaceOriginBuilder /
// PhasorBuilder, psim/src/phononBuilder.cpp:6-49).  Returns the time left until the step boundary.
template<unsigned S> __device__ __forceinline__ float spawn32(const StepParams& P, Ph32& p, Stream& rs, std::uint32_t jf,
                                                          std::uint32_t j) {
    const BirthGroup g = P.groups[find_group(P, P.group_begin_f[jf], P.group_begin_f[jf + 1], j)];
    p.id = P.id_base_f[jf] + j;
    rs.init(P.key0, P.key1, P.step + jf, p.id);
    p.tts = 0.f;
    if (g.source >= 0) {
        const std::uint32_t cell = static_cast<std::uint32_t>(g.source);
        const CellF32& c = cells_of<S>(P)[cell];
        p.meta = make_meta(cell, kNoEdge, 0, g.sign, false);
        sample_freq<S>(P, p, rs, sensors_of<S>(P)[c.sensor].base_table, c.material);
        float r1 = rs.uf();
        float r2 = rs.uf();
        if (r1 + r2 > 1.f) {
            r1 = 1.f - r1;
            r2 = 1.f - r2;
        }
        p.px = c.v1.x * r1 + c.v2.x * r2;
        p.py = c.v1.y * r1 + c.v2.y * r2;
        iso_dir(p, rs);
        return P.dt;
    }
    const EmitterDev& e = emitters_of<S>(P)[static_cast<std::uint32_t>(-(g.source + 1))];
    const float t_birth = g.t0 + g.span * rs.uf();
    const bool phasor = P.phasor_sim != 0;
    p.meta = make_meta(e.cell, e.edge, 0, g.sign, phasor);
    sample_freq<S>(P, p, rs, e.table, cells_of<S>(P)[e.cell].material);
    const float r = rs.uf();
    p.px = e.a.x * r + e.b.x * (1.f - r);
    p.py = e.a.y * r + e.b.y * (1.f - r);
    if (phasor) {
        p.binw = make_binw(1U, smat_of(p.binw), 0U);
        p.meta = meta_with_pol(p.meta, 0);
        p.dx = e.nx;
        p.dy = e.ny;
    } else {
        diffuse_dir(p, rs, e.nx, e.ny);
    }
    return fmaxf(P.dt - t_birth, 0.f);
}

// A phonon in flight on one lane: its state, its random stream and where it is inside the
// current event (the drift to the next scattering event or step boundary, with the edge
// impacts on the way).
struct Lane {
    Ph32 p;
    Stream rs;
    float rem;      // time left until the step boundary (ns)
    float target;   // length of the current event's drift (ns)
    float drifted;  // part of it already covered by impacts
    float v;        // group velocity (m/s = nm/ns)
    std::uint32_t sensor, mat;
    int ncoll;      // impacts in the current event (MAX_COLLISIONS rule)
    unsigned events;
    float fN, fNU;  // N/sum and (N+U)/sum of the rates of the last scattering-time draw
    bool need_target, changed, rates_ok;
    // the measurement step the phonon is in: the step its random stream is keyed by
    __device__ __forceinline__ std::uint32_t step() const { return rs.step; }
};

struct Outcome {
    bool alive;
    bool boundary;// reached the step boundary (a phonon-step), alive or at the last boundary
    bool cont;    // alive, and the next step is one of this launch's
    bool tallied;
    std::uint32_t sensor;
    long long fx, fy;
};

// The lane's phonon enters 'step' at its start: that step's random stream, a full step of time.
// The same state is what a later launch would read back from the output buffer.  The rates of
// its last scattering-time draw stay valid (the scattering event uses the draw's rates,
// modelSimulator.cpp:148-153 and 186-187, and a run's sensor parameters do not change between
// steps); a phonon read back from the buffer recomputes them (lane_start).
__device__ __forceinline__ void lane_enter_step(const StepParams& P, Lane& L, std::uint32_t step) {
    L.rs.init(P.key0, P.key1, step, L.p.id);
    L.rem = P.dt;
    // A phonon that scatters or draws a new scattering time in this step needs random words:
    // make them here, where most lanes of the warp start a step together.
    if (L.p.tts < L.rem) { L.rs.prefill(); }
    L.need_target = true;
    L.events = 0;
}

template<unsigned S>
__device__ __forceinline__ void lane_start(const StepParams& P, Lane& L, std::uint32_t i, std::uint32_t n_alive, std::uint32_t n_front) {
    if (i < n_alive) {
        const float4* in_pd = static_cast<const float4*>(P.in);
        const std::uint32_t slot = i < n_front ? i : P.capacity - 1U - (i - n_front);// front group, then the back group
        const float4 a = in_pd[slot];
        const uint4 b = reinterpret_cast<const uint4*>(in_pd + P.capacity)[slot];
        L.p = Ph32{ a.x, a.y, a.z, a.w, b.x, b.y, __uint_as_float(b.z), b.w };
        lane_enter_step(P, L, P.step);
        L.rates_ok = false;
    } else {
        const std::uint32_t k = i - n_alive;
        std::uint32_t jf = 0;
        while (jf + 1U < P.n_fused && k >= P.new_begin[jf + 1U]) { ++jf; }
        L.rem = spawn32<S>(P, L.p, L.rs, jf, k - P.new_begin[jf]);// keys the stream by step P.step + jf
        L.need_target = true;
        L.rates_ok = false;
        L.events = 0;
    }
    const CellF32* C = cells_of<S>(P) + meta_cell(L.p.meta);
    L.sensor = C->sensor;
    L.mat = C->material;
    L.v = vel32<S>(P, L.p.binw, meta_pol(L.p.meta), meta_phasor(L.p.meta));
}

// Earliest exit of the straight path p + w t from cell C through an edge other than 'entry':
// the edge (or -1) and its time.
__device__ __forceinline__ void next_exit(const CellF32* C, const Ph32& p, float wx, float wy, std::uint32_t entry, float& tbest,
                                          int& ebest) {
    tbest = 3.0e38f;
    ebest = -1;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const float4 E = C->edge[e];
        const float den = E.x * wx + E.y * wy;
        if (static_cast<std::uint32_t>(e) != entry && den > 0.f) {
            const float t = fmaxf(__fdividef(E.z - (E.x * p.px + E.y * p.py), den), 0.f);
            if (t < tbest) {
                tbest = t;
                ebest = e;
            }
        }
    }
}

// The lane's phonon enters 'step' at its start without computing random words ahead (a
// coasting lane crosses boundaries at its own pace; the words are made where it next draws).
__device__ __forceinline__ void lane_enter_step_lazy(const StepParams& P, Lane& L, std::uint32_t step) {
    L.rs.init(P.key0, P.key1, step, L.p.id);
    L.rem = P.dt;
    L.need_target = true;
    L.events = 0;
}

// The phonon has reached its step's boundary: the outcome (alive into the next step or not,
// tallied or not).  Returns true (the step is over).
__device__ __forceinline__ bool boundary_outcome(const StepParams& P, const Lane& L, Outcome& out) {
    const std::uint32_t next = L.step() + 1U;
    out = Outcome{ false, true, false, false, 0U, 0, 0 };
    if (next >= P.n_steps) { return true; }
    out.alive = true;
    out.cont = next < P.step + P.n_fused;
    if (next >= P.step_adj && next - P.step_adj < P.n_recorded) {
        const float sv = static_cast<float>(meta_sign(L.p.meta)) * L.v;
        out.tallied = true;
        out.sensor = L.sensor;
        out.fx = __float2ll_rn(sv * L.p.dx * kFluxScale);
        out.fy = __float2ll_rn(sv * L.p.dy * kFluxScale);
    }
    return true;
}

// One plain step boundary, if the phonon's next segment is one: its current event ends at the
// step boundary (no scattering first) and its straight path meets no edge before it.  Then the
// phonon drifts to the boundary exactly as segment32 would move it, and the outcome is the
// boundary's; returns false (state unchanged but for the event set-up segment32 would do
// first) when the next segment holds an impact, a scattering event or a new scattering time.
template<unsigned S> __device__ __forceinline__ bool coast32(const StepParams& P, Lane& L, Outcome& out) {
    Ph32& p = L.p;
    if (L.need_target) {
        if (p.tts <= 0.f || L.events + 1U > kMaxEventsPerStep) { return false; }
        ++L.events;
        L.target = (L.rem <= p.tts) ? L.rem : p.tts;
        L.drifted = 0.f;
        L.ncoll = 0;
        L.changed = false;
        L.need_target = false;
    }
    if (L.target != L.rem) { return false; }
    const CellF32* C = cells_of<S>(P) + meta_cell(p.meta);
    const float wx = p.dx * L.v;
    const float wy = p.dy * L.v;
    float tbest;
    int ebest;
    next_exit(C, p, wx, wy, meta_edge(p.meta), tbest, ebest);
    const float left = L.target - L.drifted;
    if (!(ebest < 0 || tbest > left)) { return false; }
    p.px += wx * left;
    p.py += wy * left;
    L.drifted = L.target;
    const float used = L.target;
    L.rem -= used;
    p.tts -= used;
    L.need_target = true;
    return boundary_outcome(P, L, out);
}

// One segment of a phonon's step: the straight flight to the next edge impact or to the end of
// the current event (ModelSimulator::simulatePhonon / handleImpacts / nextImpact,
// psim/src/modelSimulator.cpp:87-225).  Returns true when the phonon's step is over (it
// reached the step boundary or was absorbed); the outcome says which.
// The rare event-limit and collision-limit hits go straight to their global counters.
template<unsigned S> __device__ __forceinline__ bool segment32(const StepParams& P, Lane& L, Outcome& out) {
    Ph32& p = L.p;
    Stream& rs = L.rs;
    const bool phasor = meta_phasor(p.meta);
    if (L.need_target) {
        if (++L.events > kMaxEventsPerStep) {// numerical corner case: end the step where the phonon is
            atomicAdd(P.counters + 4, 1ULL);
            L.rem = 0.f;
            p.tts = fmaxf(p.tts, 0.f);
        }
        if (p.tts <= 0.f) {// time to the next scattering event (modelSimulator.cpp:148-153)
            const float3 r = rates32(materials_of<S>(P)[L.mat], sensors_of<S>(P)[L.sensor], omega32<S>(P, p.binw, phasor), meta_pol(p.meta));
            const float inv = __frcp_rn(r.x + r.y + r.z);
            p.tts = 1e9f * (-__logf(rs.uf())) * inv;
            L.fN = r.x * inv;
            L.fNU = (r.x + r.y) * inv;
            L.rates_ok = true;
        }
        L.target = (L.rem <= p.tts) ? L.rem : p.tts;
        L.drifted = 0.f;
        L.ncoll = 0;
        L.changed = false;
        L.need_target = false;
    }
    std::uint32_t cell = meta_cell(p.meta);
    const CellF32* C = cells_of<S>(P) + cell;
    const float wx = p.dx * L.v;
    const float wy = p.dy * L.v;
    float tbest;
    int ebest;
    next_exit(C, p, wx, wy, meta_edge(p.meta), tbest, ebest);
    const float left = L.target - L.drifted;
    bool event_over = true;
    if (ebest < 0 || tbest > left) {
        p.px += wx * left;
        p.py += wy * left;
        L.drifted = L.target;
    } else {
        p.px += wx * tbest;
        p.py += wy * tbest;
        L.drifted += tbest;
        const float4 E = C->edge[ebest];
        const int link = edge_link(E);
        std::uint32_t entry_next = static_cast<std::uint32_t>(ebest);
        if (link >= 0) {// TransitionSurface::handlePhonon (psim/src/surface.cpp:71-109)
            const CellF32* N = cells_of<S>(P) + link;
            bool pass = true;
            if (N->material != L.mat) {
                const MaterialDev& mt = materials_of<S>(P)[N->material];
                const float w = omega32<S>(P, p.binw, phasor);
                pass = !(w > (meta_pol(p.meta) == 0 ? mt.w_max_la : mt.w_max_ta));
            }
            if (pass) {
                p.px += C->offset[ebest].x;
                p.py += C->offset[ebest].y;
                entry_next = (C->rev >> (2 * ebest)) & 3U;
                cell = static_cast<std::uint32_t>(link);
                C = N;
                if (C->sensor != L.sensor) {
                    L.sensor = C->sensor;
                    L.changed = true;
                }
                L.mat = C->material;
            } else {// backscatter: no state of this frequency in the neighbour's material
                atomicAdd(P.counters + 6, 1ULL);
                const float flip = ((C->rev >> (8 + ebest)) & 1U) ? -1.f : 1.f;
                diffuse_dir(p, rs, -E.x * flip, -E.y * flip);
            }
        } else if (link == -1) {
            reflect(p, rs, C->spec, E);
        } else {// EmitSurface::handlePhonon (psim/src/surface.cpp:61-65)
            const EmitterDev& em = emitters_of<S>(P)[static_cast<std::uint32_t>(-(link + 2))];
            if (L.step() >= em.absorb_lo && L.step() <= em.absorb_hi) {
                out = Outcome{ false, false, false, false, 0U, 0, 0 };
                return true;// absorbed
            }
            reflect(p, rs, C->spec, E);
        }
        p.meta = meta_with_cell_edge(p.meta, cell, entry_next);
        if (++L.ncoll > kMaxCollisions) {// stuck in a corner: random point in the cell
            float r1 = rs.uf();
            float r2 = rs.uf();
            if (r1 + r2 > 1.f) {
                r1 = 1.f - r1;
                r2 = 1.f - r2;
            }
            p.px = C->v1.x * r1 + C->v2.x * r2;
            p.py = C->v1.y * r1 + C->v2.y * r2;
            p.meta = meta_with_cell_edge(p.meta, cell, kNoEdge);
            L.drifted = L.target;
            atomicAdd(P.counters + 1, 1ULL);
        } else {
            event_over = L.changed;
        }
    }
    if (!event_over) { return false; }
    // The event: measurement boundary, scattering, or a new sensor area (modelSimulator.cpp:178-193)
    const float used = L.changed ? L.drifted : L.target;
    L.rem -= used;
    p.tts -= used;
    L.need_target = true;
    if (L.rem == 0.f) {
        // a new sensor area reached exactly at the boundary: its scattering rates are recomputed
        // at the next event, as they are after a launch boundary
        if (L.changed) { L.rates_ok = false; }
        return boundary_outcome(P, L, out);
    }
    if (!P.phasor_sim && p.tts == 0.f) {// ModelSimulator::scatter (modelSimulator.cpp:124-137)
        if (!L.rates_ok) {// the scattering time was drawn before this launch: recompute its rates
            const float3 r = rates32(materials_of<S>(P)[L.mat], sensors_of<S>(P)[L.sensor], omega32<S>(P, p.binw, phasor), meta_pol(p.meta));
            const float inv = __frcp_rn(r.x + r.y + r.z);
            L.fN = r.x * inv;
            L.fNU = (r.x + r.y) * inv;
        }
        const float u = rs.uf();
        const bool resample = u <= L.fNU;                          // normal or Umklapp
        const bool redirect = resample ? (u > L.fN) : (L.fNU < 1.f);// Umklapp, or impurity (positive rate)
        if (resample) {// new frequency, velocity and polarization
            sample_freq<S>(P, p, rs, sensors_of<S>(P)[L.sensor].scatter_table, L.mat);
            L.v = vel32<S>(P, p.binw, meta_pol(p.meta), phasor);
        }
        if (redirect) {// new direction
            iso_dir(p, rs);
            p.meta = meta_with_cell_edge(p.meta, cell, kNoEdge);
        }
        L.rates_ok = false;
    } else {
        p.tts = 0.f;// new sensor area (or phasor): draw a fresh scattering time
    }
    return false;
}

// Persistent lanes over the work items [first, total) of one model's launch (survivors entering
// the launch's first step below n_alive, then the steps' newborns): each lane takes the next item
// from 'fetch' (a warp-aggregated counter: fetch(k) hands out k consecutive items and returns the
// first) and advances it one segment per iteration.  A phonon that crosses a boundary into another
// of the launch's steps stays in its lane; one that leaves the launch (or dies) frees the lane for
// the next item, so the warp stays full until the items run out instead of waiting for its
// slowest phonon.  Returns the phonon-steps of this thread.
template<unsigned S, bool kCoast, typename Fetch>
__device__ __forceinline__ std::uint32_t lanes_run(const StepParams& P, std::uint32_t n_alive, std::uint32_t n_front, std::uint32_t total,
                                                   Fetch fetch) {
    const unsigned full = 0xFFFFFFFFU;
    std::uint32_t steps = 0;// phonon-steps of this thread (a launch gives each thread far fewer than 2^32)
    bool active = false;
    bool exhausted = false;// warp-uniform: the step's work counter has run out
    // With P.pool > 0 the warp takes runs of P.pool items from the counter into a pool of its own
    // [pool_lo, pool_hi) (warp-uniform) and hands them to its free lanes from there; each new run's
    // state records are prefetched into L2 when the run is taken, ahead of the lanes that start them.
    std::uint32_t pool_lo = 0;
    std::uint32_t pool_hi = 0;
    bool drained = false;// warp-uniform: the counter has handed out its last run
    Lane L;
    L.p = Ph32{ 0.f, 0.f, 0.f, 0.f, 0U, 0U, 0.f, 0U };
    while (true) {
        if (!exhausted) {
            const unsigned need = __ballot_sync(full, !active);
            if (need != 0U && (static_cast<std::uint32_t>(__popc(need)) >= P.fetch_lanes || need == full)) {
                const int lane = static_cast<int>(threadIdx.x & 31U);
                const int leader = __ffs(static_cast<int>(need)) - 1;
                const auto want = static_cast<std::uint32_t>(__popc(need));
                std::uint32_t base = 0;
                std::uint32_t avail = 0;
                if (P.pool == 0U) {
                    if (lane == leader) { base = fetch(want); }
                    base = __shfl_sync(full, base, leader);
                    if (base + want >= total) { exhausted = true; }
                    avail = base < total ? min(want, total - base) : 0U;
                } else {
                    if (pool_lo == pool_hi && !drained) {
                        std::uint32_t run = 0;
                        if (lane == leader) { run = fetch(P.pool); }
                        run = __shfl_sync(full, run, leader);
                        pool_lo = min(run, total);
                        pool_hi = min(run + P.pool, total);
                        drained = run + P.pool >= total;
                        const std::uint32_t k = pool_lo + static_cast<std::uint32_t>(lane);
                        if (k < pool_hi && k < n_alive) {// survivors' records: bring them into L2 now
                            const std::uint32_t slot = k < n_front ? k : P.capacity - 1U - (k - n_front);
                            const float4* in_pd = static_cast<const float4*>(P.in);
                            asm volatile("prefetch.global.L2 [%0];" ::"l"(in_pd + slot));
                            asm volatile("prefetch.global.L2 [%0];" ::"l"(in_pd + P.capacity + slot));
                        }
                    }
                    base = pool_lo;
                    avail = min(want, pool_hi - pool_lo);
                    pool_lo += avail;
                    if (drained && pool_lo == pool_hi) { exhausted = true; }
                }
                if (!active) {
                    const std::uint32_t rank = static_cast<std::uint32_t>(__popc(need & ((1U << lane) - 1U)));
                    if (rank < avail) {
                        lane_start<S>(P, L, base + rank, n_alive, n_front);
                        active = true;
                    }
                }
            }
        }
        if (__ballot_sync(full, active) == 0U) { break; }
        Outcome o{ false, false, false, false, 0U, 0, 0 };
        bool done = false;
        // Plain boundaries first, in a loop the warp runs while enough of its lanes cross one: a
        // phonon on its way into the launch's next step stays here, so the segment below is
        // mostly the phonon's next event (an impact, a scattering event, a new scattering time).
        if (kCoast) {
            bool coasting = active;
            while (true) {
                Outcome c{ false, false, false, false, 0U, 0, 0 };
                const bool crossed = coasting && coast32<S>(P, L, c);
                if (static_cast<std::uint32_t>(__popc(__ballot_sync(full, crossed))) < P.coast_lanes) {
                    if (crossed) {// the warp stops here: this boundary goes to the common path below
                        o = c;
                        done = true;
                    }
                    break;
                }
                if (!crossed) {
                    coasting = false;
                } else if (c.alive && c.cont) {
                    steps += 1U;
                    window_add(P, g_smem, true, c.tallied, L.step() - P.step, c.sensor, meta_sign(L.p.meta), c.fx, c.fy);
                    lane_enter_step_lazy(P, L, L.step() + 1U);
                } else {// the launch's last boundary or the run's end: the common path below finishes it
                    o = c;
                    done = true;
                    coasting = false;
                }
            }
        }
        if (active && !done) {
            // after a coasting loop most segments here draw: make their words together
            if (kCoast && L.rs.left == 0) { L.rs.prefill(); }
            done = segment32<S>(P, L, o);
        }
        const bool finishing = active && done;
        const bool crossing = finishing && o.alive;// into step L.step + 1
        const bool stays = crossing && o.cont;
        steps += (finishing && o.boundary) ? 1U : 0U;
        const bool leaving = crossing && !stays;
        if (P.tail_order != 0U && P.sort_mode == 0U) {
            // the output counter's atomic first; the tallies and the next step's set-up, which do
            // not need its result, run while it is in flight; then the slot and the store
            const unsigned out_mask = __ballot_sync(full, leaving);
            const int lane = static_cast<int>(threadIdx.x & 31U);
            std::uint32_t out_base = 0;
            if (lane == 0 && out_mask != 0U) { out_base = atomicAdd(P.count_out, static_cast<std::uint32_t>(__popc(out_mask))); }
            window_add(P, g_smem, crossing, o.tallied, L.step() - P.step, o.sensor, meta_sign(L.p.meta), o.fx, o.fy);
            if (stays) { lane_enter_step(P, L, L.step() + 1U); }
            out_base = __shfl_sync(full, out_base, 0);
            if (leaving) {
                const std::uint32_t slot = out_base + static_cast<std::uint32_t>(__popc(out_mask & ((1U << lane) - 1U)));
                if (slot < P.capacity) {
                    float4* out_pd = static_cast<float4*>(P.out);
                    out_pd[slot] = make_float4(L.p.px, L.p.py, L.p.dx, L.p.dy);
                    reinterpret_cast<uint4*>(out_pd + P.capacity)[slot] = make_uint4(L.p.meta, L.p.binw, __float_as_uint(L.p.tts), L.p.id);
                } else {
                    atomicAdd(P.counters + 2, 1ULL);
                }
            }
            if (finishing && !stays) { active = false; }
            continue;
        }
        const bool back = P.sort_mode == 1U ? L.p.tts < P.sort_after : (P.sort_mode == 2U && L.v >= P.sort_after);
        const std::uint32_t slot = reserve_slot(P, leaving, back);
        if (slot != 0xFFFFFFFFU) {// records: float4 {px, py, dx, dy}[capacity], then uint4 {meta, binw, tts, id}[capacity]
            float4* out_pd = static_cast<float4*>(P.out);
            out_pd[slot] = make_float4(L.p.px, L.p.py, L.p.dx, L.p.dy);
            reinterpret_cast<uint4*>(out_pd + P.capacity)[slot] = make_uint4(L.p.meta, L.p.binw, __float_as_uint(L.p.tts), L.p.id);
        }
        window_add(P, g_smem, crossing, o.tallied, L.step() - P.step, o.sensor, meta_sign(L.p.meta), o.fx, o.fy);
        if (stays) {
            lane_enter_step(P, L, L.step() + 1U);
        } else if (finishing) {
            active = false;
        }
    }
    return steps;
}

// Issues the TMA bulk copies of one model's read-only tables into the block's shared memory
// (the layout in P's offsets), completing on 'bar' (one thread).
template<unsigned S> __device__ __forceinline__ void stage_tables(const StepParams& P, std::uint64_t* bar) {
    const unsigned cells_b = (S & kStageCells) ? P.n_cells * static_cast<unsigned>(sizeof(CellF32)) : 0U;
    const unsigned alias_b = P.n_tables * kAliasCols * 4U;
    const unsigned vel_b = P.n_materials * 2U * kBins * 4U;
    const unsigned centre_b = P.n_materials * kBins * 4U;
    const unsigned sens_b = P.n_sensors * static_cast<unsigned>(sizeof(SensorDev));
    const unsigned mat_b = P.n_materials * static_cast<unsigned>(sizeof(MaterialDev));
    const unsigned emit_b = P.n_emitters * static_cast<unsigned>(sizeof(EmitterDev));
    mbar_expect_tx(bar, cells_b + alias_b + vel_b + centre_b + sens_b + mat_b + emit_b);
    bulk_to_shared(g_smem + P.off_sensors, P.sensors, sens_b, bar);
    bulk_to_shared(g_smem + P.off_materials, P.materials, mat_b, bar);
    if (emit_b != 0U) { bulk_to_shared(g_smem + P.off_emitters, P.emitters, emit_b, bar); }
    if (cells_b != 0U) { bulk_to_shared(g_smem + P.off_cells, P.cells32, cells_b, bar); }
    bulk_to_shared(g_smem + P.off_alias, P.alias, alias_b, bar);
    bulk_to_shared(g_smem + P.off_vel, P.vel32, vel_b, bar);
    bulk_to_shared(g_smem + P.off_centre, P.centre32, centre_b, bar);
}

// One model's launch: the blocks stage the model's tables, then their lanes share the launch's
// work items through one global counter (lanes_run).  P is a __grid_constant__ so the per-step
// arrays in it are read in place with a runtime index.
template<unsigned S, bool kCoast> __global__ void __launch_bounds__(1024, 1) step_kernel_f32(const __grid_constant__ StepParams P) {
    __shared__ std::uint64_t stage_bar;
    if constexpr (S != 0U) {// TMA bulk copies of the read-only tables into shared memory
        if (threadIdx.x == 0) { mbar_init(&stage_bar, 1U); }
        __syncthreads();
        if (threadIdx.x == 0) { stage_tables<S>(P, &stage_bar); }
    }
    BlockTally bt;
    tally_init(P, bt, g_smem, P.n_fused);
    if constexpr (S != 0U) {
        const bool ok = mbar_wait_bounded(&stage_bar);
        if (__syncthreads_or(!ok)) {// the copy did not complete: leave this step's work to other blocks
            if (threadIdx.x == 0) { atomicAdd(P.counters + 5, 1ULL); }
            mbar_wait_bounded(&stage_bar);
            return;
        }
    }
    const std::uint32_t n_alive = alive_in(P);
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) {
            *P.count_clear = 0U;
            *P.back_clear = 0U;
            *P.work_clear = 0U;
            const std::uint32_t both = *P.count_in + *P.back_in;
            if (both > P.capacity) { atomicAdd(P.counters + 2, static_cast<unsigned long long>(both - P.capacity)); }
        }
        // each step's population: its newborns here, the phonons crossing into it in window_add
        if (threadIdx.x < P.n_fused) {
            atomicAdd(P.population + P.step + threadIdx.x, P.new_begin[threadIdx.x + 1U] - P.new_begin[threadIdx.x]);
        }
    }
    const std::uint32_t total = n_alive + P.new_begin[P.n_fused];
    const std::uint32_t steps =
        lanes_run<S, kCoast>(P, n_alive, min(*P.count_in, n_alive), total, [&](std::uint32_t k) { return atomicAdd(P.work, k); });
    block_count_add(P.counters + 0, static_cast<unsigned long long>(steps));
    window_flush(P, g_smem);
}

// Numbers the work items of a batched launch (one block): model m's survivors entering the
// window plus the window's newborns, in runs of B.chunk items, at [item_begin[m], item_begin[m+1]).
// It also does for every model what block 0 of a single model's launch does: clear the counters of
// two launches ahead and add each step's newborns to its population.
__global__ void batch_plan_kernel(const __grid_constant__ BatchLaunch B) {
    for (std::uint32_t m = threadIdx.x; m < B.n_models; m += blockDim.x) {
        const StepParams& P = B.params[m];
        *P.count_clear = 0U;
        *P.back_clear = 0U;
        *P.work_clear = 0U;
        const std::uint32_t both = *P.count_in + *P.back_in;
        if (both > P.capacity) { atomicAdd(P.counters + 2, static_cast<unsigned long long>(both - P.capacity)); }
        for (std::uint32_t j = 0; j < P.n_fused; ++j) { atomicAdd(P.population + P.step + j, P.new_begin[j + 1U] - P.new_begin[j]); }
    }
    if (threadIdx.x == 0) {
        const bool abort = *B.status != 0U;// a failed launch: the rest of the run has no work
        std::uint32_t acc = 0;
        for (std::uint32_t m = 0; m < B.n_models && !abort; ++m) {
            const StepParams& P = B.params[m];
            B.item_begin[m] = acc;
            const std::uint32_t n = alive_in(P) + P.new_begin[P.n_fused];
            acc += (n + B.chunk - 1U) / B.chunk;
        }
        if (abort) {
            for (std::uint32_t m = 0; m <= B.n_models; ++m) { B.item_begin[m] = 0U; }
        }
        B.item_begin[B.n_models] = acc;
        *B.item_next = 0U;
    }
}

// The batched launch: persistent blocks take work items (a run of one model's phonons) in order.
// A block stages an item's model (its StepParams into shared memory, its tables by TMA, a cleared
// tally) when it is not the model the block holds, after flushing the previous model's tally and
// phonon-step count; its lanes then share the item's phonons through a shared-memory counter
// (lanes_run).  Results equal the model's own launches: a phonon's random stream is keyed by
// (seed, step, id), and tallies are exact integer sums.
template<unsigned S> __global__ void __launch_bounds__(1024, 1) batch_kernel_f32(const __grid_constant__ BatchLaunch B) {
    __shared__ std::uint64_t stage_bar;
    __shared__ __align__(16) StepParams sP;
    __shared__ std::uint32_t s_model, s_lo, s_hi, s_alive, s_front, s_next;
    if (threadIdx.x == 0) { mbar_init(&stage_bar, 1U); }
    __syncthreads();
    const std::uint32_t n_items = B.item_begin[B.n_models];
    constexpr std::uint32_t kNone = 0xFFFFFFFFU;
    std::uint32_t staged = kNone;
    unsigned parity = 0U;
    std::uint32_t steps = 0;
    while (true) {
        if (threadIdx.x == 0) {
            const std::uint32_t it = *reinterpret_cast<volatile std::uint32_t*>(B.status) != 0U ? n_items : atomicAdd(B.item_next, 1U);
            std::uint32_t m = kNone;
            std::uint32_t lo = 0;
            std::uint32_t hi = 0;
            std::uint32_t alive = 0;
            std::uint32_t front = 0;
            if (it < n_items) {// the model owning item 'it': the last m with item_begin[m] <= it
                std::uint32_t a = 0;
                std::uint32_t b = B.n_models;
                while (b - a > 1U) {
                    const std::uint32_t mid = (a + b) >> 1;
                    if (B.item_begin[mid] <= it) {
                        a = mid;
                    } else {
                        b = mid;
                    }
                }
                m = a;
                const StepParams& P = B.params[m];
                alive = alive_in(P);
                front = min(*P.count_in, alive);
                const std::uint32_t total = alive + P.new_begin[P.n_fused];
                lo = (it - B.item_begin[m]) * B.chunk;
                hi = min(lo + B.chunk, total);
            }
            s_model = m;
            s_lo = lo;
            s_hi = hi;
            s_alive = alive;
            s_front = front;
            s_next = 0U;
        }
        __syncthreads();
        const std::uint32_t m = s_model;
        if (m != staged) {// a new model, or no more items (m == kNone): flush the model held
            if (staged != kNone) {// the previous model's tally and phonon-steps
                block_count_add(sP.counters + 0, static_cast<unsigned long long>(steps));
                steps = 0;
                window_flush(sP, g_smem);
                __syncthreads();
            }
        }
        if (m == kNone) { break; }// also for a block that never took an item
        if (m != staged) {
            const auto* src = reinterpret_cast<const std::uint32_t*>(B.params + m);
            auto* dst = reinterpret_cast<std::uint32_t*>(&sP);
            for (std::uint32_t i = threadIdx.x; i < sizeof(StepParams) / 4U; i += blockDim.x) { dst[i] = src[i]; }
            __syncthreads();
            if (threadIdx.x == 0) { stage_tables<S>(sP, &stage_bar); }
            BlockTally bt;
            tally_init(sP, bt, g_smem, sP.n_fused);
            const bool ok = mbar_wait_bounded(&stage_bar, parity);
            parity ^= 1U;
            if (__syncthreads_or(!ok)) {// the copy did not complete: stop this block and the batch (reported)
                if (threadIdx.x == 0) {
                    atomicAdd(sP.counters + 5, 1ULL);
                    atomicAdd(B.status + 1, 1U);
                    atomicExch(B.status, 1U);
                }
                mbar_wait_bounded(&stage_bar, parity ^ 1U);
                return;
            }
            if (threadIdx.x == 0) { atomicAdd(B.status + 3, 1U); }
            staged = m;
        }
        steps += lanes_run<S, false>(sP, s_alive, s_front, s_hi, [&](std::uint32_t k) { return s_lo + atomicAdd(&s_next, k); });
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(B.status + 2, 1U);
            if (*reinterpret_cast<volatile unsigned long long*>(sP.counters + 4) > kBatchEventLimitAbort) { atomicExch(B.status, 2U); }
        }
    }
}

// The FP32 rates on given inputs (a known-answer check against Material::relaxRates).
__global__ void rates32_kernel(MaterialDev m, const SensorDev* s, const float* w, const int* pol, int n, double* out) {
    const int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) { return; }
    const float3 r = rates32(m, s[i], w[i], pol[i]);
    out[3 * i] = r.x;
    out[3 * i + 1] = r.y;
    out[3 * i + 2] = r.z;
}

}// namespace

void launch_rates32(const MaterialDev& m, const SensorDev* s, const float* w, const int* pol, int n, double* out, cudaStream_t stream) {
    if (n > 0) { rates32_kernel<<<(n + 255) / 256, 256, 0, stream>>>(m, s, w, pol, n, out); }
}

// Largest population of the run (counters[3]) from the per-step populations.
__global__ void population_max_kernel(const std::uint32_t* population, std::uint32_t n, unsigned long long* counters) {
    unsigned m = 0U;
    for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) { m = max(m, population[i]); }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { m = max(m, __shfl_down_sync(0xFFFFFFFFU, m, o)); }
    if ((threadIdx.x & 31U) == 0U && m != 0U) { atomicMax(counters + 3, static_cast<unsigned long long>(m)); }
}

void launch_population_max(const std::uint32_t* population, std::uint32_t n, unsigned long long* counters, cudaStream_t stream) {
    population_max_kernel<<<1, 1024, 0, stream>>>(population, n, counters);
}

// The kernel variant of a staging mask (0, tables only, or everything) and coasting choice.
template<bool C> const void* step_f32_fn_c(unsigned stage_mask) {
    if (stage_mask == (kStageCells | kStageTables)) { return reinterpret_cast<const void*>(step_kernel_f32<kStageCells | kStageTables, C>); }
    if (stage_mask == kStageTables) { return reinterpret_cast<const void*>(step_kernel_f32<kStageTables, C>); }
    return reinterpret_cast<const void*>(step_kernel_f32<0U, C>);
}
const void* step_f32_fn(unsigned stage_mask, bool coast) { return coast ? step_f32_fn_c<true>(stage_mask) : step_f32_fn_c<false>(stage_mask); }

template<bool C> void launch_f32_c(const StepParams& P, int grid, int block, std::size_t smem, cudaStream_t stream) {
    if (P.stage_mask == (kStageCells | kStageTables)) {
        step_kernel_f32<kStageCells | kStageTables, C><<<grid, block, smem, stream>>>(P);
    } else if (P.stage_mask == kStageTables) {
        step_kernel_f32<kStageTables, C><<<grid, block, smem, stream>>>(P);
    } else {
        step_kernel_f32<0U, C><<<grid, block, smem, stream>>>(P);
    }
}

void launch_step_f32(const StepParams& P, int grid, int block, std::size_t smem, cudaStream_t stream) {
    if (P.coast_lanes != 0U) {
        launch_f32_c<true>(P, grid, block, smem, stream);
    } else {
        launch_f32_c<false>(P, grid, block, smem, stream);
    }
}

// out[i] = *ptrs[i]: the survivor counts of a batch's models, read in one copy.
__global__ void gather_counts_kernel(const std::uint32_t* const* ptrs, std::uint32_t n, std::uint32_t* out) {
    for (std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) { out[i] = *ptrs[i]; }
}

void launch_gather_counts(const std::uint32_t* const* ptrs, std::uint32_t n, std::uint32_t* out, cudaStream_t stream) {
    if (n > 0) { gather_counts_kernel<<<(n + 255) / 256, 256, 0, stream>>>(ptrs, n, out); }
}

void launch_batch_f32(const BatchLaunch& B, int grid, std::size_t smem, cudaStream_t stream) {
    batch_plan_kernel<<<1, 1024, 0, stream>>>(B);
    batch_kernel_f32<kStageCells | kStageTables><<<grid, 1024, smem, stream>>>(B);
}

// Blocks per multiprocessor for this launch shape, 0 when it cannot launch.  The kernel's
// dynamic shared-memory limit is a process-wide attribute: it is always raised to the device's
// maximum (the same value for every caller), never to one model's need, so engines that run
// side by side on other threads cannot lower it under each other's launches.
int occupancy_of(const void* fn, int block, std::size_t smem) {
    int dev = 0;
    int optin = 0;
    cudaFuncAttributes fa{};
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess
        || cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const int max_dynamic = optin - static_cast<int>(fa.sharedSizeBytes);
    if (static_cast<long long>(smem) > max_dynamic) { return 0; }
    if (max_dynamic > 48 * 1024 && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, block, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return blocks;
}

int occupancy_batch_f32(std::size_t smem) {
    return occupancy_of(reinterpret_cast<const void*>(batch_kernel_f32<kStageCells | kStageTables>), 1024, smem);
}

// Static shared memory of the batched kernel (its StepParams copy among it).
std::size_t batch_static_smem() {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(batch_kernel_f32<kStageCells | kStageTables>)) != cudaSuccess) {
        cudaGetLastError();
        return sizeof(StepParams) + 1024;
    }
    return fa.sharedSizeBytes;
}

int occupancy_f32(unsigned stage_mask, int block, std::size_t smem) {
    return std::min(occupancy_of(step_f32_fn(stage_mask, false), block, smem), occupancy_of(step_f32_fn(stage_mask, true), block, smem));
}

}// namespace psim::gpu
