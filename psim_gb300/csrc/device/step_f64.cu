// FP64 phonon transport with the reference's geometry: the step loop of
// ModelSimulator::simulatePhonon / handleImpacts / nextImpact
// (psim/src/modelSimulator.cpp:87-225) in FP64 with global coordinates, segment
// intersections by the reference's slope-intercept routine (geom64.hpp) and the
// reference's surface lookup.  It draws the same Philox stream as the FP32 kernel and
// is the precision reference for it.  Compiled with -fmad=false so the geometry
// rounds exactly as the reference's does.
#include "../host/geom64.hpp"
#include "transport.cuh"

namespace psim::gpu {
namespace {

constexpr double kVelocityEps = 0.01;// VELOCITY_EPS (psim/src/modelSimulator.cpp:23)
constexpr double kHbar64 = 1.054517e-34;// psim/src/material.cpp:13-14
constexpr double kBoltz64 = 1.38065e-23;

struct Ph64 {
    double px, py, dx, dy, tts, w;
    std::uint32_t meta, binw, id;
};

__device__ __forceinline__ psim::Seg64 seg_of(const Line64& l) {
    psim::Seg64 s;
    s.a = psim::P2{ l.ax, l.ay };
    s.b = psim::P2{ l.bx, l.by };
    s.m = l.m;
    s.c = l.c;
    s.lo = psim::P2{ l.lox, l.loy };
    s.hi = psim::P2{ l.hix, l.hiy };
    return s;
}

__device__ __forceinline__ double vel64(const StepParams& P, const Ph64& p) {
    if (meta_phasor(p.meta)) { return 1000.; }
    return P.vel64[(smat_of(p.binw) * 2U + static_cast<std::uint32_t>(meta_pol(p.meta))) * kBins + bin_of(p.binw)];
}

// x^3 and x^4 rounded once, as a correctly rounded pow(x, 3.) / pow(x, 4.) returns them: the
// products are carried exactly as unevaluated sums of two doubles (Dekker's product, with the
// low part from an FMA) and rounded at the end.
__device__ __forceinline__ double cube64(double x) {
    const double s = x * x;
    const double se = fma(x, x, -s);     // x^2 = s + se exactly
    const double c = s * x;
    const double ce = fma(s, x, -c);     // s x = c + ce exactly
    return c + fma(se, x, ce);
}
__device__ __forceinline__ double quartic64(double x) {
    const double s = x * x;
    const double se = fma(x, x, -s);
    const double q = s * s;
    const double qe = fma(s, s, -q);     // s^2 = q + qe exactly
    return q + fma(2. * s, se, qe);      // x^4 = q + qe + 2 s se + se^2 (se^2 is below the rounding)
}

// Material rates in FP64 (Material::relaxRates, psim/src/material.cpp:54-62,207-239).
__device__ __forceinline__ void rates64(const MaterialDev& m, double T, double f, int pol, double r[3]) {
    if (pol == 0) {
        r[0] = m.b_l * f * f * cube64(T);
        r[1] = r[0];
    } else {
        r[0] = (f < m.w) ? m.b_tn * f * quartic64(T) : 0.;
        r[1] = (f >= m.w) ? m.b_tu * f * f / sinh(kHbar64 * f / (T * kBoltz64)) : 0.;
    }
    r[2] = m.b_i * quartic64(f);
}

__device__ __forceinline__ void iso_dir(Ph64& p, Stream& rs) {
    p.dx = 2. * rs.ud() - 1.;
    p.dy = sqrt(1. - p.dx * p.dx) * cos(2. * psim::kPi * rs.ud());
}

__device__ __forceinline__ void diffuse_dir(Ph64& p, Stream& rs, double nx, double ny) {
    const double u = rs.ud();
    const double a = sqrt(u);
    const double b = sqrt(1. - u) * cos(2. * psim::kPi * rs.ud());
    p.dx = nx * a - ny * b;
    p.dy = ny * a + nx * b;
}

// Surface::boundaryHandlePhonon (psim/src/surface.cpp:32-44); (nx, ny) is the inward normal.
__device__ __forceinline__ void reflect(Ph64& p, Stream& rs, double spec, double nx, double ny) {
    if (spec >= 1. || (spec > 0. && rs.ud() < spec)) {// a draw only when the choice is random (as the FP32 kernel)
        const double ndx = -p.dx * nx - p.dy * ny;
        const double ndy = -p.dx * ny + p.dy * nx;
        p.dx = nx * ndx - ny * ndy;
        p.dy = ny * ndx + nx * ndy;
    } else {
        diffuse_dir(p, rs, nx, ny);
    }
}

__device__ __forceinline__ void sample_freq(const StepParams& P, Ph64& p, Stream& rs, std::uint32_t table,
                                            std::uint32_t mat) {
    const std::uint32_t o = alias_draw(P.alias + static_cast<std::size_t>(table) * kAliasCols, rs.next());
    const std::uint32_t bin = o >> 1;
    p.binw = make_binw(bin, mat, 0U);
    p.meta = meta_with_pol(p.meta, static_cast<int>(o & 1U));
    const double c = P.centre64[mat * kBins + bin];
    p.w = P.full_sim ? c : c + (2. * rs.ud() - 1.) * P.materials[mat].width64 / 2.;
}

__device__ double spawn64(const StepParams& P, Ph64& p, Stream& rs, std::uint32_t j) {
    const BirthGroup g = P.groups[find_group(P, P.group_begin, P.group_end, j)];
    p.id = P.id_base + j;
    rs.init(P.key0, P.key1, P.step, p.id);
    p.tts = 0.;
    if (g.source >= 0) {
        const std::uint32_t cell = static_cast<std::uint32_t>(g.source);
        const CellF64& c = P.cells64[cell];
        p.meta = make_meta(cell, kNoEdge, 0, g.sign, false);
        sample_freq(P, p, rs, P.sensors[c.sensor].base_table, c.material);
        const double r1 = rs.ud();
        const double r2 = rs.ud();
        const psim::P2 q = psim::tri_point(psim::P2{ c.vx[0], c.vy[0] }, psim::P2{ c.vx[1], c.vy[1] },
                                           psim::P2{ c.vx[2], c.vy[2] }, r1, r2);
        p.px = q.x;
        p.py = q.y;
        iso_dir(p, rs);
        return P.dt64;
    }
    const EmitterDev& e = P.emitters[static_cast<std::uint32_t>(-(g.source + 1))];
    const double t_birth = g.t0_64 + g.span64 * rs.ud();
    const bool phasor = P.phasor_sim != 0;
    p.meta = make_meta(e.cell, e.edge, 0, g.sign, phasor);
    sample_freq(P, p, rs, e.table, P.cells64[e.cell].material);
    const double r = rs.ud();
    p.px = e.ax * r + e.bx * (1. - r);
    p.py = e.ay * r + e.by * (1. - r);
    if (phasor) {
        p.binw = make_binw(1U, smat_of(p.binw), 0U);
        p.meta = meta_with_pol(p.meta, 0);
        p.w = 1.;
        p.dx = e.nx64;
        p.dy = e.ny64;
    } else {
        diffuse_dir(p, rs, e.nx64, e.ny64);
    }
    const double rem = P.dt64 - t_birth;
    return rem > 0. ? rem : 0.;
}

// Cell::handleSurfaceCollision -> CompositeSurface::handlePhonon (psim/src/cell.cpp:103-108,
// psim/src/compositeSurface.cpp:47-66).  Returns false when the phonon is absorbed.
__device__ bool collide64(const StepParams& P, Ph64& p, Stream& rs, psim::P2 poi) {
    const std::uint32_t cell = meta_cell(p.meta);
    const CellF64& c = P.cells64[cell];
    for (int e = 0; e < 3; ++e) {
        if (!psim::on_line(seg_of(c.edge[e]), poi)) { continue; }
        for (std::uint32_t k = c.sub_begin[e]; k < c.sub_begin[e + 1]; ++k) {
            const Sub64& s = P.subs64[k];
            if (s.kind != 0 || !psim::on_line(seg_of(s.line), poi)) { continue; }
            const CellF64& n = P.cells64[s.target];// TransitionSurface::handlePhonon (psim/src/surface.cpp:71-109)
            if (n.material == c.material) {
                p.meta = meta_with_cell_edge(p.meta, s.target, kNoEdge);
            } else {
                const MaterialDev& mt = P.materials[n.material];
                const double max_freq = (meta_pol(p.meta) == 0) ? mt.w_max_la64 : mt.w_max_ta64;
                if (p.w > max_freq) {
                    atomicAdd(P.counters + 6, 1ULL);
                    diffuse_dir(p, rs, s.nx, s.ny);
                } else {
                    p.meta = meta_with_cell_edge(p.meta, s.target, kNoEdge);
                }
            }
            return true;
        }
        for (std::uint32_t k = c.sub_begin[e]; k < c.sub_begin[e + 1]; ++k) {
            const Sub64& s = P.subs64[k];
            if (s.kind != 1 || !psim::on_line(seg_of(s.line), poi)) { continue; }
            const EmitterDev& em = P.emitters[s.target];// EmitSurface::handlePhonon (psim/src/surface.cpp:61-65)
            if (P.step >= em.absorb_lo && P.step <= em.absorb_hi) { return false; }
            reflect(p, rs, c.spec, c.nx[e], c.ny[e]);
            return true;
        }
        reflect(p, rs, c.spec, c.nx[e], c.ny[e]);
        return true;
    }
    return true;
}

// ModelSimulator::nextImpact (psim/src/modelSimulator.cpp:87-122).  Returns 0 for no impact,
// 1 for an impact (time in *t), 2 when the impact absorbed the phonon.
__device__ int next_impact64(const StepParams& P, Ph64& p, Stream& rs, double time, double* t) {
    const double v = vel64(P, p);
    const double vx = p.dx * v;
    const double vy = p.dy * v;
    const psim::P2 start{ p.px, p.py };
    const psim::P2 end{ p.px + time * vx, p.py + time * vy };
    if (psim::coincide(start, end)) { return 0; }
    const psim::Seg64 path = psim::make_seg(start, end, nullptr);
    const CellF64& c = P.cells64[meta_cell(p.meta)];
    bool hit = false;
    psim::P2 best{ 0., 0. };
    for (int e = 0; e < 3; ++e) {
        psim::P2 poi;
        if (psim::intersection(seg_of(c.edge[e]), path, &poi) && !psim::coincide(poi, start)) {
            const double tx = (vx > kVelocityEps || vx < -kVelocityEps) ? (poi.x - start.x) / vx : time;
            const double ty = (vy > kVelocityEps || vy < -kVelocityEps) ? (poi.y - start.y) / vy : time;
            const double ti = (tx <= ty) ? tx : ty;
            if (ti <= time) {
                time = ti;
                best = poi;
                hit = true;
            }
        }
    }
    if (!hit) { return 0; }
    p.px = best.x;
    p.py = best.y;
    *t = time;
    return collide64(P, p, rs, best) ? 1 : 2;
}

struct Outcome {
    bool alive;
    bool boundary;
    bool tallied;
    std::uint32_t sensor;
    long long fx, fy;
};

__device__ Outcome transport64(const StepParams& P, Ph64& p, Stream& rs, double ttm, unsigned long long& relocations,
                               unsigned long long& limits) {
    Outcome out{ false, false, false, 0U, 0, 0 };
    unsigned events = 0;
    while (true) {
        if (++events > kMaxEventsPerStep) {// numerical corner case: end the step where the phonon is
            ++limits;
            ttm = 0.;
            if (p.tts < 0.) { p.tts = 0.; }
        }
        const std::uint32_t cell = meta_cell(p.meta);
        const CellF64& c = P.cells64[cell];
        const std::uint32_t sensor = c.sensor;
        if (p.tts <= 0.) {
            double r[3];
            rates64(P.materials[c.material], P.sensors[sensor].T, p.w, meta_pol(p.meta), r);
            p.tts = 1e9 * -log(rs.ud()) / (((0. + r[0]) + r[1]) + r[2]);
        }
        double drift = (ttm < p.tts) ? ttm : p.tts;
        // handleImpacts (psim/src/modelSimulator.cpp:205-225)
        double drifted = 0.;
        double it = 0.;
        int res = next_impact64(P, p, rs, drift, &it);
        int ncoll = 0;
        while (res != 0) {
            if (res == 2) { return out; }// absorbed by an emitting surface
            drifted += it;
            if (++ncoll > kMaxCollisions) {
                const CellF64& cc = P.cells64[meta_cell(p.meta)];
                const double r1 = rs.ud();
                const double r2 = rs.ud();
                const psim::P2 q = psim::tri_point(psim::P2{ cc.vx[0], cc.vy[0] }, psim::P2{ cc.vx[1], cc.vy[1] },
                                                   psim::P2{ cc.vx[2], cc.vy[2] }, r1, r2);
                p.px = q.x;
                p.py = q.y;
                drifted = drift;
                ++relocations;
                break;
            }
            if (P.cells64[meta_cell(p.meta)].sensor != sensor) { break; }
            res = next_impact64(P, p, rs, drift - drifted, &it);
        }
        const std::uint32_t now_sensor = P.cells64[meta_cell(p.meta)].sensor;
        if (now_sensor != sensor) { drift = drifted; }
        const double factor = vel64(P, p) * (drift - drifted);
        p.px += p.dx * factor;
        p.py += p.dy * factor;
        ttm -= drift;
        p.tts -= drift;
        if (ttm == 0.) {
            const std::uint32_t next = P.step + 1U;
            out.boundary = true;
            if (next >= P.n_steps) { return out; }
            out.alive = true;
            if (next >= P.step_adj && next - P.step_adj < P.n_recorded) {
                const double sign = static_cast<double>(meta_sign(p.meta));
                const double v = vel64(P, p);
                out.tallied = true;
                out.sensor = now_sensor;
                out.fx = __double2ll_rn((p.dx * v) * sign * static_cast<double>(kFluxScale));
                out.fy = __double2ll_rn((p.dy * v) * sign * static_cast<double>(kFluxScale));
            }
            return out;
        }
        if (!P.phasor_sim && p.tts == 0.) {// ModelSimulator::scatter (psim/src/modelSimulator.cpp:124-137)
            const CellF64& cc = P.cells64[meta_cell(p.meta)];
            double r[3];
            rates64(P.materials[cc.material], P.sensors[cc.sensor].T, p.w, meta_pol(p.meta), r);
            const double tau = ((0. + r[0]) + r[1]) + r[2];
            const double u = rs.ud();
            if (u <= (r[0] + r[1]) / tau) {
                sample_freq(P, p, rs, P.sensors[cc.sensor].scatter_table, cc.material);
                if (u > r[0] / tau) { iso_dir(p, rs); }
            } else if (r[2] > 0.) {
                iso_dir(p, rs);
            }
        } else {
            p.tts = 0.;
        }
    }
}

__global__ void __launch_bounds__(kBlock) step_kernel_f64(const StepParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    BlockTally bt;
    tally_init(P, bt, smem, 1U);
    const std::uint32_t n_alive = min(*P.count_in, P.capacity);// survivors beyond the buffer were dropped and counted
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *P.count_clear = 0U;
        atomicMax(P.counters + 3, static_cast<unsigned long long>(n_alive) + P.n_new);
        if (P.population != nullptr) { P.population[P.step] = n_alive + P.n_new; }
    }
    const std::uint32_t total = n_alive + P.n_new;
    const std::uint32_t slot_k = P.step + 1U >= P.step_adj ? P.step + 1U - P.step_adj : 0U;
    const double2* in_pos = static_cast<const double2*>(P.in);
    const double2* in_dir = in_pos + P.capacity;
    const double2* in_tw = in_dir + P.capacity;
    const uint4* in_meta = reinterpret_cast<const uint4*>(in_tw + P.capacity);
    double2* out_pos = static_cast<double2*>(P.out);
    double2* out_dir = out_pos + P.capacity;
    double2* out_tw = out_dir + P.capacity;
    uint4* out_meta = reinterpret_cast<uint4*>(out_tw + P.capacity);
    unsigned long long steps = 0;
    unsigned long long relocations = 0;
    unsigned long long limits = 0;
    const std::uint32_t stride = gridDim.x * blockDim.x;
    for (std::uint32_t base = blockIdx.x * blockDim.x; base < total; base += stride) {
        const std::uint32_t i = base + threadIdx.x;
        Outcome o{ false, false, false, 0U, 0, 0 };
        Ph64 p{ 0., 0., 0., 0., 0., 0., 0U, 0U, 0U };
        if (i < total) {
            Stream rs;
            double rem;
            if (i < n_alive) {
                const double2 a = in_pos[i];
                const double2 b = in_dir[i];
                const double2 c = in_tw[i];
                const uint4 d = in_meta[i];
                p = Ph64{ a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, d.w };
                rs.init(P.key0, P.key1, P.step, p.id);
                rem = P.dt64;
            } else {
                rem = spawn64(P, p, rs, i - n_alive);
            }
            o = transport64(P, p, rs, rem, relocations, limits);
            steps += o.boundary ? 1ULL : 0ULL;
        }
        const std::uint32_t slot = reserve_slot(P, o.alive);
        if (slot != 0xFFFFFFFFU) {
            out_pos[slot] = make_double2(p.px, p.py);
            out_dir[slot] = make_double2(p.dx, p.dy);
            out_tw[slot] = make_double2(p.tts, p.w);
            out_meta[slot] = make_uint4(p.meta, p.binw, 0U, p.id);
        }
        tally_add(P, bt, o.tallied, o.sensor, meta_sign(p.meta), o.fx, o.fy, slot_k);
    }
    block_count_add(P.counters + 0, steps);
    block_count_add(P.counters + 1, relocations);
    block_count_add(P.counters + 4, limits);
    tally_flush(P, bt, slot_k);
}

}// namespace

// The FP64 rates on given inputs (a known-answer check against Material::relaxRates).
__global__ void rates64_kernel(MaterialDev m, const double* T, const double* f, const int* pol, int n, double* out) {
    const int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) { return; }
    double r[3];
    rates64(m, T[i], f[i], pol[i], r);
    out[3 * i] = r[0];
    out[3 * i + 1] = r[1];
    out[3 * i + 2] = r[2];
}

void launch_rates64(const MaterialDev& m, const double* T, const double* f, const int* pol, int n, double* out, cudaStream_t stream) {
    if (n > 0) { rates64_kernel<<<(n + 255) / 256, 256, 0, stream>>>(m, T, f, pol, n, out); }
}

void launch_step_f64(const StepParams& P, int grid, std::size_t smem, cudaStream_t stream) {
    step_kernel_f64<<<grid, kBlock, smem, stream>>>(P);
}

int occupancy_f64(std::size_t smem) {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, step_kernel_f64, kBlock, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return blocks;
}

}// namespace psim::gpu
