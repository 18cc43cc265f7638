// FP32 engine kernels.
//
// State per bead (sorted by cell, ascending bead id inside a cell):
//   pos = (ox, oy, oz, hash)  -- FP32 offset inside the bead's integer cell, in [0, 1)
//   vel = (vx, vy, vz, 0), frc = (fx, fy, fz, 0), cellg = global cell index, ids = bead id.
// Positions are integer cell + FP32 offset, so the resolution of a position does not depend
// on the box size: a pair separation is (o_i - o_j) - (cell_j - cell_i), an O(1) quantity.
//
// One timestep (the reference's step_impl, naive_dpd_engine_half_step.hpp:239-356):
//   update_pos -> re-bin -> pair forces -> bond forces -> update_mom.
// Here the force kernel finishes step t (pair + bond forces of x(t+1), v(t+1) = vh + f dt/2)
// and, unless it is the last step of a run, goes straight on with update_pos of step t+1 and
// counts the bead into its new cell; the counting sort (pdpd_sort.cu) then re-bins.
#include <algorithm>
#include <cmath>

#include "pdpd_device.cuh"

namespace pdpd {
namespace {

constexpr int MAX_PAIR = 256;  // n_types <= 16

struct WorldCache {
    WorldDev w;
    uint32_t world;
};

__device__ __forceinline__ void load_world(const KArgs &a, uint32_t world, WorldCache &wc,
                                           float2 *s_pair)
{
    // Block-uniform: every thread sees the same tile.
    if (wc.world != world) {
        __syncthreads();
        if (threadIdx.x == 0) {
            wc.w = a.worlds[world];
            wc.world = world;
        }
        __syncthreads();
        const uint32_t np = wc.w.n_types * wc.w.n_types;
        const float2 *pair = (const float2 *)a.pair;
        for (uint32_t i = threadIdx.x; i < np && i < MAX_PAIR; i += blockDim.x)
            s_pair[i] = pair[wc.w.param_base + i];
        __syncthreads();
    }
}

// update_pos (dpd_maths_core_half_step.hpp:22-49) in cell + offset form:
//   x' = x + v dt + f dt^2/2, wrapped into the box; returns the new global cell.
__device__ __forceinline__ uint32_t advance_position(const WorldDev &w, float dt, float hdt2,
                                                     const int c[3], float o[3], const float v[3],
                                                     const float f[3], uint32_t &err)
{
    int nc[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        float on = __fadd_rn(o[d], __fmaf_rn(f[d], hdt2, __fmul_rn(v[d], dt)));
        if (!(fabsf(on) < 1.0e6f)) {  // also catches NaN / inf
            err |= ERR_NONFINITE;
            on = 0.5f;
        }
        float fl = floorf(on);
        on -= fl;
        if (on >= 1.0f) on = 0x1.fffffep-1f;  // offset rounded up to 1: stay below it
        if (on < 0.0f) on = 0.0f;
        o[d] = on;
        nc[d] = wrap_index(c[d] + (int)fl, w.L[d]);
    }
    return w.cell_base + ((uint32_t)nc[0] * (uint32_t)w.L[1] + (uint32_t)nc[1]) * (uint32_t)w.L[2] +
           (uint32_t)nc[2];
}

// Arrival rank in the new cell with the z-half mark the sort orders by (bit 31: offset
// z >= 0.5, compared exactly in FP32).
__device__ __forceinline__ uint32_t zhalf_rank(uint32_t rank, float oz)
{
    return rank | (oz >= 0.5f ? 0x80000000u : 0u);
}

// Position of bead `slot` relative to a bead at (cell c, offset o), using the
// minimum-image integer cell difference.
__device__ __forceinline__ void rel_pos(const WorldDev &w, const float4 *__restrict__ pos,
                                        const uint32_t *__restrict__ cellg, uint32_t slot,
                                        const int c[3], const float o[3], float r[3])
{
    float4 p = pos[slot];
    int pc[3];
    decode_cell(cellg[slot] - w.cell_base, w.L, pc[0], pc[1], pc[2]);
    const float po[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        int dc = pc[d] - c[d];
        if (2 * dc > w.L[d]) dc -= w.L[d];
        if (2 * dc < -w.L[d]) dc += w.L[d];
        r[d] = (float)dc + (po[d] - o[d]);
    }
}

// calc_distance_from_to's periodic rule (naive_dpd_engine_half_step.hpp:198-209).
__device__ __forceinline__ void min_image(const WorldDev &w, float d[3])
{
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float L = (float)w.L[k];
        if (d[k] > L * 0.5f)
            d[k] -= L;
        else if (d[k] < -L * 0.5f)
            d[k] += L;
    }
}

// Bond forces on one bead from its CSR row (update_hookean_bond / update_angle_bond,
// naive_dpd_engine_half_step.hpp:426-483; calc_angle_force dpd_maths_core_half_step.hpp:177-229).
__device__ __noinline__ void bond_forces32(const KArgs &a, const WorldDev &w, uint32_t id, const int c[3],
                              const float o[3], float F[3], uint32_t &err)
{
    const float4 *pos = (const float4 *)a.posA;
    const float4 *prm_tab = (const float4 *)a.bond_params;
    const uint32_t r0 = a.bond_row[id], r1 = a.bond_row[id + 1];
    for (uint32_t r = r0; r < r1; r++) {
        const BondTerm bt = a.bond_terms[r];
        const float4 prm = prm_tab[bt.param];
        const uint32_t kind = bt.meta & 0xffu, role = bt.meta >> 8;
        float ra[3], rb[3] = {0.f, 0.f, 0.f};
        rel_pos(w, pos, a.cellg, a.slot_of_id[bt.a], c, o, ra);
        if (kind == 0) {
            // Hookean: dx = tail - head; head gets -f, tail +f, f = dx * kappa (r0 - r) / r.
            float dx[3];
#pragma unroll
            for (int d = 0; d < 3; d++) dx[d] = role == 0 ? ra[d] : -ra[d];
            min_image(w, dx);
            float dr = sqrtf(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
            if (dr > 2.0f) err |= ERR_BOND_SNAPPED;
            float s = (prm.x * (prm.y - dr)) / dr;
            float sign = role == 0 ? -1.0f : 1.0f;
#pragma unroll
            for (int d = 0; d < 3; d++) F[d] += sign * (dx[d] * s);
        } else {
            rel_pos(w, pos, a.cellg, a.slot_of_id[bt.b], c, o, rb);
            float xh[3], xm[3], xt[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                xh[d] = role == 0 ? 0.f : ra[d];
                xm[d] = role == 0 ? ra[d] : (role == 1 ? 0.f : rb[d]);
                xt[d] = role == 2 ? 0.f : rb[d];
            }
            float b1[3], b2[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                b1[d] = xm[d] - xh[d];
                b2[d] = xt[d] - xm[d];
            }
            min_image(w, b1);
            min_image(w, b2);
            float r01 = sqrtf(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
            float r12 = sqrtf(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
            float mag = r01 * r12;
            if (mag > 0.0001f) {
                float dot = b1[0] * b2[0] + b1[1] * b2[1] + b1[2] * b2[2];
                float p1 = dot / (r01 * r01);
                float p2 = dot / (r12 * r12);
                float fm = prm.x / mag;
                if (fabsf(dot) > 0.000001f && prm.z > 0.0f) {
                    // 1/sqrt(1/cos^2 phi - 1) loses all precision in FP32 as the bonds turn
                    // collinear: evaluate the normalisation in FP64.
                    double b1d[3] = {b1[0], b1[1], b1[2]}, b2d[3] = {b2[0], b2[1], b2[2]};
                    double dd = b1d[0] * b2d[0] + b1d[1] * b2d[1] + b1d[2] * b2d[2];
                    double n1 = b1d[0] * b1d[0] + b1d[1] * b1d[1] + b1d[2] * b1d[2];
                    double n2 = b2d[0] * b2d[0] + b2d[1] * b2d[1] + b2d[2] * b2d[2];
                    double cos_phi_sq = (dd * dd) / (n1 * n2);
                    double ip = 1.0 / sqrt(1.0 / cos_phi_sq - 1.0);
                    fm = (float)((double)fm * ((double)prm.y - (double)prm.z * ip));
                }
                float hf[3], tf[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    hf[d] = (b1[d] * p1 - b2[d]) * fm;
                    tf[d] = (b1[d] - b2[d] * p2) * fm;
                }
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    float add = role == 0 ? hf[d] : (role == 2 ? tf[d] : -(hf[d] + tf[d]));
                    F[d] += add;
                }
            }
        }
    }
}

// Neighbour list of one bead, kept in shared memory: entry k of thread t is at
// [k * TILE_BEADS + t] (consecutive threads hit consecutive banks).  An entry is a sorted
// slot j and the direction of j's cell, packed 2 bits per axis as (d + 1).
constexpr int LIST_MAX = 48;

__device__ __forceinline__ uint32_t pack_dir(int ddx, int ddy, int ddz)
{
    return (uint32_t)(ddx + 1) | ((uint32_t)(ddy + 1) << 2) | ((uint32_t)(ddz + 1) << 4);
}

// Lower bound of the distance from offset o to the neighbour slab in direction d.
__device__ __forceinline__ float slab_gap(float o, int d)
{
    return d == 0 ? 0.0f : (d < 0 ? o : 1.0f - o);
}

// Separation of a neighbour bead pj from a home position already shifted by the neighbour
// cell's direction (a = o_home - dir), and its square.  The full-shell paths (the brick
// kernels 6 and 8, their fallback and the thread-per-bead kernel) test and evaluate every pair
// with this separation and pair_accumulate, with explicit roundings, so they give
// bit-identical forces.  For a pair close across a face in the -1 direction, o_home + 1 is
// rounded to 2^-24 (6e-8 absolute), about twice the rounding of the stored offsets themselves.
// The half shell needs an exactly antisymmetric separation and uses pair_sep; its walk keeps
// a candidate when this r^2 is below R2_PREFILTER, and the evaluation decides with the exact
// test on pair_sep's r^2, which differs from this one by at most a few units in the last
// place (|dr^2| < 4e-6), so no pair in range is lost.
constexpr float R2_PREFILTER = 1.0f + 0x1p-17f;

__device__ __forceinline__ float pair_r2(float ax, float ay, float az, const float4 pj, float &dx,
                                         float &dy, float &dz)
{
    dx = __fsub_rn(ax, pj.x);
    dy = __fsub_rn(ay, pj.y);
    dz = __fsub_rn(az, pj.z);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// One DPD pair force on the home bead, added to F (calc_force,
// dpd_maths_core_half_step.hpp:69-157): conservative a (1-r), dissipative -gamma w^2 (e.dv),
// random sqrt(gamma) w sqrt(24 kT/dt) u with kT = 1, along e = dx / r.
__device__ __forceinline__ void pair_accumulate(float dx, float dy, float dz, float r2,
                                                const float4 vi, const float4 vj, uint32_t hi,
                                                uint32_t hj, float2 pp, uint32_t th_lo,
                                                uint32_t th_hi, float scale, float F[3])
{
    const float inv_r = rsqrtf(r2);
    const float r = __fmul_rn(r2, inv_r);
    const float wr = __fsub_rn(1.0f, r);
    const float ex = __fmul_rn(dx, inv_r), ey = __fmul_rn(dy, inv_r), ez = __fmul_rn(dz, inv_r);
    const float rdotv = __fmaf_rn(ez, __fsub_rn(vi.z, vj.z),
                                  __fmaf_rn(ey, __fsub_rn(vi.y, vj.y), __fmul_rn(ex, __fsub_rn(vi.x, vj.x))));
    const float sg = __fmul_rn(pp.y, wr);
    const float u = hash_u(th_lo, th_hi, hi, hj);
    const float con_m_diss = __fmaf_rn(-__fmul_rn(sg, sg), rdotv, __fmul_rn(pp.x, wr));
    const float scaled = __fmaf_rn(__fmul_rn(sg, scale), u, con_m_diss);
    F[0] = __fmaf_rn(ex, scaled, F[0]);
    F[1] = __fmaf_rn(ey, scaled, F[1]);
    F[2] = __fmaf_rn(ez, scaled, F[2]);
}

// Separation of the pair (i, j), d = cell_j - cell_i, per axis (o_i - [d > 0]) - (o_j - [d < 0]),
// and its square: the separation the half shell evaluates a pair with.  When the pair is close
// across a cell face the offset next to the face is >= 0.5, so its shift by one cell is exact
// and the separation carries one rounding relative to its own (small) size -- the unit vector
// keeps FP32 precision however close the beads are (o_i - d - o_j in the other order loses
// up to 6e-8 absolute).  Rounding to nearest is symmetric under a change of sign, so the
// separation computed on j's side is exactly the negation and r^2 is the same to the bit.
__device__ __forceinline__ float sep_axis(float oi, float oj, int d)
{
    const float a = d > 0 ? __fsub_rn(oi, 1.0f) : oi;
    const float b = d < 0 ? __fsub_rn(oj, 1.0f) : oj;
    return __fsub_rn(a, b);
}

__device__ __forceinline__ float pair_sep(const float4 pi, const float4 pj, int ddx, int ddy, int ddz,
                                          float &dx, float &dy, float &dz)
{
    dx = sep_axis(pi.x, pj.x, ddx);
    dy = sep_axis(pi.y, pj.y, ddy);
    dz = sep_axis(pi.z, pj.z, ddz);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// The pair test of update_bead_pair (naive_dpd_engine_half_step.hpp:358-368 and
// dpd_state.hpp:138-139) on the canonical r^2.
__device__ __forceinline__ bool pair_in_range(float r2)
{
    return r2 < 1.0f && r2 >= min_dist_sqr_f();
}

// Pair forces are summed in fixed point by the half-shell kernel: each pair force component,
// scaled by 2^20, is rounded to an integer (rounding to nearest is symmetric, so the two beads
// of a pair receive exact negatives; the rounding error, <= 2^-21 per term, is far below the
// FP32 engine's tolerance) and the integers are added in 64 bits.  Integer sums do not depend
// on their order, so a bead's total force is the same whichever brick shape, batch or thread
// evaluated its pairs, and whether a pair was evaluated from one side with the reaction
// passed on (inside a brick) or from both sides (across a brick face).  Terms below 2^31 (pair
// forces below 2048) convert with the full-rate 32-bit conversion; larger ones with the
// 64-bit one (slow on this part, and rare).  A pair force of 2^20 or more, or not finite, is
// reported as ERR_NONFINITE.
constexpr float FX_ONE = 1048576.0f;             // 2^20
constexpr float FX_INV = 9.5367431640625e-07f;   // 2^-20
constexpr float FX_FAST = 2147483520.0f;         // largest float below 2^31
constexpr float FX_LIMIT = 1048576.0f;           // |pair force| reported as an error

// A 64-bit fixed-point sum as a float force: one correctly rounded conversion of the whole
// integer (converting its two 32-bit halves separately rounds the low half to 24 bits, an
// error of up to 2^7 units that cancels badly for negative sums), then an exact scaling by a
// power of two.  Once per bead and axis, so the slower 64-bit conversion costs nothing.
__device__ __forceinline__ float fx_to_float(long long q)
{
    return __fmul_rn(__ll2float_rn(q), FX_INV);
}

__device__ __forceinline__ void fx_to_force(const long long q[3], float F[3])
{
    F[0] = fx_to_float(q[0]);
    F[1] = fx_to_float(q[1]);
    F[2] = fx_to_float(q[2]);
}

// One DPD pair force on the home bead i (calc_force, dpd_maths_core_half_step.hpp:69-157):
// conservative a (1-r), dissipative -gamma w^2 (e.dv), random sqrt(gamma) w sqrt(24 kT/dt) u
// with kT = 1, along e = dx / r, from the canonical separation (dx, dy, dz) and r2 in range.
// Every operation is explicitly rounded; e and dv change sign with the side the pair is
// evaluated from and everything else does not, so the force is exactly antisymmetric.
// Returns the force in fixed point (fx_to_force's scale); a pair force of magnitude beyond
// FX_LIMIT (or not finite) contributes nothing and sets ERR_NONFINITE.
__device__ __forceinline__ void pair_force_fx(float dx, float dy, float dz, float r2, const float4 vi,
                                              const float4 vj, uint32_t hi, uint32_t hj, float2 pp,
                                              uint32_t th_lo, uint32_t th_hi, float scale,
                                              long long &qx, long long &qy, long long &qz,
                                              uint32_t &err)
{
    const float inv_r = rsqrtf(r2);
    const float r = __fmul_rn(r2, inv_r);
    const float wr = __fsub_rn(1.0f, r);
    const float ex = __fmul_rn(dx, inv_r), ey = __fmul_rn(dy, inv_r), ez = __fmul_rn(dz, inv_r);
    const float rdotv = __fmaf_rn(ez, __fsub_rn(vi.z, vj.z),
                                  __fmaf_rn(ey, __fsub_rn(vi.y, vj.y), __fmul_rn(ex, __fsub_rn(vi.x, vj.x))));
    const float sg = __fmul_rn(pp.y, wr);
    const float u = hash_u(th_lo, th_hi, hi, hj);
    const float con_m_diss = __fmaf_rn(-__fmul_rn(sg, sg), rdotv, __fmul_rn(pp.x, wr));
    float scaled = __fmaf_rn(__fmul_rn(sg, scale), u, con_m_diss);
    if (!(fabsf(scaled) < FX_LIMIT)) {
        err |= ERR_NONFINITE;
        scaled = 0.0f;
    }
    const float sq = __fmul_rn(scaled, FX_ONE);
    const float tx = __fmul_rn(ex, sq), ty = __fmul_rn(ey, sq), tz = __fmul_rn(ez, sq);
    if (fabsf(sq) < FX_FAST) {  // |e| <= 1: every component converts in 32 bits
        qx = __float2int_rn(tx);
        qy = __float2int_rn(ty);
        qz = __float2int_rn(tz);
    } else {
        qx = __float2ll_rn(tx);
        qy = __float2ll_rn(ty);
        qz = __float2ll_rn(tz);
    }
}

// The pair (i, j) at direction d = cell_j - cell_i, added to i's fixed-point sum q when in
// range.  Returns whether it was.
__device__ __forceinline__ bool pair_add_fx(const float4 pi, const float4 vi, const float4 pj, const float4 vj,
                                            int ddx, int ddy, int ddz, float2 pp, uint32_t th_lo,
                                            uint32_t th_hi, float scale, long long q[3], uint32_t &err)
{
    float dx, dy, dz;
    const float r2 = pair_sep(pi, pj, ddx, ddy, ddz, dx, dy, dz);
    if (!pair_in_range(r2)) return false;
    long long fx, fy, fz;
    pair_force_fx(dx, dy, dz, r2, vi, vj, __float_as_uint(pi.w), __float_as_uint(pj.w), pp, th_lo, th_hi,
                  scale, fx, fy, fz, err);
    q[0] += fx;
    q[1] += fy;
    q[2] += fz;
    return true;
}

// Bonds, update_mom and either the final write or the next update_pos with the cell count,
// for one bead whose pair forces are in F.
template <int FINAL>
__device__ __forceinline__ void integrate32(const KArgs &a, const WorldDev &w, uint32_t s,
                                            const int c[3], const float4 ph, const float4 vh,
                                            float F[3], uint32_t &err)
{
    const float dt = (float)w.dt, hdt = 0.5f * dt, hdt2 = 0.5f * dt * dt;
    float o[3] = {ph.x, ph.y, ph.z};
    if (!(__float_as_uint(ph.w) & (1u << 27))) {  // polymer bead: its bond force, from k_bonds32
        const float4 fb = a.fbond[s];
        F[0] = __fadd_rn(F[0], fb.x);
        F[1] = __fadd_rn(F[1], fb.y);
        F[2] = __fadd_rn(F[2], fb.z);
    }
    // update_mom (dpd_maths_core_half_step.hpp:51-61)
    float v[3] = {__fmaf_rn(F[0], hdt, vh.x), __fmaf_rn(F[1], hdt, vh.y), __fmaf_rn(F[2], hdt, vh.z)};
    if ((w.stationary >> (__float_as_uint(ph.w) >> 28)) & 1u) {
        // stationary type: v and f cleared (naive_dpd_engine_half_merge.hpp:387-394), so the
        // next update_pos leaves it where it is
        v[0] = v[1] = v[2] = 0.f;
        F[0] = F[1] = F[2] = 0.f;
    }
    if (FINAL) {
        ((float4 *)a.velB)[s] = make_float4(v[0], v[1], v[2], 0.f);
        ((float4 *)a.frc)[s] = make_float4(F[0], F[1], F[2], 0.f);
        if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) err |= ERR_NONFINITE;
    } else {
        const uint32_t key = advance_position(w, dt, hdt2, c, o, v, F, err);
        const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
        ((float4 *)a.posB)[s] = make_float4(o[0], o[1], o[2], ph.w);
        ((float4 *)a.velB)[s] = make_float4(__fmaf_rn(F[0], hdt, v[0]), __fmaf_rn(F[1], hdt, v[1]),
                                            __fmaf_rn(F[2], hdt, v[2]), 0.f);
        a.keyrank[s] = make_uint2(key, zhalf_rank(rank, o[2]));
    }
}

// Bond forces of every polymer bead (monomer bit of the hash clear), one thread per bead,
// written by sorted slot for the force kernel to add.  Running them here, on a compact list
// of the few bonded beads, keeps their dependent partner lookups out of the pair kernel's
// warps.
__global__ void __launch_bounds__(128) k_bonds32(KArgs a)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_bonded) return;
    const uint32_t id = a.bonded_ids[k];
    uint32_t lo = 0, hi = a.n_worlds;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (a.worlds[mid].bead_base <= id) lo = mid; else hi = mid;
    }
    const WorldDev &w = a.worlds[lo];
    const uint32_t s = a.slot_of_id[id];
    const float4 p = ((const float4 *)a.posA)[s];
    int c[3];
    decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
    const float o[3] = {p.x, p.y, p.z};
    float F[3] = {0.f, 0.f, 0.f};
    uint32_t err = 0;
    bond_forces32(a, w, id, c, o, F, err);
    a.fbond[s] = make_float4(F[0], F[1], F[2], 0.f);
    if (err) atomicOr(&a.worlds[lo].err, err);
}

// Thread-per-bead pair forces straight from global memory, summed one pair at a time in the
// reference's order (used by the brick kernel when a halo does not fit in shared memory).
__device__ void pair_forces32_seq(const KArgs &a, const WorldDev &w, const float2 *pair,
                                  uint32_t th_lo, uint32_t th_hi, float scale, const int c[3],
                                  const float4 ph, const float4 vh, float F[3])
{
    const float4 *__restrict__ pos = (const float4 *)a.posA;
    const float4 *__restrict__ vel = (const float4 *)a.velA;
    const uint32_t nt = w.n_types;
    const uint32_t hi = __float_as_uint(ph.w);
    const uint32_t ti = min(hi >> 28, nt - 1u);
    const float min2 = min_dist_sqr_f();
    for (int ddx = -1; ddx <= 1; ddx++) {
        const int nx = wrap_index(c[0] + ddx, w.L[0]);
        const float ax = __fsub_rn(ph.x, (float)ddx);
        for (int ddy = -1; ddy <= 1; ddy++) {
            const int ny = wrap_index(c[1] + ddy, w.L[1]);
            const float ay = __fsub_rn(ph.y, (float)ddy);
            const uint32_t row = w.cell_base + ((uint32_t)nx * (uint32_t)w.L[1] + (uint32_t)ny) * (uint32_t)w.L[2];
            for (int ddz = -1; ddz <= 1; ddz++) {
                const float az = __fsub_rn(ph.z, (float)ddz);
                const uint32_t nc = row + (uint32_t)wrap_index(c[2] + ddz, w.L[2]);
                const uint32_t j1 = a.start[nc + 1];
                for (uint32_t j = a.start[nc]; j < j1; j++) {
                    const float4 pj = pos[j];
                    float dx, dy, dz;
                    const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                    if (r2 < 1.0f && r2 >= min2) {
                        const uint32_t hj = __float_as_uint(pj.w);
                        pair_accumulate(dx, dy, dz, r2, vh, vel[j], hi, hj,
                                        pair[ti * nt + min(hj >> 28, nt - 1u)], th_lo, th_hi,
                                        scale, F);
                    }
                }
            }
        }
    }
}

// The same gather in fixed point (pair_add_fx): the half-shell kernel's path for a brick whose
// halo does not fit in shared memory, with the same sums as its staged path.
__device__ void pair_forces32_seq_fx(const KArgs &a, const WorldDev &w, const float2 *pair,
                                     uint32_t th_lo, uint32_t th_hi, float scale, const int c[3],
                                     const float4 ph, const float4 vh, float F[3], uint32_t &err)
{
    const float4 *__restrict__ pos = (const float4 *)a.posA;
    const float4 *__restrict__ vel = (const float4 *)a.velA;
    const uint32_t nt = w.n_types;
    const uint32_t ti = min(__float_as_uint(ph.w) >> 28, nt - 1u);
    long long q[3] = {0, 0, 0};
    for (int ddx = -1; ddx <= 1; ddx++) {
        const int nx = wrap_index(c[0] + ddx, w.L[0]);
        for (int ddy = -1; ddy <= 1; ddy++) {
            const int ny = wrap_index(c[1] + ddy, w.L[1]);
            const uint32_t row = w.cell_base + ((uint32_t)nx * (uint32_t)w.L[1] + (uint32_t)ny) * (uint32_t)w.L[2];
            for (int ddz = -1; ddz <= 1; ddz++) {
                const uint32_t nc = row + (uint32_t)wrap_index(c[2] + ddz, w.L[2]);
                const uint32_t j1 = a.start[nc + 1];
                for (uint32_t j = a.start[nc]; j < j1; j++) {
                    const float4 pj = pos[j];
                    pair_add_fx(ph, vh, pj, vel[j], ddx, ddy, ddz,
                                pair[ti * nt + min(__float_as_uint(pj.w) >> 28, nt - 1u)], th_lo, th_hi,
                                scale, q, err);
                }
            }
        }
    }
    fx_to_force(q, F);
}

// Pair log (pdpd_log_pair_terms) of the FP32 engine: for each sorted slot whose bead is in the
// sorted id list sel, every in-range pair of the 27-direction walk (the full-shell kernels'
// separation and test), with the terms of its force.  The force kernels fuse the terms
// (pair_accumulate: con - diss and the random term in two multiply-adds); here con, diss and
// rand are also formed one by one, and f = e * scaled is the pair's contribution exactly as
// the kernels add it.  Count pass (out null) and write pass as k_pair_log64.
__global__ void k_pair_log32(KArgs a, const uint32_t *__restrict__ sel, uint32_t n_sel,
                             const uint32_t *__restrict__ offs, uint32_t *__restrict__ counts,
                             PairLogRec *__restrict__ out)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n_beads) return;
    const uint32_t id = a.ids[s];
    uint32_t lo = 0, hi = n_sel;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (sel[mid] < id) lo = mid + 1; else hi = mid;
    }
    if (lo == n_sel || sel[lo] != id) return;
    const uint32_t k = lo;
    uint32_t wl = 0, wh = a.n_worlds;
    while (wh - wl > 1) {
        const uint32_t mid = (wl + wh) / 2;
        if (a.worlds[mid].bead_base <= id) wl = mid; else wh = mid;
    }
    const WorldDev &w = a.worlds[wl];
    const float4 *pos = (const float4 *)a.posA, *vel = (const float4 *)a.velA;
    const float4 ph = pos[s], vh = vel[s];
    int c[3];
    decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
    const uint64_t th = t_hash((uint32_t)w.t, w.seed);
    const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
    const float scale = (float)w.scale_inv_sqrt_dt;
    const float2 *pair = (const float2 *)a.pair + w.param_base;
    const float2 *cp = w.spatial ? (const float2 *)a.cellpair + w.cellpair_base : nullptr;
    const uint32_t hc = ((uint32_t)c[0] * (uint32_t)w.L[1] + (uint32_t)c[1]) * (uint32_t)w.L[2] + (uint32_t)c[2];
    const uint32_t nt = w.n_types, n2 = nt * nt;
    const uint32_t hh = __float_as_uint(ph.w), ti = min(hh >> 28, nt - 1u);
    const float min2 = min_dist_sqr_f();
    uint32_t n = 0;
    for (int ddx = -1; ddx <= 1; ddx++)
        for (int ddy = -1; ddy <= 1; ddy++)
            for (int ddz = -1; ddz <= 1; ddz++) {
                const int nx = wrap_index(c[0] + ddx, w.L[0]), ny = wrap_index(c[1] + ddy, w.L[1]),
                          nz = wrap_index(c[2] + ddz, w.L[2]);
                const uint32_t nc = w.cell_base + ((uint32_t)nx * (uint32_t)w.L[1] + (uint32_t)ny) * (uint32_t)w.L[2] + (uint32_t)nz;
                const float ax = __fsub_rn(ph.x, (float)ddx), ay = __fsub_rn(ph.y, (float)ddy),
                            az = __fsub_rn(ph.z, (float)ddz);
                for (uint32_t j = a.start[nc]; j < a.start[nc + 1]; j++) {
                    const float4 pj = pos[j];
                    float dx, dy, dz;
                    const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                    if (!(r2 < 1.0f && r2 >= min2)) continue;
                    if (out) {
                        const float4 vj = vel[j];
                        const uint32_t hj = __float_as_uint(pj.w);
                        const uint32_t pk = ti * nt + min(hj >> 28, nt - 1u);
                        float2 pp = pair[pk];
                        if (cp) {
                            const float2 hv = cp[(size_t)hc * n2 + pk], ov = cp[(size_t)(a.cellg[j] - w.cell_base) * n2 + pk];
                            pp = make_float2(__fmul_rn(__fadd_rn(hv.x, ov.x), 0.5f), __fmul_rn(__fadd_rn(hv.y, ov.y), 0.5f));
                        }
                        float F[3] = {0.f, 0.f, 0.f};
                        pair_accumulate(dx, dy, dz, r2, vh, vj, hh, hj, pp, th_lo, th_hi, scale, F);
                        const float inv_r = rsqrtf(r2);
                        const float r = __fmul_rn(r2, inv_r);
                        const float wr = __fsub_rn(1.0f, r);
                        const float ex = __fmul_rn(dx, inv_r), ey = __fmul_rn(dy, inv_r), ez = __fmul_rn(dz, inv_r);
                        const float rdotv = __fmaf_rn(ez, __fsub_rn(vh.z, vj.z),
                                                      __fmaf_rn(ey, __fsub_rn(vh.y, vj.y), __fmul_rn(ex, __fsub_rn(vh.x, vj.x))));
                        const float sg = __fmul_rn(pp.y, wr);
                        const float u = hash_u(th_lo, th_hi, hh, hj);
                        PairLogRec &rec = out[offs[k] + n];
                        rec.t = w.t;
                        rec.home_id = id;
                        rec.other_id = a.ids[j];
                        rec.home_hash = hh;
                        rec.other_hash = hj;
                        rec.dx[0] = dx;
                        rec.dx[1] = dy;
                        rec.dx[2] = dz;
                        rec.dr = r;
                        rec.inv_root_dt = scale;
                        rec.gammap = __fmul_rn(sg, sg);
                        rec.rng = u;
                        rec.con = __fmul_rn(pp.x, wr);
                        rec.diss = __fmul_rn(-__fmul_rn(sg, sg), rdotv);
                        rec.rng_scale = __fmul_rn(sg, scale);
                        rec.rand = __fmul_rn(__fmul_rn(sg, scale), u);
                        for (int d = 0; d < 3; d++) rec.f[d] = F[d];
                    }
                    n++;
                }
            }
    if (!out) counts[k] = n;
}

// Phase 2: the pair forces of the listed neighbours, in list order.
__device__ __forceinline__ void list_forces32(const float4 *__restrict__ pos,
                                              const float4 *__restrict__ vel,
                                              const uint32_t *__restrict__ s_j,
                                              const uint8_t *__restrict__ s_dir, int n,
                                              const float4 ph, const float4 vh, uint32_t ti,
                                              uint32_t nt, const float2 *__restrict__ pair,
                                              uint32_t th_lo, uint32_t th_hi, float scale,
                                              float F[3], const float2 *__restrict__ cp = nullptr,
                                              uint32_t hc = 0, const uint32_t *__restrict__ cellg = nullptr,
                                              uint32_t cell_base = 0)
{
    const uint32_t hh = __float_as_uint(ph.w);
    const uint32_t n2 = nt * nt;
    for (int k = 0; k < n; k++) {
        const uint32_t j = s_j[k * TILE_BEADS + threadIdx.x];
        const uint32_t d = s_dir[k * TILE_BEADS + threadIdx.x];
        const float4 pj = pos[j];
        const float ax = __fsub_rn(ph.x, (float)((int)(d & 3u) - 1));
        const float ay = __fsub_rn(ph.y, (float)((int)((d >> 2) & 3u) - 1));
        const float az = __fsub_rn(ph.z, (float)((int)((d >> 4) & 3u) - 1));
        float dx, dy, dz;
        const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
        const uint32_t hj = __float_as_uint(pj.w);
        const uint32_t pk = ti * nt + min(hj >> 28, nt - 1u);
        float2 pp = pair[pk];
        if (cp) {  // spatial strengths: mean of the two beads' cell values
            const float2 h = cp[(size_t)hc * n2 + pk], o = cp[(size_t)(cellg[j] - cell_base) * n2 + pk];
            pp = make_float2(__fmul_rn(__fadd_rn(h.x, o.x), 0.5f), __fmul_rn(__fadd_rn(h.y, o.y), 0.5f));
        }
        pair_accumulate(dx, dy, dz, r2, vh, vel[j], hh, hj, pp, th_lo, th_hi, scale, F);
    }
}

// Pair forces on one bead: full-shell gather over the 27 neighbour cells in the reference's
// direction order, the beads of a cell in id order (naive_dpd_engine_half_step.hpp:300-315,
// 358-424).  Phase 1 keeps the candidates with r^2 in [MIN_DISTANCE_CUTOFF^2, 1) in a list;
// phase 2 evaluates them.  Cells whose nearest face is at distance >= 1 (with margin) cannot
// hold an in-range bead and are skipped; the list is the same as without the skip.
__device__ __forceinline__ void pair_forces32(const KArgs &a, const WorldDev &w,
                                              const float2 *pair, uint32_t *s_j,
                                              uint8_t *s_dir, int cap, uint32_t th_lo,
                                              uint32_t th_hi, float scale, const int c[3],
                                              const float4 ph, const float4 vh, float F[3])
{
    const float4 *__restrict__ pos = (const float4 *)a.posA;
    const float4 *__restrict__ vel = (const float4 *)a.velA;
    const uint32_t *__restrict__ start = a.start;
    const uint32_t nt = w.n_types;
    const uint32_t ti = min(__float_as_uint(ph.w) >> 28, nt - 1u);
    const float min2 = min_dist_sqr_f();
    const float PRUNE = 1.0001f;
    const float2 *cp = w.spatial ? (const float2 *)a.cellpair + w.cellpair_base : nullptr;
    const uint32_t hc = ((uint32_t)c[0] * (uint32_t)w.L[1] + (uint32_t)c[1]) * (uint32_t)w.L[2] + (uint32_t)c[2];
    F[0] = F[1] = F[2] = 0.f;
    int n = 0;
    for (int ddx = -1; ddx <= 1; ddx++) {
        const float gx = slab_gap(ph.x, ddx);
        const int nx = wrap_index(c[0] + ddx, w.L[0]);
        const float ax = __fsub_rn(ph.x, (float)ddx);
        for (int ddy = -1; ddy <= 1; ddy++) {
            const float gy = slab_gap(ph.y, ddy);
            const float gxy = gx * gx + gy * gy;
            if (gxy >= PRUNE) continue;
            const int ny = wrap_index(c[1] + ddy, w.L[1]);
            const float ay = __fsub_rn(ph.y, (float)ddy);
            const uint32_t row = w.cell_base + ((uint32_t)nx * (uint32_t)w.L[1] + (uint32_t)ny) * (uint32_t)w.L[2];
            for (int ddz = -1; ddz <= 1; ddz++) {
                const float gz = slab_gap(ph.z, ddz);
                if (gxy + gz * gz >= PRUNE) continue;
                const int nz = wrap_index(c[2] + ddz, w.L[2]);
                const float az = __fsub_rn(ph.z, (float)ddz);
                const uint32_t nc = row + (uint32_t)nz;
                const uint32_t j1 = start[nc + 1];
                const uint8_t dpk = (uint8_t)pack_dir(ddx, ddy, ddz);
                for (uint32_t j = start[nc]; j < j1; j++) {
                    const float4 pj = pos[j];
                    float dx, dy, dz;
                    const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                    if (r2 < 1.0f && r2 >= min2) {
                        if (n == cap) {
                            list_forces32(pos, vel, s_j, s_dir, n, ph, vh, ti, nt, pair, th_lo,
                                          th_hi, scale, F, cp, hc, a.cellg, w.cell_base);
                            n = 0;
                        }
                        s_j[n * TILE_BEADS + threadIdx.x] = j;
                        s_dir[n * TILE_BEADS + threadIdx.x] = dpk;
                        n++;
                    }
                }
            }
        }
    }
    list_forces32(pos, vel, s_j, s_dir, n, ph, vh, ti, nt, pair, th_lo, th_hi, scale, F, cp, hc,
                  a.cellg, w.cell_base);
}

template <int FINAL>
__global__ void __launch_bounds__(TILE_BEADS) k_force32(KArgs a)
{
    __shared__ float2 s_pair[MAX_PAIR];
    __shared__ uint32_t s_j[LIST_MAX * TILE_BEADS];
    __shared__ uint8_t s_dir[LIST_MAX * TILE_BEADS];
    __shared__ WorldCache wc;
    if (threadIdx.x == 0) wc.world = 0xffffffffu;
    __syncthreads();
    const int cap = (a.list_capacity > 0 && a.list_capacity < LIST_MAX) ? a.list_capacity : LIST_MAX;
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        load_world(a, tl.world, wc, s_pair);
        const WorldDev &w = wc.w;
        const uint32_t s = tl.slot_begin + threadIdx.x;
        if (s >= tl.slot_end) continue;
        const float scale = (float)w.scale_inv_sqrt_dt;
        const uint64_t th = t_hash((uint32_t)w.t, w.seed);
        const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
        uint32_t err = 0;
        const float4 ph = ((const float4 *)a.posA)[s];
        const float4 vh = ((const float4 *)a.velA)[s];
        int c[3];
        decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
        float F[3];
        pair_forces32(a, w, s_pair, s_j, s_dir, cap, th_lo, th_hi, scale, c, ph, vh, F);
        integrate32<FINAL>(a, w, s, c, ph, vh, F, err);
        if (err) atomicOr(&a.worlds[tl.world].err, err);
    }
}

// First update_pos of a run, from the rest state x(t), v(t), f(t).
__global__ void __launch_bounds__(TILE_BEADS) k_begin32(KArgs a)
{
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        const uint32_t s = tl.slot_begin + threadIdx.x;
        if (s >= tl.slot_end) continue;
        const WorldDev &w = a.worlds[tl.world];
        const float dt = (float)w.dt, hdt = 0.5f * dt, hdt2 = 0.5f * dt * dt;
        uint32_t err = 0;
        const float4 ph = ((const float4 *)a.posA)[s];
        const float4 vh = ((const float4 *)a.velA)[s];
        const float4 fh = ((const float4 *)a.frc)[s];
        int c[3];
        decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
        float o[3] = {ph.x, ph.y, ph.z};
        // a stationary type is not moved and keeps its v (naive_dpd_engine_half_merge.hpp:329-333)
        const bool st = (w.stationary >> (__float_as_uint(ph.w) >> 28)) & 1u;
        const float v[3] = {st ? 0.f : vh.x, st ? 0.f : vh.y, st ? 0.f : vh.z};
        const float F[3] = {st ? 0.f : fh.x, st ? 0.f : fh.y, st ? 0.f : fh.z};
        const uint32_t key = advance_position(w, dt, hdt2, c, o, v, F, err);
        const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
        ((float4 *)a.posB)[s] = make_float4(o[0], o[1], o[2], ph.w);
        ((float4 *)a.velB)[s] = st ? make_float4(vh.x, vh.y, vh.z, 0.f)
                                   : make_float4(v[0] + F[0] * hdt, v[1] + F[1] * hdt, v[2] + F[2] * hdt, 0.f);
        a.keyrank[s] = make_uint2(key, zhalf_rank(rank, o[2]));
        if (err) atomicOr(&a.worlds[tl.world].err, err);
    }
}

// Attach: id-ordered FP64 staging (x, v, f: rows of 9 doubles, or field-major blocks of
// staging_n beads each) -> B in slot = id order, with cell counts.
__global__ void k_bin32(KArgs a, const uint32_t *__restrict__ hash_in)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n_beads) return;
    // world of bead g: worlds are in bead_base order
    uint32_t lo = 0, hi = a.n_worlds;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (a.worlds[mid].bead_base <= g) lo = mid; else hi = mid;
    }
    const WorldDev &w = a.worlds[lo];
    const size_t stride = a.staging_fields ? 3 : 9, field = a.staging_fields ? 3 * (size_t)a.staging_n : 3;
    const double *st = a.staging + stride * g;
    int c[3];
    float o[3];
    uint32_t err = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double x = st[d];
        if (!(x >= 0.0 && x < (double)w.L[d])) {
            err |= ERR_OUT_OF_BOX;
            x = 0.0;
        }
        double fl = floor(x);
        c[d] = (int)fl;
        float off = (float)(x - fl);
        if (off >= 1.0f) off = 0x1.fffffep-1f;
        o[d] = off;
    }
    if (err) atomicOr(&a.worlds[lo].err, err);
    const uint32_t key = w.cell_base + ((uint32_t)c[0] * (uint32_t)w.L[1] + (uint32_t)c[1]) * (uint32_t)w.L[2] + (uint32_t)c[2];
    const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
    ((float4 *)a.posB)[g] = make_float4(o[0], o[1], o[2], __uint_as_float(hash_in[g]));
    ((float4 *)a.velB)[g] = make_float4((float)st[field], (float)st[field + 1], (float)st[field + 2], 0.f);
    ((float4 *)a.frcB)[g] = make_float4((float)st[2 * field], (float)st[2 * field + 1], (float)st[2 * field + 2], 0.f);
    a.ids[g] = g;
    a.keyrank[g] = make_uint2(key, zhalf_rank(rank, o[2]));
}

__global__ void k_finish32(KArgs a)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.n_beads) ((float4 *)a.velA)[s] = ((const float4 *)a.velB)[s];
    if (blockIdx.x == 0)
        for (uint32_t w = threadIdx.x; w < a.n_worlds; w += blockDim.x) a.worlds[w].t += 1;
}


#include "pdpd_fp32_brick.cuh"

}  // namespace

int launch_bin32(const KArgs &a, const uint32_t *hash_in, cudaStream_t s)
{
    if (a.n_beads == 0) return 0;
    k_bin32<<<(a.n_beads + 255) / 256, 256, 0, s>>>(a, hash_in);
    return 1;
}

int launch_begin32(const KArgs &a, cudaStream_t s)
{
    k_begin32<<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    return 1;
}

// Largest staged-bead capacity of a brick for a force variant: what leaves room for two
// blocks per SM (variants 8 and 9), within the 16-bit staged indices of the list entries.
uint32_t brick_maxb_limit(int variant, uint32_t hc_max, uint32_t npair, uint32_t home_max)
{
    if (variant != 8 && variant != 9) return 2047u;  // variant 6: its bricks stay far below
    int dev = 0, smem_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess)
        return 2047u;
    const uint32_t hm = variant == 9 ? home_max : 0u;
    const BrickLayout L = brick_layout(hc_max, 0, npair, brick_variant_threads(variant), hm);
    // per staged bead: position and velocity (32 B), and for the half shell its home index
    const int per_bead = variant == 9 ? 34 : 32;
    const int budget = smem_sm / 2 - 1024 - (int)L.bytes - 64;
    return (uint32_t)std::max(64, std::min(65535, budget / per_bead));
}

// Set up the brick kernel for a brick shape: opt in to the shared memory it needs and
// return its persistent grid (resident blocks x SMs) and dynamic shared-memory bytes.
int brick_setup(int sm_count, int variant, uint32_t hc_max, uint32_t maxb, uint32_t npair, uint32_t home_max,
                int *grid, uint32_t *smem_bytes)
{
    int nb = 0;
    const uint32_t hm = variant == 9 ? home_max : 0u;
    const BrickLayout L = brick_layout(hc_max, maxb, npair, brick_variant_threads(variant), hm);
    const int bytes = (int)L.bytes;
    void (*k0)(KArgs, BrickLayout) = nullptr;
    void (*k1)(KArgs, BrickLayout) = nullptr;
    switch (variant) {
    case 9: k0 = k_force32_half<0>; k1 = k_force32_half<1>; break;
    case 8:
        k0 = k_force32_brick<0, BRICK_THREADS_WIDE>;
        k1 = k_force32_brick<1, BRICK_THREADS_WIDE>;
        break;
    default: k0 = k_force32_brick<0, BRICK_THREADS>; k1 = k_force32_brick<1, BRICK_THREADS>; break;
    }
    cudaError_t e = cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k0, (int)brick_variant_threads(variant), bytes);
    if (e != cudaSuccess) return (int)e;
    if (nb < 1) return (int)cudaErrorInvalidConfiguration;
    *grid = nb * sm_count;
    *smem_bytes = L.bytes;
    return 0;
}

static int launch_pair_forces32(const KArgs &a, int final_step, cudaStream_t s);

int launch_force32(const KArgs &a, int final_step, cudaStream_t s)
{
    int n = 0;
    if (a.n_bonded > 0) {
        k_bonds32<<<(a.n_bonded + 127) / 128, 128, 0, s>>>(a);
        n++;
    }
    return n + launch_pair_forces32(a, final_step, s);
}

static int launch_pair_forces32(const KArgs &a, int final_step, cudaStream_t s)
{
    if (a.force_kernel != 1 && a.n_bricks > 0) {
        const int v = a.force_kernel;
        const BrickLayout L = brick_layout(a.brick_hc_max, a.brick_maxb, a.brick_npair, brick_variant_threads(v),
                                           v == 9 ? a.brick_home_max : 0u);
        const int grid = (int)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)a.brick_grid, a.n_bricks));
        void (*k)(KArgs, BrickLayout);
        switch (v) {
        case 9: k = final_step ? k_force32_half<1> : k_force32_half<0>; break;
        case 8:
            k = final_step ? k_force32_brick<1, BRICK_THREADS_WIDE> : k_force32_brick<0, BRICK_THREADS_WIDE>;
            break;
        default: k = final_step ? k_force32_brick<1, BRICK_THREADS> : k_force32_brick<0, BRICK_THREADS>; break;
        }
        k<<<grid, brick_variant_threads(v), L.bytes, s>>>(a, L);
        return 1;
    }
    if (final_step)
        k_force32<1><<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    else
        k_force32<0><<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    return 1;
}

int launch_pair_log32(const KArgs &a, const uint32_t *sel, uint32_t n_sel, const uint32_t *offs,
                      uint32_t *counts, PairLogRec *out, cudaStream_t s)
{
    if (a.n_beads == 0 || n_sel == 0) return 0;
    k_pair_log32<<<(a.n_beads + 127) / 128, 128, 0, s>>>(a, sel, n_sel, offs, counts, out);
    return 1;
}

int launch_finish32(const KArgs &a, cudaStream_t s)
{
    k_finish32<<<(a.n_beads + 255) / 256 + 1, 256, 0, s>>>(a);
    return 1;
}

}  // namespace pdpd
