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
        float on = o[d] + (v[d] * dt + f[d] * hdt2);
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
__device__ void bond_forces32(const KArgs &a, const WorldDev &w, uint32_t id, const int c[3],
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

// Phase 2: the pair forces of the listed neighbours, in list order (calc_force,
// dpd_maths_core_half_step.hpp:69-157; kT = 1, sigma = sqrt(2 gamma kT) implied).
__device__ __forceinline__ void list_forces32(const float4 *__restrict__ pos,
                                              const float4 *__restrict__ vel,
                                              const uint32_t *__restrict__ s_j,
                                              const uint8_t *__restrict__ s_dir, int n,
                                              const float4 ph, const float4 vh, uint32_t ti,
                                              uint32_t nt, const float2 *__restrict__ pair,
                                              uint32_t th_lo, uint32_t th_hi, float scale,
                                              float &fx, float &fy, float &fz)
{
    const uint32_t hh = __float_as_uint(ph.w);
    for (int k = 0; k < n; k++) {
        const uint32_t j = s_j[k * TILE_BEADS + threadIdx.x];
        const uint32_t d = s_dir[k * TILE_BEADS + threadIdx.x];
        const float4 pj = pos[j];
        const float4 vj = vel[j];
        const float dx = (ph.x - (float)((int)(d & 3u) - 1)) - pj.x;
        const float dy = (ph.y - (float)((int)((d >> 2) & 3u) - 1)) - pj.y;
        const float dz = (ph.z - (float)((int)((d >> 4) & 3u) - 1)) - pj.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        const uint32_t hj = __float_as_uint(pj.w);
        const float2 pp = pair[ti * nt + min(hj >> 28, nt - 1u)];
        const float inv_r = rsqrtf(r2);
        const float r = r2 * inv_r;
        const float wr = 1.0f - r;
        const float ex = dx * inv_r, ey = dy * inv_r, ez = dz * inv_r;
        const float rdotv = ex * (vh.x - vj.x) + ey * (vh.y - vj.y) + ez * (vh.z - vj.z);
        const float sg = pp.y * wr;
        const float u = hash_u(th_lo, th_hi, hh, hj);
        const float scaled = pp.x * wr - sg * sg * rdotv + (sg * scale) * u;
        fx += ex * scaled;
        fy += ey * scaled;
        fz += ez * scaled;
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
    float fx = 0.f, fy = 0.f, fz = 0.f;
    int n = 0;
    for (int ddx = -1; ddx <= 1; ddx++) {
        const float gx = slab_gap(ph.x, ddx);
        const int nx = wrap_index(c[0] + ddx, w.L[0]);
        const float ax = ph.x - (float)ddx;
        for (int ddy = -1; ddy <= 1; ddy++) {
            const float gy = slab_gap(ph.y, ddy);
            const float gxy = gx * gx + gy * gy;
            if (gxy >= PRUNE) continue;
            const int ny = wrap_index(c[1] + ddy, w.L[1]);
            const float ay = ph.y - (float)ddy;
            const uint32_t row = w.cell_base + ((uint32_t)nx * (uint32_t)w.L[1] + (uint32_t)ny) * (uint32_t)w.L[2];
            for (int ddz = -1; ddz <= 1; ddz++) {
                const float gz = slab_gap(ph.z, ddz);
                if (gxy + gz * gz >= PRUNE) continue;
                const int nz = wrap_index(c[2] + ddz, w.L[2]);
                const float az = ph.z - (float)ddz;
                const uint32_t nc = row + (uint32_t)nz;
                const uint32_t j1 = start[nc + 1];
                const uint8_t dpk = (uint8_t)pack_dir(ddx, ddy, ddz);
                for (uint32_t j = start[nc]; j < j1; j++) {
                    const float4 pj = pos[j];
                    const float dx = ax - pj.x, dy = ay - pj.y, dz = az - pj.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < 1.0f && r2 >= min2) {
                        if (n == cap) {
                            list_forces32(pos, vel, s_j, s_dir, n, ph, vh, ti, nt, pair, th_lo,
                                          th_hi, scale, fx, fy, fz);
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
    list_forces32(pos, vel, s_j, s_dir, n, ph, vh, ti, nt, pair, th_lo, th_hi, scale, fx, fy, fz);
    F[0] = fx;
    F[1] = fy;
    F[2] = fz;
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
        const float dt = (float)w.dt, hdt = 0.5f * dt, hdt2 = 0.5f * dt * dt;
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
        float o[3] = {ph.x, ph.y, ph.z};
        if (!(__float_as_uint(ph.w) & (1u << 27)))  // polymer bead: bonds
            bond_forces32(a, w, a.ids[s], c, o, F, err);
        // update_mom (dpd_maths_core_half_step.hpp:51-61)
        float v[3] = {vh.x + F[0] * hdt, vh.y + F[1] * hdt, vh.z + F[2] * hdt};
        if (FINAL) {
            ((float4 *)a.velB)[s] = make_float4(v[0], v[1], v[2], 0.f);
            ((float4 *)a.frc)[s] = make_float4(F[0], F[1], F[2], 0.f);
            if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) err |= ERR_NONFINITE;
        } else {
            const uint32_t key = advance_position(w, dt, hdt2, c, o, v, F, err);
            const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
            ((float4 *)a.posB)[s] = make_float4(o[0], o[1], o[2], ph.w);
            ((float4 *)a.velB)[s] = make_float4(v[0] + F[0] * hdt, v[1] + F[1] * hdt, v[2] + F[2] * hdt, 0.f);
            a.keyrank[s] = make_uint2(key, rank);
        }
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
        const float v[3] = {vh.x, vh.y, vh.z};
        const float F[3] = {fh.x, fh.y, fh.z};
        const uint32_t key = advance_position(w, dt, hdt2, c, o, v, F, err);
        const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
        ((float4 *)a.posB)[s] = make_float4(o[0], o[1], o[2], ph.w);
        ((float4 *)a.velB)[s] = make_float4(v[0] + F[0] * hdt, v[1] + F[1] * hdt, v[2] + F[2] * hdt, 0.f);
        a.keyrank[s] = make_uint2(key, rank);
        if (err) atomicOr(&a.worlds[tl.world].err, err);
    }
}

// Attach: id-ordered FP64 staging (x, v, f) -> B in slot = id order, with cell counts.
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
    const double *st = a.staging + 9 * (size_t)g;
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
    ((float4 *)a.velB)[g] = make_float4((float)st[3], (float)st[4], (float)st[5], 0.f);
    ((float4 *)a.frcB)[g] = make_float4((float)st[6], (float)st[7], (float)st[8], 0.f);
    a.ids[g] = g;
    a.keyrank[g] = make_uint2(key, rank);
}

__global__ void k_finish32(KArgs a)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.n_beads) ((float4 *)a.velA)[s] = ((const float4 *)a.velB)[s];
    if (blockIdx.x == 0)
        for (uint32_t w = threadIdx.x; w < a.n_worlds; w += blockDim.x) a.worlds[w].t += 1;
}

// Rest state -> id-ordered FP64 staging (x, v, f): x = cell + offset exactly.
__global__ void __launch_bounds__(TILE_BEADS) k_unsort32(KArgs a)
{
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        const uint32_t s = tl.slot_begin + threadIdx.x;
        if (s >= tl.slot_end) continue;
        const WorldDev &w = a.worlds[tl.world];
        const float4 p = ((const float4 *)a.posA)[s];
        const float4 v = ((const float4 *)a.velA)[s];
        const float4 f = ((const float4 *)a.frc)[s];
        int c[3];
        decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
        double *st = a.staging + 9 * (size_t)a.ids[s];
        st[0] = (double)c[0] + (double)p.x;
        st[1] = (double)c[1] + (double)p.y;
        st[2] = (double)c[2] + (double)p.z;
        st[3] = v.x;
        st[4] = v.y;
        st[5] = v.z;
        st[6] = f.x;
        st[7] = f.y;
        st[8] = f.z;
    }
}

// =======================================================================================
// Brick kernel: shared-memory staged, warp-per-cell pair forces.
//
// A block takes one brick of cells (nominally 4x4x4) and stages the brick plus its one-cell
// halo -- (bx+2)(by+2)(bz+2) cells, z fastest -- into shared memory with coalesced float4
// loads: for each (x, y) halo row the cells z0-1 .. z0+bz are consecutive cells, so the row
// is one or (at a periodic wrap) a few contiguous runs of sorted slots.  Staged beads keep
// the halo cell order, so the 3 cells (dz = -1, 0, +1) of any neighbour row are one
// contiguous range of staged beads.
//
// Each warp then takes home cells.  For a home cell with nh beads and M beads in its 27
// neighbour cells, the nh*M candidate pairs (home-major, then the neighbour rows in the
// reference's direction order, then bead order) are tested 32 at a time, one pair per lane;
// the pairs with r^2 in [MIN_DISTANCE_CUTOFF^2, 1) are compacted with a warp ballot into a
// queue, and each full queue of 32 is evaluated one pair per lane.  A segmented shuffle scan
// over the queue sums the forces of each home bead; the sum order is a fixed function of the
// data, so the kernel is deterministic.  A final thread-per-bead pass adds bond forces and
// integrates.
// =======================================================================================

constexpr int BRICK_THREADS = 128;
constexpr int BRICK_WARPS = BRICK_THREADS / 32;
constexpr int QUEUE_CAP = 64;
constexpr int HOME_MAX = 32;

struct BrickSmem {
    float4 pos[BRICK_MAX_BEADS];
    float4 vel[BRICK_MAX_BEADS];
    float fx[BRICK_MAX_BEADS], fy[BRICK_MAX_BEADS], fz[BRICK_MAX_BEADS];
    uint32_t hstart[BRICK_HALO_CELLS + 1];  // staged index of each halo cell's first bead
    uint32_t hslot[BRICK_HALO_CELLS];       // global slot of each halo cell's first bead
    uint32_t queue[BRICK_WARPS][QUEUE_CAP];
    uint4 rowtab[BRICK_WARPS][9];
    float fh[BRICK_WARPS][3][HOME_MAX];
    uint32_t wsum[BRICK_WARPS];
    uint32_t home_rows[BRICK_X * BRICK_Y + 1];  // prefix of home beads per (x, y) row
    float2 pair[MAX_PAIR];
    WorldCache wc;
};

// One DPD pair force (calc_force, dpd_maths_core_half_step.hpp:69-157) on the home bead:
// conservative a (1-r), dissipative -gamma w^2 (e.dv), random sigma w sqrt(24/dt) u, along e.
__device__ __forceinline__ void dpd_pair32(float dx, float dy, float dz, float r2, const float4 vi,
                                           const float4 vj, uint32_t hi, uint32_t hj, float2 pp,
                                           uint32_t th_lo, uint32_t th_hi, float scale, float &fx,
                                           float &fy, float &fz)
{
    const float inv_r = rsqrtf(r2);
    const float r = r2 * inv_r;
    const float wr = 1.0f - r;
    const float ex = dx * inv_r, ey = dy * inv_r, ez = dz * inv_r;
    const float rdotv = ex * (vi.x - vj.x) + ey * (vi.y - vj.y) + ez * (vi.z - vj.z);
    const float sg = pp.y * wr;
    const float u = hash_u(th_lo, th_hi, hi, hj);
    const float scaled = pp.x * wr - sg * sg * rdotv + (sg * scale) * u;
    fx = ex * scaled;
    fy = ey * scaled;
    fz = ez * scaled;
}

// Evaluate queue entries [0, n) of this warp (n <= 32), one per lane, and add each home
// bead's segment sum to fh.
__device__ __forceinline__ void brick_eval_queue(BrickSmem &S, int warp, int lane, int n,
                                                 uint32_t h0, uint32_t nt, uint32_t th_lo,
                                                 uint32_t th_hi, float scale)
{
    float fx = 0.f, fy = 0.f, fz = 0.f;
    uint32_t key = 0xffffffffu;
    if (lane < n) {
        const uint32_t e = S.queue[warp][lane];
        const uint32_t j = e & 2047u, i = (e >> 11) & 31u, d = e >> 16;
        const float4 pi = S.pos[h0 + i], vi = S.vel[h0 + i];
        const float4 pj = S.pos[j], vj = S.vel[j];
        const float dx = (pi.x - (float)((int)(d & 3u) - 1)) - pj.x;
        const float dy = (pi.y - (float)((int)((d >> 2) & 3u) - 1)) - pj.y;
        const float dz = (pi.z - (float)((int)((d >> 4) & 3u) - 1)) - pj.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        const uint32_t hi = __float_as_uint(pi.w), hj = __float_as_uint(pj.w);
        const float2 pp = S.pair[min(hi >> 28, nt - 1u) * nt + min(hj >> 28, nt - 1u)];
        dpd_pair32(dx, dy, dz, r2, vi, vj, hi, hj, pp, th_lo, th_hi, scale, fx, fy, fz);
        key = i;
    }
    // segmented inclusive scan by key (keys are non-decreasing along the queue)
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float ux = __shfl_up_sync(0xffffffffu, fx, off);
        const float uy = __shfl_up_sync(0xffffffffu, fy, off);
        const float uz = __shfl_up_sync(0xffffffffu, fz, off);
        const uint32_t uk = __shfl_up_sync(0xffffffffu, key, off);
        if (lane >= off && uk == key) {
            fx += ux;
            fy += uy;
            fz += uz;
        }
    }
    const uint32_t next = __shfl_down_sync(0xffffffffu, key, 1);
    if (lane < n && (lane == n - 1 || next != key)) {
        S.fh[warp][0][key] += fx;
        S.fh[warp][1][key] += fy;
        S.fh[warp][2][key] += fz;
    }
    __syncwarp();
}

// Integration of one home bead after its force is known: bonds, update_mom and either the
// final write or the next update_pos with the cell count.
template <int FINAL>
__device__ __forceinline__ void integrate32(const KArgs &a, const WorldDev &w, uint32_t world,
                                            uint32_t s, const int c[3], const float4 ph,
                                            const float4 vh, float F[3], uint32_t &err)
{
    const float dt = (float)w.dt, hdt = 0.5f * dt, hdt2 = 0.5f * dt * dt;
    float o[3] = {ph.x, ph.y, ph.z};
    if (!(__float_as_uint(ph.w) & (1u << 27))) bond_forces32(a, w, a.ids[s], c, o, F, err);
    float v[3] = {vh.x + F[0] * hdt, vh.y + F[1] * hdt, vh.z + F[2] * hdt};
    if (FINAL) {
        ((float4 *)a.velB)[s] = make_float4(v[0], v[1], v[2], 0.f);
        ((float4 *)a.frc)[s] = make_float4(F[0], F[1], F[2], 0.f);
        if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) err |= ERR_NONFINITE;
    } else {
        const uint32_t key = advance_position(w, dt, hdt2, c, o, v, F, err);
        const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
        ((float4 *)a.posB)[s] = make_float4(o[0], o[1], o[2], ph.w);
        ((float4 *)a.velB)[s] = make_float4(v[0] + F[0] * hdt, v[1] + F[1] * hdt, v[2] + F[2] * hdt, 0.f);
        a.keyrank[s] = make_uint2(key, rank);
    }
}

// Thread-per-bead pair forces straight from global memory, summed sequentially in the
// reference's order: used for a brick whose halo does not fit in shared memory.
__device__ void pair_forces32_direct(const KArgs &a, const WorldDev &w, const float2 *pair,
                                     uint32_t th_lo, uint32_t th_hi, float scale, const int c[3],
                                     const float4 ph, const float4 vh, float F[3])
{
    const float4 *__restrict__ pos = (const float4 *)a.posA;
    const float4 *__restrict__ vel = (const float4 *)a.velA;
    const uint32_t nt = w.n_types;
    const uint32_t hi = __float_as_uint(ph.w);
    const uint32_t ti = min(hi >> 28, nt - 1u);
    const float min2 = min_dist_sqr_f();
    F[0] = F[1] = F[2] = 0.f;
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
                    const float dx = (ph.x - (float)ddx) - pj.x;
                    const float dy = (ph.y - (float)ddy) - pj.y;
                    const float dz = (ph.z - (float)ddz) - pj.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < 1.0f && r2 >= min2) {
                        const uint32_t hj = __float_as_uint(pj.w);
                        float fx, fy, fz;
                        dpd_pair32(dx, dy, dz, r2, vh, vel[j], hi, hj, pair[ti * nt + min(hj >> 28, nt - 1u)],
                                   th_lo, th_hi, scale, fx, fy, fz);
                        F[0] += fx;
                        F[1] += fy;
                        F[2] += fz;
                    }
                }
            }
        }
    }
}

template <int FINAL>
__global__ void __launch_bounds__(BRICK_THREADS) k_force32_brick(KArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BrickSmem &S = *reinterpret_cast<BrickSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) S.wc.world = 0xffffffffu;
    __syncthreads();
    const float min2 = min_dist_sqr_f();
    for (uint32_t bi = blockIdx.x; bi < a.n_bricks; bi += gridDim.x) {
        const Brick br = a.bricks[bi];
        load_world(a, br.world, S.wc, S.pair);  // syncs when the world changes
        __syncthreads();
        const WorldDev &w = S.wc.w;
        const uint32_t nt = w.n_types;
        const float scale = (float)w.scale_inv_sqrt_dt;
        const uint64_t th = t_hash((uint32_t)w.t, w.seed);
        const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
        const int HX = br.bx + 2, HY = br.by + 2, HZ = br.bz + 2;
        const int HC = HX * HY * HZ;

        // ---- 1. halo cell counts, global first slots, block exclusive scan -> hstart
        uint32_t cnt2[2];
        uint32_t tsum = 0;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int hc = 2 * tid + k;
            cnt2[k] = 0;
            if (hc < HC) {
                const int hx = hc / (HY * HZ), rem = hc - hx * HY * HZ;
                const int hy = rem / HZ, hz = rem - hy * HZ;
                const int gx = wrap_index(br.x0 - 1 + hx, w.L[0]);
                const int gy = wrap_index(br.y0 - 1 + hy, w.L[1]);
                const int gz = wrap_index(br.z0 - 1 + hz, w.L[2]);
                const uint32_t c = w.cell_base + ((uint32_t)gx * (uint32_t)w.L[1] + (uint32_t)gy) * (uint32_t)w.L[2] + (uint32_t)gz;
                const uint32_t s0 = a.start[c];
                cnt2[k] = a.start[c + 1] - s0;
                S.hslot[hc] = s0;
            }
            tsum += cnt2[k];
        }
        uint32_t inc = tsum;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += y;
        }
        if (lane == 31) S.wsum[warp] = inc;
        __syncthreads();
        uint32_t woff = 0;
        for (int k = 0; k < warp; k++) woff += S.wsum[k];
        uint32_t total = 0;
        for (int k = 0; k < BRICK_WARPS; k++) total += S.wsum[k];
        {
            uint32_t run = woff + inc - tsum;
            if (2 * tid < HC) S.hstart[2 * tid] = run;
            if (2 * tid + 1 < HC) S.hstart[2 * tid + 1] = run + cnt2[0];
            if (tid == 0) S.hstart[HC] = total;
        }
        // home rows prefix (bx*by rows of bz cells each)
        __syncthreads();
        if (tid == 0) {
            uint32_t acc = 0;
            for (int r = 0; r < br.bx * br.by; r++) {
                S.home_rows[r] = acc;
                const int lx = r / br.by, ly = r - lx * br.by;
                const int hc0 = ((lx + 1) * HY + (ly + 1)) * HZ + 1;
                acc += S.hstart[hc0 + br.bz] - S.hstart[hc0];
            }
            S.home_rows[br.bx * br.by] = acc;
        }
        __syncthreads();
        const uint32_t n_home = S.home_rows[br.bx * br.by];
        uint32_t err = 0;

        if (total > (uint32_t)BRICK_MAX_BEADS) {
            // ---- overflow: thread-per-bead straight from global memory
            for (uint32_t t = tid; t < n_home; t += BRICK_THREADS) {
                int r = 0;
                while (S.home_rows[r + 1] <= t) r++;
                const int lx = r / br.by, ly = r - lx * br.by;
                const int hc0 = ((lx + 1) * HY + (ly + 1)) * HZ + 1;
                const uint32_t s = S.hslot[hc0] + (t - S.home_rows[r]);
                const float4 ph = ((const float4 *)a.posA)[s];
                const float4 vh = ((const float4 *)a.velA)[s];
                int c[3];
                decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
                float F[3];
                pair_forces32_direct(a, w, S.pair, th_lo, th_hi, scale, c, ph, vh, F);
                integrate32<FINAL>(a, w, br.world, s, c, ph, vh, F, err);
            }
            if (err) atomicOr(&a.worlds[br.world].err, err);
            continue;
        }

        // ---- 2. stage the halo: one (x, y) halo row per warp iteration, coalesced
        for (int row = warp; row < HX * HY; row += BRICK_WARPS) {
            const int hc0 = row * HZ;
            const uint32_t base = S.hstart[hc0];
            const uint32_t len = S.hstart[hc0 + HZ] - base;
            for (uint32_t k = lane; k < len; k += 32) {
                int z = 0;
                while (S.hstart[hc0 + z + 1] - base <= k) z++;
                const uint32_t slot = S.hslot[hc0 + z] + (k - (S.hstart[hc0 + z] - base));
                S.pos[base + k] = ((const float4 *)a.posA)[slot];
                S.vel[base + k] = ((const float4 *)a.velA)[slot];
            }
        }
        __syncthreads();

        // ---- 3. pair forces, one home cell per warp
        const int n_home_cells = br.bx * br.by * br.bz;
        for (int hcell = warp; hcell < n_home_cells; hcell += BRICK_WARPS) {
            const int lx = hcell / (br.by * br.bz), rem = hcell - lx * br.by * br.bz;
            const int ly = rem / br.bz, lz = rem - ly * br.bz;
            const int hx = lx + 1, hy = ly + 1, hz = lz + 1;
            const int hc = (hx * HY + hy) * HZ + hz;
            const uint32_t h0 = S.hstart[hc];
            const uint32_t nh = S.hstart[hc + 1] - h0;
            if (nh == 0) continue;
            if (nh > HOME_MAX) {
                // A crowded cell: one lane per home bead, sequential over the neighbours.
                for (uint32_t i = lane; i < nh; i += 32) {
                    const float4 pi = S.pos[h0 + i], vi = S.vel[h0 + i];
                    const uint32_t hi = __float_as_uint(pi.w);
                    float F0 = 0.f, F1 = 0.f, F2 = 0.f;
                    for (int r = 0; r < 9; r++) {
                        const int ddx = r / 3 - 1, ddy = r % 3 - 1;
                        const int hcz = ((hx + ddx) * HY + (hy + ddy)) * HZ + hz;
                        for (int ddz = -1; ddz <= 1; ddz++) {
                            const uint32_t j1 = S.hstart[hcz + ddz + 1];
                            for (uint32_t j = S.hstart[hcz + ddz]; j < j1; j++) {
                                const float4 pj = S.pos[j];
                                const float dx = (pi.x - (float)ddx) - pj.x;
                                const float dy = (pi.y - (float)ddy) - pj.y;
                                const float dz = (pi.z - (float)ddz) - pj.z;
                                const float r2 = dx * dx + dy * dy + dz * dz;
                                if (r2 < 1.0f && r2 >= min2) {
                                    const uint32_t hj = __float_as_uint(pj.w);
                                    float fx, fy, fz;
                                    dpd_pair32(dx, dy, dz, r2, vi, S.vel[j], hi, hj,
                                               S.pair[min(hi >> 28, nt - 1u) * nt + min(hj >> 28, nt - 1u)],
                                               th_lo, th_hi, scale, fx, fy, fz);
                                    F0 += fx;
                                    F1 += fy;
                                    F2 += fz;
                                }
                            }
                        }
                    }
                    S.fx[h0 + i] = F0;
                    S.fy[h0 + i] = F1;
                    S.fz[h0 + i] = F2;
                }
                continue;
            }
            // neighbour row table: row r = (ddx + 1) * 3 + (ddy + 1), cells dz = -1, 0, +1
            uint32_t len = 0;
            if (lane < 9) {
                const int ddx = lane / 3 - 1, ddy = lane % 3 - 1;
                const int hcz = ((hx + ddx) * HY + (hy + ddy)) * HZ + hz;
                const uint32_t a0 = S.hstart[hcz - 1], c1 = S.hstart[hcz], c2 = S.hstart[hcz + 1],
                               b0 = S.hstart[hcz + 2];
                len = b0 - a0;
                S.rowtab[warp][lane] = make_uint4(a0, c1, c2, 0u);
            }
            uint32_t P = len;  // inclusive prefix over lanes 0..8
#pragma unroll
            for (int off = 1; off < 16; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, P, off);
                if (lane >= off) P += y;
            }
            const uint32_t M = __shfl_sync(0xffffffffu, P, 8);
            // exclusive prefix of rows 1..8 (P of row r-1), broadcast to all lanes
            uint32_t Pr[9];
            Pr[0] = 0;
#pragma unroll
            for (int r = 1; r < 9; r++) Pr[r] = __shfl_sync(0xffffffffu, P, r - 1);
            if (lane < HOME_MAX) {
                S.fh[warp][0][lane] = 0.f;
                S.fh[warp][1][lane] = 0.f;
                S.fh[warp][2][lane] = 0.f;
            }
            __syncwarp();
            const uint32_t pairs = nh * M;
            uint32_t ii = (uint32_t)lane / M, jj = (uint32_t)lane - ii * M;
            int qn = 0;
            for (uint32_t base = 0; base < pairs; base += 32) {
                const bool valid = base + lane < pairs;
                bool inr = false;
                uint32_t entry = 0;
                if (valid) {
                    int r = 0;
#pragma unroll
                    for (int q = 1; q < 9; q++) r += jj >= Pr[q] ? 1 : 0;
                    const uint4 rt = S.rowtab[warp][r];
                    uint32_t Prr = 0;
#pragma unroll
                    for (int q = 1; q < 9; q++) Prr = r == q ? Pr[q] : Prr;
                    const uint32_t j = rt.x + (jj - Prr);
                    const int ddx = r / 3 - 1, ddy = r % 3 - 1;
                    const int ddz = (j >= rt.y ? 1 : 0) + (j >= rt.z ? 1 : 0) - 1;
                    const float4 pi = S.pos[h0 + ii];
                    const float4 pj = S.pos[j];
                    const float dx = (pi.x - (float)ddx) - pj.x;
                    const float dy = (pi.y - (float)ddy) - pj.y;
                    const float dz = (pi.z - (float)ddz) - pj.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    inr = r2 < 1.0f && r2 >= min2;
                    entry = j | (ii << 11) | (pack_dir(ddx, ddy, ddz) << 16);
                }
                const uint32_t mask = __ballot_sync(0xffffffffu, inr);
                if (inr) S.queue[warp][qn + __popc(mask & ((1u << lane) - 1u))] = entry;
                qn += __popc(mask);
                jj += 32;
                while (jj >= M) {
                    jj -= M;
                    ii++;
                }
                __syncwarp();
                if (qn >= 32) {
                    brick_eval_queue(S, warp, lane, 32, h0, nt, th_lo, th_hi, scale);
                    const uint32_t moved = lane + 32 < qn ? S.queue[warp][lane + 32] : 0u;
                    __syncwarp();
                    if (lane + 32 < qn) S.queue[warp][lane] = moved;
                    qn -= 32;
                    __syncwarp();
                }
            }
            if (qn > 0) brick_eval_queue(S, warp, lane, qn, h0, nt, th_lo, th_hi, scale);
            if ((uint32_t)lane < nh) {
                S.fx[h0 + lane] = S.fh[warp][0][lane];
                S.fy[h0 + lane] = S.fh[warp][1][lane];
                S.fz[h0 + lane] = S.fh[warp][2][lane];
            }
            __syncwarp();
        }
        __syncthreads();

        // ---- 4. bonds + integration, one thread per home bead
        for (uint32_t t = tid; t < n_home; t += BRICK_THREADS) {
            int r = 0;
            while (S.home_rows[r + 1] <= t) r++;
            const int lx = r / br.by, ly = r - lx * br.by;
            const int hc0 = ((lx + 1) * HY + (ly + 1)) * HZ + 1;
            const uint32_t k = t - S.home_rows[r];
            const uint32_t staged = S.hstart[hc0] + k;
            const uint32_t s = S.hslot[hc0] + k;
            int z = 0;
            while (S.hstart[hc0 + z + 1] <= staged) z++;
            const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
            float F[3] = {S.fx[staged], S.fy[staged], S.fz[staged]};
            integrate32<FINAL>(a, w, br.world, s, c, S.pos[staged], S.vel[staged], F, err);
        }
        if (err) atomicOr(&a.worlds[br.world].err, err);
    }
}

}  // namespace

size_t brick_smem_bytes()
{
    return sizeof(BrickSmem);
}

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

int brick_grid_blocks(int sm_count)
{
    static int per_sm = -1;
    if (per_sm < 0) {
        const int bytes = (int)sizeof(BrickSmem);
        cudaFuncSetAttribute(k_force32_brick<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(k_force32_brick<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force32_brick<0>, BRICK_THREADS, bytes) != cudaSuccess || nb < 1)
            nb = 1;
        per_sm = nb;
    }
    return per_sm * sm_count;
}

int launch_force32(const KArgs &a, int final_step, cudaStream_t s)
{
    if (a.force_kernel == 0 && a.n_bricks > 0) {
        const size_t bytes = sizeof(BrickSmem);
        const int grid = (int)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)a.brick_grid, a.n_bricks));
        if (final_step)
            k_force32_brick<1><<<grid, BRICK_THREADS, bytes, s>>>(a);
        else
            k_force32_brick<0><<<grid, BRICK_THREADS, bytes, s>>>(a);
        return 1;
    }
    if (final_step)
        k_force32<1><<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    else
        k_force32<0><<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    return 1;
}

int launch_finish32(const KArgs &a, cudaStream_t s)
{
    k_finish32<<<(a.n_beads + 255) / 256 + 1, 256, 0, s>>>(a);
    return 1;
}

int launch_unsort32(const KArgs &a, cudaStream_t s)
{
    k_unsort32<<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    return 1;
}

}  // namespace pdpd
