// FP64 engine kernels.
//
// Same pipeline as the FP32 engine, but with absolute FP64 positions in [0, L) and every
// floating-point operation in the order the reference's FP64 half-step engine performs it
// (naive_dpd_engine_half_step.hpp, dpd_maths_core_half_step.hpp).  This translation unit is
// compiled with -fmad=false, so no multiply-add is fused; with the canonical cell order
// (ascending bead id inside a cell) each bead's force is summed in the reference's order and
// the trajectory is bit-identical to the reference's.
//
// State per bead (sorted): pos = (x, y, z, hash as the low bits of w), vel = (v, 0),
// frc = (f, 0).
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/pdpd_gpu.h"
#include "pdpd_device.cuh"

namespace pdpd {
namespace {

constexpr int MAX_PAIR = 256;

struct WorldCache {
    WorldDev w;
    uint32_t world;
};

__device__ __forceinline__ uint32_t hash_of(const Vec4d &p)
{
    return (uint32_t)__double_as_longlong(p.w);
}

__device__ __forceinline__ void load_world(const KArgs &a, uint32_t world, WorldCache &wc,
                                           Vec2d *s_pair)
{
    if (wc.world != world) {
        __syncthreads();
        if (threadIdx.x == 0) {
            wc.w = a.worlds[world];
            wc.world = world;
        }
        __syncthreads();
        const uint32_t np = wc.w.n_types * wc.w.n_types;
        const Vec2d *pair = (const Vec2d *)a.pair;
        for (uint32_t i = threadIdx.x; i < np && i < MAX_PAIR; i += blockDim.x)
            s_pair[i] = pair[wc.w.param_base + i];
        __syncthreads();
    }
}

// update_pos (dpd_maths_core_half_step.hpp:22-49): x' = (x + v dt) + f (dt dt / 2), with the
// reference's single periodic wrap.  Returns the global cell of x'.
__device__ __forceinline__ uint32_t advance_position64(const WorldDev &w, double dt, double hdt2,
                                                       double x[3], const double v[3],
                                                       const double f[3], uint32_t &err)
{
    int c[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double L = (double)w.L[d];
        double xn = x[d] + v[d] * dt + f[d] * hdt2;
        if (xn < 0) {
            xn += L;
            if (xn == L) xn = 0;
        } else if (xn >= L) {
            xn -= L;
        }
        if (!(xn >= 0.0 && xn < L)) {  // moved more than a box, or non-finite
            err |= ERR_OUT_OF_BOX;
            xn = 0.0;
        }
        x[d] = xn;
        c[d] = (int)floor(xn);
    }
    return w.cell_base + ((uint32_t)c[0] * (uint32_t)w.L[1] + (uint32_t)c[1]) * (uint32_t)w.L[2] +
           (uint32_t)c[2];
}

// calc_distance_from_to (naive_dpd_engine_half_step.hpp:198-209).
__device__ __forceinline__ void distance_from_to(const WorldDev &w, const double base[3],
                                                 const double other[3], double res[3])
{
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double len = (double)w.L[i];
        const double dx = other[i] - base[i];
        const int wrap_neg = dx > len * 0.5;
        const int wrap_pos = dx < -len * 0.5;
        res[i] = dx + (double)(wrap_pos - wrap_neg) * len;
    }
}

__device__ __forceinline__ void load_x(const Vec4d *__restrict__ pos, uint32_t slot, double x[3])
{
    const Vec4d p = pos[slot];
    x[0] = p.x;
    x[1] = p.y;
    x[2] = p.z;
}

// Bond terms of one bead, one per row of its CSR (Hookean bonds, then angle bonds), each
// evaluated exactly as update_hookean_bond / update_angle_bond
// (naive_dpd_engine_half_step.hpp:426-483) and calc_angle_force
// (dpd_maths_core_half_step.hpp:177-229), and stored with the sign it is added with: the
// force kernel adds the rows in order after the pair forces (F - t == F + (-t) in IEEE
// arithmetic), which is the reference's order of additions to the bead's force.
__device__ void bond_terms64(const KArgs &a, const WorldDev &w, uint32_t id, const double xs[3],
                             uint32_t &err)
{
    Vec4d *out = (Vec4d *)a.bterm;
    const Vec4d *pos = (const Vec4d *)a.posA;
    const Vec4d *prm_tab = (const Vec4d *)a.bond_params;
    const uint32_t r0 = a.bond_row[id], r1 = a.bond_row[id + 1];
    for (uint32_t r = r0; r < r1; r++) {
        const BondTerm bt = a.bond_terms[r];
        const Vec4d prm = prm_tab[bt.param];
        const uint32_t kind = bt.meta & 0xffu, role = bt.meta >> 8;
        double xa[3], xb[3];
        load_x(pos, a.slot_of_id[bt.a], xa);
        if (kind == 0) {
            const double *xh = role == 0 ? xs : xa;
            const double *xt = role == 0 ? xa : xs;
            double dx[3];
            distance_from_to(w, xh, xt, dx);
            const double dr = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
            if (dr > 2.0) err |= ERR_BOND_SNAPPED;
            const double dr0 = prm.y - dr;
            const double hookean_force = prm.x * dr0;
            const double s = hookean_force / dr;
            double t[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const double fd = dx[d] * s;
                t[d] = role == 0 ? -fd : fd;
            }
            out[r] = Vec4d{t[0], t[1], t[2], 0.0};
        } else {
            load_x(pos, a.slot_of_id[bt.b], xb);
            const double *xh = role == 0 ? xs : xa;
            const double *xm = role == 0 ? xa : (role == 1 ? xs : xb);
            const double *xt = role == 2 ? xs : xb;
            double first[3], second[3];
            distance_from_to(w, xh, xm, first);
            distance_from_to(w, xm, xt, second);
            const double r01 = sqrt(first[0] * first[0] + first[1] * first[1] + first[2] * first[2]);
            const double r12 = sqrt(second[0] * second[0] + second[1] * second[1] + second[2] * second[2]);
            const double kappa = prm.x, cos_theta0 = prm.y, sin_theta0 = prm.z;
            double hf[3] = {0, 0, 0}, tf[3] = {0, 0, 0}, mf[3] = {0, 0, 0};
            const double mag_product = r01 * r12;
            if (mag_product > 0.0001) {
                const double b1_mag_sq = r01 * r01;
                const double b2_mag_sq = r12 * r12;
                const double b1_dot_b2 = first[0] * second[0] + first[1] * second[1] + first[2] * second[2];
                const double p1 = b1_dot_b2 / b1_mag_sq;
                const double p2 = b1_dot_b2 / b2_mag_sq;
                const double cos_phi_sq = p1 * p2;
                double force_mag = kappa / mag_product;
                if (fabs(b1_dot_b2) > 0.000001 && sin_theta0 > 0) {
                    const double inv_prefactor = 1.0 / sqrt(1.0 / cos_phi_sq - 1.0);
                    force_mag = force_mag * (cos_theta0 - sin_theta0 * inv_prefactor);
                }
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    hf[d] = (first[d] * p1 - second[d]) * force_mag;
                    tf[d] = (first[d] - second[d] * p2) * force_mag;
                    mf[d] = -(hf[d] + tf[d]);
                }
            }
            double t[3];
#pragma unroll
            for (int d = 0; d < 3; d++) t[d] = role == 0 ? hf[d] : (role == 1 ? mf[d] : tf[d]);
            out[r] = Vec4d{t[0], t[1], t[2], 0.0};
        }
    }
}

constexpr int LIST_MAX = 32;

// make_relative_cell_pos (naive_dpd_engine_half_step.hpp:181-196) for one direction:
// neighbour cell and the periodic shift of its beads (+L, -L or +0.0: the values the
// reference's (is_right - is_left) * L takes, chosen without arithmetic).
__device__ __forceinline__ uint32_t neighbour64(const WorldDev &w, const int c[3], const int dir[3],
                                                const double Ld[3], double delta[3])
{
    int op[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int raw = c[i] + dir[i];
        const int is_left = raw < 0;
        const int is_right = raw == w.L[i];
        op[i] = raw + (is_left - is_right) * w.L[i];
        delta[i] = is_right ? Ld[i] : (is_left ? -Ld[i] : 0.0);
    }
    return w.cell_base + ((uint32_t)op[0] * (uint32_t)w.L[1] + (uint32_t)op[1]) * (uint32_t)w.L[2] +
           (uint32_t)op[2];
}

// calc_force's terms of one in-range pair (dpd_maths_core_half_step.hpp:69-157, kappa = 0,
// r0 = 0.5), each operation in the reference's order: the force pass adds e * scaled, and the
// pair log (k_pair_log64) records the terms the reference's ForceLogging logs.
struct PairTerms64 {
    double e[3], wr, sqrt_gammap, u, con, diss, rand_scale, rand, scaled;
};

__device__ __forceinline__ PairTerms64 pair_terms64(double dx0, double dx1, double dx2, double dr,
                                                    const Vec2d pp, const Vec4d &vh, const Vec4d &vj,
                                                    uint32_t hh, uint32_t hj, uint32_t th_lo,
                                                    uint32_t th_hi, double scale_inv_sqrt_dt)
{
    PairTerms64 q;
    const double kappa = 0.0, r0 = 0.5;
    const double inv_dr = 1.0 / dr;
    const double dv0 = vh.x - vj.x, dv1 = vh.y - vj.y, dv2 = vh.z - vj.z;
    q.wr = 1.0 - dr;
    q.con = pp.x * q.wr;
    q.e[0] = dx0 * inv_dr;
    q.e[1] = dx1 * inv_dr;
    q.e[2] = dx2 * inv_dr;
    const double rdotv = q.e[0] * dv0 + q.e[1] * dv1 + q.e[2] * dv2;
    q.sqrt_gammap = pp.y * q.wr;
    q.diss = -q.sqrt_gammap * q.sqrt_gammap * rdotv;
    q.u = (double)hash_u(th_lo, th_hi, hh, hj);
    q.rand_scale = q.sqrt_gammap * scale_inv_sqrt_dt;
    q.rand = q.rand_scale * q.u;
    const double dr0 = r0 - dr;
    const double hookean_force = kappa * dr0;
    q.scaled = q.con + q.diss + q.rand + hookean_force;
    return q;
}

// Phase 2: the reference's pair filter and calc_force (dpd_maths_core_half_step.hpp:69-157,
// kappa = 0, r0 = 0.5) for the listed candidates, in list order, each operation in the
// reference's order.  The list holds every neighbour that can be in range (the walk's
// prefilter is conservative); the exact FP64 test here keeps dr2 < 1 and dr2 >= 1e-18
// (naive_dpd_engine_half_step.hpp:404-411), so the terms added are the reference's.
__device__ __forceinline__ void list_forces64(const Vec4d *__restrict__ pos,
                                              const Vec4d *__restrict__ vel,
                                              const uint32_t *__restrict__ s_j,
                                              const uint8_t *__restrict__ s_dir, int col, int n,
                                              const WorldDev &w, const int c[3], const double Ld[3],
                                              const double xh[3], const Vec4d &vh, uint32_t hh,
                                              uint32_t ti, const Vec2d *__restrict__ pair,
                                              const Vec2d *__restrict__ cp, uint32_t hc,
                                              const uint32_t *__restrict__ cellg,
                                              uint32_t th_lo, uint32_t th_hi,
                                              double scale_inv_sqrt_dt, double F[3])
{
    const uint32_t nt = w.n_types;
    const uint32_t n2 = nt * nt;
    const double min2 = (double)min_dist_sqr_f();
    for (int k = 0; k < n; k++) {
        const uint32_t j = s_j[k * TILE_BEADS + col];
        const uint32_t d = s_dir[k * TILE_BEADS + col];
        const int dir[3] = {(int)(d & 3u) - 1, (int)((d >> 2) & 3u) - 1, (int)((d >> 4) & 3u) - 1};
        double delta[3];
        neighbour64(w, c, dir, Ld, delta);
        const Vec4d pj = pos[j];
        const double obx = pj.x + delta[0], oby = pj.y + delta[1], obz = pj.z + delta[2];
        const double dx0 = xh[0] - obx, dx1 = xh[1] - oby, dx2 = xh[2] - obz;
        const double dr2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
        if (dr2 >= 1 || dr2 < min2) continue;
        const Vec4d vj = vel[j];
        const double dr = sqrt(dr2);
        const uint32_t hj = hash_of(pj);
        const uint32_t pk = ti * nt + min(hj >> 28, nt - 1u);
        Vec2d pp = pair[pk];
        if (cp) {  // spatial strengths: mean of the two beads' cell values (half_merge.hpp:570-583)
            const Vec2d h = cp[(size_t)hc * n2 + pk], o = cp[(size_t)(cellg[j] - w.cell_base) * n2 + pk];
            pp.x = (h.x + o.x) * 0.5;
            pp.y = (h.y + o.y) * 0.5;
        }
        const PairTerms64 q = pair_terms64(dx0, dx1, dx2, dr, pp, vh, vj, hh, hj, th_lo, th_hi, scale_inv_sqrt_dt);
        F[0] = F[0] + q.e[0] * q.scaled;
        F[1] = F[1] + q.e[1] * q.scaled;
        F[2] = F[2] + q.e[2] * q.scaled;
    }
}

// The home bead's data the list evaluation needs.
struct Home64 {
    double x[3];
    Vec4d v;
    uint32_t hash, ti, hc;
    int c[3];
};

__device__ __forceinline__ Home64 home64(const KArgs &a, const WorldDev &w, uint32_t s)
{
    Home64 h;
    const Vec4d p = ((const Vec4d *)a.posA)[s];
    h.x[0] = p.x;
    h.x[1] = p.y;
    h.x[2] = p.z;
    h.v = ((const Vec4d *)a.velA)[s];
    h.hash = hash_of(p);
    h.ti = min(h.hash >> 28, w.n_types - 1u);
    h.hc = a.cellg[s] - w.cell_base;
    decode_cell(h.hc, w.L, h.c[0], h.c[1], h.c[2]);
    return h;
}

__device__ __forceinline__ void eval_list64(const KArgs &a, const WorldDev &w, const Vec2d *s_pair,
                                            const uint32_t *s_j, const uint8_t *s_dir, int col, int n,
                                            const Home64 &h, uint32_t th_lo, uint32_t th_hi, double F[3])
{
    const double Ld[3] = {(double)w.L[0], (double)w.L[1], (double)w.L[2]};
    const Vec2d *cp = w.spatial ? (const Vec2d *)a.cellpair + w.cellpair_base : nullptr;
    list_forces64((const Vec4d *)a.posA, (const Vec4d *)a.velA, s_j, s_dir, col, n, w, h.c, Ld, h.x, h.v,
                  h.hash, h.ti, s_pair, cp, h.hc, a.cellg, th_lo, th_hi, w.scale_inv_sqrt_dt, F);
}

__device__ __forceinline__ float slab_gap32(float o, int d)
{
    return d == 0 ? 0.0f : (d < 0 ? o : 1.0f - o);
}

// The neighbour walk of one bead: for each of the 27 directions in (-1..1)^3 order, for each
// bead of that cell in id order (the reference's update_cell_forces order,
// naive_dpd_engine_half_step.hpp:358-424), candidates are appended to the bead's list
// (column threadIdx.x); a full list is evaluated into F on the spot.  Returns the entries
// left in the list.
//
// The walk itself does no FP64 arithmetic (the GPU's FP64 pipe is the kernel's bound): it
// tests the beads' FP32 cell offsets (posf, x - floor(x) rounded to FP32, error <= 2^-25)
// against a squared distance of 1.0001, and list_forces64 applies the exact FP64 test.  The
// FP32 separation of two offsets differs from the exact one by < 3e-7 per axis, so its
// square differs by < 4e-6 for pairs in range: no neighbour with dr2 < 1 is dropped, and the
// list's in-range entries, in order, are the reference's.  Rows and cells whose nearest face
// is >= 1.0001 away (FP32 gaps of the same offsets) hold no neighbour in range.
__device__ __forceinline__ int walk64(const KArgs &a, const WorldDev &w, const Vec2d *s_pair,
                                      uint32_t *s_j, uint8_t *s_dir, int cap, uint32_t th_lo,
                                      uint32_t th_hi, const Home64 &h, const float4 oh, double F[3])
{
    const float4 *__restrict__ posf = a.posf;
    const uint32_t *__restrict__ start = a.start;
    const float PRUNE = 1.0001f;
    int n = 0;
    int dir[3];
    for (dir[0] = -1; dir[0] <= 1; dir[0]++) {
        const float gx = slab_gap32(oh.x, dir[0]);
        const float ax = oh.x - (float)dir[0];
        for (dir[1] = -1; dir[1] <= 1; dir[1]++) {
            const float gy = slab_gap32(oh.y, dir[1]);
            const float gxy = gx * gx + gy * gy;
            if (gxy >= PRUNE) continue;
            const float ay = oh.y - (float)dir[1];
            for (dir[2] = -1; dir[2] <= 1; dir[2]++) {
                const float gz = slab_gap32(oh.z, dir[2]);
                if (gxy + gz * gz >= PRUNE) continue;
                const float az = oh.z - (float)dir[2];
                int op[3];
#pragma unroll
                for (int i = 0; i < 3; i++) op[i] = wrap_index(h.c[i] + dir[i], w.L[i]);
                const uint32_t nc = w.cell_base + ((uint32_t)op[0] * (uint32_t)w.L[1] + (uint32_t)op[1]) * (uint32_t)w.L[2] + (uint32_t)op[2];
                const uint32_t j1 = start[nc + 1];
                const uint8_t dpk = (uint8_t)((dir[0] + 1) | ((dir[1] + 1) << 2) | ((dir[2] + 1) << 4));
                for (uint32_t j = start[nc]; j < j1; j++) {
                    const float4 q = posf[j];
                    const float ex = ax - q.x, ey = ay - q.y, ez = az - q.z;
                    if (ex * ex + ey * ey + ez * ez >= PRUNE) continue;
                    if (n == cap) {
                        eval_list64(a, w, s_pair, s_j, s_dir, threadIdx.x, n, h, th_lo, th_hi, F);
                        n = 0;
                    }
                    s_j[n * TILE_BEADS + threadIdx.x] = j;
                    s_dir[n * TILE_BEADS + threadIdx.x] = dpk;
                    n++;
                }
            }
        }
    }
    return n;
}

// Pair log (pdpd_log_pair_terms): for each sorted slot whose bead is in the sorted id list
// sel, every in-range pair of the 27-direction walk in the reference's order
// (naive_dpd_engine_half_step.hpp:300-424), with calc_force's terms as the reference's
// ForceLogging records them (dpd_maths_core_half_step.hpp:131-153).  Count pass (out null):
// counts[k] = pairs of sel[k]; write pass: the records of sel[k] at out + offs[k].
__global__ void k_pair_log64(KArgs a, const uint32_t *__restrict__ sel, uint32_t n_sel,
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
    const Home64 h = home64(a, w, s);
    const uint64_t th = t_hash((uint32_t)w.t, w.seed);
    const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
    const double Ld[3] = {(double)w.L[0], (double)w.L[1], (double)w.L[2]};
    const Vec2d *pair = (const Vec2d *)a.pair + w.param_base;
    const Vec2d *cp = w.spatial ? (const Vec2d *)a.cellpair + w.cellpair_base : nullptr;
    const Vec4d *pos = (const Vec4d *)a.posA, *vel = (const Vec4d *)a.velA;
    const uint32_t nt = w.n_types, n2 = nt * nt;
    const double min2 = (double)min_dist_sqr_f();
    uint32_t n = 0;
    int dir[3];
    for (dir[0] = -1; dir[0] <= 1; dir[0]++)
        for (dir[1] = -1; dir[1] <= 1; dir[1]++)
            for (dir[2] = -1; dir[2] <= 1; dir[2]++) {
                double delta[3];
                const uint32_t nc = neighbour64(w, h.c, dir, Ld, delta);
                for (uint32_t j = a.start[nc]; j < a.start[nc + 1]; j++) {
                    const Vec4d pj = pos[j];
                    const double obx = pj.x + delta[0], oby = pj.y + delta[1], obz = pj.z + delta[2];
                    const double dx0 = h.x[0] - obx, dx1 = h.x[1] - oby, dx2 = h.x[2] - obz;
                    const double dr2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
                    if (dr2 >= 1 || dr2 < min2) continue;
                    if (out) {
                        const Vec4d vj = vel[j];
                        const double dr = sqrt(dr2);
                        const uint32_t hj = hash_of(pj);
                        const uint32_t pk = h.ti * nt + min(hj >> 28, nt - 1u);
                        Vec2d pp = pair[pk];
                        if (cp) {
                            const Vec2d hv = cp[(size_t)h.hc * n2 + pk], ov = cp[(size_t)(a.cellg[j] - w.cell_base) * n2 + pk];
                            pp.x = (hv.x + ov.x) * 0.5;
                            pp.y = (hv.y + ov.y) * 0.5;
                        }
                        const PairTerms64 q =
                            pair_terms64(dx0, dx1, dx2, dr, pp, h.v, vj, h.hash, hj, th_lo, th_hi, w.scale_inv_sqrt_dt);
                        PairLogRec &r = out[offs[k] + n];
                        r.t = w.t;
                        r.home_id = id;
                        r.other_id = a.ids[j];
                        r.home_hash = h.hash;
                        r.other_hash = hj;
                        r.dx[0] = dx0;
                        r.dx[1] = dx1;
                        r.dx[2] = dx2;
                        r.dr = dr;
                        r.inv_root_dt = w.scale_inv_sqrt_dt;
                        r.gammap = q.sqrt_gammap * q.sqrt_gammap;
                        r.rng = q.u;
                        r.con = q.con;
                        r.diss = q.diss;
                        r.rng_scale = q.rand_scale;
                        r.rand = q.rand;
                        const double dpd_force = q.con + q.diss + q.rand;
                        for (int d = 0; d < 3; d++) r.f[d] = q.e[d] * dpd_force;
                    }
                    n++;
                }
            }
    if (!out) counts[k] = n;
}

// Lists of a tile, re-dealt to threads by length (see k_force64).
struct Balance64 {
    uint32_t hist[LIST_MAX + 2];
    uint8_t n[TILE_BEADS];
    uint8_t perm[TILE_BEADS];
    double f[3][TILE_BEADS];
};

// Bond terms of every polymer bead, one thread per bead (a compact list of the few bonded
// beads), stored by CSR row for the force kernel: the lanes of a warp all do bond work,
// instead of one or two lanes of a pair-force warp.
__global__ void __launch_bounds__(128) k_bonds64(KArgs a)
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
    const Vec4d p = ((const Vec4d *)a.posA)[a.slot_of_id[id]];
    const double x[3] = {p.x, p.y, p.z};
    uint32_t err = 0;
    bond_terms64(a, w, id, x, err);
    if (err) atomicOr(&a.worlds[lo].err, err);
}

// Force pass of a tile of TILE_BEADS sorted beads, one thread per bead:
//   1. each thread walks its bead's neighbours into its list;
//   2. the lists are counting-sorted by length and thread t evaluates list perm[t], so the
//      lanes of a warp evaluate lists of about the same length (the FP64 pipe executes an
//      instruction for the whole warp whatever its active lanes); every list is still
//      summed by one thread in its own order, so the result is the same;
//   3. each thread adds its bead's bond terms (k_bonds64) in CSR order, then update_mom and
//      either the final write or the next update_pos with its cell count.
template <int FINAL>
__global__ void __launch_bounds__(TILE_BEADS) k_force64(KArgs a)
{
    __shared__ Vec2d s_pair[MAX_PAIR];
    __shared__ uint32_t s_j[LIST_MAX * TILE_BEADS];
    __shared__ uint8_t s_dir[LIST_MAX * TILE_BEADS];
    __shared__ WorldCache wc;
    __shared__ Balance64 B;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) wc.world = 0xffffffffu;
    __syncthreads();
    const int cap = (a.list_capacity > 0 && a.list_capacity < LIST_MAX) ? a.list_capacity : LIST_MAX;
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        load_world(a, tl.world, wc, s_pair);
        const WorldDev &w = wc.w;
        const uint32_t s = tl.slot_begin + tid;
        const bool act = s < tl.slot_end;
        const uint64_t th = t_hash((uint32_t)w.t, w.seed);
        const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
        double F[3] = {0.0, 0.0, 0.0};
        int n = 0;
        if (act) {
            const Home64 h = home64(a, w, s);
            n = walk64(a, w, s_pair, s_j, s_dir, cap, th_lo, th_hi, h, a.posf[s], F);
        }
        if (tid < LIST_MAX + 2) B.hist[tid] = 0u;
        B.n[tid] = (uint8_t)n;
        B.f[0][tid] = F[0];
        B.f[1][tid] = F[1];
        B.f[2][tid] = F[2];
        __syncthreads();
        const uint32_t rank = atomicAdd(&B.hist[n], 1u);  // n <= LIST_MAX
        __syncthreads();
        if (warp == 0) {  // exclusive prefix of the LIST_MAX + 1 bins
            const uint32_t v = B.hist[lane];
            uint32_t inc = v;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
                if (lane >= off) inc += y;
            }
            B.hist[lane] = inc - v;
            if (lane == 31) B.hist[32] = inc;
        }
        __syncthreads();
        B.perm[B.hist[n] + rank] = (uint8_t)tid;
        __syncthreads();
        {
            const int o = B.perm[tid];
            const int no = B.n[o];
            if (no > 0) {
                const Home64 h = home64(a, w, tl.slot_begin + (uint32_t)o);
                double G[3] = {B.f[0][o], B.f[1][o], B.f[2][o]};
                eval_list64(a, w, s_pair, s_j, s_dir, o, no, h, th_lo, th_hi, G);
                B.f[0][o] = G[0];
                B.f[1][o] = G[1];
                B.f[2][o] = G[2];
            }
        }
        __syncthreads();
        if (act) {
            F[0] = B.f[0][tid];
            F[1] = B.f[1][tid];
            F[2] = B.f[2][tid];
            const double dt = w.dt, hdt = dt * 0.5, hdt2 = (dt * dt) * 0.5;
            uint32_t err = 0;
            const Vec4d ph = ((const Vec4d *)a.posA)[s];
            const Vec4d vh = ((const Vec4d *)a.velA)[s];
            const uint32_t hh = hash_of(ph);
            double x[3] = {ph.x, ph.y, ph.z};
            if (!(hh & (1u << 27))) {  // polymer bead: its bond terms, in CSR order
                const uint32_t id = a.ids[s];
                const Vec4d *bt = (const Vec4d *)a.bterm;
                for (uint32_t r = a.bond_row[id]; r < a.bond_row[id + 1]; r++) {
                    const Vec4d t = bt[r];
                    F[0] = F[0] + t.x;
                    F[1] = F[1] + t.y;
                    F[2] = F[2] + t.z;
                }
            }
            // update_mom: v += f * half(dt); a stationary type's v and f are cleared instead
            // (naive_dpd_engine_half_merge.hpp:387-394), so the next update_pos leaves it in place
            double v[3] = {vh.x + F[0] * hdt, vh.y + F[1] * hdt, vh.z + F[2] * hdt};
            if ((w.stationary >> (hh >> 28)) & 1u) {
                v[0] = v[1] = v[2] = 0.0;
                F[0] = F[1] = F[2] = 0.0;
            }
            if (FINAL) {
                Vec4d vo = {v[0], v[1], v[2], 0.0};
                Vec4d fo = {F[0], F[1], F[2], 0.0};
                ((Vec4d *)a.velB)[s] = vo;
                ((Vec4d *)a.frc)[s] = fo;
                if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) err |= ERR_NONFINITE;
            } else {
                const uint32_t key = advance_position64(w, dt, hdt2, x, v, F, err);
                const uint32_t rank2 = atomicAdd(&a.cnt[key], 1u);
                Vec4d po = {x[0], x[1], x[2], ph.w};
                Vec4d vo = {v[0] + F[0] * hdt, v[1] + F[1] * hdt, v[2] + F[2] * hdt, 0.0};
                ((Vec4d *)a.posB)[s] = po;
                ((Vec4d *)a.velB)[s] = vo;
                a.keyrank[s] = make_uint2(key, rank2);
            }
            if (err) atomicOr(&a.worlds[tl.world].err, err);
        }
        __syncthreads();  // the lists and B are reused by the next tile
    }
}

__global__ void __launch_bounds__(TILE_BEADS) k_begin64(KArgs a)
{
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        const uint32_t s = tl.slot_begin + threadIdx.x;
        if (s >= tl.slot_end) continue;
        const WorldDev &w = a.worlds[tl.world];
        const double dt = w.dt, hdt = dt * 0.5, hdt2 = (dt * dt) * 0.5;
        uint32_t err = 0;
        const Vec4d ph = ((const Vec4d *)a.posA)[s];
        const Vec4d vh = ((const Vec4d *)a.velA)[s];
        const Vec4d fh = ((const Vec4d *)a.frc)[s];
        double x[3] = {ph.x, ph.y, ph.z};
        // a stationary type is not moved and keeps its v (naive_dpd_engine_half_merge.hpp:329-333)
        const bool st = (w.stationary >> (hash_of(ph) >> 28)) & 1u;
        const double v[3] = {st ? 0.0 : vh.x, st ? 0.0 : vh.y, st ? 0.0 : vh.z};
        const double F[3] = {st ? 0.0 : fh.x, st ? 0.0 : fh.y, st ? 0.0 : fh.z};
        const uint32_t key = advance_position64(w, dt, hdt2, x, v, F, err);
        const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
        Vec4d po = {x[0], x[1], x[2], ph.w};
        Vec4d vo = st ? Vec4d{vh.x, vh.y, vh.z, 0.0}
                      : Vec4d{v[0] + F[0] * hdt, v[1] + F[1] * hdt, v[2] + F[2] * hdt, 0.0};
        ((Vec4d *)a.posB)[s] = po;
        ((Vec4d *)a.velB)[s] = vo;
        a.keyrank[s] = make_uint2(key, rank);
        if (err) atomicOr(&a.worlds[tl.world].err, err);
    }
}

__global__ void k_bin64(KArgs a, const uint32_t *__restrict__ hash_in)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n_beads) return;
    uint32_t lo = 0, hi = a.n_worlds;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (a.worlds[mid].bead_base <= g) lo = mid; else hi = mid;
    }
    const WorldDev &w = a.worlds[lo];
    // rows of 9 doubles, or field-major blocks (x, v, f) of staging_n beads each
    const size_t stride = a.staging_fields ? 3 : 9, field = a.staging_fields ? 3 * (size_t)a.staging_n : 3;
    const double *st = a.staging + stride * g;
    int c[3];
    double x[3];
    uint32_t err = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double xd = st[d];
        if (!(xd >= 0.0 && xd < (double)w.L[d])) {
            err |= ERR_OUT_OF_BOX;
            xd = 0.0;
        }
        x[d] = xd;
        c[d] = (int)floor(xd);
    }
    if (err) atomicOr(&a.worlds[lo].err, err);
    const uint32_t key = w.cell_base + ((uint32_t)c[0] * (uint32_t)w.L[1] + (uint32_t)c[1]) * (uint32_t)w.L[2] + (uint32_t)c[2];
    const uint32_t rank = atomicAdd(&a.cnt[key], 1u);
    Vec4d po = {x[0], x[1], x[2], __longlong_as_double((long long)hash_in[g])};
    Vec4d vo = {st[field], st[field + 1], st[field + 2], 0.0};
    Vec4d fo = {st[2 * field], st[2 * field + 1], st[2 * field + 2], 0.0};
    ((Vec4d *)a.posB)[g] = po;
    ((Vec4d *)a.velB)[g] = vo;
    ((Vec4d *)a.frcB)[g] = fo;
    a.ids[g] = g;
    a.keyrank[g] = make_uint2(key, rank);
}

__global__ void k_finish64(KArgs a)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.n_beads) ((Vec4d *)a.velA)[s] = ((const Vec4d *)a.velB)[s];
    if (blockIdx.x == 0)
        for (uint32_t w = threadIdx.x; w < a.n_worlds; w += blockDim.x) a.worlds[w].t += 1;
}

}  // namespace

int launch_bin64(const KArgs &a, const uint32_t *hash_in, cudaStream_t s)
{
    if (a.n_beads == 0) return 0;
    k_bin64<<<(a.n_beads + 255) / 256, 256, 0, s>>>(a, hash_in);
    return 1;
}

int launch_begin64(const KArgs &a, cudaStream_t s)
{
    k_begin64<<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    return 1;
}

int launch_pair_log64(const KArgs &a, const uint32_t *sel, uint32_t n_sel, const uint32_t *offs,
                      uint32_t *counts, PairLogRec *out, cudaStream_t s)
{
    if (a.n_beads == 0 || n_sel == 0) return 0;
    k_pair_log64<<<(a.n_beads + 127) / 128, 128, 0, s>>>(a, sel, n_sel, offs, counts, out);
    return 1;
}

int launch_force64(const KArgs &a, int final_step, cudaStream_t s)
{
    int n = 0;
    if (a.n_bonded > 0) {
        k_bonds64<<<(a.n_bonded + 127) / 128, 128, 0, s>>>(a);
        n++;
    }
    if (final_step)
        k_force64<1><<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    else
        k_force64<0><<<a.grid_blocks, TILE_BEADS, 0, s>>>(a);
    return n + 1;
}

int launch_finish64(const KArgs &a, cudaStream_t s)
{
    k_finish64<<<(a.n_beads + 255) / 256 + 1, 256, 0, s>>>(a);
    return 1;
}

}  // namespace pdpd

// =======================================================================================
// Allocation-free stepping (pdpd_step_noalloc).
//
// Some callers cannot allocate device memory: code running while a CUDA stream is being
// captured into a graph (cudaMalloc is not a capturable operation), or a host framework
// that owns every device allocation through its own pool and forbids side allocations.
// For them, pdpd_step_noalloc advances one small bond-free world with the FP64 integrator
// on device arrays the caller owns, and keeps its own scratch -- the cell counts, cell
// starts, arrival ranks and the canonical bead order of the counting sort -- in the
// file-scope array g_noalloc_scratch below instead of allocating it.  Every GPU that loads
// the library holds this array (about 1.3 MB) until the process exits.  All calls share
// it: calls that overlap on the GPU (on different streams, or from different host threads
// without ordering) race on it and corrupt each other's cell lists.
//
// The arithmetic is the engine's FP64 path: update_pos, counting sort with beads in id
// order inside each cell, pair forces in the reference's direction order, update_mom,
// compiled without fused multiply-add -- so the result equals pdpd_run's bit for bit.
// =======================================================================================

namespace pdpd {
namespace {

constexpr uint32_t NA_MAX_BEADS = 65536;
constexpr uint32_t NA_MAX_CELLS = 32768;

struct NaScratch {
    uint32_t err;
    uint32_t cnt[NA_MAX_CELLS];
    uint32_t start[NA_MAX_CELLS + 1];
    uint2 keyrank[NA_MAX_BEADS];
    uint32_t tmp[NA_MAX_BEADS];
    uint32_t order[NA_MAX_BEADS];
};

struct NaParams {
    int32_t L[3];
    uint32_t n;
    uint32_t n_cells;
    uint32_t nt;
    double dt;
    double scale_inv_sqrt_dt;
    uint64_t seed;
    int64_t t;
    double pair[256][2];  // a_ij, sqrt(gamma_ij)
};

}  // namespace
}  // namespace pdpd

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(pdpd::NaScratch)];

namespace pdpd {
namespace {

// Zeroes the cell counts before each step; the error word only before a call's first step,
// so that a bead lost in any step of the call is still reported at its end.
__global__ void k_na_clear(NaScratch *S, uint32_t n_cells, int clear_err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_cells) S->cnt[i] = 0u;
    if (i == 0 && clear_err) S->err = 0u;
}

// update_pos (dpd_maths_core_half_step.hpp:22-49) and the bead's new cell and arrival rank.
__global__ void k_na_update_pos(NaParams p, NaScratch *S, double *x, double *v, double *f)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const double dt = p.dt, hdt = dt * 0.5, hdt2 = (dt * dt) * 0.5;
    int c[3];
    for (int d = 0; d < 3; d++) {
        const double L = (double)p.L[d];
        double xn = x[3 * i + d] + v[3 * i + d] * dt + f[3 * i + d] * hdt2;
        if (xn < 0) {
            xn += L;
            if (xn == L) xn = 0;
        } else if (xn >= L) {
            xn -= L;
        }
        if (!(xn >= 0.0 && xn < L)) {
            atomicOr(&S->err, (uint32_t)ERR_OUT_OF_BOX);
            xn = 0.0;
        }
        x[3 * i + d] = xn;
        c[d] = (int)floor(xn);
        v[3 * i + d] = v[3 * i + d] + f[3 * i + d] * hdt;
        f[3 * i + d] = 0.0;
    }
    const uint32_t key = ((uint32_t)c[0] * (uint32_t)p.L[1] + (uint32_t)c[1]) * (uint32_t)p.L[2] + (uint32_t)c[2];
    const uint32_t rank = atomicAdd(&S->cnt[key], 1u);
    S->keyrank[i] = make_uint2(key, rank);
}

// Exclusive scan of the cell counts in one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_na_scan(NaScratch *S, uint32_t n_cells, uint32_t n)
{
    __shared__ uint32_t wsum[32];
    const uint32_t per = (n_cells + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(n_cells, b + per);
    uint32_t tsum = 0;
    for (uint32_t k = b; k < e; k++) tsum += S->cnt[k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = tsum;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    uint32_t run = inc - tsum;
    for (int k = 0; k < warp; k++) run += wsum[k];
    for (uint32_t k = b; k < e; k++) {
        S->start[k] = run;
        run += S->cnt[k];
    }
    if (threadIdx.x == 0) S->start[n_cells] = n;
}

__global__ void k_na_place(NaScratch *S, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 kr = S->keyrank[i];
    S->tmp[S->start[kr.x] + kr.y] = i;
}

// Canonical cell order: beads of a cell in ascending id, as the reference's cell lists.
__global__ void k_na_canon(NaScratch *S, uint32_t n)
{
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const uint32_t i = S->tmp[d];
    const uint32_t key = S->keyrank[i].x;
    const uint32_t b = S->start[key], e = S->start[key + 1];
    uint32_t rank = 0;
    for (uint32_t k = b; k < e; k++) rank += S->tmp[k] < i ? 1u : 0u;
    S->order[b + rank] = i;
}

// Pair forces (update_cell_forces + calc_force, naive_dpd_engine_half_step.hpp:300-424 and
// dpd_maths_core_half_step.hpp:69-157), the same operations in the same order as
// pair_forces64 / list_forces64.
__global__ void k_na_forces(NaParams p, NaScratch *S, const double *__restrict__ x,
                            const double *__restrict__ v, double *__restrict__ f,
                            const uint32_t *__restrict__ hash)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const uint64_t th = t_hash((uint32_t)p.t, p.seed);
    const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
    const uint32_t key = S->keyrank[i].x;
    const int c[3] = {(int)(key / ((uint32_t)p.L[1] * (uint32_t)p.L[2])),
                      (int)((key / (uint32_t)p.L[2]) % (uint32_t)p.L[1]), (int)(key % (uint32_t)p.L[2])};
    const double xh[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    const double vh[3] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
    const uint32_t hh = hash[i];
    const uint32_t ti = min(hh >> 28, p.nt - 1u);
    const double min2 = (double)min_dist_sqr_f();
    double F[3] = {0.0, 0.0, 0.0};
    int dir[3];
    for (dir[0] = -1; dir[0] <= 1; dir[0]++)
        for (dir[1] = -1; dir[1] <= 1; dir[1]++)
            for (dir[2] = -1; dir[2] <= 1; dir[2]++) {
                int op[3];
                double delta[3];
                for (int k = 0; k < 3; k++) {
                    const int raw = c[k] + dir[k];
                    const int is_left = raw < 0;
                    const int is_right = raw == p.L[k];
                    op[k] = raw + (is_left - is_right) * p.L[k];
                    delta[k] = (double)(is_right - is_left) * (double)p.L[k];
                }
                const uint32_t nc = ((uint32_t)op[0] * (uint32_t)p.L[1] + (uint32_t)op[1]) * (uint32_t)p.L[2] + (uint32_t)op[2];
                const uint32_t k1 = S->start[nc + 1];
                for (uint32_t k = S->start[nc]; k < k1; k++) {
                    const uint32_t j = S->order[k];
                    const double obx = x[3 * j] + delta[0], oby = x[3 * j + 1] + delta[1], obz = x[3 * j + 2] + delta[2];
                    const double dx0 = xh[0] - obx, dx1 = xh[1] - oby, dx2 = xh[2] - obz;
                    const double dr2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
                    if (dr2 >= 1 || dr2 < min2) continue;
                    const double dr = sqrt(dr2);
                    const uint32_t hj = hash[j];
                    const uint32_t tj = min(hj >> 28, p.nt - 1u);
                    const double con_strength = p.pair[ti * p.nt + tj][0];
                    const double sqrt_diss = p.pair[ti * p.nt + tj][1];
                    const double kappa = 0.0, r0 = 0.5;
                    const double inv_dr = 1.0 / dr;
                    const double dv0 = vh[0] - v[3 * j], dv1 = vh[1] - v[3 * j + 1], dv2 = vh[2] - v[3 * j + 2];
                    const double wr = 1.0 - dr;
                    const double con_force = con_strength * wr;
                    const double e0 = dx0 * inv_dr, e1 = dx1 * inv_dr, e2 = dx2 * inv_dr;
                    const double rdotv = e0 * dv0 + e1 * dv1 + e2 * dv2;
                    const double sqrt_gammap = sqrt_diss * wr;
                    const double diss_force = -sqrt_gammap * sqrt_gammap * rdotv;
                    const double u = (double)hash_u(th_lo, th_hi, hh, hj);
                    const double rand_scale = sqrt_gammap * p.scale_inv_sqrt_dt;
                    const double rand_force = rand_scale * u;
                    const double dr0 = r0 - dr;
                    const double hookean_force = kappa * dr0;
                    const double scaled = con_force + diss_force + rand_force + hookean_force;
                    F[0] = F[0] + e0 * scaled;
                    F[1] = F[1] + e1 * scaled;
                    F[2] = F[2] + e2 * scaled;
                }
            }
    f[3 * i] = F[0];
    f[3 * i + 1] = F[1];
    f[3 * i + 2] = F[2];
}

// update_mom (dpd_maths_core_half_step.hpp:51-61).
__global__ void k_na_update_mom(NaParams p, double *v, const double *f)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const double hdt = p.dt * 0.5;
    for (int d = 0; d < 3; d++) v[3 * i + d] = v[3 * i + d] + f[3 * i + d] * hdt;
}

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
void *g_na_scratch[NA_MAX_DEVICES];

}  // namespace
}  // namespace pdpd

extern "C" int pdpd_step_noalloc(const pdpd_world *w, double *d_x, double *d_v, double *d_f,
                                 const uint32_t *d_hash, uint32_t n_steps, void *stream)
{
    using namespace pdpd;
    auto fail = [](int code, const char *msg) {
        set_thread_error(msg);
        return code;
    };
    if (!w) return fail(PDPD_E_INVALID, "pdpd_step_noalloc: no world");
    if (w->n_bonds || w->n_angles)
        return fail(PDPD_E_UNSUPPORTED, "pdpd_step_noalloc: worlds with bonds are not supported");
    if (w->n_bead_types == 0 || w->n_bead_types > 16 || !w->conservative || !w->dissipative)
        return fail(PDPD_E_INVALID, "pdpd_step_noalloc: 1..16 bead types with interaction matrices required");
    if (w->stationary)
        for (uint32_t k = 0; k < w->n_bead_types; k++)
            if (w->stationary[k]) return fail(PDPD_E_UNSUPPORTED, "Engine does not support stationary bead types.");
    if (w->cell_conservative || w->cell_dissipative)
        return fail(PDPD_E_UNSUPPORTED, "The allocation-free entry point does not support per-cell strengths.");
    if (!(w->dt > 0 && w->dt < 1)) return fail(PDPD_E_INVALID, "pdpd_step_noalloc: dt must be in (0, 1)");
    uint64_t cells = 1;
    for (int k = 0; k < 3; k++) {
        if (w->box[k] < 2) return fail(PDPD_E_INVALID, "Distance in each direction must be at least 2");
        cells *= (uint64_t)w->box[k];
    }
    if (w->n_beads > NA_MAX_BEADS || cells > NA_MAX_CELLS)
        return fail(PDPD_E_NOMEM, "pdpd_step_noalloc: at most 65536 beads and 32768 cells (the fixed scratch size)");
    if (n_steps == 0 || w->n_beads == 0) return PDPD_OK;
    if (!d_x || !d_v || !d_f || !d_hash) return fail(PDPD_E_INVALID, "pdpd_step_noalloc: missing device array");

    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
        return fail(PDPD_E_CUDA, "pdpd_step_noalloc: no current CUDA device");
    void *scratch = nullptr;
    {
        // First call on a device: look up the device address of the scratch array.
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_scratch[dev]) {
            ce = cudaGetSymbolAddress(&g_na_scratch[dev], g_noalloc_scratch);
            if (ce != cudaSuccess) {
                g_na_scratch[dev] = nullptr;
                return fail(PDPD_E_CUDA, "pdpd_step_noalloc: cudaGetSymbolAddress failed");
            }
        }
        scratch = g_na_scratch[dev];
    }
    NaScratch *S = (NaScratch *)scratch;
    cudaStream_t s = (cudaStream_t)stream;
    NaParams p;
    memset(&p, 0, sizeof p);
    for (int k = 0; k < 3; k++) p.L[k] = w->box[k];
    p.n = w->n_beads;
    p.n_cells = (uint32_t)cells;
    p.nt = w->n_bead_types;
    p.dt = w->dt;
    p.scale_inv_sqrt_dt = sqrt(24 * 1.0 / w->dt);
    p.seed = w->seed;
    for (uint32_t k = 0; k < p.nt * p.nt; k++) {
        p.pair[k][0] = w->conservative[k];
        p.pair[k][1] = sqrt(w->dissipative[k]);
    }
    const uint32_t gb = (p.n + 255) / 256, gc = (p.n_cells + 255) / 256;
    for (uint32_t step = 0; step < n_steps; step++) {
        p.t = w->t + (int64_t)step;
        k_na_clear<<<gc, 256, 0, s>>>(S, p.n_cells, step == 0 ? 1 : 0);
        k_na_update_pos<<<gb, 256, 0, s>>>(p, S, d_x, d_v, d_f);
        k_na_scan<<<1, 1024, 0, s>>>(S, p.n_cells, p.n);
        k_na_place<<<gb, 256, 0, s>>>(S, p.n);
        k_na_canon<<<gb, 256, 0, s>>>(S, p.n);
        k_na_forces<<<gb, 256, 0, s>>>(p, S, d_x, d_v, d_f, d_hash);
        k_na_update_mom<<<gb, 256, 0, s>>>(p, d_v, d_f);
    }
    uint32_t err = 0;
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&err, &S->err, sizeof err, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return fail(PDPD_E_CUDA, cudaGetErrorString(ce));
    if (err) return fail(PDPD_E_BEAD_LOST, "pdpd_step_noalloc: a bead left the box or became non-finite");
    return PDPD_OK;
}
