// FP32 brick force kernels.  Included inside pdpd_fp32.cu's anonymous namespace (they use
// the helpers defined there: WorldCache, load_world, integrate32, pair_sep, pair_force_fx).
//
// A block takes a brick of cells of one world (from a queue shared by the persistent blocks)
// and stages the brick plus its one-cell halo -- (bx+2)(by+2)(bz+2) halo cells, z fastest --
// into shared memory with coalesced 16-byte copies: for each (x, y) halo row the cells
// z0-1 .. z0+bz are consecutive cells of the sorted state, i.e. one or (at a periodic wrap) a
// few contiguous runs of slots.  A halo cell that is a periodic image of a cell already
// staged (boxes smaller than the halo) is staged again, so every neighbour is seen at its own
// image position, as the reference's direction loop sees it
// (naive_dpd_engine_half_step.hpp:300-315).
//
// Two ways to compute the pair forces of the brick's home beads:
//   full shell (variants 6 and 8): one thread per home bead walks its 9 neighbour rows (27
//     cells) and evaluates every in-range pair from its own side, so each pair inside the
//     brick is evaluated twice, once by each bead;
//   half shell (variant 9, Newton's third law): a home bead walks only the forward half of
//     its neighbourhood (make_nhood.hpp:40-49: the rest of its own cell and the 13 forward
//     cells) and passes each pair's reaction to the other bead when that bead is also a home
//     bead of the brick; a neighbour in a halo cell belongs to another brick, which never
//     sees this bead as one of its own, so pairs across the brick's faces are evaluated from
//     both sides, backward cells included.
// The full-shell variants, their global-memory fallback and the thread-per-bead kernel add
// the same pair terms in the same order with the same roundings and give the same forces to
// the bit.  The half shell cannot keep that order (a bead's reactions arrive from other
// threads): its pair force is exactly antisymmetric and its sums are integer (pdpd_fp32.cu,
// pair_force_fx), so its forces do not depend on the order of the sums, the brick shape or
// the batch -- the same to the bit across its own configurations and its fallback, and
// within the FP32 tolerance of the full-shell result.

constexpr int BRICK_THREADS = 128;       // threads per block of variant 6
constexpr int BRICK_THREADS_WIDE = 512;  // threads per block of variant 8 (larger bricks)
constexpr int HALF_THREADS = 384;        // threads per block of variant 9
constexpr int BRICK_MAX_WARPS = BRICK_THREADS_WIDE / 32;
constexpr int BLIST_MAX = 32;            // list capacity of the full-shell row walk
constexpr int HLIST_MAX = 32;            // list capacity of the half-shell walk
constexpr int BRICK_MAX_ROWS = 64;
constexpr uint16_t NOT_HOME = 0xffffu;

struct BrickHeader {
    WorldCache wc;
    uint32_t wsum[BRICK_MAX_WARPS];
    uint32_t home_rows[BRICK_MAX_ROWS + 1];
    uint32_t next;    // the block's next brick
    uint32_t cursor;  // half shell: the next home bead a warp takes
};

// A block's next brick: after its first (blockIdx.x), blocks take bricks from a shared
// counter in the order they finish, so a block that drew small bricks takes more of them.
// Which block computes a brick does not change any result.
__device__ __forceinline__ uint32_t brick_fetch(const KArgs &a, BrickHeader &H)
{
    __syncthreads();
    if (threadIdx.x == 0) H.next = gridDim.x + atomicAdd(a.brick_next, 1u);
    __syncthreads();
    return H.next;
}

// Shared-memory layout of one block: header, pair table, hstart[HC+1], hslot[HC], hlo[HC],
// pos[maxb], vel[maxb], list[cap][threads]; the half shell adds hidx[maxb] (home index of a
// staged bead, NOT_HOME for a halo bead), hsi[home_max] (staged index of a home bead) and
// acc[6][home_max] (fixed-point force sums of the home beads: per axis a word of the terms'
// low 16 bits and a word of their high parts, so that 32-bit atomics add them exactly).
struct BrickLayout {
    uint32_t hc_max, maxb, home_max, list_cap;
    uint32_t off_pair, off_hstart, off_hslot, off_hlo, off_pos, off_vel, off_list, off_hidx, off_hsi,
        off_acc, bytes;
};

inline uint32_t brick_variant_threads(int variant)
{
    return variant == 8 ? BRICK_THREADS_WIDE : (variant == 9 ? HALF_THREADS : BRICK_THREADS);
}

// npair: the largest n_types^2 of the attached worlds (the staged pair table); home_max: the
// home-bead capacity of the half-shell variant (0 for the full-shell variants).
__host__ __device__ inline BrickLayout brick_layout(uint32_t hc_max, uint32_t maxb, uint32_t npair,
                                                    uint32_t threads, uint32_t home_max)
{
    BrickLayout L;
    L.hc_max = hc_max;
    L.maxb = maxb;
    L.home_max = home_max;
    L.list_cap = home_max ? HLIST_MAX : BLIST_MAX;
    uint32_t off = (uint32_t)((sizeof(BrickHeader) + 15) & ~size_t(15));
    L.off_pair = off;
    off += 8 * npair;
    off = (off + 15) & ~15u;
    L.off_hstart = off;
    off += 4 * (hc_max + 1);
    L.off_hslot = off;
    off += 4 * hc_max;
    L.off_hlo = off;
    off += 2 * hc_max;
    off = (off + 15) & ~15u;
    L.off_pos = off;
    off += 16 * maxb;
    L.off_vel = off;
    off += 16 * maxb;
    L.off_list = off;
    off += 2 * L.list_cap * threads;
    L.off_hidx = off;
    if (home_max) off += 2 * maxb;
    L.off_hsi = off;
    if (home_max) off += 2 * home_max;
    off = (off + 15) & ~15u;
    L.off_acc = off;
    if (home_max) off += 24 * home_max;
    L.bytes = off;
    return L;
}

// Halo cell of a staged bead, kept by the staging in the w of its staged velocity:
// hx | hy << 8 | hz << 16 (brick-local halo coordinates; a halo side is at most 34 cells).
__device__ __forceinline__ uint32_t staged_cell(const float4 v)
{
    return __float_as_uint(v.w);
}

// Row of home bead t: the largest r with home_rows[r] <= t (rows may be empty).
__device__ __forceinline__ int home_row_of(const uint32_t *rows, int nr, uint32_t t)
{
    int lo = 0, hi = nr;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (rows[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
}

// Evaluate list entries [0, n) of this thread in order, adding to F (variants 6 and 8): an
// entry is a staged index of an in-range neighbour, and the neighbour direction is the
// difference of the two beads' staged halo cells (vi is the home bead's staged velocity); the
// separation is recomputed exactly as the walk computed it.
template <int T>
__device__ __forceinline__ void brick_rows_eval(const float4 *__restrict__ spos,
                                                const float4 *__restrict__ svel,
                                                const uint16_t *__restrict__ list, int n,
                                                const float4 pi, const float4 vi,
                                                const float2 *pair, uint32_t nt, uint32_t th_lo,
                                                uint32_t th_hi, float scale, float F[3])
{
    const uint32_t hi = __float_as_uint(pi.w);
    const uint32_t ti = min(hi >> 28, nt - 1u);
    const uint32_t hc = staged_cell(vi);
    const int hx = (int)(hc & 255u), hy = (int)((hc >> 8) & 255u), hz = (int)(hc >> 16);
    for (int k = 0; k < n; k++) {
        const uint32_t j = list[k * T + threadIdx.x];
        const float4 pj = spos[j];
        const float4 vj = svel[j];
        const uint32_t cj = staged_cell(vj);
        const float ax = __fsub_rn(pi.x, (float)((int)(cj & 255u) - hx));
        const float ay = __fsub_rn(pi.y, (float)((int)((cj >> 8) & 255u) - hy));
        const float az = __fsub_rn(pi.z, (float)((int)(cj >> 16) - hz));
        float dx, dy, dz;
        const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
        const uint32_t hj = __float_as_uint(pj.w);
        pair_accumulate(dx, dy, dz, r2, vi, vj, hi, hj, pair[ti * nt + min(hj >> 28, nt - 1u)],
                        th_lo, th_hi, scale, F);
    }
}

// 16-byte asynchronous global-to-shared copy (cp.async, no register round trip) and the wait
// for all of this thread's copies.  Both addresses are 16-byte aligned (float4 arrays).
__device__ __forceinline__ void cp_async16(float4 *dst_shared, const float4 *src_global)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst_shared);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src_global) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Halo setup and staging of one brick, block-wide (ends with __syncthreads):
//   hstart[hc] = first staged index of halo cell hc (hc = (hx * HY + hy) * HZ + hz, z fastest),
//   hstart[HC] = total, hslot[hc] = its first slot in the sorted state, hlo[hc] = its beads in
//   the lower z half, H.home_rows[r] = first home index of home (x, y) row r, and, if the halo
//   fits in maxb, spos / svel = the halo's beads.  Halo coordinates lie in [-1, L] (bricks are
//   cut at the box faces), so each wraps with one conditional add or subtract.
template <int T>
__device__ __forceinline__ void brick_halo_and_stage(const KArgs &a, const WorldDev &w, const Brick &br,
                                                     BrickHeader &H, uint32_t *hstart, uint32_t *hslot,
                                                     uint16_t *hlo, float4 *spos, float4 *svel,
                                                     uint32_t maxb, uint32_t &total, uint32_t &n_home)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int HX = br.bx + 2, HY = br.by + 2, HZ = br.bz + 2;
    const int HC = HX * HY * HZ;
    const int L0 = w.L[0], L1 = w.L[1], L2 = w.L[2];

    // counts of a contiguous range of halo cells per thread, then a block exclusive scan
    const int per = (HC + T - 1) / T;
    const int hc_begin = min(HC, tid * per), hc_end = min(HC, hc_begin + per);
    uint32_t tsum = 0;
    if (hc_begin < hc_end) {
        int hx = hc_begin / (HY * HZ);
        const int rem = hc_begin - hx * HY * HZ;
        int hy = rem / HZ, hz = rem - (rem / HZ) * HZ;
        for (int hc = hc_begin; hc < hc_end; hc++) {
            int gx = br.x0 - 1 + hx, gy = br.y0 - 1 + hy, gz = br.z0 - 1 + hz;
            gx += gx < 0 ? L0 : 0;
            gx -= gx >= L0 ? L0 : 0;
            gy += gy < 0 ? L1 : 0;
            gy -= gy >= L1 ? L1 : 0;
            gz += gz < 0 ? L2 : 0;
            gz -= gz >= L2 ? L2 : 0;
            const uint32_t c = w.cell_base + ((uint32_t)gx * (uint32_t)L1 + (uint32_t)gy) * (uint32_t)L2 + (uint32_t)gz;
            const uint32_t s0 = a.start[c];
            const uint32_t n = a.start[c + 1] - s0;
            hslot[hc] = s0;
            hstart[hc] = n;  // count for now
            hlo[hc] = n ? (uint16_t)min((uint32_t)a.zlo[c], n) : (uint16_t)0;
            tsum += n;
            if (++hz == HZ) {
                hz = 0;
                if (++hy == HY) {
                    hy = 0;
                    ++hx;
                }
            }
        }
    }
    uint32_t inc = tsum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += y;
    }
    if (lane == 31) H.wsum[warp] = inc;
    __syncthreads();
    uint32_t run = inc - tsum, tot = 0;
    for (int k = 0; k < T / 32; k++) {
        if (k < warp) run += H.wsum[k];
        tot += H.wsum[k];
    }
    for (int hc = hc_begin; hc < hc_end; hc++) {
        const uint32_t n = hstart[hc];
        hstart[hc] = run;
        run += n;
    }
    if (tid == 0) hstart[HC] = tot;
    __syncthreads();
    if (warp == 0) {  // home rows (at most 64): counts, then a warp prefix sum
        const int nr = br.bx * br.by;
        uint32_t c[2] = {0u, 0u};
        for (int q = 0; q < 2; q++) {
            const int r = lane + 32 * q;
            if (r < nr) {
                const int lx = r / br.by, ly = r - lx * br.by;
                const int hc0 = ((lx + 1) * HY + (ly + 1)) * HZ + 1;
                c[q] = hstart[hc0 + br.bz] - hstart[hc0];
            }
        }
        uint32_t i0 = c[0], i1 = c[1];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y0 = __shfl_up_sync(0xffffffffu, i0, off);
            const uint32_t y1 = __shfl_up_sync(0xffffffffu, i1, off);
            if (lane >= off) {
                i0 += y0;
                i1 += y1;
            }
        }
        const uint32_t tot0 = __shfl_sync(0xffffffffu, i0, 31);
        if (lane < nr) H.home_rows[lane] = i0 - c[0];
        if (lane + 32 < nr) H.home_rows[lane + 32] = tot0 + i1 - c[1];
        if (lane == 31) H.home_rows[nr] = tot0 + i1;  // nr <= 64: lane 31 holds both totals
    }
    // staging, one (x, y) halo row per warp iteration (coalesced); a row whose z range does not
    // wrap is one contiguous run of slots.  Positions go by asynchronous 16-byte copies (no
    // register round trip); velocities through registers, to record the bead's halo cell in
    // the spare w (staged_cell).
    if (tot <= maxb) {
        const bool zrun = br.z0 >= 1 && br.z0 + br.bz + 1 <= L2;
        const float4 *pos = (const float4 *)a.posA, *vel = (const float4 *)a.velA;
        for (int row = warp; row < HX * HY; row += T / 32) {
            const int hc0 = row * HZ;
            const uint32_t base = hstart[hc0];
            const uint32_t len = hstart[hc0 + HZ] - base;
            const uint32_t rowcell = (uint32_t)(row / HY) | ((uint32_t)(row - (row / HY) * HY) << 8);
            int z = 0;  // the lane's halo z cell: k only grows, so z only moves up
            for (uint32_t k = lane; k < len; k += 32) {
                while (hstart[hc0 + z + 1] - base <= k) z++;
                const uint32_t slot = zrun ? hslot[hc0] + k : hslot[hc0 + z] + (k - (hstart[hc0 + z] - base));
                cp_async16(spos + base + k, pos + slot);
                float4 v = vel[slot];
                v.w = __uint_as_float(rowcell | ((uint32_t)z << 16));  // staged_cell
                svel[base + k] = v;
            }
        }
        cp_async_wait_all();
    }
    __syncthreads();
    total = tot;
    n_home = H.home_rows[br.bx * br.by];
}

// Full-shell row walk of one staged home bead (variants 6 and 8): the 9 neighbour rows (dx, dy)
// in order; a row's 3 cells (dz = -1, 0, +1) are one contiguous range of staged beads, trimmed
// at its ends by the same conservative test as the per-cell loop (and by the far z half of an
// end cell: a cell's beads with z offset < 0.5 come first, hlo counts them).  The warp pays the
// longest row of its lanes 9 times instead of the longest cell 27 times.  The in-range
// candidates (the reference's test, update_bead_pair, on the walk's separation) go to this
// thread's list, as staged indices, in the direction order; room for a
// whole row is made before the row (the list is evaluated into F first when it could
// overflow), so the candidate loop has no capacity check and no branch.  Returns the number
// of entries left in the list.
template <int T>
__device__ __forceinline__ int brick_rows_collect(const float4 *__restrict__ spos,
                                                  const float4 *__restrict__ svel,
                                                  uint16_t *__restrict__ list, int cap,
                                                  const uint32_t *__restrict__ hstart,
                                                  const uint16_t *__restrict__ hlo, int HY, int HZ,
                                                  int hx, int hy, int hz, const float4 pi,
                                                  const float4 vi, const float2 *pair, uint32_t nt,
                                                  uint32_t th_lo, uint32_t th_hi, float scale,
                                                  float F[3])
{
    const float PRUNE = 1.0001f;
    const float min2 = min_dist_sqr_f();
    const float azm = __fsub_rn(pi.z, -1.0f), azp = __fsub_rn(pi.z, 1.0f);
    const float gzm = pi.z, gzp = 1.0f - pi.z;
    // gaps to the far halves of the end cells: the lower half of the cell below (z offsets
    // < 0.5) and the upper half of the cell above (>= 0.5)
    const float gzm2 = pi.z + 0.5f, gzp2 = 1.5f - pi.z;
    int n = 0;
#pragma unroll 1
    for (int rr = 0; rr < 9; rr++) {
        const int ddx = rr / 3 - 1, ddy = rr - (rr / 3) * 3 - 1;
        const float gx = slab_gap(pi.x, ddx), gy = slab_gap(pi.y, ddy);
        const float gxy = gx * gx + gy * gy;
        if (gxy >= PRUNE) continue;
        const int rowc = ((hx + ddx) * HY + (hy + ddy)) * HZ + hz;
        const uint32_t c1 = hstart[rowc], c2 = hstart[rowc + 1];
        const uint32_t c0 = hstart[rowc - 1], c3 = hstart[rowc + 2];
        const uint32_t j0 = gxy + gzm * gzm >= PRUNE ? c1 : (gxy + gzm2 * gzm2 >= PRUNE ? c0 + hlo[rowc - 1] : c0);
        const uint32_t j1 = gxy + gzp * gzp >= PRUNE ? c2 : (gxy + gzp2 * gzp2 >= PRUNE ? c2 + hlo[rowc + 1] : c3);
        const float ax = __fsub_rn(pi.x, (float)ddx), ay = __fsub_rn(pi.y, (float)ddy);
        if (n + (int)(j1 - j0) > cap) {  // room for the whole row, or evaluate the list first
            brick_rows_eval<T>(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, F);
            n = 0;
        }
        if ((int)(j1 - j0) <= cap) {
#pragma unroll 2
            for (uint32_t j = j0; j < j1; j++) {
                const float4 pj = spos[j];
                const float az = j < c1 ? azm : (j < c2 ? pi.z : azp);
                float dx, dy, dz;
                const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                list[n * T + threadIdx.x] = (uint16_t)j;
                n += (r2 < 1.0f && r2 >= min2) ? 1 : 0;
            }
        } else {
            for (uint32_t j = j0; j < j1; j++) {
                const float4 pj = spos[j];
                const float az = j < c1 ? azm : (j < c2 ? pi.z : azp);
                float dx, dy, dz;
                const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                list[n * T + threadIdx.x] = (uint16_t)j;
                n += (r2 < 1.0f && r2 >= min2) ? 1 : 0;
                if (n == cap) {
                    brick_rows_eval<T>(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, F);
                    n = 0;
                }
            }
        }
    }
    return n;
}

// One home bead of a brick whose halo does not fit in shared memory: pair forces gathered
// from global memory in the same order (FX = 0) or in fixed point (FX = 1, the half shell),
// then integration.
template <int FINAL, int FX>
__device__ __forceinline__ void brick_fallback_bead(const KArgs &a, const WorldDev &w, const float2 *pair,
                                                    uint32_t th_lo, uint32_t th_hi, float scale,
                                                    uint32_t s, uint32_t &err)
{
    const float4 ph = ((const float4 *)a.posA)[s];
    const float4 vh = ((const float4 *)a.velA)[s];
    int c[3];
    decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
    float F[3] = {0.f, 0.f, 0.f};
    if (FX)
        pair_forces32_seq_fx(a, w, pair, th_lo, th_hi, scale, c, ph, vh, F, err);
    else
        pair_forces32_seq(a, w, pair, th_lo, th_hi, scale, c, ph, vh, F);
    integrate32<FINAL>(a, w, s, c, ph, vh, F, err);
}

// Full-shell brick kernel (variants 6 and 8): one thread per home bead.
template <int FINAL, int T>
__global__ void __launch_bounds__(T, T == BRICK_THREADS_WIDE ? 2 : 6) k_force32_brick(KArgs a, BrickLayout lay)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BrickHeader &H = *reinterpret_cast<BrickHeader *>(smem_raw);
    float2 *spair = reinterpret_cast<float2 *>(smem_raw + lay.off_pair);
    uint32_t *hstart = reinterpret_cast<uint32_t *>(smem_raw + lay.off_hstart);
    uint32_t *hslot = reinterpret_cast<uint32_t *>(smem_raw + lay.off_hslot);
    uint16_t *hlo = reinterpret_cast<uint16_t *>(smem_raw + lay.off_hlo);
    float4 *spos = reinterpret_cast<float4 *>(smem_raw + lay.off_pos);
    float4 *svel = reinterpret_cast<float4 *>(smem_raw + lay.off_vel);
    uint16_t *list = reinterpret_cast<uint16_t *>(smem_raw + lay.off_list);
    const int tid = threadIdx.x;
    if (tid == 0) H.wc.world = 0xffffffffu;
    __syncthreads();
    const int cap = (a.list_capacity > 0 && a.list_capacity < BLIST_MAX) ? a.list_capacity : BLIST_MAX;
    for (uint32_t bi = blockIdx.x; bi < a.n_bricks; bi = brick_fetch(a, H)) {
        const Brick br = a.bricks[bi];
        load_world(a, br.world, H.wc, spair);
        __syncthreads();
        const WorldDev &w = H.wc.w;
        const uint32_t nt = w.n_types;
        const float scale = (float)w.scale_inv_sqrt_dt;
        const uint64_t th = t_hash((uint32_t)w.t, w.seed);
        const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
        const int HY = br.by + 2, HZ = br.bz + 2;

        uint32_t total = 0, n_home = 0;
        brick_halo_and_stage<T>(a, w, br, H, hstart, hslot, hlo, spos, svel, lay.maxb, total, n_home);
        const bool staged = total <= lay.maxb;

        uint32_t err = 0;
        for (uint32_t t = tid; t < n_home; t += T) {
            const int r = home_row_of(H.home_rows, br.bx * br.by, t);
            const int lx = r / br.by, ly = r - lx * br.by;
            const int hx = lx + 1, hy = ly + 1;
            const int hc0 = (hx * HY + hy) * HZ + 1;
            const uint32_t k = t - H.home_rows[r];
            const uint32_t s = hslot[hc0] + k;
            if (!staged) {  // halo larger than the shared-memory budget: gather from global memory
                brick_fallback_bead<FINAL, 0>(a, w, spair, th_lo, th_hi, scale, s, err);
                continue;
            }
            const uint32_t si = hstart[hc0] + k;
            int z = 0;
            while (hstart[hc0 + z + 1] <= si) z++;
            const float4 pi = spos[si], vi = svel[si];
            float F[3] = {0.f, 0.f, 0.f};
            const int nl = brick_rows_collect<T>(spos, svel, list, cap, hstart, hlo, HY, HZ, hx, hy, z + 1, pi, vi,
                                                 spair, nt, th_lo, th_hi, scale, F);
            brick_rows_eval<T>(spos, svel, list, nl, pi, vi, spair, nt, th_lo, th_hi, scale, F);
            const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
            integrate32<FINAL>(a, w, s, c, pi, vi, F, err);
        }
        if (err) atomicOr(&a.worlds[br.world].err, err);
    }
}

// ---------------------------------------------------------------------------------------
// Half shell (variant 9)

// Add a fixed-point term to a home bead's shared accumulator (acc[2 * axis] low words,
// acc[2 * axis + 1] high words, each home_max long): the sum is hi * 2^16 + lo exactly, in any
// order, for far more terms than a bead has.
__device__ __forceinline__ void acc_add(uint32_t *acc, uint32_t home_max, uint32_t h, int axis, long long v)
{
    atomicAdd(acc + (2 * axis) * home_max + h, (uint32_t)v & 0xffffu);
    atomicAdd(acc + (2 * axis + 1) * home_max + h, (uint32_t)(int)(v >> 16));
}

__device__ __forceinline__ long long acc_get(const uint32_t *acc, uint32_t home_max, uint32_t h, int axis)
{
    return (long long)(int)acc[(2 * axis + 1) * home_max + h] * 65536 + (long long)acc[(2 * axis) * home_max + h];
}

// Evaluate this thread's half-shell list entries [0, n): each in-range pair's force is added
// to the home bead's own sum q and its negation to the other bead's accumulator when that
// bead is a home bead of the brick (shared-memory integer atomics: the order does not matter).
__device__ __forceinline__ void half_eval(const float4 *__restrict__ spos, const float4 *__restrict__ svel,
                                          const uint16_t *__restrict__ list, int n, const float4 pi,
                                          const float4 vi, const float2 *pair, uint32_t nt,
                                          uint32_t th_lo, uint32_t th_hi, float scale,
                                          const uint16_t *__restrict__ hidx, uint32_t *acc,
                                          uint32_t home_max, long long q[3], uint32_t &err)
{
    const uint32_t ti = min(__float_as_uint(pi.w) >> 28, nt - 1u);
    const uint32_t hc = staged_cell(vi);
    const int hx = (int)(hc & 255u), hy = (int)((hc >> 8) & 255u), hz = (int)(hc >> 16);
    for (int k = 0; k < n; k++) {
        const uint32_t j = list[k * HALF_THREADS + threadIdx.x];
        const float4 pj = spos[j];
        const float4 vj = svel[j];
        const uint32_t cj = staged_cell(vj);
        float dx, dy, dz;
        const float r2 = pair_sep(pi, pj, (int)(cj & 255u) - hx, (int)((cj >> 8) & 255u) - hy,
                                  (int)(cj >> 16) - hz, dx, dy, dz);
        if (!pair_in_range(r2)) continue;
        long long fx, fy, fz;
        pair_force_fx(dx, dy, dz, r2, vi, vj, __float_as_uint(pi.w), __float_as_uint(pj.w),
                      pair[ti * nt + min(__float_as_uint(pj.w) >> 28, nt - 1u)], th_lo, th_hi, scale,
                      fx, fy, fz, err);
        q[0] += fx;
        q[1] += fy;
        q[2] += fz;
        const uint32_t h = hidx[j];
        if (h != NOT_HOME) {
            acc_add(acc, home_max, h, 0, -fx);
            acc_add(acc, home_max, h, 1, -fy);
            acc_add(acc, home_max, h, 2, -fz);
        }
    }
}

// Append the candidates of staged range [j0, j1) (cells [c0,c1) dz = -1, [c1,c2) dz = 0, the
// rest dz = +1 of one neighbour row) that pass the prefilter to this thread's list; the list
// is evaluated and emptied first when the range could overflow it.
__device__ __forceinline__ int half_range(uint32_t j0, uint32_t j1, uint32_t c1, uint32_t c2, float ax,
                                          float ay, float azm, float azp, int n,
                                          const float4 *__restrict__ spos, const float4 *__restrict__ svel,
                                          uint16_t *__restrict__ list, const float4 pi, const float4 vi,
                                          const float2 *pair, uint32_t nt, uint32_t th_lo, uint32_t th_hi,
                                          float scale, const uint16_t *__restrict__ hidx,
                                          uint32_t *acc, uint32_t home_max, long long q[3],
                                          uint32_t &err)
{
    if (j1 <= j0) return n;
    if (n + (int)(j1 - j0) > HLIST_MAX) {
        half_eval(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, hidx, acc, home_max, q, err);
        n = 0;
    }
    if ((int)(j1 - j0) <= HLIST_MAX) {
#pragma unroll 2
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = spos[j];
            const float az = j < c1 ? azm : (j < c2 ? pi.z : azp);
            float dx, dy, dz;
            const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
            list[n * HALF_THREADS + threadIdx.x] = (uint16_t)j;
            n += r2 < R2_PREFILTER ? 1 : 0;
        }
    } else {
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = spos[j];
            const float az = j < c1 ? azm : (j < c2 ? pi.z : azp);
            float dx, dy, dz;
            const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
            list[n * HALF_THREADS + threadIdx.x] = (uint16_t)j;
            n += r2 < R2_PREFILTER ? 1 : 0;
            if (n == HLIST_MAX) {
                half_eval(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, hidx, acc, home_max, q, err);
                n = 0;
            }
        }
    }
    return n;
}

// Half-shell walk of one staged home bead at staged index si, halo cell (hx, hy, hz), in a
// brick of extents (bx, by, bz).  Rows (dx, dy) after (0, 0) in lexicographic order are
// forward and walked whole (trimmed as in the full-shell walk); the own row contributes the
// rest of the bead's own cell (staged indices above si: the same order on both sides of a
// pair) and the cell above; a backward row is walked whole when it is a halo row, else only
// its end cells that are halo cells (hz == 1: the cell below; hz == bz: the cell above).
__device__ __forceinline__ void half_walk(const float4 *__restrict__ spos, const float4 *__restrict__ svel,
                                          uint16_t *__restrict__ list, const uint32_t *__restrict__ hstart,
                                          const uint16_t *__restrict__ hlo, int by, int bz, int HY, int HZ,
                                          int hx, int hy, int hz, uint32_t si, const float4 pi,
                                          const float4 vi, const float2 *pair, uint32_t nt, uint32_t th_lo,
                                          uint32_t th_hi, float scale, const uint16_t *__restrict__ hidx,
                                          uint32_t *acc, uint32_t home_max, long long q[3],
                                          uint32_t &err)
{
    const float PRUNE = 1.0001f;
    const float azm = __fsub_rn(pi.z, -1.0f), azp = __fsub_rn(pi.z, 1.0f);
    const float gzm = pi.z, gzp = 1.0f - pi.z;
    const float gzm2 = pi.z + 0.5f, gzp2 = 1.5f - pi.z;
    int n = 0;
#pragma unroll 1
    for (int rr = 0; rr < 9; rr++) {
        const int ddx = rr / 3 - 1, ddy = rr - (rr / 3) * 3 - 1;
        const float gx = slab_gap(pi.x, ddx), gy = slab_gap(pi.y, ddy);
        const float gxy = gx * gx + gy * gy;
        if (gxy >= PRUNE) continue;
        const int rowc = ((hx + ddx) * HY + (hy + ddy)) * HZ + hz;
        const uint32_t c1 = hstart[rowc], c2 = hstart[rowc + 1];
        const uint32_t c0 = hstart[rowc - 1], c3 = hstart[rowc + 2];
        const uint32_t j0 = gxy + gzm * gzm >= PRUNE ? c1 : (gxy + gzm2 * gzm2 >= PRUNE ? c0 + hlo[rowc - 1] : c0);
        const uint32_t j1 = gxy + gzp * gzp >= PRUNE ? c2 : (gxy + gzp2 * gzp2 >= PRUNE ? c2 + hlo[rowc + 1] : c3);
        const float ax = __fsub_rn(pi.x, (float)ddx), ay = __fsub_rn(pi.y, (float)ddy);
        if (rr > 4) {  // forward row
            n = half_range(j0, j1, c1, c2, ax, ay, azm, azp, n, spos, svel, list, pi, vi, pair, nt, th_lo,
                           th_hi, scale, hidx, acc, home_max, q, err);
        } else if (rr == 4) {  // own row: the rest of the own cell and the cell above
            n = half_range(si + 1, j1 > si + 1 ? j1 : si + 1, c1, c2, ax, ay, azm, azp, n, spos, svel, list,
                           pi, vi, pair, nt, th_lo, th_hi, scale, hidx, acc, home_max, q, err);
            if (hz == 1)
                n = half_range(j0, c1, c1, c2, ax, ay, azm, azp, n, spos, svel, list, pi, vi, pair, nt,
                               th_lo, th_hi, scale, hidx, acc, home_max, q, err);
        } else {  // backward row
            const bool halo_row = hx + ddx == 0 || hy + ddy == 0 || hy + ddy == by + 1;
            if (halo_row) {
                n = half_range(j0, j1, c1, c2, ax, ay, azm, azp, n, spos, svel, list, pi, vi, pair, nt, th_lo,
                               th_hi, scale, hidx, acc, home_max, q, err);
            } else {
                if (hz == 1)
                    n = half_range(j0, c1, c1, c2, ax, ay, azm, azp, n, spos, svel, list, pi, vi, pair, nt,
                                   th_lo, th_hi, scale, hidx, acc, home_max, q, err);
                if (hz == bz)
                    n = half_range(c2 > j0 ? c2 : j0, j1, c1, c2, ax, ay, azm, azp, n, spos, svel, list, pi,
                                   vi, pair, nt, th_lo, th_hi, scale, hidx, acc, home_max, q, err);
            }
        }
    }
    half_eval(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, hidx, acc, home_max, q, err);
}

// Half-shell brick kernel (variant 9).  Per brick: stage; mark the home beads (hidx, hsi) and
// clear their accumulators; warps take the home beads 32 at a time from a shared cursor and
// walk their forward half shells (own sums and reactions into the accumulators); then one
// thread per home bead converts its sum and integrates.
template <int FINAL>
__global__ void __launch_bounds__(HALF_THREADS, 2) k_force32_half(KArgs a, BrickLayout lay)
{
    constexpr int T = HALF_THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BrickHeader &H = *reinterpret_cast<BrickHeader *>(smem_raw);
    float2 *spair = reinterpret_cast<float2 *>(smem_raw + lay.off_pair);
    uint32_t *hstart = reinterpret_cast<uint32_t *>(smem_raw + lay.off_hstart);
    uint32_t *hslot = reinterpret_cast<uint32_t *>(smem_raw + lay.off_hslot);
    uint16_t *hlo = reinterpret_cast<uint16_t *>(smem_raw + lay.off_hlo);
    float4 *spos = reinterpret_cast<float4 *>(smem_raw + lay.off_pos);
    float4 *svel = reinterpret_cast<float4 *>(smem_raw + lay.off_vel);
    uint16_t *list = reinterpret_cast<uint16_t *>(smem_raw + lay.off_list);
    uint16_t *hidx = reinterpret_cast<uint16_t *>(smem_raw + lay.off_hidx);
    uint16_t *hsi = reinterpret_cast<uint16_t *>(smem_raw + lay.off_hsi);
    uint32_t *acc = reinterpret_cast<uint32_t *>(smem_raw + lay.off_acc);
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t hm = lay.home_max;
    if (tid == 0) H.wc.world = 0xffffffffu;
    __syncthreads();
    for (uint32_t bi = blockIdx.x; bi < a.n_bricks; bi = brick_fetch(a, H)) {
        const Brick br = a.bricks[bi];
        load_world(a, br.world, H.wc, spair);
        __syncthreads();
        const WorldDev &w = H.wc.w;
        const uint32_t nt = w.n_types;
        const float scale = (float)w.scale_inv_sqrt_dt;
        const uint64_t th = t_hash((uint32_t)w.t, w.seed);
        const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
        const int HY = br.by + 2, HZ = br.bz + 2;
        const int nr = br.bx * br.by;

        uint32_t total = 0, n_home = 0;
        brick_halo_and_stage<T>(a, w, br, H, hstart, hslot, hlo, spos, svel, lay.maxb, total, n_home);
        uint32_t err = 0;
        if (total > lay.maxb || n_home > hm) {  // does not fit: gather from global memory
            for (uint32_t t = tid; t < n_home; t += T) {
                const int r = home_row_of(H.home_rows, nr, t);
                const int lx = r / br.by, ly = r - lx * br.by;
                const uint32_t s = hslot[((lx + 1) * HY + (ly + 1)) * HZ + 1] + (t - H.home_rows[r]);
                brick_fallback_bead<FINAL, 1>(a, w, spair, th_lo, th_hi, scale, s, err);
            }
            if (err) atomicOr(&a.worlds[br.world].err, err);
            continue;
        }
        // home marks and cleared accumulators
        for (uint32_t k = tid; k < total; k += T) hidx[k] = NOT_HOME;
        for (uint32_t k = tid; k < n_home; k += T)
            for (int c = 0; c < 6; c++) acc[c * hm + k] = 0u;
        if (tid == 0) H.cursor = 0;
        __syncthreads();
        for (uint32_t t = tid; t < n_home; t += T) {
            const int r = home_row_of(H.home_rows, nr, t);
            const int lx = r / br.by, ly = r - lx * br.by;
            const uint32_t si = hstart[((lx + 1) * HY + (ly + 1)) * HZ + 1] + (t - H.home_rows[r]);
            hidx[si] = (uint16_t)t;
            hsi[t] = (uint16_t)si;
        }
        __syncthreads();
        // pair forces: warps take 32 home beads at a time
        for (;;) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&H.cursor, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n_home) break;
            const uint32_t t = base + lane;
            if (t < n_home) {
                const uint32_t si = hsi[t];
                const float4 pi = spos[si], vi = svel[si];
                const uint32_t hc = staged_cell(vi);
                long long q[3] = {0, 0, 0};
                half_walk(spos, svel, list, hstart, hlo, br.by, br.bz, HY, HZ, (int)(hc & 255u),
                          (int)((hc >> 8) & 255u), (int)(hc >> 16), si, pi, vi, spair, nt, th_lo, th_hi, scale,
                          hidx, acc, hm, q, err);
                acc_add(acc, hm, t, 0, q[0]);
                acc_add(acc, hm, t, 1, q[1]);
                acc_add(acc, hm, t, 2, q[2]);
            }
        }
        __syncthreads();
        // bonds, update_mom, next update_pos
        for (uint32_t t = tid; t < n_home; t += T) {
            const uint32_t si = hsi[t];
            const float4 pi = spos[si], vi = svel[si];
            const uint32_t hc = staged_cell(vi);
            const int hx = (int)(hc & 255u), hy = (int)((hc >> 8) & 255u), hz = (int)(hc >> 16);
            const int cell = (hx * HY + hy) * HZ + hz;
            const uint32_t s = hslot[cell] + (si - hstart[cell]);
            const long long q[3] = {acc_get(acc, hm, t, 0), acc_get(acc, hm, t, 1), acc_get(acc, hm, t, 2)};
            float F[3];
            fx_to_force(q, F);
            const int c[3] = {br.x0 + hx - 1, br.y0 + hy - 1, br.z0 + hz - 1};
            integrate32<FINAL>(a, w, s, c, pi, vi, F, err);
        }
        if (err) atomicOr(&a.worlds[br.world].err, err);
    }
}
