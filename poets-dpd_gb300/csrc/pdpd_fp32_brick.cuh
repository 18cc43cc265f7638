// FP32 brick force kernel.  Included inside pdpd_fp32.cu's anonymous namespace (it uses the
// helpers defined there: WorldCache, load_world, advance_position, bond_forces32, pack_dir).
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
// Then one thread per home bead gathers its pair forces from shared memory: the 27
// neighbour cells in the reference's direction order, each cell's beads in the sorted order,
// accumulated one pair at a time.  In the list variants the thread first filters the
// candidates and keeps the in-range ones (16-bit entries: staged index, with the direction in
// its high bits for variants 0 and 3, or recovered from the staged halo cells for the row
// walks 6-8) in a shared-memory list, then evaluates the list in order; the divergent,
// expensive force evaluation then runs on denser warps.  All variants, the thread-per-bead
// global-memory kernel and the overflow fallback produce bit-identical forces: the same
// explicitly rounded pair routine, the same order.

constexpr int BRICK_THREADS = 128;       // threads per block of variants 0, 2-7
constexpr int BRICK_WARPS = BRICK_THREADS / 32;
constexpr int BRICK_THREADS_WIDE = 512;  // threads per block of variant 8 (larger bricks)
constexpr int BRICK_MAX_WARPS = BRICK_THREADS_WIDE / 32;
constexpr int BLIST_MAX = 32;
constexpr int BRICK_MAX_ROWS = 64;

struct BrickHeader {
    WorldCache wc;
    uint32_t wsum[BRICK_MAX_WARPS];
    uint32_t home_rows[BRICK_MAX_ROWS + 1];
    uint32_t next;  // the block's next brick
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

// Shared-memory layout of one block: header, hstart[HC+1], hslot[HC], pos[maxb], vel[maxb],
// list[BLIST_MAX][threads].
struct BrickLayout {
    uint32_t hc_max, maxb;
    uint32_t off_pair, off_hstart, off_hslot, off_hlo, off_pos, off_vel, off_list, off_bal, bytes;
};

// Balanced list evaluation (variant 7): per pass of BRICK_THREADS home beads, the list
// lengths are counting-sorted so that each warp evaluates lists of similar length.
struct BrickBalance {
    uint32_t hist[BLIST_MAX + 2];   // length histogram, then its exclusive prefix
    uint16_t perm[BRICK_THREADS];   // evaluation lane -> list owner (thread)
    uint16_t n[BRICK_THREADS];      // list length of each owner
    uint32_t si[BRICK_THREADS];     // staged index of each owner's home bead
    float f[3][BRICK_THREADS];      // each owner's force (partial sums of flushed entries in)
};

// npair: the largest n_types^2 of the attached worlds (the staged pair table).
__host__ __device__ inline BrickLayout brick_layout(uint32_t hc_max, uint32_t maxb, uint32_t npair,
                                                    int with_list, int with_balance = 0,
                                                    uint32_t threads = BRICK_THREADS)
{
    BrickLayout L;
    L.hc_max = hc_max;
    L.maxb = maxb;
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
    if (with_list) off += 2 * BLIST_MAX * threads;
    off = (off + 15) & ~15u;
    L.off_bal = off;
    if (with_balance) off += (uint32_t)sizeof(BrickBalance);
    L.bytes = off;
    return L;
}

// Brick variants (force_kernel) that keep per-thread neighbour lists in shared memory, and
// the one that evaluates them balanced across lanes.
inline int brick_variant_has_list(int variant)
{
    return (variant == 0 || variant == 3 || variant == 6 || variant == 7 || variant == 8) ? 1 : 0;
}
inline uint32_t brick_variant_threads(int variant)
{
    return variant == 8 ? BRICK_THREADS_WIDE : BRICK_THREADS;
}
inline int brick_variant_balanced(int variant)
{
    return variant == 7 ? 1 : 0;
}

// Evaluate list entries [0, n) of this thread in order, adding to F.
template <int T = BRICK_THREADS>
__device__ __forceinline__ void brick_list_eval_col(const float4 *__restrict__ spos,
                                                    const float4 *__restrict__ svel,
                                                    const uint16_t *__restrict__ list, int col, int n,
                                                    const float4 pi, const float4 vi,
                                                    const float2 *pair, uint32_t nt, uint32_t th_lo,
                                                    uint32_t th_hi, float scale, float F[3])
{
    const uint32_t hi = __float_as_uint(pi.w);
    const uint32_t ti = min(hi >> 28, nt - 1u);
    for (int k = 0; k < n; k++) {
        const uint32_t e = list[k * T + col];
        const uint32_t j = e & 2047u, d = e >> 11;  // d = (dx+1)*9 + (dy+1)*3 + (dz+1)
        const float4 pj = spos[j];
        const float ax = __fsub_rn(pi.x, (float)((int)(d / 9u) - 1));
        const float ay = __fsub_rn(pi.y, (float)((int)((d / 3u) % 3u) - 1));
        const float az = __fsub_rn(pi.z, (float)((int)(d % 3u) - 1));
        float dx, dy, dz;
        const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
        const uint32_t hj = __float_as_uint(pj.w);
        pair_accumulate(dx, dy, dz, r2, vi, svel[j], hi, hj, pair[ti * nt + min(hj >> 28, nt - 1u)],
                        th_lo, th_hi, scale, F);
    }
}

// This thread's own list (column threadIdx.x).
template <int T = BRICK_THREADS>
__device__ __forceinline__ void brick_list_eval(const float4 *__restrict__ spos,
                                                const float4 *__restrict__ svel,
                                                const uint16_t *__restrict__ list, int n,
                                                const float4 pi, const float4 vi,
                                                const float2 *pair, uint32_t nt, uint32_t th_lo,
                                                uint32_t th_hi, float scale, float F[3])
{
    brick_list_eval_col<T>(spos, svel, list, threadIdx.x, n, pi, vi, pair, nt, th_lo, th_hi, scale, F);
}

// Halo cell of a staged bead, kept by the staging in the w of its staged velocity:
// hx | hy << 8 | hz << 16 (brick-local halo coordinates; a halo side is at most 34 cells).
__device__ __forceinline__ uint32_t staged_cell(const float4 v)
{
    return __float_as_uint(v.w);
}

// Evaluate list entries [0, n) of column `col` in order, adding to F, for the row walk's
// lists (variants 6-8): an entry is the staged index alone, and the neighbour direction is
// the difference of the two beads' staged halo cells (vi is the home bead's staged velocity).
// The direction's values and so every operation are those of brick_list_eval_col.
template <int T = BRICK_THREADS>
__device__ __forceinline__ void brick_rows_eval_col(const float4 *__restrict__ spos,
                                                    const float4 *__restrict__ svel,
                                                    const uint16_t *__restrict__ list, int col, int n,
                                                    const float4 pi, const float4 vi,
                                                    const float2 *pair, uint32_t nt, uint32_t th_lo,
                                                    uint32_t th_hi, float scale, float F[3])
{
    const uint32_t hi = __float_as_uint(pi.w);
    const uint32_t ti = min(hi >> 28, nt - 1u);
    const uint32_t hc = staged_cell(vi);
    const int hx = (int)(hc & 255u), hy = (int)((hc >> 8) & 255u), hz = (int)(hc >> 16);
    for (int k = 0; k < n; k++) {
        const uint32_t j = list[k * T + col];
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

template <int T = BRICK_THREADS>
__device__ __forceinline__ void brick_rows_eval(const float4 *__restrict__ spos,
                                                const float4 *__restrict__ svel,
                                                const uint16_t *__restrict__ list, int n,
                                                const float4 pi, const float4 vi,
                                                const float2 *pair, uint32_t nt, uint32_t th_lo,
                                                uint32_t th_hi, float scale, float F[3])
{
    brick_rows_eval_col<T>(spos, svel, list, threadIdx.x, n, pi, vi, pair, nt, th_lo, th_hi, scale, F);
}

// Pair forces of one staged home bead, with the 27 neighbour cells walked as one flat
// sequence: the 9 neighbour rows (dx, dy) in order, each row's 3 cells (dz = -1, 0, +1) being
// one contiguous range of staged beads.  Each thread's loop then runs for its own total
// candidate count, instead of the warp paying the largest count of every cell in turn.
// The sequence -- rows in order, cells in order, beads in order -- is the reference's
// direction order, and pruned cells (nearest face >= 1 away) hold no in-range bead, so the
// accumulated force is bit-identical to the nested-loop variants.
template <int LIST, int T = BRICK_THREADS>
__device__ __forceinline__ void brick_gather_flat(const float4 *__restrict__ spos,
                                                  const float4 *__restrict__ svel,
                                                  uint16_t *__restrict__ list, int cap,
                                                  const uint32_t *__restrict__ hstart, int HY,
                                                  int HZ, int hx, int hy, int hz, const float4 pi,
                                                  const float4 vi, const float2 *pair, uint32_t nt,
                                                  uint32_t th_lo, uint32_t th_hi, float scale,
                                                  float F[3])
{
    const float PRUNE = 1.0001f;
    const float min2 = min_dist_sqr_f();
    const uint32_t hi = __float_as_uint(pi.w);
    const uint32_t ti = min(hi >> 28, nt - 1u);
    const float azm = __fsub_rn(pi.z, -1.0f), az0 = pi.z, azp = __fsub_rn(pi.z, 1.0f);
    const float gzm = pi.z, gzp = 1.0f - pi.z;
    int r = -1;
    uint32_t j = 0, jend = 0, c1 = 0, c2 = 0;
    float ax = 0.f, ay = 0.f;
    int rdx = 0, rdy = 0;
    int n = 0;
    while (true) {
        while (j >= jend) {  // next row with candidates
            if (++r == 9) break;
            rdx = r / 3 - 1;
            rdy = r - (r / 3) * 3 - 1;
            const float gx = slab_gap(pi.x, rdx), gy = slab_gap(pi.y, rdy);
            const float gxy = gx * gx + gy * gy;
            if (gxy >= PRUNE) continue;
            const int hcz = ((hx + rdx) * HY + (hy + rdy)) * HZ + hz;
            c1 = hstart[hcz];
            c2 = hstart[hcz + 1];
            j = gxy + gzm * gzm >= PRUNE ? c1 : hstart[hcz - 1];
            jend = gxy + gzp * gzp >= PRUNE ? c2 : hstart[hcz + 2];
            ax = __fsub_rn(pi.x, (float)rdx);
            ay = __fsub_rn(pi.y, (float)rdy);
        }
        if (r == 9) break;
        const float4 pj = spos[j];
        const float az = j < c1 ? azm : (j < c2 ? az0 : azp);
        float dx, dy, dz;
        const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
        if (r2 < 1.0f && r2 >= min2) {
            if (LIST) {
                if (n == cap) {
                    brick_list_eval<T>(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, F);
                    n = 0;
                }
                const int ddz = j < c1 ? -1 : (j < c2 ? 0 : 1);
                list[n * T + threadIdx.x] =
                    (uint16_t)(j | (uint32_t)(((rdx + 1) * 9 + (rdy + 1) * 3 + (ddz + 1)) << 11));
                n++;
            } else {
                const uint32_t hj = __float_as_uint(pj.w);
                pair_accumulate(dx, dy, dz, r2, vi, svel[j], hi, hj,
                                pair[ti * nt + min(hj >> 28, nt - 1u)], th_lo, th_hi, scale, F);
            }
        }
        j++;
    }
    if (LIST) brick_list_eval<T>(spos, svel, list, n, pi, vi, pair, nt, th_lo, th_hi, scale, F);
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
//   hstart[HC] = total, hslot[hc] = its first slot in the sorted state,
//   H.home_rows[r] = first home index of home (x, y) row r, and, if the halo fits in maxb,
//   spos / svel = the halo's beads.  Halo coordinates lie in [-1, L] (bricks are cut at the
//   box faces), so each wraps with one conditional add or subtract.
template <int T = BRICK_THREADS>
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


// Row walk of one staged home bead (force variants 6, 7 and 8): the 9 neighbour rows (dx, dy)
// in order; a row's 3 cells (dz = -1, 0, +1) are one contiguous range of staged beads, trimmed
// at its ends by the same conservative test as the per-cell loop (and by the far z half of an
// end cell: a cell's beads with z offset < 0.5 come first, hlo counts them).  The warp pays the
// longest row of its lanes 9 times instead of the longest cell 27 times.  The in-range
// candidates go to this thread's list, as staged indices, in the direction order; room for a
// whole row is made before the row (the list is evaluated into F first when it could
// overflow), so the candidate loop has no capacity check and no branch.  Returns the number
// of entries left in the list.
template <int T = BRICK_THREADS>
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
// from global memory in the same order, then integration.  Its accumulators are its own, so
// the hot path's never have their address taken (they stay in registers).
template <int FINAL>
__device__ __forceinline__ void brick_fallback_bead(const KArgs &a, const WorldDev &w, const float2 *pair,
                                                 uint32_t th_lo, uint32_t th_hi, float scale,
                                                 uint32_t s, uint32_t &err)
{
    const float4 ph = ((const float4 *)a.posA)[s];
    const float4 vh = ((const float4 *)a.velA)[s];
    int c[3];
    decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
    float F[3] = {0.f, 0.f, 0.f};
    pair_forces32_seq(a, w, pair, th_lo, th_hi, scale, c, ph, vh, F);
    integrate32<FINAL>(a, w, s, c, ph, vh, F, err);
}

template <int FINAL, int LIST, int FLAT, int T = BRICK_THREADS>
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
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) H.wc.world = 0xffffffffu;
    __syncthreads();
    const float min2 = min_dist_sqr_f();
    const float PRUNE = 1.0001f;
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

        // ---- 1-2. halo cells (hstart, hslot, home rows) and staging
        uint32_t total = 0, n_home = 0;
        brick_halo_and_stage<T>(a, w, br, H, hstart, hslot, hlo, spos, svel, lay.maxb, total, n_home);
        const bool staged = total <= lay.maxb;

        // ---- 3. one thread per home bead: pair forces, bonds, integration
        uint32_t err = 0;
        if (FLAT == 3 && T == BRICK_THREADS && staged) {
            // Variant 7, per pass of BRICK_THREADS home beads: (a) each thread walks the rows of
            // its bead into its list; (b) the lists are counting-sorted by length and lane l
            // evaluates list perm[l], so a warp's lanes run lists of about the same length; (c)
            // each thread integrates its own bead.  Every list is still summed by one thread
            // in its own order: the forces are those of the other variants, bit for bit.
            BrickBalance &B = *reinterpret_cast<BrickBalance *>(smem_raw + lay.off_bal);
            for (uint32_t t0 = 0; t0 < n_home; t0 += T) {
                const uint32_t t = t0 + tid;
                const bool act = t < n_home;
                float F[3] = {0.f, 0.f, 0.f};
                int n = 0, lx = 0, ly = 0, z = 0;
                uint32_t s = 0, si = 0;
                float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), vi = pi;
                if (act) {
                    int r = 0;
                    while (H.home_rows[r + 1] <= t) r++;
                    lx = r / br.by;
                    ly = r - lx * br.by;
                    const int hc0 = ((lx + 1) * HY + (ly + 1)) * HZ + 1;
                    const uint32_t k = t - H.home_rows[r];
                    s = hslot[hc0] + k;
                    si = hstart[hc0] + k;
                    while (hstart[hc0 + z + 1] <= si) z++;
                    pi = spos[si];
                    vi = svel[si];
                    n = brick_rows_collect<T>(spos, svel, list, cap, hstart, hlo, HY, HZ, lx + 1, ly + 1, z + 1,
                                           pi, vi, spair, nt, th_lo, th_hi, scale, F);
                }
                if (tid < BLIST_MAX + 2) B.hist[tid] = 0u;
                B.n[tid] = (uint16_t)n;
                B.si[tid] = si;
                B.f[0][tid] = F[0];
                B.f[1][tid] = F[1];
                B.f[2][tid] = F[2];
                __syncthreads();
                const uint32_t rank = atomicAdd(&B.hist[n], 1u);  // n <= BLIST_MAX
                __syncthreads();
                if (warp == 0) {  // exclusive prefix of the BLIST_MAX + 1 bins
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
                B.perm[B.hist[n] + rank] = (uint16_t)tid;
                __syncthreads();
                {
                    const uint32_t o = B.perm[tid];
                    const int no = B.n[o];
                    if (no > 0) {
                        const uint32_t so = B.si[o];
                        float G[3] = {B.f[0][o], B.f[1][o], B.f[2][o]};
                        brick_rows_eval_col(spos, svel, list, (int)o, no, spos[so], svel[so], spair, nt,
                                            th_lo, th_hi, scale, G);
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
                    const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
                    integrate32<FINAL>(a, w, s, c, pi, vi, F, err);
                }
                if (t0 + T < n_home) __syncthreads();  // the lists are reused
            }
            if (err) atomicOr(&a.worlds[br.world].err, err);
            continue;
        }
        for (uint32_t t = tid; t < n_home; t += T) {
            int r = 0;
            while (H.home_rows[r + 1] <= t) r++;
            const int lx = r / br.by, ly = r - lx * br.by;
            const int hx = lx + 1, hy = ly + 1;
            const int hc0 = (hx * HY + hy) * HZ + 1;
            const uint32_t k = t - H.home_rows[r];
            const uint32_t s = hslot[hc0] + k;
            if (!staged) {  // halo larger than the shared-memory budget: gather from global memory
                brick_fallback_bead<FINAL>(a, w, spair, th_lo, th_hi, scale, s, err);
                continue;
            }
            float F[3] = {0.f, 0.f, 0.f};
            const uint32_t si = hstart[hc0] + k;
            int z = 0;
            while (hstart[hc0 + z + 1] <= si) z++;
            const int hz = z + 1;
            const float4 pi = spos[si], vi = svel[si];
            const uint32_t hi = __float_as_uint(pi.w);
            const uint32_t ti = min(hi >> 28, nt - 1u);
            int n = 0;
            if (FLAT >= 2) {  // variant 6 (and 7 when not staged, never reached)
                const int nl = brick_rows_collect<T>(spos, svel, list, cap, hstart, hlo, HY, HZ, hx, hy, hz, pi,
                                                  vi, spair, nt, th_lo, th_hi, scale, F);
                brick_rows_eval<T>(spos, svel, list, nl, pi, vi, spair, nt, th_lo, th_hi, scale, F);
                const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
                integrate32<FINAL>(a, w, s, c, pi, vi, F, err);
                continue;
            }
            if (FLAT) {
                brick_gather_flat<LIST, T>(spos, svel, list, cap, hstart, HY, HZ, hx, hy, hz, pi, vi,
                                        spair, nt, th_lo, th_hi, scale, F);
                const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
                integrate32<FINAL>(a, w, s, c, pi, vi, F, err);
                continue;
            }
            for (int ddx = -1; ddx <= 1; ddx++) {
                const float gx = slab_gap(pi.x, ddx);
                const float ax = __fsub_rn(pi.x, (float)ddx);
                for (int ddy = -1; ddy <= 1; ddy++) {
                    const float gy = slab_gap(pi.y, ddy);
                    const float gxy = gx * gx + gy * gy;
                    if (gxy >= PRUNE) continue;
                    const float ay = __fsub_rn(pi.y, (float)ddy);
                    const int rowc = ((hx + ddx) * HY + (hy + ddy)) * HZ + hz;
                    for (int ddz = -1; ddz <= 1; ddz++) {
                        const float gz = slab_gap(pi.z, ddz);
                        if (gxy + gz * gz >= PRUNE) continue;
                        const float az = __fsub_rn(pi.z, (float)ddz);
                        const uint32_t j1 = hstart[rowc + ddz + 1];
                        const uint16_t dpk = (uint16_t)(((ddx + 1) * 9 + (ddy + 1) * 3 + (ddz + 1)) << 11);
                        for (uint32_t j = hstart[rowc + ddz]; j < j1; j++) {
                            const float4 pj = spos[j];
                            float dx, dy, dz;
                            const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                            if (r2 < 1.0f && r2 >= min2) {
                                if (LIST) {
                                    if (n == cap) {
                                        brick_list_eval<T>(spos, svel, list, n, pi, vi, spair, nt, th_lo,
                                                        th_hi, scale, F);
                                        n = 0;
                                    }
                                    list[n * T + tid] = (uint16_t)(j | dpk);
                                    n++;
                                } else {
                                    const uint32_t hj = __float_as_uint(pj.w);
                                    pair_accumulate(dx, dy, dz, r2, vi, svel[j], hi, hj,
                                                    spair[ti * nt + min(hj >> 28, nt - 1u)], th_lo,
                                                    th_hi, scale, F);
                                }
                            }
                        }
                    }
                }
            }
            if (LIST) brick_list_eval<T>(spos, svel, list, n, pi, vi, spair, nt, th_lo, th_hi, scale, F);
            const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
            integrate32<FINAL>(a, w, s, c, pi, vi, F, err);
        }
        if (err) atomicOr(&a.worlds[br.world].err, err);
    }
}

// =======================================================================================
// Cell kernel: one warp per home cell.
//
// Same staging as the brick kernel.  A warp then takes a home cell: it writes the cell's
// neighbourhood -- the 27 neighbour cells in the reference's direction order -- once into
// an index array (staged index + direction), and for each home bead i sweeps that array
// 32 neighbours at a time, one per lane, against a per-warp table of i's 27
// direction-shifted positions.  In-range pairs are compacted with a warp ballot into a
// queue; each full queue of 32 is evaluated one pair per lane and summed per home bead with
// a segmented shuffle scan (the order is a fixed function of the data: deterministic).  A
// thread-per-bead pass then adds bonds and integrates.
// =======================================================================================

constexpr int CELL_NBR_MAX = 384;  // neighbourhood beads per home cell handled by a warp
constexpr int CELL_HOME_MAX = 64;  // home beads per cell handled by a warp
constexpr int CELL_QCAP = 64;

struct CellWarp {
    uint32_t nbr[CELL_NBR_MAX];  // staged index | direction << 16
    float4 shome[27];            // home bead position minus each direction
    uint32_t queue[CELL_QCAP];   // staged index | direction << 11 | home index << 16
    float fh[3][CELL_HOME_MAX];
};

struct CellLayout {
    uint32_t hc_max, maxb;
    uint32_t off_pair, off_hstart, off_hslot, off_hlo, off_pos, off_vel, off_f, off_warp, bytes;
};

__host__ __device__ inline CellLayout cell_layout(uint32_t hc_max, uint32_t maxb, uint32_t npair)
{
    CellLayout L;
    L.hc_max = hc_max;
    L.maxb = maxb;
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
    L.off_f = off;
    off += 12 * maxb;
    off = (off + 15) & ~15u;
    L.off_warp = off;
    off += (uint32_t)sizeof(CellWarp) * BRICK_WARPS;
    L.bytes = off;
    return L;
}

__device__ __forceinline__ void cell_eval_queue(CellWarp &cw, int lane, int n, const float4 *spos,
                                                const float4 *svel, uint32_t h0, const float2 *pair,
                                                uint32_t nt, uint32_t th_lo, uint32_t th_hi,
                                                float scale)
{
    float F[3] = {0.f, 0.f, 0.f};
    uint32_t key = 0xffffffffu;
    if (lane < n) {
        const uint32_t e = cw.queue[lane];
        const uint32_t j = e & 2047u, d = (e >> 11) & 31u, i = e >> 16;
        const float4 pi = spos[h0 + i], vi = svel[h0 + i];
        const float4 pj = spos[j];
        const float ax = __fsub_rn(pi.x, (float)((int)(d / 9u) - 1));
        const float ay = __fsub_rn(pi.y, (float)((int)((d / 3u) % 3u) - 1));
        const float az = __fsub_rn(pi.z, (float)((int)(d % 3u) - 1));
        float dx, dy, dz;
        const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
        const uint32_t hi = __float_as_uint(pi.w), hj = __float_as_uint(pj.w);
        pair_accumulate(dx, dy, dz, r2, vi, svel[j], hi, hj,
                        pair[min(hi >> 28, nt - 1u) * nt + min(hj >> 28, nt - 1u)], th_lo, th_hi,
                        scale, F);
        key = i;
    }
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float ux = __shfl_up_sync(0xffffffffu, F[0], off);
        const float uy = __shfl_up_sync(0xffffffffu, F[1], off);
        const float uz = __shfl_up_sync(0xffffffffu, F[2], off);
        const uint32_t uk = __shfl_up_sync(0xffffffffu, key, off);
        if (lane >= off && uk == key) {
            F[0] = __fadd_rn(F[0], ux);
            F[1] = __fadd_rn(F[1], uy);
            F[2] = __fadd_rn(F[2], uz);
        }
    }
    const uint32_t next = __shfl_down_sync(0xffffffffu, key, 1);
    if (lane < n && (lane == n - 1 || next != key)) {
        cw.fh[0][key] = __fadd_rn(cw.fh[0][key], F[0]);
        cw.fh[1][key] = __fadd_rn(cw.fh[1][key], F[1]);
        cw.fh[2][key] = __fadd_rn(cw.fh[2][key], F[2]);
    }
    __syncwarp();
}

template <int FINAL>
__global__ void __launch_bounds__(BRICK_THREADS) k_force32_cells(KArgs a, CellLayout lay)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BrickHeader &H = *reinterpret_cast<BrickHeader *>(smem_raw);
    float2 *spair = reinterpret_cast<float2 *>(smem_raw + lay.off_pair);
    uint32_t *hstart = reinterpret_cast<uint32_t *>(smem_raw + lay.off_hstart);
    uint32_t *hslot = reinterpret_cast<uint32_t *>(smem_raw + lay.off_hslot);
    uint16_t *hlo = reinterpret_cast<uint16_t *>(smem_raw + lay.off_hlo);
    float4 *spos = reinterpret_cast<float4 *>(smem_raw + lay.off_pos);
    float4 *svel = reinterpret_cast<float4 *>(smem_raw + lay.off_vel);
    float *sfx = reinterpret_cast<float *>(smem_raw + lay.off_f);
    float *sfy = sfx + lay.maxb;
    float *sfz = sfy + lay.maxb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    CellWarp &cw = reinterpret_cast<CellWarp *>(smem_raw + lay.off_warp)[warp];
    if (tid == 0) H.wc.world = 0xffffffffu;
    __syncthreads();
    const float min2 = min_dist_sqr_f();
    for (uint32_t bi = blockIdx.x; bi < a.n_bricks; bi += gridDim.x) {
        const Brick br = a.bricks[bi];
        load_world(a, br.world, H.wc, spair);
        __syncthreads();
        const WorldDev &w = H.wc.w;
        const uint32_t nt = w.n_types;
        const float scale = (float)w.scale_inv_sqrt_dt;
        const uint64_t th = t_hash((uint32_t)w.t, w.seed);
        const uint32_t th_lo = (uint32_t)th, th_hi = (uint32_t)(th >> 32);
        const int HY = br.by + 2, HZ = br.bz + 2;

        // ---- 1-2. halo cells (hstart, hslot, home rows) and staging
        uint32_t total = 0, n_home = 0;
        brick_halo_and_stage(a, w, br, H, hstart, hslot, hlo, spos, svel, lay.maxb, total, n_home);
        const bool staged = total <= lay.maxb;

        // ---- pair forces: one warp per home cell
        if (staged) {
            const int n_home_cells = br.bx * br.by * br.bz;
            for (int hcell = warp; hcell < n_home_cells; hcell += BRICK_WARPS) {
                const int lx = hcell / (br.by * br.bz), rem = hcell - lx * br.by * br.bz;
                const int ly = rem / br.bz, lz = rem - ly * br.bz;
                const int hx = lx + 1, hy = ly + 1, hz = lz + 1;
                const int hc = (hx * HY + hy) * HZ + hz;
                const uint32_t h0 = hstart[hc];
                const uint32_t nh = hstart[hc + 1] - h0;
                if (nh == 0) continue;
                // neighbour rows: r = (dx+1)*3 + (dy+1), 3 cells each
                uint32_t a0 = 0, c1 = 0, c2 = 0, len = 0;
                if (lane < 9) {
                    const int hcz = ((hx + lane / 3 - 1) * HY + (hy + lane % 3 - 1)) * HZ + hz;
                    a0 = hstart[hcz - 1];
                    c1 = hstart[hcz];
                    c2 = hstart[hcz + 1];
                    len = hstart[hcz + 2] - a0;
                }
                uint32_t P = len;
#pragma unroll
                for (int off = 1; off < 16; off <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, P, off);
                    if (lane >= off) P += y;
                }
                const uint32_t M = __shfl_sync(0xffffffffu, P, 8);
                if (M > (uint32_t)CELL_NBR_MAX || nh > (uint32_t)CELL_HOME_MAX) {
                    // crowded cell: one lane per home bead, sequential over the neighbours
                    for (uint32_t i = lane; i < nh; i += 32) {
                        const float4 pi = spos[h0 + i], vi = svel[h0 + i];
                        const uint32_t hi = __float_as_uint(pi.w);
                        const uint32_t ti = min(hi >> 28, nt - 1u);
                        float F[3] = {0.f, 0.f, 0.f};
                        for (int r = 0; r < 9; r++) {
                            const int ddx = r / 3 - 1, ddy = r % 3 - 1;
                            const int hcz = ((hx + ddx) * HY + (hy + ddy)) * HZ + hz;
                            const float ax = __fsub_rn(pi.x, (float)ddx), ay = __fsub_rn(pi.y, (float)ddy);
                            for (int ddz = -1; ddz <= 1; ddz++) {
                                const float az = __fsub_rn(pi.z, (float)ddz);
                                const uint32_t j1 = hstart[hcz + ddz + 1];
                                for (uint32_t j = hstart[hcz + ddz]; j < j1; j++) {
                                    const float4 pj = spos[j];
                                    float dx, dy, dz;
                                    const float r2 = pair_r2(ax, ay, az, pj, dx, dy, dz);
                                    if (r2 < 1.0f && r2 >= min2) {
                                        const uint32_t hj = __float_as_uint(pj.w);
                                        pair_accumulate(dx, dy, dz, r2, vi, svel[j], hi, hj,
                                                        spair[ti * nt + min(hj >> 28, nt - 1u)],
                                                        th_lo, th_hi, scale, F);
                                    }
                                }
                            }
                        }
                        sfx[h0 + i] = F[0];
                        sfy[h0 + i] = F[1];
                        sfz[h0 + i] = F[2];
                    }
                    __syncwarp();
                    continue;
                }
                // neighbour index array, rows in order
                for (int r = 0; r < 9; r++) {
                    const uint32_t rb = r == 0 ? 0u : __shfl_sync(0xffffffffu, P, r - 1);
                    const uint32_t ra = __shfl_sync(0xffffffffu, a0, r);
                    const uint32_t rc1 = __shfl_sync(0xffffffffu, c1, r);
                    const uint32_t rc2 = __shfl_sync(0xffffffffu, c2, r);
                    const uint32_t rl = __shfl_sync(0xffffffffu, len, r);
                    for (uint32_t k = lane; k < rl; k += 32) {
                        const uint32_t j = ra + k;
                        const uint32_t dz = j < rc1 ? 0u : (j < rc2 ? 1u : 2u);
                        cw.nbr[rb + k] = j | ((uint32_t)(r * 3) + dz) << 16;
                    }
                }
                for (uint32_t i = lane; i < nh; i += 32) {
                    cw.fh[0][i] = 0.f;
                    cw.fh[1][i] = 0.f;
                    cw.fh[2][i] = 0.f;
                }
                __syncwarp();
                int qn = 0;
                for (uint32_t i = 0; i < nh; i++) {
                    const float4 pi = spos[h0 + i];
                    if (lane < 27) {
                        cw.shome[lane] = make_float4(__fsub_rn(pi.x, (float)(lane / 9 - 1)),
                                                     __fsub_rn(pi.y, (float)((lane / 3) % 3 - 1)),
                                                     __fsub_rn(pi.z, (float)(lane % 3 - 1)), 0.f);
                    }
                    __syncwarp();
                    for (uint32_t base = 0; base < M; base += 32) {
                        const uint32_t jj = base + lane;
                        bool inr = false;
                        uint32_t entry = 0;
                        if (jj < M) {
                            const uint32_t e = cw.nbr[jj];
                            const uint32_t j = e & 0xffffu, d = e >> 16;
                            const float4 sh = cw.shome[d];
                            float dx, dy, dz;
                            const float r2 = pair_r2(sh.x, sh.y, sh.z, spos[j], dx, dy, dz);
                            inr = r2 < 1.0f && r2 >= min2;
                            entry = j | (d << 11) | (i << 16);
                        }
                        const uint32_t mask = __ballot_sync(0xffffffffu, inr);
                        if (inr) cw.queue[qn + __popc(mask & ((1u << lane) - 1u))] = entry;
                        qn += __popc(mask);
                        __syncwarp();
                        if (qn >= 32) {
                            cell_eval_queue(cw, lane, 32, spos, svel, h0, spair, nt, th_lo, th_hi, scale);
                            const uint32_t moved = lane + 32 < qn ? cw.queue[lane + 32] : 0u;
                            __syncwarp();
                            if (lane + 32 < qn) cw.queue[lane] = moved;
                            qn -= 32;
                            __syncwarp();
                        }
                    }
                    __syncwarp();
                }
                if (qn > 0) cell_eval_queue(cw, lane, qn, spos, svel, h0, spair, nt, th_lo, th_hi, scale);
                for (uint32_t i = lane; i < nh; i += 32) {
                    sfx[h0 + i] = cw.fh[0][i];
                    sfy[h0 + i] = cw.fh[1][i];
                    sfz[h0 + i] = cw.fh[2][i];
                }
                __syncwarp();
            }
        }
        __syncthreads();

        // ---- one thread per home bead: bonds and integration
        uint32_t err = 0;
        for (uint32_t t = tid; t < n_home; t += BRICK_THREADS) {
            int r = 0;
            while (H.home_rows[r + 1] <= t) r++;
            const int lx = r / br.by, ly = r - lx * br.by;
            const int hc0 = ((lx + 1) * HY + (ly + 1)) * HZ + 1;
            const uint32_t k = t - H.home_rows[r];
            const uint32_t s = hslot[hc0] + k;
            if (!staged) {
                const float4 ph = ((const float4 *)a.posA)[s];
                const float4 vh = ((const float4 *)a.velA)[s];
                int c[3];
                decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
                float F[3] = {0.f, 0.f, 0.f};
                pair_forces32_seq(a, w, spair, th_lo, th_hi, scale, c, ph, vh, F);
                integrate32<FINAL>(a, w, s, c, ph, vh, F, err);
                continue;
            }
            const uint32_t si = hstart[hc0] + k;
            int z = 0;
            while (hstart[hc0 + z + 1] <= si) z++;
            const int c[3] = {br.x0 + lx, br.y0 + ly, br.z0 + z};
            float F[3] = {sfx[si], sfy[si], sfz[si]};
            integrate32<FINAL>(a, w, s, c, spos[si], svel[si], F, err);
        }
        if (err) atomicOr(&a.worlds[br.world].err, err);
    }
}
