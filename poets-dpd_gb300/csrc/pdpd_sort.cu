// Cell-list rebuild: a counting sort of the advanced beads by their new cell.
//
// The step kernels have already counted each cell's arrivals (one atomicAdd per bead, which
// also gives the bead a provisional rank inside its new cell).  Here:
//   1. k_scan_reduce + k_scan_final: exclusive prefix sum of the counts -> start[] (and
//      the counts are cleared for the next step);
//   2. k_place: each bead writes (old slot, id, cell, z half) at start[cell] + provisional rank;
//   3. k_canon: each placed bead re-ranks itself by (z half, bead id) inside its cell and
//      moves its payload to start[cell] + that rank.
// The result is canonical: cells in index order, beads inside a cell in ascending bead id,
// whatever order the atomics ran in.  That is the order in which the reference's cell lists
// hold beads (naive_dpd_engine_half_step.hpp:276-293), so the FP64 force kernel adds pair
// forces in the reference's order and the engine is deterministic run to run.  The FP32
// engine marks beads whose cell offset z is >= 0.5 (bit 31 of the arrival rank): they follow
// the lower-half beads of their cell, still in id order, and zlo[cell] counts the lower
// half, so the FP32 neighbour walk can skip the far half of an end cell.
#include "pdpd_device.cuh"

namespace pdpd {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr uint32_t SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

uint32_t scan_blocks(uint32_t n_cells)
{
    return (n_cells + SCAN_CHUNK - 1) / SCAN_CHUNK;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    uint32_t r = 0;
    if (warp == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (lane == 0) sh[0] = r;
    }
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t *__restrict__ cnt,
                                                               uint32_t n, uint32_t *blocksums,
                                                               WorldDev *worlds, uint32_t n_worlds,
                                                               int tick, uint32_t *brick_next)
{
    // the next force pass takes its bricks from a fresh queue
    if (brick_next && blockIdx.x == 0 && threadIdx.x == 0) *brick_next = 0u;
    __shared__ uint32_t sh[32];
    const uint32_t base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < n) s += cnt[base + k];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) blocksums[blockIdx.x] = s;
    // The force pass that produced these counts has finished: advance every world's t.
    if (tick && blockIdx.x == 0)
        for (uint32_t w = threadIdx.x; w < n_worlds; w += blockDim.x) worlds[w].t += 1;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_final(uint32_t *__restrict__ cnt, uint32_t n,
                                                              const uint32_t *__restrict__ blocksums,
                                                              uint32_t *__restrict__ start)
{
    __shared__ uint32_t sh[32];
    // Offset of this chunk: sum of the preceding chunks' totals.
    uint32_t off = 0;
    for (uint32_t b = threadIdx.x; b < blockIdx.x; b += blockDim.x) off += blocksums[b];
    off = block_sum(off, sh);

    const uint32_t base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < n) ? cnt[base + k] : 0u;
        tsum += v[k];
    }
    // Block-wide exclusive scan of the thread totals.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t inc = tsum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) sh[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        sh[lane] = wi - w;  // exclusive warp offsets
    }
    __syncthreads();
    uint32_t run = off + sh[warp] + (inc - tsum);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) {
            start[base + k] = run;
            cnt[base + k] = 0u;
        }
        run += v[k];
    }
}

__global__ void k_place(uint32_t n, const uint2 *__restrict__ keyrank,
                        const uint32_t *__restrict__ start, const uint32_t *__restrict__ ids,
                        uint4 *__restrict__ tmp)
{
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    uint2 kr = keyrank[s];
    uint32_t dst = start[kr.x] + (kr.y & 0x7fffffffu);
    tmp[dst] = make_uint4(s, ids[s], kr.x, kr.y >> 31);
}

// The bead hash carried in the w component of a position payload.
__device__ __forceinline__ uint32_t payload_hash(const float4 &p)
{
    return __float_as_uint(p.w);
}
__device__ __forceinline__ uint32_t payload_hash(const Vec4d &p)
{
    return (uint32_t)__double_as_longlong(p.w);
}

// FP64 positions as FP32 offsets inside their cell (x - floor(x) is exact in FP64, the cell
// being floor(x)), for the force kernel's distance prefilter; the hash rides along.
__device__ __forceinline__ float4 offset_shadow(const float4 &p)
{
    return p;
}
__device__ __forceinline__ float4 offset_shadow(const Vec4d &p)
{
    return make_float4((float)(p.x - floor(p.x)), (float)(p.y - floor(p.y)), (float)(p.z - floor(p.z)),
                       __uint_as_float(payload_hash(p)));
}

// slot_of_id is kept for polymer beads only (monomer bit of the hash clear): the bond kernels
// look up bond partners through it; the codec walks slots and reads ids instead.
template <class P>
__global__ void k_canon(uint32_t n, const uint4 *__restrict__ tmp, const uint32_t *__restrict__ start,
                        const P *__restrict__ pos_in, const P *__restrict__ vel_in,
                        const P *__restrict__ frc_in, P *__restrict__ pos_out,
                        P *__restrict__ vel_out, P *__restrict__ frc_out,
                        uint32_t *__restrict__ ids_out, uint32_t *__restrict__ cellg_out,
                        uint32_t *__restrict__ slot_of_id, float4 *__restrict__ shadow_out,
                        uint16_t *__restrict__ zlo)
{
    uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    uint4 e = tmp[d];
    uint32_t b = start[e.z], end = start[e.z + 1];
    uint32_t rank = 0, lo = 0;
    for (uint32_t k = b; k < end; k++) {
        const uint4 o = tmp[k];
        rank += (o.w < e.w || (o.w == e.w && o.y < e.y)) ? 1u : 0u;
        lo += o.w == 0u ? 1u : 0u;
    }
    if (zlo && rank == 0) zlo[e.z] = (uint16_t)min(lo, 0xffffu);
    uint32_t dst = b + rank;
    const P p = pos_in[e.x];
    pos_out[dst] = p;
    vel_out[dst] = vel_in[e.x];
    if (frc_in) frc_out[dst] = frc_in[e.x];
    ids_out[dst] = e.y;
    cellg_out[dst] = e.z;
    if (!(payload_hash(p) & (1u << 27))) slot_of_id[e.y] = dst;
    if (shadow_out) shadow_out[dst] = offset_shadow(p);
}

void launch_scan(uint32_t *cnt, uint32_t n, uint32_t *blocksums, uint32_t *start, cudaStream_t s)
{
    if (n == 0) return;
    const uint32_t nb = scan_blocks(n);
    k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(cnt, n, blocksums, nullptr, 0, 0, nullptr);
    k_scan_final<<<nb, SCAN_THREADS, 0, s>>>(cnt, n, blocksums, start);
}

int launch_sort(const KArgs &a, int fp64, int tick, int with_force, cudaStream_t s)
{
    const uint32_t nb = scan_blocks(a.n_cells);
    k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(a.cnt, a.n_cells, a.blocksums, a.worlds, a.n_worlds,
                                              tick, a.brick_next);
    k_scan_final<<<nb, SCAN_THREADS, 0, s>>>(a.cnt, a.n_cells, a.blocksums, a.start);
    const int T = 256;
    const uint32_t g = (a.n_beads + T - 1) / T;
    if (a.n_beads == 0) return 2;
    k_place<<<g, T, 0, s>>>(a.n_beads, a.keyrank, a.start, a.ids, a.tmp);
    if (fp64) {
        k_canon<Vec4d><<<g, T, 0, s>>>(a.n_beads, a.tmp, a.start, (const Vec4d *)a.posB,
                                       (const Vec4d *)a.velB,
                                       with_force ? (const Vec4d *)a.frcB : nullptr,
                                       (Vec4d *)a.posA, (Vec4d *)a.velA, (Vec4d *)a.frc, a.ids,
                                       a.cellg, a.slot_of_id, a.posf, nullptr);
    } else {
        k_canon<float4><<<g, T, 0, s>>>(a.n_beads, a.tmp, a.start, (const float4 *)a.posB,
                                        (const float4 *)a.velB,
                                        with_force ? (const float4 *)a.frcB : nullptr,
                                        (float4 *)a.posA, (float4 *)a.velA, (float4 *)a.frc,
                                        a.ids, a.cellg, a.slot_of_id, nullptr, a.zlo);
    }
    return 4;
}

__global__ void k_rng_eval(size_t n, const uint32_t *__restrict__ t, const uint64_t *__restrict__ seed,
                           const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                           uint32_t *__restrict__ h_out, float *__restrict__ u_out)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t th = t_hash(t[i], seed[i]);
    uint32_t lo = (uint32_t)th, hi = (uint32_t)(th >> 32);
    h_out[i] = hash_rng_sym(lo, hi, a[i], b[i]);
    u_out[i] = hash_u(lo, hi, a[i], b[i]);
}

int launch_rng_eval(size_t n, const uint32_t *t, const uint64_t *seed, const uint32_t *a,
                    const uint32_t *b, uint32_t *h_out, float *u_out, cudaStream_t s)
{
    if (n == 0) return 0;
    k_rng_eval<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, t, seed, a, b, h_out, u_out);
    return 1;
}

size_t payload_bytes(int fp64)
{
    return fp64 ? sizeof(Vec4d) : sizeof(float4);
}

}  // namespace pdpd
