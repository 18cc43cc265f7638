// The attach's upload (k_host_copy) and the read-backs (k_slot_of_id + k_read_direct) as
// kernels that read and write the caller's host arrays directly, on devices that access
// pageable host memory coherently through the host's page tables (Grace-Blackwell: the GPU
// reaches the Grace CPU's memory over NVLink-C2C with address translation services).  The
// staged alternative copies every byte on the host twice (the caller's arrays to pinned
// staging, or back) around the DMA, so host memory bandwidth, not the link, bounds it; here
// the link carries each byte once and the host's cores do nothing.  The kernels touch exactly
// the host bytes the staged copies touch, and run at the link's DMA rate.
#include <algorithm>

#include "pdpd_device.cuh"

namespace pdpd {
namespace {

constexpr int HOSTCOPY_THREADS = 256;

// One block per chunk (grid-stride over the chunks).  Contiguous runs are copied as words,
// four loads in flight per thread ahead of their stores (the link's latency is long); strided
// bead arrays as triples of doubles, a thread per bead.
__global__ void __launch_bounds__(HOSTCOPY_THREADS) k_host_copy(const HostCopySeg *__restrict__ segs,
                                                                const HostCopyChunk *__restrict__ chunks,
                                                                uint32_t n_chunks)
{
    const uint32_t T = blockDim.x;
    for (uint32_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const HostCopyChunk ch = chunks[c];
        const HostCopySeg sg = segs[ch.seg];
        const uint32_t n = ch.count;
        if (sg.kind == HOSTCOPY_WORDS8) {
            const unsigned long long *src = (const unsigned long long *)sg.src + ch.first;
            unsigned long long *dst = (unsigned long long *)sg.dst + ch.first;
            uint32_t i = threadIdx.x;
            for (; i + 3 * T < n; i += 4 * T) {
                const unsigned long long a0 = src[i], a1 = src[i + T], a2 = src[i + 2 * T], a3 = src[i + 3 * T];
                dst[i] = a0;
                dst[i + T] = a1;
                dst[i + 2 * T] = a2;
                dst[i + 3 * T] = a3;
            }
            for (; i < n; i += T) dst[i] = src[i];
        } else if (sg.kind == HOSTCOPY_WORDS4) {
            const uint32_t *src = (const uint32_t *)sg.src + ch.first;
            uint32_t *dst = (uint32_t *)sg.dst + ch.first;
            uint32_t i = threadIdx.x;
            for (; i + 3 * T < n; i += 4 * T) {
                const uint32_t a0 = src[i], a1 = src[i + T], a2 = src[i + 2 * T], a3 = src[i + 3 * T];
                dst[i] = a0;
                dst[i + T] = a1;
                dst[i + 2 * T] = a2;
                dst[i + 3 * T] = a3;
            }
            for (; i < n; i += T) dst[i] = src[i];
        } else {
            for (uint32_t i = threadIdx.x; i < n; i += T) {
                const uint64_t k = ch.first + i;
                const double *s = (const double *)((const char *)sg.src + k * sg.src_stride);
                double *d = (double *)((char *)sg.dst + k * sg.dst_stride);
                const double a0 = s[0], a1 = s[1], a2 = s[2];
                d[0] = a0;
                d[1] = a1;
                d[2] = a2;
            }
        }
    }
}

__global__ void k_slot_of_id(const uint32_t *__restrict__ ids, uint32_t first, uint32_t count, uint32_t *inv)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) inv[ids[first + k]] = first + k;
}

// The read-back without device staging: a block per tile of bead ids gathers the tile's beads
// from their sorted slots (random 16- or 32-byte reads in device memory), lays x, v and f out
// in shared memory in the caller's order, and writes each field of a stride-24 array in whole
// 128-byte lines of host memory (otherwise bead by bead).  Lines a tile's run shares with the
// next tile's are written whole by the tile whose run holds the line's first byte, which
// gathers the few beads of the next tile the line reaches: a line written in parts by two
// blocks crossed the host link a fifth slower (152 against 193 GB/s for 3 KB runs 8 bytes off
// the line boundary, on a GB300).  The link carries each byte once and the gathers overlap
// it.  x = cell + offset in FP32 and the FP32 -> FP64 conversions are those of the unsort
// kernels, so the values are the same.
constexpr int LINE_BEADS = 6;  // beads past a tile that a 128-byte line can reach (120 / 24 + 1)

template <int F64>
__global__ void __launch_bounds__(TILE_BEADS) k_read_direct(KArgs a, const uint32_t *__restrict__ inv,
                                                            const ReadDest *__restrict__ dest)
{
    __shared__ double sh[3][3 * (TILE_BEADS + LINE_BEADS)];
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        const WorldDev &w = a.worlds[tl.world];
        const uint32_t cnt = tl.slot_end - tl.slot_begin;
        const uint32_t extra = min((uint32_t)LINE_BEADS, w.bead_base + w.n_beads - tl.slot_end);
        for (uint32_t t = threadIdx.x; t < cnt + extra; t += TILE_BEADS) {
            const uint32_t s = inv[tl.slot_begin + t];
            double x[3], v[3], f[3];
            if (F64) {
                const Vec4d p = ((const Vec4d *)a.posA)[s];
                const Vec4d vv = ((const Vec4d *)a.velA)[s];
                const Vec4d ff = ((const Vec4d *)a.frc)[s];
                x[0] = p.x, x[1] = p.y, x[2] = p.z;
                v[0] = vv.x, v[1] = vv.y, v[2] = vv.z;
                f[0] = ff.x, f[1] = ff.y, f[2] = ff.z;
            } else {
                const float4 p = ((const float4 *)a.posA)[s];
                const float4 vv = ((const float4 *)a.velA)[s];
                const float4 ff = ((const float4 *)a.frc)[s];
                int c[3];
                decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
                x[0] = (double)c[0] + (double)p.x;
                x[1] = (double)c[1] + (double)p.y;
                x[2] = (double)c[2] + (double)p.z;
                v[0] = vv.x, v[1] = vv.y, v[2] = vv.z;
                f[0] = ff.x, f[1] = ff.y, f[2] = ff.z;
            }
#pragma unroll
            for (int d = 0; d < 3; d++) {
                sh[0][3 * t + d] = x[d];
                sh[1][3 * t + d] = v[d];
                sh[2][3 * t + d] = f[d];
            }
        }
        __syncthreads();
        const ReadDest D = dest[tl.world];
        const uint64_t k0 = tl.slot_begin - w.bead_base;  // the tile's first bead in its world
        double *out[3] = {D.x, D.v, D.f};
#pragma unroll
        for (int q = 0; q < 3; q++) {
            if (!out[q]) continue;
            if (D.stride == 24) {
                // the doubles [i0, i1) of the array this tile writes: from the first line boundary
                // in its run (the array's start for its first tile) to the end of the line that
                // holds its run's last byte, within the array
                const uintptr_t A = (uintptr_t)out[q];
                const uintptr_t run0 = A + 24 * k0, run1 = A + 24 * (k0 + cnt);
                const uintptr_t end = A + 24 * (uintptr_t)w.n_beads;
                const uintptr_t w0 = k0 == 0 ? A : (run0 + 127) & ~(uintptr_t)127;
                const uintptr_t w1 = min((run1 + 127) & ~(uintptr_t)127, end);
                if (w1 > w0) {
                    const uint32_t i0 = (uint32_t)((w0 - A) / 8 - 3 * k0), n = (uint32_t)((w1 - w0) / 8);
                    double *o = (double *)w0;
                    for (uint32_t i = threadIdx.x; i < n; i += TILE_BEADS) o[i] = sh[q][i0 + i];
                }
            } else {
                for (uint32_t t = threadIdx.x; t < cnt; t += TILE_BEADS) {
                    double *o = (double *)((char *)out[q] + (k0 + t) * D.stride);
                    o[0] = sh[q][3 * t];
                    o[1] = sh[q][3 * t + 1];
                    o[2] = sh[q][3 * t + 2];
                }
            }
        }
        __syncthreads();
    }
}

// The rest state to id-ordered device staging (rows of 9 doubles, or field-major blocks of
// staging_n beads each), as a gather: a thread per bead id of a tile reads the bead from its
// sorted slot through inv and writes its row or vectors where consecutive ids are adjacent, so
// the stores of a warp are contiguous (a scatter from the sorted order writes 24- or 72-byte
// pieces all over the staging, each a partial write of its sectors).
template <int F64>
__global__ void __launch_bounds__(TILE_BEADS) k_unsort_gather(KArgs a, const uint32_t *__restrict__ inv)
{
    const size_t stride = a.staging_fields ? 3 : 9, field = a.staging_fields ? 3 * (size_t)a.staging_n : 3;
    for (uint32_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const Tile tl = a.tiles[tile];
        const uint32_t id = tl.slot_begin + threadIdx.x;
        if (id >= tl.slot_end) continue;
        const uint32_t s = inv[id];
        double *st = a.staging + stride * id;
        if (F64) {
            const Vec4d p = ((const Vec4d *)a.posA)[s];
            const Vec4d v = ((const Vec4d *)a.velA)[s];
            const Vec4d f = ((const Vec4d *)a.frc)[s];
            st[0] = p.x, st[1] = p.y, st[2] = p.z;
            st[field + 0] = v.x, st[field + 1] = v.y, st[field + 2] = v.z;
            st[2 * field + 0] = f.x, st[2 * field + 1] = f.y, st[2 * field + 2] = f.z;
        } else {
            const WorldDev &w = a.worlds[tl.world];
            const float4 p = ((const float4 *)a.posA)[s];
            const float4 v = ((const float4 *)a.velA)[s];
            const float4 f = ((const float4 *)a.frc)[s];
            int c[3];
            decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
            st[0] = (double)c[0] + (double)p.x;  // x = cell + offset exactly
            st[1] = (double)c[1] + (double)p.y;
            st[2] = (double)c[2] + (double)p.z;
            st[field + 0] = v.x, st[field + 1] = v.y, st[field + 2] = v.z;
            st[2 * field + 0] = f.x, st[2 * field + 1] = f.y, st[2 * field + 2] = f.z;
        }
    }
}

}  // namespace

int launch_unsort(const KArgs &a, int fp64, const uint32_t *inv, cudaStream_t s)
{
    if (a.n_tiles == 0) return 0;
    const uint32_t grid = std::min<uint32_t>(a.n_tiles, (uint32_t)std::max(1, a.grid_blocks));
    if (fp64)
        k_unsort_gather<1><<<grid, TILE_BEADS, 0, s>>>(a, inv);
    else
        k_unsort_gather<0><<<grid, TILE_BEADS, 0, s>>>(a, inv);
    return 1;
}

int launch_slot_of_id(const KArgs &a, uint32_t first, uint32_t count, uint32_t *inv, cudaStream_t s)
{
    if (count == 0) return 0;
    k_slot_of_id<<<(count + 255) / 256, 256, 0, s>>>(a.ids, first, count, inv);
    return 1;
}

int launch_read_direct(const KArgs &a, int fp64, const uint32_t *inv, const ReadDest *dest, cudaStream_t s)
{
    if (a.n_tiles == 0) return 0;
    const uint32_t grid = std::min<uint32_t>(a.n_tiles, (uint32_t)std::max(1, a.grid_blocks));
    if (fp64)
        k_read_direct<1><<<grid, TILE_BEADS, 0, s>>>(a, inv, dest);
    else
        k_read_direct<0><<<grid, TILE_BEADS, 0, s>>>(a, inv, dest);
    return 1;
}

int launch_host_copy(const HostCopySeg *segs, const HostCopyChunk *chunks, uint32_t n_chunks, int sm_count,
                     cudaStream_t s)
{
    if (n_chunks == 0) return 0;
    const uint32_t grid = std::min<uint32_t>(n_chunks, 8u * (uint32_t)std::max(1, sm_count));
    k_host_copy<<<grid, HOSTCOPY_THREADS, 0, s>>>(segs, chunks, n_chunks);
    return 1;
}

}  // namespace pdpd
