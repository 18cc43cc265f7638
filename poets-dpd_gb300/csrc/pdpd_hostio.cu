// The attach's upload and the read-backs as one kernel that reads and writes the caller's host
// arrays directly, on devices that access pageable host memory coherently through the host's
// page tables (Grace-Blackwell: the GPU reaches the Grace CPU's memory over NVLink-C2C with
// address translation services).  The staged alternative copies every byte on the host twice
// (the caller's arrays to pinned staging, or back) around the DMA, so host memory bandwidth,
// not the link, bounds it; here the link carries each byte once and the host's cores do
// nothing.  The kernel touches exactly the host addresses the staged copies touch.
#include <algorithm>

#include "pdpd_internal.h"

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

}  // namespace

int launch_host_copy(const HostCopySeg *segs, const HostCopyChunk *chunks, uint32_t n_chunks, int sm_count,
                     cudaStream_t s)
{
    if (n_chunks == 0) return 0;
    const uint32_t grid = std::min<uint32_t>(n_chunks, 8u * (uint32_t)std::max(1, sm_count));
    k_host_copy<<<grid, HOSTCOPY_THREADS, 0, s>>>(segs, chunks, n_chunks);
    return 1;
}

}  // namespace pdpd
