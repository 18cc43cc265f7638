// Attach: the per-bead bond tables built on the device from the batch's flat bond lists.
//
// The bond kernels read each bead's bond terms from a CSR by global bead id: row[id] ..
// row[id + 1] index its BondTerm entries, Hookean terms first, then angle terms, each in the
// order of the flat lists (a bead belongs to one polymer, so this is the order in which the
// reference's per-polymer loop meets them, naive_dpd_engine_half_step.hpp:321-329).  Built
// here from the flat lists with global ids:
//   1. terms per bead, by atomic increments;
//   2. an exclusive scan of the counts -> row (the cell-list scan kernels of pdpd_sort.cu);
//   3. each term placed through an atomic per-bead cursor (an arbitrary order), then
//   4. each bead's few terms sorted by (parameter index, role), which is the flat-list order:
//      parameter k is Hookean bond k of the batch, n_bonds + g angle g.
// Also the list of polymer beads (monomer bit of the hash clear) in id order, which the bond
// kernels run over, by a scan of flags and a scatter.
#include "pdpd_device.cuh"

namespace pdpd {

namespace {

constexpr int BT = 256;
constexpr uint32_t MONOMER_BIT = 1u << 27;

__global__ void k_count_terms(const uint32_t *__restrict__ pairs, uint32_t n_bonds,
                              const uint32_t *__restrict__ triples, uint32_t n_angles, uint32_t *cnt)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_bonds) {
        atomicAdd(cnt + pairs[2 * k], 1u);
        atomicAdd(cnt + pairs[2 * k + 1], 1u);
    } else if (k - n_bonds < n_angles) {
        const uint32_t g = k - n_bonds;
        atomicAdd(cnt + triples[3 * g], 1u);
        atomicAdd(cnt + triples[3 * g + 1], 1u);
        atomicAdd(cnt + triples[3 * g + 2], 1u);
    }
}

__global__ void k_place_terms(const uint32_t *__restrict__ pairs, uint32_t n_bonds,
                              const uint32_t *__restrict__ triples, uint32_t n_angles, uint32_t *cursor,
                              BondTerm *__restrict__ terms)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_bonds) {
        const uint32_t h = pairs[2 * k], t = pairs[2 * k + 1];
        terms[atomicAdd(cursor + h, 1u)] = BondTerm{0u | (0u << 8), t, t, k};
        terms[atomicAdd(cursor + t, 1u)] = BondTerm{0u | (1u << 8), h, h, k};
    } else if (k - n_bonds < n_angles) {
        const uint32_t g = k - n_bonds;
        const uint32_t h = triples[3 * g], m = triples[3 * g + 1], t = triples[3 * g + 2];
        terms[atomicAdd(cursor + h, 1u)] = BondTerm{1u | (0u << 8), m, t, k};
        terms[atomicAdd(cursor + m, 1u)] = BondTerm{1u | (1u << 8), h, t, k};
        terms[atomicAdd(cursor + t, 1u)] = BondTerm{1u | (2u << 8), h, m, k};
    }
}

// Each bead's terms in (parameter, role) order: an insertion sort (a bead has a few terms).
__global__ void k_sort_terms(uint32_t n, const uint32_t *__restrict__ row, BondTerm *terms)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint32_t r0 = row[b], r1 = row[b + 1];
    for (uint32_t x = r0 + 1; x < r1; x++) {
        const BondTerm v = terms[x];
        uint32_t y = x;
        for (; y > r0; y--) {
            const BondTerm u = terms[y - 1];
            if (!(u.param > v.param || (u.param == v.param && u.meta > v.meta))) break;
            terms[y] = u;
        }
        terms[y] = v;
    }
}

__global__ void k_set_word(uint32_t *p, uint32_t v)
{
    *p = v;
}

__global__ void k_polymer_flags(uint32_t n, const uint32_t *__restrict__ hash, uint32_t *flag)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < n) flag[b] = (hash[b] & MONOMER_BIT) ? 0u : 1u;
}

// bonded[pos[b]] = b for the polymer beads; the thread of the last bead writes their number.
__global__ void k_polymer_list(uint32_t n, const uint32_t *__restrict__ hash, const uint32_t *__restrict__ pos,
                               uint32_t *bonded, uint32_t *count)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const bool polymer = !(hash[b] & MONOMER_BIT);
    if (polymer) bonded[pos[b]] = b;
    if (b == n - 1) *count = pos[b] + (polymer ? 1u : 0u);
}

}  // namespace

int launch_bond_tables(uint32_t n_beads, const uint32_t *pairs, uint32_t n_bonds, const uint32_t *triples,
                       uint32_t n_angles, const uint32_t *hash, uint32_t *row, BondTerm *terms, uint32_t *bonded,
                       uint32_t *n_bonded, uint32_t *scratch, uint32_t *pos, uint32_t *blocksums, cudaStream_t s)
{
    int launches = 0;
    const uint32_t n_terms = 2 * n_bonds + 3 * n_angles;
    const uint32_t gb = (n_beads + BT - 1) / BT;
    if (n_terms == 0) {
        cudaMemsetAsync(row, 0, sizeof(uint32_t) * ((size_t)n_beads + 1), s);
    } else {
        const uint32_t gt = (uint32_t)(((uint64_t)n_bonds + n_angles + BT - 1) / BT);
        cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (size_t)n_beads, s);
        k_count_terms<<<gt, BT, 0, s>>>(pairs, n_bonds, triples, n_angles, scratch);
        launch_scan(scratch, n_beads, blocksums, row, s);  // (clears the counts)
        k_set_word<<<1, 1, 0, s>>>(row + n_beads, n_terms);
        cudaMemcpyAsync(scratch, row, sizeof(uint32_t) * (size_t)n_beads, cudaMemcpyDeviceToDevice, s);
        k_place_terms<<<gt, BT, 0, s>>>(pairs, n_bonds, triples, n_angles, scratch, terms);
        k_sort_terms<<<gb, BT, 0, s>>>(n_beads, row, terms);
        launches += 6;
    }
    if (n_beads) {
        k_polymer_flags<<<gb, BT, 0, s>>>(n_beads, hash, scratch);
        launch_scan(scratch, n_beads, blocksums, pos, s);
        k_polymer_list<<<gb, BT, 0, s>>>(n_beads, hash, pos, bonded, n_bonded);
        launches += 4;
    } else {
        cudaMemsetAsync(n_bonded, 0, sizeof(uint32_t), s);
    }
    return launches;
}

}  // namespace pdpd
