// Observables of one attached world, reduced on the GPU in FP64:
//   ke2      sum over beads of |v|^2                 (kinetic temperature = ke2 / 3N, m = kT units)
//   mom      total momentum
//   virial   sum over pairs i<j with r < 1 of r * a_ij (1 - r)   (conservative pair virial)
//            + sum over Hookean bonds of r * kappa (r0 - r)
//   rdf      pair-distance histogram, r in [0, 1), per unordered bead-type pair
//   bonds    Hookean bond-length histogram, r in [0, 2)
// The pair sums visit each unordered pair once (the bead with the smaller id owns it).  Each
// block writes its partial sums to its own slot and the host adds the slots in order, so the
// result is deterministic; histograms are integer counts.
#include "pdpd_device.cuh"

namespace pdpd {

struct ObsPartial {
    double ke2, mx, my, mz, virial;
};

namespace {

template <int FP64>
__global__ void __launch_bounds__(128) k_observe(KArgs a, uint32_t world, uint32_t n_bins,
                                                 unsigned long long *rdf, uint32_t n_bond_bins,
                                                 unsigned long long *bond_hist, ObsPartial *part)
{
    __shared__ double red[5][128];
    const WorldDev w = a.worlds[world];
    const uint32_t nt = w.n_types;
    const uint32_t s = w.bead_base + blockIdx.x * blockDim.x + threadIdx.x;
    double ke2 = 0, mx = 0, my = 0, mz = 0, vir = 0;
    if (s < w.bead_base + w.n_beads) {
        int c[3];
        decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
        const uint32_t id = a.ids[s];
        double xi[3], vi[3];
        uint32_t hi;
        if (FP64) {
            const Vec4d p = ((const Vec4d *)a.posA)[s], v = ((const Vec4d *)a.velA)[s];
            xi[0] = p.x; xi[1] = p.y; xi[2] = p.z;
            vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
            hi = (uint32_t)__double_as_longlong(p.w);
        } else {
            const float4 p = ((const float4 *)a.posA)[s], v = ((const float4 *)a.velA)[s];
            xi[0] = p.x; xi[1] = p.y; xi[2] = p.z;  // offsets inside cell c
            vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
            hi = __float_as_uint(p.w);
        }
        ke2 = vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2];
        mx = vi[0];
        my = vi[1];
        mz = vi[2];
        const uint32_t ti = min(hi >> 28, nt - 1u);
        const double *pair = (const double *)a.pair;
        const float *pairf = (const float *)a.pair;
        for (int dxc = -1; dxc <= 1; dxc++)
            for (int dyc = -1; dyc <= 1; dyc++)
                for (int dzc = -1; dzc <= 1; dzc++) {
                    const int d[3] = {dxc, dyc, dzc};
                    int op[3];
                    double shift[3];
                    for (int k = 0; k < 3; k++) {
                        const int raw = c[k] + d[k];
                        op[k] = wrap_index(raw, w.L[k]);
                        // FP64 positions are absolute: the image shift is the wrap; FP32
                        // offsets are cell-relative: the shift is the direction itself.
                        shift[k] = FP64 ? (double)(raw - op[k]) : (double)d[k];
                    }
                    const uint32_t nc = w.cell_base + ((uint32_t)op[0] * (uint32_t)w.L[1] + (uint32_t)op[1]) * (uint32_t)w.L[2] + (uint32_t)op[2];
                    for (uint32_t j = a.start[nc]; j < a.start[nc + 1]; j++) {
                        if (a.ids[j] <= id) continue;
                        double xj[3];
                        uint32_t hj;
                        if (FP64) {
                            const Vec4d p = ((const Vec4d *)a.posA)[j];
                            xj[0] = p.x; xj[1] = p.y; xj[2] = p.z;
                            hj = (uint32_t)__double_as_longlong(p.w);
                        } else {
                            const float4 p = ((const float4 *)a.posA)[j];
                            xj[0] = p.x; xj[1] = p.y; xj[2] = p.z;
                            hj = __float_as_uint(p.w);
                        }
                        double r2 = 0;
                        for (int k = 0; k < 3; k++) {
                            const double dd = xi[k] - (xj[k] + shift[k]);
                            r2 += dd * dd;
                        }
                        if (r2 >= 1.0 || r2 <= 0.0) continue;
                        const double r = sqrt(r2);
                        const uint32_t tj = min(hj >> 28, nt - 1u);
                        double aij = FP64 ? pair[2 * (w.param_base + ti * nt + tj)]
                                          : (double)pairf[2 * (w.param_base + ti * nt + tj)];
                        if (w.spatial) {  // mean of the two cells' values
                            const size_t n2 = (size_t)nt * nt, pk = (size_t)ti * nt + tj;
                            const size_t h = (size_t)w.cellpair_base + (size_t)(a.cellg[s] - w.cell_base) * n2 + pk;
                            const size_t o = (size_t)w.cellpair_base + (size_t)(nc - w.cell_base) * n2 + pk;
                            aij = FP64 ? (((const double *)a.cellpair)[2 * h] + ((const double *)a.cellpair)[2 * o]) * 0.5
                                       : (double)((((const float *)a.cellpair)[2 * h] + ((const float *)a.cellpair)[2 * o]) * 0.5f);
                        }
                        vir += aij * (1.0 - r) * r;
                        if (rdf) {
                            const uint32_t lo = min(ti, tj), hi2 = max(ti, tj);
                            uint32_t bin = (uint32_t)(r * n_bins);
                            if (bin >= n_bins) bin = n_bins - 1;
                            atomicAdd(&rdf[(size_t)(lo * nt + hi2) * n_bins + bin], 1ull);
                        }
                    }
                }
        // Hookean bonds: the head bead owns the bond (role 0 of its CSR terms)
        if (!(hi & (1u << 27))) {
            for (uint32_t r0 = a.bond_row[id]; r0 < a.bond_row[id + 1]; r0++) {
                const BondTerm bt = a.bond_terms[r0];
                if ((bt.meta & 0xffu) != 0 || (bt.meta >> 8) != 0) continue;
                const uint32_t sp = a.slot_of_id[bt.a];
                double dvec[3];
                if (FP64) {
                    const Vec4d p = ((const Vec4d *)a.posA)[sp];
                    const double xp[3] = {p.x, p.y, p.z};
                    for (int k = 0; k < 3; k++) {
                        double dd = xp[k] - xi[k];
                        const double L = (double)w.L[k];
                        if (dd > 0.5 * L) dd -= L;
                        else if (dd < -0.5 * L) dd += L;
                        dvec[k] = dd;
                    }
                } else {
                    const float4 p = ((const float4 *)a.posA)[sp];
                    int pc[3];
                    decode_cell(a.cellg[sp] - w.cell_base, w.L, pc[0], pc[1], pc[2]);
                    const double xp[3] = {p.x, p.y, p.z};
                    for (int k = 0; k < 3; k++) {
                        double dd = (double)(pc[k] - c[k]) + (xp[k] - xi[k]);
                        const double L = (double)w.L[k];
                        if (dd > 0.5 * L) dd -= L;
                        else if (dd < -0.5 * L) dd += L;
                        dvec[k] = dd;
                    }
                }
                const double r = sqrt(dvec[0] * dvec[0] + dvec[1] * dvec[1] + dvec[2] * dvec[2]);
                double kap, r0v;
                if (FP64) {
                    const Vec4d prm = ((const Vec4d *)a.bond_params)[bt.param];
                    kap = prm.x;
                    r0v = prm.y;
                } else {
                    const float4 prm = ((const float4 *)a.bond_params)[bt.param];
                    kap = prm.x;
                    r0v = prm.y;
                }
                vir += kap * (r0v - r) * r;
                if (bond_hist && n_bond_bins) {
                    uint32_t bin = (uint32_t)(r / 2.0 * n_bond_bins);
                    if (bin >= n_bond_bins) bin = n_bond_bins - 1;
                    atomicAdd(&bond_hist[bin], 1ull);
                }
            }
        }
    }
    red[0][threadIdx.x] = ke2;
    red[1][threadIdx.x] = mx;
    red[2][threadIdx.x] = my;
    red[3][threadIdx.x] = mz;
    red[4][threadIdx.x] = vir;
    __syncthreads();
    for (int off = 64; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off)
            for (int k = 0; k < 5; k++) red[k][threadIdx.x] += red[k][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ObsPartial o = {red[0][0], red[1][0], red[2][0], red[3][0], red[4][0]};
        part[blockIdx.x] = o;
    }
}

}  // namespace

int launch_observe(const KArgs &a, int fp64, uint32_t world, uint32_t n_beads, uint32_t n_bins,
                   unsigned long long *rdf, uint32_t n_bond_bins, unsigned long long *bond_hist,
                   ObsPartial *part, cudaStream_t s)
{
    const uint32_t blocks = (n_beads + 127) / 128;
    if (blocks == 0) return 0;
    if (fp64)
        k_observe<1><<<blocks, 128, 0, s>>>(a, world, n_bins, rdf, n_bond_bins, bond_hist, part);
    else
        k_observe<0><<<blocks, 128, 0, s>>>(a, world, n_bins, rdf, n_bond_bins, bond_hist, part);
    return 1;
}

}  // namespace pdpd
