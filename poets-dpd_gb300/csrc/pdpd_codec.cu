// v2binary snapshot codec on the GPU: the bead records of the BinaryData section of the
// reference's "WorldState v2binary" format (dpd_state_io.hpp:182-247 write_polymer_binary,
// :249-330 read_polymer_binary), encoded straight from the sorted device state.
//
// The section's structure -- per polymer a 16-bit header and optional id deltas -- depends
// only on the topology, so the host writes it once into a device buffer (the layout) with
// the byte offset of every bead's 20-byte record.  A snapshot then fills in the records:
//   position: 3 x uint32, round(x * 65536) (half away from zero), the box side wrapping to 0;
//   v, f: CVec3Half each (cvec3.hpp:132-252): a 5-bit exponent field (e + 15, 0 for the zero
//   vector) and three 9-bit two's-complement mantissas round(c * 2^(8 - e)), low bits first,
//   where e is the largest frexp exponent of the non-zero components (e + 1 if a mantissa
//   rounds to +-256); zero and subnormal components count as zero, e < -14 gives the zero
//   vector, e > 15 or a non-finite component is an error.
// Every step is exact in IEEE double (frexp, ldexp, round), so the bytes equal the reference
// writer's for the same state.  Records start at even offsets (headers are 2 bytes, deltas 4,
// records 20) and are written as 16-bit words.
#include <cfloat>

#include "pdpd_device.cuh"

namespace pdpd {

namespace {

constexpr uint32_t V2_ERR_VECTOR = 1u;  // non-finite component or magnitude >= 2^15
constexpr uint32_t V2_ERR_BOX = 2u;     // a position outside [0, L)

__device__ __forceinline__ bool cvec3half_encode(const double po[3], uint32_t &word)
{
    double p[3];
    bool any = false;
    int e = -100000;
    for (int i = 0; i < 3; i++) {
        if (!isfinite(po[i])) return false;
        p[i] = fabs(po[i]) < DBL_MIN ? 0.0 : po[i];  // zero and subnormal components
        if (p[i] != 0.0) {
            int ex;
            frexp(p[i], &ex);
            e = max(e, ex);
            any = true;
        }
    }
    if (!any || e < -14) {
        word = 0u;
        return true;
    }
    if (e > 15) return false;
    double fr[3];
    bool over = false;
    for (int i = 0; i < 3; i++) {
        fr[i] = round(ldexp(p[i], 8 - e));
        over |= fabs(fr[i]) == 256.0;
    }
    if (over) {
        e += 1;
        if (e > 15) return false;
        for (int i = 0; i < 3; i++) fr[i] = round(ldexp(p[i], 8 - e));
    }
    word = ((uint32_t)(e + 15) & 0x1Fu) | (((uint32_t)(int)fr[0] & 0x1FFu) << 5) |
           (((uint32_t)(int)fr[1] & 0x1FFu) << 14) | (((uint32_t)(int)fr[2] & 0x1FFu) << 23);
    return true;
}

__device__ __forceinline__ void cvec3half_decode(uint32_t w, double out[3])
{
    const int ex = (int)(w & 0x1Fu);
    for (int i = 0; i < 3; i++) {
        int m = (int)((w >> (5 + 9 * i)) & 0x1FFu);
        if (m >= 256) m -= 512;
        out[i] = ldexp((double)m, ex - 23);
    }
}

__device__ __forceinline__ void store_words(uint8_t *dst, const uint32_t w[5])
{
    uint16_t *d = reinterpret_cast<uint16_t *>(dst);  // even offset
    for (int k = 0; k < 5; k++) {
        d[2 * k] = (uint16_t)(w[k] & 0xFFFFu);
        d[2 * k + 1] = (uint16_t)(w[k] >> 16);
    }
}

__device__ __forceinline__ void load_words(const uint8_t *src, uint32_t w[5])
{
    const uint16_t *s = reinterpret_cast<const uint16_t *>(src);
    for (int k = 0; k < 5; k++) w[k] = (uint32_t)s[2 * k] | ((uint32_t)s[2 * k + 1] << 16);
}

template <int FP64>
__global__ void k_v2_encode(KArgs a, uint32_t world, uint32_t n, uint8_t *__restrict__ buf,
                            const uint32_t *__restrict__ off, uint32_t *err)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const WorldDev &w = a.worlds[world];
    const uint32_t s = w.bead_base + k;        // walk the world's slots (coalesced reads)
    const uint32_t i = a.ids[s] - w.bead_base;  // the bead in slot s: its record
    double x[3], v[3], f[3];
    if (FP64) {
        const Vec4d p = ((const Vec4d *)a.posA)[s], vv = ((const Vec4d *)a.velA)[s],
                    ff = ((const Vec4d *)a.frc)[s];
        x[0] = p.x; x[1] = p.y; x[2] = p.z;
        v[0] = vv.x; v[1] = vv.y; v[2] = vv.z;
        f[0] = ff.x; f[1] = ff.y; f[2] = ff.z;
    } else {
        const float4 p = ((const float4 *)a.posA)[s], vv = ((const float4 *)a.velA)[s],
                     ff = ((const float4 *)a.frc)[s];
        int c[3];
        decode_cell(a.cellg[s] - w.cell_base, w.L, c[0], c[1], c[2]);
        x[0] = (double)c[0] + (double)p.x;
        x[1] = (double)c[1] + (double)p.y;
        x[2] = (double)c[2] + (double)p.z;
        v[0] = vv.x; v[1] = vv.y; v[2] = vv.z;
        f[0] = ff.x; f[1] = ff.y; f[2] = ff.z;
    }
    uint32_t word[5];
    uint32_t bad = 0;
    for (int d = 0; d < 3; d++) {
        const double side = (double)w.L[d] * 65536.0;
        double rr = round(x[d] * 65536.0);
        if (rr == side) rr = 0.0;
        if (!(rr >= 0.0 && rr < side)) {
            bad |= V2_ERR_BOX;
            rr = 0.0;
        }
        word[d] = (uint32_t)rr;
    }
    if (!cvec3half_encode(v, word[3])) bad |= V2_ERR_VECTOR;
    if (!cvec3half_encode(f, word[4])) bad |= V2_ERR_VECTOR;
    store_words(buf + off[i], word);
    if (bad) atomicOr(err, bad);
}

// Decode one world's records into the id-ordered staging rows (x, v, f per bead).
__global__ void k_v2_decode(KArgs a, uint32_t world, uint32_t n, const uint8_t *__restrict__ buf,
                            const uint32_t *__restrict__ off, double *__restrict__ staging,
                            uint32_t *err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const WorldDev &w = a.worlds[world];
    uint32_t word[5];
    load_words(buf + off[i], word);
    double *row = staging + 9 * (size_t)(w.bead_base + i);
    for (int d = 0; d < 3; d++) {
        const double x = ldexp((double)word[d], -16);
        if (!(x < (double)w.L[d])) atomicOr(err, V2_ERR_BOX);
        row[d] = x;
    }
    cvec3half_decode(word[3], row + 3);
    cvec3half_decode(word[4], row + 6);
}

}  // namespace

int launch_v2_encode(const KArgs &a, int fp64, uint32_t world, uint32_t n, uint8_t *buf,
                     const uint32_t *off, uint32_t *err, cudaStream_t s)
{
    if (n == 0) return 0;
    const uint32_t g = (n + 255) / 256;
    if (fp64)
        k_v2_encode<1><<<g, 256, 0, s>>>(a, world, n, buf, off, err);
    else
        k_v2_encode<0><<<g, 256, 0, s>>>(a, world, n, buf, off, err);
    return 1;
}

int launch_v2_decode(const KArgs &a, uint32_t world, uint32_t n, const uint8_t *buf,
                     const uint32_t *off, double *staging, uint32_t *err, cudaStream_t s)
{
    if (n == 0) return 0;
    k_v2_decode<<<(n + 255) / 256, 256, 0, s>>>(a, world, n, buf, off, staging, err);
    return 1;
}

}  // namespace pdpd
