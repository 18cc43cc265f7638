// Internal interface between the host runtime (pdpd_engine.cpp) and the kernel
// translation units (pdpd_fp32.cu, pdpd_fp64.cu, pdpd_sort.cu, pdpd_bondcsr.cu, pdpd_hostio.cu,
// pdpd_observe.cu, pdpd_codec.cu).  Not part of the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace pdpd {

// Per-world parameters and state, resident on the device.  Worlds of a batch share one
// arena: world w owns global cells [cell_base, cell_base+n_cells) and global bead slots /
// ids [bead_base, bead_base+n_beads).
struct WorldDev {
    int32_t L[3];
    uint32_t cell_base;
    uint32_t n_cells;
    uint32_t bead_base;
    uint32_t n_beads;
    uint32_t n_types;
    uint32_t param_base;  // first entry of this world's n_types^2 pair parameters
    uint32_t err;         // device-side error flags (ERR_*)
    uint32_t stationary;  // bit k: bead type k is stationary (not moved; v, f cleared each step)
    uint32_t spatial;     // 1: per-cell strengths at cellpair[cellpair_base + local cell * n_types^2]
    double dt;
    double scale_inv_sqrt_dt;  // sqrt(24 kT / dt), kT = 1 (dpd_maths_core.hpp:24)
    uint64_t seed;
    int64_t t;
    uint64_t cellpair_base;
};

// A run of consecutive sorted bead slots of one world: the unit of work of the step
// kernels.  A world's beads always occupy the same slot range [bead_base, bead_base+n)
// (the cell list only permutes them inside it), so the tiles are fixed at attach.
struct Tile {
    uint32_t world;
    uint32_t slot_begin;
    uint32_t slot_end;
    uint32_t pad;
};

// Beads per tile = threads per block of the step kernels.
constexpr int TILE_BEADS = 128;

// A brick of cells of one world: the unit of work of the FP32 force kernel, which stages
// the brick and its one-cell halo in shared memory.  Bricks are cut at the box faces, so
// edge bricks can be smaller than the nominal shape.
struct Brick {
    uint32_t world;
    int32_t x0, y0, z0;  // first cell of the brick (world cell coordinates)
    int32_t bx, by, bz;  // brick extent in cells
    uint32_t pad;
};

// Default brick shape (cells), the autotuner's usual pick on GB300; bx * by <= 64.
constexpr int BRICK_X = 4, BRICK_Y = 8, BRICK_Z = 8;

enum ErrFlags : uint32_t {
    ERR_BOND_SNAPPED = 1u,  // Hookean bond longer than the maximum bond length
    ERR_NONFINITE = 2u,     // non-finite position / velocity / force
    ERR_OUT_OF_BOX = 4u,    // a bead outside [0, L) on attach, or moved more than a box
};

// Bond term of the per-bead CSR: what one bead contributes to itself from one Hookean bond
// or one angle bond.  kind: 0 Hookean, 1 angle.  role: Hookean 0 head / 1 tail; angle
// 0 head / 1 middle / 2 tail.  a, b: the other bead ids of the term in (head, middle,
// tail) order.  param: index into the bond parameter table.
struct BondTerm {
    uint32_t meta;  // kind | role << 8
    uint32_t a;
    uint32_t b;
    uint32_t param;
};

// Everything a step kernel needs.  Pointers are device pointers; the payload arrays are
// float4 (FP32 engine) or Vec4d (FP64 engine).
struct KArgs {
    WorldDev *worlds;
    uint32_t n_worlds;
    const Tile *tiles;
    uint32_t n_tiles;
    const Brick *bricks;
    uint32_t n_bricks;
    uint32_t n_beads;  // total over all worlds
    uint32_t n_cells;  // total over all worlds
    uint32_t *start;   // n_cells+1: first slot of each cell (sorted order); start[n_cells] = n_beads
    uint32_t *cnt;     // n_cells: bead counts of the next cell list (zero between steps)
    uint32_t *blocksums;
    // sorted state (A)
    void *posA, *velA, *frc;
    uint32_t *ids;       // bead id of each sorted slot
    uint32_t *cellg;     // global cell of each sorted slot
    uint32_t *slot_of_id;   // sorted slot of each polymer bead, by id (monomers: not kept)
    uint16_t *zlo;       // FP32: beads of each cell in its lower z half (offset z < 0.5), which
                         // the sort places first; not written for empty cells
    // advanced, not yet sorted state (B), indexed by the A slot it came from
    void *posB, *velB, *frcB;
    uint2 *keyrank;      // (new global cell, arrival rank in that cell)
    uint4 *tmp;          // (old slot, id, cell, 0) placed by provisional rank
    // bonds
    const uint32_t *bond_row;  // n_beads+1 CSR rows by global id
    const BondTerm *bond_terms;
    const void *bond_params;   // float4 / Vec4d: (kappa, r0 | cos theta0, sin theta0, 0)
    const void *pair;          // float2 / Vec2d: (a_ij, sqrt(gamma_ij))
    const void *cellpair;      // float2 / Vec2d per (cell, type pair) of spatial worlds
    const uint32_t *bonded_ids;  // ids of the beads that have bond terms (bond kernels)
    uint32_t n_bonded;
    float4 *fbond;               // FP32: bond force of each bonded bead, by sorted slot
    float4 *posf;                // FP64: (x - floor(x), hash) in FP32, by sorted slot: the
                                 // neighbour walk's distance prefilter
    void *bterm;                 // FP64: each bond term's force (Vec4d), by CSR row
    // id-ordered staging for upload / download: 9 doubles per bead (x, v, f), or, for the
    // read-backs with staging_fields set, field-major: the x of every bead (3 doubles each),
    // then every v, then every f (staging_n beads per field)
    double *staging;
    uint32_t staging_fields;
    uint32_t staging_n;
    int block_threads;
    int grid_blocks;     // persistent grid size for the tile kernels
    int list_capacity;   // neighbour-list capacity per bead (0 = the kernel's default)
    int force_kernel;    // FP32: 9 = half-shell brick kernel (Newton's third law inside a
                         // brick), 8 = full-shell brick kernel with 512-thread blocks, 6 = the
                         // same with 128-thread blocks, 1 = thread per bead (global memory)
    int brick_grid;      // persistent grid size of the brick kernel
    uint32_t brick_hc_max;  // halo cells of the nominal brick shape
    uint32_t brick_maxb;    // staged-bead capacity of one brick
    uint32_t brick_npair;   // staged pair-table entries: the largest n_types^2 of the worlds
    uint32_t brick_home_max;  // half shell: home-bead capacity of one brick
    uint32_t *brick_next;   // FP32: the brick queue's next free entry beyond the first
                            // gridDim.x (zeroed by the sort, which precedes every force pass)
};

// Kernel launchers.  Each returns the number of kernels it launched.
//   bin:    id-ordered staging (x, v, f) -> B with counts      (attach)
//   begin:  A rest state x(t), v(t), f(t) -> B with counts      (first update_pos of a run)
//   force:  A -> B: forces, update_mom and (unless final) the next update_pos with counts;
//           final: v(t+1) -> B.vel, f(t+1) -> frc
//   finish: B.vel -> A.vel and t += 1                           (after a final force pass)
//   unsort: A rest state -> id-ordered staging (pdpd_hostio.cu)   (download)
//   sort:   B -> A counting sort (pdpd_sort.cu)
int launch_bin32(const KArgs &a, const uint32_t *hash_in, cudaStream_t s);
int launch_begin32(const KArgs &a, cudaStream_t s);
int launch_force32(const KArgs &a, int final_step, cudaStream_t s);  // includes the bond kernel
int launch_finish32(const KArgs &a, cudaStream_t s);
int launch_bin64(const KArgs &a, const uint32_t *hash_in, cudaStream_t s);
int launch_begin64(const KArgs &a, cudaStream_t s);
int launch_force64(const KArgs &a, int final_step, cudaStream_t s);
int launch_finish64(const KArgs &a, cudaStream_t s);
int launch_sort(const KArgs &a, int fp64, int tick, int with_force, cudaStream_t s);

// One record of the pair log (pdpd_log_pair_terms; the C ABI's pdpd_pair_terms has this
// layout, with world-local ids): bead ids are global here.
struct PairLogRec {
    int64_t t;
    uint32_t home_id, other_id;
    uint32_t home_hash, other_hash;
    double dx[3], dr, inv_root_dt, gammap, rng, con, diss, rng_scale, rand, f[3];
};
// Pair log of the beads whose global ids are in sel (sorted, n_sel of them): with out null,
// counts[k] = in-range pairs of sel[k]; else the records of sel[k] from out + offs[k].
int launch_pair_log32(const KArgs &a, const uint32_t *sel, uint32_t n_sel, const uint32_t *offs,
                      uint32_t *counts, PairLogRec *out, cudaStream_t s);
int launch_pair_log64(const KArgs &a, const uint32_t *sel, uint32_t n_sel, const uint32_t *offs,
                      uint32_t *counts, PairLogRec *out, cudaStream_t s);

// Copies between device memory and the caller's host arrays done by a kernel (pdpd_hostio.cu),
// on devices that access pageable host memory coherently through the host's page tables
// (Grace-Blackwell: NVLink-C2C with address translation).  A segment is one contiguous run
// of 8-byte words (n words), of 4-byte words (n words), or n triples of doubles at byte
// strides src_stride / dst_stride (the beads of a strided bead array).  Chunks split the
// segments into pieces of at most HOSTCOPY_CHUNK units, the unit of work of a block.
enum HostCopyKind : uint32_t { HOSTCOPY_WORDS8 = 0, HOSTCOPY_WORDS4 = 1, HOSTCOPY_TRIPLES = 2 };
struct HostCopySeg {
    const void *src;
    void *dst;
    uint64_t n;
    uint32_t kind;
    uint32_t src_stride, dst_stride;
    uint32_t pad;
};
struct HostCopyChunk {
    uint32_t seg;
    uint32_t count;
    uint64_t first;
};
constexpr uint32_t HOSTCOPY_CHUNK = 16384;
int launch_host_copy(const HostCopySeg *segs, const HostCopyChunk *chunks, uint32_t n_chunks, int sm_count,
                     cudaStream_t s);
// The rest state of the tiles a.tiles[0, a.n_tiles) to id-ordered device staging (a.staging:
// rows of 9 doubles, or field-major with a.staging_fields), gathered through inv (the slot of
// each bead id of those tiles, launch_slot_of_id).
int launch_unsort(const KArgs &a, int fp64, const uint32_t *inv, cudaStream_t s);
// Direct read-back of the rest state into the callers' host arrays (pdpd_hostio.cu): where
// world w's x, v, f go (host pointers, null: not read; vectors `stride` bytes apart).
struct ReadDest {
    double *x, *v, *f;
    uint64_t stride;
};
// inv[ids[s]] = s for the sorted slots [first, first + count): the slot of each bead id.
int launch_slot_of_id(const KArgs &a, uint32_t first, uint32_t count, uint32_t *inv, cudaStream_t s);
// The work tiles of a.tiles[0, a.n_tiles) (each a run of bead ids of one world): each bead's
// state gathered through inv, x = cell + offset in FP32, and each field of the tile written
// to dest[world] as one contiguous run (or bead by bead at a stride).
int launch_read_direct(const KArgs &a, int fp64, const uint32_t *inv, const ReadDest *dest, cudaStream_t s);

// Exclusive prefix sum of cnt[0, n) into start[0, n), clearing cnt (pdpd_sort.cu); blocksums
// holds scan_blocks(n) words.
void launch_scan(uint32_t *cnt, uint32_t n, uint32_t *blocksums, uint32_t *start, cudaStream_t s);
// Attach (pdpd_bondcsr.cu): the per-bead bond CSR (row: n_beads + 1 offsets, terms) from the
// batch's flat lists with global ids -- pairs (head, tail) of the Hookean bonds, parameter k
// for bond k, and triples (head, middle, tail) of the angle bonds, parameter n_bonds + g for
// angle g -- and the polymer beads' ids in id order (bonded; their number to *n_bonded).
// Scratch: scratch and pos n_beads words each, blocksums scan_blocks(n_beads) words.
int launch_bond_tables(uint32_t n_beads, const uint32_t *pairs, uint32_t n_bonds, const uint32_t *triples,
                       uint32_t n_angles, const uint32_t *hash, uint32_t *row, BondTerm *terms, uint32_t *bonded,
                       uint32_t *n_bonded, uint32_t *scratch, uint32_t *pos, uint32_t *blocksums, cudaStream_t s);

// Device RNG on arrays (device pointers), for known-answer tests.
int launch_rng_eval(size_t n, const uint32_t *t, const uint64_t *seed, const uint32_t *a,
                    const uint32_t *b, uint32_t *h_out, float *u_out, cudaStream_t s);

size_t payload_bytes(int fp64);  // bytes of one pos / vel / frc element
// Largest staged-bead capacity of a brick for force variant `variant` (two blocks per SM of
// shared memory for variants 8 and 9, the list entries' range for 6).
uint32_t brick_maxb_limit(int variant, uint32_t hc_max, uint32_t npair, uint32_t home_max);
int brick_setup(int sm_count, int variant, uint32_t hc_max, uint32_t maxb, uint32_t npair, uint32_t home_max,
                int *grid, uint32_t *smem_bytes);  // 0 or a cudaError_t
uint32_t scan_blocks(uint32_t n_cells);

// Observables of one world (pdpd_observe.cu): per-block FP64 partial sums.
struct ObsPartial;
int launch_observe(const KArgs &a, int fp64, uint32_t world, uint32_t n_beads, uint32_t n_bins,
                   unsigned long long *rdf, uint32_t n_bond_bins, unsigned long long *bond_hist,
                   ObsPartial *part, cudaStream_t s);

// v2binary codec (pdpd_codec.cu): encode one world's bead records into a prepared section
// buffer at the given per-bead byte offsets, or decode them into the id-ordered staging rows.
// err (device) collects 1 = unrepresentable vector, 2 = position outside the box.
int launch_v2_encode(const KArgs &a, int fp64, uint32_t world, uint32_t n, uint8_t *buf,
                     const uint32_t *off, uint32_t *err, cudaStream_t s);
int launch_v2_decode(const KArgs &a, uint32_t world, uint32_t n, const uint8_t *buf,
                     const uint32_t *off, double *staging, uint32_t *err, cudaStream_t s);

// Message returned by pdpd_last_error(NULL) on this thread.
void set_thread_error(const char *msg);

}  // namespace pdpd
