// Host runtime of the GB300 DPD engine: implements the C ABI declared in include/pdpd_gpu.h.
//
// The engine owns one device arena holding every attached world (a batch of one for the
// plain DPDEngine path).  A timestep is a fixed sequence of kernels on the engine's stream:
//   force (finish step t, start step t+1) -> scan x2 -> place -> canon
// which is captured once per attach into a CUDA graph of G consecutive steps and replayed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <condition_variable>
#include <mutex>
#include <unistd.h>
#include <memory>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pdpd_gpu.h"
#include "pdpd_internal.h"

using namespace pdpd;

namespace {

thread_local std::string g_last_error = "";

}  // namespace

void pdpd::set_thread_error(const char *msg)
{
    g_last_error = msg ? msg : "";
}

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Host worker threads for parallel_for, started once per process and kept: a batch attach or
// read-back runs a few dozen parallel loops, and starting 16 threads for each cost more than
// some of the loops.  One loop at a time uses the pool (a loop that finds it busy, e.g. on a
// second engine's thread, starts its own threads as before); a process that forked after the
// pool was started builds a new one.
class HostPool {
public:
    static HostPool &get()
    {
        static std::mutex init;
        static HostPool *pool = nullptr;
        std::lock_guard<std::mutex> lk(init);
        if (!pool || pool->pid_ != getpid()) pool = new HostPool();  // (kept until exit)
        return *pool;
    }
    size_t threads() const { return workers_ + 1; }
    // Run task(k) for k in [0, n_tasks) on the pool and the calling thread; false if the pool
    // is busy with another loop.
    bool run(size_t n_tasks, const std::function<void(size_t)> &task)
    {
        std::unique_lock<std::mutex> use(use_, std::try_to_lock);
        if (!use.owns_lock()) return false;
        {
            std::lock_guard<std::mutex> lk(m_);
            task_ = &task;
            n_ = n_tasks;
            next_ = 0;
            done_ = 0;
            gen_++;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(m_);
        done_cv_.wait(lk, [&] { return done_ == n_; });
        task_ = nullptr;
        return true;
    }

private:
    HostPool() : pid_(getpid())
    {
        workers_ = std::min<size_t>(15, std::max(1u, std::thread::hardware_concurrency()) - 1);
        for (size_t k = 0; k < workers_; k++)
            std::thread([this] {
                uint64_t seen = 0;
                for (;;) {
                    {
                        std::unique_lock<std::mutex> lk(m_);
                        cv_.wait(lk, [&] { return gen_ != seen; });
                        seen = gen_;
                    }
                    work();
                }
            }).detach();
    }
    void work()
    {
        for (;;) {
            size_t k;
            const std::function<void(size_t)> *t;
            {
                std::lock_guard<std::mutex> lk(m_);
                if (!task_ || next_ >= n_) return;
                k = next_++;
                t = task_;
            }
            (*t)(k);
            std::lock_guard<std::mutex> lk(m_);
            if (++done_ == n_) done_cv_.notify_all();
        }
    }
    pid_t pid_;
    size_t workers_ = 0;
    std::mutex use_, m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t)> *task_ = nullptr;
    size_t n_ = 0, next_ = 0, done_ = 0;
    uint64_t gen_ = 0;
};

// fn(begin, end) over [0, n) on up to 16 host threads (chunks of at least min_chunk items):
// the per-bead host packing and unpacking of large worlds.
template <class F> void parallel_for(size_t n, size_t min_chunk, F fn)
{
    HostPool &pool = HostPool::get();
    size_t nt = std::min<size_t>(16, pool.threads());
    nt = std::min(nt, std::max<size_t>(1, n / std::max<size_t>(1, min_chunk)));
    if (nt <= 1) {
        fn((size_t)0, n);
        return;
    }
    const size_t per = (n + nt - 1) / nt;
    const std::function<void(size_t)> task = [&](size_t k) {
        const size_t b = std::min(n, k * per), e = std::min(n, b + per);
        if (b < e) fn(b, e);
    };
    if (pool.run(nt, task)) return;
    std::vector<std::thread> th;
    for (size_t k = 0; k < nt; k++) th.emplace_back([&task, k] { task(k); });
    for (auto &t : th) t.join();
}

// Device buffer that keeps its allocation while a request fits (bytes = capacity), so that a
// re-attach of a batch of similar size allocates nothing.  A buffer that has to grow takes
// half as much again as asked (a growing batch re-allocates a few times, not at every re-pack).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }  // scratch buffers local to a call are freed on return
    cudaError_t alloc(size_t n)
    {
        if (p && n <= bytes) return cudaSuccess;
        const bool grow = p != nullptr;
        release();
        if (n == 0) n = 16;
        if (grow) n += n / 2;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return (T *)p; }
};

struct HostPinned {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t alloc(size_t n, bool exact = false)
    {
        if (n <= bytes) return cudaSuccess;
        if (p && !exact) n += n / 2;  // pinning is slow: grow by half again
        release();
        cudaError_t e = cudaMallocHost(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

// v2binary section layout of one world: the section bytes with every polymer header and id
// delta written and the bead records left to the encoder, the byte offset of each bead's
// record, and the (offset, length) runs of structure bytes (for checking a stream to decode).
struct V2Layout {
    DevBuf d_buf, d_off;
    size_t bytes = 0;
    std::vector<uint8_t> tmpl;
    std::vector<std::pair<uint32_t, uint32_t>> structure;
    ~V2Layout()
    {
        d_buf.release();
        d_off.release();
    }
};

struct WorldHost {
    WorldDev dev;
    std::shared_ptr<V2Layout> v2;
};

struct ConfigEntry {
    const char *name;
    const char *desc;
};

const ConfigEntry kConfig[] = {
    {"list_capacity", "Neighbour-list entries per bead before a flush (0 = automatic)."},
    {"grid_blocks", "Persistent grid size of the tile kernels (0 = 16 blocks per SM)."},
    {"graph_steps", "Timesteps captured per CUDA graph replay (0 = automatic)."},
    {"use_graphs", "Replay captured CUDA graphs (1) or launch kernels directly (0)."},
    {"force_kernel", "FP32 force kernel (default by size: 8 from about 1,300 cells per SM, else 6): "
                     "1 = thread per bead from global memory, "
                     "6 = shared-memory brick, full shell, neighbour rows walked into lists, "
                     "128-thread blocks; 8 = as 6 with 512-thread blocks for larger bricks; "
                     "9 = shared-memory brick, half shell (each pair inside a brick evaluated "
                     "once, its reaction passed to the other bead), fixed-point force sums, "
                     "384-thread blocks.  1, 6 and 8 give the same forces to the bit; 9 gives the "
                     "same forces to the bit whatever its brick shape, grid or batch, within the "
                     "FP32 tolerance of the others."},
    {"brick_x", "Brick extent in cells along x (FP32 brick kernel; default by size: 5x8x8, "
                "3x4x6 from about 200 cells per SM, 2x4x4 below)."},
    {"brick_y", "Brick extent in cells along y (FP32 brick kernel)."},
    {"brick_z", "Brick extent in cells along z (FP32 brick kernel)."},
    {"autotune", "FP32: time the force-kernel variants and brick shapes on the first steps of "
                 "the next run and keep the fastest (results do not depend on the choice)."},
    {"host_direct", "Attach's upload and the read-backs by a kernel that reads and writes the "
                    "caller's host arrays directly (1, default; used where the device reaches "
                    "pageable host memory through the host's page tables, as Grace-Blackwell does "
                    "over NVLink-C2C, and the arrays are 8-byte aligned), or through pinned "
                    "staging buffers and DMA (0).  The results are the same."},
};

}  // namespace

struct pdpd_engine {
    int precision = PDPD_FP32;
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;
    std::string err;
    pdpd_timings timings{-1, -1, -1, -1, -1, -1};
    uint64_t launches = 0;

    // configuration
    int cfg_list_capacity = 0;
    int cfg_grid_blocks = 0;
    int cfg_graph_steps = 0;
    int cfg_use_graphs = 1;
    int cfg_force_kernel = 8;
    int cfg_brick[3] = {BRICK_X, BRICK_Y, BRICK_Z};
    int cfg_autotune = 0;
    int cfg_host_direct = 1;
    bool host_access = false;  // the device reaches pageable host memory through the host's page tables
    bool kernel_user = false;  // force_kernel set through the config
    bool brick_user = false;   // a brick_* entry set through the config
    bool tuning = false;       // the autotuner is trying candidates
    bool tuned = false;
    std::string tune_log;
    double max_density = 0;

    // attached worlds
    bool attached = false;
    std::vector<WorldHost> worlds;
    uint32_t n_beads = 0, n_cells = 0, n_tiles = 0;

    // device arena
    DevBuf d_worlds, d_tiles, d_bricks, d_start, d_cnt, d_blocksums;
    DevBuf d_posA, d_velA, d_frc, d_posB, d_velB, d_frcB;
    DevBuf d_ids, d_cellg, d_slot_of_id, d_keyrank, d_tmp;
    DevBuf d_bond_row, d_bond_terms, d_bond_params, d_pair, d_hash, d_bonded, d_fbond, d_cellpair, d_posf, d_bterm, d_zlo, d_brick_next, d_hash_old;
    DevBuf d_staging[2];
    HostPinned h_staging[2];
    HostPinned h_meta;  // attach: the flat bond lists and parameter rows, written here and uploaded from here
    HostPinned h_err;
    HostPinned h_small;  // attach: the number of polymer beads, from the device
    HostPinned h_plan;   // the tables of a direct host copy, uploaded from here (each call
                         // that copies directly waits for the copy before it returns)
    DevBuf d_v2err;
    DevBuf d_hostio;  // segment and chunk tables of the direct host copies, or the read-back's destinations
    DevBuf d_inv;     // direct read-back: the sorted slot of each bead id; attach: scratch
    DevBuf d_blist;   // attach: the flat bond lists with global ids
    DevBuf d_scan;    // attach: scan block sums, then the number of polymer beads
    cudaEvent_t ev_snap[2] = {nullptr, nullptr};
    cudaEvent_t ev_copied[2] = {nullptr, nullptr};

    // graphs
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    int graph_kernels = 0;

    KArgs args{};

    int fail(int code, const char *fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what)
    {
        return fail(PDPD_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }

    void drop_graph()
    {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        graph_steps = 0;
    }

    // Forget the attached batch but keep the device buffers for the next attach.
    void reset()
    {
        drop_graph();
        worlds.clear();
        attached = false;
        tuned = false;
        n_beads = n_cells = n_tiles = 0;
    }

    void release()
    {
        drop_graph();
        DevBuf *bufs[] = {&d_worlds, &d_tiles, &d_bricks, &d_start, &d_cnt, &d_blocksums, &d_posA, &d_velA,
                          &d_frc, &d_posB, &d_velB, &d_frcB, &d_ids, &d_cellg, &d_slot_of_id,
                          &d_keyrank, &d_tmp, &d_bond_row, &d_bond_terms, &d_bond_params,
                          &d_pair, &d_hash, &d_bonded, &d_fbond, &d_staging[0], &d_staging[1],
                          &d_v2err, &d_cellpair, &d_posf, &d_bterm, &d_zlo, &d_brick_next, &d_hash_old,
                          &d_hostio, &d_inv, &d_blist, &d_scan};
        for (DevBuf *b : bufs) b->release();
        worlds.clear();
        attached = false;
        tuned = false;
        n_beads = n_cells = n_tiles = 0;
    }

    bool fp64() const { return precision == PDPD_FP64; }
    bool any_spatial() const
    {
        for (const WorldHost &wh : worlds)
            if (wh.dev.spatial) return true;
        return false;
    }

    // ---- step sequences ------------------------------------------------------------------
    int enqueue_begin(cudaStream_t s)
    {
        int n = fp64() ? launch_begin64(args, s) : launch_begin32(args, s);
        n += launch_sort(args, fp64(), 0, 0, s);
        return n;
    }
    int enqueue_step(cudaStream_t s)  // finish step t and start t+1
    {
        int n = fp64() ? launch_force64(args, 0, s) : launch_force32(args, 0, s);
        n += launch_sort(args, fp64(), 1, 0, s);
        return n;
    }
    int enqueue_final(cudaStream_t s)
    {
        int n = fp64() ? launch_force64(args, 1, s) : launch_force32(args, 1, s);
        n += fp64() ? launch_finish64(args, s) : launch_finish32(args, s);
        return n;
    }

    int auto_graph_steps() const
    {
        if (cfg_graph_steps > 0) return std::min(cfg_graph_steps, 256);
        uint64_t target = 4u << 20;  // about 4M bead-steps per replay
        uint64_t g = n_beads ? target / n_beads : 64;
        return (int)std::max<uint64_t>(1, std::min<uint64_t>(64, g));
    }

    int build_graph()
    {
        drop_graph();
        int G = auto_graph_steps();
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
        int k = 0;
        for (int i = 0; i < G; i++) k += enqueue_step(stream);
        e = cudaStreamEndCapture(stream, &g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            graph = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate");
        }
        graph_steps = G;
        graph_kernels = k;
        return PDPD_OK;
    }

    // Enqueue n steps (n >= 1) on stream s.
    int enqueue_run(uint32_t n, cudaStream_t s)
    {
        if (n == 0) return PDPD_OK;
        launches += enqueue_begin(s);
        uint32_t mid = n - 1;
        if (cfg_use_graphs && mid > 0 && s == stream) {
            if (!graph) {
                int rc = build_graph();
                if (rc) return rc;
            }
            while (mid >= (uint32_t)graph_steps) {
                cudaError_t e = cudaGraphLaunch(graph, s);
                if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
                launches += graph_kernels;
                mid -= graph_steps;
            }
        }
        for (uint32_t i = 0; i < mid; i++) launches += enqueue_step(s);
        launches += enqueue_final(s);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        return PDPD_OK;
    }

    // Default kernel variant and brick shape for the attached batch, where the config does not
    // name them.  The persistent brick kernels want several bricks per SM: the 512-thread row
    // walk on 5x8x8 bricks is fastest from about 1,300 cells per SM (a 58^3 box on 152 SMs),
    // the 128-thread row walk on 3x4x6 bricks from about 200, and on 2x4x4 bricks below that.
    // All of them give the same trajectory.
    void default_shape()
    {
        uint64_t cells = 0;
        for (const WorldHost &wh : worlds)
            cells += (uint64_t)wh.dev.L[0] * (uint64_t)wh.dev.L[1] * (uint64_t)wh.dev.L[2];
        const uint64_t per_sm = cells / (uint64_t)std::max(1, sm_count);
        if (!kernel_user) cfg_force_kernel = per_sm >= 1300 ? 8 : 6;
        if (brick_user) return;
        static const int big[][3] = {{5, 8, 8}, {4, 8, 8}, {4, 6, 8}, {4, 4, 6}, {3, 4, 4}};
        static const int mid[3] = {3, 4, 6}, small[3] = {2, 4, 4};
        const int *b = per_sm >= 200 ? mid : small;
        if (cfg_force_kernel == 8 || cfg_force_kernel == 9 || per_sm >= 1300) {
            // the largest brick whose halo (at the batch's highest density) fits the staging
            // capacity 5 Poisson deviations above its mean, so dense boxes do not overflow it
            const int v = cfg_force_kernel == 9 ? 9 : 8;
            uint32_t npair = 1;
            for (const WorldHost &wh : worlds) npair = std::max(npair, wh.dev.n_types * wh.dev.n_types);
            b = big[4];
            for (const auto &c : big) {
                if (v == 9 && c[0] * c[1] * c[2] > 256) continue;  // the half shell's home sums
                const uint32_t hc = (uint32_t)(c[0] + 2) * (c[1] + 2) * (c[2] + 2);
                const double mean = max_density * hc;
                const uint32_t hm = home_want((uint32_t)(c[0] * c[1] * c[2]));
                if (mean + 5.0 * std::sqrt(mean) <= (double)brick_maxb_limit(v, hc, npair, hm)) {
                    b = c;
                    break;
                }
            }
        }
        for (int d = 0; d < 3; d++) cfg_brick[d] = b[d];
    }

    // Staged beads a brick of hc halo cells should have room for: the mean halo population
    // of the densest world + 6 standard deviations (Poisson), at least 1.2x the mean, + 32.
    double staging_want(uint32_t hc) const
    {
        const double mean = max_density * hc;
        return std::max(mean + 6.0 * std::sqrt(mean), 1.2 * mean) + 32;
    }

    // Home beads the half-shell kernel keeps force sums for, for bricks of `cells` home cells:
    // the mean of the densest world + 6 standard deviations + 32 (a fuller brick takes the
    // global-memory path, with the same result).
    uint32_t home_want(uint32_t cells) const
    {
        const double mean = max_density * cells;
        return (uint32_t)(mean + 6.0 * std::sqrt(mean) + 32);
    }

    // Build the brick work queue of the FP32 force kernel for the current brick shape: every
    // world cut into bx x by x bz bricks (edge bricks cut at the box faces), uploaded, and
    // the kernel's shared-memory budget and persistent grid set up.
    int configure_bricks()
    {
        KArgs &a = args;
        if (!tuning && !tuned) default_shape();
        // worlds with per-cell strengths run on the thread-per-bead kernel
        a.force_kernel = any_spatial() ? 1 : cfg_force_kernel;
        a.bricks = nullptr;
        a.n_bricks = 0;
        if (fp64() || a.force_kernel == 1) return PDPD_OK;
        // Each axis of a world is cut into ceil(L / b) bricks of as equal extents as possible
        // (e.g. a side of 9 with b = 4 into 3 + 3 + 3, not 4 + 4 + 1): no extent exceeds the
        // configured one, and no thin remainder brick stages a halo for a few home cells.
        std::vector<Brick> bricks;
        auto cuts = [](int L, int b) {
            std::vector<int> c;
            const int n = (L + b - 1) / b;
            for (int k = 0; k <= n; k++) c.push_back((int)((int64_t)L * k / n));
            return c;
        };
        for (uint32_t i = 0; i < worlds.size(); i++) {
            const int32_t *L = worlds[i].dev.L;
            const std::vector<int> cx = cuts(L[0], cfg_brick[0]), cy = cuts(L[1], cfg_brick[1]),
                                   cz = cuts(L[2], cfg_brick[2]);
            for (size_t a0 = 0; a0 + 1 < cx.size(); a0++)
                for (size_t a1 = 0; a1 + 1 < cy.size(); a1++)
                    for (size_t a2 = 0; a2 + 1 < cz.size(); a2++)
                        bricks.push_back({i, cx[a0], cy[a1], cz[a2], cx[a0 + 1] - cx[a0],
                                          cy[a1 + 1] - cy[a1], cz[a2 + 1] - cz[a2], 0});
        }
        size_t bytes_needed = sizeof(Brick) * std::max<size_t>(1, bricks.size());
        if (d_bricks.bytes < bytes_needed) {
            cudaStreamSynchronize(stream);
            cudaError_t ce = d_bricks.alloc(bytes_needed);
            if (ce != cudaSuccess) return fail(PDPD_E_NOMEM, "brick table allocation failed");
        }
        cudaError_t ce = cudaMemcpyAsync(d_bricks.p, bricks.data(), sizeof(Brick) * bricks.size(),
                                         cudaMemcpyHostToDevice, stream);
        if (ce != cudaSuccess) return cuda_fail(ce, "brick table upload");
        a.bricks = d_bricks.as<Brick>();
        a.n_bricks = (uint32_t)bricks.size();
        a.brick_hc_max = (uint32_t)(cfg_brick[0] + 2) * (cfg_brick[1] + 2) * (cfg_brick[2] + 2);
        a.brick_npair = 1;
        for (const WorldHost &wh : worlds) a.brick_npair = std::max(a.brick_npair, wh.dev.n_types * wh.dev.n_types);
        // staged-bead capacity (staging_want) within the variant's limit; a fuller brick takes
        // the (bit-identical) global path
        a.brick_home_max = a.force_kernel == 9 ? home_want((uint32_t)(cfg_brick[0] * cfg_brick[1] * cfg_brick[2])) : 0u;
        const double want = staging_want(a.brick_hc_max);
        const double limit = (double)brick_maxb_limit(a.force_kernel, a.brick_hc_max, a.brick_npair, a.brick_home_max);
        a.brick_maxb = (uint32_t)std::min(limit, std::max(64.0, want));
        int grid = 0;
        uint32_t bytes = 0;
        int rc = brick_setup(sm_count, a.force_kernel, a.brick_hc_max, a.brick_maxb, a.brick_npair,
                             a.brick_home_max, &grid, &bytes);
        if (rc)
            return fail(PDPD_E_CUDA, "brick kernel setup (%u bytes of shared memory): %s", bytes,
                        cudaGetErrorString((cudaError_t)rc));
        a.brick_grid = cfg_grid_blocks > 0 ? cfg_grid_blocks : grid;
        drop_graph();
        return PDPD_OK;
    }

    // Autotuner: pick the fastest FP32 force-kernel variant and brick shape for the attached
    // worlds by timing a few steps of each candidate on the engine's stream.  The candidates
    // add the same pair terms in the same order with the same roundings, so the trajectory
    // does not depend on which one runs: the trial steps are ordinary steps of the run.
    // Returns the number of steps consumed.
    uint32_t autotune(uint32_t n_steps)
    {
        // (variant 9 is left out: its forces are not bit-identical with these)
        static const int cand[][4] = {{8, 5, 8, 8}, {8, 4, 10, 8}, {8, 4, 8, 10}, {8, 4, 8, 8},
                                      {8, 6, 8, 6}, {6, 3, 4, 6}, {6, 4, 4, 6}, {1, 4, 4, 4}};
        const int n_cand = (int)(sizeof cand / sizeof cand[0]);
        const uint32_t timed = 3;  // steps timed per candidate, after one warm step
        const uint32_t warm = 8;   // steps of the untimed warm-up run
        // the warm-up run (warm + 1 timesteps), then per candidate begin .. final = timed + 2
        if (!cfg_autotune || tuned || fp64() || any_spatial() ||
            n_steps < warm + 1 + (timed + 2) * n_cand + 1)
            return 0;
        const int keep[4] = {cfg_force_kernel, cfg_brick[0], cfg_brick[1], cfg_brick[2]};
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 1e30f, keep_ms = 0.f;
        int best_i = -1;
        uint32_t used = 0;
        tune_log.clear();
        tuning = true;
        // warm-up with the first candidate, untimed: the first steps after an attach run slower
        // (first launches, clocks), which would bias whichever candidate came first
        cfg_force_kernel = cand[0][0];
        cfg_brick[0] = cand[0][1];
        cfg_brick[1] = cand[0][2];
        cfg_brick[2] = cand[0][3];
        if (configure_bricks() == PDPD_OK) {
            launches += enqueue_begin(stream);
            for (uint32_t k = 0; k < warm; k++) launches += enqueue_step(stream);
            launches += enqueue_final(stream);
            used += warm + 1;
        }
        for (int i = 0; i < n_cand; i++) {
            cfg_force_kernel = cand[i][0];
            cfg_brick[0] = cand[i][1];
            cfg_brick[1] = cand[i][2];
            cfg_brick[2] = cand[i][3];
            if (configure_bricks() != PDPD_OK) continue;
            // one warm step, then the timed steps (launched one by one, no graph)
            launches += enqueue_begin(stream);
            launches += enqueue_step(stream);
            cudaEventRecord(e0, stream);
            for (uint32_t k = 0; k < timed; k++) launches += enqueue_step(stream);
            cudaEventRecord(e1, stream);
            launches += enqueue_final(stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= (float)timed;
            used += timed + 2;  // begin .. final completes timed + 2 timesteps
            char line[96];
            snprintf(line, sizeof line, "%d:%dx%dx%d=%.3fms ", cand[i][0], cand[i][1], cand[i][2],
                     cand[i][3], ms);
            tune_log += line;
            if (ms < best) {
                best = ms;
                best_i = i;
            }
            if (cand[i][0] == keep[0] && cand[i][1] == keep[1] && cand[i][2] == keep[2] && cand[i][3] == keep[3])
                keep_ms = ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        // a few timed steps resolve about 1-2%: the configuration the run started with (the
        // size-aware default, chosen from long runs) stays unless a candidate beats it by 2%
        if (keep_ms > 0.f && best > 0.98f * keep_ms) best_i = -1;
        const int *pick = best_i >= 0 ? cand[best_i] : keep;
        cfg_force_kernel = pick[0];
        cfg_brick[0] = pick[1];
        cfg_brick[1] = pick[2];
        cfg_brick[2] = pick[3];
        tuned = true;
        tuning = false;
        configure_bricks();
        return used;
    }

    int check_device_errors()
    {
        int rc = fetch_device_errors();
        if (rc) return rc;
        cudaError_t e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_fail(e, "device error check");
        return eval_device_errors();
    }
    // The worlds' flags and t copied to h_err on the stream (for eval_device_errors once the
    // copy has completed).
    bool host_direct() const { return host_access && cfg_host_direct; }
    int fetch_device_errors()
    {
        size_t nb = sizeof(WorldDev) * worlds.size();
        if (h_err.alloc(nb) != cudaSuccess) return fail(PDPD_E_NOMEM, "pinned allocation failed");
        cudaError_t e = cudaMemcpyAsync(h_err.p, d_worlds.p, nb, cudaMemcpyDeviceToHost, stream);
        if (e != cudaSuccess) return cuda_fail(e, "device error check");
        return PDPD_OK;
    }
    int eval_device_errors()
    {
        const WorldDev *wd = (const WorldDev *)h_err.p;
        for (size_t i = 0; i < worlds.size(); i++) {
            worlds[i].dev.t = wd[i].t;
            uint32_t f = wd[i].err;
            if (!f) continue;
            if (f & ERR_BOND_SNAPPED)
                return fail(PDPD_E_BOND_SNAPPED,
                            "world %zu: an angle bond has snapped (Hookean bond longer than %.1f)", i,
                            pdpd_max_bond_length());
            if (f & ERR_NONFINITE)
                return fail(PDPD_E_BEAD_LOST, "world %zu: a bead position or velocity became non-finite", i);
            if (f & ERR_OUT_OF_BOX)
                return fail(PDPD_E_BEAD_LOST, "world %zu: a bead is outside the box or moved more than a box in one step", i);
        }
        return PDPD_OK;
    }
};

// ------------------------------------------------------------------------------------------
// validation

// fresh: the world's beads come from its descriptor (bead arrays required, every element
// checked); false for a world re-packed from the device, whose descriptor was checked when it
// was first attached.
static int check_world(const pdpd_world *w, char *reason, size_t n, bool fresh = true)
{
    auto say = [&](int code, const char *msg) {
        if (reason && n) snprintf(reason, n, "%s", msg);
        return code;
    };
    if (!w) return say(PDPD_E_INVALID, "No state");
    uint64_t cells = 1;
    for (int i = 0; i < 3; i++) {
        if (w->box[i] < 2) return say(PDPD_E_INVALID, "Distance in each direction must be at least 2");
        if (w->box[i] > 4096) return say(PDPD_E_UNSUPPORTED, "Box side larger than 4096 cells.");
        cells *= (uint64_t)w->box[i];
    }
    if (cells >= (1ull << 31)) return say(PDPD_E_UNSUPPORTED, "Box has more than 2^31 cells.");
    if (!(w->dt > 0 && w->dt < 1)) return say(PDPD_E_INVALID, "dt must be in (0, 1).");
    if (w->n_bead_types == 0 || w->n_bead_types > 16)
        return say(PDPD_E_UNSUPPORTED, "Engine supports 1..16 bead types (4-bit BeadHash type field).");
    if (!w->conservative || !w->dissipative)
        return say(PDPD_E_INVALID, "Missing interaction matrices.");
    for (uint32_t i = 0; i < w->n_bead_types * w->n_bead_types; i++)
        if (!(w->dissipative[i] >= 0) || !std::isfinite(w->conservative[i]))
            return say(PDPD_E_INVALID, "Interaction strengths must be finite and gamma >= 0.");
    if (!w->cell_conservative != !w->cell_dissipative)
        return say(PDPD_E_INVALID, "Per-cell strengths need both a_ij and gamma_ij tables.");
    if (w->cell_conservative) {
        const uint64_t nv = cells * (uint64_t)w->n_bead_types * w->n_bead_types;
        if (nv >= (1ull << 32)) return say(PDPD_E_UNSUPPORTED, "Per-cell strength tables larger than 2^32 entries.");
        for (uint64_t k = 0; fresh && k < nv; k++)
            if (!std::isfinite(w->cell_conservative[k]) || !(w->cell_dissipative[k] >= 0) ||
                !std::isfinite(w->cell_dissipative[k]))
                return say(PDPD_E_INVALID, "Per-cell interaction strengths must be finite and gamma >= 0.");
    }
    if (w->n_beads && (!w->hash || (fresh && (!w->x || !w->v || !w->f))))
        return say(PDPD_E_INVALID, "Missing bead arrays.");
    if (w->n_bonds && (!w->bond_beads || !w->bond_kappa || !w->bond_r0))
        return say(PDPD_E_INVALID, "Missing bond arrays.");
    if (w->n_angles && (!w->angle_beads || !w->angle_kappa || !w->angle_theta0))
        return say(PDPD_E_INVALID, "Missing angle-bond arrays.");
    if (!fresh) return PDPD_OK;
    bool bad_type = false;  // (a large world's beads checked in parallel chunks)
    parallel_for(w->n_beads, 1 << 18, [&](size_t i0, size_t i1) {
        bool bad = false;
        for (size_t i = i0; i < i1; i++) bad |= (w->hash[i] >> 28) >= w->n_bead_types;
        if (bad) __atomic_store_n(&bad_type, true, __ATOMIC_RELAXED);
    });
    if (bad_type) return say(PDPD_E_INVALID, "Bead hash has a bead type out of range.");
    for (uint32_t k = 0; k < 2 * w->n_bonds; k++)
        if (w->bond_beads[k] >= w->n_beads) return say(PDPD_E_INVALID, "Bond refers to a bead that does not exist.");
    for (uint32_t k = 0; k < 3 * w->n_angles; k++)
        if (w->angle_beads[k] >= w->n_beads) return say(PDPD_E_INVALID, "Angle bond refers to a bead that does not exist.");
    return PDPD_OK;
}

static const double *vec_at(const double *base, size_t stride_bytes, uint32_t i)
{
    size_t s = stride_bytes ? stride_bytes : 3 * sizeof(double);
    return (const double *)((const char *)base + s * (size_t)i);
}

// A plan of direct host copies (uploads: the host is the source): segments cut into chunks of
// at most HOSTCOPY_CHUNK units.  A run of words is cut at the 128-byte lines of its source,
// so that every warp of the copy kernel reads whole lines (a short first chunk up to the
// first line boundary): lines read in parts by two blocks cross the link more slowly.
struct HostCopyPlan {
    std::vector<HostCopySeg> segs;
    std::vector<HostCopyChunk> chunks;
    void add(uint32_t kind, const void *src, void *dst, uint64_t n, uint32_t src_stride = 0, uint32_t dst_stride = 0)
    {
        if (n == 0) return;
        const uint32_t si = (uint32_t)segs.size();
        segs.push_back({src, dst, n, kind, src_stride, dst_stride, 0});
        uint64_t k = 0;
        if (kind != HOSTCOPY_TRIPLES) {
            const uint64_t wb = kind == HOSTCOPY_WORDS8 ? 8 : 4;
            const uint64_t lead = ((128 - ((uintptr_t)src & 127)) & 127) / wb;  // words before a line boundary
            if (lead > 0 && lead < n) {
                chunks.push_back({si, (uint32_t)lead, 0});
                k = lead;
            }
        }
        for (; k < n; k += HOSTCOPY_CHUNK)
            chunks.push_back({si, (uint32_t)std::min<uint64_t>(HOSTCOPY_CHUNK, n - k), k});
    }
    // n beads' vectors (3 doubles each): a packed array (stride 24) as one run of words, a
    // strided one bead by bead; the device side is always packed.
    void vectors(const double *src, size_t src_stride, double *dst, size_t dst_stride, uint64_t n)
    {
        if (src_stride == 24 && dst_stride == 24) add(HOSTCOPY_WORDS8, src, dst, 3 * n);
        else add(HOSTCOPY_TRIPLES, src, dst, n, (uint32_t)src_stride, (uint32_t)dst_stride);
    }
};

// Touch, on the host, every page of the host side of a direct copy plan before the kernel runs
// (host_write: the destinations, else the sources): the device reaches host pages through the
// host's page tables, and a page the process has never touched is a fault the device waits
// for -- tens of microseconds a page, serialised (writing 1 GiB of fresh pages from the device
// took 0.37 s on a GB300 against 5.5 ms for pages already there) -- while the host's threads
// populate them in parallel.  One aligned word of the plan's own data per page: a destination
// word is written with its own value by an atomic OR with zero (the page becomes writable, the
// data stays), a source word is read.
static void touch_pages(const HostCopyPlan &plan, bool host_write)
{
    static const size_t P = []() {
        const long ps = sysconf(_SC_PAGESIZE);
        return ps > 0 ? (size_t)ps : (size_t)4096;
    }();
    struct Span {
        const HostCopySeg *sg;
        uintptr_t base, end;  // host bytes [base, end) the copy covers
        size_t page0, first;  // its first page, and its first work item in the flat page list
    };
    std::vector<Span> spans;
    size_t total = 0;
    for (const HostCopySeg &sg : plan.segs) {
        const uintptr_t base = (uintptr_t)(host_write ? sg.dst : sg.src);
        const uint32_t stride = host_write ? sg.dst_stride : sg.src_stride;
        const uintptr_t end = sg.kind == HOSTCOPY_TRIPLES ? base + (sg.n - 1) * stride + 24
                                                          : base + sg.n * (sg.kind == HOSTCOPY_WORDS4 ? 4 : 8);
        const size_t p0 = base / P, p1 = (end - 1) / P;
        spans.push_back({&sg, base, end, p0, total});
        total += p1 - p0 + 1;
    }
    parallel_for(total, 256, [&](size_t i0, size_t i1) {
        size_t si = (size_t)(std::upper_bound(spans.begin(), spans.end(), i0,
                                              [](size_t i, const Span &sp) { return i < sp.first; }) -
                             spans.begin()) - 1;
        for (size_t i = i0; i < i1; i++) {
            while (si + 1 < spans.size() && i >= spans[si + 1].first) si++;
            const Span &sp = spans[si];
            const uintptr_t ps = std::max<uintptr_t>(sp.base, (sp.page0 + (i - sp.first)) * P), pe = (ps / P + 1) * P;
            uintptr_t a = ps;  // the first word of the copy at or after the page's start
            if (sp.sg->kind == HOSTCOPY_TRIPLES) {
                const uint32_t stride = host_write ? sp.sg->dst_stride : sp.sg->src_stride;
                const uint64_t k = (ps - sp.base) / stride;
                const uintptr_t item = sp.base + k * stride;
                const uintptr_t j = (ps - item + 7) / 8;
                a = j <= 2 ? item + 8 * j : item + stride;
                if (j > 2 && k + 1 >= sp.sg->n) continue;
            }
            if (a >= pe || a >= sp.end) continue;  // no word of the copy on this page
            if (sp.sg->kind == HOSTCOPY_WORDS4) {
                if (host_write) __atomic_fetch_or((uint32_t *)a, 0u, __ATOMIC_RELAXED);
                else (void)*(volatile const uint32_t *)a;
            } else {
                if (host_write) __atomic_fetch_or((uint64_t *)a, (uint64_t)0, __ATOMIC_RELAXED);
                else (void)*(volatile const uint64_t *)a;
            }
        }
    });
}

// Host arrays the copy kernel may access: 8-byte aligned vectors at a stride that is a
// multiple of 8 (4-byte aligned hashes); anything else goes through the staged copies.
static bool vec_ok(const void *p, size_t stride)
{
    return p == nullptr || (((uintptr_t)p & 7u) == 0 && (stride & 7u) == 0 && stride >= 24 && stride < (1u << 20));
}

// Run a host copy plan (pdpd_hostio.cu) on the engine's stream: the host pages touched first
// (touch_pages; host_write: the host side is the destination), the plan's tables uploaded.
static int run_host_copy(pdpd_engine *e, const HostCopyPlan &plan, bool host_write)
{
    if (plan.chunks.empty()) return PDPD_OK;
    touch_pages(plan, host_write);
    const size_t sb = (sizeof(HostCopySeg) * plan.segs.size() + 15) & ~size_t(15);
    const size_t cb = sizeof(HostCopyChunk) * plan.chunks.size();
    if (e->d_hostio.alloc(sb + cb) != cudaSuccess) return e->fail(PDPD_E_NOMEM, "device allocation failed");
    // (through pinned memory: a copy from pageable memory would wait for the stream's earlier
    // work -- in a re-pack the previous epoch's steps -- and hold the host up with it)
    if (e->h_plan.alloc(sb + cb) != cudaSuccess) return e->fail(PDPD_E_NOMEM, "pinned allocation failed");
    memcpy(e->h_plan.p, plan.segs.data(), sizeof(HostCopySeg) * plan.segs.size());
    memcpy((char *)e->h_plan.p + sb, plan.chunks.data(), cb);
    cudaError_t ce = cudaMemcpyAsync(e->d_hostio.p, e->h_plan.p, sb + cb, cudaMemcpyHostToDevice, e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "host copy tables");
    e->launches += launch_host_copy((const HostCopySeg *)e->d_hostio.p,
                                    (const HostCopyChunk *)((const char *)e->d_hostio.p + sb),
                                    (uint32_t)plan.chunks.size(), e->sm_count, e->stream);
    ce = cudaGetLastError();
    return ce == cudaSuccess ? PDPD_OK : e->cuda_fail(ce, "host copy");
}

// ------------------------------------------------------------------------------------------
// C ABI

extern "C" {

int pdpd_create(int precision, int device, pdpd_engine **out)
{
    if (!out) return PDPD_E_INVALID;
    *out = nullptr;
    if (precision != PDPD_FP32 && precision != PDPD_FP64) {
        g_last_error = "precision must be PDPD_FP32 or PDPD_FP64";
        return PDPD_E_INVALID;
    }
    int dev = device;
    cudaError_t e = cudaSuccess;
    if (dev < 0) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaSetDevice(dev);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        g_last_error = std::string("no usable CUDA device: ") + cudaGetErrorString(e);
        return PDPD_E_CUDA;
    }
    pdpd_engine *eng = new pdpd_engine();
    eng->precision = precision;
    eng->device = dev;
    eng->sm_count = sms;
    {  // direct host copies need coherent access to pageable memory through the host's page tables
        int pageable = 0, host_tables = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            pageable = host_tables = 0;
        }
        eng->host_access = pageable == 1 && host_tables == 1;
    }
    e = cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&eng->side, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaEventCreateWithFlags(&eng->ev_snap[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&eng->ev_copied[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        g_last_error = std::string("stream creation failed: ") + cudaGetErrorString(e);
        pdpd_destroy(eng);
        return PDPD_E_CUDA;
    }
    *out = eng;
    return PDPD_OK;
}

void pdpd_destroy(pdpd_engine *e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->side) cudaStreamSynchronize(e->side);
    e->release();
    e->h_staging[0].release();
    e->h_staging[1].release();
    e->h_err.release();
    e->h_small.release();
    e->h_plan.release();
    e->h_meta.release();
    for (int i = 0; i < 2; i++) {
        if (e->ev_snap[i]) cudaEventDestroy(e->ev_snap[i]);
        if (e->ev_copied[i]) cudaEventDestroy(e->ev_copied[i]);
    }
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->side) cudaStreamDestroy(e->side);
    delete e;
}

const char *pdpd_last_error(const pdpd_engine *e)
{
    return e ? e->err.c_str() : g_last_error.c_str();
}

int pdpd_can_support(const pdpd_world *w, char *reason, size_t reason_len)
{
    if (reason && reason_len) reason[0] = 0;
    int rc = check_world(w, reason, reason_len);
    if (rc && reason) g_last_error = reason;
    return rc;
}

double pdpd_max_bond_length(void)
{
    return 2.0;
}

int pdpd_attach(pdpd_engine *e, const pdpd_world *w)
{
    if (!e) return PDPD_E_INVALID;
    if (!w) {
        cudaSetDevice(e->device);
        cudaStreamSynchronize(e->stream);
        e->release();
        return PDPD_OK;
    }
    return pdpd_attach_batch(e, w, 1);
}

static int download(pdpd_engine *e, int buf, cudaStream_t s, bool fields);

// Attach a batch.  keep_old (optional, one entry per world): index of a world of the
// currently attached batch whose bead state (x, v, f) the new world takes over on the device
// -- no host round trip -- or -1 for a world whose bead arrays come from its descriptor.
// The descriptors of kept worlds supply everything else (box, parameters, hashes, bonds, t).
static int attach_impl(pdpd_engine *e, const pdpd_world *ws, uint32_t n_worlds, const int32_t *keep_old)
{
    if (!e) return PDPD_E_INVALID;
    if (!ws || n_worlds == 0) return e->fail(PDPD_E_INVALID, "no worlds given");
    double t0 = now_s();
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    // Resident re-pack: unsort the current arena into device staging buffer 1 first; the new
    // batch is staged in buffer 0 and takes the kept worlds' rows from buffer 1.
    const double *snap = nullptr;
    std::vector<uint32_t> old_base;
    bool any_kept = false;
    for (uint32_t i = 0; keep_old && i < n_worlds; i++) any_kept |= keep_old[i] >= 0;
    if (any_kept) {
        if (!e->attached) return e->fail(PDPD_E_STATE, "re-pack without an attached batch");
        for (uint32_t i = 0; i < n_worlds; i++)
            if (keep_old[i] >= (int32_t)e->worlds.size())
                return e->fail(PDPD_E_INVALID, "re-pack refers to a world that is not attached");
        int rc = download(e, 1, e->stream, false);
        if (rc) return rc;
        snap = e->d_staging[1].as<double>();
        for (const WorldHost &wh : e->worlds) old_base.push_back(wh.dev.bead_base);
        // the kept worlds' hashes too stay on the device (the new layout reuses d_hash)
        if (e->d_hash_old.alloc(sizeof(uint32_t) * std::max<size_t>(1, e->n_beads)) != cudaSuccess)
            return e->fail(PDPD_E_NOMEM, "device allocation failed");
        cudaError_t hce = cudaMemcpyAsync(e->d_hash_old.p, e->d_hash.p, sizeof(uint32_t) * e->n_beads,
                                          cudaMemcpyDeviceToDevice, e->stream);
        if (hce != cudaSuccess) return e->cuda_fail(hce, "re-pack hash copy");
    }
    e->reset();
    char reason[256];
    // With direct host copies (a whole batch from its descriptors, in arrays the copy kernel
    // may access) the kernel brings the beads field-major into device staging 0 and the
    // hashes, launched now so that the transfer runs while the host builds the tables below.
    // In a re-pack the kept worlds' rows come from the old arena (below) and the kernel brings
    // only the new worlds', into rows of 9 doubles (x, v, f) like theirs.
    // (Launched before the worlds' checks, which scan every bead: it needs only the arrays'
    // presence and alignment and the bead counts, checked here; a batch that then fails a
    // check waits for the copy, which only reads, before the error returns.)
    uint64_t nb_direct = 0;
    for (uint32_t i = 0; i < n_worlds; i++) nb_direct += ws[i].n_beads;
    bool direct = e->host_direct() && nb_direct < (1ull << 31);
    for (uint32_t i = 0; direct && i < n_worlds; i++) {
        const pdpd_world &w = ws[i];
        if (any_kept && keep_old[i] >= 0) continue;
        const size_t sb = w.bead_stride_bytes ? w.bead_stride_bytes : 3 * sizeof(double);
        direct = (w.n_beads == 0 || (w.x && w.v && w.f && w.hash)) && vec_ok(w.x, sb) && vec_ok(w.v, sb) &&
                 vec_ok(w.f, sb) && ((uintptr_t)w.hash & 3u) == 0;
    }
    const bool field_major = direct && !any_kept;  // the layout of device staging 0 for the bin
    if (direct) {
        const uint64_t nb = nb_direct;
        if (e->d_staging[0].alloc(sizeof(double) * 9 * nb) != cudaSuccess ||
            e->d_hash.alloc(sizeof(uint32_t) * std::max<uint64_t>(1, nb)) != cudaSuccess) {
            cudaGetLastError();
            e->release();
            return e->fail(PDPD_E_NOMEM, "device allocation failed");
        }
        HostCopyPlan plan;
        double *ds = e->d_staging[0].as<double>();
        uint32_t *dh = e->d_hash.as<uint32_t>();
        size_t bb = 0;  // the world's first global bead (its bead_base)
        for (uint32_t i = 0; i < n_worlds; i++) {
            const pdpd_world &w = ws[i];
            const size_t sb = w.bead_stride_bytes ? w.bead_stride_bytes : 3 * sizeof(double);
            if (field_major) {
                plan.vectors(w.x, sb, ds + 3 * bb, 24, w.n_beads);
                plan.vectors(w.v, sb, ds + 3 * (nb + bb), 24, w.n_beads);
                plan.vectors(w.f, sb, ds + 3 * (2 * nb + bb), 24, w.n_beads);
                plan.add(HOSTCOPY_WORDS4, w.hash, dh + bb, w.n_beads);
            } else if (keep_old[i] < 0) {
                for (int q = 0; q < 3; q++)
                    plan.vectors(q == 0 ? w.x : (q == 1 ? w.v : w.f), sb, ds + 9 * bb + 3 * q, 72, w.n_beads);
                plan.add(HOSTCOPY_WORDS4, w.hash, dh + bb, w.n_beads);
            }
            bb += w.n_beads;
        }
        int rc = run_host_copy(e, plan, false);
        if (rc) {
            std::string m = e->err;
            e->release();
            e->err = m;
            return rc;
        }
    }

    uint64_t nb = 0, nc = 0, n_pair = 0, n_terms = 0, n_bparams = 0;
    {  // the worlds' checks (each scans its beads), in parallel; the first failure is reported
        std::vector<int> wrc(n_worlds, PDPD_OK);
        std::vector<std::string> why(n_worlds);
        parallel_for(n_worlds, 1, [&](size_t i0, size_t i1) {
            for (size_t i = i0; i < i1; i++) {
                char r[256];
                const bool kept = keep_old && keep_old[i] >= 0;
                wrc[i] = check_world(&ws[i], r, sizeof r, !kept);
                if (wrc[i]) why[i] = r;
            }
        });
        for (uint32_t i = 0; i < n_worlds; i++)
            if (wrc[i]) {
                cudaStreamSynchronize(e->stream);  // (the direct copy reads the caller's arrays)
                return e->fail(wrc[i], "world %u: %s", i, why[i].c_str());
            }
    }
    (void)reason;
    for (uint32_t i = 0; i < n_worlds; i++) {
        nb += ws[i].n_beads;
        nc += (uint64_t)ws[i].box[0] * ws[i].box[1] * ws[i].box[2];
        n_pair += (uint64_t)ws[i].n_bead_types * ws[i].n_bead_types;
        n_terms += 2ull * ws[i].n_bonds + 3ull * ws[i].n_angles;
        n_bparams += ws[i].n_bonds + ws[i].n_angles;
    }
    if (nb >= (1ull << 31) || nc >= (1ull << 31) || n_terms >= (1ull << 32)) {
        cudaStreamSynchronize(e->stream);
        return e->fail(PDPD_E_UNSUPPORTED, "batch too large (%llu beads, %llu cells, %llu bond terms)",
                       (unsigned long long)nb, (unsigned long long)nc, (unsigned long long)n_terms);
    }
    e->n_beads = (uint32_t)nb;
    e->n_cells = (uint32_t)nc;

    // --- world table, tiles, pair table
    std::vector<Tile> tiles;
    double max_density = 0;
    std::vector<WorldDev> wdev(n_worlds);
    const bool f64 = e->fp64();
    std::vector<double> pair64;
    std::vector<float> pair32;
    uint32_t cell_base = 0, bead_base = 0, param_base = 0;
    for (uint32_t i = 0; i < n_worlds; i++) {
        const pdpd_world &w = ws[i];
        WorldDev &d = wdev[i];
        memset(&d, 0, sizeof d);
        for (int k = 0; k < 3; k++) d.L[k] = w.box[k];
        d.n_cells = (uint32_t)w.box[0] * w.box[1] * w.box[2];
        d.cell_base = cell_base;
        d.bead_base = bead_base;
        d.n_beads = w.n_beads;
        d.n_types = w.n_bead_types;
        d.param_base = param_base;
        d.stationary = 0;
        for (uint32_t k = 0; w.stationary && k < w.n_bead_types; k++)
            if (w.stationary[k]) d.stationary |= 1u << k;
        d.spatial = w.cell_conservative ? 1u : 0u;
        d.cellpair_base = 0;
        d.dt = w.dt;
        d.scale_inv_sqrt_dt = std::sqrt(24 * 1.0 / w.dt);  // pow_half(24 kT / dt)
        d.seed = w.seed;
        d.t = w.t;
        for (uint32_t b = 0; b < w.n_beads; b += TILE_BEADS)
            tiles.push_back({i, bead_base + b, bead_base + std::min<uint32_t>(w.n_beads, b + TILE_BEADS), 0});
        max_density = std::max(max_density, (double)w.n_beads / (double)d.n_cells);
        for (uint32_t k = 0; k < w.n_bead_types * w.n_bead_types; k++) {
            double a = w.conservative[k], sg = std::sqrt(w.dissipative[k]);
            pair64.push_back(a);
            pair64.push_back(sg);
            pair32.push_back((float)a);
            pair32.push_back((float)sg);
        }
        cell_base += d.n_cells;
        bead_base += w.n_beads;
        param_base += w.n_bead_types * w.n_bead_types;
        WorldHost wh;
        wh.dev = d;
        e->worlds.push_back(wh);
    }
    e->n_tiles = (uint32_t)tiles.size();

    // --- per-cell strengths of spatial worlds: (a_ij, sqrt(gamma_ij)) per (cell, type pair)
    std::vector<double> cp64;
    std::vector<float> cp32;
    for (uint32_t i = 0; i < n_worlds; i++) {
        const pdpd_world &w = ws[i];
        if (!w.cell_conservative) continue;
        wdev[i].cellpair_base = f64 ? cp64.size() / 2 : cp32.size() / 2;
        e->worlds[i].dev.cellpair_base = wdev[i].cellpair_base;
        const uint64_t nv = (uint64_t)wdev[i].n_cells * w.n_bead_types * w.n_bead_types;
        for (uint64_t k = 0; k < nv; k++) {
            const double a = w.cell_conservative[k], sg = std::sqrt(w.cell_dissipative[k]);
            if (f64) {
                cp64.push_back(a);
                cp64.push_back(sg);
            } else {
                cp32.push_back((float)a);
                cp32.push_back((float)sg);
            }
        }
    }

    // --- bond tables.  The host writes the batch's flat bond lists with global ids and the
    // parameter rows into pinned memory, in one pass over all the batch's bond and angle terms
    // split across host threads whatever the worlds' sizes (one large world as fast as many
    // small ones); the per-bead CSR (Hookean terms first, then angle terms, each in flat-list
    // order) and the list of polymer beads are built from them on the device
    // (pdpd_bondcsr.cu).  Parameters: every world's Hookean bonds in order, then every world's
    // angle bonds.
    std::vector<uint32_t> bond_off(n_worlds + 1, 0), angle_off(n_worlds + 1, 0);
    for (uint32_t i = 0; i < n_worlds; i++) {
        bond_off[i + 1] = bond_off[i] + ws[i].n_bonds;
        angle_off[i + 1] = angle_off[i] + ws[i].n_angles;
    }
    const uint32_t n_bond_par = bond_off[n_worlds], n_angle_par = angle_off[n_worlds];
    // fn(world, k, g) for the global terms [g0, g1) of a per-world list with offsets off
    auto over_terms = [&](const std::vector<uint32_t> &off, size_t n, auto fn) {
        parallel_for(n, 1 << 14, [&](size_t g0, size_t g1) {
            uint32_t i = (uint32_t)(std::upper_bound(off.begin(), off.end(), (uint32_t)g0) - off.begin()) - 1;
            for (size_t g = g0; g < g1; g++) {
                while (g >= off[i + 1]) i++;
                fn(i, (uint32_t)(g - off[i]), (uint32_t)g);
            }
        });
    };
    const size_t list_bytes = (sizeof(uint32_t) * (2 * (size_t)n_bond_par + 3 * (size_t)n_angle_par) + 15) & ~size_t(15);
    const size_t par_bytes = (f64 ? sizeof(double) : sizeof(float)) * 4 * (size_t)n_bparams;
    if (e->h_meta.alloc(std::max<size_t>(16, list_bytes + par_bytes)) != cudaSuccess) {
        e->release();  // (waits for the direct copy, which reads the caller's arrays)
        return e->fail(PDPD_E_NOMEM, "pinned host allocation failed");
    }
    uint32_t *h_pairs = (uint32_t *)e->h_meta.p, *h_triples = h_pairs + 2 * (size_t)n_bond_par;
    void *h_par = (char *)e->h_meta.p + list_bytes;
    auto put = [&](uint32_t pidx, const double p[4]) {
        for (int q = 0; q < 4; q++) {
            if (f64) ((double *)h_par)[4 * (size_t)pidx + q] = p[q];
            else ((float *)h_par)[4 * (size_t)pidx + q] = (float)p[q];
        }
    };
    size_t bead_base_of = 0;
    std::vector<uint32_t> bb_of(n_worlds);
    for (uint32_t i = 0; i < n_worlds; i++) {
        bb_of[i] = (uint32_t)bead_base_of;
        bead_base_of += ws[i].n_beads;
    }
    over_terms(bond_off, n_bond_par, [&](uint32_t i, uint32_t k, uint32_t g) {
        const pdpd_world &w = ws[i];
        h_pairs[2 * (size_t)g] = bb_of[i] + w.bond_beads[2 * (size_t)k];
        h_pairs[2 * (size_t)g + 1] = bb_of[i] + w.bond_beads[2 * (size_t)k + 1];
        const double p[4] = {w.bond_kappa[k], w.bond_r0[k], 0, 0};
        put(g, p);
    });
    over_terms(angle_off, n_angle_par, [&](uint32_t i, uint32_t k, uint32_t g) {
        const pdpd_world &w = ws[i];
        for (int q = 0; q < 3; q++) h_triples[3 * (size_t)g + q] = bb_of[i] + w.angle_beads[3 * (size_t)k + q];
        const double th = w.angle_theta0[k];
        const double p[4] = {w.angle_kappa[k], std::cos(th), std::sin(th), 0};
        put(n_bond_par + g, p);
    });

    // --- allocate
    const size_t P = payload_bytes(f64);
    cudaError_t ce = cudaSuccess;
    auto A = [&](DevBuf &b, size_t n) {
        if (ce == cudaSuccess) ce = b.alloc(n);
    };
    A(e->d_worlds, sizeof(WorldDev) * n_worlds);
    A(e->d_tiles, sizeof(Tile) * std::max<size_t>(1, tiles.size()));
    A(e->d_start, sizeof(uint32_t) * ((size_t)nc + 1));
    A(e->d_cnt, sizeof(uint32_t) * (size_t)nc);
    A(e->d_zlo, f64 ? 16 : sizeof(uint16_t) * std::max<size_t>(1, (size_t)nc));
    A(e->d_brick_next, 16);
    A(e->d_blocksums, sizeof(uint32_t) * (scan_blocks((uint32_t)nc) + 1));
    A(e->d_posA, P * nb);
    A(e->d_velA, P * nb);
    A(e->d_frc, P * nb);
    A(e->d_posB, P * nb);
    A(e->d_velB, P * nb);
    A(e->d_frcB, P * nb);
    A(e->d_ids, sizeof(uint32_t) * nb);
    A(e->d_cellg, sizeof(uint32_t) * nb);
    A(e->d_slot_of_id, sizeof(uint32_t) * nb);
    A(e->d_keyrank, sizeof(uint2) * nb);
    A(e->d_tmp, sizeof(uint4) * nb);
    A(e->d_bond_row, sizeof(uint32_t) * (nb + 1));
    A(e->d_bond_terms, sizeof(BondTerm) * std::max<uint64_t>(1, n_terms));
    A(e->d_bond_params, (f64 ? sizeof(double) : sizeof(float)) * 4 * std::max<uint64_t>(1, n_bparams));
    A(e->d_pair, (f64 ? sizeof(double) : sizeof(float)) * 2 * n_pair);
    A(e->d_cellpair, std::max<size_t>(16, f64 ? sizeof(double) * cp64.size() : sizeof(float) * cp32.size()));
    A(e->d_hash, sizeof(uint32_t) * nb);
    A(e->d_bonded, sizeof(uint32_t) * std::max<uint64_t>(1, nb));
    A(e->d_blist, std::max<size_t>(16, list_bytes));
    A(e->d_inv, sizeof(uint32_t) * std::max<uint64_t>(1, nb));
    A(e->d_scan, sizeof(uint32_t) * (scan_blocks((uint32_t)nb) + 1));
    A(e->d_fbond, f64 ? 16 : sizeof(float4) * std::max<uint64_t>(1, nb));
    A(e->d_posf, f64 ? sizeof(float4) * std::max<uint64_t>(1, nb) : 16);
    A(e->d_bterm, f64 ? sizeof(double) * 4 * std::max<uint64_t>(1, n_terms) : 16);
    A(e->d_staging[0], sizeof(double) * 9 * nb);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        e->release();
        return e->fail(PDPD_E_NOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    // Host staging rows of the worlds that come from their descriptors: the whole batch in
    // slot order, or in a re-pack only the new worlds, packed (the kept worlds' rows stay on
    // the device, and the pinned buffer stays the size of what a re-pack brings in).
    std::vector<size_t> hoff(n_worlds);
    size_t h_rows = 0;
    for (uint32_t i = 0; i < n_worlds; i++) {
        hoff[i] = any_kept ? h_rows : (size_t)wdev[i].bead_base;
        if (!any_kept || keep_old[i] < 0) h_rows += ws[i].n_beads;
    }
    if (!any_kept) h_rows = nb;
    if (direct) h_rows = 0;
    if (!direct && e->h_staging[0].alloc(sizeof(double) * 9 * h_rows + sizeof(uint32_t) * h_rows) != cudaSuccess) {
        e->release();
        return e->fail(PDPD_E_NOMEM, "pinned host allocation failed");
    }

    // --- stage and upload
    double *hs = direct ? nullptr : (double *)e->h_staging[0].p;
    uint32_t *hh = direct ? nullptr : (uint32_t *)(hs + 9 * h_rows);
    // Global slots [r0, r1) of the batch (slot g of world i = bead_base_i + k) into the pinned
    // rows, split across host threads whatever the worlds' sizes.
    auto stage = [&](size_t r0, size_t r1) {
        parallel_for(r1 - r0, 1 << 16, [&](size_t a0, size_t a1) {
            const size_t g0 = r0 + a0, g1 = r0 + a1;
            uint32_t i = (uint32_t)(std::upper_bound(wdev.begin(), wdev.end(), (uint32_t)g0,
                                                     [](uint32_t g, const WorldDev &d) { return g < d.bead_base; }) -
                                    wdev.begin()) - 1;
            for (size_t g = g0; g < g1;) {
                while (g >= (size_t)wdev[i].bead_base + ws[i].n_beads) i++;
                const pdpd_world &w = ws[i];
                const size_t bb = wdev[i].bead_base, k1 = std::min<size_t>(g1 - bb, w.n_beads);
                const bool kept = keep_old && keep_old[i] >= 0;  // state and hashes from the old arena (below)
                const size_t ho = hoff[i];
                for (size_t k = g - bb; k < k1 && !kept; k++) {
                    const double *x = vec_at(w.x, w.bead_stride_bytes, (uint32_t)k);
                    const double *v = vec_at(w.v, w.bead_stride_bytes, (uint32_t)k);
                    const double *f = vec_at(w.f, w.bead_stride_bytes, (uint32_t)k);
                    double *o = hs + 9 * (ho + k);
                    for (int d = 0; d < 3; d++) {
                        o[d] = x[d];
                        o[3 + d] = v[d];
                        o[6 + d] = f[d];
                    }
                    hh[ho + k] = w.hash[k];
                }
                g = bb + k1;
            }
        });
    };
    cudaStream_t s = e->stream;
    if (direct) {
        // (uploaded by the copy kernel launched above)
    } else if (!any_kept) {
        // a whole batch from its descriptors: chunks of 2^20 beads, each uploaded while the
        // next is staged
        const size_t CH = size_t(1) << 20;
        for (size_t r0 = 0; r0 < nb; r0 += CH) {
            const size_t r1 = std::min<size_t>(nb, r0 + CH);
            stage(r0, r1);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(e->d_staging[0].as<double>() + 9 * r0, hs + 9 * r0, sizeof(double) * 9 * (r1 - r0),
                                     cudaMemcpyHostToDevice, s);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(e->d_hash.as<uint32_t>() + r0, hh + r0, sizeof(uint32_t) * (r1 - r0),
                                     cudaMemcpyHostToDevice, s);
        }
    } else {
        stage(0, nb);
    }
    auto H2D = [&](DevBuf &b, const void *src, size_t n) {
        if (ce == cudaSuccess && n) ce = cudaMemcpyAsync(b.p, src, n, cudaMemcpyHostToDevice, s);
    };
    H2D(e->d_worlds, wdev.data(), sizeof(WorldDev) * n_worlds);
    H2D(e->d_tiles, tiles.data(), sizeof(Tile) * tiles.size());
    H2D(e->d_blist, h_pairs, sizeof(uint32_t) * (2 * (size_t)n_bond_par + 3 * (size_t)n_angle_par));
    H2D(e->d_bond_params, h_par, par_bytes);
    if (f64) {
        H2D(e->d_pair, pair64.data(), sizeof(double) * pair64.size());
        H2D(e->d_cellpair, cp64.data(), sizeof(double) * cp64.size());
    } else {
        H2D(e->d_pair, pair32.data(), sizeof(float) * pair32.size());
        H2D(e->d_cellpair, cp32.data(), sizeof(float) * cp32.size());
    }
    if (any_kept && !direct) {  // only the rows of the worlds that come from their descriptors
        for (uint32_t i = 0; i < n_worlds; i++)
            if (keep_old[i] < 0 && ws[i].n_beads && ce == cudaSuccess)
                ce = cudaMemcpyAsync(e->d_staging[0].as<double>() + 9 * (size_t)wdev[i].bead_base,
                                     hs + 9 * hoff[i], sizeof(double) * 9 * ws[i].n_beads,
                                     cudaMemcpyHostToDevice, s);
    }
    for (uint32_t i = 0; any_kept && i < n_worlds; i++) {
        if (keep_old[i] < 0 || ws[i].n_beads == 0 || ce != cudaSuccess) continue;
        ce = cudaMemcpyAsync(e->d_staging[0].as<double>() + 9 * (size_t)wdev[i].bead_base,
                             snap + 9 * (size_t)old_base[keep_old[i]],
                             sizeof(double) * 9 * ws[i].n_beads, cudaMemcpyDeviceToDevice, s);
    }
    if (any_kept) {
        for (uint32_t i = 0; i < n_worlds && ce == cudaSuccess; i++) {
            if (ws[i].n_beads == 0) continue;
            uint32_t *dst = e->d_hash.as<uint32_t>() + wdev[i].bead_base;
            const size_t n = sizeof(uint32_t) * ws[i].n_beads;
            if (keep_old[i] < 0 && direct) continue;  // (the copy kernel's)
            ce = keep_old[i] < 0
                     ? cudaMemcpyAsync(dst, hh + hoff[i], n, cudaMemcpyHostToDevice, s)
                     : cudaMemcpyAsync(dst, e->d_hash_old.as<uint32_t>() + old_base[keep_old[i]], n,
                                       cudaMemcpyDeviceToDevice, s);
        }
    }
    if (ce == cudaSuccess) {  // (after every write of d_hash)
        const uint32_t *d_pairs = e->d_blist.as<uint32_t>();
        e->launches += launch_bond_tables((uint32_t)nb, d_pairs, n_bond_par, d_pairs + 2 * (size_t)n_bond_par,
                                          n_angle_par, e->d_hash.as<uint32_t>(), e->d_bond_row.as<uint32_t>(),
                                          e->d_bond_terms.as<BondTerm>(), e->d_bonded.as<uint32_t>(),
                                          e->d_scan.as<uint32_t>() + scan_blocks((uint32_t)nb),
                                          e->d_inv.as<uint32_t>(), e->d_slot_of_id.as<uint32_t>(),
                                          e->d_scan.as<uint32_t>(), s);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess && e->h_small.alloc(16) != cudaSuccess) ce = cudaErrorMemoryAllocation;
    if (ce == cudaSuccess)  // the number of polymer beads, read at the end of the attach
        ce = cudaMemcpyAsync(e->h_small.p, e->d_scan.as<uint32_t>() + scan_blocks((uint32_t)nb), sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(e->d_cnt.p, 0, sizeof(uint32_t) * nc, s);
    uint32_t total = (uint32_t)nb;  // start[n_cells] = total beads, fixed for the attach
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(e->d_start.as<uint32_t>() + nc, &total, sizeof(uint32_t),
                             cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) {
        e->release();
        return e->cuda_fail(ce, "upload");
    }

    // --- kernel arguments
    KArgs &a = e->args;
    memset(&a, 0, sizeof a);
    a.worlds = e->d_worlds.as<WorldDev>();
    a.n_worlds = n_worlds;
    a.tiles = e->d_tiles.as<Tile>();
    a.n_tiles = e->n_tiles;
    a.n_beads = e->n_beads;
    a.n_cells = e->n_cells;
    a.start = e->d_start.as<uint32_t>();
    a.cnt = e->d_cnt.as<uint32_t>();
    a.blocksums = e->d_blocksums.as<uint32_t>();
    a.posA = e->d_posA.p;
    a.velA = e->d_velA.p;
    a.frc = e->d_frc.p;
    a.posB = e->d_posB.p;
    a.velB = e->d_velB.p;
    a.frcB = e->d_frcB.p;
    a.ids = e->d_ids.as<uint32_t>();
    a.cellg = e->d_cellg.as<uint32_t>();
    a.slot_of_id = e->d_slot_of_id.as<uint32_t>();
    a.keyrank = e->d_keyrank.as<uint2>();
    a.tmp = e->d_tmp.as<uint4>();
    a.bond_row = e->d_bond_row.as<uint32_t>();
    a.bond_terms = e->d_bond_terms.as<BondTerm>();
    a.bond_params = e->d_bond_params.p;
    a.pair = e->d_pair.p;
    a.cellpair = e->d_cellpair.p;
    a.bonded_ids = e->d_bonded.as<uint32_t>();
    a.n_bonded = 0;  // (known once the attach's kernels have run, below)
    a.fbond = e->d_fbond.as<float4>();
    a.posf = f64 ? e->d_posf.as<float4>() : nullptr;
    a.zlo = f64 ? nullptr : e->d_zlo.as<uint16_t>();
    a.brick_next = f64 ? nullptr : e->d_brick_next.as<uint32_t>();
    a.bterm = f64 ? e->d_bterm.p : nullptr;
    a.staging = e->d_staging[0].as<double>();
    a.block_threads = 128;
    int gb = e->cfg_grid_blocks > 0 ? e->cfg_grid_blocks : 16 * e->sm_count;
    a.list_capacity = e->cfg_list_capacity;
    e->max_density = max_density;
    {
        int rc = e->configure_bricks();
        if (rc) {
            std::string m = e->err;
            e->release();
            e->err = m;
            return rc;
        }
    }
    a.grid_blocks = (int)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)gb, e->n_tiles));

    // --- bin + sort into the rest state
    const uint32_t *hash_in = e->d_hash.as<uint32_t>();
    {
        KArgs ab = a;  // the direct copies of a whole batch left the staging field-major
        ab.staging_fields = field_major ? 1u : 0u;
        ab.staging_n = (uint32_t)nb;
        e->launches += f64 ? launch_bin64(ab, hash_in, s) : launch_bin32(ab, hash_in, s);
    }
    e->launches += launch_sort(a, f64, 0, 1, s);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        e->release();
        return e->cuda_fail(ce, "attach kernels");
    }
    e->attached = true;
    int rc = e->check_device_errors();
    a.n_bonded = *(const uint32_t *)e->h_small.p;
    if (rc) {
        std::string m = e->err;
        e->release();
        e->err = m;
        return rc;
    }
    e->timings = pdpd_timings{-1, -1, now_s() - t0, -1, -1, -1};
    return PDPD_OK;
}

int pdpd_attach_batch(pdpd_engine *e, const pdpd_world *ws, uint32_t n_worlds)
{
    return attach_impl(e, ws, n_worlds, nullptr);
}

int pdpd_run_async(pdpd_engine *e, uint32_t n_steps)
{
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "Run called with no world attached");
    cudaSetDevice(e->device);
    n_steps -= e->autotune(n_steps);
    return e->enqueue_run(n_steps, e->stream);
}

int pdpd_sync(pdpd_engine *e)
{
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    cudaSetDevice(e->device);
    cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "cudaStreamSynchronize");
    return e->check_device_errors();
}

int pdpd_run(pdpd_engine *e, uint32_t n_steps)
{
    if (!e) return PDPD_E_INVALID;
    double t0 = now_s();
    int rc = pdpd_run_async(e, n_steps);
    if (rc) return rc;
    rc = pdpd_sync(e);
    double dt = now_s() - t0;
    auto acc = [](double &slot, double v) { slot = slot < 0 ? v : slot + v; };
    acc(e->timings.execute_to_first_bead, dt);
    acc(e->timings.execute_to_last_bead, dt);
    return rc;
}

void *pdpd_stream(pdpd_engine *e)
{
    return e ? (void *)e->stream : nullptr;
}

// fields: write the staging buffer field-major (the x of every bead, then every v, then
// every f) instead of in rows of 9 doubles.
static int download(pdpd_engine *e, int buf, cudaStream_t s, bool fields = false)
{
    KArgs a = e->args;
    if (e->d_staging[buf].alloc(sizeof(double) * 9 * (size_t)e->n_beads) != cudaSuccess ||
        e->d_inv.alloc(sizeof(uint32_t) * std::max<uint32_t>(1, e->n_beads)) != cudaSuccess)
        return e->fail(PDPD_E_NOMEM, "staging allocation failed");
    a.staging = e->d_staging[buf].as<double>();
    a.staging_fields = fields ? 1u : 0u;
    a.staging_n = e->n_beads;
    e->launches += launch_slot_of_id(a, 0, e->n_beads, e->d_inv.as<uint32_t>(), s);
    e->launches += launch_unsort(a, e->fp64(), e->d_inv.as<uint32_t>(), s);
    return PDPD_OK;
}

// Unsort one world only (its own work tiles) into device staging buffer `buf`: the rows
// of its beads, so reading every world of a batch in turn costs one pass over the arena.
static int download_world(pdpd_engine *e, int buf, uint32_t world, cudaStream_t s, bool fields = false)
{
    KArgs a = e->args;
    a.staging_fields = fields ? 1u : 0u;
    a.staging_n = e->n_beads;
    if (e->d_staging[buf].alloc(sizeof(double) * 9 * (size_t)e->n_beads) != cudaSuccess)
        return e->fail(PDPD_E_NOMEM, "staging allocation failed");
    uint32_t first = 0;
    for (uint32_t k = 0; k < world; k++) first += (e->worlds[k].dev.n_beads + TILE_BEADS - 1) / TILE_BEADS;
    a.tiles = e->args.tiles + first;
    a.n_tiles = (e->worlds[world].dev.n_beads + TILE_BEADS - 1) / TILE_BEADS;
    if (a.n_tiles == 0) return PDPD_OK;
    a.grid_blocks = (int)std::min<uint32_t>((uint32_t)std::max(1, e->args.grid_blocks), a.n_tiles);
    a.staging = e->d_staging[buf].as<double>();
    const WorldDev &wd = e->worlds[world].dev;
    if (e->d_inv.alloc(sizeof(uint32_t) * std::max<uint32_t>(1, e->n_beads)) != cudaSuccess)
        return e->fail(PDPD_E_NOMEM, "staging allocation failed");
    e->launches += launch_slot_of_id(a, wd.bead_base, wd.n_beads, e->d_inv.as<uint32_t>(), s);
    e->launches += launch_unsort(a, e->fp64(), e->d_inv.as<uint32_t>(), s);
    return PDPD_OK;
}

static void scatter(const double *src, uint32_t n, double *x, double *v, double *f, size_t stride)
{
    size_t sb = stride ? stride : 3 * sizeof(double);
    parallel_for(n, 1 << 16, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; i++) {
            const double *r = src + 9 * i;
            if (x) memcpy((char *)x + sb * i, r, 3 * sizeof(double));
            if (v) memcpy((char *)v + sb * i, r + 3, 3 * sizeof(double));
            if (f) memcpy((char *)f + sb * i, r + 6, 3 * sizeof(double));
        }
    });
}

// Beads [r_begin, r_end) of device staging buffer 0, written field-major by the unsort
// kernels already on the stream (download(..., true)), to pinned host staging (field-major
// too: n x's, n v's, n f's, n = r_end - r_begin) and on to the caller: the worlds' error
// flags are fetched first, then the beads go in chunks, each handed to scatter(host, n, r0,
// r1) as soon as its x, v and f have arrived, so the host copies of one chunk overlap the
// transfer of the next.
static int read_rows(pdpd_engine *e, size_t r_begin, size_t r_end,
                     const std::function<void(const double *, size_t, size_t, size_t)> &scatter)
{
    const size_t n = r_end - r_begin, nd = e->n_beads;
    if (e->h_staging[0].alloc(sizeof(double) * 9 * std::max<size_t>(1, n)) != cudaSuccess)
        return e->fail(PDPD_E_NOMEM, "pinned allocation failed");
    int rc = e->fetch_device_errors();
    if (rc) return rc;
    cudaEvent_t ev_err;
    cudaEventCreateWithFlags(&ev_err, cudaEventDisableTiming);
    cudaEventRecord(ev_err, e->stream);
    const size_t CH = size_t(1) << 20;
    const size_t nch = (n + CH - 1) / CH;
    std::vector<cudaEvent_t> ev(nch);
    double *dst = (double *)e->h_staging[0].p;
    const double *src = e->d_staging[0].as<double>();
    cudaError_t ce = cudaSuccess;
    for (size_t k = 0; k < nch; k++) {
        const size_t r0 = k * CH, r1 = std::min(n, r0 + CH);
        cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
        for (int q = 0; q < 3 && ce == cudaSuccess; q++)  // x, v, f of the chunk's beads
            ce = cudaMemcpyAsync(dst + 3 * (q * n + r0), src + 3 * (q * nd + r_begin + r0),
                                 sizeof(double) * 3 * (r1 - r0), cudaMemcpyDeviceToHost, e->stream);
        cudaEventRecord(ev[k], e->stream);
    }
    if (ce == cudaSuccess) ce = cudaEventSynchronize(ev_err);
    rc = ce != cudaSuccess ? e->cuda_fail(ce, "download") : e->eval_device_errors();
    for (size_t k = 0; k < nch; k++) {
        if (rc == PDPD_OK) {
            ce = cudaEventSynchronize(ev[k]);
            if (ce != cudaSuccess) rc = e->cuda_fail(ce, "download");
        }
        if (rc == PDPD_OK) scatter(dst, n, k * CH, std::min(n, (k + 1) * CH));
    }
    if (rc != PDPD_OK) cudaStreamSynchronize(e->stream);
    for (cudaEvent_t x : ev) cudaEventDestroy(x);
    cudaEventDestroy(ev_err);
    return rc;
}

// The read-back without device staging (k_read_direct), for worlds [w0, w1) of the batch:
// the worlds' error flags first (the callers' arrays are not written when a world has
// failed), the callers' pages touched, then the slot of each bead id and one gather kernel
// writing dest[w] (one entry per attached world).
static int read_direct(pdpd_engine *e, uint32_t w0, uint32_t w1, const std::vector<ReadDest> &dest)
{
    int rc = e->fetch_device_errors();
    if (rc) return rc;
    cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "download");
    rc = e->eval_device_errors();
    if (rc) return rc;
    HostCopyPlan pages;  // (the destinations, for touch_pages only)
    uint32_t first_tile = 0, n_tiles = 0;
    for (uint32_t i = 0; i < w1; i++) {
        const uint32_t nb = e->worlds[i].dev.n_beads, nt = (nb + TILE_BEADS - 1) / TILE_BEADS;
        if (i < w0) {
            first_tile += nt;
            continue;
        }
        n_tiles += nt;
        for (double *o : {dest[i].x, dest[i].v, dest[i].f})
            if (o) pages.vectors(nullptr, 24, o, dest[i].stride, nb);
    }
    touch_pages(pages, true);
    const size_t db = sizeof(ReadDest) * dest.size();
    if (e->d_hostio.alloc(db) != cudaSuccess || e->d_inv.alloc(sizeof(uint32_t) * std::max<uint32_t>(1, e->n_beads)) != cudaSuccess)
        return e->fail(PDPD_E_NOMEM, "device allocation failed");
    ce = cudaMemcpyAsync(e->d_hostio.p, dest.data(), db, cudaMemcpyHostToDevice, e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "download");
    const uint32_t s0 = e->worlds[w0].dev.bead_base;
    const uint32_t s1 = w1 < e->worlds.size() ? e->worlds[w1].dev.bead_base : e->n_beads;
    KArgs a = e->args;
    a.tiles = e->args.tiles + first_tile;
    a.n_tiles = n_tiles;
    e->launches += launch_slot_of_id(a, s0, s1 - s0, e->d_inv.as<uint32_t>(), e->stream);
    e->launches += launch_read_direct(a, e->fp64(), e->d_inv.as<uint32_t>(), (const ReadDest *)e->d_hostio.p,
                                      e->stream);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    return ce == cudaSuccess ? PDPD_OK : e->cuda_fail(ce, "download");
}

// Beads [k0, k1) of one world from field-major host staging (x block at hx, v at hv, f at
// hf, indexed by the world's bead index) into the caller's vectors of byte stride sb (24:
// packed, copied as one block per vector).
static void copy_out(const double *hx, const double *hv, const double *hf, size_t k0, size_t k1, double *x,
                     double *v, double *f, size_t sb)
{
    const double *src[3] = {hx, hv, hf};
    double *out[3] = {x, v, f};
    for (int q = 0; q < 3; q++) {
        if (!out[q]) continue;
        if (sb == 3 * sizeof(double)) {
            memcpy(out[q] + 3 * k0, src[q] + 3 * k0, sizeof(double) * 3 * (k1 - k0));
        } else {
            for (size_t k = k0; k < k1; k++) memcpy((char *)out[q] + sb * k, src[q] + 3 * k, 3 * sizeof(double));
        }
    }
}

int pdpd_read_state(pdpd_engine *e, uint32_t world, double *x, double *v, double *f,
                    size_t stride, int64_t *t)
{
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (world >= e->worlds.size()) return e->fail(PDPD_E_INVALID, "world index out of range");
    cudaSetDevice(e->device);
    const WorldDev &wd = e->worlds[world].dev;
    const size_t sb = stride ? stride : 3 * sizeof(double);
    if (e->host_direct() && vec_ok(x, sb) && vec_ok(v, sb) && vec_ok(f, sb)) {
        std::vector<ReadDest> dest(e->worlds.size(), ReadDest{nullptr, nullptr, nullptr, 24});
        dest[world] = ReadDest{x, v, f, sb};
        int rc = read_direct(e, world, world + 1, dest);
        if (rc) return rc;
        if (t) *t = e->worlds[world].dev.t;
        return PDPD_OK;
    }
    int rc = download_world(e, 0, world, e->stream, true);
    if (rc) return rc;
    rc = read_rows(e, wd.bead_base, (size_t)wd.bead_base + wd.n_beads,
                   [&](const double *h, size_t n, size_t r0, size_t r1) {
                       parallel_for(r1 - r0, 1 << 15, [&](size_t a0, size_t a1) {
                           copy_out(h, h + 3 * n, h + 6 * n, r0 + a0, r0 + a1, x, v, f, sb);
                       });
                   });
    if (rc) return rc;
    if (t) *t = e->worlds[world].dev.t;
    return PDPD_OK;
}

int pdpd_read_states(pdpd_engine *e, uint32_t n_worlds, const pdpd_state_view *out,
                     size_t stride)
{
    if (!e || (!out && n_worlds)) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (n_worlds != e->worlds.size())
        return e->fail(PDPD_E_INVALID, "%u views for a batch of %zu worlds", n_worlds, e->worlds.size());
    cudaSetDevice(e->device);
    const size_t sb = stride ? stride : 3 * sizeof(double);
    std::vector<uint32_t> base(n_worlds + 1);
    for (uint32_t i = 0; i < n_worlds; i++) base[i] = e->worlds[i].dev.bead_base;
    base[n_worlds] = e->n_beads;
    bool direct = e->host_direct();
    for (uint32_t i = 0; direct && i < n_worlds; i++)
        direct = vec_ok(out[i].x, sb) && vec_ok(out[i].v, sb) && vec_ok(out[i].f, sb);
    int rc = PDPD_OK;
    if (direct) {
        std::vector<ReadDest> dest(n_worlds);
        for (uint32_t i = 0; i < n_worlds; i++) dest[i] = ReadDest{out[i].x, out[i].v, out[i].f, sb};
        rc = read_direct(e, 0, n_worlds, dest);
    } else {
        // each chunk of the batch's beads, split across host threads whatever the worlds' sizes
        rc = download(e, 0, e->stream, true);
        if (rc) return rc;
        rc = read_rows(e, 0, e->n_beads, [&](const double *h, size_t n, size_t c0, size_t c1) {
            parallel_for(c1 - c0, 1 << 15, [&](size_t a0, size_t a1) {
                const size_t g0 = c0 + a0, g1 = c0 + a1;
                uint32_t i = (uint32_t)(std::upper_bound(base.begin(), base.end() - 1, (uint32_t)g0) - base.begin()) - 1;
                for (size_t g = g0; g < g1;) {
                    while (g >= base[i + 1]) i++;
                    const size_t b = base[i], e1 = std::min<size_t>(g1, base[i + 1]);
                    copy_out(h + 3 * b, h + 3 * (n + b), h + 3 * (2 * n + b), g - b, e1 - b, out[i].x, out[i].v,
                             out[i].f, sb);
                    g = e1;
                }
            });
        });
    }
    if (rc) return rc;
    for (uint32_t i = 0; i < n_worlds; i++)
        if (out[i].t) *out[i].t = e->worlds[i].dev.t;
    return PDPD_OK;
}

int pdpd_run_intervals(pdpd_engine *e, int32_t interval_count, uint32_t interval_size, double *x,
                       double *v, double *f, size_t stride, pdpd_interval_fn cb, void *user,
                       uint32_t *steps_done)
{
    if (steps_done) *steps_done = 0;
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "Run called with no world attached");
    if (e->worlds.size() != 1) return e->fail(PDPD_E_STATE, "interval runs need exactly one attached world");
    if (!cb) return e->fail(PDPD_E_INVALID, "no callback");
    cudaSetDevice(e->device);
    double t0 = now_s();
    const WorldDev wd0 = e->worlds[0].dev;
    const uint32_t n = wd0.n_beads;
    const size_t nbytes = sizeof(double) * 9 * (size_t)n;
    for (int b = 0; b < 2; b++) {
        if (e->d_staging[b].alloc(nbytes) != cudaSuccess)
            return e->fail(PDPD_E_NOMEM, "staging allocation failed");
        if (e->h_staging[b].alloc(nbytes + sizeof(WorldDev)) != cudaSuccess)
            return e->fail(PDPD_E_NOMEM, "pinned allocation failed");
    }
    uint32_t done = 0;
    int64_t t_cur = wd0.t;
    int rc = PDPD_OK;
    if (interval_count == 0) return PDPD_OK;
    rc = e->enqueue_run(interval_size, e->stream);
    for (int64_t k = 1; rc == PDPD_OK; k++) {
        const int b = (int)(k & 1);
        // Snapshot interval k into device staging b and start copying it to the host on the
        // side stream; the main stream goes straight on with interval k+1.
        rc = download(e, b, e->stream);
        if (rc) break;
        WorldDev *herr = (WorldDev *)((char *)e->h_staging[b].p + nbytes);
        cudaMemcpyAsync(herr, e->d_worlds.p, sizeof(WorldDev), cudaMemcpyDeviceToHost, e->stream);
        cudaEventRecord(e->ev_snap[b], e->stream);
        cudaStreamWaitEvent(e->side, e->ev_snap[b], 0);
        cudaMemcpyAsync(e->h_staging[b].p, e->d_staging[b].p, nbytes, cudaMemcpyDeviceToHost, e->side);
        cudaEventRecord(e->ev_copied[b], e->side);
        const bool more = interval_count < 0 || k < interval_count;
        if (more) {
            rc = e->enqueue_run(interval_size, e->stream);
            if (rc) break;
        }
        cudaError_t ce = cudaEventSynchronize(e->ev_copied[b]);
        if (ce != cudaSuccess) {
            rc = e->cuda_fail(ce, "snapshot copy");
            break;
        }
        if (herr->err) {
            cudaStreamSynchronize(e->stream);
            rc = e->check_device_errors();
            if (!rc) rc = e->fail(PDPD_E_BEAD_LOST, "device error during interval");
            break;
        }
        t_cur = herr->t;
        scatter((const double *)e->h_staging[b].p, n, x, v, f, stride);
        done += interval_size;
        int go = cb(user, t_cur);
        if (!go || !more) {
            if (more) {
                // Roll the device back to the state the caller has just seen: re-bin the
                // snapshot (lossless in both precisions) and reset t.
                cudaStreamSynchronize(e->stream);
                KArgs a = e->args;
                a.staging = e->d_staging[b].as<double>();
                std::vector<WorldDev> wv(1);
                memcpy(wv.data(), herr, sizeof(WorldDev));
                wv[0].err = 0;
                cudaMemcpyAsync(e->d_worlds.p, wv.data(), sizeof(WorldDev), cudaMemcpyHostToDevice, e->stream);
                e->launches += e->fp64() ? launch_bin64(a, e->d_hash.as<uint32_t>(), e->stream)
                                         : launch_bin32(a, e->d_hash.as<uint32_t>(), e->stream);
                e->launches += launch_sort(a, e->fp64(), 0, 1, e->stream);
                rc = pdpd_sync(e);
            }
            break;
        }
    }
    if (rc == PDPD_OK) rc = pdpd_sync(e);
    if (steps_done) *steps_done = done;
    double dt = now_s() - t0;
    auto acc = [](double &slot, double v) { slot = slot < 0 ? v : slot + v; };
    acc(e->timings.execute_to_first_bead, dt);
    acc(e->timings.execute_to_last_bead, dt);
    return rc;
}

int pdpd_get_timings(pdpd_engine *e, pdpd_timings *out)
{
    if (!e || !out) return PDPD_E_INVALID;
    *out = e->timings;
    return PDPD_OK;
}

int pdpd_get_config(pdpd_engine *e, uint32_t index, char *name, size_t name_len, char *desc,
                    size_t desc_len, char *value, size_t value_len)
{
    if (!e) return PDPD_E_INVALID;
    if (index >= sizeof(kConfig) / sizeof(kConfig[0])) return PDPD_E_INVALID;
    int vals[] = {e->cfg_list_capacity, e->cfg_grid_blocks, e->cfg_graph_steps, e->cfg_use_graphs,
                  e->cfg_force_kernel, e->cfg_brick[0], e->cfg_brick[1], e->cfg_brick[2],
                  e->cfg_autotune, e->cfg_host_direct};
    static_assert(sizeof(vals) / sizeof(vals[0]) == sizeof(kConfig) / sizeof(kConfig[0]), "config values");
    if (name && name_len) snprintf(name, name_len, "%s", kConfig[index].name);
    if (desc && desc_len) snprintf(desc, desc_len, "%s", kConfig[index].desc);
    if (value && value_len) {
        if (std::string(kConfig[index].name) == "autotune" && e->tuned)
            snprintf(value, value_len, "%d (trials %s)", vals[index], e->tune_log.c_str());
        else if (std::string(kConfig[index].name) == "host_direct" && vals[index] && !e->host_access)
            snprintf(value, value_len, "%d (staged: this device does not reach pageable host memory)", vals[index]);
        else
            snprintf(value, value_len, "%d", vals[index]);
    }
    return PDPD_OK;
}

int pdpd_set_config(pdpd_engine *e, const char *key, const char *value)
{
    if (!e || !key || !value) return PDPD_E_INVALID;
    char *end = nullptr;
    long v = strtol(value, &end, 10);
    if (!end || *end || v < 0 || v > (1 << 24)) return e->fail(PDPD_E_INVALID, "bad value '%s' for '%s'", value, key);
    std::string k = key;
    if (k == "list_capacity") e->cfg_list_capacity = (int)v;
    else if (k == "grid_blocks") e->cfg_grid_blocks = (int)v;
    else if (k == "graph_steps") e->cfg_graph_steps = (int)v;
    else if (k == "use_graphs") e->cfg_use_graphs = v ? 1 : 0;
    else if (k == "force_kernel") {
        if (v != 1 && v != 6 && v != 8 && v != 9)
            return e->fail(PDPD_E_INVALID, "force_kernel must be 1, 6, 8 or 9");
        e->cfg_force_kernel = (int)v;
        e->kernel_user = true;
    } else if (k == "brick_x" || k == "brick_y" || k == "brick_z") {
        int idx = k == "brick_x" ? 0 : (k == "brick_y" ? 1 : 2);
        int nb[3] = {e->cfg_brick[0], e->cfg_brick[1], e->cfg_brick[2]};
        nb[idx] = (int)v;
        if (v < 1 || v > 32 || nb[0] * nb[1] > 64 || (nb[0] + 2) * (nb[1] + 2) * (nb[2] + 2) > 2048)
            return e->fail(PDPD_E_INVALID, "brick shape %dx%dx%d out of range", nb[0], nb[1], nb[2]);
        e->cfg_brick[idx] = (int)v;
        e->brick_user = true;
    } else if (k == "autotune") {
        e->cfg_autotune = v ? 1 : 0;
        e->tuned = false;
    } else if (k == "host_direct") {
        e->cfg_host_direct = v ? 1 : 0;
        return PDPD_OK;  // no bearing on the captured graphs or the kernels
    }
    else return e->fail(PDPD_E_INVALID, "Unknown engine config name '%s'", key);
    e->drop_graph();  // graphs are captured again at the next run
    if (e->attached && (k == "force_kernel" || k.rfind("brick_", 0) == 0 || k == "grid_blocks")) {
        cudaSetDevice(e->device);
        cudaStreamSynchronize(e->stream);
        return e->configure_bricks();  // kernel choice and brick shape apply from the next step
    }
    return PDPD_OK;
}

}  // extern "C"

namespace pdpd {
struct ObsPartial {
    double ke2, mx, my, mz, virial;
};
}  // namespace pdpd

extern "C" {

int pdpd_observe(pdpd_engine *e, uint32_t world, pdpd_observables *out, uint32_t n_bins,
                 uint64_t *rdf, uint32_t n_bond_bins, uint64_t *bond_hist)
{
    if (!e || !out) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (world >= e->worlds.size()) return e->fail(PDPD_E_INVALID, "world index out of range");
    cudaSetDevice(e->device);
    const WorldDev &wd = e->worlds[world].dev;
    const size_t n_rdf = rdf ? (size_t)wd.n_types * wd.n_types * n_bins : 0;
    const size_t n_bh = bond_hist ? n_bond_bins : 0;
    const uint32_t blocks = (wd.n_beads + 127) / 128;
    DevBuf d_rdf, d_bh, d_part;
    cudaError_t ce = d_rdf.alloc(8 * std::max<size_t>(1, n_rdf));
    if (ce == cudaSuccess) ce = d_bh.alloc(8 * std::max<size_t>(1, n_bh));
    if (ce == cudaSuccess) ce = d_part.alloc(sizeof(ObsPartial) * std::max<uint32_t>(1, blocks));
    if (ce != cudaSuccess) return e->fail(PDPD_E_NOMEM, "observables: device allocation failed");
    cudaStream_t s = e->stream;
    cudaMemsetAsync(d_rdf.p, 0, d_rdf.bytes, s);
    cudaMemsetAsync(d_bh.p, 0, d_bh.bytes, s);
    e->launches += launch_observe(e->args, e->fp64(), world, wd.n_beads, n_bins,
                                  n_rdf ? d_rdf.as<unsigned long long>() : nullptr, n_bond_bins,
                                  n_bh ? d_bh.as<unsigned long long>() : nullptr,
                                  d_part.as<ObsPartial>(), s);
    std::vector<ObsPartial> part(blocks);
    ce = cudaGetLastError();
    if (ce == cudaSuccess && blocks)
        ce = cudaMemcpyAsync(part.data(), d_part.p, sizeof(ObsPartial) * blocks, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess && n_rdf) ce = cudaMemcpyAsync(rdf, d_rdf.p, 8 * n_rdf, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess && n_bh) ce = cudaMemcpyAsync(bond_hist, d_bh.p, 8 * n_bh, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "observables");
    pdpd_observables o{0, {0, 0, 0}, 0};
    for (const ObsPartial &p : part) {  // block order: deterministic
        o.ke2 += p.ke2;
        o.momentum[0] += p.mx;
        o.momentum[1] += p.my;
        o.momentum[2] += p.mz;
        o.virial += p.virial;
    }
    *out = o;
    return PDPD_OK;
}

static_assert(sizeof(pdpd_pair_terms) == sizeof(PairLogRec), "pair log record layouts differ");

int pdpd_log_pair_terms(pdpd_engine *e, uint32_t world, const uint32_t *bead_ids, uint32_t n_ids,
                        pdpd_pair_terms *out, uint32_t capacity, uint32_t *n_pairs)
{
    if (n_pairs) *n_pairs = 0;
    if (!e || (n_ids && !bead_ids) || (capacity && !out)) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (world >= e->worlds.size()) return e->fail(PDPD_E_INVALID, "world index out of range");
    const WorldDev wd = e->worlds[world].dev;
    std::vector<uint32_t> sel;
    for (uint32_t k = 0; k < n_ids; k++) {
        if (bead_ids[k] >= wd.n_beads) return e->fail(PDPD_E_INVALID, "bead id %u out of range", bead_ids[k]);
        sel.push_back(wd.bead_base + bead_ids[k]);
    }
    std::sort(sel.begin(), sel.end());
    sel.erase(std::unique(sel.begin(), sel.end()), sel.end());
    cudaSetDevice(e->device);
    cudaStream_t s = e->stream;
    const uint32_t ns = (uint32_t)sel.size();
    DevBuf d_sel, d_counts, d_offs, d_out;
    cudaError_t ce = d_sel.alloc(sizeof(uint32_t) * std::max<uint32_t>(1, ns));
    if (ce == cudaSuccess) ce = d_counts.alloc(sizeof(uint32_t) * std::max<uint32_t>(1, ns));
    if (ce == cudaSuccess) ce = d_offs.alloc(sizeof(uint32_t) * std::max<uint32_t>(1, ns));
    if (ce != cudaSuccess) return e->fail(PDPD_E_NOMEM, "pair log: device allocation failed");
    if (ns) ce = cudaMemcpyAsync(d_sel.p, sel.data(), sizeof(uint32_t) * ns, cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "pair log upload");
    const bool f64 = e->fp64();
    auto log = [&](const uint32_t *offs, uint32_t *counts, PairLogRec *recs) {
        return f64 ? launch_pair_log64(e->args, d_sel.as<uint32_t>(), ns, offs, counts, recs, s)
                   : launch_pair_log32(e->args, d_sel.as<uint32_t>(), ns, offs, counts, recs, s);
    };
    // the step up to its force pass (update_pos and the cell lists of t + 1), then the log of
    // the pairs that force pass will evaluate, then the force pass and the end of the step
    e->launches += e->enqueue_begin(s);
    e->launches += log(nullptr, d_counts.as<uint32_t>(), nullptr);
    std::vector<uint32_t> counts(ns), offs(ns);
    if (ns) ce = cudaMemcpyAsync(counts.data(), d_counts.p, sizeof(uint32_t) * ns, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "pair log count");
    uint64_t total = 0;
    for (uint32_t k = 0; k < ns; k++) {
        offs[k] = (uint32_t)total;
        total += counts[k];
    }
    if (total >= (1ull << 31)) return e->fail(PDPD_E_UNSUPPORTED, "pair log too large");
    ce = d_out.alloc(sizeof(PairLogRec) * std::max<uint64_t>(1, total));
    if (ce != cudaSuccess) return e->fail(PDPD_E_NOMEM, "pair log: device allocation failed");
    if (ns) ce = cudaMemcpyAsync(d_offs.p, offs.data(), sizeof(uint32_t) * ns, cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "pair log upload");
    e->launches += log(d_offs.as<uint32_t>(), nullptr, d_out.as<PairLogRec>());
    e->launches += e->enqueue_final(s);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return e->cuda_fail(ce, "kernel launch");
    std::vector<PairLogRec> recs(total);
    if (total)
        ce = cudaMemcpyAsync(recs.data(), d_out.p, sizeof(PairLogRec) * total, cudaMemcpyDeviceToHost, s);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "pair log download");
    int rc = e->check_device_errors();  // synchronises
    if (rc) return rc;
    for (PairLogRec &r : recs) {  // world-local ids
        r.home_id -= wd.bead_base;
        r.other_id -= wd.bead_base;
    }
    const uint32_t n_copy = (uint32_t)std::min<uint64_t>(total, capacity);
    if (n_copy) memcpy(out, recs.data(), sizeof(PairLogRec) * n_copy);
    if (n_pairs) *n_pairs = (uint32_t)total;
    return PDPD_OK;
}

int pdpd_profile_run(pdpd_engine *e, uint32_t n_steps, pdpd_phase_times *out)
{
    if (!e || !out) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "Run called with no world attached");
    cudaSetDevice(e->device);
    memset(out, 0, sizeof *out);
    if (n_steps == 0) return PDPD_OK;
    const bool f64 = e->fp64();
    cudaStream_t s = e->stream;
    // events: one before and after every phase
    std::vector<cudaEvent_t> ev;
    auto mark = [&]() {
        cudaEvent_t x;
        cudaEventCreate(&x);
        cudaEventRecord(x, s);
        ev.push_back(x);
        return ev.size() - 1;
    };
    struct Span {
        size_t a, b;
        int kind;  // 0 force, 1 sort, 2 other
    };
    std::vector<Span> spans;
    size_t m0 = mark();
    e->launches += f64 ? launch_begin64(e->args, s) : launch_begin32(e->args, s);
    size_t m1 = mark();
    spans.push_back({m0, m1, 2});
    e->launches += launch_sort(e->args, f64, 0, 0, s);
    size_t m2 = mark();
    spans.push_back({m1, m2, 1});
    for (uint32_t i = 0; i + 1 < n_steps; i++) {
        size_t a = mark();
        e->launches += f64 ? launch_force64(e->args, 0, s) : launch_force32(e->args, 0, s);
        size_t b = mark();
        e->launches += launch_sort(e->args, f64, 1, 0, s);
        size_t c = mark();
        spans.push_back({a, b, 0});
        spans.push_back({b, c, 1});
    }
    size_t a = mark();
    e->launches += f64 ? launch_force64(e->args, 1, s) : launch_force32(e->args, 1, s);
    size_t b = mark();
    e->launches += f64 ? launch_finish64(e->args, s) : launch_finish32(e->args, s);
    size_t c = mark();
    spans.push_back({a, b, 0});
    spans.push_back({b, c, 2});
    cudaError_t ce = cudaGetLastError();
    int rc = ce == cudaSuccess ? pdpd_sync(e) : e->cuda_fail(ce, "kernel launch");
    if (rc == PDPD_OK) {
        for (const Span &sp : spans) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[sp.a], ev[sp.b]);
            if (sp.kind == 0) {
                out->force_ms += ms;
                out->force_launches++;
            } else if (sp.kind == 1) {
                out->sort_ms += ms;
                out->sort_launches++;
            } else {
                out->other_ms += ms;
            }
        }
    }
    for (cudaEvent_t x : ev) cudaEventDestroy(x);
    return rc;
}

int pdpd_rng_eval(size_t n, const uint32_t *t, const uint64_t *seed, const uint32_t *a,
                  const uint32_t *b, uint32_t *h_out, float *u_out)
{
    if (n == 0) return PDPD_OK;
    if (!t || !seed || !a || !b) {
        g_last_error = "pdpd_rng_eval: missing input array";
        return PDPD_E_INVALID;
    }
    DevBuf dt, ds, da, db, dh, du;
    cudaError_t ce = cudaSuccess;
    auto A = [&](DevBuf &bf, size_t bytes) {
        if (ce == cudaSuccess) ce = bf.alloc(bytes);
    };
    A(dt, 4 * n);
    A(ds, 8 * n);
    A(da, 4 * n);
    A(db, 4 * n);
    A(dh, 4 * n);
    A(du, 4 * n);
    if (ce == cudaSuccess) ce = cudaMemcpy(dt.p, t, 4 * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(ds.p, seed, 8 * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(da.p, a, 4 * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(db.p, b, 4 * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
        launch_rng_eval(n, dt.as<uint32_t>(), ds.as<uint64_t>(), da.as<uint32_t>(), db.as<uint32_t>(),
                        dh.as<uint32_t>(), du.as<float>(), 0);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess && h_out) ce = cudaMemcpy(h_out, dh.p, 4 * n, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && u_out) ce = cudaMemcpy(u_out, du.p, 4 * n, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) {
        g_last_error = std::string("pdpd_rng_eval: ") + cudaGetErrorString(ce);
        return PDPD_E_CUDA;
    }
    return PDPD_OK;
}

uint64_t pdpd_kernel_launches(pdpd_engine *e)
{
    return e ? e->launches : 0;
}

}  // extern "C"


// ==========================================================================================
// v2binary snapshots (the BinaryData section of the reference's v2binary state format)
// ==========================================================================================

extern "C" {

int pdpd_v2binary_prepare(pdpd_engine *e, uint32_t world, uint32_t n_polymers,
                          const uint32_t *polymer_ids, const uint32_t *polymer_types,
                          const uint32_t *polymer_start, const uint32_t *polymer_beads,
                          size_t *section_bytes)
{
    if (section_bytes) *section_bytes = 0;
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (world >= e->worlds.size()) return e->fail(PDPD_E_INVALID, "world index out of range");
    if (n_polymers && (!polymer_types || !polymer_start || !polymer_beads))
        return e->fail(PDPD_E_INVALID, "missing polymer arrays");
    const uint32_t n = e->worlds[world].dev.n_beads;
    if (n_polymers && polymer_start[0] != 0) return e->fail(PDPD_E_INVALID, "polymer_start[0] must be 0");
    auto L = std::make_shared<V2Layout>();
    std::vector<uint32_t> off(n, 0xFFFFFFFFu);
    std::vector<uint8_t> &t = L->tmpl;
    auto put16 = [&](uint32_t v) {
        t.push_back((uint8_t)(v & 0xFF));
        t.push_back((uint8_t)(v >> 8));
    };
    auto put32 = [&](uint32_t v) {
        for (int k = 0; k < 4; k++) t.push_back((uint8_t)(v >> (8 * k)));
    };
    auto mark = [&](size_t begin) {
        if (t.size() > begin) L->structure.push_back({(uint32_t)begin, (uint32_t)(t.size() - begin)});
    };
    // write_polymer_binary (dpd_state_io.hpp:182-247), per polymer in order
    uint32_t prev_pid = 0xFFFFFFFFu, prev_bid = 0xFFFFFFFFu;
    for (uint32_t p = 0; p < n_polymers; p++) {
        const uint32_t b0 = polymer_start[p], b1 = polymer_start[p + 1];
        if (b1 <= b0) return e->fail(PDPD_E_INVALID, "polymer %u has no beads", p);
        if (polymer_types[p] >= (1u << 13)) return e->fail(PDPD_E_INVALID, "polymer type does not fit 13 bits");
        const uint32_t pid = polymer_ids ? polymer_ids[p] : p;
        const bool nsp = pid != prev_pid + 1u;
        const bool nsi = polymer_beads[b0] != prev_bid + 1u;
        bool nsa = false;
        for (uint32_t k = b0 + 1; k < b1; k++) nsa |= polymer_beads[k - 1] + 1u != polymer_beads[k];
        size_t begin = t.size();
        put16(polymer_types[p] | (nsp ? 1u << 13 : 0u) | (nsi ? 1u << 14 : 0u) | (nsa ? 1u << 15 : 0u));
        if (nsp) put32(pid - prev_pid);
        prev_pid = pid;
        for (uint32_t k = b0; k < b1; k++) {
            const uint32_t bid = polymer_beads[k];
            if (bid >= n) return e->fail(PDPD_E_INVALID, "polymer %u refers to bead %u of %u", p, bid, n);
            if (off[bid] != 0xFFFFFFFFu) return e->fail(PDPD_E_INVALID, "bead %u appears twice", bid);
            if ((k == b0 && nsi) || (k > b0 && nsa)) put32(bid - prev_bid);
            prev_bid = bid;
            mark(begin);
            off[bid] = (uint32_t)t.size();
            t.resize(t.size() + 20, 0);
            begin = t.size();
        }
        if (t.size() >= 0xFFFFFFF0u) return e->fail(PDPD_E_UNSUPPORTED, "section larger than 4 GB");
    }
    for (uint32_t i = 0; i < n; i++)
        if (off[i] == 0xFFFFFFFFu) return e->fail(PDPD_E_INVALID, "bead %u belongs to no polymer", i);
    L->bytes = t.size();
    cudaSetDevice(e->device);
    if (L->d_buf.alloc(std::max<size_t>(L->bytes, 16)) != cudaSuccess ||
        L->d_off.alloc(sizeof(uint32_t) * std::max<uint32_t>(n, 1)) != cudaSuccess ||
        e->d_v2err.alloc(16) != cudaSuccess)
        return e->fail(PDPD_E_NOMEM, "v2binary layout allocation failed");
    cudaError_t ce = cudaMemcpyAsync(L->d_buf.p, t.data(), L->bytes, cudaMemcpyHostToDevice, e->stream);
    if (ce == cudaSuccess && n)
        ce = cudaMemcpyAsync(L->d_off.p, off.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "v2binary layout upload");
    e->worlds[world].v2 = L;
    if (section_bytes) *section_bytes = L->bytes;
    return PDPD_OK;
}

int pdpd_v2binary_encode(pdpd_engine *e, uint32_t world, uint8_t *out, size_t capacity, size_t *bytes)
{
    if (bytes) *bytes = 0;
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (world >= e->worlds.size()) return e->fail(PDPD_E_INVALID, "world index out of range");
    V2Layout *L = e->worlds[world].v2.get();
    if (!L) return e->fail(PDPD_E_STATE, "pdpd_v2binary_prepare was not called for this world");
    if (bytes) *bytes = L->bytes;
    if (!out) return PDPD_OK;
    if (capacity < L->bytes) return e->fail(PDPD_E_INVALID, "output buffer too small (%zu < %zu bytes)", capacity, L->bytes);
    cudaSetDevice(e->device);
    const WorldDev &wd = e->worlds[world].dev;
    uint32_t herr = 0;
    cudaError_t ce = cudaMemsetAsync(e->d_v2err.p, 0, sizeof(uint32_t), e->stream);
    e->launches += launch_v2_encode(e->args, e->fp64(), world, wd.n_beads, L->d_buf.as<uint8_t>(),
                                    L->d_off.as<uint32_t>(), e->d_v2err.as<uint32_t>(), e->stream);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    // through pinned staging (a copy to pageable memory would be staged by the driver)
    if (e->h_staging[1].alloc(L->bytes + 16) != cudaSuccess) return e->fail(PDPD_E_NOMEM, "pinned allocation failed");
    uint32_t *herr_p = (uint32_t *)((uint8_t *)e->h_staging[1].p + ((L->bytes + 3) & ~size_t(3)));
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(e->h_staging[1].p, L->d_buf.p, L->bytes, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(herr_p, e->d_v2err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "v2binary encode");
    herr = *herr_p;
    const uint8_t *src = (const uint8_t *)e->h_staging[1].p;
    parallel_for(L->bytes, 1 << 22, [&](size_t b, size_t en) { memcpy(out + b, src + b, en - b); });
    if (herr & 2u) return e->fail(PDPD_E_INVALID, "Bead is out of bounds.");
    if (herr & 1u)
        return e->fail(PDPD_E_INVALID, "A velocity or force is not finite or has magnitude 65536 or more "
                                       "(not representable as CVec3Half).");
    return PDPD_OK;
}

static int rebin_from_staging(pdpd_engine *e);

int pdpd_v2binary_decode(pdpd_engine *e, uint32_t world, const uint8_t *in, size_t bytes)
{
    if (!e) return PDPD_E_INVALID;
    if (!e->attached) return e->fail(PDPD_E_STATE, "no world attached");
    if (world >= e->worlds.size()) return e->fail(PDPD_E_INVALID, "world index out of range");
    V2Layout *L = e->worlds[world].v2.get();
    if (!L) return e->fail(PDPD_E_STATE, "pdpd_v2binary_prepare was not called for this world");
    if (!in || bytes != L->bytes)
        return e->fail(PDPD_E_INVALID, "section of %zu bytes, the world's layout has %zu", bytes, L->bytes);
    for (const auto &r : L->structure)
        if (memcmp(in + r.first, L->tmpl.data() + r.first, r.second) != 0)
            return e->fail(PDPD_E_INVALID, "section structure (polymer headers or id deltas) at byte %u "
                                           "differs from the world's polymers", r.first);
    cudaSetDevice(e->device);
    // every world's rows to staging buffer 0, this world's rows from the section, re-bin
    int rc = download(e, 0, e->stream);
    if (rc) return rc;
    uint32_t herr = 0;
    cudaError_t ce = cudaMemsetAsync(e->d_v2err.p, 0, sizeof(uint32_t), e->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(L->d_buf.p, in, bytes, cudaMemcpyHostToDevice, e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "v2binary upload");
    e->launches += launch_v2_decode(e->args, world, e->worlds[world].dev.n_beads, L->d_buf.as<uint8_t>(),
                                    L->d_off.as<uint32_t>(), e->d_staging[0].as<double>(),
                                    e->d_v2err.as<uint32_t>(), e->stream);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&herr, e->d_v2err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "v2binary decode");
    if (herr) return e->fail(PDPD_E_INVALID, "Bead was out of box.");
    return rebin_from_staging(e);
}

}  // extern "C"

// Rebuild the sorted state from the id-ordered staging rows in buffer 0 (as the end of an
// attach does); t and the parameters are unchanged.
static int rebin_from_staging(pdpd_engine *e)
{
    KArgs a = e->args;
    a.staging = e->d_staging[0].as<double>();
    const uint32_t *hash_in = e->d_hash.as<uint32_t>();
    e->launches += e->fp64() ? launch_bin64(a, hash_in, e->stream) : launch_bin32(a, hash_in, e->stream);
    e->launches += launch_sort(a, e->fp64(), 0, 1, e->stream);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return e->cuda_fail(ce, "re-bin kernels");
    return e->check_device_errors();
}

// ==========================================================================================
// Job server: continuous batching of independent worlds on one engine.
//
// Jobs (a world, a number of steps, a callback) arrive from any thread.  One worker thread
// admits them in arrival order while their estimated device footprint fits the memory
// budget, keeps every admitted world attached in one batch, and runs the batch in epochs that
// end at the next interval boundary of some job (every `interval` steps of it) or at its
// completion.  When jobs leave or join, the batch is re-packed on the device: continuing
// worlds take their state over from the old arena with no host round trip.  At a boundary
// the snapshot is unsorted on the main stream and copied to pinned host memory on the side
// stream; the callbacks of epoch k run on the host while epoch k+1 computes.  The worlds of a
// batch are independent and each is stepped exactly as if it ran alone, so a job's results do
// not depend on what else the server runs.
// ==========================================================================================

#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>

namespace {

struct ServerJob {
    uint64_t id = 0;
    std::vector<double> cons, diss, x, v, f, bk, br, ak, at, cell_a, cell_g;
    std::vector<uint8_t> stat;
    std::vector<uint32_t> hash, bb, ab;
    pdpd_world desc{};
    uint32_t n_steps = 0, done = 0;
    int64_t t = 0;
    pdpd_job_fn cb = nullptr;
    void *user = nullptr;
    double t_submit = 0;
    size_t bytes = 0;
    int slot = -1;           // world index in the attached batch, -1 before the first attach
    bool stopped = false;    // no further callbacks: the callback asked to stop, or it failed
    bool ended = false;      // final state delivered or owed; the world leaves the batch at the
                             // next point where every running job is at an interval boundary
    bool leave_now = false;  // ended, and stepping it on to that point costs more than a re-pack
};

// A callback owed for one job: its rows start at `row` in host snapshot buffer `buf`.
struct Delivery {
    ServerJob *job;
    size_t row;
    uint32_t n_beads;
    int64_t t;
    int final_state;
};

size_t job_bytes(const pdpd_world &w, int precision)
{
    // sorted state A and B, ids / cells / ranks, two id-ordered staging rows, hashes
    const size_t per_bead = precision == PDPD_FP64 ? 424 : 296;
    const size_t cells = (size_t)w.box[0] * w.box[1] * w.box[2];
    return per_bead * w.n_beads + 12 * cells +
           48 * (2 * (size_t)w.n_bonds + 3 * (size_t)w.n_angles) + 4096;
}

}  // namespace

struct pdpd_server {
    pdpd_engine *eng = nullptr;
    int precision = PDPD_FP32;
    size_t budget = 0;
    uint32_t interval = 100;

    // shared with submitters (under mu)
    std::mutex mu;
    std::condition_variable cv, cv_idle;
    std::deque<std::unique_ptr<ServerJob>> pending;
    bool stop = false, busy = false;
    int status = PDPD_OK;
    std::string err;
    uint64_t next_id = 1;
    pdpd_server_stats st{};
    std::vector<double> latencies;
    double t_first = -1, t_last = 0, t_busy_from = 0;

    // worker only
    std::vector<std::unique_ptr<ServerJob>> active, retiring;
    std::vector<Delivery> owed;
    int owed_buf = 0;
    bool changed = false;
    double rate_est = 2e9;        // bead-steps per second of recent epochs
    double repack_est_s = 0.005;  // recent re-pack time
    HostPinned snap[2];
    cudaEvent_t ev_unsorted = nullptr, ev_copied[2] = {nullptr, nullptr};
    cudaEvent_t ev_step0 = nullptr, ev_step1[2] = {nullptr, nullptr};  // around an epoch's steps
    int end_k = 0;           // ev_step1[end_k]: the last epoch's end
    bool have_end = false;
    std::thread worker;

    void run();
    int repack();
    void deliver();
    void fail_jobs(const std::vector<ServerJob *> &jobs, int code);
    void finish_job(ServerJob &j);
};

// Attach the active jobs as one batch, continuing worlds taking their state over on the device.
int pdpd_server::repack()
{
    if (!changed) return PDPD_OK;
    cudaStreamSynchronize(eng->side);  // no snapshot copy may still read the old arena
    changed = false;
    if (active.empty()) {
        pdpd_attach(eng, nullptr);  // release the arena while idle
        return PDPD_OK;
    }
    std::vector<pdpd_world> descs;
    std::vector<int32_t> keep;
    for (auto &j : active) {
        pdpd_world d = j->desc;
        d.t = j->t;
        descs.push_back(d);
        keep.push_back(j->slot);
    }
    const double t0 = now_s();
    int rc = attach_impl(eng, descs.data(), (uint32_t)descs.size(), keep.data());
    if (rc) return rc;
    const double t_repack = now_s() - t0;
    for (size_t i = 0; i < active.size(); i++) {
        ServerJob &j = *active[i];
        if (j.slot < 0) {  // the initial state lives on the device from now on
            std::vector<double>().swap(j.x);
            std::vector<double>().swap(j.v);
            std::vector<double>().swap(j.f);
            j.desc.x = j.desc.v = j.desc.f = nullptr;
        }
        j.slot = (int)i;
    }
    std::lock_guard<std::mutex> lk(mu);
    st.repacks++;
    st.repack_s += t_repack;
    repack_est_s = 0.7 * repack_est_s + 0.3 * t_repack;
    return PDPD_OK;
}

void pdpd_server::finish_job(ServerJob &j)
{
    const double now = now_s();
    std::lock_guard<std::mutex> lk(mu);
    latencies.push_back(now - j.t_submit);
    st.jobs_done++;
    t_last = now;
}

// Callbacks of the previous epoch (its snapshot copy overlapped the current epoch).
void pdpd_server::deliver()
{
    if (owed.empty()) return;
    cudaEventSynchronize(ev_copied[owed_buf]);
    const double *base = (const double *)snap[owed_buf].p;
    for (const Delivery &d : owed) {
        ServerJob &j = *d.job;
        if (j.stopped) continue;  // stopped by an earlier callback, or failed
        const double *row = base + d.row;
        const int status = d.final_state ? 1 : 0;
        const int go = j.cb ? j.cb(j.user, j.id, d.t, row, row + 3, row + 6, 9 * sizeof(double),
                                   d.n_beads, status)
                            : 1;
        if (d.final_state) {
            finish_job(j);
        } else if (!go && !j.stopped) {  // the job ends at this snapshot
            j.stopped = j.ended = true;
            finish_job(j);
        }
    }
    owed.clear();
    retiring.clear();
}

// Jobs whose world raised an error flag: a running job gets a failure callback; every one
// leaves the batch at the next iteration.
void pdpd_server::fail_jobs(const std::vector<ServerJob *> &jobs, int code)
{
    for (ServerJob *j : jobs) {
        const bool running = !j->ended;
        j->stopped = j->ended = true;
        if (!running) continue;  // an ended job's world kept stepping only to fill the epoch
        if (j->cb) j->cb(j->user, j->id, j->t, nullptr, nullptr, nullptr, 0, 0, -code);
        std::lock_guard<std::mutex> lk(mu);
        st.jobs_failed++;
        status = code;
        err = eng->err;
    }
    for (size_t i = 0; i < active.size();)
        if (std::find(jobs.begin(), jobs.end(), active[i].get()) != jobs.end()) {
            retiring.push_back(std::move(active[i]));
            active.erase(active.begin() + i);
            changed = true;
        } else {
            i++;
        }
}

void pdpd_server::run()
{
    cudaSetDevice(eng->device);
    int b = 0;  // host snapshot buffer of the current epoch
    double t_sync_end = -1;  // when the host saw the last epoch finish
    while (true) {
        double waited = 0;  // time idle for want of jobs (not host overhead)
        {
            std::unique_lock<std::mutex> lk(mu);
            const double t_w0 = now_s();
            cv.wait(lk, [&] { return stop || !pending.empty() || !active.empty() || !owed.empty(); });
            waited = now_s() - t_w0;
            if (stop && pending.empty() && active.empty() && owed.empty()) break;
            // Membership changes only where every running job is at one of its interval
            // boundaries: the jobs' intervals stay in phase, epochs are whole intervals (a job
            // that ends mid-interval splits one epoch in two, with no re-pack), and ended jobs
            // leave and waiting jobs join in one re-pack.
            bool in_phase = true;
            for (auto &j : active)
                if (!j->ended) in_phase &= j->done % interval == 0;
            for (size_t i = 0; i < active.size();)
                if (active[i]->ended && (in_phase || active[i]->leave_now)) {
                    retiring.push_back(std::move(active[i]));
                    active.erase(active.begin() + i);
                    changed = true;
                } else {
                    i++;
                }
            if (in_phase) {
                size_t used = 0;
                for (auto &j : active) used += j->bytes;
                while (!pending.empty() && (active.empty() || used + pending.front()->bytes <= budget)) {
                    used += pending.front()->bytes;
                    active.push_back(std::move(pending.front()));
                    pending.pop_front();
                    changed = true;
                }
            }
            if (!busy) t_busy_from = now_s();
            busy = true;
            st.max_active = std::max<uint32_t>(st.max_active, (uint32_t)active.size());
        }
        // (the callbacks still owed read the pinned snapshot buffer of the previous epoch,
        // which neither the re-pack nor the next epoch touches: they run below, while the next
        // epoch computes; the re-pack itself waits for the snapshot copies out of the arena)
        int rc = repack();
        if (rc != PDPD_OK) {
            std::vector<ServerJob *> all;
            for (auto &j : active) all.push_back(j.get());
            fail_jobs(all, rc);
            pdpd_attach(eng, nullptr);
            changed = false;
        }
        std::vector<Delivery> next;
        uint32_t epoch = UINT32_MAX;
        for (auto &j : active)
            if (!j->ended) epoch = std::min({epoch, interval - j->done % interval, j->n_steps - j->done});
        if (epoch == UINT32_MAX) epoch = 0;  // only ended jobs: they leave at the next iteration
        const double t_epoch0 = now_s();
        if (epoch > 0) {
            if (t_sync_end > 0) {  // host time between the previous epoch's end and this launch
                std::lock_guard<std::mutex> lk(mu);
                st.host_gap_s += std::max(0.0, t_epoch0 - t_sync_end - waited);
            }
            cudaEventRecord(ev_step0, eng->stream);
            rc = pdpd_run_async(eng, epoch);
            cudaEventRecord(ev_step1[end_k ^ 1], eng->stream);
            std::vector<size_t> at_boundary;
            for (size_t i = 0; i < active.size(); i++) {
                ServerJob &j = *active[i];
                if (j.ended) continue;
                j.done += epoch;
                j.t += epoch;
                if (j.done % interval == 0 || j.done == j.n_steps) at_boundary.push_back(i);
            }
            if (rc == PDPD_OK && !at_boundary.empty()) {
                // Snapshot b: the arena (or its worlds at a boundary) unsorted into device staging
                // buffer b and copied from there to pinned buffer b on the side stream.  The last
                // copy that read either buffer b is the one of two snapshots ago: once it is
                // done, the unsort needs no wait on the copy still running out of the other pair
                // (a job ending a few steps after an interval boundary would otherwise hold the
                // GPU until the whole interval snapshot had crossed to the host).
                {
                    const double t_c0 = now_s();
                    cudaEventSynchronize(ev_copied[b]);  // (normally long done)
                    std::lock_guard<std::mutex> lk(mu);
                    st.copy_wait_s += now_s() - t_c0;
                }
                {
                    // (reserved at creation for a batch that fills the budget; a job larger
                    // than the budget, which runs alone, may need more)
                    const double t_a0 = now_s();
                    const size_t need = sizeof(double) * 9 * (size_t)eng->n_beads;
                    if (need > snap[b].bytes && snap[b].alloc(need, true) != cudaSuccess)
                        rc = eng->fail(PDPD_E_NOMEM, "pinned snapshot allocation failed");
                    std::lock_guard<std::mutex> lk(mu);
                    st.snap_alloc_s += now_s() - t_a0;
                }
                // unsort the arena, or only the worlds at a boundary when they are few (a job
                // ending mid-interval splits an epoch for its own snapshot)
                if (rc == PDPD_OK && at_boundary.size() * 4 >= active.size()) rc = download(eng, b, eng->stream);
                else
                    for (size_t i : at_boundary)
                        if (rc == PDPD_OK) rc = download_world(eng, b, active[i]->slot, eng->stream);
                if (rc == PDPD_OK) {
                    cudaEventRecord(ev_unsorted, eng->stream);
                    cudaStreamWaitEvent(eng->side, ev_unsorted, 0);
                    for (size_t i : at_boundary) {
                        ServerJob &j = *active[i];
                        const WorldDev &wd = eng->worlds[j.slot].dev;
                        const size_t row = 9 * (size_t)wd.bead_base;
                        if (wd.n_beads)
                            cudaMemcpyAsync((double *)snap[b].p + row, eng->d_staging[b].as<double>() + row,
                                            sizeof(double) * 9 * wd.n_beads, cudaMemcpyDeviceToHost, eng->side);
                        next.push_back({&j, row, wd.n_beads, j.t, j.done == j.n_steps ? 1 : 0});
                    }
                    cudaEventRecord(ev_copied[b], eng->side);
                }
            }
        }
        if (epoch > 0) {
            std::lock_guard<std::mutex> lk(mu);
            st.post_launch_s += now_s() - t_epoch0;
        }
        {
            const double t_cb0 = now_s();
            deliver();  // host callbacks of the previous epoch while this one computes
            std::lock_guard<std::mutex> lk(mu);
            st.callback_s += now_s() - t_cb0;
        }
        if (epoch > 0) {
            const double t_s0 = now_s();
            if (rc == PDPD_OK) rc = pdpd_sync(eng);
            t_sync_end = now_s();
            {
                std::lock_guard<std::mutex> lk(mu);
                st.sync_wait_s += t_sync_end - t_s0;
            }
            if (rc == PDPD_E_BOND_SNAPPED || rc == PDPD_E_BEAD_LOST) {
                // worlds are independent: fail the ones that raised an error flag, keep the rest
                const WorldDev *wd = (const WorldDev *)eng->h_err.p;
                std::vector<ServerJob *> bad;
                for (auto &j : active)
                    if (wd[j->slot].err) bad.push_back(j.get());
                fail_jobs(bad, rc);
                next.erase(std::remove_if(next.begin(), next.end(),
                                          [](const Delivery &d) { return d.job->stopped; }),
                           next.end());
                rc = PDPD_OK;
            } else if (rc != PDPD_OK) {
                std::vector<ServerJob *> all;
                for (auto &j : active) all.push_back(j.get());
                fail_jobs(all, rc);
                next.clear();
                cudaStreamSynchronize(eng->side);
                pdpd_attach(eng, nullptr);
                changed = false;
            }
            uint64_t stepped = 0, live_phase = 0;
            float step_ms = 0.f;
            float between_ms = 0.f;
            if (rc == PDPD_OK && cudaEventElapsedTime(&step_ms, ev_step0, ev_step1[end_k ^ 1]) != cudaSuccess) step_ms = 0.f;
            if (rc == PDPD_OK && have_end &&
                cudaEventElapsedTime(&between_ms, ev_step1[end_k], ev_step0) != cudaSuccess)
                between_ms = 0.f;
            end_k ^= 1;
            have_end = rc == PDPD_OK;
            {
                std::lock_guard<std::mutex> lk(mu);
                st.step_s += 1e-3 * step_ms;
                st.between_s += 1e-3 * between_ms;
                st.epochs++;
                for (auto &j : active) {
                    stepped += (uint64_t)j->desc.n_beads * epoch;
                    if (!j->ended) st.bead_steps += (uint64_t)j->desc.n_beads * epoch;
                    else st.wasted_bead_steps += (uint64_t)j->desc.n_beads * epoch;
                }
            }
            const double dt_epoch = now_s() - t_epoch0;
            if (stepped && dt_epoch > 0) rate_est = 0.7 * rate_est + 0.3 * (double)stepped / dt_epoch;
            for (auto &j : active) {
                if (j->done == j->n_steps) j->ended = true;  // final state is owed
                if (!j->ended) live_phase = j->done % interval;
            }
            // Ended worlds step on until the live jobs reach their next interval boundary; when
            // that costs more than an early re-pack, they leave at once.
            uint64_t zombie = 0;
            const uint64_t rem = live_phase ? interval - live_phase : 0;
            for (auto &j : active)
                if (j->ended) zombie += (uint64_t)j->desc.n_beads * rem;
            if (zombie && (double)zombie / rate_est > repack_est_s)
                for (auto &j : active)
                    if (j->ended) j->leave_now = true;
            owed.swap(next);
            owed_buf = b;
            b ^= 1;
        }
        if (active.empty() && owed.empty()) {
            have_end = false;  // idle: the next epoch's distance from the last is not overhead
            repack();  // releases the arena
            std::lock_guard<std::mutex> lk(mu);
            if (busy) st.busy_s += now_s() - t_busy_from;
            busy = false;
            if (pending.empty()) cv_idle.notify_all();
        }
    }
}

extern "C" {

int pdpd_server_create(int precision, int device, size_t memory_budget_bytes, uint32_t interval_steps,
                       pdpd_server **out)
{
    if (!out) return PDPD_E_INVALID;
    *out = nullptr;
    if (interval_steps == 0) {
        g_last_error = "interval_steps must be at least 1";
        return PDPD_E_INVALID;
    }
    pdpd_engine *e = nullptr;
    int rc = pdpd_create(precision, device, &e);
    if (rc) return rc;
    pdpd_server *s = new pdpd_server();
    s->eng = e;
    s->precision = precision;
    s->budget = memory_budget_bytes;
    s->interval = interval_steps;
    cudaSetDevice(e->device);
    cudaEventCreateWithFlags(&s->ev_unsorted, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&s->ev_copied[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&s->ev_copied[1], cudaEventDisableTiming);
    cudaEventCreate(&s->ev_step0);
    cudaEventCreate(&s->ev_step1[0]);
    cudaEventCreate(&s->ev_step1[1]);
    // The two pinned snapshot buffers, reserved for the rows (x, v, f as doubles) of a batch
    // that fills the budget, at most 16 GiB each.  Pinning host memory is slow: in a 20 s
    // stream whose batch grew to the budget, buffers re-pinned as they grew (by half, then by
    // 4x) held the GPU idle for 7%, then 4.5% of the wall time.
    const size_t per_bead = precision == PDPD_FP64 ? 424 : 296;  // as job_bytes
    const size_t full = std::min<size_t>(sizeof(double) * 9 * (memory_budget_bytes / per_bead), size_t(16) << 30);
    for (HostPinned &h : s->snap)
        if (h.alloc(std::max<size_t>(full, 4096), true) != cudaSuccess) {
            g_last_error = "pinned snapshot buffers: allocation failed";
            for (cudaEvent_t ev : {s->ev_unsorted, s->ev_copied[0], s->ev_copied[1], s->ev_step0, s->ev_step1[0],
                                   s->ev_step1[1]})
                cudaEventDestroy(ev);
            for (HostPinned &x : s->snap) x.release();
            pdpd_destroy(e);
            delete s;
            return PDPD_E_NOMEM;
        }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return PDPD_OK;
}

int pdpd_server_config(pdpd_server *s, const char *key, const char *value)
{
    if (!s) return PDPD_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);  // the worker touches the engine only while busy
    if (!s->pending.empty() || s->busy) {
        g_last_error = "the server is running jobs: drain it before changing its configuration";
        return PDPD_E_STATE;
    }
    int rc = pdpd_set_config(s->eng, key, value);
    if (rc) g_last_error = s->eng->err;
    return rc;
}

int pdpd_server_submit(pdpd_server *s, const pdpd_world *w, uint32_t n_steps, pdpd_job_fn cb, void *user,
                       uint64_t *job_id)
{
    if (job_id) *job_id = 0;
    if (!s || !w) return PDPD_E_INVALID;
    char reason[256];
    int rc = check_world(w, reason, sizeof reason);
    if (rc) {
        g_last_error = reason;
        return rc;
    }
    auto j = std::make_unique<ServerJob>();
    const uint32_t nt = w->n_bead_types, n = w->n_beads;
    j->cons.assign(w->conservative, w->conservative + nt * nt);
    j->diss.assign(w->dissipative, w->dissipative + nt * nt);
    j->stat.assign(nt, 0);
    if (w->stationary) j->stat.assign(w->stationary, w->stationary + nt);
    j->hash.assign(w->hash, w->hash + n);
    j->x.resize(3 * (size_t)n);
    j->v.resize(3 * (size_t)n);
    j->f.resize(3 * (size_t)n);
    for (uint32_t k = 0; k < n; k++)
        for (int d = 0; d < 3; d++) {
            j->x[3 * (size_t)k + d] = vec_at(w->x, w->bead_stride_bytes, k)[d];
            j->v[3 * (size_t)k + d] = vec_at(w->v, w->bead_stride_bytes, k)[d];
            j->f[3 * (size_t)k + d] = vec_at(w->f, w->bead_stride_bytes, k)[d];
        }
    if (w->n_bonds) {
        j->bb.assign(w->bond_beads, w->bond_beads + 2 * (size_t)w->n_bonds);
        j->bk.assign(w->bond_kappa, w->bond_kappa + w->n_bonds);
        j->br.assign(w->bond_r0, w->bond_r0 + w->n_bonds);
    }
    if (w->cell_conservative) {
        const size_t nv = (size_t)w->box[0] * w->box[1] * w->box[2] * nt * nt;
        j->cell_a.assign(w->cell_conservative, w->cell_conservative + nv);
        j->cell_g.assign(w->cell_dissipative, w->cell_dissipative + nv);
    }
    if (w->n_angles) {
        j->ab.assign(w->angle_beads, w->angle_beads + 3 * (size_t)w->n_angles);
        j->ak.assign(w->angle_kappa, w->angle_kappa + w->n_angles);
        j->at.assign(w->angle_theta0, w->angle_theta0 + w->n_angles);
    }
    pdpd_world &d = j->desc;
    d = *w;
    d.conservative = j->cons.data();
    d.dissipative = j->diss.data();
    d.stationary = j->stat.data();
    d.hash = j->hash.data();
    d.x = j->x.data();
    d.v = j->v.data();
    d.f = j->f.data();
    d.bead_stride_bytes = 0;
    d.bond_beads = j->bb.data();
    d.bond_kappa = j->bk.data();
    d.bond_r0 = j->br.data();
    d.angle_beads = j->ab.data();
    d.angle_kappa = j->ak.data();
    d.angle_theta0 = j->at.data();
    d.cell_conservative = w->cell_conservative ? j->cell_a.data() : nullptr;
    d.cell_dissipative = w->cell_conservative ? j->cell_g.data() : nullptr;
    j->n_steps = n_steps;
    j->t = w->t;
    j->cb = cb;
    j->user = user;
    j->bytes = job_bytes(*w, s->precision);
    j->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        j->id = s->next_id++;
        if (job_id) *job_id = j->id;
        if (s->t_first < 0) s->t_first = j->t_submit;
        s->st.jobs_submitted++;
        if (n_steps > 0) {
            s->pending.push_back(std::move(j));
            s->cv.notify_all();
            return PDPD_OK;
        }
        s->st.jobs_done++;
        s->latencies.push_back(0.0);
        s->t_last = now_s();
    }
    // nothing to run: the final state is the initial one
    if (cb) cb(user, j->id, w->t, j->x.data(), j->v.data(), j->f.data(), 3 * sizeof(double), n, 1);
    return PDPD_OK;
}

int pdpd_server_drain(pdpd_server *s)
{
    if (!s) return PDPD_E_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_idle.wait(lk, [&] { return s->pending.empty() && !s->busy; });
    int rc = s->status;
    if (rc) g_last_error = s->err;
    s->status = PDPD_OK;
    return rc;
}

int pdpd_server_stats_get(pdpd_server *s, pdpd_server_stats *out)
{
    if (!s || !out) return PDPD_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) {
        return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)std::ceil(p * l.size()) - (p > 0 ? 1 : 0))];
    };
    out->latency_p50_s = pct(0.50);
    out->latency_p99_s = pct(0.99);
    out->latency_max_s = l.empty() ? 0.0 : l.back();
    out->wall_s = s->t_first < 0 ? 0.0 : s->t_last - s->t_first;
    if (s->busy) out->busy_s += now_s() - s->t_busy_from;
    return PDPD_OK;
}

pdpd_engine *pdpd_server_engine(pdpd_server *s)
{
    return s ? s->eng : nullptr;
}

void pdpd_server_destroy(pdpd_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->eng->device);
    cudaStreamSynchronize(s->eng->side);
    if (s->ev_unsorted) cudaEventDestroy(s->ev_unsorted);
    if (s->ev_step0) cudaEventDestroy(s->ev_step0);
    for (cudaEvent_t ev : s->ev_step1)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : s->ev_copied)
        if (ev) cudaEventDestroy(ev);
    s->snap[0].release();
    s->snap[1].release();
    pdpd_destroy(s->eng);
    delete s;
}

}  // extern "C"
