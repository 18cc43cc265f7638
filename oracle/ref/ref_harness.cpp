// Test infrastructure: drives the reference's own engines, compiled unchanged from the
// reference headers, on worlds stored in the PDW1 file format (pdw1_read.hpp).
// Only the fixture generator (tests/golden/make_golden.py) runs this program, and only
// in a container where the reference sources are present.
//
//   ref_harness step  <engine> <in.pdw1> <out.bin> <n_checkpoints> <steps_1> ... <steps_n>
//       Attach + Run(steps_k - steps_{k-1}) and dump (t, x, v, f of every bead) at each
//       checkpoint.  Engines: naive_dpd_engine_half_step (include/dpd/engines/naive/
//       naive_dpd_engine_half_step.hpp:42), naive_dpd_engine_half_merge
//       (naive_dpd_engine_half_merge.hpp) and naive_dpd_engine (NaiveDPDEngine<false>,
//       naive_dpd_engine.hpp).
//   ref_harness hash  <in.bin> <out.bin>
//       For each record (uint32 t, uint64 seed, uint32 a, uint32 b) write get_t_hash
//       (hash.hpp:61-65), hash_rng_sym (hash.hpp:81-88) and dpd_maths_core::default_hash
//       (dpd_maths_core.hpp:55-79).
//   ref_harness cansupport <engine> <in.pdw1>
//       Print the engine's CanSupport() string.
//   ref_harness time <engine> <in.pdw1> <steps>
//       Attach + Run(steps), print bead-steps/s of the Run call.
//   ref_harness v2binary <in.pdw1> <out.bin>
//       write_world_state(binary=true) (dpd_state_io.hpp:408-466): the reference's own
//       v2binary snapshot of the world as read.
//   ref_harness stepx <engine> <in.pdw1> <exprs.txt> <out.bin> <n_checkpoints> <steps...>
//       As step, with the interaction strengths replaced by Parameter expressions read from
//       exprs.txt (n^2 conservative lines, then n^2 dissipative lines, row-major) -- the
//       reference's spatially varying DPD parameters (expression.hpp:328-431).
//   ref_harness tables <in.pdw1> <exprs.txt> <out.bin>
//       The per-cell values of those expressions, evaluated as the half-merge engine does at
//       Attach (naive_dpd_engine_half_merge.hpp:221-236: x, y, z = cell coordinates,
//       ux = (x + 0.5) / Lx, ...): for each cell (x-major, z fastest) n^2 conservative then
//       n^2 dissipative doubles.
//   ref_harness v2read <in.v2> <out.bin>
//       read_world_state (dpd_state_io.hpp:481-586) of a v2binary file; dump t, x, v, f.
//   ref_harness pairlog <engine> <in.pdw1> <out.bin> <steps> <n_ids> <id...>
//       Attach + Run(steps) with a ForceLogging logger installed (logging.hpp:9-30): every
//       LogBeadPairProperty call whose home bead is one of the listed bead ids, as the
//       engine's calc_force makes them (dpd_maths_core_half_step.hpp:131-153), recorded at
//       full precision: (int64 t, uint32 home hash, uint32 other hash, char name[24],
//       int32 dims, double value[3]) per call.

#include "dpd/core/dpd_engine.hpp"
#include "dpd/core/dpd_state_validator.hpp"
#include "dpd/core/logging.hpp"
#include "dpd/core/logging_impl.hpp"
#include "dpd/core/dpd_state_io.hpp"
#include "dpd/engines/naive/naive_dpd_engine.hpp"
#include "dpd/engines/naive/naive_dpd_engine_half_step.hpp"
#include "dpd/engines/naive/naive_dpd_engine_half_merge.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "pdw1_read.hpp"

using pdw1::read_pdw1;
using pdw1::Reader;

namespace {

std::shared_ptr<DPDEngine> make_engine(const std::string &name)
{
    if (name == "naive_dpd_engine_half_step") return std::make_shared<NaiveDPDEngineHalfStep>();
    if (name == "naive_dpd_engine_half_merge") return std::make_shared<NaiveDPDEngineHalfMerge>();
    if (name == "naive_dpd_engine") return std::make_shared<NaiveDPDEngine<false>>();
    throw std::runtime_error("unknown engine " + name);
}

void dump(FILE *out, const WorldState &s)
{
    int64_t t = s.t;
    fwrite(&t, sizeof(t), 1, out);
    uint32_t n = s.beads.size();
    fwrite(&n, sizeof(n), 1, out);
    for (const Bead &b : s.beads) {
        double rec[9];
        for (int d = 0; d < 3; d++) { rec[d] = b.x[d]; rec[3 + d] = b.v[d]; rec[6 + d] = b.f[d]; }
        fwrite(rec, sizeof(double), 9, out);
    }
}

int cmd_step(int argc, char **argv)
{
    if (argc < 6) throw std::runtime_error("usage: step engine in out n steps...");
    std::string engine_name = argv[2];
    WorldState s = read_pdw1(argv[3]);
    FILE *out = fopen(argv[4], "wb");
    if (!out) throw std::runtime_error("cannot open output");
    unsigned n = atoi(argv[5]);
    auto e = make_engine(engine_name);
    std::string why = e->CanSupport(&s);
    if (!why.empty()) throw std::runtime_error("CanSupport: " + why);
    e->Attach(&s);
    unsigned done = 0;
    for (unsigned k = 0; k < n; k++) {
        unsigned target = atoi(argv[6 + k]);
        if (target > done) e->Run(target - done);
        done = target;
        dump(out, s);
    }
    fclose(out);
    return 0;
}

// A ForceLogging logger that keeps the pair properties of chosen home beads, full precision.
class PairRecorder : public ForceLogging
{
public:
    std::vector<uint32_t> homes;  // full hashes of the chosen home beads
    FILE *out = nullptr;
    long t = 0;
    void Flush() override {}
    void SetTime(long tt) override { t = tt; }
    void SetPrefix(const std::string &) override {}
    void LogProperty(const char *, int, const double *) override {}
    void LogBeadProperty(BeadHash, const char *, int, const double *) override {}
    void LogBeadTripleProperty(BeadHash, BeadHash, BeadHash, const char *, int, const double *) override {}
    void LogBeadPairProperty(BeadHash b0, BeadHash b1, const char *name, int dims, const double *x) override
    {
        if (std::find(homes.begin(), homes.end(), b0.hash) == homes.end()) return;
        int64_t tt = t;
        uint32_t h[2] = {b0.hash, b1.hash};
        char nm[24] = {0};
        strncpy(nm, name, sizeof nm - 1);
        int32_t d = dims;
        double v[3] = {0, 0, 0};
        for (int i = 0; i < dims && i < 3; i++) v[i] = x[i];
        fwrite(&tt, sizeof tt, 1, out);
        fwrite(h, sizeof h, 1, out);
        fwrite(nm, 1, sizeof nm, out);
        fwrite(&d, sizeof d, 1, out);
        fwrite(v, sizeof v, 1, out);
    }
};

int cmd_pairlog(int argc, char **argv)
{
    if (argc < 7) throw std::runtime_error("usage: pairlog engine in out steps n_ids ids...");
    WorldState s = read_pdw1(argv[3]);
    PairRecorder rec;
    rec.out = fopen(argv[4], "wb");
    if (!rec.out) throw std::runtime_error("cannot open output");
    const unsigned steps = atoi(argv[5]), n_ids = atoi(argv[6]);
    if (argc < 7 + (int)n_ids) throw std::runtime_error("pairlog: missing bead ids");
    for (unsigned k = 0; k < n_ids; k++) rec.homes.push_back(s.beads.at(atoi(argv[7 + k])).get_hash_code().hash);
    auto e = make_engine(argv[2]);
    std::string why = e->CanSupport(&s);
    if (!why.empty()) throw std::runtime_error("CanSupport: " + why);
    e->Attach(&s);
    ForceLogging::set_logger(&rec);
    e->Run(steps);
    ForceLogging::set_logger(nullptr);
    fclose(rec.out);
    return 0;
}

int cmd_hash(int argc, char **argv)
{
    Reader r(argv[2]);
    FILE *out = fopen(argv[3], "wb");
    if (!out) throw std::runtime_error("cannot open output");
    while (true) {
        uint32_t t;
        if (fread(&t, 4, 1, r.f) != 1) break;
        uint64_t seed = r.get<uint64_t>();
        uint32_t a = r.get<uint32_t>();
        uint32_t b = r.get<uint32_t>();
        uint64_t th = get_t_hash(t, seed);
        uint32_t h = hash_rng_sym(th, a, b);
        float u = dpd_maths_core::default_hash(th, a, b);
        fwrite(&th, 8, 1, out);
        fwrite(&h, 4, 1, out);
        fwrite(&u, 4, 1, out);
    }
    fclose(out);
    return 0;
}

int cmd_cansupport(int argc, char **argv)
{
    WorldState s = read_pdw1(argv[3]);
    auto e = make_engine(argv[2]);
    printf("%s\n", e->CanSupport(&s).c_str());
    return 0;
}

int cmd_time(int argc, char **argv)
{
    WorldState s = read_pdw1(argv[3]);
    unsigned steps = atoi(argv[4]);
    auto e = make_engine(argv[2]);
    e->Attach(&s);
    auto t0 = std::chrono::steady_clock::now();
    e->Run(steps);
    auto t1 = std::chrono::steady_clock::now();
    double sec = std::chrono::duration<double>(t1 - t0).count();
    printf("%.6e\n", double(s.beads.size()) * steps / sec);
    return 0;
}

int cmd_v2binary(int argc, char **argv)
{
    if (argc < 4) throw std::runtime_error("usage: v2binary in out");
    WorldState s = read_pdw1(argv[2]);
    std::ofstream out(argv[3], std::ios::binary);
    if (!out) throw std::runtime_error("cannot open output");
    write_world_state(out, s, true);
    return 0;
}

void load_exprs(WorldState &s, const char *path)
{
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open expressions");
    const size_t n2 = s.interactions.size();
    std::vector<std::string> lines;
    std::string line;
    while (std::getline(in, line))
        if (!line.empty()) lines.push_back(line);
    if (lines.size() != 2 * n2) throw std::runtime_error("expression file needs 2 n^2 lines");
    for (size_t k = 0; k < n2; k++) {
        s.interactions[k].conservative = Parameter(lines[k]);
        s.interactions[k].dissipative = Parameter(lines[n2 + k]);
    }
}

int cmd_stepx(int argc, char **argv)
{
    if (argc < 7) throw std::runtime_error("usage: stepx engine in exprs out n steps...");
    std::string engine_name = argv[2];
    WorldState s = read_pdw1(argv[3]);
    load_exprs(s, argv[4]);
    FILE *out = fopen(argv[5], "wb");
    if (!out) throw std::runtime_error("cannot open output");
    unsigned n = atoi(argv[6]);
    auto e = make_engine(engine_name);
    std::string why = e->CanSupport(&s);
    if (!why.empty()) throw std::runtime_error("CanSupport: " + why);
    e->Attach(&s);
    unsigned done = 0;
    for (unsigned k = 0; k < n; k++) {
        unsigned target = atoi(argv[7 + k]);
        if (target > done) e->Run(target - done);
        done = target;
        dump(out, s);
    }
    fclose(out);
    return 0;
}

int cmd_tables(int argc, char **argv)
{
    if (argc < 5) throw std::runtime_error("usage: tables in exprs out");
    WorldState s = read_pdw1(argv[2]);
    load_exprs(s, argv[3]);
    FILE *out = fopen(argv[4], "wb");
    if (!out) throw std::runtime_error("cannot open output");
    const int L[3] = {(int)s.box[0], (int)s.box[1], (int)s.box[2]};
    for (int x = 0; x < L[0]; x++)
        for (int y = 0; y < L[1]; y++)
            for (int z = 0; z < L[2]; z++) {
                std::unordered_map<std::string, double> b;
                b["x"] = x;
                b["y"] = y;
                b["z"] = z;
                b["ux"] = (x + 0.5) / s.box[0];
                b["uy"] = (y + 0.5) / s.box[1];
                b["uz"] = (z + 0.5) / s.box[2];
                for (auto &ii : s.interactions) {
                    double a = ii.conservative.evaluate(b);
                    fwrite(&a, 8, 1, out);
                }
                for (auto &ii : s.interactions) {
                    double g = ii.dissipative.evaluate(b);
                    fwrite(&g, 8, 1, out);
                }
            }
    fclose(out);
    return 0;
}

int cmd_v2read(int argc, char **argv)
{
    if (argc < 4) throw std::runtime_error("usage: v2read in out");
    WorldState s = read_world_state(std::string(argv[2]));
    FILE *out = fopen(argv[3], "wb");
    if (!out) throw std::runtime_error("cannot open output");
    dump(out, s);
    fclose(out);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    try {
        if (argc < 2) throw std::runtime_error("usage: ref_harness step|hash|cansupport|time ...");
        std::string cmd = argv[1];
        if (cmd == "step") return cmd_step(argc, argv);
        if (cmd == "hash") return cmd_hash(argc, argv);
        if (cmd == "cansupport") return cmd_cansupport(argc, argv);
        if (cmd == "time") return cmd_time(argc, argv);
        if (cmd == "v2binary") return cmd_v2binary(argc, argv);
        if (cmd == "v2read") return cmd_v2read(argc, argv);
        if (cmd == "stepx") return cmd_stepx(argc, argv);
        if (cmd == "tables") return cmd_tables(argc, argv);
        if (cmd == "pairlog") return cmd_pairlog(argc, argv);
        throw std::runtime_error("unknown command " + cmd);
    } catch (std::exception &e) {
        fprintf(stderr, "ref_harness: %s\n", e.what());
        return 1;
    } catch (std::string &e) {
        fprintf(stderr, "ref_harness: %s\n", e.c_str());
        return 1;
    }
}
