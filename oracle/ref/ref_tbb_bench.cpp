// Baseline infrastructure: times the reference's own TBB engines, compiled unchanged from the
// reference headers with the reference's release flags and the project's TBB stand-in
// (tbb_shim/), on worlds stored in the PDW1 file format.  Only oracle/ref/calibrate.py runs
// it, in a container where the reference sources are present.
//
//   ref_tbb_bench <engine|auto> <min_seconds> <start_steps> <in1.pdw1> [<in2.pdw1> ...]
//   ref_tbb_bench check <engine|auto> <in.pdw1> <steps> <out.bin>
//       Attach + Run(steps) and dump t, then x, v, f of every bead (9 doubles per bead): the
//       check that the engine computes the same trajectory through the TBB stand-in.
//
// Engines: naive_dpd_engine_half_merge_tbb (naive_dpd_engine_half_merge_tbb.hpp; box sides
// multiples of 4), naive_dpd_engine_half_step_tbb (naive_dpd_engine_half_step_tbb.hpp; any
// side >= 2), or "auto": half_merge_tbb for a world whose sides are all multiples of 4, else
// half_step_tbb -- the choice the reference's own engines force (half_merge rejects other
// sides, naive_dpd_engine_half_merge.hpp:47-57).
//
// Timing follows the reference's benchmark_engine.cpp:127-158: Attach, then Run(k) with k
// growing by 1.5x until the rate changed by less than 5% and the round took longer than
// min_seconds.  A step here is one step of every world in turn (each has its own engine),
// so bead-steps/s = sum of beads x k / the summed seconds of the Run calls.  Engines are
// never detached (NaiveDPDEngineHalfMergeTBB::Attach runs CanSupport on its argument, which
// must not be null), as in benchmark_engine.cpp.  Prints one JSON
// line per round and a final one with "final": true.

#include "dpd/core/dpd_engine.hpp"
#include "dpd/core/logging.hpp"
#include "dpd/core/logging_impl.hpp"
#include "dpd/engines/naive/naive_dpd_engine_half_merge_tbb.hpp"
#include "dpd/engines/naive/naive_dpd_engine_half_step_tbb.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pdw1_read.hpp"

namespace {

double now()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool sides_by4(const WorldState &s)
{
    for (int d = 0; d < 3; d++)
        if (((long)std::lround(s.box[d])) % 4 != 0) return false;
    return true;
}

std::shared_ptr<DPDEngine> make_engine(const std::string &name, const WorldState &s)
{
    std::string n = name;
    if (n == "auto") {
        const bool by4 = sides_by4(s);
        n = by4 ? "naive_dpd_engine_half_merge_tbb" : "naive_dpd_engine_half_step_tbb";
    }
    if (n == "naive_dpd_engine_half_merge_tbb") return std::make_shared<NaiveDPDEngineHalfMergeTBB>();
    if (n == "naive_dpd_engine_half_step_tbb") return std::make_shared<NaiveDPDEngineHalfStepTBB>();
    throw std::runtime_error("unknown engine " + name);
}

}  // namespace

int check(int argc, char **argv)
{
    if (argc != 6) {
        fprintf(stderr, "usage: ref_tbb_bench check <engine|auto> <in.pdw1> <steps> <out.bin>\n");
        return 2;
    }
    WorldState s = pdw1::read_pdw1(argv[3]);
    auto e = make_engine(argv[2], s);
    e->Attach(&s);
    e->Run(atoi(argv[4]));
    FILE *out = fopen(argv[5], "wb");
    if (!out) throw std::runtime_error("cannot write output");
    const int64_t t = s.t;
    fwrite(&t, sizeof t, 1, out);
    for (const Bead &b : s.beads) {
        double rec[9];
        for (int d = 0; d < 3; d++) {
            rec[d] = b.x[d];
            rec[3 + d] = b.v[d];
            rec[6 + d] = b.f[d];
        }
        fwrite(rec, sizeof(double), 9, out);
    }
    fclose(out);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc >= 2 && std::string(argv[1]) == "check") {
        try {
            return check(argc, argv);
        } catch (const std::exception &e) {
            fprintf(stderr, "ref_tbb_bench: %s\n", e.what());
            return 1;
        }
    }
    if (argc < 5) {
        fprintf(stderr, "usage: ref_tbb_bench <engine|auto> <min_seconds> <start_steps> <in.pdw1>...\n");
        return 2;
    }
    try {
        const std::string engine_name = argv[1];
        const double min_seconds = atof(argv[2]);
        int todo = std::max(1, atoi(argv[3]));
        std::vector<WorldState> states;
        std::vector<std::shared_ptr<DPDEngine>> engines;
        std::string used;
        double beads = 0;
        for (int k = 4; k < argc; k++) {
            states.push_back(pdw1::read_pdw1(argv[k]));
        }
        for (auto &s : states) {
            engines.push_back(make_engine(engine_name, s));
            beads += (double)s.beads.size();
            const bool by4 = sides_by4(s);
            used += std::string(used.empty() ? "" : ",") +
                    (engine_name != "auto" ? engine_name
                                           : (by4 ? "half_merge_tbb" : "half_step_tbb"));
        }
        double prev = 0;
        for (int round = 0; round < 64; round++) {
            double run_s = 0, t0 = now();
            for (size_t w = 0; w < states.size(); w++) {
                engines[w]->Attach(&states[w]);
                const double a = now();
                engines[w]->Run(todo);
                run_s += now() - a;
            }
            const double wall = now() - t0;
            const double rate = beads * todo / run_s;
            const bool stable = prev > 0 && wall > min_seconds && std::fabs(rate - prev) / prev < 0.05;
            printf("{\"engines\": \"%s\", \"beads\": %.0f, \"steps\": %d, \"run_s\": %.6f, "
                   "\"rate\": %.6g, \"final\": %s}\n",
                   used.c_str(), beads, todo, run_s, rate, stable ? "true" : "false");
            fflush(stdout);
            if (stable) return 0;
            prev = rate;
            todo = std::max(2, todo * 3 / 2);
        }
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_tbb_bench: %s\n", e.what());
        return 1;
    }
}
