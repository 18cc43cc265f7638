// Test infrastructure: exports the reference's own engine test suite (the TestBase families
// registered by the reference's src/test/test_engine.cpp) as replayable golden segments.
//
// For each registered test, the test's world is created and driven exactly as the
// reference's test_runner does (include/dpd/tests/test_runner.hpp:8-60) with the reference's
// NaiveDPDEngineHalfStep: todo = test.get_advance_count(state) (which checks the test's
// physical properties and may modify the state), then engine.Run(todo).  Each segment's input
// state (after get_advance_count) and output state are recorded, so another engine can replay
// the segment from the identical input and be compared with the reference's output.
//
//   testbase_export <out.bin> [max_segments_per_test]
//
// Output format (little endian):
//   u32 n_tests; per test: u32 name_len, name bytes, u32 verdict (1 = ok), u32 pdw1_len,
//   PDW1 bytes of the initial world, u32 n_segments; per segment: u32 todo, i64 t_in,
//   f64[n*9] (x v f in), i64 t_out, f64[n*9] (x v f out).
#include "dpd/core/dpd_engine.hpp"
#include "dpd/core/dpd_state_validator.hpp"
#include "dpd/core/logging.hpp"
#include "dpd/core/logging_impl.hpp"
#include "dpd/engines/naive/naive_dpd_engine_half_step.hpp"
#include "dpd/tests/test_bonded_bead_angle.hpp"
#include "dpd/tests/test_bonded_bead_pair.hpp"
#include "dpd/tests/test_bonded_bead_triple.hpp"
#include "dpd/tests/test_colliding_bead_pair.hpp"
#include "dpd/tests/test_colliding_bead_pair_diss.hpp"
#include "dpd/tests/test_isolated_moving_bead.hpp"
#include "dpd/tests/test_multiple_moving_beads.hpp"
#include "dpd/tests/test_ordered_mesh.hpp"

#include <cstdio>
#include <string>
#include <vector>

namespace {

struct Out {
    std::vector<unsigned char> buf;
    template <class T> void put(const T &v)
    {
        const unsigned char *p = (const unsigned char *)&v;
        buf.insert(buf.end(), p, p + sizeof(T));
    }
    void bytes(const void *p, size_t n)
    {
        buf.insert(buf.end(), (const unsigned char *)p, (const unsigned char *)p + n);
    }
};

// PDW1: the same layout poets-dpd_gb300/pdpd_world.py writes and pdw1_read.hpp reads.
void put_pdw1(Out &o, const WorldState &s)
{
    o.bytes("PDW1", 4);
    for (int i = 0; i < 3; i++) o.put<int32_t>((int32_t)s.box[i]);
    o.put<double>(s.dt);
    o.put<double>(s.lambda);
    o.put<uint64_t>(s.seed);
    o.put<int64_t>(s.t);
    uint32_t nt = s.bead_types.size();
    o.put<uint32_t>(nt);
    for (const auto &bt : s.bead_types) o.put<uint32_t>(bt.stationary ? 1 : 0);
    for (const auto &ii : s.interactions) o.put<double>((double)ii.conservative);
    for (const auto &ii : s.interactions) o.put<double>((double)ii.dissipative);
    o.put<uint32_t>(s.polymer_types.size());
    for (const auto &pt : s.polymer_types) {
        o.put<uint32_t>(pt.bead_types.size());
        for (auto b : pt.bead_types) o.put<uint32_t>(b);
        o.put<uint32_t>(pt.bonds.size());
        for (const auto &b : pt.bonds) {
            o.put<uint32_t>(b.bead_offset_head);
            o.put<uint32_t>(b.bead_offset_tail);
            o.put<double>((double)b.kappa);
            o.put<double>((double)b.r0);
        }
        o.put<uint32_t>(pt.bond_pairs.size());
        for (const auto &bp : pt.bond_pairs) {
            o.put<uint32_t>(bp.bond_offset_head);
            o.put<uint32_t>(bp.bond_offset_tail);
            o.put<double>((double)bp.kappa);
            o.put<double>((double)bp.theta0);
        }
    }
    o.put<uint32_t>(s.polymers.size());
    for (const auto &p : s.polymers) {
        o.put<uint32_t>(p.polymer_type);
        o.put<uint32_t>(p.bead_ids.size());
        for (auto id : p.bead_ids) o.put<uint32_t>(id);
    }
    o.put<uint32_t>(s.beads.size());
    for (const auto &b : s.beads) {
        o.put<uint32_t>(b.bead_id);
        o.put<uint32_t>(b.polymer_id);
        o.put<uint8_t>(b.polymer_offset);
        o.put<uint8_t>(b.bead_type);
        o.put<uint8_t>(b.polymer_type);
        o.put<uint8_t>(b.is_monomer ? 1 : 0);
        for (int d = 0; d < 3; d++) o.put<double>(b.x[d]);
        for (int d = 0; d < 3; d++) o.put<double>(b.v[d]);
        for (int d = 0; d < 3; d++) o.put<double>(b.f[d]);
    }
}

void put_state(Out &o, const WorldState &s)
{
    o.put<int64_t>(s.t);
    for (const auto &b : s.beads) {
        for (int d = 0; d < 3; d++) o.put<double>(b.x[d]);
        for (int d = 0; d < 3; d++) o.put<double>(b.v[d]);
        for (int d = 0; d < 3; d++) o.put<double>(b.f[d]);
    }
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: testbase_export out.bin [max_segments]\n");
        return 1;
    }
    size_t max_segments = argc > 2 ? (size_t)atoi(argv[2]) : 6;
    TestOrderedMesh::register_tests();
    TestBondedBeadAngle::register_tests();
    TestBondedBeadTriple::register_tests();
    TestBondedBeadPair::register_tests();
    TestCollidingBeadPair::register_tests();
    TestCollidingBeadPairDiss::register_tests();
    TestIsolatedMovingBead::register_tests();
    TestMultipleMovingBeads::register_tests();
    auto tests = TestBase::get_test_factories_ordered_by_complexity();

    Out out;
    out.put<uint32_t>(tests.size());
    int n_ok = 0;
    for (const auto &ttt : tests) {
        auto test = std::get<2>(ttt)();
        NaiveDPDEngineHalfStep engine;
        WorldState state = test->create_world();
        validate(state);
        Out pd;
        put_pdw1(pd, state);
        struct Seg {
            unsigned todo;
            Out in, outs;
        };
        std::vector<Seg> segs;
        bool ok = false;
        try {
            engine.Attach(&state);
            unsigned done = 0;
            while (done <= 100000) {
                unsigned todo = test->get_advance_count(state);
                if (todo == 0) {
                    ok = true;
                    break;
                }
                Seg sg;
                sg.todo = todo;
                put_state(sg.in, state);
                engine.Run(todo);
                validate(state);
                put_state(sg.outs, state);
                segs.push_back(std::move(sg));
                done += todo;
            }
        } catch (std::exception &e) {
            fprintf(stderr, "%s: %s\n", test->name().c_str(), e.what());
        }
        n_ok += ok;
        // keep an evenly spaced subset of segments, always the first and the last
        std::vector<size_t> keep;
        if (segs.size() <= max_segments) {
            for (size_t i = 0; i < segs.size(); i++) keep.push_back(i);
        } else {
            for (size_t k = 0; k < max_segments; k++)
                keep.push_back(k * (segs.size() - 1) / (max_segments - 1));
        }
        std::string name = test->name();
        out.put<uint32_t>(name.size());
        out.bytes(name.data(), name.size());
        out.put<uint32_t>(ok ? 1 : 0);
        out.put<uint32_t>(pd.buf.size());
        out.bytes(pd.buf.data(), pd.buf.size());
        out.put<uint32_t>(keep.size());
        for (size_t i : keep) {
            out.put<uint32_t>(segs[i].todo);
            out.bytes(segs[i].in.buf.data(), segs[i].in.buf.size());
            out.bytes(segs[i].outs.buf.data(), segs[i].outs.buf.size());
        }
    }
    FILE *f = fopen(argv[1], "wb");
    if (!f) return 1;
    fwrite(out.buf.data(), 1, out.buf.size(), f);
    fclose(f);
    fprintf(stderr, "%zu tests, %d ok under the reference engine, %zu bytes\n", tests.size(), n_ok,
            out.buf.size());
    return 0;
}
