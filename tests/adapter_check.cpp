// Test infrastructure: builds the DPDEngine adapter (poets-dpd_gb300/host) against the
// reference's own headers and checks, without a GPU, that it registers with
// DPDEngineFactory, answers CanSupport through the reference's base checks, and flattens a
// WorldState exactly as the Python mirror does.  Compiled and run by tests/test_adapter.py
// where the reference sources are present.
//
//   adapter_check factories
//   adapter_check cansupport <engine> <world.pdw1>
//   adapter_check flatten <world.pdw1> <out.bin>
//   adapter_check spatial <world.pdw1> <exprs.txt> <out.bin>
//       strengths replaced by Parameter expressions (n^2 conservative, then n^2 dissipative
//       lines); prints CanSupport, writes the flattened per-cell tables
//   adapter_check v2file <world.pdw1> <section.bin> <out.v2>
//       gb300_v2binary.hpp's file writer around a given BinaryData section
#include "dpd/core/dpd_state_validator.hpp"
#include "dpd/core/logging.hpp"
#include "dpd/core/logging_impl.hpp"

#include "gb300_dpd_engine.hpp"
#include "gb300_v2binary.hpp"
#include "pdw1_read.hpp"

#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

template <class T> static void put(FILE *f, const std::vector<T> &v)
{
    uint64_t n = v.size();
    fwrite(&n, 8, 1, f);
    if (n) fwrite(v.data(), sizeof(T), n, f);
}

int main(int argc, char **argv)
{
    try {
        std::string cmd = argc > 1 ? argv[1] : "";
        if (cmd == "factories") {
            for (const auto &n : DPDEngineFactory::ListFactories()) printf("%s\n", n.c_str());
            return 0;
        }
        if (cmd == "cansupport" && argc > 3) {
            WorldState s = pdw1::read_pdw1(argv[3]);
            auto e = DPDEngineFactory::create(argv[2]);
            printf("[%s]\n", e->CanSupport(&s).c_str());
            printf("max_bond_length %g\n", e->GetMaxBondLength());
            return 0;
        }
        if (cmd == "flatten" && argc > 3) {
            WorldState s = pdw1::read_pdw1(argv[2]);
            GB300DPDEngine::Flat flat;
            GB300DPDEngine::Flatten(s, flat);
            FILE *f = fopen(argv[3], "wb");
            if (!f) return 2;
            put(f, flat.hash);
            put(f, flat.conservative);
            put(f, flat.dissipative);
            put(f, flat.bond_beads);
            put(f, flat.bond_kappa);
            put(f, flat.bond_r0);
            put(f, flat.angle_beads);
            put(f, flat.angle_kappa);
            put(f, flat.angle_theta0);
            const pdpd_world &w = flat.w;
            std::vector<double> head = {(double)w.box[0], (double)w.box[1], (double)w.box[2], w.dt,
                                        w.lambda, (double)w.t, (double)w.n_beads,
                                        (double)w.bead_stride_bytes};
            put(f, head);
            std::vector<double> x;
            for (uint32_t i = 0; i < w.n_beads; i++) {
                const double *p = (const double *)((const char *)w.x + w.bead_stride_bytes * i);
                x.push_back(p[0]);
                x.push_back(p[1]);
                x.push_back(p[2]);
            }
            put(f, x);
            fclose(f);
            return 0;
        }
        if (cmd == "spatial" && argc > 4) {
            WorldState s = pdw1::read_pdw1(argv[2]);
            std::ifstream in(argv[3]);
            std::vector<std::string> lines;
            std::string line;
            while (std::getline(in, line))
                if (!line.empty()) lines.push_back(line);
            const size_t n2 = s.interactions.size();
            if (lines.size() != 2 * n2) return 2;
            for (size_t k = 0; k < n2; k++) {
                s.interactions[k].conservative = Parameter(lines[k]);
                s.interactions[k].dissipative = Parameter(lines[n2 + k]);
            }
            auto e = DPDEngineFactory::create("gb300_dpd_engine_fp64");
            printf("[%s]\n", e->CanSupport(&s).c_str());
            GB300DPDEngine::Flat flat;
            GB300DPDEngine::Flatten(s, flat);
            FILE *f = fopen(argv[4], "wb");
            if (!f) return 2;
            put(f, flat.cell_conservative);
            put(f, flat.cell_dissipative);
            fclose(f);
            return 0;
        }
        if (cmd == "v2file" && argc > 4) {
            WorldState s = pdw1::read_pdw1(argv[2]);
            std::ifstream in(argv[3], std::ios::binary);
            std::vector<uint8_t> section((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
            std::ofstream out(argv[4], std::ios::binary);
            write_world_state_v2binary(out, s, section);
            return 0;
        }
        fprintf(stderr, "usage: adapter_check factories | cansupport <engine> <pdw1> | flatten <pdw1> <out>"
                        " | v2file <pdw1> <section> <out>\n");
        return 1;
    } catch (std::exception &e) {
        fprintf(stderr, "adapter_check: %s\n", e.what());
        return 1;
    }
}
