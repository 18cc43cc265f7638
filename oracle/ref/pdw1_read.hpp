// Test infrastructure: reads a world stored in the PDW1 file format (written by
// poets-dpd_gb300/pdpd_world.py) into the reference's WorldState.  Shared by the
// reference harness and the adapter check; both compile against the reference headers.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "dpd/core/dpd_state.hpp"

namespace pdw1 {

struct Reader {
    FILE *f;
    explicit Reader(const char *path) : f(fopen(path, "rb")) {
        if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    }
    ~Reader() { if (f) fclose(f); }
    template <class T> T get() {
        T v;
        if (fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("short read");
        return v;
    }
};

WorldState read_pdw1(const char *path)
{
    Reader r(path);
    char magic[4];
    if (fread(magic, 1, 4, r.f) != 4 || memcmp(magic, "PDW1", 4) != 0)
        throw std::runtime_error("not a PDW1 file");
    WorldState s;
    for (int i = 0; i < 3; i++) s.box[i] = r.get<int32_t>();
    s.dt = r.get<double>();
    s.lambda = r.get<double>();
    s.seed = r.get<uint64_t>();
    s.t = r.get<int64_t>();
    unsigned nt = r.get<uint32_t>();
    for (unsigned i = 0; i < nt; i++) {
        BeadType bt;
        bt.name = "T" + std::to_string(i);
        bt.r = 0.5;
        bt.id = i;
        bt.stationary = r.get<uint32_t>() != 0;
        s.bead_types.push_back(bt);
    }
    s.interactions.resize(nt * nt);
    for (unsigned i = 0; i < nt * nt; i++) s.interactions[i].conservative = r.get<double>();
    for (unsigned i = 0; i < nt * nt; i++) s.interactions[i].dissipative = r.get<double>();
    unsigned npt = r.get<uint32_t>();
    for (unsigned i = 0; i < npt; i++) {
        PolymerType pt;
        pt.name = "P" + std::to_string(i);
        pt.polymer_id = i;
        unsigned nb = r.get<uint32_t>();
        for (unsigned k = 0; k < nb; k++) pt.bead_types.push_back(r.get<uint32_t>());
        unsigned nbond = r.get<uint32_t>();
        for (unsigned k = 0; k < nbond; k++) {
            Bond b;
            b.bead_offset_head = r.get<uint32_t>();
            b.bead_offset_tail = r.get<uint32_t>();
            b.kappa = r.get<double>();
            b.r0 = r.get<double>();
            pt.bonds.push_back(b);
        }
        unsigned npair = r.get<uint32_t>();
        for (unsigned k = 0; k < npair; k++) {
            BondPair bp;
            bp.bond_offset_head = r.get<uint32_t>();
            bp.bond_offset_tail = r.get<uint32_t>();
            bp.kappa = r.get<double>();
            bp.theta0 = r.get<double>();
            pt.bond_pairs.push_back(bp);
        }
        s.polymer_types.push_back(pt);
    }
    unsigned np = r.get<uint32_t>();
    s.polymers.resize(np);
    for (unsigned i = 0; i < np; i++) {
        Polymer &p = s.polymers[i];
        p.polymer_id = i;
        p.polymer_type = r.get<uint32_t>();
        unsigned n = r.get<uint32_t>();
        for (unsigned k = 0; k < n; k++) p.bead_ids.push_back(r.get<uint32_t>());
    }
    unsigned nb = r.get<uint32_t>();
    s.beads.resize(nb);
    for (unsigned i = 0; i < nb; i++) {
        Bead &b = s.beads[i];
        b.bead_id = r.get<uint32_t>();
        b.polymer_id = r.get<uint32_t>();
        b.polymer_offset = r.get<uint8_t>();
        b.bead_type = r.get<uint8_t>();
        b.polymer_type = r.get<uint8_t>();
        b.is_monomer = r.get<uint8_t>() != 0;
        for (int d = 0; d < 3; d++) b.x[d] = r.get<double>();
        for (int d = 0; d < 3; d++) b.v[d] = r.get<double>();
        for (int d = 0; d < 3; d++) b.f[d] = r.get<double>();
    }
    return s;
}

}  // namespace pdw1
