// Write a "WorldState v2binary" file whose bead section was encoded on the GPU.
//
// Include in one translation unit of a poets-dpd tool (it includes the reference's
// dpd_state_io.hpp, whose functions are defined in the header).  The text header is written
// line by line as write_world_state does (dpd_state_io.hpp:408-451), through the
// reference's own formatting: operator<< of the state's numbers and Parameters,
// write_bead_type and write_polymer_type; then "BinaryData", a newline, one zero byte
// (:452-455) and the section from GB300DPDEngine::EncodeV2BinarySection.  The result equals
// write_world_state(dst, state, true) for the engine's state, byte for byte.
#pragma once

#include <cstdint>
#include <ostream>
#include <vector>

#include "dpd/core/dpd_state_io.hpp"
#include "gb300_dpd_engine.hpp"

// Header, marker and the given section (the bytes after "BinaryData\n" and its zero byte).
inline void write_world_state_v2binary(std::ostream &dst, const WorldState &state,
                                       const std::vector<uint8_t> &section)
{
    dst << "WorldState v2binary " << state.bead_types.size() << " " << state.polymer_types.size()
        << " " << state.beads.size() << " " << state.polymers.size() << "\n";
    dst << "T " << state.t << " " << state.dt << "\n";
    dst << "Lambda " << state.lambda << "\n";
    dst << "Origin " << state.origin[0] << " " << state.origin[1] << " " << state.origin[2] << "\n";
    dst << "Box " << state.box[0] << " " << state.box[1] << " " << state.box[2] << "\n";
    dst << "Seed " << state.seed << "\n";
    const unsigned nbt = state.bead_types.size();
    for (unsigned i = 0; i < nbt; i++) {
        dst << "ConservativeStrength " << i;
        for (unsigned j = 0; j < nbt; j++) dst << " " << state.interactions[i * nbt + j].conservative;
        dst << "\n";
    }
    for (unsigned i = 0; i < nbt; i++) {
        dst << "DissipativeStrength " << i;
        for (unsigned j = 0; j < nbt; j++) dst << " " << state.interactions[i * nbt + j].dissipative;
        dst << "\n";
    }
    dst << "\n# BeadTypes\n";
    for (const auto &bt : state.bead_types) write_bead_type(dst, bt, state);
    dst << "\n# polymerTypes\n";
    for (const auto &pt : state.polymer_types) write_polymer_type(dst, pt, state);
    dst << "\nBinaryData\n";
    const char zero = 0;
    dst.write(&zero, 1);
    dst.write((const char *)section.data(), (std::streamsize)section.size());
    if (dst.bad()) throw std::runtime_error("Error while writing binary stream.");
}

// The engine's current state of the attached world (after Run: x, v, f and t are those the
// engine holds) as a v2binary file.
inline void write_world_state_v2binary(std::ostream &dst, const WorldState &state, GB300DPDEngine &engine)
{
    write_world_state_v2binary(dst, state, engine.EncodeV2BinarySection());
}
