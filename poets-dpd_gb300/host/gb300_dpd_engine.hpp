// GB300DPDEngine: the GB300 engine as a poets-dpd DPDEngine plug-in.
//
// Compiled inside a poets-dpd build (it includes the reference's own engine interface,
// include/dpd/core/dpd_engine.hpp) and linked against libpdpd_gb300.so.  It is a drop-in
// for any tool that creates engines through DPDEngineFactory (run_world, step_world,
// benchmark_engine, test_engine, ...): the registration stub gb300_dpd_engine.cpp registers
// "gb300_dpd_engine_fp32" and "gb300_dpd_engine_fp64".
//
// Every member forwards to the C ABI in include/pdpd_gpu.h:
//   CanSupport       dpd_engine.hpp:57-128  -> base checks, then pdpd_can_support
//   GetMaxBondLength dpd_engine.hpp:130     -> pdpd_max_bond_length (2.0)
//   Attach           dpd_engine.hpp:177     -> flatten the WorldState, pdpd_attach
//   Run(n)           dpd_engine.hpp:185     -> pdpd_run, then pdpd_read_state into the beads
//   Run(count, size, cb) dpd_engine.hpp:195-215 -> pdpd_run_intervals (the next interval
//                    runs on the GPU while the callback sees the previous one)
//   GetTimings       dpd_engine.hpp:145     -> pdpd_get_timings
//   Get/SetConfigEntry dpd_engine.hpp:150-169 -> pdpd_get_config / pdpd_set_config
// Errors come back as std::runtime_error, as the reference's engines throw.
#pragma once

#include <exception>
#include <functional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "dpd/core/dpd_engine.hpp"
#include "pdpd_gpu.h"

class GB300DPDEngine : public DPDEngine {
public:
    // The WorldState in the flat form of the C ABI; the vectors own the expanded data, the
    // bead vectors point straight into WorldState::beads (stride sizeof(Bead)).
    struct Flat {
        std::vector<double> conservative, dissipative;
        std::vector<uint8_t> stationary;
        std::vector<uint32_t> hash;
        std::vector<uint32_t> bond_beads;
        std::vector<double> bond_kappa, bond_r0;
        std::vector<uint32_t> angle_beads;
        std::vector<double> angle_kappa, angle_theta0;
        std::vector<double> cell_conservative, cell_dissipative;  // spatial strengths only
        pdpd_world w{};
    };

    // The GPU engine is created on first use (Attach, Run, config), so a tool can list the
    // engine, ask CanSupport and read its description on a machine without a GPU.
    explicit GB300DPDEngine(int precision = PDPD_FP32) : m_precision(precision) {}

    ~GB300DPDEngine() override
    {
        if (m_engine) pdpd_destroy(m_engine);
    }

    GB300DPDEngine(const GB300DPDEngine &) = delete;
    GB300DPDEngine &operator=(const GB300DPDEngine &) = delete;

    // Expand a WorldState into the C ABI's flat form: bonds and angle bonds polymer by
    // polymer, in polymer-type order (the order of naive_dpd_engine_half_step.hpp:321-329).
    static void Flatten(const WorldState &s, Flat &out)
    {
        const unsigned nt = s.bead_types.size();
        out.conservative.resize(nt * nt);
        out.dissipative.resize(nt * nt);
        bool spatial = false;
        for (unsigned i = 0; i < nt * nt; i++)
            spatial |= !s.interactions.at(i).conservative.is_constant() ||
                        !s.interactions.at(i).dissipative.is_constant();
        out.cell_conservative.clear();
        out.cell_dissipative.clear();
        if (spatial) {
            // Per-cell values, evaluated as the half-merge engine does at Attach
            // (naive_dpd_engine_half_merge.hpp:221-236); the matrices hold cell 0's values.
            const int L[3] = {(int)s.box[0], (int)s.box[1], (int)s.box[2]};
            std::unordered_map<std::string, double> b;
            for (int x = 0; x < L[0]; x++)
                for (int y = 0; y < L[1]; y++)
                    for (int z = 0; z < L[2]; z++) {
                        b["x"] = x;
                        b["y"] = y;
                        b["z"] = z;
                        b["ux"] = (x + 0.5) / s.box[0];
                        b["uy"] = (y + 0.5) / s.box[1];
                        b["uz"] = (z + 0.5) / s.box[2];
                        for (unsigned i = 0; i < nt * nt; i++) {
                            Parameter pc = s.interactions.at(i).conservative, pd = s.interactions.at(i).dissipative;
                            out.cell_conservative.push_back(pc.evaluate(b));
                            out.cell_dissipative.push_back(pd.evaluate(b));
                        }
                    }
            for (unsigned i = 0; i < nt * nt; i++) {
                out.conservative[i] = out.cell_conservative.empty() ? 0.0 : out.cell_conservative[i];
                out.dissipative[i] = out.cell_dissipative.empty() ? 0.0 : out.cell_dissipative[i];
            }
        } else {
            for (unsigned i = 0; i < nt * nt; i++) {
                out.conservative[i] = (double)s.interactions.at(i).conservative;
                out.dissipative[i] = (double)s.interactions.at(i).dissipative;
            }
        }
        out.stationary.resize(nt);
        for (unsigned i = 0; i < nt; i++) out.stationary[i] = s.bead_types[i].stationary ? 1 : 0;
        out.hash.resize(s.beads.size());
        for (size_t i = 0; i < s.beads.size(); i++) out.hash[i] = s.beads[i].get_hash_code().hash;
        out.bond_beads.clear();
        out.bond_kappa.clear();
        out.bond_r0.clear();
        out.angle_beads.clear();
        out.angle_kappa.clear();
        out.angle_theta0.clear();
        for (const Polymer &p : s.polymers) {
            const PolymerType &pt = s.polymer_types.at(p.polymer_type);
            for (const Bond &b : pt.bonds) {
                out.bond_beads.push_back(p.bead_ids.at(b.bead_offset_head));
                out.bond_beads.push_back(p.bead_ids.at(b.bead_offset_tail));
                out.bond_kappa.push_back((double)b.kappa);
                out.bond_r0.push_back((double)b.r0);
            }
        }
        for (const Polymer &p : s.polymers) {
            const PolymerType &pt = s.polymer_types.at(p.polymer_type);
            for (const BondPair &bp : pt.bond_pairs) {
                const Bond &head = pt.bonds.at(bp.bond_offset_head);
                const Bond &tail = pt.bonds.at(bp.bond_offset_tail);
                out.angle_beads.push_back(p.bead_ids.at(head.bead_offset_head));
                out.angle_beads.push_back(p.bead_ids.at(head.bead_offset_tail));
                out.angle_beads.push_back(p.bead_ids.at(tail.bead_offset_tail));
                out.angle_kappa.push_back((double)bp.kappa);
                out.angle_theta0.push_back((double)bp.theta0);
            }
        }
        pdpd_world &w = out.w;
        for (int d = 0; d < 3; d++) w.box[d] = (int32_t)s.box[d];
        w.dt = s.dt;
        w.lambda = s.lambda;
        w.seed = s.seed;
        w.t = s.t;
        w.n_bead_types = nt;
        w.conservative = out.conservative.data();
        w.dissipative = out.dissipative.data();
        w.stationary = out.stationary.data();
        w.n_beads = (uint32_t)s.beads.size();
        w.hash = out.hash.data();
        w.x = s.beads.empty() ? nullptr : &s.beads[0].x.x[0];
        w.v = s.beads.empty() ? nullptr : &s.beads[0].v.x[0];
        w.f = s.beads.empty() ? nullptr : &s.beads[0].f.x[0];
        w.bead_stride_bytes = sizeof(Bead);
        w.n_bonds = (uint32_t)out.bond_kappa.size();
        w.bond_beads = out.bond_beads.data();
        w.bond_kappa = out.bond_kappa.data();
        w.bond_r0 = out.bond_r0.data();
        w.n_angles = (uint32_t)out.angle_kappa.size();
        w.angle_beads = out.angle_beads.data();
        w.angle_kappa = out.angle_kappa.data();
        w.angle_theta0 = out.angle_theta0.data();
        w.cell_conservative = spatial ? out.cell_conservative.data() : nullptr;
        w.cell_dissipative = spatial ? out.cell_dissipative.data() : nullptr;
    }

    std::string CanSupport(const WorldState *s) const override
    {
        std::string base = DPDEngine::CanSupport(s);  // rejects non-constant parameters etc.
        if (!base.empty()) return base;
        for (int d = 0; d < 3; d++)
            if (s->box[d] != (double)(int32_t)s->box[d]) return "World bounds must be integer.";
        Flat flat;
        Flatten(*s, flat);
        char reason[256];
        if (pdpd_can_support(&flat.w, reason, sizeof reason) != PDPD_OK) return reason;
        return "";
    }

    double GetMaxBondLength() const override
    {
        return pdpd_max_bond_length();
    }

    void Attach(WorldState *state) override
    {
        engine();
        m_state = state;
        m_v2_state = nullptr;
        if (!state) {
            check(pdpd_attach(m_engine, nullptr), "Attach");
            return;
        }
        Flat flat;
        Flatten(*state, flat);
        check(pdpd_attach(m_engine, &flat.w), "Attach");
    }

    void Run(unsigned nSteps) override
    {
        engine();
        require_state();
        check(pdpd_run(m_engine, nSteps), "Run");
        read_back();
    }

    // The callback sees each interval's state in the beads while the device already runs the
    // next interval from that state: it must treat the beads as read-only (an edit does not
    // reach the engine and is overwritten by the next interval's write-back).  The reference's
    // engines run the callback between intervals, where an edit would take effect; a caller
    // that edits returns false, edits, and calls Attach and Run again.
    unsigned Run(int interval_count, unsigned interval_size,
                 std::function<bool()> interval_callback) override
    {
        engine();
        require_state();
        struct Ctx {
            WorldState *state;
            std::function<bool()> *cb;
            std::exception_ptr error;
        } ctx{m_state, &interval_callback, nullptr};
        // No exception may cross the C ABI: a throwing callback stops the run and the
        // exception is re-thrown here once the engine has returned.
        auto tramp = [](void *user, int64_t t) -> int {
            Ctx *c = (Ctx *)user;
            c->state->t = t;
            try {
                return (*c->cb)() ? 1 : 0;
            } catch (...) {
                c->error = std::current_exception();
                return 0;
            }
        };
        Bead *b = m_state->beads.empty() ? nullptr : &m_state->beads[0];
        uint32_t done = 0;
        check(pdpd_run_intervals(m_engine, interval_count, interval_size, b ? &b->x.x[0] : nullptr,
                                 b ? &b->v.x[0] : nullptr, b ? &b->f.x[0] : nullptr, sizeof(Bead),
                                 tramp, &ctx, &done),
              "Run");
        if (ctx.error) std::rethrow_exception(ctx.error);
        return done;
    }

    bool GetTimings(timings_t &timings) override
    {
        if (!m_engine) return false;
        pdpd_timings t;
        if (pdpd_get_timings(m_engine, &t) != PDPD_OK) return false;
        timings.compile = t.compile;
        timings.aquire = t.aquire;
        timings.configure = t.configure;
        timings.execute_to_first_bead = t.execute_to_first_bead;
        timings.execute_to_last_bead = t.execute_to_last_bead;
        timings.perf_counters = t.perf_counters;
        return true;
    }

    void GetConfigEntries(std::vector<engine_config_entry_t> &config) override
    {
        config.clear();
        engine();
        char name[128], desc[512], value[64];
        for (uint32_t i = 0;
             pdpd_get_config(m_engine, i, name, sizeof name, desc, sizeof desc, value, sizeof value) == PDPD_OK;
             i++)
            config.push_back({name, desc, value});
    }

    void SetConfigEntry(const std::string &key, const std::string &value) override
    {
        if (pdpd_set_config(engine(), key.c_str(), value.c_str()) != PDPD_OK)
            throw std::runtime_error(pdpd_last_error(m_engine));
    }

    // The BinaryData section of a "WorldState v2binary" file for the attached state as the
    // engine holds it after the last Run, encoded on the GPU (about 22 bytes per bead cross
    // the bus instead of 72).  Not a DPDEngine member: gb300_v2binary.hpp writes the whole
    // file with it.  The polymer layout is built on the first call after an Attach.
    std::vector<uint8_t> EncodeV2BinarySection()
    {
        engine();
        require_state();
        if (m_v2_state != m_state) {
            std::vector<uint32_t> types, start{0}, beads, ids;
            for (const Polymer &p : m_state->polymers) {
                ids.push_back(p.polymer_id);
                types.push_back(p.polymer_type);
                beads.insert(beads.end(), p.bead_ids.begin(), p.bead_ids.end());
                start.push_back((uint32_t)beads.size());
            }
            size_t n = 0;
            check(pdpd_v2binary_prepare(m_engine, 0, (uint32_t)types.size(), ids.data(), types.data(),
                                        start.data(), beads.data(), &n),
                  "v2binary");
            m_v2_state = m_state;
        }
        size_t n = 0;
        check(pdpd_v2binary_encode(m_engine, 0, nullptr, 0, &n), "v2binary");
        std::vector<uint8_t> out(n);
        check(pdpd_v2binary_encode(m_engine, 0, out.data(), out.size(), &n), "v2binary");
        return out;
    }

protected:
    bool CanSupportHookeanBonds() const override { return true; }
    bool CanSupportAngleBonds() const override { return true; }
    bool CanSupportStationaryBeadTypes() const override { return true; }
    bool CanSupportSpatialDPDParameters() const override { return true; }

private:
    int m_precision;
    pdpd_engine *m_engine = nullptr;
    WorldState *m_state = nullptr;
    WorldState *m_v2_state = nullptr;  // state the v2binary layout was built for

    pdpd_engine *engine()
    {
        if (!m_engine && pdpd_create(m_precision, -1, &m_engine) != PDPD_OK) {
            m_engine = nullptr;
            throw std::runtime_error(std::string("GB300DPDEngine: ") + pdpd_last_error(nullptr));
        }
        return m_engine;
    }

    void check(int rc, const char *what) const
    {
        if (rc != PDPD_OK)
            throw std::runtime_error(std::string("GB300DPDEngine::") + what + ": " + pdpd_last_error(m_engine));
    }

    void require_state() const
    {
        if (!m_state) throw std::runtime_error("GB300DPDEngine: no world attached");
    }

    // Write x(t), v(t), f(t) and t back into the attached WorldState (dpd_engine.hpp:179-184).
    void read_back()
    {
        int64_t t = 0;
        Bead *b = m_state->beads.empty() ? nullptr : &m_state->beads[0];
        check(pdpd_read_state(m_engine, 0, b ? &b->x.x[0] : nullptr, b ? &b->v.x[0] : nullptr,
                              b ? &b->f.x[0] : nullptr, sizeof(Bead), &t),
              "Run");
        m_state->t = t;
    }
};
