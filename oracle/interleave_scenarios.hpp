// ORACLE — test infrastructure only.  Scripted-policy scenarios that pin a
// charged-loop skeleton (the event interleave and the substep interleave)
// by what it hands its policies.  The same scenarios, with the same
// recording policies, are run through the reference's templates
// (O/RreaChargedInterleave.H:546-732, compiled into oracle/_ref/ref_golden)
// and through the oracle's restatement (oracle/interleave.hpp); the traces
// must agree exactly.
//
// Event-interleave scenarios use an analytic medium whose rates and
// stopping depend on the frozen energy (tau_c = (end - begin) a_c E / 1e6,
// drag = s (end - begin) E, so a wrong refreeze or a wrong segment end
// changes the trace), scripted uniforms, channel gates that open above a
// per-channel energy, scripted final-state losses and a scripted consumed
// parent.  Substep-interleave scenarios script every policy's answer per
// substep and lower the energy below the cutoff at a scripted point.
//
// A skeleton is a functor type S with
//   S::events(begin, end, kinetic&, cutoff, channels, max_ordinal, policies...)
//   S::substeps(subcycles, kinetic&, cutoff, completed&, exited&, policies...)
// whose aborts throw (any std::exception).
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <exception>
#include <utility>
#include <vector>

namespace interleave_scenarios {

// Trace record: {code, a, b, c}.
enum Code {
    kTaus = 1, kDraws, kDepth, kSegment, kStop, kPoint, kOpen, kFinal, kAbort, kEnd,
    kBuild = 11, kEvents, kStopped, kFinish, kAdvance, kExits, kSubEnd
};

struct Trace {
    std::vector<double> rec;
    void put(int code, double a = 0.0, double b = 0.0, double c = 0.0)
    {
        rec.push_back(code);
        rec.push_back(a);
        rec.push_back(b);
        rec.push_back(c);
    }
};

// splitmix64 stream for scenario generation
struct Gen {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }
    int below(int n) { return static_cast<int>(next() % static_cast<uint64_t>(n)); }
};

struct EventScenario {
    double kinetic = 1.0e6, cutoff = 1.0e3;
    int channels = 2;
    uint64_t max_ordinal = 64;
    std::array<double, 3> rate{1.0, 0.0, 0.0};        // a_c
    std::array<double, 3> open_above{0.0, 0.0, 0.0};  // channel c open when E > open_above[c]
    double stopping = 0.5;                            // s
    double begin = 0.0, end = 1.0;
    std::vector<std::pair<double, double>> draws;
    std::vector<double> losses;   // per final-state call
    int consume_at = -1;          // final-state call that consumes the parent
};

inline double u_for_tau(double tau) { return -std::expm1(-tau); }

// Deterministic random scenario `seed` (seed < 8 are the hand-written
// fixtures the reference's own smoke exercises: refreeze, survivor-energy
// segment, null event, consumed parent, cutoff stop, ordinal cap, invalid
// revalidation, channel 2 pick).
inline EventScenario event_scenario(uint64_t seed)
{
    EventScenario s;
    switch (seed) {
    case 0:  // one event at 0.25 losing 1e5: refreeze at 7.75e5
        s.draws = {{u_for_tau(0.25), 0.1}, {u_for_tau(10.0), 0.1}};
        s.losses = {1.0e5};
        return s;
    case 1:  // two events, the second from the survivor energy
        s.draws = {{u_for_tau(0.25), 0.1}, {u_for_tau(0.09375), 0.1}, {u_for_tau(10.0), 0.1}};
        s.losses = {5.0e5, 1.0e4};
        return s;
    case 2:  // closed at the event, open at the frozen energy: a null event
        s.kinetic = 9.0e5;
        s.open_above = {8.0e5, 0.0, 0.0};
        s.draws = {{u_for_tau(0.54), 0.1}, {u_for_tau(10.0), 0.1}};
        return s;
    case 3:  // the final state consumes the parent
        s.draws = {{u_for_tau(0.25), 0.1}};
        s.losses = {1.0e5};
        s.consume_at = 0;
        return s;
    case 4:  // the no-event tail reaches the cutoff
        s.kinetic = 1.5e3;
        s.draws = {{u_for_tau(10.0), 0.1}};
        return s;
    case 5:  // null events until the ordinal cap
        s.kinetic = 9.0e5;
        s.max_ordinal = 3;
        s.stopping = 0.01;
        s.open_above = {9.5e5, 0.0, 0.0};
        s.draws = std::vector<std::pair<double, double>>(8, {u_for_tau(0.01), 0.1});
        return s;
    case 6:  // closed at both energies: the skeleton aborts
        s.open_above = {2.0e6, 0.0, 0.0};
        s.draws = {{u_for_tau(0.25), 0.1}};
        return s;
    case 7:  // three channels, the channel draw picks the last one
        s.channels = 3;
        s.rate = {0.2, 0.3, 0.5};
        s.draws = {{u_for_tau(0.2), 0.95}, {u_for_tau(10.0), 0.5}};
        s.losses = {2.0e5};
        return s;
    default:
        break;
    }
    Gen g{seed * 0x2545F4914F6CDD1DULL + 17};
    s.kinetic = std::exp(std::log(2.0e3) + g.uniform() * (std::log(5.0e7) - std::log(2.0e3)));
    s.cutoff = 1.0e3 * (1.0 + 9.0 * g.uniform());
    s.channels = 1 + g.below(3);
    s.max_ordinal = 4 + static_cast<uint64_t>(g.below(40));
    for (int c = 0; c < 3; ++c) {
        s.rate[c] = g.below(4) == 0 ? 0.0 : g.uniform() * 3.0;
        s.open_above[c] = g.below(3) == 0 ? s.kinetic * g.uniform() * 1.2 : 0.0;
    }
    s.stopping = g.uniform() < 0.2 ? 2.0 + 3.0 * g.uniform() : 0.6 * g.uniform();
    s.begin = g.below(2) ? 0.0 : 0.3 * g.uniform();
    s.end = g.below(4) == 0 ? s.begin + 0.5 * g.uniform() : 1.0;
    int const nd = 1 + g.below(12);
    for (int i = 0; i < nd; ++i) {
        double const u1 = g.below(8) == 0 ? 1.0 - 1.0e-17 : g.uniform();
        double const u2 = g.below(10) == 0 ? 1.0 : g.uniform();
        s.draws.push_back({u1, u2});
    }
    int const nl = g.below(10);
    for (int i = 0; i < nl; ++i) s.losses.push_back(s.kinetic * 0.6 * g.uniform());
    s.consume_at = g.below(3) == 0 ? g.below(4) : -1;
    return s;
}

struct Limit {
    bool reaches_cutoff;
    double effective_end_fraction;
};

template <class S>
Trace run_event_scenario(EventScenario const& sc)
{
    Trace t;
    double kinetic = sc.kinetic;
    std::size_t draw = 0, calls = 0;
    try {
        S::events(
            sc.begin, sc.end, kinetic, sc.cutoff, sc.channels, sc.max_ordinal,
            [&](double frozen, double b, double e) {
                t.put(kTaus, frozen, b, e);
                std::array<double, 3> taus{};
                for (int c = 0; c < 3; ++c) taus[c] = (e - b) * sc.rate[c] * frozen / 1.0e6;
                return taus;
            },
            [&](uint64_t ordinal) {
                t.put(kDraws, static_cast<double>(ordinal));
                // an exhausted script draws "no event"
                std::pair<double, double> d = draw < sc.draws.size() ? sc.draws[draw] : std::make_pair(0.0, 0.5);
                ++draw;
                return d;
            },
            [&](double tau, double b, double e) {
                t.put(kDepth, tau, b, e);
                double total = 0.0;
                for (int c = 0; c < sc.channels; ++c) total += sc.rate[c];
                double const per = total * kinetic / 1.0e6;
                return per > 0.0 ? b + tau / per : e;
            },
            [&](double b, double e, double frozen) {
                double const loss = sc.stopping * (e - b) * frozen;
                kinetic -= loss;
                bool const reaches = kinetic < sc.cutoff;
                t.put(kSegment, b, e, frozen);
                return Limit{reaches, reaches ? 0.5 * (b + e) : e};
            },
            [&](double f) { t.put(kStop, f); },
            [&](double f) { t.put(kPoint, f); },
            [&](int ch, double energy) {
                bool const open = energy > sc.open_above[static_cast<std::size_t>(ch)];
                t.put(kOpen, ch, energy, open ? 1.0 : 0.0);
                return open;
            },
            [&](int ch, double f) {
                t.put(kFinal, ch, f);
                if (calls < sc.losses.size()) kinetic -= sc.losses[calls];
                bool const consumed = static_cast<int>(calls) == sc.consume_at;
                ++calls;
                return !consumed;
            });
    } catch (std::exception const&) {
        t.put(kAbort);
    }
    t.put(kEnd, kinetic, static_cast<double>(draw), static_cast<double>(calls));
    return t;
}

struct SubstepScenario {
    uint64_t subcycles = 3;
    double kinetic = 1.0e6, cutoff = 1.0e3;
    std::vector<int> build_ok, stop_after_events, finish_ends, advance_ok, exits;
    int drop_below_cutoff_at = -1;  // the finish of this substep lowers E below the cutoff
    int drop_in_build = -1;         // the build of this substep lowers E below the cutoff and refuses
};

inline SubstepScenario substep_scenario(uint64_t seed)
{
    SubstepScenario s;
    Gen g{seed * 0x9E3779B97F4A7C15ULL + 3};
    s.subcycles = seed == 0 ? 3 : static_cast<uint64_t>(g.below(7));
    if (seed == 1) s.kinetic = 0.5e3;  // a sub-cutoff parent never builds
    for (uint64_t i = 0; i < s.subcycles + 1; ++i) {
        bool const plain = seed == 0;
        s.build_ok.push_back(plain || g.below(8) != 0);
        s.stop_after_events.push_back(!plain && g.below(8) == 0);
        s.finish_ends.push_back(!plain && g.below(10) == 0);
        s.advance_ok.push_back(plain || g.below(8) != 0);
        s.exits.push_back(!plain && g.below(10) == 0);
    }
    if (seed > 1 && g.below(4) == 0) s.drop_below_cutoff_at = g.below(static_cast<int>(s.subcycles) + 1);
    if (seed > 1 && g.below(6) == 0) s.drop_in_build = g.below(static_cast<int>(s.subcycles) + 1);
    return s;
}

template <class S>
Trace run_substep_scenario(SubstepScenario const& sc)
{
    Trace t;
    double kinetic = sc.kinetic;
    uint64_t completed = 0;
    bool exited = false;
    uint64_t current = 0;
    auto at = [](std::vector<int> const& v, uint64_t i) { return i < v.size() && v[i] != 0; };
    try {
        S::substeps(
            sc.subcycles, kinetic, sc.cutoff, completed, exited,
            [&](uint64_t sub, double& b, double& e) {
                current = sub;
                b = 0.0;
                e = 1.0;
                bool ok = at(sc.build_ok, sub);
                if (static_cast<int>(sub) == sc.drop_in_build) {
                    kinetic = 0.5 * sc.cutoff;
                    ok = false;
                }
                t.put(kBuild, static_cast<double>(sub), ok ? 1.0 : 0.0, kinetic);
                return ok;
            },
            [&](uint64_t sub, double b, double e) { t.put(kEvents, static_cast<double>(sub), b, e); },
            [&] {
                bool const st = at(sc.stop_after_events, current);
                t.put(kStopped, st ? 1.0 : 0.0);
                return st;
            },
            [&](uint64_t sub, double, double) {
                bool ends = at(sc.finish_ends, sub);
                if (static_cast<int>(sub) == sc.drop_below_cutoff_at) kinetic = 0.5 * sc.cutoff;
                t.put(kFinish, static_cast<double>(sub), ends ? 1.0 : 0.0, kinetic);
                return ends;
            },
            [&](double e) {
                bool const ok = at(sc.advance_ok, current);
                t.put(kAdvance, e, ok ? 1.0 : 0.0, static_cast<double>(completed));
                return ok;
            },
            [&] {
                bool const ex = at(sc.exits, current);
                t.put(kExits, ex ? 1.0 : 0.0, static_cast<double>(completed));
                return ex;
            });
    } catch (std::exception const&) {
        t.put(kAbort);
    }
    t.put(kSubEnd, static_cast<double>(completed), exited ? 1.0 : 0.0, kinetic);
    return t;
}

}  // namespace interleave_scenarios
