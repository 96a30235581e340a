// ORACLE — test infrastructure only.  The charged-particle loop skeletons of
// the overlay restated as templates with the reference's policy interface:
//
//   RunChargedEventInterleave   RreaRunChargedEventInterleave
//                               (O/RreaChargedInterleave.H:546-664)
//   RunChargedSubstepInterleave RreaRunChargedSubstepInterleave
//                               (O/RreaChargedInterleave.H:686-732)
//   SelectCompetingHazard       RreaSelectCompetingHazard
//                               (O/RreaParticleInteraction.H:1398-1447)
//   ResolveRemainingSegmentHazard, SplitChargedSegmentAtEvent
//                               (O/RreaParticleInteraction.H:1371-1392, 1449-1492)
//
// The oracle's electron, positron and newborn loops run through these
// templates, and the templates themselves are pinned against the
// reference's own (compiled from its header into oracle/_ref/ref_golden)
// by driving both with the same scripted policies
// (oracle/interleave_scenarios.hpp, tests/test_oracle_interleave.py).
// Where the reference calls amrex::Abort, these call interleave_abort,
// which throws the oracle's error with the matching status code.
//   O/ = native_amrex_rrea/warpx_overlay/Source/Rrea/
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <string>
#include <utility>

namespace oracle {

// Status codes of the skeleton's aborts (rrea_gpu_status values).
enum InterleaveAbort { kAbortOrdinal = 6, kAbortInvalid = 9 };
[[noreturn]] void interleave_abort(int code, std::string const& message);

struct HazardSelection {
    bool valid = false, event = false;
    int channel = -1;
    double sampled = 0.0, total = 0.0;
};

// O/RreaParticleInteraction.H:1398-1447: the first draw is an exponential
// optical depth against the total, the second picks the channel by share.
inline HazardSelection SelectCompetingHazard(std::array<double, 3> const& taus, int count, double u1, double u2)
{
    HazardSelection r;
    if (count < 1 || count > 3 || !std::isfinite(u1) || !std::isfinite(u2)) return r;
    for (int i = 0; i < count; ++i) {
        double const t = taus[static_cast<std::size_t>(i)];
        if (!std::isfinite(t) || t < 0.0) return r;
        r.total += t;
    }
    r.valid = std::isfinite(r.total);
    if (!r.valid) return r;
    u1 = std::max(0.0, std::min(1.0, u1));
    r.sampled = -std::log(std::max(1.0e-30, 1.0 - u1));
    if (!(r.sampled < r.total)) return r;
    r.event = true;
    u2 = std::max(0.0, std::min(1.0, u2));
    double const target = u2 * r.total;
    double cum = 0.0;
    int last_open = -1;
    for (int i = 0; i < count; ++i) {
        double const t = taus[static_cast<std::size_t>(i)];
        if (t > 0.0) last_open = i;
        cum += t;
        if (target < cum) {
            r.channel = i;
            return r;
        }
    }
    r.channel = last_open;  // u2 rounded to one: the last nonzero channel
    r.valid = r.channel >= 0;
    r.event = r.valid;
    return r;
}

// O/RreaParticleInteraction.H:1371-1392: the pieces before and after the
// event share its fraction exactly.
inline bool SplitChargedSegmentAtEvent(double begin, double event, double end)
{
    return std::isfinite(begin) && std::isfinite(event) && std::isfinite(end) && end > begin && !(event < begin)
        && !(event > end);
}

// What a continuous_segment policy returns (the cutoff limiter's verdict).
struct SegmentLimit {
    bool reaches_cutoff = false;
    double effective_end_fraction = 0.0;
};

struct RemainingSegmentHazard {
    HazardSelection selection;
    bool split_valid = false;
    double event_fraction = 0.0;
};

// O/RreaParticleInteraction.H:1459-1492
template <typename DepthToFraction>
RemainingSegmentHazard ResolveRemainingSegmentHazard(std::array<double, 3> const& taus, int count, double begin,
                                                     double end, double u1, double u2, DepthToFraction&& to_fraction)
{
    RemainingSegmentHazard r;
    r.selection = SelectCompetingHazard(taus, count, u1, u2);
    if (!r.selection.valid || !r.selection.event) return r;
    r.event_fraction = to_fraction(r.selection.sampled);
    r.split_valid = SplitChargedSegmentAtEvent(begin, r.event_fraction, end);
    return r;
}

// The repeated competing hazard of one substep, O/RreaChargedInterleave.H:546-664.
// Policies as there:
//   channel_taus(frozen_eV, begin, end) -> std::array<double, 3>
//   hazard_draws(ordinal) -> std::pair<double, double>
//   depth_to_fraction(tau, begin, end) -> double
//   continuous_segment(begin, end, frozen_eV) -> {reaches_cutoff, effective_end_fraction}
//   mark_stopped_at(fraction), event_point_at(fraction)
//   channel_open_at(channel, energy_eV) -> bool
//   final_state(channel, event_fraction) -> bool (false: parent consumed)
template <typename ChannelTaus, typename HazardDraws, typename DepthToFraction, typename ContinuousSegment,
          typename MarkStoppedAt, typename EventPointAt, typename ChannelOpenAt, typename FinalState>
void RunChargedEventInterleave(double begin, double end, double const& kinetic_eV, double cutoff_eV, int channel_count,
                               uint64_t max_ordinal, char const* label, ChannelTaus&& channel_taus,
                               HazardDraws&& hazard_draws, DepthToFraction&& depth_to_fraction,
                               ContinuousSegment&& continuous_segment, MarkStoppedAt&& mark_stopped_at,
                               EventPointAt&& event_point_at, ChannelOpenAt&& channel_open_at,
                               FinalState&& final_state)
{
    double remaining = begin;
    uint64_t ordinal = 0;
    while (remaining < end && kinetic_eV >= cutoff_eV) {
        if (ordinal >= max_ordinal) {
            interleave_abort(kAbortOrdinal, std::string(label) + " event ordinal overflow");
        }
        // rates and depth are refrozen at the survivor energy every iteration
        double const frozen = kinetic_eV;
        std::array<double, 3> const taus = channel_taus(frozen, remaining, end);
        std::pair<double, double> const draws = hazard_draws(ordinal);
        RemainingSegmentHazard const hz = ResolveRemainingSegmentHazard(
            taus, channel_count, remaining, end, draws.first, draws.second,
            [&](double tau) { return depth_to_fraction(tau, remaining, end); });
        if (!hz.selection.valid) interleave_abort(kAbortInvalid, std::string(label) + " hazard selection invalid");
        if (!hz.selection.event) {
            auto const lim = continuous_segment(remaining, end, frozen);
            if (lim.reaches_cutoff) mark_stopped_at(lim.effective_end_fraction);
            break;
        }
        double const ev = hz.event_fraction;
        if (!hz.split_valid) interleave_abort(kAbortInvalid, std::string(label) + " event depth outside its subcycle");
        event_point_at(ev);
        // continuous loss to the exact sampled depth, at the frozen energy
        auto const lim = continuous_segment(remaining, ev, frozen);
        if (lim.reaches_cutoff) {
            mark_stopped_at(lim.effective_end_fraction);
            break;
        }
        bool const open_ev = kinetic_eV >= cutoff_eV && channel_open_at(hz.selection.channel, kinetic_eV);
        if (!open_ev) {
            bool const open_fr = frozen >= cutoff_eV && channel_open_at(hz.selection.channel, frozen);
            if (!open_fr) interleave_abort(kAbortInvalid, std::string(label) + " channel closed before its event");
            remaining = ev;  // a null event on a new ordinal
            ++ordinal;
            continue;
        }
        if (!final_state(hz.selection.channel, ev)) return;  // parent consumed
        if (kinetic_eV <= cutoff_eV) {
            mark_stopped_at(ev);
            break;
        }
        remaining = ev;
        ++ordinal;
    }
}

// The substep skeleton of one charged step, O/RreaChargedInterleave.H:686-732:
// build, events, (stop check), finish, advance, exit check; completed
// counts only fully committed substeps and an exit is sticky.
template <typename BuildSubstep, typename RunEvents, typename StoppedMidChord, typename FinishSubstep,
          typename AdvancePosition, typename PathExitsDomain>
void RunChargedSubstepInterleave(uint64_t subcycles, double const& kinetic_eV, double cutoff_eV, uint64_t& completed,
                                 bool& exited, BuildSubstep&& build_substep, RunEvents&& run_events,
                                 StoppedMidChord&& stopped_mid_chord, FinishSubstep&& finish_substep,
                                 AdvancePosition&& advance_position, PathExitsDomain&& path_exits_domain)
{
    for (uint64_t sub = 0; sub < subcycles; ++sub) {
        if (kinetic_eV < cutoff_eV) break;
        double b = 0.0, e = 0.0;
        if (!build_substep(sub, b, e)) break;
        run_events(sub, b, e);
        if (stopped_mid_chord()) break;
        if (finish_substep(sub, b, e)) break;
        if (!advance_position(e)) {
            exited = true;
            break;
        }
        if (path_exits_domain()) {
            exited = true;
            break;
        }
        completed = sub + 1U;
    }
}

}  // namespace oracle
