// tuner.h -- online autotuner of the gradient kernel's tile-table shape rule.
//
// Opt-in (sad_train_config_t::autotune): on the 256^2-1024^2 fits the arms differ by 1-2%
// of the fit, about what two 8-iteration windows per arm can resolve, and the tuned fits
// came out no faster than the fixed default rule (1024^2: 545 vs 543 ms; 512^2: 132.3 vs
// 129.2 ms, where it settled on "never wide"; 256^2: 46.4 vs 46.2 ms).
//
// Each candidate-field refresh registers every 16x16 tile's keys once (register_tiles_kernel)
// and gives the tile one of two word-table shapes (accum.cuh: TileWords): narrow (four
// copies of 128 entries, far entries through global atomics) or wide (two copies of 256
// entries).  A tile is wide when more than `rule` of its (pixel, candidate) references name
// far entries.  Every rule gives the same fixed-point sums -- the fit is bit-identical --
// but which rule is fastest depends on the image size, the site density and the phase of
// the fit (measured on the 1024^2 fit: never wide is 1% faster; on 512^2 and 256^2 a low
// rule is 1-2% faster).  So the trainer tunes it while it fits:
//
//   * a round times one refresh window per arm, in palindromic order (a b c d d c b a, so a
//     drift of the fit's cost over the round weighs every arm alike).  A window runs from
//     the iteration after a refresh (the first to use the field registered with the arm) to
//     the iteration after the next refresh; it is timed with two CUDA events recorded on
//     the trainer's stream between iterations, so graph replays need no re-capture.  Only
//     windows without a densify or prune step, and that end inside the current run call,
//     are timed; others run the best arm so far and the round resumes at the next clean one;
//   * when the round's last window is recorded the host waits for it (one synchronisation
//     per round), sums each arm's two windows and keeps the fastest until the next round;
//   * rounds start at the second refresh window and then every kRoundInterval iterations,
//     so the choice follows the fit from its dense start to its sparse end.
//
// The rule lives in the trainer's device state (DevState::wide_far_refs); a one-thread
// kernel on the trainer's stream sets it before the refresh that registers with it.
#pragma once

#include <algorithm>
#include <cuda_runtime.h>
#include <vector>

#include "accum.cuh"
#include "kernels.h"

namespace sad {

class ShapeTuner {
public:
    static constexpr int kArms = 4;
    // rules tried: wide at 64 far references, at 256 (the default), at 1024, and never
    static constexpr int kArmRule[kArms] = {64, kWideFarRefs, 1024, 1 << 29};
    static constexpr int kRoundWindows = 2 * kArms;
    static constexpr int kRoundInterval = 1024;

    ShapeTuner() = default;
    ShapeTuner(const ShapeTuner&) = delete;
    ShapeTuner& operator=(const ShapeTuner&) = delete;
    ~ShapeTuner() { release(); }

    // A new fit: the default rule on the device (set by the state reset), no rounds yet.
    void reset(bool enabled, int refresh_every) {
        enabled_ = enabled;
        best_ = kWideFarRefs;
        current_ = kWideFarRefs;
        rounds_ = 0;
        next_round_at_ = 2 * std::max(1, refresh_every);
        abort_round();
    }

    int rule() const { return current_; }
    int rounds() const { return rounds_; }

    // Called by the run loop before it launches iteration `it` on stream s; plan is the
    // fit's schedule (upd / dens / prune per iteration), state its device state, `end` the
    // last iteration (exclusive) of this run call.  Returns a CUDA error, if any.
    template <class Plan>
    cudaError_t before_iteration(const std::vector<Plan>& plan, DevState* state, int it, int end,
                                 cudaStream_t s) {
        if (!enabled_) return cudaSuccess;
        cudaError_t e = cudaSuccess;
        if (active_) {
            // a window ending here, then one starting here (consecutive windows share the
            // boundary; the end is recorded first)
            for (int w = 0; w < kRoundWindows; ++w) {
                if (win_[w].state == kOpen && win_[w].end == it) {
                    if ((e = cudaEventRecord(ev_[2 * w + 1], s)) != cudaSuccess) return fail(e);
                    win_[w].state = kClosed;
                    if (w == kRoundWindows - 1) {
                        if ((e = finish_round()) != cudaSuccess) return fail(e);
                        next_round_at_ = it + kRoundInterval;
                    }
                }
            }
            for (int w = 0; active_ && w < kRoundWindows; ++w) {
                if (win_[w].state == kAssigned && win_[w].start == it) {
                    if ((e = cudaEventRecord(ev_[2 * w], s)) != cudaSuccess) return fail(e);
                    win_[w].state = kOpen;
                }
            }
        }
        if (!plan[it].upd) return cudaSuccess;
        if (!active_ && it >= next_round_at_) {
            if ((e = ensure_events()) != cudaSuccess) return fail(e);
            active_ = true;
            assign_ = 0;
        }
        int rule = best_;
        if (active_ && assign_ < kRoundWindows) {
            const int next = next_refresh(plan, it);
            // the window [it + 1, next + 1) runs on the field registered in this iteration;
            // it must hold no densify or prune step and close inside this run call
            if (next > it && next + 1 < end && clean(plan, it, next + 1)) {
                Window& w = win_[assign_++];
                w.start = it + 1;
                w.end = next + 1;
                w.state = kAssigned;
                rule = kArmRule[arm_of(static_cast<int>(&w - win_))];
            }
        }
        if (rule != current_) {
            launch_set_wide_far_refs(state, rule, s);
            current_ = rule;
        }
        return cudaSuccess;
    }

    // The run call ends: windows not yet closed are dropped (the next call may come after
    // an idle gap) and are assigned again at the next clean refreshes of the round.
    void end_run() {
        if (!active_) return;
        for (int w = 0; w < kRoundWindows; ++w) {
            if (win_[w].state == kAssigned || win_[w].state == kOpen) {
                win_[w].state = kUnused;
                assign_ = std::min(assign_, w);
            }
        }
    }

private:
    enum { kUnused, kAssigned, kOpen, kClosed };
    struct Window {
        int start = 0, end = 0;  // iterations [start, end)
        int state = kUnused;
    };

    static int arm_of(int window) { return window < kArms ? window : kRoundWindows - 1 - window; }

    template <class Plan>
    static int next_refresh(const std::vector<Plan>& plan, int it) {
        for (int j = it + 1; j < static_cast<int>(plan.size()); ++j)
            if (plan[j].upd) return j;
        return -1;
    }
    template <class Plan>
    static bool clean(const std::vector<Plan>& plan, int from, int to) {
        for (int j = from; j < to && j < static_cast<int>(plan.size()); ++j)
            if (plan[j].dens || plan[j].prune) return false;
        return true;
    }

    cudaError_t ensure_events() {
        if (!ev_.empty()) return cudaSuccess;
        ev_.assign(2 * kRoundWindows, nullptr);
        for (auto& ev : ev_) {
            cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    cudaError_t finish_round() {
        cudaError_t e = cudaEventSynchronize(ev_[2 * kRoundWindows - 1]);
        if (e != cudaSuccess) return e;
        float total[kArms] = {};
        for (int w = 0; w < kRoundWindows; ++w) {
            float ms = 0.0f;
            if ((e = cudaEventElapsedTime(&ms, ev_[2 * w], ev_[2 * w + 1])) != cudaSuccess) return e;
            total[arm_of(w)] += ms;
        }
        int b = 0;
        for (int a = 1; a < kArms; ++a)
            if (total[a] < total[b]) b = a;
        best_ = kArmRule[b];
        rounds_ += 1;
        abort_round();
        return cudaSuccess;
    }

    void abort_round() {
        active_ = false;
        assign_ = 0;
        for (Window& w : win_) w = Window{};
    }

    // a failed CUDA call ends tuning for this fit (every rule gives the same sums)
    cudaError_t fail(cudaError_t e) {
        enabled_ = false;
        abort_round();
        return e;
    }

    void release() {
        for (cudaEvent_t ev : ev_)
            if (ev) cudaEventDestroy(ev);
        ev_.clear();
    }

    bool enabled_ = false, active_ = false;
    int best_ = kWideFarRefs, current_ = kWideFarRefs;
    int rounds_ = 0, next_round_at_ = 0;
    int assign_ = 0;  // next window of the round to assign an arm
    Window win_[kRoundWindows];
    std::vector<cudaEvent_t> ev_;
};

}  // namespace sad
