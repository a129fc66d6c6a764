// minimize.h -- one instance's Simulator::minimize (MC/src/sim.cpp:174-211) as a state
// machine, with every decision in functions that compile for the host and the device.
//
// A solver round gives each instance with work one search direction (stage A), one
// evaluation (stage B: the start point, a line-search candidate or the final state) and the
// decisions that follow it (stage C: the reference's convergence test, Armijo test, halving,
// steepest-descent retry and best-state fallback).  The host-stepped solver calls these
// functions between its launches; the device-resident solver calls the same functions from
// its stage kernels, so both take the same decisions from the same FP64 numbers.
#pragma once

#include <math.h>

#include "kernels.h"

#ifdef __CUDACC__
#define MCG_HD __host__ __device__
#else
#define MCG_HD
#endif

namespace mcg {

constexpr double kMzInf = __builtin_huge_val();

struct HostStats {
    int iterations = 0, backtracks = 0;
    double rms = kMzInf, max = kMzInf, energy = kMzInf;
    bool converged = false;
};

struct Minimizer {
    enum Phase { kIdle, kStart, kIterate, kDirection, kSteepest, kTrial, kFinish, kDone };
    Phase phase = kIdle;
    double top = 0;
    bool zero_first = false;  // z = 0 before the first evaluation (run(): zeroVars, sim.cpp:398)
    bool restore = false;     // z = best before the final evaluation
    HostStats st;
    EvalOut cur{}, cand{}, fin{};
    double cur_rms = 0, cur_max = 0, rms0 = 0, best_energy = 0, dg = 0, step = 1;
    int it = 0, bt = 0;
    bool retry = false;       // in the steepest-descent retry of this iteration
    bool fresh = false;       // the trial is the first of a new direction (dg to be read)
    bool accepted = false;    // the trial of this round passed the Armijo test
};

// The configuration the decisions read.
struct MzParams {
    int max_iterations, max_line_search, H;
    double relative_gradient_tolerance, translation_scale, reaction_relative_tolerance;
    double gradient_rms_tolerance, gradient_max_tolerance, penetration_tolerance;
    double armijo, min_line_step;
    double slack_rel;  // Armijo allowance for energy noise, relative to |E| (mixed form)
};

// Convergence (sim.cpp:177), or the relative-gradient mode rms <= tol rms0.
MCG_HD inline bool mz_converged(const MzParams& p, const EvalOut& o, double rms, double mx, double rms0) {
    if (p.relative_gradient_tolerance > 0)
        return (rms <= p.relative_gradient_tolerance * rms0) && o.max_pen <= p.penetration_tolerance;
    const double rel = rms / fmax(1e-6, p.translation_scale * fmax(1.0, o.reaction));
    const double rrt = p.reaction_relative_tolerance == 0 ? 1.5e-3 : p.reaction_relative_tolerance;
    const bool forceOK = (rms <= p.gradient_rms_tolerance && mx <= p.gradient_max_tolerance) || rel < rrt;
    return forceOK && o.max_pen <= p.penetration_tolerance;
}

// Start of an iteration (sim.cpp:176-177): record, test convergence, continue with a
// direction or finish.
MCG_HD inline void mz_iterate(const MzParams& p, Minimizer& s) {
    using M = Minimizer;
    if (s.it >= p.max_iterations) {
        s.phase = M::kFinish;
        s.restore = !s.st.converged && s.best_energy < s.cur.energy;
        return;
    }
    s.st.iterations = s.it + 1;
    s.st.rms = s.cur_rms;
    s.st.max = s.cur_max;
    s.st.energy = s.cur.energy;
    if (mz_converged(p, s.cur, s.cur_rms, s.cur_max, s.rms0)) {
        s.st.converged = true;
        s.phase = M::kFinish;
        s.restore = false;
        return;
    }
    s.phase = M::kDirection;
}

// Stage A: the operation of the instance's search direction, two-loop (sim.cpp:184-190) or
// the steepest-descent retry (:193-196); 0 when the instance computes none this round.
MCG_HD inline int mz_stage_direction(Minimizer& s, bool fused) {
    using M = Minimizer;
    int flags;
    if (s.phase == M::kDirection) flags = fused ? kOpDirFused : kOpDirection;
    else if (s.phase == M::kSteepest) flags = kOpSteepest;
    else return 0;
    s.phase = M::kTrial;  // first trial of the new direction, step 1
    s.step = 1.0;
    s.bt = 0;
    s.fresh = true;
    return flags;
}

// Stage B: what the instance evaluates this round; 0 when it evaluates nothing.
MCG_HD inline int mz_stage_eval(const Minimizer& s, double& step, bool& trials) {
    using M = Minimizer;
    switch (s.phase) {
        case M::kStart:
            return kOpResetHistory | (s.zero_first ? kOpZero : 0) | kOpEvalAtZ | kOpKeepBest;
        case M::kTrial:
            step = s.step;
            return kOpCandidate;
        case M::kFinish:
            trials = true;
            return (s.restore ? kOpRestore : 0) | kOpEvalAtZ | kOpFinal;
        default:
            return 0;
    }
}

// Stage C: the decisions after the evaluation o (dg: <g, p> of the direction, read on the
// first trial of a direction), and the operations they imply for the accept step.  An
// accepted trial moves on to the next iteration here as well (the curvature pair and the
// history are the device's, sim.cpp:205-206).
MCG_HD inline int mz_stage_decide(const MzParams& p, Minimizer& s, const EvalOut& o, double dg) {
    using M = Minimizer;
    int flags = 0;
    switch (s.phase) {
        case M::kStart:
            s.cur = o;
            s.cur_rms = o.rms;
            s.cur_max = o.gmax;
            s.best_energy = o.energy;
            s.rms0 = o.rms;
            s.it = 0;
            flags = kOpTakeGrad;
            s.phase = M::kIterate;
            break;
        case M::kTrial: {
            if (s.fresh) {
                s.dg = dg;
                s.fresh = false;
            }
            s.cand = o;
            s.st.backtracks++;
            // Armijo (sim.cpp:180), with the mixed form's allowance for its energy noise
            const double slack = p.slack_rel * fabs(s.cur.energy);
            if (isfinite(o.energy) && o.energy <= s.cur.energy + p.armijo * s.step * s.dg + slack) {
                flags = kOpAccept | (p.H > 0 ? kOpPair : 0) | (o.energy < s.best_energy ? kOpKeepBestAfter : 0);
                s.accepted = true;
                break;
            }
            s.step *= .5;
            s.bt++;
            if (!(s.step < p.min_line_step) && s.bt < p.max_line_search) break;
            // line search failed (sim.cpp:193-209)
            if (!s.retry) {
                s.retry = true;
                s.phase = M::kSteepest;
            } else {
                s.phase = M::kFinish;
                s.restore = !s.st.converged && s.best_energy < s.cur.energy;
            }
            break;
        }
        case M::kFinish:
            s.fin = o;
            s.st.rms = o.rms;
            s.st.max = o.gmax;
            s.st.energy = o.energy;
            s.st.converged = mz_converged(p, o, o.rms, o.gmax, s.rms0);
            flags = kOpTakeGrad;
            s.phase = M::kDone;
            break;
        default:
            break;
    }
    if (s.phase == M::kTrial && s.accepted) {
        s.accepted = false;
        s.cur = s.cand;
        s.cur_rms = s.cand.rms;
        s.cur_max = s.cand.gmax;
        if (s.cur.energy < s.best_energy) s.best_energy = s.cur.energy;
        s.retry = false;
        s.it++;
        s.phase = M::kIterate;
    }
    if (s.phase == M::kIterate) mz_iterate(p, s);
    return flags;
}

// ---- the device-resident solver (minimize_dev.cu) --------------------------------------------
// Device view of a round's control: per-instance minimizers, directions' kind, the
// evaluation's active and trial masks, platen heights, and a status word.
struct MzStatus {
    int rounds;     // rounds run by the current launch
    int overflow;   // the last evaluation overflowed a contact buffer (nothing was decided)
    int done;       // an instance finished its minimization
    int pad_;
    // device time of the launch's rounds by stage (global timer, ns): directions (stage A
    // to B), evaluations (B to C, with the vector preparation), decisions and accept steps
    // (C to the next round's A); t_last is the last stage boundary
    unsigned long long t_dir, t_eval, t_post, t_last;
};
struct MzDev {
    int I;
    Minimizer* mins;         // [I]
    const uint8_t* fused;    // [I] the instance's direction is computed by one CTA
    SolveCtl* ctl;           // [I]
    uint8_t* active;         // [I] evaluated this round
    uint8_t* trial_inst;     // [I] writes trial states this round
    double* tops;            // [I]
    const double* dg;        // [I]
    const EvalOut* out;      // [I]
    uint32_t* contact_flags; // the contact pipeline's flags (flags[2]: force a build), or null
    MzStatus* status;
    int round_cap;           // rounds a launch may run before it returns to the host
};
// Stage kernels of one round; each sets the conditional handles of the graph nodes that
// follow it (directions of each kind; the accept step; the loop).
void launch_mz_direction(const MzDev& d, cudaGraphConditionalHandle h_fused, cudaGraphConditionalHandle h_multi,
                         cudaGraphConditionalHandle h_dir, cudaGraphConditionalHandle h_sd, cudaStream_t s);
void launch_mz_eval(const MzDev& d, cudaStream_t s);
void launch_mz_decide(const MzDev& d, const MzParams& p, cudaGraphConditionalHandle h_post,
                      cudaGraphConditionalHandle h_loop, cudaStream_t s);
void launch_mz_reset(const MzDev& d, cudaStream_t s);

}  // namespace mcg
