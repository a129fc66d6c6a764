// minimize_dev.cu -- the stage kernels of the device-resident solver round.
//
// One round of Simulator::minimize (MC/src/sim.cpp:174-211) for every instance, as the
// body of a CUDA-graph WHILE node: stage A (directions), stage B (what to evaluate), the
// evaluation, stage C (decisions).  Each stage kernel runs the decision functions of
// minimize.h -- the ones the host-stepped solver calls -- over the instances' minimizers,
// writes their control records and sets the conditional handles of the graph nodes that
// follow: the kinds of direction computed this round, the accept step, and the loop itself.
// The loop runs while some instance is still minimizing and none has finished (the host
// commits finished instances and starts their next increment), up to a round cap.  No
// kernel waits on another: the graph orders them.
#include "minimize.h"

namespace mcg {

namespace {

constexpr int kMzThreads = 256;  // one block walks all instances

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Adds the time since the last stage boundary to *acc and moves the boundary (thread 0).
__device__ __forceinline__ void stage_mark(MzStatus* st, unsigned long long* acc) {
    const unsigned long long t = global_ns();
    if (st->t_last && acc) *acc += t - st->t_last;
    st->t_last = t;
}

__global__ void __launch_bounds__(kMzThreads) k_mz_direction(MzDev d, cudaGraphConditionalHandle h_fused,
                                                             cudaGraphConditionalHandle h_multi,
                                                             cudaGraphConditionalHandle h_dir,
                                                             cudaGraphConditionalHandle h_sd) {
    int fused = 0, multi = 0, sd = 0;
    for (int i = threadIdx.x; i < d.I; i += blockDim.x) {
        Minimizer s = d.mins[i];
        const int f = mz_stage_direction(s, d.fused[i] != 0);
        if (f) d.mins[i] = s;
        d.ctl[i] = SolveCtl{0.0, f, 0, 0, 0};
        fused |= f == kOpDirFused;
        multi |= f == kOpDirection;
        sd |= f == kOpSteepest;
    }
    fused = __syncthreads_or(fused);
    multi = __syncthreads_or(multi);
    sd = __syncthreads_or(sd);
    if (threadIdx.x == 0) {
        stage_mark(d.status, &d.status->t_post);
        cudaGraphSetConditional(h_fused, fused ? 1u : 0u);
        cudaGraphSetConditional(h_multi, multi ? 1u : 0u);
        cudaGraphSetConditional(h_dir, (fused | multi) ? 1u : 0u);
        cudaGraphSetConditional(h_sd, sd ? 1u : 0u);
    }
}

__global__ void __launch_bounds__(kMzThreads) k_mz_eval(MzDev d) {
    int joined = 0;
    for (int i = threadIdx.x; i < d.I; i += blockDim.x) {
        const Minimizer s = d.mins[i];
        double step = 0.0;
        bool trials = false;
        const int f = mz_stage_eval(s, step, trials);
        d.ctl[i] = SolveCtl{step, f, 0, 0, 0};
        const uint8_t a = f ? 1 : 0;
        joined |= a && !d.active[i];  // a joining instance needs its shapes in the candidate list
        d.active[i] = a;
        d.trial_inst[i] = trials ? 1 : 0;
        if (a) d.tops[i] = s.top;
    }
    joined = __syncthreads_or(joined);
    if (threadIdx.x == 0) {
        stage_mark(d.status, &d.status->t_dir);
        if (joined && d.contact_flags) d.contact_flags[2] = 1u;
    }
}

__global__ void __launch_bounds__(kMzThreads) k_mz_decide(MzDev d, MzParams p, cudaGraphConditionalHandle h_post,
                                                          cudaGraphConditionalHandle h_loop) {
    // an evaluation that overflowed a contact buffer decided nothing: the host grows the
    // buffers and the next launch repeats the round's evaluation (stages A and B leave the
    // minimizers ready for it)
    if (threadIdx.x == 0) stage_mark(d.status, &d.status->t_eval);
    if (d.out[0].overflow) {
        if (threadIdx.x == 0) {
            d.status->overflow = 1;
            cudaGraphSetConditional(h_post, 0u);
            cudaGraphSetConditional(h_loop, 0u);
        }
        return;
    }
    int post = 0, done = 0, running = 0;
    for (int i = threadIdx.x; i < d.I; i += blockDim.x) {
        Minimizer s = d.mins[i];
        const int f = mz_stage_decide(p, s, d.out[i], d.dg[i]);
        d.mins[i] = s;
        d.ctl[i] = SolveCtl{0.0, f, 0, 0, 0};
        post |= f != 0;
        done |= s.phase == Minimizer::kDone;
        running |= s.phase != Minimizer::kDone && s.phase != Minimizer::kIdle;
    }
    post = __syncthreads_or(post);
    done = __syncthreads_or(done);
    running = __syncthreads_or(running);
    if (threadIdx.x == 0) {
        const int rounds = ++d.status->rounds;
        if (done) d.status->done = 1;
        cudaGraphSetConditional(h_post, post ? 1u : 0u);
        cudaGraphSetConditional(h_loop, (!done && running && rounds < d.round_cap) ? 1u : 0u);
    }
}

__global__ void k_mz_reset(MzStatus* st) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *st = MzStatus{0, 0, 0, 0, 0, 0, 0, 0};
}

}  // namespace

void launch_mz_direction(const MzDev& d, cudaGraphConditionalHandle h_fused, cudaGraphConditionalHandle h_multi,
                         cudaGraphConditionalHandle h_dir, cudaGraphConditionalHandle h_sd, cudaStream_t s) {
    k_mz_direction<<<1, kMzThreads, 0, s>>>(d, h_fused, h_multi, h_dir, h_sd);
    note_launches(1);
}

void launch_mz_eval(const MzDev& d, cudaStream_t s) {
    k_mz_eval<<<1, kMzThreads, 0, s>>>(d);
    note_launches(1);
}

void launch_mz_decide(const MzDev& d, const MzParams& p, cudaGraphConditionalHandle h_post,
                      cudaGraphConditionalHandle h_loop, cudaStream_t s) {
    k_mz_decide<<<1, kMzThreads, 0, s>>>(d, p, h_post, h_loop);
    note_launches(1);
}

void launch_mz_reset(const MzDev& d, cudaStream_t s) {
    k_mz_reset<<<1, 32, 0, s>>>(d.status);
    note_launches(1);
}

}  // namespace mcg
