// context.cpp -- the C ABI (include/mcg.h): device context, topology upload, the
// energy/gradient evaluation, the L-BFGS minimizer and the load/unload driver.
//
// The solver logic follows the reference's Simulator::minimize / commit / run
// (MC/src/sim.cpp:174-213, 312-467) decision for decision; the vectors live on the device
// and only the scalars each decision needs are read back.
//
// A context holds I lattices (instances): one for the plain API, many for the batched sweep.
// Every evaluation evaluates all of them in the same launches, and the minimizer and the
// load/unload driver are per-instance state machines stepped together: in each round every
// instance that needs one gets its direction, its next candidate and one evaluation, and
// decides as the reference would.  An instance's arithmetic does not depend on the others,
// so a lattice solved in a batch gives bit for bit what it gives alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mcg.h"
#include "kernels.h"
#include "minimize.h"

namespace mcg {
std::atomic<long long> g_launch_count{0};
}

using namespace mcg;

namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();

struct Fail : std::runtime_error {
    int code;
    Fail(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Smallest float not below x.
float round_up_float(double x) {
    float f = float(x);
    if (double(f) < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Fail(MCG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
void h2d(T* d, const T* h, size_t n, cudaStream_t s) {
    if (n) ck(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, s), "copy to device");
}
template <class T>
void d2h(T* h, const T* d, size_t n, cudaStream_t s) {
    if (n) ck(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, s), "copy to host");
}

struct DevArena {
    std::vector<void*> ptrs;
    template <class T>
    T* get(size_t n) {
        void* p = nullptr;
        ck(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    void release() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
    ~DevArena() { release(); }
};

// Page-locked staging for the per-instance scalars the host reads and writes every round.
struct Pinned {
    void* base = nullptr;
    EvalOut* outs = nullptr;   // [I]
    double* tops = nullptr;    // [I]
    SolveCtl* ctl = nullptr;   // [3 I]: the three uploads of a solver round (directions,
                               // evaluation, accept) each have their own, so none is
                               // rewritten before its copy has run
    double* dg = nullptr;      // [I]
    double* pstats = nullptr;  // [6 I]
    double* cen = nullptr;     // [9 (I + 1)]
    uint32_t* u32 = nullptr;   // [8]
    Minimizer* mins = nullptr; // [I] the device-resident solver's minimizers, in and out
    MzStatus* mz = nullptr;    // its status word
    void alloc(int I) {
        release();
        const size_t bytes = I * sizeof(EvalOut) + 3 * I * sizeof(SolveCtl) +
                             sizeof(double) * (I + I + 6 * I + 9 * (I + 1)) + 8 * 4 + I * sizeof(Minimizer) +
                             sizeof(MzStatus) + 1024;
        ck(cudaMallocHost(&base, bytes), "cudaMallocHost");
        std::memset(base, 0, bytes);
        char* p = static_cast<char*>(base);
        auto take = [&](size_t b) {
            char* r = p;
            p += (b + 15) & ~size_t(15);
            return r;
        };
        outs = reinterpret_cast<EvalOut*>(take(I * sizeof(EvalOut)));
        ctl = reinterpret_cast<SolveCtl*>(take(3 * I * sizeof(SolveCtl)));
        tops = reinterpret_cast<double*>(take(I * sizeof(double)));
        dg = reinterpret_cast<double*>(take(I * sizeof(double)));
        pstats = reinterpret_cast<double*>(take(6 * I * sizeof(double)));
        cen = reinterpret_cast<double*>(take(9 * (I + 1) * sizeof(double)));
        u32 = reinterpret_cast<uint32_t*>(take(8 * sizeof(uint32_t)));
        mins = reinterpret_cast<Minimizer*>(take(I * sizeof(Minimizer)));
        mz = reinterpret_cast<MzStatus*>(take(sizeof(MzStatus)));
    }
    void release() {
        if (base) cudaFreeHost(base);
        base = nullptr;
    }
    ~Pinned() { release(); }
};

// Energy noise allowance of the mixed form's line search, relative to |E| (the state
// machine of one instance's Simulator::minimize is in minimize.h).
constexpr double kMixedArmijoSlack = 1e-9;

// One instance of the load/unload driver (Simulator::run, MC/src/sim.cpp:374-467).
struct Task {
    double top;
    bool loading;
    int refinement;
};
struct Runner {
    bool done = false;
    int status = MCG_OK;
    std::string error;
    int next_step = 0;  // 0: the settle at top0, then load steps, then unload steps
    std::vector<Task> stack;
    Task task{};
    double time = 0, currentTop = 0;
    bool first = true;
    int accepted = 0;
    double loadingWork = 0, recoveredWork = 0, prevDisp = 0, prevForce = 0, reactionOffset = 0;
    std::vector<mcg_frame> frames;
};

// Host description of one instance.
struct InstHost {
    int node0 = 0, N = 0, beam0 = 0, B = 0;
    long long n_free = 0;
    mcg_geometry geom{};
    double sy = 0;
    float2 off{0.f, 0.f};
};

// One instance's input to the upload.
struct InstIn {
    const mcg_topology* t;
    const mcg_geometry* g;
    const double* x0;
    const double* r0;
    double sy;
};

}  // namespace

struct mcg_ctx {
    mcg_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int N = 0, B = 0, I = 0;
    std::vector<InstHost> inst;
    bool have_topo = false;
    double jr = 0, rmax = 0;

    DevArena topo_mem, eval_mem, contact_mem, solver_mem;
    DevTopo topo{};
    Material mat{};
    PhysParams phys{};
    EvalBufs ev{};
    ContactBufs cb{};
    long long last_contacts = 0;
    // The last evaluation was mcg_objective_noalloc's: its contacts lived in the shared
    // fixed scratch, so the pair and statistics queries have nothing current to report.
    bool contacts_stale = false;
    // Device address of mcg_objective_noalloc's fixed scratch on this context's device,
    // looked up by that entry point's first call on this context (noalloc.cu).
    void* noalloc_scratch = nullptr;
    Pinned hp;

    double *d_baseX = nullptr, *d_baseR = nullptr, *d_plastic = nullptr;
    bool mixed = false;  // MCG_MIXED: FP32 bulk arithmetic (objective_mixed.cu)
    MixedBeams mb{};
    MixedNodes mn{};
    // Re-derives the mixed form's per-increment base terms after the base state changed.
    void rebase() {
        if (mixed) launch_rebase_mixed(topo, d_baseX, d_baseR, mb, mn, stream);
    }
    double *d_zin = nullptr, *d_grad = nullptr;

    // solver vectors (all instances), history H slots of 6N, per-instance scalars
    int H = 0;
    double *d_z = nullptr, *d_zeval = nullptr, *d_p = nullptr, *d_g = nullptr, *d_geval = nullptr,
           *d_best = nullptr, *d_zfinal = nullptr, *d_S = nullptr, *d_Y = nullptr;
    double *d_rho = nullptr, *d_alpha = nullptr, *d_part = nullptr, *d_dg = nullptr, *d_dots3 = nullptr,
           *d_pstats = nullptr;
    SolveCtl* d_ctl = nullptr;
    int2* d_hist = nullptr;       // per instance: history pairs held, oldest slot
    uint8_t* d_mask = nullptr;
    uint8_t *d_active = nullptr, *d_all = nullptr;  // instances evaluated / all instances
    std::vector<uint8_t> active;                    // host copy of d_active
    // Evaluates only the instances with a[i] != 0 from now on.  An instance that joins
    // needs its shapes in the contact candidate list: the next evaluation rebuilds it.
    void set_active(const std::vector<uint8_t>& a) {
        if (a == active) return;
        bool joined = false;
        for (int i = 0; i < I; i++) joined |= a[size_t(i)] && active[size_t(i)] != 1;  // 2: unknown
        active = a;
        h2d(d_active, active.data(), size_t(I), stream);
        if (joined) ck(cudaMemsetAsync(cb.flags + 2, 1, 1, stream), "memset");
        sync();  // the host vector may change before the copy runs
    }
    std::vector<Minimizer> mins;
    std::vector<uint8_t> fused;  // the instance's direction is computed by one CTA
    bool have_final = false;  // instance 0 has a final state from minimize, not yet committed

    // ---- the device-resident round loop ------------------------------------------------
    // Rounds run as the body of a CUDA-graph WHILE node (minimize_dev.cu): the host launches
    // the loop once and reads the minimizers back when an instance has finished (or a round
    // cap was reached, or an evaluation overflowed a contact buffer), instead of
    // synchronising after every round.  Off while timing phases (direct launches) or when
    // the graph cannot be built (loop_error says why); the host-stepped rounds then run.
    Minimizer* d_mins = nullptr;
    uint8_t* d_fused = nullptr;
    uint8_t* d_trial = nullptr;   // per-instance trial mask of the loop's evaluations
    MzStatus* d_mz = nullptr;
    cudaGraphExec_t loop_exec = nullptr;
    cudaStream_t side = nullptr;  // captures the bodies of the loop's conditional nodes
    bool device_loop = true;
    std::string loop_error;
    static constexpr int kLoopRoundCap = 4096;
    // the loop's device time by stage (ns; minimize_dev.cu), its rounds, and the host's wall
    // time from each loop launch to the synchronisation that ends it
    unsigned long long loop_ns[3] = {0, 0, 0};
    long long loop_rounds = 0;
    double loop_wall_ms = 0;

    // optional per-phase timing of evaluations (events on the context stream)
    // state, beams, contact grid (up to the pair enumeration), pair enumeration (k_bin_pairs),
    // narrow phase and contact lists, gather, finalize
    static constexpr int kPhases = 7;
    bool timing = false;
    cudaEvent_t ev_t[kPhases + 1] = {};
    double phase_ms[kPhases] = {};
    long long phase_n = 0;
    void mark(int k) {
        if (timing) ck(cudaEventRecord(ev_t[k], stream), "cudaEventRecord");
    }
    void collect() {
        if (!timing) return;
        ck(cudaEventSynchronize(ev_t[kPhases]), "cudaEventSynchronize");
        for (int k = 0; k < kPhases; k++) {
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, ev_t[k], ev_t[k + 1]), "cudaEventElapsedTime");
            phase_ms[k] += ms;
        }
        phase_n++;
    }

    ~mcg_ctx() {
        drop_graphs();
        for (auto& e : ev_t)
            if (e) cudaEventDestroy(e);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    void set_device() { ck(cudaSetDevice(device), "cudaSetDevice"); }
    void sync() { ck(cudaStreamSynchronize(stream), "stream sync"); }
    void check_launch() { ck(cudaGetLastError(), "kernel launch"); }

    // occupancy variants of the beam kernel and the gather (shape_blocks), picked by
    // mcg_autotune; results do not depend on them
    int beam_variant = 0, gather_variant = 0;
    void set_kernel_variants(int beams, int gather) {
        if (beams != beam_variant || gather != gather_variant) drop_graphs();
        beam_variant = beams;
        gather_variant = gather;
    }

    // ---- contact buffers ---------------------------------------------------------------
    double broad_cell = 0;   // current grid cell (the reference's size unless coarsened)
    float contact_skin = 0;  // candidate-list reuse distance (m); 0 rebuilds every evaluation
    int pair_blocks_set = 0; // blocks of the pair enumeration; 0: contact_pair_blocks(shapes)
    double default_cell() const { return std::max(2.8 * jr, .72 * cfg.cell_size); }
    int pair_blocks_for(long long shapes) const {
        return pair_blocks_set > 0 ? pair_blocks_set : contact_pair_blocks(shapes);
    }
    // bin_slots: entries a grid bin holds (rounded up to a power of two, at least 8)
    long long builds_before = 0;  // candidate-list builds counted by buffers since released
    void alloc_contacts(long long bin_slots, long long contact_cap, long long bin_cap, long long cand_cap) {
        drop_graphs();
        if (cb.flags) {
            d2h(hp.u32, cb.flags + 4, 1, stream);
            sync();
            builds_before += hp.u32[0];
        }
        contact_mem.release();
        const long long S = (long long)N + B;
        ContactBufs c{};
        c.cell_lo = contact_mem.get<int4>(size_t(S));
        c.cell_hi = contact_mem.get<int4>(size_t(S));
        c.rec = contact_mem.get<uint4>(size_t(S));
        c.grid = contact_mem.get<int>(16);
        c.flags = contact_mem.get<uint32_t>(5);
        c.xref = contact_mem.get<float4>(size_t(std::max(N, 1)));
        int slots = 8;
        while (slots < bin_slots && slots < (1 << 20)) slots <<= 1;
        c.bin_slots = slots;
        c.bin_cap = bin_cap;
        c.bin_count = contact_mem.get<uint32_t>(size_t(bin_cap + 1));
        c.bin_items = contact_mem.get<uint32_t>(size_t(bin_cap) * size_t(slots));
        c.nentries = contact_mem.get<uint32_t>(3);
        c.pair_blocks = pair_blocks_for(S);
        c.cand_cap = std::max<long long>(1024, (cand_cap + 31) / 32 * 32);
        c.cand = contact_mem.get<uint2>(size_t(c.cand_cap));
        c.ncand = contact_mem.get<uint32_t>(1);
        const long long chunks = c.cand_cap / 32;
        c.cand2 = contact_mem.get<uint2>(size_t(c.cand_cap));
        c.fbits = contact_mem.get<uint32_t>(size_t(chunks));
        c.fcount = contact_mem.get<uint32_t>(size_t(chunks + 1));
        c.foff = contact_mem.get<uint32_t>(size_t(chunks + 1));
        c.hitbits = contact_mem.get<uint32_t>(size_t(chunks));
        c.hcount = contact_mem.get<uint32_t>(size_t(chunks + 1));
        c.hoff = contact_mem.get<uint32_t>(size_t(chunks + 1));
        c.contact_cap = contact_cap;
        c.c_a = contact_mem.get<uint32_t>(size_t(contact_cap));
        c.c_b = contact_mem.get<uint32_t>(size_t(contact_cap));
        c.c_s = contact_mem.get<double>(size_t(contact_cap));
        c.c_t = contact_mem.get<double>(size_t(contact_cap));
        c.c_n = contact_mem.get<double>(size_t(3 * contact_cap));
        c.c_pen = contact_mem.get<double>(size_t(contact_cap));
        c.n_count = contact_mem.get<uint32_t>(size_t(N + 1));
        c.n_start = contact_mem.get<uint32_t>(size_t(N + 1));
        c.n_cursor = contact_mem.get<uint32_t>(size_t(N));
        c.n_items = contact_mem.get<uint32_t>(size_t(4 * contact_cap));
        c.n_sorted = contact_mem.get<uint32_t>(size_t(4 * contact_cap));
        c.n_long = contact_mem.get<uint32_t>(size_t(N + 1));
        c.long_sum = contact_mem.get<double>(6 * size_t(std::max(N, 1)));
        c.scan_tmp_bytes = scan_tmp_bytes(std::max({(long long)N + 1, chunks + 1}));
        c.scan_tmp = contact_mem.get<unsigned char>(c.scan_tmp_bytes);
        ck(cudaMemsetAsync(c.flags, 0, 5 * sizeof(uint32_t), stream), "memset");
        ck(cudaMemsetAsync(c.ncand, 0, sizeof(uint32_t), stream), "memset");
        ck(cudaMemsetAsync(c.nentries, 0, 3 * sizeof(uint32_t), stream), "memset");
        ck(cudaMemsetAsync(c.flags + 2, 1, 1, stream), "memset");  // the first evaluation builds the list
        cb = c;
    }
    long long contact_chunks() const { return cb.cand_cap / 32; }

    // Grows whatever the last evaluation overflowed; false when nothing did.
    bool grow_contacts(int flags) {
        if (!(flags & (kOverEntries | kOverContacts | kOverBins | kOverSpan | kOverCandidates))) return false;
        uint32_t need[3] = {0, 0, 0};
        int grid[16];
        ck(cudaMemcpyAsync(&need[0], cb.nentries + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "copy");
        ck(cudaMemcpyAsync(&need[1], cb.hoff + contact_chunks(), sizeof(uint32_t), cudaMemcpyDeviceToHost, stream),
           "copy");
        ck(cudaMemcpyAsync(&need[2], cb.ncand, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "copy");
        ck(cudaMemcpyAsync(grid, cb.grid, sizeof(grid), cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        long long slots = cb.bin_slots, ccap = cb.contact_cap, bcap = cb.bin_cap, kcap = cb.cand_cap;
        if (flags & kOverCandidates) kcap = std::max(kcap, (long long)need[2] + need[2] / 4 + 1024);
        if (flags & kOverSpan) broad_cell *= 2;
        if (flags & kOverEntries) slots = std::max(slots, (long long)need[0] + need[0] / 4);
        if (flags & kOverContacts) ccap = std::max(ccap, (long long)need[1] + need[1] / 4 + 1024);
        if (flags & kOverBins) {
            const long long want = (long long)grid[9] + grid[9] / 4 + 1024;
            if (want <= (1LL << 28)) bcap = std::max(bcap, want);
            else broad_cell *= 2;  // a huge extent: coarser cells instead of more bins
        }
        alloc_contacts(slots, ccap, bcap, kcap);
        return true;
    }

    // ---- evaluation ----------------------------------------------------------------------
    // Platen heights of all instances from hp.tops (the host changes them only after a sync).
    void upload_tops() { h2d(ev.tops, hp.tops, size_t(I), stream); }

    // Captured evaluations: the launch sequence of eval_launches for one (z, gradient,
    // trials) combination, replayed as one graph.  Any change of what the launches bake in
    // (contact buffers, grid cell, skin) drops them.
    struct EvalGraph {
        const double* dz;
        double* d_gout;
        bool trials;
        cudaGraphExec_t exec;
        long long kernels;  // kernel launches a replay performs
    };
    std::vector<EvalGraph> graphs;
    bool use_graphs = true;
    // Solver launch sequences (directions, vectors around an evaluation, accepts): their
    // kernels read what to do from the control records on the device, so one capture per
    // sequence variant serves every round.
    struct SeqGraph {
        int key;
        cudaGraphExec_t exec;
        long long kernels;
    };
    std::vector<SeqGraph> seq_graphs;
    void drop_graphs() {
        if (loop_exec) cudaGraphExecDestroy(loop_exec);
        loop_exec = nullptr;
        for (EvalGraph& g : graphs) cudaGraphExecDestroy(g.exec);
        graphs.clear();
        for (SeqGraph& g : seq_graphs) cudaGraphExecDestroy(g.exec);
        seq_graphs.clear();
    }
    // Captures launches() once per key and replays it (runs it directly while timing).
    template <typename F>
    void replay(int key, F&& launches) {
        if (!use_graphs || timing) {
            launches();
            return;
        }
        const SeqGraph* found = nullptr;
        for (const SeqGraph& g : seq_graphs)
            if (g.key == key) found = &g;
        if (!found) {
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            const long long before = g_launch_count.load();
            ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
            launches();
            ck(cudaStreamEndCapture(stream, &graph), "cudaStreamEndCapture");
            const long long kernels = g_launch_count.load() - before;
            g_launch_count -= kernels;
            const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            ck(e, "cudaGraphInstantiate");
            seq_graphs.push_back(SeqGraph{key, exec, kernels});
            found = &seq_graphs.back();
        }
        ck(cudaGraphLaunch(found->exec, stream), "cudaGraphLaunch");
        note_launches(int(found->kernels));
    }

    // One evaluation of every instance at device z; grad written to d_gout; totals in
    // ev.out[0..I).  Enqueues only: no host synchronisation.
    void eval(const double* dz, bool trials, double* d_gout) {
        if (!use_graphs || timing) {
            eval_launches(dz, trials, d_gout);
        } else {
            const EvalGraph* found = nullptr;
            for (const EvalGraph& g : graphs)
                if (g.dz == dz && g.d_gout == d_gout && g.trials == trials) found = &g;
            if (!found) {
                cudaGraph_t graph = nullptr;
                cudaGraphExec_t exec = nullptr;
                const long long before = g_launch_count.load();
                ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
                eval_launches(dz, trials, d_gout);
                ck(cudaStreamEndCapture(stream, &graph), "cudaStreamEndCapture");
                const long long kernels = g_launch_count.load() - before;
                g_launch_count -= kernels;  // counted when the graph runs
                const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                ck(e, "cudaGraphInstantiate");
                graphs.push_back(EvalGraph{dz, d_gout, trials, exec, kernels});
                found = &graphs.back();
            }
            ck(cudaGraphLaunch(found->exec, stream), "cudaGraphLaunch");
            note_launches(int(found->kernels));
        }
        last_z = dz;
        last_trials = trials;
        last_grad = d_gout;
    }

    // trials: 0 none, 1 every instance, 2 the instances of d_trial (device-resident loop)
    void eval_launches(const double* dz, int trials, double* d_gout) {
        PhysParams p = phys;
        p.broad_cell = broad_cell;
        p.inv_cell_f = float(1.0 / broad_cell);
        mark(0);
        if (mixed) launch_state_mixed(topo, p, dz, d_baseX, mn, ev, stream);
        else launch_state(topo, p, dz, d_baseX, d_baseR, ev, stream);
        mark(1);
        if (mixed) launch_beams_mixed(topo, mat, mb, mn, trials, ev, stream, beam_variant);
        else launch_beams(topo, mat, d_plastic, trials, ev, stream, beam_variant);
        mark(2);
        const ContactBufs* cptr = nullptr;
        if (p.self_contact) {
            launch_contacts(topo, p, ev, cb, rmax + cfg.contact_margin, contact_skin, stream,
                            timing ? ev_t[3] : nullptr, timing ? ev_t[4] : nullptr);
            cptr = &cb;
        } else {
            mark(3);
            mark(4);
        }
        mark(5);
        if (mixed) launch_gather_mixed(topo, p, cptr, d_gout, ev, stream, gather_variant);
        else launch_gather(topo, p, cptr, d_gout, ev, stream, gather_variant);
        mark(6);
        launch_finalize(topo, p, cptr, d_gout, ev, stream);
        mark(7);
        check_launch();
        collect();
    }
    const double* last_z = nullptr;
    bool last_trials = false;
    double* last_grad = nullptr;

    // Evaluation whose totals are read back (hp.outs); repeats it with larger contact
    // buffers when a capacity was exceeded.
    // host_grad: the gradient is also copied there, in the same synchronisation.
    const EvalOut* eval_read(const double* dz, bool trials, double* d_gout, double* host_grad = nullptr) {
        eval(dz, trials, d_gout);
        if (host_grad) d2h(host_grad, d_gout, 6 * size_t(N), stream);
        read_outs();
        for (int tries = 0; hp.outs[0].overflow && tries < 16; tries++) {
            if (!grow_contacts(hp.outs[0].overflow)) break;
            eval(dz, trials, d_gout);
            if (host_grad) d2h(host_grad, d_gout, 6 * size_t(N), stream);
            read_outs();
        }
        if (hp.outs[0].overflow) throw Fail(MCG_ERR_CAPACITY, "contact buffers could not be sized");
        if (cfg.self_contact) last_contacts = hp.u32[0];
        contacts_stale = false;
        return hp.outs;
    }
    long long read_contact_count() {
        d2h(hp.u32, cb.hoff + contact_chunks(), 1, stream);
        sync();
        return hp.u32[0];
    }
    void read_outs() {
        d2h(hp.outs, ev.out, size_t(I), stream);
        if (cfg.self_contact) d2h(hp.u32, cb.hoff + contact_chunks(), 1, stream);
        d2h(hp.u32 + 6, ev.err, 1, stream);
        sync();
        check_kernel_error();
    }
    // A kernel's bounded wait that gave up (ev.err, read into hp.u32[6] with the totals)
    // leaves its evaluation invalid: an error, after which the context stays usable.
    void check_kernel_error() {
        if (!hp.u32[6]) return;
        hp.u32[6] = 0;
        ck(cudaMemsetAsync(ev.err, 0, sizeof(unsigned), stream), "memset");
        sync();
        throw Fail(MCG_ERR_CUDA, "a staging wait of the beam kernel gave up; the evaluation is invalid");
    }
    // Totals of the last evaluation, repeating it if it overflowed a contact buffer.
    EvalOut read_out() {
        read_outs();
        if (hp.outs[0].overflow) eval_read(last_z, last_trials, last_grad);
        else if (cfg.self_contact) last_contacts = hp.u32[0];
        contacts_stale = false;
        return hp.outs[0];
    }

    // ---- solver rounds --------------------------------------------------------------------
    // Control records of stage k (0 directions, 1 evaluation, 2 accept) of a round.
    SolveCtl* ctl_stage(int k) { return hp.ctl + size_t(k) * size_t(I); }
    void upload_ctl(int k) { h2d(d_ctl, ctl_stage(k), size_t(I), stream); }
    void clear_ctl(int k) {
        SolveCtl* c = ctl_stage(k);
        for (int i = 0; i < I; i++) c[i] = SolveCtl{0.0, 0, 0, 0, 0};
    }
    // The configuration the minimize decisions read (minimize.h).
    MzParams mz_params() const {
        MzParams p{};
        p.max_iterations = cfg.max_iterations;
        p.max_line_search = cfg.max_line_search;
        p.H = H;
        p.relative_gradient_tolerance = cfg.relative_gradient_tolerance;
        p.translation_scale = cfg.translation_scale;
        p.reaction_relative_tolerance = cfg.reaction_relative_tolerance;
        p.gradient_rms_tolerance = cfg.gradient_rms_tolerance;
        p.gradient_max_tolerance = cfg.gradient_max_tolerance;
        p.penetration_tolerance = cfg.penetration_tolerance;
        p.armijo = cfg.armijo;
        p.min_line_step = cfg.min_line_step;
        // The mixed form's energy carries rounding noise of ~3e-10 |E| (compensated FP32
        // sums of FP32 beam energies); near equilibrium a step's decrease falls below it, so
        // its Armijo test allows that much slack.  The FP64 form tests exactly.
        p.slack_rel = mixed ? kMixedArmijoSlack : 0.0;
        return p;
    }
    // Starts instance i's minimization at platen height `top` from the current d_z (or from
    // z = 0 with zero_first), with an empty history.
    void start_minimize(int i, double top, bool zero_first) {
        Minimizer& s = mins[size_t(i)];
        s = Minimizer{};
        s.phase = Minimizer::kStart;
        s.top = top;
        s.zero_first = zero_first;
    }
    bool pending() const {
        for (const Minimizer& s : mins)
            if (s.phase != Minimizer::kIdle && s.phase != Minimizer::kDone) return true;
        return false;
    }

    // One round for every instance with an unfinished minimization, stepped from the host:
    // directions, one evaluation each, decisions, accepted steps.  The decisions are
    // minimize.h's (the reference's, sim.cpp:174-211); the history (pairs, slots, rho) and
    // the fallback to steepest descent when a direction does not descend are decided on the
    // device (sim.cpp:191, 205-206); the host reads back once per round: the evaluation's
    // totals and each instance's dg.  False when no instance had work.
    bool minimize_round() {
        const double mt = cfg.max_translation_step / cfg.translation_scale, mr = cfg.max_rotation_step;
        const MzParams P = mz_params();
        // A. search directions: two-loop (sim.cpp:184-190), or steepest descent for the retry
        //    after a failed line search (:193-196)
        bool any_dir = false, any_multi = false, any_sd = false;
        clear_ctl(0);
        SolveCtl* ca = ctl_stage(0);
        for (int i = 0; i < I; i++) {
            const int f = mz_stage_direction(mins[size_t(i)], fused[size_t(i)] != 0);
            ca[i].flags = f;
            any_dir |= f == kOpDirFused || f == kOpDirection;
            any_multi |= f == kOpDirection;
            any_sd |= f == kOpSteepest;
        }
        if (any_dir || any_sd) {
            upload_ctl(0);
            replay(1 | (any_dir ? 2 : 0) | (any_multi ? 4 : 0) | (any_sd ? 8 : 0), [&] {
                if (any_dir)
                    bl_direction(topo, d_ctl, d_hist, std::max(H, 1), any_multi, d_p, d_g, d_S, d_Y, 6LL * N, d_rho,
                                 d_alpha, d_part, d_dg, mt, mr, stream);
                if (any_sd) bl_steepest(topo, d_ctl, d_hist, d_p, d_g, d_part, d_dg, mt, mr, stream);
            });
        }
        // B. one evaluation per instance: the start point, a line-search candidate
        //    (sim.cpp:179) or the final state with trials (sim.cpp:210)
        clear_ctl(1);
        SolveCtl* cb1 = ctl_stage(1);
        bool any = false, trials = false;
        std::vector<uint8_t> a(size_t(I), 0);
        for (int i = 0; i < I; i++) {
            double step = 0;
            bool tr = false;
            const int f = mz_stage_eval(mins[size_t(i)], step, tr);
            if (!f) continue;
            cb1[i].flags = f;
            cb1[i].step = step;
            trials |= tr;
            any = true;
            a[size_t(i)] = 1;
            hp.tops[i] = mins[size_t(i)].top;
        }
        if (!any) return false;
        set_active(a);
        upload_ctl(1);
        upload_tops();
        replay(16, [&] { bl_prepare(topo, d_ctl, d_hist, d_z, d_best, d_zeval, d_p, d_zfinal, stream); });
        d2h(hp.dg, d_dg, size_t(I), stream);  // read back with the evaluation's totals
        const EvalOut* out = eval_read(d_zeval, trials, d_geval);
        // C. decisions (the reference's, per instance) and the vectors they imply
        clear_ctl(2);
        SolveCtl* cc = ctl_stage(2);
        bool any_post = false;
        for (int i = 0; i < I; i++) {
            const int f = mz_stage_decide(P, mins[size_t(i)], out[i], hp.dg[i]);
            cc[i].flags = f;
            any_post |= f != 0;
        }
        if (any_post) {
            upload_ctl(2);
            replay(32, [&] {
                bl_accept(topo, d_ctl, d_hist, H, d_z, d_g, d_zeval, d_geval, d_S, d_Y, 6LL * N, d_best, d_rho,
                          d_part, d_dots3, stream);
            });
        }
        check_launch();
        return true;
    }

    // Adds, to the graph being captured on `stream`, an IF node on handle h whose body is
    // what inner(side) launches (captured on the side stream).
    template <typename F>
    void capture_if(cudaGraphConditionalHandle h, F&& inner) {
        cudaStreamCaptureStatus st;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* edges = nullptr;
        size_t nd = 0;
        ck(cudaStreamGetCaptureInfo(stream, &st, nullptr, &g, &deps, &edges, &nd), "cudaStreamGetCaptureInfo");
        cudaGraphNodeParams prm{};
        prm.type = cudaGraphNodeTypeConditional;
        prm.conditional.handle = h;
        prm.conditional.type = cudaGraphCondTypeIf;
        prm.conditional.size = 1;
        cudaGraphNode_t node;
        ck(cudaGraphAddNode(&node, g, deps, edges, nd, &prm), "cudaGraphAddNode (IF)");
        cudaGraph_t body = prm.conditional.phGraph_out[0];
        ck(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
           "cudaStreamUpdateCaptureDependencies");
        ck(cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
           "cudaStreamBeginCaptureToGraph");
        inner(side);
        cudaGraph_t out = nullptr;
        ck(cudaStreamEndCapture(side, &out), "cudaStreamEndCapture (IF body)");
    }

    MzDev mz_dev() {
        MzDev d{};
        d.I = I;
        d.mins = d_mins;
        d.fused = d_fused;
        d.ctl = d_ctl;
        d.active = d_active;
        d.trial_inst = d_trial;
        d.tops = ev.tops;
        d.dg = d_dg;
        d.out = ev.out;
        d.contact_flags = cfg.self_contact ? cb.flags : nullptr;
        d.status = d_mz;
        d.round_cap = kLoopRoundCap;
        return d;
    }

    // The round loop as one graph: WHILE(loop) { A; IF(fused) one-CTA directions;
    // IF(multi) two-loop; IF(any direction) descent fix; IF(steepest) retry; B; prepare;
    // evaluation (trial states per instance); C; IF(accept) accept step }.
    void build_loop() {
        if (!side) ck(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking), "cudaStreamCreate");
        const double mt = cfg.max_translation_step / cfg.translation_scale, mr = cfg.max_rotation_step;
        const MzDev md = mz_dev();
        const MzParams P = mz_params();
        cudaGraph_t g = nullptr;
        ck(cudaGraphCreate(&g, 0), "cudaGraphCreate");
        try {
            cudaGraphConditionalHandle h_loop;
            ck(cudaGraphConditionalHandleCreate(&h_loop, g, 1, cudaGraphCondAssignDefault), "conditional handle");
            cudaGraphNodeParams wp{};
            wp.type = cudaGraphNodeTypeConditional;
            wp.conditional.handle = h_loop;
            wp.conditional.type = cudaGraphCondTypeWhile;
            wp.conditional.size = 1;
            cudaGraphNode_t wnode;
            ck(cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp), "cudaGraphAddNode (WHILE)");
            cudaGraph_t body = wp.conditional.phGraph_out[0];
            cudaGraphConditionalHandle hf, hm, hd, hs, hpost;
            for (cudaGraphConditionalHandle* h : {&hf, &hm, &hd, &hs, &hpost})
                ck(cudaGraphConditionalHandleCreate(h, body, 0, cudaGraphCondAssignDefault), "conditional handle");
            const long long before = g_launch_count.load();
            ck(cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
               "cudaStreamBeginCaptureToGraph");
            try {
                const int Hs = std::max(H, 1);
                launch_mz_direction(md, hf, hm, hd, hs, stream);
                capture_if(hf, [&](cudaStream_t s2) {
                    bl_direction_fused(topo, d_ctl, d_hist, Hs, d_p, d_g, d_S, d_Y, 6LL * N, d_rho, d_dg, mt, mr, s2);
                });
                capture_if(hm, [&](cudaStream_t s2) {
                    bl_direction_multi(topo, d_ctl, d_hist, Hs, d_p, d_g, d_S, d_Y, 6LL * N, d_rho, d_alpha, d_part,
                                       d_dg, mt, mr, s2);
                });
                capture_if(hd, [&](cudaStream_t s2) {
                    bl_descent_fix(topo, d_ctl, d_hist, d_p, d_g, d_part, d_dg, mt, mr, s2);
                });
                capture_if(hs, [&](cudaStream_t s2) {
                    bl_steepest(topo, d_ctl, d_hist, d_p, d_g, d_part, d_dg, mt, mr, s2);
                });
                launch_mz_eval(md, stream);
                bl_prepare(topo, d_ctl, d_hist, d_z, d_best, d_zeval, d_p, d_zfinal, stream);
                eval_launches(d_zeval, 2, d_geval);
                launch_mz_decide(md, P, hpost, h_loop, stream);
                capture_if(hpost, [&](cudaStream_t s2) {
                    bl_accept(topo, d_ctl, d_hist, H, d_z, d_g, d_zeval, d_geval, d_S, d_Y, 6LL * N, d_best, d_rho,
                              d_part, d_dots3, s2);
                });
            } catch (...) {
                cudaGraph_t junk = nullptr;
                cudaStreamEndCapture(stream, &junk);
                cudaGetLastError();
                throw;
            }
            cudaGraph_t out = nullptr;
            ck(cudaStreamEndCapture(stream, &out), "cudaStreamEndCapture (loop body)");
            loop_round_kernels = g_launch_count.load() - before;
            g_launch_count -= loop_round_kernels;  // counted per round run (rounds_device)
            ck(cudaGraphInstantiate(&loop_exec, g, 0), "cudaGraphInstantiate (loop)");
        } catch (...) {
            cudaGraphDestroy(g);
            throw;
        }
        cudaGraphDestroy(g);
    }

    // Rounds on the device until an instance finishes, none has work, the round cap is
    // reached or an evaluation overflows a contact buffer (then the buffers grow and the
    // loop runs again from that evaluation).  The host minimizers are copied in before and
    // out after.  False when no instance had work.
    bool rounds_device() {
        if (!pending()) return false;
        for (int tries = 0;; tries++) {
            if (!loop_exec) build_loop();
            std::copy(mins.begin(), mins.end(), hp.mins);
            h2d(d_mins, hp.mins, size_t(I), stream);
            launch_mz_reset(mz_dev(), stream);
            const auto w0 = std::chrono::steady_clock::now();
            ck(cudaGraphLaunch(loop_exec, stream), "cudaGraphLaunch (loop)");
            d2h(hp.mins, d_mins, size_t(I), stream);
            d2h(hp.mz, d_mz, 1, stream);
            d2h(hp.outs, ev.out, size_t(I), stream);
            if (cfg.self_contact) d2h(hp.u32, cb.hoff + contact_chunks(), 1, stream);
            d2h(hp.u32 + 6, ev.err, 1, stream);
            sync();
            check_launch();
            check_kernel_error();
            loop_wall_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
            loop_ns[0] += hp.mz->t_dir;
            loop_ns[1] += hp.mz->t_eval;
            loop_ns[2] += hp.mz->t_post;
            loop_rounds += hp.mz->rounds;
            note_launches(int(hp.mz->rounds) * int(loop_kernels_per_round()));
            std::copy(hp.mins, hp.mins + I, mins.begin());
            active.assign(size_t(I), 2);  // the loop wrote d_active: the host mirror is unknown
            last_z = d_zeval;
            last_trials = false;
            last_grad = d_geval;
            if (hp.mz->overflow) {
                if (tries >= 16 || !grow_contacts(hp.outs[0].overflow))
                    throw Fail(MCG_ERR_CAPACITY, "contact buffers could not be sized");
                continue;
            }
            if (hp.mz->rounds <= 0)  // the body did not run: never loop on the host for it
                throw Fail(MCG_ERR_CUDA, "the device-resident round loop ran no round");
            break;
        }
        if (cfg.self_contact) last_contacts = hp.u32[0];
        contacts_stale = false;
        return true;
    }
    // Kernels one loop round launches (the device counts no launches; this estimate keeps
    // the library's launch counter meaningful): stage kernels plus the evaluation's.
    long long loop_kernels_per_round() const { return loop_round_kernels; }
    long long loop_round_kernels = 0;

    // One step of rounds: on the device when the loop is available, else host-stepped.
    bool step_rounds() {
        if (device_loop && use_graphs && !timing) {
            try {
                return rounds_device();
            } catch (const Fail& f) {
                if (f.code == MCG_ERR_CAPACITY) throw;
                device_loop = false;  // e.g. the driver refuses the conditional nodes
                loop_error = f.what();
                drop_graphs();
            }
        }
        return minimize_round();
    }

    // Steps the minimizations started with start_minimize until all are done.
    void minimize_all() {
        while (step_rounds()) {
        }
    }

    // ---- Simulator::commit, MC/src/sim.cpp:212, for the instances with m[i] != 0 ----------
    void commit(const std::vector<uint8_t>& m) {
        h2d(d_mask, m.data(), size_t(I), stream);
        PhysParams p = phys;
        DevTopo all = topo;  // the committed instances' states (others are recomputed before use)
        all.active = d_all;
        launch_state(all, p, d_zfinal, d_baseX, d_baseR, ev, stream);
        if (mixed) {
            launch_commit(topo, d_mask, ev, d_baseX, d_baseR, nullptr, stream);
            launch_plastic_mixed(topo, d_mask, nullptr, ev.trial_nextf, mb, stream);
            launch_plastic_mixed_to_f64(topo, d_mask, mb, d_plastic, stream);
        } else {
            launch_commit(topo, d_mask, ev, d_baseX, d_baseR, d_plastic, stream);
        }
        rebase();
        check_launch();
        sync();  // the mask is pageable host memory
    }

    double top_y(const mcg_geometry& g, double s, bool loading) const {
        const double compressed = g.top0 - cfg.max_strain * g.height;
        const double t = std::max(0.0, std::min(1.0, s));
        return loading ? g.top0 * (1.0 - t) + compressed * t : compressed * (1.0 - t) + g.top0 * t;
    }

    // ---- Simulator::diagnostics, MC/src/sim.cpp:312-372 -------------------------------------
    // Reads the plastic statistics and node boxes of all instances after a commit.
    void read_diagnostics() {
        launch_plastic_stats(topo, d_plastic, d_part, d_pstats, stream);
        d2h(hp.pstats, d_pstats, 6 * size_t(I), stream);
        d2h(hp.cen, ev.cen, 9 * size_t(I + 1), stream);
        sync();
    }
    mcg_frame diagnostics(int i, const Runner& r, double time, double top, bool loading, const EvalOut& o,
                          const HostStats& s) const {
        const mcg_geometry& g = inst[size_t(i)].geom;
        const int Bi = inst[size_t(i)].B;
        mcg_frame d;
        std::memset(&d, 0, sizeof(d));
        d.time = time;
        d.platen_y = top;
        d.displacement = g.top0 - top;
        d.engineering_strain = d.displacement / std::max(1e-12, g.height);
        d.reaction_force = std::max(0.0, o.reaction - r.reactionOffset);
        d.engineering_stress = d.reaction_force / std::max(1e-12, g.area);
        d.loading_work = r.loadingWork;
        d.recovered_work = r.recoveredWork;
        d.dissipated_work = std::max(0.0, r.loadingWork - r.recoveredWork);
        d.specific_energy_absorption = d.dissipated_work / std::max(1e-12, g.mass);
        d.elastic_energy = o.elastic;
        d.plastic_dissipation = o.plastic;
        d.contact_energy = o.contact;
        d.residual_rms = s.rms;
        d.residual_max = s.max;
        d.max_penetration = o.max_pen;
        d.active_contacts = o.contacts;
        d.iterations = s.iterations;
        d.converged = s.converged;
        d.loading = loading;
        const double* ps = hp.pstats + 6 * size_t(i);
        if (Bi > 0) {
            d.mean_plastic_strain = ps[0] / Bi;
            d.max_plastic_strain = ps[1];
            d.mean_plastic_rotation = ps[2] / Bi;
            d.max_plastic_rotation = ps[3];
        }
        d.plastic_beams = int(ps[4]);
        d.plastic_hinges = int(ps[5]);
        const double* box = hp.cen + 9 * size_t(i);
        const double currentHeight = std::max(0.0, box[7] - box[4]);
        d.permanent_set = std::max(0.0, 1.0 - currentHeight / std::max(1e-12, g.height));
        return d;
    }

    // ---- Simulator::run, MC/src/sim.cpp:374-467, for every instance ---------------------------
    // advanceTo's recursion (bisection of a failed increment) is an explicit stack per
    // instance: a failed target is replaced by its midpoint followed by itself.
    void run(std::vector<Runner>& rs, bool verbose) {
        rs.assign(size_t(I), Runner{});
        for (int i = 0; i < I; i++) {
            rs[size_t(i)].currentTop = inst[size_t(i)].geom.top0;
            mins[size_t(i)] = Minimizer{};
        }
        have_final = false;
        auto next_task = [&](int i) -> bool {
            Runner& r = rs[size_t(i)];
            const mcg_geometry& g = inst[size_t(i)].geom;
            if (!r.stack.empty()) {
                r.task = r.stack.back();
                r.stack.pop_back();
                return true;
            }
            const int L = cfg.load_steps, U = cfg.unload_steps;
            const int k = r.next_step++;
            if (k == 0) r.task = Task{g.top0, true, 0};
            else if (k <= L) r.task = Task{top_y(g, double(k) / std::max(1, L), true), true, 0};
            else if (k <= L + U) r.task = Task{top_y(g, double(k - L) / std::max(1, U), false), false, 0};
            else return false;
            return true;
        };
        std::vector<uint8_t> cm(size_t(I), 0);
        for (;;) {
            bool pending = false;
            for (int i = 0; i < I; i++) {
                Runner& r = rs[size_t(i)];
                if (r.done) continue;
                if (mins[size_t(i)].phase == Minimizer::kIdle) {
                    if (!next_task(i)) {
                        r.done = true;
                        continue;
                    }
                    start_minimize(i, r.task.top, true);
                }
                pending = true;
            }
            if (!pending) break;
            step_rounds();
            bool any_commit = false;
            std::fill(cm.begin(), cm.end(), uint8_t(0));
            for (int i = 0; i < I; i++) {
                Minimizer& s = mins[size_t(i)];
                if (s.phase != Minimizer::kDone) continue;
                Runner& r = rs[size_t(i)];
                const Task t = r.task;
                const bool acceptable = s.st.converged && s.fin.max_pen <= cfg.penetration_tolerance &&
                                        std::isfinite(s.fin.energy);
                if (acceptable) {
                    cm[size_t(i)] = 1;
                    any_commit = true;
                    continue;
                }
                s.phase = Minimizer::kIdle;
                if (t.refinement < cfg.max_adaptive_refinements && std::abs(t.top - r.currentTop) > 2.5e-5) {
                    const double midpoint = 0.5 * (r.currentTop + t.top);
                    r.stack.push_back(Task{t.top, t.loading, t.refinement + 1});
                    r.stack.push_back(Task{midpoint, t.loading, t.refinement + 1});
                    continue;
                }
                char msg[256];
                std::snprintf(msg, sizeof msg,
                              "quasi-static equilibrium failed at platen=%g m, residual=%g, penetration=%g mm after %d "
                              "iterations",
                              t.top, s.st.rms, s.fin.max_pen * 1000.0, s.st.iterations);
                r.status = MCG_ERR_EQUILIBRIUM;
                r.error = msg;
                r.done = true;
            }
            if (!any_commit) continue;
            commit(cm);
            read_diagnostics();
            for (int i = 0; i < I; i++) {
                if (!cm[size_t(i)]) continue;
                Minimizer& s = mins[size_t(i)];
                Runner& r = rs[size_t(i)];
                const Task t = r.task;
                if (r.first) r.reactionOffset = s.fin.reaction;
                const double force = std::max(0.0, s.fin.reaction - r.reactionOffset);
                const double displacement = inst[size_t(i)].geom.top0 - t.top;
                if (!r.first) {
                    const double dd = displacement - r.prevDisp;
                    const double work = 0.5 * (r.prevForce + force) * dd;
                    if (dd >= 0.0) r.loadingWork += std::max(0.0, work);
                    else r.recoveredWork += std::max(0.0, -work);
                }
                r.prevDisp = displacement;
                r.prevForce = force;
                r.currentTop = t.top;
                mcg_frame d = diagnostics(i, r, r.time, t.top, t.loading, s.fin, s.st);
                d.refinement = t.refinement;
                r.frames.push_back(d);
                if (verbose)
                    std::printf("[equilibrium] %3d %s strain=%.4f force=%.3f N residual=%.2e pen=%.3f mm iter=%d %s\n",
                                r.accepted, t.loading ? "load  " : "unload", d.engineering_strain, d.reaction_force,
                                d.residual_rms, d.max_penetration * 1000.0, d.iterations,
                                t.refinement ? "[REFINED]" : "[OK]");
                r.accepted++;
                r.first = false;
                r.time += cfg.step_time;
                s.phase = Minimizer::kIdle;
            }
        }
    }
};

namespace {

int fail(mcg_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

template <class F>
int guarded(mcg_ctx* c, F&& f) {
    if (!c) return MCG_ERR_INVALID;
    try {
        c->set_device();
        f();
        c->err.clear();
        return MCG_OK;
    } catch (const Fail& e) {
        return fail(c, e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(c, MCG_ERR_INVALID, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(c, MCG_ERR_INVALID, e.what());
    }
}

void need_topo(const mcg_ctx* c) {
    if (!c->have_topo) throw Fail(MCG_ERR_STATE, "no topology uploaded");
}
void need_single(const mcg_ctx* c) {
    need_topo(c);
    if (c->I != 1) throw Fail(MCG_ERR_STATE, "a batched context: use the mcg_batch_* functions");
}

// Builds the device model of one or more instances (stored one after another).
void upload_instances(mcg_ctx* c, const std::vector<InstIn>& ins) {
    const mcg_config& cf = c->cfg;
    const int I = int(ins.size());
    if (I <= 0) throw Fail(MCG_ERR_INVALID, "no instance");
    long long Nt = 0, Bt = 0;
    for (int k = 0; k < I; k++) {
        const mcg_topology* t = ins[size_t(k)].t;
        if (!t || !ins[size_t(k)].g) throw Fail(MCG_ERR_INVALID, "null topology or geometry");
        if (t->n_nodes <= 0 || t->n_beams < 0)
            throw Fail(MCG_ERR_INVALID, "node count must be positive and beam count non-negative");
        if (t->n_beams > 0 &&
            (!t->beam_a || !t->beam_b || !t->L0 || !t->radius || !t->area || !t->I || !t->J || !t->e0))
            throw Fail(MCG_ERR_INVALID, "missing beam array");
        if (!t->mass || !t->locked) throw Fail(MCG_ERR_INVALID, "missing node array");
        if (t->n_connected < 0 || (t->n_connected > 0 && !t->connected))
            throw Fail(MCG_ERR_INVALID, "bad connected list");
        if (!(ins[size_t(k)].sy > 0) || !std::isfinite(ins[size_t(k)].sy))
            throw Fail(MCG_ERR_INVALID, "yield stress must be positive");
        Nt += t->n_nodes;
        Bt += t->n_beams;
    }
    if (Nt + Bt >= (1LL << 31) / 4) throw Fail(MCG_ERR_INVALID, "model too large for 32-bit shape indices");
    const int N = int(Nt), B = int(Bt);
    const double E = cf.material.young, G = E / (2 * (1 + cf.material.nu));
    std::vector<int2> ab(static_cast<size_t>(B));
    std::vector<double> kb(B), kt(B), my(B), ty(B), hb(B), ht(B), cs(B), aL(B), aLsy(B), syb(B);
    std::vector<double> invL0(B), inv_kbh(B), inv_kth(B);
    std::vector<double> e0x(B), e0y(B), e0z(B), L0v(B), areav(B), radv(B), massv(N);
    std::vector<uint8_t> lockedv(6 * size_t(N));
    std::vector<float> padf(B);
    double rmax = cf.joint_scale * cf.max_radius;
    // whether every section is the circular one (area pi r^2, I = pi r^4 / 4, J = 2 I,
    // MC/src/sim.cpp:115): then the mixed form derives its section constants from r and L0
    bool circular = true;
    const double kPiD = 3.14159265358979323846;
    auto near = [](double a, double b) { return std::abs(a - b) <= 1e-9 * std::abs(b); };
    std::vector<int> deg(size_t(N) + 1, 0);
    std::vector<InstHost> ih(static_cast<size_t>(I));
    std::vector<std::vector<int>> adj(static_cast<size_t>(N));
    int node0 = 0, beam0 = 0;
    for (int k = 0; k < I; k++) {
        const mcg_topology* t = ins[size_t(k)].t;
        const int Ni = t->n_nodes, Bi = t->n_beams;
        const double sy = ins[size_t(k)].sy;
        InstHost& h = ih[size_t(k)];
        h.node0 = node0;
        h.N = Ni;
        h.beam0 = beam0;
        h.B = Bi;
        h.geom = *ins[size_t(k)].g;
        h.sy = sy;
        for (int b = 0; b < Bi; b++) {
            const int a = t->beam_a[b], bb = t->beam_b[b];
            if (a < 0 || a >= Ni || bb < 0 || bb >= Ni || a == bb)
                throw Fail(MCG_ERR_INVALID, "beam " + std::to_string(b) + " has invalid end nodes");
            const double L0 = t->L0[b], r = t->radius[b];
            if (!(L0 > 0) || !std::isfinite(L0) || !(r > 0) || !std::isfinite(r) || !std::isfinite(t->area[b]) ||
                !std::isfinite(t->I[b]) || !std::isfinite(t->J[b]))
                throw Fail(MCG_ERR_INVALID, "beam " + std::to_string(b) + " has invalid section data");
            const size_t g = size_t(beam0 + b);
            ab[g] = make_int2(node0 + a, node0 + bb);
            deg[size_t(node0 + a)]++;
            deg[size_t(node0 + bb)]++;
            // Section constants, evaluated with the reference's expressions
            // (sim.cpp:139-141); this file is compiled without FMA contraction, so the
            // values equal the ones the reference recomputes on every call.
            const double area = t->area[b], Is = t->I[b], J = t->J[b];
            kb[g] = E * Is / L0;
            kt[g] = G * J / L0;
            my[g] = sy * Is / r;
            ty[g] = (sy / std::sqrt(3.0)) * J / r;
            hb[g] = cf.material.bend_hardening * kb[g];
            ht[g] = cf.material.torsion_hardening * kt[g];
            cs[g] = .5 * cf.shear_correction * G * area * L0;
            aL[g] = area * L0;
            aLsy[g] = area * L0 * sy;
            syb[g] = sy;
            invL0[g] = 1.0 / L0;
            inv_kbh[g] = 1.0 / std::max(1e-20, kb[g] + hb[g]);
            inv_kth[g] = 1.0 / std::max(1e-20, kt[g] + ht[g]);
            circular = circular && near(area, kPiD * r * r) && near(Is, .25 * kPiD * r * r * r * r) && near(J, 2 * Is);
            e0x[g] = t->e0[3 * size_t(b)];
            e0y[g] = t->e0[3 * size_t(b) + 1];
            e0z[g] = t->e0[3 * size_t(b) + 2];
            L0v[g] = L0;
            areav[g] = area;
            radv[g] = r;
            rmax = std::max(rmax, r);
            padf[g] = round_up_float(r + cf.contact_margin);
        }
        for (int i = 0; i < Ni; i++) {
            if (!std::isfinite(t->mass[i])) throw Fail(MCG_ERR_INVALID, "non-finite node mass");
            massv[size_t(node0 + i)] = t->mass[i];
        }
        long long nfree = 0;
        for (long long q = 0; q < 6LL * Ni; q++) {
            if (t->locked[q] > 1) throw Fail(MCG_ERR_INVALID, "locked flags must be 0 or 1");
            nfree += t->locked[q] ? 0 : 1;
            lockedv[size_t(6LL * node0 + q)] = t->locked[q];
        }
        h.n_free = nfree;
        for (int64_t q = 0; q < t->n_connected; q++) {
            const uint64_t key = t->connected[q];
            const uint32_t u = uint32_t(key >> 32), v = uint32_t(key & 0xffffffffu);
            if (u >= uint32_t(Ni) || v >= uint32_t(Ni) || u > v)
                throw Fail(MCG_ERR_INVALID, "connected key " + std::to_string(q) + " is not a node pair key");
            adj[size_t(node0) + u].push_back(int(node0 + v));
            if (u != v) adj[size_t(node0) + v].push_back(int(node0 + u));
        }
        node0 += Ni;
        beam0 += Bi;
    }
    // incidence CSR in ascending beam order (the reference's scatter order)
    std::vector<int> inc_start(size_t(N) + 1, 0), inc(2 * size_t(B));
    for (int i = 0; i < N; i++) inc_start[size_t(i) + 1] = inc_start[size_t(i)] + deg[size_t(i)];
    {
        std::vector<int> cur(inc_start.begin(), inc_start.end() - 1);
        for (int b = 0; b < B; b++) {
            inc[size_t(cur[size_t(ab[size_t(b)].x)]++)] = (b << 1) | 0;
            inc[size_t(cur[size_t(ab[size_t(b)].y)]++)] = (b << 1) | 1;
        }
    }
    // connected pairs as an open-addressing hash set (at most half full)
    long long npairs = 0;
    for (int i = 0; i < N; i++) {
        auto& l = adj[size_t(i)];
        std::sort(l.begin(), l.end());
        l.erase(std::unique(l.begin(), l.end()), l.end());
        for (int v : l) npairs += v >= i ? 1 : 0;
    }
    int hbits = 4;
    while ((1LL << hbits) < 2 * npairs) hbits++;
    std::vector<unsigned long long> conn_hash(size_t(1) << hbits, ~0ull);
    const unsigned long long hmask = (1ull << hbits) - 1;
    for (int i = 0; i < N; i++)
        for (int v : adj[size_t(i)]) {
            if (v < i) continue;
            const unsigned long long key = ((unsigned long long)i << 32) | uint32_t(v);
            unsigned long long h = (key * 0x9E3779B97F4A7C15ull) >> (64 - hbits);
            while (conn_hash[h] != ~0ull) h = (h + 1) & hmask;
            conn_hash[h] = key;
        }
    // blocks that never straddle two instances
    std::vector<int4> nblk, bblk, irange(static_cast<size_t>(I));
    for (int k = 0; k < I; k++) {
        const InstHost& h = ih[size_t(k)];
        irange[size_t(k)].x = int(nblk.size());
        for (int f = 0; f < h.N; f += kMapBlock)
            nblk.push_back(make_int4(h.node0 + f, std::min(kMapBlock, h.N - f), k, 0));
        irange[size_t(k)].y = int(nblk.size());
        irange[size_t(k)].z = int(bblk.size());
        for (int f = 0; f < h.B; f += kMapBlock)
            bblk.push_back(make_int4(h.beam0 + f, std::min(kMapBlock, h.B - f), k, 0));
        irange[size_t(k)].w = int(bblk.size());
    }
    // contact-grid offsets: the instances' footprints (x-z extent with room to widen under
    // compression) packed in rows, so that the shared grid stays small; offsets are
    // multiples of 2^-10 m, exact in FP32.  (Pairs of two instances are never contacts in
    // any case: the narrow phase rejects them.)
    {
        struct Fp {
            int k;
            double lo_x, lo_z, w, d;
        };
        std::vector<Fp> fp;
        for (int k = 0; k < I; k++) {
            const InstIn& in = ins[size_t(k)];
            double lx = 0, hx = 0, lz = 0, hz = 0;
            if (in.x0 && in.t->n_nodes > 0) {
                lx = hx = in.x0[0];
                lz = hz = in.x0[2];
                for (int i = 0; i < in.t->n_nodes; i++) {
                    lx = std::min(lx, in.x0[3 * size_t(i)]);
                    hx = std::max(hx, in.x0[3 * size_t(i)]);
                    lz = std::min(lz, in.x0[3 * size_t(i) + 2]);
                    hz = std::max(hz, in.x0[3 * size_t(i) + 2]);
                }
            }
            const double mw = 0.3 * (hx - lx) + 4 * rmax + 0.005, md = 0.3 * (hz - lz) + 4 * rmax + 0.005;
            fp.push_back(Fp{k, lx - mw, lz - md, (hx - lx) + 2 * mw, (hz - lz) + 2 * md});
        }
        double area = 0;
        for (const Fp& f : fp) area += f.w * f.d;
        const double row_max = std::sqrt(area) * 1.2;
        std::vector<Fp> order = fp;
        std::sort(order.begin(), order.end(), [](const Fp& a, const Fp& b) { return a.d > b.d || (a.d == b.d && a.k < b.k); });
        double x = 0, z = 0, row_d = 0;
        auto q = [](double v) { return std::ceil(v * 1024.0) / 1024.0; };
        for (const Fp& f : order) {
            if (x > 0 && x + f.w > row_max) {
                z = q(z + row_d);
                x = 0;
                row_d = 0;
            }
            ih[size_t(f.k)].off = I == 1 ? float2{0.f, 0.f} : float2{float(q(x - f.lo_x)), float(q(z - f.lo_z))};
            x = q(x + f.w + 1e-3);
            row_d = std::max(row_d, f.d + 1e-3);
        }
    }

    c->sync();
    c->drop_graphs();
    c->topo_mem.release();
    c->eval_mem.release();
    c->contact_mem.release();
    c->solver_mem.release();
    c->have_topo = false;
    c->have_final = false;
    c->N = N;
    c->B = B;
    c->I = I;
    c->inst = ih;
    c->jr = cf.joint_scale * cf.max_radius;
    c->rmax = rmax;
    c->H = std::max(cf.history, 0);
    c->hp.alloc(I);
    cudaStream_t s = c->stream;
    DevArena& M = c->topo_mem;
    DevTopo T{};
    T.N = N;
    T.B = B;
    auto upd = [&](const std::vector<double>& v) {
        double* d = M.get<double>(v.size());
        h2d(d, v.data(), v.size(), s);
        return static_cast<const double*>(d);
    };
    int2* dab = M.get<int2>(size_t(B));
    h2d(dab, ab.data(), size_t(B), s);
    T.ab = dab;
    T.L0 = upd(L0v);
    T.area = upd(areav);
    T.radius = upd(radv);
    T.e0x = upd(e0x); T.e0y = upd(e0y); T.e0z = upd(e0z);
    T.kb = upd(kb); T.kt = upd(kt); T.my = upd(my); T.ty = upd(ty); T.hb = upd(hb); T.ht = upd(ht);
    T.cs = upd(cs); T.aL = upd(aL); T.aLsy = upd(aLsy);
    T.invL0 = upd(invL0); T.inv_kbh = upd(inv_kbh); T.inv_kth = upd(inv_kth);
    T.sy = upd(syb);
    T.mass = upd(massv);
    uint8_t* dl = M.get<uint8_t>(6 * size_t(N));
    h2d(dl, lockedv.data(), 6 * size_t(N), s);
    T.locked = dl;
    int* dis = M.get<int>(inc_start.size());
    h2d(dis, inc_start.data(), inc_start.size(), s);
    T.inc_start = dis;
    int* di = M.get<int>(inc.size());
    h2d(di, inc.data(), inc.size(), s);
    T.inc = di;
    {
        unsigned long long* dh = M.get<unsigned long long>(conn_hash.size());
        h2d(dh, conn_hash.data(), conn_hash.size(), s);
        T.conn_hash = dh;
        T.conn_mask = hmask;
        T.conn_shift = 64 - hbits;
    }
    {
        float* dp = M.get<float>(size_t(B));
        h2d(dp, padf.data(), size_t(B), s);
        T.padf = dp;
    }
    T.I = I;
    T.n_nblk = int(nblk.size());
    T.n_bblk = int(bblk.size());
    {
        int4* d = M.get<int4>(nblk.size());
        h2d(d, nblk.data(), nblk.size(), s);
        T.nblk = d;
        int4* e = M.get<int4>(bblk.size());
        h2d(e, bblk.data(), bblk.size(), s);
        T.bblk = e;
        int4* r = M.get<int4>(irange.size());
        h2d(r, irange.data(), irange.size(), s);
        T.irange = r;
        std::vector<int> nn(static_cast<size_t>(I));
        std::vector<long long> nf(static_cast<size_t>(I));
        std::vector<float2> off(static_cast<size_t>(I));
        for (int k = 0; k < I; k++) {
            nn[size_t(k)] = ih[size_t(k)].N;
            nf[size_t(k)] = ih[size_t(k)].n_free;
            off[size_t(k)] = ih[size_t(k)].off;
        }
        int* dn = M.get<int>(nn.size());
        h2d(dn, nn.data(), nn.size(), s);
        T.inst_n = dn;
        long long* dnf = M.get<long long>(nf.size());
        h2d(dnf, nf.data(), nf.size(), s);
        T.inst_free = dnf;
        float2* doff = M.get<float2>(off.size());
        h2d(doff, off.data(), off.size(), s);
        T.off = doff;
        std::vector<int> ni(static_cast<size_t>(N));
        for (int k = 0; k < I; k++)
            std::fill(ni.begin() + ih[size_t(k)].node0, ni.begin() + ih[size_t(k)].node0 + ih[size_t(k)].N, k);
        int* dni = M.get<int>(ni.size());
        h2d(dni, ni.data(), ni.size(), s);
        T.node_inst = dni;
        std::vector<uint8_t> ones(static_cast<size_t>(I), 1);
        c->d_active = M.get<uint8_t>(size_t(I));
        c->d_all = M.get<uint8_t>(size_t(I));
        h2d(c->d_active, ones.data(), ones.size(), s);
        h2d(c->d_all, ones.data(), ones.size(), s);
        T.active = c->d_active;
        c->active = ones;
        c->d_trial = M.get<uint8_t>(size_t(I));
        ck(cudaMemsetAsync(c->d_trial, 0, size_t(I), s), "memset");
        T.trial_inst = c->d_trial;
        c->sync();  // the host vectors above go out of scope
    }
    c->topo = T;
    c->mat = Material{E,
                      G,
                      cf.material.yield,
                      cf.material.hardening,
                      cf.material.bend_hardening,
                      cf.material.torsion_hardening,
                      1.0 / std::max(1e-20, E + cf.material.hardening),
                      float(E),
                      float(cf.material.hardening),
                      float(cf.material.bend_hardening),
                      float(cf.material.torsion_hardening)};
    PhysParams P{};
    P.translation_scale = cf.translation_scale;
    P.gravity = cf.gravity;
    P.centering = cf.centering_stiffness;
    P.contact_k = cf.contact_stiffness;
    P.contact_margin = cf.contact_margin;
    P.joint_radius = c->jr;
    P.broad_cell = std::max(2.8 * c->jr, .72 * cf.cell_size);
    P.top = ih[0].geom.top0;
    P.self_contact = cf.self_contact ? 1 : 0;
    P.joint_padf = round_up_float(c->jr + cf.contact_margin);
    c->phys = P;
    // state
    c->d_baseX = M.get<double>(3 * size_t(N));
    c->d_baseR = M.get<double>(4 * size_t(N));
    c->d_plastic = M.get<double>(7 * size_t(B));
    ck(cudaMemsetAsync(c->d_plastic, 0, 7 * size_t(B) * sizeof(double), s), "memset");
    {
        std::vector<double> x(3 * size_t(N), 0.0), r(4 * size_t(N), 0.0);
        bool have_x = true;
        for (int k = 0; k < I; k++) {
            const InstIn& in = ins[size_t(k)];
            const InstHost& h = ih[size_t(k)];
            have_x &= in.x0 != nullptr;
            if (in.x0) std::copy(in.x0, in.x0 + 3 * size_t(h.N), x.begin() + 3 * size_t(h.node0));
            for (int i = 0; i < h.N; i++) {
                double* q = r.data() + 4 * size_t(h.node0 + i);
                if (in.r0) std::copy(in.r0 + 4 * size_t(i), in.r0 + 4 * size_t(i) + 4, q);
                else q[0] = 1.0;
            }
        }
        if (have_x) h2d(c->d_baseX, x.data(), x.size(), s);
        h2d(c->d_baseR, r.data(), r.size(), s);
        c->sync();
    }
    // evaluation buffers
    DevArena& V = c->eval_mem;
    EvalBufs e{};
    e.x = V.get<double4_32a>(size_t(N));
    e.R = V.get<double4_32a>(size_t(N));
    e.M = V.get<double4_32a>(3 * size_t(N));
    e.xf_lo = V.get<float4>(size_t(N));
    e.xf_hi = V.get<float4>(size_t(N));
    e.slotA = V.get<double>(6 * size_t(B));
    e.slotB = V.get<double>(6 * size_t(B));
    e.part_state = V.get<double>(9 * size_t(T.n_nblk));
    e.part_beam = V.get<double>(3 * size_t(std::max(T.n_bblk, 1)));
    e.err = V.get<unsigned>(1);
    ck(cudaMemsetAsync(e.err, 0, sizeof(unsigned), s), "memset");
    e.part_node = V.get<double>(kNodeParts * size_t(T.n_nblk));
    e.part_fin = V.get<double>(size_t(kFinPartDoubles) * size_t(I));
    e.cen = V.get<double>(9 * size_t(I + 1));
    e.tops = V.get<double>(size_t(I));
    e.out = V.get<EvalOut>(size_t(I));
    e.trial_next = V.get<double>(7 * size_t(B));
    e.trial_aux = V.get<double>(7 * size_t(B));
    e.trial_flags = V.get<uint8_t>(3 * size_t(B));
    c->mixed = cf.precision == MCG_MIXED;
    if (c->mixed) {
        e.slotAf = V.get<float>(6 * size_t(B));
        e.slotBf = V.get<float>(6 * size_t(B));
        e.trial_nextf = V.get<float>(7 * size_t(B));
        e.trial_auxf = V.get<float>(7 * size_t(B));
        MixedBeams mb{};
        float4** fields[] = {&mb.B0, &mb.B1, &mb.B2, &mb.B5, &mb.P0, &mb.P1};
        for (float4** f : fields) *f = V.get<float4>(size_t(B));
        if (!circular) {
            mb.C0 = V.get<float4>(size_t(B));
            mb.C1 = V.get<float4>(size_t(B));
        }
        std::vector<float4> ic(static_cast<size_t>(I));
        for (int k = 0; k < I; k++) {
            const double sy = ih[size_t(k)].sy;
            ic[size_t(k)] = make_float4(float(sy), float(sy * kPiD / 4), float(sy / std::sqrt(3.0) * kPiD / 2),
                                        float(sy * kPiD));
        }
        mb.ic = V.get<float4>(size_t(I));
        h2d(mb.ic, ic.data(), ic.size(), s);
        mb.kg = make_float4(float(E * kPiD / 4), float(G * kPiD / 2), float(.5 * cf.shear_correction * G * kPiD),
                            float(kPiD));
        c->mb = mb;
        c->sync();  // ic goes out of scope
        c->mn = MixedNodes{V.get<float4>(2 * size_t(N)), V.get<float4>(size_t(N))};
    }
    c->ev = e;
    for (int k = 0; k < I; k++) c->hp.tops[k] = ih[size_t(k)].geom.top0;
    c->upload_tops();
    c->d_zin = V.get<double>(6 * size_t(N));
    c->d_grad = V.get<double>(6 * size_t(N));
    ck(cudaMemsetAsync(c->d_zin, 0, 6 * size_t(N) * sizeof(double), s), "memset");
    // contact buffers: a first guess, grown on demand
    const long long S = (long long)N + B;
    c->broad_cell = P.broad_cell;
    c->contact_skin = float(cf.cell_size / 32);
    {
        // bins: the Morton range of the rest-state extent (in the grid's frame) with room to
        // grow, or row-major bins when that range is too large
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        bool any = false;
        for (int k = 0; k < I; k++) {
            const InstIn& in = ins[size_t(k)];
            if (!in.x0) continue;
            any = true;
            const double o[3] = {ih[size_t(k)].off.x, 0.0, ih[size_t(k)].off.y};
            for (int i = 0; i < in.t->n_nodes; i++)
                for (int d = 0; d < 3; d++) {
                    lo[d] = std::min(lo[d], in.x0[3 * size_t(i) + d] + o[d]);
                    hi[d] = std::max(hi[d], in.x0[3 * size_t(i) + d] + o[d]);
                }
        }
        long long dims[3] = {8, 8, 8};
        long long dmax = 8;
        if (any)
            for (int d = 0; d < 3; d++) {
                dims[d] = (long long)((hi[d] - lo[d] + 2 * c->rmax) / P.broad_cell * 1.15) + 4;
                dmax = std::max(dmax, dims[d]);
            }
        int bits = 3;
        while ((1LL << bits) < dmax && bits < 10) bits++;
        const long long dense = dims[0] * dims[1] * dims[2];
        long long bin_cap = std::min(1LL << (3 * bits), 1LL << 27);
        // row-major bins when the Morton range does not fit or is mostly empty
        if ((1LL << bits) < dmax || bin_cap > 4 * dense) bin_cap = std::min(dense, 1LL << 28);
        c->alloc_contacts(64, std::max<long long>(S / 2, 4096), bin_cap, std::max<long long>(4 * S, 4096));
    }
    // solver vectors
    DevArena& Q = c->solver_mem;
    const size_t n = 6 * size_t(N);
    const int Hs = std::max(c->H, 1);
    c->d_z = Q.get<double>(n); c->d_zeval = Q.get<double>(n); c->d_p = Q.get<double>(n);
    c->d_g = Q.get<double>(n); c->d_geval = Q.get<double>(n); c->d_best = Q.get<double>(n);
    c->d_zfinal = Q.get<double>(n);
    c->d_S = Q.get<double>(size_t(Hs) * n);
    c->d_Y = Q.get<double>(size_t(Hs) * n);
    c->d_rho = Q.get<double>(size_t(I) * Hs);
    c->d_alpha = Q.get<double>(size_t(I) * Hs);
    c->d_part = Q.get<double>(std::max(lbfgs_part_doubles(std::max(T.n_nblk, T.n_bblk)), 6 * size_t(T.n_bblk) + 8));
    c->d_dg = Q.get<double>(size_t(I));
    c->d_dots3 = Q.get<double>(3 * size_t(I));
    c->d_pstats = Q.get<double>(6 * size_t(I));
    c->d_ctl = Q.get<SolveCtl>(size_t(I));
    c->d_hist = Q.get<int2>(size_t(I));
    ck(cudaMemsetAsync(c->d_hist, 0, size_t(I) * sizeof(int2), s), "memset");
    ck(cudaMemsetAsync(c->d_rho, 0, size_t(I) * Hs * sizeof(double), s), "memset");
    c->d_mask = Q.get<uint8_t>(size_t(I));
    c->mins.assign(size_t(I), Minimizer{});
    c->fused.assign(size_t(I), 0);
    for (int k = 0; k < I; k++) {
        const int4 r = irange[size_t(k)];
        c->fused[size_t(k)] = r.y - r.x <= fused_direction_limit() && c->H <= 64;
    }
    c->d_mins = Q.get<Minimizer>(size_t(I));
    c->d_mz = Q.get<MzStatus>(1);
    c->d_fused = Q.get<uint8_t>(size_t(I));
    h2d(c->d_fused, c->fused.data(), size_t(I), s);

    ck(cudaMemsetAsync(c->d_z, 0, n * sizeof(double), s), "memset");
    if (c->mixed) {
        prepare_beams_mixed(c->device);
        launch_mixed_constants(c->topo, c->mb, s);
        launch_plastic_mixed(c->topo, nullptr, c->d_plastic, nullptr, c->mb, s);
        c->rebase();
    }
    c->sync();
    c->have_topo = true;
}

void fill_diag(mcg_diag* d, const EvalOut& o) {
    if (!d) return;
    d->elastic = o.elastic; d->plastic = o.plastic; d->contact = o.contact;
    d->reaction = o.reaction; d->max_pen = o.max_pen; d->contacts = o.contacts; d->pad_ = 0;
}

}  // namespace

extern "C" {

int mcg_abi_version(void) { return MCG_ABI_VERSION; }

void mcg_config_defaults(mcg_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->cells_x = 4; c->cells_y = 6; c->cells_z = 4; c->elements_per_strut = 3;
    c->cell_size = .010; c->min_radius = .00082; c->max_radius = .00122; c->joint_scale = 1.18;
    c->trigger_scale = .38; c->imperfection = .00022; c->member_imperfection = .00022;
    c->material = mcg_material{1180, 26e6, .485, 5.2e6, 1.4e6, .06, .045};
    c->gravity = 9.81; c->shear_correction = .62; c->contact_stiffness = 1.2e6; c->contact_margin = 2e-5;
    c->centering_stiffness = 1.5; c->contact_samples = 3; c->load_steps = 52; c->unload_steps = 30;
    c->max_iterations = 130; c->history = 10; c->max_line_search = 22; c->max_strain = .62; c->step_time = .06;
    c->translation_scale = .010; c->max_translation_step = .0022; c->max_rotation_step = .30;
    c->gradient_rms_tolerance = 1.2e-3; c->gradient_max_tolerance = 1.5e-2; c->armijo = 1e-4;
    c->min_line_step = 1e-9; c->penetration_tolerance = .00012; c->max_adaptive_refinements = 7;
    c->fps = 24; c->frames = 83; c->threads = 0; c->seed = 0x494e445553545259ULL;
    c->relative_gradient_tolerance = 0; c->precision = MCG_FP64; c->self_contact = 1;
    c->reaction_relative_tolerance = 1.5e-3;
}

const char* mcg_status_string(int s) {
    switch (s) {
        case MCG_OK: return "ok";
        case MCG_ERR_INVALID: return "invalid argument";
        case MCG_ERR_CUDA: return "CUDA error";
        case MCG_ERR_NO_DEVICE: return "no CUDA device";
        case MCG_ERR_STATE: return "invalid call order";
        case MCG_ERR_EQUILIBRIUM: return "equilibrium failed";
        case MCG_ERR_CAPACITY: return "output capacity too small";
        case MCG_ERR_TIMEOUT: return "device wait timed out";
        default: return "unknown status";
    }
}

int mcg_create(const mcg_config* cfg, int device, mcg_ctx** out) {
    if (!cfg || !out) return MCG_ERR_INVALID;
    *out = nullptr;
    if (cfg->precision != MCG_FP64 && cfg->precision != MCG_MIXED) return MCG_ERR_INVALID;
    if (!(cfg->translation_scale > 0) || cfg->history < 0 || cfg->history > 64 || cfg->max_line_search < 0)
        return MCG_ERR_INVALID;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return MCG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return MCG_ERR_INVALID;
    mcg_ctx* c = new (std::nothrow) mcg_ctx;
    if (!c) return MCG_ERR_INVALID;
    c->cfg = *cfg;
    c->device = device;
    try {
        c->set_device();
        ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        c->hp.alloc(1);
    } catch (const Fail&) {
        delete c;
        return MCG_ERR_CUDA;
    }
    *out = c;
    return MCG_OK;
}

void mcg_destroy(mcg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->drop_graphs();
    c->topo_mem.release();
    c->eval_mem.release();
    c->contact_mem.release();
    c->solver_mem.release();
    c->hp.release();
    delete c;
}

const char* mcg_last_error(const mcg_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* mcg_stream(mcg_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int64_t mcg_launch_count(const mcg_ctx*) { return g_launch_count.load(); }

int mcg_upload_topology(mcg_ctx* c, const mcg_topology* t, const mcg_geometry* g, const double* x0, const double* r0) {
    return guarded(c, [&] {
        if (!t || !g) throw Fail(MCG_ERR_INVALID, "null topology or geometry");
        upload_instances(c, std::vector<InstIn>{InstIn{t, g, x0, r0, c->cfg.material.yield}});
    });
}

int mcg_upload_batch(mcg_ctx* c, int32_t count, const mcg_topology* topos, const mcg_geometry* geoms,
                     const double* const* x0, const double* const* r0, const double* yield) {
    return guarded(c, [&] {
        if (count <= 0 || !topos || !geoms) throw Fail(MCG_ERR_INVALID, "empty batch");
        std::vector<InstIn> ins;
        for (int k = 0; k < count; k++)
            ins.push_back(InstIn{topos + k, geoms + k, x0 ? x0[k] : nullptr, r0 ? r0[k] : nullptr,
                                 yield ? yield[k] : c->cfg.material.yield});
        upload_instances(c, ins);
    });
}

int32_t mcg_instance_count(const mcg_ctx* c) { return c && c->have_topo ? c->I : 0; }

int mcg_set_state(mcg_ctx* c, const double* bx, const double* br, const double* pl) {
    return guarded(c, [&] {
        need_topo(c);
        cudaStream_t s = c->stream;
        if (bx) h2d(c->d_baseX, bx, 3 * size_t(c->N), s);
        if (br) h2d(c->d_baseR, br, 4 * size_t(c->N), s);
        if (pl) {
            const size_t B = size_t(c->B);
            std::vector<double> soa(7 * B);
            for (size_t b = 0; b < B; b++)
                for (int k = 0; k < 7; k++) soa[size_t(k) * B + b] = pl[7 * b + size_t(k)];
            h2d(c->d_plastic, soa.data(), soa.size(), s);
            if (c->mixed) launch_plastic_mixed(c->topo, nullptr, c->d_plastic, nullptr, c->mb, s);
            c->sync();
        }
        if (bx || br) c->rebase();
        c->sync();
        c->have_final = false;
    });
}

int mcg_get_state(mcg_ctx* c, double* bx, double* br, double* pl) {
    return guarded(c, [&] {
        need_topo(c);
        cudaStream_t s = c->stream;
        if (bx) d2h(bx, c->d_baseX, 3 * size_t(c->N), s);
        if (br) d2h(br, c->d_baseR, 4 * size_t(c->N), s);
        if (pl) {
            const size_t B = size_t(c->B);
            std::vector<double> soa(7 * B);
            d2h(soa.data(), c->d_plastic, soa.size(), s);
            c->sync();
            for (size_t b = 0; b < B; b++)
                for (int k = 0; k < 7; k++) pl[7 * b + size_t(k)] = soa[size_t(k) * B + b];
        }
        c->sync();
    });
}

int mcg_objective(mcg_ctx* c, const double* z, double top, int trials, double* energy, double* grad,
                  mcg_diag* diag, double* trial_next, double* trial_aux, uint8_t* trial_flags) {
    return guarded(c, [&] {
        need_single(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        cudaStream_t s = c->stream;
        const size_t n = 6 * size_t(c->N), B = size_t(c->B);
        h2d(c->d_zin, z, n, s);
        c->hp.tops[0] = top;
        c->upload_tops();
        c->set_active(std::vector<uint8_t>(1, 1));
        const EvalOut o = c->eval_read(c->d_zin, trials != 0, c->d_grad, grad)[0];
        if (trials) c->have_final = false;
        if (energy) *energy = o.energy;
        fill_diag(diag, o);
        if (trials && c->mixed) {
            launch_f32_to_f64(7LL * c->B, c->ev.trial_nextf, c->ev.trial_next, s);
            launch_f32_to_f64(7LL * c->B, c->ev.trial_auxf, c->ev.trial_aux, s);
        }
        if (trials && (trial_next || trial_aux || trial_flags)) {
            std::vector<double> soa(7 * B);
            auto aos = [&](const double* d, double* out) {
                d2h(soa.data(), d, soa.size(), s);
                c->sync();
                for (size_t b = 0; b < B; b++)
                    for (int k = 0; k < 7; k++) out[7 * b + size_t(k)] = soa[size_t(k) * B + b];
            };
            if (trial_next) aos(c->ev.trial_next, trial_next);
            if (trial_aux) aos(c->ev.trial_aux, trial_aux);
            if (trial_flags) {
                std::vector<uint8_t> f(3 * B);
                d2h(f.data(), c->ev.trial_flags, f.size(), s);
                c->sync();
                for (size_t b = 0; b < B; b++)
                    for (int k = 0; k < 3; k++) trial_flags[3 * b + size_t(k)] = f[size_t(k) * B + b];
            }
        }
        c->sync();
    });
}

int mcg_batch_objective(mcg_ctx* c, const double* z, const double* tops, double* energies, double* grad,
                        mcg_diag* diags) {
    return guarded(c, [&] {
        need_topo(c);
        if (!z || !tops) throw Fail(MCG_ERR_INVALID, "null z or platen heights");
        const size_t n = 6 * size_t(c->N);
        h2d(c->d_zin, z, n, c->stream);
        for (int i = 0; i < c->I; i++) c->hp.tops[i] = tops[i];
        c->upload_tops();
        c->set_active(std::vector<uint8_t>(size_t(c->I), 1));
        const EvalOut* o = c->eval_read(c->d_zin, false, c->d_grad, grad);
        for (int i = 0; i < c->I; i++) {
            if (energies) energies[i] = o[i].energy;
            if (diags) fill_diag(diags + i, o[i]);
        }
    });
}

int mcg_upload_z(mcg_ctx* c, const double* z) {
    return guarded(c, [&] {
        need_topo(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        h2d(c->d_zin, z, 6 * size_t(c->N), c->stream);
        c->sync();
    });
}

int mcg_objective_resident(mcg_ctx* c, double top, int trials) {
    return guarded(c, [&] {
        need_single(c);
        c->set_active(std::vector<uint8_t>(1, 1));
        if (c->hp.tops[0] != top) {
            c->sync();
            c->hp.tops[0] = top;
            c->upload_tops();
        }
        c->eval(c->d_zin, trials != 0, c->d_grad);
        if (trials) c->have_final = false;
    });
}

int mcg_read_result(mcg_ctx* c, double* energy, double* grad, mcg_diag* diag) {
    return guarded(c, [&] {
        need_single(c);
        if (!c->last_z) throw Fail(MCG_ERR_STATE, "no evaluation to read");
        const EvalOut o = c->read_out();
        if (grad) d2h(grad, c->d_grad, 6 * size_t(c->N), c->stream);
        c->sync();
        if (energy) *energy = o.energy;
        fill_diag(diag, o);
    });
}

}  // extern "C"

namespace mcg {

// One evaluation whose self-contact scratch is `fixed` (caller-provided, never grown) and
// which allocates nothing: the building block of mcg_objective_noalloc (noalloc.cu).
int objective_with_fixed_contacts(mcg_ctx* c, ContactBufs& fixed, const double* z, double top, double* energy,
                                  double* grad, mcg_diag* diag) {
    return guarded(c, [&] {
        need_single(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        cudaStream_t s = c->stream;
        const size_t n = 6 * size_t(c->N);
        h2d(c->d_zin, z, n, s);
        c->hp.tops[0] = top;
        c->upload_tops();
        c->set_active(std::vector<uint8_t>(1, 1));
        PhysParams p = c->phys;
        p.broad_cell = c->broad_cell;
        p.inv_cell_f = float(1.0 / c->broad_cell);
        if (c->mixed) launch_state_mixed(c->topo, p, c->d_zin, c->d_baseX, c->mn, c->ev, s);
        else launch_state(c->topo, p, c->d_zin, c->d_baseX, c->d_baseR, c->ev, s);
        if (c->mixed) launch_beams_mixed(c->topo, c->mat, c->mb, c->mn, false, c->ev, s, c->beam_variant);
        else launch_beams(c->topo, c->mat, c->d_plastic, false, c->ev, s, c->beam_variant);
        const ContactBufs* cptr = nullptr;
        if (p.self_contact) {
            launch_contacts(c->topo, p, c->ev, fixed, c->rmax + c->cfg.contact_margin, 0.f, s);  // always rebuilds
            cptr = &fixed;
        }
        if (c->mixed) launch_gather_mixed(c->topo, p, cptr, c->d_grad, c->ev, s, c->gather_variant);
        else launch_gather(c->topo, p, cptr, c->d_grad, c->ev, s, c->gather_variant);
        launch_finalize(c->topo, p, cptr, c->d_grad, c->ev, s);
        c->check_launch();
        c->contacts_stale = p.self_contact != 0;
        d2h(c->hp.outs, c->ev.out, 1, s);
        c->sync();
        const EvalOut o = c->hp.outs[0];
        if (o.overflow) {
            std::string what;
            if (o.overflow & kOverEntries) what += " entries in one grid bin";
            if (o.overflow & kOverBins) what += " grid bins";
            if (o.overflow & kOverCandidates) what += " candidate pairs";
            if (o.overflow & kOverContacts) what += " contacts";
            if (o.overflow & kOverSpan) what += " cells spanned by one shape";
            throw Fail(MCG_ERR_CAPACITY, "this state needs more" + what +
                                             " than the fixed scratch of mcg_objective_noalloc holds");
        }
        if (grad) d2h(grad, c->d_grad, n, s);
        c->sync();
        if (energy) *energy = o.energy;
        fill_diag(diag, o);
    });
}

int ctx_counts(const mcg_ctx* c, int* n_nodes, int* n_beams, int* device) {
    if (!c || !c->have_topo || c->I != 1) return MCG_ERR_STATE;
    *n_nodes = c->N;
    *n_beams = c->B;
    *device = c->device;
    return MCG_OK;
}

void** ctx_noalloc_scratch(mcg_ctx* c) { return &c->noalloc_scratch; }

void ctx_set_error(mcg_ctx* c, const char* msg) {
    if (c) c->err = msg;
}

}  // namespace mcg

extern "C" {

int mcg_contact_pairs(mcg_ctx* c, uint64_t* keys, int64_t capacity, int64_t* count) {
    if (!c || !count) return MCG_ERR_INVALID;
    int rc = guarded(c, [&] {
        need_topo(c);
        if (c->contacts_stale)
            throw Fail(MCG_ERR_STATE, "the last evaluation was mcg_objective_noalloc's, whose contact pairs are not kept");
        const long long nc = c->phys.self_contact ? c->last_contacts : 0;
        *count = nc;
        if (nc > capacity) throw Fail(MCG_ERR_CAPACITY, "pair buffer too small");
        std::vector<uint32_t> a(static_cast<size_t>(nc)), b(static_cast<size_t>(nc));
        if (nc) {
            d2h(a.data(), c->cb.c_a, size_t(nc), c->stream);
            d2h(b.data(), c->cb.c_b, size_t(nc), c->stream);
        }
        c->sync();
        std::vector<uint64_t> k(static_cast<size_t>(nc));
        for (size_t i = 0; i < size_t(nc); i++) {
            const uint32_t u = std::min(a[i], b[i]), v = std::max(a[i], b[i]);
            k[i] = (uint64_t(u) << 32) | v;
        }
        std::sort(k.begin(), k.end());
        if (keys) std::copy(k.begin(), k.end(), keys);
    });
    return rc;
}

int mcg_minimize(mcg_ctx* c, double top, double* z, mcg_optstats* stats, double* final_energy, mcg_diag* fd) {
    return guarded(c, [&] {
        need_single(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        const size_t n = 6 * size_t(c->N);
        h2d(c->d_z, z, n, c->stream);
        c->start_minimize(0, top, false);
        c->minimize_all();
        const Minimizer& m = c->mins[0];
        d2h(z, c->d_z, n, c->stream);
        c->sync();
        c->have_final = true;
        if (stats) {
            stats->iterations = m.st.iterations; stats->backtracks = m.st.backtracks; stats->rms = m.st.rms;
            stats->max = m.st.max; stats->energy = m.st.energy; stats->converged = m.st.converged; stats->pad_ = 0;
        }
        if (final_energy) *final_energy = m.fin.energy;
        fill_diag(fd, m.fin);
        c->mins[0].phase = Minimizer::kIdle;
    });
}

int mcg_commit(mcg_ctx* c) {
    return guarded(c, [&] {
        need_single(c);
        if (!c->have_final) throw Fail(MCG_ERR_STATE, "commit without a preceding minimize");
        c->commit(std::vector<uint8_t>(1, 1));
        c->have_final = false;
    });
}

int mcg_set_contact_capacity(mcg_ctx* c, int64_t entries, int64_t candidates, int64_t contacts, int64_t bins) {
    return guarded(c, [&] {
        need_topo(c);
        if (entries < 0 || candidates < 0 || contacts < 0 || bins < 0 || bins > (1LL << 28))
            throw Fail(MCG_ERR_INVALID, "capacities must be non-negative and bins at most 2^28");
        const long long lo = 4096;
        c->sync();
        c->alloc_contacts(std::min<long long>(entries, 1LL << 20), std::max<long long>(contacts, lo),
                          std::max<long long>(bins, lo), std::max<long long>(candidates, lo));
    });
}

int mcg_set_contact_skin(mcg_ctx* c, double skin) {
    return guarded(c, [&] {
        need_topo(c);
        if (!(skin >= 0) || skin > 1e3) throw Fail(MCG_ERR_INVALID, "skin must be a distance >= 0 (m)");
        c->contact_skin = float(skin);
        c->drop_graphs();
        // the stored list was built for the previous skin
        ck(cudaMemsetAsync(c->cb.flags + 2, 1, 1, c->stream), "memset");
    });
}

int mcg_contact_stats(mcg_ctx* c, int64_t* out5) {
    return guarded(c, [&] {
        need_topo(c);
        if (!out5) throw Fail(MCG_ERR_INVALID, "null output");
        if (c->contacts_stale)
            throw Fail(MCG_ERR_STATE, "the last evaluation was mcg_objective_noalloc's, whose contact statistics are not kept");
        d2h(c->hp.u32, c->cb.nentries, 1, c->stream);
        d2h(c->hp.u32 + 1, c->cb.nentries + 2, 1, c->stream);
        d2h(c->hp.u32 + 2, c->cb.ncand, 1, c->stream);
        d2h(c->hp.u32 + 3, c->cb.foff + c->contact_chunks(), 1, c->stream);
        d2h(c->hp.u32 + 4, c->cb.hoff + c->contact_chunks(), 1, c->stream);
        c->sync();
        for (int k = 0; k < 5; k++) out5[k] = c->hp.u32[k];
    });
}

int mcg_set_solver_loop(mcg_ctx* c, int device) {
    return guarded(c, [&] {
        c->sync();
        c->device_loop = device != 0;
        c->loop_error.clear();
        for (auto& v : c->loop_ns) v = 0;
        c->loop_rounds = 0;
        c->loop_wall_ms = 0;
        c->drop_graphs();
    });
}

int mcg_solver_times(mcg_ctx* c, double* ms4, int64_t* rounds) {
    return guarded(c, [&] {
        if (!ms4) throw Fail(MCG_ERR_INVALID, "null output");
        for (int k = 0; k < 3; k++) ms4[k] = double(c->loop_ns[k]) * 1e-6;
        ms4[3] = c->loop_wall_ms;
        if (rounds) *rounds = c->loop_rounds;
    });
}

int mcg_solver_loop(mcg_ctx* c, int32_t* device) {
    return guarded(c, [&] {
        if (!device) throw Fail(MCG_ERR_INVALID, "null output");
        *device = c->device_loop ? 1 : 0;
        if (!c->device_loop && !c->loop_error.empty()) c->err = c->loop_error;
    });
}

int mcg_contact_builds(mcg_ctx* c, int64_t* builds) {
    return guarded(c, [&] {
        need_topo(c);
        if (!builds) throw Fail(MCG_ERR_INVALID, "null output");
        long long n = c->builds_before;
        if (c->cb.flags) {
            d2h(c->hp.u32, c->cb.flags + 4, 1, c->stream);
            c->sync();
            n += c->hp.u32[0];
        }
        *builds = n;
    });
}

int mcg_set_contact_cell(mcg_ctx* c, double cell) {
    return guarded(c, [&] {
        need_topo(c);
        if (!(cell >= 0) || cell > 1e3) throw Fail(MCG_ERR_INVALID, "cell must be a length >= 0 (m)");
        c->broad_cell = cell > 0 ? cell : c->default_cell();
        c->sync();
        c->alloc_contacts(c->cb.bin_slots, c->cb.contact_cap, c->cb.bin_cap, c->cb.cand_cap);
    });
}

int mcg_set_contact_shapes(mcg_ctx* c, double cell, int32_t pair_blocks) {
    return guarded(c, [&] {
        need_topo(c);
        if (!(cell >= 0) || cell > 1e3) throw Fail(MCG_ERR_INVALID, "cell must be a length >= 0 (m)");
        if (pair_blocks < 0 || pair_blocks > (1 << 20)) throw Fail(MCG_ERR_INVALID, "pair_blocks must be in 0 .. 2^20");
        c->broad_cell = cell > 0 ? cell : c->default_cell();
        c->pair_blocks_set = pair_blocks;
        c->sync();
        c->alloc_contacts(c->cb.bin_slots, c->cb.contact_cap, c->cb.bin_cap, c->cb.cand_cap);
    });
}

int mcg_set_kernel_shapes(mcg_ctx* c, int32_t beam_blocks, int32_t gather_blocks) {
    return guarded(c, [&] {
        need_topo(c);
        const ShapeKernel bk = c->mixed ? ShapeKernel::kBeamsMixed : ShapeKernel::kBeams;
        auto find = [](ShapeKernel k, int32_t blocks) {
            if (blocks == 0) return 0;
            for (int v = 0; v < shape_variants(k); v++)
                if (shape_blocks(k, v) == blocks) return v;
            throw Fail(MCG_ERR_INVALID, "no kernel variant with " + std::to_string(blocks) + " CTAs per SM");
        };
        const int bv = find(bk, beam_blocks), gv = find(ShapeKernel::kGather, gather_blocks);
        c->sync();
        c->set_kernel_variants(bv, gv);
    });
}

int mcg_autotune(mcg_ctx* c, const double* z, const double* tops, int32_t reps, mcg_tuning* out) {
    return guarded(c, [&] {
        need_topo(c);
        if (reps < 1 || reps > 1000) throw Fail(MCG_ERR_INVALID, "reps must be in 1 .. 1000");
        if (!c->cfg.self_contact) throw Fail(MCG_ERR_INVALID, "self-contact is off: nothing to tune");
        cudaStream_t s = c->stream;
        const size_t n = 6 * size_t(c->N);
        c->sync();
        if (z) h2d(c->d_zin, z, n, s);
        else ck(cudaMemsetAsync(c->d_zin, 0, n * sizeof(double), s), "memset");
        for (int i = 0; i < c->I; i++) c->hp.tops[i] = tops ? tops[i] : c->inst[size_t(i)].geom.top0;
        c->upload_tops();
        c->set_active(std::vector<uint8_t>(size_t(c->I), 1));
        const float skin = c->contact_skin;
        c->contact_skin = 0.f;  // time full builds
        const long long S = (long long)c->N + c->B;
        std::vector<int> blocks{0};
        for (int b : {152, 304, 608, 1216})
            if (b != contact_pair_blocks(S) && (long long)b * 8 * 32 <= std::max<long long>(S, 8 * 32)) blocks.push_back(b);
        const double cell0 = c->default_cell();
        std::vector<double> ref_e, e(size_t(c->I));
        std::vector<double> ref_g, g(n);
        cudaEvent_t t0 = nullptr, t1 = nullptr;
        ck(cudaEventCreate(&t0), "cudaEventCreate");
        ck(cudaEventCreate(&t1), "cudaEventCreate");
        struct Pick { double cell; int blocks; double ms; };
        std::vector<Pick> timed;
        double ms_default = 0;
        int tried = 0;
        try {
            for (double scale : {1.0, 0.9, 1.1, 1.25, 1.4})
                for (int b : blocks) {
                    c->broad_cell = scale * cell0;
                    c->pair_blocks_set = b;
                    c->alloc_contacts(c->cb.bin_slots, c->cb.contact_cap, c->cb.bin_cap, c->cb.cand_cap);
                    const EvalOut* o = c->eval_read(c->d_zin, false, c->d_grad);  // sizes the buffers
                    for (int i = 0; i < c->I; i++) e[size_t(i)] = o[i].energy;
                    d2h(g.data(), c->d_grad, n, s);
                    c->sync();
                    if (ref_e.empty()) {
                        ref_e = e;
                        ref_g = g;
                    } else if (std::memcmp(e.data(), ref_e.data(), e.size() * sizeof(double)) != 0 ||
                               std::memcmp(g.data(), ref_g.data(), n * sizeof(double)) != 0) {
                        throw Fail(MCG_ERR_MISMATCH, "broad-phase shapes changed an evaluation");
                    }
                    c->eval(c->d_zin, false, c->d_grad);  // captures the graph
                    ck(cudaEventRecord(t0, s), "cudaEventRecord");
                    for (int r = 0; r < reps; r++) c->eval(c->d_zin, false, c->d_grad);
                    ck(cudaEventRecord(t1, s), "cudaEventRecord");
                    c->read_outs();
                    if (c->hp.outs[0].overflow) throw Fail(MCG_ERR_CAPACITY, "contact buffers overflowed in tuning");
                    float ms = 0;
                    ck(cudaEventElapsedTime(&ms, t0, t1), "cudaEventElapsedTime");
                    const double per = double(ms) / reps;
                    if (tried == 0) ms_default = per;
                    tried++;
                    timed.push_back(Pick{c->broad_cell, c->pair_blocks_for(S), per});
                }
        } catch (...) {
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            c->contact_skin = skin;
            throw;
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        c->contact_skin = skin;
        // the fastest; among candidates within 1 % of it (timing noise) the one with the most
        // pair blocks, then the smallest cell, so that repeated tunings agree
        double fastest = 1e300;
        for (const Pick& q : timed) fastest = std::min(fastest, q.ms);
        Pick best{cell0, 0, 1e300};
        for (const Pick& q : timed)
            if (q.ms <= 1.01 * fastest &&
                (best.ms > 1e299 || q.blocks > best.blocks || (q.blocks == best.blocks && q.cell < best.cell)))
                best = q;
        c->broad_cell = best.cell;
        c->pair_blocks_set = best.blocks;
        c->alloc_contacts(c->cb.bin_slots, c->cb.contact_cap, c->cb.bin_cap, c->cb.cand_cap);
        // then the occupancy variants of the beam kernel and of the gather, one after the
        // other, timed on the same evaluation with the same bitwise check (ties within 1 %
        // keep the default)
        const ShapeKernel beam_kernel = c->mixed ? ShapeKernel::kBeamsMixed : ShapeKernel::kBeams;
        double best_ms = best.ms;
        ck(cudaEventCreate(&t0), "cudaEventCreate");
        ck(cudaEventCreate(&t1), "cudaEventCreate");
        c->contact_skin = 0.f;
        // each variant is timed on its own kernel (the evaluation's phase events): its share
        // of a whole evaluation is small enough to drown in the other kernels' variation
        if (!c->ev_t[0])
            for (auto& ev : c->ev_t) ck(cudaEventCreate(&ev), "cudaEventCreate");
        auto time_variant = [&](int bv, int gv, int phase) {
            c->set_kernel_variants(bv, gv);
            const EvalOut* o = c->eval_read(c->d_zin, false, c->d_grad);
            for (int i = 0; i < c->I; i++) e[size_t(i)] = o[i].energy;
            d2h(g.data(), c->d_grad, n, s);
            c->sync();
            if (std::memcmp(e.data(), ref_e.data(), e.size() * sizeof(double)) != 0 ||
                std::memcmp(g.data(), ref_g.data(), n * sizeof(double)) != 0)
                throw Fail(MCG_ERR_MISMATCH, "a kernel occupancy variant changed an evaluation");
            const bool timing_was = c->timing;
            double saved[mcg_ctx::kPhases];
            std::copy(c->phase_ms, c->phase_ms + mcg_ctx::kPhases, saved);
            const long long saved_n = c->phase_n;
            c->timing = true;
            std::fill(c->phase_ms, c->phase_ms + mcg_ctx::kPhases, 0.0);
            c->phase_n = 0;
            const int runs = std::max(reps, 5);
            for (int r = 0; r < runs; r++) c->eval(c->d_zin, false, c->d_grad);
            c->read_outs();
            const double ms = c->phase_ms[phase] / double(std::max(1LL, c->phase_n));
            c->timing = timing_was;
            std::copy(saved, saved + mcg_ctx::kPhases, c->phase_ms);
            c->phase_n = saved_n;
            tried++;
            return ms;
        };
        try {
            int bv = 0, gv = 0;
            double best_beam = time_variant(0, 0, 1);  // phase 1: the beam kernel
            for (int v = 1; v < shape_variants(beam_kernel); v++) {
                const double ms = time_variant(v, gv, 1);
                if (ms < 0.99 * best_beam) { best_beam = ms; bv = v; }
            }
            double best_gather = time_variant(bv, 0, 5);  // phase 5: the gather
            for (int v = 1; v < shape_variants(ShapeKernel::kGather); v++) {
                const double ms = time_variant(bv, v, 5);
                if (ms < 0.99 * best_gather) { best_gather = ms; gv = v; }
            }
            c->set_kernel_variants(bv, gv);
            // the whole evaluation with the chosen shapes
            c->eval(c->d_zin, false, c->d_grad);  // captures the graph
            ck(cudaEventRecord(t0, s), "cudaEventRecord");
            for (int r = 0; r < reps; r++) c->eval(c->d_zin, false, c->d_grad);
            ck(cudaEventRecord(t1, s), "cudaEventRecord");
            c->read_outs();
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, t0, t1), "cudaEventElapsedTime");
            best_ms = double(ms) / reps;
        } catch (...) {
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            c->contact_skin = skin;
            c->set_kernel_variants(0, 0);
            throw;
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        c->contact_skin = skin;
        c->sync();
        if (out)
            *out = mcg_tuning{best.cell, c->pair_blocks_for(S), tried, best_ms, ms_default,
                              shape_blocks(beam_kernel, c->beam_variant),
                              shape_blocks(ShapeKernel::kGather, c->gather_variant)};
    });
}

int mcg_set_timing(mcg_ctx* c, int on) {
    return guarded(c, [&] {
        if (on && !c->ev_t[0])
            for (auto& e : c->ev_t) ck(cudaEventCreate(&e), "cudaEventCreate");
        c->timing = on != 0;
        for (double& v : c->phase_ms) v = 0;
        c->phase_n = 0;
    });
}

int mcg_phase_times(mcg_ctx* c, double* ms, int32_t n, int64_t* evaluations) {
    if (!c || !ms || n < 0) return MCG_ERR_INVALID;
    for (int k = 0; k < n && k < mcg_ctx::kPhases; k++) ms[k] = c->phase_ms[k];
    if (evaluations) *evaluations = c->phase_n;
    return MCG_OK;
}

int mcg_run(mcg_ctx* c, mcg_frame* frames, int32_t capacity, int32_t* count, int verbose) {
    if (!c || !count) return MCG_ERR_INVALID;
    std::vector<Runner> rs;
    int rc = guarded(c, [&] {
        need_single(c);
        c->run(rs, verbose != 0);
    });
    const std::vector<mcg_frame> none;
    const std::vector<mcg_frame>& out = rs.empty() ? none : rs[0].frames;
    *count = int32_t(out.size());
    if (frames)
        for (size_t f = 0; f < out.size() && int32_t(f) < capacity; f++) frames[f] = out[f];
    if (rc == MCG_OK && !rs.empty() && rs[0].status != MCG_OK) {
        c->err = rs[0].error;
        rc = rs[0].status;
    }
    if (rc == MCG_OK && int32_t(out.size()) > capacity) {
        c->err = "frame buffer too small";
        return MCG_ERR_CAPACITY;
    }
    return rc;
}

int mcg_batch_run(mcg_ctx* c, mcg_frame* frames, int32_t capacity, int32_t* counts, int32_t* status) {
    if (!c || !counts || !status) return MCG_ERR_INVALID;
    std::vector<Runner> rs;
    int rc = guarded(c, [&] {
        need_topo(c);
        c->run(rs, false);
    });
    if (rc != MCG_OK) return rc;
    bool small = false;
    for (int i = 0; i < c->I; i++) {
        const std::vector<mcg_frame>& out = rs[size_t(i)].frames;
        counts[i] = int32_t(out.size());
        status[i] = rs[size_t(i)].status;
        small |= int32_t(out.size()) > capacity;
        if (frames)
            for (size_t f = 0; f < out.size() && int32_t(f) < capacity; f++)
                frames[size_t(i) * size_t(capacity) + f] = out[f];
    }
    if (small) {
        c->err = "frame buffer too small";
        return MCG_ERR_CAPACITY;
    }
    return MCG_OK;
}

}  // extern "C"
