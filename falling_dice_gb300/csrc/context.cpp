// context.cpp -- the C ABI (include/mcg.h): device context, topology upload, the
// energy/gradient evaluation, the L-BFGS minimizer and the load/unload driver.
//
// The solver logic follows the reference's Simulator::minimize / commit / run
// (MC/src/sim.cpp:174-213, 312-467) decision for decision; the vectors live on the device
// and only the scalars each decision needs are read back.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mcg.h"
#include "kernels.h"

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

struct Pinned {
    EvalOut out;
    double rmsmax[2];
    double dots[4];
    uint32_t u32[8];
    int grid[8];
};

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

struct HostStats {
    int iterations = 0, backtracks = 0;
    double rms = kInf, max = kInf, energy = kInf;
    bool converged = false;
};

}  // namespace

struct mcg_ctx {
    mcg_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int N = 0, B = 0;
    long long n_free = 0;
    bool have_topo = false;
    mcg_geometry geom{};
    double jr = 0, rmax = 0;

    DevArena topo_mem, eval_mem, contact_mem, solver_mem;
    DevTopo topo{};
    Material mat{};
    PhysParams phys{};
    EvalBufs ev{};
    ContactBufs cb{};
    long long last_contacts = 0;
    int last_sort_res = 0;

    double *d_baseX = nullptr, *d_baseR = nullptr, *d_plastic = nullptr;
    bool mixed = false;  // MCG_MIXED: FP32 bulk arithmetic (objective_mixed.cu)
    MixedBeams mb{};
    MixedNodes mn{};
    // Re-derives the mixed form's per-increment base terms after the base state changed.
    void rebase() {
        if (mixed) launch_rebase_mixed(topo, d_baseX, d_baseR, mb, mn, stream);
    }
    double *d_zin = nullptr, *d_grad = nullptr;
    Pinned* hp = nullptr;

    // solver vectors
    double *d_z = nullptr, *d_zc = nullptr, *d_p = nullptr, *d_g = nullptr, *d_gc = nullptr, *d_best = nullptr;
    std::vector<double*> d_S, d_Y;
    double *d_rho = nullptr, *d_alpha = nullptr, *d_scal = nullptr, *d_part = nullptr, *d_stats = nullptr;
    double* d_zfinal = nullptr;
    bool have_final = false;
    EvalOut final_out{};

    // run() bookkeeping (sim.hpp:47)
    double loadingWork = 0, recoveredWork = 0, prevDisp = 0, prevForce = 0, reactionOffset = 0;

    // optional per-phase timing of evaluations (events on the context stream)
    static constexpr int kPhases = 5;  // state, beams, contacts, gather, finalize
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
        for (auto& e : ev_t)
            if (e) cudaEventDestroy(e);
        if (hp) cudaFreeHost(hp);
        if (stream) cudaStreamDestroy(stream);
    }

    void set_device() { ck(cudaSetDevice(device), "cudaSetDevice"); }
    void sync() { ck(cudaStreamSynchronize(stream), "stream sync"); }
    void check_launch() { ck(cudaGetLastError(), "kernel launch"); }

    // ---- contact buffers ---------------------------------------------------------------
    double broad_cell = 0;   // current grid cell (the reference's size unless coarsened)
    float contact_skin = 0;  // candidate-list reuse distance (m); 0 rebuilds every evaluation
    void alloc_contacts(long long entry_cap, long long contact_cap, long long bin_cap, int region) {
        contact_mem.release();
        const long long S = (long long)N + B;
        ContactBufs c{};
        c.cell_lo = contact_mem.get<int4>(size_t(S));
        c.cell_hi = contact_mem.get<int4>(size_t(S));
        c.rec = contact_mem.get<uint4>(size_t(S));
        c.count = contact_mem.get<uint32_t>(size_t(S + 1));
        c.offset = contact_mem.get<uint32_t>(size_t(S + 1));
        c.grid = contact_mem.get<int>(16);
        c.flags = contact_mem.get<uint32_t>(4);
        c.xref = contact_mem.get<float4>(size_t(std::max(N, 1)));
        c.entry_cap = entry_cap;
        c.ekey = contact_mem.get<uint32_t>(size_t(entry_cap));
        c.erank = contact_mem.get<uint32_t>(size_t(entry_cap));
        c.sorted = contact_mem.get<uint32_t>(size_t(entry_cap));
        c.sorted2 = contact_mem.get<uint32_t>(size_t(entry_cap));
        c.bin_cap = bin_cap;
        c.bin_count = contact_mem.get<uint32_t>(size_t(bin_cap + 1));
        c.bin_start = contact_mem.get<uint32_t>(size_t(bin_cap + 1));
        c.bcount = contact_mem.get<uint32_t>(size_t(bin_cap + 1));
        c.boffset = contact_mem.get<uint32_t>(size_t(bin_cap + 1));
        c.occ = contact_mem.get<uint32_t>(size_t(bin_cap));
        c.pair_blocks = contact_pair_blocks(S);
        const long long W = (long long)c.pair_blocks * 8;
        c.region = std::max(32, (region + 31) / 32 * 32);
        c.cand = contact_mem.get<uint2>(size_t(W * c.region));
        c.wcount = contact_mem.get<uint32_t>(size_t(W));
        c.wcap = contact_mem.get<uint32_t>(size_t(W + 1));
        c.woff = contact_mem.get<uint32_t>(size_t(W + 1));
        const long long chunks = W * c.region / 32;
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
        c.part = contact_mem.get<double>(size_t(3 * contact_part_blocks(contact_cap)));
        c.scan_tmp_bytes = scan_tmp_bytes(std::max({S + 1, bin_cap + 1, (long long)N + 1, W + 1, chunks + 1}));
        c.scan_tmp = contact_mem.get<unsigned char>(c.scan_tmp_bytes);
        ck(cudaMemsetAsync(c.flags, 0, 4 * sizeof(uint32_t), stream), "memset");
        ck(cudaMemsetAsync(c.flags + 2, 1, 1, stream), "memset");  // the first evaluation builds the list
        cb = c;
    }

    // Grows whatever the last evaluation overflowed; false when nothing did.
    bool grow_contacts(int flags) {
        if (!(flags & (kOverEntries | kOverContacts | kOverBins | kOverSpan | kOverCandidates))) return false;
        const long long S = (long long)N + B;
        const long long W = (long long)cb.pair_blocks * 8;
        uint32_t need[2] = {0, 0};
        int grid[16];
        std::vector<uint32_t> wc(static_cast<size_t>(W));
        ck(cudaMemcpyAsync(&need[0], cb.offset + S, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "copy");
        ck(cudaMemcpyAsync(&need[1], cb.hoff + W * cb.region / 32, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream),
           "copy");
        ck(cudaMemcpyAsync(grid, cb.grid, sizeof(grid), cudaMemcpyDeviceToHost, stream), "copy");
        ck(cudaMemcpyAsync(wc.data(), cb.wcount, size_t(W) * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        long long ecap = cb.entry_cap, ccap = cb.contact_cap, bcap = cb.bin_cap;
        int region = cb.region;
        if (flags & kOverCandidates) {
            const long long mx = *std::max_element(wc.begin(), wc.end());
            region = int(std::min<long long>(std::max<long long>(region, mx + mx / 4 + 32), 1LL << 26));
        }
        if (flags & kOverSpan) broad_cell *= 2;
        if (flags & kOverEntries) ecap = std::max(ecap, (long long)need[0] + need[0] / 4 + 1024);
        if (flags & kOverContacts) ccap = std::max(ccap, (long long)need[1] + need[1] / 4 + 1024);
        if (flags & kOverBins) {
            const long long want = (long long)grid[9] + grid[9] / 4 + 1024;
            if (want <= (1LL << 28)) bcap = std::max(bcap, want);
            else broad_cell *= 2;  // a huge extent: coarser cells instead of more bins
        }
        alloc_contacts(ecap, ccap, bcap, region);
        return true;
    }

    // One evaluation of the objective at device z; grad written to d_gout; totals in ev.out.
    // Enqueues only: no host synchronisation.
    void eval(const double* dz, double top, bool trials, double* d_gout) {
        PhysParams p = phys;
        p.top = top;
        p.broad_cell = broad_cell;
        p.inv_cell_f = float(1.0 / broad_cell);
        mark(0);
        if (mixed) launch_state_mixed(topo, p, dz, d_baseX, mn, ev, stream);
        else launch_state(topo, p, dz, d_baseX, d_baseR, ev, stream);
        mark(1);
        if (mixed) launch_beams_mixed(topo, mat, mb, mn, trials, ev, stream);
        else launch_beams(topo, mat, d_plastic, trials, ev, stream);
        mark(2);
        const ContactBufs* cptr = nullptr;
        if (p.self_contact) {
            launch_contacts(topo, p, ev, cb, rmax + cfg.contact_margin, contact_skin, stream);
            cptr = &cb;
        }
        mark(3);
        if (mixed) launch_gather_mixed(topo, p, cptr, d_gout, ev, stream);
        else launch_gather(topo, p, cptr, d_gout, ev, stream);
        mark(4);
        launch_finalize(topo, p, cptr, d_gout, ev, stream);
        mark(5);
        check_launch();
        collect();
        last_top = top;
        last_z = dz;
        last_trials = trials;
        last_grad = d_gout;
    }
    double last_top = 0;
    const double* last_z = nullptr;
    bool last_trials = false;
    double* last_grad = nullptr;

    // Evaluation whose totals are read back; repeats it with larger contact buffers when a
    // capacity was exceeded.
    EvalOut eval_read(const double* dz, double top, bool trials, double* d_gout) {
        eval(dz, top, trials, d_gout);
        EvalOut o = read_out_raw();
        for (int tries = 0; o.overflow && tries < 16; tries++) {
            if (!grow_contacts(o.overflow)) break;
            eval(dz, top, trials, d_gout);
            o = read_out_raw();
        }
        if (o.overflow) throw Fail(MCG_ERR_CAPACITY, "contact buffers could not be sized");
        if (cfg.self_contact) last_contacts = read_contact_count();
        return o;
    }
    long long read_contact_count() {
        uint32_t nc = 0;
        ck(cudaMemcpyAsync(&nc, cb.hoff + (long long)cb.pair_blocks * 8 * cb.region / 32, sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        return nc;
    }
    EvalOut read_out_raw() {
        ck(cudaMemcpyAsync(&hp->out, ev.out, sizeof(EvalOut), cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        return hp->out;
    }
    // Totals of the last evaluation, repeating it if it overflowed a contact buffer.
    EvalOut read_out() {
        EvalOut o = read_out_raw();
        if (o.overflow) o = eval_read(last_z, last_top, last_trials, last_grad);
        else if (cfg.self_contact) last_contacts = read_contact_count();
        return o;
    }
    void read_rms_max(const double* g, double& rms, double& mx) {
        rms_max(g, topo.locked, 6LL * N, n_free, d_part, d_stats, stream);
        ck(cudaMemcpyAsync(hp->rmsmax, d_stats, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        rms = hp->rmsmax[0];
        mx = hp->rmsmax[1];
    }
    double read_dot(const double* a, const double* b) {
        dots(1, a, b, nullptr, nullptr, nullptr, nullptr, 6LL * N, d_part, d_stats + 4, stream);
        ck(cudaMemcpyAsync(hp->dots, d_stats + 4, sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        return hp->dots[0];
    }

    // ---- Simulator::minimize, MC/src/sim.cpp:174-211 --------------------------------------
    HostStats minimize(double top, EvalOut& fin) {
        const long long n = 6LL * N;
        const int H = std::max(0, cfg.history);
        HostStats st;
        int m = 0, head = 0;  // history: slots (head + h) % H, h = 0 oldest
        auto slot = [&](int h) { return (head + h) % std::max(H, 1); };
        EvalOut cur = eval_read(d_z, top, false, d_g);
        double cur_rms, cur_max;
        read_rms_max(d_g, cur_rms, cur_max);
        double best_energy = cur.energy;
        vcopy(d_best, d_z, n, stream);
        const double rms0 = cur_rms;
        auto converged = [&](const EvalOut& o, double rms, double mx) {
            if (cfg.relative_gradient_tolerance > 0)
                return (rms <= cfg.relative_gradient_tolerance * rms0) && o.max_pen <= cfg.penetration_tolerance;
            const double rel = rms / std::max(1e-6, cfg.translation_scale * std::max(1.0, o.reaction));
            const bool forceOK = (rms <= cfg.gradient_rms_tolerance && mx <= cfg.gradient_max_tolerance) || rel < 1.5e-3;
            return forceOK && o.max_pen <= cfg.penetration_tolerance;
        };
        EvalOut cand{};
        auto line_search = [&](double dg) {
            double step = 1.0;
            for (int bt = 0; bt < cfg.max_line_search; bt++) {
                candidate(d_zc, d_z, d_p, step, topo.locked, n, stream);
                cand = eval_read(d_zc, top, false, d_gc);
                st.backtracks++;
                if (std::isfinite(cand.energy) && cand.energy <= cur.energy + cfg.armijo * step * dg) return true;
                step *= .5;
                if (step < cfg.min_line_step) break;
            }
            return false;
        };
        std::vector<const double*> S(H), Y(H), R(H);
        for (int it = 0; it < cfg.max_iterations; it++) {
            st.iterations = it + 1;
            st.rms = cur_rms;
            st.max = cur_max;
            st.energy = cur.energy;
            if (converged(cur, cur_rms, cur_max)) {
                st.converged = true;
                break;
            }
            for (int h = 0; h < m; h++) {
                S[h] = d_S[slot(h)];
                Y[h] = d_Y[slot(h)];
                R[h] = d_rho + slot(h);
            }
            two_loop(d_p, d_g, S.data(), Y.data(), R.data(), m, d_alpha, d_scal, d_part, n, stream);
            finish_direction(d_p, d_p, topo.locked, N, cfg.max_translation_step / cfg.translation_scale,
                             cfg.max_rotation_step, stream);
            double dg = read_dot(d_g, d_p);
            if (!(dg < 0)) {  // not a descent direction: steepest descent (sim.cpp:191)
                m = 0;
                finish_direction(d_p, d_g, topo.locked, N, cfg.max_translation_step / cfg.translation_scale,
                                 cfg.max_rotation_step, stream);
                dg = read_dot(d_g, d_p);
            }
            bool ok = line_search(dg);
            if (!ok) {  // steepest-descent retry (sim.cpp:193-203)
                m = 0;
                finish_direction(d_p, d_g, topo.locked, N, cfg.max_translation_step / cfg.translation_scale,
                                 cfg.max_rotation_step, stream);
                dg = read_dot(d_g, d_p);
                ok = line_search(dg);
            }
            if (!ok) break;
            // curvature pair (sim.cpp:205-206) into the slot it would occupy
            const int target = H == 0 ? 0 : (m < H ? slot(m) : slot(0));
            double sy = 0, ss = 0, yy = 0;
            if (H > 0) {
                make_sy(d_S[target], d_Y[target], d_zc, d_z, d_gc, d_g, n, stream);
                dots(3, d_S[target], d_Y[target], d_S[target], d_S[target], d_Y[target], d_Y[target], n, d_part,
                     d_stats + 4, stream);
            }
            rms_max(d_gc, topo.locked, n, n_free, d_part, d_stats, stream);
            ck(cudaMemcpyAsync(hp->rmsmax, d_stats, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
            ck(cudaMemcpyAsync(hp->dots, d_stats + 4, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
            sync();
            if (H > 0) {
                sy = hp->dots[0];
                ss = hp->dots[1];
                yy = hp->dots[2];
                if (sy > 1e-12 * std::sqrt(std::max(1e-30, ss * yy))) {
                    set_rho(d_rho + target, d_stats + 4, stream);
                    if (m == H) head = (head + 1) % H;
                    else m++;
                } else {
                    m = 0;
                }
            }
            std::swap(d_z, d_zc);
            std::swap(d_g, d_gc);
            cur = cand;
            cur_rms = hp->rmsmax[0];
            cur_max = hp->rmsmax[1];
            if (cur.energy < best_energy) {
                best_energy = cur.energy;
                vcopy(d_best, d_z, n, stream);
            }
        }
        if (!st.converged && best_energy < cur.energy) vcopy(d_z, d_best, n, stream);
        fin = eval_read(d_z, top, true, d_g);
        read_rms_max(d_g, st.rms, st.max);
        st.energy = fin.energy;
        st.converged = converged(fin, st.rms, st.max);
        vcopy(d_zfinal, d_z, n, stream);
        have_final = true;
        final_out = fin;
        check_launch();
        return st;
    }

    // ---- Simulator::commit, MC/src/sim.cpp:212 --------------------------------------------
    void commit() {
        if (!have_final) throw Fail(MCG_ERR_STATE, "commit without a preceding minimize");
        PhysParams p = phys;
        launch_state(topo, p, d_zfinal, d_baseX, d_baseR, ev, stream);
        if (mixed) {
            launch_commit(N, B, ev, d_baseX, d_baseR, nullptr, stream);
            launch_plastic_mixed(B, nullptr, ev.trial_nextf, mb, stream);
            launch_plastic_mixed_to_f64(B, mb, d_plastic, stream);
        } else {
            launch_commit(N, B, ev, d_baseX, d_baseR, d_plastic, stream);
        }
        rebase();
        have_final = false;
        check_launch();
    }

    double top_y(double s, bool loading) const {
        const double compressed = geom.top0 - cfg.max_strain * geom.height;
        const double t = std::max(0.0, std::min(1.0, s));
        return loading ? geom.top0 * (1.0 - t) + compressed * t : compressed * (1.0 - t) + geom.top0 * t;
    }

    // ---- Simulator::diagnostics, MC/src/sim.cpp:312-372 -------------------------------------
    mcg_frame diagnostics(double time, double top, bool loading, const EvalOut& o, const HostStats& s) {
        mcg_frame d;
        std::memset(&d, 0, sizeof(d));
        d.time = time;
        d.platen_y = top;
        d.displacement = geom.top0 - top;
        d.engineering_strain = d.displacement / std::max(1e-12, geom.height);
        d.reaction_force = std::max(0.0, o.reaction - reactionOffset);
        d.engineering_stress = d.reaction_force / std::max(1e-12, geom.area);
        d.loading_work = loadingWork;
        d.recovered_work = recoveredWork;
        d.dissipated_work = std::max(0.0, loadingWork - recoveredWork);
        d.specific_energy_absorption = d.dissipated_work / std::max(1e-12, geom.mass);
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
        // plastic statistics and the node height extent of the committed state
        double ps[8];
        launch_plastic_stats(B, d_plastic, d_part, d_stats, stream);
        ck(cudaMemcpyAsync(ps, d_stats, 6 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
        double box[9];
        ck(cudaMemcpyAsync(box, ev.cen, 9 * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
        sync();
        if (B > 0) {
            d.mean_plastic_strain = ps[0] / B;
            d.max_plastic_strain = ps[1];
            d.mean_plastic_rotation = ps[2] / B;
            d.max_plastic_rotation = ps[3];
        }
        d.plastic_beams = int(ps[4]);
        d.plastic_hinges = int(ps[5]);
        const double currentHeight = std::max(0.0, box[7] - box[4]);
        d.permanent_set = std::max(0.0, 1.0 - currentHeight / std::max(1e-12, geom.height));
        return d;
    }

    // ---- Simulator::run, MC/src/sim.cpp:374-467 ----------------------------------------------
    int run(std::vector<mcg_frame>& frames, bool verbose) {
        loadingWork = recoveredWork = prevDisp = prevForce = reactionOffset = 0;
        double time = 0, currentTop = geom.top0;
        bool first = true;
        int accepted = 0;
        const long long n = 6LL * N;
        std::function<void(double, bool, int)> advanceTo = [&](double targetTop, bool loading, int refinement) {
            ck(cudaMemsetAsync(d_z, 0, size_t(n) * sizeof(double), stream), "memset");
            EvalOut fin{};
            const HostStats stats = minimize(targetTop, fin);
            const bool acceptable = stats.converged && fin.max_pen <= cfg.penetration_tolerance && std::isfinite(fin.energy);
            if (!acceptable && refinement < cfg.max_adaptive_refinements && std::abs(targetTop - currentTop) > 2.5e-5) {
                const double midpoint = 0.5 * (currentTop + targetTop);
                advanceTo(midpoint, loading, refinement + 1);
                advanceTo(targetTop, loading, refinement + 1);
                return;
            }
            if (!acceptable) {
                char msg[256];
                std::snprintf(msg, sizeof msg,
                              "quasi-static equilibrium failed at platen=%g m, residual=%g, penetration=%g mm after %d iterations",
                              targetTop, stats.rms, fin.max_pen * 1000.0, stats.iterations);
                throw Fail(MCG_ERR_EQUILIBRIUM, msg);
            }
            commit();
            if (first) reactionOffset = fin.reaction;
            const double force = std::max(0.0, fin.reaction - reactionOffset);
            const double displacement = geom.top0 - targetTop;
            if (!first) {
                const double dd = displacement - prevDisp;
                const double work = 0.5 * (prevForce + force) * dd;
                if (dd >= 0.0) loadingWork += std::max(0.0, work);
                else recoveredWork += std::max(0.0, -work);
            }
            prevDisp = displacement;
            prevForce = force;
            currentTop = targetTop;
            mcg_frame d = diagnostics(time, targetTop, loading, fin, stats);
            d.refinement = refinement;
            frames.push_back(d);
            if (verbose)
                std::printf("[equilibrium] %3d %s strain=%.4f force=%.3f N residual=%.2e pen=%.3f mm iter=%d %s\n",
                            accepted, loading ? "load  " : "unload", d.engineering_strain, d.reaction_force,
                            d.residual_rms, d.max_penetration * 1000.0, d.iterations, refinement ? "[REFINED]" : "[OK]");
            accepted++;
            first = false;
            time += cfg.step_time;
        };
        advanceTo(geom.top0, true, 0);
        for (int step = 1; step <= cfg.load_steps; ++step)
            advanceTo(top_y(double(step) / std::max(1, cfg.load_steps), true), true, 0);
        for (int step = 1; step <= cfg.unload_steps; ++step)
            advanceTo(top_y(double(step) / std::max(1, cfg.unload_steps), false), false, 0);
        return MCG_OK;
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

template <class T>
void h2d(T* d, const T* h, size_t n, cudaStream_t s) {
    ck(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, s), "copy to device");
}
template <class T>
void d2h(T* h, const T* d, size_t n, cudaStream_t s) {
    ck(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, s), "copy to host");
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
    if (!(cfg->translation_scale > 0) || cfg->history < 0 || cfg->max_line_search < 0) return MCG_ERR_INVALID;
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
        ck(cudaMallocHost(reinterpret_cast<void**>(&c->hp), sizeof(Pinned)), "cudaMallocHost");
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
    c->topo_mem.release();
    c->eval_mem.release();
    c->contact_mem.release();
    c->solver_mem.release();
    delete c;
}

const char* mcg_last_error(const mcg_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* mcg_stream(mcg_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int64_t mcg_launch_count(const mcg_ctx*) { return g_launch_count.load(); }

int mcg_upload_topology(mcg_ctx* c, const mcg_topology* t, const mcg_geometry* g, const double* x0, const double* r0) {
    return guarded(c, [&] {
        if (!t || !g) throw Fail(MCG_ERR_INVALID, "null topology or geometry");
        const int N = t->n_nodes, B = t->n_beams;
        if (N <= 0 || B < 0) throw Fail(MCG_ERR_INVALID, "node count must be positive and beam count non-negative");
        if ((long long)N + B >= (1LL << 31) / 4) throw Fail(MCG_ERR_INVALID, "model too large for 32-bit shape indices");
        if (B > 0 && (!t->beam_a || !t->beam_b || !t->L0 || !t->radius || !t->area || !t->I || !t->J || !t->e0))
            throw Fail(MCG_ERR_INVALID, "missing beam array");
        if (!t->mass || !t->locked) throw Fail(MCG_ERR_INVALID, "missing node array");
        if (t->n_connected < 0 || (t->n_connected > 0 && !t->connected))
            throw Fail(MCG_ERR_INVALID, "bad connected list");
        const mcg_config& cf = c->cfg;
        const double E = cf.material.young, G = E / (2 * (1 + cf.material.nu)), sy = cf.material.yield;
        std::vector<int2> ab(static_cast<size_t>(B));
        std::vector<double> kb(B), kt(B), my(B), ty(B), hb(B), ht(B), cs(B), aL(B), aLsy(B);
        std::vector<double> invL0(B), inv_kbh(B), inv_kth(B);
        std::vector<double> e0x(B), e0y(B), e0z(B);
        std::vector<float> padf(B);
        double rmax = cf.joint_scale * cf.max_radius;
        std::vector<int> deg(size_t(N) + 1, 0);
        for (int b = 0; b < B; b++) {
            const int a = t->beam_a[b], bb = t->beam_b[b];
            if (a < 0 || a >= N || bb < 0 || bb >= N || a == bb)
                throw Fail(MCG_ERR_INVALID, "beam " + std::to_string(b) + " has invalid end nodes");
            const double L0 = t->L0[b], r = t->radius[b];
            if (!(L0 > 0) || !std::isfinite(L0) || !(r > 0) || !std::isfinite(r) || !std::isfinite(t->area[b]) ||
                !std::isfinite(t->I[b]) || !std::isfinite(t->J[b]))
                throw Fail(MCG_ERR_INVALID, "beam " + std::to_string(b) + " has invalid section data");
            ab[size_t(b)] = make_int2(a, bb);
            deg[size_t(a)]++;
            deg[size_t(bb)]++;
            // Section constants, evaluated with the reference's expressions
            // (sim.cpp:139-141); this file is compiled without FMA contraction, so the
            // values equal the ones the reference recomputes on every call.
            const double area = t->area[b], I = t->I[b], J = t->J[b];
            kb[b] = E * I / L0;
            kt[b] = G * J / L0;
            my[b] = sy * I / r;
            ty[b] = (sy / std::sqrt(3.0)) * J / r;
            hb[b] = cf.material.bend_hardening * kb[b];
            ht[b] = cf.material.torsion_hardening * kt[b];
            cs[b] = .5 * cf.shear_correction * G * area * L0;
            aL[b] = area * L0;
            aLsy[b] = area * L0 * sy;
            invL0[b] = 1.0 / L0;
            inv_kbh[b] = 1.0 / std::max(1e-20, kb[b] + hb[b]);
            inv_kth[b] = 1.0 / std::max(1e-20, kt[b] + ht[b]);
            e0x[b] = t->e0[3 * size_t(b)];
            e0y[b] = t->e0[3 * size_t(b) + 1];
            e0z[b] = t->e0[3 * size_t(b) + 2];
            rmax = std::max(rmax, r);
            padf[b] = round_up_float(r + cf.contact_margin);
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
        // connected-pair adjacency
        std::vector<std::vector<int>> adj(static_cast<size_t>(N));
        for (int64_t k = 0; k < t->n_connected; k++) {
            const uint64_t key = t->connected[k];
            const uint32_t u = uint32_t(key >> 32), v = uint32_t(key & 0xffffffffu);
            if (u >= uint32_t(N) || v >= uint32_t(N) || u > v)
                throw Fail(MCG_ERR_INVALID, "connected key " + std::to_string(k) + " is not a node pair key");
            adj[u].push_back(int(v));
            if (u != v) adj[v].push_back(int(u));
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
        long long nfree = 0;
        for (long long k = 0; k < 6LL * N; k++) {
            if (t->locked[k] > 1) throw Fail(MCG_ERR_INVALID, "locked flags must be 0 or 1");
            nfree += t->locked[k] ? 0 : 1;
        }
        for (int i = 0; i < N; i++)
            if (!std::isfinite(t->mass[i])) throw Fail(MCG_ERR_INVALID, "non-finite node mass");

        c->sync();
        c->topo_mem.release();
        c->eval_mem.release();
        c->contact_mem.release();
        c->solver_mem.release();
        c->have_topo = false;
        c->have_final = false;
        c->N = N;
        c->B = B;
        c->n_free = nfree;
        c->geom = *g;
        c->jr = cf.joint_scale * cf.max_radius;
        c->rmax = rmax;
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
        T.L0 = upd(std::vector<double>(t->L0, t->L0 + B));
        T.area = upd(std::vector<double>(t->area, t->area + B));
        T.radius = upd(std::vector<double>(t->radius, t->radius + B));
        T.e0x = upd(e0x); T.e0y = upd(e0y); T.e0z = upd(e0z);
        T.kb = upd(kb); T.kt = upd(kt); T.my = upd(my); T.ty = upd(ty); T.hb = upd(hb); T.ht = upd(ht);
        T.cs = upd(cs); T.aL = upd(aL); T.aLsy = upd(aLsy);
        T.invL0 = upd(invL0); T.inv_kbh = upd(inv_kbh); T.inv_kth = upd(inv_kth);
        T.mass = upd(std::vector<double>(t->mass, t->mass + N));
        uint8_t* dl = M.get<uint8_t>(6 * size_t(N));
        h2d(dl, t->locked, 6 * size_t(N), s);
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
            if (B) h2d(dp, padf.data(), size_t(B), s);
            T.padf = dp;
        }
        c->topo = T;
        c->mat = Material{E, G, sy, cf.material.hardening, cf.material.bend_hardening, cf.material.torsion_hardening,
                          1.0 / std::max(1e-20, E + cf.material.hardening)};
        PhysParams P{};
        P.translation_scale = cf.translation_scale;
        P.gravity = cf.gravity;
        P.centering = cf.centering_stiffness;
        P.contact_k = cf.contact_stiffness;
        P.contact_margin = cf.contact_margin;
        P.joint_radius = c->jr;
        P.broad_cell = std::max(2.8 * c->jr, .72 * cf.cell_size);
        P.top = g->top0;
        P.self_contact = cf.self_contact ? 1 : 0;
        P.joint_padf = round_up_float(c->jr + cf.contact_margin);
        c->phys = P;
        // state
        c->d_baseX = M.get<double>(3 * size_t(N));
        c->d_baseR = M.get<double>(4 * size_t(N));
        c->d_plastic = M.get<double>(7 * size_t(B));
        ck(cudaMemsetAsync(c->d_plastic, 0, 7 * size_t(B) * sizeof(double), s), "memset");
        if (x0) h2d(c->d_baseX, x0, 3 * size_t(N), s);
        if (r0) {
            h2d(c->d_baseR, r0, 4 * size_t(N), s);
        } else if (x0) {
            std::vector<double> id(4 * size_t(N), 0.0);
            for (int i = 0; i < N; i++) id[4 * size_t(i)] = 1.0;
            h2d(c->d_baseR, id.data(), id.size(), s);
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
        e.part_state = V.get<double>(9 * size_t(nb_nodes(N)));
        e.part_beam = V.get<double>(3 * size_t(nb_beams(std::max(B, 1))));
        e.part_node = V.get<double>(kNodeParts * size_t(nb_nodes(N)));
        e.cen = V.get<double>(9);
        e.out = V.get<EvalOut>(1);
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
            float4** fields[] = {&mb.B0, &mb.B1, &mb.B2, &mb.B3, &mb.B4, &mb.B5, &mb.C0, &mb.C1, &mb.P0, &mb.P1};
            for (float4** f : fields) *f = V.get<float4>(size_t(B));
            c->mb = mb;
            c->mn = MixedNodes{V.get<float4>(size_t(N)), V.get<float4>(size_t(N)), V.get<float4>(size_t(N))};
        }
        c->ev = e;
        c->d_zin = V.get<double>(6 * size_t(N));
        c->d_grad = V.get<double>(6 * size_t(N));
        ck(cudaMemsetAsync(c->d_zin, 0, 6 * size_t(N) * sizeof(double), s), "memset");
        // contact buffers: a first guess, grown on demand
        const long long S = (long long)N + B;
        c->broad_cell = P.broad_cell;
        c->contact_skin = float(0.125 * cf.cell_size);
        {
            // bins: the Morton range of the rest-state extent, with room to grow
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            if (x0)
                for (int i = 0; i < N; i++)
                    for (int d = 0; d < 3; d++) {
                        lo[d] = std::min(lo[d], x0[3 * size_t(i) + d]);
                        hi[d] = std::max(hi[d], x0[3 * size_t(i) + d]);
                    }
            long long dmax = 8;
            if (x0)
                for (int d = 0; d < 3; d++)
                    dmax = std::max(dmax, (long long)((hi[d] - lo[d] + 2 * c->rmax) / P.broad_cell * 1.15) + 4);
            int bits = 3;
            while ((1LL << bits) < dmax && bits < 10) bits++;
            const long long bin_cap = std::min(1LL << (3 * bits), 1LL << 27);
            c->alloc_contacts(std::max<long long>(8 * S, 4096), std::max<long long>(S / 2, 4096), bin_cap, 1024);
        }
        // solver vectors
        DevArena& Q = c->solver_mem;
        const size_t n = 6 * size_t(N);
        c->d_z = Q.get<double>(n); c->d_zc = Q.get<double>(n); c->d_p = Q.get<double>(n);
        c->d_g = Q.get<double>(n); c->d_gc = Q.get<double>(n); c->d_best = Q.get<double>(n);
        c->d_zfinal = Q.get<double>(n);
        c->d_S.assign(size_t(cf.history), nullptr);
        c->d_Y.assign(size_t(cf.history), nullptr);
        for (int h = 0; h < cf.history; h++) { c->d_S[size_t(h)] = Q.get<double>(n); c->d_Y[size_t(h)] = Q.get<double>(n); }
        c->d_rho = Q.get<double>(size_t(std::max(cf.history, 1)));
        c->d_alpha = Q.get<double>(size_t(std::max(cf.history, 1)));
        c->d_scal = Q.get<double>(8);
        c->d_part = Q.get<double>(lbfgs_part_doubles());
        c->d_stats = Q.get<double>(16);
        ck(cudaMemsetAsync(c->d_z, 0, n * sizeof(double), s), "memset");
        if (c->mixed) {
            launch_mixed_constants(c->topo, c->mb, s);
            launch_plastic_mixed(B, c->d_plastic, nullptr, c->mb, s);
            c->rebase();
        }
        c->sync();
        c->have_topo = true;
    });
}

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
            if (c->mixed) launch_plastic_mixed(c->B, c->d_plastic, nullptr, c->mb, s);
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
        need_topo(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        cudaStream_t s = c->stream;
        const size_t n = 6 * size_t(c->N), B = size_t(c->B);
        h2d(c->d_zin, z, n, s);
        const EvalOut o = c->eval_read(c->d_zin, top, trials != 0, c->d_grad);
        if (trials) c->have_final = false;
        if (grad) d2h(grad, c->d_grad, n, s);
        if (energy) *energy = o.energy;
        if (diag) {
            diag->elastic = o.elastic; diag->plastic = o.plastic; diag->contact = o.contact;
            diag->reaction = o.reaction; diag->max_pen = o.max_pen; diag->contacts = o.contacts; diag->pad_ = 0;
        }
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
        need_topo(c);
        c->eval(c->d_zin, top, trials != 0, c->d_grad);
        if (trials) c->have_final = false;
    });
}

int mcg_read_result(mcg_ctx* c, double* energy, double* grad, mcg_diag* diag) {
    return guarded(c, [&] {
        need_topo(c);
        if (!c->last_z) throw Fail(MCG_ERR_STATE, "no evaluation to read");
        const EvalOut o = c->read_out();
        if (grad) d2h(grad, c->d_grad, 6 * size_t(c->N), c->stream);
        c->sync();
        if (energy) *energy = o.energy;
        if (diag) {
            diag->elastic = o.elastic; diag->plastic = o.plastic; diag->contact = o.contact;
            diag->reaction = o.reaction; diag->max_pen = o.max_pen; diag->contacts = o.contacts; diag->pad_ = 0;
        }
    });
}

}  // extern "C"

namespace mcg {

// One evaluation whose self-contact scratch is `fixed` (caller-provided, never grown) and
// which allocates nothing: the building block of mcg_objective_noalloc (noalloc.cu).
int objective_with_fixed_contacts(mcg_ctx* c, ContactBufs& fixed, const double* z, double top, double* energy,
                                  double* grad, mcg_diag* diag) {
    return guarded(c, [&] {
        need_topo(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        cudaStream_t s = c->stream;
        const size_t n = 6 * size_t(c->N);
        h2d(c->d_zin, z, n, s);
        PhysParams p = c->phys;
        p.top = top;
        p.broad_cell = c->broad_cell;
        p.inv_cell_f = float(1.0 / c->broad_cell);
        if (c->mixed) launch_state_mixed(c->topo, p, c->d_zin, c->d_baseX, c->mn, c->ev, s);
        else launch_state(c->topo, p, c->d_zin, c->d_baseX, c->d_baseR, c->ev, s);
        if (c->mixed) launch_beams_mixed(c->topo, c->mat, c->mb, c->mn, false, c->ev, s);
        else launch_beams(c->topo, c->mat, c->d_plastic, false, c->ev, s);
        const ContactBufs* cptr = nullptr;
        if (p.self_contact) {
            launch_contacts(c->topo, p, c->ev, fixed, c->rmax + c->cfg.contact_margin, 0.f, s);  // always rebuilds
            cptr = &fixed;
        }
        if (c->mixed) launch_gather_mixed(c->topo, p, cptr, c->d_grad, c->ev, s);
        else launch_gather(c->topo, p, cptr, c->d_grad, c->ev, s);
        launch_finalize(c->topo, p, cptr, c->d_grad, c->ev, s);
        c->check_launch();
        const EvalOut o = c->read_out_raw();
        if (o.overflow) {
            std::string what;
            if (o.overflow & kOverEntries) what += " cell entries";
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
        if (diag) {
            diag->elastic = o.elastic; diag->plastic = o.plastic; diag->contact = o.contact;
            diag->reaction = o.reaction; diag->max_pen = o.max_pen; diag->contacts = o.contacts; diag->pad_ = 0;
        }
    });
}

int ctx_counts(const mcg_ctx* c, int* n_nodes, int* n_beams, int* device) {
    if (!c || !c->have_topo) return MCG_ERR_STATE;
    *n_nodes = c->N;
    *n_beams = c->B;
    *device = c->device;
    return MCG_OK;
}

void ctx_set_error(mcg_ctx* c, const char* msg) {
    if (c) c->err = msg;
}

}  // namespace mcg

extern "C" {

int mcg_contact_pairs(mcg_ctx* c, uint64_t* keys, int64_t capacity, int64_t* count) {
    if (!c || !count) return MCG_ERR_INVALID;
    int rc = guarded(c, [&] {
        need_topo(c);
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
        need_topo(c);
        if (!z) throw Fail(MCG_ERR_INVALID, "null z");
        const size_t n = 6 * size_t(c->N);
        h2d(c->d_z, z, n, c->stream);
        EvalOut fin{};
        const HostStats st = c->minimize(top, fin);
        d2h(z, c->d_z, n, c->stream);
        c->sync();
        if (stats) {
            stats->iterations = st.iterations; stats->backtracks = st.backtracks; stats->rms = st.rms;
            stats->max = st.max; stats->energy = st.energy; stats->converged = st.converged; stats->pad_ = 0;
        }
        if (final_energy) *final_energy = fin.energy;
        if (fd) {
            fd->elastic = fin.elastic; fd->plastic = fin.plastic; fd->contact = fin.contact;
            fd->reaction = fin.reaction; fd->max_pen = fin.max_pen; fd->contacts = fin.contacts; fd->pad_ = 0;
        }
    });
}

int mcg_commit(mcg_ctx* c) {
    return guarded(c, [&] {
        need_topo(c);
        c->commit();
        c->sync();
    });
}

int mcg_set_contact_capacity(mcg_ctx* c, int64_t entries, int64_t candidates, int64_t contacts, int64_t bins) {
    return guarded(c, [&] {
        need_topo(c);
        if (entries < 0 || candidates < 0 || contacts < 0 || bins < 0 || bins > (1LL << 28))
            throw Fail(MCG_ERR_INVALID, "capacities must be non-negative and bins at most 2^28");
        const long long lo = 4096;
        c->sync();
        const long long W = (long long)contact_pair_blocks((long long)c->N + c->B) * 8;
        c->alloc_contacts(std::max<long long>(entries, lo), std::max<long long>(contacts, lo),
                          std::max<long long>(bins, lo), int(std::min<long long>((candidates + W - 1) / W, 1LL << 26)));
    });
}

int mcg_set_contact_skin(mcg_ctx* c, double skin) {
    return guarded(c, [&] {
        need_topo(c);
        if (!(skin >= 0) || skin > 1e3) throw Fail(MCG_ERR_INVALID, "skin must be a distance >= 0 (m)");
        c->contact_skin = float(skin);
        // the stored list was built for the previous skin
        ck(cudaMemsetAsync(c->cb.flags + 2, 1, 1, c->stream), "memset");
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
    std::vector<mcg_frame> out;
    int rc = guarded(c, [&] {
        need_topo(c);
        c->run(out, verbose != 0);
    });
    *count = int32_t(out.size());
    if (frames)
        for (size_t f = 0; f < out.size() && int32_t(f) < capacity; f++) frames[f] = out[f];
    if (rc == MCG_OK && int32_t(out.size()) > capacity) {
        c->err = "frame buffer too small";
        return MCG_ERR_CAPACITY;
    }
    return rc;
}

}  // extern "C"
