// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY: a C harness around the reference's own
// solver, compiled from the unmodified reference sources where they lie (build recipe:
// oracle/Makefile, target `ref`, output oracle/_ref/libmcref.so).  It is only built where
// the reference tree exists; it never ships and no product code links it.
//
// The reference keeps everything on the path private (MC/include/sim.hpp:44-53) and its
// helpers in an anonymous namespace (MC/src/sim.cpp:4-47), so this translation unit
// includes MC/src/sim.cpp itself with `private` opened.  core.hpp must be included before
// `private` is redefined, or libstdc++'s <sstream> stops compiling.
#include "include/core.hpp"
#define private public
#include "src/sim.cpp"
#undef private

#include <algorithm>
#include <cstring>
#include <iostream>
#include <memory>

#include "oracle.h"

using namespace meta;

struct orc_model {
    std::unique_ptr<Simulator> sim;
    std::vector<double> lastZ;
    Objective lastFinal;
    bool haveFinal = false;
};

namespace {

SimulationConfig toConfig(const mcg_config& c) {
    SimulationConfig s;
    s.cellsX = c.cells_x; s.cellsY = c.cells_y; s.cellsZ = c.cells_z;
    s.cellSize = c.cell_size; s.minRadius = c.min_radius; s.maxRadius = c.max_radius;
    s.jointScale = c.joint_scale; s.triggerScale = c.trigger_scale;
    s.imperfection = c.imperfection; s.memberImperfection = c.member_imperfection;
    s.elementsPerStrut = c.elements_per_strut;
    s.material.density = c.material.density; s.material.young = c.material.young;
    s.material.nu = c.material.nu; s.material.yield = c.material.yield;
    s.material.hardening = c.material.hardening;
    s.material.bendHardening = c.material.bend_hardening;
    s.material.torsionHardening = c.material.torsion_hardening;
    s.gravity = c.gravity; s.shearCorrection = c.shear_correction;
    s.contactStiffness = c.contact_stiffness; s.contactMargin = c.contact_margin;
    s.centeringStiffness = c.centering_stiffness; s.contactSamples = c.contact_samples;
    s.loadSteps = c.load_steps; s.unloadSteps = c.unload_steps;
    s.maxIterations = c.max_iterations; s.history = c.history;
    s.maxLineSearch = c.max_line_search; s.maxStrain = c.max_strain; s.stepTime = c.step_time;
    s.translationScale = c.translation_scale; s.maxTranslationStep = c.max_translation_step;
    s.maxRotationStep = c.max_rotation_step;
    s.gradientRmsTolerance = c.gradient_rms_tolerance;
    s.gradientMaxTolerance = c.gradient_max_tolerance; s.armijo = c.armijo;
    s.minLineStep = c.min_line_step; s.penetrationTolerance = c.penetration_tolerance;
    s.maxAdaptiveRefinements = c.max_adaptive_refinements; s.fps = c.fps;
    s.frames = c.frames; s.threads = c.threads; s.seed = c.seed;
    return s;
}

void fillDiag(const ObjectiveDiag& d, mcg_diag* out) {
    if (!out) return;
    out->elastic = d.elastic; out->plastic = d.plastic; out->contact = d.contact;
    out->reaction = d.reaction; out->max_pen = d.maxPen; out->contacts = d.contacts;
    out->pad_ = 0;
}

void fillStats(const OptStats& s, mcg_optstats* out) {
    if (!out) return;
    out->iterations = s.iterations; out->backtracks = s.backtracks; out->rms = s.rms;
    out->max = s.max; out->energy = s.energy; out->converged = s.converged ? 1 : 0;
    out->pad_ = 0;
}

std::vector<double> vec(const double* p, size_t n) { return std::vector<double>(p, p + n); }

}  // namespace

extern "C" {

int orc_is_reference(void) { return 1; }

orc_model* orc_create_builder(const mcg_config* cfg) {
    auto m = new orc_model;
    m->sim = std::make_unique<Simulator>(toConfig(*cfg));
    return m;
}

orc_model* orc_create_injected(const mcg_config* cfg, const mcg_topology* t,
                               const mcg_geometry* g, const double* x0, const double* r0,
                               const int32_t* layer) {
    // Construct a minimal reference model, then overwrite every member the path reads.
    SimulationConfig tiny = toConfig(*cfg);
    tiny.cellsX = tiny.cellsY = tiny.cellsZ = 1;
    auto m = new orc_model;
    m->sim = std::make_unique<Simulator>(tiny);
    Simulator& s = *m->sim;
    s.cfg_ = toConfig(*cfg);
    const size_t N = size_t(t->n_nodes), B = size_t(t->n_beams);
    s.nodes_.assign(N, Node{});
    for (size_t i = 0; i < N; i++) {
        Node& n = s.nodes_[i];
        n.x0 = {x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]};
        n.x = n.x0;
        n.R = r0 ? Quat{r0[4 * i], r0[4 * i + 1], r0[4 * i + 2], r0[4 * i + 3]} : Quat{};
        n.mass = t->mass[i];
        n.layer = layer ? layer[i] : 0;
    }
    s.beams_.assign(B, Beam{});
    for (size_t b = 0; b < B; b++) {
        Beam& e = s.beams_[b];
        e.a = t->beam_a[b]; e.b = t->beam_b[b]; e.L0 = t->L0[b]; e.radius = t->radius[b];
        e.area = t->area[b]; e.I = t->I[b]; e.J = t->J[b];
        e.e0 = {t->e0[3 * b], t->e0[3 * b + 1], t->e0[3 * b + 2]};
    }
    s.connected_.clear();
    for (int64_t k = 0; k < t->n_connected; k++) s.connected_.insert(t->connected[k]);
    s.locked_.assign(t->locked, t->locked + 6 * N);
    s.baseX_.resize(N); s.baseR_.resize(N);
    for (size_t i = 0; i < N; i++) { s.baseX_[i] = s.nodes_[i].x; s.baseR_[i] = s.nodes_[i].R; }
    s.width_ = g->width; s.height_ = g->height; s.depth_ = g->depth;
    s.area_ = g->area; s.mass_ = g->mass; s.top0_ = g->top0;
    return m;
}

void orc_free(orc_model* m) { delete m; }

void orc_counts(const orc_model* m, int32_t* n, int32_t* b, int64_t* nc) {
    const Simulator& s = *m->sim;
    if (n) *n = int32_t(s.nodes_.size());
    if (b) *b = int32_t(s.beams_.size());
    if (nc) *nc = int64_t(s.connected_.size());
}

void orc_export(const orc_model* m, double* x0, double* r0, int32_t* layer, double* mass,
                uint8_t* locked, int32_t* beam_a, int32_t* beam_b, double* L0, double* radius,
                double* area, double* I, double* J, double* e0, uint64_t* connected,
                mcg_geometry* geom, double* translation_scale) {
    const Simulator& s = *m->sim;
    for (size_t i = 0; i < s.nodes_.size(); i++) {
        const Node& n = s.nodes_[i];
        if (x0) { x0[3 * i] = n.x0.x; x0[3 * i + 1] = n.x0.y; x0[3 * i + 2] = n.x0.z; }
        if (r0) { r0[4 * i] = n.R.w; r0[4 * i + 1] = n.R.x; r0[4 * i + 2] = n.R.y; r0[4 * i + 3] = n.R.z; }
        if (layer) layer[i] = n.layer;
        if (mass) mass[i] = n.mass;
    }
    if (locked) std::copy(s.locked_.begin(), s.locked_.end(), locked);
    for (size_t b = 0; b < s.beams_.size(); b++) {
        const Beam& e = s.beams_[b];
        if (beam_a) beam_a[b] = e.a;
        if (beam_b) beam_b[b] = e.b;
        if (L0) L0[b] = e.L0;
        if (radius) radius[b] = e.radius;
        if (area) area[b] = e.area;
        if (I) I[b] = e.I;
        if (J) J[b] = e.J;
        if (e0) { e0[3 * b] = e.e0.x; e0[3 * b + 1] = e.e0.y; e0[3 * b + 2] = e.e0.z; }
    }
    if (connected) {
        std::vector<uint64_t> keys(s.connected_.begin(), s.connected_.end());
        std::sort(keys.begin(), keys.end());
        std::copy(keys.begin(), keys.end(), connected);
    }
    if (geom) {
        geom->width = s.width_; geom->height = s.height_; geom->depth = s.depth_;
        geom->area = s.area_; geom->mass = s.mass_; geom->top0 = s.top0_;
    }
    if (translation_scale) *translation_scale = s.cfg_.translationScale;
}

void orc_set_state(orc_model* m, const double* bx, const double* br, const double* pl) {
    Simulator& s = *m->sim;
    for (size_t i = 0; i < s.nodes_.size(); i++) {
        if (bx) {
            s.baseX_[i] = {bx[3 * i], bx[3 * i + 1], bx[3 * i + 2]};
            s.nodes_[i].x = s.baseX_[i];
        }
        if (br) {
            s.baseR_[i] = {br[4 * i], br[4 * i + 1], br[4 * i + 2], br[4 * i + 3]};
            s.nodes_[i].R = s.baseR_[i];
        }
    }
    if (pl)
        for (size_t b = 0; b < s.beams_.size(); b++) {
            PlasticState& p = s.beams_[b].plastic;
            const double* q = pl + 7 * b;
            p.epsp = q[0]; p.alpha = q[1]; p.rotp = {q[2], q[3], q[4]}; p.alphaB = q[5]; p.alphaT = q[6];
        }
}

void orc_get_state(const orc_model* m, double* bx, double* br, double* pl) {
    const Simulator& s = *m->sim;
    for (size_t i = 0; i < s.nodes_.size(); i++) {
        if (bx) { bx[3 * i] = s.baseX_[i].x; bx[3 * i + 1] = s.baseX_[i].y; bx[3 * i + 2] = s.baseX_[i].z; }
        if (br) { br[4 * i] = s.baseR_[i].w; br[4 * i + 1] = s.baseR_[i].x; br[4 * i + 2] = s.baseR_[i].y; br[4 * i + 3] = s.baseR_[i].z; }
    }
    if (pl)
        for (size_t b = 0; b < s.beams_.size(); b++) {
            const PlasticState& p = s.beams_[b].plastic;
            double* q = pl + 7 * b;
            q[0] = p.epsp; q[1] = p.alpha; q[2] = p.rotp.x; q[3] = p.rotp.y; q[4] = p.rotp.z;
            q[5] = p.alphaB; q[6] = p.alphaT;
        }
}

static void exportTrials(const Objective& o, double* next, double* aux, uint8_t* flags) {
    for (size_t b = 0; b < o.trial.size(); b++) {
        const TrialBeam& t = o.trial[b];
        if (next) {
            double* q = next + 7 * b;
            q[0] = t.next.epsp; q[1] = t.next.alpha; q[2] = t.next.rotp.x; q[3] = t.next.rotp.y;
            q[4] = t.next.rotp.z; q[5] = t.next.alphaB; q[6] = t.next.alphaT;
        }
        if (aux) {
            double* q = aux + 7 * b;
            q[0] = t.strain; q[1] = t.stress; q[2] = t.moment.x; q[3] = t.moment.y;
            q[4] = t.moment.z; q[5] = t.elastic; q[6] = t.dissipation;
        }
        if (flags) {
            flags[3 * b] = t.axialPlastic; flags[3 * b + 1] = t.bendPlastic;
            flags[3 * b + 2] = t.torsionPlastic;
        }
    }
}

double orc_objective(const orc_model* m, const double* z, double top, int trials,
                     double* grad, mcg_diag* diag, double* next, double* aux, uint8_t* flags) {
    const Simulator& s = *m->sim;
    Objective o = s.objective(vec(z, 6 * s.nodes_.size()), top, trials != 0);
    if (grad) std::copy(o.grad.begin(), o.grad.end(), grad);
    fillDiag(o.d, diag);
    if (trials) exportTrials(o, next, aux, flags);
    return o.energy;
}

int64_t orc_contact_pairs(const orc_model* m, const double* z, uint64_t* keys, int64_t cap) {
    // Every pair whose distance is below target shares a grid cell in the reference's
    // broad phase (the cell lists hold the margin-inflated AABBs, MC/src/sim.cpp:154), so
    // the reference's contact set is exactly the set of non-local pairs closer than
    // target.  This enumerates that set with a sweep over x, using the reference's own
    // geometry and exclusion functions.
    const Simulator& s = *m->sim;
    std::vector<Vec3> x; std::vector<Quat> R;
    s.state(vec(z, 6 * s.nodes_.size()), x, R);
    const double jr = s.cfg_.jointScale * s.cfg_.maxRadius;
    std::vector<ContactShape> shapes;
    for (int i = 0; i < int(s.nodes_.size()); i++) shapes.push_back({x[size_t(i)], x[size_t(i)], jr, i, -1, -1, false});
    for (int bi = 0; bi < int(s.beams_.size()); bi++) {
        const Beam& e = s.beams_[size_t(bi)];
        shapes.push_back({x[size_t(e.a)], x[size_t(e.b)], e.radius, e.a, e.b, bi, true});
    }
    const double m_ = s.cfg_.contactMargin;
    struct Box { Vec3 lo, hi; int id; };
    std::vector<Box> boxes;
    for (int si = 0; si < int(shapes.size()); si++) {
        const ContactShape& c = shapes[size_t(si)];
        boxes.push_back({minVec(c.a, c.b) - Vec3(c.r + m_), maxVec(c.a, c.b) + Vec3(c.r + m_), si});
    }
    std::sort(boxes.begin(), boxes.end(), [](const Box& a, const Box& b) {
        return a.lo.x < b.lo.x || (a.lo.x == b.lo.x && a.id < b.id);
    });
    std::vector<uint64_t> out;
    for (size_t p = 0; p < boxes.size(); p++)
        for (size_t q = p + 1; q < boxes.size() && boxes[q].lo.x <= boxes[p].hi.x; q++) {
            const Box &A = boxes[p], &Bx = boxes[q];
            if (A.lo.y > Bx.hi.y || Bx.lo.y > A.hi.y || A.lo.z > Bx.hi.z || Bx.lo.z > A.hi.z) continue;
            int ai = std::min(A.id, Bx.id), bi = std::max(A.id, Bx.id);
            const ContactShape &a = shapes[size_t(ai)], &b = shapes[size_t(bi)];
            if (localShapes(a, b, s.connected_)) continue;
            ClosestPair cp = closestShapes(a, b);
            double dist = length(cp.pb - cp.pa), target = a.r + b.r + m_;
            if (dist >= target) continue;
            out.push_back(pairKey(ai, bi));
        }
    std::sort(out.begin(), out.end());
    for (int64_t k = 0; k < int64_t(out.size()) && k < cap; k++) keys[k] = out[size_t(k)];
    return int64_t(out.size());
}

int orc_minimize(orc_model* m, double top, double* z, mcg_optstats* stats, double* fe,
                 mcg_diag* fd) {
    Simulator& s = *m->sim;
    std::vector<double> zz = vec(z, 6 * s.nodes_.size());
    Objective final;
    OptStats st = s.minimize(top, zz, final);
    std::copy(zz.begin(), zz.end(), z);
    fillStats(st, stats);
    if (fe) *fe = final.energy;
    fillDiag(final.d, fd);
    m->lastZ = zz;
    m->lastFinal = std::move(final);
    m->haveFinal = true;
    return 0;
}

int orc_commit(orc_model* m) {
    if (!m->haveFinal) return MCG_ERR_STATE;
    m->sim->commit(m->lastZ, m->lastFinal);
    m->haveFinal = false;
    return 0;
}

static void fillFrame(const FrameDiagnostics& d, mcg_frame* f) {
    std::memset(f, 0, sizeof(*f));
    f->time = d.time; f->platen_y = d.platenY; f->displacement = d.displacement;
    f->engineering_strain = d.engineeringStrain; f->engineering_stress = d.engineeringStress;
    f->reaction_force = d.reactionForce; f->loading_work = d.loadingWork;
    f->recovered_work = d.recoveredWork; f->dissipated_work = d.dissipatedWork;
    f->specific_energy_absorption = d.specificEnergyAbsorption;
    f->elastic_energy = d.elasticEnergy; f->plastic_dissipation = d.plasticDissipation;
    f->contact_energy = d.contactEnergy; f->residual_rms = d.residualRms;
    f->residual_max = d.residualMax; f->max_penetration = d.maxPenetration;
    f->mean_plastic_strain = d.meanPlasticStrain; f->max_plastic_strain = d.maxPlasticStrain;
    f->mean_plastic_rotation = d.meanPlasticRotation;
    f->max_plastic_rotation = d.maxPlasticRotation; f->permanent_set = d.permanentSet;
    f->active_contacts = d.activeContacts; f->plastic_beams = d.plasticBeams;
    f->plastic_hinges = d.plasticHinges; f->iterations = d.iterations;
    f->converged = d.converged; f->loading = d.loading;
}

int orc_run(orc_model* m, mcg_frame* frames, int32_t cap, int32_t* count, int verbose) {
    std::streambuf* saved = std::cout.rdbuf();
    std::ostringstream sink;
    if (!verbose) std::cout.rdbuf(sink.rdbuf());
    int rc = 0;
    *count = 0;
    try {
        SimulationResult r = m->sim->run();
        for (size_t f = 0; f < r.diagnostics.size() && int32_t(f) < cap; f++) fillFrame(r.diagnostics[f], frames + f);
        *count = int32_t(r.diagnostics.size());
    } catch (const std::exception& e) {
        rc = MCG_ERR_EQUILIBRIUM;
    }
    std::cout.rdbuf(saved);
    return rc;
}

double orc_rigid_rotation_error(const orc_model* m) {
    double e = 0;
    m->sim->rigidRotationTest(&e);
    return e;
}

double orc_gradient_check_error(const orc_model* m) {
    double e = 0;
    m->sim->gradientCheck(&e);
    return e;
}

double orc_beam_potential(const orc_model* m, const double* x, const double* r) {
    const Simulator& s = *m->sim;
    std::vector<Vec3> xv(s.nodes_.size());
    std::vector<Quat> rv(s.nodes_.size());
    for (size_t i = 0; i < xv.size(); i++) {
        xv[i] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
        rv[i] = {r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]};
    }
    return s.beamPotential(xv, rv);
}

double orc_top_y(const orc_model* m, double s, int loading) { return m->sim->topY(s, loading != 0); }

int orc_set_variant(orc_model*, int variant) { return variant == 0 ? 0 : -1; }  // the reference has one order

}  // extern "C"
