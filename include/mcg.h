/*
 * mcg.h -- C ABI of the GB300 beam-lattice energy/gradient + L-BFGS library.
 *
 * The reference solver (projects/metamaterial-compression/industry-grade, "MC/"
 * below) keeps this path behind one private C++ member,
 *   Objective Simulator::objective(const std::vector<double>& z, double top,
 *                                  bool trials) const          (MC/include/sim.hpp:49,
 *                                                               MC/src/sim.cpp:138-172)
 * and its caller Simulator::minimize (MC/src/sim.cpp:174-211).  The reference has no
 * FFI of its own; the entry points below are what its solver binds to replace that
 * member: plain pointers and sizes, no C++ or torch types.  Every function returns an int
 * status (MCG_OK = 0); mcg_last_error() gives the message.  Contexts own their device
 * memory and are not thread-safe: use one context per host thread, as the reference uses
 * one Simulator per thread.  Every call on a context makes the context's CUDA device the
 * current device of the calling thread.
 *
 * Layouts (all host arrays are caller-owned, copied in/out):
 *   z, grad      6 doubles per node: [tx, ty, tz, rx, ry, rz]; translations in units of
 *                translation_scale, rotations as a rotation vector (MC/src/sim.cpp:136).
 *   base_x       3 doubles per node (m).       base_r   4 doubles per node (w, x, y, z).
 *   plastic      7 doubles per beam: [epsp, alpha, rotp.x, rotp.y, rotp.z, alphaB, alphaT]
 *                (PlasticState, MC/include/sim.hpp:28).
 *   e0           3 doubles per beam (material director, MC/include/sim.hpp:29).
 *   connected    pair keys (min << 32 | max) of node pairs excluded from self-contact
 *                (Simulator::connected_, MC/src/sim.cpp:115-117; key as core.hpp:47 pairKey).
 *   locked       one byte per DOF (Simulator::locked_, MC/src/sim.cpp:134).
 */
#ifndef MCG_H
#define MCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCG_ABI_VERSION 2

enum mcg_status {
    MCG_OK = 0,
    MCG_ERR_INVALID = 1,     /* bad argument, size or topology */
    MCG_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    MCG_ERR_NO_DEVICE = 3,   /* no usable GPU */
    MCG_ERR_STATE = 4,       /* call order (objective before topology, commit before minimize) */
    MCG_ERR_EQUILIBRIUM = 5, /* run(): an increment failed after all bisections (the
                                reference throws std::runtime_error, MC/src/sim.cpp:412-419) */
    MCG_ERR_CAPACITY = 6,    /* an output buffer is too small; the needed count is returned */
    MCG_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up */
    MCG_ERR_MISMATCH = 8,    /* a self-check failed: results that must agree bit for bit did not */
};

enum mcg_precision {
    MCG_FP64 = 0,  /* plain form: FP64 throughout (the correctness oracle on the GPU); the
                      solver takes the reference's decisions exactly */
    MCG_MIXED = 1, /* FP32 bulk element/contact arithmetic, FP64 reductions; energies carry
                      ~3e-10 relative rounding noise, so the line search accepts a step when
                      E_new <= E + armijo step dg + 1e-9 |E| (convergence is still judged on
                      the gradient) */
};

/* MaterialConfig, MC/include/sim.hpp:16 (the name string is not carried). */
typedef struct mcg_material {
    double density, young, nu, yield, hardening, bend_hardening, torsion_hardening;
} mcg_material;

/* SimulationConfig, MC/include/sim.hpp:17-26, field for field, plus two extensions at
 * the end.  mcg_config_defaults() fills the reference defaults. */
typedef struct mcg_config {
    int32_t cells_x, cells_y, cells_z, elements_per_strut;
    double cell_size, min_radius, max_radius, joint_scale, trigger_scale;
    double imperfection, member_imperfection;
    mcg_material material;
    double gravity, shear_correction, contact_stiffness, contact_margin, centering_stiffness;
    int32_t contact_samples, load_steps, unload_steps, max_iterations, history, max_line_search;
    double max_strain, step_time, translation_scale, max_translation_step, max_rotation_step;
    double gradient_rms_tolerance, gradient_max_tolerance, armijo, min_line_step;
    double penetration_tolerance;
    int32_t max_adaptive_refinements, fps, frames, threads;
    uint64_t seed;
    /* Extensions (no reference counterpart). */
    double relative_gradient_tolerance; /* > 0: converge when rms(g)/rms(g at iteration 0)
                                           <= this, in place of the absolute test */
    int32_t precision;                  /* enum mcg_precision */
    int32_t self_contact;               /* 1 = on (reference behaviour), 0 = off */
    double reaction_relative_tolerance; /* the alternative convergence test
                                           rms/(translation_scale max(1, reaction)) < this
                                           (sim.cpp:177); 0: the reference's 1.5e-3;
                                           < 0: off (only the absolute rms/max test) */
} mcg_config;

void mcg_config_defaults(mcg_config* cfg);

/* The model arrays the objective reads (Node/Beam, MC/include/sim.hpp:27-29). */
typedef struct mcg_topology {
    int32_t n_nodes, n_beams;
    const int32_t* beam_a;      /* [B] */
    const int32_t* beam_b;      /* [B] */
    const double* L0;           /* [B] */
    const double* radius;       /* [B] */
    const double* area;         /* [B] */
    const double* I;            /* [B] */
    const double* J;            /* [B] */
    const double* e0;           /* [3B] */
    const double* mass;         /* [N] */
    const uint8_t* locked;      /* [6N] */
    int64_t n_connected;
    const uint64_t* connected;  /* [n_connected] */
} mcg_topology;

/* Specimen scalars used by the load schedule and diagnostics
 * (Simulator::width_/height_/depth_/area_/mass_/top0_, MC/include/sim.hpp:46). */
typedef struct mcg_geometry {
    double width, height, depth, area, mass, top0;
} mcg_geometry;

/* ObjectiveDiag, MC/include/sim.hpp:31. */
typedef struct mcg_diag {
    double elastic, plastic, contact, reaction, max_pen;
    int32_t contacts, pad_;
} mcg_diag;

/* OptStats, MC/include/sim.hpp:33. */
typedef struct mcg_optstats {
    int32_t iterations, backtracks;
    double rms, max, energy;
    int32_t converged, pad_;
} mcg_optstats;

/* FrameDiagnostics, MC/include/sim.hpp:8-14 (one per accepted increment of run()). */
typedef struct mcg_frame {
    double time, platen_y, displacement, engineering_strain, engineering_stress, reaction_force;
    double loading_work, recovered_work, dissipated_work, specific_energy_absorption;
    double elastic_energy, plastic_dissipation, contact_energy, residual_rms, residual_max;
    double max_penetration, mean_plastic_strain, max_plastic_strain, mean_plastic_rotation;
    double max_plastic_rotation, permanent_set;
    int32_t active_contacts, plastic_beams, plastic_hinges, iterations, converged, loading;
    int32_t refinement, pad_;
} mcg_frame;

typedef struct mcg_ctx mcg_ctx;

/* ---- context ------------------------------------------------------------------- */

/* Creates a context on CUDA device `device` with its own stream.  Replaces the
 * construction of the solver state in Simulator::Simulator (MC/src/sim.cpp:49); the
 * configuration is copied.  translation_scale is used as given (the reference sets it
 * to cell_size in its constructor; mcg_config_defaults does not). */
int mcg_create(const mcg_config* cfg, int device, mcg_ctx** out);
void mcg_destroy(mcg_ctx* ctx);
const char* mcg_last_error(const mcg_ctx* ctx);
const char* mcg_status_string(int status);
int mcg_abi_version(void);

/* Uploads the model (MC/src/sim.cpp:51-134 produce it in the reference).  Validates
 * indices, lengths and the connected keys; builds the node incidence lists used by the
 * deterministic gradient gather.  Resets the base state to the rest state
 * base_x = x0, base_r = R0 when x0/R0 are given (NULL leaves the state undefined until
 * mcg_set_state), and plastic state to zero. */
int mcg_upload_topology(mcg_ctx* ctx, const mcg_topology* topo, const mcg_geometry* geom,
                        const double* x0, const double* r0);

/* Base configuration (baseX_/baseR_, MC/include/sim.hpp:46) and plastic state
 * (Beam::plastic).  Any pointer may be NULL to leave that part unchanged. */
int mcg_set_state(mcg_ctx* ctx, const double* base_x, const double* base_r,
                  const double* plastic);
int mcg_get_state(mcg_ctx* ctx, double* base_x, double* base_r, double* plastic);

/* ---- the energy/gradient evaluation --------------------------------------------- */

/* Simulator::objective(z, top, trials), MC/src/sim.cpp:138-172.
 *   z [6N] in; energy, grad [6N], diag out (grad/diag may be NULL).
 *   With trials != 0 the per-beam trial plastic state is kept on the device for
 *   mcg_commit and, when the pointers are non-NULL, copied out:
 *     trial_next [7B]  TrialBeam::next (layout as `plastic`)
 *     trial_aux  [7B]  strain, stress, moment.x, moment.y, moment.z, elastic, dissipation
 *     trial_flags[3B]  axialPlastic, bendPlastic, torsionPlastic
 *   Non-finite energy gives energy = +inf and grad = 0, as the reference does. */
int mcg_objective(mcg_ctx* ctx, const double* z, double top, int trials, double* energy,
                  double* grad, mcg_diag* diag, double* trial_next, double* trial_aux,
                  uint8_t* trial_flags);

/* The same evaluation as mcg_objective (without trial states) for callers that must not
 * allocate device memory when they evaluate: real-time loops with a fixed device-memory
 * budget, hosts whose device memory belongs to another allocator, schedulers that cannot
 * afford cudaFree's wait for the whole device.  mcg_objective may re-allocate its
 * self-contact buffers to fit a state; this entry point uses a fixed 4 MiB __device__ array
 * instead and calls no allocating routine.  Limits: at most 4096 nodes and 8192 nodes +
 * beams, and per evaluation 4096 grid bins (the grid box of the deformed specimen at the
 * reference's grid cell: about 9 cells per axis of a cube) of at most 128 entries each,
 * 32768 candidate pairs and 8192 contacts; beyond them it returns MCG_ERR_CAPACITY, naming
 * what overflowed.  The first call on a context sets up: it looks up the array's device
 * address on the context's device (cudaGetSymbolAddress) and keeps it in the context.  All
 * calls on a device share the array, which keeps the last call's contents: calls that
 * overlap on the GPU race.  After such a call mcg_contact_pairs and mcg_contact_stats
 * return MCG_ERR_STATE until the next allocating evaluation (its contacts are not kept).
 * A call made while another stream captures a CUDA graph (in relaxed capture mode, or in
 * thread-local mode from a thread other than the capturing one) runs at once on the
 * context's own stream and returns its results: none of its work enters that graph.
 * No counterpart in the reference. */
int mcg_objective_noalloc(mcg_ctx* ctx, const double* z, double top, double* energy, double* grad,
                          mcg_diag* diag);

/* Device-resident form used for throughput measurement: mcg_upload_z copies z once;
 * mcg_objective_resident evaluates at that z, leaving energy/grad on the device;
 * mcg_read_result copies them out.  The same kernels as mcg_objective. */
int mcg_upload_z(mcg_ctx* ctx, const double* z);
int mcg_objective_resident(mcg_ctx* ctx, double top, int trials);
int mcg_read_result(mcg_ctx* ctx, double* energy, double* grad, mcg_diag* diag);

/* Contact pair set of the most recent evaluation, sorted ascending, as pair keys over
 * shape indices (nodes 0..N-1 are joint spheres, N+b is beam b's capsule;
 * MC/src/sim.cpp:148-150).  Platen contacts are not pairs and are not listed.
 * With capacity too small: MCG_ERR_CAPACITY and *count = the needed size. */
int mcg_contact_pairs(mcg_ctx* ctx, uint64_t* keys, int64_t capacity, int64_t* count);

/* ---- the solver ---------------------------------------------------------------- */

/* Simulator::minimize(top, z, final), MC/src/sim.cpp:174-211: L-BFGS with Armijo
 * backtracking, steepest-descent retry and best-state fallback; vectors stay on the
 * device.  z [6N] in/out.  The final evaluation (with trials) is kept for mcg_commit.
 * final_diag / final_energy may be NULL. */
int mcg_minimize(mcg_ctx* ctx, double top, double* z, mcg_optstats* stats,
                 double* final_energy, mcg_diag* final_diag);

/* Simulator::commit(z, final), MC/src/sim.cpp:212: re-bases base_x/base_r at the
 * minimizer's z and writes the plastic state from its final trial evaluation. */
int mcg_commit(mcg_ctx* ctx);

/* Simulator::run(), MC/src/sim.cpp:374-467: tare, load_steps loading and unload_steps
 * unloading increments with adaptive bisection, trapezoidal work and per-increment
 * diagnostics.  frames [capacity] out; *count = accepted increments.  Returns
 * MCG_ERR_EQUILIBRIUM where the reference throws; the frames accepted so far are
 * returned.  With `verbose` one line per increment goes to stdout in the reference's
 * format (MC/src/sim.cpp:441-451). */
int mcg_run(mcg_ctx* ctx, mcg_frame* frames, int32_t capacity, int32_t* count, int verbose);

/* The reference CLI's run outputs from run() frames (host only, no context needed):
 * mcg_write_metrics_csv writes the per-increment metrics CSV of MC/src/main.cpp:112-128
 * (writeMetrics: 28 columns, 14 significant digits); mcg_write_summary_json the run summary
 * of MC/src/main.cpp:130-155 (writeSummary: peak force and stress, works, SEA, permanent
 * set, maximum penetration, unconverged increments; 12 significant digits).  `material` is
 * the material's name (MaterialConfig::name, MC/include/sim.hpp:16; NULL: empty) and mass_kg
 * the specimen's mass (mcg_geometry.mass).  MCG_ERR_INVALID when the file cannot be written. */
int mcg_write_metrics_csv(const mcg_frame* frames, int32_t count, const char* path);
int mcg_write_summary_json(const mcg_frame* frames, int32_t count, const mcg_config* cfg, double mass_kg,
                           const char* material, const char* path);

/* The CUDA stream the context launches on (a cudaStream_t), for callers that time
 * or order work around it. */
void* mcg_stream(mcg_ctx* ctx);

/* Number of kernel launches the library has issued in this process. */
int64_t mcg_launch_count(const mcg_ctx* ctx);

/* Capacities of the self-contact buffers (no reference counterpart): entries one grid bin
 * holds (rounded up to a power of two, at least 8), narrow-phase candidates, contacts and
 * grid bins.  They grow by themselves when an evaluation needs more (the evaluation is then
 * repeated); setting them ahead avoids that repeat for a known workload.  Candidates,
 * contacts and bins below the minimum (4096) are raised to it. */
int mcg_set_contact_capacity(mcg_ctx* ctx, int64_t entries, int64_t candidates, int64_t contacts,
                             int64_t bins);

/* ---- batched contexts (no reference counterpart) ------------------------------------
 * One context can hold `count` lattices of uneven size (the reference solves one).  They
 * share the configuration except the yield stress, and every evaluation, minimizer step and
 * load/unload increment of all of them runs in the same kernel launches; each lattice's
 * arithmetic is independent of the others, so a lattice solved in a batch gives exactly the
 * results it gives in a context of its own.  The single-lattice functions (mcg_objective,
 * mcg_minimize, mcg_commit, mcg_run, ...) refuse a context with more than one lattice. */

/* Uploads `count` lattices: topos[k], geoms[k], rest state x0[k] / r0[k] (NULL arrays or
 * entries: undefined state / identity orientations) and yield[k] (NULL: the configuration's
 * yield stress).  Replaces any model the context held. */
int mcg_upload_batch(mcg_ctx* ctx, int32_t count, const mcg_topology* topos, const mcg_geometry* geoms,
                     const double* const* x0, const double* const* r0, const double* yield);

/* Number of lattices in the context (0 before an upload). */
int32_t mcg_instance_count(const mcg_ctx* ctx);

/* One evaluation of every lattice: z holds the lattices' 6-DOF vectors one after another
 * (the order of the upload), tops[k] the platen heights; energies[k], diags[k] and the
 * gradient in the layout of z are written (each may be NULL). */
int mcg_batch_objective(mcg_ctx* ctx, const double* z, const double* tops, double* energies, double* grad,
                        mcg_diag* diags);

/* Simulator::run (MC/src/sim.cpp:374-467) for every lattice at once: lattice k's frames go
 * to frames[k * capacity ...], counts[k] frames, status[k] = MCG_OK or
 * MCG_ERR_EQUILIBRIUM (the frames before the failure are kept).  MCG_ERR_CAPACITY when some
 * lattice produced more than `capacity` frames (counts[] holds the needed sizes). */
int mcg_batch_run(mcg_ctx* ctx, mcg_frame* frames, int32_t capacity, int32_t* counts, int32_t* status);

/* Reuse of the self-contact candidate list (no reference counterpart; results are
 * unchanged).  The list of shape pairs whose boxes may overlap is built with boxes grown
 * by `skin` metres and rebuilt only when some node has moved more than `skin` along an
 * axis since the build (checked on the GPU at every evaluation), so consecutive solver
 * evaluations skip the grid and pair enumeration.  Every pair the reference would test is
 * still tested exactly, and contact sums do not depend on the list, so energies,
 * gradients and pair sets are bitwise those of a rebuild.  0 rebuilds at every evaluation;
 * the default after mcg_upload_topology is cell_size / 32. */
int mcg_set_contact_skin(mcg_ctx* ctx, double skin);

/* Cell size of the self-contact grid in metres (no reference counterpart; 0: the
 * reference's max(2.8 joint radius, 0.72 cell_size)).  Pair sets and results do not depend
 * on it: a pair is examined once whatever the grid, and the narrow phase decides. */
int mcg_set_contact_cell(mcg_ctx* ctx, double cell);

/* Both broad-phase shapes at once, as mcg_autotune reports them (no reference counterpart):
 * the grid cell in metres (0: the reference's) and the blocks of the pair enumeration (0: a
 * default from the lattice size), e.g. to re-apply a tuning without timing again. */
int mcg_set_contact_shapes(mcg_ctx* ctx, double cell, int32_t pair_blocks);

/* Shapes of the evaluation's kernels picked by measurement (no reference counterpart).
 * First the self-contact broad phase: grid cells 0.9, 1, 1.1, 1.25 and 1.4 times the
 * reference's max(2.8 joint radius, 0.72 cell_size), and pair-enumeration grids of 152 ..
 * 1216 blocks (at most one warp per 32 shapes) besides the default; then the occupancy of the
 * beam kernel (FP64: 1, 2 or 3 CTAs of 256 threads per SM; mixed: 3, 4, 5 or 6, and -3 or
 * -4 for the mixed kernel whose beam records arrive in shared memory by bulk copies, two
 * blocks ahead, in persistent CTAs at 3 or 4 per SM) and of the gradient gather (1, 2 or
 * 4), one after the other.  Each candidate evaluates every lattice
 * `reps` times at z (host, 6 N values in the layout of mcg_batch_objective; NULL: z = 0) and
 * platen heights `tops` (NULL: each lattice's top0), with the candidate list rebuilt at
 * every evaluation; the fastest by CUDA-event time is kept for the context (broad phase:
 * among candidates within 1 % of it, the one with the most pair blocks, then the smallest
 * cell; kernel occupancy: timed on the kernel itself, a variant must be 1 % faster than the
 * one before to replace it).
 * All candidates must agree bit for bit on energies and gradients (pair sets and sums do
 * not depend on the grid, nor arithmetic on register allocation); MCG_ERR_MISMATCH if one
 * does not. */
typedef struct mcg_tuning {
    double cell;             /* chosen grid cell (m) */
    int32_t pair_blocks;     /* chosen blocks of the pair enumeration (8 warps each) */
    int32_t tried;           /* candidates timed */
    double ms_chosen;        /* ms per evaluation with the chosen shapes */
    double ms_default;       /* ms per evaluation with the default shapes */
    int32_t beam_blocks;     /* chosen CTAs per SM of the beam kernel */
    int32_t gather_blocks;   /* chosen CTAs per SM of the gather */
} mcg_tuning;
int mcg_autotune(mcg_ctx* ctx, const double* z, const double* tops, int32_t reps, mcg_tuning* out);
/* Re-applies kernel occupancy shapes as mcg_autotune reports them (0: the default). */
int mcg_set_kernel_shapes(mcg_ctx* ctx, int32_t beam_blocks, int32_t gather_blocks);

/* Where the solver's rounds are stepped (no reference counterpart).  With device != 0
 * (the default) mcg_minimize, mcg_run and mcg_batch_run run their rounds as one CUDA-graph
 * loop on the device: each round's directions, evaluation, decisions and accepted step are
 * graph nodes, the decisions (the reference's, sim.cpp:174-211) are taken by device kernels
 * from the same FP64 numbers, and the host synchronises only when an instance has finished
 * its minimization.  With device == 0 the host takes the decisions after every round.  Both
 * give the same results bit for bit.  While phase timing is on (mcg_set_timing) the host
 * steps the rounds.  mcg_solver_loop reports whether the device loop is in use; when it
 * could not be built it is switched off, and mcg_last_error then says why. */
int mcg_set_solver_loop(mcg_ctx* ctx, int device);
int mcg_solver_loop(mcg_ctx* ctx, int32_t* device);
/* Time of the device-resident loop's rounds since the upload or the last
 * mcg_set_solver_loop (no reference counterpart): ms4 = {directions, evaluations (with the
 * vectors they read), decisions and accept steps} as device time between the rounds' stage
 * kernels, and ms4[3] the host's wall time from each loop launch to its synchronisation;
 * *rounds the rounds run. */
int mcg_solver_times(mcg_ctx* ctx, double* ms4, int64_t* rounds);

/* Candidate-list builds of the self-contact broad phase since the lattice was uploaded
 * (no reference counterpart): every evaluation checks whether a node moved farther than the
 * skin from its position at the last build and builds again if so (mcg_set_contact_skin). */
int mcg_contact_builds(mcg_ctx* ctx, int64_t* builds);

/* Sizes of the last self-contact candidate-list build and evaluation (no reference
 * counterpart): out5 = {cell entries, occupied bins, box-overlap candidates, candidates kept
 * by the distance filter, contacts}. */
int mcg_contact_stats(mcg_ctx* ctx, int64_t* out5);

/* Per-phase timing of evaluations with CUDA events on the context stream (no reference
 * counterpart).  While on, every evaluation synchronizes at its end and adds its phase
 * durations: [0] node state, [1] beam kernel, [2] contact grid (skin check, cells, bins),
 * [3] pair enumeration, [4] narrow phase and contact lists, [5] gradient gather,
 * [6] totals.  mcg_set_timing resets the sums. */
int mcg_set_timing(mcg_ctx* ctx, int on);
int mcg_phase_times(mcg_ctx* ctx, double* ms, int32_t n, int64_t* evaluations);

/* ---- synthetic lattices (no reference counterpart; the reference's own builder is
 *      MC/src/sim.cpp:51-135) --------------------------------------------------- */

enum mcg_lattice_kind {
    MCG_LATTICE_CUBIC = 0,     /* cell-edge struts */
    MCG_LATTICE_CUBIC_BCC = 1, /* cell edges + 8 centre-to-corner half-diagonals per cell */
    MCG_LATTICE_REFERENCE_BCC = 2, /* the reference's own specimen, Simulator::build
                                      (MC/src/sim.cpp:51-132) bit for bit: graded BCC with
                                      face grids, seeded imperfections, elements_per_strut
                                      (2..5) elements per strut.  Built from cfg (cells,
                                      cell_size, radii, joint/trigger scales, imperfections,
                                      elements_per_strut, seed); the spec's other fields are
                                      ignored.  As in the reference, set translation_scale to
                                      cell_size (MC/src/sim.cpp:49). */
};

enum mcg_radius_mode {
    MCG_RADIUS_GRADED_Y = 0,   /* linear in height from r0 (bottom) to r1 (top) */
    MCG_RADIUS_UNIFORM = 1,    /* uniform random in [r0, r1] per strut */
};

typedef struct mcg_lattice_spec {
    int32_t kind, radius_mode;
    int32_t cells_x, cells_y, cells_z, pad_;
    double cell_size, r0, r1;
    double jitter;            /* node jitter amplitude as a fraction of cell_size */
    uint64_t seed;
} mcg_lattice_spec;

/* Arrays of a generated lattice; the memory belongs to the lattice object. */
typedef struct mcg_lattice_view {
    int32_t n_nodes, n_beams;
    int64_t n_connected;
    const double* x0;       /* [3N] rest positions */
    const double* r0;       /* [4N] rest orientations (identity) */
    const int32_t* layer;   /* [N] */
    const double* mass;     /* [N] */
    const uint8_t* locked;  /* [6N] */
    const int32_t* beam_a;
    const int32_t* beam_b;
    const double* L0;
    const double* radius;
    const double* area;
    const double* I;
    const double* J;
    const double* e0;       /* [3B] */
    const uint64_t* connected;
    mcg_geometry geometry;
} mcg_lattice_view;

typedef struct mcg_lattice mcg_lattice;

/* Builds a lattice; mass and locks follow the reference rules
 * (Simulator::distributeMass, MC/src/sim.cpp:134) with cfg's density, joint_scale and
 * max_radius.  For MCG_LATTICE_REFERENCE_BCC the whole lattice comes from cfg. */
int mcg_lattice_generate(const mcg_lattice_spec* spec, const mcg_config* cfg,
                         mcg_lattice** out);
int mcg_lattice_view_of(const mcg_lattice* lat, mcg_lattice_view* view);
void mcg_lattice_free(mcg_lattice* lat);
/* Fills a topology description that points into the lattice's arrays. */
int mcg_lattice_topology(const mcg_lattice* lat, mcg_topology* topo);

/* Seeded deformed state: z translations ~ N(0, sigma_t) (units of cell), rotation
 * vectors with uniform axis and angle ~ N(0, sigma_r); plastic epsp ~ U[0, epsp_max],
 * alpha = epsp, the rest zero.  Locked DOFs are zero.  Either output may be NULL. */
int mcg_random_state(int32_t n_nodes, int32_t n_beams, const uint8_t* locked,
                     double sigma_t, double sigma_r, double epsp_max, uint64_t seed,
                     double* z, double* plastic);

#ifdef __cplusplus
}
#endif

#endif /* MCG_H */
