/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.  Common C API of the two CPU oracles:
 *
 *   oracle/_build/libmco.so   the CPU restatement of the reference path (mco_oracle.cpp),
 *                             compiled on every machine, including the GPU machine;
 *   oracle/_ref/libmcref.so   the reference's own MC/src/sim.cpp compiled unmodified
 *                             with a harness (ref_harness.cpp); only where the reference
 *                             sources exist, i.e. not on the GPU machine.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load these libraries, and
 * only as the checker or as the timed CPU baseline.  The product library (libmcg.so)
 * never links or calls them.
 *
 * Both export the same symbols, so a test can run the same case through either and
 * compare.  Types come from include/mcg.h.
 */
#ifndef MCG_ORACLE_H
#define MCG_ORACLE_H

#include "../include/mcg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model orc_model;

/* 1 for the reference harness, 0 for the restatement. */
int orc_is_reference(void);

/* A model built by the reference's own lattice builder (MC/src/sim.cpp:49-135). */
orc_model* orc_create_builder(const mcg_config* cfg);

/* A model whose topology is injected (any generator); rest state x0/r0, layer per node. */
orc_model* orc_create_injected(const mcg_config* cfg, const mcg_topology* topo,
                               const mcg_geometry* geom, const double* x0, const double* r0,
                               const int32_t* layer);
void orc_free(orc_model* m);

void orc_counts(const orc_model* m, int32_t* n_nodes, int32_t* n_beams, int64_t* n_connected);
/* Copies the model out; every pointer may be NULL.  `connected` comes out sorted. */
void orc_export(const orc_model* m, double* x0, double* r0, int32_t* layer, double* mass,
                uint8_t* locked, int32_t* beam_a, int32_t* beam_b, double* L0, double* radius,
                double* area, double* I, double* J, double* e0, uint64_t* connected,
                mcg_geometry* geom, double* translation_scale);

void orc_set_state(orc_model* m, const double* base_x, const double* base_r,
                   const double* plastic);
void orc_get_state(const orc_model* m, double* base_x, double* base_r, double* plastic);

/* Simulator::objective (MC/src/sim.cpp:138-172).  Returns the energy. */
double orc_objective(const orc_model* m, const double* z, double top, int trials,
                     double* grad, mcg_diag* diag, double* trial_next, double* trial_aux,
                     uint8_t* trial_flags);

/* Sorted set of shape pairs in contact at state z (MC/src/sim.cpp:148-165); returns the
 * count, writing at most `capacity` keys. */
int64_t orc_contact_pairs(const orc_model* m, const double* z, uint64_t* keys,
                          int64_t capacity);

/* Simulator::minimize (MC/src/sim.cpp:174-211); keeps the final objective for commit. */
int orc_minimize(orc_model* m, double top, double* z, mcg_optstats* stats,
                 double* final_energy, mcg_diag* final_diag);
/* Simulator::commit (MC/src/sim.cpp:212) with the last minimize's z and final. */
int orc_commit(orc_model* m);
/* Simulator::run (MC/src/sim.cpp:374-467).  Returns 0, or MCG_ERR_EQUILIBRIUM. */
int orc_run(orc_model* m, mcg_frame* frames, int32_t capacity, int32_t* count, int verbose);

double orc_rigid_rotation_error(const orc_model* m);   /* MC/src/sim.cpp:511-536 */
double orc_gradient_check_error(const orc_model* m);   /* MC/src/sim.cpp:538-577 */
double orc_beam_potential(const orc_model* m, const double* x, const double* r); /* :468 */
double orc_top_y(const orc_model* m, double s, int loading);                        /* :213 */

/* Rounding-order variant of the restatement's gradient accumulation (0 = the reference's
 * order; see mco_oracle.cpp).  The reference harness accepts only 0 and returns -1. */
int orc_set_variant(orc_model* m, int variant);

/* ---- restatement only (libmco.so) ---------------------------------------------------- */

/* The drop-in seam.  With a hook set, the restatement's objective (MC/src/sim.cpp:138,
 * called by minimize at :176,179,210 and by gradientCheck at :552,564-565) forwards every
 * evaluation to `objective` with ctx as its first argument -- the signature is
 * mcg_objective's, so libmcg's entry point can be passed as it is -- and commit()/set_state
 * hand the base and plastic state to `state` (mcg_set_state's signature).  minimize, run and
 * the checks are unchanged.  NULL objective removes the hook. */
typedef int (*orc_objective_fn)(void* ctx, const double* z, double top, int trials, double* energy,
                                double* grad, mcg_diag* diag, double* trial_next, double* trial_aux,
                                uint8_t* trial_flags);
typedef int (*orc_state_fn)(void* ctx, const double* base_x, const double* base_r, const double* plastic);
void orc_set_objective_hook(orc_model* m, orc_objective_fn objective, orc_state_fn state, void* ctx);
/* First non-zero status a hook returned since it was set (0: none); calls = evaluations. */
int orc_hook_status(const orc_model* m, int64_t* calls);

/* With on != 0 every evaluation keeps its sorted self-contact pair set (the same keys as
 * orc_contact_pairs) for orc_last_pairs, so one evaluation gives both. */
void orc_record_pairs(orc_model* m, int on);
int64_t orc_last_pairs(const orc_model* m, uint64_t* keys, int64_t capacity);

/* A model of the synthetic cubic / cubic+BCC specimen that mcg_lattice_generate builds
 * for (spec, cfg), built here without the product library (oracle/specimens.cpp). */
orc_model* orc_create_specimen(const mcg_config* cfg, const mcg_lattice_spec* spec);
/* The seeded deformed state of mcg_random_state. */
void orc_random_state(int32_t n_nodes, int32_t n_beams, const uint8_t* locked, double sigma_t,
                      double sigma_r, double epsp_max, uint64_t seed, double* z, double* plastic);

#ifdef __cplusplus
}
#endif

#endif
