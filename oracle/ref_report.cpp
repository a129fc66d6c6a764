// ref_report.cpp -- TEST INFRASTRUCTURE ONLY: the reference CLI's own output writers
// (writeMetrics and writeSummary, MC/src/main.cpp:112-155) behind a C entry point, so that
// tests/golden/make_golden.py can produce the reference's metrics CSV and summary JSON of a
// run.  Built into oracle/_ref/libmcref.so with the unmodified MC/src/main.cpp included here
// (its main() renamed so that it does not collide) and MC/src/render.cpp compiled beside it
// (main.cpp's renderer calls need its definitions); only where the reference tree exists.
#include "include/core.hpp"
#define main mcref_cli_main
#include "src/main.cpp"
#undef main

#include "oracle.h"

namespace {

meta::FrameDiagnostics fromFrame(const mcg_frame& f) {
    meta::FrameDiagnostics d;
    d.time = f.time; d.platenY = f.platen_y; d.displacement = f.displacement;
    d.engineeringStrain = f.engineering_strain; d.engineeringStress = f.engineering_stress;
    d.reactionForce = f.reaction_force; d.loadingWork = f.loading_work; d.recoveredWork = f.recovered_work;
    d.dissipatedWork = f.dissipated_work; d.specificEnergyAbsorption = f.specific_energy_absorption;
    d.elasticEnergy = f.elastic_energy; d.plasticDissipation = f.plastic_dissipation;
    d.contactEnergy = f.contact_energy; d.residualRms = f.residual_rms; d.residualMax = f.residual_max;
    d.maxPenetration = f.max_penetration; d.meanPlasticStrain = f.mean_plastic_strain;
    d.maxPlasticStrain = f.max_plastic_strain; d.meanPlasticRotation = f.mean_plastic_rotation;
    d.maxPlasticRotation = f.max_plastic_rotation; d.permanentSet = f.permanent_set;
    d.activeContacts = f.active_contacts; d.plasticBeams = f.plastic_beams; d.plasticHinges = f.plastic_hinges;
    d.iterations = f.iterations; d.converged = f.converged != 0; d.loading = f.loading != 0;
    return d;
}

meta::SimulationResult resultOf(const mcg_frame* frames, int32_t count) {
    meta::SimulationResult r;
    for (int32_t k = 0; k < count; k++) r.diagnostics.push_back(fromFrame(frames[k]));
    return r;
}

}  // namespace

extern "C" int orc_ref_write_outputs(const mcg_frame* frames, int32_t count, const mcg_config* cfg, double mass_kg,
                                     const char* metrics_path, const char* summary_path) {
    try {
        const meta::SimulationResult r = resultOf(frames, count);
        meta::SimulationConfig c;  // the material name and cell counts the summary prints
        c.cellsX = cfg->cells_x; c.cellsY = cfg->cells_y; c.cellsZ = cfg->cells_z;
        meta::writeMetrics(metrics_path, r);
        meta::writeSummary(summary_path, r, c, mass_kg);
    } catch (...) {
        return MCG_ERR_INVALID;
    }
    return MCG_OK;
}
