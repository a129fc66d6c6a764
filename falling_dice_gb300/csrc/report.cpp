// report.cpp -- the run outputs of the reference's CLI from a load/unload run's frames:
// the per-increment metrics CSV (MC/src/main.cpp:112-128) and the run summary JSON
// (MC/src/main.cpp:130-155), in the same columns, keys and number formatting (14 significant
// digits in the CSV, 12 in the summary), so that a GPU run's files can be compared with the
// reference's mechanically.  Host code only.
#include <cstdio>
#include <string>
#include <utility>

#include "../../include/mcg.h"

namespace {

// A file written through stdio, closed on every path.
struct Out {
    FILE* f;
    explicit Out(const char* path) : f(path ? std::fopen(path, "w") : nullptr) {}
    ~Out() {
        if (f) std::fclose(f);
    }
    bool ok() const { return f != nullptr; }
};

const char* kMetricsHeader =
    "frame,time,loading,platen_y_m,displacement_m,engineering_strain,engineering_stress_pa,"
    "reaction_force_n,loading_work_j,recovered_work_j,dissipated_work_j,sea_j_per_kg,"
    "elastic_energy_j,incremental_plastic_dissipation_j,contact_energy_j,residual_rms,residual_max,"
    "max_penetration_m,mean_plastic_strain,max_plastic_strain,mean_plastic_rotation_rad,"
    "max_plastic_rotation_rad,permanent_set,active_contacts,plastic_beams,plastic_hinges,iterations,converged\n";

}  // namespace

extern "C" {

int mcg_write_metrics_csv(const mcg_frame* frames, int32_t count, const char* path) {
    if (count < 0 || (count > 0 && !frames) || !path) return MCG_ERR_INVALID;
    Out o(path);
    if (!o.ok()) return MCG_ERR_INVALID;
    std::fputs(kMetricsHeader, o.f);
    for (int32_t k = 0; k < count; k++) {
        const mcg_frame& d = frames[k];
        const double reals[] = {d.platen_y, d.displacement, d.engineering_strain, d.engineering_stress,
                                d.reaction_force, d.loading_work, d.recovered_work, d.dissipated_work,
                                d.specific_energy_absorption, d.elastic_energy, d.plastic_dissipation,
                                d.contact_energy, d.residual_rms, d.residual_max, d.max_penetration,
                                d.mean_plastic_strain, d.max_plastic_strain, d.mean_plastic_rotation,
                                d.max_plastic_rotation, d.permanent_set};
        std::fprintf(o.f, "%d,%.14g,%d", int(k), d.time, d.loading ? 1 : 0);
        for (double v : reals) std::fprintf(o.f, ",%.14g", v);
        std::fprintf(o.f, ",%d,%d,%d,%d,%d\n", d.active_contacts, d.plastic_beams, d.plastic_hinges, d.iterations,
                     d.converged ? 1 : 0);
    }
    return std::ferror(o.f) ? MCG_ERR_INVALID : MCG_OK;
}

int mcg_write_summary_json(const mcg_frame* frames, int32_t count, const mcg_config* cfg, double mass_kg,
                           const char* material, const char* path) {
    if (count < 0 || (count > 0 && !frames) || !cfg || !path) return MCG_ERR_INVALID;
    // the reference's summarize(): peaks over the frames, works and set of the last frame
    double peak_force = 0, peak_stress = 0, max_pen = 0;
    int unconverged = 0;
    for (int32_t k = 0; k < count; k++) {
        const mcg_frame& d = frames[k];
        if (d.reaction_force > peak_force) peak_force = d.reaction_force;
        if (peak_stress < d.engineering_stress) peak_stress = d.engineering_stress;  // std::max order
        if (max_pen < d.max_penetration) max_pen = d.max_penetration;
        if (!d.converged) ++unconverged;
    }
    mcg_frame last{};
    if (count > 0) last = frames[count - 1];
    Out o(path);
    if (!o.ok()) return MCG_ERR_INVALID;
    std::fprintf(o.f,
                 "{\n"
                 "  \"solver\": \"incremental quasi-static 6-DOF corotational beam/contact energy minimization\",\n"
                 "  \"material\": \"%s\",\n"
                 "  \"cells\": [%d, %d, %d],\n"
                 "  \"frames\": %d,\n",
                 material ? material : "", cfg->cells_x, cfg->cells_y, cfg->cells_z, int(count));
    const std::pair<const char*, double> rows[] = {
        {"mass_kg", mass_kg},
        {"peak_force_n", peak_force},
        {"peak_stress_pa", peak_stress},
        {"loading_work_j", last.loading_work},
        {"recovered_work_j", last.recovered_work},
        {"dissipated_work_j", last.dissipated_work},
        {"specific_energy_absorption_j_per_kg", last.specific_energy_absorption},
        {"permanent_set", last.permanent_set},
        {"max_penetration_m", max_pen}};
    for (const auto& r : rows) std::fprintf(o.f, "  \"%s\": %.12g,\n", r.first, r.second);
    std::fprintf(o.f, "  \"unconverged_steps\": %d\n}\n", unconverged);
    return std::ferror(o.f) ? MCG_ERR_INVALID : MCG_OK;
}

}  // extern "C"
