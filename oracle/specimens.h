// specimens.h -- TEST INFRASTRUCTURE ONLY: CPU-side restatement of the synthetic specimens
// of the throughput workloads (see specimens.cpp).
#ifndef ORC_SPECIMENS_H
#define ORC_SPECIMENS_H

#include <cstdint>
#include <vector>

#include "../include/mcg.h"

namespace orcspec {

struct Specimen {
    std::vector<double> x0, r0, mass, L0, radius, area, I, J, e0;
    std::vector<int32_t> layer, beam_a, beam_b;
    std::vector<uint8_t> locked;
    std::vector<uint64_t> connected;
    mcg_geometry geometry{};
};

// The specimen mcg_lattice_generate builds for (spec, cfg); false on an invalid spec.
bool build(const mcg_lattice_spec& spec, const mcg_config& cfg, Specimen& out);

// The state mcg_random_state produces.
void random_state(int32_t n_nodes, int32_t n_beams, const uint8_t* locked, double sigma_t, double sigma_r,
                  double epsp_max, uint64_t seed, double* z, double* plastic);

}  // namespace orcspec

#endif
