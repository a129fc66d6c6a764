// specimens.cpp -- TEST INFRASTRUCTURE ONLY: the synthetic cubic and cubic+BCC specimens and
// the seeded deformed state of the throughput workloads, restated for the CPU side so that
// the timed CPU baseline builds its inputs without loading the product library.
//
// The workloads are defined by the product's generator (mcg_lattice_generate and
// mcg_random_state, falling_dice_gb300/csrc/lattice.cpp); this file computes the same
// arrays in the same floating-point order (tests/test_oracle.py checks them bit for bit).
// Shared with the reference are the corner numbering (MC/src/sim.cpp:54), the section
// formulas (MC/src/sim.cpp:115), lumped mass and anti-drift locks (MC/src/sim.cpp:134), the
// platen height (MC/src/sim.cpp:131) and the splitmix64 generator (MC/include/core.hpp:46).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#include "specimens.h"

namespace orcspec {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795;

uint64_t splitmix(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

// The stream of core.hpp:46's RNG, plus Box-Muller normals drawn from two of its uniforms.
class Stream {
  public:
    explicit Stream(uint64_t seed) : s_(splitmix(seed)) {}
    double u() {
        s_ = splitmix(s_);
        return (double(uint32_t(s_ >> 32)) + .5) / 4294967296.0;
    }
    double su() { return 2 * u() - 1; }
    double gauss() {
        const double a = u(), b = u();
        return std::sqrt(-2.0 * std::log(a)) * std::cos(2.0 * kPi * b);
    }

  private:
    uint64_t s_;
};

}  // namespace

bool build(const mcg_lattice_spec& sp, const mcg_config& cfg, Specimen& out) {
    const int nx = sp.cells_x, ny = sp.cells_y, nz = sp.cells_z;
    const bool bcc = sp.kind == MCG_LATTICE_CUBIC_BCC;
    if (nx < 1 || ny < 1 || nz < 1 || !(sp.cell_size > 0) || !(sp.r0 > 0) || !(sp.r1 > 0)) return false;
    if (sp.kind != MCG_LATTICE_CUBIC && !bcc) return false;
    const long long nc = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    const long long nb = bcc ? (long long)nx * ny * nz : 0;
    const double h = sp.cell_size, W = nx * h, H = ny * h, D = nz * h;
    const double jr = cfg.joint_scale * cfg.max_radius;
    const double x0 = -.5 * W, y0 = jr, z0 = -.5 * D;
    auto corner_id = [&](int i, int j, int k) { return int((j * (nz + 1) + k) * (nx + 1) + i); };
    auto centre_id = [&](int i, int j, int k) { return int(nc + (j * nz + k) * nx + i); };
    const size_t N = size_t(nc + nb);
    Specimen s;
    s.x0.assign(3 * N, 0.0);
    s.r0.assign(4 * N, 0.0);
    s.layer.assign(N, 0);
    const double amp = sp.jitter * h;
    Stream js(sp.seed);
    // corners in (layer, depth, width) order; planar top and bottom faces
    for (int j = 0; j <= ny; j++)
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                double* p = &s.x0[3 * size_t(corner_id(i, j, k))];
                const double ex = amp * js.su(), ey = amp * js.su(), ez = amp * js.su();
                const bool face = j == 0 || j == ny;
                p[0] = x0 + i * h + ex;
                p[1] = y0 + j * h + (face ? 0.0 : ey);
                p[2] = z0 + k * h + ez;
                s.layer[size_t(corner_id(i, j, k))] = j;
            }
    // cell centres in node order, continuing the same stream
    for (int j = 0; j < ny && bcc; j++)
        for (int k = 0; k < nz; k++)
            for (int i = 0; i < nx; i++) {
                double* p = &s.x0[3 * size_t(centre_id(i, j, k))];
                p[0] = x0 + (i + .5) * h + amp * js.su();
                p[1] = y0 + (j + .5) * h + amp * js.su();
                p[2] = z0 + (k + .5) * h + amp * js.su();
                s.layer[size_t(centre_id(i, j, k))] = j;
            }
    for (size_t n = 0; n < N; n++) s.r0[4 * n] = 1.0;
    // struts: per corner the +x, +y, +z edges, then the eight half-diagonals of each cell
    for (int j = 0; j <= ny; j++)
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                const int a = corner_id(i, j, k);
                if (i < nx) { s.beam_a.push_back(a); s.beam_b.push_back(corner_id(i + 1, j, k)); }
                if (j < ny) { s.beam_a.push_back(a); s.beam_b.push_back(corner_id(i, j + 1, k)); }
                if (k < nz) { s.beam_a.push_back(a); s.beam_b.push_back(corner_id(i, j, k + 1)); }
            }
    for (int j = 0; j < ny && bcc; j++)
        for (int k = 0; k < nz; k++)
            for (int i = 0; i < nx; i++)
                for (int q = 0; q < 8; q++) {
                    s.beam_a.push_back(centre_id(i, j, k));
                    s.beam_b.push_back(corner_id(i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1)));
                }
    const size_t B = s.beam_a.size();
    s.L0.resize(B); s.radius.resize(B); s.area.resize(B); s.I.resize(B); s.J.resize(B);
    s.e0.resize(3 * B);
    Stream rs(splitmix(sp.seed ^ 0x5241444949ULL));
    std::vector<uint64_t> keys(B);
    for (size_t b = 0; b < B; b++) {
        const int a = s.beam_a[b], c = s.beam_b[b];
        const double* pa = &s.x0[3 * size_t(a)];
        const double* pc = &s.x0[3 * size_t(c)];
        const double d[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
        const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        const double inv = 1.0 / len;
        s.L0[b] = len;
        for (int q = 0; q < 3; q++) s.e0[3 * b + size_t(q)] = d[q] * inv;
        double r;
        if (sp.radius_mode == MCG_RADIUS_GRADED_Y) {
            const double mid = .5 * (pa[1] + pc[1]);
            r = sp.r0 + (sp.r1 - sp.r0) * std::clamp((mid - jr) / H, 0.0, 1.0);
        } else {
            r = sp.r0 + (sp.r1 - sp.r0) * rs.u();
        }
        s.radius[b] = r;
        s.area[b] = kPi * r * r;
        s.I[b] = .25 * kPi * std::pow(r, 4);
        s.J[b] = 2 * s.I[b];
        const uint32_t lo = uint32_t(std::min(a, c)), hi = uint32_t(std::max(a, c));
        keys[b] = (uint64_t(lo) << 32) | hi;
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    s.connected = std::move(keys);
    // lumped mass: half of each strut to either end, then one joint mass per node
    s.mass.assign(N, 0.0);
    double total = 0;
    for (size_t b = 0; b < B; b++) {
        const double m = cfg.material.density * s.area[b] * s.L0[b];
        s.mass[size_t(s.beam_a[b])] += .5 * m;
        s.mass[size_t(s.beam_b[b])] += .5 * m;
        total += m;
    }
    const double joint = cfg.material.density * (4.0 / 3.0) * kPi * std::pow(jr, 3) * .28;
    for (size_t n = 0; n < N; n++) {
        s.mass[n] += joint;
        total += joint;
    }
    // anti-drift locks on the two bottom nodes nearest the (-x, -z) and (+x, -z) corners
    s.locked.assign(6 * N, 0);
    int best_a = -1, best_b = -1;
    double qa_min = std::numeric_limits<double>::infinity(), qb_min = qa_min;
    for (size_t n = 0; n < N; n++) {
        if (s.layer[n] != 0) continue;
        const double px = s.x0[3 * n], pz = s.x0[3 * n + 2];
        const double qa = (px + .5 * W) * (px + .5 * W) + (pz + .5 * D) * (pz + .5 * D);
        const double qb = (px - .5 * W) * (px - .5 * W) + (pz + .5 * D) * (pz + .5 * D);
        if (qa < qa_min) { qa_min = qa; best_a = int(n); }
        if (qb < qb_min) { qb_min = qb; best_b = int(n); }
    }
    if (best_a < 0 || best_b < 0) return false;
    s.locked[6 * size_t(best_a)] = 1;
    s.locked[6 * size_t(best_a) + 2] = 1;
    s.locked[6 * size_t(best_b) + 2] = 1;
    s.geometry = mcg_geometry{W, H, D, W * D, total, jr + H + jr};
    out = std::move(s);
    return true;
}

void random_state(int32_t n_nodes, int32_t n_beams, const uint8_t* locked, double sigma_t, double sigma_r,
                  double epsp_max, uint64_t seed, double* z, double* plastic) {
    if (z) {
        Stream g(seed);
        for (int32_t i = 0; i < n_nodes; i++) {
            double* zi = z + 6 * size_t(i);
            for (int d = 0; d < 3; d++) zi[d] = sigma_t * g.gauss();
            double v[3] = {g.gauss(), g.gauss(), g.gauss()};
            double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (!(n > 1e-12)) { v[0] = 0; v[1] = 0; v[2] = 1; n = 1; }
            const double angle = sigma_r * g.gauss();
            for (int d = 0; d < 3; d++) zi[3 + d] = v[d] / n * angle;
            for (int d = 0; d < 6 && locked; d++)
                if (locked[6 * size_t(i) + size_t(d)]) zi[d] = 0;
        }
    }
    if (plastic) {
        Stream g(splitmix(seed ^ 0x504c4153ULL));
        for (int32_t b = 0; b < n_beams; b++) {
            double* q = plastic + 7 * size_t(b);
            const double e = epsp_max * g.u();
            std::fill(q, q + 7, 0.0);
            q[0] = e;
            q[1] = e;
        }
    }
}

}  // namespace orcspec
