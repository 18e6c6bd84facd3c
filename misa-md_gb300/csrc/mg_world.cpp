// Creation mode of the reference (WorldBuilder::build, src/world_builder.cpp:64-199) on the host:
// a BCC crystal on the slot grid with random alloy types, uniform random velocities, zero total
// momentum and velocities rescaled to the set temperature (configuration::rescale,
// src/system_configuration.cpp:86-111). Every operation follows the reference's order, with each
// product and sum rounded on its own, so the slot array equals the reference's for the same seed.
//
// Random streams (src/utils/random/random.cpp:14-37): velocities draw from md_rand's engine, which
// the build selects (MD_RAND in config.cmake; "MT" by default). Atom types draw from the C library's
// rand(), which the reference never seeds outside its development mode, so it starts in its default
// state (seed 1). That generator is restated here (GlibcRand) instead of calling the process's
// rand(): the caller's own libc state is left alone.

#include <cmath>
#include <cstring>
#include <random>
#include <string>

#include "mg_internal.h"

namespace mg {
void set_global_error(const char *msg);
}

namespace {

using mg::atom_mass;
using mg::kBoltz;
using mg::kMvv2e;

// glibc's default rand() (random_r with the TYPE_3 additive feedback table of 31 words):
// r[0] = seed; r[i] = 16807 r[i-1] mod (2^31 - 1) for i < 31 (Schrage's method); r[i] = r[i-31] for
// 31 <= i < 34; then r[i] = r[i-31] + r[i-3] (mod 2^32), the first 310 discarded, output r[i] >> 1.
class GlibcRand {
public:
    explicit GlibcRand(uint32_t seed) {
        int32_t r[34];
        r[0] = seed == 0 ? 1 : static_cast<int32_t>(seed);
        for (int i = 1; i < 31; i++) {
            const int64_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
            int64_t w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            r[i] = static_cast<int32_t>(w);
        }
        for (int i = 31; i < 34; i++) r[i] = r[i - 31];
        for (int i = 0; i < 34; i++) ring_[i] = static_cast<uint32_t>(r[i]);
        pos_ = 34;
        for (int i = 0; i < 310; i++) step();
    }
    int32_t operator()() { return static_cast<int32_t>(step() >> 1); }

private:
    uint32_t step() {
        const uint32_t v = ring_[(pos_ - 31) % kLen] + ring_[(pos_ - 3) % kLen];
        ring_[pos_ % kLen] = v;
        pos_++;
        return v;
    }
    static constexpr int kLen = 34;
    uint32_t ring_[kLen];
    uint64_t pos_ = 0;
};

// md_rand::LegacyRand (src/utils/random/legacy_random.hpp): Park-Miller minimal standard, Schrage.
class LegacyRand {
public:
    explicit LegacyRand(uint32_t seed) : s_(static_cast<int32_t>(seed)) {}
    uint32_t operator()() {
        const int32_t k = s_ / 127773;
        s_ = 16807 * (s_ - k * 127773) - 2836 * k;
        if (s_ < 0) s_ += 0x7fffffff;
        return static_cast<uint32_t>(s_);
    }
    static constexpr double max() { return 2147483647.0; }

private:
    int32_t s_;
};

// md_rand::random() for the engines of the non-development build: rand32() * (1.0 / rng.max())
template <class Engine>
struct Uniform {
    Engine e;
    explicit Uniform(uint32_t seed) : e(seed) {}
    double operator()() { return static_cast<double>(e()) * (1.0 / static_cast<double>(Engine::max())); }
};
template <>
struct Uniform<LegacyRand> {
    LegacyRand e;
    explicit Uniform(uint32_t seed) : e(seed) {}
    double operator()() { return static_cast<double>(e()) * (1.0 / LegacyRand::max()); }
};

template <class U>
void build_world(const int64_t ps[3], double a0, double rcf, double t_set, uint32_t seed, const int32_t ratio[3],
                 mg_atom_element *atoms) {
    const int64_t g = static_cast<int64_t>(std::ceil(rcf)) + 1;  // src/simulation.cpp:46
    const int64_t bx = 2 * ps[0], by = ps[1], bz = ps[2];
    const int64_t Sx = 2 * (ps[0] + 2 * g), Sy = ps[1] + 2 * g;
    const int64_t gx = 2 * g, gy = g, gz = g;
    auto slot = [&](int64_t i, int64_t j, int64_t k) { return ((k + gz) * Sy + (j + gy)) * Sx + (i + gx); };
    U uniform(seed);
    GlibcRand crand(1);
    int ratio_total = 0;
    for (int t = 0; t < 3; t++) ratio_total += ratio[t];
    // createPhaseSpace (src/world_builder.cpp:105-131), one rank: lattice region lows are 0
    uint64_t id = 0;
    for (int64_t k = 0; k < bz; k++) {
        for (int64_t j = 0; j < by; j++) {
            for (int64_t i = 0; i < bx; i++) {
                mg_atom_element &a = atoms[slot(i, j, k)];
                a.id = ++id;
                // randomAtomsType (src/world_builder.cpp:183-199)
                const int r = crand() % ratio_total;
                int acc = 0, type = 0;
                for (int t = 0; t < 3; t++) {
                    acc += ratio[t];
                    if (r < acc) { type = t; break; }
                }
                a.type = type;
                const double mass = atom_mass(type);
                a.x[0] = (static_cast<double>(i) * 0.5) * a0;
                a.x[1] = static_cast<double>(j) * a0 + static_cast<double>(i % 2) * (a0 / 2);
                a.x[2] = static_cast<double>(k) * a0 + static_cast<double>(i % 2) * (a0 / 2);
                a.v[0] = (uniform() - 0.5) / mass;
                a.v[1] = (uniform() - 0.5) / mass;
                a.v[2] = (uniform() - 0.5) / mass;
            }
        }
    }
    // vcm and zeroMomentum (src/world_builder.cpp:70-95, 145-181)
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t k = 0; k < bz; k++)
        for (int64_t j = 0; j < by; j++)
            for (int64_t i = 0; i < bx; i++) {
                const mg_atom_element &a = atoms[slot(i, j, k)];
                const double m = atom_mass(a.type);
                p[0] += a.v[0] * m;
                p[1] += a.v[1] * m;
                p[2] += a.v[2] * m;
                p[3] += m;
            }
    const uint64_t n = static_cast<uint64_t>(bx * by * bz);
    if (p[3] > 0.0) {
        p[0] /= n;
        p[1] /= n;
        p[2] /= n;
    }
    for (int64_t k = 0; k < bz; k++)
        for (int64_t j = 0; j < by; j++)
            for (int64_t i = 0; i < bx; i++) {
                mg_atom_element &a = atoms[slot(i, j, k)];
                const double m = atom_mass(a.type);
                a.v[0] -= (p[0] / m);
                a.v[1] -= (p[1] / m);
                a.v[2] -= (p[2] / m);
            }
    if (t_set == 0.0) return;
    // configuration::rescale with configuration::temperature and mvv (src/system_configuration.cpp:51-111)
    double mvv = 0.0;
    for (int64_t k = 0; k < bz; k++)
        for (int64_t j = 0; j < by; j++)
            for (int64_t i = 0; i < bx; i++) {
                const mg_atom_element &a = atoms[slot(i, j, k)];
                mvv += (a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]) * atom_mass(a.type);
            }
    const uint64_t dof = 3 * n - 3;
    const double t_now = mvv * kMvv2e / (static_cast<double>(dof) * kBoltz);
    const double factor = std::sqrt(t_set / t_now);
    for (int64_t k = 0; k < bz; k++)
        for (int64_t j = 0; j < by; j++)
            for (int64_t i = 0; i < bx; i++) {
                mg_atom_element &a = atoms[slot(i, j, k)];
                a.v[0] *= factor;
                a.v[1] *= factor;
                a.v[2] *= factor;
            }
}

}  // namespace

extern "C" mg_status mg_world_build(const int64_t phase_space[3], double lattice_const, double cutoff_radius_factor,
                                    double t_set, uint32_t seed, const int32_t alloy_ratio[3], int32_t rng,
                                    mg_atom_element *atoms, int64_t n_slots) {
    if (!phase_space || !alloy_ratio || !atoms || !(lattice_const > 0) || !(cutoff_radius_factor > 0) || t_set < 0) {
        mg::set_global_error("mg_world_build: bad argument");
        return MG_ERR_ARG;
    }
    const int64_t g = static_cast<int64_t>(std::ceil(cutoff_radius_factor)) + 1;
    for (int d = 0; d < 3; d++) {
        if (phase_space[d] < 1) { mg::set_global_error("mg_world_build: empty box"); return MG_ERR_ARG; }
    }
    const int64_t need = 2 * (phase_space[0] + 2 * g) * (phase_space[1] + 2 * g) * (phase_space[2] + 2 * g);
    if (n_slots != need) { mg::set_global_error("mg_world_build: slot array size differs from the grid"); return MG_ERR_ARG; }
    if (alloy_ratio[0] < 0 || alloy_ratio[1] < 0 || alloy_ratio[2] < 0 || alloy_ratio[0] + alloy_ratio[1] + alloy_ratio[2] <= 0) {
        mg::set_global_error("mg_world_build: alloy ratio must be non-negative with a positive sum");
        return MG_ERR_ARG;
    }
    std::memset(atoms, 0, sizeof(mg_atom_element) * static_cast<size_t>(n_slots));
    for (int64_t s = 0; s < n_slots; s++) atoms[s].type = mg::kInvalid;
    switch (rng) {
        case MG_RNG_MT: build_world<Uniform<std::mt19937>>(phase_space, lattice_const, cutoff_radius_factor, t_set, seed, alloy_ratio, atoms); break;
        case MG_RNG_LCG: build_world<Uniform<std::minstd_rand>>(phase_space, lattice_const, cutoff_radius_factor, t_set, seed, alloy_ratio, atoms); break;
        case MG_RNG_STC: build_world<Uniform<std::ranlux24>>(phase_space, lattice_const, cutoff_radius_factor, t_set, seed, alloy_ratio, atoms); break;
        case MG_RNG_LEGACY: build_world<Uniform<LegacyRand>>(phase_space, lattice_const, cutoff_radius_factor, t_set, seed, alloy_ratio, atoms); break;
        default: mg::set_global_error("mg_world_build: unknown random engine"); return MG_ERR_ARG;
    }
    return MG_OK;
}
