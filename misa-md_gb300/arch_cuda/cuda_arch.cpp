// MISA-MD's accelerator plugin for ARCH_NAME = cuda: the seven hooks that src/arch/arch_imp.h:16-32
// declares (named by token pasting, src/arch/arch_macros.h:10-11), forwarding to libmisa_gb300's C ABI.
// Built as libmisa_arch_cuda.so; a MISA-MD build with its CUDA accelerator switched on links it in
// place of the plugin directory its CMake expects (src/arch/arch_libs.cmake), and the reference's own
// loop then calls these functions unchanged:
//   cuda_env_init / cuda_env_clean      archEnvInit / archEnvFinalize (src/arch/arch_env.hpp:15-25)
//   cuda_domain_init                    simulation::createDomain (src/simulation.cpp:52-54)
//   cuda_nei_offset_init                simulation::createAtoms (src/simulation.cpp:67-69)
//   cuda_pot_init                       simulation::prepareForStart (src/simulation.cpp:133)
//   cuda_eam_rho/df/force_calc          atom::latRho / latDf / latForce (src/atom.cpp:159-160, 293-294, 320-321)
//
// The hooks return void and the reference has no error channel for them (its own errors end the MPI
// job), so a failed call prints the library's message and aborts the process.
//
// Settings the hooks' arguments do not carry are read from the environment once, at cuda_env_init:
//   MISA_GB300_DEVICE     CUDA device ordinal (default 0)
//   MISA_GB300_PRECISION  "fp64" (default) or "mixed"
//   MISA_GB300_SETFL      the setfl file the run's potential was read from. The pot package's eam
//                         class (pot v0.1.0) exposes no accessor for its tables, so cuda_pot_init
//                         parses the same file again and builds the same FP64 splines from it.

// arch_imp.h first: it includes the atom headers and then declares the hooks, with NeighbourIndex
// already complete, exactly as the reference's own translation units see them.
#include "arch/arch_imp.h"

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "misa_gb300.h"
#include "misa_gb300_arch.h"

#ifndef ACCELERATE_ENABLED
#error "the plugin needs ACCELERATE_ENABLED (arch_building_config.h with the CUDA accelerator on)"
#endif

// The host slot array crosses the C ABI as it is: AtomElement and mg_atom_element must agree byte for
// byte. These checks run against whichever atom_element.h the build includes.
static_assert(sizeof(AtomElement) == sizeof(mg_atom_element), "AtomElement is 104 bytes on LP64");
static_assert(std::is_standard_layout<AtomElement>::value, "AtomElement must stay a plain record");
static_assert(offsetof(AtomElement, id) == offsetof(mg_atom_element, id), "id");
static_assert(offsetof(AtomElement, type) == offsetof(mg_atom_element, type), "type");
static_assert(sizeof(AtomElement::type) == sizeof(int32_t), "type is a 4-byte enum");
static_assert(offsetof(AtomElement, x) == offsetof(mg_atom_element, x), "x");
static_assert(offsetof(AtomElement, v) == offsetof(mg_atom_element, v), "v");
static_assert(offsetof(AtomElement, f) == offsetof(mg_atom_element, f), "f");
static_assert(offsetof(AtomElement, rho) == offsetof(mg_atom_element, rho), "rho");
static_assert(offsetof(AtomElement, df) == offsetof(mg_atom_element, df), "df");
static_assert(sizeof(NeiOffset) == sizeof(int64_t), "offset tables hold 64-bit linear offsets");

namespace {

mg_context *g_ctx = nullptr;
int g_device = 0;
int g_precision = MG_PREC_FP64;
const char *g_setfl = nullptr;

[[noreturn]] void fail(const char *hook, mg_status st, const char *why) {
    std::fprintf(stderr, "misa_gb300 %s failed (status %d): %s\n", hook, static_cast<int>(st), why ? why : "");
    std::fflush(stderr);
    std::abort();
}
void check(const char *hook, mg_status st) {
    if (st != MG_OK) fail(hook, st, mg_last_error(g_ctx));
}
mg_context *context(const char *hook) {
    if (!g_ctx) fail(hook, MG_ERR_STATE, "cuda_domain_init has not run");
    return g_ctx;
}

}  // namespace

void cuda_env_init() {
    const char *dev = std::getenv("MISA_GB300_DEVICE");
    g_device = dev ? std::atoi(dev) : 0;
    const char *prec = std::getenv("MISA_GB300_PRECISION");
    if (prec && std::strcmp(prec, "mixed") == 0) g_precision = MG_PREC_MIXED;
    else if (prec && std::strcmp(prec, "fp64") != 0) fail("cuda_env_init", MG_ERR_ARG, "MISA_GB300_PRECISION is neither fp64 nor mixed");
    g_setfl = std::getenv("MISA_GB300_SETFL");
    check("cuda_env_init", mg_env_init(g_device));
}

void cuda_env_clean() {
    if (g_ctx) mg_destroy(g_ctx);
    g_ctx = nullptr;
    check("cuda_env_clean", mg_env_clean());
}

// One GPU owns the whole periodic box: the single-rank decomposition, whose sub-box is the box.
void cuda_domain_init(const comm::BccDomain *domain) {
    if (!domain) fail("cuda_domain_init", MG_ERR_ARG, "null domain");
    int64_t cells[3];
    for (int d = 0; d < 3; d++) {
        cells[d] = static_cast<int64_t>(domain->phase_space[d]);
        if (static_cast<int64_t>(domain->sub_box_lattice_size[d]) != cells[d])
            fail("cuda_domain_init", MG_ERR_ARG, "the plugin runs the whole box on one GPU (one MPI rank)");
    }
    if (g_ctx) mg_destroy(g_ctx);
    g_ctx = nullptr;
    check("cuda_domain_init", mg_create(cells, domain->lattice_const, domain->cutoff_radius_factor, g_precision, 0, &g_ctx));
}

// A friend of NeighbourIndex (src/atom/neighbour_index.h:21-24): the four offset tables of the host,
// which the context checks against its own (same entries, same order).
void cuda_nei_offset_init(const NeighbourIndex<AtomElement> *nei_offset) {
    mg_context *ctx = context("cuda_nei_offset_init");
    if (!nei_offset) fail("cuda_nei_offset_init", MG_ERR_ARG, "null neighbour index");
    const auto &fe = nei_offset->nei_even_offsets, &fo = nei_offset->nei_odd_offsets;
    const auto &he = nei_offset->nei_half_even_offsets, &ho = nei_offset->nei_half_odd_offsets;
    if (fe.size() != fo.size() || he.size() != ho.size())
        fail("cuda_nei_offset_init", MG_ERR_ARG, "even and odd tables differ in length");
    check("cuda_nei_offset_init",
          mg_nei_offset_init(ctx, reinterpret_cast<const int64_t *>(fe.data()), reinterpret_cast<const int64_t *>(fo.data()),
                             static_cast<int32_t>(fe.size()), reinterpret_cast<const int64_t *>(he.data()),
                             reinterpret_cast<const int64_t *>(ho.data()), static_cast<int32_t>(he.size())));
}

void cuda_pot_init(eam *) {
    mg_context *ctx = context("cuda_pot_init");
    if (!g_setfl || !*g_setfl) fail("cuda_pot_init", MG_ERR_POTENTIAL, "MISA_GB300_SETFL names no setfl file");
    check("cuda_pot_init", mg_pot_init_setfl(ctx, g_setfl));
}

void cuda_eam_rho_calc(eam *, AtomElement *atoms, const double cutoff_radius) {
    check("cuda_eam_rho_calc", mg_eam_rho_calc(context("cuda_eam_rho_calc"), reinterpret_cast<mg_atom_element *>(atoms), cutoff_radius));
}

void cuda_eam_df_calc(eam *, AtomElement *atoms, const double cutoff_radius) {
    check("cuda_eam_df_calc", mg_eam_df_calc(context("cuda_eam_df_calc"), reinterpret_cast<mg_atom_element *>(atoms), cutoff_radius));
}

void cuda_eam_force_calc(eam *, AtomElement *atoms, const double cutoff_radius) {
    check("cuda_eam_force_calc", mg_eam_force_calc(context("cuda_eam_force_calc"), reinterpret_cast<mg_atom_element *>(atoms), cutoff_radius));
}
