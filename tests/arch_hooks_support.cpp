// Test support for the plugin's GPU test (compiled by the test with the plugin's include layout):
// builds the host objects MISA-MD would pass to its accelerator hooks, a comm::BccDomain of one rank
// owning the whole box and a NeighbourIndex<AtomElement> holding given offset tables, so a test can
// call the cuda_* hooks of libmisa_arch_cuda.so through ctypes in the order the reference's loop does.
#include <cstdint>
#include <vector>

#include "arch/arch_imp.h"

extern "C" {

void *th_domain_new(const int64_t cells[3], double lattice_const, double cutoff_radius_factor, int cut_lattice) {
    auto *d = new comm::BccDomain();
    for (int k = 0; k < 3; k++) {
        d->phase_space[k] = cells[k];
        d->sub_box_lattice_size[k] = cells[k];
    }
    d->lattice_const = lattice_const;
    d->cutoff_radius_factor = cutoff_radius_factor;
    d->cut_lattice = cut_lattice;
    return d;
}

void th_domain_free(void *d) { delete static_cast<comm::BccDomain *>(d); }

void *th_neighbour_index_new(const int64_t *full_even, const int64_t *full_odd, int32_t n_full,
                             const int64_t *half_even, const int64_t *half_odd, int32_t n_half) {
    auto vec = [](const int64_t *p, int32_t n) { return std::vector<NeiOffset>(p, p + n); };
    return new NeighbourIndex<AtomElement>(vec(full_even, n_full), vec(full_odd, n_full), vec(half_even, n_half),
                                           vec(half_odd, n_half));
}

void th_neighbour_index_free(void *n) { delete static_cast<NeighbourIndex<AtomElement> *>(n); }
}
