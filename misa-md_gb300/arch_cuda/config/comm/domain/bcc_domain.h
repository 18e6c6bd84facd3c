// Stand-in for libcomm v0.3.3's comm::BccDomain (git.hpcer.dev/HPCer/CrystalMD/libcomm), which MISA-MD
// fetches at build time and does not ship. It declares only the members the CUDA plugin reads, under
// the names MISA-MD's own code reads them by (e.g. src/world_builder.cpp:98-100, src/atom.cpp:15,
// src/lattice/ws_utils.cpp:92), so the plugin compiles unchanged against the real header.
#ifndef MISA_GB300_STANDIN_COMM_BCC_DOMAIN_H
#define MISA_GB300_STANDIN_COMM_BCC_DOMAIN_H

#include <cstdint>

#include "domain.h"

namespace comm {
class BccDomain : public Domain {
public:
    int64_t phase_space[3];           // unit cells of the whole box per dimension
    int64_t sub_box_lattice_size[3];  // unit cells of this rank's sub-box
    double lattice_const;             // Angstrom
    double cutoff_radius_factor;      // cutoff radius / lattice_const
    int cut_lattice;                  // ceil(cutoff_radius_factor)
};
}  // namespace comm

#endif
