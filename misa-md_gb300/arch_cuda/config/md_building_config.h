// What MISA-MD's CMake writes from src/md_building_config.h.in for a default build (reached from the
// reference's "../md_building_config.h" includes through the gen/ include directory): no development
// mode, and the lattice cutoff the neighbour offsets widen their search by (line 24 of the template).
#ifndef MISA_MD_PRE_CONFIG_H
#define MISA_MD_PRE_CONFIG_H
#define RAND_MT
#define LAT_CUTOFF 0.5
namespace config {
const double nei_lat_cutoff = LAT_CUTOFF;
}
#endif
