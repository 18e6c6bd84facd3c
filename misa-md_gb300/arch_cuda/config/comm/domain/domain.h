// Stand-in for libcomm v0.3.3's comm::Domain (not shipped with MISA-MD): MISA-MD's headers only name it
// (src/atom/atom_list.h:187).
#ifndef MISA_GB300_STANDIN_COMM_DOMAIN_H
#define MISA_GB300_STANDIN_COMM_DOMAIN_H
namespace comm {
class Domain {};
}  // namespace comm
#endif
