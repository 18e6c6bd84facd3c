// The record of MISA-MD's lattice-indexed atom store (src/atom/atom_element.h:18-41), declared here for
// builds without the MISA-MD tree (the GPU machine): same class name, members, order and types, so the
// hooks' mangled names and the record layout are those of the reference. Builds inside the tree use
// the reference's own header instead, and the plugin's layout checks run against that.
#ifndef MISA_MD_ATOM_ELEMENT_H
#define MISA_MD_ATOM_ELEMENT_H

namespace atom_type {
enum atom_type { INVALID = -1, Fe = 0, Cu = 1, Ni = 2 };
}

typedef long NeiOffset;

class AtomElement {
public:
    unsigned long id;
    atom_type::atom_type type;
    double x[3];
    double v[3];
    double f[3];
    double rho;
    double df;
};

#endif
