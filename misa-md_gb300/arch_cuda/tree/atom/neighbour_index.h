// MISA-MD's neighbour offset tables (src/atom/neighbour_index.h:16-77), declared here for builds
// without the MISA-MD tree: the class template, its four protected tables and the friend declaration
// through which the plugin's cuda_nei_offset_init reads them. The reference fills the tables in make();
// here they are given to the constructor, which is all a host without the tree can do.
#ifndef MISA_MD_NEIGHBOUR_INDEX_H
#define MISA_MD_NEIGHBOUR_INDEX_H

#include <utility>
#include <vector>

#include "arch/arch_macros.h"
#include "atom/atom_element.h"

template <class T>
class NeighbourIndex;
class AtomElement;
void ARCH_PREFIX(ARCH_NAME, nei_offset_init)(const NeighbourIndex<AtomElement> *);

template <class T>
class NeighbourIndex {
    friend void ARCH_PREFIX(ARCH_NAME, nei_offset_init)(const NeighbourIndex<T> *);

public:
    NeighbourIndex(std::vector<NeiOffset> full_even, std::vector<NeiOffset> full_odd, std::vector<NeiOffset> half_even,
                   std::vector<NeiOffset> half_odd)
        : nei_even_offsets(std::move(full_even)), nei_odd_offsets(std::move(full_odd)),
          nei_half_even_offsets(std::move(half_even)), nei_half_odd_offsets(std::move(half_odd)) {}

protected:
    std::vector<NeiOffset> nei_even_offsets;
    std::vector<NeiOffset> nei_odd_offsets;
    std::vector<NeiOffset> nei_half_even_offsets;
    std::vector<NeiOffset> nei_half_odd_offsets;
};

#endif
