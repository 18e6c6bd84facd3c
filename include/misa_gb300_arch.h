/*
 * misa_gb300_arch: MISA-MD's accelerator plugin for ARCH_NAME = cuda (libmisa_arch_cuda.so).
 *
 * The eight C++ hooks that MISA-MD declares in src/arch/arch_imp.h:16-32 (names pasted by
 * src/arch/arch_macros.h:10-11 from ARCH_NAME = cuda), with the same signatures, so a MISA-MD build with
 * its CUDA accelerator switched on links this library where its CMake expects the plugin
 * (src/arch/arch_libs.cmake) and its own loop calls these functions unchanged. Each forwards to the C ABI
 * of misa_gb300.h; the hooks return void and, like the reference's own failures, a failed call ends the
 * process (the library's message goes to stderr). C++ linkage, as the reference declares them.
 *
 * The hooks keep one context per process (the reference calls them from its single rank thread); they
 * are not thread-safe.
 *
 * Settings the arguments do not carry are read from the environment at cuda_env_init:
 * MISA_GB300_DEVICE (default 0), MISA_GB300_PRECISION ("fp64", default, or "mixed") and
 * MISA_GB300_SETFL (the setfl file the run's potential came from; pot v0.1.0's eam class has no
 * accessor for its tables, so cuda_pot_init reads the file again).
 */
#ifndef MISA_GB300_ARCH_H
#define MISA_GB300_ARCH_H

#ifdef __cplusplus
class AtomElement;                  /* src/atom/atom_element.h:18-41, the 104-byte slot record */
class eam;                          /* pot v0.1.0's potential, passed through untouched */
namespace comm {
class BccDomain;                    /* libcomm v0.3.3's domain: phase_space, sub_box_lattice_size,
                                       lattice_const, cutoff_radius_factor are read */
}
template <class T>
class NeighbourIndex;               /* src/atom/neighbour_index.h:16-77, read as a friend */

/* archEnvInit / archEnvFinalize (src/arch/arch_env.hpp:15-25): device selection, context teardown. */
void cuda_env_init();
void cuda_env_clean();
/* simulation::createDomain (src/simulation.cpp:52-54): one GPU owns the whole periodic box, so the
 * domain must be the single-rank one (sub-box = box); creates the context (mg_create). */
void cuda_domain_init(const comm::BccDomain *domain);
/* simulation::createAtoms (src/simulation.cpp:67-69): the host's four offset tables, checked against
 * the context's own (mg_nei_offset_init). */
void cuda_nei_offset_init(const NeighbourIndex<AtomElement> *nei_offset);
/* simulation::prepareForStart (src/simulation.cpp:133): the potential, from MISA_GB300_SETFL
 * (mg_pot_init_setfl). */
void cuda_pot_init(eam *pot);
/* atom::latRho / latDf / latForce (src/atom.cpp:159-160, 293-294, 320-321), on the host slot array of
 * the whole ghost-extended grid: mg_eam_rho_calc / mg_eam_df_calc / mg_eam_force_calc. */
void cuda_eam_rho_calc(eam *pot, AtomElement *atoms, const double cutoff_radius);
void cuda_eam_df_calc(eam *pot, AtomElement *atoms, const double cutoff_radius);
void cuda_eam_force_calc(eam *pot, AtomElement *atoms, const double cutoff_radius);
#endif

#endif
