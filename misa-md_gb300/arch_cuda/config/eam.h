// Stand-in for the pot package's eam class (pot v0.1.0, git.hpcer.dev/HPCer/CrystalMD/potential), which
// MISA-MD fetches at build time and does not ship. The plugin passes eam pointers through without
// touching them, so the class only needs its name.
#ifndef MISA_GB300_STANDIN_EAM_H
#define MISA_GB300_STANDIN_EAM_H
class eam;
#endif
