// MISA-MD's hook-name pasting (src/arch/arch_macros.h:10-11), for builds without the MISA-MD tree.
#ifndef MISA_MD_ARCH_MACROS_H
#define MISA_MD_ARCH_MACROS_H
#include "arch_building_config.h"
#define _ARCH_PREFIX_(arch_name, func_name) arch_name##_##func_name
#define ARCH_PREFIX(arch_name, func_name) _ARCH_PREFIX_(arch_name, func_name)
#endif
