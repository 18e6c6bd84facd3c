// What MISA-MD's CMake writes from src/arch/arch_building_config.h.in with the CUDA accelerator switched
// on (MD_CUDA_ARCH_ENABLE_FLAG=ON, src/arch/arch_configure.cmake): the hooks are named cuda_*.
#ifndef MISA_MD_ARCH_BUILDING_CONFIG_H
#define MISA_MD_ARCH_BUILDING_CONFIG_H
#define ACCELERATE_ENABLED
#define ARCH_NAME cuda
#define ARCH_CUDA
#endif
