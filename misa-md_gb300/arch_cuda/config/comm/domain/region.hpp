// Stand-in for libcomm v0.3.3's region header (not shipped with MISA-MD); nothing the plugin includes
// uses its declarations.
#ifndef MISA_GB300_STANDIN_COMM_REGION_HPP
#define MISA_GB300_STANDIN_COMM_REGION_HPP
#endif
