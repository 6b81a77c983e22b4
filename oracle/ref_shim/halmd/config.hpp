/*
 * Minimal stand-in for the reference's generated halmd/config.hpp, used only
 * to compile the reference's own header-only Hilbert map and DSFUN routines
 * into the pinning harness (oracle/ref_harness.cpp).  Test infrastructure.
 */
#ifndef HALMD_CONFIG_HPP
#define HALMD_CONFIG_HPP
#define HALMD_GPU_ENABLED
#endif
