/*
 * Configuration header for compiling the heFFTe reference as a CPU oracle:
 * the stock backend only (no FFTW, MKL or GPU backends; no x86 SIMD, so the
 * same recipe builds on Arm hosts).  Written for this recipe; it plays the
 * role of the CMake-generated heffte_config.h of the reference build.
 */
#ifndef HEFFTE_CONFIG_H
#define HEFFTE_CONFIG_H

#define Heffte_VERSION_MAJOR 2
#define Heffte_VERSION_MINOR 4
#define Heffte_VERSION_PATCH 1
#define Heffte_GIT_HASH "oracle-build"

#endif
