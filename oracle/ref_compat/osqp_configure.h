/*
 * Test infrastructure (oracle only).  Build configuration used when the
 * reference's builtin (CPU, FP64, direct LDL^T) algebra is compiled from its
 * own sources for parity checks; it stands in for the CMake-generated header
 * described by configure/osqp_configure.h.in.
 */
#ifndef OSQP_CONFIGURE_H
#define OSQP_CONFIGURE_H
#define IS_LINUX
#define OSQP_ALGEBRA_BUILTIN
#define OSQP_ENABLE_PRINTING
#define OSQP_ENABLE_PROFILING
#define OSQP_ENABLE_INTERRUPT
#endif
