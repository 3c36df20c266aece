/*
 * Test infrastructure: configuration of the reference's C core as it is built
 * against a CUDA-class algebra backend (configure/osqp_configure.h.in with
 * OSQP_ALGEBRA_CUDA), used only to link that unmodified core against the
 * GB300 algebra library and prove the boundary is complete.
 */
#ifndef OSQP_CONFIGURE_H
#define OSQP_CONFIGURE_H
#define IS_LINUX
#define OSQP_ALGEBRA_CUDA
#define OSQP_ENABLE_PRINTING
#define OSQP_ENABLE_PROFILING
#define OSQP_ENABLE_INTERRUPT
#endif
