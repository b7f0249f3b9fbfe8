/* Stub build configuration for compiling the reference's headers with nvcc
 * (the device-side cell tests compile the reference's own TestCell): as
 * ref_config/, plus the CUDA options its CUDA headers need. */
#ifndef LGD_REF_STUB_LIBGEODECOMP_CONFIG_H
#define LGD_REF_STUB_LIBGEODECOMP_CONFIG_H
#define LIBGEODECOMP_WITH_CPP14
#define LIBGEODECOMP_WITH_THREADS
#define LIBGEODECOMP_WITH_CUDA
#define LIBGEODECOMP_DEBUG_LEVEL 0
#endif
