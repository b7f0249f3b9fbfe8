/* Stub build configuration for compiling the reference's header-only
 * hot path (SerialSimulator, OpenMPSimulator, SoAGrid, SELL-C-sigma) with
 * plain g++ and no CMake.  Only the options the hot path needs are set. */
#ifndef LGD_REF_STUB_LIBGEODECOMP_CONFIG_H
#define LGD_REF_STUB_LIBGEODECOMP_CONFIG_H
#define LIBGEODECOMP_WITH_CPP14
#define LIBGEODECOMP_WITH_THREADS
#define LIBGEODECOMP_DEBUG_LEVEL 0
#endif
