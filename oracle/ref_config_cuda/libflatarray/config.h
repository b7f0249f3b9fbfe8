/* Stub build configuration for libflatarray (vendored with the reference)
 * under nvcc. */
#ifndef LGD_REF_STUB_LIBFLATARRAY_CONFIG_H
#define LGD_REF_STUB_LIBFLATARRAY_CONFIG_H
#define LIBFLATARRAY_WITH_CPP14
#define LIBFLATARRAY_WITH_CUDA
#endif
