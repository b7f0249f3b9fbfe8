/* Stub build configuration for libflatarray (vendored with the reference). */
#ifndef LGD_REF_STUB_LIBFLATARRAY_CONFIG_H
#define LGD_REF_STUB_LIBFLATARRAY_CONFIG_H
#define LIBFLATARRAY_WITH_CPP14
#endif
