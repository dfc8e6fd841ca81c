/* Host stand-in for the one cuFFT type common/filter.h names in its
 * (no-op) filter kernel signature. Used only by the oracle's reference
 * shim build (oracle/ref_shim.cpp). */
#ifndef FV_REF_SHIM_CUFFT_H
#define FV_REF_SHIM_CUFFT_H
typedef struct { float x, y; } cufftComplex;
typedef float cufftReal;
#endif
