/*
 * shim.h -- force-included when compiling the reference's sources for the
 * oracle pin (oracle/ref/Makefile).  It does three things and nothing else:
 *   1. stands in for headers/bpd_common.h so that ACCEL_USELEN can be set per
 *      build (-DACCEL_USELEN=...); the other compile-time constants keep the
 *      reference's values (bpd_common.h:24-45);
 *   2. supplies the two names CUDA 12+ removed (texture<>, used only by an
 *      unused global at bpd_search.cu:12, and cudaThreadSynchronize);
 *   3. redirects cudaMalloc/cudaMemcpy/cudaFree in the reference's host code
 *      to host memory so that createSubharmonicInfo runs on a machine without
 *      a GPU.  No reference kernel is ever launched by the harness.
 */
#ifndef ORACLE_REF_SHIM_H_
#define ORACLE_REF_SHIM_H_

#define BPD_COMMON_H_ 1
#ifndef ACCEL_USELEN
#define ACCEL_USELEN 32000
#endif
#define ACCEL_NUMBETWEEN 2
#define ACCEL_DR 0.5
#define ACCEL_RDR 2
#define ACCEL_DZ 2
#define ACCEL_RDZ 0.5
#define ACCEL_PADDING 2000
#define DBLCORRECT 1e-14
#define NUMLOCPOWAVG 20
#define DELTAAVGBINS 5
#define NUMFINTBINS 16

#include <string.h>
#include <stdlib.h>
#include <stdio.h>
#include <stdarg.h>
#ifdef __cplusplus
#include <cuda_runtime.h>
#endif
#include <cufft.h>

#ifdef __cplusplus
extern "C" {
#endif
#include "app_utilities.h"
#ifdef __cplusplus
}

template <class T> struct texture {};
#define cudaThreadSynchronize cudaDeviceSynchronize

cudaError_t refshim_malloc(void **p, size_t n);
cudaError_t refshim_memcpy(void *d, const void *s, size_t n, cudaMemcpyKind k);
cudaError_t refshim_free(void *p);
#define cudaMalloc(p, n) refshim_malloc((void **)(p), (n))
#define cudaMemcpy refshim_memcpy
#define cudaFree refshim_free
#endif

#endif
