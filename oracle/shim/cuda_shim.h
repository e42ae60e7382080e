/*
 * cuda_shim.h -- forced-include prelude that lets the reference's CUDA C
 * sources compile as host C++ (g++ -include oracle/shim/cuda_shim.h).
 *
 * TEST INFRASTRUCTURE ONLY: used by oracle/build_ref.sh to build
 * oracle/_ref/libcmsl_ref.so from the reference sources where they lie.
 * Kernel qualifiers are defined away, the built-in index variables become
 * thread-local globals set by the launch emulation in oracle/ref_harness.cpp,
 * and the few runtime calls the host set-up code makes map to libc.
 */
#ifndef CMSL_CUDA_SHIM_H
#define CMSL_CUDA_SHIM_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <climits>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline
#define __shared__ static

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

typedef int cudaError_t;
enum { cudaSuccess = 0 };
typedef void *cudaEvent_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
                      cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
static inline const char *cudaGetErrorString(cudaError_t) { return "shim"; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind)
{ std::memcpy(d, s, n); return cudaSuccess; }
static inline cudaError_t cudaMemset(void *d, int v, size_t n) { std::memset(d, v, n); return cudaSuccess; }
static inline cudaError_t cudaMalloc(void **p, size_t n) { *p = std::calloc(n ? n : 1, 1); return cudaSuccess; }
static inline cudaError_t cudaFree(void *p) { std::free(p); return cudaSuccess; }
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }

/* Device pointers the reference declares in include/cuda_deps.h:44-48; the
 * definitions come from the reference's own src/global.cu. */
extern dim3 threads, blocks;
extern int threadsPerBlock, numBlocks;
extern double *Pmx_old_d, *Pmy_old_d, *Pmz_old_d, *Pmx_d, *Pmy_d, *Pmz_d;
extern double *Psx_old_d, *Psy_old_d, *Psz_old_d, *Psx_d, *Psy_d, *Psz_d;
extern double *phi_old_d, *phi_dep_d;
extern bool phi_dep_initialized;
extern double *delecX_d, *delecY_d, *delecZ_d, *divP_d;
extern double *eta_d;
extern int *omega_d;
extern double *phi_d, *theta_d, *psi_d, *TR_d;
extern double *Pmx_local_d, *Pmy_local_d, *Pmz_local_d;
extern double *Psx_local_d, *Psy_local_d, *Psz_local_d;
extern cudaEvent_t start, stop;
extern double *Psum_d;
extern void *t_storage;
extern size_t t_storage_bytes;
extern int *d_grain_mat;
extern int d_zbc_type;
extern int d_ref_id;

#endif
