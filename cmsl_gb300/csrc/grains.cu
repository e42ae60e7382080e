// grains.cu -- grain maps on the GPU.
//
// The interface flags of a device-resident map (cmsl_interface_flags_gpu,
// the reference's build_interface_flag), for maps that never leave the GPU.
//
// The columnar periodic Voronoi map of cmsl_voronoi_columnar (the stand-in for
// the reference's genpolycr_layered/voronoi.c, a brute-force nearest-seed
// search per voxel) computed on the device: one thread per (i, j) column,
// the seed points staged in shared memory, the distances in explicitly
// rounded FP64 so the map is identical to the host generator's.  The seeds,
// centres and orientations come from the same host SplitMix64 stream.
#include <algorithm>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "cmsl.h"
#include "cmsl_io.h"

void cmsl_internal_set_error(const char *msg);
void cmsl_internal_voronoi_seeds(int nx, int ny, int nz, int ng, uint64_t seed, double *sx, double *sy,
                                 double *cent, double *euler);

namespace {

constexpr int VB = 256;     // threads per block
constexpr int VCHUNK = 512; // seeds staged per pass

__global__ void __launch_bounds__(VB) k_voronoi(int nx, int ny, int nz, int ng, const double *__restrict__ sx,
                                                const double *__restrict__ sy, int32_t *__restrict__ omega)
{
    __shared__ double s_x[VCHUNK], s_y[VCHUNK];
    const long long plane = (long long)nx * ny;
    const long long c = (long long)blockIdx.x * VB + threadIdx.x;
    const bool live = c < plane;
    const int i = live ? (int)(c % nx) : 0, j = live ? (int)(c / nx) : 0;
    const double x = i + 0.5, y = j + 0.5, fx = nx, fy = ny;
    int best = 0;
    double bd = 1e300;
    for (int g0 = 0; g0 < ng; g0 += VCHUNK) {
        const int n = min(VCHUNK, ng - g0);
        __syncthreads();
        for (int t = threadIdx.x; t < n; t += VB) {
            s_x[t] = sx[g0 + t];
            s_y[t] = sy[g0 + t];
        }
        __syncthreads();
        if (live)
            for (int t = 0; t < n; ++t) {
                double dx = fabs(__dsub_rn(x, s_x[t])), dy = fabs(__dsub_rn(y, s_y[t]));
                dx = fmin(dx, __dsub_rn(fx, dx));
                dy = fmin(dy, __dsub_rn(fy, dy));
                const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
                if (d2 < bd) { bd = d2; best = g0 + t; }
            }
    }
    if (live)
        for (int k = 0; k < nz; ++k) omega[c + plane * k] = best;
}

// build_interface_flag (main.cu:13-42): an FE voxel off the first and last
// planes is an interface voxel when the voxel above or below it is not FE (a
// grain id outside [0, ng) counts as not FE); 1 / 0 per voxel.
__global__ void k_interface(int nx, int ny, int nz, int ng, const int32_t *__restrict__ omega,
                            const int32_t *__restrict__ gmat, int32_t *__restrict__ flag)
{
    const long long plane = (long long)nx * ny, n = plane * nz;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int g = omega[i];
        const long long k = i / plane;
        int v = 0;
        if (g >= 0 && g < ng && gmat[g] == CMSL_FE && k > 0 && k < nz - 1) {
            const int gu = omega[i + plane], gd = omega[i - plane];
            const int mu = (gu >= 0 && gu < ng) ? gmat[gu] : -1, md = (gd >= 0 && gd < ng) ? gmat[gd] : -1;
            v = (mu != CMSL_FE || md != CMSL_FE) ? 1 : 0;
        }
        flag[i] = v;
    }
}

cmsl_status gfail(cmsl_status s, const char *msg)
{
    cmsl_internal_set_error(msg);
    return s;
}

}  // namespace

extern "C" cmsl_status cmsl_voronoi_columnar_gpu(int nx, int ny, int nz, int ng, uint64_t seed, int32_t *omega,
                                                 double *cent, double *euler)
{
    if (nx < 1 || ny < 1 || nz < 1 || ng < 1 || !omega) return gfail(CMSL_ERR_ARG, "bad arguments");
    std::vector<double> sx(ng), sy(ng);
    cmsl_internal_voronoi_seeds(nx, ny, nz, ng, seed, sx.data(), sy.data(), cent, euler);
    const size_t N = (size_t)nx * ny * nz, plane = (size_t)nx * ny;
    double *d_s = nullptr;
    int32_t *d_om = nullptr;
    cudaError_t e = cudaMalloc(&d_s, sizeof(double) * 2 * ng);
    if (e == cudaSuccess) e = cudaMalloc(&d_om, sizeof(int32_t) * N);
    if (e == cudaSuccess) e = cudaMemcpy(d_s, sx.data(), sizeof(double) * ng, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_s + ng, sy.data(), sizeof(double) * ng, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const unsigned blocks = (unsigned)((plane + VB - 1) / VB);
        k_voronoi<<<blocks, VB>>>(nx, ny, nz, ng, d_s, d_s + ng, d_om);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(omega, d_om, sizeof(int32_t) * N, cudaMemcpyDeviceToHost);
    cudaFree(d_s);
    cudaFree(d_om);
    if (e != cudaSuccess) {
        cmsl_internal_set_error(cudaGetErrorString(e));
        return CMSL_ERR_CUDA;
    }
    return CMSL_OK;
}

// Interface flags of a grain map held in device memory (a map generated on
// the GPU stays there): omega_dev[N], grain_mat_dev[n_grains], flags_dev[N],
// grain ids outside [0, n_grains) count as not FE (never read beyond the table),
// all device pointers; runs on `stream` and returns without synchronising.
extern "C" cmsl_status cmsl_interface_flags_gpu(int nx, int ny, int nz, int n_grains, const int32_t *omega_dev,
                                                const int32_t *grain_mat_dev, int32_t *flags_dev, void *stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || n_grains < 1 || !omega_dev || !grain_mat_dev || !flags_dev)
        return gfail(CMSL_ERR_ARG, "bad arguments");
    const long long n = (long long)nx * ny * nz;
    const unsigned blocks = (unsigned)std::min<long long>((n + VB - 1) / VB, 152LL * 16);
    k_interface<<<blocks, VB, 0, (cudaStream_t)stream>>>(nx, ny, nz, n_grains, omega_dev, grain_mat_dev, flags_dev);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        cmsl_internal_set_error(cudaGetErrorString(e));
        return CMSL_ERR_CUDA;
    }
    return CMSL_OK;
}
