// spectral.cuh -- direct solve of the FP32 inner system for films whose
// materials share one permittivity (the configurations' eps_b).
//
// With a uniform eps the operator of depol_varEPS.cu:37-124 on the interior
// planes k = 1..nz-2 is (eps/h^2)(6 x_c - sum of the 6 neighbours), periodic
// in x and y, with x = 0 on the Dirichlet planes.  The in-plane discrete
// Fourier transform diagonalises the x/y part (eigenvalues 2 - 2 cos(2 pi m / n)),
// which leaves one real tridiagonal system along z per in-plane mode:
//   (lam_x + lam_y + 2) X_k - X_{k-1} - X_{k+1} = (h^2 / eps) R_k.
// The solve is: 2D FFT of every interior plane of r -> Thomas algorithm per
// mode -> inverse 2D FFT (as the forward transform of the conjugate, the
// system being real) -> x.  It is exact up to FP32 rounding (~1e-6 relative),
// so one solve per refinement pass replaces the PCG iterations; the outer
// double-float refinement keeps the potential at the reference's tolerance.
//
// FFTs: mixed radix-2/3 self-sorting (Stockham) passes in shared memory, one
// block per group of rows (x) or of columns (y); twiddles exp(-2 pi i t / n)
// and eigenvalues come from host tables computed in double.
#pragma once
#include "kernels.cuh"

namespace cmsl {

constexpr int SPEC_MAX_STAGES = 13;       // 2^12 = 4096
constexpr int SPEC_ELEMS = 4096;          // complex values staged per block
constexpr int SPEC_NT = 256;

struct SpecAxis {
    int n, nst;
    int rad[SPEC_MAX_STAGES];
};

struct SpecDev {
    float2 *C;                  // [M][ny][nx] spectra of the interior planes
    float *cp;                  // [M][ny*nx] Thomas coefficients
    const float2 *twx, *twy;    // exp(-2 pi i t / n)
    const float *lamx, *lamy;   // 2 - 2 cos(2 pi t / n)
    SpecAxis ax, ay;
    int nx, ny, nz, M;
    float scale;                // h^2 / (eps nx ny)
};

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// nseq sequences of length n, [seq][n] in a; transforms them with scratch b;
// returns the buffer holding the result.  All threads of the block call it.
__device__ __forceinline__ float2 *fft_seqs(float2 *a, float2 *b, int nseq, const SpecAxis &pl,
                                            const float2 *__restrict__ tw)
{
    const int n = pl.n;
    int Ns = 1;
    for (int st = 0; st < pl.nst; ++st) {
        const int R = pl.rad[st];
        const int nbf = n / R;
        const int tstride = n / (Ns * R);
        for (int t = threadIdx.x; t < nseq * nbf; t += blockDim.x) {
            const int s = t / nbf, j = t - s * nbf;
            const int jm = j % Ns;
            const float2 *src = a + s * n;
            float2 *dst = b + s * n;
            const int o = (j / Ns) * Ns * R + jm;
            const float2 v0 = src[j];
            const float2 v1 = c_mul(src[j + nbf], __ldg(tw + jm * tstride));
            if (R == 2) {
                dst[o] = c_add(v0, v1);
                dst[o + Ns] = c_sub(v0, v1);
            } else {
                const float2 v2 = c_mul(src[j + 2 * nbf], __ldg(tw + 2 * jm * tstride));
                const float2 s12 = c_add(v1, v2), d12 = c_sub(v1, v2);
                const float2 m = make_float2(v0.x - 0.5f * s12.x, v0.y - 0.5f * s12.y);
                const float k3 = 0.86602540378443865f;   // sin(2 pi / 3)
                const float2 rot = make_float2(k3 * d12.y, -k3 * d12.x);
                dst[o] = c_add(v0, s12);
                dst[o + Ns] = c_add(m, rot);
                dst[o + 2 * Ns] = c_sub(m, rot);
            }
        }
        __syncthreads();
        float2 *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Whether the film's inner solve runs through the spectra this step.
__device__ __forceinline__ bool spec_run(const Dev &d)
{
    return d.force || *(volatile const int *)&d.solve[0].active != 0;
}

// x transforms of rows (kk, y), kk = interior plane - 1.  IN_REAL: from the
// FP32 residual r into the spectra; otherwise from the spectra into the real
// correction x (and x = 0 on the Dirichlet planes).
template <bool IN_REAL>
__global__ void __launch_bounds__(SPEC_NT) k_spec_x(Dev d, Fields<float> F, SpecDev sp)
{
    extern __shared__ float2 sm2[];
    if (!spec_run(d)) return;
    const int nx = sp.nx, rows = sp.M * sp.ny, rb = max(1, SPEC_ELEMS / nx);
    const int r0 = blockIdx.x * rb, nr = min(rb, rows - r0);
    const long long plane = (long long)nx * sp.ny;
    float2 *a = sm2, *b = sm2 + rb * nx;
    for (int t = threadIdx.x; t < nr * nx; t += blockDim.x) {
        const int s = t / nx, i = t - s * nx;
        const long long row = r0 + s;              // (kk, y)
        if (IN_REAL) {
            const long long kk = row / sp.ny, y = row - kk * sp.ny;
            a[t] = make_float2(F.r[(kk + 1) * plane + y * nx + i], 0.f);
        } else {
            a[t] = sp.C[row * nx + i];
        }
    }
    __syncthreads();
    const float2 *res = fft_seqs(a, b, nr, sp.ax, sp.twx);
    for (int t = threadIdx.x; t < nr * nx; t += blockDim.x) {
        const int s = t / nx, i = t - s * nx;
        const long long row = r0 + s;
        if (IN_REAL) {
            sp.C[row * nx + i] = res[t];
        } else {
            const long long kk = row / sp.ny, y = row - kk * sp.ny;
            F.x[(kk + 1) * plane + y * nx + i] = res[t].x;
            if (kk == 0) F.x[y * nx + i] = 0.f;
            if (kk == sp.M - 1) F.x[(sp.nz - 1) * plane + y * nx + i] = 0.f;
        }
    }
}

// y transforms of column groups of one interior plane, in place on the spectra.
static __global__ void __launch_bounds__(SPEC_NT) k_spec_y(Dev d, SpecDev sp)
{
    extern __shared__ float2 sm2[];
    if (!spec_run(d)) return;
    const int nx = sp.nx, ny = sp.ny, cb = max(1, SPEC_ELEMS / ny);
    const int groups = (nx + cb - 1) / cb;
    const int kk = blockIdx.x / groups, x0 = (blockIdx.x - kk * groups) * cb, nc = min(cb, nx - x0);
    float2 *base = sp.C + (long long)kk * nx * ny;
    float2 *a = sm2, *b = sm2 + cb * ny;
    for (int t = threadIdx.x; t < nc * ny; t += blockDim.x) {
        const int y = t / nc, c = t - y * nc;      // coalesced along x
        a[c * ny + y] = base[(long long)y * nx + x0 + c];
    }
    __syncthreads();
    const float2 *res = fft_seqs(a, b, nc, sp.ay, sp.twy);
    for (int t = threadIdx.x; t < nc * ny; t += blockDim.x) {
        const int y = t / nc, c = t - y * nc;
        base[(long long)y * nx + x0 + c] = res[c * ny + y];
    }
}

// Thomas algorithm along z for every in-plane mode; writes the conjugate of
// the scaled solution so that the next forward transforms invert.
static __global__ void __launch_bounds__(SPEC_NT) k_spec_z(Dev d, SpecDev sp)
{
    if (!spec_run(d)) return;
    const long long modes = (long long)sp.nx * sp.ny;
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= modes) return;
    const int x = (int)(m % sp.nx), y = (int)(m / sp.nx);
    const float dg = __ldg(sp.lamx + x) + __ldg(sp.lamy + y) + 2.f;
    const float s = sp.scale;
    float2 *C = sp.C + m;
    float *cp = sp.cp + m;
    float c_prev = 0.f;
    float2 d_prev = make_float2(0.f, 0.f);
    for (int k = 0; k < sp.M; ++k) {                 // forward sweep (sub/super-diagonal -1)
        const float piv = dg + c_prev;
        const float inv = 1.f / piv;
        const float2 rk = C[k * modes];
        const float2 dk = make_float2((rk.x * s + d_prev.x) * inv, (rk.y * s + d_prev.y) * inv);
        c_prev = -inv;
        cp[k * modes] = c_prev;
        C[k * modes] = dk;
        d_prev = dk;
    }
    float2 xn = d_prev;                              // back substitution
    C[(sp.M - 1) * modes] = make_float2(xn.x, -xn.y);
    for (int k = sp.M - 2; k >= 0; --k) {
        const float2 dk = C[k * modes];
        const float c = cp[k * modes];
        xn = make_float2(dk.x - c * xn.x, dk.y - c * xn.y);
        C[k * modes] = make_float2(xn.x, -xn.y);
    }
}

// After the solve: the inner solve of this pass is done (one "iteration").
static __global__ void k_spec_done(Dev d)
{
    if (threadIdx.x == 0 && blockIdx.x == 0 && spec_run(d) && !d.force) {
        SolveDev *S = d.solve;
        S->iters = 1;
        S->total_iters += 1;
        S->active = 0;
    }
}

}  // namespace cmsl
