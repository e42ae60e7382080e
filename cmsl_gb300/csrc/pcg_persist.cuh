// pcg_persist.cuh -- persistent single-reduction Jacobi-PCG for the FP32 inner
// solve of CMSL_FP32_REFINED.
//
// The reference runs textbook PCG with two blocking dot products per
// iteration (depol_varEPS.cu:472-522).  Here the inner solve of each
// refinement pass is one cooperative kernel that stays resident for all its
// iterations.  It uses the Chronopoulos-Gear recurrences, which need a single
// reduction (two dots) per iteration, so every iteration is one sweep over the
// film and one grid barrier:
//
//   p_i = u_i + b_i p_{i-1}      s_i = w_i + b_i s_{i-1}
//   x  += a_i p_i                r_{i+1} = r_i - a_i s_i
//   u_{i+1} = D^-1 r_{i+1}       w_{i+1} = A u_{i+1}
//   g_{i+1} = (r_{i+1}, u_{i+1}) d_{i+1} = (w_{i+1}, u_{i+1})
//   b_{i+1} = g_{i+1}/g_i        a_{i+1} = g_{i+1} / (d_{i+1} - b_{i+1} g_{i+1} / a_i)
//
// w = A u needs u at the x/y/z neighbours; u there is recomputed from the
// neighbour's r_i, w_i, s_{i-1} (r, w, s ping-pong by iteration parity so
// that no block overwrites a value another block still reads).
//
// Grid barrier: arrival counter + bounded spin (about a second), after which
// the block records a timeout and leaves; no wait is unbounded.  Every block
// then sums all blocks' partials in block order, so all blocks hold the same
// scalars and take the same loop decisions without a second barrier.
#pragma once
#include "kernels.cuh"

namespace cmsl {

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

constexpr unsigned long long BARRIER_SPIN_LIMIT = 20000000ull;   // x ~100 ns sleeps

// Brick geometry of the persistent solver: a block of PBX x PBY threads owns
// the TX x TY column tile plus its one-cell x/y halo; it stages u = D^-1 r for
// PZ planes (+1 above and below) in shared memory, then applies the stencil.
constexpr int PBX = TX + 2;
constexpr int PBY = TY + 2;
constexpr int PNT = PBX * PBY;          // 340 threads
constexpr int PNW = (PNT + 31) / 32;    // 11 warps
constexpr int PZ = 8;
constexpr int PBP = PZ + 2;

// Block sum over PNT threads: FP32 within a warp, FP64 across warps.
template <int NV, class T>
__device__ __forceinline__ void block_sum_p(T (&v)[NV], double (*sm)[NV], double (&out)[NV])
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
        const T s = warp_sum(v[i]);
        if (lane == 0) sm[w][i] = (double)s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        #pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int q = 0; q < PNW; ++q) s += sm[q][i];
            out[i] = s;
        }
    }
    __syncthreads();
}

// Writes this block's two partial sums, waits for all blocks, and returns the
// grid totals (identical in every block).  False if the wait timed out.
// Block partials are stored as double-float pairs and summed across blocks by
// one warp in double-float, so the all-reduce issues no FP64 instruction
// beyond a handful of conversions.
__device__ __forceinline__ df warp_sum_df(df v)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const df w{__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
        v = df_add(v, w);
    }
    return v;
}

__device__ __forceinline__ bool grid_allreduce2(const CgBuf &B, int parity, unsigned int &target,
                                                float v0, float v1, double (*sm)[2], double &t0,
                                                double &t1)
{
    __shared__ int s_ok;
    __shared__ double s_tot[2];
    float a[2] = {v0, v1};
    double blk[2];
    block_sum_p<2, float>(a, sm, blk);
    float4 *part = B.part + (size_t)parity * gridDim.x;
    target += gridDim.x;
    if (threadIdx.x == 0) {
        const float h0 = (float)blk[0], h1 = (float)blk[1];
        __stcg(part + blockIdx.x, make_float4(h0, (float)(blk[0] - (double)h0), h1, (float)(blk[1] - (double)h1)));
        __threadfence();
        atomicAdd(B.arrive, 1u);
        int ok = 1;
        unsigned long long spins = 0;
        while (ld_acquire(B.arrive) < target) {
            if (++spins > BARRIER_SPIN_LIMIT) { ok = 0; atomicExch(B.err, 1); break; }
            __nanosleep(64);
        }
        s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) return false;
    if (threadIdx.x < 32) {
        df q0{0.f, 0.f}, q1{0.f, 0.f};
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {
            const float4 v = __ldcg(part + b);
            q0 = df_add(q0, df{v.x, v.y});
            q1 = df_add(q1, df{v.z, v.w});
        }
        q0 = warp_sum_df(q0);
        q1 = warp_sum_df(q1);
        if (threadIdx.x == 0) {
            s_tot[0] = (double)q0.h + (double)q0.l;
            s_tot[1] = (double)q1.h + (double)q1.l;
        }
    }
    __syncthreads();
    t0 = s_tot[0];
    t1 = s_tot[1];
    return true;
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared-memory carve-up of one brick (dynamic shared memory).
constexpr int PNPL = PBP * PBY * PBX;   // staged cells, all planes
constexpr int PNOWN = PZ * PBY * PBX;   // own planes
struct BrickSmem {
    float *r, *w, *s, *d, *u, *x, *p;
    uint32_t *c;
};
constexpr size_t PSMEM_BYTES = sizeof(float) * (6 * PNPL + 2 * PNOWN);

__device__ __forceinline__ BrickSmem brick_smem(float *base)
{
    BrickSmem m;
    m.r = base; m.w = base + PNPL; m.s = base + 2 * PNPL; m.d = base + 3 * PNPL;
    m.c = (uint32_t *)(base + 4 * PNPL); m.u = base + 5 * PNPL;
    m.x = base + 6 * PNPL; m.p = base + 6 * PNPL + PNOWN;
    return m;
}

// Film constants held in registers for the whole solve (the compiler would
// otherwise reload them from global memory after every float store).
struct FilmC {
    int nx, ny, nz, zbc, ref_id, plane;
    long long off;
    float inv_h2;
    float dinv_uni;
};

__device__ __forceinline__ bool id_row(const FilmC &F, int k, int pl)
{
    if (F.zbc == 0) return k == 0 || k == F.nz - 1;
    return pl + k * F.plane == F.ref_id;
}

// One brick (tile x0,y0; planes z0..z1-1, z1 - z0 <= PZ).  INIT: w_0 = A D^-1 r_0
// and its dots.  Otherwise iteration i with parity c and (alpha, beta) = (a_i, b_i).
// Stage (cp.async, every load of the brick in flight at once) -> pointwise
// phase from shared memory -> stencil phase.  UNI: all materials share one
// eps, so A is the constant-coefficient 7-point operator and no material codes
// are read.
template <bool INIT, bool UNI>
__device__ __forceinline__ void cg_brick(const FilmC &F, const CgBuf &B, const uint32_t *__restrict__ code,
                                         const float *__restrict__ dv, int x0, int y0, int z0, int z1, int c,
                                         bool first, float alpha, float beta, float &gacc, float &dacc,
                                         const BrickSmem &sm, const float *sEps)
{
    const int nx = F.nx, ny = F.ny, nz = F.nz, plane = F.plane;
    const int bx = threadIdx.x % PBX, by = threadIdx.x / PBX;
    const int wx = min(TX, nx - x0), wy = min(TY, ny - y0);
    const bool own = bx >= 1 && bx <= wx && by >= 1 && by <= wy;
    const bool ex = bx == 0 || bx == wx + 1, ey = by == 0 || by == wy + 1;
    const bool need = bx <= wx + 1 && by <= wy + 1 && !(ex && ey);
    const int gx = (x0 - 1 + bx + nx) % nx, gy = (y0 - 1 + by + ny) % ny;
    const int pl = gx + nx * gy;
    // parity selects by value: a dynamically indexed parameter array would be
    // copied to local memory
    const float *__restrict__ rA = (c ? B.r[1] : B.r[0]) + F.off;
    const float *__restrict__ wA = (c ? B.w[1] : B.w[0]) + F.off;
    const float *__restrict__ sA = (c ? B.s[1] : B.s[0]) + F.off;
    float *__restrict__ rB = (c ? B.r[0] : B.r[1]) + F.off;
    float *__restrict__ sB = (c ? B.s[0] : B.s[1]) + F.off;
    float *__restrict__ wB = (INIT ? B.w[0] : (c ? B.w[0] : B.w[1])) + F.off;
    float *__restrict__ x = B.x + F.off;
    float *__restrict__ p = B.p + F.off;
    constexpr int PP = PBY * PBX;
    const int col = by * PBX + bx;
    const int klo = own ? max(z0 - 1, 0) : z0;
    const int khi = own ? min(z1, nz - 1) : z1 - 1;

    if (need) {
        for (int k = klo; k <= khi; ++k) {
            const int o = pl + k * plane;
            const int si = (k - z0 + 1) * PP + col;
            cp_async4(sm.r + si, rA + o);
            cp_async4(sm.d + si, dv + o);
            if (!UNI) cp_async4(sm.c + si, code + o);
            if (!INIT) {
                cp_async4(sm.w + si, wA + o);
                if (!first) cp_async4(sm.s + si, sA + o);
                if (!first && own && k >= z0 && k < z1) {
                    const int oi = (k - z0) * PP + col;
                    cp_async4(sm.x + oi, x + o);
                    cp_async4(sm.p + oi, p + o);
                }
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // u_{i+1} = D^-1 r_{i+1} for every staged cell; own cells do their pointwise updates
    if (need) {
        for (int k = klo; k <= khi; ++k) {
            const int si = (k - z0 + 1) * PP + col;
            const float dd = sm.d[si], ri = sm.r[si];
            const bool mine = own && k >= z0 && k < z1;
            float u, rn;
            if (INIT) {
                rn = ri;
                u = dd * ri;
            } else {
                const float wi = sm.w[si];
                const float sv = first ? wi : fmaf(beta, sm.s[si], wi);
                rn = fmaf(-alpha, sv, ri);
                u = dd * rn;
                if (mine) {
                    const int o = pl + k * plane;
                    const int oi = (k - z0) * PP + col;
                    const float ui = dd * ri;
                    const float pi = first ? ui : fmaf(beta, sm.p[oi], ui);
                    x[o] = first ? alpha * pi : fmaf(alpha, pi, sm.x[oi]);
                    p[o] = pi;
                    sB[o] = sv;
                    rB[o] = rn;
                }
            }
            if (mine) gacc = fmaf(rn, u, gacc);
            sm.u[si] = u;
        }
    }
    __syncthreads();
    // w_{i+1} = A u_{i+1} on own cells (depol_varEPS.cu:101-123 operator order)
    if (own) {
        for (int k = z0; k < z1; ++k) {
            const int zi = k - z0 + 1;
            const int si = zi * PP + col;
            const float uc = sm.u[si];
            float wv;
            if (id_row(F, k, pl)) {
                wv = uc;
            } else {
                int zu = zi + 1, zd = zi - 1;
                if (F.zbc != 0) {
                    if (k == 0) zd = zu;
                    else if (k == nz - 1) zu = zd;
                }
                const int su = zu * PP + col, sd = zd * PP + col;
                const float ue = sm.u[si + 1], uw = sm.u[si - 1], un = sm.u[si + PBX], us = sm.u[si - PBX];
                const float uu = sm.u[su], ud = sm.u[sd];
                float a;
                if (UNI) {
                    const float e0 = sEps[0];
                    a = e0 * ((((((ue - uc) - (uc - uw)) + (un - uc)) - (uc - us)) + (uu - uc)) - (uc - ud));
                } else {
                    const int mc = code_mat(sm.c[si]) * 3;
                    a = sEps[mc + code_mat(sm.c[si + 1])] * (ue - uc) - sEps[mc + code_mat(sm.c[si - 1])] * (uc - uw);
                    a += sEps[mc + code_mat(sm.c[si + PBX])] * (un - uc);
                    a -= sEps[mc + code_mat(sm.c[si - PBX])] * (uc - us);
                    a += sEps[mc + code_mat(sm.c[su])] * (uu - uc);
                    a -= sEps[mc + code_mat(sm.c[sd])] * (uc - ud);
                }
                wv = -(a * F.inv_h2);
            }
            wB[pl + k * plane] = wv;
            dacc = fmaf(wv, uc, dacc);
        }
    }
    __syncthreads();
}

template <bool INIT, bool UNI>
__device__ __forceinline__ void cg_sweep_all(const Dev &d, const FilmC &F, const CgBuf &B, const float *dinv,
                                             int c, bool first, float alpha, float beta, float &ga, float &da,
                                             const BrickSmem &sm, const float *sEps)
{
    const uint32_t *code = d.code + F.off;
    const float *dv = dinv + F.off;
    for (int i = blockIdx.x; i < d.n_items; i += gridDim.x) {
        const int4 it = d.items[i];
        const int z0 = it.w & 0xffff, z1 = it.w >> 16;
        for (int zz = z0; zz < z1; zz += PZ)
            cg_brick<INIT, UNI>(F, B, code, dv, it.y, it.z, zz, min(zz + PZ, z1), c, first, alpha, beta, ga, da,
                                sm, sEps);
    }
}

// Thread 0's scalar step of the single-reduction (Chronopoulos-Gear)
// recurrence after an iteration produced gn = (r,u) and dn = (w,u), w = A u.
// Returns 1 to go on (s_ab = {alpha, beta} of the next iteration), 0 to end
// this inner pass; status = 1 only for a non-finite residual.  Rounding can
// make the recurrence's estimate of (p, A p) non-positive on ill-conditioned
// operators (a Neumann film pinned at one cell); the iteration then restarts
// from p = u (beta = 0, alpha = gn / dn), which needs only (u, A u) > 0.  With
// no positive direction left the pass ends and the outer refinement, which
// recomputes the true residual, decides what follows.
__device__ __forceinline__ int cg_scalars(double gn, double dn, double &gam, double &alpha, float *s_ab,
                                          int &status)
{
    if (!isfinite(gn) || !isfinite(dn) || gn < 0.0) {
        status = 1;
        gam = gn;
        return 0;
    }
    const double bn = gn / gam;
    const double den = dn - bn * gn / alpha;
    gam = gn;
    if (gn == 0.0) return 0;
    if (den > 0.0) {
        alpha = gn / den;
        s_ab[0] = (float)alpha;
        s_ab[1] = (float)bn;
        return 1;
    }
    if (dn > 0.0) {
        alpha = gn / dn;
        s_ab[0] = (float)alpha;
        s_ab[1] = 0.f;
        return 1;
    }
    return 0;
}

// The inner FP32 solve of one refinement pass on a single film: starts from
// r_0 in B.r[0] (written by k_refine) and x = 0, runs until
// (r,u) <= inner_tol2 (r_0,u_0) or inner_max iterations, leaves the
// correction in B.x.  Cooperative launch of PNT-thread blocks; grid <=
// co-resident blocks.  The scalar recurrences run in FP64 on thread 0 only
// and are broadcast through shared memory.
template <bool UNI>
__global__ void __launch_bounds__(PNT, 2) k_pcg_cg1(Dev d, CgBuf B, const float *dinv)
{
    extern __shared__ float4 dsm4[];
    const BrickSmem sm = brick_smem((float *)dsm4);
    __shared__ double sRed[PNW][2];
    __shared__ float sEps[9];
    __shared__ float s_ab[2];
    __shared__ int s_go;
    const FilmDev *f = d.films;
    SolveDev *S = d.solve;
    const bool run = f->dep_flag != 0 && *(volatile int *)&S->active != 0;
    if (!run) return;                       // uniform: k_refine decided for every block
    FilmC F;
    F.nx = f->nx; F.ny = f->ny; F.nz = f->nz; F.zbc = f->zbc; F.ref_id = f->ref_id;
    F.plane = f->nx * f->ny; F.off = f->off; F.inv_h2 = f->inv_h2f; F.dinv_uni = f->dinv_uni;
    if (threadIdx.x < 9) sEps[threadIdx.x] = f->epsf32[threadIdx.x];
    __syncthreads();
    const double tol2 = S->inner_tol2;
    const int imax = S->inner_max;
    unsigned int target = 0;
    float ga = 0.f, da = 0.f;
    cg_sweep_all<true, UNI>(d, F, B, dinv, 0, true, 0.f, 0.f, ga, da, sm, sEps);
    double g0, dl;
    if (!grid_allreduce2(B, 0, target, ga, da, sRed, g0, dl)) return;
    // thread 0 owns the recurrences
    double gam = g0, alpha = (dl > 0.0) ? g0 / dl : 0.0;
    int it = 0, status = 0;
    if (threadIdx.x == 0) {
        s_go = isfinite(g0) && g0 > 0.0 && dl > 0.0 && gam > tol2 * g0 && imax > 0;
        if (!(isfinite(g0) && g0 > 0.0 && dl > 0.0)) status = (g0 == 0.0) ? 0 : 1;
        s_ab[0] = (float)alpha;
        s_ab[1] = 0.f;
    }
    __syncthreads();
    while (s_go) {
        const float a = s_ab[0], b = s_ab[1];
        ga = 0.f; da = 0.f;
        cg_sweep_all<false, UNI>(d, F, B, dinv, it & 1, it == 0, a, b, ga, da, sm, sEps);
        double gn, dn;
        if (!grid_allreduce2(B, (it + 1) & 1, target, ga, da, sRed, gn, dn)) return;
        ++it;
        if (threadIdx.x == 0) {
            const int go = cg_scalars(gn, dn, gam, alpha, s_ab, status);
            s_go = go && gam > tol2 * g0 && it < imax;
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S->iters = it;
        S->total_iters += it;
        S->rz = gam;
        S->rz0 = g0;
        S->active = 0;
        if (status) { S->status = 1; S->outer_active = 0; }
    }
}

// ------------------------------------------------------------------------
// Two-phase persistent solver.  Per iteration:
//   P (pointwise, float4, every cell, no halo):
//       s = w + b s,  p = D^-1 r + b p,  x += a p,  r -= a s,  u = D^-1 r,
//       gamma += r.u
//   grid sync
//   S (stencil bricks staging only u): w = A u,  delta += w.u
//   grid sync + all-reduce (gamma, delta)
// All updates are in place (P touches only its own cells; S reads u, which P
// does not write again before the next grid sync).
// ------------------------------------------------------------------------

// Plain grid barrier (no reduction), same bounded wait.
__device__ __forceinline__ bool grid_sync(const CgBuf &B, unsigned int &target)
{
    __shared__ int s_ok2;
    __syncthreads();
    target += gridDim.x;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(B.arrive, 1u);
        int ok = 1;
        unsigned long long spins = 0;
        while (ld_acquire(B.arrive) < target) {
            if (++spins > BARRIER_SPIN_LIMIT) { ok = 0; atomicExch(B.err, 1); break; }
            __nanosleep(32);
        }
        s_ok2 = ok;
    }
    __syncthreads();
    return s_ok2 != 0;
}

// Phase P over all cells of the film.  INIT: u = D^-1 r, gamma = r.u.
template <bool INIT, bool UNI>
__device__ __forceinline__ void cg2_point(const FilmC &F, const CgBuf &B, const float *__restrict__ dv,
                                          long long n, bool first, float a, float b, float &gacc)
{
    // UNI: D^-1 is 1 on the identity rows (Dirichlet planes / Neumann pin) and
    // one constant elsewhere, so it is not read from memory
    const long long id_lo = (long long)F.plane, id_hi = (long long)F.plane * (F.nz - 1);
    auto dinv_of = [&](long long c) -> float {
        const bool idr = F.zbc == 0 ? (c < id_lo || c >= id_hi) : (c == (long long)F.ref_id);
        return idr ? 1.f : F.dinv_uni;
    };
    float *__restrict__ r = B.r[0] + F.off;
    float *__restrict__ u = B.r[1] + F.off;
    float *__restrict__ w = B.w[0] + F.off;
    float *__restrict__ s = B.s[0] + F.off;
    float *__restrict__ x = B.x + F.off;
    float *__restrict__ p = B.p + F.off;
    const float *__restrict__ d = dv + F.off;
    const long long n4 = n >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
        float dd[4];
        if (UNI) {
            #pragma unroll
            for (int j = 0; j < 4; ++j) dd[j] = dinv_of(4 * q + j);
        } else {
            const float4 D4 = reinterpret_cast<const float4 *>(d)[q];
            dd[0] = D4.x; dd[1] = D4.y; dd[2] = D4.z; dd[3] = D4.w;
        }
        const float4 R4 = reinterpret_cast<const float4 *>(r)[q];
        const float ri[4] = {R4.x, R4.y, R4.z, R4.w};
        float uo[4], ro[4];
        if (INIT) {
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                ro[j] = ri[j];
                uo[j] = dd[j] * ri[j];
                gacc = fmaf(ro[j], uo[j], gacc);
            }
        } else {
            const float4 W4 = reinterpret_cast<const float4 *>(w)[q];
            const float wi[4] = {W4.x, W4.y, W4.z, W4.w};
            float si[4] = {0.f, 0.f, 0.f, 0.f}, pi[4] = {0.f, 0.f, 0.f, 0.f}, xi[4] = {0.f, 0.f, 0.f, 0.f};
            if (!first) {
                const float4 S4 = reinterpret_cast<const float4 *>(s)[q];
                const float4 P4 = reinterpret_cast<const float4 *>(p)[q];
                const float4 X4 = reinterpret_cast<const float4 *>(x)[q];
                si[0] = S4.x; si[1] = S4.y; si[2] = S4.z; si[3] = S4.w;
                pi[0] = P4.x; pi[1] = P4.y; pi[2] = P4.z; pi[3] = P4.w;
                xi[0] = X4.x; xi[1] = X4.y; xi[2] = X4.z; xi[3] = X4.w;
            }
            float so[4], po[4], xo[4];
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                so[j] = first ? wi[j] : fmaf(b, si[j], wi[j]);
                const float ui = dd[j] * ri[j];
                po[j] = first ? ui : fmaf(b, pi[j], ui);
                xo[j] = first ? a * po[j] : fmaf(a, po[j], xi[j]);
                ro[j] = fmaf(-a, so[j], ri[j]);
                uo[j] = dd[j] * ro[j];
                gacc = fmaf(ro[j], uo[j], gacc);
            }
            reinterpret_cast<float4 *>(s)[q] = make_float4(so[0], so[1], so[2], so[3]);
            reinterpret_cast<float4 *>(p)[q] = make_float4(po[0], po[1], po[2], po[3]);
            reinterpret_cast<float4 *>(x)[q] = make_float4(xo[0], xo[1], xo[2], xo[3]);
            reinterpret_cast<float4 *>(r)[q] = make_float4(ro[0], ro[1], ro[2], ro[3]);
        }
        reinterpret_cast<float4 *>(u)[q] = make_float4(uo[0], uo[1], uo[2], uo[3]);
    }
    // tail (n not a multiple of 4): block 0
    if (blockIdx.x == 0) {
        for (long long c = 4 * n4 + threadIdx.x; c < n; c += blockDim.x) {
            const float dd = UNI ? dinv_of(c) : d[c], ri = r[c];
            float ro, uo;
            if (INIT) {
                ro = ri;
                uo = dd * ri;
            } else {
                const float wi = w[c];
                const float so = first ? wi : fmaf(b, s[c], wi);
                const float ui = dd * ri;
                const float po = first ? ui : fmaf(b, p[c], ui);
                x[c] = first ? a * po : fmaf(a, po, x[c]);
                ro = fmaf(-a, so, ri);
                uo = dd * ro;
                s[c] = so;
                p[c] = po;
                r[c] = ro;
            }
            u[c] = uo;
            gacc = fmaf(ro, uo, gacc);
        }
    }
}

// Phase S on one brick: stage u (and material codes) with a one-cell halo,
// then w = A u and delta += w.u on own cells.
template <bool UNI>
__device__ __forceinline__ void cg2_brick(const FilmC &F, const CgBuf &B, const uint32_t *__restrict__ code,
                                          int x0, int y0, int z0, int z1, float &dacc, float *sUb,
                                          uint32_t *sCb, const float *sEps)
{
    const int nx = F.nx, ny = F.ny, nz = F.nz, plane = F.plane;
    const int bx = threadIdx.x % PBX, by = threadIdx.x / PBX;
    const int wx = min(TX, nx - x0), wy = min(TY, ny - y0);
    const bool own = bx >= 1 && bx <= wx && by >= 1 && by <= wy;
    const bool ex = bx == 0 || bx == wx + 1, ey = by == 0 || by == wy + 1;
    const bool need = bx <= wx + 1 && by <= wy + 1 && !(ex && ey);
    const int gx = (x0 - 1 + bx + nx) % nx, gy = (y0 - 1 + by + ny) % ny;
    const int pl = gx + nx * gy;
    const float *__restrict__ u = B.r[1] + F.off;
    float *__restrict__ w = B.w[0] + F.off;
    constexpr int PP = PBY * PBX;
    const int col = by * PBX + bx;
    if (need) {
        const int klo = own ? max(z0 - 1, 0) : z0;
        const int khi = own ? min(z1, nz - 1) : z1 - 1;
        for (int k = klo; k <= khi; ++k) {
            const int o = pl + k * plane;
            const int si = (k - z0 + 1) * PP + col;
            cp_async4(sUb + si, u + o);
            if (!UNI) cp_async4(sCb + si, code + o);
        }
    }
    cp_async_wait_all();
    __syncthreads();
    if (own) {
        for (int k = z0; k < z1; ++k) {
            const int zi = k - z0 + 1;
            const int si = zi * PP + col;
            const float uc = sUb[si];
            float wv;
            if (id_row(F, k, pl)) {
                wv = uc;
            } else {
                int zu = zi + 1, zd = zi - 1;
                if (F.zbc != 0) {
                    if (k == 0) zd = zu;
                    else if (k == nz - 1) zu = zd;
                }
                const int su = zu * PP + col, sd = zd * PP + col;
                const float ue = sUb[si + 1], uw = sUb[si - 1], un = sUb[si + PBX], us = sUb[si - PBX];
                const float uu = sUb[su], ud = sUb[sd];
                float a;
                if (UNI) {
                    a = sEps[0] * ((((((ue - uc) - (uc - uw)) + (un - uc)) - (uc - us)) + (uu - uc)) - (uc - ud));
                } else {
                    const int mc = code_mat(sCb[si]) * 3;
                    a = sEps[mc + code_mat(sCb[si + 1])] * (ue - uc) - sEps[mc + code_mat(sCb[si - 1])] * (uc - uw);
                    a += sEps[mc + code_mat(sCb[si + PBX])] * (un - uc);
                    a -= sEps[mc + code_mat(sCb[si - PBX])] * (uc - us);
                    a += sEps[mc + code_mat(sCb[su])] * (uu - uc);
                    a -= sEps[mc + code_mat(sCb[sd])] * (uc - ud);
                }
                wv = -(a * F.inv_h2);
            }
            w[pl + k * plane] = wv;
            dacc = fmaf(wv, uc, dacc);
        }
    }
    __syncthreads();
}

template <bool UNI>
__device__ __forceinline__ void cg2_stencil(const Dev &d, const FilmC &F, const CgBuf &B, float &dacc,
                                            float *sUb, uint32_t *sCb, const float *sEps)
{
    const uint32_t *code = d.code + F.off;
    for (int i = blockIdx.x; i < B.n_bricks; i += gridDim.x) {
        const int4 it = B.bricks[i];
        cg2_brick<UNI>(F, B, code, it.y, it.z, it.w & 0xffff, it.w >> 16, dacc, sUb, sCb, sEps);
    }
}

constexpr size_t P2SMEM_BYTES = sizeof(float) * 2 * PNPL;

template <bool UNI>
__global__ void __launch_bounds__(PNT, 2) k_pcg_cg2(Dev d, CgBuf B, const float *dinv)
{
    extern __shared__ float4 dsm4[];
    float *sUb = (float *)dsm4;
    uint32_t *sCb = (uint32_t *)(sUb + PNPL);
    __shared__ double sRed[PNW][2];
    __shared__ float sEps[9];
    __shared__ float s_ab[2];
    __shared__ int s_go;
    const FilmDev *f = d.films;
    SolveDev *S = d.solve;
    const bool run = f->dep_flag != 0 && *(volatile int *)&S->active != 0;
    if (!run) return;
    FilmC F;
    F.nx = f->nx; F.ny = f->ny; F.nz = f->nz; F.zbc = f->zbc; F.ref_id = f->ref_id;
    F.plane = f->nx * f->ny; F.off = f->off; F.inv_h2 = f->inv_h2f; F.dinv_uni = f->dinv_uni;
    const long long n = (long long)F.plane * F.nz;
    if (threadIdx.x < 9) sEps[threadIdx.x] = f->epsf32[threadIdx.x];
    __syncthreads();
    const double tol2 = S->inner_tol2;
    const int imax = S->inner_max;
    unsigned int target = 0;
    float ga = 0.f, da = 0.f;
    cg2_point<true, UNI>(F, B, dinv, n, true, 0.f, 0.f, ga);
    if (!grid_sync(B, target)) return;
    cg2_stencil<UNI>(d, F, B, da, sUb, sCb, sEps);
    double g0, dl;
    if (!grid_allreduce2(B, 0, target, ga, da, sRed, g0, dl)) return;
    double gam = g0, alpha = (dl > 0.0) ? g0 / dl : 0.0;
    int it = 0, status = 0;
    if (threadIdx.x == 0) {
        s_go = isfinite(g0) && g0 > 0.0 && dl > 0.0 && gam > tol2 * g0 && imax > 0;
        if (!(isfinite(g0) && g0 > 0.0 && dl > 0.0)) status = (g0 == 0.0) ? 0 : 1;
        s_ab[0] = (float)alpha;
        s_ab[1] = 0.f;
    }
    __syncthreads();
    while (s_go) {
        const float a = s_ab[0], b = s_ab[1];
        ga = 0.f; da = 0.f;
        cg2_point<false, UNI>(F, B, dinv, n, it == 0, a, b, ga);
        if (!grid_sync(B, target)) return;
        cg2_stencil<UNI>(d, F, B, da, sUb, sCb, sEps);
        double gn, dn;
        if (!grid_allreduce2(B, (it + 1) & 1, target, ga, da, sRed, gn, dn)) return;
        ++it;
        if (threadIdx.x == 0) {
            const int go = cg_scalars(gn, dn, gam, alpha, s_ab, status);
            s_go = go && gam > tol2 * g0 && it < imax;
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S->iters = it;
        S->total_iters += it;
        S->rz = gam;
        S->rz0 = g0;
        S->active = 0;
        if (status) { S->status = 1; S->outer_active = 0; }
    }
}

}  // namespace cmsl
