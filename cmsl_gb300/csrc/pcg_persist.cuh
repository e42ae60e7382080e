// pcg_persist.cuh -- persistent single-reduction Jacobi-PCG for the FP32 inner
// solve of CMSL_FP32_REFINED, over one film or a batch of films.
//
// The reference runs textbook PCG with two blocking dot products per
// iteration (depol_varEPS.cu:472-522).  Here the inner solve of each
// refinement pass is one cooperative kernel that stays resident for all its
// iterations.  It uses the Chronopoulos-Gear recurrences, which need a single
// reduction (two dots) per iteration, so every iteration is one sweep over the
// films and one grid all-reduce:
//
//   p_i = u_i + b_i p_{i-1}      s_i = w_i + b_i s_{i-1}
//   x  += a_i p_i                r_{i+1} = r_i - a_i s_i
//   u_{i+1} = D^-1 r_{i+1}       w_{i+1} = A u_{i+1}
//   g_{i+1} = (r_{i+1}, u_{i+1}) d_{i+1} = (w_{i+1}, u_{i+1})
//   b_{i+1} = g_{i+1}/g_i        a_{i+1} = g_{i+1} / (d_{i+1} - b_{i+1} g_{i+1} / a_i)
//
// Batches: every film owns a contiguous range of the grid's blocks (in
// proportion to its cells) and a contiguous range of the stencil bricks, so
// a block works on one film only and its partial sums belong to that film.
// After each all-reduce every block forms every film's totals from that
// film's block range (same order everywhere), so all blocks hold the same
// per-film scalars and convergence flags and take the same loop decisions
// without a second barrier.  A film that has converged (or failed) stops
// working while the others iterate: its blocks only take part in the
// barriers.  The loop ends when no film is active.
//
// Grid barrier: arrival counter + bounded spin (about a second), after which
// the block records a timeout and leaves; no wait is unbounded.
#pragma once
#include "kernels.cuh"

namespace cmsl {

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Spins of a grid-barrier wait before it gives up (x ~100 ns sleeps): the
// default of CgBuf::spin_limit (about 1 s).
constexpr unsigned long long BARRIER_SPIN_LIMIT = 20000000ull;

// Brick geometry of the persistent solver: a block of PBX x PBY threads owns
// the TX x TY column tile plus its one-cell x/y halo; it stages u = D^-1 r for
// PZ planes (+1 above and below) in shared memory, then applies the stencil.
constexpr int PBX = TX + 2;
constexpr int PBY = TY + 2;
constexpr int PNT = PBX * PBY;          // 340 threads
constexpr int PNW = (PNT + 31) / 32;    // 11 warps
constexpr int PZ = 8;
constexpr int PBP = PZ + 2;
constexpr int PNPL = PBP * PBY * PBX;   // staged cells of one brick, all planes

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

// Double-float warp sum (lane 0 holds the result).
__device__ __forceinline__ df warp_sum_df(df v)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const df w{__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
        v = df_add(v, w);
    }
    return v;
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

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
        if ((int)blockIdx.x != B.hold_block) atomicAdd(B.arrive, 1u);
        int ok = 1;
        unsigned long long spins = 0;
        while (ld_acquire(B.arrive) < target) {
            if (++spins > B.spin_limit) { ok = 0; atomicExch(B.err, 1); break; }
            __nanosleep(32);
        }
        s_ok2 = ok;
    }
    __syncthreads();
    return s_ok2 != 0;
}

// Phase P over the film's n cells, shared by its nb blocks (this one is lb).
// INIT: u = D^-1 r, gamma = r.u.  The film's first cell is 16-byte aligned.
template <bool INIT, bool UNI>
__device__ __forceinline__ void cg2_point(const FilmC &F, const CgBuf &B, const float *__restrict__ dv,
                                          long long n, int lb, int nb, bool first, float a, float b,
                                          float &gacc)
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
    const long long stride = (long long)nb * blockDim.x;
    for (long long q = (long long)lb * blockDim.x + threadIdx.x; q < n4; q += stride) {
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
    // tail (n not a multiple of 4): the film's first block
    if (lb == 0) {
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

// Phase S over the bricks [first, end) of the film, stride nb (its blocks).
template <bool UNI>
__device__ __forceinline__ void cg2_stencil(const Dev &d, const FilmC &F, const CgBuf &B, int first, int end,
                                            int nb, float &dacc, float *sUb, uint32_t *sCb, const float *sEps)
{
    const uint32_t *code = d.code + F.off;
    for (int i = first; i < end; i += nb) {
        const int4 it = B.bricks[i];
        cg2_brick<UNI>(F, B, code, it.y, it.z, it.w & 0xffff, it.w >> 16, dacc, sUb, sCb, sEps);
    }
}

constexpr size_t P2SMEM_BYTES = sizeof(float) * 2 * PNPL;

// Films one persistent launch can carry (their scalars live in shared memory
// behind the brick staging area: dynamic size P2SMEM_BYTES + films * 72 B).
constexpr int CG_MAX_FILMS = 128;

// One film's recurrence state; every block holds an identical copy.
struct FilmState {
    double gam, alpha, g0, tol2;
    float a, b;                 // alpha and beta of the film's next iteration
    int it, go, status, imax;
    int pb0, pb1;               // the film's block range
    int ran, pad;
};
static_assert(sizeof(FilmState) % 8 == 0 && P2SMEM_BYTES % 16 == 0, "shared-memory layout of the persistent solver");

// Publishes this block's (gamma, delta) partials, waits for every block, then
// updates every active film's state from the partials of its block range
// (double-float sums, one warp per film).  INIT: the partials are the
// starting (r0,u0) and (w0,u0).  False if the wait timed out.
__device__ __forceinline__ bool grid_allreduce_films(const CgBuf &B, int n_films, int parity, unsigned int &target,
                                                     float v0, float v1, double (*sm)[2], FilmState *st,
                                                     bool init)
{
    __shared__ int s_ok;
    float a[2] = {v0, v1};
    double blk[2];
    block_sum_p<2, float>(a, sm, blk);
    float4 *part = B.part + (size_t)parity * gridDim.x;
    target += gridDim.x;
    if (threadIdx.x == 0) {
        const float h0 = (float)blk[0], h1 = (float)blk[1];
        __stcg(part + blockIdx.x, make_float4(h0, (float)(blk[0] - (double)h0), h1, (float)(blk[1] - (double)h1)));
        __threadfence();
        if ((int)blockIdx.x != B.hold_block) atomicAdd(B.arrive, 1u);
        int ok = 1;
        unsigned long long spins = 0;
        while (ld_acquire(B.arrive) < target) {
            if (++spins > B.spin_limit) { ok = 0; atomicExch(B.err, 1); break; }
            __nanosleep(64);
        }
        s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) return false;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int FULL_WARPS = PNT / 32;
    for (int f = warp; warp < FULL_WARPS && f < n_films; f += FULL_WARPS) {
        FilmState &s = st[f];
        if (!s.go) continue;
        df q0{0.f, 0.f}, q1{0.f, 0.f};
        for (int b = s.pb0 + lane; b < s.pb1; b += 32) {
            const float4 v = __ldcg(part + b);
            q0 = df_add(q0, df{v.x, v.y});
            q1 = df_add(q1, df{v.z, v.w});
        }
        q0 = warp_sum_df(q0);
        q1 = warp_sum_df(q1);
        if (lane == 0) {
            const double tg = (double)q0.h + (double)q0.l, td = (double)q1.h + (double)q1.l;
            if (init) {
                s.g0 = tg;
                s.gam = tg;
                s.alpha = td > 0.0 ? tg / td : 0.0;
                const bool ok = isfinite(tg) && tg > 0.0 && td > 0.0;
                if (!ok) s.status = tg == 0.0 ? 0 : 1;
                s.go = ok && s.gam > s.tol2 * tg && s.imax > 0;
                s.a = (float)s.alpha;
                s.b = 0.f;
            } else {
                s.it += 1;
                const int go = cg_scalars(tg, td, s.gam, s.alpha, &s.a, s.status);
                s.go = go && s.gam > s.tol2 * s.g0 && s.it < s.imax;
            }
        }
    }
    __syncthreads();
    return true;
}

// Single film: publishes this block's partials, waits for every block, and
// returns the grid totals (identical in every block).  False on a timeout.
__device__ __forceinline__ bool grid_allreduce_all(const CgBuf &B, int parity, unsigned int &target, float v0,
                                                   float v1, double (*sm)[2], double &t0, double &t1)
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
        if ((int)blockIdx.x != B.hold_block) atomicAdd(B.arrive, 1u);
        int ok = 1;
        unsigned long long spins = 0;
        while (ld_acquire(B.arrive) < target) {
            if (++spins > B.spin_limit) { ok = 0; atomicExch(B.err, 1); break; }
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

// The inner FP32 solve of one refinement pass for every film whose solve is
// active: starts from r_0 in B.r[0] (written by k_refine32) and x = 0, runs
// until (r,u) <= inner_tol2 (r_0,u_0) or inner_max iterations per film, and
// leaves each film's correction in B.x.  Cooperative launch of PNT-thread
// blocks; every block is co-resident.  MULTI = false is the single-film
// instance: its scalars stay in thread 0's registers (the per-film
// shared-memory state costs about a microsecond per iteration and registers).
template <bool UNI, bool MULTI>
__global__ void __launch_bounds__(PNT, 2) k_pcg_cg2(Dev d, CgBuf B, const float *dinv)
{
    extern __shared__ float4 dsm4[];
    float *sUb = (float *)dsm4;
    uint32_t *sCb = (uint32_t *)(sUb + PNPL);
    __shared__ double sRed[PNW][2];
    __shared__ float sEps[9];
    FilmState *st = reinterpret_cast<FilmState *>(sCb + PNPL);
    const int nf = min(d.n_films, CG_MAX_FILMS);
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
        const FilmDev *ff = d.films + i;
        const SolveDev *S = d.solve + i;
        FilmState s{};
        s.tol2 = S->inner_tol2;
        s.imax = S->inner_max;
        s.go = ff->dep_flag != 0 && *(volatile const int *)&S->active != 0;
        s.ran = s.go;
        s.pb0 = ff->pb_begin;
        s.pb1 = ff->pb_end;
        st[i] = s;
    }
    const int mf = B.blk_film[blockIdx.x];
    const FilmDev *f = d.films + mf;
    FilmC F;
    F.nx = f->nx; F.ny = f->ny; F.nz = f->nz; F.zbc = f->zbc; F.ref_id = f->ref_id;
    F.plane = f->nx * f->ny; F.off = f->off; F.inv_h2 = f->inv_h2f; F.dinv_uni = f->dinv_uni;
    // single film: the whole grid and brick list (special registers and
    // kernel parameters, which cost no registers)
    const int lb = MULTI ? (int)blockIdx.x - f->pb_begin : (int)blockIdx.x;
    const int nb = MULTI ? f->pb_end - f->pb_begin : (int)gridDim.x;
    const int br0 = MULTI ? f->brick_begin + lb : (int)blockIdx.x;
    const int br1 = MULTI ? f->brick_end : B.n_bricks;
    const long long n = (long long)F.plane * F.nz;
    if (threadIdx.x < 9) sEps[threadIdx.x] = f->epsf32[threadIdx.x];
    // uniform in every block: no film active means nothing to do
    if (!__syncthreads_or(threadIdx.x < nf && st[threadIdx.x].go)) return;
    unsigned int target = 0;
    float ga = 0.f, da = 0.f;
    bool on = st[mf].go != 0;
    if (on) cg2_point<true, UNI>(F, B, dinv, n, lb, nb, true, 0.f, 0.f, ga);
    if (!grid_sync(B, target)) return;
    if (on) cg2_stencil<UNI>(d, F, B, br0, br1, nb, da, sUb, sCb, sEps);
    if (!grid_allreduce_films(B, nf, 0, target, ga, da, sRed, st, true)) return;
    if constexpr (!MULTI) {
        __shared__ int s_go;
        __shared__ float s_ab[2];
        double gam = st[0].gam, alpha = st[0].alpha;
        const double stop = st[0].tol2 * st[0].g0;
        const int imax = st[0].imax;
        int it = 0, status = 0;
        if (threadIdx.x == 0) { s_go = st[0].go; s_ab[0] = st[0].a; s_ab[1] = 0.f; }
        __syncthreads();
        while (s_go) {
            const float a = s_ab[0], b = s_ab[1];
            ga = 0.f; da = 0.f;
            cg2_point<false, UNI>(F, B, dinv, n, lb, nb, it == 0, a, b, ga);
            if (!grid_sync(B, target)) return;
            cg2_stencil<UNI>(d, F, B, br0, br1, nb, da, sUb, sCb, sEps);
            double gn, dn;
            if (!grid_allreduce_all(B, (it + 1) & 1, target, ga, da, sRed, gn, dn)) return;
            ++it;
            if (threadIdx.x == 0) {
                const int go = cg_scalars(gn, dn, gam, alpha, s_ab, status);
                s_go = go && gam > stop && it < imax;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            st[0].it = it;
            st[0].gam = gam;
            st[0].status |= status;
        }
        __syncthreads();
    } else {
        int k = 0;
        while (__syncthreads_or(threadIdx.x < nf && st[threadIdx.x].go)) {
            on = st[mf].go != 0;
            ga = 0.f; da = 0.f;
            if (on) cg2_point<false, UNI>(F, B, dinv, n, lb, nb, st[mf].it == 0, st[mf].a, st[mf].b, ga);
            if (!grid_sync(B, target)) return;
            if (on) cg2_stencil<UNI>(d, F, B, br0, br1, nb, da, sUb, sCb, sEps);
            if (!grid_allreduce_films(B, nf, (k + 1) & 1, target, ga, da, sRed, st, false)) return;
            ++k;
        }
    }
    if (lb == 0 && threadIdx.x == 0 && st[mf].ran) {
        const FilmState &s = st[mf];
        SolveDev *S = d.solve + mf;
        S->iters = s.it;
        S->total_iters += s.it;
        S->rz = s.gam;
        S->rz0 = s.g0;
        S->active = 0;
        if (s.status) { S->status = 1; S->outer_active = 0; }
    }
}

}  // namespace cmsl
