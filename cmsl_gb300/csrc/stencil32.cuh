// stencil32.cuh -- the CMSL_FP32_REFINED stencil passes: the TDGL step and
// the double-float residual pass of the depolarisation solve.
//
// Same work items as the FP64 kernels (a TX x TY column tile of one film
// marching through z0..z1), but every plane of every field a pass reads is
// brought into a ring of NS shared-memory stages by cp.async copies, NS-3
// planes ahead of the plane being computed.  The z neighbours are read from
// the ring as well, so a thread carries no plane-to-plane state beyond its
// partial sums, several blocks share an SM, and each plane costs one barrier.
//
// Each thread owns one cell of the tile and copies it (4 bytes per field)
// and at most one x/y halo cell.  (Pair tiles -- two x-adjacent cells per
// thread with 8-byte copies -- execute a third fewer instructions but halve
// the warps an SM holds within the same shared memory, and measured slower.)
//
// Ring protocol (identical in both kernels): planes zlo = max(z0-1, 0) ..
// zhi = min(z1, nz-1) are staged, plane p in stage (p - zlo) % NS, one
// commit group per plane (empty groups keep the count uniform across
// threads).  Before computing plane k a thread waits until plane k+1 has
// landed (NS-4 younger groups may still be in flight), the block syncs --
// which also retires every read of plane k-2 -- and plane k+NS-2 is issued
// into that stage.
#pragma once
#include "kernels.cuh"

namespace cmsl {

constexpr int TR32 = 12;     // FP32 rotation per grain: 9 values + 3 pad (three 16-byte loads)

// Warm start of a step's first refinement pass (own cell): 0 the previous
// potential a, 1 linear 2a - q, 2 quadratic 3(a - q) + u, 3 cubic
// 4(a + u) - 6q - v, with a, q, u, v the potentials of steps n .. n-3.
__device__ __forceinline__ df extrap_phi(int warm, df a, df q, df u, df v)
{
    if (warm == 1) return df_sub(df{2.f * a.h, 2.f * a.l}, q);
    if (warm == 2) return df_add(df_mul_f(df_sub(a, q), 3.f), u);
    if (warm == 3) return df_sub(df_sub(df_mul_f(df_add(a, u), 4.f), df_mul_f(q, 6.f)), v);
    return a;
}

// The free one of the five potential buffers of film S.
__device__ __forceinline__ int phi_free(const SolveDev *S)
{
    return 10 - S->phi_cur - S->phi_prev - S->phi_prev2 - S->phi_prev3;
}

// ------------------------------------------------------------ TDGL step
// kernelCalc_antiferro (kernels_evol.cu:47-231) with E_dep of the current
// potential (depol_varEPS.cu:223-276) and the sweep-row sums
// (evolve.cu:256-357) in FP32, plus the warm start of the coming solve:
// the extrapolated potential is written to the film's free buffer, which the
// step's first residual pass then reads.

// Coefficients of one (material, interface) class as three float4:
// (relax, A, LdT, ag), (ags, b4, b12, g6), (a02, -, -, -).
__device__ __forceinline__ void load_coef4(const FilmDev *f, float4 (*sC)[3])
{
    if (threadIdx.x < 6) {
        const Coef<float> &c = f->coef32[threadIdx.x];
        sC[threadIdx.x][0] = make_float4(c.relax, c.A, c.LdT, c.ag);
        sC[threadIdx.x][1] = make_float4(c.ags, c.b4, c.b12, c.g6);
        sC[threadIdx.x][2] = make_float4(c.a02, 0.f, 0.f, 0.f);
    }
}

// One cell: P^{n+1} (pn) from P^n (pc), the 6-neighbour sums, -E (ex, ey, ez)
// and -Ez_applied (mEz); pMZl, pSZl (crystal frame) for the sweep rows.
__device__ __forceinline__ void tdgl_cell32(const float4 *K, const float4 *tr, const float (&pc)[6],
                                            const float (&sum)[6], float ex, float ey, float ez, float mEz,
                                            float (&pn)[6], float &pMZl, float &pSZl)
{
    const float4 t0 = __ldg(tr), t1 = __ldg(tr + 1), t2 = __ldg(tr + 2);
    const float t[9] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w, t2.x};
    const float4 ka = K[0], kb = K[1], kc = K[2];
    const float relax = ka.x, A = ka.y, LdT = ka.z, ag = ka.w, ags = kb.x, b4 = kb.y, b12 = kb.z, g6 = kb.w;
    const float a02 = kc.x;
    // crystal frame (kernels_evol.cu:162-168)
    const float pMXl = t[0] * pc[0] + t[1] * pc[1] + t[2] * pc[2];
    const float pMYl = t[3] * pc[0] + t[4] * pc[1] + t[5] * pc[2];
    pMZl = t[6] * pc[0] + t[7] * pc[1] + t[8] * pc[2];
    const float pSXl = t[0] * pc[3] + t[1] * pc[4] + t[2] * pc[5];
    const float pSYl = t[3] * pc[3] + t[4] * pc[4] + t[5] * pc[5];
    pSZl = t[6] * pc[3] + t[7] * pc[4] + t[8] * pc[5];
    // two-sublattice Landau derivative (kernels_evol.cu:178-199)
    const float dmx = a02 * pMXl, dmy = a02 * pMYl;
    const float dsx = a02 * pSXl, dsy = a02 * pSYl;
    const float m2 = pMZl * pMZl, m3 = m2 * pMZl, m4 = m3 * pMZl, m5 = m4 * pMZl;
    const float q2 = pSZl * pSZl, q3 = q2 * pSZl, q4 = q3 * pSZl, q5 = q4 * pSZl;
    float dmz = ag * pMZl + b4 * m3;
    dmz = dmz + b12 * pMZl * q2;
    dmz = dmz + g6 * (m5 + 10.f * m3 * q2 + 5.f * pMZl * q4);
    float dsz = ags * pSZl + b4 * q3;
    dsz = dsz + b12 * pSZl * m2;
    dsz = dsz + g6 * (q5 + 10.f * m2 * q3 + 5.f * pSZl * m4);
    // back to the lab frame (kernels_evol.cu:202-208) + fields (:210-220)
    float b[6];
    b[0] = t[0] * dmx + t[3] * dmy + t[6] * dmz + ex;
    b[1] = t[1] * dmx + t[4] * dmy + t[7] * dmz + ey;
    b[2] = t[2] * dmx + t[5] * dmy + t[8] * dmz + (mEz + ez);
    b[3] = t[0] * dsx + t[3] * dsy + t[6] * dsz;
    b[4] = t[1] * dsx + t[4] * dsy + t[7] * dsz;
    b[5] = t[2] * dsx + t[5] * dsy + t[8] * dsz;
    // explicit Euler with the 6-neighbour Laplacian (kernels_evol.cu:223-229)
    #pragma unroll
    for (int q = 0; q < 6; ++q) pn[q] = pc[q] * relax + A * sum[q] - LdT * b[q];
}

// z neighbours of the potential for E (depol_varEPS.cu:246-273): zero beyond
// the Dirichlet planes, mirrored for the Neumann boundary.
__device__ __forceinline__ void efield_z(const FilmDev *f, int k, df fu, df fd, df &pu, df &pd)
{
    if (f->zbc == 0) {
        pu = (k == f->nz - 1) ? df{0.f, 0.f} : fu;
        pd = (k == 0) ? df{0.f, 0.f} : fd;
    } else {
        op_z<df>(f, k, fu, fd, pu, pd);
    }
}

__device__ __forceinline__ void row_acc(float (&acc)[7], int mat, const float (&pn)[6], float pMZl, float pSZl)
{
    acc[0] += pn[2];
    acc[1] += pn[5];
    acc[2] += pMZl;
    acc[3] += pSZl;
    acc[4] += (mat == 1) ? pn[2] : 0.f;
    acc[5] += (mat == 0) ? pn[2] : 0.f;
    acc[6] += (mat == 2) ? pn[2] : 0.f;
}

constexpr int T32_NS = 4;
constexpr int T32_STAGE = 8 * SPL + NT;      // floats: P[6], phi hi, phi lo (own + halo); code (own)
constexpr size_t T32_SMEM = sizeof(float) * T32_NS * T32_STAGE;

template <int NS>
__global__ void __launch_bounds__(NT, 4) k_tdgl32(Dev d, Fields<float> F)
{
    static_assert(NS >= 4, "the ring holds planes k-1, k, k+1 and at least one in flight");
    extern __shared__ float4 smem_t32[];
    float *ring = (float *)smem_t32;
    __shared__ float4 sC[6][3];
    __shared__ double sRed[NT / 32][7];
    __shared__ double sTot[7];
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    load_coef4(f, sC);
    const Geom g = make_geom(f, it.y, it.z);
    const int cur = d.ctl->cur, rs = d.ctl->run_step;
    const float mEz = (float)(-d.wave[(long long)it.x * d.wstride + rs]);   // dfdPmz_app, kernels_evol.cu:210
    const int row = d.rows[(long long)it.x * d.wstride + rs];
    const int dep = f->dep_flag, nz = g.nz;
    const long long off = f->off, lo = d.ncells;
    const SolveDev *S = d.solve + it.x;
    const float *ph = (const float *)phi_sel(d, S->phi_cur) + off;
    const float *qh = (const float *)phi_sel(d, S->phi_prev) + off;
    const float *uh = (const float *)phi_sel(d, S->phi_prev2) + off;
    const float *vh = (const float *)phi_sel(d, S->phi_prev3) + off;
    float *nh = (float *)phi_sel(d, phi_free(S)) + off;
    const int warm = f->warm;
    const uint32_t *code = d.code + off;
    const float4 *TR4 = (const float4 *)(F.TR + (long long)TR32 * f->g_off);
    const float inv_2hf = f->inv_2hf;
    const int zlo = max(z0 - 1, 0), zhi = min(z1, nz - 1);

    auto Pold = [&](int q) { return (cur ? F.P[1][q] : F.P[0][q]) + off; };
    auto stage = [&](int p) { return ring + ((p - zlo) % NS) * T32_STAGE; };
    auto issue = [&](int p) {
        if (p <= zhi) {
            float *st = stage(p);
            const long long pp = (long long)p * g.plane;
            if (g.valid) {
                const long long o = g.own_pl + pp;
                #pragma unroll
                for (int q = 0; q < 6; ++q) cp4(st + q * SPL + g.own_slot, Pold(q) + o);
                if (dep) {
                    cp4(st + 6 * SPL + g.own_slot, ph + o);
                    cp4(st + 7 * SPL + g.own_slot, ph + lo + o);
                }
                cp4(st + 8 * SPL + threadIdx.x, code + o);
            }
            if (g.halo) {
                const long long o = g.halo_pl + pp;
                #pragma unroll
                for (int q = 0; q < 6; ++q) cp4(st + q * SPL + g.halo_slot, Pold(q) + o);
                if (dep) {
                    cp4(st + 6 * SPL + g.halo_slot, ph + o);
                    cp4(st + 7 * SPL + g.halo_slot, ph + lo + o);
                }
            }
        }
        cp_commit();
    };
    for (int p = zlo; p <= z0 + NS - 3; ++p) issue(p);

    float acc[7];
    #pragma unroll
    for (int q = 0; q < 7; ++q) acc[q] = 0.f;
    const int s0 = g.own_slot;
    for (int k = z0; k < z1; ++k) {
        cp_wait<NS - 4>();
        __syncthreads();
        issue(k + NS - 2);
        if (!g.valid) continue;
        const long long o = g.own_pl + (long long)k * g.plane;
        // older potentials for the warm start (consumed after the step's arithmetic)
        df wq{0.f, 0.f}, wu{0.f, 0.f}, wv{0.f, 0.f};
        if (dep && warm >= 1) wq = df{qh[o], qh[lo + o]};
        if (dep && warm >= 2) wu = df{uh[o], uh[lo + o]};
        if (dep && warm >= 3) wv = df{vh[o], vh[lo + o]};
        const int ku = k == nz - 1 ? k : k + 1, kd = k == 0 ? k : k - 1;
        const float *sk = stage(k), *su = stage(ku), *sd = stage(kd);
        const uint32_t c = ((const uint32_t *)sk)[8 * SPL + threadIdx.x];
        float pc[6], sum[6];
        #pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float *a = sk + q * SPL;
            pc[q] = a[s0];
            // neighbour sums e, w, n, s, u, d (kernels_evol.cu:101-122); z clamped
            float sm = a[s0 + 1] + a[s0 - 1];
            sm = sm + a[s0 + SX];
            sm = sm + a[s0 - SX];
            sm = sm + su[q * SPL + s0];
            sum[q] = sm + sd[q * SPL + s0];
        }
        float ex = 0.f, ey = 0.f, ez = 0.f;
        df a0{0.f, 0.f};
        if (dep) {
            const float *fh = sk + 6 * SPL, *fl = sk + 7 * SPL;
            a0 = df{fh[s0], fl[s0]};
            df pu, pd;
            efield_z(f, k, df{su[6 * SPL + s0], su[7 * SPL + s0]}, df{sd[6 * SPL + s0], sd[7 * SPL + s0]}, pu, pd);
            // -1 * E with E = -(phi_+ - phi_-) / (2h)
            ex = phi_diff(df{fh[s0 + 1], fl[s0 + 1]}, df{fh[s0 - 1], fl[s0 - 1]}) * inv_2hf;
            ey = phi_diff(df{fh[s0 + SX], fl[s0 + SX]}, df{fh[s0 - SX], fl[s0 - SX]}) * inv_2hf;
            ez = phi_diff(pu, pd) * inv_2hf;
        }
        float pn[6], pMZl, pSZl;
        tdgl_cell32(sC[code_mat(c) * 2 + code_iface(c)], TR4 + 3LL * code_gid(c), pc, sum, ex, ey, ez, mEz, pn,
                    pMZl, pSZl);
        #pragma unroll
        for (int q = 0; q < 6; ++q) (cur ? F.P[0][q] : F.P[1][q])[off + o] = pn[q];
        if (row >= 0) row_acc(acc, code_mat(c), pn, pMZl, pSZl);
        if (dep) {
            const df w = extrap_phi(warm, a0, wq, wu, wv);
            nh[o] = w.h;
            nh[lo + o] = w.l;
        }
    }
    cp_wait<0>();

    if (row >= 0) {
        double tot[7];
        block_sum<7, float>(acc, sRed, tot);
        if (threadIdx.x == 0) {
            #pragma unroll
            for (int q = 0; q < 7; ++q) d.partial[(long long)blockIdx.x * NPART + q] = tot[q];
        }
    }
    if (!ticket_last(d.counter)) return;
    tdgl_finish(d, rs, sRed, sTot);
}

// Warm start alone (own cells): the free buffer of every depolarised film
// gets the extrapolated potential.  Used before a solve that does not follow
// a TDGL step (cmsl_film_depol).
static __global__ void __launch_bounds__(NT) k_extrap(Dev d)
{
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    if (!f->dep_flag || !g.valid) return;
    const SolveDev *S = d.solve + it.x;
    const long long off = f->off, lo = d.ncells;
    const float *ph = (const float *)phi_sel(d, S->phi_cur) + off;
    const float *qh = (const float *)phi_sel(d, S->phi_prev) + off;
    const float *uh = (const float *)phi_sel(d, S->phi_prev2) + off;
    const float *vh = (const float *)phi_sel(d, S->phi_prev3) + off;
    float *nh = (float *)phi_sel(d, phi_free(S)) + off;
    for (int k = z0; k < z1; ++k) {
        const long long o = g.own_pl + (long long)k * g.plane;
        const df w = extrap_phi(f->warm, df{ph[o], ph[lo + o]}, df{qh[o], qh[lo + o]}, df{uh[o], uh[lo + o]},
                                df{vh[o], vh[lo + o]});
        nh[o] = w.h;
        nh[lo + o] = w.l;
    }
}

// ------------------------------------------------- double-float residual
// One refinement pass of CMSL_FP32_REFINED's depolarisation solve: with x the
// potential -- on a step's first pass the warm start in the free buffer, on
// later passes the current potential plus the pending FP32 correction dx of
// the inner solve, written to the free buffer -- form b = -eps_0_nd div Pm
// (depol_varEPS.cu:279-329, zero on the Dirichlet planes / Neumann pin) and
// r = b - A x in double-float, and the partial sums r.r, b.b, r.D^-1.r.
// x = phi + dx is formed in double-float at every stencil point (dx can be
// as large as phi itself, e.g. the first solve after a cold start).  UNI:
// every material has the same eps, the operator is eps/h^2 times the 7-point
// Laplacian (one double-float product per cell, no material codes).
// An update pass (after the direct solve, once ||r|| <= 1e-4 ||b||) instead
// forms r <- r - A dx in FP32: dx is then small, and the FP32 rounding of
// A dx stays far below the refinement target.
// No FP64 instruction is executed.
constexpr int R32_NS = 5;

// sum of six double-float values minus 6 c; the hi parts are summed error-free
__device__ __forceinline__ df lap7(df e, df w, df n, df s, df u, df dn, df c)
{
    df t = two_sum(e.h, w.h);
    float l = t.l + (e.l + w.l);
    df t2 = two_sum(t.h, n.h);
    l += t2.l + n.l;
    t = two_sum(t2.h, s.h);
    l += t.l + s.l;
    t2 = two_sum(t.h, u.h);
    l += t2.l + u.l;
    t = two_sum(t2.h, dn.h);
    l += t.l + dn.l;
    const df p = two_prod(c.h, -6.f);
    l += fmaf(c.l, -6.f, p.l);
    t2 = two_sum(t.h, p.h);
    l += t2.l;
    return fast_two_sum(t2.h, l);
}

// (a - b) + (c - e) + (g - h) of FP32 values as double-float (hi parts error-free)
__device__ __forceinline__ df div3(float a, float b, float c, float e, float g, float h)
{
    const df x = two_sum(a, -b), y = two_sum(c, -e), z = two_sum(g, -h);
    const df s = two_sum(x.h, y.h);
    float l = s.l + (x.l + y.l);
    const df s2 = two_sum(s.h, z.h);
    l += s2.l + z.l;
    return fast_two_sum(s2.h, l);
}

// The neighbourhood of one cell as a residual pass sees it.
struct RCell {
    df xc, xe, xw, xn, xs, xu, xd;          // x = phi + dx (z neighbours as loaded, k+1 / k-1 clamped)
    float dc, de, dw, dn, ds, du, dd;        // pending correction (update passes)
    float pxe, pxw, pyn, pys, pzu, pzd;      // Pm for the divergence (z clamped)
    int mc, me, mw, mn, ms, mu, md;          // materials (general eps only)
};

// -A dx of one non-identity row in FP32 (dx: the pending correction).
template <bool UNI>
__device__ __forceinline__ float minus_adx(const FilmDev *f, int k, const RCell &c)
{
    float du, ddn;
    op_z<float>(f, k, c.du, c.dd, du, ddn);
    if (UNI) return f->cf_h[0] * ((c.de + c.dw) + (c.dn + c.ds) + (du + ddn) - 6.f * c.dc);
    int mu, md;
    op_z<int>(f, k, c.mu, c.md, mu, md);
    const float *ch = f->cf_h + c.mc * 3;
    return ch[c.me] * (c.de - c.dc) - ch[c.mw] * (c.dc - c.dw) + ch[c.mn] * (c.dn - c.dc) -
           ch[c.ms] * (c.dc - c.ds) + ch[mu] * (du - c.dc) - ch[md] * (c.dc - ddn);
}

// r (FP32 value of b - A x, double-float arithmetic) and b.h of one non-identity row.
template <bool UNI>
__device__ __forceinline__ void refine_row(const FilmDev *f, int k, const RCell &c, float &rv, float &bh)
{
    const df cb{f->cb_h, f->cb_l};
    const df bm = df_mul(div3(c.pxe, c.pxw, c.pyn, c.pys, c.pzu, c.pzd), cb);   // -b
    df xu, xd;
    op_z<df>(f, k, c.xu, c.xd, xu, xd);
    df s;            // b - A phi
    if (UNI) {
        const df cu{f->cf_h[0], f->cf_l[0]};   // eps/h^2 on every face
        s = df_sub(df_mul(cu, lap7(c.xe, c.xw, c.xn, c.xs, xu, xd, c.xc)), bm);
    } else {
        int mu, md;
        op_z<int>(f, k, c.mu, c.md, mu, md);
        const int m3 = c.mc * 3;
        auto cf = [&](int i) { return df{f->cf_h[m3 + i], f->cf_l[m3 + i]}; };
        df a = df_sub(df_mul(cf(c.me), df_sub(c.xe, c.xc)), df_mul(cf(c.mw), df_sub(c.xc, c.xw)));
        a = df_add(a, df_mul(cf(c.mn), df_sub(c.xn, c.xc)));
        a = df_sub(a, df_mul(cf(c.ms), df_sub(c.xc, c.xs)));
        a = df_add(a, df_mul(cf(mu), df_sub(xu, c.xc)));
        a = df_sub(a, df_mul(cf(md), df_sub(c.xc, xd)));
        s = df_sub(a, bm);
    }
    rv = s.h + s.l;
    bh = -bm.h;
}

// The last part of a residual pass of one cell: r and the partial sums.
// upd: r = r_old - A dx (b.b is not formed); otherwise r = b - A x.
template <bool UNI>
__device__ __forceinline__ void refine_cell(const FilmDev *f, int k, bool ident, bool upd, const RCell &c,
                                            float r_old, float dinv, float &rv, float (&acc)[3])
{
    float bh = 0.f, wj = 1.f;
    if (ident) {
        rv = -(c.xc.h + c.xc.l);              // x - g with g = 0, b = 0
    } else {
        if (upd) rv = r_old + minus_adx<UNI>(f, k, c);
        else refine_row<UNI>(f, k, c, rv, bh);
        wj = UNI ? f->dinv_uni : dinv;
    }
    acc[0] = fmaf(rv, rv, acc[0]);
    acc[1] = fmaf(bh, bh, acc[1]);
    acc[2] = fmaf(rv, rv * wj, acc[2]);
}

// Common set-up of a residual pass.
struct RefineSrc {
    const float *xh, *dx, *Pmx, *Pmy, *Pmz, *dinv;
    const uint32_t *code;
    float *nh, *r;
    long long lo;
    bool run, apply, upd;
};

__device__ __forceinline__ RefineSrc refine_src(const Dev &d, const Fields<float> &F, const FilmDev *f,
                                                const SolveDev *S)
{
    RefineSrc q;
    q.run = f->dep_flag != 0 && (d.force || S->outer_active);
    q.apply = S->refine > 0;     // later pass: x = phi + dx; first pass: x = the warm start
    q.upd = q.apply && S->upd && f->upd_ok;   // r <- r - A dx
    const int cur = d.ctl->cur, fr = phi_free(S);
    const long long off = f->off;
    q.lo = d.ncells;
    q.xh = (const float *)phi_sel(d, q.apply ? S->phi_cur : fr) + off;
    q.nh = (float *)phi_sel(d, fr) + off;
    q.dx = F.x + off;
    q.Pmx = (cur ? F.P[0][0] : F.P[1][0]) + off;
    q.Pmy = (cur ? F.P[0][1] : F.P[1][1]) + off;
    q.Pmz = (cur ? F.P[0][2] : F.P[1][2]) + off;
    q.code = d.code + off;
    q.dinv = F.dinv + off;
    q.r = F.r + off;
    return q;
}

__device__ __forceinline__ void refine_partials(const Dev &d, float (&acc)[3], double (*sRed)[3])
{
    double t[3];
    block_sum<3, float>(acc, sRed, t);
    if (threadIdx.x == 0) {
        d.partial[(long long)blockIdx.x * NPART + 0] = t[0];
        d.partial[(long long)blockIdx.x * NPART + 1] = t[1];
        d.partial[(long long)blockIdx.x * NPART + 2] = t[2];
    }
}

template <bool UNI> struct R32Lay {
    static constexpr int FH = 0, FL = SPL, DX = 2 * SPL, PX = 3 * SPL, PY = 4 * SPL, PZ = 5 * SPL;
    static constexpr int CODE = 5 * SPL + NT, DINV = 6 * SPL + NT;   // general eps only
    static constexpr int STAGE = UNI ? 5 * SPL + NT : 6 * SPL + 2 * NT;
};
template <bool UNI> constexpr size_t r32_smem() { return sizeof(float) * R32_NS * R32Lay<UNI>::STAGE; }

template <bool UNI, int NS>
__global__ void __launch_bounds__(NT, 4) k_refine32(Dev d, Fields<float> F)
{
    static_assert(NS >= 4, "the ring holds planes k-1, k, k+1 and at least one in flight");
    using L = R32Lay<UNI>;
    extern __shared__ float4 smem_r32[];
    float *ring = (float *)smem_r32;
    __shared__ double sRed[NT / 32][3];
    __shared__ double sTot[3];
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    const int nz = g.nz;
    const RefineSrc q = refine_src(d, F, f, d.solve + it.x);
    const long long lo = q.lo;
    const bool apply = q.apply, upd = UNI && q.upd;   // update passes follow the direct solve (one eps)
    const int zlo = max(z0 - 1, 0), zhi = min(z1, nz - 1);

    auto stage = [&](int p) { return ring + ((p - zlo) % NS) * L::STAGE; };
    auto issue = [&](int p) {
        if (q.run && p <= zhi && upd) {
            // update pass: dx with its halo; phi and the old r of the own cell
            float *st = stage(p);
            const long long pp = (long long)p * g.plane;
            if (g.valid) {
                const long long o = g.own_pl + pp;
                const int s = g.own_slot;
                cp4(st + L::FH + s, q.xh + o);
                cp4(st + L::FL + s, q.xh + lo + o);
                cp4(st + L::DX + s, q.dx + o);
                cp4(st + L::PX + s, q.r + o);
                if (!UNI) {
                    cp4(st + L::CODE + s, q.code + o);
                    cp4(st + L::DINV + threadIdx.x, q.dinv + o);
                }
            }
            if (g.halo) {
                const long long o = g.halo_pl + pp;
                const int s = g.halo_slot;
                cp4(st + L::DX + s, q.dx + o);
                if (!UNI) cp4(st + L::CODE + s, q.code + o);
            }
        } else if (q.run && p <= zhi) {
            float *st = stage(p);
            const long long pp = (long long)p * g.plane;
            if (g.valid) {
                const long long o = g.own_pl + pp;
                const int s = g.own_slot;
                cp4(st + L::FH + s, q.xh + o);
                cp4(st + L::FL + s, q.xh + lo + o);
                if (apply) cp4(st + L::DX + s, q.dx + o);
                cp4(st + L::PX + s, q.Pmx + o);
                cp4(st + L::PY + s, q.Pmy + o);
                cp4(st + L::PZ + threadIdx.x, q.Pmz + o);
                if (!UNI) {
                    cp4(st + L::CODE + s, q.code + o);
                    cp4(st + L::DINV + threadIdx.x, q.dinv + o);
                }
            }
            if (g.halo) {
                const long long o = g.halo_pl + pp;
                const int s = g.halo_slot;
                cp4(st + L::FH + s, q.xh + o);
                cp4(st + L::FL + s, q.xh + lo + o);
                if (apply) cp4(st + L::DX + s, q.dx + o);
                cp4(st + L::PX + s, q.Pmx + o);
                cp4(st + L::PY + s, q.Pmy + o);
                if (!UNI) cp4(st + L::CODE + s, q.code + o);
            }
        }
        cp_commit();
    };
    for (int p = zlo; p <= z0 + NS - 3; ++p) issue(p);

    const int s0 = g.own_slot, tz = threadIdx.x;
    float acc[3] = {0.f, 0.f, 0.f};
    for (int k = z0; k < z1; ++k) {
        cp_wait<NS - 4>();
        __syncthreads();
        issue(k + NS - 2);
        if (!q.run || !g.valid) continue;
        const long long o = g.own_pl + (long long)k * g.plane;
        const int ku = k == nz - 1 ? k : k + 1, kd = k == 0 ? k : k - 1;
        const float *sk = stage(k), *su = stage(ku), *sd = stage(kd);
        auto D = [&](const float *st, int s) { return st[L::DX + s]; };
        auto X = [&](const float *st, int s) {        // x = phi (+ dx on later passes)
            const df p{st[L::FH + s], st[L::FL + s]};
            return apply ? df_add_f(p, D(st, s)) : p;
        };
        auto M = [&](const float *st, int s) { return UNI ? 0 : code_mat(((const uint32_t *)st)[L::CODE + s]); };
        RCell c;
        c.xc = X(sk, s0);
        c.mc = M(sk, s0); c.me = M(sk, s0 + 1); c.mw = M(sk, s0 - 1); c.mn = M(sk, s0 + SX); c.ms = M(sk, s0 - SX);
        c.mu = M(su, s0); c.md = M(sd, s0);
        if (upd) {
            c.dc = D(sk, s0); c.de = D(sk, s0 + 1); c.dw = D(sk, s0 - 1); c.dn = D(sk, s0 + SX);
            c.ds = D(sk, s0 - SX); c.du = D(su, s0); c.dd = D(sd, s0);
        } else {
            c.xe = X(sk, s0 + 1); c.xw = X(sk, s0 - 1); c.xn = X(sk, s0 + SX); c.xs = X(sk, s0 - SX);
            c.xu = X(su, s0); c.xd = X(sd, s0);
            c.pxe = sk[L::PX + s0 + 1]; c.pxw = sk[L::PX + s0 - 1];
            c.pyn = sk[L::PY + s0 + SX]; c.pys = sk[L::PY + s0 - SX];
            c.pzu = su[L::PZ + tz]; c.pzd = sd[L::PZ + tz];
        }
        float rv;
        refine_cell<UNI>(f, k, identity_row(f, k, g.own_pl), upd, c, upd ? sk[L::PX + s0] : 0.f,
                         UNI ? 0.f : sk[L::DINV + tz], rv, acc);
        q.r[o] = rv;
        if (apply) {
            q.nh[o] = c.xc.h;
            q.nh[lo + o] = c.xc.l;
        }
    }
    cp_wait<0>();
    refine_partials(d, acc, sRed);
    if (!ticket_last(d.counter)) return;
    refine_finish(d, sRed, sTot);
}

}  // namespace cmsl
