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
// FP32 storage (CMSL_FP32_REFINED): P is kept as three float2 arrays per set,
// the pairs (Pmx, Pmy), (Pmz, Psx), (Psy, Psz) (pair j at j * ncells float2
// of the set's allocation), and every double-float potential interleaves its
// (hi, lo) halves per cell; a stencil point of a pair is one 8-byte copy and
// one 8-byte shared load.
//
// Each thread owns one cell of the tile and copies it and at most one x/y
// halo cell.  The tile is TX x TYc columns (TYc 4, 8 or 16: 128, 256 or 512
// threads), the autotuner's choice; the blocks take the stencil item list
// (Dev::sitems) of that tile height.  (Pair tiles -- two x-adjacent cells per thread -- execute a
// third fewer instructions but halve the warps an SM holds within the same
// shared memory, and measured slower.)
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
// 4(a + u) - 6q - v, with a, q, u, v the potentials of steps n .. n-3.  In
// double-float: FP32 rounding noise in the start would be amplified by the
// operator's high-frequency end (~12/h^2) well above the smooth truncation
// error, and the first residual would miss the update pass's 1e-4 ||b||.
__device__ __forceinline__ df extrap_phi(int warm, df a, df q, df u, df v)
{
    if (warm == 1) return df_sub(df{2.f * a.h, 2.f * a.l}, q);
    if (warm == 2) return df_add(df_mul_f(df_sub(a, q), 3.f), u);
    if (warm == 3) return df_sub(df_sub(df_mul_f(df_add(a, u), 4.f), df_mul_f(q, 6.f)), v);
    return a;
}

// The extrapolation order a film's next warm start can take: its warm start
// order, lowered while fewer potentials than it needs are valid (after a
// state upload; a state without a potential starts from zero).
__device__ __forceinline__ int warm_order(const FilmDev *f, const SolveDev *S)
{
    return min(f->warm, max(S->hist - 1, 0));
}

// Difference of two double-float potentials rounded to FP32, for E: the hi
// difference of neighbouring values is exact when they lie within a factor
// of two of each other (Sterbenz) and one FP32 rounding off otherwise; the
// lo difference is added.  E enters the FP32 step, which rounds at that
// level anyway.
__device__ __forceinline__ float phi_diff32(df a, df b) { return (a.h - b.h) + (a.l - b.l); }

// The free one of the five potential buffers of film S.
__device__ __forceinline__ int phi_free(const SolveDev *S)
{
    return 10 - S->phi_cur - S->phi_prev - S->phi_prev2 - S->phi_prev3;
}

// The (hi, lo) pairs of double-float potential buffer i.
__device__ __forceinline__ float2 *phi2_sel(const Dev &d, int i) { return (float2 *)phi_sel(d, i); }
__device__ __forceinline__ df ld_df(const float2 *p)
{
    const float2 v = *p;
    return df{v.x, v.y};
}
// The three P pairs of FP32 set s (pair j at j * ncells).
__device__ __forceinline__ float2 *pairs32(const Fields<float> &F, int s) { return (float2 *)F.P[s][0]; }

// Stage bookkeeping of the ring: s is the stage of the plane being computed.
template <int NS> struct RingIdx {
    int s;
    __device__ __forceinline__ int up(bool top) const { return top ? s : (s + 1 == NS ? 0 : s + 1); }
    __device__ __forceinline__ int dn(bool bottom) const { return bottom ? s : (s == 0 ? NS - 1 : s - 1); }
    __device__ __forceinline__ int ahead() const { return s >= 2 ? s - 2 : s + NS - 2; }   // plane k + NS - 2
    __device__ __forceinline__ void next() { s = s + 1 == NS ? 0 : s + 1; }
};

// The neighbourhood of one cell as a residual pass sees it.
struct RCell {
    df xc, xe, xw, xn, xs, xu, xd;          // x = phi + dx (z neighbours as loaded, k+1 / k-1 clamped)
    float dc, de, dw, dn, ds, du, dd;        // pending correction (update passes)
    float pxe, pxw, pyn, pys, pzu, pzd;      // Pm for the divergence (z clamped)
    int mc, me, mw, mn, ms, mu, md;          // materials (general eps only)
};

// Film constants of a residual pass, held in registers.
struct RConst {
    df cb, cu;                  // eps_0_nd / (2h); eps / h^2 on every face (one eps)
    float dinv_u;               // Jacobi weight of the non-identity rows (one eps)
    int nz;
    bool neu;                   // Neumann z boundary (mirrored end rows, one pinned cell)
    long long ref;              // the pinned cell (film-local)
    const float *cf_h, *cf_l;   // general eps: face coefficient tables (through the film table)
};

// z neighbours of the operator (depol_varEPS.cu:86-99), given the loaded
// k+1 and k-1 values (clamped at the ends).
template <class V>
__device__ __forceinline__ void zpick(const RConst &rc, int k, V up, V dn, V &u, V &dd)
{
    if (!rc.neu || (k > 0 && k < rc.nz - 1)) { u = up; dd = dn; }
    else if (k == 0) { u = up; dd = up; }
    else { u = dn; dd = dn; }
}

// -A dx of one non-identity row in FP32 (dx: the pending correction).
template <bool UNI>
__device__ __forceinline__ float minus_adx(const RConst &rc, int k, const RCell &c)
{
    float du, ddn;
    zpick<float>(rc, k, c.du, c.dd, du, ddn);
    if (UNI) return rc.cu.h * ((c.de + c.dw) + (c.dn + c.ds) + (du + ddn) - 6.f * c.dc);
    int mu, md;
    zpick<int>(rc, k, c.mu, c.md, mu, md);
    const float *ch = rc.cf_h + c.mc * 3;
    return ch[c.me] * (c.de - c.dc) - ch[c.mw] * (c.dc - c.dw) + ch[c.mn] * (c.dn - c.dc) -
           ch[c.ms] * (c.dc - c.ds) + ch[mu] * (du - c.dc) - ch[md] * (c.dc - ddn);
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
// The grain's rotation t (row major) given.
__device__ __forceinline__ void tdgl_cell32t(const float4 *K, const float (&t)[9], const float (&pc)[6],
                                             const float (&sum)[6], float ex, float ey, float ez, float mEz,
                                             float (&pn)[6], float &pMZl, float &pSZl)
{
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

__device__ __forceinline__ void load_tr32(const float4 *tr, float (&t)[9])
{
    const float4 t0 = __ldg(tr), t1 = __ldg(tr + 1), t2 = __ldg(tr + 2);
    t[0] = t0.x; t[1] = t0.y; t[2] = t0.z; t[3] = t0.w;
    t[4] = t1.x; t[5] = t1.y; t[6] = t1.z; t[7] = t1.w; t[8] = t2.x;
}

// The rotation loaded from the grain's entry tr.
__device__ __forceinline__ void tdgl_cell32(const float4 *K, const float4 *tr, const float (&pc)[6],
                                            const float (&sum)[6], float ex, float ey, float ez, float mEz,
                                            float (&pn)[6], float &pMZl, float &pSZl)
{
    float t[9];
    load_tr32(tr, t);
    tdgl_cell32t(K, t, pc, sum, ex, ey, ez, mEz, pn, pMZl, pSZl);
}

// z neighbours of the potential for E (depol_varEPS.cu:246-273): zero beyond
// the Dirichlet planes, mirrored for the Neumann boundary.
__device__ __forceinline__ void efield_z(bool neumann, int k, int nz, df fu, df fd, df &pu, df &pd)
{
    if (!neumann) {
        pu = (k == nz - 1) ? df{0.f, 0.f} : fu;
        pd = (k == 0) ? df{0.f, 0.f} : fd;
    } else {
        pu = (k == nz - 1) ? fd : fu;         // mirrored (depol_varEPS.cu:86-99)
        pd = (k == 0) ? fu : fd;
    }
}

template <int NV>
__device__ __forceinline__ void row_acc(float (&acc)[NV], int mat, const float (&pn)[6], float pMZl, float pSZl)
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
// Stage layout (own + halo slots): P as three float2 planes (P0, P1), (P2, P3),
// (P4, P5), the potential as one (hi, lo) float2 plane, then the code (own),
// and with DEF the pending correction dx (own + halo): a stencil point of a
// pair is one 8-byte shared load.
template <int TYc, bool DEF = false> __host__ __device__ constexpr int t32_stage()      // floats
{
    return 8 * TileShape<TYc>::SPLt + TileShape<TYc>::NTt + (DEF ? TileShape<TYc>::SPLt : 0);
}
template <int TYc, bool DEF = false> constexpr size_t t32_smem()
{
    return sizeof(float) * T32_NS * t32_stage<TYc, DEF>();
}

template <int NV>
__device__ __forceinline__ void tdgl_def_film(const Dev &d, int rs, int fi, double (*sRed)[NV], double (&sTot)[NV]);
__device__ __forceinline__ void tdgl_def_grid(const Dev &d, int rs);

// TYc: the tile height (TX x TYc threads, one column each).
// DEF: a film whose previous step ended on its direct solve (SolveDev::pending;
// every depolarised film under kernel timing) has the potential x0 + dx -- the
// warm start in phi_cur plus the pending correction dx.  The step takes E
// from x0 + dx, writes x0 + dx to the free buffer (where the update pass
// would have put it), extrapolates the next warm start into the third-oldest
// potential's buffer (a warm start of at most quadratic order never reads
// it), and forms the check the update pass would have formed: r <- r - A dx
// in FP32 (r.r in the eighth partial sum).  The last block decides whether
// the previous step stands (tdgl_def_film, tdgl_def_grid).
// The check's values raise the registers a thread needs: the DEF kernels are
// built for three quarters of the blocks per SM (80 registers at 32 x 8
// tiles, where the 64 of four blocks spilled and ran 15 % slower).
template <int TYc, bool DEF> constexpr int tdgl32_minb()
{
    return DEF && TYc < 16 ? TileShape<TYc>::MINB * 3 / 4 : TileShape<TYc>::MINB;
}

template <int NS, int TYc = TY, bool DEF = false, bool FB = false>
__global__ void __launch_bounds__(TileShape<TYc>::NTt, tdgl32_minb<TYc, DEF>()) k_tdgl32(Dev d, Fields<float> F)
{
    static_assert(NS >= 4, "the ring holds planes k-1, k, k+1 and at least one in flight");
    constexpr int SPL = TileShape<TYc>::SPLt, NT = TileShape<TYc>::NTt, T32_STAGE = t32_stage<TYc, DEF>();
    constexpr int NV = DEF ? 8 : 7;         // row sums (+ the check's r.r)
    constexpr int DXO = 8 * SPL + NT;       // DEF: the dx plane of a stage
    extern __shared__ float4 smem_t32[];
    float *ring = (float *)smem_t32;
    __shared__ float4 sC[6][3];
    __shared__ double sRed[NT / 32][NV];
    __shared__ double sTot[NV];
    const int4 it = d.sitems[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    load_coef4(f, sC);
    const Geom g = make_geom<TYc>(f, it.y, it.z);
    const int cur = d.ctl->cur, rs = d.ctl->run_step;
    const float mEz = (float)(-d.wave[(long long)it.x * d.wstride + rs]);   // dfdPmz_app, kernels_evol.cu:210
    const int row = d.rows[(long long)it.x * d.wstride + rs];
    // film constants in registers (the stores below might alias the film table)
    const SolveDev *S = d.solve + it.x;
    const int dep = f->dep_flag, nz = g.nz, warm = warm_order(f, S);
    const bool neu = f->zbc != 0;
    const float inv_2hf = f->inv_2hf;
    const long long off = f->off, lo = d.ncells, fs = d.ncells;
    const bool pend = DEF && dep && (d.force || S->pending != 0);
    const float2 *ph = phi2_sel(d, S->phi_cur) + off;
    const float2 *qh = phi2_sel(d, S->phi_prev) + off;
    const float2 *uh = phi2_sel(d, S->phi_prev2) + off;
    const float2 *vh = phi2_sel(d, S->phi_prev3) + off;
    float2 *nh = phi2_sel(d, pend ? S->phi_prev3 : phi_free(S)) + off;
    float2 *xh = phi2_sel(d, phi_free(S)) + off;     // DEF: the checked potential x0 + dx
    const float *dxg = F.x + off, *rg = F.r + off;
    const uint32_t *code = d.code + off;
    const float4 *TR4 = (const float4 *)(F.TR + (long long)TR32 * f->g_off);
    const float2 *Po = pairs32(F, cur) + off;   // the three pairs of a set at j * fs
    float2 *Pn = pairs32(F, cur ^ 1) + off;
    const int zlo = max(z0 - 1, 0), zhi = min(z1, nz - 1);
    (void)lo;
    // the check's operator (one eps) and identity rows, as the update pass has them
    RConst rc;
    rc.cu = df{f->cf_h[0], f->cf_l[0]};
    rc.nz = nz;
    rc.neu = neu;
    const long long pin = neu ? (long long)f->ref_id - g.own_pl : -1;

    // copies of plane p (planes are issued in order, p = zlo, zlo + 1, ...)
    long long own_o = g.own_pl + (long long)zlo * g.plane, halo_o = g.halo_pl + (long long)zlo * g.plane;
    auto issue = [&](int p, float *st) {
        if (p <= zhi) {
            if (g.valid) {
                #pragma unroll
                for (int j = 0; j < 3; ++j) cp8(st + 2 * (j * SPL + g.own_slot), Po + j * fs + own_o);
                if (dep) cp8(st + 2 * (3 * SPL + g.own_slot), ph + own_o);
                cp4(st + 8 * SPL + threadIdx.x, code + own_o);
                if (pend) cp4(st + DXO + g.own_slot, dxg + own_o);
            }
            if (g.halo) {
                #pragma unroll
                for (int j = 0; j < 3; ++j) cp8(st + 2 * (j * SPL + g.halo_slot), Po + j * fs + halo_o);
                if (dep) cp8(st + 2 * (3 * SPL + g.halo_slot), ph + halo_o);
                if (pend) cp4(st + DXO + g.halo_slot, dxg + halo_o);
            }
        }
        cp_commit();
        own_o += g.plane;
        halo_o += g.plane;
    };
    for (int p = zlo; p <= z0 + NS - 3; ++p) issue(p, ring + (p - zlo) * T32_STAGE);

    float acc[NV];
    #pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = 0.f;
    const int s0 = g.own_slot;
    RingIdx<NS> ri{z0 - zlo};
    long long o = g.own_pl + (long long)z0 * g.plane;
    for (int k = z0; k < z1; ++k, o += g.plane, ri.next()) {
        cp_wait<NS - 4>();
        __syncthreads();
        issue(k + NS - 2, ring + ri.ahead() * T32_STAGE);
        if (!g.valid) continue;
        // older potentials for the warm start (consumed after the step's arithmetic)
        df wq{0.f, 0.f}, wu{0.f, 0.f}, wv{0.f, 0.f};
        if (dep && warm >= 1) wq = ld_df(qh + o);
        if (dep && warm >= 2) wu = ld_df(uh + o);
        if (dep && warm >= 3) wv = ld_df(vh + o);
        const float rold = pend ? rg[o] : 0.f;          // DEF: r of the step's first pass
        const float *sk = ring + ri.s * T32_STAGE;
        const float *su = ring + ri.up(k == nz - 1) * T32_STAGE, *sd = ring + ri.dn(k == 0) * T32_STAGE;
        const uint32_t c = ((const uint32_t *)sk)[8 * SPL + threadIdx.x];
        const float2 *k2 = (const float2 *)sk, *u2 = (const float2 *)su, *d2 = (const float2 *)sd;
        float pc[6], sum[6];
        #pragma unroll
        for (int p = 0; p < 3; ++p) {
            const float2 *a = k2 + p * SPL;
            const float2 cc = a[s0], xe = a[s0 + 1], xw = a[s0 - 1], yn = a[s0 + SX], ys = a[s0 - SX];
            const float2 zu = u2[p * SPL + s0], zd = d2[p * SPL + s0];
            pc[2 * p] = cc.x;
            pc[2 * p + 1] = cc.y;
            // neighbour sums e, w, n, s, u, d (kernels_evol.cu:101-122); z clamped
            sum[2 * p] = ((((xe.x + xw.x) + yn.x) + ys.x) + zu.x) + zd.x;
            sum[2 * p + 1] = ((((xe.y + xw.y) + yn.y) + ys.y) + zu.y) + zd.y;
        }
        float ex = 0.f, ey = 0.f, ez = 0.f;
        df a0{0.f, 0.f};
        float chk = 0.f;                                // DEF: the check's r, formed here
        if (dep) {
            const float2 *f2 = k2 + 3 * SPL;
            const float2 fc = f2[s0], fu = u2[3 * SPL + s0], fd = d2[3 * SPL + s0];
            const float2 fe = f2[s0 + 1], fw = f2[s0 - 1], fn = f2[s0 + SX], fsth = f2[s0 - SX];
            a0 = df{fc.x, fc.y};
            df pu, pd;
            efield_z(neu, k, nz, df{fu.x, fu.y}, df{fd.x, fd.y}, pu, pd);
            // -1 * E with E = -(phi_+ - phi_-) / (2h)
            ex = phi_diff32(df{fe.x, fe.y}, df{fw.x, fw.y});
            ey = phi_diff32(df{fn.x, fn.y}, df{fsth.x, fsth.y});
            ez = phi_diff32(pu, pd);
            if (pend) {
                // phi = x0 + dx: the differences of dx added, the own value
                // resolved and stored; the update pass's r <- r - A dx
                // (identity rows: x - g with g = 0)
                RCell cd;
                const float *dk = sk + DXO;
                cd.dc = dk[s0]; cd.de = dk[s0 + 1]; cd.dw = dk[s0 - 1]; cd.dn = dk[s0 + SX]; cd.ds = dk[s0 - SX];
                cd.du = su[DXO + s0]; cd.dd = sd[DXO + s0];
                df du{cd.du, 0.f}, dd{cd.dd, 0.f};
                efield_z(neu, k, nz, du, dd, du, dd);
                ex += cd.de - cd.dw;
                ey += cd.dn - cd.ds;
                ez += du.h - dd.h;
                a0 = df_add_f(a0, cd.dc);
                xh[o] = make_float2(a0.h, a0.l);
                const bool ident = neu ? (long long)k * g.plane == pin : (k == 0 || k == nz - 1);
                chk = ident ? -(a0.h + a0.l) : rold + minus_adx<true>(rc, k, cd);
            }
            ex *= inv_2hf;
            ey *= inv_2hf;
            ez *= inv_2hf;
        }
        float pn[6], pMZl, pSZl;
        tdgl_cell32(sC[code_mat(c) * 2 + code_iface(c)], TR4 + 3LL * code_gid(c), pc, sum, ex, ey, ez, mEz, pn,
                    pMZl, pSZl);
        #pragma unroll
        for (int j = 0; j < 3; ++j) Pn[j * fs + o] = make_float2(pn[2 * j], pn[2 * j + 1]);
        if (row >= 0) row_acc(acc, code_mat(c), pn, pMZl, pSZl);
        if (dep) {
            const df w = extrap_phi(warm, a0, wq, wu, wv);
            nh[o] = make_float2(w.h, w.l);
        }
        if (pend) acc[NV - 1] = fmaf(chk, chk, acc[NV - 1]);
    }
    cp_wait<0>();

    if (row >= 0 || pend) block_partial32<NV>(d, acc, sRed);
    if constexpr (DEF)
        finish32<FB>(d, [&](int fi) { tdgl_def_film<NV>(d, rs, fi, sRed, sTot); }, [&] { tdgl_def_grid(d, rs); });
    else
        finish32<FB>(d, [&](int fi) { tdgl_film32(d, rs, fi, sRed, sTot); }, [&] { tdgl_grid32(d, rs); });
}

// The end of a TDGL step that may carry deferred checks (finish32): every
// pending film's r.r of its check decides whether its previous step stands
// (the update pass's test, ||r|| <= refine_tol ||b||).  If every check
// passes, the checked potentials become current and the step begins as
// tdgl_grid32 begins it.  If one fails, the previous step is reopened: the
// step counters and the P sets roll back, the failed films are set up for
// the update pass that the step's next residual pass then is, the films
// whose checks passed stay pending (the repeated step checks them again, to
// the same result), and the step loop runs this step again after that pass
// has ended the previous one.
// Film fi's part: its sweep row and its check's r.r (S->rr64).  Under
// Dev::row_off the row is left to the step's first residual pass
// (row_from_tdgl): only the check's r.r is totalled here, one value instead
// of eight at the end of the grid.
template <int NV>
__device__ __forceinline__ void tdgl_def_film(const Dev &d, int rs, int fi, double (*sRed)[NV], double (&sTot)[NV])
{
    static_assert(NV == 8, "seven row sums and the check's r.r");
    const FilmDev *ff = d.films + fi;
    SolveDev *S = d.solve + fi;
    const int frow = d.rows[(long long)fi * d.wstride + rs];
    if (d.row_off) {
        if (!ff->dep_flag || !(d.force || uniform_flag(&S->pending))) return;
        double rr[1];
        film_total32<1, NV - 1>(d, ff, (double (*)[1])sRed, rr);
        if (threadIdx.x == 0 && !d.force) S->rr64 = rr[0];
        return;
    }
    if (d.force) {              // kernel timing: the totals as a step forms them; the state stays as it is
        if (ff->dep_flag || frow >= 0) film_total32<NV>(d, ff, sRed, sTot);
        return;
    }
    const bool pend = ff->dep_flag != 0 && uniform_flag(&S->pending);
    if (frow < 0 && !pend) return;
    film_total32<NV>(d, ff, sRed, sTot);
    if (threadIdx.x == 0) {
        if (frow >= 0) row_write(d, fi, frow, sTot);
        if (pend) S->rr64 = sTot[NV - 1];
    }
}

// A pending film's check passed (NaN fails); rr read past this block's L1.
__device__ __forceinline__ bool def_check_ok(const Dev &d, int fi)
{
    const double rr = *(volatile const double *)&d.solve[fi].rr64;
    return rr <= d.films[fi].refine_tol2 * d.solve[fi].bb || rr == 0.0;
}

// What depends on every film: resolve and begin, or reopen.
__device__ __forceinline__ void tdgl_def_grid(const Dev &d, int rs)
{
    if (threadIdx.x != 0) return;
    if (d.force) {
        *d.counter = 0u;
        return;
    }
    bool fail = false;
    for (int fi = 0; fi < d.n_films; ++fi)
        if (d.films[fi].dep_flag && d.solve[fi].pending && !def_check_ok(d, fi)) fail = true;
    if (!fail) {
        for (int fi = 0; fi < d.n_films; ++fi) {
            SolveDev *S = d.solve + fi;
            if (S->pending) {
                // this launch wrote x0 + dx to the free buffer; the warm start
                // buffer (x0) takes the third-oldest slot, which held the next
                // warm start and now becomes the free one
                const int fr = phi_free(S);
                S->phi_prev3 = S->phi_cur;
                S->phi_cur = fr;
                S->pending = 0;
            }
            step_reset(d, fi);
            if (d.row_off) {    // the step's first residual pass totals and writes the row
                const int frow = d.rows[(long long)fi * d.wstride + rs];
                S->row_pend = frow >= 0 ? frow + 1 : 0;
            }
        }
        step_begin(d, rs);
    } else {
        for (int fi = 0; fi < d.n_films; ++fi) {
            SolveDev *S = d.solve + fi;
            if (S->pending && !def_check_ok(d, fi)) {
                S->pending = 0;
                S->outer_active = 1;
                S->active = 0;
                S->refine = 1;
                S->upd = 1;
            }
        }
        step_reopen(d);
        set_cond(d, d.h_steps, 1);
    }
    *d.counter = 0u;
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
    const long long off = f->off;
    const float2 *ph = phi2_sel(d, S->phi_cur) + off;
    const float2 *qh = phi2_sel(d, S->phi_prev) + off;
    const float2 *uh = phi2_sel(d, S->phi_prev2) + off;
    const float2 *vh = phi2_sel(d, S->phi_prev3) + off;
    float2 *nh = phi2_sel(d, phi_free(S)) + off;
    const int warm = warm_order(f, S);
    for (int k = z0; k < z1; ++k) {
        const long long o = g.own_pl + (long long)k * g.plane;
        const df w = extrap_phi(warm, ld_df(ph + o), ld_df(qh + o), ld_df(uh + o), ld_df(vh + o));
        nh[o] = make_float2(w.h, w.l);
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

// r (FP32 value of b - A x, double-float arithmetic) and b.h of one non-identity row.
template <bool UNI>
__device__ __forceinline__ void refine_row(const RConst &rc, int k, const RCell &c, float &rv, float &bh)
{
    const df bm = df_mul(div3(c.pxe, c.pxw, c.pyn, c.pys, c.pzu, c.pzd), rc.cb);   // -b
    df xu, xd;
    zpick<df>(rc, k, c.xu, c.xd, xu, xd);
    df s;            // b - A phi
    if (UNI) {
        s = df_sub(df_mul(rc.cu, lap7(c.xe, c.xw, c.xn, c.xs, xu, xd, c.xc)), bm);
    } else {
        int mu, md;
        zpick<int>(rc, k, c.mu, c.md, mu, md);
        const int m3 = c.mc * 3;
        auto cf = [&](int i) { return df{rc.cf_h[m3 + i], rc.cf_l[m3 + i]}; };
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
__device__ __forceinline__ void refine_cell(const RConst &rc, int k, bool ident, bool upd, const RCell &c,
                                            float r_old, float dinv, float &rv, float (&acc)[3])
{
    float bh = 0.f, wj = 1.f;
    if (ident) {
        rv = -(c.xc.h + c.xc.l);              // x - g with g = 0, b = 0
    } else {
        if (upd) rv = r_old + minus_adx<UNI>(rc, k, c);
        else refine_row<UNI>(rc, k, c, rv, bh);
        wj = UNI ? rc.dinv_u : dinv;
    }
    acc[0] = fmaf(rv, rv, acc[0]);
    acc[1] = fmaf(bh, bh, acc[1]);
    acc[2] = fmaf(rv, rv * wj, acc[2]);
}

__device__ __forceinline__ void refine_partials(const Dev &d, float (&acc)[3], double (*sRed)[3])
{
    block_partial32<3>(d, acc, sRed, d.rpartial);
}

// Dev::row_off (a single film with deferred checks): block 0 of the step's
// first residual pass totals the sweep row from the TDGL step's item
// partials (slots 0-6, which the residual passes leave alone) and writes it,
// while the other blocks run their items; the TDGL step's last block formed
// only the check's r.r.  Under kernel timing the total is formed and nothing
// written.  Every thread of block 0.
__device__ __forceinline__ void row_from_tdgl(const Dev &d, double (*sRow)[7])
{
    SolveDev *S = d.solve;
    const int rp = d.force ? 1 : S->row_pend;
    if (rp <= 0) return;
    double t[7];
    film_total32<7>(d, d.films, sRow, t);
    if (threadIdx.x == 0 && !d.force) {
        row_write(d, 0, rp - 1, t);
        S->row_pend = 0;
    }
}

// Stage layout (floats): x = phi (+ dx) as one (hi, lo) float2 plane, dx,
// the (Pmx, Pmy) pair plane, Pmz (own), then the general-eps code and D^-1.
// The update pass keeps the old r of the own cell in the Pmz slot.
template <bool UNI, int TYc = TY> struct R32Lay {
    static constexpr int SPL = TileShape<TYc>::SPLt, NT = TileShape<TYc>::NTt;
    static constexpr int FX = 0, DX = 2 * SPL, PA = 3 * SPL, PZ = 5 * SPL;
    static constexpr int CODE = 5 * SPL + NT, DINV = 6 * SPL + NT;   // general eps only
    static constexpr int STAGE = UNI ? 5 * SPL + NT : 6 * SPL + 2 * NT;
};
template <bool UNI, int TYc = TY> constexpr size_t r32_smem()
{
    return sizeof(float) * R32_NS * R32Lay<UNI, TYc>::STAGE;
}

template <bool UNI, int NS, int TYc = TY, bool FB = false>
__global__ void __launch_bounds__(TileShape<TYc>::NTt, TileShape<TYc>::MINB) k_refine32(Dev d, Fields<float> F)
{
    static_assert(NS >= 4, "the ring holds planes k-1, k, k+1 and at least one in flight");
    using L = R32Lay<UNI, TYc>;
    constexpr int NT = TileShape<TYc>::NTt;
    extern __shared__ float4 smem_r32[];
    float *ring = (float *)smem_r32;
    __shared__ double sRed[NT / 32][3];
    __shared__ double sTot[3];
    if (!FB && d.row_off && blockIdx.x == 0) {
        __shared__ double sRow[NT / 32][7];
        row_from_tdgl(d, sRow);
    }
    const int4 it = d.sitems[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const SolveDev *S = d.solve + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom<TYc>(f, it.y, it.z);
    const int nz = g.nz;
    // film constants in registers (the stores below might alias the film table)
    RConst rc;
    rc.cb = df{f->cb_h, f->cb_l};
    rc.cu = df{f->cf_h[0], f->cf_l[0]};
    rc.dinv_u = f->dinv_uni;
    rc.nz = nz;
    rc.neu = f->zbc != 0;
    rc.ref = f->ref_id;
    rc.cf_h = f->cf_h;
    rc.cf_l = f->cf_l;
    const bool run = f->dep_flag != 0 && (d.force || S->outer_active);
    const bool apply = S->refine > 0;                   // later pass: x = phi + dx; first: the warm start
    const bool upd = UNI && apply && S->upd && f->upd_ok;   // r <- r - A dx (after the direct solve, one eps)
    const int cur = d.ctl->cur, fr = phi_free(S);
    const long long off = f->off, fs = d.ncells;
    const float2 *xh = phi2_sel(d, apply ? S->phi_cur : fr) + off;
    float2 *nh = phi2_sel(d, fr) + off;
    const float *dx = F.x + off;
    const float2 *PA = pairs32(F, cur ^ 1) + off;            // the new (Pmx, Pmy)
    const float *PZ = (const float *)(PA + fs);              // the new Pmz: .x of the (Pmz, Psx) pairs
    const uint32_t *code = d.code + off;
    const float *dinv = F.dinv + off;
    float *r = F.r + off;
    const int zlo = max(z0 - 1, 0), zhi = min(z1, nz - 1);

    // copies of plane p (planes are issued in order, p = zlo, zlo + 1, ...)
    long long own_o = g.own_pl + (long long)zlo * g.plane, halo_o = g.halo_pl + (long long)zlo * g.plane;
    auto issue = [&](int p, float *st) {
        if (run && p <= zhi) {
            const int so = g.own_slot, sh = g.halo_slot;
            if (upd) {
                // update pass: dx with its halo; phi and the old r of the own cell
                if (g.valid) {
                    cp8(st + L::FX + 2 * so, xh + own_o);
                    cp4(st + L::DX + so, dx + own_o);
                    cp4(st + L::PZ + threadIdx.x, r + own_o);
                }
                if (g.halo) cp4(st + L::DX + sh, dx + halo_o);
            } else {
                if (g.valid) {
                    cp8(st + L::FX + 2 * so, xh + own_o);
                    if (apply) cp4(st + L::DX + so, dx + own_o);
                    cp8(st + L::PA + 2 * so, PA + own_o);
                    cp4(st + L::PZ + threadIdx.x, PZ + 2 * own_o);
                    if (!UNI) {
                        cp4(st + L::CODE + so, code + own_o);
                        cp4(st + L::DINV + threadIdx.x, dinv + own_o);
                    }
                }
                if (g.halo) {
                    cp8(st + L::FX + 2 * sh, xh + halo_o);
                    if (apply) cp4(st + L::DX + sh, dx + halo_o);
                    cp8(st + L::PA + 2 * sh, PA + halo_o);
                    if (!UNI) cp4(st + L::CODE + sh, code + halo_o);
                }
            }
        }
        cp_commit();
        own_o += g.plane;
        halo_o += g.plane;
    };
    for (int p = zlo; p <= z0 + NS - 3; ++p) issue(p, ring + (p - zlo) * L::STAGE);

    const int s0 = g.own_slot, tz = threadIdx.x;
    const long long pin = rc.neu ? rc.ref - g.own_pl : -1;   // the pinned cell's plane offset in this column
    float acc[3] = {0.f, 0.f, 0.f};
    RingIdx<NS> ri{z0 - zlo};
    long long o = g.own_pl + (long long)z0 * g.plane;
    for (int k = z0; k < z1; ++k, o += g.plane, ri.next()) {
        cp_wait<NS - 4>();
        __syncthreads();
        issue(k + NS - 2, ring + ri.ahead() * L::STAGE);
        if (!run || !g.valid) continue;
        const float *sk = ring + ri.s * L::STAGE;
        const float *su = ring + ri.up(k == nz - 1) * L::STAGE, *sd = ring + ri.dn(k == 0) * L::STAGE;
        auto D = [&](const float *st, int s) { return st[L::DX + s]; };
        auto X = [&](const float *st, int s) {        // x = phi (+ dx on later passes)
            const float2 v = ((const float2 *)(st + L::FX))[s];
            const df p{v.x, v.y};
            return apply ? df_add_f(p, D(st, s)) : p;
        };
        auto PAx = [&](const float *st, int s) { return ((const float2 *)(st + L::PA))[s].x; };
        auto PAy = [&](const float *st, int s) { return ((const float2 *)(st + L::PA))[s].y; };
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
            c.pxe = PAx(sk, s0 + 1); c.pxw = PAx(sk, s0 - 1);
            c.pyn = PAy(sk, s0 + SX); c.pys = PAy(sk, s0 - SX);
            c.pzu = su[L::PZ + tz]; c.pzd = sd[L::PZ + tz];
        }
        // identity rows: the Dirichlet planes, or the Neumann pin
        const bool ident = rc.neu ? (long long)k * g.plane == pin : (k == 0 || k == nz - 1);
        float rv;
        refine_cell<UNI>(rc, k, ident, upd, c, upd ? sk[L::PZ + tz] : 0.f, UNI ? 0.f : sk[L::DINV + tz], rv, acc);
        r[o] = rv;
        if (apply) nh[o] = make_float2(c.xc.h, c.xc.l);
    }
    cp_wait<0>();
    refine_partials(d, acc, sRed);
    finish32<FB>(d, [&](int fi) { refine_film(d, fi, sRed, sTot); }, [&] { refine_grid(d); });
}

}  // namespace cmsl
