// stencil_tma.cuh -- the CMSL_FP32_REFINED stencil passes with tensor-copy
// (TMA) staging: the TDGL step (k_tdgl32t) and the double-float residual
// pass (k_refine32t).
//
// Same work items (the stencil list, Dev::sitems, with the tile height TY)
// and arithmetic as stencil32.cuh, but a plane of every field
// is brought into the ring by cp.async.bulk.tensor copies that the first
// lane of each warp issues (a few boxes each) and that complete on the
// stage's mbarrier; no thread computes a per-cell copy address.  A field of a plane lands as five boxes:
//
//   [S row: TX][tile: TY x TX][N row: TX][W strip: TY x 16 B][E strip: TY x 16 B]
//
// the y halo rows at (y0 - 1) mod ny and (y0 + TY) mod ny and the x halo
// strips ending at x0 - 1 and starting at x0 + TX (mod nx), so the periodic
// halo needs no special case: the S row sits just before the tile and the N
// row just after it (the y neighbours are always +-TX elements away), and
// only the first and last thread of a row read their x neighbour from a
// strip.  Films must have nx % 32 == 0 and ny % 8 == 0 (full tiles).
//
// Ring protocol: planes zlo = max(z0-1, 0) .. zhi = min(z1, nz-1) are staged,
// plane p in stage (p - zlo) % NS, whose barrier completes phase
// (p - zlo) / NS when the plane has landed.  Before computing plane k every
// thread waits for plane k+1, the block syncs (retiring every read of plane
// k-2) and the warps' first lanes issue plane k+NS-2 into that stage.
#pragma once
#include "stencil32.cuh"
#include "tma.cuh"

namespace cmsl {

// one field region, in elements of the field's type
constexpr int TR_S = 0, TR_BODY = TX, TR_N = TX + NT, TR_W = 2 * TX + NT;
__host__ __device__ constexpr int tr_e(int esz) { return TR_W + TY * (16 / esz); }
__host__ __device__ constexpr int tr_elems(int esz) { return tr_e(esz) + TY * (16 / esz); }
constexpr int REG2 = 8 * tr_elems(8);     // bytes of a float2 region (2816)
constexpr int REG1 = 4 * tr_elems(4);     // bytes of a float region (1536)
constexpr int BODY2 = 8 * NT, BODY1 = 4 * NT;
static_assert(REG2 % 128 == 0 && REG1 % 128 == 0, "regions keep 128-byte alignment");

// Per-thread neighbour offsets (elements) inside a region of element size
// esz: the own cell, and the x / y neighbours (an x neighbour beyond the tile
// comes from the strip; the y rows adjoin the tile).
struct NbOff {
    int c, e, w, n, s;
};
__device__ __forceinline__ NbOff nb_off(int esz)
{
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX, per = 16 / esz;
    NbOff o;
    o.c = TR_BODY + ly * TX + lx;
    o.n = o.c + TX;
    o.s = o.c - TX;
    o.w = lx > 0 ? o.c - 1 : TR_W + ly * per + per - 1;
    o.e = lx < TX - 1 ? o.c + 1 : tr_e(esz) + ly * per;
    return o;
}

// Map sets by buffer index, clamped as phi_sel clamps its pointers (any
// index outside 0..4 selects buffer 4), so a stale or unset solver slot can
// never select memory outside the film's table.
__device__ __forceinline__ const CUtensorMap *phi_maps(const FilmMaps *M, int i)
{
    return M->phi[(i >= 0 && i < 5) ? i : 4];
}
__device__ __forceinline__ const CUtensorMap *p_maps(const FilmMaps *M, int set) { return M->P[set & 1]; }

// Appends the five boxes of one field region (base: byte offset in the
// stage) for tile (x0, y0); q is the 4D map's field index or -1 (3D map).
struct OpBuilder {
    TmaOp *ops;
    int n;
    int x0, y0, nx, ny;
    __device__ __forceinline__ void add(const CUtensorMap *m, int dst, int x, int y, int q)
    {
        ops[n++] = TmaOp{m, dst, x, y, q, 0};
    }
    // all five boxes; esz 8 (float2) or 4 (float / uint32)
    __device__ __forceinline__ void region(const CUtensorMap *m3, int base, int q, int esz)
    {
        const int per = 16 / esz;
        add(&m3[TM_ROW], base + esz * TR_S, x0, (y0 - 1 + ny) % ny, q);
        add(&m3[TM_BODY], base + esz * TR_BODY, x0, y0, q);
        add(&m3[TM_ROW], base + esz * TR_N, x0, (y0 + TY) % ny, q);
        add(&m3[TM_COL], base + esz * TR_W, (x0 - per + nx) % nx, y0, q);
        add(&m3[TM_COL], base + esz * tr_e(esz), (x0 + TX) % nx, y0, q);
    }
    // the tile body only, at the region's body position
    __device__ __forceinline__ void body(const CUtensorMap *m3, int base, int q, int esz)
    {
        add(&m3[TM_BODY], base + esz * TR_BODY, x0, y0, q);
    }
};

// The ring of one block: NS stages of STAGE bytes from a 128-byte aligned
// base of the dynamic shared memory, their barriers, and the copy table.
template <int NS, int MAXOPS> struct TmaRing {
    uint32_t base;                // shared address of stage 0
    const unsigned char *ptr;     // generic address of stage 0
    uint64_t *bar;
    TmaOp *ops;
    int n_ops, zlo, zhi, stage_bytes;
    uint32_t tx;                  // bytes per plane
    __device__ __forceinline__ int st(int p) const { return (p - zlo) % NS; }
    __device__ __forceinline__ void issue(int p) const
    {
        if (p <= zhi) {
            const int s = st(p);
            tma_issue_plane(ops, n_ops, base + (uint32_t)(s * stage_bytes), p, &bar[s], tx);
        }
    }
    __device__ __forceinline__ void wait(int p, int *err) const
    {
        if (p <= zhi) mbar_wait(&bar[st(p)], (uint32_t)(((p - zlo) / NS) & 1), err);
    }
    __device__ __forceinline__ const unsigned char *stage(int s) const { return ptr + s * stage_bytes; }
};

template <int NS, int MAXOPS>
__device__ __forceinline__ TmaRing<NS, MAXOPS> ring_setup(unsigned char *dyn, uint64_t *bar, TmaOp *ops, int zlo,
                                                         int zhi, int stage_bytes)
{
    TmaRing<NS, MAXOPS> r;
    const uint32_t raw = smem_u32(dyn);
    r.base = (raw + 127u) & ~127u;
    r.ptr = dyn + (r.base - raw);
    r.bar = bar;
    r.ops = ops;
    r.zlo = zlo;
    r.zhi = zhi;
    r.stage_bytes = stage_bytes;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        fence_barrier_init();
    }
    return r;
}

// ------------------------------------------------------------ TDGL step
// kernelCalc_antiferro (kernels_evol.cu:47-231) + E of the current potential
// (depol_varEPS.cu:223-276) + the sweep-row sums (evolve.cu:256-357) + the
// extrapolated warm start, as k_tdgl32.
constexpr int TT_NS = 4;
constexpr int TT_PHI = 3 * REG2, TT_CODE = 4 * REG2, TT_STAGE = 4 * REG2 + BODY1;   // bytes
constexpr size_t TT_SMEM = (size_t)TT_NS * TT_STAGE + 128;
constexpr int TT_OPS = 3 * 5 + 5 + 1;

template <int NS, bool FB = false>
__global__ void __launch_bounds__(NT, 4) k_tdgl32t(Dev d, Fields<float> F)
{
    static_assert(NS >= 4, "the ring holds planes k-1, k, k+1 and at least one in flight");
    extern __shared__ unsigned char smem_tt[];
    __shared__ __align__(8) uint64_t bar[NS];
    __shared__ TmaOp ops[TT_OPS];
    __shared__ float4 sC[6][3];
    __shared__ double sRed[NT / 32][7];
    __shared__ double sTot[7];
    const int4 it = d.sitems[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    load_coef4(f, sC);
    const int nx = f->nx, ny = f->ny, nz = f->nz, x0 = it.y, y0 = it.z;
    const int cur = d.ctl->cur, rs = d.ctl->run_step;
    const float mEz = (float)(-d.wave[(long long)it.x * d.wstride + rs]);   // dfdPmz_app, kernels_evol.cu:210
    const int row = d.rows[(long long)it.x * d.wstride + rs];
    const SolveDev *S = d.solve + it.x;
    const int dep = f->dep_flag, warm = warm_order(f, S);
    const bool neu = f->zbc != 0;
    const float inv_2hf = f->inv_2hf;
    const long long off = f->off, fs = d.ncells, plane = (long long)nx * ny;
    const int pcur = S->phi_cur;
    const float2 *qh = phi2_sel(d, S->phi_prev) + off;
    const float2 *uh = phi2_sel(d, S->phi_prev2) + off;
    const float2 *vh = phi2_sel(d, S->phi_prev3) + off;
    float2 *nh = phi2_sel(d, phi_free(S)) + off;
    const float4 *TR4 = (const float4 *)(F.TR + (long long)TR32 * f->g_off);
    float2 *Pn = pairs32(F, cur ^ 1) + off;
    const int zlo = max(z0 - 1, 0), zhi = min(z1, nz - 1);
    const FilmMaps *M = d.maps + it.x;

    auto R = ring_setup<NS, TT_OPS>(smem_tt, bar, ops, zlo, zhi, TT_STAGE);
    R.n_ops = 3 * 5 + (dep ? 5 : 0) + 1;
    R.tx = (uint32_t)(3 * REG2 + (dep ? REG2 : 0) + BODY1);
    if (threadIdx.x == 0) {
        OpBuilder b{ops, 0, x0, y0, nx, ny};
        for (int j = 0; j < 3; ++j) b.region(p_maps(M, cur), j * REG2, j, 8);
        if (dep) b.region(phi_maps(M, pcur), TT_PHI, -1, 8);
        b.body(M->code, TT_CODE - 4 * TR_BODY, -1, 4);
    }
    __syncthreads();

    for (int p = zlo; p <= z0 + NS - 3; ++p) R.issue(p);
    for (int p = zlo; p <= z0; ++p) R.wait(p, d.err);

    const NbOff o2 = nb_off(8);
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    float acc[7];
    #pragma unroll
    for (int q = 0; q < 7; ++q) acc[q] = 0.f;
    RingIdx<NS> ri{z0 - zlo};
    long long o = (long long)(x0 + lx) + (long long)nx * (y0 + ly) + (long long)z0 * plane;
    const long long plane_step = plane;
    float2 oq{0.f, 0.f}, ou{0.f, 0.f};
    auto ld_old = [&](long long oo) {
        if (dep && warm >= 1) oq = qh[oo];
        if (dep && warm >= 2) ou = uh[oo];
    };
    ld_old(o);
    for (int k = z0; k < z1; ++k, o += plane, ri.next()) {
        R.wait(k + 1, d.err);
        __syncthreads();
        R.issue(k + NS - 2);
        // older potentials for the warm start, loaded one plane ahead (the
        // cubic start's third one in place), consumed after the step's arithmetic
        const df wq{oq.x, oq.y}, wu{ou.x, ou.y};
        const df wv = (dep && warm >= 3) ? ld_df(vh + o) : df{0.f, 0.f};
        if (k + 1 < z1) ld_old(o + plane_step);
        const unsigned char *sk = R.stage(ri.s);
        const unsigned char *su = R.stage(ri.up(k == nz - 1)), *sd = R.stage(ri.dn(k == 0));
        const uint32_t c = ((const uint32_t *)(sk + TT_CODE))[threadIdx.x];
        float pc[6], sum[6];
        #pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float2 *a = (const float2 *)(sk + j * REG2);
            const float2 cc = a[o2.c], xe = a[o2.e], xw = a[o2.w], yn = a[o2.n], ys = a[o2.s];
            const float2 zu = ((const float2 *)(su + j * REG2))[o2.c], zd = ((const float2 *)(sd + j * REG2))[o2.c];
            pc[2 * j] = cc.x;
            pc[2 * j + 1] = cc.y;
            // neighbour sums e, w, n, s, u, d (kernels_evol.cu:101-122); z clamped
            sum[2 * j] = ((((xe.x + xw.x) + yn.x) + ys.x) + zu.x) + zd.x;
            sum[2 * j + 1] = ((((xe.y + xw.y) + yn.y) + ys.y) + zu.y) + zd.y;
        }
        float ex = 0.f, ey = 0.f, ez = 0.f;
        df a0{0.f, 0.f};
        if (dep) {
            const float2 *f2 = (const float2 *)(sk + TT_PHI);
            const float2 fc = f2[o2.c], fe = f2[o2.e], fw = f2[o2.w], fn = f2[o2.n], fsth = f2[o2.s];
            const float2 fu = ((const float2 *)(su + TT_PHI))[o2.c], fd = ((const float2 *)(sd + TT_PHI))[o2.c];
            a0 = df{fc.x, fc.y};
            df pu, pd;
            efield_z(neu, k, nz, df{fu.x, fu.y}, df{fd.x, fd.y}, pu, pd);
            // -1 * E with E = -(phi_+ - phi_-) / (2h)
            ex = phi_diff32(df{fe.x, fe.y}, df{fw.x, fw.y}) * inv_2hf;
            ey = phi_diff32(df{fn.x, fn.y}, df{fsth.x, fsth.y}) * inv_2hf;
            ez = phi_diff32(pu, pd) * inv_2hf;
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
    }

    if (row >= 0) block_partial32<7>(d, acc, sRed);
    finish32<FB>(d, [&](int fi) { tdgl_film32(d, rs, fi, sRed, sTot); }, [&] { tdgl_grid32(d, rs); });
}

// ------------------------------------------------- double-float residual
// One refinement pass (as k_refine32): b - A x in double-float with x the
// warm start (first pass) or phi + dx (later passes), or the FP32 update
// r <- r - A dx (update pass), and the partial sums r.r, b.b, r.D^-1.r.
// Stage: x (float2 region), dx (float region), (Pmx, Pmy) (float2 region),
// the (Pmz, Psx) tile body (Pmz of the own cell; the update pass keeps the
// old r there), then for several eps the material codes and D^-1.
constexpr int RT_NS = 5;
constexpr int RT_X = 0, RT_DX = REG2, RT_PA = REG2 + REG1, RT_PZ = 2 * REG2 + REG1;
constexpr int RT_CODE = RT_PZ + BODY2, RT_DINV = RT_CODE + REG1;
template <bool UNI> __host__ __device__ constexpr int rt_stage() { return UNI ? RT_CODE : RT_DINV + BODY1; }
template <bool UNI> constexpr size_t rt_smem() { return (size_t)RT_NS * rt_stage<UNI>() + 128; }
constexpr int RT_OPS = 5 + 5 + 5 + 1 + 5 + 1;

template <bool UNI, int NS, bool FB = false>
__global__ void __launch_bounds__(NT, 4) k_refine32t(Dev d, Fields<float> F)
{
    static_assert(NS >= 4, "the ring holds planes k-1, k, k+1 and at least one in flight");
    constexpr int STAGE = rt_stage<UNI>();
    extern __shared__ unsigned char smem_rt[];
    __shared__ __align__(8) uint64_t bar[NS];
    __shared__ TmaOp ops[RT_OPS];
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
    const int nx = f->nx, ny = f->ny, nz = f->nz, x0 = it.y, y0 = it.z;
    const long long plane = (long long)nx * ny;
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
    const int cur = d.ctl->cur, fr = phi_free(S), xb = apply ? S->phi_cur : fr;
    const long long off = f->off;
    float2 *nh = phi2_sel(d, fr) + off;
    float *r = F.r + off;
    const int zlo = max(z0 - 1, 0), zhi = min(z1, nz - 1);
    const FilmMaps *M = d.maps + it.x;

    auto R = ring_setup<NS, RT_OPS>(smem_rt, bar, ops, zlo, run ? zhi : -1, STAGE);
    // update pass: dx with its halo, phi and the old r of the own cell;
    // otherwise x with its halo, dx (later passes), (Pmx, Pmy), Pmz, codes and D^-1
    R.n_ops = upd ? 7 : 5 + (apply ? 5 : 0) + 5 + 1 + (UNI ? 0 : 6);
    R.tx = (uint32_t)(upd ? BODY2 + REG1 + BODY1
                          : REG2 + (apply ? REG1 : 0) + REG2 + BODY2 + (UNI ? 0 : REG1 + BODY1));
    if (threadIdx.x == 0) {
        OpBuilder b{ops, 0, x0, y0, nx, ny};
        if (upd) {
            b.body(phi_maps(M, xb), RT_X, -1, 8);
            b.region(M->x, RT_DX, -1, 4);
            b.add(&M->r, RT_PZ, x0, y0, -1);
        } else {
            b.region(phi_maps(M, xb), RT_X, -1, 8);
            if (apply) b.region(M->x, RT_DX, -1, 4);
            b.region(p_maps(M, cur ^ 1), RT_PA, 0, 8);
            b.add(&p_maps(M, cur ^ 1)[TM_BODY], RT_PZ, x0, y0, 1);
            if (!UNI) {
                b.region(M->code, RT_CODE, -1, 4);
                b.add(&M->dinv, RT_DINV, x0, y0, -1);
            }
        }
    }
    __syncthreads();

    for (int p = zlo; p <= z0 + NS - 3; ++p) R.issue(p);
    for (int p = zlo; p <= z0; ++p) R.wait(p, d.err);

    const NbOff o2 = nb_off(8), o1 = nb_off(4);
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX, tz = threadIdx.x;
    const long long own_pl = (long long)(x0 + lx) + (long long)nx * (y0 + ly);
    const long long pin = rc.neu ? rc.ref - own_pl : -1;   // the pinned cell's plane offset in this column
    float acc[3] = {0.f, 0.f, 0.f};
    RingIdx<NS> ri{z0 - zlo};
    long long o = own_pl + (long long)z0 * plane;
    for (int k = z0; k < z1; ++k, o += plane, ri.next()) {
        R.wait(k + 1, d.err);
        __syncthreads();
        R.issue(k + NS - 2);
        if (!run) continue;
        const unsigned char *sk = R.stage(ri.s);
        const unsigned char *su = R.stage(ri.up(k == nz - 1)), *sd = R.stage(ri.dn(k == 0));
        auto D = [&](const unsigned char *st, int s) { return ((const float *)(st + RT_DX))[s]; };
        auto X = [&](const unsigned char *st, int s2, int s1) {   // x = phi (+ dx on later passes)
            const float2 v = ((const float2 *)(st + RT_X))[s2];
            const df p{v.x, v.y};
            return apply ? df_add_f(p, D(st, s1)) : p;
        };
        auto PA = [&](const unsigned char *st, int s) { return ((const float2 *)(st + RT_PA))[s]; };
        auto M_ = [&](const unsigned char *st, int s) {
            return UNI ? 0 : code_mat(((const uint32_t *)(st + RT_CODE))[s]);
        };
        RCell c;
        c.xc = X(sk, o2.c, o1.c);
        c.mc = M_(sk, o1.c); c.me = M_(sk, o1.e); c.mw = M_(sk, o1.w); c.mn = M_(sk, o1.n); c.ms = M_(sk, o1.s);
        c.mu = M_(su, o1.c); c.md = M_(sd, o1.c);
        if (upd) {
            c.dc = D(sk, o1.c); c.de = D(sk, o1.e); c.dw = D(sk, o1.w); c.dn = D(sk, o1.n);
            c.ds = D(sk, o1.s); c.du = D(su, o1.c); c.dd = D(sd, o1.c);
        } else {
            c.xe = X(sk, o2.e, o1.e); c.xw = X(sk, o2.w, o1.w); c.xn = X(sk, o2.n, o1.n); c.xs = X(sk, o2.s, o1.s);
            c.xu = X(su, o2.c, o1.c); c.xd = X(sd, o2.c, o1.c);
            c.pxe = PA(sk, o2.e).x; c.pxw = PA(sk, o2.w).x;
            c.pyn = PA(sk, o2.n).y; c.pys = PA(sk, o2.s).y;
            c.pzu = ((const float2 *)(su + RT_PZ))[tz].x;
            c.pzd = ((const float2 *)(sd + RT_PZ))[tz].x;
        }
        // identity rows: the Dirichlet planes, or the Neumann pin
        const bool ident = rc.neu ? (long long)k * plane == pin : (k == 0 || k == nz - 1);
        float rv;
        const float r_old = upd ? ((const float *)(sk + RT_PZ))[tz] : 0.f;
        refine_cell<UNI>(rc, k, ident, upd, c, r_old, UNI ? 0.f : ((const float *)(sk + RT_DINV))[tz], rv, acc);
        r[o] = rv;
        if (apply) nh[o] = make_float2(c.xc.h, c.xc.l);
    }
    refine_partials(d, acc, sRed);
    finish32<FB>(d, [&](int fi) { refine_film(d, fi, sRed, sTot); }, [&] { refine_grid(d); });
}


}  // namespace cmsl
