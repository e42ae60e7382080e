// kernels.cuh -- sm_103a kernels of the TDGL + Jacobi-PCG path.
//
// All stencil kernels share one scheme: a thread block owns a TX x TY column
// tile of one film and marches it through z (2.5D).  Each thread keeps its
// own column's values for planes k-1, k, k+1 in registers; plane k of every
// stencil field is staged with a one-cell halo in shared memory for the x/y
// neighbours.  Plane k+2 (own column) and the halo of plane k+1 are loaded
// while plane k is computed.  x/y are periodic; z is clamped or mirrored as
// in the reference.
//
// Reductions (PCG dots, sweep-row sums) are deterministic: block sums go to a
// per-item partial array and the last block of the grid (ticket counter)
// reduces each film's items in item order, then updates the film's scalars
// and, inside a CUDA graph, the WHILE-node conditions.  No block waits on
// another.
//
// Arithmetic policy M: Exact (FP64, every operation an explicitly rounded
// intrinsic in the reference's order, so results equal the reference kernels
// bit for bit) or Fast (FP32 with contraction to FMA).
#pragma once
#include <type_traits>
#include "cmsl_dev.cuh"
#include "dfloat.cuh"

namespace cmsl {

struct Exact {};
struct Fast {};

__device__ __forceinline__ double add(Exact, double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(Exact, double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(Exact, double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dvd(Exact, double a, double b) { return __ddiv_rn(a, b); }
template <class T> __device__ __forceinline__ T add(Fast, T a, T b) { return a + b; }
template <class T> __device__ __forceinline__ T sub(Fast, T a, T b) { return a - b; }
template <class T> __device__ __forceinline__ T mul(Fast, T a, T b) { return a * b; }
template <class T> __device__ __forceinline__ T dvd(Fast, T a, T b) { return a / b; }

template <class T> __device__ __forceinline__ const Coef<T> &coef_of(const FilmDev *f, int i);
template <> __device__ __forceinline__ const Coef<double> &coef_of<double>(const FilmDev *f, int i) { return f->coef[i]; }
template <> __device__ __forceinline__ const Coef<float> &coef_of<float>(const FilmDev *f, int i) { return f->coef32[i]; }
template <class T> __device__ __forceinline__ T inv_h2_of(const FilmDev *f);
template <> __device__ __forceinline__ double inv_h2_of<double>(const FilmDev *f) { return f->inv_h2; }
template <> __device__ __forceinline__ float inv_h2_of<float>(const FilmDev *f) { return f->inv_h2f; }
template <class T> __device__ __forceinline__ T epsf_of(const FilmDev *f, int i);
template <> __device__ __forceinline__ double epsf_of<double>(const FilmDev *f, int i) { return f->epsf[i]; }
template <> __device__ __forceinline__ float epsf_of<float>(const FilmDev *f, int i) { return f->epsf32[i]; }

// phi buffer by index without dynamically indexing the parameter array
__device__ __forceinline__ double *phi_sel(const Dev &d, int i)
{
    return i == 0 ? d.phi[0] : i == 1 ? d.phi[1] : i == 2 ? d.phi[2] : i == 3 ? d.phi[3] : d.phi[4];
}

// Potential storage: FP64 mode keeps doubles; FP32_REFINED keeps double-float
// (hi, lo) pairs, one float2 per cell.
template <class T> struct PhiAcc;
template <> struct PhiAcc<double> {
    using V = double;
    const double *p;
    __device__ __forceinline__ PhiAcc(const Dev &d, int buf, long long off) : p(phi_sel(d, buf) + off) {}
    __device__ __forceinline__ V ld(long long o) const { return p[o]; }
    static __device__ __forceinline__ V zero() { return 0.0; }
};
template <> struct PhiAcc<float> {
    using V = df;
    const float2 *p;
    __device__ __forceinline__ PhiAcc(const Dev &d, int buf, long long off) : p((const float2 *)phi_sel(d, buf) + off) {}
    __device__ __forceinline__ V ld(long long o) const { const float2 v = p[o]; return df{v.x, v.y}; }
    static __device__ __forceinline__ V zero() { return df{0.f, 0.f}; }
};
__device__ __forceinline__ float phi_diff(df a, df b)
{
    const df d = df_sub(a, b);
    return d.h + d.l;
}

// Asynchronous global -> shared copies (cp.async, 4 or 8 bytes, both
// addresses aligned to the size), grouped per commit; cp_wait<N> returns
// once at most N of this thread's groups are still in flight.  The copies
// carry no compiler memory clobber: their destinations are read only after
// cp_wait (which has one) and a barrier, and their sources are not written
// while they are in flight.
__device__ __forceinline__ void cp4(void *dst, const void *src)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src));
}
__device__ __forceinline__ void cp8(void *dst, const void *src)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ------------------------------------------------------------------ tiles
struct Geom {
    int nx, ny, nz, x0, y0, wx, wy;
    bool valid, halo;
    int own_slot, halo_slot;
    long long own_pl, halo_pl, plane;
};

template <int TYc = TY>
__device__ __forceinline__ Geom make_geom(const FilmDev *f, int x0, int y0)
{
    Geom g;
    g.nx = f->nx; g.ny = f->ny; g.nz = f->nz; g.x0 = x0; g.y0 = y0;
    g.plane = (long long)g.nx * g.ny;
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    g.wx = min(TX, g.nx - x0);
    g.wy = min(TYc, g.ny - y0);
    g.valid = lx < g.wx && ly < g.wy;
    g.own_slot = (ly + 1) * SX + lx + 1;
    g.own_pl = (long long)(x0 + lx) + (long long)g.nx * (y0 + ly);
    const int t = threadIdx.x;
    int hx = 0, hy = 0;
    g.halo = t < 2 * (g.wx + g.wy);
    if (t < g.wx) { hx = t; hy = -1; }
    else if (t < 2 * g.wx) { hx = t - g.wx; hy = g.wy; }
    else if (t < 2 * g.wx + g.wy) { hx = -1; hy = t - 2 * g.wx; }
    else { hx = g.wx; hy = t - 2 * g.wx - g.wy; }
    g.halo_slot = (hy + 1) * SX + hx + 1;
    const int gi = (x0 + hx + g.nx) % g.nx, gj = (y0 + hy + g.ny) % g.ny;
    g.halo_pl = (long long)gi + (long long)g.nx * gj;
    return g;
}

// ------------------------------------------------------------ reductions
template <class T> __device__ __forceinline__ T warp_sum(T v)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sums NV values over the block; the result is valid in thread 0.  Values are
// summed in T within a warp and in FP64 across warps, in warp order: thread
// i of the first warp sums value i, so the FP64 adds of all NV values issue
// together (FP64 instructions are scarce on this part).
template <int NV, class T>
__device__ __forceinline__ void block_sum(T (&v)[NV], double (*sm)[NV], double (&out)[NV])
{
    static_assert(NV <= 32, "one lane per value");
    static_assert(sizeof(T) <= sizeof(double), "warp sums are kept in sm");
    __shared__ double s_tot[NV];
    T *ws = (T *)&sm[0][0];                       // [warps][NV] warp sums
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
        const T s = warp_sum(v[i]);
        if (lane == 0) ws[w * NV + i] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        const int nw = (int)(blockDim.x >> 5);      // any block of up to NT threads
        double s = 0.0;
        for (int q = 0; q < nw; ++q) s += (double)ws[q * NV + threadIdx.x];
        s_tot[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        #pragma unroll
        for (int i = 0; i < NV; ++i) out[i] = s_tot[i];
    }
    __syncthreads();
}

// Ticket: true in every thread of the last block of the grid to arrive.
__device__ __forceinline__ bool ticket_last(unsigned int *counter)
{
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        // modulo: a stale counter can never leave a grid without a last block
        s_last = ((t + 1u) % gridDim.x) == 0u;
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last;
}

// Batches: true in every thread of the last block of film fi's stencil items
// to arrive.  That block forms the film's totals
// while the other films' blocks still run, instead of the grid's last block
// forming every film's one after another.
__device__ __forceinline__ bool film_ticket_last(const Dev &d, int fi)
{
    __shared__ bool s_flast;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const FilmDev *f = d.films + fi;
        const unsigned int n = (unsigned int)(f->sitem_end - f->sitem_begin);
        unsigned int *fc = d.counter + 4 + fi;
        const unsigned int t = atomicAdd(fc, 1u);
        s_flast = t + 1u == n;
        if (s_flast) *fc = 0u;                   // every block of the film has arrived
    }
    __syncthreads();
    if (s_flast) __threadfence();
    return s_flast;
}

// The end of an FP32 stencil pass has a film part (film fi's totals and
// state, every thread of one block) and a grid part (what depends on every
// film).  FB false: the grid's last block runs every film's part and the grid
// part.  FB true (kernels built for batches): each film's last block runs its
// film part while other films' blocks still run, and the grid's last block
// the grid part.  A compile-time choice: the single-film kernels keep their
// register allocation.
template <bool FB, class FilmFn, class GridFn>
__device__ __forceinline__ void finish32(const Dev &d, FilmFn film, GridFn grid)
{
    if constexpr (FB) {
        const int mine = d.sitems[blockIdx.x].x;
        for (int fi = 0; fi < d.n_films; ++fi)      // the loop form keeps the stencil loop's registers
            if (fi == mine && film_ticket_last(d, fi)) film(fi);
        if (!ticket_last(d.counter)) return;
    } else {
        if (!ticket_last(d.counter)) return;
        for (int fi = 0; fi < d.n_films; ++fi) film(fi);
    }
    grid();
}

// In the last block: sums the NV partials of film f's items (item order,
// thread-strided then block tree).  Result valid in thread 0.
template <int NV>
__device__ __forceinline__ void film_total(const Dev &d, const FilmDev *f, double (*sm)[NV],
                                           double (&out)[NV])
{
    double v[NV];
    #pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = 0.0;
    for (int it = f->item_begin + (int)threadIdx.x; it < f->item_end; it += (int)blockDim.x) {
        #pragma unroll
        for (int i = 0; i < NV; ++i) v[i] += __ldcg(d.partial + (long long)it * NPART + i);
    }
    block_sum<NV, double>(v, sm, out);
}

// FP32 passes: the partial sums of an item are double-float pairs (float2
// in the item's double slots) formed and added with FP32 instructions only,
// so that neither the blocks' epilogues nor the last block's film totals
// queue on the FP64 pipe.  The summation order is fixed (deterministic).
template <int NV>
__device__ __forceinline__ void block_partial32(const Dev &d, float (&v)[NV], double (*sm)[NV], double *part = nullptr)
{
    static_assert(NV <= 32, "one lane per value");
    float *ws = (float *)&sm[0][0];               // [warps][NV] warp sums
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
        const float s = warp_sum(v[i]);
        if (lane == 0) ws[w * NV + i] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        const int nw = (int)(blockDim.x >> 5);
        df s{0.f, 0.f};
        for (int q = 0; q < nw; ++q) s = df_add_f(s, ws[q * NV + threadIdx.x]);
        *(float2 *)((part ? part : d.partial) + (long long)blockIdx.x * NPART + threadIdx.x) = make_float2(s.h, s.l);
    }
    __syncthreads();
}

// In the last block: film f's totals of the block_partial32 pairs of its
// stencil items (Dev::sitems; item order: thread-strided U items a round,
// warp tree, then warps in order), valid in thread 0.  The last block runs
// alone at the end of its grid, so the sum is laid out for latency: every
// load of a round is issued before its sums, and the values' warp trees
// interleave.  OFF: the first slot; part: the partials (default the TDGL's).
template <int NV, int OFF = 0>
__device__ __forceinline__ void film_total32(const Dev &d, const FilmDev *f, double (*sm)[NV],
                                             double (&out)[NV], const double *part = nullptr)
{
    static_assert(OFF + NV <= NPART, "slots of an item");
    const double *pp = part ? part : d.partial;
    static_assert(NV <= 32 && sizeof(float2) == sizeof(double), "one lane and one slot per value");
    __shared__ double s_tot[NV];
    float2 *ws = (float2 *)&sm[0][0];             // [warps][NV] warp totals
    df v[NV];
    #pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = df{0.f, 0.f};
    const int b1 = f->sitem_end, stride = (int)blockDim.x;
    auto ld = [&](int it, int i) { return __ldcg((const float2 *)(pp + (long long)it * NPART + OFF + i)); };
    // U items a round, all their loads issued before the sums (about 16
    // values in flight per thread: one round for a 1536-item film's single
    // value instead of six)
    constexpr int U = 16 / NV > 8 ? 8 : (16 / NV < 2 ? 2 : 16 / NV);
    for (int it = f->sitem_begin + (int)threadIdx.x; it < b1; it += U * stride) {
        float2 p[U][NV];
        #pragma unroll
        for (int u = 0; u < U; ++u)
            #pragma unroll
            for (int i = 0; i < NV; ++i)
                p[u][i] = it + u * stride < b1 ? ld(it + u * stride, i) : make_float2(0.f, 0.f);
        #pragma unroll
        for (int u = 0; u < U; ++u)
            #pragma unroll
            for (int i = 0; i < NV; ++i) v[i] = df_add_acc(v[i], df{p[u][i].x, p[u][i].y});
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const df u{__shfl_down_sync(0xffffffffu, v[i].h, o), __shfl_down_sync(0xffffffffu, v[i].l, o)};
            v[i] = df_add_acc(v[i], u);
        }
        if (lane == 0) ws[w * NV + i] = make_float2(v[i].h, v[i].l);
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        const int nw = (int)(blockDim.x >> 5);
        df s{0.f, 0.f};
        for (int q = 0; q < nw; ++q) {
            const float2 p = ws[q * NV + threadIdx.x];
            s = df_add_acc(s, df{p.x, p.y});
        }
        s_tot[threadIdx.x] = (double)s.h + (double)s.l;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        #pragma unroll
        for (int i = 0; i < NV; ++i) out[i] = s_tot[i];
    }
    __syncthreads();
}

// Block-uniform read of a flag another block may have written.
__device__ __forceinline__ bool uniform_flag(const int *p)
{
    __shared__ int s_flag;
    __syncthreads();
    if (threadIdx.x == 0) s_flag = *(volatile const int *)p;
    __syncthreads();
    return s_flag != 0;
}

__device__ __forceinline__ void set_cond(const Dev &d, cudaGraphConditionalHandle h, int value)
{
    if (d.use_cond && h) cudaGraphSetConditional(h, value ? 1u : 0u);
}

// Step rs in a graph whose WHILE node runs the steps (one thread of the
// TDGL launch's last block): whether another step follows, and the entry
// value of the outer refinement loop (a handle's default is applied per
// graph launch, not per step).
__device__ __forceinline__ void step_begin(const Dev &d, int rs)
{
    set_cond(d, d.h_steps, rs + 1 < d.ctl->stop);
    set_cond(d, d.h_outer, 1);
}

// ------------------------------------------------------------- operator
// One row of A x = -div(eps grad x)/h^2 (depol_varEPS.cu:37-124).  Neighbour
// values and materials are passed in; Dirichlet planes and the Neumann pin
// are identity rows (x - g with g = 0).
template <class T, class M>
__device__ __forceinline__ T op_row(const FilmDev *f, int mc, int me, int mw, int mn, int ms,
                                    int mu, int md, T xc, T xe, T xw, T xn, T xs, T xu, T xd)
{
    const M m{};
    const T ex_p = epsf_of<T>(f, mc * 3 + me), ex_m = epsf_of<T>(f, mc * 3 + mw);
    const T ey_p = epsf_of<T>(f, mc * 3 + mn), ey_m = epsf_of<T>(f, mc * 3 + ms);
    const T ez_p = epsf_of<T>(f, mc * 3 + mu), ez_m = epsf_of<T>(f, mc * 3 + md);
    T a = sub(m, mul(m, ex_p, sub(m, xe, xc)), mul(m, ex_m, sub(m, xc, xw)));
    a = add(m, a, mul(m, ey_p, sub(m, xn, xc)));
    a = sub(m, a, mul(m, ey_m, sub(m, xc, xs)));
    a = add(m, a, mul(m, ez_p, sub(m, xu, xc)));
    a = sub(m, a, mul(m, ez_m, sub(m, xc, xd)));
    if constexpr (sizeof(T) == 8 && std::is_same<M, Exact>::value)
        a = dvd(m, a, (T)f->h2);
    else
        a = a * inv_h2_of<T>(f);
    return -a;
}

// Row kind of cell (k, plane index): 0 interior, 1 identity (Dirichlet plane
// or Neumann pin).
__device__ __forceinline__ bool identity_row(const FilmDev *f, int k, long long pl)
{
    if (f->zbc == 0) return k == 0 || k == f->nz - 1;
    return (pl + (long long)k * f->nx * f->ny) == (long long)f->ref_id;
}

// z neighbours of the operator (depol_varEPS.cu:86-99): returns the value to
// use for "up" and "down" given the loaded k+1 and k-1 values.
template <class V>
__device__ __forceinline__ void op_z(const FilmDev *f, int k, V up, V dn, V &u, V &dd)
{
    if (f->zbc == 0 || (k > 0 && k < f->nz - 1)) { u = up; dd = dn; }
    else if (k == 0) { u = up; dd = up; }
    else { u = dn; dd = dn; }
}

template <bool DF>
__device__ __forceinline__ void tdgl_finish(const Dev &d, int rs, double (*sRed)[7], double (&sTot)[7]);

// ---------------------------------------------------------- TDGL kernel
// kernelCalc_antiferro (kernels_evol.cu:47-231) + Calc_EfieldMag
// (depol_varEPS.cu:223-276) of the previous potential + the sweep-row sums
// of evolve.cu:256-357, fused; the old/new buffers ping-pong (no
// kernelUpdate_P copies).
template <class T, class M>
__global__ void __launch_bounds__(NT) k_tdgl(Dev d, Fields<T> F)
{
    using PV = typename PhiAcc<T>::V;
    __shared__ T sP[6][SPL];
    __shared__ PV sF[SPL];
    __shared__ Coef<T> sC[6];
    __shared__ double sRed[NT / 32][7];
    __shared__ double sTot[7];
    const M m{};
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    if (threadIdx.x < 6) sC[threadIdx.x] = coef_of<T>(f, threadIdx.x);
    const Geom g = make_geom(f, it.y, it.z);
    const int cur = d.ctl->cur, rs = d.ctl->run_step;
    const double Ez_ext = d.wave[(long long)it.x * d.wstride + rs];
    const T mEz = (T)(-Ez_ext);                   // dfdPmz_app, kernels_evol.cu:210
    const int row = d.rows[(long long)it.x * d.wstride + rs];
    const int dep = f->dep_flag, nz = g.nz;
    const long long off = f->off;
    const T *Po[6];
    T *Pn[6];
    #pragma unroll
    for (int q = 0; q < 6; ++q) { Po[q] = F.P[cur][q] + off; Pn[q] = F.P[cur ^ 1][q] + off; }
    const PhiAcc<T> phi(d, d.solve[it.x].phi_cur, off);
    const uint32_t *code = d.code + off;
    const double two_h = f->two_h;
    const float inv_2hf = f->inv_2hf;

    T cdn[6], ccu[6], cup[6], hv[6];
    PV fdn = PhiAcc<T>::zero(), fcu = fdn, fup = fdn, hf = fdn;
    if (g.valid) {
        const long long o = g.own_pl + (long long)z0 * g.plane;
        #pragma unroll
        for (int q = 0; q < 6; ++q) ccu[q] = Po[q][o];
        fcu = phi.ld(o);
        const long long od = g.own_pl + (long long)(z0 > 0 ? z0 - 1 : z0) * g.plane;
        const long long ou = g.own_pl + (long long)(z0 + 1 < nz ? z0 + 1 : z0) * g.plane;
        #pragma unroll
        for (int q = 0; q < 6; ++q) { cdn[q] = Po[q][od]; cup[q] = Po[q][ou]; }
        fdn = phi.ld(od); fup = phi.ld(ou);
    }
    if (g.halo) {
        const long long o = g.halo_pl + (long long)z0 * g.plane;
        #pragma unroll
        for (int q = 0; q < 6; ++q) hv[q] = Po[q][o];
        hf = phi.ld(o);
    }
    T acc[7];
    #pragma unroll
    for (int q = 0; q < 7; ++q) acc[q] = (T)0;

    for (int k = z0; k < z1; ++k) {
        __syncthreads();
        if (g.valid) {
            #pragma unroll
            for (int q = 0; q < 6; ++q) sP[q][g.own_slot] = ccu[q];
            sF[g.own_slot] = fcu;
        }
        if (g.halo) {
            #pragma unroll
            for (int q = 0; q < 6; ++q) sP[q][g.halo_slot] = hv[q];
            sF[g.halo_slot] = hf;
        }
        __syncthreads();
        T cnx[6];
        PV fnx = PhiAcc<T>::zero();
        const bool pre = g.valid && (k + 2 < nz) && (k + 1 < z1);
        if (pre) {
            const long long o = g.own_pl + (long long)(k + 2) * g.plane;
            #pragma unroll
            for (int q = 0; q < 6; ++q) cnx[q] = Po[q][o];
            fnx = phi.ld(o);
        }
        if (g.halo && k + 1 < z1) {
            const long long o = g.halo_pl + (long long)(k + 1) * g.plane;
            #pragma unroll
            for (int q = 0; q < 6; ++q) hv[q] = Po[q][o];
            hf = phi.ld(o);
        }
        if (g.valid) {
            const int s0 = g.own_slot;
            const long long o = g.own_pl + (long long)k * g.plane;
            const uint32_t c = code[o];
            const int gid = code_gid(c), mat = code_mat(c);
            const Coef<T> K = sC[mat * 2 + code_iface(c)];
            const T *trp = F.TR + 9LL * (f->g_off + gid);
            T t[9];
            #pragma unroll
            for (int q = 0; q < 9; ++q) t[q] = __ldg(trp + q);
            // neighbour sums e, w, n, s, u, d (kernels_evol.cu:101-122)
            T sum[6];
            #pragma unroll
            for (int q = 0; q < 6; ++q) {
                const T u = (k == nz - 1) ? ccu[q] : cup[q];
                const T dn = (k == 0) ? ccu[q] : cdn[q];
                T s = add(m, sP[q][s0 + 1], sP[q][s0 - 1]);
                s = add(m, s, sP[q][s0 + SX]);
                s = add(m, s, sP[q][s0 - SX]);
                s = add(m, s, u);
                sum[q] = add(m, s, dn);
            }
            // E_dep from the previous potential (depol_varEPS.cu:246-273)
            T ex = (T)0, ey = (T)0, ez = (T)0;
            if (dep) {
                PV pu, pd;
                if (f->zbc == 0) {
                    pu = (k == nz - 1) ? PhiAcc<T>::zero() : fup;
                    pd = (k == 0) ? PhiAcc<T>::zero() : fdn;
                } else {
                    op_z<PV>(f, k, fup, fdn, pu, pd);
                }
                if constexpr (std::is_same<M, Exact>::value) {
                    const double Ex = __ddiv_rn(-__dsub_rn(sF[s0 + 1], sF[s0 - 1]), two_h);
                    const double Ey = __ddiv_rn(-__dsub_rn(sF[s0 + SX], sF[s0 - SX]), two_h);
                    const double Ezd = __ddiv_rn(-__dsub_rn(pu, pd), two_h);
                    ex = (T)(-1.0 * Ex);
                    ey = (T)(-1.0 * Ey);
                    ez = (T)(-1.0 * Ezd);
                } else {
                    // -1 * E with E = -(phi_+ - phi_-) / (2h)
                    ex = (T)(phi_diff(sF[s0 + 1], sF[s0 - 1]) * inv_2hf);
                    ey = (T)(phi_diff(sF[s0 + SX], sF[s0 - SX]) * inv_2hf);
                    ez = (T)(phi_diff(pu, pd) * inv_2hf);
                }
            }
            // crystal frame (kernels_evol.cu:162-168)
            const T pMXl = add(m, add(m, mul(m, t[0], ccu[0]), mul(m, t[1], ccu[1])), mul(m, t[2], ccu[2]));
            const T pMYl = add(m, add(m, mul(m, t[3], ccu[0]), mul(m, t[4], ccu[1])), mul(m, t[5], ccu[2]));
            const T pMZl = add(m, add(m, mul(m, t[6], ccu[0]), mul(m, t[7], ccu[1])), mul(m, t[8], ccu[2]));
            const T pSXl = add(m, add(m, mul(m, t[0], ccu[3]), mul(m, t[1], ccu[4])), mul(m, t[2], ccu[5]));
            const T pSYl = add(m, add(m, mul(m, t[3], ccu[3]), mul(m, t[4], ccu[4])), mul(m, t[5], ccu[5]));
            const T pSZl = add(m, add(m, mul(m, t[6], ccu[3]), mul(m, t[7], ccu[4])), mul(m, t[8], ccu[5]));
            // two-sublattice Landau derivative (kernels_evol.cu:178-199)
            const T dmx = mul(m, K.a02, pMXl), dmy = mul(m, K.a02, pMYl);
            const T dsx = mul(m, K.a02, pSXl), dsy = mul(m, K.a02, pSYl);
            const T m2 = mul(m, pMZl, pMZl), m3 = mul(m, m2, pMZl), m4 = mul(m, m3, pMZl), m5 = mul(m, m4, pMZl);
            const T q2 = mul(m, pSZl, pSZl), q3 = mul(m, q2, pSZl), q4 = mul(m, q3, pSZl), q5 = mul(m, q4, pSZl);
            T dmz = add(m, mul(m, K.ag, pMZl), mul(m, K.b4, m3));
            dmz = add(m, dmz, mul(m, mul(m, K.b12, pMZl), q2));
            dmz = add(m, dmz, mul(m, K.g6, add(m, add(m, m5, mul(m, mul(m, (T)10.0, m3), q2)),
                                                mul(m, mul(m, (T)5.0, pMZl), q4))));
            T dsz = add(m, mul(m, K.ags, pSZl), mul(m, K.b4, q3));
            dsz = add(m, dsz, mul(m, mul(m, K.b12, pSZl), m2));
            dsz = add(m, dsz, mul(m, K.g6, add(m, add(m, q5, mul(m, mul(m, (T)10.0, m2), q3)),
                                                mul(m, mul(m, (T)5.0, pSZl), m4))));
            // back to the lab frame (kernels_evol.cu:202-208) + fields (:210-220)
            T b[6];
            b[0] = add(m, add(m, mul(m, t[0], dmx), mul(m, t[3], dmy)), mul(m, t[6], dmz));
            b[1] = add(m, add(m, mul(m, t[1], dmx), mul(m, t[4], dmy)), mul(m, t[7], dmz));
            b[2] = add(m, add(m, mul(m, t[2], dmx), mul(m, t[5], dmy)), mul(m, t[8], dmz));
            b[3] = add(m, add(m, mul(m, t[0], dsx), mul(m, t[3], dsy)), mul(m, t[6], dsz));
            b[4] = add(m, add(m, mul(m, t[1], dsx), mul(m, t[4], dsy)), mul(m, t[7], dsz));
            b[5] = add(m, add(m, mul(m, t[2], dsx), mul(m, t[5], dsy)), mul(m, t[8], dsz));
            b[0] = add(m, b[0], ex);
            b[1] = add(m, b[1], ey);
            b[2] = add(m, b[2], add(m, mEz, ez));
            // explicit Euler with the 6-neighbour Laplacian (kernels_evol.cu:223-229)
            T pn[6];
            #pragma unroll
            for (int q = 0; q < 6; ++q) {
                pn[q] = sub(m, add(m, mul(m, ccu[q], K.relax), mul(m, K.A, sum[q])), mul(m, K.LdT, b[q]));
                Pn[q][o] = pn[q];
            }
            if (row >= 0) {
                acc[0] += pn[2];
                acc[1] += pn[5];
                acc[2] += pMZl;
                acc[3] += pSZl;
                const T pz = pn[2];
                acc[4] += (mat == 1) ? pz : (T)0;
                acc[5] += (mat == 0) ? pz : (T)0;
                acc[6] += (mat == 2) ? pz : (T)0;
            }
        }
        if (g.valid) {
            #pragma unroll
            for (int q = 0; q < 6; ++q) { cdn[q] = ccu[q]; ccu[q] = cup[q]; }
            fdn = fcu; fcu = fup;
            if (pre) {
                #pragma unroll
                for (int q = 0; q < 6; ++q) cup[q] = cnx[q];
                fup = fnx;
            }
        }
    }

    // sweep-row partial sums of this item
    if (row >= 0) {
        double tot[7];
        block_sum<7, T>(acc, sRed, tot);
        if (threadIdx.x == 0) {
            #pragma unroll
            for (int q = 0; q < 7; ++q) d.partial[(long long)blockIdx.x * NPART + q] = tot[q];
        }
    }
    if (!ticket_last(d.counter)) return;
    tdgl_finish<false>(d, rs, sRed, sTot);
}

// Last block of a TDGL step: every film's sweep row from its items' partial
// sums (evolve.cu:256-357 scaled as in :391-400), and the per-step reset of
// the solver state.
// DF: the partials are block_partial32 pairs (FP32 kernel).
// Film fi's sweep row frow from the totals of its seven row sums (one thread).
template <int NV>
__device__ __forceinline__ void row_write(const Dev &d, int fi, int frow, const double (&sTot)[NV])
{
    const FilmDev *ff = d.films + fi;
    double *R = d.rowbuf + ((long long)fi * d.rstride + frow) * 11;
    const double N = (double)ff->nx * ff->ny * ff->nz;
    R[0] = sTot[0] * ff->inv_N;
    R[1] = sTot[1] * ff->inv_N;
    R[2] = sTot[2] * ff->inv_N;
    R[3] = sTot[3] * ff->inv_N;
    const double nFE = ff->n_mat[1], nAFE = ff->n_mat[0], nDE = ff->n_mat[2];
    R[4] = nFE > 0.0 ? sTot[4] / nFE : 0.0;
    R[5] = nFE > 0.0 ? nFE / N : 0.0;
    R[6] = nAFE > 0.0 ? sTot[5] / nAFE : 0.0;
    R[7] = nAFE > 0.0 ? nAFE / N : 0.0;
    R[8] = nDE > 0.0 ? sTot[6] / nDE : 0.0;
    R[9] = nDE > 0.0 ? nDE / N : 0.0;
    R[10] = (double)(d.ctl->step + 1);
}

// Film fi's solver state at the start of a step (one thread).
__device__ __forceinline__ void step_reset(const Dev &d, int fi)
{
    SolveDev *S = d.solve + fi;
    S->outer_active = d.films[fi].dep_flag ? 1 : 0;
    S->active = 0;
    S->status = 0;
    S->refine = 0;
    S->upd = 0;
    S->total_iters = 0;
    S->iters = 0;
}

// Reopens the step that step_end ended last (one thread): the counters and
// the P sets as they were before it, so that the residual pass that ends the
// step again advances them once more.
__device__ __forceinline__ void step_reopen(const Dev &d)
{
    d.ctl->step -= 1;
    d.ctl->run_step -= 1;
    d.ctl->cur ^= 1;
    d.ctl->redo = 1;
}

// The FP32 TDGL step's end (finish32): film fi's sweep row and the reset of
// its solver state; then the step's conditions.  Under kernel timing
// (d.force) the totals are formed as a step forms them and nothing is written.
__device__ __forceinline__ void tdgl_film32(const Dev &d, int rs, int fi, double (*sRed)[7], double (&sTot)[7])
{
    const int frow = d.rows[(long long)fi * d.wstride + rs];
    if (frow >= 0) {
        film_total32<7>(d, d.films + fi, sRed, sTot);
        if (threadIdx.x == 0 && !d.force) row_write(d, fi, frow, sTot);
    }
    if (threadIdx.x == 0 && !d.force) step_reset(d, fi);
}
__device__ __forceinline__ void tdgl_grid32(const Dev &d, int rs)
{
    if (threadIdx.x == 0) {
        if (!d.force) step_begin(d, rs);
        *d.counter = 0u;
    }
}

// Under kernel timing (d.force) the totals are formed as a step forms them
// and nothing is written.
template <bool DF>
__device__ __forceinline__ void tdgl_finish(const Dev &d, int rs, double (*sRed)[7], double (&sTot)[7])
{
    for (int fi = 0; fi < d.n_films; ++fi) {
        const FilmDev *ff = d.films + fi;
        const int frow = d.rows[(long long)fi * d.wstride + rs];
        if (frow >= 0) {
            if (DF) film_total32<7>(d, ff, sRed, sTot);
            else film_total<7>(d, ff, sRed, sTot);
            if (threadIdx.x == 0 && !d.force) row_write(d, fi, frow, sTot);
        }
        if (threadIdx.x == 0 && !d.force) step_reset(d, fi);
    }
    if (threadIdx.x == 0) {
        if (!d.force) step_begin(d, rs);
        *d.counter = 0u;
    }
}

// In the last block of a solve's set-up kernel (partials r.z, r.r, b.b per
// item): every film's starting scalars and the stop test of
// depol_varEPS.cu:447-474 (or the relative-residual test); drives the inner
// WHILE node.
__device__ __forceinline__ void start_solves(const Dev &d, double (*sRed)[3], double (&sTot)[3])
{
    int any = 0;
    for (int fi = 0; fi < d.n_films; ++fi) {
        const FilmDev *ff = d.films + fi;
        film_total<3>(d, ff, sRed, sTot);
        if (threadIdx.x == 0) {
            SolveDev *S = d.solve + fi;
            S->iters = 0;
            S->active = 0;
            S->status = 0;
            if (ff->dep_flag) {
                S->rz = S->rz0 = sTot[0];
                S->rr = sTot[1];
                S->bb = sTot[2];
                S->refine = 1;
                if (!isfinite(S->rz) || S->rz < 0.0) {
                    S->status = 2;
                } else if (ff->crit == 0) {
                    S->active = ff->max_iter > 0 && S->rz > ff->tol_abs2 &&
                                (S->rz0 <= 0.0 || (S->rz / S->rz0) > ff->tol_rel2);
                } else {
                    S->active = ff->max_iter > 0 && S->rr > ff->tol_rel2 * S->bb;
                }
                any |= S->active;
            }
        }
    }
    if (threadIdx.x == 0) {
        set_cond(d, d.h_inner, any);
        *d.counter = 0u;
    }
}

// ------------------------------------------------- FP64 solve: RHS + r0
// divergence (depol_varEPS.cu:279-329), b = -divP with zero rows on the
// Dirichlet planes / Neumann pin (:401-424), r = b - A x0 with the warm start
// x0 = phi (:429-445), z = D^-1 r, r.z (:447-460).  p = z is formed by the
// first k_spmv.
template <class T, class M>
__global__ void __launch_bounds__(NT) k_rhs(Dev d, Fields<T> F)
{
    __shared__ T sX[SPL], sY[SPL];
    __shared__ double sF[SPL];
    __shared__ int sM[SPL];
    __shared__ double sRed[NT / 32][3];
    __shared__ double sTot[3];
    const M m{};
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    const int nz = g.nz;
    const bool run = f->dep_flag != 0;
    const int cur = d.ctl->cur;
    const long long off = f->off;
    const T *Pmx = F.P[cur ^ 1][0] + off, *Pmy = F.P[cur ^ 1][1] + off, *Pmz = F.P[cur ^ 1][2] + off;
    const int pcur = d.solve[it.x].phi_cur;
    const double *x = phi_sel(d, pcur) + off;
    const uint32_t *code = d.code + off;
    T *r = F.r + off;
    const T *dinv = F.dinv + off;
    T acc[3] = {(T)0, (T)0, (T)0};
    if (run) {
        double xd = 0, xc = 0, xu = 0, hx = 0;
        T zd = 0, zc = 0, zu = 0, hPx = 0, hPy = 0;
        int md = 0, mc = 0, mu = 0, hm = 0;
        auto ld_own = [&](int k, double &xv, T &zv, int &mv) {
            const long long o = g.own_pl + (long long)k * g.plane;
            xv = x[o]; zv = Pmz[o]; mv = code_mat(code[o]);
        };
        if (g.valid) {
            ld_own(z0, xc, zc, mc);
            ld_own(z0 > 0 ? z0 - 1 : z0, xd, zd, md);
            ld_own(z0 + 1 < nz ? z0 + 1 : z0, xu, zu, mu);
        }
        auto ld_halo = [&](int k) {
            const long long o = g.halo_pl + (long long)k * g.plane;
            hx = x[o]; hPx = Pmx[o]; hPy = Pmy[o]; hm = code_mat(code[o]);
        };
        if (g.halo) ld_halo(z0);
        for (int k = z0; k < z1; ++k) {
            __syncthreads();
            if (g.valid) {
                const long long o = g.own_pl + (long long)k * g.plane;
                sF[g.own_slot] = xc; sX[g.own_slot] = Pmx[o]; sY[g.own_slot] = Pmy[o]; sM[g.own_slot] = mc;
            }
            if (g.halo) { sF[g.halo_slot] = hx; sX[g.halo_slot] = hPx; sY[g.halo_slot] = hPy; sM[g.halo_slot] = hm; }
            __syncthreads();
            double xn2 = 0; T zn2 = 0; int mn2 = 0;
            const bool pre = g.valid && (k + 2 < nz) && (k + 1 < z1);
            if (pre) ld_own(k + 2, xn2, zn2, mn2);
            if (g.halo && k + 1 < z1) ld_halo(k + 1);
            if (g.valid) {
                const int s0 = g.own_slot;
                const long long o = g.own_pl + (long long)k * g.plane;
                // b (divergence with z clamped)
                const T pzu = (k == nz - 1) ? zc : zu, pzd = (k == 0) ? zc : zd;
                T dv = add(m, add(m, sub(m, sX[s0 + 1], sX[s0 - 1]), sub(m, sY[s0 + SX], sY[s0 - SX])),
                           sub(m, pzu, pzd));
                dv = dvd(m, dv, (T)f->two_h);
                dv = mul(m, dv, (T)f->eps0nd);
                T b = mul(m, (T)-1.0, dv);
                T ax;
                if (identity_row(f, k, g.own_pl)) {
                    b = (T)0;
                    ax = (T)xc;   // x - g, g = 0
                } else {
                    double u, dd; int mmu, mmd;
                    op_z<double>(f, k, xu, xd, u, dd);
                    op_z<int>(f, k, mu, md, mmu, mmd);
                    ax = op_row<T, M>(f, mc, sM[s0 + 1], sM[s0 - 1], sM[s0 + SX], sM[s0 - SX], mmu, mmd,
                                      (T)xc, (T)sF[s0 + 1], (T)sF[s0 - 1], (T)sF[s0 + SX],
                                      (T)sF[s0 - SX], (T)u, (T)dd);
                }
                const T rv = sub(m, b, ax);
                r[o] = rv;
                const T z = mul(m, rv, dinv[o]);
                acc[0] += rv * z;
                acc[1] += rv * rv;
                acc[2] += b * b;
            }
            if (g.valid) {
                xd = xc; xc = xu; zd = zc; zc = zu; md = mc; mc = mu;
                if (pre) { xu = xn2; zu = zn2; mu = mn2; }
            }
        }
    }
    double tot[3];
    block_sum<3, T>(acc, sRed, tot);
    if (threadIdx.x == 0) {
        #pragma unroll
        for (int q = 0; q < 3; ++q) d.partial[(long long)blockIdx.x * NPART + q] = tot[q];
    }
    if (!ticket_last(d.counter)) return;
    start_solves(d, sRed, sTot);
}

// End of a time step (one block): every film's solve counts into the logs,
// the first failure into its sticky status, then the step counters and the
// P set advance.
__device__ __forceinline__ void step_end(const Dev &d)
{
    for (int fi = threadIdx.x; fi < d.n_films; fi += blockDim.x) {
        SolveDev *S = d.solve + fi;
        const long long w = (long long)fi * d.wstride + d.ctl->run_step;
        d.iters_log[w] = S->total_iters;
        d.refine_log[w] = S->refine + (S->pending ? 1 : 0);   // a deferred check counts as a pass
        if (S->status != 0 && S->status != 3 && S->sticky == 0) S->sticky = S->status;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        d.ctl->step += 1;
        d.ctl->run_step += 1;
        d.ctl->cur ^= 1;
    }
}

// ----------------------------- FP32 refinement: end of a residual pass
// The potential of CMSL_FP32_REFINED is stored as double-float ((hi, lo)
// pairs, one float2 per cell) in five rotating
// buffers: the current one, the three before it (extrapolated warm start) and
// a free one.  A residual pass (k_refine32, stencil32.cuh) forms r = b - A phi
// in double-float; in the last block this function takes every film's
// reduced r.r, b.b and r.D^-1.r, applies the refinement stop test
// ||r|| <= refine_tol ||b||, rotates the buffers and sets the next inner
// solve's target.
// Film fi's part (finish32): its totals, the stop test and its next pass.
__device__ __forceinline__ void refine_film(const Dev &d, int fi, double (*sRed)[3], double (&sTot)[3])
{
    if (d.force) {              // kernel timing: the totals as a pass forms them; the state stays as it is
        if (d.films[fi].dep_flag) film_total32<3>(d, d.films + fi, sRed, sTot, d.rpartial);
        return;
    }
    {
        const FilmDev *ff = d.films + fi;
        SolveDev *S = d.solve + fi;
        const bool was = ff->dep_flag != 0 && uniform_flag(&S->outer_active);
        if (was) film_total32<3>(d, ff, sRed, sTot, d.rpartial);
        if (threadIdx.x == 0 && was) {
            // an update pass (r <- r - A dx) leaves b.b as the last full pass formed it
            const bool was_upd = ff->upd_ok && S->upd && S->refine > 0;
            const double bb = was_upd ? S->bb : sTot[1];
            const int c0 = S->phi_cur, p0 = S->phi_prev, q0 = S->phi_prev2, r0 = S->phi_prev3;
            const int fr = 10 - c0 - p0 - q0 - r0;
            const bool first = S->refine == 0;
            if (first) {                     // keep phi_n .. phi_{n-2} for the next step's extrapolation
                S->phi_prev3 = q0;
                S->phi_prev2 = p0;
                S->phi_prev = c0;
                S->hist = min(S->hist + 1, 4);   // this step's potential joins the history
                (void)r0;                    // phi_{n-3} is no longer needed: it becomes the free buffer
            }
            S->phi_cur = fr;                 // this pass wrote the free buffer
            S->refine += 1;
            S->rr64 = sTot[0];
            S->bb = bb;
            const bool conv = sTot[0] <= ff->refine_tol2 * bb || sTot[0] == 0.0;
            // the next pass may update r when this one formed it in full and
            // ||r|| <= 1e-4 ||b||: the FP32 rounding of A dx (relative ~1e-7,
            // times the stencil's cancellation) then stays far below the
            // refinement target; never two update passes in a row
            S->upd = !was_upd && ff->upd_ok && sTot[0] <= 1e-8 * bb;
            // the next direct solve's increment (Chebyshev semi-iteration for a
            // direct solve preconditioning several eps, M^-1 A's spectrum in
            // [1 - delta, 1 + delta]): solve 0 of a step dx = M^-1 r, then
            // rho_k = 1 / (2 / delta - rho_{k-1}), dx_k = (2 rho_k / delta) M^-1 r
            // + rho_k rho_{k-1} dx_{k-1}
            {
                const double dl = ff->cheb_delta;
                if (dl <= 0.0 || S->refine == 1) {
                    S->cheb_rho = dl;
                    S->cheb_w = 1.f;
                    S->cheb_m = 0.f;
                } else {
                    const double rp = S->cheb_rho, rk = 1.0 / (2.0 / dl - rp);
                    S->cheb_rho = rk;
                    S->cheb_w = (float)(2.0 * rk / dl);
                    S->cheb_m = (float)(rk * rp);
                }
            }
            S->iters = 0;
            S->rz = S->rz0 = sTot[2];
            if (conv || !isfinite(sTot[0])) {
                S->outer_active = 0;
                S->active = 0;
                if (!isfinite(sTot[0])) S->status = 2;
            } else if (S->refine > ff->max_refine) {
                S->outer_active = 0;
                S->active = 0;
                S->status = 3;
            } else {
                S->active = isfinite(S->rz) && S->rz > 0.0;
                if (!S->active) { S->outer_active = 0; S->status = 2; }
                // inner target: just enough reduction to reach the refinement
                // tolerance in this pass (half-margin), between the FP32 floor
                // inner_tol and 1e-2
                double want = 0.25 * ff->refine_tol2 * bb / sTot[0];
                want = fmax(want, ff->inner_tol2);
                S->inner_tol2 = fmin(want, 1e-4);
                S->inner_max = ff->inner_max;
                // the step's first pass before an exact direct solve: the step
                // ends on that solve, and the next TDGL step forms the check
                // the update pass would have formed (SolveDev::pending)
                if (d.defer && ff->defer_ok && first && S->upd && S->active) {
                    S->pending = 1;
                    S->outer_active = 0;
                }
            }
        }
    }
}

// What depends on every film (finish32): the loop conditions, and the end of
// the step when no film continues (d.step_end).
__device__ __forceinline__ void refine_grid(const Dev &d)
{
    if (d.force) {
        if (threadIdx.x == 0) *d.counter = 0u;
        return;
    }
    // other blocks updated the films' slots (volatile: not from this block's L1)
    int any_outer = 0, any_inner = 0;
    if (threadIdx.x == 0)
        for (int fi = 0; fi < d.n_films; ++fi) {
            any_outer |= *(volatile const int *)&d.solve[fi].outer_active;
            any_inner |= *(volatile const int *)&d.solve[fi].active;
        }
    __shared__ int s_any;
    if (threadIdx.x == 0) {
        set_cond(d, d.h_outer, any_outer);
        set_cond(d, d.h_inner, any_inner);
        if (d.arrive) *d.arrive = 0u;
        *d.counter = 0u;
        s_any = any_outer;
    }
    __syncthreads();
    if (d.step_end && !s_any) step_end(d);
}

// ------------------------------------------- PCG: p-update + SpMV + p.Ap
// p = z + beta p (z = D^-1 r; p = z on the first iteration), q = A p,
// partial p.q (depol_varEPS.cu:478-492, 515-519).  p ping-pongs so that
// halo cells can be recomputed from the previous p.
template <class T, class M>
__global__ void __launch_bounds__(NT) k_spmv(Dev d, Fields<T> F)
{
    __shared__ T sP[SPL];
    __shared__ int sM[SPL];
    __shared__ double sRed[NT / 32][1];
    __shared__ double sTot[1];
    constexpr bool REFINE_T = sizeof(T) == 4;   // FP32 PCG runs only as the inner solve of a refinement
    const M m{};
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const SolveDev *S0 = d.solve + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    const int nz = g.nz;
    const bool run = d.force || S0->active != 0;
    const int par = S0->iters & 1;
    const bool first = S0->iters == 0;
    const T beta = (T)S0->beta;
    const long long off = f->off;
    const T *r = F.r + off, *dinv = F.dinv + off, *po = F.p[par] + off;
    T *pn = F.p[par ^ 1] + off, *q = F.q + off;
    const uint32_t *code = d.code + off;
    T acc[1] = {(T)0};
    if (run) {
        auto pnew = [&](long long o) {
            const T z = mul(m, r[o], dinv[o]);
            return first ? z : add(m, mul(m, beta, po[o]), z);
        };
        T pd = 0, pc = 0, pu = 0, hp = 0;
        int md = 0, mc = 0, mu = 0, hm = 0;
        auto ld_own = [&](int k, T &pv, int &mv) {
            const long long o = g.own_pl + (long long)k * g.plane;
            pv = pnew(o); mv = code_mat(code[o]);
        };
        if (g.valid) {
            ld_own(z0, pc, mc);
            ld_own(z0 > 0 ? z0 - 1 : z0, pd, md);
            ld_own(z0 + 1 < nz ? z0 + 1 : z0, pu, mu);
        }
        auto ld_halo = [&](int k) {
            const long long o = g.halo_pl + (long long)k * g.plane;
            hp = pnew(o); hm = code_mat(code[o]);
        };
        if (g.halo) ld_halo(z0);
        for (int k = z0; k < z1; ++k) {
            __syncthreads();
            if (g.valid) { sP[g.own_slot] = pc; sM[g.own_slot] = mc; }
            if (g.halo) { sP[g.halo_slot] = hp; sM[g.halo_slot] = hm; }
            __syncthreads();
            T pn2 = 0; int mn2 = 0;
            const bool pre = g.valid && (k + 2 < nz) && (k + 1 < z1);
            if (pre) ld_own(k + 2, pn2, mn2);
            if (g.halo && k + 1 < z1) ld_halo(k + 1);
            if (g.valid) {
                const int s0 = g.own_slot;
                const long long o = g.own_pl + (long long)k * g.plane;
                T qv;
                if (identity_row(f, k, g.own_pl)) {
                    qv = pc;
                } else {
                    T u, dd; int mmu, mmd;
                    op_z<T>(f, k, pu, pd, u, dd);
                    op_z<int>(f, k, mu, md, mmu, mmd);
                    qv = op_row<T, M>(f, mc, sM[s0 + 1], sM[s0 - 1], sM[s0 + SX], sM[s0 - SX], mmu, mmd,
                                      pc, sP[s0 + 1], sP[s0 - 1], sP[s0 + SX], sP[s0 - SX], u, dd);
                }
                pn[o] = pc;
                q[o] = qv;
                acc[0] += pc * qv;
            }
            if (g.valid) {
                pd = pc; pc = pu; md = mc; mc = mu;
                if (pre) { pu = pn2; mu = mn2; }
            }
        }
    }
    double tot[1];
    block_sum<1, T>(acc, sRed, tot);
    if (threadIdx.x == 0) d.partial[(long long)blockIdx.x * NPART] = tot[0];
    if (!ticket_last(d.counter)) return;
    for (int fi = 0; fi < d.n_films; ++fi) {
        const FilmDev *ff = d.films + fi;
        SolveDev *S = d.solve + fi;
        const bool was = uniform_flag(&S->active);
        if (was) film_total<1>(d, ff, sRed, sTot);
        if (threadIdx.x == 0 && was) {
            const double den = sTot[0];
            S->pq = den;
            if (!isfinite(den) || (!REFINE_T && !(den > 0.0))) {   // depol_varEPS.cu:486-490
                S->status = 1;
                S->active = 0;
                S->outer_active = 0;
            } else if (!(den > 0.0)) {
                // FP32 inner solve: p.Ap lost positivity to rounding; end this
                // pass, the outer refinement recomputes the true residual
                S->active = 0;
            } else {
                S->alpha = S->rz / den;
            }
        }
    }
    if (threadIdx.x == 0) *d.counter = 0u;
}

// ------------------------------------------- PCG: x, r update + r.z
// x += alpha p, r -= alpha Ap, z = D^-1 r, r.z (depol_varEPS.cu:492-521);
// decides whether the film continues and drives the inner WHILE node.
// refine_mode: x is the FP32 correction, overwritten on the first iteration.
template <class T, class M, bool REFINE>
__global__ void __launch_bounds__(NT) k_update(Dev d, Fields<T> F)
{
    __shared__ double sRed[NT / 32][2];
    __shared__ double sTot[2];
    const M m{};
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const SolveDev *S0 = d.solve + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    const bool run = d.force || S0->active != 0;
    const int par = S0->iters & 1;
    const bool first = S0->iters == 0;
    const T alpha = (T)S0->alpha, nalpha = (T)(-S0->alpha);
    const long long off = f->off;
    const T *p = F.p[par ^ 1] + off, *q = F.q + off, *dinv = F.dinv + off;
    T *r = F.r + off;
    T *x;
    if constexpr (REFINE) x = F.x + off;
    else {
        const int pcur = S0->phi_cur;
        x = (T *)(phi_sel(d, pcur) + off);
    }
    T acc[2] = {(T)0, (T)0};
    if (run && g.valid) {
        for (int k = z0; k < z1; ++k) {
            const long long o = g.own_pl + (long long)k * g.plane;
            const T pv = p[o];
            if (REFINE && first) x[o] = alpha * pv;
            else x[o] = add(m, x[o], mul(m, alpha, pv));
            const T rv = add(m, r[o], mul(m, nalpha, q[o]));
            r[o] = rv;
            const T z = mul(m, rv, dinv[o]);
            acc[0] += rv * z;
            acc[1] += rv * rv;
        }
    }
    double tot[2];
    block_sum<2, T>(acc, sRed, tot);
    if (threadIdx.x == 0) {
        d.partial[(long long)blockIdx.x * NPART] = tot[0];
        d.partial[(long long)blockIdx.x * NPART + 1] = tot[1];
    }
    if (!ticket_last(d.counter)) return;
    int any = 0;
    for (int fi = 0; fi < d.n_films; ++fi) {
        const FilmDev *ff = d.films + fi;
        SolveDev *S = d.solve + fi;
        const bool was = uniform_flag(&S->active);
        if (was) film_total<2>(d, ff, sRed, sTot);
        if (threadIdx.x == 0 && was) {
            S->iters += 1;
            S->total_iters += 1;
            const double rzn = sTot[0];
            S->rr = sTot[1];
            if (!isfinite(rzn) || rzn < 0.0) {          // depol_varEPS.cu:508-513
                S->status = 1;
                S->active = 0;
                S->outer_active = 0;
            } else {
                S->beta = rzn / S->rz;
                S->rz = rzn;
                if (REFINE) {
                    S->active = S->iters < S->inner_max && rzn > S->inner_tol2 * S->rz0 && rzn > 0.0;
                } else if (ff->crit == 0) {
                    S->active = S->iters < ff->max_iter && rzn > ff->tol_abs2 &&
                                (S->rz0 <= 0.0 || (rzn / S->rz0) > ff->tol_rel2);
                } else {
                    S->active = S->iters < ff->max_iter && S->rr > ff->tol_rel2 * S->bb;
                }
            }
            any |= S->active;
        }
    }
    if (threadIdx.x == 0) {
        set_cond(d, d.h_inner, any);
        *d.counter = 0u;
    }
}

// ------------------------------------------------------------ step end
static __global__ void k_step_end(Dev d)
{
    step_end(d);
}

// A fixed pseudo-random P of amplitude 0.05 (FP32 pairs, n floats) for the
// autotuner's trial steps on films that have no state yet.
static __global__ void k_trial_P(float *P, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        P[i] = 0.05f * ((float)(h & 0xffffu) / 32768.f - 1.f);
    }
}

// After the last step of a run (one thread): every film whose last step
// ended on its direct solve gets its check as an update pass.  That step is
// reopened, so that the residual pass that ends it again leaves the counters
// where the run left them; h_open (the IF node over those passes) is set
// when there is such a film.
static __global__ void k_defer_open(Dev d, cudaGraphConditionalHandle h_open)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int any = 0;
    for (int fi = 0; fi < d.n_films; ++fi) {
        SolveDev *S = d.solve + fi;
        if (!S->pending) continue;
        S->pending = 0;
        S->outer_active = 1;
        S->active = 0;
        S->refine = 1;
        S->upd = 1;
        any = 1;
    }
    if (any) step_reopen(d);
    else d.ctl->redo = 0;
    set_cond(d, h_open, any);
}

// ----------------------------------------------------------- utilities
// Jacobi diagonal inverse, built once per film (depol_varEPS.cu:126-180):
// exact FP64 arithmetic in the reference order, stored in T.
template <class T>
__global__ void k_dinv(Dev d, T *dinv)
{
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    if (!g.valid) return;
    const Exact m{};
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    const int i = g.x0 + lx, j = g.y0 + ly, nx = g.nx, ny = g.ny, nz = g.nz;
    const uint32_t *code = d.code + f->off;
    dinv += f->off;
    for (int k = z0; k < z1; ++k) {
        const long long o = g.own_pl + (long long)k * g.plane;
        double v = 1.0;
        if (!identity_row(f, k, g.own_pl)) {
            const int ip = (i + 1) % nx, im = (i - 1 + nx) % nx, jp = (j + 1) % ny, jm = (j - 1 + ny) % ny;
            int up = k + 1, dn = k - 1;
            if (f->zbc != 0) {
                if (k == 0) { up = 1; dn = 1; }
                else if (k == nz - 1) { up = nz - 2; dn = nz - 2; }
            }
            auto mt = [&](int a, int b, int c) { return code_mat(code[a + (long long)nx * (b + (long long)ny * c)]); };
            const int mc = code_mat(code[o]);
            const double e1 = f->epsf[mc * 3 + mt(ip, j, k)], e2 = f->epsf[mc * 3 + mt(im, j, k)];
            const double e3 = f->epsf[mc * 3 + mt(i, jp, k)], e4 = f->epsf[mc * 3 + mt(i, jm, k)];
            const double e5 = f->epsf[mc * 3 + mt(i, j, up)], e6 = f->epsf[mc * 3 + mt(i, j, dn)];
            double D = add(m, add(m, add(m, add(m, add(m, e1, e2), e3), e4), e5), e6);
            D = dvd(m, D, f->h2);
            v = (D > 1e-30 ? dvd(m, 1.0, D) : 1.0);
        }
        dinv[o] = (T)v;
    }
}

// y = A x on one film, one thread per cell, for the parity tests.
template <class T, class M>
__global__ void k_apply_op(Dev d, const T *x, T *y)
{
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    if (!g.valid) return;
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    const int i = g.x0 + lx, j = g.y0 + ly, nx = g.nx, ny = g.ny, nz = g.nz;
    const uint32_t *code = d.code + f->off;
    x += f->off;
    y += f->off;
    for (int k = z0; k < z1; ++k) {
        const long long o = g.own_pl + (long long)k * g.plane;
        if (identity_row(f, k, g.own_pl)) { y[o] = x[o]; continue; }
        const int ip = (i + 1) % nx, im = (i - 1 + nx) % nx, jp = (j + 1) % ny, jm = (j - 1 + ny) % ny;
        int up = k + 1, dn = k - 1;
        if (f->zbc != 0) {
            if (k == 0) { up = 1; dn = 1; }
            else if (k == nz - 1) { up = nz - 2; dn = nz - 2; }
        }
        auto id = [&](int a, int b, int c) { return a + (long long)nx * (b + (long long)ny * c); };
        const long long ie = id(ip, j, k), iw = id(im, j, k), in = id(i, jp, k), is = id(i, jm, k);
        const long long iu = id(i, j, up), idn = id(i, j, dn);
        y[o] = op_row<T, M>(f, code_mat(code[o]), code_mat(code[ie]), code_mat(code[iw]), code_mat(code[in]),
                            code_mat(code[is]), code_mat(code[iu]), code_mat(code[idn]), x[o], x[ie], x[iw],
                            x[in], x[is], x[iu], x[idn]);
    }
}

// E = -grad(phi) of the current potential (Calc_EfieldMag), for the tests.
static __global__ void k_efield(Dev d, double *Ex, double *Ey, double *Ez)
{
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    if (!g.valid) return;
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    const int i = g.x0 + lx, j = g.y0 + ly, nx = g.nx, ny = g.ny, nz = g.nz;
    const int pcur = d.solve[it.x].phi_cur;
    const double *phi = phi_sel(d, pcur) + f->off;
    Ex += f->off; Ey += f->off; Ez += f->off;
    const double two_h = f->two_h;
    for (int k = z0; k < z1; ++k) {
        const long long o = g.own_pl + (long long)k * g.plane;
        auto id = [&](int a, int b, int c) { return a + (long long)nx * (b + (long long)ny * c); };
        Ex[o] = __ddiv_rn(-__dsub_rn(phi[id((i + 1) % nx, j, k)], phi[id((i - 1 + nx) % nx, j, k)]), two_h);
        Ey[o] = __ddiv_rn(-__dsub_rn(phi[id(i, (j + 1) % ny, k)], phi[id(i, (j - 1 + ny) % ny, k)]), two_h);
        double pu, pd;
        if (f->zbc == 0) {
            pu = (k == nz - 1) ? 0.0 : phi[id(i, j, k + 1)];
            pd = (k == 0) ? 0.0 : phi[id(i, j, k - 1)];
        } else {
            const int up = (k == 0) ? 1 : (k == nz - 1 ? nz - 2 : k + 1);
            const int dn = (k == 0) ? 1 : (k == nz - 1 ? nz - 2 : k - 1);
            pu = phi[id(i, j, up)];
            pd = phi[id(i, j, dn)];
        }
        Ez[o] = __ddiv_rn(-__dsub_rn(pu, pd), two_h);
    }
}

// E = -grad(phi) of the double-float potential of CMSL_FP32_REFINED films
// ((hi, lo) pairs per cell): each value is formed as hi + lo in FP64, then
// differenced as in k_efield.
static __global__ void k_efield_df(Dev d, double *Ex, double *Ey, double *Ez)
{
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom g = make_geom(f, it.y, it.z);
    if (!g.valid) return;
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    const int i = g.x0 + lx, j = g.y0 + ly, nx = g.nx, ny = g.ny, nz = g.nz;
    const float2 *hl = (const float2 *)phi_sel(d, d.solve[it.x].phi_cur) + f->off;
    Ex += f->off; Ey += f->off; Ez += f->off;
    const double two_h = f->two_h;
    auto id = [&](int a, int b, int c) { return a + (long long)nx * (b + (long long)ny * c); };
    auto phi = [&](long long c) { const float2 v = hl[c]; return (double)v.x + (double)v.y; };
    for (int k = z0; k < z1; ++k) {
        const long long o = g.own_pl + (long long)k * g.plane;
        Ex[o] = __ddiv_rn(-__dsub_rn(phi(id((i + 1) % nx, j, k)), phi(id((i - 1 + nx) % nx, j, k))), two_h);
        Ey[o] = __ddiv_rn(-__dsub_rn(phi(id(i, (j + 1) % ny, k)), phi(id(i, (j - 1 + ny) % ny, k))), two_h);
        double pu, pd;
        if (f->zbc == 0) {
            pu = (k == nz - 1) ? 0.0 : phi(id(i, j, k + 1));
            pd = (k == 0) ? 0.0 : phi(id(i, j, k - 1));
        } else {
            const int up = (k == 0) ? 1 : (k == nz - 1 ? nz - 2 : k + 1);
            const int dn = (k == 0) ? 1 : (k == nz - 1 ? nz - 2 : k - 1);
            pu = phi(id(i, j, up));
            pd = phi(id(i, j, dn));
        }
        Ez[o] = __ddiv_rn(-__dsub_rn(pu, pd), two_h);
    }
}

}  // namespace cmsl
