// engine.cu -- film and batch lifecycle, CUDA-graph construction and the run loop.
//
// A handle holds F >= 1 independent films (a cmsl_film is a batch of one).
// Their cells, grains and work items are concatenated; every kernel launch
// covers all films, each work item carrying its film index, and every
// per-film quantity (solver scalars, convergence flags, waveform, sweep rows)
// lives in per-film device slots.  A run is one CUDA graph launch: a WHILE
// node over the steps whose body is one time step,
//   CMSL_FP64:          k_tdgl -> k_rhs -> WHILE(inner){ k_spmv -> k_update } -> k_step_end
//   CMSL_FP32_REFINED:  k_tdgl32 -> k_refine32 -> solve -> k_refine32
//                       -> WHILE(outer){ solve -> k_refine32 }
// where the FP32 inner solve is the direct spectral solve (films of one eps,
// spectral.cuh), or one persistent cooperative PCG launch over all films
// (each film on its own block range with its own convergence flag, under an
// IF node), or, for films with the Neumann z boundary, the residual pass
// followed by WHILE(inner){ k_spmv -> k_update } inside the outer WHILE.
// Converged films drop out of the masked kernels; a loop runs while any film
// is active.  The conditions are set on the device by the last block of
// k_tdgl32 / k_tdgl (the step loop), k_rhs, k_refine32 and k_update (the
// residual pass that leaves no film active also ends the step, in place of
// k_step_end), so a run never returns to the host: the
// PCG loop of the reference (depol_varEPS.cu:472-522, two blocking Ddot per
// iteration) and its per-step cudaMalloc/cublasCreate churn (:373-393,
// :585-593) are gone.  The applied field and the output-row schedule of the
// P-E loop are device arrays indexed by a device step counter, which the
// step loop's condition compares with the run's length.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cudaTypedefs.h>

#include "engine.h"
#include "cmsl_io.h"

using namespace cmsl;

namespace cmsl_eng {

namespace {
thread_local std::string g_err;
}

cmsl_status fail(cmsl_status s, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

}  // namespace cmsl_eng

using namespace cmsl_eng;

void cmsl_internal_set_error(const char *msg) { g_err = msg; }

namespace {

double harm(double a, double b)   // depol_varEPS.cu:10-15
{
    const double eps = 1e-20;
    double denom = a + b;
    if (denom < eps) denom = eps;
    return (2.0 * a * b) / denom;
}

}  // namespace

namespace {

// z chunk of the stencil items (xy_tiles: the column tiles of all films of
// the handle together); CMSL_ZCHUNK overrides.
int pick_zchunk(long long xy_tiles, int nz)
{
    const char *env = getenv("CMSL_ZCHUNK");
    if (env && atoi(env) > 0) return std::min(nz, atoi(env));
    // about 1.5 waves of the stencil passes (4 resident blocks on each of
    // 152 SMs), chunks of at least 8 planes: the ring prologue and the two
    // halo planes of a chunk cost more than the tail of a partial wave
    const long long target = 6LL * 152;
    const long long chunks = (target + xy_tiles - 1) / xy_tiles;
    int zc = (int)std::max<long long>(1, (nz + chunks - 1) / chunks);
    zc = std::max(zc, std::min(nz, 8));
    return std::min(zc, nz);
}

// Work items of every film for z chunk zc (0: pick_zchunk per film); how
// many there are, or the items themselves with each film's item range.
constexpr int ZCHUNK_MIN = 4;       // the finest chunk the autotuner tries

int film_zchunk(const Engine *e, int fi, int zc)
{
    const int nz = e->fh[fi].nz;
    return zc > 0 ? std::min(zc, nz) : pick_zchunk(e->xy_tiles, nz);
}

// A column of nz planes in chunks of at most c planes: ceil(nz / c) chunks
// whose sizes differ by one at most (chunk i starts at i * nz / nchunks), so
// that no short last chunk leaves blocks of the last wave idle.
int z_chunks(int nz, int c) { return (nz + c - 1) / c; }
int z_chunk_start(int nz, int nchunks, int i) { return (int)((long long)i * nz / nchunks); }

size_t count_items(const Engine *e, int zc, int ty = TY)
{
    size_t n = 0;
    for (int fi = 0; fi < e->n_films; ++fi) {
        const FilmHost &h = e->fh[fi];
        const int c = film_zchunk(e, fi, zc);
        n += (size_t)((h.nx + TX - 1) / TX) * ((h.ny + ty - 1) / ty) * z_chunks(h.nz, c);
    }
    return n;
}

// Rebuilds and uploads the items for z chunk zc (the graph is rebuilt at the
// next run).
cmsl_status set_items(Engine *e, int zc)
{
    if (count_items(e, zc) > e->items_cap || count_items(e, zc, e->stile_ty) > e->sitems_cap)
        return fail(CMSL_ERR_ARG, "z chunk %d: too many work items", zc);
    // the item kernels' list (TX x TY tiles) and the FP32 stencil passes'
    // list (TX x stile_ty tiles); the same z chunk
    for (int list = 0; list < 2; ++list) {
        std::vector<int4> &v = list ? e->sitems : e->items;
        const int ty = list ? e->stile_ty : TY;
        v.clear();
        for (int fi = 0; fi < e->n_films; ++fi) {
            const FilmHost &h = e->fh[fi];
            const int nc = z_chunks(h.nz, film_zchunk(e, fi, zc));
            FilmDev &fd = e->fdh[fi];
            (list ? fd.sitem_begin : fd.item_begin) = (int)v.size();
            for (int y0 = 0; y0 < h.ny; y0 += ty)
                for (int x0 = 0; x0 < h.nx; x0 += TX)
                    for (int i = 0; i < nc; ++i)
                        v.push_back(make_int4(fi, x0, y0, z_chunk_start(h.nz, nc, i) |
                                                              (z_chunk_start(h.nz, nc, i + 1) << 16)));
            (list ? fd.sitem_end : fd.item_end) = (int)v.size();
        }
    }
    CK(cudaMemcpy(e->d_films, e->fdh.data(), sizeof(FilmDev) * e->fdh.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_items, e->items.data(), sizeof(int4) * e->items.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_sitems, e->sitems.data(), sizeof(int4) * e->sitems.size(), cudaMemcpyHostToDevice));
    e->zchunk = zc;
    e->graph_valid = false;
    return CMSL_OK;
}

// Tile shapes tuned in this process, by film-shape class: the z chunk and
// the staging of the TDGL and of the residual passes.
struct Tuned {
    int zchunk;
    int stg_tdgl, stg_refine;
    int tile_y;                 // tile height of the FP32 stencil passes
};
std::map<std::string, Tuned> g_tuned;
std::mutex g_tuned_mu;

std::string shape_key(const Engine *e)
{
    std::string k = std::to_string(e->precision) + (e->spectral ? "s" : e->persistent ? "p" : "k");
    for (const FilmHost &h : e->fh)
        k += ":" + std::to_string(h.nx) + "x" + std::to_string(h.ny) + "x" + std::to_string(h.nz) + (h.dep ? "d" : "");
    return k;
}

// n = 2^a 3^b <= 4096 (the FFT radices of spectral.cuh)
bool spec_radix_ok(int n)
{
    if (n < 1 || n > 4096) return false;
    while (n % 3 == 0) n /= 3;
    while (n % 2 == 0) n /= 2;
    return n == 1;
}

SpecAxis spec_plan(int n)
{
    SpecAxis a{};
    a.n = n;
    a.lg = (n & (n - 1)) == 0 ? __builtin_ctz((unsigned)n) : -1;
    while (n % 3 == 0) { a.rad[a.nst++] = 3; n /= 3; }
    while (n % 2 == 0) { a.rad[a.nst++] = 2; n /= 2; }
    return a;
}

// Shared memory of the z solve per thread: the staged / eliminated plane
// pairs (16 bytes each) and the pivots (4 bytes per plane).
size_t spec_zbytes(int M) { return (size_t)16 * ((M + 1) / 2) + (size_t)4 * M; }

// Threads per block of the z solve: its shared memory stays within 96 KB;
// 0 if M is too large.
int spec_zthreads(int M)
{
    for (int t = 128; t >= 32; t /= 2)
        if ((size_t)t * spec_zbytes(M) <= 96 * 1024) return t;
    return 0;
}

template <class T> void fill_coef(Coef<T> &c, const cmsl_material &mt, int iface, double h, double dt)
{
    // kernels_evol.cu:139-153, :212, :223 -- reference operation order
    const double A_loc = mt.kappa * dt / (h * h);
    double g_loc = mt.g, Lfac = mt.L;
    if (iface) {
        g_loc *= 0.4;
        Lfac *= (1.0 + 10.0);
    }
    c.relax = (T)(1.0 - 6.0 * A_loc);
    c.A = (T)A_loc;
    c.LdT = (T)(Lfac * dt);
    c.ag = (T)(2.0 * (mt.alpha + g_loc));
    c.ags = (T)(2.0 * (mt.alpha - g_loc));
    c.b4 = (T)(4.0 * mt.beta);
    c.b12 = (T)(12.0 * mt.beta);
    c.g6 = (T)(6.0 * mt.gamma);
    c.a02 = (T)(2.0 * mt.a0);
}

// Permittivities of the materials a film's grains use: the reference value
// of its direct solve (the middle of their range, which minimises the
// spectral radius of I - M^-1 A for M = eps_ref times the Laplacian, the
// discrete operator's face permittivities lying between the smallest and the
// largest) and the ratio largest / smallest.
double spec_eps_ref(const cmsl_film_desc &d, double *kappa)
{
    bool used[3] = {false, false, false};
    for (int g = 0; g < d.n_grains; ++g)
        if (d.grain_mat[g] >= 0 && d.grain_mat[g] <= 2) used[d.grain_mat[g]] = true;
    double lo = 0.0, hi = 0.0;
    bool any = false;
    for (int m = 0; m < 3; ++m) {
        if (!used[m]) continue;
        const double e = d.mats[m].eps_r;
        lo = any ? std::min(lo, e) : e;
        hi = any ? std::max(hi, e) : e;
        any = true;
    }
    if (!any || !(lo > 0.0)) {
        if (kappa) *kappa = 1.0;
        return d.mats[0].eps_r;
    }
    if (kappa) *kappa = hi / lo;
    return 0.5 * (lo + hi);
}

// Several permittivities with the direct solve: the solve is a
// preconditioner (M = eps_ref times the Laplacian) of the double-float
// refinement, whose increments follow the Chebyshev semi-iteration for M^-1
// A's spectrum [1 - delta, 1 + delta], delta = (kappa - 1) / (kappa + 1):
// the residual contracts by about (sqrt(kappa) - 1) / (sqrt(kappa) + 1) per
// pass; CMSL_INNER_AUTO takes it up to this ratio of permittivities.
constexpr double SPEC_PRECOND_KAPPA = 16.0;

// Refinement passes such a film may take: enough for the plain (fixed-step)
// contraction (kappa - 1) / (kappa + 1) to reach the refinement target from
// a zero start, plus a margin -- a safe bound for the Chebyshev iteration.
int spec_precond_refine_cap(double kappa, double refine_tol)
{
    // twice the Chebyshev estimate, and never fewer than plain Richardson's passes would need
    const double rho = (kappa - 1.0) / (kappa + 1.0);
    const double tol = refine_tol > 0.0 ? std::min(refine_tol, 1e-2) : 1e-8;
    const double n = rho > 0.0 ? std::ceil(std::log(tol) / std::log(rho)) : 1.0;
    return (int)std::min(500.0, std::max(16.0, n + 8.0));
}

// The film-constant table of one film (set-up of main.cu:261-359 and
// depol_varEPS.cu:126-180 reduced to per-material constants).
void fill_film(FilmDev &fd, const cmsl_film_desc *dsc, int precision)
{
    fd.nx = dsc->nx; fd.ny = dsc->ny; fd.nz = dsc->nz; fd.zbc = dsc->zbc;
    fd.dep_flag = dsc->dep_flag != 0;
    fd.warm = precision != CMSL_FP64 ? std::min(std::max(dsc->warm_start, 0), 3) : 0;
    fd.ref_id = dsc->nx / 2 + dsc->nx * (dsc->ny / 2 + (dsc->nz / 2) * dsc->ny);   // depol_varEPS.cu:339-346
    fd.crit = dsc->pcg_crit;
    fd.max_iter = dsc->max_iter;
    fd.max_refine = std::max(1, dsc->max_refine);
    fd.inner_max = std::max(1, dsc->inner_max_iter);
    const double h = dsc->del_h;
    fd.h = h; fd.dt = dsc->del_t; fd.eps0nd = dsc->eps_0_nd;
    fd.inv_N = 1.0 / ((double)dsc->nx * dsc->ny * dsc->nz);              // main.cu:405
    fd.two_h = 2.0 * h; fd.h2 = h * h; fd.inv_h2 = 1.0 / (h * h); fd.inv_2h = 1.0 / (2.0 * h);
    fd.inv_h2f = (float)fd.inv_h2; fd.inv_2hf = (float)fd.inv_2h; fd.eps0f = (float)dsc->eps_0_nd;
    {
        const df cb = df_from_double(dsc->eps_0_nd * fd.inv_2h);
        fd.cb_h = cb.h; fd.cb_l = cb.l;
    }
    fd.tol_abs2 = dsc->tol_abs * dsc->tol_abs;
    fd.tol_rel2 = dsc->tol_rel * dsc->tol_rel;
    fd.refine_tol2 = dsc->refine_tol * dsc->refine_tol;
    fd.inner_tol2 = dsc->inner_tol * dsc->inner_tol;
    fd.uni_eps = dsc->mats[0].eps_r == dsc->mats[1].eps_r && dsc->mats[1].eps_r == dsc->mats[2].eps_r;
    {
        // depol_varEPS.cu:177-179 with six equal faces
        const double e = harm(dsc->mats[0].eps_r, dsc->mats[0].eps_r);
        const double D = (e + e + e + e + e + e) / (h * h);
        fd.dinv_uni = (float)(D > 1e-30 ? 1.0 / D : 1.0);
    }
    for (int mt = 0; mt < 3; ++mt)
        for (int fl = 0; fl < 2; ++fl) {
            fill_coef<double>(fd.coef[mt * 2 + fl], dsc->mats[mt], fl, h, dsc->del_t);
            fill_coef<float>(fd.coef32[mt * 2 + fl], dsc->mats[mt], fl, h, dsc->del_t);
        }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            fd.epsf[a * 3 + b] = harm(dsc->mats[a].eps_r, dsc->mats[b].eps_r);
            fd.epsf32[a * 3 + b] = (float)fd.epsf[a * 3 + b];
            const df c = df_from_double(fd.epsf[a * 3 + b] * fd.inv_h2);
            fd.cf_h[a * 3 + b] = c.h; fd.cf_l[a * 3 + b] = c.l;
        }
}

cmsl_status check_desc(const cmsl_film_desc *dsc, int idx, int n)
{
    char who[32] = "";
    if (n > 1) snprintf(who, sizeof who, "film %d: ", idx);
    if (dsc->nx < 1 || dsc->ny < 1 || dsc->nz < 3)
        return fail(CMSL_ERR_ARG, "%sgrid %dx%dx%d: need nx, ny >= 1 and nz >= 3", who, dsc->nx, dsc->ny, dsc->nz);
    if (dsc->nx > 32767 || dsc->ny > 32767 || dsc->nz > 32767)
        return fail(CMSL_ERR_ARG, "%sgrid dimension above 32767", who);
    if (dsc->n_grains < 1 || dsc->n_grains > (int)GID_MASK)
        return fail(CMSL_ERR_ARG, "%sn_grains %d out of range", who, dsc->n_grains);
    if (!dsc->omega || !dsc->grain_mat || !dsc->TR) return fail(CMSL_ERR_ARG, "%somega/grain_mat/TR NULL", who);
    if (dsc->precision != CMSL_FP64 && dsc->precision != CMSL_FP32_REFINED)
        return fail(CMSL_ERR_ARG, "%sprecision %d unknown", who, dsc->precision);
    if (dsc->zbc != CMSL_DIRICHLET && dsc->zbc != CMSL_NEUMANN) return fail(CMSL_ERR_ARG, "%szbc %d", who, dsc->zbc);
    if (dsc->inner_solver < CMSL_INNER_AUTO || dsc->inner_solver > CMSL_INNER_DIRECT)
        return fail(CMSL_ERR_ARG, "%sinner_solver %d unknown", who, dsc->inner_solver);
    if (!(dsc->del_h > 0.0) || !(dsc->del_t > 0.0)) return fail(CMSL_ERR_ARG, "%sdel_h and del_t must be > 0", who);
    for (int g = 0; g < dsc->n_grains; ++g)
        if (dsc->grain_mat[g] < 0 || dsc->grain_mat[g] > 2)
            return fail(CMSL_ERR_ARG, "%sgrain %d has material %d (need 0..2)", who, g, dsc->grain_mat[g]);
    return CMSL_OK;
}

// Rotations per grain: 9 values (FP64), or 9 values and 3 zeros (FP32: three
// 16-byte loads per cell in the TDGL step).
template <class T> cmsl_status upload_TR(Engine *e, const cmsl_film_desc *descs, int n)
{
    constexpr int stride = sizeof(T) == 4 ? TR32 : 9;
    std::vector<T> tr;
    for (int i = 0; i < n; ++i)
        for (int g = 0; g < descs[i].n_grains; ++g)
            for (int q = 0; q < stride; ++q) tr.push_back(q < 9 ? (T)descs[i].TR[9 * g + q] : (T)0);
    TRY(e->alloc(&e->d_TR, tr.size() * sizeof(T)));
    CK(cudaMemcpy(e->d_TR, tr.data(), tr.size() * sizeof(T), cudaMemcpyHostToDevice));
    return CMSL_OK;
}

}  // namespace

namespace cmsl_eng {

cmsl_status ensure_schedule(Engine *e, int n_steps, int n_rows)
{
    const size_t F = (size_t)e->n_films;
    if (n_steps > e->wstride) {
        const int w = std::max(n_steps, 16);
        if (e->d_wave) { cudaFree(e->d_wave); cudaFree(e->d_rows); cudaFree(e->d_iters); cudaFree(e->d_refine); }
        e->d_wave = nullptr; e->d_rows = nullptr; e->d_iters = nullptr; e->d_refine = nullptr;
        CK(cudaMalloc(&e->d_wave, sizeof(double) * w * F));
        CK(cudaMalloc(&e->d_rows, sizeof(int) * w * F));
        CK(cudaMalloc(&e->d_iters, sizeof(int) * w * F));
        CK(cudaMalloc(&e->d_refine, sizeof(int) * w * F));
        e->wstride = w;
        e->graph_valid = false;
    }
    if (n_rows > e->rstride || !e->d_rowbuf) {
        const int r = std::max(n_rows, 16);
        if (e->d_rowbuf) cudaFree(e->d_rowbuf);
        e->d_rowbuf = nullptr;
        CK(cudaMalloc(&e->d_rowbuf, sizeof(double) * 11 * r * F));
        CK(cudaMemset(e->d_rowbuf, 0, sizeof(double) * 11 * r * F));
        e->rstride = r;
        e->graph_valid = false;
    }
    return CMSL_OK;
}

constexpr int CG_TIMING_ITERS = 50;

struct KArgs {
    Dev d;
    Fields<double> F64;
    Fields<float> F32;
};

cmsl_status add_kernel(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *dep, int ndep,
                       void *fn, int grid, int block, void **args, size_t smem)
{
    cudaKernelNodeParams kp{};
    kp.func = fn;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.sharedMemBytes = (unsigned int)smem;
    kp.kernelParams = args;
    kp.extra = nullptr;
    CK(cudaGraphAddKernelNode(node, g, dep, ndep, &kp));
    return CMSL_OK;
}

cmsl_status add_while(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *dep, int ndep,
                      cudaGraphConditionalHandle h, cudaGraph_t *body)
{
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    CK(cudaGraphAddNode(node, g, dep, nullptr, ndep, &cp));
    *body = cp.conditional.phGraph_out[0];
    return CMSL_OK;
}

cmsl_status add_if(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *dep, int ndep,
                   cudaGraphConditionalHandle h, cudaGraph_t *body)
{
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    CK(cudaGraphAddNode(node, g, dep, nullptr, ndep, &cp));
    *body = cp.conditional.phGraph_out[0];
    return CMSL_OK;
}

// Arguments must outlive graph instantiation only (node params are copied).
cmsl_status build_graph(Engine *e)
{
    if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
    if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
    cudaGraph_t top, g;
    CK(cudaGraphCreate(&top, 0));
    e->graph = top;
    // One launch runs the steps of a run: a WHILE node whose body is one
    // step; the TDGL kernel sets its condition (run_step + 1 < ctl->stop).
    cudaGraphConditionalHandle h_steps = 0;
    cudaGraphNode_t n_loop;
    CK(cudaGraphConditionalHandleCreate(&h_steps, top, 1, cudaGraphCondAssignDefault));
    TRY(add_while(top, &n_loop, nullptr, 0, h_steps, &g));
    auto dev = [&](cudaGraphConditionalHandle hi, cudaGraphConditionalHandle ho) {
        Dev d = e->dev(1, hi, ho);
        d.h_steps = h_steps;
        return d;
    };
    const int nit = (int)e->items.size();
    const int nsit = (int)e->sitems.size();        // the FP32 stencil passes' blocks
    KArgs a;
    a.F64 = e->fields<double>();
    a.F32 = e->fields<float>();
    cudaGraphConditionalHandle h_outer = 0, h_inner = 0;
    const bool fp64 = e->precision == CMSL_FP64;
    cudaGraphNode_t n_tdgl, n_solve, n_end;
    if (!fp64 && e->any_dep) CK(cudaGraphConditionalHandleCreate(&h_outer, g, 1, cudaGraphCondAssignDefault));
    if (fp64 && e->any_dep) CK(cudaGraphConditionalHandleCreate(&h_inner, g, 0, cudaGraphCondAssignDefault));
    a.d = dev(h_inner, h_outer);
    void *args64[] = {&a.d, &a.F64};
    void *args32[] = {&a.d, &a.F32};
    void *args_d[] = {&a.d};
    void *a_x[] = {&a.d, &a.F32, &e->spec};
    void *a_s[] = {&a.d, &e->spec};
    void *a_cg[] = {&a.d, &e->cg, &e->d_dinv};
    // the inner solve of one pass, after *dep (or first in graph gs)
    auto add_solve = [&](cudaGraph_t gs, const cudaGraphNode_t *dep, cudaGraphNode_t *out) -> cmsl_status {
        if (e->persistent) {
            TRY(add_kernel(gs, out, dep, dep ? 1 : 0, e->cg_fn, e->cg_grid, PNT, a_cg, e->cg_smem));
            cudaLaunchAttributeValue av{};
            av.cooperative = 1;
            CK(cudaGraphKernelNodeSetAttribute(*out, cudaLaunchAttributeCooperative, &av));
            return CMSL_OK;
        }
        struct Node { void *fn; int grid, block; void **args; size_t smem; };
        const Node rows[] = {
            {(void *)k_spec_x<true>, e->spec_grid[0], SPEC_NT, a_x, e->spec_smem[0]},
            {(void *)k_spec_y, e->spec_grid[1], SPEC_NT, a_s, e->spec_smem[1]},
            {(void *)k_spec_z<false>, e->spec_grid[2], e->spec_zt, a_s, e->spec_smem[2]},
            {(void *)k_spec_y, e->spec_grid[1], SPEC_NT, a_s, e->spec_smem[1]},
            {(void *)k_spec_x<false>, e->spec_grid[0], SPEC_NT, a_x, e->spec_smem[0]}};
        const Node cols[] = {
            {(void *)k_spec_x<true, true>, e->spec_grid[0], SPEC_NT, a_x, e->spec_smem[0]},
            {(void *)k_spec_yzy, e->spec_grid[3], SPEC_YZY_NT, a_s, e->spec_smem[3]},
            {(void *)k_spec_x<false, true>, e->spec_grid[0], SPEC_NT, a_x, e->spec_smem[0]}};
        const Node clus[] = {
            {(void *)k_spec_cxy, e->spec_grid[4], SPEC_CL_NT, a_x, e->spec_smem[4]},
            {(void *)k_spec_z<true>, e->spec_grid[2], e->spec_zt, a_s, e->spec_smem[2]},
            {(void *)k_spec_cyx, e->spec_grid[4], SPEC_CL_NT, a_x, e->spec_smem[4]}};
        const Node *seq = e->spec_cl ? clus : e->spec_col ? cols : rows;
        const int nseq = e->spec_cl || e->spec_col ? 3 : 5;
        const cudaGraphNode_t *prev = dep;
        for (int qi = 0; qi < nseq; ++qi) {
            const Node &q = seq[qi];
            TRY(add_kernel(gs, out, prev, prev ? 1 : 0, q.fn, q.grid, q.block, q.args, q.smem));
            prev = out;
        }
        return CMSL_OK;
    };
    if (fp64) TRY(add_kernel(g, &n_tdgl, nullptr, 0, (void *)k_tdgl<double, Exact>, nit, NT, args64));
    else TRY(add_kernel(g, &n_tdgl, nullptr, 0, e->tdgl_fn, nsit, e->tdgl_nt, args32, e->tdgl_smem));
    cudaGraphNode_t last = n_tdgl;
    if (e->any_dep) {
        if (fp64) {
            cudaGraphNode_t n_rhs, n_sp, n_up;
            cudaGraph_t body;
            TRY(add_kernel(g, &n_rhs, &last, 1, (void *)k_rhs<double, Exact>, nit, NT, args64));
            TRY(add_while(g, &n_solve, &n_rhs, 1, h_inner, &body));
            TRY(add_kernel(body, &n_sp, nullptr, 0, (void *)k_spmv<double, Exact>, nit, NT, args64));
            TRY(add_kernel(body, &n_up, &n_sp, 1, (void *)k_update<double, Exact, false>, nit, NT, args64));
            last = n_solve;
        } else if (e->spectral || e->persistent) {
            // A step almost always takes two refinement passes (the warm
            // start's residual, then the check after one inner solve), so
            // they are laid out flat: pass -> solve -> pass -> WHILE(some
            // film not converged) { solve -> pass } for the rare further
            // passes.  The direct solve's kernels skip converged films; the
            // cooperative PCG launch sits under an IF node.  (Programmatic
            // edges along this chain measured no gain.)  With deferred
            // checks the second pass of a step moves into the next TDGL
            // step, and the passes after the solve sit under an IF node.
            cudaGraphNode_t n_r1, n_s1, n_r2, n_sb, n_rb;
            cudaGraph_t body;
            if (e->persistent) CK(cudaGraphConditionalHandleCreate(&h_inner, g, 0, cudaGraphCondAssignDefault));
            a.d = dev(h_inner, h_outer);
            if (e->defer) {
                // deferred checks: pass -> solve (which ends the step when no
                // film continues) -> IF(some film continues) { pass ->
                // WHILE(some film not converged) { solve -> pass } }
                cudaGraph_t cont;
                cudaGraphNode_t n_if, n_w;
                cudaGraphConditionalHandle h_cont = 0;
                a.d.defer = 1;
                TRY(add_kernel(g, &n_r1, &last, 1, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
                a.d.step_end = 1;
                TRY(add_solve(g, &n_r1, &n_s1));
                TRY(add_if(g, &n_if, &n_s1, 1, h_outer, &cont));
                CK(cudaGraphConditionalHandleCreate(&h_cont, cont, 0, cudaGraphCondAssignDefault));
                a.d = dev(0, h_cont);
                a.d.defer = 1;
                a.d.step_end = 1;
                TRY(add_kernel(cont, &n_r2, nullptr, 0, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
                TRY(add_while(cont, &n_w, &n_r2, 1, h_cont, &body));
                a.d.step_end = 0;
                TRY(add_solve(body, nullptr, &n_sb));
                a.d.step_end = 1;
                TRY(add_kernel(body, &n_rb, &n_sb, 1, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
                last = nullptr;
            } else {
                TRY(add_kernel(g, &n_r1, &last, 1, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
                if (e->persistent) {
                    cudaGraph_t solve1;
                    cudaGraphNode_t n_c1;
                    TRY(add_if(g, &n_s1, &n_r1, 1, h_inner, &solve1));
                    TRY(add_solve(solve1, nullptr, &n_c1));
                } else {
                    TRY(add_solve(g, &n_r1, &n_s1));
                }
                // the pass that leaves no film active ends the step (no k_step_end node)
                a.d.step_end = 1;
                TRY(add_kernel(g, &n_r2, &n_s1, 1, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
                TRY(add_while(g, &n_solve, &n_r2, 1, h_outer, &body));
                a.d = dev(0, h_outer);
                a.d.step_end = 1;
                TRY(add_solve(body, nullptr, &n_sb));
                TRY(add_kernel(body, &n_rb, &n_sb, 1, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
                last = nullptr;
            }
        } else {
            // the inner loop's handle belongs to the outer body graph it lives in
            cudaGraph_t outer, inner;
            cudaGraphNode_t n_ref, n_in, n_sp, n_up;
            TRY(add_while(g, &n_solve, &last, 1, h_outer, &outer));
            CK(cudaGraphConditionalHandleCreate(&h_inner, outer, 0, cudaGraphCondAssignDefault));
            a.d = dev(h_inner, h_outer);
            TRY(add_kernel(outer, &n_ref, nullptr, 0, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
            TRY(add_while(outer, &n_in, &n_ref, 1, h_inner, &inner));
            TRY(add_kernel(inner, &n_sp, nullptr, 0, (void *)k_spmv<float, Fast>, nit, NT, args32));
            TRY(add_kernel(inner, &n_up, &n_sp, 1, (void *)k_update<float, Fast, true>, nit, NT, args32));
            last = n_solve;
        }
    }
    if (last) TRY(add_kernel(g, &n_end, &last, 1, (void *)k_step_end, 1, 32, args_d));
    if (e->defer) {
        // after the last step: the checks still pending run as update passes
        // (k_defer_open reopens that step) -> WHILE(some film not converged)
        // { solve -> pass }, under an IF that skips them when none is pending
        cudaGraphConditionalHandle h_open = 0, h_fin = 0;
        cudaGraphNode_t n_open, n_fif, n_u, n_fw, n_fs, n_fr;
        cudaGraph_t fin, fbody;
        CK(cudaGraphConditionalHandleCreate(&h_open, top, 0, cudaGraphCondAssignDefault));
        Dev dopen = e->dev(1);
        void *a_open[] = {&dopen, &h_open};
        TRY(add_kernel(top, &n_open, &n_loop, 1, (void *)k_defer_open, 1, 32, a_open));
        TRY(add_if(top, &n_fif, &n_open, 1, h_open, &fin));
        CK(cudaGraphConditionalHandleCreate(&h_fin, fin, 0, cudaGraphCondAssignDefault));
        a.d = e->dev(1, 0, h_fin);
        a.d.step_end = 1;
        TRY(add_kernel(fin, &n_u, nullptr, 0, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
        TRY(add_while(fin, &n_fw, &n_u, 1, h_fin, &fbody));
        a.d.step_end = 0;
        TRY(add_solve(fbody, nullptr, &n_fs));
        a.d.step_end = 1;
        TRY(add_kernel(fbody, &n_fr, &n_fs, 1, e->refine_fn, nsit, e->refine_nt, args32, e->refine_smem));
    }
    CK(cudaGraphInstantiate(&e->exec, top, 0));
    e->graph_valid = true;
    return CMSL_OK;
}

// State transfers.  Where the device reads the host's page tables
// (cudaDevAttrPageableMemoryAccess: Grace-Blackwell's coherent NVLink-C2C),
// kernels read the caller's double arrays in place and convert on the GPU.
// Downloads into page-locked caller arrays (cmsl_host_alloc, or registered
// by the caller) are converted and written by kernels as well; other
// downloads go through one pinned array and are converted on the host cores
// (a GPU writing fresh pageable pages pays a page fault per page).  Without
// that device attribute uploads are converted on the host too.
template <class T>
__global__ void k_host_in(const double *__restrict__ src, T *__restrict__ dst, long long n, int stride)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i * stride] = (T)src[i];
}
// potential as double-float pairs: hi = (float)x, lo = (float)(x - hi)
__global__ void k_phi_in(const double *__restrict__ src, float2 *__restrict__ dst, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = src[i];
        const float h = (float)x;
        dst[i] = make_float2(h, (float)(x - (double)h));
    }
}
template <class T>
__global__ void k_host_out(const T *__restrict__ src, double *__restrict__ dst, long long n, int stride)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = (double)src[i * stride];
}
__global__ void k_phi_out(const float2 *__restrict__ src, double *__restrict__ dst, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        dst[i] = (double)v.x + (double)v.y;
    }
}

// The whole state of one FP32 film in one launch each way, the P set and
// the potential buffer picked on the device (Ctl::cur, SolveDev::phi_cur):
// no host round trip for them and no launch per field.  The link to the
// host's memory is the bound (measured ~205 GB/s in, ~190 GB/s out with
// either one launch per field or one for all; one launch saves the launches
// and host synchronisations between them).
struct StateIn {
    const double *P[6];         // the caller's fields (device-readable)
    const double *phi;          // the caller's potential, or null (zero)
    float2 *pair[2][3];         // the film's (P[2j], P[2j+1]) pairs of both sets
    float2 *phi0;               // the film's slice of potential buffer 0
    float *x;                   // the film's slice of the correction
    const Ctl *ctl;
    long long n;
};
__global__ void k_state_in(StateIn s)
{
    float2 *const *pr = s.pair[s.ctl->cur];     // the set the next step reads
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += (long long)gridDim.x * blockDim.x) {
        double v[6];
        #pragma unroll
        for (int q = 0; q < 6; ++q) v[q] = s.P[q][i];
        const double p = s.phi ? s.phi[i] : 0.0;
        #pragma unroll
        for (int j = 0; j < 3; ++j) pr[j][i] = make_float2((float)v[2 * j], (float)v[2 * j + 1]);
        const float h = (float)p;
        s.phi0[i] = make_float2(h, (float)(p - (double)h));
        s.x[i] = 0.f;
    }
}
struct StateOut {
    double *P[6];               // page-locked outputs (device addresses), null where not wanted
    double *phi;
    const float2 *pair[2][3];
    const float2 *phib[5];      // the film's slice of every potential buffer
    const Ctl *ctl;
    const SolveDev *S;
    long long n;
};
__global__ void k_state_out(StateOut s)
{
    const float2 *const *pr = s.pair[s.ctl->cur];
    const float2 *ph = s.phi ? s.phib[s.S->phi_cur] : nullptr;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += (long long)gridDim.x * blockDim.x) {
        float2 v[3];
        #pragma unroll
        for (int j = 0; j < 3; ++j)
            if (s.P[2 * j] || s.P[2 * j + 1]) v[j] = pr[j][i];
        const float2 w = ph ? ph[i] : make_float2(0.f, 0.f);
        #pragma unroll
        for (int j = 0; j < 3; ++j) {
            if (s.P[2 * j]) s.P[2 * j][i] = (double)v[j].x;
            if (s.P[2 * j + 1]) s.P[2 * j + 1][i] = (double)v[j].y;
        }
        if (ph) s.phi[i] = (double)w.x + (double)w.y;
    }
}
// Per-cell codes of one film on the device (the set-up of main.cu:13-52 and
// init_conf.cu:68-106 reduced to one word per cell): grain id | material
// << 24 | interface << 26, the interface flag of build_interface_flag unless
// the caller gave one; the voxels of each material counted per block and
// added in integers (exact).  Grain ids were checked on the host.
__global__ void k_film_code(const int32_t *__restrict__ omega, const int32_t *__restrict__ gmat,
                            const int32_t *__restrict__ iface, int nx, int ny, int nz, uint32_t *__restrict__ code,
                            unsigned long long *__restrict__ counts)
{
    __shared__ unsigned int s_cnt[3];
    if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    const long long plane = (long long)nx * ny, n = plane * nz;
    unsigned int c0 = 0, c1 = 0, c2 = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int g = omega[i], m = gmat[g];
        int fl = 0;
        if (iface) {
            fl = iface[i] != 0;
        } else {
            const long long k = i / plane;
            if (m == CMSL_FE && k > 0 && k < nz - 1)
                fl = gmat[omega[i + plane]] != CMSL_FE || gmat[omega[i - plane]] != CMSL_FE;
        }
        code[i] = (uint32_t)g | ((uint32_t)m << 24) | ((uint32_t)fl << 26);
        c0 += m == 0;
        c1 += m == 1;
        c2 += m == 2;
    }
    atomicAdd(&s_cnt[0], c0);
    atomicAdd(&s_cnt[1], c1);
    atomicAdd(&s_cnt[2], c2);
    __syncthreads();
    if (threadIdx.x < 3) atomicAdd(&counts[threadIdx.x], (unsigned long long)s_cnt[threadIdx.x]);
}

constexpr int XFER_GRID = 152 * 8, XFER_NT = 256;

// The device address of page-locked host memory at p (null for pageable
// memory, which cudaPointerGetAttributes reports as unregistered).
inline double *locked_dst(double *p)
{
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? (double *)a.devicePointer : nullptr;
}

}  // namespace cmsl_eng

namespace {

// Reads every film's solver slot; *active / *outer: any film still running.
cmsl_status read_flags(Engine *e, cudaStream_t st, bool *active, bool *outer)
{
    std::vector<SolveDev> S((size_t)e->n_films);
    CK(cudaMemcpyAsync(S.data(), e->d_solve, sizeof(SolveDev) * S.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *active = false;
    if (outer) *outer = false;
    for (const SolveDev &s : S) {
        *active |= s.active != 0;
        if (outer) *outer |= s.outer_active != 0;
    }
    return CMSL_OK;
}

// One FP32 residual pass (k_refine32) launched from the host.
cmsl_status launch_refine(Engine *e, cudaStream_t st, const Dev &d, const Fields<float> &F32)
{
    Dev dd = d;
    Fields<float> ff = F32;
    void *args[] = {&dd, &ff};
    CK(cudaLaunchKernel(e->refine_fn, dim3((unsigned)e->sitems.size()), dim3(e->refine_nt), args, e->refine_smem, st));
    return CMSL_OK;
}

// One FP32 TDGL step (k_tdgl32 / k_tdgl32p) launched from the host.
cmsl_status launch_tdgl32(Engine *e, cudaStream_t st, const Dev &d, const Fields<float> &F32)
{
    Dev dd = d;
    Fields<float> ff = F32;
    void *args[] = {&dd, &ff};
    CK(cudaLaunchKernel(e->tdgl_fn, dim3((unsigned)e->sitems.size()), dim3(e->tdgl_nt), args, e->tdgl_smem, st));
    return CMSL_OK;
}

// The direct spectral solve of the correction, launched from the host.
cmsl_status spec_launch(Engine *e, cudaStream_t st, const Dev &d, const Fields<float> &F32)
{
    const SpecDev &sp = e->spec;
    if (e->spec_cl) {
        k_spec_cxy<<<e->spec_grid[4], SPEC_CL_NT, e->spec_smem[4], st>>>(d, F32, sp);
        k_spec_z<true><<<e->spec_grid[2], e->spec_zt, e->spec_smem[2], st>>>(d, sp);
        k_spec_cyx<<<e->spec_grid[4], SPEC_CL_NT, e->spec_smem[4], st>>>(d, F32, sp);
        CK(cudaGetLastError());
        return CMSL_OK;
    }
    if (e->spec_col) {
        k_spec_x<true, true><<<e->spec_grid[0], SPEC_NT, e->spec_smem[0], st>>>(d, F32, sp);
        k_spec_yzy<<<e->spec_grid[3], SPEC_YZY_NT, e->spec_smem[3], st>>>(d, sp);
        k_spec_x<false, true><<<e->spec_grid[0], SPEC_NT, e->spec_smem[0], st>>>(d, F32, sp);
        CK(cudaGetLastError());
        return CMSL_OK;
    }
    k_spec_x<true><<<e->spec_grid[0], SPEC_NT, e->spec_smem[0], st>>>(d, F32, sp);
    k_spec_y<<<e->spec_grid[1], SPEC_NT, e->spec_smem[1], st>>>(d, sp);
    k_spec_z<false><<<e->spec_grid[2], e->spec_zt, e->spec_smem[2], st>>>(d, sp);
    k_spec_y<<<e->spec_grid[1], SPEC_NT, e->spec_smem[1], st>>>(d, sp);
    k_spec_x<false><<<e->spec_grid[0], SPEC_NT, e->spec_smem[0], st>>>(d, F32, sp);
    CK(cudaGetLastError());
    return CMSL_OK;
}

// The depolarisation solve launched from the host, one kernel at a time,
// reading the loop flags back after each iteration.  Used by the
// single-piece test hooks and when graphs are disabled (CMSL_NO_GRAPH=1).
cmsl_status solve_direct(Engine *e, cudaStream_t st, const Dev &d, const Fields<double> &F64,
                         const Fields<float> &F32)
{
    const int nit = (int)e->items.size();
    bool act = false, out = false;
    if (e->precision == CMSL_FP64) {
        k_rhs<double, Exact><<<nit, NT, 0, st>>>(d, F64);
        CK(cudaGetLastError());
        for (int guard = 0;; ++guard) {
            TRY(read_flags(e, st, &act, nullptr));
            if (!act) break;
            if (guard > e->max_iter_cap + 1) return fail(CMSL_ERR_STATE, "PCG loop did not stop");
            k_spmv<double, Exact><<<nit, NT, 0, st>>>(d, F64);
            k_update<double, Exact, false><<<nit, NT, 0, st>>>(d, F64);
            CK(cudaGetLastError());
        }
    } else {
        for (int og = 0;; ++og) {
            if (og > e->max_refine_cap + 1) return fail(CMSL_ERR_STATE, "refinement loop did not stop");
            TRY(launch_refine(e, st, d, F32));
            TRY(read_flags(e, st, &act, &out));
            if (act && e->spectral) {
                TRY(spec_launch(e, st, d, F32));
                TRY(read_flags(e, st, &act, &out));
            }
            if (act && e->persistent) {
                Dev dd = d;
                CgBuf B = e->cg;
                const float *dv = (const float *)e->d_dinv;
                void *args[] = {&dd, &B, &dv};
                CK(cudaLaunchCooperativeKernel(e->cg_fn, e->cg_grid, PNT, args, e->cg_smem, st));
                TRY(read_flags(e, st, &act, &out));
            }
            for (int guard = 0; act && !e->persistent && !e->spectral; ++guard) {
                if (guard > e->inner_max_cap + 1) return fail(CMSL_ERR_STATE, "inner PCG loop did not stop");
                k_spmv<float, Fast><<<nit, NT, 0, st>>>(d, F32);
                k_update<float, Fast, true><<<nit, NT, 0, st>>>(d, F32);
                CK(cudaGetLastError());
                TRY(read_flags(e, st, &act, &out));
            }
            if (!out) break;
        }
    }
    return CMSL_OK;
}

cmsl_status step_direct(Engine *e, cudaStream_t st)
{
    const int nit = (int)e->items.size();
    Dev d = e->dev(0);
    d.defer = e->defer ? 1 : 0;
    const Fields<double> F64 = e->fields<double>();
    const Fields<float> F32 = e->fields<float>();
    if (e->precision == CMSL_FP64) {
        k_tdgl<double, Exact><<<nit, NT, 0, st>>>(d, F64);
    } else {
        for (int tries = 0;; ++tries) {
            if (e->defer) CK(cudaMemsetAsync(&e->d_ctl->redo, 0, sizeof(int), st));
            TRY(launch_tdgl32(e, st, d, F32));
            if (!e->defer) break;
            // a failed deferred check reopened the previous step: its passes
            // end it again, then this step runs again
            int redo = 0;
            CK(cudaMemcpyAsync(&redo, &e->d_ctl->redo, sizeof(int), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (!redo) break;
            if (tries > 1) return fail(CMSL_ERR_STATE, "a reopened step failed its check again");
            TRY(solve_direct(e, st, d, F64, F32));
            k_step_end<<<1, 32, 0, st>>>(d);
        }
    }
    CK(cudaGetLastError());
    if (e->any_dep) TRY(solve_direct(e, st, d, F64, F32));
    k_step_end<<<1, 32, 0, st>>>(d);
    CK(cudaGetLastError());
    return CMSL_OK;
}

// After the last step of a run launched from the host: the checks still
// pending run as update passes of that step, reopened (see k_defer_open).
cmsl_status defer_close_direct(Engine *e, cudaStream_t st)
{
    std::vector<SolveDev> S((size_t)e->n_films);
    CK(cudaMemcpyAsync(S.data(), e->d_solve, sizeof(SolveDev) * S.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    bool any = false;
    for (const SolveDev &s : S) any |= s.pending != 0;
    if (!any) return CMSL_OK;
    const Dev d = e->dev(0);
    k_defer_open<<<1, 32, 0, st>>>(d, 0);
    CK(cudaGetLastError());
    TRY(solve_direct(e, st, d, e->fields<double>(), e->fields<float>()));
    k_step_end<<<1, 32, 0, st>>>(d);
    CK(cudaGetLastError());
    return CMSL_OK;
}


// Field q of P set s: FP64 -- its own array; FP32 -- one half of the pair
// (q & ~1, q | 1), element i at stride 2 (pstride).
template <class T>
cmsl_status put_fields(Engine *e, int film, int set, const double *const P[6])
{
    const FilmHost &h = e->fh[film];
    const int ps = e->pstride();
    for (int q = 0; q < 6; ++q)
        if (!P[q]) return fail(CMSL_ERR_ARG, "P[%d] is NULL", q);
    if (e->host_direct) {
        for (int q = 0; q < 6; ++q)
            k_host_in<T><<<XFER_GRID, XFER_NT>>>(P[q], (T *)e->d_P[set][q] + ps * h.off, h.N, ps);
        CK(cudaGetLastError());
        CK(cudaDeviceSynchronize());
        return CMSL_OK;
    }
    std::vector<T> tmp((size_t)(ps * h.N));
    for (int q = 0; q < 6; q += ps) {
        for (long long i = 0; i < h.N; ++i)
            for (int u = 0; u < ps; ++u) tmp[ps * i + u] = (T)P[q + u][i];
        CK(cudaMemcpy((T *)e->d_P[set][q] + ps * h.off, tmp.data(), ps * h.N * sizeof(T), cudaMemcpyHostToDevice));
    }
    return CMSL_OK;
}

// Pinned host array of the largest film's cells (two floats or one double per
// cell), for state downloads (allocated on first use).
cmsl_status pinned_stage(Engine *e, void **out)
{
    if (!e->h_stage) {
        long long nmax = 0;
        for (const FilmHost &h : e->fh) nmax = std::max(nmax, h.N);
        CK(cudaMallocHost(&e->h_stage, sizeof(double) * (size_t)nmax));
    }
    *out = e->h_stage;
    return CMSL_OK;
}

// fn(i0, i1) over [0, n) on the host cores: the conversion of a download is
// dominated by the first touch of the caller's fresh output pages.
template <class F> void parallel_for(long long n, F fn)
{
    const long long chunk = 1 << 20;
    const int nt = (int)std::min<long long>(std::max(1u, std::thread::hardware_concurrency()), (n + chunk - 1) / chunk);
    if (nt <= 1) {
        fn(0LL, n);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] { fn(n * t / nt, n * (t + 1) / nt); });
    for (std::thread &x : th) x.join();
}

template <class T>
cmsl_status get_fields(Engine *e, int film, int set, double *const P[6])
{
    const FilmHost &h = e->fh[film];
    const int ps = e->pstride();
    bool rest = false;                  // arrays left for the paths below
    for (int q = 0; q < 6; ++q) {
        double *dv = locked_dst(P[q]);
        if (dv) k_host_out<T><<<XFER_GRID, XFER_NT>>>((const T *)e->d_P[set][q] + ps * h.off, dv, h.N, ps);
        else rest = rest || P[q];
    }
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if (!rest) return CMSL_OK;
    double *Pr[6];
    for (int q = 0; q < 6; ++q) Pr[q] = locked_dst(P[q]) ? nullptr : P[q];
    P = Pr;
    // one DMA copy of each field (FP64) or pair (FP32) into pinned memory,
    // then the conversion into the caller's arrays on the host cores
    void *stg = nullptr;
    std::vector<T> tmp;
    if (e->host_direct) {
        TRY(pinned_stage(e, &stg));
    } else {
        tmp.resize((size_t)(ps * h.N));
        stg = tmp.data();
    }
    const T *st = (const T *)stg;
    for (int q = 0; q < 6; q += ps) {
        bool want = false;
        for (int u = 0; u < ps; ++u) want = want || P[q + u];
        if (!want) continue;
        CK(cudaMemcpy((void *)st, (const T *)e->d_P[set][q] + ps * h.off, sizeof(T) * ps * h.N,
                      cudaMemcpyDeviceToHost));
        for (int u = 0; u < ps; ++u) {
            double *dst = P[q + u];
            if (!dst) continue;
            parallel_for(h.N, [&](long long i0, long long i1) {
                for (long long i = i0; i < i1; ++i) dst[i] = (double)st[ps * i + u];
            });
        }
    }
    return CMSL_OK;
}

// Builds every film's codes into d_code (film f at its offset) and the
// per-material voxel counts of the film tables.
cmsl_status build_film_codes(Engine *e, const cmsl_film_desc *descs, std::vector<FilmDev> &fds)
{
    long long nmax = 0;
    int gmax = 0;
    for (const FilmHost &h : e->fh) {
        nmax = std::max(nmax, h.N);
        gmax = std::max(gmax, h.ng);
    }
    int32_t *t = nullptr;
    unsigned long long *cnt = nullptr;
    CK(cudaMalloc(&t, sizeof(int32_t) * (size_t)(2 * nmax + gmax)));
    cudaError_t err = cudaMalloc(&cnt, sizeof(unsigned long long) * 3);
    for (int fi = 0; fi < e->n_films && err == cudaSuccess; ++fi) {
        const cmsl_film_desc *dsc = descs + fi;
        const FilmHost &h = e->fh[fi];
        int32_t *om = t, *fl = t + nmax, *gm = t + 2 * nmax;
        unsigned long long c[3] = {0, 0, 0};
        err = cudaMemcpy(om, dsc->omega, sizeof(int32_t) * h.N, cudaMemcpyHostToDevice);
        if (err == cudaSuccess) err = cudaMemcpy(gm, dsc->grain_mat, sizeof(int32_t) * h.ng, cudaMemcpyHostToDevice);
        if (err == cudaSuccess && dsc->is_interface)
            err = cudaMemcpy(fl, dsc->is_interface, sizeof(int32_t) * h.N, cudaMemcpyHostToDevice);
        if (err == cudaSuccess) err = cudaMemset(cnt, 0, sizeof(unsigned long long) * 3);
        if (err == cudaSuccess) {
            const unsigned blocks = (unsigned)std::min<long long>((h.N + 255) / 256, 152LL * 16);
            k_film_code<<<blocks, 256>>>(om, gm, dsc->is_interface ? fl : nullptr, h.nx, h.ny, h.nz,
                                         e->d_code + h.off, cnt);
            err = cudaGetLastError();
        }
        if (err == cudaSuccess) err = cudaMemcpy(c, cnt, sizeof c, cudaMemcpyDeviceToHost);
        for (int q = 0; q < 3; ++q) fds[fi].n_mat[q] = (double)c[q];
    }
    cudaFree(t);
    if (cnt) cudaFree(cnt);
    if (err != cudaSuccess) return fail(CMSL_ERR_CUDA, "building the cell codes failed: %s", cudaGetErrorString(err));
    return CMSL_OK;
}

// Tensor maps of every film for the tensor-copy staging (FilmMaps): the P
// sets as 4D {nx, ny, nz, 3} float2-pair tensors, the five potential buffers
// and the correction dx, the codes, r and D^-1 as 3D tensors, each in the
// three box shapes the stencil passes copy (tile body, x row, x halo strip).
cmsl_status make_maps(Engine *e)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (!fn || q != cudaDriverEntryPointSuccess) return fail(CMSL_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    const int F = e->n_films;
    std::vector<FilmMaps> maps((size_t)F);
    const cuuint64_t cells = (cuuint64_t)e->ncells;
    for (int fi = 0; fi < F; ++fi) {
        const FilmHost &h = e->fh[fi];
        FilmMaps &M = maps[fi];
        // box shapes: tile body, one x row, a 16-byte x strip
        auto enc = [&](CUtensorMap *m3, void *base, int esz, int rank, int nq, int n_shapes) -> cmsl_status {
            const cuuint64_t dims[4] = {(cuuint64_t)h.nx, (cuuint64_t)h.ny, (cuuint64_t)h.nz, (cuuint64_t)nq};
            const cuuint64_t strides[3] = {(cuuint64_t)h.nx * esz, (cuuint64_t)h.nx * h.ny * esz, cells * esz};
            const cuuint32_t shapes[3][4] = {{TX, TY, 1, 1}, {TX, 1, 1, 1}, {(cuuint32_t)(16 / esz), TY, 1, 1}};
            const cuuint32_t unit[4] = {1, 1, 1, 1};
            for (int sh = 0; sh < n_shapes; ++sh) {
                const CUresult r = encode(m3 + sh, esz == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32,
                                          rank, base, dims, strides, shapes[sh], unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                if (r != CUDA_SUCCESS) return fail(CMSL_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
            }
            return CMSL_OK;
        };
        for (int s = 0; s < 2; ++s) TRY(enc(M.P[s], (float2 *)e->d_P[s][0] + h.off, 8, 4, 3, 3));
        for (int b = 0; b < 5; ++b) TRY(enc(M.phi[b], (float2 *)e->d_phi[b] + h.off, 8, 3, 1, 3));
        TRY(enc(M.code, (uint32_t *)e->d_code + h.off, 4, 3, 1, 3));
        TRY(enc(M.x, (float *)e->d_x + h.off, 4, 3, 1, 3));
        TRY(enc(&M.r, (float *)e->d_r + h.off, 4, 3, 1, 1));
        TRY(enc(&M.dinv, (float *)e->d_dinv + h.off, 4, 3, 1, 1));
    }
    TRY(e->alloc((void **)&e->d_maps, sizeof(FilmMaps) * F));
    CK(cudaMemcpy(e->d_maps, maps.data(), sizeof(FilmMaps) * F, cudaMemcpyHostToDevice));
    return CMSL_OK;
}

cmsl_status engine_create(Engine *e, const cmsl_film_desc *descs, int n)
{
    for (int i = 0; i < n; ++i) TRY(check_desc(descs + i, i, n));
    for (int i = 1; i < n; ++i)
        if (descs[i].precision != descs[0].precision)
            return fail(CMSL_ERR_ARG, "film %d: precision %d differs from film 0 (%d)", i, descs[i].precision,
                        descs[0].precision);
    e->precision = descs[0].precision;
    e->n_films = n;
    e->esz = e->precision == CMSL_FP64 ? 8 : 4;
    const char *ng = getenv("CMSL_NO_GRAPH");
    e->use_graph = !(ng && atoi(ng) != 0);
    long long xy_tiles = 0;
    for (int i = 0; i < n; ++i) {
        const cmsl_film_desc &d = descs[i];
        FilmHost h;
        h.nx = d.nx; h.ny = d.ny; h.nz = d.nz; h.ng = d.n_grains; h.dep = d.dep_flag != 0; h.zbc = d.zbc; h.h = d.del_h;
        h.N = (long long)d.nx * d.ny * d.nz;
        h.off = (e->ncells + 31) / 32 * 32;   // 128-byte aligned FP32 film start
        e->ncells = h.off + h.N;
        e->fh.push_back(h);
        e->any_dep |= h.dep != 0;
        xy_tiles += (long long)((d.nx + TX - 1) / TX) * ((d.ny + TY - 1) / TY);
        e->max_iter_cap = std::max(e->max_iter_cap, d.max_iter);
        e->max_refine_cap = std::max(e->max_refine_cap, std::max(1, d.max_refine));
        e->inner_max_cap = std::max(e->inner_max_cap, std::max(1, d.inner_max_iter));
    }
    e->ncells = (e->ncells + 31) / 32 * 32;
    // FP32_REFINED inner solver.  The persistent solver's single-reduction
    // recurrence assumes a symmetric operator; with the Neumann z boundary
    // the mirrored rows of the first and last planes (depol_varEPS.cu:93-98)
    // make A non-symmetric, so a batch holding such a film takes the
    // two-kernel PCG, the reference's own algorithm.  So does a batch with
    // more films than one cooperative launch carries.
    const char *tk = getenv("CMSL_PCG_TWO_KERNEL");
    bool all_dirichlet = true, all_uni = true;
    for (int i = 0; i < n; ++i) {
        all_dirichlet &= descs[i].zbc == CMSL_DIRICHLET;
        all_uni &= descs[i].mats[0].eps_r == descs[i].mats[1].eps_r && descs[i].mats[1].eps_r == descs[i].mats[2].eps_r;
    }
    // direct (spectral) inner solve: every film with a depolarisation solve
    // has the Dirichlet z boundary and 2^a 3^b sides; with one eps it is the
    // exact inverse, with several a preconditioner of the refinement
    int spec_mmax = 1;
    {
        bool want = false, forced = false, ok = e->precision != CMSL_FP64, anydep = false, ok_auto = true;
        for (int i = 0; i < n; ++i) {
            const cmsl_film_desc &d = descs[i];
            forced |= d.inner_solver == CMSL_INNER_DIRECT;
            want |= d.inner_solver != CMSL_INNER_PCG;
            if (!d.dep_flag) continue;
            anydep = true;
            double kappa = 1.0;
            spec_eps_ref(d, &kappa);
            // several permittivities: the solve preconditions the refinement
            // (AUTO up to SPEC_PRECOND_KAPPA, any ratio when DIRECT is asked for)
            ok_auto &= kappa <= SPEC_PRECOND_KAPPA;
            ok &= d.zbc == CMSL_DIRICHLET && d.nz >= 3 && spec_radix_ok(d.nx) && spec_radix_ok(d.ny);
            spec_mmax = std::max(spec_mmax, d.nz - 2);
        }
        ok &= anydep && spec_zthreads(spec_mmax) > 0;
        if (forced && !ok)
            return fail(CMSL_ERR_ARG, "inner_solver DIRECT needs FP32_REFINED films whose depolarisation solves have "
                                      "the Dirichlet z boundary and nx, ny of the form 2^a 3^b <= 4096");
        e->spectral = ok && want && (forced || ok_auto);
    }
    int cg_per = 0, cg_nsm = 0;
    e->persistent = e->precision != CMSL_FP64 && !e->spectral && all_dirichlet && n <= CG_MAX_FILMS &&
                    !(tk && atoi(tk) != 0);
    if (e->persistent) {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&cg_nsm, cudaDevAttrMultiProcessorCount, dev));
        if (n == 1) e->cg_fn = all_uni ? (void *)k_pcg_cg2<true, false> : (void *)k_pcg_cg2<false, false>;
        else e->cg_fn = all_uni ? (void *)k_pcg_cg2<true, true> : (void *)k_pcg_cg2<false, true>;
        e->cg_smem = P2SMEM_BYTES + sizeof(FilmState) * n;
        CK(cudaFuncSetAttribute(e->cg_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->cg_smem));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cg_per, e->cg_fn, PNT, e->cg_smem));
        if (cg_per < 1) return fail(CMSL_ERR_CUDA, "persistent PCG kernel cannot be resident");
        if (n > cg_per * cg_nsm) e->persistent = false;
    }

    // grain ids are checked on the host (before any device work); the
    // per-cell codes, interface flags and material voxel counts are built on
    // the device below (build_film_codes); work items, film tables
    std::vector<FilmDev> fds((size_t)n);
    int g_off = 0;
    for (int fi = 0; fi < n; ++fi) {
        const cmsl_film_desc *dsc = descs + fi;
        const FilmHost &h = e->fh[fi];
        const std::string who = n > 1 ? "film " + std::to_string(fi) + ": " : "";
        for (long long i = 0; i < h.N; ++i) {
            const int gid = dsc->omega[i];
            if (gid < 0 || gid >= h.ng)
                return fail(CMSL_ERR_ARG, "%scell %lld has grain id %d outside [0,%d)", who.c_str(), i, gid, h.ng);
        }
        FilmDev &fd = fds[fi];
        fill_film(fd, dsc, e->precision);
        // the FP32 update pass r <- r - A dx follows an exact (one-eps) direct solve only;
        // its check may run inside the next TDGL step when that step's warm start
        // leaves the third-oldest potential unread
        fd.upd_ok = e->spectral && fd.uni_eps ? 1 : 0;
        fd.defer_ok = fd.upd_ok && fd.dep_flag && fd.warm <= 2 ? 1 : 0;
        fd.cheb_delta = 0.f;
        if (e->spectral && !fd.uni_eps && fd.dep_flag) {
            double kappa = 1.0;
            spec_eps_ref(*dsc, &kappa);
            fd.cheb_delta = (float)((kappa - 1.0) / (kappa + 1.0));
            const int cap = spec_precond_refine_cap(kappa, dsc->refine_tol);
            fd.max_refine = std::max(fd.max_refine, cap);
            e->max_refine_cap = std::max(e->max_refine_cap, cap);
        }
        fd.off = h.off;
        fd.g_off = g_off;
        g_off += h.ng;
    }
    e->xy_tiles = xy_tiles;

    // persistent PCG partition: stencil bricks of PZ planes film by film;
    // each film gets a contiguous block range in proportion to its cells
    // (one film: as many blocks as give every block the same brick count)
    std::vector<int4> bricks;
    std::vector<int> blk_film;
    if (e->persistent) {
        for (int fi = 0; fi < n; ++fi) {
            const FilmHost &h = e->fh[fi];
            fds[fi].brick_begin = (int)bricks.size();
            for (int y0 = 0; y0 < h.ny; y0 += TY)
                for (int x0 = 0; x0 < h.nx; x0 += TX)
                    for (int z0 = 0; z0 < h.nz; z0 += PZ)
                        bricks.push_back(make_int4(fi, x0, y0, z0 | (std::min(h.nz, z0 + PZ) << 16)));
            fds[fi].brick_end = (int)bricks.size();
        }
        const int maxg = cg_per * cg_nsm;
        std::vector<int> nb((size_t)n, 1);
        if (n == 1) {
            const int nbk = (int)bricks.size(), per_block = (nbk + maxg - 1) / maxg;
            nb[0] = (nbk + per_block - 1) / per_block;
        } else {
            long long tot = 0;
            for (const FilmHost &h : e->fh) tot += h.N;
            int sum = 0;
            auto cap = [&](int fi) { return std::max(1, fds[fi].brick_end - fds[fi].brick_begin); };
            for (int fi = 0; fi < n; ++fi) {
                nb[fi] = std::min(cap(fi), std::max(1, (int)((double)maxg * e->fh[fi].N / tot)));
                sum += nb[fi];
            }
            while (sum > maxg) {             // cannot happen with n <= maxg unless rounding up
                int big = 0;
                for (int fi = 1; fi < n; ++fi) if (nb[fi] > nb[big]) big = fi;
                if (nb[big] <= 1) break;
                --nb[big]; --sum;
            }
            while (sum < maxg) {             // hand out the rest to the most loaded films
                int best = -1;
                double load = 0.0;
                for (int fi = 0; fi < n; ++fi) {
                    if (nb[fi] >= cap(fi)) continue;
                    const double l = (double)e->fh[fi].N / nb[fi];
                    if (l > load) { load = l; best = fi; }
                }
                if (best < 0) break;
                ++nb[best]; ++sum;
            }
        }
        for (int fi = 0; fi < n; ++fi) {
            fds[fi].pb_begin = (int)blk_film.size();
            for (int j = 0; j < nb[fi]; ++j) blk_film.push_back(fi);
            fds[fi].pb_end = (int)blk_film.size();
        }
        e->cg_grid = (int)blk_film.size();
    }

    // device memory; the work items (and their partial sums) are sized for
    // the finest z chunk the autotuner tries
    const size_t cells = (size_t)e->ncells;
    {
        int dev = 0, pageable = 0, host_tables = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
        CK(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
        const char *hd = getenv("CMSL_HOST_COPY");   // 1: host-side conversion and copies
        e->host_direct = pageable && host_tables && !(hd && atoi(hd) != 0);
    }
    TRY(e->alloc((void **)&e->d_code, sizeof(uint32_t) * cells));
    TRY(build_film_codes(e, descs, fds));
    e->fdh = fds;
    TRY(e->alloc((void **)&e->d_films, sizeof(FilmDev) * n));
    e->items_cap = std::max(count_items(e, ZCHUNK_MIN), count_items(e, 0));
    e->sitems_cap = std::max(count_items(e, ZCHUNK_MIN, TILE_YS[0]), count_items(e, 0, TILE_YS[0]));
    TRY(e->alloc((void **)&e->d_items, sizeof(int4) * e->items_cap));
    TRY(e->alloc((void **)&e->d_sitems, sizeof(int4) * e->sitems_cap));
    e->part_cap = std::max(e->items_cap, e->sitems_cap);
    TRY(e->alloc((void **)&e->d_partial, sizeof(double) * NPART * 2 * e->part_cap));
    {
        // tile height of the FP32 stencil passes: CMSL_TILE_Y (4, 8 or 16)
        // fixes it; else a tuned handle of the same shape class, else TY
        int zc = 0;
        const char *tyv = getenv("CMSL_TILE_Y");
        const int ty_env = tyv ? atoi(tyv) : 0;
        e->tile_fixed = e->precision != CMSL_FP64 && (ty_env == 4 || ty_env == 8 || ty_env == 16);
        e->stile_ty = e->tile_fixed ? ty_env : TY;
        std::lock_guard<std::mutex> lk(g_tuned_mu);
        const auto hit = g_tuned.find(shape_key(e));
        if (hit != g_tuned.end()) {
            zc = hit->second.zchunk;
            if (!e->tile_fixed && e->precision != CMSL_FP64) e->stile_ty = hit->second.tile_y;
        }
        TRY(set_items(e, zc));
    }
    if (e->precision == CMSL_FP64) TRY(upload_TR<double>(e, descs, n));
    else TRY(upload_TR<float>(e, descs, n));
    for (int s = 0; s < 2; ++s) {
        // FP64: the six fields of a set back to back (field q at q * cells);
        // FP32: the pairs (Pmx, Pmy), (Pmz, Psx), (Psy, Psz) as float2 arrays
        // back to back, field q the half q & 1 of pair q / 2 (stride 2)
        TRY(e->alloc(&e->d_P[s][0], 6 * e->esz * cells));
        for (int q = 1; q < 6; ++q)
            e->d_P[s][q] = e->precision == CMSL_FP64 ? (char *)e->d_P[s][0] + q * e->esz * cells
                                                      : (void *)((float *)e->d_P[s][0] + (q >> 1) * 2 * cells + (q & 1));
    }
    TRY(e->alloc(&e->d_r, e->esz * cells));
    TRY(e->alloc(&e->d_q, e->esz * cells));
    TRY(e->alloc(&e->d_dinv, e->esz * cells));
    TRY(e->alloc(&e->d_p[0], e->esz * cells));
    TRY(e->alloc(&e->d_p[1], e->esz * cells));
    if (e->precision != CMSL_FP64) TRY(e->alloc(&e->d_x, e->esz * cells));
    if (e->persistent) {
        // persistent single-reduction PCG: r (the shared r), u, w, s; x =
        // correction, p in place
        CgBuf &B = e->cg;
        B.r[0] = (float *)e->d_r;
        TRY(e->alloc((void **)&B.r[1], 4 * cells));
        TRY(e->alloc((void **)&B.w[0], 4 * cells));
        TRY(e->alloc((void **)&B.s[0], 4 * cells));
        B.w[1] = B.w[0];
        B.s[1] = B.s[0];
        B.x = (float *)e->d_x;
        B.p = (float *)e->d_p[0];
        TRY(e->alloc((void **)&B.bricks, sizeof(int4) * bricks.size()));
        CK(cudaMemcpy((void *)B.bricks, bricks.data(), sizeof(int4) * bricks.size(), cudaMemcpyHostToDevice));
        B.n_bricks = (int)bricks.size();
        TRY(e->alloc((void **)&B.blk_film, sizeof(int) * blk_film.size()));
        CK(cudaMemcpy((void *)B.blk_film, blk_film.data(), sizeof(int) * blk_film.size(), cudaMemcpyHostToDevice));
        TRY(e->alloc((void **)&B.part, sizeof(float4) * 2 * e->cg_grid));
        TRY(e->alloc((void **)&B.arrive, sizeof(unsigned int) * 2));
        TRY(e->alloc((void **)&B.err, sizeof(int) * 2));
        // the barrier waits' limit, and a block that withholds its arrivals,
        // for the host test that makes a barrier run out (CMSL_PCG_SPIN_LIMIT,
        // CMSL_PCG_HOLD_BLOCK); the kernel then returns and reports the timeout
        const char *sl = getenv("CMSL_PCG_SPIN_LIMIT"), *hb = getenv("CMSL_PCG_HOLD_BLOCK");
        B.spin_limit = sl && atoll(sl) > 0 ? (unsigned long long)atoll(sl) : BARRIER_SPIN_LIMIT;
        B.hold_block = hb ? atoi(hb) : -1;
    }
    if (e->spectral) {
        // per-film plans, tables and block ranges of the three passes
        const int zt = spec_zthreads(spec_mmax);
        std::vector<SpecFilm> sf((size_t)n);
        std::vector<int> bxf, byf, bzf, bqf, bcf;
        size_t smq = 0, smc = 0;
        int dev_o = 0, optin = 0;
        CK(cudaGetDevice(&dev_o));
        CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev_o));
        // the cluster transforms (CMSL_SPEC_CL=1, where every depolarised
        // film takes them): a shorter solve at 64x64x16 and 128x128x16 (24.7
        // against 32.7 us, 28.0 against 31.8) but no shorter a step there,
        // and a longer solve at 256x256x32 (55.4 against 43.0 us, one block
        // of 512 threads per SM on 120 SMs), so it stays opt-in (64x64x16
        // steps: 59.3 us against 55.8 for the column layout)
        const char *clv = getenv("CMSL_SPEC_CL");
        bool cl_ok = clv && atoi(clv) != 0;
        for (int fi = 0; fi < n; ++fi)
            if (e->fh[fi].dep)
                cl_ok = cl_ok && spec_cl_ok(spec_plan(e->fh[fi].nx), spec_plan(e->fh[fi].ny), e->fh[fi].nx,
                                            e->fh[fi].ny, (size_t)optin);
        e->spec_cl = cl_ok;
        long long ioff = 0;
        std::vector<float2> tw;
        std::vector<float> lam;
        long long coff = 0;
        size_t smx = 0, smy = 0;
        auto tables = [&](int nn, int *two, int *lamo) {
            *two = (int)tw.size();
            *lamo = (int)lam.size();
            for (int q = 0; q < nn; ++q) {
                const double ang = 2.0 * M_PI * q / nn;
                tw.push_back(make_float2((float)std::cos(ang), (float)-std::sin(ang)));
                const double sn = std::sin(M_PI * q / nn);
                lam.push_back((float)(4.0 * sn * sn));                 // 2 - 2 cos(2 pi q / n)
            }
        };
        for (int fi = 0; fi < n; ++fi) {
            const FilmHost &h = e->fh[fi];
            SpecFilm &P = sf[fi];
            P.nx = h.nx; P.ny = h.ny; P.nz = h.nz; P.off = h.off;
            P.bx0 = (int)bxf.size(); P.by0 = (int)byf.size(); P.bz0 = (int)bzf.size(); P.bq0 = (int)bqf.size();
            P.bc0 = (int)bcf.size();
            if (!h.dep) continue;                                    // no solve, no blocks
            P.M = h.nz - 2;
            P.Mp = (P.M + 1) / 2;
            P.ax = spec_plan(h.nx);
            P.ay = spec_plan(h.ny);
            P.coff = coff;
            coff += (long long)P.Mp * h.nx * h.ny;
            P.ioff = ioff;
            ioff += (long long)P.M * h.nx * h.ny;
            // harm(eps, eps) = eps on every face; several eps: the reference value
            const double eps = spec_eps_ref(descs[fi], nullptr);
            P.scale = (float)(h.h * h.h / (eps * (double)h.nx * h.ny));
            tables(h.nx, &P.twx, &P.lamx);
            tables(h.ny, &P.twy, &P.lamy);
            // rows (columns) per transform block: about two blocks per SM for
            // the film's Mp ny rows (Mp nx columns), a power of two, at most
            // SPEC_ELEMS values (8 rows of 256 at 256x256x32, 8 of 512 at
            // 512x512x64, 1 of 64 at 64x64x16); CMSL_SPEC_RB fixes it
            const char *rbe = getenv("CMSL_SPEC_RB");
            auto per_block = [&](long long lines, int len) {
                const int cap = std::max(1, SPEC_ELEMS / len);
                int r = 1;
                while (2LL * r * 2 * 152 <= lines && 2 * r <= cap) r *= 2;
                if (rbe && atoi(rbe) > 0) r = std::min(cap, atoi(rbe));
                return r;
            };
            const int rbx = per_block((long long)P.Mp * h.ny, h.nx), cby = per_block((long long)P.Mp * h.nx, h.ny);
            P.rb = rbx;
            P.cb = cby;
            const long long gx = ((long long)P.Mp * h.ny + rbx - 1) / rbx;
            const long long gy = (long long)P.Mp * ((h.nx + cby - 1) / cby);
            // one thread per mode pair (column by column: the count with nx and ny swapped)
            const long long gz = ((e->spec_cl ? spec_canon_count(h.ny, h.nx) : spec_canon_count(h.nx, h.ny)) + zt - 1) / zt;
            bxf.insert(bxf.end(), (size_t)gx, fi);
            byf.insert(byf.end(), (size_t)gy, fi);
            bzf.insert(bzf.end(), (size_t)gz, fi);
            bqf.insert(bqf.end(), (size_t)(h.nx / 2 + 1), fi);                  // mirror pairs of columns
            if (e->spec_cl) {
                bcf.insert(bcf.end(), (size_t)P.Mp * SPEC_CL, fi);               // a cluster per packed plane
                smc = std::max(smc, spec_cl_bytes(h.nx, h.ny));
            }
            smq = std::max(smq, spec_yzy_bytes(h.ny, P.Mp, P.M));
            smx = std::max(smx, sizeof(float2) * (2 * (spec_pad(rbx * spec_x_pitch(h.nx, true)) + 1) + h.nx));   // two tiles + twiddles
            smy = std::max(smy, sizeof(float2) * (2 * cby * h.ny + h.ny));
        }
        // the column layout (three launches per solve instead of five) where
        // the column pairs fit one block and every film has at most 128 x 128
        // columns: there the shorter solve shortens the step (64x64x16: 55.6
        // against 60.3 us per step, 128x128x16: 62.2 against 66.3), while at
        // 256x256x32 the row layout's step is shorter (151.0 against 152.8
        // us).  CMSL_SPEC_COLS=1 / 0 selects either where the column pairs fit.
        {
            bool small = true;
            for (int fi = 0; fi < n; ++fi) small = small && (long long)e->fh[fi].nx * e->fh[fi].ny <= 128 * 128;
            const char *cl = getenv("CMSL_SPEC_COLS");
            const bool want = cl && *cl ? atoi(cl) != 0 : small;
            e->spec_col = e->spec_cl || (smq <= (size_t)optin && want);
        }
        // Thomas pivots of every film, mode and interior plane, in double:
        // dg = lam_x + lam_y + 2, inv_k = 1 / (dg - c'_{k-1}) with c'_k = -inv_k
        std::vector<float> piv((size_t)std::max<long long>(ioff, 1));
        for (int fi = 0; fi < n; ++fi) {
            const FilmHost &h = e->fh[fi];
            const SpecFilm &P = sf[fi];
            if (!h.dep) continue;
            const long long modes = (long long)h.nx * h.ny;
            for (int ky = 0; ky < h.ny; ++ky)
                for (int kx = 0; kx < h.nx; ++kx) {
                    const double sx = std::sin(M_PI * kx / h.nx), sy = std::sin(M_PI * ky / h.ny);
                    const double dg = 4.0 * sx * sx + 4.0 * sy * sy + 2.0;
                    const long long mode = e->spec_col ? (long long)kx * h.ny + ky : (long long)ky * h.nx + kx;
                    double c = 0.0;
                    for (int k = 0; k < P.M; ++k) {
                        const double inv = 1.0 / (dg + c);
                        piv[(size_t)(P.ioff + k * modes + mode)] = (float)inv;
                        c = -inv;
                    }
                }
        }
        SpecDev &sp = e->spec;
        auto upload = [&](const void *src, size_t bytes, void **dst) -> cmsl_status {
            TRY(e->alloc(dst, bytes));
            CK(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
            return CMSL_OK;
        };
        void *p = nullptr;
        TRY(upload(sf.data(), sizeof(SpecFilm) * sf.size(), &p)); sp.films = (const SpecFilm *)p;
        TRY(upload(bxf.data(), sizeof(int) * bxf.size(), &p)); sp.bx_film = (const int *)p;
        TRY(upload(byf.data(), sizeof(int) * byf.size(), &p)); sp.by_film = (const int *)p;
        TRY(upload(bzf.data(), sizeof(int) * bzf.size(), &p)); sp.bz_film = (const int *)p;
        TRY(upload(bqf.data(), sizeof(int) * bqf.size(), &p)); sp.bq_film = (const int *)p;
        if (bcf.empty()) bcf.push_back(0);
        TRY(upload(bcf.data(), sizeof(int) * bcf.size(), &p)); sp.bc_film = (const int *)p;
        TRY(upload(tw.data(), sizeof(float2) * tw.size(), &p)); sp.tw = (const float2 *)p;
        TRY(upload(lam.data(), sizeof(float) * lam.size(), &p)); sp.lam = (const float *)p;
        TRY(upload(piv.data(), sizeof(float) * piv.size(), &p)); sp.piv = (const float *)p;
        TRY(e->alloc((void **)&sp.C, sizeof(float2) * (size_t)coff));
        e->spec_zt = zt;
        e->spec_grid[0] = (int)bxf.size();
        e->spec_grid[1] = (int)byf.size();
        e->spec_grid[2] = (int)bzf.size();
        e->spec_smem[0] = smx;
        e->spec_smem[1] = smy;
        e->spec_smem[2] = spec_zbytes(spec_mmax) * zt;
        CK(cudaFuncSetAttribute(k_spec_x<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->spec_smem[0]));
        CK(cudaFuncSetAttribute(k_spec_x<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->spec_smem[0]));
        CK(cudaFuncSetAttribute(k_spec_y, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->spec_smem[1]));
        CK(cudaFuncSetAttribute(k_spec_z<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->spec_smem[2]));
        CK(cudaFuncSetAttribute(k_spec_z<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->spec_smem[2]));
        if (e->spec_cl) {
            e->spec_grid[4] = (int)bcf.size();
            e->spec_smem[4] = smc;
            CK(cudaFuncSetAttribute(k_spec_cxy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
            CK(cudaFuncSetAttribute(k_spec_cyx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
        }
        {
            e->spec_grid[3] = (int)bqf.size();
            e->spec_smem[3] = smq;
            if (e->spec_col && !e->spec_cl) {
                CK(cudaFuncSetAttribute(k_spec_x<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)e->spec_smem[0]));
                CK(cudaFuncSetAttribute(k_spec_x<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)e->spec_smem[0]));
                CK(cudaFuncSetAttribute(k_spec_yzy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smq));
            }
        }
    }
    TRY(e->alloc((void **)&e->d_phi[0], sizeof(double) * cells));
    TRY(e->alloc((void **)&e->d_phi[1], sizeof(double) * cells));
    if (e->precision != CMSL_FP64) {
        TRY(e->alloc((void **)&e->d_phi[2], sizeof(double) * cells));
        TRY(e->alloc((void **)&e->d_phi[3], sizeof(double) * cells));
        TRY(e->alloc((void **)&e->d_phi[4], sizeof(double) * cells));
    }
    TRY(e->alloc((void **)&e->d_counter, sizeof(unsigned int) * (4 + n)));
    TRY(e->alloc((void **)&e->d_err, sizeof(int)));
    TRY(e->alloc((void **)&e->d_solve, sizeof(SolveDev) * n));
    {
        // every film's potential rotation valid from creation on (set_state
        // sets the same): FP32_REFINED buffers 0..3 in use, 4 free
        std::vector<SolveDev> S0((size_t)n);
        for (SolveDev &x : S0) {
            x = SolveDev{};
            if (e->precision != CMSL_FP64) { x.phi_prev = 1; x.phi_prev2 = 2; x.phi_prev3 = 3; }
        }
        CK(cudaMemcpy(e->d_solve, S0.data(), sizeof(SolveDev) * n, cudaMemcpyHostToDevice));
    }
    TRY(e->alloc((void **)&e->d_ctl, sizeof(Ctl)));
    TRY(ensure_schedule(e, 16, 16));

    if (e->precision != CMSL_FP64) {
        // FP32 stencil passes: the one-eps residual pass when every
        // depolarised film has one eps
        bool uni = true;
        for (int fi = 0; fi < n; ++fi) uni &= !e->fh[fi].dep || fds[fi].uni_eps != 0;
        // tensor-copy staging when every film has full tiles (CMSL_NO_TMA=1:
        // the cp.async ring for all)
        const char *nt = getenv("CMSL_NO_TMA");
        e->tma = !(nt && atoi(nt) != 0);
        for (int fi = 0; fi < n; ++fi) e->tma = e->tma && e->fh[fi].nx % TX == 0 && e->fh[fi].ny % TY == 0;
        // the cp.async ring at every tile height, the tensor copies at TY
        // rows; batches take the kernels that finish each film in its own
        // last block
        const bool fb = n > 1;
        if (fb) {
            e->refine_cp[0] = uni ? (void *)k_refine32<true, R32_NS, 4, true> : (void *)k_refine32<false, R32_NS, 4, true>;
            e->refine_cp[1] = uni ? (void *)k_refine32<true, R32_NS, 8, true> : (void *)k_refine32<false, R32_NS, 8, true>;
            e->refine_cp[2] = uni ? (void *)k_refine32<true, R32_NS, 16, true> : (void *)k_refine32<false, R32_NS, 16, true>;
            e->tdgl_cp[0] = (void *)k_tdgl32<T32_NS, 4, false, true>;
            e->tdgl_cp[1] = (void *)k_tdgl32<T32_NS, 8, false, true>;
            e->tdgl_cp[2] = (void *)k_tdgl32<T32_NS, 16, false, true>;
            e->tdgl_def[0] = (void *)k_tdgl32<T32_NS, 4, true, true>;
            e->tdgl_def[1] = (void *)k_tdgl32<T32_NS, 8, true, true>;
            e->tdgl_def[2] = (void *)k_tdgl32<T32_NS, 16, true, true>;
        } else {
            e->refine_cp[0] = uni ? (void *)k_refine32<true, R32_NS, 4> : (void *)k_refine32<false, R32_NS, 4>;
            e->refine_cp[1] = uni ? (void *)k_refine32<true, R32_NS, 8> : (void *)k_refine32<false, R32_NS, 8>;
            e->refine_cp[2] = uni ? (void *)k_refine32<true, R32_NS, 16> : (void *)k_refine32<false, R32_NS, 16>;
            e->tdgl_cp[0] = (void *)k_tdgl32<T32_NS, 4>;
            e->tdgl_cp[1] = (void *)k_tdgl32<T32_NS, 8>;
            e->tdgl_cp[2] = (void *)k_tdgl32<T32_NS, 16>;
            e->tdgl_def[0] = (void *)k_tdgl32<T32_NS, 4, true>;
            e->tdgl_def[1] = (void *)k_tdgl32<T32_NS, 8, true>;
            e->tdgl_def[2] = (void *)k_tdgl32<T32_NS, 16, true>;
        }
        e->refine_cp_smem[0] = uni ? r32_smem<true, 4>() : r32_smem<false, 4>();
        e->refine_cp_smem[1] = uni ? r32_smem<true, 8>() : r32_smem<false, 8>();
        e->refine_cp_smem[2] = uni ? r32_smem<true, 16>() : r32_smem<false, 16>();
        e->tdgl_cp_smem[0] = t32_smem<4>();
        e->tdgl_cp_smem[1] = t32_smem<8>();
        e->tdgl_cp_smem[2] = t32_smem<16>();
        // deferred checks: some film's step can end on an exact direct solve
        const char *df = getenv("CMSL_DEFER");
        e->defer = e->spectral && !e->persistent && !(df && atoi(df) == 0);
        bool any_def = false;
        for (int fi = 0; fi < n; ++fi) any_def |= fds[fi].defer_ok != 0;
        e->defer = e->defer && any_def;
        e->tdgl_def_smem[0] = t32_smem<4, true>();
        e->tdgl_def_smem[1] = t32_smem<8, true>();
        e->tdgl_def_smem[2] = t32_smem<16, true>();
        for (int v = 0; v < 3; ++v) {
            CK(cudaFuncSetAttribute(e->refine_cp[v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)e->refine_cp_smem[v]));
            CK(cudaFuncSetAttribute(e->tdgl_cp[v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)e->tdgl_cp_smem[v]));
            CK(cudaFuncSetAttribute(e->tdgl_def[v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)e->tdgl_def_smem[v]));
        }
        if (e->tma) {
            TRY(make_maps(e));
            if (fb) e->refine_tma = uni ? (void *)k_refine32t<true, RT_NS, true> : (void *)k_refine32t<false, RT_NS, true>;
            else e->refine_tma = uni ? (void *)k_refine32t<true, RT_NS> : (void *)k_refine32t<false, RT_NS>;
            e->refine_tma_smem = uni ? rt_smem<true>() : rt_smem<false>();
            e->tdgl_tma = fb ? (void *)k_tdgl32t<TT_NS, true> : (void *)k_tdgl32t<TT_NS>;
            e->tdgl_tma_smem = TT_SMEM;
            CK(cudaFuncSetAttribute(e->refine_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)e->refine_tma_smem));
            CK(cudaFuncSetAttribute(e->tdgl_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->tdgl_tma_smem));
        }
        // CMSL_STAGING=<tdgl><residual> (digits 0 cp.async ring, 1 tensor
        // copies) fixes the staging of films with full tiles; the autotuner
        // then keeps it
        int st_t = STG_TMA, st_r = STG_TMA;
        const char *sg = getenv("CMSL_STAGING");
        e->staging_fixed = false;
        if (sg && strlen(sg) == 2 && sg[0] >= '0' && sg[0] < '0' + N_STG && sg[1] >= '0' && sg[1] < '0' + N_STG) {
            st_t = sg[0] - '0';
            st_r = sg[1] - '0';
            e->staging_fixed = true;
        }
        e->stage(st_t, st_r);
        if (!e->staging_fixed) {
            std::lock_guard<std::mutex> lk(g_tuned_mu);
            const auto hit = g_tuned.find(shape_key(e));
            if (hit != g_tuned.end()) e->stage(hit->second.stg_tdgl, hit->second.stg_refine);
        }
    }
    const Dev d = e->dev(0);
    if (e->precision == CMSL_FP64) k_dinv<double><<<(int)e->items.size(), NT>>>(d, (double *)e->d_dinv);
    else k_dinv<float><<<(int)e->items.size(), NT>>>(d, (float *)e->d_dinv);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    return CMSL_OK;
}

// State of one film.  P goes into the set the next step reads (Ctl::cur);
// phi into the film's slice of every potential buffer; the film's solver
// slot restarts.  reset_clock also zeroes the shared step counters.
cmsl_status set_state(Engine *e, int film, const double *const P[6], const double *phi, bool reset_clock)
{
    if (!P) return fail(CMSL_ERR_ARG, "NULL argument");
    if (film < 0 || film >= e->n_films) return fail(CMSL_ERR_ARG, "film %d outside [0,%d)", film, e->n_films);
    for (int q = 0; q < 6; ++q)
        if (!P[q]) return fail(CMSL_ERR_ARG, "P[%d] is NULL", q);
    CK(cudaDeviceSynchronize());
    e->has_state = true;
    if (reset_clock) CK(cudaMemset(e->d_ctl, 0, sizeof(Ctl)));
    const FilmHost &hf = e->fh[film];
    if (e->precision != CMSL_FP64 && e->host_direct) {
        // one launch: P into set cur, phi (or zero) into buffer 0, x = 0.
        // The other potential buffers are not read before they hold this
        // run's potentials (SolveDev::hist starts at 1, or 0 without phi).
        StateIn s{};
        for (int q = 0; q < 6; ++q) s.P[q] = P[q];
        s.phi = phi;
        for (int set = 0; set < 2; ++set)
            for (int j = 0; j < 3; ++j) s.pair[set][j] = (float2 *)e->d_P[set][2 * j] + hf.off;
        s.phi0 = (float2 *)e->d_phi[0] + hf.off;
        s.x = (float *)e->d_x + hf.off;
        s.ctl = e->d_ctl;
        s.n = hf.N;
        k_state_in<<<XFER_GRID, XFER_NT>>>(s);
        CK(cudaGetLastError());
        SolveDev S0{};
        S0.phi_prev = 1;
        S0.phi_prev2 = 2;
        S0.phi_prev3 = 3;
        S0.hist = phi ? 1 : 0;
        CK(cudaMemcpyAsync(e->d_solve + film, &S0, sizeof(SolveDev), cudaMemcpyHostToDevice, 0));
        CK(cudaDeviceSynchronize());
        return CMSL_OK;
    }
    Ctl c;
    CK(cudaMemcpy(&c, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    if (e->precision == CMSL_FP64) TRY(put_fields<double>(e, film, c.cur, P));
    else TRY(put_fields<float>(e, film, c.cur, P));
    const FilmHost &h = e->fh[film];
    if (e->precision == CMSL_FP64) {
        double *dst = e->d_phi[0] + h.off;
        if (phi) CK(cudaMemcpy(dst, phi, sizeof(double) * h.N, cudaMemcpyHostToDevice));
        else CK(cudaMemset(dst, 0, sizeof(double) * h.N));
        CK(cudaMemcpy(e->d_phi[1] + h.off, dst, sizeof(double) * h.N, cudaMemcpyDeviceToDevice));
    } else if (e->host_direct) {
        // double-float (hi, lo) pairs per cell; the previous potentials
        // start equal to the given one
        float2 *b0 = (float2 *)e->d_phi[0] + h.off;
        if (phi) {
            k_phi_in<<<XFER_GRID, XFER_NT>>>(phi, b0, h.N);
            CK(cudaGetLastError());
        } else {
            CK(cudaMemset(b0, 0, sizeof(float2) * h.N));
        }
        for (int q = 1; q < 4; ++q)
            CK(cudaMemcpy((float2 *)e->d_phi[q] + h.off, b0, sizeof(float2) * h.N, cudaMemcpyDeviceToDevice));
        CK(cudaMemset((float *)e->d_x + h.off, 0, sizeof(float) * h.N));
    } else {
        // double-float (hi, lo) pairs per cell
        std::vector<float2> hl((size_t)h.N, make_float2(0.f, 0.f));
        if (phi)
            for (long long i = 0; i < h.N; ++i) {
                const df v = df_from_double(phi[i]);
                hl[i] = make_float2(v.h, v.l);
            }
        // the previous potentials start equal to the given one (no extrapolation on step 1)
        for (int q = 0; q < 4; ++q)
            CK(cudaMemcpy((float2 *)e->d_phi[q] + h.off, hl.data(), sizeof(float2) * h.N, cudaMemcpyHostToDevice));
        CK(cudaMemset((float *)e->d_x + h.off, 0, sizeof(float) * h.N));
    }
    SolveDev S0{};
    S0.phi_cur = 0;
    S0.phi_prev = e->precision == CMSL_FP64 ? 0 : 1;
    S0.phi_prev2 = e->precision == CMSL_FP64 ? 0 : 2;
    S0.phi_prev3 = e->precision == CMSL_FP64 ? 0 : 3;
    S0.hist = phi ? 1 : 0;              // a state without a potential starts from zero
    CK(cudaMemcpy(e->d_solve + film, &S0, sizeof(SolveDev), cudaMemcpyHostToDevice));
    return CMSL_OK;
}

cmsl_status get_state(Engine *e, int film, double *const P[6], double *phi)
{
    if (film < 0 || film >= e->n_films) return fail(CMSL_ERR_ARG, "film %d outside [0,%d)", film, e->n_films);
    CK(cudaDeviceSynchronize());
    if (e->precision != CMSL_FP64) {
        // every wanted output page-locked: one launch
        StateOut s{};
        bool all = true;
        for (int q = 0; q < 6 && P; ++q)
            if (P[q]) all = all && (s.P[q] = locked_dst(P[q])) != nullptr;
        if (phi) all = all && (s.phi = locked_dst(phi)) != nullptr;
        if (all) {
            const FilmHost &hf = e->fh[film];
            for (int set = 0; set < 2; ++set)
                for (int j = 0; j < 3; ++j) s.pair[set][j] = (const float2 *)e->d_P[set][2 * j] + hf.off;
            for (int b = 0; b < 5; ++b) s.phib[b] = (const float2 *)e->d_phi[b] + hf.off;
            s.ctl = e->d_ctl;
            s.S = e->d_solve + film;
            s.n = hf.N;
            k_state_out<<<XFER_GRID, XFER_NT>>>(s);
            CK(cudaGetLastError());
            CK(cudaDeviceSynchronize());
            return CMSL_OK;
        }
    }
    Ctl c;
    SolveDev S;
    CK(cudaMemcpy(&c, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&S, e->d_solve + film, sizeof(SolveDev), cudaMemcpyDeviceToHost));
    if (P) {
        if (e->precision == CMSL_FP64) TRY(get_fields<double>(e, film, c.cur, P));
        else TRY(get_fields<float>(e, film, c.cur, P));
    }
    const FilmHost &h = e->fh[film];
    if (phi) {
        double *dv = e->precision == CMSL_FP64 ? nullptr : locked_dst(phi);
        if (e->precision == CMSL_FP64) {
            CK(cudaMemcpy(phi, e->d_phi[S.phi_cur] + h.off, sizeof(double) * h.N, cudaMemcpyDeviceToHost));
        } else if (dv) {
            k_phi_out<<<XFER_GRID, XFER_NT>>>((const float2 *)e->d_phi[S.phi_cur] + h.off, dv, h.N);
            CK(cudaGetLastError());
            CK(cudaDeviceSynchronize());
        } else {
            const float2 *b = (const float2 *)e->d_phi[S.phi_cur] + h.off;
            void *stg = nullptr;
            std::vector<float2> tmp;
            if (e->host_direct) {
                TRY(pinned_stage(e, &stg));
            } else {
                tmp.resize((size_t)h.N);
                stg = tmp.data();
            }
            const float2 *hl = (const float2 *)stg;
            CK(cudaMemcpy((void *)hl, b, sizeof(float2) * h.N, cudaMemcpyDeviceToHost));
            parallel_for(h.N, [&](long long i0, long long i1) {
                for (long long i = i0; i < i1; ++i) phi[i] = (double)hl[i].x + (double)hl[i].y;
            });
        }
    }
    return CMSL_OK;
}

// Ez and row are [n_films][n_steps] host arrays (row may be NULL).
cmsl_status run(Engine *e, int n_steps, const double *Ez, const int32_t *row, void *stream)
{
    if (n_steps < 0 || (n_steps > 0 && !Ez)) return fail(CMSL_ERR_ARG, "bad run arguments");
    if (n_steps == 0) return CMSL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t F = (size_t)e->n_films, ns = (size_t)n_steps;
    int nrows = 0;
    std::vector<int> rows(F * ns, -1);
    if (row)
        for (size_t s = 0; s < F * ns; ++s) {
            rows[s] = row[s] < 0 ? -1 : row[s];
            nrows = std::max(nrows, rows[s] + 1);
        }
    TRY(ensure_schedule(e, n_steps, nrows));
    CK(cudaMemcpy2DAsync(e->d_wave, sizeof(double) * e->wstride, Ez, sizeof(double) * ns, sizeof(double) * ns, F,
                         cudaMemcpyHostToDevice, st));
    CK(cudaMemcpy2DAsync(e->d_rows, sizeof(int) * e->wstride, rows.data(), sizeof(int) * ns, sizeof(int) * ns, F,
                         cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(&e->d_ctl->run_step, 0, sizeof(int), st));
    for (int fi = 0; fi < e->n_films; ++fi) CK(cudaMemsetAsync(&e->d_solve[fi].sticky, 0, sizeof(int), st));
    e->stream = st;
    e->last_steps = n_steps;
    if (e->use_graph) {
        if (!e->graph_valid) TRY(build_graph(e));
        // one launch: the graph's step loop runs until run_step == stop
        CK(cudaMemcpyAsync(&e->d_ctl->stop, &n_steps, sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaGraphLaunch(e->exec, st));
    } else {
        for (int s = 0; s < n_steps; ++s) TRY(step_direct(e, st));
        if (e->defer) TRY(defer_close_direct(e, st));
    }
    // the host rows vector must stay alive until the copy above has run
    CK(cudaStreamSynchronize(st));
    return CMSL_OK;
}

cmsl_status sync(Engine *e, int32_t *film_status)
{
    CK(cudaStreamSynchronize(e->stream));
    CK(cudaGetLastError());
    std::vector<SolveDev> S((size_t)e->n_films);
    CK(cudaMemcpy(S.data(), e->d_solve, sizeof(SolveDev) * S.size(), cudaMemcpyDeviceToHost));
    if (e->cg.err) {
        int err = 0;
        CK(cudaMemcpy(&err, e->cg.err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) return fail(CMSL_ERR_CUDA, "persistent PCG grid barrier timed out");
    }
    if (e->d_err) {
        int err = 0;
        CK(cudaMemcpy(&err, e->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err & TMA_ERR_WAIT) return fail(CMSL_ERR_CUDA, "a tensor-copy wait of a stencil pass timed out");
    }
    int first = -1;
    for (int fi = 0; fi < e->n_films; ++fi) {
        if (film_status) film_status[fi] = S[fi].sticky;
        if (S[fi].sticky != 0 && first < 0) first = fi;
    }
    if (first >= 0) {
        const int s = S[first].sticky;
        const char *what = s == 1 ? "breakdown" : "invalid initial residual";
        if (e->n_films > 1)
            return fail(CMSL_ERR_PCG, "PCG failure (status %d: %s) in at least one step of film %d", s, what, first);
        return fail(CMSL_ERR_PCG, "PCG failure (status %d: %s) in at least one step", s, what);
    }
    return CMSL_OK;
}

cmsl_status get_rows(Engine *e, int film, int first, int n, double *out)
{
    if (!out || film < 0 || film >= e->n_films || first < 0 || n < 0 || first + n > e->rstride)
        return fail(CMSL_ERR_ARG, "bad row range");
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(out, e->d_rowbuf + ((size_t)film * e->rstride + first) * 11, sizeof(double) * 11 * n,
                  cudaMemcpyDeviceToHost));
    return CMSL_OK;
}

cmsl_status get_iters(Engine *e, int film, int n, int32_t *iters, int32_t *refine)
{
    if (film < 0 || film >= e->n_films || n < 0 || n > e->wstride) return fail(CMSL_ERR_ARG, "bad count");
    CK(cudaDeviceSynchronize());
    const size_t o = (size_t)film * e->wstride;
    if (iters) CK(cudaMemcpy(iters, e->d_iters + o, sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (refine) CK(cudaMemcpy(refine, e->d_refine + o, sizeof(int) * n, cudaMemcpyDeviceToHost));
    return CMSL_OK;
}

// ms[0] TDGL, ms[1] solve set-up / first refinement pass, ms[2] and ms[3] the
// PCG kernels (persistent FP32 solver: ms[2] per iteration, ms[3] the step
// end; direct solve: ms[2] the solve, ms[3] the update pass, 0 under
// deferred checks, whose TDGL kernel forms the check and is timed with every
// depolarised film pending).  The kernels run in force mode, which leaves the
// solver state as it is, so every repetition times the same kind of pass; the
// TDGL step forms a sweep row and every launch's last block its film totals,
// as in a step, without writing them.
cmsl_status time_kernels(Engine *e, int reps, void *stream, double *ms)
{
    if (!ms || reps < 1) return fail(CMSL_ERR_ARG, "bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaDeviceSynchronize());
    const int nit = (int)e->items.size();
    const size_t F = (size_t)e->n_films;
    Dev d = e->dev(0);
    d.force = 1;
    const Fields<double> F64 = e->fields<double>();
    const Fields<float> F32 = e->fields<float>();
    std::vector<double> e0(F, 0.0);
    std::vector<int> row0(F, 0);        // a sweep row, as every step of the benchmark schedules forms one
    CK(cudaMemcpy2D(e->d_wave, sizeof(double) * e->wstride, e0.data(), sizeof(double), sizeof(double), F,
                    cudaMemcpyHostToDevice));
    CK(cudaMemcpy2D(e->d_rows, sizeof(int) * e->wstride, row0.data(), sizeof(int), sizeof(int), F,
                    cudaMemcpyHostToDevice));
    CK(cudaMemset(&e->d_ctl->run_step, 0, sizeof(int)));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    const bool fp64 = e->precision == CMSL_FP64;
    std::vector<SolveDev> S(F);
    for (int kind = 0; kind < 4; ++kind) {
        if (kind == 3 && !fp64 && e->defer) {
            ms[3] = 0.0;                // the check runs inside the TDGL step (ms[0])
            continue;
        }
        CK(cudaMemcpy(S.data(), e->d_solve, sizeof(SolveDev) * F, cudaMemcpyDeviceToHost));
        for (SolveDev &s : S) {
            // FP32 passes: kind 1 a step's first residual pass, kind 3 (direct
            // solve) the update pass that follows it
            s.outer_active = 1; s.active = 1; s.iters = 1; s.status = 0;
            s.refine = (!fp64 && kind == 1) ? 0 : 1;
            s.upd = (e->spectral && kind == 3) ? 1 : 0;
            s.alpha = 1e-3; s.beta = 0.5; s.rz = s.rz0 = 1.0;
            s.inner_tol2 = 0.0; s.inner_max = CG_TIMING_ITERS;
        }
        CK(cudaMemcpy(e->d_solve, S.data(), sizeof(SolveDev) * F, cudaMemcpyHostToDevice));
        // one untimed launch, then `reps` timed ones
        for (int r = -1; r < reps; ++r) {
            if (r == 0) CK(cudaEventRecord(a, st));
            switch (kind) {
            case 0:
                if (fp64) k_tdgl<double, Exact><<<nit, NT, 0, st>>>(d, F64);
                else TRY(launch_tdgl32(e, st, d, F32));
                break;
            case 1:
                if (fp64) k_rhs<double, Exact><<<nit, NT, 0, st>>>(d, F64);
                else TRY(launch_refine(e, st, d, F32));
                break;
            case 2:
                if (fp64) {
                    k_spmv<double, Exact><<<nit, NT, 0, st>>>(d, F64);
                } else if (e->spectral) {
                    TRY(spec_launch(e, st, d, F32));
                } else if (e->persistent) {
                    // one persistent solve of CG_TIMING_ITERS iterations
                    Dev dd = d;
                    CgBuf B = e->cg;
                    const float *dv = (const float *)e->d_dinv;
                    void *args[] = {&dd, &B, &dv};
                    CK(cudaMemsetAsync(e->cg.arrive, 0, sizeof(unsigned int), st));
                    CK(cudaLaunchCooperativeKernel(e->cg_fn, e->cg_grid, PNT, args, e->cg_smem, st));
                    CK(cudaMemcpyAsync(e->d_solve, S.data(), sizeof(SolveDev) * F, cudaMemcpyHostToDevice, st));
                } else {
                    k_spmv<float, Fast><<<nit, NT, 0, st>>>(d, F32);
                }
                break;
            default:
                if (fp64) k_update<double, Exact, false><<<nit, NT, 0, st>>>(d, F64);
                else if (e->spectral) TRY(launch_refine(e, st, d, F32));                 // update pass
                else if (e->persistent) k_step_end<<<1, 32, 0, st>>>(d);                 // no fourth kernel
                else k_update<float, Fast, true><<<nit, NT, 0, st>>>(d, F32);
                break;
            }
            CK(cudaGetLastError());
        }
        CK(cudaEventRecord(b, st));
        CK(cudaEventSynchronize(b));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, a, b));
        ms[kind] = (double)t / reps;
        if (kind == 2 && !fp64 && e->persistent) ms[kind] /= CG_TIMING_ITERS;
        CK(cudaMemcpy(e->d_solve, S.data(), sizeof(SolveDev) * F, cudaMemcpyHostToDevice));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return CMSL_OK;
}

cmsl_status autotune_items(Engine *e, int32_t *zchunk);

// The autotuner's trial steps (FP32): every buffer a step reads or writes is
// copied aside before the trials and back before each, so that every
// candidate tiling runs the same steps from the same state -- a sweep row a
// step, field 0 -- and the films end the tuning as they began.  Films that
// have no state yet (P = 0 gives b = 0 and no solve) get a fixed pseudo-random
// P of amplitude 0.05 for the trials.
struct StepSnapshot {
    std::vector<std::pair<void *, size_t>> regions;
    char *store = nullptr;
    ~StepSnapshot() { if (store) cudaFree(store); }
};

static size_t snap_pad(size_t n) { return (n + 255) & ~(size_t)255; }

cmsl_status snapshot_take(Engine *e, StepSnapshot &s)
{
    const size_t cells = (size_t)e->ncells, F = (size_t)e->n_films;
    for (int set = 0; set < 2; ++set) s.regions.push_back({e->d_P[set][0], 6 * e->esz * cells});
    for (int b = 0; b < 5; ++b)
        if (e->d_phi[b]) s.regions.push_back({e->d_phi[b], sizeof(double) * cells});
    s.regions.push_back({e->d_x, e->esz * cells});
    s.regions.push_back({e->d_r, e->esz * cells});
    s.regions.push_back({e->d_solve, sizeof(SolveDev) * F});
    s.regions.push_back({e->d_ctl, sizeof(Ctl)});
    s.regions.push_back({e->d_rowbuf, sizeof(double) * 11 * (size_t)e->rstride * F});
    s.regions.push_back({e->d_iters, sizeof(int) * (size_t)e->wstride * F});
    s.regions.push_back({e->d_refine, sizeof(int) * (size_t)e->wstride * F});
    size_t bytes = 0;
    for (const auto &r : s.regions) bytes += snap_pad(r.second);
    CK(cudaMalloc(&s.store, bytes));
    size_t o = 0;
    for (const auto &r : s.regions) {
        CK(cudaMemcpy(s.store + o, r.first, r.second, cudaMemcpyDeviceToDevice));
        o += snap_pad(r.second);
    }
    return CMSL_OK;
}

cmsl_status snapshot_put(const StepSnapshot &s)
{
    size_t o = 0;
    for (const auto &r : s.regions) {
        CK(cudaMemcpy(r.first, s.store + o, r.second, cudaMemcpyDeviceToDevice));
        o += snap_pad(r.second);
    }
    return CMSL_OK;
}

// ms per step of W + K trial steps (the last K timed) from snapshot s.
cmsl_status trial_steps(Engine *e, const StepSnapshot &s, bool synthetic, double *ms)
{
    constexpr int W = 4, K = 8;
    TRY(snapshot_put(s));
    if (synthetic) {
        for (int set = 0; set < 2; ++set)
            k_trial_P<<<XFER_GRID, XFER_NT>>>((float *)e->d_P[set][0], 6LL * e->ncells);
        CK(cudaGetLastError());
    }
    const size_t F = (size_t)e->n_films;
    std::vector<double> Ez(F * (W + K), 0.0);
    std::vector<int32_t> rows(F * (W + K), 0);
    TRY(run(e, W, Ez.data(), rows.data(), nullptr));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, nullptr));
    TRY(run(e, K, Ez.data(), rows.data(), nullptr));
    CK(cudaEventRecord(b, nullptr));
    CK(cudaEventSynchronize(b));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = (double)t / K;
    return CMSL_OK;
}

// Tile-shape autotuner: times trial steps (FP32, trial_steps) or the TDGL
// step and the PCG kernels (FP64) for z chunks 4, 8, 16, ... up to the
// thickest film, tile heights and stagings, keeps the fastest, and remembers
// it for handles of the same film-shape class.
cmsl_status autotune(Engine *e, int32_t *zchunk)
{
    // the FP64 PCG kernels update the potential in place when timed: keep a copy
    const size_t pbytes = sizeof(double) * (size_t)e->ncells;
    double *saved = nullptr;
    if (e->precision == CMSL_FP64) {
        CK(cudaMalloc(&saved, 2 * pbytes));
        CK(cudaMemcpy(saved, e->d_phi[0], pbytes, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(saved + e->ncells, e->d_phi[1], pbytes, cudaMemcpyDeviceToDevice));
    }
    const cmsl_status st = autotune_items(e, zchunk);
    if (saved) {
        cudaMemcpy(e->d_phi[0], saved, pbytes, cudaMemcpyDeviceToDevice);
        cudaMemcpy(e->d_phi[1], saved + e->ncells, pbytes, cudaMemcpyDeviceToDevice);
        cudaFree(saved);
    }
    if (st != CMSL_OK) return st;
    CK(cudaGetLastError());
    return CMSL_OK;
}

cmsl_status autotune_items(Engine *e, int32_t *zchunk)
{
    int maxnz = 1;
    for (const FilmHost &h : e->fh) maxnz = std::max(maxnz, h.nz);
    // every chunk count of the thickest film down to chunks of ZCHUNK_MIN
    // planes (the wave count of the stencil passes is what differs)
    std::vector<int> cands;
    for (int nc = 1; nc == 1 || (maxnz + nc - 1) / nc >= ZCHUNK_MIN; ++nc) {
        const int c = (maxnz + nc - 1) / nc;
        if (cands.empty() || cands.back() != c) cands.push_back(c);
    }
    // per tile height (FP32; 4, 8 and 16 rows unless CMSL_TILE_Y fixed one)
    // and z chunk: every pair of stagings of the TDGL and the residual passes
    // where the tensor copies apply (8-row tiles of films with full tiles; a
    // staging fixed by CMSL_STAGING is kept)
    const bool fp32 = e->precision != CMSL_FP64;
    std::unique_ptr<StepSnapshot> snap;
    if (fp32) {
        snap.reset(new StepSnapshot());
        TRY(snapshot_take(e, *snap));
    }
    std::vector<int> tys;
    if (!fp32 || e->tile_fixed) tys.push_back(e->stile_ty);
    else tys.assign(TILE_YS, TILE_YS + 3);
    Tuned best{0, e->stg_tdgl, e->stg_refine, e->stile_ty};
    double best_ms = 0.0;
    std::vector<std::pair<double, Tuned>> tried;       // FP32: every candidate's trial time
    for (int ty : tys) {
        if (fp32 && e->staging_fixed && (e->stg_tdgl || e->stg_refine) && ty != TY) continue;
        e->stile_ty = ty;
        const bool tune_stg = fp32 && e->tma && !e->staging_fixed && ty == TY;
        const int nst = tune_stg ? N_STG : 1;
        const int fixed_t = e->stg_tdgl, fixed_r = e->stg_refine;
        for (int c : cands) {
            TRY(set_items(e, c));
            if (!fp32) {
                double ms[4] = {0, 0, 0, 0};
                TRY(time_kernels(e, 5, nullptr, ms));
                const double t = ms[0] + ms[1] + ms[2] + ms[3];
                if (best.zchunk == 0 || t < best_ms) {
                    best = Tuned{c, e->stg_tdgl, e->stg_refine, ty};
                    best_ms = t;
                }
                continue;
            }
            // every staging pair of the TDGL and the residual passes (the
            // TDGL that forms deferred checks has the cp.async ring only)
            for (int vt = 0; vt < nst; ++vt)
                for (int vr = 0; vr < nst; ++vr) {
                    if (vt && e->defer) continue;
                    if (tune_stg) e->stage(vt, vr);
                    else e->stage(e->staging_fixed ? fixed_t : STG_CP, e->staging_fixed ? fixed_r : STG_CP);
                    double t = 0.0;
                    TRY(trial_steps(e, *snap, !e->has_state, &t));
                    const Tuned cand = tune_stg ? Tuned{c, vt, vr, ty} : Tuned{c, e->stg_tdgl, e->stg_refine, ty};
                    tried.emplace_back(t, cand);
                    if (best.zchunk == 0 || t < best_ms) {
                        best = cand;
                        best_ms = t;
                    }
                }
        }
    }
    // the three fastest again, twice each in turn, warm: one short trial
    // (8 steps) can rank candidates within a few percent of each other
    // wrongly; the least total of the three trials wins
    if (tried.size() > 1) {
        std::stable_sort(tried.begin(), tried.end(),
                         [](const std::pair<double, Tuned> &x, const std::pair<double, Tuned> &y) { return x.first < y.first; });
        tried.resize(std::min<size_t>(3, tried.size()));
        for (int round = 0; round < 2; ++round)
            for (auto &c : tried) {
                e->stile_ty = c.second.tile_y;
                TRY(set_items(e, c.second.zchunk));
                e->stage(c.second.stg_tdgl, c.second.stg_refine);
                double t = 0.0;
                TRY(trial_steps(e, *snap, !e->has_state, &t));
                c.first += t;
            }
        size_t bi = 0;
        for (size_t q = 1; q < tried.size(); ++q)
            if (tried[q].first < tried[bi].first) bi = q;
        best = tried[bi].second;
    }
    if (snap) TRY(snapshot_put(*snap));
    e->stile_ty = best.tile_y;
    TRY(set_items(e, best.zchunk));
    if (fp32) e->stage(best.stg_tdgl, best.stg_refine);
    if (!e->staging_fixed && !e->tile_fixed) {
        std::lock_guard<std::mutex> lk(g_tuned_mu);
        g_tuned[shape_key(e)] = best;
    }
    if (zchunk) *zchunk = best.zchunk;
    return CMSL_OK;
}

void tile_config(const Engine *e, int32_t cfg[4])
{
    cfg[0] = TX;
    cfg[1] = e->precision != CMSL_FP64 ? e->stile_ty : TY;
    cfg[2] = e->zchunk;
    cfg[3] = e->stg_tdgl | (e->stg_refine << 2);
}

size_t device_bytes(const Engine *e)
{
    return e->bytes + (size_t)e->n_films * ((size_t)e->wstride * (sizeof(double) + 3 * sizeof(int)) +
                                            (size_t)e->rstride * 11 * sizeof(double));
}

}  // namespace

extern "C" {

const char *cmsl_last_error(void) { return g_err.c_str(); }
const char *cmsl_version(void) { return "cmsl_gb300 0.2 (sm_103a)"; }

cmsl_status cmsl_film_create(const cmsl_film_desc *dsc, cmsl_film **out)
{
    if (!dsc || !out) return fail(CMSL_ERR_ARG, "NULL argument");
    *out = nullptr;
    std::unique_ptr<cmsl_film> f(new cmsl_film());
    TRY(engine_create(f.get(), dsc, 1));
    *out = f.release();
    return CMSL_OK;
}

cmsl_status cmsl_film_destroy(cmsl_film *f)
{
    if (f) {
        cudaDeviceSynchronize();
        delete f;
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_set_state(cmsl_film *f, const double *const P[6], const double *phi)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL argument");
    return set_state(f, 0, P, phi, true);
}

cmsl_status cmsl_film_get_state(cmsl_film *f, double *const P[6], double *phi)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    return get_state(f, 0, P, phi);
}

cmsl_status cmsl_host_alloc(size_t bytes, void **out)
{
    if (!out) return fail(CMSL_ERR_ARG, "NULL out");
    *out = nullptr;
    CK(cudaMallocHost(out, bytes ? bytes : 16));
    return CMSL_OK;
}

cmsl_status cmsl_host_free(void *p)
{
    if (p) CK(cudaFreeHost(p));
    return CMSL_OK;
}

cmsl_status cmsl_film_run(cmsl_film *f, int n_steps, const double *Ez, const int32_t *row, void *stream)
{
    if (!f) return fail(CMSL_ERR_ARG, "bad run arguments");
    return run(f, n_steps, Ez, row, stream);
}

cmsl_status cmsl_film_sync(cmsl_film *f)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    return sync(f, nullptr);
}

cmsl_status cmsl_film_get_rows(cmsl_film *f, int first, int n, double *out)
{
    if (!f) return fail(CMSL_ERR_ARG, "bad row range");
    return get_rows(f, 0, first, n, out);
}

cmsl_status cmsl_film_get_iters(cmsl_film *f, int n, int32_t *iters, int32_t *refine)
{
    if (!f) return fail(CMSL_ERR_ARG, "bad count");
    return get_iters(f, 0, n, iters, refine);
}

cmsl_status cmsl_film_tdgl_step(cmsl_film *f, double Ez)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    const int rowm1 = -1;
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(f->d_wave, &Ez, sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(f->d_rows, &rowm1, sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(&f->d_ctl->run_step, 0, sizeof(int)));
    const int nit = (int)f->items.size();
    const Dev d = f->dev(0);
    if (f->precision == CMSL_FP64) k_tdgl<double, Exact><<<nit, NT>>>(d, f->fields<double>());
    else TRY(launch_tdgl32(f, nullptr, d, f->fields<float>()));
    k_step_end<<<1, 32>>>(d);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    return CMSL_OK;
}

cmsl_status cmsl_film_depol(cmsl_film *f, int32_t *iters, int32_t *status)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    CK(cudaDeviceSynchronize());
    // the solve kernels read the new Pm from set cur^1: point it at the current state
    Ctl c;
    CK(cudaMemcpy(&c, f->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    Fields<double> F64 = f->fields<double>();
    Fields<float> F32 = f->fields<float>();
    for (int q = 0; q < 6; ++q) {
        F64.P[c.cur ^ 1][q] = F64.P[c.cur][q];
        F32.P[c.cur ^ 1][q] = F32.P[c.cur][q];
    }
    SolveDev S;
    CK(cudaMemcpy(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
    S.outer_active = 1; S.active = 0; S.refine = 0; S.total_iters = 0; S.iters = 0; S.status = 0; S.upd = 0;
    CK(cudaMemcpy(f->d_solve, &S, sizeof(SolveDev), cudaMemcpyHostToDevice));
    const Dev d = f->dev(0);
    if (f->precision != CMSL_FP64) {
        // the first residual pass reads the warm start from the free buffer
        k_extrap<<<(unsigned)f->items.size(), NT>>>(d);
        CK(cudaGetLastError());
    }
    TRY(solve_direct(f, nullptr, d, F64, F32));
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
    if (iters) { iters[0] = S.total_iters; if (f->precision != CMSL_FP64) iters[1] = S.refine; }
    if (status) *status = S.status;
    return CMSL_OK;
}

// Depol_field over caller device arrays: Pm in, phi (warm start in,
// solution out) and E out, converted by kernels on `stream`; nothing passes
// through the host and nothing is allocated.
cmsl_status cmsl_film_depol_device(cmsl_film *f, const double *Pmx, const double *Pmy, const double *Pmz,
                                   double *phi, double *Ex, double *Ey, double *Ez, void *stream, int32_t *iters,
                                   int32_t *status)
{
    if (!f || !Pmx || !Pmy || !Pmz || !phi) return fail(CMSL_ERR_ARG, "NULL argument");
    if (f->n_films != 1) return fail(CMSL_ERR_ARG, "depol_device: single films only");
    if (!f->any_dep) return fail(CMSL_ERR_STATE, "depol_device: the film has no depolarisation solve");
    cudaStream_t st = (cudaStream_t)stream;
    const FilmHost &h = f->fh[0];
    Ctl c;
    SolveDev S;
    CK(cudaMemcpyAsync(&c, f->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    f->has_state = true;
    const double *src[3] = {Pmx, Pmy, Pmz};
    const int ps = f->pstride();
    for (int q = 0; q < 3; ++q) {
        if (f->precision == CMSL_FP64)
            k_host_in<double><<<XFER_GRID, XFER_NT, 0, st>>>(src[q], (double *)f->d_P[c.cur][q] + h.off, h.N, 1);
        else
            k_host_in<float><<<XFER_GRID, XFER_NT, 0, st>>>(src[q], (float *)f->d_P[c.cur][q] + ps * h.off, h.N, ps);
    }
    // the warm start: every potential buffer holds phi (no extrapolation)
    if (f->precision == CMSL_FP64) {
        for (int q = 0; q < 2; ++q)
            CK(cudaMemcpyAsync(f->d_phi[q] + h.off, phi, sizeof(double) * h.N, cudaMemcpyDeviceToDevice, st));
    } else {
        float2 *b0 = (float2 *)f->d_phi[0] + h.off;
        k_phi_in<<<XFER_GRID, XFER_NT, 0, st>>>(phi, b0, h.N);
        for (int q = 1; q < 4; ++q)
            CK(cudaMemcpyAsync((float2 *)f->d_phi[q] + h.off, b0, sizeof(float2) * h.N, cudaMemcpyDeviceToDevice, st));
    }
    CK(cudaGetLastError());
    S = SolveDev{};
    S.phi_cur = 0;
    S.phi_prev = f->precision == CMSL_FP64 ? 0 : 1;
    S.phi_prev2 = f->precision == CMSL_FP64 ? 0 : 2;
    S.phi_prev3 = f->precision == CMSL_FP64 ? 0 : 3;
    S.hist = 1;                         // the caller's potential
    S.outer_active = 1;
    CK(cudaMemcpyAsync(f->d_solve, &S, sizeof(SolveDev), cudaMemcpyHostToDevice, st));
    // the solve kernels read the new Pm from set cur^1: point it at set cur
    Fields<double> F64 = f->fields<double>();
    Fields<float> F32 = f->fields<float>();
    for (int q = 0; q < 6; ++q) {
        F64.P[c.cur ^ 1][q] = F64.P[c.cur][q];
        F32.P[c.cur ^ 1][q] = F32.P[c.cur][q];
    }
    const Dev d = f->dev(0);
    const unsigned nit = (unsigned)f->items.size();
    if (f->precision != CMSL_FP64) {
        k_extrap<<<nit, NT, 0, st>>>(d);
        CK(cudaGetLastError());
    }
    TRY(solve_direct(f, st, d, F64, F32));
    CK(cudaMemcpyAsync(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (f->precision == CMSL_FP64) {
        CK(cudaMemcpyAsync(phi, f->d_phi[S.phi_cur] + h.off, sizeof(double) * h.N, cudaMemcpyDeviceToDevice, st));
    } else {
        k_phi_out<<<XFER_GRID, XFER_NT, 0, st>>>((const float2 *)f->d_phi[S.phi_cur] + h.off, phi, h.N);
    }
    if (Ex && Ey && Ez) {
        if (f->precision == CMSL_FP64) k_efield<<<nit, NT, 0, st>>>(d, Ex - h.off, Ey - h.off, Ez - h.off);
        else k_efield_df<<<nit, NT, 0, st>>>(d, Ex - h.off, Ey - h.off, Ez - h.off);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    if (iters) { iters[0] = S.total_iters; iters[1] = f->precision != CMSL_FP64 ? S.refine : 0; }
    if (status) *status = S.status;
    return CMSL_OK;
}

cmsl_status cmsl_film_apply_operator(cmsl_film *f, const double *x, double *y)
{
    if (!f || !x || !y) return fail(CMSL_ERR_ARG, "NULL argument");
    CK(cudaDeviceSynchronize());
    const int nit = (int)f->items.size();
    const long long N = f->fh[0].N;   // the film's cells (the buffers are padded beyond)
    const Dev d = f->dev(0);
    if (f->precision == CMSL_FP64) {
        CK(cudaMemcpy(f->d_q, x, sizeof(double) * N, cudaMemcpyHostToDevice));
        k_apply_op<double, Exact><<<nit, NT>>>(d, (const double *)f->d_q, (double *)f->d_r);
        CK(cudaGetLastError());
        CK(cudaMemcpy(y, f->d_r, sizeof(double) * N, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> t((size_t)N);
        for (long long i = 0; i < N; ++i) t[i] = (float)x[i];
        CK(cudaMemcpy(f->d_q, t.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
        k_apply_op<float, Fast><<<nit, NT>>>(d, (const float *)f->d_q, (float *)f->d_r);
        CK(cudaGetLastError());
        CK(cudaMemcpy(t.data(), f->d_r, sizeof(float) * N, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < N; ++i) y[i] = t[i];
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_efield(cmsl_film *f, double *Ex, double *Ey, double *Ez)
{
    if (!f || !Ex || !Ey || !Ez) return fail(CMSL_ERR_ARG, "NULL argument");
    CK(cudaDeviceSynchronize());
    const long long N = f->fh[0].N;   // the film's cells (the buffers are padded beyond)
    double *e = nullptr;
    CK(cudaMalloc(&e, sizeof(double) * 3 * N));
    const Dev d = f->dev(0);
    if (f->precision == CMSL_FP64) k_efield<<<(int)f->items.size(), NT>>>(d, e, e + N, e + 2 * N);
    else k_efield_df<<<(int)f->items.size(), NT>>>(d, e, e + N, e + 2 * N);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpy(Ex, e, sizeof(double) * N, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(Ey, e + N, sizeof(double) * N, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(Ez, e + 2 * N, sizeof(double) * N, cudaMemcpyDeviceToHost);
    cudaFree(e);
    if (err != cudaSuccess) return fail(CMSL_ERR_CUDA, "efield: %s", cudaGetErrorString(err));
    return CMSL_OK;
}

cmsl_status cmsl_film_diag_inv(cmsl_film *f, double *dinv)
{
    if (!f || !dinv) return fail(CMSL_ERR_ARG, "NULL argument");
    CK(cudaDeviceSynchronize());
    const long long N = f->fh[0].N;   // the film's cells (the buffers are padded beyond)
    if (f->precision == CMSL_FP64) {
        CK(cudaMemcpy(dinv, f->d_dinv, sizeof(double) * N, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> t((size_t)N);
        CK(cudaMemcpy(t.data(), f->d_dinv, sizeof(float) * N, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < N; ++i) dinv[i] = t[i];
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_checkpoint_write(cmsl_film *f, const char *path, int peloop, int count, double Ez_ext,
                                       double incEz)
{
    if (!f || !path) return fail(CMSL_ERR_ARG, "NULL argument");
    const FilmHost &h = f->fh[0];
    const size_t N = (size_t)h.N;
    std::vector<double> P[6], E[3], phi(N);
    double *Pp[6], *Ep[3];
    for (int q = 0; q < 6; ++q) { P[q].resize(N); Pp[q] = P[q].data(); }
    for (int q = 0; q < 3; ++q) { E[q].resize(N); Ep[q] = E[q].data(); }
    TRY(get_state(f, 0, Pp, phi.data()));
    TRY(cmsl_efield_host(h.nx, h.ny, h.nz, h.h, h.zbc, phi.data(), Ep[0], Ep[1], Ep[2]));
    return cmsl_checkpoint_write(path, h.nx, h.ny, h.nz, peloop, count, Ez_ext, incEz, Pp, Ep);
}

cmsl_status cmsl_film_checkpoint_read(cmsl_film *f, const char *path, int *peloop, int *count, double *Ez_ext,
                                      double *incEz)
{
    if (!f || !path) return fail(CMSL_ERR_ARG, "NULL argument");
    const FilmHost &h = f->fh[0];
    const size_t N = (size_t)h.N;
    std::vector<double> P[6];
    double *Pp[6];
    for (int q = 0; q < 6; ++q) { P[q].resize(N); Pp[q] = P[q].data(); }
    TRY(cmsl_checkpoint_read(path, h.nx, h.ny, h.nz, peloop, count, Ez_ext, incEz, Pp, nullptr));
    const double *Pc[6] = {Pp[0], Pp[1], Pp[2], Pp[3], Pp[4], Pp[5]};
    TRY(set_state(f, 0, Pc, nullptr, true));
    if (h.dep) {
        // the file holds E of the potential solved from these P (the last
        // step's solve): solve for it again
        int32_t it[2] = {0, 0}, st = 0;
        TRY(cmsl_film_depol(f, it, &st));
        if (st != 0 && st != 3) return fail(CMSL_ERR_PCG, "checkpoint restart: PCG failure (status %d)", st);
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_time_kernels(cmsl_film *f, int reps, void *stream, double *ms)
{
    if (!f) return fail(CMSL_ERR_ARG, "bad arguments");
    return time_kernels(f, reps, stream, ms);
}

cmsl_status cmsl_film_inner_solver(cmsl_film *f, int *solver)
{
    if (!f || !solver) return fail(CMSL_ERR_ARG, "NULL argument");
    *solver = f->spectral ? CMSL_INNER_DIRECT : CMSL_INNER_PCG;
    return CMSL_OK;
}

cmsl_status cmsl_film_autotune(cmsl_film *f, int32_t *zchunk)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    return autotune(f, zchunk);
}

cmsl_status cmsl_film_tile_config(cmsl_film *f, int32_t cfg[4])
{
    if (!f || !cfg) return fail(CMSL_ERR_ARG, "NULL argument");
    tile_config(f, cfg);
    return CMSL_OK;
}

cmsl_status cmsl_film_device_bytes(cmsl_film *f, size_t *bytes)
{
    if (!f || !bytes) return fail(CMSL_ERR_ARG, "NULL argument");
    *bytes = device_bytes(f);
    return CMSL_OK;
}

// ----------------------------------------------------------------- batches

cmsl_status cmsl_batch_create(const cmsl_film_desc *descs, int n_films, cmsl_batch **out)
{
    if (!descs || !out) return fail(CMSL_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (n_films < 1 || n_films > (1 << 20)) return fail(CMSL_ERR_ARG, "n_films %d out of range", n_films);
    std::unique_ptr<cmsl_batch> b(new cmsl_batch());
    TRY(engine_create(b.get(), descs, n_films));
    *out = b.release();
    return CMSL_OK;
}

cmsl_status cmsl_batch_destroy(cmsl_batch *b)
{
    if (b) {
        cudaDeviceSynchronize();
        delete b;
    }
    return CMSL_OK;
}

cmsl_status cmsl_batch_set_state(cmsl_batch *b, int film, const double *const P[6], const double *phi)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return set_state(b, film, P, phi, false);
}

cmsl_status cmsl_batch_get_state(cmsl_batch *b, int film, double *const P[6], double *phi)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return get_state(b, film, P, phi);
}

cmsl_status cmsl_batch_run(cmsl_batch *b, int n_steps, const double *Ez, const int32_t *row, void *stream)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return run(b, n_steps, Ez, row, stream);
}

cmsl_status cmsl_batch_sync(cmsl_batch *b, int32_t *film_status)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return sync(b, film_status);
}

cmsl_status cmsl_batch_get_rows(cmsl_batch *b, int film, int first, int n, double *out)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return get_rows(b, film, first, n, out);
}

cmsl_status cmsl_batch_get_iters(cmsl_batch *b, int film, int n, int32_t *iters, int32_t *refine)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return get_iters(b, film, n, iters, refine);
}

cmsl_status cmsl_batch_time_kernels(cmsl_batch *b, int reps, void *stream, double *ms)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return time_kernels(b, reps, stream, ms);
}

cmsl_status cmsl_batch_inner_solver(cmsl_batch *b, int *solver)
{
    if (!b || !solver) return fail(CMSL_ERR_ARG, "NULL argument");
    *solver = b->spectral ? CMSL_INNER_DIRECT : CMSL_INNER_PCG;
    return CMSL_OK;
}

cmsl_status cmsl_batch_autotune(cmsl_batch *b, int32_t *zchunk)
{
    if (!b) return fail(CMSL_ERR_ARG, "NULL batch");
    return autotune(b, zchunk);
}

cmsl_status cmsl_batch_tile_config(cmsl_batch *b, int32_t cfg[4])
{
    if (!b || !cfg) return fail(CMSL_ERR_ARG, "NULL argument");
    tile_config(b, cfg);
    return CMSL_OK;
}

cmsl_status cmsl_batch_device_bytes(cmsl_batch *b, size_t *bytes)
{
    if (!b || !bytes) return fail(CMSL_ERR_ARG, "NULL argument");
    *bytes = device_bytes(b);
    return CMSL_OK;
}

}  // extern "C"
