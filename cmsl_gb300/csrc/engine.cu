// engine.cu -- film lifecycle, CUDA-graph construction and the run loop.
//
// One time step is one CUDA graph:
//   CMSL_FP64:          k_tdgl -> k_rhs -> WHILE(inner){ k_spmv -> k_update } -> k_step_end
//   CMSL_FP32_REFINED:  k_tdgl -> WHILE(outer){ k_refine -> WHILE(inner){ k_spmv -> k_update } }
//                       -> k_step_end
// The WHILE conditions are set on the device by the last block of k_rhs,
// k_refine and k_update, so a step never returns to the host: the PCG loop of
// the reference (depol_varEPS.cu:472-522, two blocking Ddot per iteration) and
// its per-step cudaMalloc/cublasCreate churn (:373-393, :585-593) are gone.
// The applied field and the output-row schedule of the P-E loop are device
// arrays indexed by a device step counter, so the same graph is relaunched
// for every step.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cmsl.h"
#include "kernels.cuh"
#include "pcg_persist.cuh"

using namespace cmsl;

namespace {

thread_local std::string g_err;

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

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(CMSL_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                  \
    } while (0)

double harm(double a, double b)   // depol_varEPS.cu:10-15
{
    const double eps = 1e-20;
    double denom = a + b;
    if (denom < eps) denom = eps;
    return (2.0 * a * b) / denom;
}

}  // namespace

void cmsl_internal_set_error(const char *msg) { g_err = msg; }

struct cmsl_film {
    int precision = CMSL_FP64;
    int nx = 0, ny = 0, nz = 0, dep = 0, ng = 0;
    long long N = 0;
    size_t esz = 8;
    std::vector<int4> items;
    FilmDev fd{};
    // device buffers
    std::vector<void *> allocs;
    size_t bytes = 0;
    FilmDev *d_films = nullptr;
    int4 *d_items = nullptr;
    uint32_t *d_code = nullptr;
    void *d_TR = nullptr;
    double *d_phi[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    double *d_partial = nullptr;
    unsigned int *d_counter = nullptr;
    SolveDev *d_solve = nullptr;
    Ctl *d_ctl = nullptr;
    void *d_P[2][6] = {};
    void *d_r = nullptr, *d_q = nullptr, *d_dinv = nullptr, *d_x = nullptr, *d_p[2] = {};
    // schedule buffers (grown on demand)
    double *d_wave = nullptr;
    int *d_rows = nullptr;
    double *d_rowbuf = nullptr;
    int *d_iters = nullptr, *d_refine = nullptr;
    int wstride = 0, rstride = 0;
    int last_steps = 0;
    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_valid = false;
    bool use_graph = true;
    cudaStream_t stream = nullptr;
    CgBuf cg{};                 // FP32_REFINED persistent PCG vectors
    int cg_grid = 0;
    bool uni_eps = false;       // every material has the same eps_r
    bool cg_fused = false;      // single-sweep variant (CMSL_PCG_FUSED=1) instead of two-phase
    void *cg_fn = nullptr;      // the persistent solver kernel in use
    size_t cg_smem = 0;

    ~cmsl_film()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void *p : allocs) cudaFree(p);
        if (d_wave) cudaFree(d_wave);
        if (d_rows) cudaFree(d_rows);
        if (d_rowbuf) cudaFree(d_rowbuf);
        if (d_iters) cudaFree(d_iters);
        if (d_refine) cudaFree(d_refine);
    }

    template <class T> Fields<T> fields() const
    {
        Fields<T> F{};
        for (int s = 0; s < 2; ++s)
            for (int q = 0; q < 6; ++q) F.P[s][q] = (T *)d_P[s][q];
        F.r = (T *)d_r; F.q = (T *)d_q; F.dinv = (T *)d_dinv; F.x = (T *)d_x;
        F.p[0] = (T *)d_p[0]; F.p[1] = (T *)d_p[1];
        F.TR = (const T *)d_TR;
        return F;
    }

    Dev dev(int use_cond, cudaGraphConditionalHandle hi = 0, cudaGraphConditionalHandle ho = 0) const
    {
        Dev d{};
        d.films = d_films; d.items = d_items; d.n_films = 1; d.n_items = (int)items.size();
        d.code = d_code; d.ncells = N; d.phi[0] = d_phi[0]; d.phi[1] = d_phi[1]; d.phi[2] = d_phi[2]; d.phi[3] = d_phi[3]; d.phi[4] = d_phi[4];
        d.partial = d_partial; d.counter = d_counter; d.solve = d_solve; d.ctl = d_ctl;
        d.wave = d_wave; d.rows = d_rows; d.rowbuf = d_rowbuf;
        d.iters_log = d_iters; d.refine_log = d_refine;
        d.wstride = wstride; d.rstride = rstride;
        d.use_cond = use_cond; d.h_inner = hi; d.h_outer = ho;
        d.arrive = cg.arrive;
        return d;
    }

    cmsl_status alloc(void **p, size_t n)
    {
        cudaError_t e = cudaMalloc(p, n ? n : 16);
        if (e != cudaSuccess) {
            *p = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? CMSL_ERR_NOMEM : CMSL_ERR_CUDA,
                        "cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
        }
        allocs.push_back(*p);
        bytes += n;
        e = cudaMemset(*p, 0, n ? n : 16);
        if (e != cudaSuccess) return fail(CMSL_ERR_CUDA, "cudaMemset failed: %s", cudaGetErrorString(e));
        return CMSL_OK;
    }
};

namespace {

#define TRY(x)                               \
    do {                                     \
        cmsl_status s_ = (x);                \
        if (s_ != CMSL_OK) return s_;        \
    } while (0)

// z chunk: enough items to fill the 152 SMs a few times over, chunks >= 4 planes.
int pick_zchunk(int nx, int ny, int nz)
{
    const long long xy = (long long)((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
    const char *env = getenv("CMSL_ZCHUNK");
    if (env && atoi(env) > 0) return std::min(nz, atoi(env));
    const long long target = 8LL * 152;
    long long chunks = (target + xy - 1) / xy;
    int zc = (int)std::max<long long>(1, (nz + chunks - 1) / chunks);
    zc = std::max(zc, std::min(nz, 4));
    return std::min(zc, nz);
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

template <class T> cmsl_status upload_TR(cmsl_film *f, const double *TR)
{
    std::vector<T> tr((size_t)9 * f->ng);
    for (size_t i = 0; i < tr.size(); ++i) tr[i] = (T)TR[i];
    TRY(f->alloc(&f->d_TR, tr.size() * sizeof(T)));
    CK(cudaMemcpy(f->d_TR, tr.data(), tr.size() * sizeof(T), cudaMemcpyHostToDevice));
    return CMSL_OK;
}

cmsl_status ensure_schedule(cmsl_film *f, int n_steps, int n_rows)
{
    if (n_steps > f->wstride) {
        const int w = std::max(n_steps, 16);
        if (f->d_wave) { cudaFree(f->d_wave); cudaFree(f->d_rows); cudaFree(f->d_iters); cudaFree(f->d_refine); }
        f->d_wave = nullptr; f->d_rows = nullptr; f->d_iters = nullptr; f->d_refine = nullptr;
        CK(cudaMalloc(&f->d_wave, sizeof(double) * w));
        CK(cudaMalloc(&f->d_rows, sizeof(int) * w));
        CK(cudaMalloc(&f->d_iters, sizeof(int) * w));
        CK(cudaMalloc(&f->d_refine, sizeof(int) * w));
        f->wstride = w;
        f->graph_valid = false;
    }
    if (n_rows > f->rstride || !f->d_rowbuf) {
        const int r = std::max(n_rows, 16);
        if (f->d_rowbuf) cudaFree(f->d_rowbuf);
        f->d_rowbuf = nullptr;
        CK(cudaMalloc(&f->d_rowbuf, sizeof(double) * 11 * r));
        CK(cudaMemset(f->d_rowbuf, 0, sizeof(double) * 11 * r));
        f->rstride = r;
        f->graph_valid = false;
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
                       void *fn, int grid, int block, void **args, size_t smem = 0)
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

// Arguments must outlive graph instantiation only (node params are copied).
cmsl_status build_graph(cmsl_film *f)
{
    if (f->exec) { cudaGraphExecDestroy(f->exec); f->exec = nullptr; }
    if (f->graph) { cudaGraphDestroy(f->graph); f->graph = nullptr; }
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    f->graph = g;
    const int nit = (int)f->items.size();
    KArgs a;
    a.F64 = f->fields<double>();
    a.F32 = f->fields<float>();
    cudaGraphConditionalHandle h_outer = 0, h_inner = 0;
    const bool fp64 = f->precision == CMSL_FP64;
    cudaGraphNode_t n_tdgl, n_solve, n_end;
    if (!fp64 && f->dep) CK(cudaGraphConditionalHandleCreate(&h_outer, g, 1, cudaGraphCondAssignDefault));
    if (fp64 && f->dep) CK(cudaGraphConditionalHandleCreate(&h_inner, g, 0, cudaGraphCondAssignDefault));
    a.d = f->dev(1, h_inner, h_outer);
    void *args64[] = {&a.d, &a.F64};
    void *args32[] = {&a.d, &a.F32};
    void *args_d[] = {&a.d};
    if (fp64) TRY(add_kernel(g, &n_tdgl, nullptr, 0, (void *)k_tdgl<double, Exact>, nit, NT, args64));
    else TRY(add_kernel(g, &n_tdgl, nullptr, 0, (void *)k_tdgl<float, Fast>, nit, NT, args32));
    cudaGraphNode_t last = n_tdgl;
    if (f->dep) {
        if (fp64) {
            cudaGraphNode_t n_rhs, n_sp, n_up;
            cudaGraph_t body;
            TRY(add_kernel(g, &n_rhs, &last, 1, (void *)k_rhs<double, Exact>, nit, NT, args64));
            TRY(add_while(g, &n_solve, &n_rhs, 1, h_inner, &body));
            TRY(add_kernel(body, &n_sp, nullptr, 0, (void *)k_spmv<double, Exact>, nit, NT, args64));
            TRY(add_kernel(body, &n_up, &n_sp, 1, (void *)k_update<double, Exact, false>, nit, NT, args64));
            last = n_solve;
        } else {
            cudaGraph_t outer;
            cudaGraphNode_t n_ref, n_cg;
            TRY(add_while(g, &n_solve, &last, 1, h_outer, &outer));
            a.d = f->dev(1, 0, h_outer);
            TRY(add_kernel(outer, &n_ref, nullptr, 0, (void *)k_refine, nit, NT, args32));
            void *args_cg[] = {&a.d, &f->cg, &f->d_dinv};
            TRY(add_kernel(outer, &n_cg, &n_ref, 1, f->cg_fn, f->cg_grid, PNT, args_cg, f->cg_smem));
            cudaLaunchAttributeValue av{};
            av.cooperative = 1;
            CK(cudaGraphKernelNodeSetAttribute(n_cg, cudaLaunchAttributeCooperative, &av));
            last = n_solve;
        }
    }
    TRY(add_kernel(g, &n_end, &last, 1, (void *)k_step_end, 1, 32, args_d));
    CK(cudaGraphInstantiate(&f->exec, g, 0));
    f->graph_valid = true;
    return CMSL_OK;
}

cmsl_status read_flags(cmsl_film *f, cudaStream_t st, SolveDev *S)
{
    CK(cudaMemcpyAsync(S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return CMSL_OK;
}

// The depolarisation solve launched from the host, one kernel at a time,
// reading the loop flags back after each iteration.  Used by the
// single-piece test hooks and when graphs are disabled (CMSL_NO_GRAPH=1).
cmsl_status solve_direct(cmsl_film *f, cudaStream_t st, const Dev &d, const Fields<double> &F64,
                         const Fields<float> &F32)
{
    const int nit = (int)f->items.size();
    SolveDev S;
    if (f->precision == CMSL_FP64) {
        k_rhs<double, Exact><<<nit, NT, 0, st>>>(d, F64);
        CK(cudaGetLastError());
        for (int guard = 0;; ++guard) {
            TRY(read_flags(f, st, &S));
            if (!S.active) break;
            if (guard > f->fd.max_iter + 1) return fail(CMSL_ERR_STATE, "PCG loop did not stop");
            k_spmv<double, Exact><<<nit, NT, 0, st>>>(d, F64);
            k_update<double, Exact, false><<<nit, NT, 0, st>>>(d, F64);
            CK(cudaGetLastError());
        }
    } else {
        for (int og = 0;; ++og) {
            if (og > f->fd.max_refine + 1) return fail(CMSL_ERR_STATE, "refinement loop did not stop");
            k_refine<<<nit, NT, 0, st>>>(d, F32);
            CK(cudaGetLastError());
            TRY(read_flags(f, st, &S));
            if (S.active) {
                Dev dd = d;
                CgBuf B = f->cg;
                const float *dv = (const float *)f->d_dinv;
                void *args[] = {&dd, &B, &dv};
                CK(cudaLaunchCooperativeKernel(f->cg_fn, f->cg_grid, PNT, args, f->cg_smem, st));
                TRY(read_flags(f, st, &S));
            }
            if (!S.outer_active) break;
        }
    }
    return CMSL_OK;
}

cmsl_status step_direct(cmsl_film *f, cudaStream_t st)
{
    const int nit = (int)f->items.size();
    const Dev d = f->dev(0);
    const Fields<double> F64 = f->fields<double>();
    const Fields<float> F32 = f->fields<float>();
    if (f->precision == CMSL_FP64) k_tdgl<double, Exact><<<nit, NT, 0, st>>>(d, F64);
    else k_tdgl<float, Fast><<<nit, NT, 0, st>>>(d, F32);
    CK(cudaGetLastError());
    if (f->dep) TRY(solve_direct(f, st, d, F64, F32));
    k_step_end<<<1, 32, 0, st>>>(d);
    CK(cudaGetLastError());
    return CMSL_OK;
}

template <class T>
cmsl_status put_fields(cmsl_film *f, int set, const double *const P[6])
{
    std::vector<T> tmp((size_t)f->N);
    for (int q = 0; q < 6; ++q) {
        if (!P[q]) return fail(CMSL_ERR_ARG, "P[%d] is NULL", q);
        for (long long i = 0; i < f->N; ++i) tmp[i] = (T)P[q][i];
        CK(cudaMemcpy(f->d_P[set][q], tmp.data(), f->N * sizeof(T), cudaMemcpyHostToDevice));
    }
    return CMSL_OK;
}

template <class T>
cmsl_status get_fields(cmsl_film *f, int set, double *const P[6])
{
    std::vector<T> tmp((size_t)f->N);
    for (int q = 0; q < 6; ++q) {
        if (!P[q]) continue;
        CK(cudaMemcpy(tmp.data(), f->d_P[set][q], f->N * sizeof(T), cudaMemcpyDeviceToHost));
        for (long long i = 0; i < f->N; ++i) P[q][i] = (double)tmp[i];
    }
    return CMSL_OK;
}

}  // namespace

extern "C" {

const char *cmsl_last_error(void) { return g_err.c_str(); }
const char *cmsl_version(void) { return "cmsl_gb300 0.1 (sm_103a)"; }

cmsl_status cmsl_film_create(const cmsl_film_desc *dsc, cmsl_film **out)
{
    if (!dsc || !out) return fail(CMSL_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (dsc->nx < 1 || dsc->ny < 1 || dsc->nz < 3)
        return fail(CMSL_ERR_ARG, "grid %dx%dx%d: need nx, ny >= 1 and nz >= 3", dsc->nx, dsc->ny, dsc->nz);
    if (dsc->nx > 32767 || dsc->ny > 32767 || dsc->nz > 32767)
        return fail(CMSL_ERR_ARG, "grid dimension above 32767");
    if (dsc->n_grains < 1 || dsc->n_grains > (int)GID_MASK)
        return fail(CMSL_ERR_ARG, "n_grains %d out of range", dsc->n_grains);
    if (!dsc->omega || !dsc->grain_mat || !dsc->TR) return fail(CMSL_ERR_ARG, "omega/grain_mat/TR NULL");
    if (dsc->precision != CMSL_FP64 && dsc->precision != CMSL_FP32_REFINED)
        return fail(CMSL_ERR_ARG, "precision %d unknown", dsc->precision);
    if (dsc->zbc != CMSL_DIRICHLET && dsc->zbc != CMSL_NEUMANN) return fail(CMSL_ERR_ARG, "zbc %d", dsc->zbc);
    if (!(dsc->del_h > 0.0) || !(dsc->del_t > 0.0)) return fail(CMSL_ERR_ARG, "del_h and del_t must be > 0");

    cmsl_film *f = new cmsl_film();
    std::unique_ptr<cmsl_film> guard(f);
    f->precision = dsc->precision;
    f->nx = dsc->nx; f->ny = dsc->ny; f->nz = dsc->nz;
    f->N = (long long)f->nx * f->ny * f->nz;
    f->dep = dsc->dep_flag != 0;
    f->ng = dsc->n_grains;
    f->esz = f->precision == CMSL_FP64 ? 8 : 4;
    const char *ng = getenv("CMSL_NO_GRAPH");
    f->use_graph = !(ng && atoi(ng) != 0);

    // per-cell code, interface flags (main.cu:13-42), material voxel counts
    const long long N = f->N, plane = (long long)f->nx * f->ny;
    std::vector<uint32_t> code((size_t)N);
    double nmat[3] = {0, 0, 0};
    for (int g = 0; g < f->ng; ++g)
        if (dsc->grain_mat[g] < 0 || dsc->grain_mat[g] > 2)
            return fail(CMSL_ERR_ARG, "grain %d has material %d (need 0..2)", g, dsc->grain_mat[g]);
    for (long long i = 0; i < N; ++i) {
        const int gid = dsc->omega[i];
        if (gid < 0 || gid >= f->ng) return fail(CMSL_ERR_ARG, "cell %lld has grain id %d outside [0,%d)", i, gid, f->ng);
        const int mat = dsc->grain_mat[gid];
        int iface;
        if (dsc->is_interface) {
            iface = dsc->is_interface[i] != 0;
        } else {
            const long long k = i / plane;
            iface = 0;
            if (mat == CMSL_FE && k > 0 && k < f->nz - 1) {
                const int mu = dsc->grain_mat[dsc->omega[i + plane]];
                const int md = dsc->grain_mat[dsc->omega[i - plane]];
                iface = (mu != CMSL_FE || md != CMSL_FE);
            }
        }
        code[i] = (uint32_t)gid | ((uint32_t)mat << 24) | ((uint32_t)iface << 26);
        nmat[mat] += 1.0;
    }

    // items: TX x TY x zchunk tiles
    const int zc = pick_zchunk(f->nx, f->ny, f->nz);
    for (int y0 = 0; y0 < f->ny; y0 += TY)
        for (int x0 = 0; x0 < f->nx; x0 += TX)
            for (int z0 = 0; z0 < f->nz; z0 += zc) {
                const int z1 = std::min(f->nz, z0 + zc);
                f->items.push_back(make_int4(0, x0, y0, z0 | (z1 << 16)));
            }

    FilmDev &fd = f->fd;
    fd.nx = f->nx; fd.ny = f->ny; fd.nz = f->nz; fd.zbc = dsc->zbc;
    fd.off = 0; fd.g_off = 0; fd.item_begin = 0; fd.item_end = (int)f->items.size();
    fd.dep_flag = f->dep;
    fd.warm = f->precision != CMSL_FP64 ? std::min(std::max(dsc->warm_start, 0), 3) : 0;
    fd.ref_id = f->nx / 2 + f->nx * (f->ny / 2 + (f->nz / 2) * f->ny);   // depol_varEPS.cu:339-346
    fd.crit = dsc->pcg_crit;
    fd.max_iter = dsc->max_iter;
    fd.max_refine = std::max(1, dsc->max_refine);
    fd.inner_max = std::max(1, dsc->inner_max_iter);
    const double h = dsc->del_h;
    fd.h = h; fd.dt = dsc->del_t; fd.eps0nd = dsc->eps_0_nd;
    fd.inv_N = 1.0 / ((double)f->nx * f->ny * f->nz);              // main.cu:405
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
    for (int q = 0; q < 3; ++q) fd.n_mat[q] = nmat[q];
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

    // device memory
    const size_t cells = (size_t)N;
    TRY(f->alloc((void **)&f->d_films, sizeof(FilmDev)));
    CK(cudaMemcpy(f->d_films, &fd, sizeof(FilmDev), cudaMemcpyHostToDevice));
    TRY(f->alloc((void **)&f->d_items, sizeof(int4) * f->items.size()));
    CK(cudaMemcpy(f->d_items, f->items.data(), sizeof(int4) * f->items.size(), cudaMemcpyHostToDevice));
    TRY(f->alloc((void **)&f->d_code, sizeof(uint32_t) * cells));
    CK(cudaMemcpy(f->d_code, code.data(), sizeof(uint32_t) * cells, cudaMemcpyHostToDevice));
    if (f->precision == CMSL_FP64) TRY(upload_TR<double>(f, dsc->TR));
    else TRY(upload_TR<float>(f, dsc->TR));
    for (int s = 0; s < 2; ++s)
        for (int q = 0; q < 6; ++q) TRY(f->alloc(&f->d_P[s][q], f->esz * cells));
    TRY(f->alloc(&f->d_r, f->esz * cells));
    TRY(f->alloc(&f->d_q, f->esz * cells));
    TRY(f->alloc(&f->d_dinv, f->esz * cells));
    TRY(f->alloc(&f->d_p[0], f->esz * cells));
    TRY(f->alloc(&f->d_p[1], f->esz * cells));
    if (f->precision != CMSL_FP64) {
        TRY(f->alloc(&f->d_x, f->esz * cells));
        // persistent single-reduction PCG: r ping-pong (r[0] is the shared r),
        // w and s ping-pong, x = correction, p in place
        CgBuf &B = f->cg;
        B.r[0] = (float *)f->d_r;
        TRY(f->alloc((void **)&B.r[1], 4 * cells));
        TRY(f->alloc((void **)&B.w[0], 4 * cells));
        TRY(f->alloc((void **)&B.w[1], 4 * cells));
        TRY(f->alloc((void **)&B.s[0], 4 * cells));
        TRY(f->alloc((void **)&B.s[1], 4 * cells));
        B.x = (float *)f->d_x;
        B.p = (float *)f->d_p[0];
        int dev = 0, nsm = 0, per = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        CK(cudaFuncSetAttribute(k_pcg_cg1<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PSMEM_BYTES));
        CK(cudaFuncSetAttribute(k_pcg_cg1<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PSMEM_BYTES));
        CK(cudaFuncSetAttribute(k_pcg_cg2<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P2SMEM_BYTES));
        CK(cudaFuncSetAttribute(k_pcg_cg2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P2SMEM_BYTES));
        f->uni_eps = dsc->mats[0].eps_r == dsc->mats[1].eps_r && dsc->mats[1].eps_r == dsc->mats[2].eps_r;
        const char *solver = getenv("CMSL_PCG_FUSED");
        f->cg_fused = solver && atoi(solver) != 0;
        if (f->cg_fused) {
            f->cg_fn = f->uni_eps ? (void *)k_pcg_cg1<true> : (void *)k_pcg_cg1<false>;
            f->cg_smem = PSMEM_BYTES;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg_cg1<false>, PNT, PSMEM_BYTES));
        } else {
            f->cg_fn = f->uni_eps ? (void *)k_pcg_cg2<true> : (void *)k_pcg_cg2<false>;
            f->cg_smem = P2SMEM_BYTES;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg_cg2<false>, PNT, P2SMEM_BYTES));
        }
        if (per < 1) return fail(CMSL_ERR_CUDA, "persistent PCG kernel cannot be resident");
        // stencil bricks of PZ planes; the grid is sized so that every block
        // gets the same number of bricks
        std::vector<int4> bricks;
        for (int y0 = 0; y0 < f->ny; y0 += TY)
            for (int x0 = 0; x0 < f->nx; x0 += TX)
                for (int z0 = 0; z0 < f->nz; z0 += PZ)
                    bricks.push_back(make_int4(0, x0, y0, z0 | (std::min(f->nz, z0 + PZ) << 16)));
        const int nb = (int)bricks.size(), maxg = per * nsm;
        const int per_block = (nb + maxg - 1) / maxg;
        f->cg_grid = f->cg_fused ? std::min<int>((int)f->items.size(), maxg) : (nb + per_block - 1) / per_block;
        TRY(f->alloc((void **)&B.bricks, sizeof(int4) * nb));
        CK(cudaMemcpy((void *)B.bricks, bricks.data(), sizeof(int4) * nb, cudaMemcpyHostToDevice));
        B.n_bricks = nb;
        TRY(f->alloc((void **)&B.part, sizeof(float4) * 2 * f->cg_grid));
        TRY(f->alloc((void **)&B.arrive, sizeof(unsigned int) * 2));
        TRY(f->alloc((void **)&B.err, sizeof(int) * 2));
    }
    TRY(f->alloc((void **)&f->d_phi[0], sizeof(double) * cells));
    TRY(f->alloc((void **)&f->d_phi[1], sizeof(double) * cells));
    if (f->precision != CMSL_FP64) {
        TRY(f->alloc((void **)&f->d_phi[2], sizeof(double) * cells));
        TRY(f->alloc((void **)&f->d_phi[3], sizeof(double) * cells));
        TRY(f->alloc((void **)&f->d_phi[4], sizeof(double) * cells));
    }
    TRY(f->alloc((void **)&f->d_partial, sizeof(double) * NPART * f->items.size()));
    TRY(f->alloc((void **)&f->d_counter, sizeof(unsigned int) * 4));
    TRY(f->alloc((void **)&f->d_solve, sizeof(SolveDev)));
    TRY(f->alloc((void **)&f->d_ctl, sizeof(Ctl)));
    TRY(ensure_schedule(f, 16, 16));

    const Dev d = f->dev(0);
    if (f->precision == CMSL_FP64) k_dinv<double><<<(int)f->items.size(), NT>>>(d, (double *)f->d_dinv);
    else k_dinv<float><<<(int)f->items.size(), NT>>>(d, (float *)f->d_dinv);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    *out = guard.release();
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
    if (!f || !P) return fail(CMSL_ERR_ARG, "NULL argument");
    CK(cudaDeviceSynchronize());
    CK(cudaMemset(f->d_ctl, 0, sizeof(Ctl)));
    CK(cudaMemset(f->d_solve, 0, sizeof(SolveDev)));
    if (f->precision == CMSL_FP64) TRY(put_fields<double>(f, 0, P));
    else TRY(put_fields<float>(f, 0, P));
    if (f->precision == CMSL_FP64) {
        if (phi) CK(cudaMemcpy(f->d_phi[0], phi, sizeof(double) * f->N, cudaMemcpyHostToDevice));
        else CK(cudaMemset(f->d_phi[0], 0, sizeof(double) * f->N));
    } else {
        // double-float: hi half then lo half
        std::vector<float> t((size_t)2 * f->N, 0.f);
        if (phi)
            for (long long i = 0; i < f->N; ++i) {
                const df v = df_from_double(phi[i]);
                t[i] = v.h;
                t[f->N + i] = v.l;
            }
        CK(cudaMemcpy(f->d_phi[0], t.data(), sizeof(float) * 2 * f->N, cudaMemcpyHostToDevice));
    }
    // the previous potential starts equal to the given one (no extrapolation on step 1)
    CK(cudaMemcpy(f->d_phi[1], f->d_phi[0], sizeof(double) * f->N, cudaMemcpyDeviceToDevice));
    for (int q = 2; q < 4; ++q)
        if (f->d_phi[q]) CK(cudaMemcpy(f->d_phi[q], f->d_phi[0], sizeof(double) * f->N, cudaMemcpyDeviceToDevice));
    SolveDev S0{};
    S0.phi_cur = 0;
    S0.phi_prev = f->precision == CMSL_FP64 ? 0 : 1;
    S0.phi_prev2 = f->precision == CMSL_FP64 ? 0 : 2;
    S0.phi_prev3 = f->precision == CMSL_FP64 ? 0 : 3;
    CK(cudaMemcpy(f->d_solve, &S0, sizeof(SolveDev), cudaMemcpyHostToDevice));
    if (f->precision != CMSL_FP64) CK(cudaMemset(f->d_x, 0, f->esz * f->N));
    return CMSL_OK;
}

cmsl_status cmsl_film_get_state(cmsl_film *f, double *const P[6], double *phi)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    CK(cudaDeviceSynchronize());
    Ctl c;
    SolveDev S;
    CK(cudaMemcpy(&c, f->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
    if (P) {
        if (f->precision == CMSL_FP64) TRY(get_fields<double>(f, c.cur, P));
        else TRY(get_fields<float>(f, c.cur, P));
    }
    if (phi) {
        if (f->precision == CMSL_FP64) {
            CK(cudaMemcpy(phi, f->d_phi[S.phi_cur], sizeof(double) * f->N, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> t((size_t)2 * f->N);
            CK(cudaMemcpy(t.data(), f->d_phi[S.phi_cur], sizeof(float) * 2 * f->N, cudaMemcpyDeviceToHost));
            for (long long i = 0; i < f->N; ++i) phi[i] = (double)t[i] + (double)t[f->N + i];
        }
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_run(cmsl_film *f, int n_steps, const double *Ez, const int32_t *row, void *stream)
{
    if (!f || n_steps < 0 || (n_steps > 0 && !Ez)) return fail(CMSL_ERR_ARG, "bad run arguments");
    if (n_steps == 0) return CMSL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int nrows = 0;
    std::vector<int> rows((size_t)n_steps, -1);
    if (row)
        for (int s = 0; s < n_steps; ++s) {
            rows[s] = row[s] < 0 ? -1 : row[s];
            nrows = std::max(nrows, rows[s] + 1);
        }
    TRY(ensure_schedule(f, n_steps, nrows));
    CK(cudaMemcpyAsync(f->d_wave, Ez, sizeof(double) * n_steps, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(f->d_rows, rows.data(), sizeof(int) * n_steps, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(&f->d_ctl->run_step, 0, sizeof(int), st));
    CK(cudaMemsetAsync(&f->d_solve->sticky, 0, sizeof(int), st));
    f->stream = st;
    f->last_steps = n_steps;
    if (f->use_graph) {
        if (!f->graph_valid) TRY(build_graph(f));
        for (int s = 0; s < n_steps; ++s) CK(cudaGraphLaunch(f->exec, st));
    } else {
        for (int s = 0; s < n_steps; ++s) TRY(step_direct(f, st));
    }
    // the host rows vector must stay alive until the copy above has run
    CK(cudaStreamSynchronize(st));
    return CMSL_OK;
}

cmsl_status cmsl_film_sync(cmsl_film *f)
{
    if (!f) return fail(CMSL_ERR_ARG, "NULL film");
    CK(cudaStreamSynchronize(f->stream));
    CK(cudaGetLastError());
    SolveDev S;
    CK(cudaMemcpy(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
    if (f->cg.err) {
        int e = 0;
        CK(cudaMemcpy(&e, f->cg.err, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) return fail(CMSL_ERR_CUDA, "persistent PCG grid barrier timed out");
    }
    if (S.sticky != 0)
        return fail(CMSL_ERR_PCG, "PCG failure (status %d: %s) in at least one step", S.sticky,
                    S.sticky == 1 ? "breakdown" : "invalid initial residual");
    return CMSL_OK;
}

cmsl_status cmsl_film_get_rows(cmsl_film *f, int first, int n, double *out)
{
    if (!f || !out || first < 0 || n < 0 || first + n > f->rstride) return fail(CMSL_ERR_ARG, "bad row range");
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(out, f->d_rowbuf + (size_t)first * 11, sizeof(double) * 11 * n, cudaMemcpyDeviceToHost));
    return CMSL_OK;
}

cmsl_status cmsl_film_get_iters(cmsl_film *f, int n, int32_t *iters, int32_t *refine)
{
    if (!f || n < 0 || n > f->wstride) return fail(CMSL_ERR_ARG, "bad count");
    CK(cudaDeviceSynchronize());
    if (iters) CK(cudaMemcpy(iters, f->d_iters, sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (refine) CK(cudaMemcpy(refine, f->d_refine, sizeof(int) * n, cudaMemcpyDeviceToHost));
    return CMSL_OK;
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
    else k_tdgl<float, Fast><<<nit, NT>>>(d, f->fields<float>());
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
    S.outer_active = 1; S.active = 0; S.refine = 0; S.total_iters = 0; S.iters = 0; S.status = 0;
    CK(cudaMemcpy(f->d_solve, &S, sizeof(SolveDev), cudaMemcpyHostToDevice));
    const Dev d = f->dev(0);
    TRY(solve_direct(f, nullptr, d, F64, F32));
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
    if (iters) { iters[0] = S.total_iters; if (f->precision != CMSL_FP64) iters[1] = S.refine; }
    if (status) *status = S.status;
    return CMSL_OK;
}

cmsl_status cmsl_film_apply_operator(cmsl_film *f, const double *x, double *y)
{
    if (!f || !x || !y) return fail(CMSL_ERR_ARG, "NULL argument");
    CK(cudaDeviceSynchronize());
    const int nit = (int)f->items.size();
    const Dev d = f->dev(0);
    if (f->precision == CMSL_FP64) {
        CK(cudaMemcpy(f->d_q, x, sizeof(double) * f->N, cudaMemcpyHostToDevice));
        k_apply_op<double, Exact><<<nit, NT>>>(d, (const double *)f->d_q, (double *)f->d_r);
        CK(cudaGetLastError());
        CK(cudaMemcpy(y, f->d_r, sizeof(double) * f->N, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> t((size_t)f->N);
        for (long long i = 0; i < f->N; ++i) t[i] = (float)x[i];
        CK(cudaMemcpy(f->d_q, t.data(), sizeof(float) * f->N, cudaMemcpyHostToDevice));
        k_apply_op<float, Fast><<<nit, NT>>>(d, (const float *)f->d_q, (float *)f->d_r);
        CK(cudaGetLastError());
        CK(cudaMemcpy(t.data(), f->d_r, sizeof(float) * f->N, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < f->N; ++i) y[i] = t[i];
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_efield(cmsl_film *f, double *Ex, double *Ey, double *Ez)
{
    if (!f || !Ex || !Ey || !Ez) return fail(CMSL_ERR_ARG, "NULL argument");
    if (f->precision != CMSL_FP64) return fail(CMSL_ERR_STATE, "efield: FP64 films only");
    CK(cudaDeviceSynchronize());
    double *e = nullptr;
    CK(cudaMalloc(&e, sizeof(double) * 3 * f->N));
    const Dev d = f->dev(0);
    k_efield<<<(int)f->items.size(), NT>>>(d, e, e + f->N, e + 2 * f->N);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpy(Ex, e, sizeof(double) * f->N, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(Ey, e + f->N, sizeof(double) * f->N, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(Ez, e + 2 * f->N, sizeof(double) * f->N, cudaMemcpyDeviceToHost);
    cudaFree(e);
    if (err != cudaSuccess) return fail(CMSL_ERR_CUDA, "efield: %s", cudaGetErrorString(err));
    return CMSL_OK;
}

cmsl_status cmsl_film_diag_inv(cmsl_film *f, double *dinv)
{
    if (!f || !dinv) return fail(CMSL_ERR_ARG, "NULL argument");
    CK(cudaDeviceSynchronize());
    if (f->precision == CMSL_FP64) {
        CK(cudaMemcpy(dinv, f->d_dinv, sizeof(double) * f->N, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> t((size_t)f->N);
        CK(cudaMemcpy(t.data(), f->d_dinv, sizeof(float) * f->N, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < f->N; ++i) dinv[i] = t[i];
    }
    return CMSL_OK;
}

cmsl_status cmsl_film_time_kernels(cmsl_film *f, int reps, void *stream, double *ms)
{
    if (!f || !ms || reps < 1) return fail(CMSL_ERR_ARG, "bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaDeviceSynchronize());
    const int nit = (int)f->items.size();
    Dev d = f->dev(0);
    d.force = 1;
    const Fields<double> F64 = f->fields<double>();
    const Fields<float> F32 = f->fields<float>();
    const int rowm1 = -1;
    const double e0 = 0.0;
    CK(cudaMemcpy(f->d_wave, &e0, sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(f->d_rows, &rowm1, sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(&f->d_ctl->run_step, 0, sizeof(int)));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    const bool fp64 = f->precision == CMSL_FP64;
    SolveDev S;
    for (int kind = 0; kind < 4; ++kind) {
        CK(cudaMemcpy(&S, f->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
        S.outer_active = 1; S.active = 1; S.iters = 1; S.refine = 1; S.status = 0;
        S.alpha = 1e-3; S.beta = 0.5; S.rz = S.rz0 = 1.0;
        S.inner_tol2 = 0.0; S.inner_max = CG_TIMING_ITERS;
        CK(cudaMemcpy(f->d_solve, &S, sizeof(SolveDev), cudaMemcpyHostToDevice));
        // one untimed launch, then `reps` timed ones
        for (int r = -1; r < reps; ++r) {
            if (r == 0) CK(cudaEventRecord(a, st));
            switch (kind) {
            case 0:
                if (fp64) k_tdgl<double, Exact><<<nit, NT, 0, st>>>(d, F64);
                else k_tdgl<float, Fast><<<nit, NT, 0, st>>>(d, F32);
                break;
            case 1:
                if (fp64) k_rhs<double, Exact><<<nit, NT, 0, st>>>(d, F64);
                else k_refine<<<nit, NT, 0, st>>>(d, F32);
                break;
            case 2:
                if (fp64) {
                    k_spmv<double, Exact><<<nit, NT, 0, st>>>(d, F64);
                } else {
                    // one persistent solve of CG_TIMING_ITERS iterations
                    Dev dd = d;
                    CgBuf B = f->cg;
                    const float *dv = (const float *)f->d_dinv;
                    void *args[] = {&dd, &B, &dv};
                    CK(cudaMemsetAsync(f->cg.arrive, 0, sizeof(unsigned int), st));
                    CK(cudaLaunchCooperativeKernel(f->cg_fn, f->cg_grid, PNT, args, f->cg_smem, st));
                    CK(cudaMemcpyAsync(f->d_solve, &S, sizeof(SolveDev), cudaMemcpyHostToDevice, st));
                }
                break;
            default:
                if (fp64) k_update<double, Exact, false><<<nit, NT, 0, st>>>(d, F64);
                else k_step_end<<<1, 32, 0, st>>>(d);   // FP32 mode has no fourth kernel
                break;
            }
            CK(cudaGetLastError());
        }
        CK(cudaEventRecord(b, st));
        CK(cudaEventSynchronize(b));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, a, b));
        ms[kind] = (double)t / reps;
        if (kind == 2 && !fp64) ms[kind] /= CG_TIMING_ITERS;
        // the TDGL kernel flips nothing by itself; keep the state consistent
        CK(cudaMemcpy(f->d_solve, &S, sizeof(SolveDev), cudaMemcpyHostToDevice));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return CMSL_OK;
}

cmsl_status cmsl_film_device_bytes(cmsl_film *f, size_t *bytes)
{
    if (!f || !bytes) return fail(CMSL_ERR_ARG, "NULL argument");
    *bytes = f->bytes + (size_t)f->wstride * (sizeof(double) + 3 * sizeof(int)) +
             (size_t)f->rstride * 11 * sizeof(double);
    return CMSL_OK;
}

}  // extern "C"
