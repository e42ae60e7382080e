// engine.h -- the film/batch engine shared by the C-ABI translation units
// (engine.cu: lifecycle, graphs, run loop; adjoint.cu: loop gradients).
#pragma once
#include <cstdarg>
#include <string>
#include <vector>

#include "cmsl.h"
#include "kernels.cuh"
#include "pcg_persist.cuh"
#include "spectral.cuh"
#include "stencil32.cuh"
#include "stencil_tma.cuh"

namespace cmsl_eng {

using namespace cmsl;

// Records the message returned by cmsl_last_error() and returns s.
cmsl_status fail(cmsl_status s, const char *fmt, ...);

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ::cmsl_eng::fail(CMSL_ERR_CUDA, "%s failed: %s (%s:%d)", #call,            \
                                    cudaGetErrorString(e_), __FILE__, __LINE__);              \
    } while (0)

#define TRY(x)                               \
    do {                                     \
        cmsl_status s_ = (x);                \
        if (s_ != CMSL_OK) return s_;        \
    } while (0)

// Staging of the FP32 stencil passes (Engine::stage).
enum { STG_CP = 0, STG_TMA = 1, N_STG = 2 };

// Host view of one film of a handle.
struct FilmHost {
    int nx, ny, nz, ng, dep, zbc;
    long long N, off;   // cells, first cell
    double h;           // grid spacing (non-dimensional)
};

struct Engine {
    int precision = CMSL_FP64;
    int n_films = 0;
    long long ncells = 0;
    bool any_dep = false;
    size_t esz = 8;
    int max_iter_cap = 0, max_refine_cap = 0, inner_max_cap = 0;
    std::vector<FilmHost> fh;
    std::vector<FilmDev> fdh;           // host copy of the film tables
    std::vector<int4> items;
    size_t items_cap = 0;               // items the device arrays hold
    std::vector<int4> sitems;           // items of the FP32 stencil passes (tile height stile_ty)
    size_t sitems_cap = 0;
    int stile_ty = TY;
    long long xy_tiles = 0;             // column tiles of all films
    int zchunk = 0;                     // z chunk of the items (0: per-film heuristic)
    // device buffers
    std::vector<void *> allocs;
    size_t bytes = 0;
    FilmDev *d_films = nullptr;
    int4 *d_items = nullptr;
    int4 *d_sitems = nullptr;
    uint32_t *d_code = nullptr;
    void *d_TR = nullptr;
    double *d_phi[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    double *d_partial = nullptr;        // the TDGL's item partials, then the residual passes'
    size_t part_cap = 0;                // items of each half
    unsigned int *d_counter = nullptr;  // [4 + n_films] (Dev::counter)
    SolveDev *d_solve = nullptr;
    Ctl *d_ctl = nullptr;
    void *d_P[2][6] = {};
    void *d_r = nullptr, *d_q = nullptr, *d_dinv = nullptr, *d_x = nullptr, *d_p[2] = {};
    // schedule buffers, [n_films][stride], grown on demand
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
    bool host_direct = false;           // state uploads read the host arrays from kernels
    bool has_state = false;             // some film's state has been set (the autotuner's trial steps)
    void *h_stage = nullptr;            // pinned buffer of state downloads (first use)
    cudaStream_t stream = nullptr;
    // FP32_REFINED inner solver: the persistent cooperative kernel, or the
    // masked two-kernel PCG (Neumann films, or CMSL_PCG_TWO_KERNEL=1)
    // FP32_REFINED stencil passes (stencil32.cuh): the residual pass for
    // one-eps films (all films) or the general one, and their ring sizes
    void *refine_fn = nullptr, *tdgl_fn = nullptr;
    size_t refine_smem = 0, tdgl_smem = 0;
    int refine_nt = 0, tdgl_nt = 0;     // threads per block
    bool spectral = false;      // FP32 inner solve by the direct spectral solve (one film, uniform eps)
    SpecDev spec{};
    int spec_grid[5] = {0, 0, 0, 0, 0};   // blocks of the x, y, z passes, the column-pair pass, the cluster passes
    int spec_zt = 0;            // threads per block of the z solve
    size_t spec_smem[5] = {0, 0, 0, 0, 0};
    bool spec_col = false;      // column layout: x, fused y-z-y, x (three launches per solve)
    bool spec_cl = false;       // column layout by cluster transforms: xy, z, yx (three launches per solve)
    bool persistent = false;
    // staging of the FP32 stencil passes: STG_CP the cp.async ring (any
    // film), STG_TMA tensor copies (every film's nx % 32 == 0, ny % 8 == 0).
    // The TDGL and the residual passes each take the staging the autotuner
    // measured faster (STG_TMA until tuned)
    // The cp.async ring has a kernel per tile height (TILE_YS: 4, 8, 16 rows
    // of 32 columns); the tensor copies run 8-row tiles only.
    bool tma = false;
    int stg_tdgl = 0, stg_refine = 0;
    bool staging_fixed = false;         // CMSL_STAGING set the staging: the autotuner keeps it
    bool tile_fixed = false;            // CMSL_TILE_Y set the tile height: the autotuner keeps it
    void *tdgl_cp[3] = {nullptr, nullptr, nullptr}, *refine_cp[3] = {nullptr, nullptr, nullptr};
    size_t tdgl_cp_smem[3] = {0, 0, 0}, refine_cp_smem[3] = {0, 0, 0};
    void *tdgl_tma = nullptr, *refine_tma = nullptr;
    size_t tdgl_tma_smem = 0, refine_tma_smem = 0;
    // deferred checks: a step of films with defer_ok ends on its direct
    // solve and the next TDGL step (the cp.async ring kernels below; a
    // tensor-copy variant at three blocks per SM measured 20 % slower) forms
    // the check the update pass formed (CMSL_DEFER=0: the update pass)
    bool defer = false;
    void *tdgl_def[3] = {nullptr, nullptr, nullptr};
    size_t tdgl_def_smem[3] = {0, 0, 0};
    static int ty_index(int ty) { return ty == 4 ? 0 : ty == 16 ? 2 : 1; }
    // Stagings for the current tile height (tensor copies only with TY rows).
    void stage(int tdgl_stg, int refine_stg)
    {
        const bool t_ok = tma && stile_ty == TY;
        stg_tdgl = t_ok ? tdgl_stg : 0;
        stg_refine = t_ok ? refine_stg : 0;
        const int yi = ty_index(stile_ty);
        if (defer) stg_tdgl = 0;
        tdgl_fn = defer ? tdgl_def[yi] : stg_tdgl ? tdgl_tma : tdgl_cp[yi];
        tdgl_smem = defer ? tdgl_def_smem[yi] : stg_tdgl ? tdgl_tma_smem : tdgl_cp_smem[yi];
        refine_fn = stg_refine ? refine_tma : refine_cp[yi];
        refine_smem = stg_refine ? refine_tma_smem : refine_cp_smem[yi];
        tdgl_nt = refine_nt = TX * stile_ty;
        graph_valid = false;
    }
    FilmMaps *d_maps = nullptr;
    int *d_err = nullptr;               // device error word
    CgBuf cg{};
    int cg_grid = 0;
    void *cg_fn = nullptr;
    size_t cg_smem = 0;

    // element stride of one P field in its set: FP32 fields are halves of float2 pairs
    int pstride() const { return precision == CMSL_FP64 ? 1 : 2; }

    ~Engine()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void *p : allocs) cudaFree(p);
        if (h_stage) cudaFreeHost(h_stage);
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
        d.films = d_films; d.items = d_items; d.n_films = n_films; d.n_items = (int)items.size();
        d.sitems = d_sitems; d.n_sitems = (int)sitems.size();
        d.code = d_code; d.ncells = ncells;
        for (int q = 0; q < 5; ++q) d.phi[q] = d_phi[q];
        d.partial = d_partial; d.counter = d_counter; d.solve = d_solve; d.ctl = d_ctl;
        d.rpartial = d_partial + (size_t)NPART * part_cap;
        // the residual pass's block 0 hides the row total only where the
        // pass has more blocks than one wave (152 SMs, 32 / TY' resident
        // blocks each); otherwise the total stays at the TDGL step's end
        d.row_off = defer && n_films == 1 && (long long)sitems.size() > 152LL * 32 / stile_ty ? 1 : 0;
        d.wave = d_wave; d.rows = d_rows; d.rowbuf = d_rowbuf;
        d.iters_log = d_iters; d.refine_log = d_refine;
        d.wstride = wstride; d.rstride = rstride;
        d.use_cond = use_cond; d.h_inner = hi; d.h_outer = ho;
        d.arrive = cg.arrive;
        d.maps = d_maps;
        d.err = d_err;
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


// Shared pieces of the engine.
cmsl_status ensure_schedule(Engine *e, int n_steps, int n_rows);
cmsl_status add_kernel(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *dep, int ndep, void *fn,
                       int grid, int block, void **args, size_t smem = 0);
cmsl_status add_while(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *dep, int ndep,
                      cudaGraphConditionalHandle h, cudaGraph_t *body);
cmsl_status build_graph(Engine *e);

}  // namespace cmsl_eng

struct cmsl_film : cmsl_eng::Engine {};
struct cmsl_batch : cmsl_eng::Engine {};
