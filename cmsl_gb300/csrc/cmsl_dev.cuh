// cmsl_dev.cuh -- device-side data layout shared by the kernels and the engine.
//
// Layout in HBM (one "batch" = one or more films, concatenated):
//   * every per-cell array holds all films back to back; film f's cells start
//     at FilmDev::off (a multiple of 32 cells: 128-byte aligned FP32 rows for
//     the vectorised passes) and are in the reference's C order
//     i + nx*(j + ny*k);
//   * P fields: two ping-pong sets, each one allocation: CMSL_FP64 -- six
//     SoA double arrays (Pmx..Psz), field q at q * ncells; CMSL_FP32_REFINED
//     -- three float2 arrays of the pairs (Pmx, Pmy), (Pmz, Psx), (Psy, Psz),
//     pair j at j * ncells float2 (a stencil point of a pair is one 8-byte
//     load or one 8-byte tensor-copy element);
//   * code[c]: grain id (bits 0-23, film-local) | material (bits 24-25) |
//     interface flag (bit 26) -- replaces the reference's seven per-voxel FP64
//     parameter arrays, omega and is_interface (kernels_evol.cu:133-146);
//   * phi: FP64 potentials (two buffers), or five double-float buffers in
//     FP32_REFINED mode ((hi, lo) float2 per cell) for the extrapolated warm
//     start; PCG vectors r, p[2], q, dinv, x in T;
//   * per-grain rotations TR (9 per grain, row major) in T.
// Work is cut into items (film, x0, y0, z0..z1): one thread block per item,
// a TX x TY thread tile marching through z0..z1.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cmsl {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;
constexpr int SX = TX + 2;
constexpr int SY = TY + 2;
constexpr int SPL = SX * SY;        // smem cells of one staged plane

// Tiles of the FP32 stencil passes (TDGL and residual passes, cp.async ring):
// TX x TYc columns, one thread per column; the tile autotuner picks TYc among
// TILE_YS (the tensor-copy staging and every other item kernel use TY).
template <int TYc> struct TileShape {
    static constexpr int SYt = TYc + 2;
    static constexpr int SPLt = SX * SYt;   // smem cells of one staged plane
    static constexpr int NTt = TX * TYc;    // threads per block
    static constexpr int MINB = 1024 / NTt; // resident blocks per SM the kernels are built for
};
constexpr int TILE_YS[3] = {4, 8, 16};
constexpr int NPART = 8;            // doubles of partial sums per item

constexpr uint32_t GID_MASK = 0x00ffffffu;
__host__ __device__ inline int code_gid(uint32_t c) { return (int)(c & GID_MASK); }
__host__ __device__ inline int code_mat(uint32_t c) { return (int)((c >> 24) & 3u); }
__host__ __device__ inline int code_iface(uint32_t c) { return (int)((c >> 26) & 1u); }
constexpr uint32_t CODE_INVALID = 0x80000000u;   // grain id out of range: cell frozen

// Per (material, interface) TDGL coefficients, computed on the host in the
// reference's operation order (kernels_evol.cu:139-153, :212, :223).
template <class T> struct Coef {
    T relax;   // 1 - 6 A
    T A;       // kappa dt / h^2
    T LdT;     // Lfac * dt
    T ag, ags; // 2 (alpha +- g_loc)
    T b4, b12, g6, a02;
};

struct FilmDev {
    int nx, ny, nz, zbc;
    long long off;              // first cell of the film
    int g_off;                  // first grain of the film in TR
    int item_begin, item_end;
    int sitem_begin, sitem_end; // the film's range of the FP32 stencil passes' items (Dev::sitems)
    int pb_begin, pb_end;       // persistent PCG: the film's block range of the cooperative grid
    int brick_begin, brick_end; // persistent PCG: the film's stencil bricks
    int dep_flag;
    int warm;                   // FP32_REFINED warm start: 0 previous phi, 1 linear, 2 quadratic, 3 cubic extrapolation
    int ref_id;                 // Neumann pinned cell (film-local)
    int crit;
    int max_iter, max_refine, inner_max;
    double h, dt, eps0nd, inv_N, two_h, h2, inv_h2, inv_2h;
    double tol_abs2, tol_rel2, refine_tol2, inner_tol2;
    float inv_h2f, inv_2hf, eps0f;
    float dinv_uni;             // Jacobi D^-1 of non-identity rows when every material has one eps
    int uni_eps;                // all materials share eps_r
    float cheb_delta;           // direct solve preconditioning several eps: (kappa - 1) / (kappa + 1),
                                // the half-width of M^-1 A's spectrum around 1 (0: exact solve)
    int upd_ok;                 // FP32_REFINED: the inner solve leaves r intact (direct solve), so a
                                // later refinement pass may update r instead of recomputing it
    int defer_ok;               // the check after a step's one direct solve may run inside the next
                                // TDGL step (upd_ok, warm start at most quadratic)
    double n_mat[3];            // voxels per material (sum of the reference's masks)
    Coef<double> coef[6];       // index mat*2 + iface
    Coef<float> coef32[6];
    double epsf[9];             // harmonic face eps for (mat_c, mat_nb), depol_varEPS.cu:10-15
    float epsf32[9];
    float cf_h[9], cf_l[9];     // epsf / h^2 as double-float pairs (FP32_REFINED residual)
    float cb_h, cb_l;           // eps_0_nd / (2 h) as a double-float pair
};

struct SolveDev {               // per film, lives in device memory
    double rz, rz0, pq, alpha, beta, rr, bb, rr64;
    int iters;                  // PCG iterations of the current (inner) solve
    int active;                 // inner PCG still running
    int status;                 // 0 ok, 1 breakdown, 2 bad initial residual, 3 refine cap
    int outer_active;           // FP32_REFINED: refinement still running
    int refine;                 // refinement passes this step
    int total_iters;            // PCG iterations this step
    int phi_cur;                // which phi buffer is current
    int phi_prev;               // previous step's potential (extrapolated warm start)
    int phi_prev2;              // the one before (quadratic extrapolation)
    int phi_prev3;              // and the one before that (cubic extrapolation)
    int hist;                   // FP32_REFINED: valid potentials among phi_cur, phi_prev, ... (0: phi_cur is
                                // the zero start of a state without a potential; at most 4); the warm
                                // start extrapolates to order min(warm, hist - 1)
    int sticky;                 // first non-zero status seen since set_state
    double inner_tol2;          // inner target of the current refinement pass
    int inner_max;              // inner iteration cap of the current pass
    int upd;                    // the next refinement pass updates r <- r - A dx (FP32) instead of
                                // forming b - A phi in double-float
    double cheb_rho;            // Chebyshev recurrence of the preconditioned refinement (rho_k)
    float cheb_w, cheb_m;       // the next direct solve's increment: dx <- w M^-1 r + m dx
    int row_pend;               // Dev::row_off: the sweep row (+1; 0 none) whose item partials the
                                // TDGL step left for the next residual pass to total and write
    int pending;                // the step ended on its direct solve: the potential is phi_cur (the
                                // warm start) + dx, its check r <- r - A dx still to come (next TDGL)
};

// Extra vectors of the single-reduction FP32 PCG (FP32_REFINED mode).
struct CgBuf {
    float *r[2], *w[2], *s[2];  // ping-pong by iteration parity
    float *x, *p;
    unsigned int *arrive;       // grid-barrier arrival counter (reset by k_refine32)
    float4 *part;               // [2][grid] per-block partial sums (two double-float pairs), by parity
    int *err;                   // barrier timeout flag
    unsigned long long spin_limit;   // sleeps of a barrier wait before it gives up
    int hold_block;             // failure injection: this block never arrives at a barrier (-1: none)
    const int4 *bricks;         // stencil work list: TX x TY x (<= PZ planes) bricks, film by film
    const int *blk_film;        // film of each block of the cooperative grid
    int n_bricks;
};

struct Ctl {
    int step;                   // steps done since set_state
    int cur;                    // which P set is "old"
    int run_step;               // step index within the current run (waveform index)
    int stop;                   // run_step at which the step loop of a graph launch ends
    int redo;                   // a TDGL step found a pending check failed and reopened the step before
};

template <class T> struct Fields {
    T *P[2][6];
    T *r, *q, *dinv, *x;
    T *p[2];
    const T *TR;
};

// Tensor maps of one film for the tensor-copy (TMA) staging of the FP32
// stencil passes (films with nx % 32 == 0 and ny % 8 == 0).  Each tensor has
// maps of three box shapes: the tile body {TX, TY}, one x row {TX, 1} (the
// y halo rows) and a column strip {16 bytes, TY} (the x halo columns).
enum { TM_BODY = 0, TM_ROW = 1, TM_COL = 2 };
struct FilmMaps {            // CUtensorMap carries its own alignment
    CUtensorMap P[2][3];        // P set s: 4D {nx, ny, nz, 3} of float2 pairs
    CUtensorMap phi[5][3];      // potential buffer b: 3D {nx, ny, nz} of (hi, lo) float2
    CUtensorMap code[3];        // 3D uint32
    CUtensorMap x[3];           // the inner solve's correction dx: 3D float
    CUtensorMap r;              // 3D float (body)
    CUtensorMap dinv;           // 3D float (body)
};

struct Dev {
    const FilmDev *films;
    const int4 *items;
    int n_films, n_items;
    const int4 *sitems;         // items of the FP32 stencil passes (tile height of the autotuner's choice)
    int n_sitems;
    int row_off;                // single films with deferred checks: block 0 of the step's first
                                // residual pass totals and writes the TDGL step's sweep row
                                // (SolveDev::row_pend) while the other blocks run their items.
                                // (Kept in the padding after n_sitems: a Dev above 256 bytes
                                // measured 1-2 us more per graph step.)
    const uint32_t *code;
    long long ncells;           // cells of all films (stride of the FP32 P pairs)
    double *phi[5];
    double *partial;            // [n_items * NPART]
    double *rpartial;           // [n_items * NPART] the FP32 residual passes' partial sums (apart from
                                // the TDGL's, which the step's first residual pass may still total)
    unsigned int *counter;      // [4 + n_films] the grid's ticket counter (reset by the last block);
                                // from 4 on the per-film ones of the FP32 stencil passes (batches)
    SolveDev *solve;            // [n_films]
    Ctl *ctl;
    const double *wave;         // [n_films * wstride] applied field per run step
    const int *rows;            // [n_films * wstride] output row per run step (-1 none)
    double *rowbuf;             // [n_films * rstride * 11]
    int *iters_log;             // [n_films * wstride]
    int *refine_log;            // [n_films * wstride]
    int wstride, rstride;
    int use_cond;
    int force;                  // run the PCG kernels whatever the flags (kernel timing)
    int step_end;               // a residual pass that leaves no film active also ends the step
    int defer;                  // films with defer_ok end a step on its direct solve (SolveDev::pending)
    unsigned int *arrive;       // grid-barrier counter of the persistent PCG (or null)
    cudaGraphConditionalHandle h_inner, h_outer;
    cudaGraphConditionalHandle h_steps;   // the graph's step loop (0: one step per launch)
    const FilmMaps *maps;       // [n_films] tensor maps (TMA stencil passes), or null
    int *err;                   // device error word (bounded waits that gave up)
};

}  // namespace cmsl
