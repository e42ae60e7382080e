/*
 * cmsl.h -- C ABI of libcmsl_gb, the GB300 (sm_103a) implementation of the
 * HZO phase-field hot path of jhb6617-arch/cmsl: the explicit TDGL step, the
 * Jacobi-PCG depolarisation solve and the P-E loop driver that sequences them.
 *
 * Conventions: plain C types only; host pointers unless a name says _dev;
 * every call returns cmsl_status and never exits the process (the reference
 * prints and calls exit(1), HZO_Code_github/include/check.h:9-83);
 * cmsl_last_error() gives the text of the last failure on the calling thread.
 * A film handle is not thread-safe; distinct handles are independent.
 *
 * Cell order is the reference's C order id = i + nx*(j + ny*k)
 * (HZO_Code_github/src/kernels_evol.cu:65).  Field arrays are the six
 * polarisation components Pmx, Pmy, Pmz, Psx, Psy, Psz (non-dimensional).
 */
#ifndef CMSL_H
#define CMSL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CMSL_OK = 0,
    CMSL_ERR_ARG = 1,      /* bad argument or size */
    CMSL_ERR_CUDA = 2,     /* CUDA runtime failure (no device, launch error) */
    CMSL_ERR_IO = 3,       /* file missing, short or malformed */
    CMSL_ERR_PCG = 4,      /* PCG breakdown or non-finite residual in some step */
    CMSL_ERR_STATE = 5,    /* call out of order */
    CMSL_ERR_NOMEM = 6
} cmsl_status;

typedef enum { CMSL_AFE = 0, CMSL_FE = 1, CMSL_DE = 2 } cmsl_material_id;
typedef enum { CMSL_DIRICHLET = 0, CMSL_NEUMANN = 1 } cmsl_zbc;

/* CMSL_FP64: FP64 storage and arithmetic, TDGL and operator bit-identical to
 *   the reference kernels; one PCG solve per step.
 * CMSL_FP32_REFINED: FP32 fields, stencils and PCG vectors; PCG dots summed in
 *   FP32 within a warp and FP64 above it; the potential is kept in
 *   double-float (two FP32 halves, ~48 significand bits) and an outer
 *   residual-refinement loop evaluated in double-float drives
 *   ||b - A phi|| / ||b|| below refine_tol. */
typedef enum { CMSL_FP64 = 0, CMSL_FP32_REFINED = 1 } cmsl_precision;

/* Stop test of the (inner) PCG.  CMSL_CRIT_REF is the reference's
 * (depol_varEPS.cu:472-474): continue while r.z > tol_abs^2 and
 * r.z/r0.z0 > tol_rel^2.  CMSL_CRIT_RELRES: continue while
 * ||r||_2 > tol_rel * ||b||_2. */
typedef enum { CMSL_CRIT_REF = 0, CMSL_CRIT_RELRES = 1 } cmsl_pcg_crit;

/* Non-dimensional material parameters, as make_nd_wrt_reference produces them
 * (HZO_Code_github/src/main.cu:232-256, include/types.h:22-28). */
typedef struct {
    double alpha, beta, gamma, g, a0, kappa, L, eps_r;
} cmsl_material;

typedef struct {
    int nx, ny, nz;
    double del_h, del_t;
    int dep_flag;                 /* 0: no depolarisation solve (E_dep = 0) */
    int zbc;                      /* cmsl_zbc for the potential */
    double eps_0_nd;              /* main.cu:343-344 */
    int n_grains;
    const int32_t *omega;         /* [N] grain id per cell, 0 <= id < n_grains */
    const int32_t *grain_mat;     /* [n_grains] cmsl_material_id */
    const double *TR;             /* [9*n_grains] lab->crystal rotation, row major */
    const int32_t *is_interface;  /* [N] 0/1, or NULL: built as main.cu:13-42 does */
    cmsl_material mats[3];        /* indexed by cmsl_material_id */
    int precision;                /* cmsl_precision */
    int pcg_crit;                 /* cmsl_pcg_crit (FP64 solve; FP32 inner solve uses RELRES-free rz test) */
    double tol_abs, tol_rel;      /* reference defaults 1e-3, 1e-2 (global.cu:140-144) */
    int max_iter;                 /* reference default 4000 */
    double refine_tol;            /* FP32_REFINED: outer ||r||/||b|| target, e.g. 1e-8 */
    int max_refine;               /* FP32_REFINED: outer passes per step (>= 2) */
    double inner_tol;             /* FP32_REFINED: inner sqrt(r.z/r0.z0) target, e.g. 1e-4 */
    int inner_max_iter;           /* FP32_REFINED: inner iterations per pass */
    int warm_start;               /* FP32_REFINED: 0 = previous phi (the reference's warm
                                     start, depol_varEPS.cu:429-430), 1 = linear
                                     extrapolation 2 phi_n - phi_{n-1}, 2 = quadratic
                                     3 phi_n - 3 phi_{n-1} + phi_{n-2}, 3 = cubic
                                     4 phi_n - 6 phi_{n-1} + 4 phi_{n-2} - phi_{n-3}
                                     (2 is the fastest with the direct inner solve: its
                                     first residual is small enough for the FP32 update
                                     pass, at two fewer potentials read per step) */
    int inner_solver;             /* FP32_REFINED inner solve: CMSL_INNER_AUTO (direct
                                     spectral solve where it applies, else PCG),
                                     CMSL_INNER_PCG, CMSL_INNER_DIRECT (CMSL_ERR_ARG where
                                     it does not apply) */
} cmsl_film_desc;

/* The direct inner solve applies to FP32_REFINED films (or batches) whose
 * depolarisation solves have the Dirichlet z boundary and nx, ny of the form
 * 2^a 3^b (<= 4096): an in-plane FFT, a tridiagonal solve along z per mode and
 * the inverse FFT.  With one permittivity for all materials it is exact for
 * the operator up to FP32 rounding.  With several it solves with one
 * reference permittivity (the middle of the range the film's grains use) and
 * preconditions the double-float refinement, whose residual applies the true
 * operator; the refinement's increments follow the Chebyshev semi-iteration
 * for the preconditioned spectrum [2 e_min, 2 e_max] / (e_min + e_max), so
 * each pass contracts the residual by about (sqrt(kappa) - 1) / (sqrt(kappa)
 * + 1), kappa = e_max / e_min, and such a film may take more refinement
 * passes than max_refine (enough for (kappa - 1) / (kappa + 1) per pass to
 * reach refine_tol from a zero potential).  CMSL_INNER_AUTO takes it for
 * kappa <= 16 and the PCG otherwise. */
typedef enum { CMSL_INNER_AUTO = 0, CMSL_INNER_PCG = 1, CMSL_INNER_DIRECT = 2 } cmsl_inner_solver;

typedef struct cmsl_film cmsl_film;

/* One sweep row: the 11 averages the reference writes per output step
 * (evolve.cu:256-357): <Pm_z>, <Ps_z>, <Pm_z^loc>, <Ps_z^loc>, <Pm_z>_FE, f_FE,
 * <Pm_z>_AFE, f_AFE, <Pm_z>_DE, f_DE, N_steps_done.  Non-dimensional. */
#define CMSL_ROW_WIDTH 11

const char *cmsl_last_error(void);
const char *cmsl_version(void);

/* Replaces the film set-up of SetupAndRunSimulation/AllocateData/Init_Conf
 * (main.cu:261-359, allocateVars.cu:4-112, init_conf.cu:68-106): uploads the
 * grain map, builds the per-cell code, the coefficient tables and the Jacobi
 * diagonal (depol_varEPS.cu:126-180, built once instead of every step), and
 * zeroes P, phi and the work vectors. */
cmsl_status cmsl_film_create(const cmsl_film_desc *desc, cmsl_film **out);
cmsl_status cmsl_film_destroy(cmsl_film *film);

/* Host <-> device state.  P: 6 arrays of N doubles; phi: N doubles or NULL
 * (leaves phi unchanged / not read).  set_state also resets the step counter. */
cmsl_status cmsl_film_set_state(cmsl_film *film, const double *const P[6], const double *phi);
cmsl_status cmsl_film_get_state(cmsl_film *film, double *const P[6], double *phi);

/* Page-locked host memory for state arrays (no reference counterpart: the
 * reference keeps its state in its own globals).  get_state converts on the
 * GPU straight into page-locked arrays (these, or memory the caller
 * registered with CUDA) instead of converting on the host cores, and a
 * caller that reuses its arrays across calls avoids first-touch page faults.
 * cmsl_host_free(NULL) is a no-op. */
cmsl_status cmsl_host_alloc(size_t bytes, void **out);
cmsl_status cmsl_host_free(void *p);

/* The P-E loop driver body (Evolve, evolve.cu:217-409): runs n_steps TDGL steps,
 * each followed by the depolarisation solve when dep_flag.  Ez[s] is the
 * applied non-dimensional field of step s (host array); row[s] >= 0 stores the
 * sweep averages of step s as row row[s] (host array or NULL).  The whole loop
 * is enqueued on `stream` (a cudaStream_t, NULL = legacy default) as CUDA
 * graphs with device-side PCG loops; the call returns after enqueueing.
 * cmsl_film_sync waits and reports a PCG failure seen by any step. */
cmsl_status cmsl_film_run(cmsl_film *film, int n_steps, const double *Ez, const int32_t *row,
                          void *stream);
cmsl_status cmsl_film_sync(cmsl_film *film);

/* Copies rows [first, first+n) (n*CMSL_ROW_WIDTH doubles) of the last run. */
cmsl_status cmsl_film_get_rows(cmsl_film *film, int first, int n, double *out);

/* Per-step solver counters of the last run: PCG iterations (summed over the
 * refinement passes) and refinement passes (1 in FP64 mode). */
cmsl_status cmsl_film_get_iters(cmsl_film *film, int n, int32_t *pcg_iters, int32_t *refine_passes);

/* Single pieces of the path on the film's current state, for parity tests:
 *  - tdgl_step: one TDGL step with applied field Ez (no solve), the E_dep of
 *    kernelCalc_antiferro computed from the current phi (Calc_EfieldMag);
 *  - depol: one Depol_field (RHS from the current Pm, warm-started PCG);
 *  - apply_operator: y = A x with the film's operator (apply_A), FP64 or FP32;
 *  - efield: E = -grad(phi) of the current phi (Calc_EfieldMag; FP32-refined
 *    films difference the double-float potential in FP64). */
cmsl_status cmsl_film_tdgl_step(cmsl_film *film, double Ez);
cmsl_status cmsl_film_depol(cmsl_film *film, int32_t *iters, int32_t *status);
cmsl_status cmsl_film_apply_operator(cmsl_film *film, const double *x, double *y);
cmsl_status cmsl_film_efield(cmsl_film *film, double *Ex, double *Ey, double *Ez);
cmsl_status cmsl_film_diag_inv(cmsl_film *film, double *dinv);

/* Depol_field (depol_varEPS.cu:332-595) over the caller's DEVICE arrays, as
 * the reference's global-state solve sees them: the new Pm (Pmx/Pmy/Pmz_d),
 * phi_dep_d (warm start in, solution out, in place) and delecX/Y/Z_d (E out;
 * pass NULLs to skip).  Everything is converted and copied by kernels on
 * `stream`; nothing goes through the host and nothing is allocated per call,
 * so a caller keeps one film for its grid and calls this once per step.  The
 * film's own P state is overwritten (its Pm with the given one).  Single
 * films with a depolarisation solve; iters[0] PCG iterations, iters[1]
 * refinement passes (FP32_REFINED). */
cmsl_status cmsl_film_depol_device(cmsl_film *film, const double *Pmx, const double *Pmy, const double *Pmz,
                                   double *phi, double *Ex, double *Ey, double *Ez, void *stream,
                                   int32_t *iters, int32_t *status);

/* Average device time (ms, CUDA events on the launch stream) of each kernel
 * of a step, each launched `reps` times back to back on the current state:
 * ms[0] TDGL step, ms[1] solve set-up (FP64 RHS + r0, or FP32_REFINED FP64
 * residual pass), ms[2] PCG p-update + SpMV + p.Ap, ms[3] PCG x/r update +
 * r.z.  The PCG kernels run with the solve forced active, so the call
 * changes the film's work vectors; run it after the steps being measured. */
cmsl_status cmsl_film_time_kernels(cmsl_film *film, int reps, void *stream, double *ms);

/* The FP32_REFINED inner solve the film uses: CMSL_INNER_DIRECT or
 * CMSL_INNER_PCG (CMSL_INNER_PCG for FP64 films, whose solve is the
 * reference's PCG). */
cmsl_status cmsl_film_inner_solver(cmsl_film *film, int *solver);

/* Tile-shape autotuner: times the stencil passes of this film for work-item z
 * chunks ceil(nz / n), n = 1, 2, ... down to 4 planes (a column's chunks
 * differ by one plane at most) on the device -- and, for CMSL_FP32_REFINED
 * films with full 32 x 8 tiles, both stagings of the TDGL and of the
 * residual passes (tensor copies or the cp.async ring) -- keeps the fastest
 * (the z chunk in *zchunk, may be NULL) and remembers it for films of the same
 * shape class created later in the process.  Leaves the state (P, phi) as it
 * is; results of later steps equal the untuned ones up to the order of the
 * row sums.  CMSL_ZCHUNK=<n> fixes the chunk of untuned handles,
 * CMSL_NO_TMA=1 the cp.async staging. */
cmsl_status cmsl_film_autotune(cmsl_film *film, int32_t *zchunk);

/* The stencil-pass configuration in use: cfg[0] tile x, cfg[1] tile y,
 * cfg[2] z chunk (0: the per-film heuristic), cfg[3] the stagings: bits 0-1
 * the TDGL's, bits 2-3 the residual passes' (0 the cp.async ring, 1 tensor
 * copies). */
cmsl_status cmsl_film_tile_config(cmsl_film *film, int32_t cfg[4]);

/* Bytes of device memory the film holds. */
cmsl_status cmsl_film_device_bytes(cmsl_film *film, size_t *bytes);

/* ---- Batches: many independent films advancing together.
 * The reference runs its simulations one after another, each with its own
 * allocation and P-E loop (the campaign loop main.cu:455-498 calling
 * SetupAndRunSimulation -> Evolve, main.cu:261-359 / evolve.cu:73-440).  A
 * batch holds films of any sizes, grain maps, materials and tolerances (one
 * precision for all) and advances them in lockstep: every step is one graph
 * whose kernels cover all films, with per-film PCG convergence masks -- a
 * film that has converged drops out of the PCG kernels while the others
 * iterate, and a PCG failure marks that film only.  Per-film results equal
 * those of the same film run alone through cmsl_film_* (same kernels, same
 * per-film reductions), except that the FP32_REFINED inner solve of a batch
 * is the two-kernel masked PCG instead of the single-film persistent one. */
typedef struct cmsl_batch cmsl_batch;

/* descs: n_films film descriptions (as cmsl_film_create; equal precision). */
cmsl_status cmsl_batch_create(const cmsl_film_desc *descs, int n_films, cmsl_batch **out);
cmsl_status cmsl_batch_destroy(cmsl_batch *batch);

/* State of film `film` (0-based), as cmsl_film_set_state/get_state.  Setting
 * one film restarts its solver state and leaves the other films and the
 * batch's step counter alone. */
cmsl_status cmsl_batch_set_state(cmsl_batch *batch, int film, const double *const P[6], const double *phi);
cmsl_status cmsl_batch_get_state(cmsl_batch *batch, int film, double *const P[6], double *phi);

/* n_steps steps of every film.  Ez: [n_films][n_steps] applied fields (film
 * major); row: [n_films][n_steps] output rows (-1 none) or NULL.  Returns once
 * the loop is enqueued and the host arrays have been consumed. */
cmsl_status cmsl_batch_run(cmsl_batch *batch, int n_steps, const double *Ez, const int32_t *row, void *stream);

/* Waits for the run.  film_status (n_films entries, or NULL) receives each
 * film's first PCG failure of the run (0 none, 1 breakdown, 2 invalid
 * initial residual); returns CMSL_ERR_PCG if any film failed. */
cmsl_status cmsl_batch_sync(cmsl_batch *batch, int32_t *film_status);

/* Rows and solver counters of one film, as cmsl_film_get_rows/get_iters. */
cmsl_status cmsl_batch_get_rows(cmsl_batch *batch, int film, int first, int n, double *out);
cmsl_status cmsl_batch_get_iters(cmsl_batch *batch, int film, int n, int32_t *pcg_iters, int32_t *refine_passes);

/* As cmsl_film_time_kernels over the whole batch (ms[2], ms[3] are the
 * masked PCG's SpMV and update kernels in FP32_REFINED mode). */
cmsl_status cmsl_batch_time_kernels(cmsl_batch *batch, int reps, void *stream, double *ms);
cmsl_status cmsl_batch_device_bytes(cmsl_batch *batch, size_t *bytes);
/* The batch's FP32_REFINED inner solve, as cmsl_film_inner_solver. */
cmsl_status cmsl_batch_inner_solver(cmsl_batch *batch, int *solver);

/* The batch's tile-shape autotuner, as cmsl_film_autotune (one z chunk for
 * all films of the batch). */
cmsl_status cmsl_batch_autotune(cmsl_batch *batch, int32_t *zchunk);
cmsl_status cmsl_batch_tile_config(cmsl_batch *batch, int32_t cfg[4]);

/* Restart files in the reference's checkpoint layout (generate.cu:90-264;
 * cmsl_io.h cmsl_checkpoint_write/read).  write: P and E = -grad(phi) of the
 * film's current state with the loop counters given.  read: sets P from the
 * file (its grid must match the film's), resets the step counter, and, with
 * dep_flag, solves for the potential of that P (the file's E is the field of
 * that same solve); returns the loop counters. */
cmsl_status cmsl_film_checkpoint_write(cmsl_film *film, const char *path, int peloop, int count, double Ez_ext,
                                       double incEz);
cmsl_status cmsl_film_checkpoint_read(cmsl_film *film, const char *path, int *peloop, int *count, double *Ez_ext,
                                      double *incEz);

/* Gradient of a P-E loop misfit by a hand-written adjoint of the TDGL step and
 * the depolarisation solve (no counterpart in the reference, which has no
 * derivatives; for fitting Landau coefficients to measured loops).  From the
 * film's current state it runs n_steps steps (Ez, row as cmsl_film_run; every
 * row index < n_rows) and
 *   loss = (1/n_rows) sum_r (<Pm_z>_r - target[r])^2,
 * <Pm_z>_r the first column of sweep row r; then the adjoint backwards in
 * time, recomputing each segment of checkpoint_every steps from a checkpoint
 * of P and phi taken by the forward pass (the last segment keeps the states
 * of the forward pass; checkpoint_every >= n_steps recomputes nothing).
 * grad[5*m + p] = d loss / d of the
 * non-dimensional parameter p in (alpha, beta, gamma, g, kappa) of material m
 * (cmsl_material_id), through every voxel of that material (interfaces
 * included).  FP64 films; with dep_flag, the Dirichlet z boundary.  The
 * forward solves are taken as exact: converge them tightly (e.g.
 * CMSL_CRIT_RELRES, tol_rel 1e-12) for a gradient that matches finite
 * differences.  Work memory (about 8 * N * (7 * segments + 6 *
 * checkpoint_every + 14) bytes) is allocated for the call.  Leaves the film
 * in an unspecified state: set it again before the next run. */
cmsl_status cmsl_film_loop_gradient(cmsl_film *film, int n_steps, const double *Ez, const int32_t *row,
                                    const double *target, int n_rows, int checkpoint_every, double *loss,
                                    double *grad);

/* Depolarisation solve that allocates nothing.  No counterpart in the
 * reference: it is for callers that cannot call cudaMalloc (an application
 * that owns all device memory through its own pool, a plugin handed fixed
 * buffers).  It runs the FP64 Jacobi-PCG of cmsl_film_depol -- the same
 * kernels and stop test -- with every work buffer in one fixed device array
 * of about 6.3 MB that stays resident on each GPU that loads the library.
 *   - grids up to 131072 cells (nx*ny*nz; nz >= 3) and up to 32767 cells
 *     along each side; other grids return CMSL_ERR_ARG and do nothing;
 *   - inputs and outputs are device pointers: material id per cell (0 AFE,
 *     1 FE, 2 DE), eps_r per material (host), the new Pm components, and phi
 *     (warm start in, solution out, in place);
 *   - the first call on a device looks up the array's device address with
 *     that device current; make it before any stream capture; the address
 *     is kept for the life of the process and does not survive
 *     cudaDeviceReset (no call may follow one);
 *   - all calls share the array: calls whose GPU work overlaps race, so
 *     serialise them; each call clears the state it reads;
 *   - returns after the solve (it reads the loop flags on `stream`). */
cmsl_status cmsl_depol_solve_noalloc(int nx, int ny, int nz, double del_h, int zbc, double eps_0_nd,
                                     const int32_t *material_dev, const double eps_r[3],
                                     const double *Pmx_dev, const double *Pmy_dev, const double *Pmz_dev,
                                     double *phi_dev, double tol_abs, double tol_rel, int max_iter,
                                     int pcg_crit, void *stream, int32_t *iters_out, int32_t *status_out);

#ifdef __cplusplus
}
#endif
#endif
