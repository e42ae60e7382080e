/*
 * cmsl_oracle.h -- CPU FP64 restatement of the HZO TDGL + Jacobi-PCG hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library is checked
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  The product library never links or calls it.
 *
 * Every function restates one piece of the reference (jhb6617-arch/cmsl,
 * HZO_Code_github/) and cites the file:line it follows.  Arithmetic is
 * written in the reference's operation order and the file is compiled with
 * -ffp-contract=off, so the TDGL step, divergence, operator, diagonal and
 * E-field restatements are bit-identical to the reference kernels compiled
 * for the host (pinned by tests/test_oracle_pin.py against oracle/_ref).
 * Dot products use a fixed-chunk order (deterministic for any thread count);
 * the reference's cuBLAS Ddot order is unknown, so PCG results agree with it
 * to rounding, not bitwise.
 */
#ifndef CMSL_ORACLE_H
#define CMSL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_AFE = 0, ORC_FE = 1, ORC_DE = 2 };
enum { ORC_DIRICHLET = 0, ORC_NEUMANN = 1 };
/* PCG stop tests: the reference's (sqrt(r.z) vs tol_abs and vs tol_rel*sqrt(r0.z0))
 * or a true relative residual ||r||_2 <= tol_rel * ||b||_2. */
enum { ORC_CRIT_REF = 0, ORC_CRIT_RELRES = 1 };

/* Non-dimensional per-material parameters (types.h:22-28 MaterialNorm subset). */
typedef struct {
    double alpha, beta, gamma, g, a0, kappa, L, eps_r;
} orc_mat;

typedef struct {
    int nx, ny, nz;
    double del_h, del_t;
    int dep_flag;
    int zbc;                 /* ORC_DIRICHLET / ORC_NEUMANN */
    double eps_0_nd;
    double g_bot, g_top;     /* electrode potentials (0 in the reference) */
    int ng;                  /* number of grains */
    const int32_t *omega;    /* [N] grain id per cell, C order i + nx*(j + ny*k) */
    const int32_t *grain_mat;/* [ng] material per grain */
    const double *TR;        /* [9*ng] row-major rotation lab->crystal per grain */
    const int32_t *is_interface; /* [N] 0/1 */
    orc_mat mats[3];         /* indexed by material id */
    /* PCG controls */
    int crit;
    double tol_abs, tol_rel;
    int max_iter;
} orc_film;

typedef struct {
    int iters;
    int status;    /* 0 ok, 1 breakdown (p.Ap <= 0 or non-finite), 2 bad initial residual */
    double rz0, rz;
    double rr, bb; /* final ||r||^2 and ||b||^2 */
} orc_pcg_info;

/* ---- kernels ---------------------------------------------------------- */

/* One explicit TDGL step: kernels_evol.cu:47-231 (kernelCalc_antiferro).
 * P_old/P_new: 6 arrays each, order Pmx,Pmy,Pmz,Psx,Psy,Psz.
 * E: 3 arrays (delecX/Y/Z) or NULL when dep_flag == 0.
 * local_out: 6 arrays (Pmx_l,Pmy_l,Pmz_l,Psx_l,Psy_l,Psz_l) or NULL.
 * Cells whose grain id is out of range are left untouched (kernels_evol.cu:68). */
void orc_tdgl_step(const orc_film *f, const double *const P_old[6], double *const P_new[6],
                   double Ez_ext, const double *const E[3], double *const local_out[6]);

/* eps_0_nd * div(Pm), central differences, x/y periodic, z clamped
 * (depol_varEPS.cu:279-329). */
void orc_divergence(const orc_film *f, const double *Pmx, const double *Pmy,
                    const double *Pmz, double *divP);

/* y = A x, the variable-eps 7-point operator (depol_varEPS.cu:10-15, 37-124). */
void orc_apply_A(const orc_film *f, const double *x, double *y);

/* Jacobi diagonal inverse (depol_varEPS.cu:126-180). */
void orc_diag_inv(const orc_film *f, double *dinv);

/* E = -grad(phi) (depol_varEPS.cu:223-276). */
void orc_efield(const orc_film *f, const double *phi, double *Ex, double *Ey, double *Ez);

/* Per-cell eps_r (InitConfKernel eps_m, init_conf.cu:105). */
void orc_eps_field(const orc_film *f, double *eps);

/* The depolarisation solve of one step: Depol_field (depol_varEPS.cu:332-595).
 * phi is the warm start on entry and the solution on exit.  E (3 arrays) is
 * written from the solution.  divP (may be NULL) receives eps_0_nd*div(Pm). */
void orc_depol_field(const orc_film *f, const double *Pmx, const double *Pmy,
                     const double *Pmz, double *phi, double *const E[3],
                     double *divP, orc_pcg_info *info);

/* PCG for A x = b with Jacobi preconditioning (depol_varEPS.cu:426-523).
 * x: warm start in, solution out. */
void orc_pcg(const orc_film *f, const double *b, double *x, orc_pcg_info *info);

/* The 11 averages of one sweep row (evolve.cu:256-357, kernels_evol.cu:23-44):
 * out[0..10] = <Pm_z>, <Ps_z>, <Pm_z^loc>, <Ps_z^loc>, <Pm_z>_FE, f_FE,
 * <Pm_z>_AFE, f_AFE, <Pm_z>_DE, f_DE, N  (unscaled, non-dimensional). */
void orc_sweep_stats(const orc_film *f, const double *Pmz, const double *Psz,
                     const double *Pmz_loc, const double *Psz_loc, double out[11]);

/* ---- driver ----------------------------------------------------------- */

/* Runs n_steps TDGL steps (plus the depolarisation solve when dep_flag) on the
 * state P (6 arrays, updated in place), E (3 arrays, in/out), phi (in/out).
 * Ez[s] is the applied field of step s; row[s] >= 0 asks for the sweep stats
 * of step s to be written to stats[row[s]*11 ..].  pcg_iters[s] (may be NULL)
 * receives the PCG iteration count.  Mirrors the step body of Evolve
 * (evolve.cu:217-241).  Returns 0, or the first PCG status that was not 0. */
int orc_run(const orc_film *f, double *const P[6], double *const E[3], double *phi,
            int n_steps, const double *Ez, const int *row, double *stats, int *pcg_iters);

/* ---- set-up ----------------------------------------------------------- */

/* main.cu:200-213 */
double orc_compute_p0(double alpha, double beta, double g, double gamma1, int transition_type);

typedef struct { double alpha, beta, gamma1, g, a0; int transition_type; double L, kappa, eps_r; } orc_raw;
typedef struct { double alpha_ref, P0_ref, L_ref, kappa_ref; } orc_refs;

/* main.cu:215-230 */
orc_refs orc_make_phase_refs(orc_raw raw);
/* main.cu:232-256; t0 and l0 are global.cu:30-31 (3e-9 s, 1e-9 m). */
orc_mat orc_make_nd(orc_raw raw, orc_refs ref, double t0, double l0);

/* Grain -> material assignment by voxel-fraction targets (init_conf.cu:108-260).
 * Uses the C library's srand(123456)/rand() exactly as the reference does.
 * Returns 0, or -1 (grain outside every layer), -2 (layer with no voxels). */
int orc_assign_materials(int nx, int ny, int nz, int ng, const int32_t *omega,
                         const double *centz, int n_layers, const int *layer_counts,
                         const double *afe, const double *fe, const double *de,
                         int32_t *grain_mat);

/* build_interface_flag (main.cu:13-42) */
void orc_interface_flags(int nx, int ny, int nz, const int32_t *omega,
                         const int32_t *grain_mat, int32_t *flag);

/* Bunge ZXZ rotation per grain (grain_io.cu:103-126). */
void orc_tr_from_euler(int ng, const double *phi, const double *theta, const double *psi,
                       double *TR);

#ifdef __cplusplus
}
#endif
#endif
