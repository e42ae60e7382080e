/*
 * cmsl_oracle.c -- CPU FP64 restatement of the HZO TDGL + Jacobi-PCG hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Loaded by tests/, the smoke check
 * and bench.py's CPU-baseline leg; never by the product library.
 *
 * Build: -O2 -fPIC -ffp-contract=off -fopenmp (see oracle/Makefile).  The
 * no-contraction flag keeps the arithmetic bit-identical to the reference's
 * kernels compiled for the host on both x86-64 and aarch64.
 */
#include "cmsl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_CHUNK 4096

static inline long long orc_id(const orc_film *f, int i, int j, int k)
{
    return (long long)i + (long long)f->nx * ((long long)j + (long long)k * f->ny);
}

/* Deterministic dot product: fixed chunks summed in chunk order. */
static double orc_dot(const double *a, const double *b, long long n)
{
    long long nch = (n + ORC_CHUNK - 1) / ORC_CHUNK;
    double *part = (double *)malloc((size_t)(nch > 0 ? nch : 1) * sizeof(double));
    #pragma omp parallel for schedule(static)
    for (long long c = 0; c < nch; ++c) {
        long long lo = c * ORC_CHUNK, hi = lo + ORC_CHUNK < n ? lo + ORC_CHUNK : n;
        double s = 0.0;
        for (long long t = lo; t < hi; ++t) s += a[t] * b[t];
        part[c] = s;
    }
    double s = 0.0;
    for (long long c = 0; c < nch; ++c) s += part[c];
    free(part);
    return s;
}

static double orc_sum(const double *a, long long n)
{
    long long nch = (n + ORC_CHUNK - 1) / ORC_CHUNK;
    double *part = (double *)malloc((size_t)(nch > 0 ? nch : 1) * sizeof(double));
    #pragma omp parallel for schedule(static)
    for (long long c = 0; c < nch; ++c) {
        long long lo = c * ORC_CHUNK, hi = lo + ORC_CHUNK < n ? lo + ORC_CHUNK : n;
        double s = 0.0;
        for (long long t = lo; t < hi; ++t) s += a[t];
        part[c] = s;
    }
    double s = 0.0;
    for (long long c = 0; c < nch; ++c) s += part[c];
    free(part);
    return s;
}

/* ------------------------------------------------------------------------
 * TDGL step -- kernels_evol.cu:47-231.  Operation order follows the
 * reference expression by expression (required for bit parity).
 * ---------------------------------------------------------------------- */
void orc_tdgl_step(const orc_film *f, const double *const Po[6], double *const Pn[6],
                   double Ez_ext, const double *const E[3], double *const loc[6])
{
    const int nx = f->nx, ny = f->ny, nz = f->nz;
    const double del_h = f->del_h, del_t = f->del_t;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
        const long long id = orc_id(f, i, j, k);
        const int gid = f->omega[id];
        if (gid < 0 || gid >= f->ng) continue;              /* kernels_evol.cu:68 */

        const int e = (i + 1) % nx, w = (i - 1 + nx) % nx;  /* :71-76 */
        const int n = (j + 1) % ny, s = (j - 1 + ny) % ny;
        const int u = (k == nz - 1) ? k : (k + 1);
        const int d = (k == 0) ? k : (k - 1);
        const long long nb[6] = { orc_id(f, e, j, k), orc_id(f, w, j, k), orc_id(f, i, n, k),
                                  orc_id(f, i, s, k), orc_id(f, i, j, u), orc_id(f, i, j, d) };

        double sum[6], c0[6];
        for (int q = 0; q < 6; ++q) {                          /* :87-122 */
            const double *a = Po[q];
            sum[q] = a[nb[0]] + a[nb[1]] + a[nb[2]] + a[nb[3]] + a[nb[4]] + a[nb[5]];
            c0[q] = a[id];                                     /* :125-130 */
        }

        const orc_mat *m = &f->mats[f->grain_mat[gid]];         /* per-voxel params :133-140 */
        const double alpha_nd = m->alpha, beta_nd = m->beta, gamma_nd = m->gamma;
        double g_loc = m->g;
        const double a0_nd = m->a0, kappa_nd = m->kappa;
        double Lfac = m->L;
        if (f->is_interface[id]) {                              /* :142-146 */
            g_loc *= 0.4;
            Lfac *= (1.0 + 10.0);
        }
        const double alpha_g_nd = 2.0 * (alpha_nd + g_loc);     /* :148-153 */
        const double alpha_g_nd_s = 2.0 * (alpha_nd - g_loc);
        const double beta_4 = 4.0 * beta_nd;
        const double beta_12 = 12.0 * beta_nd;
        const double gamma_6 = 6.0 * gamma_nd;
        const double a0_2 = 2.0 * a0_nd;

        const double *T = f->TR + 9 * (long long)gid;            /* :157-159 */
        const double pMx0 = c0[0], pMy0 = c0[1], pMz0 = c0[2];
        const double pSx0 = c0[3], pSy0 = c0[4], pSz0 = c0[5];
        const double pMXl = T[0] * pMx0 + T[1] * pMy0 + T[2] * pMz0; /* :162-168 */
        const double pMYl = T[3] * pMx0 + T[4] * pMy0 + T[5] * pMz0;
        const double pMZl = T[6] * pMx0 + T[7] * pMy0 + T[8] * pMz0;
        const double pSXl = T[0] * pSx0 + T[1] * pSy0 + T[2] * pSz0;
        const double pSYl = T[3] * pSx0 + T[4] * pSy0 + T[5] * pSz0;
        const double pSZl = T[6] * pSx0 + T[7] * pSy0 + T[8] * pSz0;
        if (loc) {                                              /* :170-175 */
            loc[0][id] = pMXl; loc[1][id] = pMYl; loc[2][id] = pMZl;
            loc[3][id] = pSXl; loc[4][id] = pSYl; loc[5][id] = pSZl;
        }

        const double dfdPmxl = a0_2 * pMXl, dfdPmyl = a0_2 * pMYl; /* :178-181 */
        const double dfdPsxl = a0_2 * pSXl, dfdPsyl = a0_2 * pSYl;
        const double m2 = pMZl * pMZl, m3 = m2 * pMZl, m4 = m3 * pMZl, m5 = m4 * pMZl;
        const double s2 = pSZl * pSZl, s3 = s2 * pSZl, s4 = s3 * pSZl, s5 = s4 * pSZl;
        const double dfdPmzl = alpha_g_nd * pMZl + beta_4 * m3 + beta_12 * pMZl * s2
                             + gamma_6 * (m5 + 10.0 * m3 * s2 + 5.0 * pMZl * s4); /* :193-195 */
        const double dfdPszl = alpha_g_nd_s * pSZl + beta_4 * s3 + beta_12 * pSZl * m2
                             + gamma_6 * (s5 + 10.0 * m2 * s3 + 5.0 * pSZl * m4); /* :197-199 */

        double bMx = T[0] * dfdPmxl + T[3] * dfdPmyl + T[6] * dfdPmzl;  /* :202-208 */
        double bMy = T[1] * dfdPmxl + T[4] * dfdPmyl + T[7] * dfdPmzl;
        double bMz = T[2] * dfdPmxl + T[5] * dfdPmyl + T[8] * dfdPmzl;
        const double bSx = T[0] * dfdPsxl + T[3] * dfdPsyl + T[6] * dfdPszl;
        const double bSy = T[1] * dfdPsxl + T[4] * dfdPsyl + T[7] * dfdPszl;
        const double bSz = T[2] * dfdPsxl + T[5] * dfdPsyl + T[8] * dfdPszl;

        const double dfdPmz_app = -Ez_ext;                      /* :210 */
        const double A_loc = kappa_nd * del_t / (del_h * del_h); /* :212 */
        const double ex = (f->dep_flag != 0) ? -1.0 * E[0][id] : 0.0; /* :214-216 */
        const double ey = (f->dep_flag != 0) ? -1.0 * E[1][id] : 0.0;
        const double ez = (f->dep_flag != 0) ? -1.0 * E[2][id] : 0.0;
        bMx += ex;                                              /* :218-220 */
        bMy += ey;
        bMz += dfdPmz_app + ez;

        const double relax = 1.0 - 6.0 * A_loc;                 /* :223-229 */
        Pn[0][id] = pMx0 * relax + A_loc * sum[0] - Lfac * del_t * bMx;
        Pn[1][id] = pMy0 * relax + A_loc * sum[1] - Lfac * del_t * bMy;
        Pn[2][id] = pMz0 * relax + A_loc * sum[2] - Lfac * del_t * bMz;
        Pn[3][id] = pSx0 * relax + A_loc * sum[3] - Lfac * del_t * bSx;
        Pn[4][id] = pSy0 * relax + A_loc * sum[4] - Lfac * del_t * bSy;
        Pn[5][id] = pSz0 * relax + A_loc * sum[5] - Lfac * del_t * bSz;
    }
}

/* depol_varEPS.cu:279-329 */
void orc_divergence(const orc_film *f, const double *Pmx, const double *Pmy,
                    const double *Pmz, double *divP)
{
    const int nx = f->nx, ny = f->ny, nz = f->nz;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
        const int e = (i + 1) % nx, w = (i - 1 + nx) % nx;
        const int n = (j + 1) % ny, s = (j - 1 + ny) % ny;
        const int u = (k == nz - 1) ? k : (k + 1);
        const int d = (k == 0) ? k : (k - 1);
        double v = ((Pmx[orc_id(f, e, j, k)] - Pmx[orc_id(f, w, j, k)]) +
                    (Pmy[orc_id(f, i, n, k)] - Pmy[orc_id(f, i, s, k)]) +
                    (Pmz[orc_id(f, i, j, u)] - Pmz[orc_id(f, i, j, d)])) / (2.0 * f->del_h);
        v *= f->eps_0_nd;
        divP[orc_id(f, i, j, k)] = v;
    }
}

/* depol_varEPS.cu:10-15 */
static inline double orc_harm(double a, double b)
{
    const double eps = 1e-20;
    double denom = a + b;
    if (denom < eps) denom = eps;
    return (2.0 * a * b) / denom;
}

static inline long long orc_ref_id(const orc_film *f)
{
    return orc_id(f, f->nx / 2, f->ny / 2, f->nz / 2);  /* depol_varEPS.cu:339-346 */
}

void orc_eps_field(const orc_film *f, double *eps)
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    for (long long t = 0; t < N; ++t) {
        const int g = f->omega[t];
        eps[t] = (g >= 0 && g < f->ng) ? f->mats[f->grain_mat[g]].eps_r : 0.0;
    }
}

/* z neighbours of the operator rows (depol_varEPS.cu:86-99). */
static inline void orc_zn(const orc_film *f, int k, int *up, int *dn)
{
    if (f->zbc == ORC_DIRICHLET) { *up = k + 1; *dn = k - 1; }
    else if (k == 0) { *up = 1; *dn = 1; }
    else if (k == f->nz - 1) { *up = f->nz - 2; *dn = f->nz - 2; }
    else { *up = k + 1; *dn = k - 1; }
}

/* depol_varEPS.cu:37-124 */
static void orc_apply_A_eps(const orc_film *f, const double *eps, const double *x, double *y)
{
    const int nx = f->nx, ny = f->ny, nz = f->nz;
    const double h = f->del_h;
    const long long ref = orc_ref_id(f);
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
        const long long id = orc_id(f, i, j, k);
        if (f->zbc == ORC_NEUMANN && id == ref) { y[id] = x[id]; continue; }
        if (f->zbc == ORC_DIRICHLET) {
            if (k == 0) { y[id] = x[id] - f->g_bot; continue; }
            if (k == nz - 1) { y[id] = x[id] - f->g_top; continue; }
        }
        const int ip = (i + 1) % nx, im = (i - 1 + nx) % nx;
        const int jp = (j + 1) % ny, jm = (j - 1 + ny) % ny;
        int up, dn;
        orc_zn(f, k, &up, &dn);
        const double ec = eps[id];
        const double ex_p = orc_harm(ec, eps[orc_id(f, ip, j, k)]);
        const double ex_m = orc_harm(ec, eps[orc_id(f, im, j, k)]);
        const double ey_p = orc_harm(ec, eps[orc_id(f, i, jp, k)]);
        const double ey_m = orc_harm(ec, eps[orc_id(f, i, jm, k)]);
        const double ez_p = orc_harm(ec, eps[orc_id(f, i, j, up)]);
        const double ez_m = orc_harm(ec, eps[orc_id(f, i, j, dn)]);
        const double xc = x[id];
        const double xe = x[orc_id(f, ip, j, k)], xw = x[orc_id(f, im, j, k)];
        const double xn = x[orc_id(f, i, jp, k)], xs = x[orc_id(f, i, jm, k)];
        const double xu = x[orc_id(f, i, j, up)], xd = x[orc_id(f, i, j, dn)];
        const double Ax = (ex_p * (xe - xc) - ex_m * (xc - xw)
                         + ey_p * (xn - xc) - ey_m * (xc - xs)
                         + ez_p * (xu - xc) - ez_m * (xc - xd)) / (h * h);
        y[id] = -Ax;
    }
}

void orc_apply_A(const orc_film *f, const double *x, double *y)
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    double *eps = (double *)malloc((size_t)N * sizeof(double));
    orc_eps_field(f, eps);
    orc_apply_A_eps(f, eps, x, y);
    free(eps);
}

/* depol_varEPS.cu:126-180 */
static void orc_diag_inv_eps(const orc_film *f, const double *eps, double *dinv)
{
    const int nx = f->nx, ny = f->ny, nz = f->nz;
    const double h = f->del_h;
    const long long ref = orc_ref_id(f);
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
        const long long id = orc_id(f, i, j, k);
        if (f->zbc == ORC_NEUMANN && id == ref) { dinv[id] = 1.0; continue; }
        if (f->zbc == ORC_DIRICHLET && (k == 0 || k == nz - 1)) { dinv[id] = 1.0; continue; }
        const int ip = (i + 1) % nx, im = (i - 1 + nx) % nx;
        const int jp = (j + 1) % ny, jm = (j - 1 + ny) % ny;
        int up, dn;
        orc_zn(f, k, &up, &dn);
        const double ec = eps[id];
        const double ex_p = orc_harm(ec, eps[orc_id(f, ip, j, k)]);
        const double ex_m = orc_harm(ec, eps[orc_id(f, im, j, k)]);
        const double ey_p = orc_harm(ec, eps[orc_id(f, i, jp, k)]);
        const double ey_m = orc_harm(ec, eps[orc_id(f, i, jm, k)]);
        const double ez_p = orc_harm(ec, eps[orc_id(f, i, j, up)]);
        const double ez_m = orc_harm(ec, eps[orc_id(f, i, j, dn)]);
        const double D = (ex_p + ex_m + ey_p + ey_m + ez_p + ez_m) / (h * h);
        dinv[id] = (D > 1e-30 ? 1.0 / D : 1.0);
    }
}

void orc_diag_inv(const orc_film *f, double *dinv)
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    double *eps = (double *)malloc((size_t)N * sizeof(double));
    orc_eps_field(f, eps);
    orc_diag_inv_eps(f, eps, dinv);
    free(eps);
}

/* depol_varEPS.cu:223-276 */
void orc_efield(const orc_film *f, const double *phi, double *Ex, double *Ey, double *Ez)
{
    const int nx = f->nx, ny = f->ny, nz = f->nz;
    const double del_h = f->del_h;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
        const long long id = orc_id(f, i, j, k);
        const int e = (i + 1) % nx, w = (i - 1 + nx) % nx;
        const int n = (j + 1) % ny, s = (j - 1 + ny) % ny;
        Ex[id] = -(phi[orc_id(f, e, j, k)] - phi[orc_id(f, w, j, k)]) / (2.0 * del_h);
        Ey[id] = -(phi[orc_id(f, i, n, k)] - phi[orc_id(f, i, s, k)]) / (2.0 * del_h);
        if (f->zbc == ORC_DIRICHLET) {
            const int up = (k == nz - 1 ? k : k + 1), dn = (k == 0 ? k : k - 1);
            const double phi_up = (k == nz - 1 ? f->g_top : phi[orc_id(f, i, j, up)]);
            const double phi_dn = (k == 0 ? f->g_bot : phi[orc_id(f, i, j, dn)]);
            Ez[id] = -(phi_up - phi_dn) / (2 * del_h);
        } else {
            int up, dn;
            orc_zn(f, k, &up, &dn);
            Ez[id] = -(phi[orc_id(f, i, j, up)] - phi[orc_id(f, i, j, dn)]) / (2 * del_h);
        }
    }
}

/* depol_varEPS.cu:426-523, with an optional true-relative-residual stop test. */
static void orc_pcg_eps(const orc_film *f, const double *eps, const double *b, double *x,
                        orc_pcg_info *info)
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    double *r = (double *)malloc((size_t)N * sizeof(double));
    double *z = (double *)malloc((size_t)N * sizeof(double));
    double *p = (double *)malloc((size_t)N * sizeof(double));
    double *Ap = (double *)malloc((size_t)N * sizeof(double));
    double *dinv = (double *)malloc((size_t)N * sizeof(double));

    orc_diag_inv_eps(f, eps, dinv);
    orc_apply_A_eps(f, eps, x, Ap);
    #pragma omp parallel for schedule(static)
    for (long long t = 0; t < N; ++t) {
        r[t] = b[t] - Ap[t];
        z[t] = r[t] * dinv[t];
        p[t] = z[t];
    }
    double rz = orc_dot(r, z, N);
    const double rz0 = rz;
    const double bb = orc_dot(b, b, N);
    double rr = orc_dot(r, r, N);
    int k = 0, status = 0;
    const double ta2 = f->tol_abs * f->tol_abs, tr2 = f->tol_rel * f->tol_rel;

    if (!isfinite(rz) || rz < 0.0) {
        status = 2;
    } else {
        for (;;) {
            int go;
            if (f->crit == ORC_CRIT_REF)
                go = k < f->max_iter && rz > ta2 && (rz0 <= 0.0 || (rz / rz0) > tr2);
            else
                go = k < f->max_iter && rr > tr2 * bb;
            if (!go) break;
            ++k;
            orc_apply_A_eps(f, eps, p, Ap);
            const double denom = orc_dot(p, Ap, N);
            if (!isfinite(denom) || !(denom > 0.0)) { status = 1; break; }
            const double alpha = rz / denom;
            const double nalpha = -alpha;
            #pragma omp parallel for schedule(static)
            for (long long t = 0; t < N; ++t) {
                x[t] = x[t] + alpha * p[t];
                r[t] = r[t] + nalpha * Ap[t];
                z[t] = r[t] * dinv[t];
            }
            const double rz_new = orc_dot(r, z, N);
            if (f->crit != ORC_CRIT_REF) rr = orc_dot(r, r, N);
            if (!isfinite(rz_new) || rz_new < 0.0) { status = 1; break; }
            const double beta = rz_new / rz;
            #pragma omp parallel for schedule(static)
            for (long long t = 0; t < N; ++t) p[t] = beta * p[t] + z[t];
            rz = rz_new;
        }
    }
    if (info) {
        info->iters = k; info->status = status; info->rz0 = rz0; info->rz = rz;
        info->rr = orc_dot(r, r, N); info->bb = bb;
    }
    free(r); free(z); free(p); free(Ap); free(dinv);
}

void orc_pcg(const orc_film *f, const double *b, double *x, orc_pcg_info *info)
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    double *eps = (double *)malloc((size_t)N * sizeof(double));
    orc_eps_field(f, eps);
    orc_pcg_eps(f, eps, b, x, info);
    free(eps);
}

/* depol_varEPS.cu:332-550 */
void orc_depol_field(const orc_film *f, const double *Pmx, const double *Pmy,
                     const double *Pmz, double *phi, double *const E[3], double *divP,
                     orc_pcg_info *info)
{
    const int nx = f->nx, ny = f->ny, nz = f->nz;
    const long long N = (long long)nx * ny * nz;
    double *b = (double *)malloc((size_t)N * sizeof(double));
    double *eps = (double *)malloc((size_t)N * sizeof(double));
    orc_eps_field(f, eps);
    orc_divergence(f, Pmx, Pmy, Pmz, b);                       /* :382-385 */
    if (divP) memcpy(divP, b, (size_t)N * sizeof(double));
    for (long long t = 0; t < N; ++t) b[t] = -1.0 * b[t];      /* :401-402 */
    if (f->zbc == ORC_NEUMANN) b[orc_ref_id(f)] = 0.0;        /* :405-414 */
    if (f->zbc == ORC_DIRICHLET) {                             /* :417-424 */
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                b[orc_id(f, i, j, 0)] = 0.0;
                b[orc_id(f, i, j, nz - 1)] = 0.0;
            }
    }
    orc_pcg_eps(f, eps, b, phi, info);                          /* :429-543 */
    orc_efield(f, phi, E[0], E[1], E[2]);                       /* :547-550 */
    free(b);
    free(eps);
}

/* evolve.cu:256-357 with build_mat_mask_and_p (kernels_evol.cu:23-44) */
void orc_sweep_stats(const orc_film *f, const double *Pmz, const double *Psz,
                     const double *Pmz_loc, const double *Psz_loc, double out[11])
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    const double one_by = 1.0 / ((double)f->nx * f->ny * f->nz);
    out[0] = orc_sum(Pmz, N) * one_by;
    out[1] = orc_sum(Psz, N) * one_by;
    out[2] = orc_sum(Pmz_loc, N) * one_by;
    out[3] = orc_sum(Psz_loc, N) * one_by;
    double *pm = (double *)malloc((size_t)N * sizeof(double));
    double *mk = (double *)malloc((size_t)N * sizeof(double));
    const int order[3] = { ORC_FE, ORC_AFE, ORC_DE };
    for (int q = 0; q < 3; ++q) {
        const int target = order[q];
        for (long long t = 0; t < N; ++t) {
            const int g = f->omega[t];
            double mm = 0.0;
            if (g >= 0 && f->grain_mat[g] == target) mm = 1.0;
            mk[t] = mm;
            pm[t] = mm * Pmz[t];
        }
        const double ps = orc_sum(pm, N), ms = orc_sum(mk, N);
        out[4 + 2 * q] = ms > 0.0 ? ps / ms : 0.0;
        out[5 + 2 * q] = ms > 0.0 ? ms / (double)N : 0.0;
    }
    free(pm);
    free(mk);
}

/* evolve.cu:217-241 (one step body) repeated n_steps times. */
int orc_run(const orc_film *f, double *const P[6], double *const E[3], double *phi,
            int n_steps, const double *Ez, const int *row, double *stats, int *pcg_iters)
{
    const long long N = (long long)f->nx * f->ny * f->nz;
    double *Pn[6], *loc[6];
    for (int q = 0; q < 6; ++q) {
        Pn[q] = (double *)malloc((size_t)N * sizeof(double));
        memcpy(Pn[q], P[q], (size_t)N * sizeof(double));
        loc[q] = (double *)calloc((size_t)N, sizeof(double));
    }
    int rc = 0;
    for (int s = 0; s < n_steps; ++s) {
        orc_tdgl_step(f, (const double *const *)P, Pn, Ez[s], (const double *const *)E, loc);
        for (int q = 0; q < 6; ++q) memcpy(P[q], Pn[q], (size_t)N * sizeof(double));
        if (f->dep_flag != 0) {
            orc_pcg_info info;
            orc_depol_field(f, P[0], P[1], P[2], phi, E, NULL, &info);
            if (pcg_iters) pcg_iters[s] = info.iters;
            if (info.status != 0 && rc == 0) rc = info.status;
        } else if (pcg_iters) {
            pcg_iters[s] = 0;
        }
        if (row && row[s] >= 0 && stats)
            orc_sweep_stats(f, P[2], P[5], loc[2], loc[5], stats + 11 * (long long)row[s]);
    }
    for (int q = 0; q < 6; ++q) { free(Pn[q]); free(loc[q]); }
    return rc;
}

/* ------------------------------------------------------------------------
 * Set-up restatements
 * ---------------------------------------------------------------------- */

/* main.cu:200-213 */
double orc_compute_p0(double alpha, double beta, double g, double gamma1, int transition_type)
{
    if (transition_type == 2) return 2.0 * sqrt((g - alpha) / beta);
    double disc = beta * beta - 4.0 * gamma1 * (alpha - g);
    if (disc < 0.0 && disc > -1e-14) disc = 0.0;
    if (disc < 0.0) return 1.0;
    const double Num = 2.0 * fabs(beta) + 2.0 * sqrt(disc);
    if (gamma1 == 0.0) return 1.0;
    return sqrt(Num / gamma1);
}

/* main.cu:215-230 */
orc_refs orc_make_phase_refs(orc_raw raw)
{
    orc_refs R;
    R.alpha_ref = fabs(raw.alpha);
    if (raw.beta == 0.0 && raw.gamma1 == 0.0 && raw.g == 0.0) {
        R.P0_ref = 1.0;
    } else {
        R.P0_ref = orc_compute_p0(raw.alpha, raw.beta, raw.g, raw.gamma1, raw.transition_type);
        if (!isfinite(R.P0_ref) || R.P0_ref <= 0.0) R.P0_ref = 1.0;
    }
    R.L_ref = raw.L;
    R.kappa_ref = raw.kappa;
    return R;
}

/* main.cu:232-256 */
orc_mat orc_make_nd(orc_raw raw, orc_refs ref, double t0, double l0)
{
    orc_mat N;
    memset(&N, 0, sizeof(N));
    N.alpha = raw.alpha / ref.alpha_ref;
    if (!(raw.beta == 0.0 && raw.gamma1 == 0.0 && raw.g == 0.0)) {
        N.beta = (raw.beta * ref.P0_ref * ref.P0_ref) / (8.0 * ref.alpha_ref);
        N.gamma = (raw.gamma1 * pow(ref.P0_ref, 4.0)) / (48.0 * ref.alpha_ref);
        N.g = raw.g / ref.alpha_ref;
    }
    N.a0 = (4.0 * raw.a0) / ref.alpha_ref;
    N.L = 0.25 * raw.L * ref.alpha_ref * t0;
    N.kappa = raw.kappa / (ref.alpha_ref * l0 * l0);
    N.eps_r = raw.eps_r;
    return N;
}

/* init_conf.cu:108-260 */
int orc_assign_materials(int nx, int ny, int nz, int ng, const int32_t *omega,
                         const double *centz, int n_layers, const int *layer_counts,
                         const double *afe, const double *fe, const double *de,
                         int32_t *grain_mat)
{
    int rc = 0;
    int *z_start = (int *)malloc((size_t)n_layers * sizeof(int));
    int *z_end = (int *)malloc((size_t)n_layers * sizeof(int));
    int *layer = (int *)malloc((size_t)(ng > 0 ? ng : 1) * sizeof(int));
    int *vox = (int *)calloc((size_t)(ng > 0 ? ng : 1), sizeof(int));
    int *lst = (int *)malloc((size_t)(ng > 0 ? ng : 1) * sizeof(int));
    z_start[0] = 0;
    z_end[0] = layer_counts[0];
    for (int L = 1; L < n_layers; L++) {
        z_start[L] = z_end[L - 1];
        z_end[L] = z_start[L] + layer_counts[L];
    }
    for (int g = 0; g < ng; g++) {
        const double zc = centz[g];
        int found = 0;
        for (int L = 0; L < n_layers; L++) {
            if (zc >= z_start[L] && zc < z_end[L]) { layer[g] = L; found = 1; break; }
        }
        if (!found) { rc = -1; goto done; }
    }
    for (long long id = 0; id < (long long)nx * ny * nz; id++) {
        const int g = omega[id];
        if (g >= 0 && g < ng) vox[g]++;
    }
    for (int g = 0; g < ng; g++) grain_mat[g] = -1;
    srand(123456);
    for (int L = 0; L < n_layers; L++) {
        double A = afe[L], F = fe[L], D = de[L];
        double sum = A + F + D;
        if (sum <= 0) { A = 0; F = 0; D = 1; sum = 1; }
        A /= sum; F /= sum; D /= sum;
        int cnt = 0;
        for (int g = 0; g < ng; g++)
            if (layer[g] == L) lst[cnt++] = g;
        long long tot = 0;
        for (int i = 0; i < cnt; i++) tot += vox[lst[i]];
        if (tot <= 0) { rc = -2; goto done; }
        const long long tA = llround(A * tot), tD = llround(D * tot);
        for (int i = 0; i < cnt; i++) {
            const int r = i + rand() % (cnt - i);
            const int tmp = lst[i]; lst[i] = lst[r]; lst[r] = tmp;
        }
        long long acc = 0;
        int p = 0;
        while (p < cnt && acc < tD) { const int g = lst[p++]; grain_mat[g] = ORC_DE; acc += vox[g]; }
        acc = 0;
        while (p < cnt && acc < tA) { const int g = lst[p++]; grain_mat[g] = ORC_AFE; acc += vox[g]; }
        while (p < cnt) { const int g = lst[p++]; if (grain_mat[g] == -1) grain_mat[g] = ORC_FE; }
    }
done:
    free(z_start); free(z_end); free(layer); free(vox); free(lst);
    return rc;
}

/* main.cu:13-42 */
void orc_interface_flags(int nx, int ny, int nz, const int32_t *omega,
                         const int32_t *grain_mat, int32_t *flag)
{
    const long long N = (long long)nx * ny * nz, plane = (long long)nx * ny;
    for (long long id = 0; id < N; ++id) {
        const int gid = omega[id];
        if (gid < 0 || grain_mat[gid] != ORC_FE) { flag[id] = 0; continue; }
        const long long k = id / plane;
        if (k == 0 || k == nz - 1) { flag[id] = 0; continue; }
        const int gu = omega[id + plane], gd = omega[id - plane];
        const int mu = gu >= 0 ? grain_mat[gu] : -1;
        const int md = gd >= 0 ? grain_mat[gd] : -1;
        flag[id] = (mu != ORC_FE || md != ORC_FE);
    }
}

/* grain_io.cu:103-126 */
void orc_tr_from_euler(int ng, const double *phi, const double *theta, const double *psi,
                       double *TR)
{
    for (int kp = 0; kp < ng; ++kp) {
        const double sph = sin(phi[kp]), cph = cos(phi[kp]);
        const double sth = sin(theta[kp]), cth = cos(theta[kp]);
        const double sps = sin(psi[kp]), cps = cos(psi[kp]);
        const double cth_sph = cth * sph, cth_cph = cth * cph;
        const double sth_sph = sth * sph, sth_cph = sth * cph;
        double *T = TR + 9 * (long long)kp;
        T[0] = cph * cps - cth_sph * sps;
        T[1] = sph * cps + cth_cph * sps;
        T[2] = sth * sps;
        T[3] = -cph * sps - cth_sph * cps;
        T[4] = -sph * sps + cth_cph * cps;
        T[5] = sth * cps;
        T[6] = sth_sph;
        T[7] = -sth_cph;
        T[8] = cth;
    }
}
