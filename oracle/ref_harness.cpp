/*
 * ref_harness.cpp -- host launch harness around the reference's own kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
 * with the reference sources (HZO_Code_github/src/kernels_evol.cu,
 * global.cu, get_InputParams.cu, grain_io.cu whole; depol_varEPS.cu:5-329,
 * main.cu:13-42 and :200-256, init_conf.cu:108-279 extracted at build time)
 * into oracle/_ref/libcmsl_ref.so.  Nothing of the reference is committed.
 *
 * Each ref_* entry point emulates a CUDA launch: blocks run in parallel
 * (OpenMP), threads of a block run in sequence, and the built-in index
 * variables are thread-local globals.  None of the reference kernels used
 * here synchronises within a block, so sequential threads are exact.
 */
#include <omp.h>
#include "header.h"
#include "kernels_evol.h"
#include "io_utils.h"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

/* prototypes of the extracted reference kernels (depol_varEPS.cu, main.cu) */
void apply_A(double *y, const double *x, const double *eps_r, int nx, int ny, int nz,
             double h, double g_bot, double g_top);
void build_diag_inv(double *dinv, const double *eps_r, int nx, int ny, int nz, double h);
void applyJacobiPreconditioner(int N, const double *r, const double *dinv, double *z);
void rhs_zero_on_planes(double *b, int nx, int ny, int nz);
void init_phi_linear(double *phi, int nx, int ny, int nz, double g_bot, double g_top);
void Calc_EfieldMag(double *Ex, double *Ey, double *Ez, const double *phi, double del_h,
                    int nx, int ny, int nz, double g_bot, double g_top, int count, double *divP_d);
void divergence(double *divP_d, double *Pmx_d, double *Pmy_d, double *Pmz_d, double del_h,
                int nx, int ny, int nz, int count, double eps_0_nd);
void build_interface_flag(const int *omega, const int *grain_mat, int *is_interface,
                          int nx, int ny, int nz);

template <class F>
static void launch(dim3 grid, dim3 block, F body)
{
    const long long nb = (long long)grid.x * grid.y * grid.z;
    #pragma omp parallel for schedule(dynamic, 4)
    for (long long b = 0; b < nb; ++b) {
        blockIdx.x = (unsigned)(b % grid.x);
        blockIdx.y = (unsigned)((b / grid.x) % grid.y);
        blockIdx.z = (unsigned)(b / ((long long)grid.x * grid.y));
        blockDim = block;
        gridDim = grid;
        for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = tz;
                    body();
                }
    }
}

static dim3 grid3(int nx, int ny, int nz, dim3 b)
{
    return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y, (nz + b.z - 1) / b.z);
}

static const dim3 kBlock(8, 4, 4);   /* InputParams dimx/dimy/dimz of the shipped decks */

extern "C" {

void ref_tdgl_step(int nx_, int ny_, int nz_, int ng, double *const Po[6], double *const Pn[6],
                   int *omega, const double *TR, const double *const prm[7], double h,
                   double dt, double *const E[3], int dep, double Ez, double *const loc[6],
                   const int *is_interface)
{
    const dim3 g = grid3(nx_, ny_, nz_, kBlock);
    launch(g, kBlock, [&]() {
        kernelCalc_antiferro(Pn[0], Po[0], Pn[3], Po[3], Pn[1], Po[1], Pn[4], Po[4],
                             Pn[2], Po[2], Pn[5], Po[5], omega, TR, prm[0], prm[1], prm[2],
                             prm[3], prm[4], prm[5], prm[6], h, dt, E[0], E[1], E[2], dep,
                             nx_, ny_, nz_, ng, 0, Ez, g_top, g_bot, loc[0], loc[3], loc[1],
                             loc[4], loc[2], loc[5], is_interface);
    });
}

void ref_divergence(int nx_, int ny_, int nz_, double *Pmx, double *Pmy, double *Pmz,
                    double h, double eps0nd, double *out)
{
    launch(grid3(nx_, ny_, nz_, kBlock), kBlock,
           [&]() { divergence(out, Pmx, Pmy, Pmz, h, nx_, ny_, nz_, 0, eps0nd); });
}

static void set_bc(int nx_, int ny_, int nz_, int zbc)
{
    d_zbc_type = zbc;
    d_ref_id = nx_ / 2 + nx_ * (ny_ / 2 + (nz_ / 2) * ny_);
}

void ref_apply_A(int nx_, int ny_, int nz_, int zbc, const double *x, const double *eps,
                 double h, double *y)
{
    set_bc(nx_, ny_, nz_, zbc);
    launch(grid3(nx_, ny_, nz_, kBlock), kBlock,
           [&]() { apply_A(y, x, eps, nx_, ny_, nz_, h, g_bot, g_top); });
}

void ref_diag_inv(int nx_, int ny_, int nz_, int zbc, const double *eps, double h, double *dinv)
{
    set_bc(nx_, ny_, nz_, zbc);
    launch(grid3(nx_, ny_, nz_, kBlock), kBlock,
           [&]() { build_diag_inv(dinv, eps, nx_, ny_, nz_, h); });
}

void ref_efield(int nx_, int ny_, int nz_, int zbc, const double *phi_, double h,
                double *Ex, double *Ey, double *Ez)
{
    set_bc(nx_, ny_, nz_, zbc);
    launch(grid3(nx_, ny_, nz_, kBlock), kBlock,
           [&]() { Calc_EfieldMag(Ex, Ey, Ez, phi_, h, nx_, ny_, nz_, g_bot, g_top, 0, nullptr); });
}

void ref_interface_flag(int nx_, int ny_, int nz_, const int *omega_, const int *gmat, int *out)
{
    const int N = nx_ * ny_ * nz_;
    launch(dim3((N + 255) / 256), dim3(256),
           [&]() { build_interface_flag(omega_, gmat, out, nx_, ny_, nz_); });
}

void ref_mat_mask(const double *Pmz, const int *omega_, const int *gmat, double *pm,
                  double *mask, int N, int target)
{
    launch(dim3((N + 255) / 256), dim3(256),
           [&]() { build_mat_mask_and_p(Pmz, omega_, gmat, pm, mask, N, target); });
}

double ref_compute_p0(double a, double b, double g, double c, int tt)
{
    return compute_p0(a, b, g, c, tt);
}

/* raw[9] = alpha, beta, gamma1, g, a0, transition_type, L, kappa, eps_r (types.h:15-20)
 * of the material and of the reference phase; out[8] = alpha, beta, gamma, g, a0,
 * kappa, L, eps_r non-dimensional; refs[2] = alpha_ref, P0_ref. */
void ref_make_nd(const double *raw, const double *ref_raw, double *out, double *refs)
{
    MaterialParamsRaw r{}, rr{};
    r.alpha = raw[0]; r.beta = raw[1]; r.gamma1 = raw[2]; r.g = raw[3]; r.a0 = raw[4];
    r.transition_type = (int)raw[5]; r.L = raw[6]; r.kappa = raw[7]; r.eps_r = raw[8];
    rr.alpha = ref_raw[0]; rr.beta = ref_raw[1]; rr.gamma1 = ref_raw[2]; rr.g = ref_raw[3];
    rr.a0 = ref_raw[4]; rr.transition_type = (int)ref_raw[5]; rr.L = ref_raw[6];
    rr.kappa = ref_raw[7]; rr.eps_r = ref_raw[8];
    PhaseRefs R = make_phase_refs(rr);
    MaterialNorm N = make_nd_wrt_reference(r, R);
    out[0] = N.alpha_nd; out[1] = N.beta_nd; out[2] = N.gamma_nd; out[3] = N.g_nd;
    out[4] = N.a0_nd; out[5] = N.kappa_nd; out[6] = N.L_nd; out[7] = N.eps_r;
    refs[0] = R.alpha_ref; refs[1] = R.P0_ref;
}

/* processInputParams (get_InputParams.cu:8-151).  ints[10] = nx, ny, nz, dep_flag,
 * num_steps, dimx, dimy, dimz, n_layers, do_pre_relax; dbl[12] = del_h, del_t, delEap,
 * Eap, kappa_fe, L_fe, kappa_afe, L_afe, kappa_de, L_de, eps_fe, eps_afe (eps_de in
 * dbl[12]); strs: crystal_type (20 chars) then z_bc_type (20 chars). */
void ref_read_deck(const char *path, const char *out_path, int *ints, double *dbl,
                   char *strs, int *layer_counts)
{
    processInputParams(path, out_path);
    ints[0] = nx; ints[1] = ny; ints[2] = nz; ints[3] = dep_flag; ints[4] = num_steps;
    ints[5] = dimx; ints[6] = dimy; ints[7] = dimz; ints[8] = h_n_layers; ints[9] = do_pre_relax;
    dbl[0] = del_h; dbl[1] = del_t; dbl[2] = delEap; dbl[3] = Eap;
    dbl[4] = FE_raw.kappa; dbl[5] = FE_raw.L; dbl[6] = AFE_raw.kappa; dbl[7] = AFE_raw.L;
    dbl[8] = DE_raw.kappa; dbl[9] = DE_raw.L; dbl[10] = FE_raw.eps_r; dbl[11] = AFE_raw.eps_r;
    dbl[12] = DE_raw.eps_r;
    std::memcpy(strs, crystal_type, 20);
    std::memcpy(strs + 20, z_bc_type, 20);
    for (int i = 0; i < h_n_layers && i < 16; ++i) layer_counts[i] = h_layer_counts[i];
}

/* LoadGrainStructureFromDir (grain_io.cu:26-135) with the grain count given. */
void ref_load_grain(const char *dir, const char *tag, int nx_, int ny_, int nz_, int ng,
                    int *omega_out, double *eta_out, double *TR_out, double *cent_out,
                    double *euler_out)
{
    nx = nx_; ny = ny_; nz = nz_; ng_total = ng;
    const size_t N = (size_t)nx_ * ny_ * nz_;
    omega = (int *)std::malloc(N * sizeof(int));       omega_d = (int *)std::malloc(N * sizeof(int));
    eta = (double *)std::malloc(N * sizeof(double));   eta_d = (double *)std::malloc(N * sizeof(double));
    centx = (double *)std::malloc(ng * sizeof(double)); centy = (double *)std::malloc(ng * sizeof(double));
    centz = (double *)std::malloc(ng * sizeof(double));
    phi = (double *)std::malloc(ng * sizeof(double));  theta = (double *)std::malloc(ng * sizeof(double));
    psi = (double *)std::malloc(ng * sizeof(double));
    phi_d = (double *)std::malloc(ng * sizeof(double)); theta_d = (double *)std::malloc(ng * sizeof(double));
    psi_d = (double *)std::malloc(ng * sizeof(double));
    TR_h = (double *)std::malloc(9 * ng * sizeof(double)); TR_d = (double *)std::malloc(9 * ng * sizeof(double));
    LoadGrainStructureFromDir(dir, tag);
    std::memcpy(omega_out, omega, N * sizeof(int));
    std::memcpy(eta_out, eta, N * sizeof(double));
    std::memcpy(TR_out, TR_h, 9 * ng * sizeof(double));
    for (int g = 0; g < ng; ++g) {
        cent_out[3 * g] = centx[g]; cent_out[3 * g + 1] = centy[g]; cent_out[3 * g + 2] = centz[g];
        euler_out[3 * g] = phi[g]; euler_out[3 * g + 1] = theta[g]; euler_out[3 * g + 2] = psi[g];
    }
    std::free(omega); std::free(omega_d); std::free(eta); std::free(eta_d);
    std::free(centx); std::free(centy); std::free(centz);
    std::free(phi); std::free(theta); std::free(psi);
    std::free(phi_d); std::free(theta_d); std::free(psi_d); std::free(TR_h); std::free(TR_d);
}

/* Grain -> material assignment: the host part of Init_Conf (init_conf.cu:108-279). */
void ref_assign_materials(int nx_, int ny_, int nz_, int ng, const int *omega_in,
                          const double *centz_in, int n_layers, const int *counts,
                          const double *afe, const double *fe, const double *de, int *out)
{
    nx = nx_; ny = ny_; nz = nz_; ng_total = ng; h_n_layers = n_layers;
    for (int L = 0; L < n_layers; ++L) {
        h_layer_counts[L] = counts[L];
        afe_frac_layer[L] = afe[L]; fe_frac_layer[L] = fe[L]; de_frac_layer[L] = de[L];
    }
    const size_t N = (size_t)nx_ * ny_ * nz_;
    omega = (int *)std::malloc(N * sizeof(int));
    std::memcpy(omega, omega_in, N * sizeof(int));
    centz = (double *)std::malloc(ng * sizeof(double));
    std::memcpy(centz, centz_in, ng * sizeof(double));
    grain_mat = (int *)std::malloc(ng * sizeof(int));
    Init_Conf();
    std::memcpy(out, grain_mat, ng * sizeof(int));
    std::free(omega); std::free(centz); std::free(grain_mat);
    omega = nullptr; centz = nullptr; grain_mat = nullptr;
}

/* One Depol_field call (depol_varEPS.cu:332-550): the reference kernels in the
 * reference launch order; the cuBLAS level-1 calls are plain loops. */
void ref_depol_field(int nx_, int ny_, int nz_, int zbc, const double *eps, double *Pmx,
                     double *Pmy, double *Pmz, double h, double eps0nd, double *phi_io,
                     double *Ex, double *Ey, double *Ez, double tola, double tolr,
                     int maxit, int *iters_out)
{
    set_bc(nx_, ny_, nz_, zbc);
    const int N = nx_ * ny_ * nz_;
    double *b = (double *)std::calloc(N, sizeof(double));
    double *x = (double *)std::calloc(N, sizeof(double));
    double *r = (double *)std::calloc(N, sizeof(double));
    double *z = (double *)std::calloc(N, sizeof(double));
    double *p = (double *)std::calloc(N, sizeof(double));
    double *Ap = (double *)std::calloc(N, sizeof(double));
    double *dinv = (double *)std::calloc(N, sizeof(double));
    const dim3 g = grid3(nx_, ny_, nz_, kBlock);
    launch(g, kBlock, [&]() { divergence(b, Pmx, Pmy, Pmz, h, nx_, ny_, nz_, 0, eps0nd); });
    for (int t = 0; t < N; ++t) b[t] = -1.0 * b[t];
    if (zbc == NEUMANN) b[d_ref_id] = 0.0;
    if (zbc == DIRICHLET) {
        const dim3 b2(16, 16, 1), g2((nx_ + 15) / 16, (ny_ + 15) / 16, 1);
        launch(g2, b2, [&]() { rhs_zero_on_planes(b, nx_, ny_, nz_); });
    }
    std::memcpy(x, phi_io, N * sizeof(double));
    launch(g, kBlock, [&]() { build_diag_inv(dinv, eps, nx_, ny_, nz_, h); });
    launch(g, kBlock, [&]() { apply_A(Ap, x, eps, nx_, ny_, nz_, h, g_bot, g_top); });
    for (int t = 0; t < N; ++t) r[t] = b[t] + (-1.0) * Ap[t];
    const dim3 b1(256), g1((N + 255) / 256);
    launch(g1, b1, [&]() { applyJacobiPreconditioner(N, r, dinv, z); });
    std::memcpy(p, z, N * sizeof(double));
    double rz = 0.0;
    for (int t = 0; t < N; ++t) rz += r[t] * z[t];
    const double rz0 = rz;
    int k = 0;
    if (std::isfinite(rz) && rz >= 0.0) {
        while (k < maxit && rz > tola * tola && (rz0 <= 0.0 || (rz / rz0) > tolr * tolr)) {
            ++k;
            launch(g, kBlock, [&]() { apply_A(Ap, p, eps, nx_, ny_, nz_, h, g_bot, g_top); });
            double den = 0.0;
            for (int t = 0; t < N; ++t) den += p[t] * Ap[t];
            if (!std::isfinite(den) || !(den > 0.0)) break;
            const double al = rz / den;
            for (int t = 0; t < N; ++t) x[t] = x[t] + al * p[t];
            for (int t = 0; t < N; ++t) r[t] = r[t] + (-al) * Ap[t];
            launch(g1, b1, [&]() { applyJacobiPreconditioner(N, r, dinv, z); });
            double rzn = 0.0;
            for (int t = 0; t < N; ++t) rzn += r[t] * z[t];
            if (!std::isfinite(rzn) || rzn < 0.0) break;
            const double be = rzn / rz;
            for (int t = 0; t < N; ++t) p[t] = be * p[t];
            for (int t = 0; t < N; ++t) p[t] = p[t] + 1.0 * z[t];
            rz = rzn;
        }
    }
    std::memcpy(phi_io, x, N * sizeof(double));
    launch(g, kBlock, [&]() { Calc_EfieldMag(Ex, Ey, Ez, x, h, nx_, ny_, nz_, g_bot, g_top, 0, b); });
    *iters_out = k;
    std::free(b); std::free(x); std::free(r); std::free(z); std::free(p); std::free(Ap); std::free(dinv);
}

// generate.cu: the reference's checkpoint and field writers/readers (host
// copies through the shim's cudaMemcpy).
void ref_write_checkpoint(const char *fname, double *const P[6], double *const E[3], int nx_, int ny_, int nz_,
                          double Ez_ext_, int peloop_, int count_, double incEz_)
{
    write_checkpoint(fname, P[0], P[1], P[2], P[3], P[4], P[5], E[0], E[1], E[2], nx_, ny_, nz_, Ez_ext_, peloop_,
                     count_, incEz_);
}

void ref_read_checkpoint(const char *fname, double *const P[6], double *const E[3], int nx_, int ny_, int nz_,
                         int *peloop_, int *count_, double *Ez_ext_, double *incEz_)
{
    read_checkpoint(fname, P[0], P[1], P[2], P[3], P[4], P[5], E[0], E[1], E[2], nx_, ny_, nz_, peloop_, count_,
                    Ez_ext_, incEz_);
}

void ref_write_vector_field(const char *fname, double *Px, double *Py, double *Pz, int nx_, int ny_, int nz_,
                            double p0)
{
    write_vector_field_binary(fname, Px, Py, Pz, nx_, ny_, nz_, p0);
}

void ref_write_midplane_slice(const char *fname, const double *v, int nx_, int ny_, int nz_)
{
    write_midplane_slice(fname, v, nx_, ny_, nz_);
}

}  // extern "C"
