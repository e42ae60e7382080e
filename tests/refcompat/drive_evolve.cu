// Test driver: sets the reference globals from a setup file, calls the
// reference entry points (provided by libcmsl_gb's refcompat object) and
// writes the result.  Modes (argv[4]):
//   evolve (default)  Evolve(); writes the final P, count and peloop
//   pre               the same with do_pre_relax = 1 (the slice files land in
//                     the working directory)
//   depol             Depol_field() twice on the device arrays: P as the new
//                     state, then 0.9 P, the second call warm-started from
//                     the first's phi_dep_d; writes phi and E of both calls
// Setup file layout (native endianness):
//   int32  nx ny nz ng dep_flag zbc num_steps
//   double del_h del_t eps_0_nd maxEz delEz E0_ref P0_ref
//   double mats[3][8] (AFE, FE, DE: alpha beta gamma g a0 kappa L eps_r)
//   int32  omega[N], grain_mat[ng]; double TR[9 ng], P[6][N]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>

typedef struct MaterialNorm {
    double alpha_nd, beta_nd, gamma_nd, g_nd, a0_nd;
    double p0, f0, t0, E0;
    double L_nd, kappa_nd;
    double eps_r;
} MaterialNorm;
extern MaterialNorm N_FE, N_AFE, N_DE;
extern int nx, ny, nz, ng_total, count, peloop, time_to_change, dep_flag, do_pre_relax, zbc_flag, sim_index;
extern double del_h, del_t, Ez_ext, maxEz, delEz, E0_ref, P0_ref, eps_0_nd;
extern char crystal_type[20];
extern char output_dir[4000];
extern int *omega, *grain_mat;
extern double *TR_h;
extern double *Pmx_old_d, *Pmy_old_d, *Pmz_old_d, *Pmx_d, *Pmy_d, *Pmz_d;
extern double *Psx_old_d, *Psy_old_d, *Psz_old_d, *Psx_d, *Psy_d, *Psz_d;
extern double *delecX_d, *delecY_d, *delecZ_d;
extern double *phi_dep_d;
extern bool phi_dep_initialized;
void Evolve(void);
void Depol_field(void);
void evolve_resources_cleanup(void);

int main(int argc, char **argv)
{
    if (argc < 4) { std::fprintf(stderr, "usage: drive_evolve setup.bin out_dir result.bin [evolve|pre|depol]\n"); return 2; }
    const char *mode = argc > 4 ? argv[4] : "evolve";
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int iv[7];
    double dv[7], m[24];
    if (std::fread(iv, sizeof iv, 1, f) != 1 || std::fread(dv, sizeof dv, 1, f) != 1 || std::fread(m, sizeof m, 1, f) != 1) return 2;
    nx = iv[0]; ny = iv[1]; nz = iv[2]; ng_total = iv[3]; dep_flag = iv[4]; zbc_flag = iv[5]; time_to_change = iv[6];
    del_h = dv[0]; del_t = dv[1]; eps_0_nd = dv[2]; maxEz = dv[3]; delEz = dv[4]; E0_ref = dv[5]; P0_ref = dv[6];
    MaterialNorm *mn[3] = {&N_AFE, &N_FE, &N_DE};
    for (int q = 0; q < 3; ++q) {
        const double *r = m + 8 * q;
        mn[q]->alpha_nd = r[0]; mn[q]->beta_nd = r[1]; mn[q]->gamma_nd = r[2]; mn[q]->g_nd = r[3];
        mn[q]->a0_nd = r[4]; mn[q]->kappa_nd = r[5]; mn[q]->L_nd = r[6]; mn[q]->eps_r = r[7];
    }
    const size_t N = (size_t)nx * ny * nz;
    omega = (int *)std::malloc(N * sizeof(int));
    grain_mat = (int *)std::malloc(ng_total * sizeof(int));
    TR_h = (double *)std::malloc(9 * ng_total * sizeof(double));
    std::vector<double> P(6 * N);
    if (std::fread(omega, sizeof(int), N, f) != N || std::fread(grain_mat, sizeof(int), ng_total, f) != (size_t)ng_total ||
        std::fread(TR_h, sizeof(double), 9 * ng_total, f) != (size_t)(9 * ng_total) ||
        std::fread(P.data(), sizeof(double), 6 * N, f) != 6 * N)
        return 2;
    std::fclose(f);
    std::strcpy(crystal_type, "poly");
    std::snprintf(output_dir, sizeof output_dir, "%s", argv[2]);
    sim_index = 1;
    double **olds[6] = {&Pmx_old_d, &Pmy_old_d, &Pmz_old_d, &Psx_old_d, &Psy_old_d, &Psz_old_d};
    double **news[6] = {&Pmx_d, &Pmy_d, &Pmz_d, &Psx_d, &Psy_d, &Psz_d};
    for (int q = 0; q < 6; ++q) {
        cudaMalloc(olds[q], N * sizeof(double));
        cudaMalloc(news[q], N * sizeof(double));
        cudaMemcpy(*olds[q], P.data() + q * N, N * sizeof(double), cudaMemcpyHostToDevice);
    }
    double **E[3] = {&delecX_d, &delecY_d, &delecZ_d};
    for (auto e : E) { cudaMalloc(e, N * sizeof(double)); cudaMemset(*e, 0, N * sizeof(double)); }
    if (std::strcmp(mode, "depol") == 0) {
        // the new Pm is what Depol_field reads
        for (int q = 0; q < 6; ++q)
            cudaMemcpy(*news[q], P.data() + q * N, N * sizeof(double), cudaMemcpyHostToDevice);
        f = std::fopen(argv[3], "wb");
        std::vector<double> v(N);
        for (int call = 0; call < 2; ++call) {
            if (call == 1)
                for (int q = 0; q < 3; ++q) {
                    for (size_t i = 0; i < N; ++i) v[i] = 0.9 * P[q * N + i];
                    cudaMemcpy(*news[q], v.data(), N * sizeof(double), cudaMemcpyHostToDevice);
                }
            Depol_field();
            double *out[4] = {phi_dep_d, delecX_d, delecY_d, delecZ_d};
            for (double *o : out) {
                cudaMemcpy(v.data(), o, N * sizeof(double), cudaMemcpyDeviceToHost);
                std::fwrite(v.data(), sizeof(double), N, f);
            }
        }
        std::fclose(f);
        evolve_resources_cleanup();
        return cudaGetLastError() == cudaSuccess ? 0 : 3;
    }
    if (std::strcmp(mode, "pre") == 0) do_pre_relax = 1;
    Evolve();
    for (int q = 0; q < 6; ++q) cudaMemcpy(P.data() + q * N, *olds[q], N * sizeof(double), cudaMemcpyDeviceToHost);
    f = std::fopen(argv[3], "wb");
    std::fwrite(P.data(), sizeof(double), 6 * N, f);
    std::fwrite(&count, sizeof(int), 1, f);
    std::fwrite(&peloop, sizeof(int), 1, f);
    std::fclose(f);
    return 0;
}
