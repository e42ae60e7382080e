// Test driver: sets the reference globals from a setup file, calls the
// reference entry point Evolve() (provided by libcmsl_gb's refcompat object),
// and writes the final P.  Setup file layout (native endianness):
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
void Evolve(void);

int main(int argc, char **argv)
{
    if (argc < 4) { std::fprintf(stderr, "usage: drive_evolve setup.bin out_dir final_P.bin\n"); return 2; }
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
    Evolve();
    for (int q = 0; q < 6; ++q) cudaMemcpy(P.data() + q * N, *olds[q], N * sizeof(double), cudaMemcpyDeviceToHost);
    f = std::fopen(argv[3], "wb");
    std::fwrite(P.data(), sizeof(double), 6 * N, f);
    std::fwrite(&count, sizeof(int), 1, f);
    std::fwrite(&peloop, sizeof(int), 1, f);
    std::fclose(f);
    return 0;
}
