// Definitions of the reference globals that refcompat.cu reads, with the
// reference's names and types (HZO_Code_github/include/globals.h,
// cuda_deps.h, types.h).  Stands in for the reference's global.cu where the
// reference sources are absent.
#include <cstdio>

typedef struct MaterialNorm {
    double alpha_nd, beta_nd, gamma_nd, g_nd, a0_nd;
    double p0, f0, t0, E0;
    double L_nd, kappa_nd;
    double eps_r;
} MaterialNorm;

MaterialNorm N_FE, N_AFE, N_DE;
int nx = 0, ny = 0, nz = 0, ng_total = 0, count = 0, peloop = 0, time_to_change = 0, dep_flag = 0;
int do_pre_relax = 0, zbc_flag = 0, sim_index = 1;
double del_h = 0, del_t = 0, Ez_ext = 0, Ez_prev = 0, incEz = 0, maxEz = 0, delEz = 0, E0_ref = 1, P0_ref = 1;
double eps_0_nd = 0, sim_time = 0;
char crystal_type[20] = {0};
char output_dir[4000] = "output";
int *omega = nullptr, *grain_mat = nullptr;
double *TR_h = nullptr;
double *Pmx_old_d = nullptr, *Pmy_old_d = nullptr, *Pmz_old_d = nullptr, *Pmx_d = nullptr, *Pmy_d = nullptr,
       *Pmz_d = nullptr;
double *Psx_old_d = nullptr, *Psy_old_d = nullptr, *Psz_old_d = nullptr, *Psx_d = nullptr, *Psy_d = nullptr,
       *Psz_d = nullptr;
double *delecX_d = nullptr, *delecY_d = nullptr, *delecZ_d = nullptr;
double *phi_dep_d = nullptr;
bool phi_dep_initialized = false;
double *Pmx = nullptr, *Pmy = nullptr, *Pmz = nullptr, *Psx = nullptr, *Psy = nullptr, *Psz = nullptr;
