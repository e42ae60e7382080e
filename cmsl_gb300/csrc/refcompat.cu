// refcompat.cu -- the reference's driver entry points over its own globals.
//
// Linked together with the reference's main.cu, init_conf.cu, grain_io.cu,
// get_InputParams.cu, global.cu, allocateVars.cu, cleanup.cu and generate.cu,
// this file replaces evolve.cu, kernels_evol.cu and depol_varEPS.cu: it
// defines Evolve(), Depol_field(), evolve_resources_init() and
// evolve_resources_cleanup() (HZO_Code_github/include/header.h:25-32) with
// the same effect on the same globals, and runs them on libcmsl_gb.
//
// The globals are declared here with the reference's names and types
// (include/globals.h, include/cuda_deps.h, include/types.h); the definitions
// come from the reference's global.cu.  The precision is FP64 (bit-identical
// TDGL) unless CMSL_PRECISION=fp32 selects FP32_REFINED.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "cmsl.h"
#include "cmsl_io.h"

// ---- the reference's types and globals (layouts must match include/types.h)
typedef struct MaterialNorm {
    double alpha_nd, beta_nd, gamma_nd, g_nd, a0_nd;
    double p0, f0, t0, E0;
    double L_nd, kappa_nd;
    double eps_r;
} MaterialNorm;

extern MaterialNorm N_FE, N_AFE, N_DE;
extern int nx, ny, nz, ng_total, count, peloop, time_to_change, dep_flag, do_pre_relax, zbc_flag, sim_index;
extern double del_h, del_t, Ez_ext, Ez_prev, incEz, maxEz, delEz, E0_ref, P0_ref, eps_0_nd, sim_time;
extern char crystal_type[20];
extern char output_dir[4000];
extern int *omega, *grain_mat;
extern double *TR_h;
extern double *Pmx_old_d, *Pmy_old_d, *Pmz_old_d, *Pmx_d, *Pmy_d, *Pmz_d;
extern double *Psx_old_d, *Psy_old_d, *Psz_old_d, *Psx_d, *Psy_d, *Psz_d;
extern double *delecX_d, *delecY_d, *delecZ_d;
extern double *phi_dep_d;
extern bool phi_dep_initialized;
extern double *Pmx, *Pmy, *Pmz, *Psx, *Psy, *Psz;

namespace {

void die(const char *what)
{
    std::fprintf(stderr, "Error: %s: %s\n", what, cmsl_last_error());
    std::exit(1);   // the reference's convention for fatal errors (include/check.h)
}

void cuda_or_die(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        std::fprintf(stderr, "CUDA error in %s: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

cmsl_material nd_mat(const MaterialNorm &m)
{
    cmsl_material r;
    r.alpha = m.alpha_nd; r.beta = m.beta_nd; r.gamma = m.gamma_nd; r.g = m.g_nd; r.a0 = m.a0_nd;
    r.kappa = m.kappa_nd; r.L = m.L_nd; r.eps_r = m.eps_r;
    return r;
}

// A film over the reference's current state (host grain map, materials, TR).
cmsl_film *make_film(std::vector<int32_t> &gm)
{
    const int ng = ng_total;
    gm.assign(grain_mat, grain_mat + ng);
    for (int &g : gm)
        if (g < 0 || g > 2) g = CMSL_FE;
    cmsl_film_desc d = {};
    d.nx = nx; d.ny = ny; d.nz = nz; d.del_h = del_h; d.del_t = del_t;
    d.dep_flag = dep_flag; d.zbc = zbc_flag; d.eps_0_nd = eps_0_nd;
    d.n_grains = ng; d.omega = omega; d.grain_mat = gm.data(); d.TR = TR_h;
    d.mats[CMSL_AFE] = nd_mat(N_AFE); d.mats[CMSL_FE] = nd_mat(N_FE); d.mats[CMSL_DE] = nd_mat(N_DE);
    const char *p = std::getenv("CMSL_PRECISION");
    d.precision = (p && std::string(p) == "fp32") ? CMSL_FP32_REFINED : CMSL_FP64;
    d.pcg_crit = CMSL_CRIT_REF;
    d.tol_abs = 1.0e-3; d.tol_rel = 1.0e-2; d.max_iter = 4000;   // global.cu:140-144
    d.refine_tol = 1e-8; d.max_refine = 6; d.inner_tol = 1e-5; d.inner_max_iter = 2000; d.warm_start = 2;
    cmsl_film *f = nullptr;
    if (cmsl_film_create(&d, &f) != CMSL_OK) die("cmsl_film_create");
    return f;
}

void load_state(cmsl_film *f, double *const dev[6], bool use_phi)
{
    const size_t N = (size_t)nx * ny * nz;
    std::vector<double> P[6];
    const double *Pp[6];
    for (int q = 0; q < 6; ++q) {
        P[q].resize(N);
        cuda_or_die(cudaMemcpy(P[q].data(), dev[q], N * sizeof(double), cudaMemcpyDeviceToHost), "state copy");
        Pp[q] = P[q].data();
    }
    std::vector<double> phi(N, 0.0);
    if (use_phi && phi_dep_initialized && phi_dep_d)
        cuda_or_die(cudaMemcpy(phi.data(), phi_dep_d, N * sizeof(double), cudaMemcpyDeviceToHost), "phi copy");
    if (cmsl_film_set_state(f, Pp, phi.data()) != CMSL_OK) die("cmsl_film_set_state");
}

// Writes P back to both the old and new device sets, phi to phi_dep_d and
// E = -grad(phi) to delecX/Y/Z_d, as the reference leaves them.
void store_state(cmsl_film *f)
{
    const size_t N = (size_t)nx * ny * nz;
    std::vector<double> P[6], phi(N);
    double *Pp[6];
    for (int q = 0; q < 6; ++q) { P[q].resize(N); Pp[q] = P[q].data(); }
    if (cmsl_film_get_state(f, Pp, phi.data()) != CMSL_OK) die("cmsl_film_get_state");
    double *olds[6] = {Pmx_old_d, Pmy_old_d, Pmz_old_d, Psx_old_d, Psy_old_d, Psz_old_d};
    double *news[6] = {Pmx_d, Pmy_d, Pmz_d, Psx_d, Psy_d, Psz_d};
    for (int q = 0; q < 6; ++q) {
        if (olds[q]) cuda_or_die(cudaMemcpy(olds[q], P[q].data(), N * sizeof(double), cudaMemcpyHostToDevice), "P");
        if (news[q]) cuda_or_die(cudaMemcpy(news[q], P[q].data(), N * sizeof(double), cudaMemcpyHostToDevice), "P");
    }
    if (dep_flag != 0) {
        if (!phi_dep_d) cuda_or_die(cudaMalloc(&phi_dep_d, N * sizeof(double)), "phi alloc");
        phi_dep_initialized = true;
        cuda_or_die(cudaMemcpy(phi_dep_d, phi.data(), N * sizeof(double), cudaMemcpyHostToDevice), "phi");
        std::vector<double> E[3];
        for (auto &e : E) e.resize(N);
        // the E field needs the FP64 potential; FP32 films get it from a copy
        if (cmsl_film_efield(f, E[0].data(), E[1].data(), E[2].data()) == CMSL_OK) {
            double *dst[3] = {delecX_d, delecY_d, delecZ_d};
            for (int q = 0; q < 3; ++q)
                if (dst[q]) cuda_or_die(cudaMemcpy(dst[q], E[q].data(), N * sizeof(double), cudaMemcpyHostToDevice), "E");
        }
    }
}

// The film Depol_field solves on, kept between calls: it is rebuilt only
// when the grid, the materials, the grain map or the rotations change (a
// content hash of the host arrays, far cheaper than rebuilding the film).
struct DepolCache {
    cmsl_film *f = nullptr;
    std::vector<int32_t> gm;
    uint64_t key = 0;
} g_depol;

uint64_t mix(uint64_t h, uint64_t v)
{
    h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    return h;
}

uint64_t hash_words(uint64_t h, const void *p, size_t bytes)
{
    const unsigned char *b = (const unsigned char *)p;
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
        uint64_t v;
        std::memcpy(&v, b + i, 8);
        h = mix(h, v);
    }
    for (; i < bytes; ++i) h = mix(h, b[i]);
    return h;
}

uint64_t depol_key()
{
    const size_t N = (size_t)nx * ny * nz;
    uint64_t h = mix(mix(mix(0x1234, (uint64_t)nx), (uint64_t)ny), (uint64_t)nz);
    h = mix(mix(mix(h, (uint64_t)ng_total), (uint64_t)dep_flag), (uint64_t)zbc_flag);
    const double sc[3] = {del_h, del_t, eps_0_nd};
    h = hash_words(h, sc, sizeof sc);
    const MaterialNorm *m[3] = {&N_AFE, &N_FE, &N_DE};
    for (const MaterialNorm *q : m) h = hash_words(h, q, sizeof(MaterialNorm));
    const char *p = std::getenv("CMSL_PRECISION");
    h = mix(h, (p && std::string(p) == "fp32") ? 1u : 0u);
    if (omega) h = hash_words(h, omega, N * sizeof(int));
    if (grain_mat) h = hash_words(h, grain_mat, (size_t)ng_total * sizeof(int));
    if (TR_h) h = hash_words(h, TR_h, (size_t)ng_total * 9 * sizeof(double));
    return h;
}

cmsl_film *depol_film()
{
    const uint64_t key = depol_key();
    if (!g_depol.f || g_depol.key != key) {
        if (g_depol.f) cmsl_film_destroy(g_depol.f);
        g_depol.f = make_film(g_depol.gm);
        g_depol.key = key;
    }
    return g_depol.f;
}

}  // namespace

void evolve_resources_init(void) {}

// evolve.cu:67-71: frees the host P buffers (and the film Depol_field keeps)
void evolve_resources_cleanup(void)
{
    if (g_depol.f) {
        cmsl_film_destroy(g_depol.f);
        g_depol.f = nullptr;
    }
    double **h[6] = {&Pmx, &Pmy, &Pmz, &Psx, &Psy, &Psz};
    for (double **p : h) {
        std::free(*p);
        *p = nullptr;
    }
}

// depol_varEPS.cu:332-595: one solve on the new Pm (Pmx/Pmy/Pmz_d),
// warm-started from phi_dep_d (allocated and zeroed on first use, as
// init_phi_linear with g_bot = g_top = 0), writing phi_dep_d and
// delecX/Y/Z_d in place on the device.  The film is kept between calls.
void Depol_field(void)
{
    if (!dep_flag) return;
    const size_t N = (size_t)nx * ny * nz;
    if (!phi_dep_initialized || !phi_dep_d) {
        if (!phi_dep_d) cuda_or_die(cudaMalloc(&phi_dep_d, N * sizeof(double)), "phi alloc");
        cuda_or_die(cudaMemset(phi_dep_d, 0, N * sizeof(double)), "phi init");
        phi_dep_initialized = true;
    }
    cmsl_film *f = depol_film();
    int32_t it[2] = {0, 0}, st = 0;
    if (cmsl_film_depol_device(f, Pmx_d, Pmy_d, Pmz_d, phi_dep_d, delecX_d, delecY_d, delecZ_d, nullptr, it, &st) !=
        CMSL_OK)
        die("cmsl_film_depol_device");
    if (st != 0 && st != 3) std::printf("PCG breakdown (status %d)\n", st);
}

// The two slice files of the pre-relax stage (evolve.cu:202-210): Psz of
// the relaxed state, and Psz in the crystal frame of the state the last
// pre-relax step started from (the kernel's Psz_local output).
void pre_relax_slices(cmsl_film *f, int pre)
{
    const size_t N = (size_t)nx * ny * nz;
    std::vector<double> P[6], phi(N), loc(N);
    double *Pp[6];
    for (int q = 0; q < 6; ++q) { P[q].resize(N); Pp[q] = P[q].data(); }
    std::vector<double> Ez0((size_t)pre, 0.0);
    std::vector<int32_t> r0((size_t)pre, -1);
    if (pre > 1 && cmsl_film_run(f, pre - 1, Ez0.data(), r0.data(), nullptr) != CMSL_OK) die("cmsl_film_run");
    if (cmsl_film_sync(f) != CMSL_OK) std::printf("PCG ERROR reported during the pre-relax: %s\n", cmsl_last_error());
    if (cmsl_film_get_state(f, Pp, phi.data()) != CMSL_OK) die("cmsl_film_get_state");
    if (cmsl_crystal_z((long long)N, omega, TR_h, Pp[3], Pp[4], Pp[5], loc.data()) != CMSL_OK) die("cmsl_crystal_z");
    if (cmsl_film_run(f, 1, Ez0.data(), r0.data(), nullptr) != CMSL_OK) die("cmsl_film_run");
    if (cmsl_film_sync(f) != CMSL_OK) std::printf("PCG ERROR reported during the pre-relax: %s\n", cmsl_last_error());
    if (cmsl_film_get_state(f, Pp, phi.data()) != CMSL_OK) die("cmsl_film_get_state");
    if (cmsl_midplane_slice_write("slice_E0_midplane.dat", Pp[5], nx, ny, nz) != CMSL_OK ||
        cmsl_midplane_slice_write("slice_E0_midplane_local.dat", loc.data(), nx, ny, nz) != CMSL_OK)
        std::fprintf(stderr, "Cannot write the midplane slices: %s\n", cmsl_last_error());
}

// evolve.cu:73-440: the P-E loop with the sweep file output.
void Evolve(void)
{
    std::printf("Now in evolve.\n");
    const bool single = std::strcmp(crystal_type, "single") == 0;
    std::vector<int32_t> gm;
    cmsl_film *f = make_film(gm);
    double *olds[6] = {Pmx_old_d, Pmy_old_d, Pmz_old_d, Psx_old_d, Psy_old_d, Psz_old_d};
    load_state(f, olds, true);

    int ns = 0, nr = 0;
    if (cmsl_evolve_schedule(maxEz, delEz, time_to_change, 1, single, E0_ref, 100000000, nullptr, nullptr, &ns,
                             nullptr, nullptr, &nr) != CMSL_OK)
        die("cmsl_evolve_schedule");
    const int pre = do_pre_relax ? 15000 : 0;                             // evolve.cu:171-211
    std::vector<double> Ez(ns, 0.0), rowE(nr);
    std::vector<int32_t> row(ns, -1), rowc(nr);
    cmsl_evolve_schedule(maxEz, delEz, time_to_change, 1, single, E0_ref, 100000000, Ez.data(), row.data(), &ns,
                         rowE.data(), rowc.data(), &nr);

    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, 0);
    if (pre > 0) pre_relax_slices(f, pre);                                // stage A at E = 0
    if (cmsl_film_run(f, (int)Ez.size(), Ez.data(), row.data(), nullptr) != CMSL_OK) die("cmsl_film_run");
    if (cmsl_film_sync(f) != CMSL_OK) std::printf("PCG ERROR reported during the loop: %s\n", cmsl_last_error());
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);

    std::vector<double> rows((size_t)nr * CMSL_ROW_WIDTH);
    if (nr > 0 && cmsl_film_get_rows(f, 0, nr, rows.data()) != CMSL_OK) die("cmsl_film_get_rows");
    char path[4100];
    std::snprintf(path, sizeof path, "%s/sweep%03d.txt", output_dir, sim_index);
    FILE *fo = std::fopen(path, "a");
    if (!fo) {
        std::printf("Error opening %s\n", path);
        std::exit(1);
    }
    const double Es = E0_ref / 1.0e+08, Ps = P0_ref * 100.0;             // evolve.cu:117-118
    for (int r = 0; r < nr; ++r) {
        const double *v = rows.data() + (size_t)r * CMSL_ROW_WIDTH;
        std::fprintf(fo, "%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%d\n", rowE[r] * Es, v[0] * Ps,
                     v[1] * Ps, v[2] * Ps, v[3] * Ps, v[4] * Ps, v[5], v[6] * Ps, v[7], v[8] * Ps, v[9],
                     count + pre + rowc[r]);
    }
    std::fclose(fo);
    store_state(f);
    cmsl_film_destroy(f);

    // leave the loop counters as the reference does
    const int steps = pre + ns;
    sim_time += steps * del_t;
    count += steps;
    peloop = 2;
    if (nr > 0) {
        Ez_prev = rowE[nr - 1];
        incEz = -delEz;
        Ez_ext = Ez_prev + incEz;
    }
    std::printf("Kernel execution time: %f s\n", ms / 1000.0);
    std::fflush(stdout);
}
