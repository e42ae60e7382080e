/*
 * cmsl_io.h -- the reference's input formats and simulation set-up, in C ABI
 * form (host code, no GPU needed).  These are the steps that feed the hot
 * path in the reference: the InputParams deck, the grain-map files, the
 * Landau and phase-fraction pools, the non-dimensionalisation, the
 * grain-to-material assignment and the P-E loop field schedule.
 *
 * Every function returns cmsl_status (never exits); text of the last failure
 * is in cmsl_last_error().
 */
#ifndef CMSL_IO_H
#define CMSL_IO_H

#include "cmsl.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The InputParams deck (HZO_Code_github/src/get_InputParams.cu:8-92). */
typedef struct {
    int device_flag, nx, ny, nz, dep_flag, num_steps, out_flag, dimx, dimy, dimz;
    double del_h, del_t, delEap, Eap;
    double kappa_fe, L_fe, kappa_afe, L_afe, kappa_de, L_de;
    double eps_fe, eps_afe, eps_de;
    double PsNoise, G0, omg;
    int do_pre_relax;
    int n_layers;
    int layer_counts[16];
    char crystal_type[20];
    char z_bc_type[20];
} cmsl_deck;

/* processInputParams (get_InputParams.cu:8-127): prefix-matched "key = value"
 * lines in the reference's matching order; layer_counts must sum to nz. */
cmsl_status cmsl_deck_read(const char *path, cmsl_deck *out);
/* The OutputParams summary file the reference writes (get_InputParams.cu:130-150). */
cmsl_status cmsl_deck_write_summary(const cmsl_deck *deck, const char *path);

/* ReadGrainCount (grain_io.cu:10-25): the first integer of a gnumb file. */
cmsl_status cmsl_grain_count(const char *gnumb_path, int *n_grains);

/* LoadGrainStructureFromDir (grain_io.cu:26-135): <dir>/gdata_<tag>.bin
 * (int32 omega[N] then float64 eta[N], z fastest) transposed to C order,
 * <dir>/gchar_<tag>.txt (gid cx cy cz phi theta psi), rotations TR.
 * cent and euler are [3*n_grains]; any output may be NULL. */
cmsl_status cmsl_grain_read(const char *dir, const char *tag, int nx, int ny, int nz, int n_grains,
                            int32_t *omega, double *eta, double *cent, double *euler, double *TR);
/* Writes the three files of a grain map in the same formats (gnumb into
 * gnumb_path); the inverse of cmsl_grain_read. */
cmsl_status cmsl_grain_write(const char *dir, const char *tag, const char *gnumb_path, int nx, int ny,
                             int nz, int n_grains, const int32_t *omega, const double *eta,
                             const double *cent, const double *euler);

/* Bunge ZXZ lab->crystal rotation per grain (grain_io.cu:103-126). */
cmsl_status cmsl_tr_from_euler(int n_grains, const double *phi, const double *theta, const double *psi,
                               double *TR);

/* One Landau coefficient set: AFE (alpha, beta, gamma1, g, a0), FE (same), DE
 * (alpha, a0), the reference phase (0 AFE, 1 FE, 2 DE) and, from 16-column
 * tables, phase fractions in percent (negative when absent). */
typedef struct {
    double afe[5], fe[5], de[2];
    int ref_type;
    double frac_afe, frac_fe, frac_de;
} cmsl_landau_set;

/* LoadLandauPool (main.cu:123-155): 12 numbers + label per line; 16-column
 * lines (12 numbers, 3 fractions, label) are accepted too. */
cmsl_status cmsl_landau_pool_read(const char *path, cmsl_landau_set *out, int max_sets, int *n_sets);
/* LoadPhasePool (main.cu:81-98): triples of percentages, lines with DE > 50
 * skipped; returned as fractions. */
cmsl_status cmsl_phase_pool_read(const char *path, double *afe, double *fe, double *de, int max_entries,
                                 int *n_entries);

/* Raw (SI) material parameters, types.h:15-20. */
typedef struct {
    double alpha, beta, gamma1, g, a0;
    int transition_type;
    double L, kappa, eps_r;
} cmsl_raw_material;

/* Scalars of SetupAndRunSimulation (main.cu:261-349). */
typedef struct {
    double alpha_ref, P0_ref, L_ref, kappa_ref, f0_ref, E0_ref, eps_0_nd, maxEz, delEz;
} cmsl_scales;

/* compute_p0 / make_phase_refs / make_nd_wrt_reference against the reference
 * phase ref_type (main.cu:200-256, t0 = 3e-9 s, l0 = 1e-9 m, global.cu:30-31),
 * plus E0_ref, eps_0_nd, maxEz = Eap/E0_ref and delEz = delEap/E0_ref.
 * raw[3] and nd[3] are indexed AFE, FE, DE. */
cmsl_status cmsl_nondim(const cmsl_raw_material raw[3], int ref_type, double Eap, double delEap,
                        cmsl_material nd[3], cmsl_scales *scales);

/* Grain -> material by voxel-fraction targets per layer (init_conf.cu:108-260).
 * Uses the C library's srand(123456)/rand() as the reference does (so it
 * reseeds the process-wide rand() state). fractions in [0,1] per layer. */
cmsl_status cmsl_assign_materials(int nx, int ny, int nz, int n_grains, const int32_t *omega,
                                  const double *centz, int n_layers, const int *layer_counts,
                                  const double *afe, const double *fe, const double *de,
                                  int32_t *grain_mat);

/* build_interface_flag (main.cu:13-42). */
cmsl_status cmsl_interface_flags(int nx, int ny, int nz, const int32_t *omega, const int32_t *grain_mat,
                                 int32_t *flag);

/* build_interface_flag (main.cu:13-52) on DEVICE arrays (omega[N],
 * grain_mat[n_grains], flags[N]), e.g. a grain map generated on the GPU;
 * grain ids outside [0, n_grains) count as not FE; runs on `stream` without
 * synchronising. */
cmsl_status cmsl_interface_flags_gpu(int nx, int ny, int nz, int n_grains, const int32_t *omega_dev,
                                     const int32_t *grain_mat_dev, int32_t *flags_dev, void *stream);

/* The field schedule of Evolve (evolve.cu:123-409): Ez[s] per step and
 * row[s] (output row index or -1); row_E/row_count per row.  n_periods = 1 is
 * the reference's peloop < 2.  Pass NULL arrays to query the sizes. */
cmsl_status cmsl_evolve_schedule(double maxEz, double delEz, int num_steps, int n_periods, int single_crystal,
                                 double E0_ref, int max_steps, double *Ez, int32_t *row, int *n_steps,
                                 double *row_E, int32_t *row_count, int *n_rows);

/* Seeded columnar periodic Voronoi grain map (in-plane seeds, grains through
 * z) with orientations |cos theta| ~ U[0.3, 1]; a stand-in generator for the
 * reference's genpolycr_layered/voronoi.c, whose maps are not shipped.
 * cent/euler are [3*n_grains]. */
cmsl_status cmsl_voronoi_columnar(int nx, int ny, int nz, int n_grains, uint64_t seed, int32_t *omega,
                                  double *cent, double *euler);

/* cmsl_voronoi_columnar computed on the GPU (one thread per column, seeds in
 * shared memory, distances in explicitly rounded FP64): the same map, centres
 * and orientations as the host generator.  omega, cent, euler are host arrays. */
cmsl_status cmsl_voronoi_columnar_gpu(int nx, int ny, int nz, int n_grains, uint64_t seed, int32_t *omega,
                                      double *cent, double *euler);

/* Checkpoint file of the reference (generate.cu:90-264, write_checkpoint /
 * read_checkpoint): header int nx, ny, nz, peloop, count; double Ez_ext,
 * incEz; then Pmx, Pmy, Pmz, Psx, Psy, Psz, Ex, Ey, Ez (N doubles each), host
 * byte order.  read: the file's grid must equal (nx, ny, nz) (CMSL_ERR_IO
 * otherwise); P or E may be NULL to skip them. */
cmsl_status cmsl_checkpoint_write(const char *path, int nx, int ny, int nz, int peloop, int count, double Ez_ext,
                                  double incEz, const double *const P[6], const double *const E[3]);
cmsl_status cmsl_checkpoint_read(const char *path, int nx, int ny, int nz, int *peloop, int *count, double *Ez_ext,
                                 double *incEz, double *const P[6], double *const E[3]);

/* write_vector_field_binary (generate.cu:11-30): the interleaved
 * (x, y, z) * scale of n cells as doubles. */
cmsl_status cmsl_vector_field_write(const char *path, const double *Px, const double *Py, const double *Pz,
                                    long long n, double scale);

/* write_midplane_slice (generate.cu:67-88): the plane k = nz/2 of v as text
 * lines "i j value" (%.16e), a blank line after each row j. */
cmsl_status cmsl_midplane_slice_write(const char *path, const double *v, int nx, int ny, int nz);

/* The crystal-frame z component of a lab-frame vector field per cell,
 * TR[9 omega + 6] x + TR[9 omega + 7] y + TR[9 omega + 8] z in that order
 * (kernelCalc_antiferro's *_local outputs, kernels_evol.cu:160-175). */
cmsl_status cmsl_crystal_z(long long n, const int32_t *omega, const double *TR, const double *x, const double *y,
                           const double *z, double *out);

/* Calc_EfieldMag (depol_varEPS.cu:223-276) on the host: E = -grad(phi). */
cmsl_status cmsl_efield_host(int nx, int ny, int nz, double del_h, int zbc, const double *phi, double *Ex,
                             double *Ey, double *Ez);

#ifdef __cplusplus
}
#endif
#endif
