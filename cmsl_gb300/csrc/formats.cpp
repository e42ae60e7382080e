// formats.cpp -- the reference's input formats and set-up steps (host C++).
//
// Compiled with -ffp-contract=off: the non-dimensionalisation and the rotation
// matrices then round exactly as the reference's host code does.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cmsl_io.h"

void cmsl_internal_set_error(const char *msg);   // engine.cu

namespace {

cmsl_status io_fail(cmsl_status s, const std::string &m)
{
    cmsl_internal_set_error(m.c_str());
    return s;
}

// FILE* closed on scope exit
struct FileCloser {
    void operator()(FILE *f) const
    {
        if (f) std::fclose(f);
    }
};
using File = std::unique_ptr<FILE, FileCloser>;

bool starts(const char *line, const char *key) { return std::strncmp(line, key, std::strlen(key)) == 0; }

// "key = value" scanned with the key itself as the literal prefix, as the
// reference's sscanf calls do (whitespace around '=' is free; a line whose
// text after the key is not " = value" leaves the field unchanged)
template <class V> bool scan_kv(const char *line, const char *key, const char *conv, V *v)
{
    char fmt[64];
    std::snprintf(fmt, sizeof fmt, "%s = %s", key, conv);
    return std::sscanf(line, fmt, v) == 1;
}

bool get_int(const char *line, const char *key, int *v) { return scan_kv(line, key, "%d", v); }
bool get_dbl(const char *line, const char *key, double *v) { return scan_kv(line, key, "%lf", v); }

bool get_word(const char *line, const char *key, char *dst, size_t cap)
{
    char tmp[256];
    if (!scan_kv(line, key, "%255s", tmp)) return false;
    std::strncpy(dst, tmp, cap - 1);
    dst[cap - 1] = '\0';
    return true;
}

}  // namespace

extern "C" {

// get_InputParams.cu:18-92.  The first matching prefix wins, in this order
// (so e.g. "delEap" is tested before "Eap", "L_fe" before "L_afe").
cmsl_status cmsl_deck_read(const char *path, cmsl_deck *d)
{
    if (!path || !d) return io_fail(CMSL_ERR_ARG, "NULL argument");
    std::memset(d, 0, sizeof(*d));
    FILE *fp = std::fopen(path, "r");
    if (!fp) return io_fail(CMSL_ERR_IO, std::string("cannot open deck ") + path);
    char line[256];
    cmsl_status st = CMSL_OK;
    while (std::fgets(line, sizeof line, fp)) {
        if (starts(line, "device_flag")) get_int(line, "device_flag", &d->device_flag);
        else if (starts(line, "nx")) get_int(line, "nx", &d->nx);
        else if (starts(line, "ny")) get_int(line, "ny", &d->ny);
        else if (starts(line, "nz")) get_int(line, "nz", &d->nz);
        else if (starts(line, "dep_flag")) get_int(line, "dep_flag", &d->dep_flag);
        else if (starts(line, "del_h")) get_dbl(line, "del_h", &d->del_h);
        else if (starts(line, "del_t")) get_dbl(line, "del_t", &d->del_t);
        else if (starts(line, "delEap")) get_dbl(line, "delEap", &d->delEap);
        else if (starts(line, "Eap")) get_dbl(line, "Eap", &d->Eap);
        else if (starts(line, "num_steps")) get_int(line, "num_steps", &d->num_steps);
        else if (starts(line, "out_flag")) get_int(line, "out_flag", &d->out_flag);
        else if (starts(line, "dimx")) get_int(line, "dimx", &d->dimx);
        else if (starts(line, "dimy")) get_int(line, "dimy", &d->dimy);
        else if (starts(line, "dimz")) get_int(line, "dimz", &d->dimz);
        else if (starts(line, "kappa_fe")) get_dbl(line, "kappa_fe", &d->kappa_fe);
        else if (std::strncmp(line, "L_fe", 4) == 0) get_dbl(line, "L_fe", &d->L_fe);
        else if (starts(line, "kappa_afe")) get_dbl(line, "kappa_afe", &d->kappa_afe);
        else if (std::strncmp(line, "L_afe", 4) == 0) get_dbl(line, "L_afe", &d->L_afe);
        else if (starts(line, "kappa_de")) get_dbl(line, "kappa_de", &d->kappa_de);
        else if (starts(line, "L_de")) get_dbl(line, "L_de", &d->L_de);
        else if (starts(line, "PsNoise")) get_dbl(line, "PsNoise", &d->PsNoise);
        else if (starts(line, "do_pre_relax")) get_int(line, "do_pre_relax", &d->do_pre_relax);
        else if (starts(line, "crystal_type")) get_word(line, "crystal_type", d->crystal_type, sizeof d->crystal_type);
        else if (starts(line, "G0")) get_dbl(line, "G0", &d->G0);
        else if (starts(line, "eps_de")) get_dbl(line, "eps_de", &d->eps_de);
        else if (starts(line, "eps_fe")) get_dbl(line, "eps_fe", &d->eps_fe);
        else if (starts(line, "eps_afe")) get_dbl(line, "eps_afe", &d->eps_afe);
        else if (starts(line, "omg")) get_dbl(line, "omg", &d->omg);
        else if (starts(line, "z_bc_type")) get_word(line, "z_bc_type", d->z_bc_type, sizeof d->z_bc_type);
        else if (starts(line, "n_layers")) get_int(line, "n_layers", &d->n_layers);
        else if (starts(line, "layer_counts")) {
            const char *p = std::strchr(line, '=');
            if (p) ++p;
            int i = 0, used = 0;
            const int want = d->n_layers < 16 ? d->n_layers : 16;
            while (p && i < want && std::sscanf(p, "%d%n", &d->layer_counts[i], &used) == 1) {
                p += used;
                ++i;
            }
            if (i != d->n_layers) {
                st = io_fail(CMSL_ERR_IO, "layer_counts: expected " + std::to_string(d->n_layers) + ", got " +
                                              std::to_string(i));
                break;
            }
        }
    }
    std::fclose(fp);
    if (st != CMSL_OK) return st;
    int sum = 0;
    for (int i = 0; i < d->n_layers && i < 16; ++i) sum += d->layer_counts[i];
    if (sum != d->nz)   // get_InputParams.cu:122-127
        return io_fail(CMSL_ERR_IO, "layer_counts sum " + std::to_string(sum) + " != nz " + std::to_string(d->nz));
    return CMSL_OK;
}

// get_InputParams.cu:130-150
cmsl_status cmsl_deck_write_summary(const cmsl_deck *d, const char *path)
{
    if (!d || !path) return io_fail(CMSL_ERR_ARG, "NULL argument");
    FILE *f = std::fopen(path, "w");
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot write ") + path);
    std::fprintf(f, "Device Flag: %d\n\n", d->device_flag);
    std::fprintf(f, "Print Flag for Ps and Pm: %d\n\n", d->out_flag);
    std::fprintf(f, "Grid Spacing (del_h): %lf\n\n", d->del_h);
    std::fprintf(f, "Time Step (del_t): %lf\n\n", d->del_t);
    std::fprintf(f, "Electric Field Increment (delE): %lf\n\n", d->delEap);
    std::fprintf(f, "Maximum Electric Field (maxE): %lf\n\n", d->Eap);
    std::fprintf(f, "Grid Points (nx, ny, nz): %d, %d, %d\n\n", d->nx, d->ny, d->nz);
    std::fprintf(f, "Number of Steps: %d\n\n", d->num_steps);
    std::fprintf(f, "Grid Dimensions (dimx, dimy, dimz): %d, %d, %d\n\n", d->dimx, d->dimy, d->dimz);
    std::fprintf(f, "\nNoise added to Ps: %le\n\n", d->PsNoise);
    std::fprintf(f, "---------------------------------\n");
    std::fclose(f);
    return CMSL_OK;
}

cmsl_status cmsl_grain_count(const char *path, int *ng)
{
    if (!path || !ng) return io_fail(CMSL_ERR_ARG, "NULL argument");
    FILE *f = std::fopen(path, "r");
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot open grain count file ") + path);
    const int ok = std::fscanf(f, "%d", ng);
    std::fclose(f);
    if (ok != 1) return io_fail(CMSL_ERR_IO, std::string("no grain count in ") + path);
    return CMSL_OK;
}

cmsl_status cmsl_tr_from_euler(int ng, const double *phi, const double *theta, const double *psi, double *TR)
{
    if (ng < 0 || (ng && (!phi || !theta || !psi || !TR))) return io_fail(CMSL_ERR_ARG, "bad arguments");
    for (int g = 0; g < ng; ++g) {
        const double sph = std::sin(phi[g]), cph = std::cos(phi[g]);
        const double sth = std::sin(theta[g]), cth = std::cos(theta[g]);
        const double sps = std::sin(psi[g]), cps = std::cos(psi[g]);
        const double cth_sph = cth * sph, cth_cph = cth * cph;
        double *T = TR + 9 * (size_t)g;
        T[0] = cph * cps - cth_sph * sps;
        T[1] = sph * cps + cth_cph * sps;
        T[2] = sth * sps;
        T[3] = -cph * sps - cth_sph * cps;
        T[4] = -sph * sps + cth_cph * cps;
        T[5] = sth * cps;
        T[6] = sth * sph;
        T[7] = -(sth * cph);
        T[8] = cth;
    }
    return CMSL_OK;
}

cmsl_status cmsl_grain_read(const char *dir, const char *tag, int nx, int ny, int nz, int ng, int32_t *omega,
                            double *eta, double *cent, double *euler, double *TR)
{
    if (!dir || !tag || nx < 1 || ny < 1 || nz < 1 || ng < 1) return io_fail(CMSL_ERR_ARG, "bad arguments");
    const size_t N = (size_t)nx * ny * nz;
    std::string pd = std::string(dir) + "/gdata_" + tag + ".bin";
    FILE *f = std::fopen(pd.c_str(), "rb");
    if (!f) return io_fail(CMSL_ERR_IO, "cannot open " + pd);
    std::vector<int32_t> om(N);
    std::vector<double> et(N);
    const size_t a = std::fread(om.data(), sizeof(int32_t), N, f);
    const size_t b = std::fread(et.data(), sizeof(double), N, f);
    std::fclose(f);
    if (a != N || b != N) return io_fail(CMSL_ERR_IO, "short grain map " + pd);
    // z-fastest file order id_f = k + nz*(j + ny*i) -> C order (grain_io.cu:61-69)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const size_t idf = (size_t)k + (size_t)nz * ((size_t)j + (size_t)i * ny);
                const size_t idc = (size_t)i + (size_t)nx * ((size_t)j + (size_t)k * ny);
                if (omega) omega[idc] = om[idf];
                if (eta) eta[idc] = et[idf];
            }
    std::string pc = std::string(dir) + "/gchar_" + tag + ".txt";
    f = std::fopen(pc.c_str(), "r");
    if (!f) return io_fail(CMSL_ERR_IO, "cannot open " + pc);
    std::vector<double> c(3 * (size_t)ng, -1.0), e(3 * (size_t)ng, 0.0);
    for (int k = 0; k < ng; ++k) {
        int gid;
        double x, y, z, p, t, s;
        if (std::fscanf(f, "%d %lf %lf %lf %lf %lf %lf", &gid, &x, &y, &z, &p, &t, &s) != 7) {
            std::fclose(f);
            return io_fail(CMSL_ERR_IO, "bad line " + std::to_string(k) + " in " + pc);
        }
        if (gid < 0 || gid >= ng) {
            std::fclose(f);
            return io_fail(CMSL_ERR_IO, "grain id " + std::to_string(gid) + " out of range in " + pc);
        }
        c[3 * gid] = x; c[3 * gid + 1] = y; c[3 * gid + 2] = z;
        e[3 * gid] = p; e[3 * gid + 1] = t; e[3 * gid + 2] = s;
    }
    std::fclose(f);
    if (cent) std::memcpy(cent, c.data(), sizeof(double) * c.size());
    if (euler) std::memcpy(euler, e.data(), sizeof(double) * e.size());
    if (TR) {
        std::vector<double> ph(ng), th(ng), ps(ng);
        for (int g = 0; g < ng; ++g) { ph[g] = e[3 * g]; th[g] = e[3 * g + 1]; ps[g] = e[3 * g + 2]; }
        cmsl_tr_from_euler(ng, ph.data(), th.data(), ps.data(), TR);
    }
    return CMSL_OK;
}

cmsl_status cmsl_grain_write(const char *dir, const char *tag, const char *gnumb_path, int nx, int ny, int nz,
                             int ng, const int32_t *omega, const double *eta, const double *cent,
                             const double *euler)
{
    if (!dir || !tag || !omega || !cent || !euler || nx < 1 || ny < 1 || nz < 1 || ng < 1)
        return io_fail(CMSL_ERR_ARG, "bad arguments");
    const size_t N = (size_t)nx * ny * nz;
    std::vector<int32_t> om(N);
    std::vector<double> et(N, 0.0);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const size_t idf = (size_t)k + (size_t)nz * ((size_t)j + (size_t)i * ny);
                const size_t idc = (size_t)i + (size_t)nx * ((size_t)j + (size_t)k * ny);
                om[idf] = omega[idc];
                et[idf] = eta ? eta[idc] : 0.0;
            }
    std::string pd = std::string(dir) + "/gdata_" + tag + ".bin";
    FILE *f = std::fopen(pd.c_str(), "wb");
    if (!f) return io_fail(CMSL_ERR_IO, "cannot write " + pd);
    const bool ok = std::fwrite(om.data(), sizeof(int32_t), N, f) == N && std::fwrite(et.data(), sizeof(double), N, f) == N;
    std::fclose(f);
    if (!ok) return io_fail(CMSL_ERR_IO, "short write " + pd);
    std::string pc = std::string(dir) + "/gchar_" + tag + ".txt";
    f = std::fopen(pc.c_str(), "w");
    if (!f) return io_fail(CMSL_ERR_IO, "cannot write " + pc);
    for (int g = 0; g < ng; ++g)
        std::fprintf(f, "%d\t%.17g\t%.17g\t%.17g\t%.17g\t%.17g\t%.17g\n", g, cent[3 * g], cent[3 * g + 1],
                     cent[3 * g + 2], euler[3 * g], euler[3 * g + 1], euler[3 * g + 2]);
    std::fclose(f);
    if (gnumb_path) {
        f = std::fopen(gnumb_path, "w");
        if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot write ") + gnumb_path);
        std::fprintf(f, "%d\n", ng);
        std::fclose(f);
    }
    return CMSL_OK;
}

// main.cu:123-155 (13 tokens) and the 16-column tables of the shipped inputs
cmsl_status cmsl_landau_pool_read(const char *path, cmsl_landau_set *out, int max_sets, int *n_sets)
{
    if (!path || !out || !n_sets || max_sets < 0) return io_fail(CMSL_ERR_ARG, "bad arguments");
    FILE *f = std::fopen(path, "r");
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot open Landau pool ") + path);
    char line[1024];
    int n = 0;
    while (n < max_sets && std::fgets(line, sizeof line, f)) {
        const char *p = line;
        while (std::isspace((unsigned char)*p)) ++p;
        if (*p == '\0' || *p == '#') continue;
        std::vector<std::string> tok;
        char buf[1024];
        std::strncpy(buf, p, sizeof buf - 1);
        buf[sizeof buf - 1] = '\0';
        for (char *t = std::strtok(buf, " \t\r\n"); t; t = std::strtok(nullptr, " \t\r\n")) tok.emplace_back(t);
        if (tok.size() != 13 && tok.size() != 16) continue;
        double v[15];
        bool num = true;
        for (size_t i = 0; i + 1 < tok.size(); ++i) {
            char *end = nullptr;
            v[i] = std::strtod(tok[i].c_str(), &end);
            if (!end || *end) { num = false; break; }
        }
        if (!num) continue;
        const std::string &lab = tok.back();
        const int ref = lab == "AFE" ? 0 : lab == "FE" ? 1 : lab == "DE" ? 2 : -1;
        if (ref < 0) continue;
        cmsl_landau_set &s = out[n];
        for (int i = 0; i < 5; ++i) { s.afe[i] = v[i]; s.fe[i] = v[5 + i]; }
        s.de[0] = v[10]; s.de[1] = v[11];
        s.ref_type = ref;
        if (tok.size() == 16) { s.frac_afe = v[12]; s.frac_fe = v[13]; s.frac_de = v[14]; }
        else { s.frac_afe = s.frac_fe = s.frac_de = -1.0; }
        ++n;
    }
    std::fclose(f);
    *n_sets = n;
    return CMSL_OK;
}

// main.cu:81-98
// generate.cu:90-163 (write_checkpoint) layout: int nx, ny, nz, peloop, count;
// double Ez_ext, incEz; then Pmx, Pmy, Pmz, Psx, Psy, Psz, Ex, Ey, Ez, N
// doubles each, host byte order.
cmsl_status cmsl_checkpoint_write(const char *path, int nx, int ny, int nz, int peloop, int count, double Ez_ext,
                                  double incEz, const double *const P[6], const double *const E[3])
{
    if (!path || !P || !E || nx < 1 || ny < 1 || nz < 1) return io_fail(CMSL_ERR_ARG, "bad arguments");
    for (int q = 0; q < 6; ++q)
        if (!P[q]) return io_fail(CMSL_ERR_ARG, "P[" + std::to_string(q) + "] is NULL");
    for (int q = 0; q < 3; ++q)
        if (!E[q]) return io_fail(CMSL_ERR_ARG, "E[" + std::to_string(q) + "] is NULL");
    const size_t N = (size_t)nx * ny * nz;
    File f(std::fopen(path, "wb"));
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot write ") + path);
    const int hdr[5] = {nx, ny, nz, peloop, count};
    const double hd[2] = {Ez_ext, incEz};
    bool ok = std::fwrite(hdr, sizeof(int), 5, f.get()) == 5 && std::fwrite(hd, sizeof(double), 2, f.get()) == 2;
    for (int q = 0; ok && q < 6; ++q) ok = std::fwrite(P[q], sizeof(double), N, f.get()) == N;
    for (int q = 0; ok && q < 3; ++q) ok = std::fwrite(E[q], sizeof(double), N, f.get()) == N;
    if (!ok) return io_fail(CMSL_ERR_IO, std::string("short write ") + path);
    return CMSL_OK;
}

// generate.cu:165-264 (read_checkpoint): the grid in the file must match.
cmsl_status cmsl_checkpoint_read(const char *path, int nx, int ny, int nz, int *peloop, int *count, double *Ez_ext,
                                 double *incEz, double *const P[6], double *const E[3])
{
    if (!path || nx < 1 || ny < 1 || nz < 1) return io_fail(CMSL_ERR_ARG, "bad arguments");
    const size_t N = (size_t)nx * ny * nz;
    File f(std::fopen(path, "rb"));
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot open checkpoint ") + path);
    int hdr[5];
    double hd[2];
    if (std::fread(hdr, sizeof(int), 5, f.get()) != 5 || std::fread(hd, sizeof(double), 2, f.get()) != 2)
        return io_fail(CMSL_ERR_IO, std::string("checkpoint header read failed: ") + path);
    if (hdr[0] != nx || hdr[1] != ny || hdr[2] != nz)
        return io_fail(CMSL_ERR_IO, "checkpoint grid mismatch: file (" + std::to_string(hdr[0]) + "," +
                                        std::to_string(hdr[1]) + "," + std::to_string(hdr[2]) + "), expected (" +
                                        std::to_string(nx) + "," + std::to_string(ny) + "," + std::to_string(nz) + ")");
    std::vector<double> skip;
    for (int q = 0; q < 9; ++q) {
        double *dst = q < 6 ? (P ? P[q] : nullptr) : (E ? E[q - 6] : nullptr);
        if (!dst) {
            skip.resize(N);
            dst = skip.data();
        }
        if (std::fread(dst, sizeof(double), N, f.get()) != N)
            return io_fail(CMSL_ERR_IO, std::string("checkpoint data read failed: ") + path);
    }
    if (peloop) *peloop = hdr[3];
    if (count) *count = hdr[4];
    if (Ez_ext) *Ez_ext = hd[0];
    if (incEz) *incEz = hd[1];
    return CMSL_OK;
}

// generate.cu:11-30 (write_vector_field_binary): (x, y, z) * scale per cell.
cmsl_status cmsl_vector_field_write(const char *path, const double *Px, const double *Py, const double *Pz,
                                    long long n, double scale)
{
    if (!path || !Px || !Py || !Pz || n < 0) return io_fail(CMSL_ERR_ARG, "bad arguments");
    File f(std::fopen(path, "wb"));
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot write ") + path);
    std::vector<double> buf;
    buf.reserve(3 * 4096);
    for (long long i = 0; i < n;) {
        buf.clear();
        const long long e = std::min(n, i + 4096);
        for (; i < e; ++i) {
            buf.push_back(Px[i] * scale);
            buf.push_back(Py[i] * scale);
            buf.push_back(Pz[i] * scale);
        }
        if (std::fwrite(buf.data(), sizeof(double), buf.size(), f.get()) != buf.size())
            return io_fail(CMSL_ERR_IO, std::string("short write ") + path);
    }
    return CMSL_OK;
}

// write_midplane_slice (generate.cu:67-88): "i j value" lines of the plane
// k = nz/2, rows j in order, a blank line after each.
cmsl_status cmsl_midplane_slice_write(const char *path, const double *v, int nx, int ny, int nz)
{
    if (!path || !v || nx < 1 || ny < 1 || nz < 1) return io_fail(CMSL_ERR_ARG, "bad arguments");
    File f(std::fopen(path, "w"));
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot write ") + path);
    const long long base = (long long)nx * ny * (nz / 2);
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) std::fprintf(f.get(), "%d %d %.16e\n", i, j, v[base + i + (long long)nx * j]);
        std::fprintf(f.get(), "\n");
    }
    return std::ferror(f.get()) ? io_fail(CMSL_ERR_IO, std::string("short write ") + path) : CMSL_OK;
}

// The crystal-frame z component (row 3 of the grain's rotation applied to
// the lab vector), in the order of kernels_evol.cu:162-167.
cmsl_status cmsl_crystal_z(long long n, const int32_t *omega, const double *TR, const double *x, const double *y,
                           const double *z, double *out)
{
    if (n < 0 || !omega || !TR || !x || !y || !z || !out) return io_fail(CMSL_ERR_ARG, "bad arguments");
    for (long long i = 0; i < n; ++i) {
        const double *t = TR + 9LL * omega[i];
        out[i] = t[6] * x[i] + t[7] * y[i] + t[8] * z[i];
    }
    return CMSL_OK;
}

// Calc_EfieldMag (depol_varEPS.cu:223-276) on the host: E = -grad(phi), x/y
// periodic; Dirichlet z with phi = 0 beyond the planes, or the mirrored
// Neumann neighbours.
cmsl_status cmsl_efield_host(int nx, int ny, int nz, double del_h, int zbc, const double *phi, double *Ex,
                             double *Ey, double *Ez)
{
    if (nx < 1 || ny < 1 || nz < 3 || !phi || !Ex || !Ey || !Ez) return io_fail(CMSL_ERR_ARG, "bad arguments");
    auto id = [&](int i, int j, int k) { return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k); };
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t c = id(i, j, k);
                Ex[c] = -(phi[id((i + 1) % nx, j, k)] - phi[id((i - 1 + nx) % nx, j, k)]) / (2.0 * del_h);
                Ey[c] = -(phi[id(i, (j + 1) % ny, k)] - phi[id(i, (j - 1 + ny) % ny, k)]) / (2.0 * del_h);
                double pu, pd;
                if (zbc == CMSL_DIRICHLET) {
                    pu = k == nz - 1 ? 0.0 : phi[id(i, j, k + 1)];
                    pd = k == 0 ? 0.0 : phi[id(i, j, k - 1)];
                } else {
                    const int up = k == 0 ? 1 : (k == nz - 1 ? nz - 2 : k + 1);
                    const int dn = k == 0 ? 1 : (k == nz - 1 ? nz - 2 : k - 1);
                    pu = phi[id(i, j, up)];
                    pd = phi[id(i, j, dn)];
                }
                Ez[c] = -(pu - pd) / (2.0 * del_h);
            }
    return CMSL_OK;
}

cmsl_status cmsl_phase_pool_read(const char *path, double *afe, double *fe, double *de, int max_entries, int *n)
{
    if (!path || !n || max_entries < 0) return io_fail(CMSL_ERR_ARG, "bad arguments");
    FILE *f = std::fopen(path, "r");
    if (!f) return io_fail(CMSL_ERR_IO, std::string("cannot open phase pool ") + path);
    int k = 0;
    while (k < max_entries) {
        double a, b, c;
        if (std::fscanf(f, "%lf %lf %lf", &a, &b, &c) != 3) break;
        if (c > 50.0) continue;
        if (afe) afe[k] = a / 100.0;
        if (fe) fe[k] = b / 100.0;
        if (de) de[k] = c / 100.0;
        ++k;
    }
    std::fclose(f);
    *n = k;
    return CMSL_OK;
}

}  // extern "C"

namespace {

// main.cu:200-213
double p0_of(double alpha, double beta, double g, double gamma1, int transition_type)
{
    if (transition_type == 2) return 2.0 * std::sqrt((g - alpha) / beta);
    double disc = beta * beta - 4.0 * gamma1 * (alpha - g);
    if (disc < 0.0 && disc > -1e-14) disc = 0.0;
    if (disc < 0.0) return 1.0;
    const double num = 2.0 * std::fabs(beta) + 2.0 * std::sqrt(disc);
    if (gamma1 == 0.0) return 1.0;
    return std::sqrt(num / gamma1);
}

cmsl_material nd_of(const cmsl_raw_material &r, double alpha_ref, double P0_ref)
{
    const double t0 = 3.0e-09, l0 = 1.0e-09;   // global.cu:30-31
    cmsl_material m{};
    m.alpha = r.alpha / alpha_ref;
    if (!(r.beta == 0.0 && r.gamma1 == 0.0 && r.g == 0.0)) {
        m.beta = (r.beta * P0_ref * P0_ref) / (8.0 * alpha_ref);
        m.gamma = (r.gamma1 * std::pow(P0_ref, 4.0)) / (48.0 * alpha_ref);
        m.g = r.g / alpha_ref;
    }
    m.a0 = (4.0 * r.a0) / alpha_ref;
    m.L = 0.25 * r.L * alpha_ref * t0;
    m.kappa = r.kappa / (alpha_ref * l0 * l0);
    m.eps_r = r.eps_r;
    return m;
}

}  // namespace

extern "C" {

cmsl_status cmsl_nondim(const cmsl_raw_material raw[3], int ref_type, double Eap, double delEap, cmsl_material nd[3],
                        cmsl_scales *sc)
{
    if (!raw || !nd || !sc) return io_fail(CMSL_ERR_ARG, "NULL argument");
    const cmsl_raw_material &R = raw[(ref_type >= 0 && ref_type <= 2) ? ref_type : 1];  // main.cu:185-198
    cmsl_scales s{};
    s.alpha_ref = std::fabs(R.alpha);                                                     // main.cu:215-230
    if (R.beta == 0.0 && R.gamma1 == 0.0 && R.g == 0.0) {
        s.P0_ref = 1.0;
    } else {
        s.P0_ref = p0_of(R.alpha, R.beta, R.g, R.gamma1, R.transition_type);
        if (!std::isfinite(s.P0_ref) || s.P0_ref <= 0.0) s.P0_ref = 1.0;
    }
    s.L_ref = R.L;
    s.kappa_ref = R.kappa;
    s.f0_ref = 0.25 * s.alpha_ref * s.P0_ref * s.P0_ref;                                 // main.cu:273-274
    s.E0_ref = s.f0_ref / s.P0_ref;
    for (int q = 0; q < 3; ++q) nd[q] = nd_of(raw[q], s.alpha_ref, s.P0_ref);
    s.eps_0_nd = 4.0 / (8.854e-12 * std::fabs(R.alpha));                                 // main.cu:343-344
    s.maxEz = Eap / s.E0_ref;                                                             // main.cu:347-348
    s.delEz = delEap / s.E0_ref;
    *sc = s;
    return CMSL_OK;
}

cmsl_status cmsl_assign_materials(int nx, int ny, int nz, int ng, const int32_t *omega, const double *centz,
                                  int n_layers, const int *counts, const double *afe, const double *fe,
                                  const double *de, int32_t *grain_mat)
{
    if (!omega || !centz || !counts || !afe || !fe || !de || !grain_mat || ng < 1 || n_layers < 1)
        return io_fail(CMSL_ERR_ARG, "bad arguments");
    std::vector<int> zs(n_layers), ze(n_layers), layer(ng, -1), vox(ng, 0), lst;
    zs[0] = 0;
    ze[0] = counts[0];
    for (int L = 1; L < n_layers; ++L) { zs[L] = ze[L - 1]; ze[L] = zs[L] + counts[L]; }
    for (int g = 0; g < ng; ++g) {                                   // init_conf.cu:132-149
        for (int L = 0; L < n_layers; ++L)
            if (centz[g] >= zs[L] && centz[g] < ze[L]) { layer[g] = L; break; }
        if (layer[g] < 0)
            return io_fail(CMSL_ERR_IO, "grain " + std::to_string(g) + " is in no layer");
    }
    const long long N = (long long)nx * ny * nz;
    for (long long i = 0; i < N; ++i)
        if (omega[i] >= 0 && omega[i] < ng) vox[omega[i]]++;
    for (int g = 0; g < ng; ++g) grain_mat[g] = -1;
    std::srand(123456);                                              // init_conf.cu:169
    for (int L = 0; L < n_layers; ++L) {
        double A = afe[L], F = fe[L], D = de[L];
        double sum = A + F + D;
        if (sum <= 0) { A = 0; F = 0; D = 1; sum = 1; }
        A /= sum; F /= sum; D /= sum;
        lst.clear();
        for (int g = 0; g < ng; ++g)
            if (layer[g] == L) lst.push_back(g);
        const int cnt = (int)lst.size();
        long long tot = 0;
        for (int g : lst) tot += vox[g];
        if (tot <= 0) return io_fail(CMSL_ERR_IO, "layer " + std::to_string(L) + " has no voxels");
        const long long tA = std::llround(A * tot), tD = std::llround(D * tot);
        for (int i = 0; i < cnt; ++i) {                              // Fisher-Yates with rand()
            const int r = i + std::rand() % (cnt - i);
            std::swap(lst[i], lst[r]);
        }
        long long acc = 0;
        int p = 0;
        while (p < cnt && acc < tD) { const int g = lst[p++]; grain_mat[g] = CMSL_DE; acc += vox[g]; }
        acc = 0;
        while (p < cnt && acc < tA) { const int g = lst[p++]; grain_mat[g] = CMSL_AFE; acc += vox[g]; }
        while (p < cnt) { const int g = lst[p++]; if (grain_mat[g] == -1) grain_mat[g] = CMSL_FE; }
    }
    return CMSL_OK;
}

cmsl_status cmsl_interface_flags(int nx, int ny, int nz, const int32_t *omega, const int32_t *gm, int32_t *flag)
{
    if (!omega || !gm || !flag) return io_fail(CMSL_ERR_ARG, "NULL argument");
    const long long N = (long long)nx * ny * nz, plane = (long long)nx * ny;
    for (long long id = 0; id < N; ++id) {
        const int g = omega[id];
        if (g < 0 || gm[g] != CMSL_FE) { flag[id] = 0; continue; }
        const long long k = id / plane;
        if (k == 0 || k == nz - 1) { flag[id] = 0; continue; }
        const int gu = omega[id + plane], gd = omega[id - plane];
        const int mu = gu >= 0 ? gm[gu] : -1, md = gd >= 0 ? gm[gd] : -1;
        flag[id] = (mu != CMSL_FE || md != CMSL_FE);
    }
    return CMSL_OK;
}

cmsl_status cmsl_evolve_schedule(double maxEz, double delEz, int num_steps, int n_periods, int single, double E0_ref,
                                 int max_steps, double *Ez, int32_t *row, int *n_steps, double *row_E,
                                 int32_t *row_count, int *n_rows)
{
    if (!(delEz > 0.0) || num_steps < 1 || n_periods < 1 || !n_steps || !n_rows || max_steps < 1)
        return io_fail(CMSL_ERR_ARG, "bad schedule arguments");
    double E = 0.0, inc = delEz;                       // evolve.cu:123, main.cu:66-70
    int peloop = 0, since = 0, s = 0, r = 0;
    long long count = 0;
    const double win = 0.2e8 / E0_ref;                 // evolve.cu:243
    while (peloop < n_periods + 1) {
        if (s >= max_steps) return io_fail(CMSL_ERR_ARG, "schedule longer than max_steps");
        if (Ez) Ez[s] = E;
        if (row) row[s] = -1;
        ++since;
        ++count;
        const int relax = (single && std::fabs(E) < win) ? num_steps * 10 : num_steps;
        if (since >= relax) {
            if (E > maxEz) { inc = -delEz; ++peloop; }  // evolve.cu:362-369
            if (E < -maxEz) inc = delEz;
            if (peloop > 0) {                          // evolve.cu:390-403
                if (row) row[s] = r;
                if (row_E) row_E[r] = E;
                if (row_count) row_count[r] = (int32_t)count;
                ++r;
            }
            E += inc;                                  // evolve.cu:407
            since = 0;
        }
        ++s;
    }
    *n_steps = s;
    *n_rows = r;
    return CMSL_OK;
}

}  // extern "C"

// The seed points, centres and orientations of cmsl_voronoi_columnar (shared
// with the device generator, grains.cu).
void cmsl_internal_voronoi_seeds(int nx, int ny, int nz, int ng, uint64_t seed, double *sx, double *sy,
                                 double *cent, double *euler)
{
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    auto next = [&]() {   // SplitMix64
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto uni = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
    for (int g = 0; g < ng; ++g) { sx[g] = uni() * nx; sy[g] = uni() * ny; }
    for (int g = 0; g < ng; ++g) {
        if (cent) { cent[3 * g] = sx[g]; cent[3 * g + 1] = sy[g]; cent[3 * g + 2] = 0.5 * (nz - 1); }
        if (euler) {
            const double phi = 2.0 * M_PI * uni();
            const double c = (0.3 + 0.7 * uni()) * (uni() < 0.5 ? -1.0 : 1.0);
            const double psi = 2.0 * M_PI * uni();
            euler[3 * g] = phi; euler[3 * g + 1] = std::acos(c); euler[3 * g + 2] = psi;
        }
    }
}

extern "C" {

cmsl_status cmsl_voronoi_columnar(int nx, int ny, int nz, int ng, uint64_t seed, int32_t *omega, double *cent,
                                  double *euler)
{
    if (nx < 1 || ny < 1 || nz < 1 || ng < 1 || !omega) return io_fail(CMSL_ERR_ARG, "bad arguments");
    std::vector<double> sx(ng), sy(ng);
    cmsl_internal_voronoi_seeds(nx, ny, nz, ng, seed, sx.data(), sy.data(), cent, euler);
    const long long plane = (long long)nx * ny;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double x = i + 0.5, y = j + 0.5;
            int best = 0;
            double bd = 1e300;
            for (int g = 0; g < ng; ++g) {
                double dx = std::fabs(x - sx[g]), dy = std::fabs(y - sy[g]);
                dx = std::fmin(dx, nx - dx);
                dy = std::fmin(dy, ny - dy);
                const double d2 = dx * dx + dy * dy;
                if (d2 < bd) { bd = d2; best = g; }
            }
            for (int k = 0; k < nz; ++k) omega[i + (long long)nx * j + plane * k] = best;
        }
    return CMSL_OK;
}

}  // extern "C"
