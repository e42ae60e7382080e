// noalloc.cu -- the depolarisation solve for callers that cannot allocate
// device memory.
//
// Some hosts of this library cannot call cudaMalloc: code running inside an
// application that owns every device allocation through its own pool
// allocator, plugins that are handed pre-sized device buffers, or a
// process whose memory budget is fixed before the solver is loaded.
// cmsl_depol_solve_noalloc serves them: it runs the same FP64 Jacobi-PCG as
// cmsl_film_depol (the same kernels), but every piece of work memory -- the
// film table, the work-item list, the cell codes, the Jacobi diagonal, the
// PCG vectors, the reduction partials and the solver state -- lives in one
// file-scope device array, g_noalloc_scratch, of fixed size.  The caller
// passes the inputs (materials, Pm) and the output (phi) as device pointers.
//
// The array exists once per device for as long as the library is loaded.
// Its device address is looked up once per device, with that device current,
// on the first call made on that device: make that first call before any
// stream capture.  The looked-up address is kept for the life of the process
// and does not survive cudaDeviceReset (or any other destruction of the
// device's primary context): after one, no further call may be made.  Every
// call shares the array, so calls whose GPU work overlaps (different streams,
// different host threads on one device) race; serialise them.  Each call
// re-initialises every part of the array it reads.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "cmsl.h"
#include "kernels.cuh"

using namespace cmsl;

void cmsl_internal_set_error(const char *msg);   // engine.cu: text for cmsl_last_error()

namespace {

constexpr long long NA_MAX_CELLS = 131072;       // e.g. 64 x 64 x 32
constexpr int NA_MAX_ITEMS = 8192;

constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t NA_OFF_FILM = 0;
constexpr size_t NA_OFF_SOLVE = NA_OFF_FILM + na_align(sizeof(FilmDev));
constexpr size_t NA_OFF_CTL = NA_OFF_SOLVE + na_align(sizeof(SolveDev));
constexpr size_t NA_OFF_COUNTER = NA_OFF_CTL + na_align(sizeof(Ctl));
constexpr size_t NA_OFF_ITEMS = NA_OFF_COUNTER + 256;
constexpr size_t NA_OFF_PART = NA_OFF_ITEMS + na_align(sizeof(int4) * NA_MAX_ITEMS);
constexpr size_t NA_OFF_CODE = NA_OFF_PART + na_align(sizeof(double) * NPART * NA_MAX_ITEMS);
constexpr size_t NA_OFF_VEC = NA_OFF_CODE + na_align(sizeof(uint32_t) * NA_MAX_CELLS);
constexpr size_t NA_VEC = na_align(sizeof(double) * NA_MAX_CELLS);
constexpr size_t NA_BYTES = NA_OFF_VEC + 5 * NA_VEC;   // dinv, r, q, p0, p1

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {

std::mutex g_na_mutex;
void *g_na_base[256] = {};

cmsl_status na_fail(cmsl_status s, const char *msg, cudaError_t e = cudaSuccess)
{
    std::string m = msg;
    if (e != cudaSuccess) {
        m += ": ";
        m += cudaGetErrorString(e);
    }
    cmsl_internal_set_error(m.c_str());
    return s;
}

// Device address of the scratch array on the current device (looked up once).
cmsl_status na_base(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(CMSL_ERR_CUDA, "cudaGetDevice failed", e);
    if (dev < 0 || dev >= 256) return na_fail(CMSL_ERR_CUDA, "device index out of range");
    std::lock_guard<std::mutex> lk(g_na_mutex);
    if (!g_na_base[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return na_fail(CMSL_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch) failed", e);
        g_na_base[dev] = p;
    }
    *out = g_na_base[dev];
    return CMSL_OK;
}

double na_harm(double a, double b)   // depol_varEPS.cu:10-15
{
    const double eps = 1e-20;
    double denom = a + b;
    if (denom < eps) denom = eps;
    return (2.0 * a * b) / denom;
}

// code = material << 24 (grain id and interface bit are not used by the solve)
__global__ void k_na_codes(const int32_t *mat, uint32_t *code, long long n, int *bad)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int m = mat[i];
        if (m < 0 || m > 2) { atomicExch(bad, 1); code[i] = 0u; }
        else code[i] = (uint32_t)m << 24;
    }
}

}  // namespace

extern "C" cmsl_status cmsl_depol_solve_noalloc(int nx, int ny, int nz, double del_h, int zbc, double eps_0_nd,
                                                const int32_t *material_dev, const double eps_r[3],
                                                const double *Pmx_dev, const double *Pmy_dev,
                                                const double *Pmz_dev, double *phi_dev, double tol_abs,
                                                double tol_rel, int max_iter, int pcg_crit, void *stream,
                                                int32_t *iters_out, int32_t *status_out)
{
    if (nx < 1 || ny < 1 || nz < 3) return na_fail(CMSL_ERR_ARG, "grid: need nx, ny >= 1 and nz >= 3");
    // work items pack z0 and z1 into 16-bit fields (the film API's limit too)
    if (nx > 32767 || ny > 32767 || nz > 32767) return na_fail(CMSL_ERR_ARG, "grid: each side must be <= 32767");
    const long long N = (long long)nx * ny * nz;
    if (N > NA_MAX_CELLS) return na_fail(CMSL_ERR_ARG, "grid larger than the 131072-cell scratch of the no-alloc solve");
    if (!material_dev || !eps_r || !Pmx_dev || !Pmy_dev || !Pmz_dev || !phi_dev)
        return na_fail(CMSL_ERR_ARG, "NULL argument");
    if (zbc != CMSL_DIRICHLET && zbc != CMSL_NEUMANN) return na_fail(CMSL_ERR_ARG, "zbc");
    if (!(del_h > 0.0) || max_iter < 0) return na_fail(CMSL_ERR_ARG, "del_h must be > 0, max_iter >= 0");

    // work items: the same tiling as cmsl_film_create
    std::vector<int4> items;
    {
        const long long xy = (long long)((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
        const long long target = 8LL * 152;
        const long long chunks = (target + xy - 1) / xy;
        int zc = (int)std::max<long long>(1, (nz + chunks - 1) / chunks);
        zc = std::min(std::max(zc, std::min(nz, 4)), nz);
        const long long n_items = xy * ((nz + zc - 1) / zc);
        if (n_items > NA_MAX_ITEMS) return na_fail(CMSL_ERR_ARG, "grid shape needs more than 8192 work items");
        for (int y0 = 0; y0 < ny; y0 += TY)
            for (int x0 = 0; x0 < nx; x0 += TX)
                for (int z0 = 0; z0 < nz; z0 += zc)
                    items.push_back(make_int4(0, x0, y0, z0 | (std::min(nz, z0 + zc) << 16)));
    }
    FilmDev fd{};
    fd.nx = nx; fd.ny = ny; fd.nz = nz; fd.zbc = zbc;
    fd.off = 0; fd.g_off = 0; fd.item_begin = 0; fd.item_end = (int)items.size();
    fd.dep_flag = 1;
    fd.ref_id = nx / 2 + nx * (ny / 2 + (nz / 2) * ny);
    fd.crit = pcg_crit;
    fd.max_iter = max_iter;
    fd.h = del_h; fd.eps0nd = eps_0_nd;
    fd.two_h = 2.0 * del_h; fd.h2 = del_h * del_h; fd.inv_h2 = 1.0 / (del_h * del_h);
    fd.inv_2h = 1.0 / (2.0 * del_h);
    fd.tol_abs2 = tol_abs * tol_abs;
    fd.tol_rel2 = tol_rel * tol_rel;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            fd.epsf[a * 3 + b] = na_harm(eps_r[a], eps_r[b]);
            fd.epsf32[a * 3 + b] = (float)fd.epsf[a * 3 + b];
        }

    void *base = nullptr;
    cmsl_status st = na_base(&base);
    if (st != CMSL_OK) return st;
    unsigned char *B = (unsigned char *)base;
    cudaStream_t s = (cudaStream_t)stream;
    FilmDev *d_film = (FilmDev *)(B + NA_OFF_FILM);
    SolveDev *d_solve = (SolveDev *)(B + NA_OFF_SOLVE);
    Ctl *d_ctl = (Ctl *)(B + NA_OFF_CTL);
    unsigned int *d_counter = (unsigned int *)(B + NA_OFF_COUNTER);
    int4 *d_items = (int4 *)(B + NA_OFF_ITEMS);
    double *d_part = (double *)(B + NA_OFF_PART);
    uint32_t *d_code = (uint32_t *)(B + NA_OFF_CODE);
    double *v[5];
    for (int q = 0; q < 5; ++q) v[q] = (double *)(B + NA_OFF_VEC + q * NA_VEC);

    // clear what must start at zero; upload the tables
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_film, &fd, sizeof(FilmDev), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_solve, 0, sizeof(SolveDev), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_ctl, 0, sizeof(Ctl), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_counter, 0, 256, s)) != cudaSuccess)
        return na_fail(CMSL_ERR_CUDA, "scratch initialisation failed", e);
    int *d_bad = (int *)(d_counter + 8);
    const int nit = (int)items.size();
    k_na_codes<<<std::max(1, (int)std::min<long long>((N + 255) / 256, 1024)), 256, 0, s>>>(material_dev, d_code, N, d_bad);

    Dev d{};
    d.films = d_film; d.items = d_items; d.n_films = 1; d.n_items = nit;
    d.code = d_code; d.ncells = N; d.phi[0] = phi_dev;
    d.partial = d_part; d.counter = d_counter; d.solve = d_solve; d.ctl = d_ctl;
    Fields<double> F{};
    for (int c = 0; c < 2; ++c) {
        F.P[c][0] = (double *)Pmx_dev; F.P[c][1] = (double *)Pmy_dev; F.P[c][2] = (double *)Pmz_dev;
    }
    F.dinv = v[0]; F.r = v[1]; F.q = v[2]; F.p[0] = v[3]; F.p[1] = v[4];
    k_dinv<double><<<nit, NT, 0, s>>>(d, v[0]);
    k_rhs<double, Exact><<<nit, NT, 0, s>>>(d, F);
    if ((e = cudaGetLastError()) != cudaSuccess) return na_fail(CMSL_ERR_CUDA, "launch failed", e);
    SolveDev S{};
    int bad = 0;
    for (int guard = 0;; ++guard) {
        // the material check is read on the caller's stream with the first state read
        if (guard == 0 && (e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return na_fail(CMSL_ERR_CUDA, "reading the material check failed", e);
        if ((e = cudaMemcpyAsync(&S, d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return na_fail(CMSL_ERR_CUDA, "reading the solver state failed", e);
        if (guard == 0 && bad) return na_fail(CMSL_ERR_ARG, "material ids must be 0 (AFE), 1 (FE) or 2 (DE)");
        if (!S.active) break;
        if (guard > max_iter + 1) return na_fail(CMSL_ERR_STATE, "PCG loop did not stop");
        k_spmv<double, Exact><<<nit, NT, 0, s>>>(d, F);
        k_update<double, Exact, false><<<nit, NT, 0, s>>>(d, F);
        if ((e = cudaGetLastError()) != cudaSuccess) return na_fail(CMSL_ERR_CUDA, "launch failed", e);
    }
    if (iters_out) *iters_out = S.iters;
    if (status_out) *status_out = S.status;
    return S.status == 0 ? CMSL_OK : na_fail(CMSL_ERR_PCG, "PCG breakdown or invalid residual");
}
