// adjoint.cu -- gradient of a P-E loop misfit by a hand-written adjoint of the
// TDGL step and the depolarisation solve, with checkpointing.
//
// Forward model of step n (FP64 film, Dirichlet z boundary):
//   P^{n+1} = T(P^n, phi^n; theta)        (k_tdgl: kernels_evol.cu:47-231)
//   A phi^{n+1} = b(P^{n+1})              (Depol_field: depol_varEPS.cu:332-595)
//   row r = mean(Pm_z^{n+1}) when step n writes row r
//   loss  = (1/R) sum_r (row_r - target_r)^2
// phi enters T linearly (through E = -grad phi), so the backward pass only
// needs P^n: the forward stores P and phi every `checkpoint_every` steps and
// each segment is recomputed, storing P^n for its steps, before it is
// traversed backwards:
//   mu      = A^{-1} g~,  g~ = lambda_phi^{n+1} with the Dirichlet rows zeroed
//             (b is zero there, and the interior block of A is symmetric, so
//             the forward PCG solves the adjoint system)
//   lam^{n+1} += (db/dP)^T mu + d loss / d P^{n+1}
//   lam^n    = (dT/dP)^T lam^{n+1};  lambda_phi^n = (dT/dphi)^T lam^{n+1}
//   d loss / d theta += (dT/dtheta)^T lam^{n+1}
// where theta are the TDGL coefficients of each (material, interface) set:
// 2(alpha +- g), 4 beta, 12 beta, 6 gamma, kappa dt/h^2; the host maps them
// to the non-dimensional (alpha, beta, gamma, g, kappa) of each material.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "engine.h"

using namespace cmsl;
using namespace cmsl_eng;

namespace {

constexpr int NTH = 36;   // theta partials per item: 6 sets x (ag, ags, b4, b12, g6, A)

struct Lam {
    double *q[6];
};
struct CLam {
    const double *q[6];
};

// r = g~ - A mu, z = D^-1 r, partial (r.z, r.r, b.b); the last block starts
// every film's solve (stop test of the film).
__global__ void __launch_bounds__(NT) k_adj_rhs(Dev d, Fields<double> F, const double *g)
{
    __shared__ double sRed[NT / 32][3];
    __shared__ double sTot[3];
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom gm = make_geom(f, it.y, it.z);
    const long long off = f->off;
    const uint32_t *code = d.code + off;
    const double *x = phi_sel(d, d.solve[it.x].phi_cur) + off;
    const double *gg = g + off, *dinv = F.dinv + off;
    double *r = F.r + off;
    double acc[3] = {0.0, 0.0, 0.0};
    if (f->dep_flag && gm.valid) {
        const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
        const int i = gm.x0 + lx, j = gm.y0 + ly, nx = gm.nx, ny = gm.ny;
        for (int k = z0; k < z1; ++k) {
            const long long o = gm.own_pl + (long long)k * gm.plane;
            double b, ax;
            if (identity_row(f, k, gm.own_pl)) {
                b = 0.0;
                ax = x[o];
            } else {
                b = gg[o];
                const int ip = (i + 1) % nx, im = (i - 1 + nx) % nx, jp = (j + 1) % ny, jm = (j - 1 + ny) % ny;
                auto id = [&](int a, int bb, int c) { return a + (long long)nx * (bb + (long long)ny * c); };
                const long long ie = id(ip, j, k), iw = id(im, j, k), in = id(i, jp, k), is = id(i, jm, k);
                const long long iu = id(i, j, k + 1), idn = id(i, j, k - 1);
                ax = op_row<double, Fast>(f, code_mat(code[o]), code_mat(code[ie]), code_mat(code[iw]),
                                          code_mat(code[in]), code_mat(code[is]), code_mat(code[iu]),
                                          code_mat(code[idn]), x[o], x[ie], x[iw], x[in], x[is], x[iu], x[idn]);
            }
            const double rv = b - ax;
            r[o] = rv;
            acc[0] += rv * (rv * dinv[o]);
            acc[1] += rv * rv;
            acc[2] += b * b;
        }
    }
    double tot[3];
    block_sum<3, double>(acc, sRed, tot);
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) d.partial[(long long)blockIdx.x * NPART + q] = tot[q];
    if (!ticket_last(d.counter)) return;
    start_solves(d, sRed, sTot);
}

// lam_m += (db/dPm)^T mu (b = -eps_0_nd div(Pm) / (2h) on interior rows,
// depol_varEPS.cu:279-329, 401-424) and lam_mz += seed (the loss term of the
// row this step wrote).
__global__ void __launch_bounds__(NT) k_adj_div(Dev d, Lam L, const double *mu, double seed)
{
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom gm = make_geom(f, it.y, it.z);
    if (!gm.valid) return;
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    const int i = gm.x0 + lx, j = gm.y0 + ly, nx = gm.nx, ny = gm.ny, nz = gm.nz;
    const long long off = f->off;
    const double s = f->dep_flag ? f->eps0nd / f->two_h : 0.0;
    const double *m = mu + off;
    auto id = [&](int a, int b, int c) { return a + (long long)nx * (b + (long long)ny * c); };
    for (int k = z0; k < z1; ++k) {
        const long long o = gm.own_pl + (long long)k * gm.plane;
        if (s != 0.0) {
            const double dx = m[id((i + 1) % nx, j, k)] - m[id((i - 1 + nx) % nx, j, k)];
            const double dy = m[id(i, (j + 1) % ny, k)] - m[id(i, (j - 1 + ny) % ny, k)];
            const double up = k + 1 < nz ? m[id(i, j, k + 1)] : 0.0, dn = k > 0 ? m[id(i, j, k - 1)] : 0.0;
            L.q[0][off + o] += s * dx;
            L.q[1][off + o] += s * dy;
            L.q[2][off + o] += s * (up - dn) + seed;
        } else {
            L.q[2][off + o] += seed;
        }
    }
}

// The adjoint of one TDGL step at P^n (kernels_evol.cu:47-231 transposed):
// lam_out = (dT/dP)^T lam_in, lam_phi = (dT/dphi)^T lam_in, and the theta
// partials of the item added to tacc[item][36].
__global__ void __launch_bounds__(NT) k_adj_tdgl(Dev d, Fields<double> F, CLam P, CLam Lin, Lam Lout,
                                                  double *lam_phi, double *tacc)
{
    __shared__ double sAcc[NT / 32][NTH];
    const int4 it = d.items[blockIdx.x];
    const FilmDev *f = d.films + it.x;
    const int z0 = it.w & 0xffff, z1 = it.w >> 16;
    const Geom gm = make_geom(f, it.y, it.z);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = lane; q < NTH; q += 32) sAcc[warp][q] = 0.0;
    const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
    const int i = gm.x0 + lx, j = gm.y0 + ly, nx = gm.nx, ny = gm.ny, nz = gm.nz;
    const long long off = f->off;
    const uint32_t *code = d.code + off;
    const bool dep = f->dep_flag != 0;
    const double inv2h = 1.0 / f->two_h;
    auto id = [&](int a, int b, int c) { return off + a + (long long)nx * (b + (long long)ny * c); };
    auto coef = [&](long long gc) -> const Coef<double> & {
        const uint32_t c = d.code[gc];
        return f->coef[code_mat(c) * 2 + code_iface(c)];
    };
    for (int k = z0; k < z1; ++k) {
        double th[6] = {0, 0, 0, 0, 0, 0};
        int set = -1;
        if (gm.valid) {
            const long long c = id(i, j, k);
            const uint32_t cc = code[c - off];
            set = code_mat(cc) * 2 + code_iface(cc);
            const Coef<double> &K = f->coef[set];
            const double *t = F.TR + 9LL * (f->g_off + code_gid(cc));
            double lam[6], p[6];
            for (int q = 0; q < 6; ++q) { lam[q] = Lin.q[q][c]; p[q] = P.q[q][c]; }
            // neighbours: x/y periodic; z clamped to the cell itself at the
            // first and last planes (kernels_evol.cu:71-83), transposed
            const long long ce = id((i + 1) % nx, j, k), cw = id((i - 1 + nx) % nx, j, k);
            const long long cn = id(i, (j + 1) % ny, k), cs = id(i, (j - 1 + ny) % ny, k);
            const double Ae = coef(ce).A, Aw = coef(cw).A, An = coef(cn).A, As = coef(cs).A;
            double Au = 0.0, Ad = 0.0;
            long long cu = c, cd = c;
            if (k + 1 < nz) { cu = id(i, j, k + 1); Au = coef(cu).A; }   // cell above uses c as its "down"
            if (k > 0) { cd = id(i, j, k - 1); Ad = coef(cd).A; }        // cell below uses c as its "up"
            double self = 0.0;
            if (k == nz - 1) self += K.A;
            if (k == 0) self += K.A;
            double out[6];
            for (int q = 0; q < 6; ++q) {
                double tl = Ae * Lin.q[q][ce] + Aw * Lin.q[q][cw] + An * Lin.q[q][cn] + As * Lin.q[q][cs];
                if (k + 1 < nz) tl += Au * Lin.q[q][cu];
                if (k > 0) tl += Ad * Lin.q[q][cd];
                tl += self * lam[q];
                out[q] = K.relax * lam[q] + tl;
            }
            // Landau term: (TR^T H TR)^T v = TR^T H (TR v), v = LdT lam
            double v[6];
            for (int q = 0; q < 6; ++q) v[q] = K.LdT * lam[q];
            const double vmx = t[0] * v[0] + t[1] * v[1] + t[2] * v[2];
            const double vmy = t[3] * v[0] + t[4] * v[1] + t[5] * v[2];
            const double vmz = t[6] * v[0] + t[7] * v[1] + t[8] * v[2];
            const double vsx = t[0] * v[3] + t[1] * v[4] + t[2] * v[5];
            const double vsy = t[3] * v[3] + t[4] * v[4] + t[5] * v[5];
            const double vsz = t[6] * v[3] + t[7] * v[4] + t[8] * v[5];
            const double mz = t[6] * p[0] + t[7] * p[1] + t[8] * p[2];
            const double sz = t[6] * p[3] + t[7] * p[4] + t[8] * p[5];
            const double m2 = mz * mz, s2 = sz * sz;
            const double Hmm = K.ag + 3.0 * K.b4 * m2 + K.b12 * s2 + K.g6 * (5.0 * m2 * m2 + 30.0 * m2 * s2 + 5.0 * s2 * s2);
            const double Hss = K.ags + 3.0 * K.b4 * s2 + K.b12 * m2 + K.g6 * (5.0 * s2 * s2 + 30.0 * s2 * m2 + 5.0 * m2 * m2);
            const double Hms = 2.0 * K.b12 * mz * sz + K.g6 * (20.0 * m2 * mz * sz + 20.0 * mz * s2 * sz);
            const double hmx = K.a02 * vmx, hmy = K.a02 * vmy, hsx = K.a02 * vsx, hsy = K.a02 * vsy;
            const double hmz = Hmm * vmz + Hms * vsz, hsz = Hms * vmz + Hss * vsz;
            out[0] -= t[0] * hmx + t[3] * hmy + t[6] * hmz;
            out[1] -= t[1] * hmx + t[4] * hmy + t[7] * hmz;
            out[2] -= t[2] * hmx + t[5] * hmy + t[8] * hmz;
            out[3] -= t[0] * hsx + t[3] * hsy + t[6] * hsz;
            out[4] -= t[1] * hsx + t[4] * hsy + t[7] * hsz;
            out[5] -= t[2] * hsx + t[5] * hsy + t[8] * hsz;
            for (int q = 0; q < 6; ++q) Lout.q[q][c] = out[q];
            // E = -grad(phi^n) enters as +LdT * (phi_+ - phi_-)/(2h) in dfdPm
            if (dep) {
                auto w = [&](int q, long long gc) { return coef(gc).LdT * Lin.q[q][gc]; };
                double lp = (w(0, ce) - w(0, cw)) + (w(1, cn) - w(1, cs));
                if (k + 1 < nz) lp += w(2, cu);
                if (k > 0) lp -= w(2, cd);
                lam_phi[c] = lp * inv2h;
            }
            // theta partials of this cell's set
            const double m3 = m2 * mz, s3 = s2 * sz;
            th[0] = -vmz * mz;
            th[1] = -vsz * sz;
            th[2] = -(vmz * m3 + vsz * s3);
            th[3] = -(vmz * mz * s2 + vsz * sz * m2);
            th[4] = -(vmz * (m3 * m2 + 10.0 * m3 * s2 + 5.0 * mz * s2 * s2) +
                      vsz * (s3 * s2 + 10.0 * s3 * m2 + 5.0 * sz * m2 * m2));
            double lap_minus = 0.0;
            for (int q = 0; q < 6; ++q) {
                const double pu = k + 1 < nz ? P.q[q][cu] : p[q], pd = k > 0 ? P.q[q][cd] : p[q];
                const double sum = P.q[q][ce] + P.q[q][cw] + P.q[q][cn] + P.q[q][cs] + pu + pd;
                lap_minus += lam[q] * (sum - 6.0 * p[q]);
            }
            th[5] = lap_minus;
        }
        // warp reduction per set present in the warp (fixed order)
        const unsigned present = __ballot_sync(0xffffffffu, set >= 0);
        if (present) {
            for (int s = 0; s < 6; ++s) {
                const unsigned has = __ballot_sync(0xffffffffu, set == s);
                if (!has) continue;
                for (int q = 0; q < 6; ++q) {
                    const double v = warp_sum(set == s ? th[q] : 0.0);
                    if (lane == 0) sAcc[warp][s * 6 + q] += v;
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < NTH) {
        double t = 0.0;
        for (int w = 0; w < NT / 32; ++w) t += sAcc[w][threadIdx.x];
        tacc[(long long)blockIdx.x * NTH + threadIdx.x] += t;
    }
}

struct AdjWork {
    std::vector<void *> mem;
    ~AdjWork()
    {
        for (void *p : mem) cudaFree(p);
    }
    cmsl_status alloc(void **p, size_t n)
    {
        cudaError_t e = cudaMalloc(p, n ? n : 16);
        if (e != cudaSuccess) {
            *p = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? CMSL_ERR_NOMEM : CMSL_ERR_CUDA, "adjoint: cudaMalloc(%zu): %s",
                        n, cudaGetErrorString(e));
        }
        mem.push_back(*p);
        e = cudaMemset(*p, 0, n ? n : 16);
        if (e != cudaSuccess) return fail(CMSL_ERR_CUDA, "adjoint: cudaMemset: %s", cudaGetErrorString(e));
        return CMSL_OK;
    }
};

__global__ void k_set_stop(Ctl *ctl, int stop) { ctl->stop = stop; }

// Enqueues steps [0, len) of Ez_seg from the film's current state on st
// (forward graph, one launch per step, its step loop stopped after that
// step).  store: P^n before each step, as [len][6][N].  cur: the film's
// current P set, advanced per step.
cmsl_status forward_segment(Engine *e, cudaStream_t st, const double *Ez_seg, const int32_t *rows_seg, int len,
                            double *store, int &cur)
{
    TRY(ensure_schedule(e, len, 0));
    std::vector<int> rows((size_t)len, -1);
    if (rows_seg)
        for (int s = 0; s < len; ++s) rows[s] = rows_seg[s] < 0 ? -1 : rows_seg[s];
    CK(cudaMemcpy(e->d_wave, Ez_seg, sizeof(double) * len, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_rows, rows.data(), sizeof(int) * len, cudaMemcpyHostToDevice));
    CK(cudaMemset(&e->d_ctl->run_step, 0, sizeof(int)));
    if (!e->graph_valid) TRY(build_graph(e));
    const size_t N = (size_t)e->fh[0].N;
    for (int s = 0; s < len; ++s) {
        if (store)
            for (int q = 0; q < 6; ++q)
                CK(cudaMemcpyAsync(store + ((size_t)s * 6 + q) * N, e->d_P[cur][q], sizeof(double) * N,
                                   cudaMemcpyDeviceToDevice, st));
        k_set_stop<<<1, 1, 0, st>>>(e->d_ctl, s + 1);
        CK(cudaGraphLaunch(e->exec, st));
        cur ^= 1;
    }
    return CMSL_OK;
}

}  // namespace

extern "C" cmsl_status cmsl_film_loop_gradient(cmsl_film *f, int n_steps, const double *Ez, const int32_t *row,
                                               const double *target, int n_rows, int checkpoint_every,
                                               double *loss, double *grad)
{
    if (!f || !Ez || !row || !target || !loss || !grad || n_steps < 1 || n_rows < 1 || checkpoint_every < 1)
        return fail(CMSL_ERR_ARG, "loop gradient: bad arguments");
    if (f->precision != CMSL_FP64) return fail(CMSL_ERR_ARG, "loop gradient: CMSL_FP64 films only");
    if (f->fh[0].dep && f->fh[0].zbc != CMSL_DIRICHLET)
        return fail(CMSL_ERR_ARG, "loop gradient: the adjoint solve needs the Dirichlet z boundary");
    int seen = 0;
    for (int s = 0; s < n_steps; ++s) {
        if (row[s] >= n_rows) return fail(CMSL_ERR_ARG, "loop gradient: row[%d] = %d >= n_rows %d", s, row[s], n_rows);
        seen += row[s] >= 0;
    }
    if (seen == 0) return fail(CMSL_ERR_ARG, "loop gradient: no step writes a row");
    Engine *e = f;
    cudaStream_t st = nullptr;
    const size_t N = (size_t)e->fh[0].N;
    const long long off = e->fh[0].off;
    const int K = std::min(checkpoint_every, n_steps);
    const int nseg = (n_steps + K - 1) / K;
    const int nit = (int)e->items.size();
    CK(cudaDeviceSynchronize());
    Ctl c0;
    CK(cudaMemcpy(&c0, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    int cur = c0.cur;
    AdjWork W;
    double *ckpt = nullptr, *store = nullptr, *lam = nullptr, *lphi = nullptr, *mu = nullptr, *tacc = nullptr;
    SolveDev *sadj = nullptr;
    TRY(W.alloc((void **)&ckpt, sizeof(double) * 7 * N * nseg));
    TRY(W.alloc((void **)&store, sizeof(double) * 6 * N * K));
    TRY(W.alloc((void **)&lam, sizeof(double) * 12 * e->ncells));
    TRY(W.alloc((void **)&lphi, sizeof(double) * e->ncells));
    TRY(W.alloc((void **)&mu, sizeof(double) * e->ncells));
    TRY(W.alloc((void **)&tacc, sizeof(double) * NTH * nit));
    TRY(W.alloc((void **)&sadj, sizeof(SolveDev)));
    // rows of the whole loop stay in the row buffer
    TRY(ensure_schedule(e, K, n_rows));

    // ---- forward with checkpoints (P^{jK}, phi^{jK}); the last segment, the
    // first one traversed backwards, keeps its P^n and is not recomputed
    for (int j = 0; j < nseg; ++j) {
        const int s0 = j * K, len = std::min(K, n_steps - s0);
        double *ck = ckpt + (size_t)j * 7 * N;
        for (int q = 0; q < 6; ++q)
            CK(cudaMemcpyAsync(ck + q * N, e->d_P[cur][q], sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(ck + 6 * N, e->d_phi[0] + off, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        TRY(forward_segment(e, st, Ez + s0, row + s0, len, j == nseg - 1 ? store : nullptr, cur));
        CK(cudaStreamSynchronize(st));
    }
    {
        SolveDev S;
        CK(cudaMemcpy(&S, e->d_solve, sizeof(SolveDev), cudaMemcpyDeviceToHost));
        if (S.sticky != 0) return fail(CMSL_ERR_PCG, "loop gradient: PCG failure (status %d) in the forward loop", S.sticky);
    }
    std::vector<double> rows((size_t)n_rows * 11);
    CK(cudaMemcpy(rows.data(), e->d_rowbuf, sizeof(double) * 11 * n_rows, cudaMemcpyDeviceToHost));
    double L = 0.0;
    std::vector<double> dl((size_t)n_rows);
    for (int r = 0; r < n_rows; ++r) {
        const double dv = rows[(size_t)r * 11] - target[r];
        L += dv * dv;
        dl[r] = 2.0 * dv / n_rows;
    }
    *loss = L / n_rows;

    // ---- adjoint solve graph: k_adj_rhs -> WHILE { k_spmv -> k_update } on mu
    cudaGraph_t g = nullptr;
    cudaGraphExec_t gx = nullptr;
    struct GraphGuard {
        cudaGraph_t &g;
        cudaGraphExec_t &x;
        ~GraphGuard()
        {
            if (x) cudaGraphExecDestroy(x);
            if (g) cudaGraphDestroy(g);
        }
    } gguard{g, gx};
    const bool dep = e->fh[0].dep != 0;
    Fields<double> F = e->fields<double>();
    if (dep) {
        CK(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle h = 0;
        CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
        Dev da = e->dev(1, h, 0);
        da.phi[0] = mu;
        da.solve = sadj;
        const double *gp = lphi;
        void *a_rhs[] = {&da, &F, &gp};
        void *a_pcg[] = {&da, &F};
        cudaGraphNode_t n_rhs, n_loop, n_sp, n_up;
        cudaGraph_t body;
        TRY(add_kernel(g, &n_rhs, nullptr, 0, (void *)k_adj_rhs, nit, NT, a_rhs));
        TRY(add_while(g, &n_loop, &n_rhs, 1, h, &body));
        TRY(add_kernel(body, &n_sp, nullptr, 0, (void *)k_spmv<double, Fast>, nit, NT, a_pcg));
        TRY(add_kernel(body, &n_up, &n_sp, 1, (void *)k_update<double, Fast, false>, nit, NT, a_pcg));
        CK(cudaGraphInstantiate(&gx, g, 0));
    }
    const Dev d0 = e->dev(0);

    // ---- backward, segment by segment
    Lam la, lb;
    for (int q = 0; q < 6; ++q) { la.q[q] = lam + q * e->ncells; lb.q[q] = lam + (6 + q) * e->ncells; }
    for (int j = nseg - 1; j >= 0; --j) {
        const int s0 = j * K, len = std::min(K, n_steps - s0);
        if (j < nseg - 1) {
            const double *ck = ckpt + (size_t)j * 7 * N;
            for (int q = 0; q < 6; ++q)
                CK(cudaMemcpyAsync(e->d_P[cur][q], ck + q * N, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(e->d_phi[0] + off, ck + 6 * N, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            TRY(forward_segment(e, st, Ez + s0, nullptr, len, store, cur));
        }
        for (int s = len - 1; s >= 0; --s) {
            const int n = s0 + s;
            if (dep) CK(cudaGraphLaunch(gx, st));
            const double seed = row[n] >= 0 ? dl[row[n]] / (double)N : 0.0;
            k_adj_div<<<nit, NT, 0, st>>>(d0, la, mu, seed);
            CLam P, Lin;
            for (int q = 0; q < 6; ++q) {
                P.q[q] = store + ((size_t)s * 6 + q) * N - off;
                Lin.q[q] = la.q[q];
            }
            k_adj_tdgl<<<nit, NT, 0, st>>>(d0, F, P, Lin, lb, lphi, tacc);
            CK(cudaGetLastError());
            std::swap(la, lb);
        }
        CK(cudaStreamSynchronize(st));
    }

    // ---- theta partials -> d loss / d (alpha, beta, gamma, g, kappa) per material
    std::vector<double> th((size_t)NTH * nit);
    CK(cudaMemcpy(th.data(), tacc, sizeof(double) * th.size(), cudaMemcpyDeviceToHost));
    double tot[NTH] = {0};
    for (int b = 0; b < nit; ++b)
        for (int q = 0; q < NTH; ++q) tot[q] += th[(size_t)b * NTH + q];
    FilmDev fd;
    CK(cudaMemcpy(&fd, e->d_films, sizeof(FilmDev), cudaMemcpyDeviceToHost));
    for (int m = 0; m < 3; ++m) {
        double da = 0, db = 0, dg = 0, dgl = 0, dk = 0;
        for (int fl = 0; fl < 2; ++fl) {
            const double *t = tot + (m * 2 + fl) * 6;
            const double sf = fl ? 0.4 : 1.0;                 // interface g (kernels_evol.cu:142-146)
            da += 2.0 * (t[0] + t[1]);                        // ag = 2(alpha + g), ags = 2(alpha - g)
            dgl += 2.0 * sf * (t[0] - t[1]);
            db += 4.0 * t[2] + 12.0 * t[3];                   // b4 = 4 beta, b12 = 12 beta
            dg += 6.0 * t[4];                                 // g6 = 6 gamma
            dk += fd.dt / fd.h2 * t[5];                       // A = kappa dt / h^2
        }
        grad[m * 5 + 0] = da;
        grad[m * 5 + 1] = db;
        grad[m * 5 + 2] = dg;
        grad[m * 5 + 3] = dgl;
        grad[m * 5 + 4] = dk;
    }
    return CMSL_OK;
}
