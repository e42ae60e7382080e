// spectral.cuh -- direct solve of the FP32 inner system for films whose
// materials share one permittivity (the configurations' eps_b).
//
// With a uniform eps the operator of depol_varEPS.cu:37-124 on the interior
// planes k = 1..nz-2 is (eps/h^2)(6 x_c - sum of the 6 neighbours), periodic
// in x and y, with x = 0 on the Dirichlet planes.  The in-plane discrete
// Fourier transform diagonalises the x/y part (eigenvalues 2 - 2 cos(2 pi m / n)),
// which leaves one real tridiagonal system along z per in-plane mode:
//   (lam_x + lam_y + 2) X_k - X_{k-1} - X_{k+1} = (h^2 / eps) R_k.
// The solve is: 2D FFT of the interior planes of r -> Thomas algorithm per
// mode -> inverse 2D FFT (as the forward transform of the conjugate) -> x.
// r and x are real, so interior planes 2j and 2j+1 travel as the real and
// imaginary parts of one complex plane j (half the transforms); the z solve
// separates a mode m and its mirror -m of the packed spectrum into the two
// real planes' spectra (R_2j = (Z(m) + conj Z(-m))/2, R_2j+1 = (Z(m) -
// conj Z(-m))/2i), solves for m (the mirror's solution is the conjugate) and
// packs the pair back.  It is exact up to FP32 rounding (~1e-6 relative), so
// one solve per refinement pass replaces the PCG iterations; the outer
// double-float refinement keeps the potential at the reference's tolerance.
//
// FFTs: self-sorting (Stockham) passes through shared memory, the butterflies
// in registers -- radix 16 (8, 4 or 2 for the remainder) for powers of two,
// radix 3 and 2 otherwise -- one block per group of rows (x) or of columns
// (y); twiddles exp(-2 pi i t / n) and eigenvalues come from host tables
// computed in double.  The z solve keeps the Thomas elimination in shared
// memory, so each spectrum value is read and written once per sweep.
//
// Two layouts of the spectra.  Row layout ([Mp][ny][nx], five launches, the
// default): x transforms, y transforms, z solve, y transforms, x transforms.
// Column layout ([Mp][nx][ny], three launches, films whose column pairs fit
// one block's shared memory, selected by CMSL_SPEC_COLS=1): the x transforms store (and the last ones load)
// through shared memory transposed, and one block per mirror pair of
// columns {kx, nx - kx} holds both columns of every packed plane, so it runs
// the y transforms, the z solve of all modes (kx, ky) with their mirrors
// (nx - kx, ny - ky), and the y transforms back, with contiguous column reads
// and writes (k_spec_yzy).
#pragma once
#include <cooperative_groups.h>
#include "kernels.cuh"

namespace cmsl {

constexpr int SPEC_MAX_STAGES = 13;       // 2^12 = 4096
constexpr int SPEC_ELEMS = 4096;          // complex values staged per block at most
constexpr int SPEC_NT = 256;

struct SpecAxis {
    int n, nst;
    int lg;                     // log2(n) when n is a power of two, else -1
    int rad[SPEC_MAX_STAGES];
};

// One film of the direct solve.
struct SpecFilm {
    SpecAxis ax, ay;
    long long off;              // first cell of the film
    long long coff;             // first spectrum value: [Mp][ny][nx], plane j = interior planes 2j, 2j+1
    int nx, ny, nz, M, Mp;      // M = nz - 2 interior planes, Mp = ceil(M / 2) packed planes
    int twx, twy, lamx, lamy;   // offsets into the twiddle / eigenvalue tables
    float scale;                // h^2 / (eps nx ny)
    int bx0, by0, bz0;          // first block of the film in the x, y and z grids
    int bq0;                    // first block of the film in the column-pair grid (column layout)
    int bc0;                    // first block of the film in the cluster grids (SPEC_CL blocks per packed plane)
    int rb, cb;                 // rows of an x-transform block, columns of a y-transform block
    long long ioff;             // first pivot of the film in SpecDev::piv
};

struct SpecDev {
    const SpecFilm *films;
    float2 *C;                  // spectra of every film
    const float2 *tw;           // exp(-2 pi i t / n) per film and axis
    const float *lam;           // 2 - 2 cos(2 pi t / n) per film and axis
    const int *bx_film, *by_film, *bz_film;   // film of every block of the three grids
    const int *bq_film;         // film of every block of the column-pair grid (column layout)
    const int *bc_film;         // film of every block of the cluster grids
    // Thomas pivots 1 / (dg - c'_{k-1}) of every interior plane k and mode,
    // [k][mode] per film (mode kx * ny + ky in the column layout, ky * nx + kx
    // in the row layout), computed on the host in double: the z solves run
    // without divisions on their serial chain
    const float *piv;
};

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Element e of sequence s of a block's tile sits at a[e * es + s * ss].  The
// transforms run in place between two such tiles (a, b) and return the one
// holding the result.  SEQ_FAST: consecutive threads take consecutive
// sequences (interleaved tiles, the y pass); otherwise consecutive butterflies
// of one sequence (the x pass), whose tiles are padded by one element every
// 16 (spec_pad) so that the strided Stockham writes of a warp fall on
// distinct banks.  tw: the n twiddles, staged in shared memory.
__host__ __device__ __forceinline__ int spec_pad(int i) { return i + (i >> 4); }

// Forward DFTs of 4, 8 and 16 values held in registers, y_k = sum_n v_n
// exp(-2 pi i n k / R).  dft4 and dft8 leave y in natural order; dft16 (4 x 4
// split) leaves y_k at v[4 (k mod 4) + k / 4] (dft_out gives the slot's k).
__device__ __forceinline__ void dft4(float2 &a, float2 &b, float2 &c, float2 &d)
{
    const float2 s02 = c_add(a, c), d02 = c_sub(a, c), s13 = c_add(b, d), d13 = c_sub(b, d);
    const float2 rot = make_float2(d13.y, -d13.x);     // -i (b - d)
    a = c_add(s02, s13);
    b = c_add(d02, rot);
    c = c_sub(s02, s13);
    d = c_sub(d02, rot);
}

constexpr float SPEC_R2 = 0.70710678118654752f;    // cos(pi/4)
constexpr float SPEC_C8 = 0.92387953251128676f;    // cos(pi/8)
constexpr float SPEC_S8 = 0.38268343236508977f;    // sin(pi/8)

__device__ __forceinline__ float2 c_mulc(float2 v, float wr, float wi)
{
    return make_float2(v.x * wr - v.y * wi, v.x * wi + v.y * wr);
}

__device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
    const float2 t = a;
    a = c_add(t, b);
    b = c_sub(t, b);
}

__device__ __forceinline__ void dft8(float2 (&v)[8])
{
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4(e0, e1, e2, e3);
    dft4(o0, o1, o2, o3);
    o1 = c_mulc(o1, SPEC_R2, -SPEC_R2);                // w8^1
    o2 = make_float2(o2.y, -o2.x);                     // w8^2 = -i
    o3 = c_mulc(o3, -SPEC_R2, -SPEC_R2);               // w8^3
    v[0] = c_add(e0, o0); v[4] = c_sub(e0, o0);
    v[1] = c_add(e1, o1); v[5] = c_sub(e1, o1);
    v[2] = c_add(e2, o2); v[6] = c_sub(e2, o2);
    v[3] = c_add(e3, o3); v[7] = c_sub(e3, o3);
}

// v * w16^e for the exponents e = n2 k1 (n2, k1 < 4) of the 4 x 4 split
__device__ __forceinline__ float2 w16(int e, float2 v)
{
    switch (e) {
    case 0: return v;
    case 1: return c_mulc(v, SPEC_C8, -SPEC_S8);
    case 2: return c_mulc(v, SPEC_R2, -SPEC_R2);
    case 3: return c_mulc(v, SPEC_S8, -SPEC_C8);
    case 4: return make_float2(v.y, -v.x);
    case 6: return c_mulc(v, -SPEC_R2, -SPEC_R2);
    default: return c_mulc(v, -SPEC_C8, SPEC_S8);     // e = 9
    }
}

__device__ __forceinline__ void dft16(float2 (&v)[16])
{
    // n = 4 n1 + n2, k = k1 + 4 k2: DFT4 over n1, twiddle w16^(n2 k1), DFT4 over n2
    #pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
    #pragma unroll
    for (int k1 = 1; k1 < 4; ++k1)
        #pragma unroll
        for (int n2 = 1; n2 < 4; ++n2) v[4 * k1 + n2] = w16(n2 * k1, v[4 * k1 + n2]);
    #pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

template <int R> __device__ __forceinline__ constexpr int dft_out(int i) { return R == 16 ? (i >> 2) + 4 * (i & 3) : i; }

template <int R> __device__ __forceinline__ void dft_reg(float2 (&v)[R])
{
    if constexpr (R == 2) dft2(v[0], v[1]);
    else if constexpr (R == 4) dft4(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8) dft8(v);
    else dft16(v);
}

// One self-sorting (Stockham) pass of radix R on a tile: butterfly j of a
// sequence takes elements j + r n/R (r < R), twiddled by w_n^(r (j mod Ns)
// n / (Ns R)), and writes its DFT to (j / Ns) Ns R + (j mod Ns) + k Ns.
// The first pass reads through ld(sequence, element) instead of tile a, the
// last writes through st(sequence, element, value) instead of tile b, so the
// data goes from global memory to registers and back with one shared-memory
// exchange per further pass.
template <int R, bool SEQ_FAST, class LD, class ST>
__device__ __forceinline__ void stockham_pass(const float2 *a, float2 *b, int nseq, int lgs, int lgn, int lgNs,
                                              int es, int ss, const float2 *tw, bool first, bool last, LD &ld,
                                              ST &st)
{
    constexpr int lgR = R == 16 ? 4 : R == 8 ? 3 : R == 4 ? 2 : 1;
    const int lgnbf = lgn - lgR, nbf = 1 << lgnbf;
    const int Ns = 1 << lgNs;
    const int lgstep = lgn - lgNs - lgR;              // twiddle stride n / (Ns R)
    const int total = nseq << lgnbf;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int sq, j;
        if (SEQ_FAST) {
            if (lgs >= 0) { j = t >> lgs; sq = t & (nseq - 1); }
            else { j = t / nseq; sq = t - j * nseq; }
        } else {
            sq = t >> lgnbf; j = t & (nbf - 1);
        }
        const int jm = j & (Ns - 1);
        const int o = ((j >> lgNs) << (lgNs + lgR)) + jm;
        const int base = sq * ss;
        auto at = [&](int e) { return SEQ_FAST ? base + e * es : spec_pad(base + e * es); };
        const int tj = jm << lgstep;
        float2 v[R];
        if (first) {
            #pragma unroll
            for (int r = 0; r < R; ++r) v[r] = ld(sq, j + r * nbf);
        } else {
            #pragma unroll
            for (int r = 0; r < R; ++r) v[r] = a[at(j + r * nbf)];
        }
        if (lgNs > 0) {
            #pragma unroll
            for (int r = 1; r < R; ++r) v[r] = c_mul(v[r], tw[r * tj]);
        }
        dft_reg<R>(v);
        if (last) {
            #pragma unroll
            for (int i = 0; i < R; ++i) st(sq, o + dft_out<R>(i) * Ns, v[i]);
        } else {
            #pragma unroll
            for (int i = 0; i < R; ++i) b[at(o + dft_out<R>(i) * Ns)] = v[i];
        }
    }
}

// n = 2^lgn: passes of radix 16 (8, 4 or 2 for the remainder; a radix-8
// pass first when the remainder would be a lone radix-2), between ld and st
// (see stockham_pass) with tiles a and b for the exchanges.  The twiddles
// must be visible to the block (a barrier after staging them).
template <bool SEQ_FAST, class LD, class ST>
__device__ __forceinline__ void fft_pow2(float2 *a, float2 *b, int nseq, int lgn, int es, int ss, const float2 *tw,
                                         LD ld, ST st)
{
    const int lgs = (nseq & (nseq - 1)) == 0 ? __ffs(nseq) - 1 : -1;   // sequences per tile, as a shift
    if (lgn == 0)                                                     // n = 1: the identity
        for (int t = threadIdx.x; t < nseq; t += blockDim.x) st(t, 0, ld(t, 0));
    int lgNs = 0;
    while (lgNs < lgn) {
        const int rem = lgn - lgNs;
        const int lgR = (rem >= 4 && (rem & 3) != 1) ? 4 : rem >= 3 ? 3 : rem;
        const bool first = lgNs == 0, last = lgNs + lgR == lgn;
        if (lgR == 4) stockham_pass<16, SEQ_FAST>(a, b, nseq, lgs, lgn, lgNs, es, ss, tw, first, last, ld, st);
        else if (lgR == 3) stockham_pass<8, SEQ_FAST>(a, b, nseq, lgs, lgn, lgNs, es, ss, tw, first, last, ld, st);
        else if (lgR == 2) stockham_pass<4, SEQ_FAST>(a, b, nseq, lgs, lgn, lgNs, es, ss, tw, first, last, ld, st);
        else stockham_pass<2, SEQ_FAST>(a, b, nseq, lgs, lgn, lgNs, es, ss, tw, first, last, ld, st);
        if (!last) __syncthreads();
        float2 *tmp = a;
        a = b;
        b = tmp;
        lgNs += lgR;
    }
}

// Any 2^a 3^b length: radix-3 and radix-2 passes.
template <bool SEQ_FAST>
__device__ __forceinline__ float2 *fft_mixed(float2 *a, float2 *b, int nseq, const SpecAxis &pl, int es, int ss,
                                             const float2 *tw)
{
    const int n = pl.n;
    int Ns = 1;
    for (int st = 0; st < pl.nst; ++st) {
        const int R = pl.rad[st];
        const int nbf = n / R;
        const int tstride = n / (Ns * R);
        for (int t = threadIdx.x; t < nseq * nbf; t += blockDim.x) {
            int sq, j;
            if (SEQ_FAST) { j = t / nseq; sq = t - j * nseq; }
            else { sq = t / nbf; j = t - sq * nbf; }
            const int jm = j % Ns;
            const int base = sq * ss;
            auto at = [&](int e) { return SEQ_FAST ? base + e * es : spec_pad(base + e * es); };
            const int o = (j / Ns) * Ns * R + jm;
            const float2 v0 = a[at(j)];
            const float2 v1 = c_mul(a[at(j + nbf)], tw[jm * tstride]);
            if (R == 2) {
                b[at(o)] = c_add(v0, v1);
                b[at(o + Ns)] = c_sub(v0, v1);
            } else {
                const float2 v2 = c_mul(a[at(j + 2 * nbf)], tw[2 * jm * tstride]);
                const float2 s12 = c_add(v1, v2), d12 = c_sub(v1, v2);
                const float2 m = make_float2(v0.x - 0.5f * s12.x, v0.y - 0.5f * s12.y);
                const float k3 = 0.86602540378443865f;   // sin(2 pi / 3)
                const float2 rot = make_float2(k3 * d12.y, -k3 * d12.x);
                b[at(o)] = c_add(v0, s12);
                b[at(o + Ns)] = c_add(m, rot);
                b[at(o + 2 * Ns)] = c_sub(m, rot);
            }
        }
        __syncthreads();
        float2 *tmp = a;
        a = b;
        b = tmp;
        Ns *= R;
    }
    return a;
}


// Whether film f's inner solve runs through the spectra in this pass.
__device__ __forceinline__ bool spec_run(const Dev &d, int f)
{
    return d.force || *(volatile const int *)&d.solve[f].active != 0;
}

// The inverse transform closes the solve: its last block marks every active
// film's inner solve done (one "iteration").
// Under deferred checks (Dev::defer, the solve node of a step) a step whose
// films all end on this solve ends here.
__device__ __forceinline__ void spec_finish(const Dev &d)
{
    if (!ticket_last(d.counter)) return;
    __shared__ int s_out;
    if (threadIdx.x == 0) {
        int out = 0;
        if (!d.force)
            for (int f = 0; f < d.n_films; ++f) {
                SolveDev *S = d.solve + f;
                if (S->active) {
                    S->iters = 1;
                    S->total_iters += 1;
                    S->active = 0;
                }
                out |= S->outer_active;
            }
        *d.counter = 0u;
        s_out = out;
    }
    __syncthreads();
    if (d.defer && d.step_end && !d.force && !s_out) step_end(d);
}

// x transforms of rows (j, y) of the packed planes, j = 0 .. Mp-1.  IN_REAL:
// from the FP32 residual r (interior planes 2j and 2j+1, i.e. z planes 2j+1
// and 2j+2, as real and imaginary parts) into the spectra; otherwise from the
// spectra into the real correction x (and x = 0 on the Dirichlet planes).
// COL: the spectra in the column layout, stored (IN_REAL) or loaded through a
// shared-memory tile transposed, so that a warp touches runs of consecutive
// y.  Shared memory: two padded tiles of rb rows and the twiddles.
__host__ __device__ inline int spec_x_pitch(int nx, bool col) { return col ? nx + 1 : nx; }

__device__ __forceinline__ int fft_pow2_passes(int lgn)
{
    int n = 0;
    for (int lgNs = 0; lgNs < lgn; ++n) {
        const int rem = lgn - lgNs;
        lgNs += (rem >= 4 && (rem & 3) != 1) ? 4 : rem >= 3 ? 3 : rem;
    }
    return n;
}

template <bool IN_REAL, bool COL = false>
__global__ void __launch_bounds__(SPEC_NT, 4) k_spec_x(Dev d, Fields<float> F, SpecDev sp)
{
    extern __shared__ float2 sm2[];
    const int f = __ldg(sp.bx_film + blockIdx.x);
    if (!spec_run(d, f)) {
        if (!IN_REAL) spec_finish(d);
        return;
    }
    const SpecFilm &P = sp.films[f];
    const int nx = P.nx, ny = P.ny, rows = P.Mp * ny, rb = P.rb;
    const int r0 = (blockIdx.x - P.bx0) * rb, nr = min(rb, rows - r0);
    const long long plane = (long long)nx * ny;
    const float *rr = F.r + P.off;
    float *xx = F.x + P.off;
    float2 *Cf = sp.C + P.coff;
    const SpecAxis ax = P.ax;
    const int M = P.M, Mp = P.Mp;
    // row pitch of the tiles: nx, or nx + 1 in the column layout, whose
    // transposed copies read a column of the tile (an odd pitch in 8-byte
    // words spreads its rows over the banks)
    const int pitch = spec_x_pitch(nx, COL);
    const int tile = spec_pad(rb * pitch) + 1;
    float2 *a = sm2, *b = sm2 + tile, *tw = sm2 + 2 * tile;
    for (int t = threadIdx.x; t < nx; t += blockDim.x) tw[t] = __ldg(sp.tw + P.twx + t);
    // spectrum value (row r0 + sq, x element e) in the column layout
    auto col_at = [&](int sq, int e) -> long long {
        const int rw = r0 + sq, j = rw / ny;
        return ((long long)j * nx + e) * ny + (rw - j * ny);
    };
    if (COL && !IN_REAL) {
        // transposed load: consecutive threads take consecutive rows of one column
        const int total = nr * nx;
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int e = t / nr, sq = t - e * nr;
            a[spec_pad(sq * pitch + e)] = Cf[col_at(sq, e)];
        }
        __syncthreads();
    }
    // row r0 + sq is (j, y) = packed plane j, in-plane row y; its residual
    // rows in r are z planes 2j+1 and 2j+2
    auto ld = [&](int sq, int e) -> float2 {
        if (!IN_REAL) return COL ? a[spec_pad(sq * pitch + e)] : Cf[(long long)(r0 + sq) * nx + e];
        const int rw = r0 + sq, j = rw / ny;
        const long long o = (long long)(2 * j + 1) * plane + (long long)(rw - j * ny) * nx + e;
        return make_float2(rr[o], 2 * j + 1 < M ? rr[o + plane] : 0.f);
    };
    // the tile that receives the transform in the column layout's store
    float2 *res = (ax.lg >= 0 && (fft_pow2_passes(ax.lg) & 1) == 0) ? a : b;
    // the increment of this solve: w M^-1 r + m (the previous increment), from
    // the film's Chebyshev recurrence (w = 1, m = 0 for an exact solve)
    const SolveDev *Sf = d.solve + f;
    const float cw = IN_REAL ? 1.f : (d.force || Sf->cheb_w == 0.f ? 1.f : Sf->cheb_w);
    const float cm = IN_REAL || d.force ? 0.f : Sf->cheb_m;
    auto st = [&](int sq, int e, float2 v) {
        if (IN_REAL) {
            if (COL) res[spec_pad(sq * pitch + e)] = v;
            else Cf[(long long)(r0 + sq) * nx + e] = v;
            return;
        }
        // the transform of conj(W) is conj(x_2j + i x_2j+1) (scale folded into the z solve)
        const int rw = r0 + sq, j = rw / ny;
        const long long yx = (long long)(rw - j * ny) * nx + e, o = (long long)(2 * j + 1) * plane + yx;
        if (cm != 0.f) {
            xx[o] = cw * v.x + cm * xx[o];
            if (2 * j + 1 < M) xx[o + plane] = cw * -v.y + cm * xx[o + plane];
        } else {
            xx[o] = cw * v.x;
            if (2 * j + 1 < M) xx[o + plane] = cw * -v.y;
        }
        if (j == 0) xx[yx] = 0.f;                                        // first Dirichlet plane
        if (j == Mp - 1) xx[(long long)(M + 1) * plane + yx] = 0.f;      // last one
    };
    if (ax.lg >= 0) {
        __syncthreads();                                                 // twiddles
        fft_pow2<false>(a, b, nr, ax.lg, 1, pitch, tw, ld, st);
    } else {
        const int total = nr * nx;
        if (!(COL && !IN_REAL))
            for (int t = threadIdx.x; t < total; t += blockDim.x) {
                const int sq = t / nx, e = t - sq * nx;
                a[spec_pad(sq * pitch + e)] = ld(sq, e);
            }
        __syncthreads();
        res = fft_mixed<false>(a, b, nr, ax, 1, pitch, tw);
        if (!(COL && IN_REAL))
            for (int t = threadIdx.x; t < total; t += blockDim.x) {
                const int sq = t / nx, e = t - sq * nx;
                st(sq, e, res[spec_pad(sq * pitch + e)]);
            }
    }
    if (COL && IN_REAL) {
        // transposed store: consecutive threads write consecutive rows of one column
        __syncthreads();
        const int total = nr * nx;
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int e = t / nr, sq = t - e * nr;
            Cf[col_at(sq, e)] = res[spec_pad(sq * pitch + e)];
        }
    }
    if (!IN_REAL) spec_finish(d);
}

// y transforms of column groups of one packed plane, in place on the
// spectra; the tile keeps the plane's row-major layout (sequences interleaved).
static __global__ void __launch_bounds__(SPEC_NT, 4) k_spec_y(Dev d, SpecDev sp)
{
    extern __shared__ float2 sm2[];
    const int f = __ldg(sp.by_film + blockIdx.x);
    if (!spec_run(d, f)) return;
    const SpecFilm &P = sp.films[f];
    const int nx = P.nx, ny = P.ny, cb = P.cb;
    const int groups = (nx + cb - 1) / cb;
    const int lb = blockIdx.x - P.by0;
    const int kk = lb / groups, x0 = (lb - kk * groups) * cb, nc = min(cb, nx - x0);
    const SpecAxis ay = P.ay;
    float2 *base = sp.C + P.coff + (long long)kk * nx * ny + x0;
    float2 *a = sm2, *b = sm2 + cb * ny, *tw = sm2 + 2 * cb * ny;
    for (int t = threadIdx.x; t < ny; t += blockDim.x) tw[t] = __ldg(sp.tw + P.twy + t);
    // sequence c = column x0 + c, element e = row y (coalesced along x)
    auto ld = [&](int c, int e) { return base[(long long)e * nx + c]; };
    auto st = [&](int c, int e, float2 v) { base[(long long)e * nx + c] = v; };
    __syncthreads();                                                     // twiddles
    if (ay.lg >= 0) {
        fft_pow2<true>(a, b, nc, ay.lg, nc, 1, tw, ld, st);
    } else {
        const int total = nc * ny;
        for (int t = threadIdx.x; t < total; t += blockDim.x) a[t] = ld(t % nc, t / nc);
        __syncthreads();
        const float2 *res = fft_mixed<true>(a, b, nc, ay, nc, 1, tw);
        for (int t = threadIdx.x; t < total; t += blockDim.x) st(t % nc, t / nc, res[t]);
    }
}

// In-plane modes m whose mirror -m has an index >= m's, one per z solve:
// rows y = 1 .. (ny-1)/2 in full, then row 0 and, for even ny, row ny/2
// with x = 0 .. nx/2.  Returns false past the last one.
__device__ __forceinline__ bool spec_canon_mode(long long t, int nx, int ny, int &x, int &y)
{
    const long long full = (long long)((ny - 1) / 2) * nx;
    if (t < full) {
        y = 1 + (int)(t / nx);
        x = (int)(t - (long long)(y - 1) * nx);
        return true;
    }
    const int hx = nx / 2 + 1, t2 = (int)(t - full);
    if (t2 < hx) { y = 0; x = t2; return true; }
    if ((ny & 1) == 0 && t2 < 2 * hx) { y = ny / 2; x = t2 - hx; return true; }
    return false;
}
__host__ __device__ inline long long spec_canon_count(int nx, int ny)
{
    return (long long)((ny - 1) / 2) * nx + (long long)(nx / 2 + 1) * ((ny & 1) == 0 ? 2 : 1);
}
// The same set column by column (the column layout: consecutive threads take
// consecutive y): columns x = 1 .. (nx-1)/2 in full, then column 0 and, for
// even nx, column nx/2 with y = 0 .. ny/2.
__device__ __forceinline__ bool spec_canon_mode_col(long long t, int nx, int ny, int &x, int &y)
{
    const long long full = (long long)((nx - 1) / 2) * ny;
    if (t < full) {
        x = 1 + (int)(t / ny);
        y = (int)(t - (long long)(x - 1) * ny);
        return true;
    }
    const int hy = ny / 2 + 1, t2 = (int)(t - full);
    if (t2 < hy) { x = 0; y = t2; return true; }
    if ((nx & 1) == 0 && t2 < 2 * hy) { x = nx / 2; y = t2 - hy; return true; }
    return false;
}

// Thomas algorithm along z, one thread per canonical mode m (the mirror's
// solution is the conjugate).  The thread's packed spectra at m and -m for
// every plane pair are first copied into shared memory at once (cp.async),
// then eliminated there: [Mp][blockDim] float4 (Z(m), Z(-m)), overwritten by
// the eliminated right-hand sides (d'_2j, d'_2j+1), and [M][blockDim] of
// the mode's pivots (SpecDev::piv) staged with them.
// Writes the conjugates of the packed scaled solutions, so that the next
// forward transforms invert.  COL: the spectra (and the pivots) in the column
// layout [Mp][nx][ny] of the cluster transforms, modes taken column by column.
template <bool COL = false>
static __global__ void k_spec_z(Dev d, SpecDev sp)
{
    extern __shared__ float2 sm2[];
    const int f = __ldg(sp.bz_film + blockIdx.x);
    if (!spec_run(d, f)) return;
    const SpecFilm &P = sp.films[f];
    const int M = P.M, Mp = P.Mp, T = blockDim.x, tx = threadIdx.x;
    float4 *dp = (float4 *)sm2;
    int x, y;
    const long long t = (long long)(blockIdx.x - P.bz0) * T + tx;
    if (!(COL ? spec_canon_mode_col(t, P.nx, P.ny, x, y) : spec_canon_mode(t, P.nx, P.ny, x, y))) return;
    const long long modes = (long long)P.nx * P.ny;
    const int xm = x == 0 ? 0 : P.nx - x, ym = y == 0 ? 0 : P.ny - y;
    const long long m = COL ? (long long)x * P.ny + y : (long long)y * P.nx + x;
    const long long mm = COL ? (long long)xm * P.ny + ym : (long long)ym * P.nx + xm;
    float2 *Ca = sp.C + P.coff + m, *Cb = sp.C + P.coff + mm;
    float *pvs = (float *)(dp + (size_t)Mp * T) + tx;   // this thread's pivots, plane k at pvs[k * T]
    {
        const float *pv = sp.piv + P.ioff + m;          // pivot of plane k at pv[k * modes]
        for (int k = 0; k < M; ++k) cp4(pvs + (size_t)k * T, pv + k * modes);
    }
    for (int j = 0; j < Mp; ++j) {
        float2 *s = (float2 *)(dp + (size_t)j * T + tx);
        cp8(s, Ca + j * modes);
        cp8(s + 1, Cb + j * modes);
    }
    cp_commit();
    const float s = 0.5f * P.scale;
    cp_wait<0>();
    float2 d_prev = make_float2(0.f, 0.f);
    auto sweep = [&](int k, float2 rk) {             // forward elimination (sub/super-diagonal -1)
        const float inv = pvs[(size_t)k * T];
        d_prev = make_float2((rk.x * s + d_prev.x) * inv, (rk.y * s + d_prev.y) * inv);
        return d_prev;
    };
    for (int j = 0; j < Mp; ++j) {
        const float4 ab = dp[(size_t)j * T + tx];    // a = Z(m), b = Z(-m)
        const float2 d0 = sweep(2 * j, make_float2(ab.x + ab.z, ab.y - ab.w));   // 2 (Z(m) + conj Z(-m)) / 2
        float2 d1 = make_float2(0.f, 0.f);
        if (2 * j + 1 < M) d1 = sweep(2 * j + 1, make_float2(ab.y + ab.w, ab.z - ab.x));   // (Z(m) - conj Z(-m)) / i
        dp[(size_t)j * T + tx] = make_float4(d0.x, d0.y, d1.x, d1.y);
    }
    // back substitution (x_k = d'_k + pivot_k x_{k+1}), two planes at a time;
    // store conj of the packed pair W(m) = X_2j + i X_2j+1 and
    // W(-m) = conj X_2j + i conj X_2j+1
    auto put = [&](int j, float2 p0, float2 p1) {
        Ca[j * modes] = make_float2(p0.x - p1.y, -(p0.y + p1.x));
        Cb[j * modes] = make_float2(p0.x + p1.y, p0.y - p1.x);
    };
    float2 xn = make_float2(0.f, 0.f);               // x_{k+1} of the plane above the pair
    for (int j = Mp - 1; j >= 0; --j) {
        const float4 dd = dp[(size_t)j * T + tx];
        float2 v = make_float2(0.f, 0.f);
        if (2 * j + 1 < M) {
            const float c = pvs[(size_t)(2 * j + 1) * T];
            v = make_float2(dd.z + c * xn.x, dd.w + c * xn.y);
        }
        const float c = pvs[(size_t)(2 * j) * T];
        const float2 u = make_float2(dd.x + c * v.x, dd.y + c * v.y);
        put(j, u, v);
        xn = u;
    }
}


// Column layout: the y transforms, the z solve and the y transforms back of
// one mirror pair of columns {kx, kx2 = (nx - kx) mod nx} of every packed
// plane of a film (one block; kx = kx2 for kx = 0 and, for even nx, nx/2).
// Sequence s = j * ncol + c of the shared tiles is column c (0: kx, 1: kx2)
// of packed plane j, its ny values contiguous (padded every 16).  Modes
// (kx, ky) pair with (kx2, (ny - ky) mod ny); a self-mirror column pairs ky
// with ny - ky inside itself, one thread per pair (ky <= ny - ky).  The
// elimination runs in place: the pair's slots at plane j take the eliminated
// right-hand sides of interior planes 2j and 2j+1 (for a mode that is its
// own mirror both are real and share its one slot), then the conjugates of
// the packed solutions, whose forward y transforms go back to the spectra.
// Shared memory: two tiles, the y twiddles and the column's pivots
// (SpecDev::piv).
__host__ __device__ inline size_t spec_yzy_bytes(int ny, int Mp, int M)
{
    return sizeof(float2) * (2 * (size_t)(spec_pad(2 * Mp * ny) + 1) + ny) + sizeof(float) * (size_t)M * ny;
}

constexpr int SPEC_YZY_NT = 512;

static __global__ void __launch_bounds__(SPEC_YZY_NT, 1) k_spec_yzy(Dev d, SpecDev sp)
{
    extern __shared__ float2 sm2[];
    const int f = __ldg(sp.bq_film + blockIdx.x);
    if (!spec_run(d, f)) return;
    const SpecFilm &P = sp.films[f];
    const int nx = P.nx, ny = P.ny, M = P.M, Mp = P.Mp;
    const int kx = blockIdx.x - P.bq0, kx2 = kx == 0 ? 0 : nx - kx;
    const int ncol = kx == kx2 ? 1 : 2, nseq = ncol * Mp;
    const int tile = spec_pad(2 * Mp * ny) + 1;
    float2 *A = sm2, *B = sm2 + tile, *tw = sm2 + 2 * tile;
    const SpecAxis ay = P.ay;
    const long long modes = (long long)nx * ny;
    float2 *Cf = sp.C + P.coff;
    auto gcol = [&](int sq) {                    // first value of sequence sq in the spectra
        const int j = sq / ncol, c = sq - j * ncol;
        return Cf + ((long long)j * nx + (c ? kx2 : kx)) * ny;
    };
    // the pivots of column kx (its mirror column's are the same: lam(nx - kx) =
    // lam(kx), lam(ny - ky) = lam(ky)), staged while the transforms run
    float *pvs = (float *)(tw + ny);
    for (int t = threadIdx.x; t < M * ny; t += blockDim.x) {
        const int k = t / ny, ky = t - k * ny;
        cp4(pvs + t, sp.piv + P.ioff + k * modes + (long long)kx * ny + ky);
    }
    cp_commit();
    for (int t = threadIdx.x; t < ny; t += blockDim.x) tw[t] = __ldg(sp.tw + P.twy + t);
    __syncthreads();
    // forward y transforms: spectra -> tile R
    float2 *R;
    if (ay.lg >= 0) {
        R = (fft_pow2_passes(ay.lg) & 1) == 0 ? A : B;
        auto ld = [&](int sq, int e) { return gcol(sq)[e]; };
        auto st = [&](int sq, int e, float2 v) { R[spec_pad(sq * ny + e)] = v; };
        fft_pow2<false>(A, B, nseq, ay.lg, 1, ny, tw, ld, st);
    } else {
        for (int t = threadIdx.x; t < nseq * ny; t += blockDim.x) A[spec_pad(t)] = gcol(t / ny)[t - (t / ny) * ny];
        __syncthreads();
        R = fft_mixed<false>(A, B, nseq, ay, 1, ny, tw);
    }
    __syncthreads();
    cp_wait<0>();
    __syncthreads();
    // z solve, one thread per mode pair (as k_spec_z)
    const int npair = ncol == 2 ? ny : ny / 2 + 1;
    const float s = 0.5f * P.scale;
    for (int ky = threadIdx.x; ky < npair; ky += blockDim.x) {
        const int ky2 = ky == 0 ? 0 : ny - ky;
        const bool self = ncol == 1 && ky == ky2;
        const float *pv = pvs + ky;              // pivot of plane k at pv[k * ny]
        auto slot_a = [&](int j) { return &R[spec_pad((j * ncol) * ny + ky)]; };
        auto slot_b = [&](int j) { return &R[spec_pad((j * ncol + ncol - 1) * ny + ky2)]; };
        float2 d_prev = make_float2(0.f, 0.f);
        auto sweep = [&](int k, float2 rk) {     // forward elimination (sub/super-diagonal -1)
            const float inv = pv[k * ny];
            d_prev = make_float2((rk.x * s + d_prev.x) * inv, (rk.y * s + d_prev.y) * inv);
            return d_prev;
        };
        for (int j = 0; j < Mp; ++j) {
            const float2 a = *slot_a(j), b = *slot_b(j);       // Z(m), Z(-m)
            const float2 d0 = sweep(2 * j, make_float2(a.x + b.x, a.y - b.y));
            float2 d1 = make_float2(0.f, 0.f);
            if (2 * j + 1 < M) d1 = sweep(2 * j + 1, make_float2(a.y + b.y, b.x - a.x));
            if (self) {
                *slot_a(j) = make_float2(d0.x, d1.x);
            } else {
                *slot_a(j) = d0;
                *slot_b(j) = d1;
            }
        }
        // back substitution (x_k = d'_k + pivot_k x_{k+1}), two planes at a
        // time; the slots take the conjugates of W(m) = X_2j + i X_2j+1 and
        // W(-m) = conj X_2j + i conj X_2j+1
        float2 xn = make_float2(0.f, 0.f);
        for (int j = Mp - 1; j >= 0; --j) {
            float2 d0, d1;
            if (self) {
                const float2 q = *slot_a(j);
                d0 = make_float2(q.x, 0.f);
                d1 = make_float2(q.y, 0.f);
            } else {
                d0 = *slot_a(j);
                d1 = *slot_b(j);
            }
            float2 v = make_float2(0.f, 0.f);
            if (2 * j + 1 < M) {
                const float c = pv[(2 * j + 1) * ny];
                v = make_float2(d1.x + c * xn.x, d1.y + c * xn.y);
            }
            const float c = pv[2 * j * ny];
            const float2 u = make_float2(d0.x + c * v.x, d0.y + c * v.y);
            *slot_a(j) = make_float2(u.x - v.y, -(u.y + v.x));
            if (!self) *slot_b(j) = make_float2(u.x + v.y, u.y - v.x);
            xn = u;
        }
    }
    __syncthreads();
    // y transforms of the conjugated solutions: tile R -> spectra
    if (ay.lg >= 0) {
        float2 *other = R == A ? B : A;
        auto ld = [&](int sq, int e) { return R[spec_pad(sq * ny + e)]; };
        auto st = [&](int sq, int e, float2 v) { gcol(sq)[e] = v; };
        fft_pow2<false>(R, other, nseq, ay.lg, 1, ny, tw, ld, st);
    } else {
        const float2 *res = fft_mixed<false>(R, R == A ? B : A, nseq, ay, 1, ny, tw);
        for (int t = threadIdx.x; t < nseq * ny; t += blockDim.x) gcol(t / ny)[t - (t / ny) * ny] = res[spec_pad(t)];
    }
}

// ------------------------------------------------- cluster transforms
// The in-plane transforms of a packed plane in one thread-block cluster of
// SPEC_CL blocks (films with power-of-two sides divisible by SPEC_CL whose
// tiles fit one block's shared memory): block q of the cluster owns rows
// y0 = q ny / SPEC_CL .. and columns x0 = q nx / SPEC_CL .. of the plane.
// Forward (k_spec_cxy): x transforms of its rows into its tile T, a cluster
// barrier, then y transforms of its columns whose first pass reads the other
// blocks' tiles through distributed shared memory, written to the spectra
// in the column layout [Mp][nx][ny].  Inverse (k_spec_cyx): y transforms of
// its columns into T (column-major), a cluster barrier, x transforms of its
// rows reading the tiles of the cluster, written to dx.  A solve is these
// two launches around the column-layout z solve, with no pass over the
// spectra between the x and the y transforms.  T's rows (columns) are
// padded to an odd pitch in 8-byte words so that the strided reads of
// another block's tile spread over the banks; a last cluster barrier keeps
// every block resident until the others have read its tile.
constexpr int SPEC_CL = 8;
constexpr int SPEC_CL_NT = 512;

__host__ __device__ inline int spec_cl_tile(int nx, int ny)     // float2 of T, A or B
{
    const int rows = ny / SPEC_CL, cols = nx / SPEC_CL;
    const int t = rows * (nx + 1) > cols * (ny + 1) ? rows * (nx + 1) : cols * (ny + 1);
    const int a = spec_pad(rows * nx) + 1;                      // = spec_pad(cols * ny) + 1
    return t > a ? t : a;
}
__host__ __device__ inline size_t spec_cl_bytes(int nx, int ny)
{
    return sizeof(float2) * (3 * (size_t)spec_cl_tile(nx, ny) + nx + ny);
}
__host__ inline bool spec_cl_ok(const SpecAxis &ax, const SpecAxis &ay, int nx, int ny, size_t smem_max)
{
    return ax.lg >= 0 && ay.lg >= 0 && nx % SPEC_CL == 0 && ny % SPEC_CL == 0 && nx >= 32 && ny >= 32 &&
           spec_cl_bytes(nx, ny) <= smem_max;
}

static __global__ void __cluster_dims__(SPEC_CL, 1, 1) __launch_bounds__(SPEC_CL_NT, 1)
    k_spec_cxy(Dev d, Fields<float> F, SpecDev sp)
{
    namespace cgr = cooperative_groups;
    extern __shared__ float2 sm2[];
    const cgr::cluster_group cl = cgr::this_cluster();
    const int f = __ldg(sp.bc_film + blockIdx.x);
    if (!spec_run(d, f)) return;                     // the whole cluster: one film
    const SpecFilm &P = sp.films[f];
    const int nx = P.nx, ny = P.ny, M = P.M;
    const int j = (blockIdx.x - P.bc0) / SPEC_CL, q = (int)cl.block_rank();
    const int rows = ny / SPEC_CL, cols = nx / SPEC_CL, y0 = q * rows, x0 = q * cols;
    const int tile = spec_cl_tile(nx, ny), pitch = nx + 1;
    float2 *T = sm2, *A = T + tile, *B = A + tile, *twx = B + tile, *twy = twx + nx;
    for (int t = threadIdx.x; t < nx; t += blockDim.x) twx[t] = __ldg(sp.tw + P.twx + t);
    for (int t = threadIdx.x; t < ny; t += blockDim.x) twy[t] = __ldg(sp.tw + P.twy + t);
    __syncthreads();
    // x transforms of rows y0 + sq: interior z planes 2j+1 and 2j+2 of r as
    // real and imaginary parts
    const long long plane = (long long)nx * ny;
    const float *rr = F.r + P.off;
    auto ldr = [&](int sq, int e) -> float2 {
        const long long o = (long long)(2 * j + 1) * plane + (long long)(y0 + sq) * nx + e;
        return make_float2(rr[o], 2 * j + 1 < M ? rr[o + plane] : 0.f);
    };
    auto stT = [&](int sq, int e, float2 v) { T[sq * pitch + e] = v; };
    fft_pow2<false>(A, B, rows, P.ax.lg, 1, nx, twx, ldr, stT);
    cl.sync();
    // y transforms of columns x0 + sq: element y sits in block y / rows, row y % rows
    float2 *Cf = sp.C + P.coff;
    auto ldT = [&](int sq, int e) -> float2 {
        const int p = e / rows, r = e - p * rows;
        return cl.map_shared_rank(T, p)[r * pitch + x0 + sq];
    };
    auto stC = [&](int sq, int e, float2 v) { Cf[((long long)j * nx + x0 + sq) * ny + e] = v; };
    fft_pow2<false>(A, B, cols, P.ay.lg, 1, ny, twy, ldT, stC);
    cl.sync();
}

static __global__ void __cluster_dims__(SPEC_CL, 1, 1) __launch_bounds__(SPEC_CL_NT, 1)
    k_spec_cyx(Dev d, Fields<float> F, SpecDev sp)
{
    namespace cgr = cooperative_groups;
    extern __shared__ float2 sm2[];
    const cgr::cluster_group cl = cgr::this_cluster();
    const int f = __ldg(sp.bc_film + blockIdx.x);
    if (!spec_run(d, f)) {
        spec_finish(d);
        return;
    }
    const SpecFilm &P = sp.films[f];
    const int nx = P.nx, ny = P.ny, M = P.M, Mp = P.Mp;
    const int j = (blockIdx.x - P.bc0) / SPEC_CL, q = (int)cl.block_rank();
    const int rows = ny / SPEC_CL, cols = nx / SPEC_CL, y0 = q * rows, x0 = q * cols;
    const int tile = spec_cl_tile(nx, ny), pitch = ny + 1;
    float2 *T = sm2, *A = T + tile, *B = A + tile, *twx = B + tile, *twy = twx + nx;
    for (int t = threadIdx.x; t < nx; t += blockDim.x) twx[t] = __ldg(sp.tw + P.twx + t);
    for (int t = threadIdx.x; t < ny; t += blockDim.x) twy[t] = __ldg(sp.tw + P.twy + t);
    __syncthreads();
    // y transforms of the conjugated solutions, columns x0 + sq, into T (column-major)
    const float2 *Cf = sp.C + P.coff;
    auto ldC = [&](int sq, int e) { return Cf[((long long)j * nx + x0 + sq) * ny + e]; };
    auto stT = [&](int sq, int e, float2 v) { T[sq * pitch + e] = v; };
    fft_pow2<false>(A, B, cols, P.ay.lg, 1, ny, twy, ldC, stT);
    cl.sync();
    // x transforms of rows y0 + sq (element x in block x / cols, column x % cols)
    // into the correction: the transform of conj(W) is conj(x_2j + i x_2j+1),
    // combined with the previous increment as k_spec_x
    float *xx = F.x + P.off;
    const long long plane = (long long)nx * ny;
    const SolveDev *Sf = d.solve + f;
    const float cw = d.force || Sf->cheb_w == 0.f ? 1.f : Sf->cheb_w;
    const float cm = d.force ? 0.f : Sf->cheb_m;
    auto ldT = [&](int sq, int e) -> float2 {
        const int p = e / cols, c = e - p * cols;
        return cl.map_shared_rank(T, p)[c * pitch + y0 + sq];
    };
    auto st = [&](int sq, int e, float2 v) {
        const long long yx = (long long)(y0 + sq) * nx + e, o = (long long)(2 * j + 1) * plane + yx;
        if (cm != 0.f) {
            xx[o] = cw * v.x + cm * xx[o];
            if (2 * j + 1 < M) xx[o + plane] = cw * -v.y + cm * xx[o + plane];
        } else {
            xx[o] = cw * v.x;
            if (2 * j + 1 < M) xx[o + plane] = cw * -v.y;
        }
        if (j == 0) xx[yx] = 0.f;                                        // first Dirichlet plane
        if (j == Mp - 1) xx[(long long)(M + 1) * plane + yx] = 0.f;      // last one
    };
    fft_pow2<false>(A, B, rows, P.ax.lg, 1, nx, twx, ldT, st);
    cl.sync();
    spec_finish(d);
}

}  // namespace cmsl
