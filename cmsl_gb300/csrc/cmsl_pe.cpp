// cmsl_pe.cpp -- the P-E loop campaign driver on libcmsl_gb.
//
// Same inputs, flow and outputs as the reference executable
// (HZO_Code_github/src/main.cu:361-506 and SetupAndRunSimulation :261-359):
//
//   cmsl_pe <offset_sims> <landau_pool> <phase_pool> [max_sims]
//           [--seed N] [--precision fp64|fp32] [--root DIR]
//
// reads <root>/inputs/InputParams, the Landau and phase pools, the structures
// <root>/inputs/struc1..N (gdata_<tag>.bin, gchar_<tag>.txt) and
// <root>/inputs/gnumb_<tag>.txt; writes <root>/OutputParams,
// <root>/microstructure.txt and <root>/output/sweepNNN.txt rows (appended, the
// reference's 12-column format).  Every simulation runs on the GPU through the
// C ABI.  Differences from the reference: the seed can be fixed (--seed); the
// initial FE polarisation noise comes from a seeded SplitMix64 stream instead
// of cuRAND; single-crystal Ps noise injection is not done.
#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "cmsl.h"
#include "cmsl_io.h"

namespace {

int die(const std::string &m)
{
    std::fprintf(stderr, "cmsl_pe: %s\n", m.c_str());
    return 1;
}

bool is_dir(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

struct SplitMix {
    uint64_t s;
    double next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
};

}  // namespace

int main(int argc, char **argv)
{
    std::vector<std::string> pos;
    long long seed = -1;
    int precision = CMSL_FP64;
    std::string root = ".";
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--seed" && i + 1 < argc) seed = std::atoll(argv[++i]);
        else if (a == "--precision" && i + 1 < argc) precision = std::string(argv[++i]) == "fp32" ? CMSL_FP32_REFINED : CMSL_FP64;
        else if (a == "--root" && i + 1 < argc) root = argv[++i];
        else pos.push_back(a);
    }
    if (pos.size() < 3)
        return die("usage: cmsl_pe <offset_sims> <landau_pool> <phase_pool> [max_sims] [--seed N] "
                   "[--precision fp64|fp32] [--root DIR]");
    int offset = std::atoi(pos[0].c_str());
    if (offset < 0) offset = 0;
    int max_sims = pos.size() >= 4 ? std::atoi(pos[3].c_str()) : 500;   // main.cu:379-384
    if (max_sims < 1) max_sims = 1;
    std::srand(seed >= 0 ? (unsigned)seed : (unsigned)(std::time(nullptr) + (unsigned)offset * 1234567u));

    cmsl_deck deck;
    if (cmsl_deck_read((root + "/inputs/InputParams").c_str(), &deck) != CMSL_OK) return die(cmsl_last_error());
    cmsl_deck_write_summary(&deck, (root + "/OutputParams").c_str());

    std::vector<cmsl_landau_set> pool(2000);
    int n_pool = 0;
    if (cmsl_landau_pool_read(pos[1].c_str(), pool.data(), (int)pool.size(), &n_pool) != CMSL_OK) return die(cmsl_last_error());
    std::vector<double> pa(20000), pf(20000), pd(20000);
    int n_phase = 0;
    if (cmsl_phase_pool_read(pos[2].c_str(), pa.data(), pf.data(), pd.data(), 20000, &n_phase) != CMSL_OK)
        return die(cmsl_last_error());
    if (n_pool < 1 || n_phase < 1) return die("empty Landau or phase pool");

    const std::string tag = deck.crystal_type;
    if (tag != "single" && tag != "poly") return die("invalid crystal_type");
    int zbc;
    if (std::string(deck.z_bc_type) == "diri") zbc = CMSL_DIRICHLET;
    else if (std::string(deck.z_bc_type) == "neu") zbc = CMSL_NEUMANN;
    else return die(std::string("unsupported z_bc_type: ") + deck.z_bc_type);
    int n_struct = 0;
    while (is_dir(root + "/inputs/struc" + std::to_string(n_struct + 1))) ++n_struct;
    if (n_struct == 0) return die("no inputs/struc1 folder found");
    const std::string outdir = root + "/output";
    mkdir(outdir.c_str(), 0755);

    const int nx = deck.nx, ny = deck.ny, nz = deck.nz;
    const long long N = (long long)nx * ny * nz;
    for (int sim = 0; sim < max_sims; ++sim) {
        const int sim_index = offset + sim + 1;
        const cmsl_landau_set &ls = pool[std::rand() % n_pool];               // main.cu:159-178
        const int pidx = std::rand() % n_phase;                              // main.cu:100-106
        const int sid = 1 + std::rand() % n_struct;                          // main.cu:478
        const std::string sdir = root + "/inputs/struc" + std::to_string(sid);
        int ng = 0;
        if (cmsl_grain_count((root + "/inputs/gnumb_" + tag + ".txt").c_str(), &ng) != CMSL_OK) return die(cmsl_last_error());
        if (ng > 8500) { std::fprintf(stderr, "skipping %s: %d grains\n", sdir.c_str(), ng); continue; }
        std::vector<int32_t> omega(N);
        std::vector<double> cent(3 * ng), euler(3 * ng), TR(9 * ng);
        if (cmsl_grain_read(sdir.c_str(), tag.c_str(), nx, ny, nz, ng, omega.data(), nullptr, cent.data(),
                            euler.data(), TR.data()) != CMSL_OK)
            return die(cmsl_last_error());

        // SetupAndRunSimulation: materials from the picked set and the deck
        cmsl_raw_material raw[3] = {};
        raw[CMSL_AFE] = {ls.afe[0], ls.afe[1], ls.afe[2], ls.afe[3], ls.afe[4], 0, deck.L_afe, deck.kappa_afe, deck.eps_afe};
        raw[CMSL_FE] = {ls.fe[0], ls.fe[1], ls.fe[2], ls.fe[3], ls.fe[4], 0, deck.L_fe, deck.kappa_fe, deck.eps_fe};
        raw[CMSL_DE] = {ls.de[0], 0.0, 0.0, 0.0, ls.de[1], 0, deck.L_de, deck.kappa_de, deck.eps_de};
        cmsl_material nd[3];
        cmsl_scales sc;
        if (cmsl_nondim(raw, ls.ref_type, deck.Eap, deck.delEap, nd, &sc) != CMSL_OK) return die(cmsl_last_error());

        // Init_Conf: per-layer fractions, grain -> material (reseeds rand())
        std::vector<double> fa(deck.n_layers, pa[pidx]), ff(deck.n_layers, pf[pidx]), fd(deck.n_layers, pd[pidx]);
        std::vector<double> centz(ng);
        for (int g = 0; g < ng; ++g) centz[g] = cent[3 * g + 2];
        std::vector<int32_t> gmat(ng);
        if (cmsl_assign_materials(nx, ny, nz, ng, omega.data(), centz.data(), deck.n_layers, deck.layer_counts,
                                  fa.data(), ff.data(), fd.data(), gmat.data()) != CMSL_OK)
            return die(cmsl_last_error());
        for (int g = 0; g < ng; ++g)
            if (gmat[g] < 0) gmat[g] = CMSL_FE;
        {   // microstructure.txt (init_conf.cu:302-308, generate.cu write_field)
            FILE *mf = std::fopen((root + "/microstructure.txt").c_str(), "w");
            if (mf) {
                for (int i = 0; i < nx; i++) {
                    for (int j = 0; j < ny; j++) {
                        for (int k = 0; k < nz; k++) {
                            const int h = gmat[omega[i + (long long)nx * (j + (long long)k * ny)]];
                            std::fprintf(mf, "%d\t%d\t%d\t%d\n", i, j, k, h);
                        }
                        std::fprintf(mf, "\n");
                    }
                    std::fprintf(mf, "\n");
                }
                std::fclose(mf);
            }
        }
        // initial P (init_conf.cu:14-66): FE Pm = 0.1 (2u - 1) on all components,
        // AFE Ps = 1, DE 0
        std::vector<double> P[6];
        for (auto &v : P) v.assign(N, 0.0);
        SplitMix rng{34635ull};
        for (long long c = 0; c < N; ++c) {
            const int m = gmat[omega[c]];
            const double r = 2.0 * rng.next() - 1.0;
            if (m == CMSL_FE) P[0][c] = P[1][c] = P[2][c] = 0.1 * r;
            else if (m == CMSL_AFE) P[3][c] = P[4][c] = P[5][c] = 1.0;
        }

        // the schedule of Evolve, with the optional pre-relax at E = 0
        int ns = 0, nr = 0;
        const int single = tag == "single";
        if (cmsl_evolve_schedule(sc.maxEz, sc.delEz, deck.num_steps, 1, single, sc.E0_ref, 100000000, nullptr,
                                 nullptr, &ns, nullptr, nullptr, &nr) != CMSL_OK)
            return die(cmsl_last_error());
        const int pre = deck.do_pre_relax ? 15000 : 0;                          // evolve.cu:171-211
        std::vector<double> Ez(ns, 0.0), rowE(nr);
        std::vector<int32_t> row(ns, -1), rowc(nr);
        cmsl_evolve_schedule(sc.maxEz, sc.delEz, deck.num_steps, 1, single, sc.E0_ref, 100000000, Ez.data(),
                             row.data(), &ns, rowE.data(), rowc.data(), &nr);

        cmsl_film_desc d = {};
        d.nx = nx; d.ny = ny; d.nz = nz; d.del_h = deck.del_h; d.del_t = deck.del_t;
        d.dep_flag = deck.dep_flag; d.zbc = zbc; d.eps_0_nd = sc.eps_0_nd;
        d.n_grains = ng; d.omega = omega.data(); d.grain_mat = gmat.data(); d.TR = TR.data();
        for (int q = 0; q < 3; ++q) d.mats[q] = nd[q];
        d.precision = precision; d.pcg_crit = CMSL_CRIT_REF;
        d.tol_abs = 1e-3; d.tol_rel = 1e-2; d.max_iter = 4000;                    // global.cu:140-144
        d.refine_tol = 1e-8; d.max_refine = 6; d.inner_tol = 1e-5; d.inner_max_iter = 2000; d.warm_start = 2;
        cmsl_film *film = nullptr;
        if (cmsl_film_create(&d, &film) != CMSL_OK) return die(cmsl_last_error());
        const double *Pp[6] = {P[0].data(), P[1].data(), P[2].data(), P[3].data(), P[4].data(), P[5].data()};
        cmsl_status st = cmsl_film_set_state(film, Pp, nullptr);
        if (st == CMSL_OK && pre > 0) {
            // stage A: pre-relax at E = 0, then the two midplane slices of
            // evolve.cu:202-210 (Psz of the relaxed state; Psz in the crystal
            // frame of the state the last pre-relax step started from)
            std::vector<double> Ez0((size_t)pre, 0.0), S[6], phi((size_t)N), loc((size_t)N);
            std::vector<int32_t> r0((size_t)pre, -1);
            double *Sp[6];
            for (int q = 0; q < 6; ++q) { S[q].resize((size_t)N); Sp[q] = S[q].data(); }
            if (pre > 1) st = cmsl_film_run(film, pre - 1, Ez0.data(), r0.data(), nullptr);
            if (st == CMSL_OK) st = cmsl_film_sync(film);
            if (st == CMSL_OK) st = cmsl_film_get_state(film, Sp, phi.data());
            if (st == CMSL_OK) st = cmsl_crystal_z(N, omega.data(), TR.data(), Sp[3], Sp[4], Sp[5], loc.data());
            if (st == CMSL_OK) st = cmsl_film_run(film, 1, Ez0.data(), r0.data(), nullptr);
            if (st == CMSL_OK) st = cmsl_film_sync(film);
            if (st == CMSL_OK) st = cmsl_film_get_state(film, Sp, phi.data());
            if (st == CMSL_OK) st = cmsl_midplane_slice_write("slice_E0_midplane.dat", Sp[5], nx, ny, nz);
            if (st == CMSL_OK) st = cmsl_midplane_slice_write("slice_E0_midplane_local.dat", loc.data(), nx, ny, nz);
        }
        if (st == CMSL_OK) st = cmsl_film_run(film, (int)Ez.size(), Ez.data(), row.data(), nullptr);
        if (st == CMSL_OK) st = cmsl_film_sync(film);
        std::vector<double> rows((size_t)nr * CMSL_ROW_WIDTH);
        if (st == CMSL_OK && nr > 0) st = cmsl_film_get_rows(film, 0, nr, rows.data());
        if (st != CMSL_OK) {
            const std::string m = cmsl_last_error();
            cmsl_film_destroy(film);
            return die(m);
        }
        cmsl_film_destroy(film);

        char name[64];
        std::snprintf(name, sizeof name, "/sweep%03d.txt", sim_index);
        FILE *fo = std::fopen((outdir + name).c_str(), "a");
        if (!fo) return die("cannot open " + outdir + name);
        const double Es = sc.E0_ref / 1.0e+08, Ps = sc.P0_ref * 100.0;       // evolve.cu:117-118
        for (int r = 0; r < nr; ++r) {
            const double *v = rows.data() + (size_t)r * CMSL_ROW_WIDTH;
            std::fprintf(fo, "%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%le\t%d\n", rowE[r] * Es, v[0] * Ps,
                         v[1] * Ps, v[2] * Ps, v[3] * Ps, v[4] * Ps, v[5], v[6] * Ps, v[7], v[8] * Ps, v[9],
                         rowc[r] + pre);
        }
        std::fclose(fo);
        std::printf("simulation %d: %d steps, %d rows -> %s\n", sim_index, pre + (int)Ez.size(), nr,
                    (outdir + name).c_str());
    }
    return 0;
}
