// main_portal.x on GB300: the same command line, input files and outputs as
// the reference program (main_para.f90), with the node loop
// (main_para.f90:210-257) run by the library.
//
//   main_portal.x <input_file> <output_map> <pop> <grid> <mol> <dust>
//
// Outputs: <output_map>/pol_pops.dat (one line per node, rho^0_0 and
// rho^2_0 per level, main_para.f90:271-275); with extra_info = 1 also
// mag_field.dat (:158-167), the rate files spont_rates.dat, rad_rates.dat,
// col_rates.dat (:277-294) and rad_anis.dat (J^2_0 / J^0_0 per line,
// :296-300).
//
// Two inputs the reference leaves implicit are explicit here:
//   PORTAL_GVEC="gx gy gz"   the gauge vector (the reference draws it with an
//                            unseeded random_number, main_para.f90:172-176);
//                            default: drawn from seed 0
//   PORTAL_BVEC_FILE=path    per-node field directions (N lines of three
//                            numbers) instead of global_magfield /
//                            dipole_magfield, for clouds whose field those
//                            models cannot express (e.g. a uniform field)
//   PORTAL_DEVICE=n          CUDA device (default 0)
//   PORTAL_LAMBDA="tol [n]"  iterate the node loop to convergence (largest
//                            relative change of rho^0_0 per pass below tol,
//                            at most n passes, accelerated) before the pass
//                            whose results are written (no reference
//                            counterpart: the reference makes one pass)
//   PORTAL_POPS_BINARY=1     also write pol_pops.bin, a binary copy of
//                            pol_pops.dat that finish_portal.x reads instead
//                            of parsing the text (same values to the bit)
//   PORTAL_DUMP_INGESTED=dir write the ingested arrays (what the library
//                            receives) as .npy files into dir and stop
//                            before any device work
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "portal_gb300.h"
#include "portal_io.h"

using namespace portal_io;

static int fail(const std::string &m) {
    fprintf(stderr, "main_portal: %s\n", m.c_str());
    return 1;
}

// .npy (format 1.0) of a 1-D array
template <typename T>
static bool npy(const std::string &path, const std::vector<T> &v, const char *descr) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    std::string h = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': (" +
                    std::to_string(v.size()) + ",), }";
    while ((10 + h.size() + 1) % 64) h.push_back(' ');
    h.push_back('\n');
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    fwrite(magic, 1, 8, f);
    const unsigned short hl = (unsigned short)h.size();
    fputc(hl & 0xff, f);
    fputc(hl >> 8, f);
    fwrite(h.data(), 1, h.size(), f);
    fwrite(v.data(), sizeof(T), v.size(), f);
    return fclose(f) == 0;
}

static bool dump(const std::string &d, const Molecule &m, const Cloud &c, const std::vector<double> &bvec) {
    bool ok = true;
    ok &= npy(d + "/xyz.npy", c.xyz, "<f8") && npy(d + "/vel.npy", c.vel, "<f8");
    ok &= npy(d + "/b_all.npy", c.b_all, "<f8") && npy(d + "/temp_all.npy", c.temp_all, "<f8");
    ok &= npy(d + "/dust_p.npy", c.dust_p, "<f8") && npy(d + "/h2_dens.npy", c.h2_dens, "<f8");
    ok &= npy(d + "/ab_all.npy", c.ab_all, "<f8") && npy(d + "/lev_p.npy", c.lev_p, "<f8");
    ok &= npy(d + "/bvec.npy", bvec, "<f8") && npy(d + "/del_ne.npy", c.del_ne, "<i4");
    ok &= npy(d + "/del_num_ne.npy", c.del_num_ne, "<i4");
    ok &= npy(d + "/e_levs.npy", m.e_levs, "<f8") && npy(d + "/nu.npy", m.nu, "<f8");
    ok &= npy(d + "/A.npy", m.A, "<f8") && npy(d + "/Bij.npy", m.Bij, "<f8") && npy(d + "/kd_v.npy", m.kd_v, "<f8");
    ok &= npy(d + "/j_lev.npy", m.j_lev, "<i4") && npy(d + "/r_trans.npy", m.r_trans, "<i4");
    ok &= npy(d + "/c_trans.npy", m.c_trans, "<i4") && npy(d + "/C.npy", m.C, "<f8");
    ok &= npy(d + "/col_temps.npy", m.col_temps, "<f8");
    std::vector<double> sc = {c.tx, (double)c.bulk_node_num, (double)c.maxne, m.mass};
    ok &= npy(d + "/scalars.npy", sc, "<f8");
    return ok;
}

int main(int argc, char **argv) {
    if (argc < 7)
        return fail("usage: main_portal.x <input_file> <output_map> <pop> <grid> <mol> <dust>");
    const std::string input = argv[1], out = argv[2], pop = argv[3], grid = argv[4], mol = argv[5],
                      dust = argv[6];
    std::string err;
    MainInput in;
    if (!read_main_input(input, in, err)) return fail(err);
    if (in.star_mod != 0 && in.star_mod != 1) return fail("star_mod must be 0 or 1");
    Molecule m;
    Cloud c;
    // the neighbour lists are built on the device (portal_adj_list), by the
    // context the run then uses; PORTAL_HOST_NEIGHBOURS=1 builds them on the
    // host instead (the same lists); the dump of the ingested
    // arrays (PORTAL_DUMP_INGESTED) needs no device and builds them on the host
    const int dev = getenv("PORTAL_DEVICE") ? atoi(getenv("PORTAL_DEVICE")) : 0;
    portal_ctx *ctx = nullptr;
    const bool device_lists = !getenv("PORTAL_DUMP_INGESTED") && !getenv("PORTAL_HOST_NEIGHBOURS");
    if (device_lists && portal_create(&ctx, dev))
        return fail(std::string("portal_create: ") + portal_last_error(nullptr));
    const NeighbourBuilder on_device = [&](int N, const std::vector<int> &tets, int max_ne_temp, Cloud &cl,
                                           std::string &e) {
        int mx = 0;
        cl.del_ne.assign((size_t)N * max_ne_temp, 0);
        cl.del_num_ne.assign(N, 0);
        if (portal_adj_list(ctx, N, (long long)(tets.size() / 4), tets.data(), max_ne_temp, cl.del_ne.data(),
                            cl.del_num_ne.data(), &mx, nullptr)) {
            e = std::string("neighbour lists: ") + portal_last_error(ctx);
            return false;
        }
        cl.maxne = mx;
        cl.del_ne.resize((size_t)N * mx);  // main_para.f90:124-128: the first maxne columns
        return true;
    };
    if (!read_lime(pop, grid, mol, dust, 0.01, in.max_ne_temp, m, c, err, device_lists ? &on_device : nullptr))
        return fail(err);
    std::vector<double> bvec;
    if (const char *bf = getenv("PORTAL_BVEC_FILE")) {
        std::vector<double> rows;  // (N,3) column-major: N lines of 3 numbers
        if (!read_rows(bf, rows, c.node_num, 3, err)) return fail(err);
        bvec.resize(3 * (size_t)c.node_num);
        for (int i = 0; i < c.node_num; i++)
            for (int k = 0; k < 3; k++) bvec[3 * (size_t)i + k] = rows[(size_t)i + (size_t)c.node_num * k];
    } else {
        magfield(c, in.x1, in.x2, in.x3, in.x_dip, bvec);
    }
    double g[3];
    if (const char *gv = getenv("PORTAL_GVEC")) {
        if (sscanf(gv, "%lf %lf %lf", &g[0], &g[1], &g[2]) != 3) return fail("PORTAL_GVEC: three numbers");
        const double n = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        for (auto &v : g) v /= n;
    } else {
        gauge_vector(0, g);
    }
    if (const char *dd = getenv("PORTAL_DUMP_INGESTED")) {
        if (!dump(dd, m, c, bvec)) return fail(std::string("cannot write the dump into ") + dd);
        printf("main_portal: %d nodes (%d bulk), %d levels ingested into %s\n", c.node_num, c.bulk_node_num,
               m.nlev, dd);
        return 0;
    }
    if (!ctx && portal_create(&ctx, dev)) return fail(std::string("portal_create: ") + portal_last_error(nullptr));
    auto chk = [&](int r, const char *what) {
        if (r) {
            fprintf(stderr, "main_portal: %s: %s (%s)\n", what, portal_strerror(r), portal_last_error(ctx));
            portal_destroy(ctx);
            exit(1);
        }
    };
    chk(portal_set_molecule(ctx, m.nlev, m.j_lev.data(), m.e_levs.data(), m.r_num, m.r_trans.data(),
                            m.A.data(), m.nu.data(), m.Bij.data(), m.kd_v.data(), m.c_num, m.c_trans.data(),
                            m.c_temp, m.c_par, m.col_temps.data(), m.C.data()),
        "portal_set_molecule");
    chk(portal_set_cloud(ctx, c.node_num, c.bulk_node_num, c.nlev, c.xyz.data(), c.vel.data(), c.b_all.data(),
                         c.temp_all.data(), c.dust_p.data(), c.h2_dens.data(), c.ab_all.data(), c.lev_p.data(),
                         bvec.data(), c.maxne, c.del_ne.data(), c.del_num_ne.data(), c.tx),
        "portal_set_cloud");
    if (in.star_mod == 1)  // R_star in metres; X_star as read (main_para.f90:75, :122)
        chk(portal_set_star(ctx, 1, in.T_star, in.R_star, in.XYZ_star), "portal_set_star");
    long long nseg = 0;
    const double dx = (double)1e-6f;  // main_para.f90:135
    if (const char *li = getenv("PORTAL_LAMBDA")) {
        // iterate the node loop to convergence first (accelerated: local
        // operator + Ng every 4 passes); the pass below then starts from the
        // converged populations, so its outputs are those of the fixed point
        double tol = 1e-6;
        int max_iter = 500;
        if (sscanf(li, "%lf %d", &tol, &max_iter) < 1 || !(tol > 0.0) || max_iter < 1)
            return fail("PORTAL_LAMBDA: \"tol [max_iter]\"");
        int iters = 0;
        long long ns = 0;
        std::vector<double> res((size_t)max_iter);
        chk(portal_lambda_iterate(ctx, in.nth, in.nph, in.nvel, g, dx, in.n_depth, in.kmax, tol, max_iter, 4, 1,
                                  nullptr, nullptr, nullptr, &iters, res.data(), &ns),
            "portal_lambda_iterate");
        const double last = iters ? res[iters - 1] : 0.0;
        printf("main_portal: Lambda iteration, %d passes, last change %.3e%s\n", iters, last,
               last < tol ? "" : " (not converged)");
    }
    chk(portal_radiation_field(ctx, in.nth, in.nph, in.nvel, g, dx, in.n_depth, nullptr, nullptr, nullptr, &nseg),
        "portal_radiation_field");
    const int N = c.node_num, nlev = m.nlev;
    std::vector<double> pops((size_t)N * 2 * nlev), jj((size_t)N * m.r_num), rates;
    if (in.extra_info == 1) rates.resize((size_t)N * 3 * 2 * nlev);
    chk(portal_solve_se(ctx, in.kmax, nullptr, nullptr, pops.data(), rates.empty() ? nullptr : rates.data(),
                        jj.data(), nullptr),
        "portal_solve_se");
    portal_destroy(ctx);
    if (!write_rows(out + "/pol_pops.dat", pops, N, 2 * nlev)) return fail("cannot write " + out + "/pol_pops.dat");
    if (const char *pb = getenv("PORTAL_POPS_BINARY"))
        if (atoi(pb) == 1 && !write_sidecar(out + "/pol_pops.bin", pops, N, 2 * nlev))
            return fail("cannot write " + out + "/pol_pops.bin");
    if (in.extra_info == 1) {
        std::vector<double> mf((size_t)N * 6);
        for (int i = 0; i < N; i++)
            for (int k = 0; k < 3; k++) {
                mf[(size_t)i + (size_t)N * k] = c.xyz[3 * (size_t)i + k];
                mf[(size_t)i + (size_t)N * (3 + k)] = bvec[3 * (size_t)i + k];
            }
        if (!write_rows(out + "/mag_field.dat", mf, N, 6))
            return fail("cannot write the extra_info files");
        // pol_rates(N, 3, 2 nlev): one file per kind (main_para.f90:277-294)
        const char *names[3] = {"/spont_rates.dat", "/rad_rates.dat", "/col_rates.dat"};
        std::vector<double> one((size_t)N * 2 * nlev);
        for (int k = 0; k < 3; k++) {
            for (int cc = 0; cc < 2 * nlev; cc++)
                for (int i = 0; i < N; i++)
                    one[(size_t)i + (size_t)N * cc] = rates[(size_t)i + (size_t)N * (k + 3 * (size_t)cc)];
            if (!write_rows(out + names[k], one, N, 2 * nlev)) return fail("cannot write the extra_info files");
        }
        if (!write_rows(out + "/rad_anis.dat", jj, N, m.r_num)) return fail("cannot write the extra_info files");
    }
    printf("main_portal: %d nodes, %lld ray segments\n", c.bulk_node_num, nseg);
    return 0;
}
