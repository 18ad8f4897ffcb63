// finish_portal.x on GB300: the same command line, input file and outputs as
// the reference program (para_finish.f90), with the pixel loops
// (para_finish.f90:382-448) or the per-node loops (:287-320) run by the
// library.
//
//   finish_portal.x <input_file> <output_map> <pop> <grid> <mol> <dust>
//
// Reads <output_map>/pol_pops.dat (para_finish.f90:222-240; or its binary
// sidecar pol_pops.bin when that is present and not older) and writes, per
// line i and inclination j, inc{j}-trans{i}-im_{i,q,u,tau}.fits and the
// centre-channel dust maps inc{j}-trans{i}-dust_{i,q,u,tau}.fits
// (para_finish.f90:460-652), I, Q and U scaled by I_to_T = 3.255e39/nu0^2.
// With fits = 0 the .dat maps of the same routine are written instead: one
// file per channel of FP64 rows, the dust maps included.
// pix_mod = 0 (para_finish.f90:245-350): per inclination j the node positions
// inc{j}-xy.dat, then per line i, inclination j and channel k the per-node
// rows inc{j}-trans{i}-vel{k}-im.dat (I_to_T I, I_to_T Q, I_to_T U, tau); the
// numbers in the names are written like Fortran's i2.2 ("**" above 99).
// PORTAL_BVEC_FILE and PORTAL_DEVICE as for main_portal.x.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "portal_gb300.h"
#include "portal_io.h"

using namespace portal_io;

static int fail(const std::string &m) {
    fprintf(stderr, "finish_portal: %s\n", m.c_str());
    return 1;
}

// Fortran's i2.2 edit descriptor: two digits, "**" when the value needs more
static std::string i2(int v) {
    if (v < 0 || v > 99) return "**";
    char b[4];
    snprintf(b, sizeof b, "%02d", v);
    return b;
}

// pix_mod = 0: para_finish.f90:245-350
static int node_maps(portal_ctx *ctx, const FinishInput &in, const std::string &out, const Cloud &c,
                     const std::vector<double> &pops, double nu0, double dx) {
    const int nb = c.bulk_node_num, nch = 2 * in.nvel + 1, nl = in.nlevels;
    const double I_to_T = 3.255e39 / (nu0 * nu0);  // :333
    const size_t cube = (size_t)nb * nch * nl;
    std::vector<float> q[4];
    for (auto &v : q) v.assign(cube, 0.f);
    std::vector<double> xy(2 * (size_t)nb), rows;
    for (int j = 0; j < in.nincs; j++) {
        const int r = portal_image_nodes(ctx, pops.data(), nl, in.l1.data(), in.l2.data(), in.th_inc[j], in.ph_az[j],
                                         in.nvel, in.dvel, in.v0, 0.15, dx, in.n_depth_rt, xy.data(), q[0].data(),
                                         q[1].data(), q[2].data(), q[3].data(), nullptr, nullptr, nullptr, nullptr,
                                         nullptr);
        if (r) return fail(std::string("portal_image_nodes: ") + portal_strerror(r) + " (" + portal_last_error(ctx) + ")");
        rows.resize(2 * (size_t)nb);
        for (int n = 0; n < nb; n++) {
            rows[n] = xy[2 * (size_t)n];
            rows[(size_t)nb + n] = xy[2 * (size_t)n + 1];
        }
        std::string name = out + "/inc" + i2(j + 1) + "-xy.dat";
        if (!write_rows(name, rows, nb, 2)) return fail("cannot write " + name);
        rows.resize(4 * (size_t)nb);
        for (int i = 0; i < nl; i++)
            for (int k = 0; k < nch; k++) {
                const size_t base = (size_t)nb * ((size_t)k + (size_t)nch * i);
                for (int n = 0; n < nb; n++) {
                    rows[n] = I_to_T * (double)q[0][base + n];
                    rows[(size_t)nb + n] = I_to_T * (double)q[1][base + n];
                    rows[2 * (size_t)nb + n] = I_to_T * (double)q[2][base + n];
                    rows[3 * (size_t)nb + n] = (double)q[3][base + n];
                }
                name = out + "/inc" + i2(j + 1) + "-trans" + i2(i + 1) + "-vel" + i2(k + 1) + "-im.dat";
                if (!write_rows(name, rows, nb, 4)) return fail("cannot write " + name);
            }
    }
    printf("finish_portal: %d inclinations, %d lines, %d nodes, %d channels\n", in.nincs, nl, nb, nch);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 7)
        return fail("usage: finish_portal.x <input_file> <output_map> <pop> <grid> <mol> <dust>");
    const std::string input = argv[1], out = argv[2], pop = argv[3], grid = argv[4], mol = argv[5],
                      dust = argv[6];
    std::string err;
    FinishInput in;
    if (!read_finish_input(input, in, err)) return fail(err);
    if (in.star_mod != 0 && in.star_mod != 1) return fail("star_mod must be 0 or 1");
    Molecule m;
    Cloud c;
    // the neighbour lists are built on the device (portal_adj_list), by the
    // context the run then uses; PORTAL_HOST_NEIGHBOURS=1 builds them on the
    // host instead (the same lists)
    const int dev = getenv("PORTAL_DEVICE") ? atoi(getenv("PORTAL_DEVICE")) : 0;
    portal_ctx *ctx = nullptr;
    const bool device_lists = !getenv("PORTAL_HOST_NEIGHBOURS");
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
        std::vector<double> rows;
        if (!read_rows(bf, rows, c.node_num, 3, err)) return fail(err);
        bvec.resize(3 * (size_t)c.node_num);
        for (int i = 0; i < c.node_num; i++)
            for (int k = 0; k < 3; k++) bvec[3 * (size_t)i + k] = rows[(size_t)i + (size_t)c.node_num * k];
    } else {
        magfield(c, in.x1, in.x2, in.x3, in.x_dip, bvec);
    }
    const int N = c.node_num, nlev = m.nlev;
    std::vector<double> pops;
    // the binary sidecar main_portal.x writes with PORTAL_POPS_BINARY=1, when it
    // is current; else the text file
    if (read_sidecar(out + "/pol_pops.bin", out + "/pol_pops.dat", pops, N, 2 * nlev))
        printf("finish_portal: populations from pol_pops.bin\n");
    else if (!read_rows(out + "/pol_pops.dat", pops, N, 2 * nlev, err))
        return fail(err);
    if (!ctx && portal_create(&ctx, dev)) return fail(std::string("portal_create: ") + portal_last_error(nullptr));
    auto chk = [&](int r, const char *what) {
        if (r) {
            fprintf(stderr, "finish_portal: %s: %s (%s)\n", what, portal_strerror(r), portal_last_error(ctx));
            portal_destroy(ctx);
            exit(1);
        }
    };
    chk(portal_set_molecule(ctx, m.nlev, m.j_lev.data(), m.e_levs.data(), m.r_num, m.r_trans.data(),
                            m.A.data(), m.nu.data(), m.Bij.data(), m.kd_v.data(), m.c_num, m.c_trans.data(),
                            m.c_temp, m.c_par, m.col_temps.data(), m.C.data()),
        "portal_set_molecule");
    chk(portal_set_cloud(ctx, N, c.bulk_node_num, nlev, c.xyz.data(), c.vel.data(), c.b_all.data(),
                         c.temp_all.data(), c.dust_p.data(), c.h2_dens.data(), c.ab_all.data(), c.lev_p.data(),
                         bvec.data(), c.maxne, c.del_ne.data(), c.del_num_ne.data(), c.tx),
        "portal_set_cloud");
    if (in.star_mod == 1)  // R_star in metres; X_star as read (para_finish.f90:116, :187)
        chk(portal_set_star(ctx, 1, in.T_star, in.R_star, in.XYZ_star), "portal_set_star");
    const int npx = 2 * in.im_pix + 1, nch = 2 * in.nvel + 1, nl = in.nlevels;
    // every line takes the frequency of the last (l1, l2) pair (para_finish.f90:173-175)
    const double nu0 = m.e_levs[in.l2[nl - 1] - 1] - m.e_levs[in.l1[nl - 1] - 1];
    const double dx = (double)1e-4f;  // para_finish.f90:201
    if (in.pix == 0) {
        const int r = node_maps(ctx, in, out, c, pops, nu0, dx);
        portal_destroy(ctx);
        return r;
    }
    const size_t cube = (size_t)npx * npx * nch * nl;
    std::vector<float> q[8];
    for (auto &v : q) v.assign(cube, 0.f);
    const double I_to_T = 3.255e39 / (nu0 * nu0);
    const double pi = std::acos(-1.0);
    const double ang = -180.0 * std::asin(2.0 * in.im_size * c.tx / in.distance) / (pi * (in.im_pix * 2 + 1));
    for (int j = 0; j < in.nincs; j++) {
        chk(portal_image(ctx, pops.data(), nl, in.l1.data(), in.l2.data(), in.th_inc[j], in.ph_az[j], in.nvel,
                         in.dvel, in.v0, in.im_pix, in.im_size, 0.15, dx, in.n_depth_rt, q[0].data(), q[1].data(),
                         q[2].data(), q[3].data(), q[4].data(), q[5].data(), q[6].data(), q[7].data(), nullptr),
            "portal_image");
        for (int i = 0; i < nl; i++) {
            const char *names[8] = {"im_i", "im_q", "im_u", "im_tau", "dust_i", "dust_q", "dust_u", "dust_tau"};
            for (int k = 0; k < 8; k++) {
                const bool dustmap = k >= 4;
                const bool scale = (k % 4) != 3;
                // the value the reference forms, I_to_T times the Stokes value
                // (para_finish.f90:477-480, :583-586)
                auto val = [&](size_t p, int ch) {
                    const double v = q[k][p + (size_t)npx * npx * (ch + (size_t)nch * i)];
                    return scale ? I_to_T * v : v;
                };
                if (in.fits == 1) {
                    // REAL*4 cubes; the dust maps hold the centre channel only (:592-613)
                    const int nv = dustmap ? 1 : nch;
                    std::vector<float> a((size_t)npx * npx * nv);
                    for (int c3 = 0; c3 < nv; c3++) {
                        const int ch = dustmap ? in.nvel : c3;
                        for (size_t p = 0; p < (size_t)npx * npx; p++) a[p + (size_t)npx * npx * c3] = (float)val(p, ch);
                    }
                    const std::string name = out + "/inc" + i2(j + 1) + "-trans" + i2(i + 1) + "-" + names[k] + ".fits";
                    if (!write_fits(name, a.data(), npx, nv, (float)nu0, (float)ang, (float)(in.im_pix + 1),
                                    (float)(-ang), (float)(in.im_pix + 1), (float)in.dvel, (float)(in.nvel + 1),
                                    0.f, 0.f, 0.f))
                        return fail("cannot write " + name);
                } else {
                    // list-directed rows of FP64 values, one file per channel, the dust
                    // maps too (:513-545, :619-650)
                    std::vector<double> rows((size_t)npx * npx);
                    for (int c3 = 0; c3 < nch; c3++) {
                        const std::string name = out + "/inc" + i2(j + 1) + "-trans" + i2(i + 1) + "-vel" + i2(c3 + 1) +
                                                 "-" + names[k] + ".dat";
                        for (size_t p = 0; p < rows.size(); p++) rows[p] = val(p, c3);
                        if (!write_rows(name, rows, npx, npx)) return fail("cannot write " + name);
                    }
                }
            }
        }
    }
    portal_destroy(ctx);
    printf("finish_portal: %d inclinations, %d lines, %dx%d pixels, %d channels\n", in.nincs, nl, npx, npx, nch);
    return 0;
}
