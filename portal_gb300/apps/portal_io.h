// File formats of PORTAL's two executables: the input files, LIME's
// grid.vtk / .pop, LAMDA molecule files, the dust table, pol_pops.dat and the
// FITS cubes.  Readers follow the reference's own read statements (Fortran
// list-directed semantics), so that every file the reference accepts is read
// into the same values.
#pragma once

#include <functional>
#include <string>
#include <vector>

namespace portal_io {

// Fortran list-directed reading of one file: read(u,*) with an empty list
// skips one record; read(u,*) v1,...,vn takes values from the next record and,
// when it runs out, from the following ones, then drops the rest of the last
// record used.  Separators are blanks and commas; r*c repeat counts expand;
// D exponents are accepted.
class ListReader {
public:
    explicit ListReader(const std::string &path);
    bool ok() const { return ok_; }
    bool skip();
    bool read(std::vector<std::string> &out, size_t n);
    bool read_doubles(std::vector<double> &out, size_t n);
    bool read_ints(std::vector<int> &out, size_t n);
    const std::string &path() const { return path_; }
    // Up to n_rec consecutive reads of n values each into out (n_rec * n):
    // the same values as n_rec calls of read_doubles / read_ints.  When every
    // record is one line of exactly n plain numbers (the form LIME and the
    // reference's writers produce), the lines are parsed by `threads` threads
    // at once; otherwise the records are read one by one.  Returns the number
    // of records read (fewer than n_rec only at the end of the file).
    size_t read_block_doubles(double *out, size_t n_rec, size_t n, int threads);
    size_t read_block_ints(int *out, size_t n_rec, size_t n, int threads);

private:
    bool next_record();
    template <typename T>
    size_t read_block(T *out, size_t n_rec, size_t n, int threads);
    std::string path_;
    std::string buf_;                   // the whole file
    std::vector<size_t> lbeg_, lend_;   // line extents in buf_ (no line end characters)
    size_t line_ = 0;
    std::vector<std::string> toks_;
    size_t pos_ = 0;
    bool ok_ = false;
};

// threads for the bulk readers: PORTAL_THREADS, else the hardware's
int io_threads();

double to_double(const std::string &tok);
int to_int(const std::string &tok);

struct MainInput {                    // main_para.f90:72-80
    int star_mod = 0;
    double T_star = 0, R_star = 0, XYZ_star[3] = {0, 0, 0};
    int nth = 0, nph = 0, nvel = 0;
    double x1 = 0, x2 = 0, x3 = 0, x_dip = 0;
    int kmax = 0, extra_info = 0, max_ne_temp = 0, n_depth = 0;
};
struct FinishInput {                  // para_finish.f90:88-122
    int nlevels = 0;
    std::vector<int> l1, l2;
    int nincs = 0;
    std::vector<double> th_inc, ph_az;
    int nvel = 0;
    double dvel = 0, v0 = 0;
    int star_mod = 0;
    double T_star = 0, R_star = 0, XYZ_star[3] = {0, 0, 0};
    double x1 = 0, x2 = 0, x3 = 0, x_dip = 0;
    int kmax = 0, extra_info = 0, pix = 0, im_pix = 0;
    double im_size = 0;
    int fits = 0;
    double distance = 0;
    int max_ne_temp = 0, n_depth_rt = 0;
};
bool read_main_input(const std::string &path, MainInput &in, std::string &err);
bool read_finish_input(const std::string &path, FinishInput &in, std::string &err);

// The molecule and cloud in the state eat_lime_no_delaunay
// (eat_lime.f90:71-313) leaves them, plus main_para.f90:119-120 (Hz) and
// :124-133, :178-185 (compacted neighbours, degeneracies, t_Bij).
struct Molecule {
    int nlev = 0, r_num = 0, c_num = 0, c_temp = 0, c_par = 0;
    double mass = 0;
    std::vector<int> j_lev, r_trans, c_trans;        // (2,n) (lower, upper) 1-based
    std::vector<double> e_levs, A, nu, Bij, kd_v, col_temps, C;  // C(c_temp,c_num,c_par)
};
struct Cloud {
    int node_num = 0, bulk_node_num = 0, nlev = 0, maxne = 0;
    double tx = 0;
    std::vector<double> xyz, vel, b_all, temp_all, dust_p, h2_dens, ab_all, lev_p;  // Fortran layouts
    std::vector<int> del_ne, del_num_ne;   // del_ne(N,maxne) column-major, 1-based
};
// Builds del_ne / del_num_ne / maxne of a cloud of N nodes from its
// tetrahedra (4 vertices each, 0-based as grid.vtk lists them): the step of
// adj_list_no_delaunay (miscellaneous.f90:910-1015).  Returns false with err
// set on failure.
using NeighbourBuilder = std::function<bool(int N, const std::vector<int> &tets, int max_ne_temp, Cloud &c,
                                            std::string &err)>;
// build_neighbours: the construction of the neighbour lists, or null for the
// host's (parallel CSR + per-node sort / unique)
bool read_lime(const std::string &pop, const std::string &grid, const std::string &mol,
               const std::string &dust, double dust_ii_gas, int max_ne_temp, Molecule &m, Cloud &c,
               std::string &err, const NeighbourBuilder *build_neighbours = nullptr);

// global_magfield / dipole_magfield miscellaneous.f90:553-641
void magfield(const Cloud &c, double x1, double x2, double x3, double x_dip, std::vector<double> &bvec);

// gvec: three uniform numbers normalised (main_para.f90:172-176), drawn from
// a seeded generator
void gauge_vector(unsigned long long seed, double g[3]);

// pol_pops.dat: one line per node, 2*nlev values (main_para.f90:271-275),
// each as printf's " %24.17E" (17 significant digits: read back, the same
// doubles); formatted in parallel, byte-identical to the printf loop
bool write_rows(const std::string &path, const std::vector<double> &colmajor, int rows, int cols);
bool read_rows(const std::string &path, std::vector<double> &colmajor, int rows, int cols, std::string &err);

// Binary sidecar of pol_pops.dat (no reference counterpart): the magic
// "PORTALPP", rows and cols as little-endian int32, then the rows x cols
// doubles column-major -- the array pol_pops(N, 2 nlev) itself, the same
// values the text file holds to the last bit.
bool write_sidecar(const std::string &path, const std::vector<double> &colmajor, int rows, int cols);
// Reads the sidecar when it exists, has the expected shape and is not older
// than the text file it accompanies; false (and cm untouched) otherwise.
bool read_sidecar(const std::string &path, const std::string &text_path, std::vector<double> &colmajor, int rows,
                  int cols);

// FITS primary HDU, BITPIX -32, NAXIS 3, keywords of writeimage
// fits_writing.f90:1-159; array (npix, npix, nvel) column-major
bool write_fits(const std::string &path, const float *array, int npix, int nvel, float restfreq,
                float cdelt1, float crpix1, float cdelt2, float crpix2, float cdelt3, float crpix3,
                float crval1, float crval2, float crval3);

}  // namespace portal_io
