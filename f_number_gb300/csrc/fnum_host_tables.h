// Host-side tables and checks shared by the plan path (fnum_host.cpp) and the
// allocation-free entry point (fnum_noalloc.cu): the DFT order and band, the
// F table, the geometry and transmit tables the kernels read, and the argument
// checks of the plane-wave gateway.  One definition serves both, so a change to
// a table or a check reaches both entry points.  Host code only.
#pragma once
#include <vector>

#include "../../include/fnum.h"
#include "fnum_internal.h"

namespace fnum {

// DFT order, band bins and the phase constants of +cuda/gpu_bf_das_pw_rf.cu:494-556
struct Band {
  int N, k_lb, k_ub, K;
  double coef, add, M;
};

// geometry tables of both plan kinds (layouts as in PWDev / SADev)
struct GeomTables {
  std::vector<dfl> col_u, col_p, col_m, row_u2, row_p, el_u, el_m, el_lb, el_ub;
  std::vector<int> col_emid;
  std::vector<float> px_f, pz_f, ctr_f, lb_f, ub_f;
};

dfl to_df(double v);
// MEX band (N_dft padded with positions_z[1]); das_pw.m band (padded with positions_z[0])
int compute_band(const double* pz, int nz, int nt, int ne, double fs, double width, double pitch, double c,
                 const double* fb, double t0, Band* b);
int compute_band_m(const double* pz, int nt, int ne, double fs, double pitch, double c, const double* fb, double t0,
                   Band* b);
// F per band bin from the class parameters or caller values; err = status for invalid values
int band_f_table(const fnum_f_number* fn, const double* values, int n_values, const Band& b, double pitch,
                 double fs, double c, int err, std::vector<double>& F);
// F non-decreasing over the band (values at or below FLT_EPSILON count as 0)
bool f_monotone(const std::vector<double>& F);
// 1 / (2F) per bin in double-float; hi < 0 marks F <= FLT_EPSILON (full aperture)
void g_table(const std::vector<double>& F, std::vector<dfl>& g);
void build_geometry(const double* px, int nx, const double* pz, int nz, int ne, double width, double pitch,
                    double Ku, double M, GeomTables& g);
// per-angle transmit tables: ax[a][i] = K_u e_x (x_i - x_ref) + t0 / N, az[a][j] = K_u e_z z_j
void build_tx_tables(const double* px, int nx, const double* pz, int nz, const double* angles, int na, double Ku,
                     double M, double pitch, double t0, int N, std::vector<dfl>& ax, std::vector<dfl>& az);
// plane-wave gateway checks in the order and with the identifiers of gpu_bf_das_pw_rf.cu:126-485
int check_pw(const fnum_pw_desc* d, const double* angles, int na);

}  // namespace fnum
