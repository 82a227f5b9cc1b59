// md_io.cpp -- the reference's text output files, written from host arrays:
// saveData, WriteCoords2TXT, WriteData2TXT and ExportDiffVis
// (src/postprocessing.cpp:15-32, 82-133, 222-231 of MD_Sim_Wolfschwenger) and
// the m_z / time exports at the end of RunSimulation (src/simulation.cpp:532-536).
//
// The reference streams Eigen matrices with the default IOFormat: the
// stream's precision (6 significant digits, %g style), every coefficient
// right-aligned to the width of the widest one in the matrix, one space
// between coefficients, one row per line; saveData then adds "\n" and endl,
// so each matrix is followed by one empty line.  A file is truncated when the
// time label passed to saveData is exactly 0 and appended to otherwise.  The
// writers below produce those bytes from plain arrays (no Eigen).
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/md_gb300.h"
#include "md_err.h"
#include "md_host.h"

namespace {

// One coefficient as `std::ostream << double` prints it by default.
std::string coeff_text(double v) {
  std::ostringstream s;
  s << v;
  return s.str();
}

// rows x cols matrix, element (i, j) at a[i + j * rows] (column-major) or
// a[i * cols + j] (row-major).
void print_matrix(std::ostream& os, const double* a, int64_t rows, int64_t cols, bool col_major) {
  if (rows <= 0 || cols <= 0) return;
  auto at = [&](int64_t i, int64_t j) { return col_major ? a[i + j * rows] : a[i * cols + j]; };
  std::vector<std::string> txt((size_t)(rows * cols));
  size_t width = 0;
  for (int64_t i = 0; i < rows; i++)
    for (int64_t j = 0; j < cols; j++) {
      std::string& t = txt[(size_t)(i * cols + j)];
      t = coeff_text(at(i, j));
      width = std::max(width, t.size());
    }
  for (int64_t i = 0; i < rows; i++) {
    for (int64_t j = 0; j < cols; j++) {
      const std::string& t = txt[(size_t)(i * cols + j)];
      if (j) os << ' ';
      for (size_t k = t.size(); k < width; k++) os << ' ';
      os << t;
    }
    if (i < rows - 1) os << '\n';
  }
}

int save_data(const std::string& path, const double* a, int64_t rows, int64_t cols, bool col_major, double tInt) {
  std::ofstream f(path, tInt == 0 ? (std::ios::out | std::ios::trunc) : (std::ios::out | std::ios::app));
  if (!f.is_open()) return set_err(nullptr, MD_ERR_INVALID, "cannot open %s for writing", path.c_str());
  print_matrix(f, a, rows, cols, col_major);
  f << "\n" << std::endl;
  if (!f) return set_err(nullptr, MD_ERR_INVALID, "write to %s failed", path.c_str());
  return MD_OK;
}

std::string join(const char* dir, const char* name) {
  if (!dir || !*dir) return name;
  std::string d(dir);
  if (d.back() != '/') d += '/';
  return d + name;
}

}  // namespace

extern "C" {

int md_write_matrix_txt(const char* path, const double* a, int64_t rows, int64_t cols, int col_major, double tInt) {
  if (!path || (!a && rows * cols > 0) || rows < 0 || cols < 0)
    return set_err(nullptr, MD_ERR_INVALID, "md_write_matrix_txt: bad argument");
  return save_data(path, a, rows, cols, col_major != 0, tInt);
}

int md_write_coords_txt(const char* path, int64_t n, const double* pos, const double* mm, const double* ea,
                        double tInt) {
  if (!path || n < 1 || !pos || !mm || !ea) return set_err(nullptr, MD_ERR_INVALID, "md_write_coords_txt: bad argument");
  // columns x y z | m_x m_y m_z | n_x n_y n_z | time label in row 0, zeros below
  std::vector<double> res((size_t)(10 * n), 0.0);
  const double* src[3] = {pos, mm, ea};
  for (int b = 0; b < 3; b++)
    for (int c = 0; c < 3; c++)
      std::copy(src[b] + c * n, src[b] + (c + 1) * n, res.begin() + (3 * b + c) * n);
  res[(size_t)(9 * n)] = tInt;
  return save_data(path, res.data(), n, 10, true, tInt);
}

int md_write_data_txt(const char* path, const md_config* cfg, int64_t n, const double* rMag, const double* rHydr,
                      double lBox) {
  if (!path || !cfg || n < 1 || !rMag || !rHydr)
    return set_err(nullptr, MD_ERR_INVALID, "md_write_data_txt: bad argument");
  const md_config& c = *cfg;
  // column 2 (src/postprocessing.cpp:112-133); rows beyond n are dropped
  const double meta[22] = {lBox,
                           (double)mdh::numb_part(&c),
                           c.magFluxDens,
                           c.satMag,
                           c.temp,
                           c.tMag,
                           c.tRelax,
                           c.tEnd,
                           c.volFrac,
                           (double)c.INIT_CONFIG_ROT,
                           (double)c.INIT_CONFIG_TRANS,
                           (double)c.seed,
                           c.anisEn,
                           c.densSurfMol,
                           c.effLenSurfMol,
                           c.hamaker,
                           c.z_valency,
                           c.epsilon_r,
                           c.gamma_0,
                           c.absTol,
                           c.errTolEwald,
                           c.errTolSR};
  std::vector<double> res((size_t)(3 * n), 0.0);
  std::copy(rHydr, rHydr + n, res.begin());
  std::copy(rMag, rMag + n, res.begin() + n);
  for (int64_t i = 0; i < std::min<int64_t>(n, 22); i++) res[(size_t)(2 * n + i)] = meta[i];
  return save_data(path, res.data(), n, 3, true, 0.0);
}

int md_export_records_txt(const char* dir, const double* obs, int64_t count, double tInt, int64_t steps) {
  if ((!obs && count > 0) || count < 0 || steps < 1)
    return set_err(nullptr, MD_ERR_INVALID, "md_export_records_txt: bad argument");
  const double dtMean = tInt / (double)steps;
  int st = save_data(join(dir, "dtMean.txt"), &dtMean, 1, 1, true, 0.0);
  // record columns {t, mz, MSDx, MSDy, MSDz, Pxy, Pxz, Pyz}
  const char* names[8] = {"t.txt", "mz.txt", "MSDx.txt", "MSDy.txt", "MSDz.txt", "Pxy.txt", "Pxz.txt", "Pyz.txt"};
  const int order[8] = {5, 6, 7, 2, 3, 4, 1, 0};  // the reference's write order
  std::vector<double> col((size_t)count);
  for (int q = 0; q < 8 && st == MD_OK; q++) {
    const int k = order[q];
    for (int64_t i = 0; i < count; i++) col[(size_t)i] = obs[i * 8 + k];
    st = save_data(join(dir, names[k]), col.data(), count, 1, true, 0.0);
  }
  return st;
}

}  // extern "C"
