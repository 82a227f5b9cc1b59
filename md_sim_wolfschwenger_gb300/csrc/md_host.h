// md_host.h -- host-side logic shared by the library and the drop-in
// executable: configuration (INI) handling, the Ewald error model, the
// k-vector segment list, the cell-grid choice and particle properties.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/md_gb300.h"
#include "md_types.h"

namespace mdh {

// ------------------------------------------------------- configuration
void config_defaults(md_config* c);
void config_derive(md_config* c);
// Returns MD_OK or MD_ERR_CONFIG (message in *err).
int config_load_ini(const char* path, md_config* c, std::string* err);
int64_t numb_part(const md_config* c);

// ----------------------------------------------------- particle props
struct Props {
  std::vector<double> rMag, rHydr, volMag, volHydr, magMom, zetaRot, zetaTrans, velEa1, velEa2;
  double lBox = 0, muMax = 0, rCutSR = 0, vis = 0;
};
// InitParticleProps derived quantities + box length + InitCutOffSR.
// rHydr may be empty (then rMag + dShell, or the Rosensweig equivalent
// diameter with coating potentials).  Returns MD_OK / MD_ERR_INVALID.
int make_props(const md_config& c, const double* rMag, const double* rHydr, int64_t n, Props* p,
               std::string* err);
double integral_eff_diameter(const md_config& c, double dMag);
// DefThermFluct scale factors for a step dt.
void noise_scales(const md_config& c, const Props& p, double dt, std::vector<double>* sT,
                  std::vector<double>* sB, std::vector<double>* sF);

// ------------------------------------------------------------ Ewald
struct EwaldModel {
  double M = 0, fAl = 0, tAl = 0, L = 0, n = 0;
};
EwaldModel ewald_model(const md_config& c, const Props& p);
double fun_real_error(const md_config& c, const EwaldModel& m, double alpha, double rc);
double fun_rez_error(const md_config& c, const EwaldModel& m, double alpha, double kc);
// alpha (first root in alpha) and unrounded kc for the cutoff rc.
bool ewald_for_rc(const md_config& c, const EwaldModel& m, double rc, double* alpha, double* kc_raw);
// Predicted RMS force / torque error relative to the contact values
// (src/interaction.cpp:313-323).
void predicted_errors(const md_config& c, const EwaldModel& m, double alpha, double rc, double kc,
                      double* errF, double* errT);
// Cost-model choice of rc (box fraction in [0.08, 0.5]) for n particles.
// kc_tc: largest kc the tensor-core k space takes (0: none).
double choose_rc(const md_config& c, const EwaldModel& m, int64_t n, double* alpha, int64_t* kc, int kc_tc);
double model_cost(double rc_box, int64_t kc, int64_t n, int kc_tc);

// ------------------------------------------------------ k-vector list
struct KList {
  std::vector<md::KSeg> seg;   // length-sorted (structure factor)
  std::vector<int> koff;
  std::vector<double> ek;
  // scatter layout: whole k rows (split evenly above kScatSeg), each padded
  // to a multiple of 4, in row order
  std::vector<md::KSeg> rseg;
  std::vector<int> rowpos;     // sorted padded k -> scatter-layout k (-1: padding)
  std::vector<int> chunks;     // pairs (first row segment, first row k), nchk + 1 pairs
  int nchk = 0;
  int nk_scat = 0;             // length of the scatter layout
  std::vector<int> kx, ky, kz;  // per padded k (padding k's are marked by kreal = 0)
  std::vector<char> kreal;
  int nk = 0, nk_real = 0;
};
KList build_klist(int kc, double w);

// ------------------------------------------------------ initial systems
// Sizes, box, positions and orientations of a new system (md_init_system).
int init_system(const md_config& c, int64_t n, uint64_t seed, double* rMag, double* rHydr, double* pos, double* mm,
                double* ea, double* lBox, std::string* err);

// ----------------------------------------------------------- cell grid
md::CellGrid choose_grid(double rc_box, int64_t n, int reach);

}  // namespace mdh
