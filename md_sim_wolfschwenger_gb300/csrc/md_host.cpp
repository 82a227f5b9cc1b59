// md_host.cpp -- host-side logic (no CUDA): configuration, Ewald error
// model, k-vector list, cell grid, particle properties.  See md_host.h.
#include "md_host.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

namespace mdh {

// ================================================================ config

// Values of the reference's shipped src/configuration.ini (lines 1-79).
void config_defaults(md_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->INIT_CONFIG_ROT = 2;
  c->INIT_CONFIG_TRANS = 1;
  c->READ_FROM_FILE = 0;
  c->SIZE_DIST = 0;
  c->ENABLE_MOBILIZATION = 1;
  c->ENABLE_THERM_FIELD = 1;
  c->ENABLE_THERM_TORQUE = 1;
  c->ENABLE_THERM_FORCE = 1;
  c->seed = 1;
  c->ENABLE_COATING_POT = 0;
  c->SOLVER = 2;
  c->npDim = 10;
  c->magDamp = 0.001;
  c->temp = 300.0;
  c->satMag = 4.5e5;
  c->anisEn = 1e4;
  c->rMagMean = 8e-9;
  c->dShell = 0;
  c->volFrac = 0.0001;
  c->densSurfMol = 5e17;
  c->hamaker = 33e-21;
  c->z_valency = 1;
  c->epsilon_r = 78.5;
  c->gamma_0 = 0.04;
  c->conc = 50;
  c->tMag = 0;
  c->tRelax = 1e-8;
  c->deltaTinit = 1e-12;
  c->magFluxDens = 0.03;
  c->absTol = 1e-4;
  c->deltaTmin = 1e-14;
  c->deltaTmax = 1e-9;
  c->errTolEwald = 1e-7;
  c->errTolSR = 0.01;
  c->npCoords = 100;
  c->my_pi = 3.14159265359;
  c->kB = 1.380648e-23;
  c->gyroMr = 1.7595e11;
  c->avogadro = 6.02214076e23;
  c->epsilon_0 = 8.8541e-12;
  c->el = 1.6e-19;
  c->facEwald = 1e-7;
  c->precision = MD_PREC_MIXED;
  c->noise = MD_NOISE_PHILOX;
  c->fieldKind = MD_FIELD_STEP;
  config_derive(c);
}

// Derived constants exactly as src/configuration.cpp:39, 64, 71-84.
void config_derive(md_config* c) {
  const double pi = c->my_pi, T = c->temp, kB = c->kB, el = c->el, z = c->z_valency;
  c->effLenSurfMol = 0.2 * c->rMagMean;
  c->mu0 = 4.0 * pi * std::pow(10, -7);
  c->numbPart = c->npDim * c->npDim * c->npDim;
  c->velMmConst = c->gyroMr / (1.0 + std::pow(c->magDamp, 2.0));
  c->anisConst = 2.0 * c->anisEn / c->satMag;
  c->sterRepFac = 4 * kB * T * pi * c->densSurfMol / (2 * c->effLenSurfMol);
  c->gamma = std::tanh(z * el * c->gamma_0 / (4 * kB * T));
  c->epsilon = c->epsilon_0 * c->epsilon_r;
  c->kappa = std::sqrt(el * el * c->avogadro * c->conc * z * z / (c->epsilon * kB * T));
  c->electrostatRepFac = c->kappa * 64 * pi * c->epsilon * std::pow(kB * T / (z * el), 2.0) * c->gamma * c->gamma;
  c->irPi = 1 / std::sqrt(pi);
  c->vis = (2.414e-5) * std::pow(10, 247.8 / (T - 140));
  c->sigma = std::sqrt(0.1) * 2.0 * c->rMagMean;
  c->tEnd = c->tMag + c->tRelax;
}

int64_t numb_part(const md_config* c) { return c->numbPartOverride > 0 ? c->numbPartOverride : c->npDim * c->npDim * c->npDim; }

namespace {

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

std::string lower(std::string s) {
  for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

// The INI dialect of the reference's vendored inih (src/INIReader.h): [section],
// name = value or name: value, ';'/'#' full-line comments, ';' inline comments
// after whitespace, case-insensitive section and key names.
struct Ini {
  std::map<std::string, std::string> kv;
  bool get(const char* sec, const char* key, std::string* v) const {
    auto it = kv.find(lower(sec) + "=" + lower(key));
    if (it == kv.end()) return false;
    *v = it->second;
    return true;
  }
  long get_int(const char* sec, const char* key, long dflt) const {
    std::string v;
    if (!get(sec, key, &v)) return dflt;
    const char* s = v.c_str();
    char* end;
    long r = std::strtol(s, &end, 0);
    return end > s ? r : dflt;
  }
  double get_real(const char* sec, const char* key, double dflt) const {
    std::string v;
    if (!get(sec, key, &v)) return dflt;
    const char* s = v.c_str();
    char* end;
    double r = std::strtod(s, &end);
    return end > s ? r : dflt;
  }
  bool get_bool(const char* sec, const char* key, bool dflt) const {
    std::string v;
    if (!get(sec, key, &v)) return dflt;
    v = lower(v);
    if (v == "true" || v == "yes" || v == "on" || v == "1") return true;
    if (v == "false" || v == "no" || v == "off" || v == "0") return false;
    return dflt;
  }
};

int parse_ini(const char* path, Ini* ini, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = std::string("cannot open configuration file ") + path;
    return -1;
  }
  std::string line, section;
  int lineno = 0;
  while (std::getline(f, line)) {
    lineno++;
    if (lineno == 1 && line.size() >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
        (unsigned char)line[2] == 0xBF)
      line = line.substr(3);
    std::string t = trim(line);
    if (t.empty() || t[0] == ';' || t[0] == '#') continue;
    if (t[0] == '[') {
      size_t e = t.find(']');
      if (e == std::string::npos) {
        *err = "line " + std::to_string(lineno) + ": ']' expected";
        return lineno;
      }
      section = trim(t.substr(1, e - 1));
      continue;
    }
    size_t eq = t.find_first_of("=:");
    if (eq == std::string::npos) {
      *err = "line " + std::to_string(lineno) + ": '=' or ':' expected";
      return lineno;
    }
    std::string name = trim(t.substr(0, eq)), value = t.substr(eq + 1);
    for (size_t k = 0; k < value.size(); k++)
      if (value[k] == ';' && (k == 0 || std::isspace((unsigned char)value[k - 1]))) {
        value = value.substr(0, k);
        break;
      }
    ini->kv[lower(section) + "=" + lower(name)] = trim(value);
  }
  return 0;
}

}  // namespace

// Configuration::Configuration (src/configuration.cpp:6-85), the same
// defaults for missing keys (-1, false), plus the optional [gb300] keys.
int config_load_ini(const char* path, md_config* c, std::string* err) {
  Ini ini;
  if (parse_ini(path, &ini, err) != 0) return MD_ERR_CONFIG;
  std::memset(c, 0, sizeof(*c));
  c->INIT_CONFIG_ROT = ini.get_int("initial_configuration", "INIT_CONFIG_ROT", -1);
  c->INIT_CONFIG_TRANS = ini.get_int("initial_configuration", "INIT_CONFIG_TRANS", -1);
  c->READ_FROM_FILE = ini.get_bool("initial_configuration", "READ_FROM_FILE", false);
  c->SIZE_DIST = ini.get_int("size_distribution", "SIZE_DIST", -1);
  c->ENABLE_MOBILIZATION = ini.get_bool("mobilization", "ENABLE_MOBILIZATION", false);
  c->ENABLE_THERM_FIELD = ini.get_bool("thermal_fluctuations", "ENABLE_THERM_FIELD", false);
  c->ENABLE_THERM_TORQUE = ini.get_bool("thermal_fluctuations", "ENABLE_THERM_TORQUE", false);
  c->ENABLE_THERM_FORCE = ini.get_bool("thermal_fluctuations", "ENABLE_THERM_FORCE", false);
  c->seed = ini.get_int("thermal_fluctuations", "seed", -1);
  c->ENABLE_COATING_POT = ini.get_bool("interactions", "ENABLE_COATING_POT", false);
  c->SOLVER = ini.get_int("adaptive_timestepping_solver", "SOLVER", -1);
  c->npDim = ini.get_int("particle_properties", "npDim", -1);
  c->magDamp = ini.get_real("particle_properties", "magDamp", -1);
  c->temp = ini.get_real("particle_properties", "temp", -1);
  c->satMag = ini.get_real("particle_properties", "satMag", -1);
  c->anisEn = ini.get_real("particle_properties", "anisEn", -1);
  c->rMagMean = ini.get_real("assemble_properties", "rMagMean", -1);
  c->dShell = ini.get_real("assemble_properties", "dShell", -1);
  c->volFrac = ini.get_real("assemble_properties", "volFrac", -1);
  c->densSurfMol = ini.get_real("steric_repulsion", "densSurfMol", -1);
  c->hamaker = ini.get_real("vdw_attraction", "hamaker", -1);
  c->z_valency = ini.get_real("electrostat_repulsion", "z_valency", -1);
  c->epsilon_r = ini.get_real("electrostat_repulsion", "epsilon_r", -1);
  c->gamma_0 = ini.get_real("electrostat_repulsion", "gamma_0", -1);
  c->conc = ini.get_real("electrostat_repulsion", "conc", -1);
  c->tMag = ini.get_real("time_settings", "tMag", -1);
  c->tRelax = ini.get_real("time_settings", "tRelax", -1);
  c->deltaTinit = ini.get_real("time_settings", "deltaTinit", -1);
  c->magFluxDens = ini.get_real("external_magnetic_field_t", "magFluxDens", -1);
  c->absTol = ini.get_real("solver_settings", "absTol", -1);
  c->deltaTmin = ini.get_real("solver_settings", "deltaTmin", -1);
  c->deltaTmax = ini.get_real("solver_settings", "deltaTmax", -1);
  c->errTolEwald = ini.get_real("long_range_interactions", "errTolEwald", -1);
  c->errTolSR = ini.get_real("short_range_interactions", "errTolSR", -1);
  c->npCoords = ini.get_real("output_settings", "npCoords", -1);
  c->my_pi = ini.get_real("physical_constants", "my_pi", -1);
  c->kB = ini.get_real("physical_constants", "kB", -1);
  c->gyroMr = ini.get_real("physical_constants", "gyroMr", -1);
  c->avogadro = ini.get_real("physical_constants", "avogadro", -1);
  c->epsilon_0 = ini.get_real("physical_constants", "epsilon_0", -1);
  c->el = ini.get_real("physical_constants", "el", -1);
  c->facEwald = ini.get_real("faster_calculation", "facEwald", -1);
  // extension keys
  c->numbPartOverride = ini.get_int("gb300", "NUMB_PART", 0);
  c->visOverride = ini.get_real("gb300", "vis", 0);
  c->sigmaLog = ini.get_real("gb300", "sigmaLog", 0);
  c->fieldKind = ini.get_int("gb300", "FIELD_KIND", MD_FIELD_STEP);
  c->fieldAmp = ini.get_real("gb300", "fieldAmp", 0);
  c->fieldFreq = ini.get_real("gb300", "fieldFreq", 0);
  c->precision = ini.get_int("gb300", "PRECISION", MD_PREC_MIXED);
  c->noise = ini.get_int("gb300", "NOISE", MD_NOISE_PHILOX);
  config_derive(c);
  return MD_OK;
}

// =============================================================== particles

// funEffDiameter / IntegralEffDiameter (src/mathFun.cpp:27-54): Simpson rule.
static double fun_eff_diameter(const md_config& c, double dMag, double r) {
  double dDelta = dMag + 2 * c.effLenSurfMol;
  return 1 - std::exp(-c.my_pi * dMag * dMag * c.densSurfMol / (2 * c.effLenSurfMol) *
                      (dDelta - r * (std::log(dDelta / (r + 1e-20)) + 1)));
}

double integral_eff_diameter(const md_config& c, double dMag) {
  double area = 0, lo = 0, hi = dMag + 2 * c.effLenSurfMol;
  const int steps = 1000;
  double h = (hi - lo) / steps;
  for (int i = 0; i < steps; i++)
    area += h / 6 * (fun_eff_diameter(c, dMag, i * h) + 4 * fun_eff_diameter(c, dMag, (i + 0.5) * h) +
                     fun_eff_diameter(c, dMag, (i + 1) * h));
  return area;
}

int make_props(const md_config& c, const double* rMag, const double* rHydr, int64_t n, Props* p, std::string* err) {
  if (n <= 0 || !rMag) {
    *err = "no particles";
    return MD_ERR_INVALID;
  }
  const double pi = c.my_pi;
  p->vis = c.visOverride > 0 ? c.visOverride : c.vis;
  p->rMag.assign(rMag, rMag + n);
  p->rHydr.resize(n);
  for (int64_t i = 0; i < n; i++) {
    if (!(rMag[i] > 0) || !std::isfinite(rMag[i])) {
      *err = "particle radius must be positive and finite";
      return MD_ERR_INVALID;
    }
    if (rHydr) {
      p->rHydr[i] = rHydr[i];
    } else if (c.ENABLE_COATING_POT) {
      double dH = integral_eff_diameter(c, 2 * rMag[i]);
      p->rHydr[i] = dH >= 2 * rMag[i] ? dH / 2.0 : rMag[i];
    } else {
      p->rHydr[i] = rMag[i] + c.dShell;
    }
  }
  p->volMag.resize(n);
  p->volHydr.resize(n);
  p->magMom.resize(n);
  p->zetaRot.resize(n);
  p->zetaTrans.resize(n);
  p->velEa1.resize(n);
  p->velEa2.resize(n);
  double vh = 0, mmax = 0, rmax = 0, rhmax = 0;
  for (int64_t i = 0; i < n; i++) {
    p->volMag[i] = 4.0 / 3.0 * pi * std::pow(p->rMag[i], 3.0);
    p->volHydr[i] = 4.0 / 3.0 * pi * std::pow(p->rHydr[i], 3.0);
    p->magMom[i] = c.satMag * p->volMag[i];
    p->zetaRot[i] = 8.0 * pi * p->vis * std::pow(p->rHydr[i], 3.0);
    p->zetaTrans[i] = 6.0 * pi * p->vis * p->rHydr[i];
    p->velEa1[i] = 2.0 * c.anisEn * (p->volMag[i] / p->zetaRot[i]);
    p->velEa2[i] = 1 / p->zetaRot[i];
    vh += p->volHydr[i];
    mmax = std::max(mmax, p->magMom[i]);
    rmax = std::max(rmax, p->rMag[i]);
    rhmax = std::max(rhmax, p->rHydr[i]);
  }
  if (!(c.volFrac > 0)) {
    *err = "volFrac must be positive";
    return MD_ERR_INVALID;
  }
  p->lBox = std::pow(vh / c.volFrac, 1.0 / 3.0);
  p->muMax = mmax;
  // InitCutOffSR (src/interaction.cpp:20-57)
  if (c.ENABLE_COATING_POT) {
    double c1 = 128 * c.hamaker * std::pow(rmax, 6.0) * pi / (18 * c.mu0 * mmax * mmax);
    auto f = [&](double x, bool der) {
      if (der) return c1 * (4 * rmax * rmax + 3 * x * x) / std::pow(4 * rmax * rmax - x * x, 3.0);
      return c1 * x / std::pow(x * x - 4 * rmax * rmax, 2.0) - c.errTolSR;
    };
    double x = 1.1 * 2 * rmax;
    for (int it = 0; it < 1000; it++) {
      x -= f(x, false) / f(x, true);
      if (std::fabs(f(x, false)) <= 1e-7) break;
    }
    if (!(x >= 2 * rhmax)) {
      *err = "short-range cutoff below 2 rHydr: particles can only interact if they overlap";
      return MD_ERR_INVALID;
    }
    p->rCutSR = x;
  } else {
    p->rCutSR = 2 * rmax;
  }
  return MD_OK;
}

void noise_scales(const md_config& c, const Props& p, double dt, std::vector<double>* sT, std::vector<double>* sB,
                  std::vector<double>* sF) {
  const size_t n = p.rMag.size();
  sT->assign(n, 0.0);
  sB->assign(n, 0.0);
  sF->assign(n, 0.0);
  for (size_t i = 0; i < n; i++) {
    if (c.ENABLE_THERM_TORQUE) (*sT)[i] = std::sqrt((2.0 * c.kB * c.temp / dt) * p.zetaRot[i]);
    if (c.ENABLE_THERM_FIELD)
      (*sB)[i] = std::sqrt(2.0 * c.kB * c.temp * c.magDamp / (c.gyroMr * c.satMag * dt) * (1.0 / p.volMag[i]));
    if (c.ENABLE_THERM_FORCE) (*sF)[i] = std::sqrt((2.0 * c.kB * c.temp / dt) * p.zetaTrans[i]);
  }
}

// ================================================================== Ewald

EwaldModel ewald_model(const md_config& c, const Props& p) {
  EwaldModel m;
  double mmin = 1e300, rhmin = 1e300;
  for (size_t i = 0; i < p.magMom.size(); i++) {
    m.M += std::pow(p.magMom[i], 2.0);
    mmin = std::min(mmin, p.magMom[i]);
    rhmin = std::min(rhmin, p.rHydr[i]);
  }
  m.fAl = 3 * c.mu0 * std::pow(mmin, 2.0) / (2.0 * c.my_pi * std::pow(2.0 * rhmin, 4.0));
  m.tAl = std::pow(mmin, 2.0) * c.mu0 / (16.0 * c.my_pi * std::pow(rhmin, 3.0));
  m.L = p.lBox;
  m.n = (double)p.magMom.size();
  return m;
}

// FunRealError (src/interaction.cpp:330-338).
double fun_real_error(const md_config& c, const EwaldModel& m, double x, double rc) {
  const double a = x * rc, a2 = a * a, a4 = a2 * a2, a6 = a4 * a2;
  const double rc3 = rc * rc * rc, L3 = m.L * m.L * m.L;
  const double b = m.M / (x * x * std::sqrt(L3 * rc3 * rc3 * rc3 * m.n));
  const double cc = 4.0 * a4 + 6.0 * a2 + 3.0;
  const double d = 8.0 * a6 + 20.0 * a4 + 30.0 * a2 + 15.0;
  return c.facEwald * b * std::sqrt(13.0 / 6.0 * cc * cc + 2.0 / 15.0 * d * d - 13.0 / 15.0 * cc * d) *
             std::exp(-a2) / m.fAl -
         c.errTolEwald / std::sqrt(2.0);
}

// FunRezError (src/interaction.cpp:344-347).
double fun_rez_error(const md_config& c, const EwaldModel& m, double alpha, double x) {
  const double pi = c.my_pi, q = pi * x / (alpha * m.L);
  return c.facEwald * 8.0 * m.M * pi / (m.L * m.L * m.L) * alpha * std::sqrt(2.0 * pi * x * x * x / (15.0 * m.n)) *
             std::exp(-q * q) / m.fAl -
         c.errTolEwald / std::sqrt(2.0);
}

// alpha: the first sign change of FunRealError going up in alpha (the
// reference scans [0, 2e8] on a uniform grid, interaction.cpp:192-213), then
// bisection to full precision.  kc: the root on the decaying side of
// FunRezError after its maximum (interaction.cpp:219-249), kc >= 2.
bool ewald_for_rc(const md_config& c, const EwaldModel& m, double rc, double* alpha, double* kc_raw) {
  // first sign change on the grid a_i = 1e-4 / rc 10^(6 i / 4000): located on
  // every 10th grid point, then among the 10 points before it (the error
  // function is smooth on the 3.5 % span of ten grid points)
  auto grid = [&](int i) { return 1e-4 / rc * std::pow(10.0, 6.0 * i / 4000.0); };
  double lo = 0, hi = 0;
  if (!(fun_real_error(c, m, grid(0), rc) > 0)) return false;
  for (int j = 10; j <= 4000 + 9 && hi == 0; j += 10) {
    const int jj = std::min(j, 4000);
    if (fun_real_error(c, m, grid(jj), rc) < 0) {
      for (int i = jj - 9 > 1 ? jj - 9 : 1; i <= jj; i++)
        if (fun_real_error(c, m, grid(i), rc) < 0) {
          lo = grid(i - 1);
          hi = grid(i);
          break;
        }
    }
    if (jj == 4000) break;
  }
  if (hi == 0) return false;
  for (int it = 0; it < 200 && hi - lo > 1e-15 * hi; it++) {
    double mid = 0.5 * (lo + hi);
    (fun_real_error(c, m, mid, rc) > 0 ? lo : hi) = mid;
  }
  const double a = 0.5 * (lo + hi);
  *alpha = a;
  const double xs = std::sqrt(3.0) * a * m.L / (2.0 * c.my_pi);  // maximum of FunRezError
  if (!(fun_rez_error(c, m, a, xs) > 0)) {
    *kc_raw = 2.0;
    return true;
  }
  double klo = xs, khi = 2 * xs + 4;
  while (fun_rez_error(c, m, a, khi) > 0) khi *= 2;
  for (int it = 0; it < 200 && khi - klo > 1e-13 * khi; it++) {
    double mid = 0.5 * (klo + khi);
    (fun_rez_error(c, m, a, mid) > 0 ? klo : khi) = mid;
  }
  *kc_raw = std::max(2.0, 0.5 * (klo + khi));
  return true;
}

void predicted_errors(const md_config& c, const EwaldModel& m, double alpha, double rc, double kc, double* errF,
                      double* errT) {
  const double ar = alpha * rc, pi = c.my_pi, L = m.L, N = m.n, M = m.M;
  const double cc = 4.0 * std::pow(ar, 4.0) + 6.0 * std::pow(ar, 2.0) + 3.0;
  const double dc = 8.0 * std::pow(ar, 6.0) + 20.0 * std::pow(ar, 4.0) + 30.0 * std::pow(ar, 2.0) + 15.0;
  const double bc = 2.0 * std::pow(ar, 2.0) + 1.0;
  const double eRF = c.facEwald * M / std::sqrt(std::pow(L, 3.0) * std::pow(alpha, 4.0) * std::pow(rc, 9.0) * N) *
                     std::sqrt(13.0 / 6.0 * cc * cc + 2.0 / 15.0 * dc * dc - 13.0 / 15.0 * cc * dc) *
                     std::exp(-std::pow(ar, 2.0));
  const double eKF = c.facEwald * 8.0 * pi * M / std::pow(L, 3.0) * alpha *
                     std::sqrt(2.0 * pi * std::pow(kc, 3.0) / (15.0 * N)) *
                     std::exp(-std::pow(pi * kc / (alpha * L), 2.0));
  const double eRT = c.facEwald * M / std::sqrt(std::pow(L, 3.0) * std::pow(alpha, 4.0) * std::pow(rc, 7.0) * N) *
                     std::sqrt(0.5 * bc * bc + 0.2 * cc * cc) * std::exp(-std::pow(ar, 2.0));
  const double eKT = c.facEwald * 4.0 * M / std::pow(L, 2.0) * alpha * std::sqrt(pi * kc / (5.0 * N)) *
                     std::exp(-std::pow(pi * kc / (alpha * L), 2.0));
  if (errF) *errF = std::sqrt(eKF * eKF + eRF * eRF) / m.fAl;
  if (errT) *errT = std::sqrt(eKT * eKT + eRT * eRT) / m.tAl;
}

// Instruction-count model of one step (two field evaluations): per neighbour
// ~75 for the candidate tests and ~155 for the pair maths; per (k, particle)
// ~44 (structure factor twice, full and field-only scatter).
// Relative cost of one step for cutoff rc (box units) and kc: per particle,
// the ordered pairs within rc (field + force and field-only passes over the
// Verlet list, which is rebuilt only every many steps) and the k vectors of
// the half space (structure factor twice, scatter twice).  The weights are
// the measured per-unit times on GB300 at N = 32768: 9.5 ps per ordered
// pair; per (k, particle) 2.5 ps on the FP32 CUDA-core k-space kernels and
// 1.7 ps on the tensor-core ones (used for kc <= kc_tc).
double model_cost(double rc_box, int64_t kc, int64_t n, int kc_tc) {
  const double pi = 3.141592653589793;
  const double nr = (double)n * 4.0 / 3.0 * pi * rc_box * rc_box * rc_box;
  const double nk = 2.0 * pi / 3.0 * (double)kc * kc * kc;
  return (double)n * (9.5 * nr + (kc <= kc_tc ? 1.7 : 2.5) * nk);
}

double choose_rc(const md_config& c, const EwaldModel& m, int64_t n, double* alpha_out, int64_t* kc_out,
                 int kc_tc) {
  // every candidate rc = 0.08 L .. 0.5 L in steps of 0.005 L (the cost is not
  // unimodal in rc, so no candidate is skipped)
  double best = 1e300, best_rc = 0.5;
  for (int q = 0; q <= 84; q++) {
    const double x = 0.08 + 0.005 * q;
    double a, k;
    if (!ewald_for_rc(c, m, x * m.L, &a, &k)) continue;
    const int64_t kc = (int64_t)std::floor(k + 0.5);
    if (kc > 64) continue;
    const double cost = model_cost(x, kc, n, kc_tc);
    if (cost < best) {
      best = cost;
      best_rc = x;
      *alpha_out = a;
      *kc_out = kc;
    }
  }
  return best_rc * m.L;
}

// ========================================================== k-vector list

// Rows (ny, nz) of the half space |n|^2 <= kc^2, nz >= 0, with half of the
// nz = 0 plane; each row split into segments of <= 16 consecutive nx, each
// padded to a multiple of 4 with zero-weight k's; sorted by padded length.
KList build_klist(int kc, double w) {
  KList L;
  const int kc2 = kc * kc;
  // rows of the half space: (ny, nz) with nx in [x0, x1]
  struct Row {
    int ny, nz, x0, x1;
  };
  std::vector<Row> rows;
  for (int nz = 0; nz <= kc; nz++)
    for (int ny = -kc; ny <= kc; ny++) {
      if (nz == 0 && ny < 0) continue;
      int rem = kc2 - ny * ny - nz * nz;
      if (rem < 0) continue;
      int m = (int)std::floor(std::sqrt((double)rem));
      while ((m + 1) * (m + 1) <= rem) m++;
      while (m * m > rem) m--;
      int x0 = (nz == 0 && ny == 0) ? 1 : -m, x1 = m;
      if (x1 < x0) continue;
      rows.push_back({ny, nz, x0, x1});
    }
  // rows split evenly into pieces of at most `maxlen`, padded to multiples of 4
  auto split = [&](int maxlen, std::vector<md::KSeg>* segs, std::vector<int>* reals) {
    for (const Row& r : rows) {
      const int len = r.x1 - r.x0 + 1, ns = (len + maxlen - 1) / maxlen;
      const int base = len / ns, extra = len % ns;
      int x = r.x0;
      for (int s = 0; s < ns; s++) {
        const int l = base + (s < extra ? 1 : 0);
        segs->push_back(md::KSeg{x, r.ny, r.nz, (l + 3) & ~3});
        reals->push_back(l);
        x += l;
      }
    }
  };
  // structure factor: segments of <= 16, sorted by length (uniform warps)
  std::vector<md::KSeg> segs;
  std::vector<int> reals;
  split(16, &segs, &reals);
  std::vector<int> order(segs.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return segs[a].len > segs[b].len; });
  // scatter: whole rows (<= kScatSeg), row order, chunks of <= kKChunk k's
  std::vector<int> sreals;
  split(md::kScatSeg, &L.rseg, &sreals);
  std::map<std::pair<int, int>, int> row_first;  // (ny, nz) -> first scatter segment
  std::vector<int> soff(L.rseg.size());
  int roff = 0, chunk_k = 0;
  for (size_t s = 0; s < L.rseg.size(); s++) {
    if (s == 0 || chunk_k + L.rseg[s].len > md::kKChunk) {
      L.chunks.push_back((int)s);
      L.chunks.push_back(roff);
      chunk_k = 0;
    }
    soff[s] = roff;
    roff += L.rseg[s].len;
    chunk_k += L.rseg[s].len;
    row_first.emplace(std::make_pair(L.rseg[s].ny, L.rseg[s].nz), (int)s);
  }
  L.nchk = (int)L.chunks.size() / 2;
  L.chunks.push_back((int)L.rseg.size());
  L.chunks.push_back(roff);
  L.nk_scat = roff;
  // position of k = (nx, ny, nz) in the scatter layout
  auto scat_pos = [&](int nx, int ny, int nz) {
    int s = row_first.at(std::make_pair(ny, nz));
    while (nx >= L.rseg[s].nx0 + sreals[s]) s++;
    return soff[s] + (nx - L.rseg[s].nx0);
  };
  L.rowpos.clear();
  int off = 0;
  for (int idx : order) {
    const md::KSeg& sg = segs[idx];
    L.seg.push_back(sg);
    L.koff.push_back(off);
    for (int t = 0; t < sg.len; t++) {
      const int nx = sg.nx0 + t;
      const bool real = t < reals[idx];
      L.rowpos.push_back(real ? scat_pos(nx, sg.ny, sg.nz) : -1);
      const double n2 = (double)nx * nx + (double)sg.ny * sg.ny + (double)sg.nz * sg.nz;
      L.ek.push_back(real ? 2.0 * std::exp(-w * n2) / n2 : 0.0);
      L.kx.push_back(nx);
      L.ky.push_back(sg.ny);
      L.kz.push_back(sg.nz);
      L.kreal.push_back(real ? 1 : 0);
      L.nk_real += real ? 1 : 0;
    }
    off += sg.len;
  }
  L.nk = off;
  return L;
}

// ============================================================ cell grid

// Cells of edge >= rc / reach; a stencil of +-reach cells must not wrap onto
// itself (ncx >= 2 reach + 1), otherwise all pairs are scanned (ncx = 1).
md::CellGrid choose_grid(double rc_box, int64_t n, int reach) {
  md::CellGrid g{1, 1, 0};
  if (reach < 1) reach = 2;
  int ncx = (int)std::floor(reach / rc_box * (1.0 - 1e-12));
  // keep cells from becoming much smaller than needed for tiny systems
  const int cap = std::max(1, (int)std::cbrt((double)n * 4.0));
  ncx = std::min(ncx, std::max(2 * reach + 1, cap));
  if (ncx >= 2 * reach + 1) {
    g.ncx = ncx;
    g.ncell = ncx * ncx * ncx;
    g.reach = reach;
  }
  return g;
}

}  // namespace mdh

namespace mdh {

// ----------------------------------------------------- initial systems

namespace {

// xoshiro256** (Blackman & Vigna, 2018), seeded through splitmix64.
struct Xoshiro {
  uint64_t s[4];
  explicit Xoshiro(uint64_t seed) {
    for (int i = 0; i < 4; i++) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s[i] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
  double balanced() { return 2.0 * uniform() - 1.0; }              // [-1, 1)
  double normal() {                                                 // Marsaglia polar method
    for (;;) {
      const double u = balanced(), v = balanced(), q = u * u + v * v;
      if (q > 0 && q < 1) return u * std::sqrt(-2.0 * std::log(q) / q);
    }
  }
};

}  // namespace

int init_system(const md_config& c, int64_t n, uint64_t seed, double* rMag, double* rHydr, double* pos, double* mm,
                double* ea, double* lBox, std::string* err) {
  if (n < 1 || !rMag || !pos || !mm || !ea) {
    *err = "bad arguments";
    return MD_ERR_INVALID;
  }
  Xoshiro rng(seed);
  // sizes (InitParticleProps, src/simulation.cpp:162-212)
  if (c.SIZE_DIST == 1) {
    double mu, sl;
    if (c.sigmaLog > 0) {
      mu = std::log(c.rMagMean);
      sl = c.sigmaLog;
    } else {
      mu = std::log(c.rMagMean * c.rMagMean / std::sqrt(c.rMagMean * c.rMagMean + c.sigma * c.sigma));
      sl = std::sqrt(std::log(1.0 + std::pow(c.sigma / c.rMagMean, 2.0)));
    }
    for (int64_t i = 0; i < n; i++) rMag[i] = std::exp(mu + sl * rng.normal());
  } else {
    for (int64_t i = 0; i < n; i++) rMag[i] = c.rMagMean;
  }
  Props p;
  int st = make_props(c, rMag, nullptr, n, &p, err);
  if (st) return st;
  if (rHydr)
    for (int64_t i = 0; i < n; i++) rHydr[i] = p.rHydr[i];
  const double L = p.lBox;
  *lBox = L;
  // positions (InitCoordsFromSketch, src/simulation.cpp:229-288)
  if (c.INIT_CONFIG_TRANS == 2) {
    const int64_t d = (int64_t)std::llround(std::cbrt((double)n));
    if (d * d * d != n) {
      *err = "INIT_CONFIG_TRANS = 2 needs a cubic particle count";
      return MD_ERR_INVALID;
    }
    const double gap = L / (double)d;
    int64_t ip = 0;
    for (int64_t ix = 0; ix < d; ix++)
      for (int64_t iy = 0; iy < d; iy++)
        for (int64_t iz = 0; iz < d; iz++, ip++) {
          pos[ip] = (ix + 0.5) * gap - L / 2.0;
          pos[n + ip] = (iy + 0.5) * gap - L / 2.0;
          pos[2 * n + ip] = (iz + 0.5) * gap - L / 2.0;
        }
  } else {
    // random sequential addition on a cell grid (cells >= the largest
    // contact distance, so a candidate only meets the 27 cells around it)
    double rhmax = 0, rhmin = 1e300;
    for (int64_t i = 0; i < n; i++) {
      rhmax = std::max(rhmax, p.rHydr[i]);
      rhmin = std::min(rhmin, p.rHydr[i]);
    }
    const int64_t nc = std::max<int64_t>(1, std::min<int64_t>(1024, (int64_t)std::floor(L / (2.0 * rhmax))));
    const double cs = L / (double)nc;
    std::vector<int64_t> head((size_t)(nc * nc * nc), -1), next((size_t)n, -1);
    std::vector<int64_t> order((size_t)n);
    for (int64_t i = 0; i < n; i++) order[i] = i;
    if (rhmax > rhmin)
      std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return p.rHydr[a] > p.rHydr[b]; });
    auto cell_of = [&](double x) {
      int64_t k = (int64_t)std::floor((x + L / 2.0) / cs);
      return std::min<int64_t>(nc - 1, std::max<int64_t>(0, k));
    };
    const int64_t max_tries = 2000000;
    for (int64_t q = 0; q < n; q++) {
      const int64_t i = order[q];
      const double ri = p.rHydr[i], ext = L / 2.0 - ri;
      bool placed = false;
      for (int64_t t = 0; t < max_tries && !placed; t++) {
        const double x = rng.balanced() * ext, y = rng.balanced() * ext, z = rng.balanced() * ext;
        const int64_t cx = cell_of(x), cy = cell_of(y), cz = cell_of(z);
        bool ok = true;
        for (int64_t dz = -1; dz <= 1 && ok; dz++)
          for (int64_t dy = -1; dy <= 1 && ok; dy++)
            for (int64_t dx = -1; dx <= 1 && ok; dx++) {
              const int64_t ux = cx + dx, uy = cy + dy, uz = cz + dz;
              if (ux < 0 || uy < 0 || uz < 0 || ux >= nc || uy >= nc || uz >= nc) continue;
              for (int64_t j = head[(size_t)((uz * nc + uy) * nc + ux)]; j >= 0; j = next[(size_t)j]) {
                const double ddx = pos[j] - x, ddy = pos[n + j] - y, ddz = pos[2 * n + j] - z;
                const double rr = ri + p.rHydr[j];
                if (ddx * ddx + ddy * ddy + ddz * ddz < rr * rr) {
                  ok = false;
                  break;
                }
              }
            }
        if (ok) {
          pos[i] = x;
          pos[n + i] = y;
          pos[2 * n + i] = z;
          const size_t cell = (size_t)((cz * nc + cy) * nc + cx);
          next[(size_t)i] = head[cell];
          head[cell] = i;
          placed = true;
        }
      }
      if (!placed) {
        *err = "random sequential addition failed: volume fraction too high";
        return MD_ERR_INVALID;
      }
    }
  }
  // orientations (src/simulation.cpp:292-349): azimuth 2 pi u, elevation
  // 2 asin(sqrt(u)) -- uniform on the sphere
  auto draw = [&](double* v) {
    for (int64_t i = 0; i < n; i++) {
      const double az = rng.uniform() * 2.0 * c.my_pi;
      const double el = 2.0 * std::asin(std::sqrt(rng.uniform()));
      v[i] = std::sin(el) * std::cos(az);
      v[n + i] = std::sin(el) * std::sin(az);
      v[2 * n + i] = std::cos(el);
    }
  };
  auto set_z = [&](double* v) {
    for (int64_t i = 0; i < n; i++) {
      v[i] = 0.0;
      v[n + i] = 0.0;
      v[2 * n + i] = 1.0;
    }
  };
  switch (c.INIT_CONFIG_ROT) {
    case 1:
      draw(ea);
      set_z(mm);
      break;
    case 3:
      set_z(ea);
      std::copy(ea, ea + 3 * n, mm);
      break;
    case 4:
      draw(ea);
      draw(mm);
      break;
    default:
      draw(ea);
      std::copy(ea, ea + 3 * n, mm);
      break;
  }
  return MD_OK;
}

}  // namespace mdh
