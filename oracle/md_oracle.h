/* md_oracle.h -- TEST INFRASTRUCTURE ONLY: CPU restatement (FP64, plain C) of
 * the reference's coupled LLG + Brownian-dynamics time step
 * (MD_Sim_Wolfschwenger, src/simulation.cpp:466-520 and the functions it
 * calls).  It is the checker for the CUDA path: only tests/, the smoke test
 * and bench.py's CPU-baseline leg may load it.  The product never links it.
 *
 * Parity pin: this restatement is compared against the reference's own code
 * (oracle/_ref/ref_harness, built from the reference sources) by
 * tests/test_oracle_vs_reference.py and by the committed fixtures under
 * tests/golden/ that the harness produced.
 *
 * Arrays are N x 3 column-major FP64 (Eigen ArrayXXd layout, src/typedefs.h).
 */
#ifndef MD_ORACLE_H
#define MD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Values the reference reads from its Configuration singleton and Params_S. */
typedef struct orc_cfg {
  int64_t n;
  double lBox;
  double alpha, rCutLR;  /* Ewald real-space parameters (Params_S) */
  int64_t nc;            /* k-space cut-off as an integer (Params_S::nc)      */
  double rCutSR;         /* short-range cut-off (InitCutOffSR)                 */
  double my_pi, facEwald, irPi, kB, temp, magDamp, gyroMr, satMag, anisEn, anisConst, velMmConst;
  double effLenSurfMol, sterRepFac, electrostatRepFac, kappa, hamaker;
  double magFluxDens, tMag;
  int64_t enable_mobilization, enable_therm_torque, enable_therm_field, enable_therm_force;
  int64_t enable_coating;
  /* Extensions (0 = reference behaviour). */
  int64_t field_kind;     /* 0: B0 for t < tMag (DefExtField); 1: amp*sin(2 pi freq t) */
  double field_amp, field_freq;
  int64_t overlap_mode;   /* 0: sequential in-place push (reference), 1: Jacobi  */
} orc_cfg;

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(const orc_cfg* cfg);
void orc_destroy(orc_ctx* c);
/* Per-particle radii; derived properties as InitParticleProps
 * (simulation.cpp:204-210) with the given viscosity. */
void orc_set_props(orc_ctx* c, const double* rMag, const double* rHydr, double vis);
void orc_set_state(orc_ctx* c, const double* pos, const double* mm, const double* ea, double t);
void orc_get_state(const orc_ctx* c, double* pos, double* mm, double* ea, double* t);
/* Re-anchors the MSD reference positions (InitSimulation, simulation.cpp:108-109). */
void orc_reset_observables(orc_ctx* c);

/* CompInteractions (simulation.cpp:628-680) preceded by EvalSinCos, on the
 * current state with the current thermal force.  Positions are overlap
 * corrected in place as the reference does.  Outputs may be NULL. */
void orc_compute_interactions(orc_ctx* c, double* B, double* F, double* P3);
/* CompDemagField (simulation.cpp:688-697) for the given moment directions,
 * reusing the pair list and tables of the last orc_compute_interactions. */
void orc_compute_field(orc_ctx* c, const double* mm, double* B);

/* noise_mode: 0 off (also honours the ENABLE_THERM_* flags), 1 uploaded unit
 * normals (xi: [torque N*3][field N*3][force N*3], column-major), 2 Philox. */
enum { ORC_NOISE_OFF = 0, ORC_NOISE_UPLOADED = 1, ORC_NOISE_PHILOX = 2 };

/* One step of the reference loop body (simulation.cpp:469-518) with fixed dt.
 * Optional dumps (may be NULL): B1, F1 after CompInteractions, B2 at the Heun
 * predictor, obs[8] = {t, mz, MSDx, MSDy, MSDz, Pxy, Pxz, Pyz}. */
void orc_step(orc_ctx* c, double dt, int noise_mode, const double* xi, uint64_t seed,
              double* B1, double* F1, double* B2, double* obs);

/* Adaptive time stepping (IntegrationRot + AdjustTimeStep,
 * simulation.cpp:707-871, 912-951): solver 0 Heun-Euler 1(2), 1
 * Bogacki-Shampine 2(3), 2 Dormand-Prince 4(5) (the SOLVER key). */
typedef struct orc_adapt {
  int64_t solver;
  double absTol, dtMin, dtMax;
} orc_adapt;

/* One accepted step of the reference loop with the adaptive solver: deltaT is
 * the trial step on entry and the next trial step on exit; *used_out the step
 * taken, *attempts_out the attempts (1 + rejections). */
void orc_step_adaptive(orc_ctx* c, const orc_adapt* ad, double* deltaT, int noise_mode, const double* xi,
                       uint64_t seed, double* obs, double* used_out, int* attempts_out);

/* Thermal noise scaled as DefThermFluct (simulation.cpp:563-603). */
void orc_thermal(orc_ctx* c, double dt, int noise_mode, const double* xi, uint64_t seed,
                 double* torque, double* field, double* force);

/* Philox4x32-10 normals: 9 per particle per step, layout as uploaded xi. */
void orc_philox_normals(uint64_t seed, uint64_t step, int64_t n, double* xi);
/* One Philox4x32-10 block (Salmon et al., SC'11): counter ctr, key key. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Ewald error model (interaction.cpp:330-347).  Returns the real-space and
 * k-space RMS force errors divided by F_contact, minus errTol/sqrt(2). */
double orc_fun_real_error(double x, double M, double fAl, double lBox, double rc, double n,
                          double facEwald, double errTol);
double orc_fun_rez_error(double x, double M, double fAl, double lBox, double alpha, double n,
                         double facEwald, double my_pi, double errTol);
/* The reference's grid scan + linear interpolation for alpha and kc at a
 * given rc (interaction.cpp:190-257).  Returns 0 on success. */
int orc_ewald_for_rc(double rc, double M, double fAl, double lBox, double n, double facEwald,
                     double my_pi, double errTol, double* alpha, double* kc);

int64_t orc_pairs(const orc_ctx* c);
/* Threads of the pair list and the Ewald sums (default 1); t > 1 needs
 * overlap_mode 1.  Returns 0, or nonzero for a bad request. */
int orc_set_threads(orc_ctx* c, int t);
/* Random sequential addition in index order (InitCoordsFromSketch,
 * simulation.cpp:241-264) with a seeded splitmix64 generator. */
int orc_rsa(int64_t n, double lBox, const double* rHydr, uint64_t seed, int64_t max_tries, double* pos);
/* Random sequential addition with a Philox stream per particle (the GPU
 * placement's restatement; order NULL: index order). */
int orc_rsa_philox(int64_t n, double lBox, const double* rHydr, uint64_t seed, const int64_t* order,
                   int64_t max_tries, double* pos, int64_t* tries);
double orc_last_seconds(const orc_ctx* c);

#ifdef __cplusplus
}
#endif
#endif
