/* md_gb300.h -- C ABI of the GB300 implementation of the coupled LLG +
 * Brownian-dynamics time step for magnetic nanoparticles.
 *
 * This is the drop-in boundary for the reference simulator
 * MD_Sim_Wolfschwenger (C++, single-threaded, FP64).  Every entry point names
 * the reference interface it replaces (paths relative to that repository).
 * Plain pointers and sizes only; all arrays are FP64 N x 3 column-major
 * (x[0..N), y[0..N), z[0..N)), which is the memory layout of the reference's
 * Eigen ArrayXXd members (src/typedefs.h:37-47), so a caller can pass
 * `pWorkVar->coordsTrans.pos.data()` directly.
 *
 * Every function returns an md_status; md_strerror() describes it and
 * md_last_error() returns the context's last message.  Nothing here calls
 * exit(): the reference's `cout` + `exit(-1)` error paths
 * (src/interaction.cpp:49-50, 235) become MD_ERR_INVALID / MD_ERR_CONFIG.
 *
 * Threading: a context owns one CUDA stream on one device; calls on one
 * context must be serialised by the caller (the reference is single-threaded
 * and non-reentrant, src/simulation.cpp:12-20).  Different contexts are
 * independent.
 */
#ifndef MD_GB300_H
#define MD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum md_status {
  MD_OK = 0,
  MD_ERR_INVALID = 1,     /* bad argument or state                         */
  MD_ERR_CUDA = 2,        /* CUDA runtime error (message in md_last_error)  */
  MD_ERR_NOMEM = 3,       /* device or host allocation failed / over budget */
  MD_ERR_NONFINITE = 4,   /* NaN/Inf detected in fields, forces or state    */
  MD_ERR_CONFIG = 5,      /* configuration file missing or malformed        */
  MD_ERR_UNSUPPORTED = 6, /* feature not available in this build            */
  MD_ERR_NO_DEVICE = 7    /* no CUDA device visible                          */
} md_status;

/* Arithmetic of the hot path. */
enum {
  MD_PREC_FP64 = 0,  /* everything FP64: the plain GPU path               */
  MD_PREC_MIXED = 1  /* FP32 pair math, sincos and integrator; FP64
                        structure-factor sums, self/surface terms,
                        positions and reductions                           */
};

/* Thermal noise source (DefThermFluct, src/simulation.cpp:563-603). */
enum {
  MD_NOISE_OFF = 0,      /* no thermal torque, field or force                 */
  MD_NOISE_UPLOADED = 1, /* caller supplies unit normals per step (the
                            reference's own Rand::normal stream can be fed) */
  MD_NOISE_PHILOX = 2    /* counter-based Philox4x32-10 on the device        */
};

/* Reciprocal-space engine of the mixed path (md_set_kspace_engine). */
enum {
  MD_KSPACE_AUTO = 0, /* tensor cores when kc allows, else the FP32 kernels   */
  MD_KSPACE_SIMT = 1, /* FP32 CUDA-core kernels (row segments, phase recurrences) */
  MD_KSPACE_TC = 2    /* tensor cores (3-pass TF32 matrix products over k rows) */
};

/* External field program (DefExtField, src/simulation.cpp:546-556). */
enum {
  MD_FIELD_STEP = 0,  /* B = magFluxDens e_z for t < tMag, else 0 (reference) */
  MD_FIELD_SIN = 1    /* B = fieldAmp sin(2 pi fieldFreq t) e_z (extension)   */
};

/* Every key of the reference's configuration.ini (src/configuration.ini:1-79,
 * read by Configuration::Configuration, src/configuration.cpp:6-70) and every
 * derived constant (src/configuration.cpp:71-84), plus optional extension
 * keys from an extra [gb300] section.  Integers and flags are int64_t. */
typedef struct md_config {
  /* [initial_configuration] [size_distribution] [mobilization] */
  int64_t INIT_CONFIG_ROT, INIT_CONFIG_TRANS, READ_FROM_FILE, SIZE_DIST, ENABLE_MOBILIZATION;
  /* [thermal_fluctuations] [interactions] [adaptive_timestepping_solver] */
  int64_t ENABLE_THERM_FIELD, ENABLE_THERM_TORQUE, ENABLE_THERM_FORCE, seed, ENABLE_COATING_POT, SOLVER;
  /* [particle_properties] */
  int64_t npDim;
  double magDamp, temp, satMag, anisEn;
  /* [assemble_properties] [steric_repulsion] [vdw_attraction] [electrostat_repulsion] */
  double rMagMean, dShell, volFrac, densSurfMol, hamaker, z_valency, epsilon_r, gamma_0, conc;
  /* [time_settings] [external_magnetic_field_t] [solver_settings] */
  double tMag, tRelax, deltaTinit, magFluxDens, absTol, deltaTmin, deltaTmax;
  /* [long_range_interactions] [short_range_interactions] [output_settings] */
  double errTolEwald, errTolSR, npCoords;
  /* [physical_constants] [faster_calculation] */
  double my_pi, kB, gyroMr, avogadro, epsilon_0, el, facEwald;
  /* derived (src/configuration.cpp:39, 64, 71-84) */
  int64_t numbPart;
  double mu0, effLenSurfMol, velMmConst, anisConst, sterRepFac, gamma, epsilon, kappa;
  double electrostatRepFac, irPi, vis, sigma, tEnd;
  /* [gb300] extension keys; 0 means "reference behaviour" */
  int64_t numbPartOverride; /* particle count that is not npDim^3            */
  double visOverride;       /* viscosity instead of the Vogel formula        */
  double sigmaLog;          /* log-normal sigma of ln(rMag) instead of sigma */
  int64_t fieldKind;        /* MD_FIELD_STEP or MD_FIELD_SIN                 */
  double fieldAmp, fieldFreq;
  int64_t precision;        /* MD_PREC_*                                      */
  int64_t noise;            /* MD_NOISE_*; default PHILOX                     */
} md_config;

typedef struct md_ctx md_ctx;

/* ------------------------------------------------------------ status */
const char* md_strerror(int status);
/* Copies the context's last error message (or the process-wide one when ctx
 * is NULL) into buf; returns the status that produced it. */
int md_last_error(const md_ctx* ctx, char* buf, size_t len);
/* Library version string and the CUDA architecture it was built for. */
const char* md_version(void);

/* ------------------------------------------------------ configuration */
/* Replaces Configuration::getInstance() + its getters
 * (src/configuration.h:12-180, src/configuration.cpp:6-93).  Unlike the
 * reference, the path is explicit (the reference reads ../configuration.ini
 * relative to the working directory, src/configuration.cpp:6) and a parse
 * error is returned instead of leaving zeroed members. */
int md_config_load_ini(const char* path, md_config* cfg);
/* The reference's shipped configuration.ini values (src/configuration.ini). */
int md_config_default(md_config* cfg);
/* Recomputes the derived constants (src/configuration.cpp:39, 64, 71-84)
 * after fields were edited. */
int md_config_derive(md_config* cfg);
/* Effective particle count: numbPartOverride if set, else npDim^3. */
int64_t md_config_numb_part(const md_config* cfg);
/* sizeof(md_config), for bindings that mirror the struct. */
size_t md_config_size(void);

/* ------------------------------------------------------------ context */
/* Makes `device` the calling thread's current CUDA device for this library
 * (contexts are created on the current device). */
int md_select_device(int device);
/* Creates a context for n particles on the current CUDA device
 * (the storage InitSimulation sizes, src/simulation.cpp:37-113). */
int md_ctx_create(const md_config* cfg, int64_t n, int precision, md_ctx** out);
int md_ctx_destroy(md_ctx* ctx);
/* The context's CUDA stream (cudaStream_t) for callers that order work. */
int md_ctx_stream(md_ctx* ctx, void** stream);
/* Device bytes held by this context. */
int md_ctx_device_bytes(const md_ctx* ctx, int64_t* bytes);

/* Per-particle radii (InitParticleProps, src/simulation.cpp:118-214):
 * derives volumes, moments, friction coefficients and easy-axis constants,
 * and the box length L = (sum V_hydr / volFrac)^(1/3) (simulation.cpp:56-57).
 * rHydr may be NULL: then rHydr = rMag + dShell (simulation.cpp:201). */
int md_set_particles(md_ctx* ctx, const double* rMag, const double* rHydr);
int md_get_box(const md_ctx* ctx, double* lBox);
/* Overrides the box length (e.g. a restart written by another run). */
int md_set_box(md_ctx* ctx, double lBox);

/* Coordinates (CoordsTrans_S::pos, CoordsRot_S::posMm / posEa), N x 3
 * column-major FP64.  Upload also re-anchors the diffusion reference
 * positions like InitSimulation (simulation.cpp:108-109) when reset != 0. */
int md_state_upload(md_ctx* ctx, const double* pos, const double* mm, const double* ea, int reset);
int md_state_download(md_ctx* ctx, double* pos, double* mm, double* ea);
/* Checkpoint / resume (the reference's READ_FROM_FILE path reads columns
 * its own writer does not produce, src/simulation.cpp:357-382 vs
 * src/postprocessing.cpp:84-97; this one restores everything): a binary file
 * with the radii, box, Ewald parameters, noise mode and seed, time and step
 * counter, and the positions, moments, easy axes, unwrapped positions and MSD
 * reference positions.  Loading needs a context of the same particle count
 * and precision (created with the same configuration); a run continued from
 * the file equals the saving run continued, step for step (both rebuild
 * their cell order and neighbour list at the next step).  Per-step records
 * are not part of the file. */
int md_checkpoint_save(md_ctx* ctx, const char* path);
int md_checkpoint_load(md_ctx* ctx, const char* path);
/* Integration time and step counter (RunSimulation's tInt / steps). */
int md_set_time(md_ctx* ctx, double t, int64_t step);
int md_get_time(const md_ctx* ctx, double* t, int64_t* step);

/* ------------------------------------------------------------- Ewald */
/* Ewald error model of CompEwaldParams/FunRealError/FunRezError
 * (src/interaction.cpp:164-347): for a real-space cutoff rc (metres; if
 * rc <= 0 the cutoff is chosen by the library's cost model) returns alpha
 * and the integer k-space cutoff kc that meet errTolEwald.  The particles
 * must be set.  Predicted relative force/torque errors are returned when
 * the pointers are non-NULL. */
int md_ewald_params(md_ctx* ctx, double rc, double* alpha, double* rc_out, int64_t* kc,
                    double* err_force, double* err_torque);
/* Host-only form of md_ewald_params (no context, no GPU): the same error
 * model for n particles with radii rMag (and rHydr, may be NULL); also
 * returns the box length of InitSimulation (src/simulation.cpp:56). */
int md_ewald_params_host(const md_config* cfg, int64_t n, const double* rMag, const double* rHydr, double rc,
                         double* alpha, double* rc_out, int64_t* kc, double* err_force, double* err_torque,
                         double* lBox);
/* Sets the Ewald parameters (Params_S alpha, rCutLR, nCutLR) and derives
 * the constants of InitEwaldConst (src/interaction.cpp:353-374). */
int md_set_ewald(md_ctx* ctx, double alpha, double rc, int64_t kc);
/* Chooses how the mixed path evaluates CompDipInteractEwaldF /
 * CompDipFieldEwaldF (src/interaction.cpp:429-514, 588-672): MD_KSPACE_*.
 * Both engines compute the same sums.  MD_KSPACE_TC returns
 * MD_ERR_UNSUPPORTED on the FP64 path or when kc is too large for the
 * tensor-core kernels' shared memory (kc <= 25).  Applies to the current
 * and later Ewald parameters. */
int md_set_kspace_engine(md_ctx* ctx, int engine);
/* *tensor_cores = 1 when the current Ewald parameters use the tensor cores. */
int md_kspace_engine_active(const md_ctx* ctx, int* tensor_cores);
/* Tiling of the tensor-core structure factor (no counterpart in the
 * reference; the autotuner's knobs): ring = the operand-ring option (0..5,
 * deeper rings first; -1: the deepest that fits shared memory), waves = the
 * multiple (1..4) of the chunk count that fills whole waves of resident
 * blocks (more, smaller particle chunks).  The same sums, to the kernels'
 * precision (smaller chunks add fewer terms per tensor-memory accumulator). */
int md_set_kspace_tiling(md_ctx* ctx, int ring, int waves);
/* The tiling in use; chunk = particles per structure-factor chunk (0 when
 * the tensor cores are off). */
int md_get_kspace_tiling(const md_ctx* ctx, int* ring, int* waves, int* chunk);
/* Times candidate cut-offs on the device and sets the fastest that meets
 * the error model; the GPU counterpart of the timing sweep of
 * CompEwaldParams (src/interaction.cpp:185-296).  Candidates: the cost
 * model's cut-off (md_ewald_params) and ncand cut-offs from 0.75 to 1.35
 * times it; each is timed as the median of 5 field + force and field-only
 * evaluations, each after an L2 flush (a temporary device buffer of twice
 * the L2), and replaces the cost model's choice only when faster by more
 * than 3 %.  At the chosen cut-off it times the k-space engines and the
 * tensor-core tilings (md_set_kspace_tiling) on the mixed path the same way,
 * the default tiling first. */
int md_autotune_ewald(md_ctx* ctx, int ncand, double* alpha, double* rc, int64_t* kc,
                      double* best_ms);

/* ------------------------------------------------------ interactions */
/* EvalSinCos + CompInteractions (src/interaction.cpp:521-548,
 * src/simulation.cpp:628-680) on the current state: demagnetising flux
 * density B (T) and interaction force F (N, without thermal force), the
 * real-space + short-range pressure sums P3 = {Pxy, Pxz, Pyz} before the
 * division by the box volume.  Overlapping cores are pushed apart like
 * CompInteractVecs (src/interaction.cpp:120-129) -- all overlaps resolved
 * from the same starting positions.  Outputs may be NULL. */
int md_compute_interactions(md_ctx* ctx, double* B, double* F, double* P3);
/* CompDemagField (src/simulation.cpp:688-697): B for moment directions mm
 * (N x 3, need not be unit length) with the geometry of the last
 * md_compute_interactions. */
int md_compute_field(md_ctx* ctx, const double* mm, double* B);

/* ---------------------------------------------------------- stepping */
/* Noise source and seed for md_step. */
int md_set_noise(md_ctx* ctx, int mode, uint64_t seed);
/* nsteps iterations of RunSimulation's loop body (src/simulation.cpp:469-518)
 * with the fixed step dt: DefExtField, DefThermFluct, EvalSinCos,
 * CompInteractions, IntegrationRot (Heun, SOLVER = 0), IntegrationTrans,
 * ApplyBoundaryCondArr, EvalTransCoeffs and the mz record.
 * xi: MD_NOISE_UPLOADED only, nsteps blocks of 9N unit normals, each block
 * [torque N x 3][field N x 3][force N x 3] column-major (the order of the
 * three Rand::normal draws of DefThermFluct); NULL otherwise. */
int md_step(md_ctx* ctx, int64_t nsteps, double dt, const double* xi);
/* The state in, nsteps of md_step, the state out, in one call with one
 * synchronisation: md_state_upload(pos, mm, ea, reset = 0), md_step(nsteps,
 * dt) with the context's drawn noise (Philox or off; MD_NOISE_UPLOADED is
 * MD_ERR_INVALID), md_state_download(pos_out, mm_out, ea_out).  For a caller
 * that keeps the state on the host between steps, as the reference's own
 * loop does (src/simulation.cpp:469-518).  Page-locked host buffers
 * (cudaHostAlloc, cudaHostRegister, a pinned framework tensor) are read and
 * written by kernels through their device mapping (on GB300 over
 * NVLink-C2C), which saves the copies' overhead; other host memory goes
 * through cudaMemcpyAsync.  md_state_upload does the same for its input. */
int md_step_io(md_ctx* ctx, const double* pos, const double* mm, const double* ea, int64_t nsteps, double dt,
               double* pos_out, double* mm_out, double* ea_out);
/* RunSimulation's loop with the adaptive solvers of IntegrationRot
 * (src/simulation.cpp:707-871; the configuration's SOLVER: 0 Heun-Euler 1(2),
 * 1 Bogacki-Shampine 2(3), 2 Dormand-Prince 4(5)) and the step control
 * AdjustTimeStep (src/simulation.cpp:912-951; absTol, deltaTmin, deltaTmax
 * of the configuration), stage fields by CompDemagField.  Runs accepted
 * steps while the time is <= t_end (the loop condition of RunSimulation),
 * at most max_steps of them.  *dt: the trial step on entry (deltaTinit for
 * the first step), the next trial step on exit.  The reference's behaviour is
 * kept: deltaTmax is never applied (its clamp is overwritten), a retried
 * attempt's first slope uses the field of the rejected attempt's last stage,
 * and a rejection rescales the thermal field and torque by sqrt(new/old) but
 * not the thermal force already in the interaction force.  A step rejected at
 * deltaTmin, where the reference retries forever, returns MD_ERR_INVALID.
 * xi: MD_NOISE_UPLOADED only, max_steps blocks of 9N unit normals as for
 * md_step (scaled with each step's trial dt, like DefThermFluct).
 * *steps_done: accepted steps; md_records holds one record per step. */
int md_step_adaptive(md_ctx* ctx, int64_t max_steps, double t_end, double* dt, const double* xi,
                     int64_t* steps_done);
/* Per-step records {t, mz, MSDx, MSDy, MSDz, Pxy, Pxz, Pyz} (the vectors of
 * OutputVar_S, src/typedefs.h:129-137, filled by EvalTransCoeffs and
 * simulation.cpp:514-515) for steps [first, first + count) since the last
 * md_clear_records; obs is count x 8 row-major. */
int md_records(md_ctx* ctx, int64_t first, int64_t count, double* obs);
int md_num_records(const md_ctx* ctx, int64_t* count);
int md_clear_records(md_ctx* ctx);
/* Waits for the context's stream. */
int md_sync(md_ctx* ctx);

/* ----------------------------------------------------- test hooks */
/* Cell list of the last interaction evaluation: cell_start[ncell + 1],
 * perm[N] (sorted slot -> particle index); ncell and ncx are returned. */
int md_debug_cells(md_ctx* ctx, int64_t* ncell, int64_t* ncx, int32_t* cell_start, int32_t* perm);
/* Structure factor of the last evaluation: nk entries {nx, ny, nz, Sc, Ss}
 * (as doubles, e(k) not applied).  nk_inout: capacity in, count out. */
int md_debug_structure_factor(md_ctx* ctx, int64_t* nk_inout, double* out5);
/* Number of kernel launches issued by the last md_step / md_compute_*. */
int md_debug_launches(const md_ctx* ctx, int64_t* launches);
/* In-range particle pairs (each unordered pair once) of the last full
 * real-space evaluation: the entries CompInteractVecs would list. */
int md_debug_pairs(md_ctx* ctx, int64_t* pairs);
/* Real-space field and force alone (no k-space, self or surface terms) of
 * the last md_compute_interactions, N x 3 column-major SI: the part of
 * CompDipInteractEwaldR (src/interaction.cpp:383-422). */
int md_debug_real_part(md_ctx* ctx, double* B, double* F);
/* Skin of the real-space neighbour list as a fraction of rc (default 0.005):
 * the list holds pairs within rc (1 + skin) and is rebuilt on the device when
 * a particle has moved more than skin rc / 2 since the last build. */
int md_set_neighbor_skin(md_ctx* ctx, double skin_frac);
/* Mixed path: real-space pairs whose force weight
 * (|mu_i| |mu_j| / mu_min^2) (2 rHydr_min / r)^4 exceeds theta (contact
 * forces of the smallest particles, the scale of CheckEwaldSum's relative
 * error, src/interaction.cpp:180, 741-754) are evaluated in FP64 with the
 * reference's pair formula (src/interaction.cpp:396-417) instead of FP32.
 * Classified at each neighbour-list build; default theta = 3 (about 0.2 % of
 * the pairs of a log-normal sigma 0.2 system); 0 turns it off; no effect on
 * the FP64 path, with coating potentials on, or on a system without pairs
 * above theta (monodisperse: none for theta >= 1). */
int md_set_strong_pairs(md_ctx* ctx, double theta);
/* Limit of every mbarrier wait in the tensor-core kernels, in SM clock
 * cycles (default 2e9, about a second).  A wait that reaches it gives up;
 * the kernel frees its tensor memory and returns, and the call reports
 * MD_ERR_CUDA ("a pipeline wait gave up").  No counterpart in the
 * reference (it has no GPU code). */
int md_set_wait_limit(md_ctx* ctx, int64_t cycles);
/* Test hook for that error path: one warp takes tensor memory and waits on
 * an mbarrier that is signalled only when `arrive` is nonzero, with the
 * given limit; returns MD_ERR_CUDA when the wait gave up (the context stays
 * usable), MD_OK otherwise. */
int md_debug_wait_probe(md_ctx* ctx, int arrive, int64_t cycles);
/* Entries of the strong-pair list of the last build (each ordered pair
 * once); 0 when the path is off, -1 while the list is not in use. */
int md_debug_strong_pairs(md_ctx* ctx, int64_t* entries);
/* Test hook: caps the neighbour-list capacity (entries); a list that does not
 * fit makes the real-space kernels scan the cells directly for that step. */
int md_debug_neighbor_capacity(md_ctx* ctx, int64_t cap, int64_t* used);

/* ------------------------------------------------------ profiling */
/* Kernel segments of one step, in launch order. */
enum {
  MD_SEG_CELLS = 0,      /* cell list (a)                          */
  MD_SEG_REAL_FULL,      /* real space, field + force (b)          */
  MD_SEG_KSF_FULL,       /* structure factor (c)                   */
  MD_SEG_KRED_FULL,      /* structure-factor reduction (c)         */
  MD_SEG_KSCAT_FULL,     /* k-space scatter, field + force (c)     */
  MD_SEG_HEUN1,          /* integrator stage 1 (d)                 */
  MD_SEG_REAL_FIELD,     /* real space, field only (b)             */
  MD_SEG_KSF_FIELD,
  MD_SEG_KRED_FIELD,
  MD_SEG_KSCAT_FIELD,
  MD_SEG_HEUN2,          /* integrator stage 2 (d)                 */
  MD_SEG_OBS,            /* per-step records                       */
  MD_NSEG
};
/* With enable != 0, every following step records CUDA events between its
 * kernel segments (inside the replayed graph, on the context's stream). */
int md_profile(md_ctx* ctx, int enable);
/* Milliseconds per segment of the last step (ms[MD_NSEG]). */
int md_profile_read(md_ctx* ctx, double* ms);
/* Measured FP32 FMA throughput of the current device (TFLOP/s, FMA = 2
 * FLOPs) from a register-resident FMA-chain kernel on all SMs. */
int md_calibrate_fp32(double* tflops);

/* ------------------------------------------------------ initial systems */
/* InitParticleProps size draws and InitCoordsFromSketch
 * (src/simulation.cpp:118-351) for n particles: radii rMag, rHydr (n), pos,
 * mm, ea (n x 3 column-major FP64) and the box length (src/simulation.cpp:56).
 *   sizes:     SIZE_DIST 0: rMagMean; 1: log-normal with the reference's
 *              (mu, sigmaLog) from rMagMean and sigma, or ln r ~ N(ln rMagMean,
 *              sigmaLog) when the [gb300] sigmaLog key is set;
 *   positions: INIT_CONFIG_TRANS 1: random sequential addition of
 *              non-overlapping hydrodynamic spheres in [-(L/2 - r_h), L/2 - r_h]^3
 *              (cell grid, O(n); polydisperse sizes are placed largest first);
 *              2: cubic grid (n must be a cube);
 *   rotations: INIT_CONFIG_ROT 1, 2, 3 as the reference; 4 (extension): mm
 *              and ea independent and uniform on the sphere.
 * rHydr may be NULL.  Random numbers: a seeded xoshiro256** stream, not the
 * reference's Mersenne-Twister stream. */
int md_init_system(const md_config* cfg, int64_t n, uint64_t seed, double* rMag, double* rHydr, double* pos,
                   double* mm, double* ea, double* lBox);

/* Initial positions on the GPU (the calling thread's device) by random
 * sequential addition, the placement of InitCoordsFromSketch
 * (src/simulation.cpp:241-264) with its box-interior draw and overlap rule
 * (plain distance below the sum of the hydrodynamic radii): in placement order
 * (largest_first = 0: index order, as the reference; 1: decreasing radius,
 * for dense polydisperse systems) each particle takes the first attempt that
 * overlaps no particle placed before it.  Attempt t of particle i is drawn
 * from Philox4x32-10 with counters {i, t} (the reference draws all attempts
 * from one generator), so the parallel placement equals the sequential rule
 * exactly.  pos: 3 x n column-major, box centred at 0.  MD_ERR_INVALID when
 * a particle finds no place in 1e5 attempts or all particles together need
 * more than 100 n + 1e6 (volume fraction too high for random addition);
 * MD_ERR_UNSUPPORTED when more than 64 particles fall into one cell of its
 * search grid (cells span the largest contact distance, 2N cells at most: an
 * extremely wide size distribution). */
int md_place_rsa(int64_t n, double lBox, const double* rHydr, uint64_t seed, int largest_first, double* pos);

/* Ewald cutoff tuned per (N, volume fraction) bucket: the first system of a
 * bucket runs md_autotune_ewald (timed field evaluations over candidate
 * cutoffs, each with alpha and kc from the error model); later systems of the
 * bucket reuse the winning rc / L.  *hit = 1 when the cache answered.  The
 * cache is process-wide; md_tune_cache_save/load keep it in a text file. */
int md_autotune_ewald_cached(md_ctx* ctx, double volFrac, double* alpha, double* rc, int64_t* kc, int* hit);
int md_tune_cache_save(const char* path);
int md_tune_cache_load(const char* path);
int md_tune_cache_clear(void);

/* ------------------------------------------------------ packed systems */
/* Independent systems (replicas of uneven N: field sweeps, seed ensembles,
 * served requests) advanced together: every kernel of the step is launched
 * once for all systems of the batch (one grid over all their blocks, one
 * captured CUDA graph per step), and each system's results equal those of
 * md_step on it alone, bit for bit.  Systems keep their own contexts (the
 * caller owns them); the batch holds at most `capacity` of them.
 * Requirements: MD_PREC_MIXED, noise MD_NOISE_OFF or MD_NOISE_PHILOX, state
 * uploaded and Ewald parameters set.  While a round is in flight
 * (md_batch_launch .. md_batch_wait) the contexts in the batch must not be
 * used. */
typedef struct md_batch md_batch;
int md_batch_create(int64_t capacity, md_batch** out);
int md_batch_destroy(md_batch* batch);
/* Adds ctx to run nsteps steps of size dt; *id identifies it in the batch. */
int md_batch_add(md_batch* batch, md_ctx* ctx, int64_t nsteps, double dt, int64_t* id);
int md_batch_remove(md_batch* batch, int64_t id);
/* Launches min(max_steps, fewest steps left of any system) steps of every
 * system (asynchronous; *steps gets that count) ... */
int md_batch_launch(md_batch* batch, int64_t max_steps, int64_t* steps);
/* ... and waits for them: MD_ERR_NONFINITE if some system's state became
 * non-finite (md_batch_remaining tells which). */
int md_batch_wait(md_batch* batch);
/* launch + wait. */
int md_batch_run(md_batch* batch, int64_t max_steps, int64_t* steps);
/* Steps still to run and the status of the last round of system id. */
int md_batch_remaining(const md_batch* batch, int64_t id, int64_t* left, int* status);
/* Systems, particles, kernel launches per packed step, GPU time of the last
 * round (ms, CUDA events on the batch's stream). */
int md_batch_info(const md_batch* batch, int64_t* systems, int64_t* particles, int64_t* launches_per_step,
                  double* last_round_ms);

/* ------------------------------------------------------------ serving */
/* One simulation request of a served stream. */
typedef struct md_request {
  int64_t n;          /* particles                                           */
  double volFrac;     /* volume fraction of hydrodynamic spheres             */
  int64_t steps;      /* Heun steps                                          */
  double dt;          /* step (s)                                            */
  int64_t fieldKind;  /* MD_FIELD_STEP: fieldAmp along z for all t;
                         MD_FIELD_SIN: fieldAmp sin(2 pi fieldFreq t) along z */
  double fieldAmp;    /* T                                                   */
  double fieldFreq;   /* Hz                                                  */
  uint64_t seed;      /* initial system and Philox noise                     */
  double arrival;     /* s after the start of md_serve_run                  */
} md_request;

typedef struct md_request_result {
  int status;         /* MD_OK or the error that ended the request           */
  double admitted;    /* s after the start: state on the device              */
  double finished;    /* s after the start: last step done                   */
  double latency;     /* finished - arrival                                  */
  double mz;          /* mean m_z after the last step                        */
  double checksum;    /* sum of pos / L + mm + ea over all particles (final) */
  int64_t steps_done;
  int64_t device_bytes;
} md_request_result;

typedef struct md_serve_opts {
  double hbm_budget;     /* device bytes the admitted systems may hold        */
  int64_t max_systems;   /* systems packed at once                            */
  int64_t round_steps;   /* steps per packed round (admission granularity)    */
  int realtime;          /* 1: admit a request no earlier than its arrival    */
  int autotune;          /* 1: Ewald cutoff from md_autotune_ewald_cached     */
} md_serve_opts;

typedef struct md_serve_stats {
  double wall;            /* s from start to the last completion              */
  double particle_steps;  /* sum over requests of n * steps                   */
  double gpu_ms;          /* GPU time of all packed rounds (CUDA events)      */
  double admit_ms;        /* host time creating contexts (upload, setup), on
                             the admitting thread, overlapping the rounds      */
  int64_t rounds, repacks, peak_systems;
  double peak_bytes;
} md_serve_stats;

/* Continuous batching over a request stream: requests are admitted in
 * arrival order as device memory (hbm_budget) and batch slots free up; each
 * admitted request becomes a system (md_init_system with base's keys and the
 * request's n, volFrac, field and seed; Ewald parameters for
 * base.errTolEwald) that joins the packed batch at the next round; a second
 * host thread admits while this one keeps the rounds going.  Finished systems
 * leave the batch and free their memory.  results[i] belongs to reqs[i]. */
int md_serve_run(const md_config* base, const md_request* reqs, int64_t nreq, const md_serve_opts* opts,
                 md_request_result* results, md_serve_stats* stats);

/* ------------------------------------------------------ post-processing */
/* Radial distribution function of the current positions, as the reference's
 * analysis script computes it per frame (mFiles/radial_dist_fun.m:19-66):
 * pairs i < j at their minimum-image distance, distances below 2 r_mag0
 * clamped to 2 r_mag0 (the script uses rMag of the first particle), pairs
 * closer than `range` (m; the script: 8 r_mag0) counted in `bins` equal bins
 * (<= 8192), g[k] = count[k] L^3 / (2 pi dr^3 N^2) / (k + 1/2)^2.  With
 * include_last = 0 the pairs with the last particle are left out, as the
 * script's loop bound does; 1 counts all pairs.  counts (may be NULL) gets
 * the integer pair counts. */
int md_rdf(md_ctx* ctx, int64_t bins, double range, double r_mag0, int include_last, double* g, uint64_t* counts);

/* ------------------------------------------------------ output files */
/* The reference's text outputs, written from host arrays with the bytes its
 * Eigen stream output produces (6 significant digits, columns aligned to the
 * widest coefficient, each matrix followed by an empty line).  A time label
 * tInt of exactly 0 truncates the file, any other value appends -- the rule
 * of saveData (src/postprocessing.cpp:15-32). */
/* saveData: rows x cols matrix a (col_major != 0: a[i + j rows], else
 * a[i cols + j]). */
int md_write_matrix_txt(const char* path, const double* a, int64_t rows, int64_t cols, int col_major, double tInt);
/* WriteCoords2TXT (src/postprocessing.cpp:82-101): one frame of n rows
 * {x y z m_x m_y m_z n_x n_y n_z label}, the label column holding tInt in
 * row 0 and zeros below. */
int md_write_coords_txt(const char* path, int64_t n, const double* pos, const double* mm, const double* ea,
                        double tInt);
/* WriteData2TXT (src/postprocessing.cpp:106-133): n rows {rHydr rMag meta},
 * meta = box length, N, field, Ms, T, tMag, tRelax, tEnd, volFrac, the two
 * INIT_CONFIG keys, seed, K, surfactant density and length, Hamaker constant,
 * valency, epsilon_r, gamma_0, absTol, errTolEwald, errTolSR in rows 0..21
 * (rows beyond n are left out; the reference needs n >= 22). */
int md_write_data_txt(const char* path, const md_config* cfg, int64_t n, const double* rMag, const double* rHydr,
                      double lBox);
/* ExportDiffVis (src/postprocessing.cpp:222-231) and the m_z / time exports
 * of RunSimulation (src/simulation.cpp:532-536): dtMean.txt = tInt / steps,
 * then Pxy, Pxz, Pyz, MSDx, MSDy, MSDz, mz and t .txt as column vectors from
 * count records {t, mz, MSDx, MSDy, MSDz, Pxy, Pxz, Pyz} (row-major, as
 * md_records returns them).  dir NULL or "": the working directory. */
int md_export_records_txt(const char* dir, const double* obs, int64_t count, double tInt, int64_t steps);

/* ------------------------------------------- structure factor, no allocation */
/* This entry point has no counterpart in the reference.  It exists for
 * callers that cannot call cudaMalloc -- a host framework that owns all
 * device memory through its own pool, a real-time loop that must not allocate
 * after start-up, a process under a fixed device-memory budget.  It computes
 * the Ewald structure factor S(n) = sum_j (n . mu_j) exp(2 pi i n . r_j / L)
 * (FP64) with caller-owned device buffers and no allocation of its own: its
 * scratch is one file-scope device array of md_noalloc_scratch_bytes()
 * (2,430,592 bytes) that every GPU loading the library holds until exit.
 *   n:        1 .. 2^30 particles.
 *   pos, mom: device pointers, N x 3 column-major FP64 (positions in m,
 *             moment vectors in A m^2);  out5: device pointer with room for
 *             nk x 5 doubles {nx, ny, nz, Sc, Ss}, the k vectors of the
 *             reference's loops (nz = 0..kc, ny and nx = -kc..kc,
 *             0 < |n|^2 <= kc^2, in that loop order); nk_out (host) gets nk.
 *   stream:   cudaStream_t (NULL: the default stream); the call is
 *             asynchronous on it.
 * kc above MD_NOALLOC_MAX_KC is rejected with MD_ERR_INVALID.  The first
 * call on a device looks up the array's device address (make it before any
 * stream capture); the address is kept for the process, so do not call it
 * on a device after cudaDeviceReset.  All calls share the array and it keeps
 * the last call's contents, so calls whose work overlaps on the GPU race:
 * serialise them.  Launch failures are read from each launch's own return
 * code; an error left pending by earlier work is not consumed here. */
#define MD_NOALLOC_MAX_KC 16
size_t md_noalloc_scratch_bytes(void);
int md_structure_factor_noalloc(const double* pos, const double* mom, int64_t n, double lBox, int64_t kc,
                                double my_pi, double* out5, int64_t* nk_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MD_GB300_H */
