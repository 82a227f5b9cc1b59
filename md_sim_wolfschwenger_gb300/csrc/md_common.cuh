// md_common.cuh -- shared definitions of the GB300 kernels.
//
// Unit system of the device kernels (both precisions): lengths in units of
// the box length L, magnetic moments in units of mu_u = max_i |mu_i|.  Then
// a real-space term like a3 ~ 1/r^7 stays inside FP32 range (it would
// overflow in SI units), and the results convert to SI with
//   B_unit = facEwald * mu_u / L^3        [T]
//   F_unit = facEwald * mu_u^2 / L^4      [N].
// All Ewald formulas are those of the reference (src/interaction.cpp:353-674)
// rewritten in these units; the conversion factors are applied once per
// particle in the integrator.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "md_types.h"

namespace md {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

template <typename T> struct V4;
template <> struct V4<float> { using t = float4; };
template <> struct V4<double> { using t = double4_32a; };
template <typename T> struct V2;
template <> struct V2<float> { using t = float2; };
template <> struct V2<double> { using t = double2; };

// ------------------------------------------------------------ cell list
// Sorted particle data (cell order).  Written by the cell-list build and,
// for the moments, by the integrator between the two Heun stages.
struct SortedView {
  float4* xf;     // box coordinates (float) + rMag/L: candidate test
  int4* xi;       // fixed-point box coordinates (2^32 per L) + particle index
  double4_32a* xd;  // box coordinates (double) + rMag/L (FP64 path)
  void* mu;       // T4: moment / mu_u, .w = rMag / L
  int* cell;      // cell id of the sorted slot
  int* perm;      // sorted slot -> particle index
  int* rank;      // particle index -> sorted slot
  int* cell_start;  // [ncell + 1]
};

// Per-step control words in device memory (written by the step's own kernels,
// so one captured graph serves every step).
struct StepFlags {
  int rebuild;        // this step rebuilds the cell list and neighbour list
  int overflow;       // the neighbour list did not fit: real space scans cells
  int force;          // host request: rebuild on the next step
  unsigned maxdisp;   // float bits of the largest displacement since the build (box units)
  int soverflow;      // the strong-pair list did not fit: every pair stays on the FP32 path
};

// Cell-list build of one system (positions in particle order, FP64).
struct CellParams {
  int n;
  double invL;
  CellGrid grid;
  float half_skin;          // rebuild threshold: half the list skin, box units
  const double* pos;
  const double* mm;
  const double* magMom_u;
  const double* rMag_u;
  int* cellOf;
  int* count;               // [ncell] zero between builds
  int* tmp;
  SortedView s;
  double* xbuild;           // positions at the last build (may be null)
  StepFlags* flags;
};

// A packed launch runs one kernel over the blocks of several independent
// systems: block b of the grid executes block tasks[b].blk of system
// tasks[b].rep, with that system's parameters.  The kernel bodies are the
// same as for a single system, so every system gets the same results alone
// and packed.
struct Task {
  int rep, blk;
};

// Work queue of one persistent packed launch: blocks claim tasks in turn
// (atomic ticket), and the last block to finish resets the counters for the
// next launch (the next replay of the step graph).  Which block runs a task
// does not change the task's result.
struct WorkQ {
  unsigned next, done;
};

// Task loop of a persistent packed kernel: body(t) for every task claimed by
// this block; SYNC adds a block barrier after each task (kernels whose tasks
// use shared memory).
template <bool SYNC, typename F>
__device__ __forceinline__ void for_tasks(const Task* __restrict__ tk, int ntask, WorkQ* wq, F&& body) {
  __shared__ int s_task;
  for (;;) {
    if (threadIdx.x == 0) s_task = (int)atomicAdd(&wq->next, 1u);
    __syncthreads();
    const int q = s_task;
    __syncthreads();  // every thread has read the ticket before thread 0 takes the next
    if (q >= ntask) break;
    body(tk[q]);
    if (SYNC) __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&wq->done, 1u) == gridDim.x - 1) {  // all blocks have stopped claiming
      wq->next = 0;
      wq->done = 0;
      __threadfence();
    }
  }
}

// ------------------------------------------------------- real space
// FP32 loop constants of the packed pair terms (mixed path), computed once on
// the host: the pair loop reads them from the kernel parameters, so nothing
// in it is recomputed from the FP64 fields (GB300's FP64 rate is ~1/64 of
// FP32).  Pair vectors arrive in the fixed-point unit (2^-32 box lengths):
// d_fix = 2^32 d, r2f = 2^64 r^2; the unit scale and the exp -> 2^x
// conversion are folded into the factors.
struct PairK {
  float ke;     // -alpha^2 log2(e) 2^-64: exp(-alpha^2 r^2) = 2^(ke r2f)
  float kz;     // alpha 2^-32 / 2: erfc denominator 1 + alpha r / 2 = 1 + kz r_fix
  float c2a;    // 2 alpha / sqrt(pi)
  float ka2n;   // -3 2^-64 and -2 alpha^2 2^-64: field-pass a2 r^2 from a1, t
  float kt2n;   //   with the pair weight negated
  float al2x2;  // 2 alpha^2
  float al4x4;  // 4 alpha^4
  float eps;    // contact offset
  float rc2f;   // rc^2 2^64: the cutoff test on r2f
};
inline PairK make_pair_consts(double alpha, double c2a, double cont_eps, double rc2) {
  const double s64 = 5.421010862427522e-20;  // 2^-64
  const double al2 = alpha * alpha;
  PairK k;
  k.ke = (float)(-al2 * 1.4426950408889634 * s64);
  k.kz = (float)(0.5 * alpha * 2.3283064365386963e-10);
  k.c2a = (float)c2a;
  k.ka2n = (float)(-3.0 * s64);
  k.kt2n = (float)(-2.0 * al2 * s64);
  k.al2x2 = (float)(2.0 * al2);
  k.al4x4 = (float)(4.0 * al2 * al2);
  k.eps = (float)cont_eps;
  k.rc2f = (float)(rc2 * 18446744073709551616.0);
  return k;
}

struct RealParams {
  int n;
  CellGrid grid;
  double alpha, rc;      // box units
  double rc2, rc2_test;  // exact and (slightly larger) candidate cutoff
  double c2a;            // 2 alpha / sqrt(pi)
  double al2, al4;       // alpha^2, alpha^4
  double cont_eps;       // 1e-10 m / L (contact offset, interaction.cpp:120)
  PairK pk;              // FP32 constants of the packed pair terms
  // coating potentials (src/interaction.cpp:766-832), box units / F_unit
  int coat;
  double rcut_sr2;       // (rCutSR / L)^2
  double eff_len;        // effLenSurfMol / L
  double ster, elec, kappa, vdw;  // scaled prefactors
  const double* rMag_u;  // rMag / L by particle index (coating potentials)
  SortedView s;
  void* B;      // [3][n] T, sorted order
  void* F;      // [3][n] T, sorted order (FULL only)
  void* ov;     // [3][n] T, overlap displacement, box units (FULL only)
  double* Ppart;  // [n][3] per-particle pressure sums (FULL only)
  unsigned long long* npairs;  // in-range ordered pairs (FULL only, may be null)
  int* err;       // device error word
  // Verlet neighbour list (sorted indices) with a skin: rebuilt when a
  // particle has moved more than skin/2 since the last build.
  double rl2;                 // (rc + skin)^2, box units
  int* nbr;                   // [cap] neighbour indices
  int* nbr_cnt;               // [n]
  int* nbr_off;               // [n + 1]
  long long nbr_cap;
  StepFlags* flags;           // rebuild / overflow
  // Strong pairs (mixed path): list entries with |mu_i|^2 |mu_j|^2 >
  // strong_w4sq r^8 at the build (box units, moments in mu_max) carry the
  // sign bit in nbr, are left out of the FP32 field, force and pressure sums
  // (the FP32 pass still pushes them apart when they overlap) and are
  // evaluated in FP64 from the list snbr by the same kernel's warps, one
  // term set per entry into svals; the integrator adds each particle's
  // entries (StrongView).
  int strong;                 // 1: classify at builds and honour the flags
  float strong_w4sq;
  int2* snbr;                 // [scap] (i, j) sorted indices, grouped by i
  int* snbr_cnt;              // [n]
  int* snbr_off;              // [n + 1]
  long long scap;
  double* svals;              // [3][scap] B (+ [3][scap] F, [3][scap] P when FULL) per entry
  // moments of the strong entries: FP64 master directions x |mu| / mu_max
  // (particle order, via s.perm) when the evaluated moments are the master
  // state; null: the sorted view's (FP32 stage moments, exact there)
  const double* smm;
  const double* smag;
};

// The FP64 strong-pair terms of one evaluation, as the integrator reads
// them.  The real-space kernel stores, per 32-entry chunk of the strong list
// and owner particle, the owner's field and force sums at its first entry in
// the chunk, and the chunk's pressure sum at the chunk's first entry.  Slot
// r (entries off[r] .. off[r + 1]) thus adds its partials at off[r] and at
// every chunk start inside its range, in that fixed order; the pressure
// partial of a chunk belongs to the owner of the chunk's first entry.
// off == nullptr: the path is off; the flags say whether the list of the
// last build is in use.
struct StrongView {
  const int* off;
  long long cap;
  const double* B;  // [3][cap] (field of the evaluation)
  const double* F;  // [3][cap] (force, full evaluation)
  const double* P;  // [3][cap] (pressure, full evaluation)
  const StepFlags* flags;
  __device__ __forceinline__ bool usable() const { return off && !flags->overflow && !flags->soverflow; }
  // sums of the 3-component arrays a (and b when given) over slot r's
  // partials; pc: the pressure partials of the chunks slot r starts
  __device__ __forceinline__ bool sums(int r, const double* a, double oa[3], const double* b = nullptr,
                                       double* ob = nullptr, const double* pc = nullptr, double* op = nullptr) const {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      oa[q] = 0.0;
      if (ob) ob[q] = 0.0;
      if (op) op[q] = 0.0;
    }
    if (!usable() || !a) return false;
    const int e0 = max(off[r], 0), e1 = (int)min((long long)off[r + 1], cap);
    for (int e = e0; e < e1; e = (e & ~31) + 32) {
#pragma unroll
      for (int q = 0; q < 3; q++) {
        oa[q] += a[q * cap + e];
        if (b) ob[q] += b[q * cap + e];
        if (pc && (e & 31) == 0) op[q] += pc[q * cap + e];
      }
    }
    return true;
  }
  __device__ __forceinline__ bool sum3(const double* a, int r, double out[3]) const { return sums(r, a, out); }
};

// --------------------------------------------------------- k space
struct KParams {
  int n;
  int kc;
  int nseg, nk;          // segments, padded k count
  int chunk;             // particles per chunk of the structure-factor grid
  int nchunk;
  double two_pi;         // 2 * my_pi (FP64 phases follow the reference's pi)
  const KSeg* seg;       // [nseg] sorted by len (desc): structure-factor threads
  const int* koff;       // [nseg] k index of the segment's first k (sorted order)
  const double* ek;      // [nk] 2 exp(-w n^2) / n^2 (0 for padding), sorted order
  const KSeg* rseg;      // [nseg] the same segments in row order (nz, ny ascending)
  const int* rowpos;     // [nk] sorted k index -> row-order k index
  const int2* chunks;    // [nchk + 1] (first row segment, first row-order k)
  int nchk;              // chunks of <= kKChunk row-order k's (scatter staging)
  double2* Spart;        // [nchunk][nk] partial structure factors
  double* musum_part;    // [nchunk][3]
  double* musum;         // [3]
  void* eS;              // [nk] T2: e(k) * (Sc, Ss)
  double2* S;            // [nk] full structure factor (debug / FP64)
  void* tab;             // [n][3][kc + 1] T2 phase tables of the sorted particles
  double cflux, cforce;  // 4 pi, 8 pi^2 (box units)
  SortedView s;
  void* B;   // [3][n] T sorted
  void* F;   // [3][n] T sorted (FULL only)
  // Tensor-core engine (mixed path): k rows r = (ny, nz), each with nx in
  // [-kc, kc] (column q = nx + kc; k's outside the sphere or the half space
  // have kmap -1 and a zero operand).
  int tc_rows;           // R
  int tc_mt;             // structure-factor M tiles of 64 rows (x U, V)
  int tc_ns;             // structure-factor N: 2 (2kc + 1) rounded up to 16
  int tc_kp;             // scatter K: 2 (2kc + 1) rounded up to 8
  int tc_rt;             // k rows per 128-column scatter tile: 20 (field + force) or 32
  int tc_nt;             // scatter tiles: ceil(R / tc_rt)
  int tc_nst;            // scatter pipeline stages (2 or 3)
  int tc_chunk, tc_nchunk;  // structure-factor particle chunks (multiple of 16)
  const int2* tc_row;    // [R] (ny, nz)
  const float4* tc_rowd; // scatter row descriptors (kspace_tc_row_desc)
  const int* tc_kmap;    // [R][2kc + 1] sorted k index, or -1
  float* tc_part;        // [nchunk][mt][ns][128] FP32 chunk partials (column-major tiles)
  float* tc_w;           // scatter operand image [nt][hi, lo][128][kp] (this evaluation's layout)
  float* tc_bimg;        // per step: X operand tiles per 16 particles [n/16][hi, lo][ns][32]
  float2* tc_tblk;       // per step: Y, Z of each 16 particles [n/16][2][kc + 1][17]
  int tc_scat_smem;      // dynamic shared memory of the scatter launch
  int tc_yz;             // the scatter stages the Y, Z phases in shared memory
  int tc_sfa, tc_sfb;    // structure-factor ring slots (generated, copied)
  long long tc_wait;     // SM clock cycles after which an mbarrier wait gives up
  int* err;              // device error word (kErrTcWait on a wait that gave up)
};

// ----------------------------------------------------- integrator
struct IntParams {
  int n;
  double dt, L;
  double B_unit, F_unit;     // SI per unit
  double cself, csurf;       // box units
  double anisConst, velMmConst, magDamp;
  int mobil;
  int noise;                 // MD_NOISE_*
  uint64_t seed;
  int field_kind;
  double magFluxDens, tMag, fieldAmp, fieldFreq;
  const double* xi;          // uploaded unit normals [9][n] for this step
  // master state (orig order, FP64 SoA)
  double *pos, *mm, *ea, *truePos, *posRef;
  // particle constants (orig order)
  const double* magMom_u;    // |mu_i| / mu_u
  const double* rMag_u;      // rMag / L
  const double* invZt;       // 1 / zeta_trans
  const double* velEa1;
  const double* velEa2;
  const double* sT;          // thermal torque scale (DefThermFluct)
  const double* sB;          // thermal field scale
  const double* sF;          // thermal force scale
  // work arrays (orig order, T)
  void *k1m, *k1e, *m2, *e2, *th;   // th: [9][n] scaled noise
  // stage outputs (sorted order, T)
  const void *Br, *Bk, *Fr, *Fk, *ov;
  // FP64 strong-pair terms: sv.B belongs to the evaluation that gave Br,
  // sv.F and sv.P to the full evaluation (Fr, Ppart); sv.off null when off
  StrongView sv;
  // Reported field only (R = double in demag_si): FP64 unit moments of the
  // evaluation (particle order) and the k-space self-interaction matrix
  // kself = cflux sum_k e(k) n n^T (xx, yy, zz, xy, xz, yz; box units); the
  // k-space sum holds -kself mu_i of each particle's own FP32 moment, which
  // is moved to the FP64 moment.  mexact null: no correction.
  const double* mexact;
  double kself[6];
  SortedView s;
  const double* musum;       // [3] sum of mu' of the evaluated stage
  const double* Ppart;       // [n][3] per-particle pressure sums of the full real-space pass
  double* obs_part;          // [gridDim.x][7]: msd x,y,z, mz, Pxy, Pxz, Pyz
  const double* time;        // device t (double) and step
  const long long* stepno;
  int* err;
  const double* xbuild;      // [3][n] positions at the last neighbour-list build
  StepFlags* flags;          // maxdisp is raised here
};

// One stage (or the accept step) of an adaptive Runge-Kutta attempt.
struct RKStage {
  IntParams p;              // p.Br / p.Bk: the field last evaluated; p.dt: the attempt's step
  void* km[7];              // stage slopes of m, [3][n] T, original order
  void* ke[7];              // stage slopes of n
  void* cm;                 // stage coordinates (m), [3][n] T
  void* ce;                 // stage coordinates (n)
  double a[7];              // weights of k_0..k_s: next stage (stage kernel) / solution (accept)
  double e[7];              // error weights (last stage)
  int s;                    // stage index (0-based); accept: last weight index
  int last;                 // stage: no next stage, form the error; accept: take (cm, ce)
  double nf;                // factor on the thermal field and torque (rescaled on rejections)
  unsigned long long* errmax;  // max over particles of the error norm (double bits)
};

struct ObsParams {
  int nblk_int;
  const double* obs_part;
  double p_scale;            // L * F_unit / (2 * volBox) (pair double count)
  double inv_n;
  double dt;
  double* time;
  long long* stepno;
  double* records;           // [cap][8]
  long long* nrec;
  long long cap;
  // packed runs: the system's error word and list overflow, copied to status
  const int* err;
  const StepFlags* flags;
  int* status;               // may be null
};

// ------------------------------------------------------ device helpers
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): the published
// multipliers and Weyl increments; counter {i, block, step_lo, step_hi}.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Nine standard normals of particle i at step s (torque xyz, field xyz,
// force xyz), Box-Muller on uniforms (x + 0.5) 2^-32.
template <typename T>
__device__ __forceinline__ void philox_normals9(uint64_t seed, uint64_t step, uint32_t i, T z[9]) {
  T w[12];
#pragma unroll
  for (uint32_t b = 0; b < 3; b++) {
    uint4 r = philox4x32_10(make_uint4(i, b, (uint32_t)step, (uint32_t)(step >> 32)), (uint32_t)seed,
                            (uint32_t)(seed >> 32));
    uint32_t u[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if constexpr (std::is_same<T, float>::value) {
        float u1 = ((float)u[2 * h] + 0.5f) * 2.3283064365386963e-10f;
        float u2 = ((float)u[2 * h + 1] + 0.5f) * 2.3283064365386963e-10f;
        float rr = sqrtf(-2.0f * logf(u1)), s, c;
        sincospif(2.0f * u2, &s, &c);
        w[4 * b + 2 * h] = rr * c;
        w[4 * b + 2 * h + 1] = rr * s;
      } else {
        double u1 = ((double)u[2 * h] + 0.5) * 2.3283064365386963e-10;
        double u2 = ((double)u[2 * h + 1] + 0.5) * 2.3283064365386963e-10;
        double rr = sqrt(-2.0 * log(u1)), s, c;
        sincospi(2.0 * u2, &s, &c);
        w[4 * b + 2 * h] = rr * c;
        w[4 * b + 2 * h + 1] = rr * s;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 9; k++) z[k] = w[k];
}

template <typename T>
__device__ __forceinline__ void cmul(T ar, T ai, T br, T bi, T& cr, T& ci) {
  cr = ar * br - ai * bi;
  ci = ar * bi + ai * br;
}

// Device error word bits.
enum : int { kErrNonFinite = 1, kErrQueue = 2, kErrTcWait = 4 };

}  // namespace md
