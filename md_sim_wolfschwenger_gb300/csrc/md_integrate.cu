// md_integrate.cu -- kernel (d): fused stochastic Heun step of the moment
// (LLG), the easy axis and the translation, with the thermal noise.
// Restates, per particle:
//   DefExtField                   src/simulation.cpp:546-556
//   DefThermFluct                 src/simulation.cpp:563-603
//   RKCoeffs                      src/simulation.cpp:876-902
//   IntegrationRot (HEUN_EULER)   src/simulation.cpp:721-749, 866-867
//   IntegrationTrans              src/simulation.cpp:959-962
//   ApplyBoundaryCondArr          src/simulation.cpp:610-620
//   EvalTransCoeffs, mz record    src/postprocessing.cpp:167-187,
//                                 src/simulation.cpp:514-515
// Stage 1 (k_heun1) evaluates k1 with the interaction field, forms the
// predictor (m2, n2) and writes its moments into the sorted view for the
// second field evaluation.  Stage 2 (k_heun2) evaluates k2, applies the
// corrector, renormalises, translates with the force of the step start plus
// the overlap push, wraps, and accumulates MSD and m_z.  The thermal torque,
// field and force are drawn once per step and frozen across the two stages
// (the reference draws them once in DefThermFluct).
//
// Precision: T = float (mixed) or double.  Positions, the master copies of
// m and n, the self/surface Ewald terms and all reductions are FP64.
//
// Roofline: HBM/L2 bound, tiny; per particle and step ~250 B of algorithmic
// traffic (state 72 B read + 72 B written, stage outputs, work arrays).
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kIntThreads = 256;  // largest block (packed batches, adaptive solvers)
// Single-system Heun launches: 128-thread blocks, so that N = 32768 spreads
// over every SM (256 blocks; these short kernels are latency bound).
constexpr int kIntOne = 128;

__device__ __forceinline__ double ext_field_z(const IntParams& p, double t) {
  if (p.field_kind == 1) return p.fieldAmp * sinpi(2.0 * p.fieldFreq * t);
  return t < p.tMag ? p.magFluxDens : 0.0;
}

// RKCoeffs: Beff = ext + demag + anisConst (m.n) n + B_th;
// dn/dt = velEa1 (m.n)(m - (m.n) n) + velEa2 (tau_th x n);
// dm/dt = -velMmConst (m x Beff + magDamp m x (m x Beff)).
template <typename T>
__device__ __forceinline__ void rk(const IntParams& p, const T m[3], const T e[3], const T bd[3], T bz_ext,
                                   const T bth[3], const T tau[3], T v1, T v2, T km[3], T ke[3]) {
  const T dot = m[0] * e[0] + m[1] * e[1] + m[2] * e[2];
  const T ac = (T)p.anisConst;
  T be[3];
  be[0] = bd[0] + ac * (e[0] * dot) + bth[0];
  be[1] = bd[1] + ac * (e[1] * dot) + bth[1];
  be[2] = (bz_ext + bd[2]) + ac * (e[2] * dot) + bth[2];
  if (p.mobil) {
    const T c0 = tau[1] * e[2] - tau[2] * e[1];
    const T c1 = tau[2] * e[0] - tau[0] * e[2];
    const T c2 = tau[0] * e[1] - tau[1] * e[0];
    const T f = v1 * dot;
    ke[0] = (m[0] - e[0] * dot) * f + c0 * v2;
    ke[1] = (m[1] - e[1] * dot) * f + c1 * v2;
    ke[2] = (m[2] - e[2] * dot) * f + c2 * v2;
  } else {
    ke[0] = ke[1] = ke[2] = 0;
  }
  const T x0 = m[1] * be[2] - m[2] * be[1];
  const T x1 = m[2] * be[0] - m[0] * be[2];
  const T x2 = m[0] * be[1] - m[1] * be[0];
  const T y0 = m[1] * x2 - m[2] * x1;
  const T y1 = m[2] * x0 - m[0] * x2;
  const T y2 = m[0] * x1 - m[1] * x0;
  const T vm = (T)p.velMmConst, md = (T)p.magDamp;
  km[0] = -vm * (x0 + md * y0);
  km[1] = -vm * (x1 + md * y1);
  km[2] = -vm * (x2 + md * y2);
}

// Demagnetising field of particle i (sorted slot r) in SI: the real- and
// k-space sums and the self and surface terms combined in FP64, then
// returned in the integrator's type T.
// sbs: the strong-pair field sums of slot r when the caller has them already.
template <typename T, typename R = T>
__device__ __forceinline__ void demag_si(const IntParams& p, int r, R b[3], const double* sbs = nullptr) {
  using T4 = typename V4<T>::t;
  const int n = p.n;
  const T* Br = (const T*)p.Br;
  const T* Bk = (const T*)p.Bk;
  double sb[3];  // strong pairs (FP64 terms), mixed path
  bool hs;
  if (sbs) {
    sb[0] = sbs[0];
    sb[1] = sbs[1];
    sb[2] = sbs[2];
    hs = true;
  } else {
    hs = p.sv.sum3(p.sv.B, r, sb);
  }
  const T4 mu = ((const T4*)p.s.mu)[r];
  if constexpr (std::is_same<R, float>::value) {
    // mixed integrator: the FP32 stage outputs combined in FP32 (FP64 runs
    // at ~1/64 of the FP32 rate on GB300; the self term that cancels the
    // k-space self field is small against the pair fields, so the FP32 sum
    // loses nothing measurable)
    const float cs = (float)p.cself, cu = (float)p.csurf, bu = (float)p.B_unit;
    const float mu3[3] = {(float)mu.x, (float)mu.y, (float)mu.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float br = hs ? (float)Br[a * n + r] + (float)sb[a] : (float)Br[a * n + r];
      b[a] = ((br + (float)Bk[a * n + r]) + (cs * mu3[a] - cu * (float)p.musum[a])) * bu;
    }
  } else {
    double mu3[3] = {(double)mu.x, (double)mu.y, (double)mu.z};
    double kfix[3] = {0.0, 0.0, 0.0};
    if (std::is_same<R, double>::value && p.mexact) {
      // FP64 moment of particle i (sorted slot r): the self term uses it, and
      // the k-space sum's self-interaction -kself mu is moved from the moment
      // it was evaluated with (the sorted view's) to this one
      const int i = p.s.perm[r];
      const double g = p.magMom_u[i];
      const double me[3] = {p.mexact[i] * g, p.mexact[n + i] * g, p.mexact[2 * n + i] * g};
      const double d[3] = {mu3[0] - me[0], mu3[1] - me[1], mu3[2] - me[2]};
      const double* K = p.kself;
      kfix[0] = K[0] * d[0] + K[3] * d[1] + K[4] * d[2];
      kfix[1] = K[3] * d[0] + K[1] * d[1] + K[5] * d[2];
      kfix[2] = K[4] * d[0] + K[5] * d[1] + K[2] * d[2];
      mu3[0] = me[0];
      mu3[1] = me[1];
      mu3[2] = me[2];
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const double selfsurf = p.cself * mu3[a] - p.csurf * p.musum[a];
      const double br = (double)Br[a * n + r] + sb[a];
      b[a] = (R)(((br + ((double)Bk[a * n + r] + kfix[a])) + selfsurf) * p.B_unit);
    }
  }
}

template <typename T>
__device__ __forceinline__ void heun1(const IntParams& p, int bx) {
  using T4 = typename V4<T>::t;
  const int i = bx * (int)blockDim.x + threadIdx.x;
  const int n = p.n;
  if (i >= n) return;
  const int r = p.s.rank[i];
  T m[3], e[3], bd[3], z[9];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    m[a] = (T)p.mm[a * n + i];
    e[a] = (T)p.ea[a * n + i];
  }
  demag_si<T>(p, r, bd);
  if (p.noise == 2) {
    philox_normals9<T>(p.seed, (uint64_t)*p.stepno, (uint32_t)i, z);
  } else if (p.noise == 1) {
#pragma unroll
    for (int q = 0; q < 9; q++) z[q] = (T)p.xi[(q / 3) * 3 * n + (q % 3) * n + i];
  } else {
#pragma unroll
    for (int q = 0; q < 9; q++) z[q] = 0;
  }
  const T sT = (T)p.sT[i], sB = (T)p.sB[i], sF = (T)p.sF[i];
  T tau[3], bth[3];
  T* th = (T*)p.th;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    tau[a] = sT * z[a];
    bth[a] = sB * z[3 + a];
    th[a * n + i] = tau[a];
    th[(3 + a) * n + i] = bth[a];
    th[(6 + a) * n + i] = sF * z[6 + a];
  }
  const T bz = (T)ext_field_z(p, *p.time);
  T km[3], ke[3];
  rk<T>(p, m, e, bd, bz, bth, tau, (T)p.velEa1[i], (T)p.velEa2[i], km, ke);
  const T dt = (T)p.dt;
  T* k1m = (T*)p.k1m;
  T* k1e = (T*)p.k1e;
  T* m2 = (T*)p.m2;
  T* e2 = (T*)p.e2;
  T mm2[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    k1m[a * n + i] = km[a];
    k1e[a * n + i] = ke[a];
    e2[a * n + i] = e[a] + dt * ke[a];
    mm2[a] = m[a] + dt * km[a];
    m2[a * n + i] = mm2[a];
  }
  const T mu = (T)p.magMom_u[i];
  T4 v;
  v.x = mm2[0] * mu;
  v.y = mm2[1] * mu;
  v.z = mm2[2] * mu;
  v.w = (T)p.rMag_u[i];
  ((T4*)p.s.mu)[r] = v;
}

// End of a step for particle i (sorted slot r): renormalised m and n
// (simulation.cpp:869-870) from the solver's mn, en; translation with the
// step-start force plus thermal force fth and the overlap push, the single
// wrap (IntegrationTrans + ApplyBoundaryCondArr); unwrapped MSD, m_z and the
// pressure partials into acc; squared displacement since the last list build.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so FP64 is spent only where the
// value needs it (positions, MSD).  The multiples of L that wrap and unwrap
// are integers taken from FP32 quotients that sit next to an integer (a
// step moves a particle far less than L / 2), so they equal the FP64
// round(.../L) of the reference; the displacement since the list build only
// feeds the rebuild test and is FP32.
// sfp: the strong-pair force and pressure sums of slot r (6 values) when the
// caller has them already.
template <typename T>
__device__ __forceinline__ void finish_particle(const IntParams& p, int i, int r, const T mn[3], const T en[3],
                                                const T fth[3], double acc[7], float& disp2,
                                                const double* sfp = nullptr) {
  const int n = p.n;
  acc[4] = p.Ppart[3 * i];
  acc[5] = p.Ppart[3 * i + 1];
  acc[6] = p.Ppart[3 * i + 2];
  double sp[3], sf[3];  // strong pairs of the full evaluation (FP64 terms)
  bool hs;
  if (sfp) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      sf[q] = sfp[q];
      sp[q] = sfp[3 + q];
    }
    hs = true;
  } else {
    hs = p.sv.sums(r, p.sv.F, sf, nullptr, nullptr, p.sv.P, sp);
  }
  acc[4] += sp[0];
  acc[5] += sp[1];
  acc[6] += sp[2];
  const T nm = sqrt(mn[0] * mn[0] + mn[1] * mn[1] + mn[2] * mn[2]);
  const T ne = sqrt(en[0] * en[0] + en[1] * en[1] + en[2] * en[2]);
  const T* Fr = (const T*)p.Fr;
  const T* Fk = (const T*)p.Fk;
  const T* ov = (const T*)p.ov;
  const double L = p.L, half = 0.5 * L, dtd = p.dt;
  const float Lf = (float)L, iLf = 1.0f / Lf;
  const T izt = (T)p.invZt[i];
  bool bad = false;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const T mf = mn[a] / nm, ef = en[a] / ne;
    p.mm[a * n + i] = (double)mf;
    p.ea[a * n + i] = (double)ef;
    T f;
    const T fr = hs ? Fr[a * n + r] + (T)sf[a] : Fr[a * n + r];
    if constexpr (std::is_same<T, float>::value)
      f = (fr + Fk[a * n + r]) * (float)p.F_unit + fth[a];
    else
      f = (fr + Fk[a * n + r]) * p.F_unit + fth[a];
    double x = p.pos[a * n + i] + (double)ov[a * n + r] * L + dtd * (double)(f * izt);
    if (x > half) x -= L;
    if (x < -half) x += L;
    p.pos[a * n + i] = x;
    if (p.xbuild) {
      float db = (float)(x - p.xbuild[a * n + i]);
      db -= Lf * rintf(db * iLf);
      disp2 += db * db;
    }
    double tp = p.truePos[a * n + i];
    const float wraps = rintf((float)(tp - x) * iLf);
    tp = x + (double)wraps * L;
    p.truePos[a * n + i] = tp;
    const double d = tp - p.posRef[a * n + i];
    acc[a] = d * d;
    bad |= !isfinite(x) || !isfinite((double)mf) || !isfinite((double)ef);
  }
  acc[3] = p.mm[2 * n + i];
  if (bad) atomicOr(p.err, kErrNonFinite);
}

// Block sums of the step records and the largest displacement since the
// last list build (every thread of the block calls this; blocks of up to
// kIntThreads threads).  The seven sums go through shared memory: a warp
// adds a record's column of values with one FP64 addition per warp of the
// block and five butterfly steps per lane (a butterfly per record and warp
// would take 7 x 5 per warp).
__device__ __forceinline__ void step_block_sums(const IntParams& p, int bx, const double acc[7], float disp2) {
  if (p.flags) {
    float d = sqrtf(disp2) * (1.0f / (float)p.L);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(kFull, d, o));
    if ((threadIdx.x & 31) == 0 && d > 0.f) atomicMax(&p.flags->maxdisp, __float_as_uint(d));
  }
  __shared__ double red[7][kIntThreads];
#pragma unroll
  for (int q = 0; q < 7; q++) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (int)blockDim.x >> 5;
  for (int q = w; q < 7; q += nw) {
    double s = red[q][l];
    for (int k = 1; k < nw; k++) s += red[q][l + 32 * k];
    s = warp_sum(s);
    if (l == 0) p.obs_part[7 * bx + q] = s;
  }
}

template <typename T>
__device__ __forceinline__ void heun2(const IntParams& p, int bx) {
  const int i = bx * (int)blockDim.x + threadIdx.x;
  const int n = p.n;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  float disp2 = 0;  // squared displacement since the last neighbour-list build
  if (i < n) {
    const int r = p.s.rank[i];
    const T* th = (const T*)p.th;
    T m[3], e[3], m2[3], e2[3], bd[3], tau[3], bth[3], k1m[3], k1e[3], fth[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      m[a] = (T)p.mm[a * n + i];
      e[a] = (T)p.ea[a * n + i];
      m2[a] = ((const T*)p.m2)[a * n + i];
      e2[a] = ((const T*)p.e2)[a * n + i];
      k1m[a] = ((const T*)p.k1m)[a * n + i];
      k1e[a] = ((const T*)p.k1e)[a * n + i];
      tau[a] = th[a * n + i];
      bth[a] = th[(3 + a) * n + i];
      fth[a] = th[(6 + a) * n + i];
    }
    // strong-pair partials: the field of this (field-only) evaluation, the
    // force and pressure of the step's full evaluation, in one pass
    double sb[3], sfp[6];
    const bool hs = p.sv.sums(r, p.sv.B, sb, p.sv.F, sfp, p.sv.P, sfp + 3);
    demag_si<T>(p, r, bd, hs ? sb : nullptr);
    const T bz = (T)ext_field_z(p, *p.time);
    T km[3], ke[3];
    rk<T>(p, m2, e2, bd, bz, bth, tau, (T)p.velEa1[i], (T)p.velEa2[i], km, ke);
    const T dt = (T)p.dt, h = (T)0.5;
    T mn[3], en[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      en[a] = e[a] + dt * (h * k1e[a] + h * ke[a]);
      mn[a] = m[a] + dt * (h * k1m[a] + h * km[a]);
    }
    finish_particle<T>(p, i, r, mn, en, fth, acc, disp2, hs ? sfp : nullptr);
  }
  step_block_sums(p, bx, acc, disp2);
}

__device__ __forceinline__ void obs(const ObsParams& p) {
  __shared__ double red[7][8];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < p.nblk_int; b += blockDim.x)
    for (int q = 0; q < 7; q++) acc[q] += __ldcg(p.obs_part + 7 * b + q);
  for (int q = 0; q < 7; q++) {
    const double v = warp_sum(acc[q]);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[7];
    for (int q = 0; q < 7; q++) {
      s[q] = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) s[q] += red[q][w];
    }
    const long long k = *p.nrec;
    if (k < p.cap) {
      double* o = p.records + 8 * k;
      o[0] = *p.time;
      o[1] = s[3] * p.inv_n;
      o[2] = s[0] * p.inv_n;
      o[3] = s[1] * p.inv_n;
      o[4] = s[2] * p.inv_n;
      o[5] = s[4] * p.p_scale;
      o[6] = s[5] * p.p_scale;
      o[7] = s[6] * p.p_scale;
      *p.nrec = k + 1;
    }
    *p.time += p.dt;
    *p.stepno += 1;
    if (p.status) *p.status = *p.err | (p.flags->overflow ? 4 : 0);
  }
}

template <typename T>
__global__ void __launch_bounds__(kIntThreads) k_heun1(IntParams p) {
  heun1<T>(p, blockIdx.x);
}
__global__ void __launch_bounds__(256) k_obs(ObsParams p) { obs(p); }

// Stage 2 and the step records in one launch: the block that finishes last
// (counted in *done) sums the blocks' partials in block order, so the
// records do not depend on which block that is, and clears the counter.
// Launched in blocks of kIntOne threads (bounded so: 72 registers and no
// spills, where the bound of kIntThreads gave 64 and spilled).
template <typename T>
__global__ void __launch_bounds__(kIntOne) k_heun2_obs(IntParams p, ObsParams o, unsigned* done) {
  heun2<T>(p, blockIdx.x);
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  obs(o);
  if (threadIdx.x == 0) *done = 0;
}

// persistent: blocks stride over the task table (see md_cells.cu)
__global__ void __launch_bounds__(kIntThreads, 4) k_heun1_packed(const IntParams* __restrict__ ps,
                                                             const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<false>(tk, ntask, wq, [&](const Task& t) {
      heun1<float>(ps[t.rep], t.blk);
  });
}
__global__ void __launch_bounds__(kIntThreads, 4) k_heun2_packed(const IntParams* __restrict__ ps,
                                                             const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      heun2<float>(ps[t.rep], t.blk);
  });
}
// The step's last packed kernel: it also clears the batch's rebuild word
// (raised by k_step_begin_packed; every reader of it ran earlier in the step).
__global__ void __launch_bounds__(256) k_obs_packed(const ObsParams* __restrict__ ps, unsigned* anyrb) {
  const ObsParams p = ps[blockIdx.x];
  obs(p);
  if (blockIdx.x == 0 && threadIdx.x == 0) *anyrb = 0u;
}

// B and F in SI, particle order; optional overlap push of the positions
// (CompInteractVecs moves the positions, src/interaction.cpp:126-127).
template <typename T>
__global__ void k_combine(IntParams p, double* Bout, double* Fout, int apply_overlap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = p.n;
  if (i >= n) return;
  const int r = p.s.rank[i];
  double b[3];  // reported field: no rounding to the integrator's type
  demag_si<T, double>(p, r, b);
  double sf[3];
  p.sv.sum3(p.sv.F, r, sf);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (Bout) Bout[a * n + i] = b[a];
    if (Fout) Fout[a * n + i] = ((double)((const T*)p.Fr)[a * n + r] + sf[a] + (double)((const T*)p.Fk)[a * n + r]) *
                                p.F_unit;
    if (apply_overlap) p.pos[a * n + i] += (double)((const T*)p.ov)[a * n + r] * p.L;
  }
}

// Real-space part alone (field without the k-space, self and surface terms;
// force without the k-space force), particle order, SI.
template <typename T>
__global__ void k_real_part(IntParams p, double* Bout, double* Fout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = p.n;
  if (i >= n) return;
  const int r = p.s.rank[i];
  double sb[3], sf[3];
  p.sv.sum3(p.sv.B, r, sb);
  p.sv.sum3(p.sv.F, r, sf);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    Bout[a * n + i] = ((double)((const T*)p.Br)[a * n + r] + sb[a]) * p.B_unit;
    Fout[a * n + i] = ((double)((const T*)p.Fr)[a * n + r] + sf[a]) * p.F_unit;
  }
}

int launch_real_part(cudaStream_t st, const IntParams& p, double* Bout, double* Fout, bool fp64) {
  if (fp64)
    k_real_part<double><<<(p.n + 255) / 256, 256, 0, st>>>(p, Bout, Fout);
  else
    k_real_part<float><<<(p.n + 255) / 256, 256, 0, st>>>(p, Bout, Fout);
  return 1;
}

// ------------------------------------------------ adaptive Runge-Kutta
// IntegrationRot with SOLVER = 0, 1, 2 and the reference's step control
// (src/simulation.cpp:707-871): one kernel per stage s evaluates the slopes
// k_s at the stage coordinates with the field last evaluated there, and
// forms the next stage's coordinates (written into the sorted view for the
// next field evaluation) or, at the last stage, the error norm
// max_i |sum_j e_j km_j,i|.  The host runs the step control
// (AdjustTimeStep) and launches the accept kernel with the step used.

template <typename T>
__device__ __forceinline__ void noise9(const IntParams& p, int i, T z[9]) {
  const int n = p.n;
  if (p.noise == 2) {
    philox_normals9<T>(p.seed, (uint64_t)*p.stepno, (uint32_t)i, z);
  } else if (p.noise == 1) {
#pragma unroll
    for (int q = 0; q < 9; q++) z[q] = (T)p.xi[(q / 3) * 3 * n + (q % 3) * n + i];
  } else {
#pragma unroll
    for (int q = 0; q < 9; q++) z[q] = 0;
  }
}

template <typename T>
__global__ void __launch_bounds__(kIntThreads) k_rk_stage(RKStage q) {
  using T4 = typename V4<T>::t;
  const IntParams& p = q.p;
  const int i = blockIdx.x * kIntThreads + threadIdx.x;
  const int n = p.n;
  double err = 0.0;
  if (i < n) {
    const int r = p.s.rank[i];
    T m[3], e[3], bd[3], z[9], tau[3], bth[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      m[a] = q.s == 0 ? (T)p.mm[a * n + i] : ((const T*)q.cm)[a * n + i];
      e[a] = q.s == 0 ? (T)p.ea[a * n + i] : ((const T*)q.ce)[a * n + i];
    }
    demag_si<T>(p, r, bd);
    noise9<T>(p, i, z);
    const T sT = (T)(p.sT[i] * q.nf), sB = (T)(p.sB[i] * q.nf);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      tau[a] = sT * z[a];
      bth[a] = sB * z[3 + a];
    }
    const T bz = (T)ext_field_z(p, *p.time);
    T km[3], ke[3];
    rk<T>(p, m, e, bd, bz, bth, tau, (T)p.velEa1[i], (T)p.velEa2[i], km, ke);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      ((T*)q.km[q.s])[a * n + i] = km[a];
      ((T*)q.ke[q.s])[a * n + i] = ke[a];
    }
    if (!q.last) {
      // next stage: y0 + dt sum_{j <= s} a_j k_j, formed in FP64 (the
      // Dormand-Prince weights reach ~12 and cancel)
      T nm[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        double sm = 0, se = 0;
        for (int j = 0; j <= q.s; j++) {
          if (q.a[j] == 0.0) continue;
          const double kmj = j == q.s ? (double)km[a] : (double)((const T*)q.km[j])[a * n + i];
          const double kej = j == q.s ? (double)ke[a] : (double)((const T*)q.ke[j])[a * n + i];
          sm += q.a[j] * kmj;
          se += q.a[j] * kej;
        }
        ((T*)q.ce)[a * n + i] = (T)(p.ea[a * n + i] + p.dt * se);
        nm[a] = (T)(p.mm[a * n + i] + p.dt * sm);
        ((T*)q.cm)[a * n + i] = nm[a];
      }
      const T mu = (T)p.magMom_u[i];
      T4 v;
      v.x = nm[0] * mu;
      v.y = nm[1] * mu;
      v.z = nm[2] * mu;
      v.w = (T)p.rMag_u[i];
      ((T4*)p.s.mu)[r] = v;
    } else {
      double ev[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        double sm = 0;
        for (int j = 0; j <= q.s; j++) {
          if (q.e[j] == 0.0) continue;
          const double kmj = j == q.s ? (double)km[a] : (double)((const T*)q.km[j])[a * n + i];
          sm += q.e[j] * kmj;
        }
        ev[a] = sm;
      }
      err = sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
    }
  }
  if (q.last) {
    // non-negative doubles order like their bit patterns
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(kFull, err, o));
    if ((threadIdx.x & 31) == 0 && err > 0.0)
      atomicMax(q.errmax, (unsigned long long)__double_as_longlong(err));
  }
}

template <typename T>
__global__ void __launch_bounds__(kIntThreads) k_rk_accept(RKStage q) {
  const IntParams& p = q.p;
  const int i = blockIdx.x * kIntThreads + threadIdx.x;
  const int n = p.n;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  float disp2 = 0;
  if (i < n) {
    const int r = p.s.rank[i];
    T mn[3], en[3], z[9], fth[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (q.last) {  // Bogacki-Shampine: the last stage's coordinates
        mn[a] = ((const T*)q.cm)[a * n + i];
        en[a] = ((const T*)q.ce)[a * n + i];
      } else {
        double sm = 0, se = 0;
        for (int j = 0; j <= q.s; j++) {
          if (q.a[j] == 0.0) continue;
          sm += q.a[j] * (double)((const T*)q.km[j])[a * n + i];
          se += q.a[j] * (double)((const T*)q.ke[j])[a * n + i];
        }
        en[a] = (T)(p.ea[a * n + i] + p.dt * se);
        mn[a] = (T)(p.mm[a * n + i] + p.dt * sm);
      }
    }
    // the thermal force at the scale of the step's first trial (the
    // reference rescales it on rejections only after it entered the force)
    noise9<T>(p, i, z);
    const T sF = (T)p.sF[i];
#pragma unroll
    for (int a = 0; a < 3; a++) fth[a] = sF * z[6 + a];
    finish_particle<T>(p, i, r, mn, en, fth, acc, disp2);
  }
  step_block_sums(p, blockIdx.x, acc, disp2);
}

int launch_rk_stage(cudaStream_t st, const RKStage& q, bool fp64) {
  const int g = (q.p.n + kIntThreads - 1) / kIntThreads;
  if (fp64)
    k_rk_stage<double><<<g, kIntThreads, 0, st>>>(q);
  else
    k_rk_stage<float><<<g, kIntThreads, 0, st>>>(q);
  return 1;
}

int launch_rk_accept(cudaStream_t st, const RKStage& q, bool fp64) {
  const int g = (q.p.n + kIntThreads - 1) / kIntThreads;
  if (fp64)
    k_rk_accept<double><<<g, kIntThreads, 0, st>>>(q);
  else
    k_rk_accept<float><<<g, kIntThreads, 0, st>>>(q);
  return 1;
}

int int_blocks(int n) { return (n + kIntThreads - 1) / kIntThreads; }
int int_blocks_one(int n) { return (n + kIntOne - 1) / kIntOne; }

int launch_heun1(cudaStream_t st, const IntParams& p, bool fp64) {
  if (fp64)
    k_heun1<double><<<int_blocks_one(p.n), kIntOne, 0, st>>>(p);
  else
    k_heun1<float><<<int_blocks_one(p.n), kIntOne, 0, st>>>(p);
  return 1;
}

int launch_heun2_obs(cudaStream_t st, const IntParams& p, const ObsParams& o_in, unsigned* done, bool fp64) {
  ObsParams o = o_in;
  o.nblk_int = int_blocks_one(p.n);  // partials of this launch's blocks
  if (fp64)
    k_heun2_obs<double><<<int_blocks_one(p.n), kIntOne, 0, st>>>(p, o, done);
  else
    k_heun2_obs<float><<<int_blocks_one(p.n), kIntOne, 0, st>>>(p, o, done);
  return 1;
}

int launch_obs(cudaStream_t st, const ObsParams& p) {
  k_obs<<<1, 256, 0, st>>>(p);
  return 1;
}

int launch_heun1_packed(cudaStream_t st, const IntParams* ps, const Packed& n256) {
  if (!n256.n) return 0;
  k_heun1_packed<<<persistent_grid((const void*)k_heun1_packed, kIntThreads, 0, n256.n), kIntThreads, 0, st>>>(ps, n256.tasks, n256.n, n256.wq);
  return 1;
}

int launch_heun2_packed(cudaStream_t st, const IntParams* ps, const Packed& n256) {
  if (!n256.n) return 0;
  k_heun2_packed<<<persistent_grid((const void*)k_heun2_packed, kIntThreads, 0, n256.n), kIntThreads, 0, st>>>(ps, n256.tasks, n256.n, n256.wq);
  return 1;
}

int launch_obs_packed(cudaStream_t st, const ObsParams* ps, int R, unsigned* anyrb) {
  if (!R) return 0;
  k_obs_packed<<<R, 256, 0, st>>>(ps, anyrb);
  return 1;
}

int launch_combine(cudaStream_t st, const IntParams& p, double* Bout, double* Fout, int apply_overlap, bool fp64) {
  if (fp64)
    k_combine<double><<<(p.n + 255) / 256, 256, 0, st>>>(p, Bout, Fout, apply_overlap);
  else
    k_combine<float><<<(p.n + 255) / 256, 256, 0, st>>>(p, Bout, Fout, apply_overlap);
  return 1;
}

}  // namespace md
