// md_kspace.cu -- kernel (c): reciprocal-space Ewald sum.  Restates
// CompDipInteractEwaldF / CompDipFieldEwaldF (src/interaction.cpp:429-514,
// 588-672) with the phases of EvalSinCos (src/interaction.cpp:521-548):
//   S_c(n) + i S_s(n) = sum_j (n . mu_j) exp(2 pi i n . r_j / L)
//   B_i -= cFluxDens e(n) (S_c pc_i + S_s ps_i) n
//   F_i += cForce e(n) (n . mu_i) (S_c ps_i - S_s pc_i) n
// over 0 < |n|^2 <= kc^2 in the half space.  The reference sums the whole
// nz = 0 plane with e/2; since the n and -n terms of that plane are equal,
// this code sums half of the plane (ny > 0, or ny = 0 and nx > 0) with the
// full e(n).  The self and surface terms are added in the integrator.
//
// Phase tables (k_phase_tables, once per step -- positions are frozen across
// the two Heun stages): X(n) = exp(2 pi i n x / L) per particle and axis,
// n = 0..kc, evaluated directly for n < 4 and multiples of 4, otherwise as one
// product of two direct entries.  Direct phases: on the mixed path n x / L is
// reduced exactly in 32-bit fixed point before sincospif; the FP64 path uses
// sincos(2 my_pi n x / L) like the reference.  Layout [3][kc+1][n].
//
// k vectors are row segments (fixed ny, nz; up to 16 consecutive nx, padded
// to a multiple of 4 with e = 0).  Within a segment the phase is advanced by
// one complex multiply per k from a table entry (<= 15 recurrence steps).
//
// Structure factor (k_sk): threads = segments (sorted by length so warps are
// uniform), particles staged through shared-memory tiles of 64; FP32 sums over
// a chunk of <= 512 particles, FP64 across chunks (k_sk_reduce), which also
// applies e(n) and writes e*S in row order for the scatter.
// Scatter (k_kscatter): threads = (particle, partition); whole k rows (its own
// layout: one segment per row up to 64 k's, so the per-segment work of phase
// setup and sums is paid once per row) are grouped into chunks staged in
// shared memory and dealt round-robin to 4 partitions
// of threads that share the particle's tables; FP32 per segment, blocks of 8
// segments added with Kahan compensation (mixed path); the partitions are
// summed in a fixed order.
//
// Roofline: FP32 issue bound.  Algorithmic FLOPs per (k, particle): 11 for
// the structure factor, 12 for the field scatter, 21 for field + force.
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kSkThreads = 128;
constexpr int kSkTile = 64;
constexpr int kSegMax = 16;

// exp(2 pi i n x) evaluated directly.
template <typename T>
__device__ __forceinline__ typename V2<T>::t phase_direct(int nn, unsigned sfix, double xb, double two_pi) {
  using T2 = typename V2<T>::t;
  T2 v;
  if constexpr (std::is_same<T, float>::value) {
    const int ph = (int)((unsigned)nn * sfix);  // exact reduction mod one box length
    float s, c;
    sincospif(2.0f * ((float)ph * 2.3283064365386963e-10f), &s, &c);
    v.x = c;
    v.y = s;
  } else {
    double s, c;
    sincos(two_pi * (double)nn * xb, &s, &c);
    v.x = c;
    v.y = s;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ void particle_coord(const SortedView& s, int k, int ax, unsigned& sfix, double& xb) {
  if constexpr (std::is_same<T, float>::value) {
    const int4 q = s.xi[k];
    sfix = (unsigned)(ax == 0 ? q.x : (ax == 1 ? q.y : q.z));
    xb = 0.0;
  } else {
    const double4_32a q = s.xd[k];
    xb = ax == 0 ? q.x : (ax == 1 ? q.y : q.z);
    sfix = 0;
  }
}

// ------------------------------------------------------------ phase tables

constexpr int kPhaseThreads = 256;

template <typename T>
__device__ __forceinline__ void phase_tables(const KParams& p, int bx) {
  using T2 = typename V2<T>::t;
  const int t = bx * kPhaseThreads + threadIdx.x;
  if (t >= 3 * p.n) return;
  const int ax = t / p.n, k = t - ax * p.n;
  unsigned sf;
  double xb;
  particle_coord<T>(p.s, k, ax, sf, xb);
  T2* tab = (T2*)p.tab;
  const int K1 = p.kc + 1;
  const size_t stride = (size_t)p.n;
  T2* out = tab + (size_t)ax * K1 * stride + k;
  T2 d[4];
  for (int nn = 0; nn <= p.kc; nn++) {
    T2 v;
    if (nn < 4) {
      v = phase_direct<T>(nn, sf, xb, p.two_pi);
      d[nn] = v;
    } else if ((nn & 3) == 0) {
      v = phase_direct<T>(nn, sf, xb, p.two_pi);
      d[0] = v;  // anchor of this block of 4
    } else {
      const T2 a = d[0];
      const T2 b = (nn & 3) == 1 ? d[1] : ((nn & 3) == 2 ? d[2] : d[3]);
      cmul<T>(a.x, a.y, b.x, b.y, v.x, v.y);
    }
    out[(size_t)nn * stride] = v;
  }
}

// ------------------------------------------------------ structure factor

template <typename T>
__device__ __forceinline__ void sk_body(const KParams& p, int bx, int by) {
  using T2 = typename V2<T>::t;
  using T4 = typename V4<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K1 = p.kc + 1, E3 = 3 * K1;
  T2* tab = (T2*)smem_raw;                   // [kSkTile][3][K1]
  T4* mus = (T4*)(tab + kSkTile * E3);       // [kSkTile]
  const T2* gtab = (const T2*)p.tab;
  const int tid = threadIdx.x;
  const int sidx = bx * kSkThreads + tid;
  const int chunk = by;
  const int p0 = chunk * p.chunk, p1 = min(p.n, p0 + p.chunk);
  const bool has = sidx < p.nseg;
  KSeg sg = {0, 0, 0, 0};
  if (has) sg = p.seg[sidx];
  const int len = sg.len;
  const int ax0 = sg.nx0 < 0 ? -sg.nx0 : sg.nx0, ay = sg.ny < 0 ? -sg.ny : sg.ny;
  const T nx0f = (T)sg.nx0, nyf = (T)sg.ny, nzf = (T)sg.nz;
  T sc[kSegMax], ss[kSegMax];
#pragma unroll
  for (int c = 0; c < kSegMax; c++) sc[c] = ss[c] = 0;

  for (int t0 = p0; t0 < p1; t0 += kSkTile) {
    const int tn = min(kSkTile, p1 - t0);
    __syncthreads();
    for (int i = tid; i < tn * E3; i += kSkThreads) {
      const int e = i / tn, pp = i - e * tn;
      tab[pp * E3 + e] = gtab[(size_t)e * p.n + t0 + pp];
    }
    for (int pp = tid; pp < tn; pp += kSkThreads) mus[pp] = ((const T4*)p.s.mu)[t0 + pp];
    __syncthreads();
    if (!has) continue;
    for (int pp = 0; pp < tn; pp++) {
      const T2* tb = tab + pp * E3;
      T2 X = tb[ax0], Y = tb[K1 + ay];
      const T2 Z = tb[2 * K1 + sg.nz], E = tb[1];
      if (sg.nx0 < 0) X.y = -X.y;
      if (sg.ny < 0) Y.y = -Y.y;
      T yr, yi, pr, pi;
      cmul<T>(Y.x, Y.y, Z.x, Z.y, yr, yi);
      cmul<T>(X.x, X.y, yr, yi, pr, pi);
      const T4 mu = mus[pp];
      T w = nx0f * mu.x + nyf * mu.y + nzf * mu.z;
#pragma unroll
      for (int c = 0; c < kSegMax; c += 4) {
        if (c >= len) break;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          sc[c + u] += w * pr;
          ss[c + u] += w * pi;
          const T npr = pr * E.x - pi * E.y;
          pi = pr * E.y + pi * E.x;
          pr = npr;
          w += mu.x;
        }
      }
    }
  }
  if (has) {
    double2* out = p.Spart + (size_t)chunk * p.nk + p.koff[sidx];
#pragma unroll
    for (int c = 0; c < kSegMax; c++)
      if (c < len) out[c] = make_double2((double)sc[c], (double)ss[c]);
  }
  if (bx == 0) {
    // sum of moments of this chunk (surface term), FP64
    double m0 = 0, m1 = 0, m2 = 0;
    for (int q = p0 + tid; q < p1; q += kSkThreads) {
      const T4 mu = ((const T4*)p.s.mu)[q];
      m0 += (double)mu.x;
      m1 += (double)mu.y;
      m2 += (double)mu.z;
    }
    __shared__ double red[3][kSkThreads / 32];
    m0 = warp_sum(m0);
    m1 = warp_sum(m1);
    m2 = warp_sum(m2);
    if ((tid & 31) == 0) {
      red[0][tid >> 5] = m0;
      red[1][tid >> 5] = m1;
      red[2][tid >> 5] = m2;
    }
    __syncthreads();
    if (tid < 3) {
      double s = 0;
      for (int w = 0; w < kSkThreads / 32; w++) s += red[tid][w];
      p.musum_part[3 * chunk + tid] = s;
    }
  }
}

// Sum of the chunk partials: block = 32 k's x 8 chunk groups, fixed order.
template <typename T>
__device__ __forceinline__ void sk_reduce(const KParams& p, int bx) {
  using T2 = typename V2<T>::t;
  __shared__ double2 red[8][32];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int kk = bx * 32 + tx;
  double a = 0, b = 0;
  if (kk < p.nk)
    for (int c = ty; c < p.nchunk; c += 8) {
      const double2 v = p.Spart[(size_t)c * p.nk + kk];
      a += v.x;
      b += v.y;
    }
  red[ty][tx] = make_double2(a, b);
  __syncthreads();
  if (ty == 0 && kk < p.nk) {
    for (int g = 1; g < 8; g++) {
      a += red[g][tx].x;
      b += red[g][tx].y;
    }
    p.S[kk] = make_double2(a, b);
    const double e = p.ek[kk];
    T2 o;
    o.x = (T)(e * a);
    o.y = (T)(e * b);
    const int pos = p.rowpos[kk];
    if (pos >= 0) ((T2*)p.eS)[pos] = o;
  }
  if (bx == 0 && threadIdx.x < 3) {
    double s = 0;
    for (int c = 0; c < p.nchunk; c++) s += p.musum_part[3 * c + threadIdx.x];
    p.musum[threadIdx.x] = s;
  }
}

// ---------------------------------------------------------------- scatter

template <typename T>
__device__ __forceinline__ void kahan_add(T& s, T& c, T v) {
  if constexpr (std::is_same<T, float>::value) {
    const float y = v - c, t = s + y;
    c = (t - s) - y;
    s = t;
  } else {
    s += v;
  }
}

template <typename T, int NP, bool FULL>
__device__ __forceinline__ void kscatter(const KParams& p, int bx, int kcmax) {
  using T2 = typename V2<T>::t;
  using T4 = typename V4<T>::t;
  constexpr int NT = NP * kScatterParts;
  constexpr int kSegChunk = kKChunk / 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K1 = p.kc + 1, E3 = 3 * K1;
  T2* tab = (T2*)smem_raw;                       // [3 * K1][NP]
  T2* es_all = tab + 3 * (kcmax + 1) * NP;       // [parts][kKChunk]
  KSeg* seg_all = (KSeg*)(es_all + kScatterParts * kKChunk);  // [parts][kSegChunk]
  T* red = (T*)es_all;                           // [parts][6][NP], after the loop
  const int tid = threadIdx.x;
  const int part = tid / NP, lp = tid - part * NP;
  const int base = bx * NP;
  const int k = base + lp;
  const bool active = k < p.n;
  const int kk = active ? k : p.n - 1;
  const T2* gtab = (const T2*)p.tab;
  for (int i = tid; i < E3 * NP; i += NT) {
    const int e = i / NP, q = i - e * NP;
    tab[i] = gtab[(size_t)e * p.n + min(base + q, p.n - 1)];
  }
  const T4 mu = ((const T4*)p.s.mu)[kk];
  T2* es_s = es_all + part * kKChunk;
  KSeg* seg_s = seg_all + part * kSegChunk;
  __syncthreads();
  const T2 E = tab[1 * NP + lp];
  T b[3] = {0, 0, 0}, f[3] = {0, 0, 0}, cb[3] = {0, 0, 0}, cf[3] = {0, 0, 0};
  T bb[3] = {0, 0, 0}, fb[3] = {0, 0, 0};
  int cur_ny = 1 << 30, cur_nz = 1 << 30, nflush = 0;
  T yzr = 0, yzi = 0;
  const int rounds = (p.nchk + kScatterParts - 1) / kScatterParts;
  for (int r = 0; r < rounds; r++) {
    const int c = r * kScatterParts + part;
    const bool mine = c < p.nchk;
    int nsg = 0;
    __syncthreads();
    if (mine) {
      const int2 c0 = p.chunks[c], c1 = p.chunks[c + 1];
      nsg = c1.x - c0.x;
      const int nkc = c1.y - c0.y;
      for (int i = lp; i < nkc; i += NP) es_s[i] = ((const T2*)p.eS)[c0.y + i];
      for (int i = lp; i < nsg; i += NP) seg_s[i] = p.rseg[c0.x + i];
    }
    __syncthreads();
    int ko = 0;
    for (int s = 0; s < nsg; s++) {
      const KSeg sg = seg_s[s];
      if (sg.nz != cur_nz || sg.ny != cur_ny) {
        T2 Y = tab[(K1 + (sg.ny < 0 ? -sg.ny : sg.ny)) * NP + lp];
        const T2 Z = tab[(2 * K1 + sg.nz) * NP + lp];
        if (sg.ny < 0) Y.y = -Y.y;
        cmul<T>(Y.x, Y.y, Z.x, Z.y, yzr, yzi);
        cur_ny = sg.ny;
        cur_nz = sg.nz;
      }
      T2 X = tab[(sg.nx0 < 0 ? -sg.nx0 : sg.nx0) * NP + lp];
      if (sg.nx0 < 0) X.y = -X.y;
      T pr, pi;
      cmul<T>(X.x, X.y, yzr, yzi, pr, pi);
      // k = (nx0 + u, ny, nz), u = 0..len-1: the field takes G n with
      // G = Re(conj(eS) phase), the force H (n . mu) n with H = Im(conj(eS)
      // phase); n_x and n . mu advance by 1 and mu_x per k
      T nxf = (T)sg.nx0;
      T w = 0;
      if constexpr (FULL) w = nxf * mu.x + (T)sg.ny * mu.y + (T)sg.nz * mu.z;
      T gx = 0, gs = 0, hx = 0, hs = 0;
      const T2* es_seg = es_s + ko;
#pragma unroll
      for (int q = 0; q < kScatSeg; q += 4) {
        if (q >= sg.len) break;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const T2 es = es_seg[q + u];
          const T g = es.x * pr + es.y * pi;
          gx += g * nxf;
          gs += g;
          if constexpr (FULL) {
            const T h = (es.x * pi - es.y * pr) * w;
            hx += h * nxf;
            hs += h;
            w += mu.x;
          }
          const T npr = pr * E.x - pi * E.y;
          pi = pr * E.y + pi * E.x;
          pr = npr;
          nxf += (T)1;
        }
      }
      ko += sg.len;
      bb[0] += gx;
      bb[1] += gs * (T)sg.ny;
      bb[2] += gs * (T)sg.nz;
      if constexpr (FULL) {
        fb[0] += hx;
        fb[1] += hs * (T)sg.ny;
        fb[2] += hs * (T)sg.nz;
      }
      if (++nflush == 8) {
        nflush = 0;
#pragma unroll
        for (int a = 0; a < 3; a++) {
          kahan_add<T>(b[a], cb[a], bb[a]);
          bb[a] = 0;
          if constexpr (FULL) {
            kahan_add<T>(f[a], cf[a], fb[a]);
            fb[a] = 0;
          }
        }
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 3; a++) {
    kahan_add<T>(b[a], cb[a], bb[a]);
    if constexpr (FULL) kahan_add<T>(f[a], cf[a], fb[a]);
  }
  __syncthreads();  // staging buffers are reused for the partition reduction
#pragma unroll
  for (int a = 0; a < 3; a++) {
    red[(part * 6 + a) * NP + lp] = b[a] - cb[a];
    if constexpr (FULL) red[(part * 6 + 3 + a) * NP + lp] = f[a] - cf[a];
  }
  __syncthreads();
  if (part == 0 && active) {
    T* B = (T*)p.B;
    const int n = p.n;
    const T cfl = (T)p.cflux, cfo = (T)p.cforce;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      T s = 0;
      for (int q = 0; q < kScatterParts; q++) s += red[(q * 6 + a) * NP + lp];
      B[a * n + k] = -cfl * s;
    }
    if constexpr (FULL) {
      T* F = (T*)p.F;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        T s = 0;
        for (int q = 0; q < kScatterParts; q++) s += red[(q * 6 + 3 + a) * NP + lp];
        F[a * n + k] = cfo * s;
      }
    }
  }
}

// ------------------------------------------------------------ entry points

template <typename T>
__global__ void __launch_bounds__(kPhaseThreads) k_phase_tables(KParams p) {
  phase_tables<T>(p, blockIdx.x);
}
template <typename T>
__global__ void __launch_bounds__(kSkThreads, 6) k_sk(KParams p) {
  sk_body<T>(p, blockIdx.x, blockIdx.y);
}
template <typename T>
__global__ void __launch_bounds__(256) k_sk_reduce(KParams p) {
  sk_reduce<T>(p, blockIdx.x);
}
template <typename T, int NP, bool FULL>
__global__ void __launch_bounds__(NP * kScatterParts) k_kscatter(KParams p) {
  kscatter<T, NP, FULL>(p, blockIdx.x, p.kc);
}

// persistent: blocks stride over the task table (see md_cells.cu)
__global__ void __launch_bounds__(kPhaseThreads) k_phase_tables_packed(const KParams* __restrict__ ps,
                                                                       const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<false>(tk, ntask, wq, [&](const Task& t) {
      phase_tables<float>(ps[t.rep], t.blk);
  });
}
__global__ void __launch_bounds__(kSkThreads, 6) k_sk_packed(const KParams* __restrict__ ps,
                                                              const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      const KParams p = ps[t.rep];
      const int nsb = (p.nseg + kSkThreads - 1) / kSkThreads;
      sk_body<float>(p, t.blk % nsb, t.blk / nsb);
  });
}
__global__ void __launch_bounds__(256) k_sk_reduce_packed(const KParams* __restrict__ ps,
                                                          const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      sk_reduce<float>(ps[t.rep], t.blk);
  });
}
template <int NP, bool FULL>
__global__ void __launch_bounds__(NP * kScatterParts) k_kscatter_packed(const KParams* __restrict__ ps,
                                                                        const Task* __restrict__ tk, int kcmax,
                                                                        int ntask, WorkQ* wq) {
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      kscatter<float, NP, FULL>(ps[t.rep], t.blk, kcmax);
  });
}

int sk_threads() { return kSkThreads; }

int sk_resident_blocks(int kc, bool fp64) {
  int nb = 0;
  const size_t sm = ksf_smem(kc, fp64);
  cudaError_t e;
  if (fp64) {
    cudaFuncSetAttribute(k_sk<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_sk<double>, kSkThreads, sm);
  } else {
    cudaFuncSetAttribute(k_sk<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_sk<float>, kSkThreads, sm);
  }
  return (e == cudaSuccess && nb > 0) ? nb : 1;
}

int phase_blocks(int n) { return (3 * n + kPhaseThreads - 1) / kPhaseThreads; }
int sk_blocks(const KParams& p) { return (p.nseg + kSkThreads - 1) / kSkThreads * p.nchunk; }
int skred_blocks(const KParams& p) { return (p.nk + 31) / 32; }
int scatter_blocks(const KParams& p, int np) { return (p.n + np - 1) / np; }

size_t ksf_smem(int kc, bool fp64) {
  const size_t e = fp64 ? 16 : 8;
  return (size_t)kSkTile * 3 * (kc + 1) * e + (size_t)kSkTile * (fp64 ? 32 : 16);
}

static size_t scatter_bytes(int kc, bool fp64, int np) {
  const size_t e = fp64 ? 16 : 8;
  return (size_t)3 * (kc + 1) * np * e + (size_t)kScatterParts * kKChunk * e +
         (size_t)kScatterParts * (kKChunk / 4) * sizeof(KSeg);
}

int scatter_particles(int kc, bool fp64) {
  for (int np : {64, 32})
    if (scatter_bytes(kc, fp64, np) <= 200 * 1024) return np;
  return 0;
}

size_t kscatter_smem(int kc, bool fp64) {
  const int np = scatter_particles(kc, fp64);
  return np ? scatter_bytes(kc, fp64, np) : 0;
}

template <typename T, int NP>
static void scatter_launch(cudaStream_t st, const KParams& p, bool full, size_t smem) {
  dim3 grid((p.n + NP - 1) / NP);
  if (full) {
    cudaFuncSetAttribute(k_kscatter<T, NP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_kscatter<T, NP, true><<<grid, NP * kScatterParts, smem, st>>>(p);
  } else {
    cudaFuncSetAttribute(k_kscatter<T, NP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_kscatter<T, NP, false><<<grid, NP * kScatterParts, smem, st>>>(p);
  }
}

template <typename T>
static int kspace_t(cudaStream_t st, const KParams& p, bool full, cudaEvent_t* ev) {
  const bool fp64 = std::is_same<T, double>::value;
  const size_t sm1 = ksf_smem(p.kc, fp64);
  cudaFuncSetAttribute(k_sk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  dim3 g1((p.nseg + kSkThreads - 1) / kSkThreads, p.nchunk);
  k_sk<T><<<g1, kSkThreads, sm1, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[0], st, cudaEventRecordExternal);
  k_sk_reduce<T><<<(p.nk + 31) / 32, 256, 0, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[1], st, cudaEventRecordExternal);
  const size_t sm2 = kscatter_smem(p.kc, fp64);
  if (scatter_particles(p.kc, fp64) == 64)
    scatter_launch<T, 64>(st, p, full, sm2);
  else
    scatter_launch<T, 32>(st, p, full, sm2);
  return 3;
}

int launch_kspace(cudaStream_t st, const KParams& p, bool full, bool fp64, cudaEvent_t* ev) {
  if (!fp64 && p.tc_rows > 0) return launch_kspace_tc(st, p, full, ev);
  return fp64 ? kspace_t<double>(st, p, full, ev) : kspace_t<float>(st, p, full, ev);
}

int launch_phase_tables(cudaStream_t st, const KParams& p, bool fp64) {
  if (fp64)
    k_phase_tables<double><<<phase_blocks(p.n), kPhaseThreads, 0, st>>>(p);
  else
    k_phase_tables<float><<<phase_blocks(p.n), kPhaseThreads, 0, st>>>(p);
  if (!fp64 && p.tc_rows > 0) return 1 + launch_kspace_tc_prep(st, p);
  return 1;
}

int launch_phase_tables_packed(cudaStream_t st, const KParams* ps, const Packed& phase) {
  if (!phase.n) return 0;
  k_phase_tables_packed<<<persistent_grid((const void*)k_phase_tables_packed, kPhaseThreads, 0, phase.n),
                          kPhaseThreads, 0, st>>>(ps, phase.tasks, phase.n, phase.wq);
  return 1;
}

template <int NP>
static void scatter_packed(cudaStream_t st, const KParams* ps, const Packed& sc, bool full, int kcmax, size_t smem) {
  const int th = NP * kScatterParts;
  if (full) {
    cudaFuncSetAttribute(k_kscatter_packed<NP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int g = persistent_grid((const void*)k_kscatter_packed<NP, true>, th, smem, sc.n);
    k_kscatter_packed<NP, true><<<g, th, smem, st>>>(ps, sc.tasks, kcmax, sc.n, sc.wq);
  } else {
    cudaFuncSetAttribute(k_kscatter_packed<NP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int g = persistent_grid((const void*)k_kscatter_packed<NP, false>, th, smem, sc.n);
    k_kscatter_packed<NP, false><<<g, th, smem, st>>>(ps, sc.tasks, kcmax, sc.n, sc.wq);
  }
}

int launch_kspace_packed(cudaStream_t st, const KParams* ps, const Packed& sk, const Packed& red, const Packed& sc,
                         bool full, int kcmax, int np) {
  int l = 0;
  if (sk.n) {
    const size_t sm1 = ksf_smem(kcmax, false);
    cudaFuncSetAttribute(k_sk_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
    k_sk_packed<<<persistent_grid((const void*)k_sk_packed, kSkThreads, sm1, sk.n), kSkThreads, sm1, st>>>(
        ps, sk.tasks, sk.n, sk.wq);
    l++;
  }
  if (red.n) {
    k_sk_reduce_packed<<<persistent_grid((const void*)k_sk_reduce_packed, 256, 0, red.n), 256, 0, st>>>(
        ps, red.tasks, red.n, red.wq);
    l++;
  }
  if (sc.n) {
    const size_t sm2 = scatter_bytes(kcmax, false, np);
    if (np == 64)
      scatter_packed<64>(st, ps, sc, full, kcmax, sm2);
    else
      scatter_packed<32>(st, ps, sc, full, kcmax, sm2);
    l++;
  }
  return l;
}

// FP32 throughput calibration: 8 independent FMA chains per thread, 4096
// iterations, operands in registers.  The result is stored so the chains are
// not removed.
__global__ void __launch_bounds__(256) k_fma_calibration(float* out, float seed) {
  float a[8];
#pragma unroll
  for (int q = 0; q < 8; q++) a[q] = seed + (float)(threadIdx.x + q);
  const float b = 0.9999f, c = 1e-7f;
  for (int it = 0; it < 4096; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) a[q] = fmaf(a[q], b, c);
  }
  float s = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += a[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

double launch_fma_calibration(cudaStream_t st, float* out, int blocks, int threads) {
  k_fma_calibration<<<blocks, threads, 0, st>>>(out, 1.0f);
  return 2.0 * 8.0 * 4096.0 * (double)blocks * (double)threads;
}

}  // namespace md
