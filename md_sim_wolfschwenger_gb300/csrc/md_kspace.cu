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
// k vectors are stored as row segments (fixed ny, nz; up to 16 consecutive
// nx, padded to a multiple of 4 with e = 0).  Within a segment the phase is
// advanced by one complex multiply per k, starting from a directly evaluated
// phase (at most 16 recurrence steps).  Direct phases: on the mixed path the
// argument n x / L is reduced exactly in 32-bit fixed point before
// sincospif; the FP64 path uses sincos(2 my_pi n x / L) like the reference.
//
// Structure factor (k_sk): threads = segments (sorted by length so warps are
// uniform), particles staged through shared-memory tiles of 64 with their
// per-axis phase tables; FP32 sums over a chunk of <= 512 particles, FP64
// across chunks (k_sk_reduce), which also applies e(n) and writes e*S in row
// order for the scatter.
// Scatter (k_kscatter): threads = particles; the block walks the k rows in
// order, staging e*S and the segments chunk by chunk in shared memory; the
// x phase comes from a per-thread table, y and z phases per row (direct
// every 8th row, otherwise one multiply).  FP32 per segment, blocks of 8
// segments added with Kahan compensation (mixed path).
//
// Roofline: FP32 issue bound.  Algorithmic FLOPs per (k, particle): 11 for
// the structure factor, 12 for the field scatter, 21 for field + force.
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kSkThreads = 256;
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

// Table of exp(2 pi i n x) for n = 0..kc at out[n * stride]: direct for
// n < 4 and multiples of 4, otherwise the product of two direct entries.
template <typename T>
__device__ __forceinline__ void fill_table(typename V2<T>::t* out, int stride, int kc, unsigned sfix, double xb,
                                           double two_pi) {
  using T2 = typename V2<T>::t;
  for (int nn = 0; nn <= kc; nn++) {
    T2 v;
    if (nn < 4 || (nn & 3) == 0) {
      v = phase_direct<T>(nn, sfix, xb, two_pi);
    } else {
      const T2 a = out[(nn & ~3) * stride], b = out[(nn & 3) * stride];
      cmul<T>(a.x, a.y, b.x, b.y, v.x, v.y);
    }
    out[nn * stride] = v;
  }
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

// ------------------------------------------------------ structure factor

template <typename T>
__global__ void __launch_bounds__(kSkThreads, 2) k_sk(KParams p) {
  using T2 = typename V2<T>::t;
  using T4 = typename V4<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K1 = p.kc + 1;
  T2* tab = (T2*)smem_raw;                   // [kSkTile][3][K1]
  T4* mus = (T4*)(tab + kSkTile * 3 * K1);   // [kSkTile]
  const int tid = threadIdx.x;
  const int sidx = blockIdx.x * kSkThreads + tid;
  const int chunk = blockIdx.y;
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
    for (int job = tid; job < tn * 3; job += kSkThreads) {
      const int pp = job / 3, ax = job - 3 * pp;
      unsigned sf;
      double xb;
      particle_coord<T>(p.s, t0 + pp, ax, sf, xb);
      fill_table<T>(tab + (pp * 3 + ax) * K1, 1, p.kc, sf, xb, p.two_pi);
    }
    for (int pp = tid; pp < tn; pp += kSkThreads) mus[pp] = ((const T4*)p.s.mu)[t0 + pp];
    __syncthreads();
    if (!has) continue;
    for (int pp = 0; pp < tn; pp++) {
      const T2* tb = tab + pp * 3 * K1;
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
  if (blockIdx.x == 0) {
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

template <typename T>
__global__ void k_sk_reduce(KParams p) {
  using T2 = typename V2<T>::t;
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk < p.nk) {
    double a = 0, b = 0;
    for (int c = 0; c < p.nchunk; c++) {
      const double2 v = p.Spart[(size_t)c * p.nk + kk];
      a += v.x;
      b += v.y;
    }
    p.S[kk] = make_double2(a, b);
    const double e = p.ek[kk];
    T2 o;
    o.x = (T)(e * a);
    o.y = (T)(e * b);
    ((T2*)p.eS)[p.rowpos[kk]] = o;
  }
  if (blockIdx.x == 0 && threadIdx.x < 3) {
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

template <typename T, int NT, bool FULL>
__global__ void __launch_bounds__(NT) k_kscatter(KParams p) {
  using T2 = typename V2<T>::t;
  using T4 = typename V4<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K1 = p.kc + 1;
  T2* tab = (T2*)smem_raw;                 // x phase table [K1][NT]
  T2* es_s = tab + K1 * NT;                // e*S of the chunk [kKChunk]
  KSeg* seg_s = (KSeg*)(es_s + kKChunk);   // segments of the chunk [kKChunk / 4]
  const int tid = threadIdx.x;
  const int k = blockIdx.x * NT + tid;
  const bool active = k < p.n;
  const int kk = active ? k : p.n - 1;
  unsigned sx, sy, sz;
  double xbx, xby, xbz;
  particle_coord<T>(p.s, kk, 0, sx, xbx);
  particle_coord<T>(p.s, kk, 1, sy, xby);
  particle_coord<T>(p.s, kk, 2, sz, xbz);
  fill_table<T>(tab + tid, NT, p.kc, sx, xbx, p.two_pi);
  const T4 mu = ((const T4*)p.s.mu)[kk];
  const T2 E = tab[NT + tid];
  const T2 EY = phase_direct<T>(1, sy, xby, p.two_pi);
  T b[3] = {0, 0, 0}, f[3] = {0, 0, 0}, cb[3] = {0, 0, 0}, cf[3] = {0, 0, 0};
  T bb[3] = {0, 0, 0}, fb[3] = {0, 0, 0};
  int cur_ny = 1 << 30, cur_nz = 1 << 30, anchor = 0, nflush = 0;
  T2 Y = {0, 0}, Z = {0, 0};
  T yzr = 0, yzi = 0;
  for (int c = 0; c < p.nchk; c++) {
    const int2 c0 = p.chunks[c], c1 = p.chunks[c + 1];
    const int nsg = c1.x - c0.x, nkc = c1.y - c0.y;
    __syncthreads();
    for (int i = tid; i < nkc; i += NT) es_s[i] = ((const T2*)p.eS)[c0.y + i];
    for (int i = tid; i < nsg; i += NT) seg_s[i] = p.rseg[c0.x + i];
    __syncthreads();
    int ko = 0;
    for (int s = 0; s < nsg; s++) {
      const KSeg sg = seg_s[s];
      if (sg.nz != cur_nz) {
        Z = phase_direct<T>(sg.nz, sz, xbz, p.two_pi);
        Y = phase_direct<T>(sg.ny, sy, xby, p.two_pi);
        cur_nz = sg.nz;
        cur_ny = anchor = sg.ny;
        cmul<T>(Y.x, Y.y, Z.x, Z.y, yzr, yzi);
      } else if (sg.ny != cur_ny) {
        if (sg.ny - anchor >= 8) {
          Y = phase_direct<T>(sg.ny, sy, xby, p.two_pi);
          anchor = sg.ny;
        } else {
          T nr, ni;
          cmul<T>(Y.x, Y.y, EY.x, EY.y, nr, ni);
          Y.x = nr;
          Y.y = ni;
        }
        cur_ny = sg.ny;
        cmul<T>(Y.x, Y.y, Z.x, Z.y, yzr, yzi);
      }
      const int ax0 = sg.nx0 < 0 ? -sg.nx0 : sg.nx0;
      T2 X = tab[ax0 * NT + tid];
      if (sg.nx0 < 0) X.y = -X.y;
      T pr, pi;
      cmul<T>(X.x, X.y, yzr, yzi, pr, pi);
      T nxf = (T)sg.nx0;
      T w = 0;
      if constexpr (FULL) w = nxf * mu.x + (T)sg.ny * mu.y + (T)sg.nz * mu.z;
      T gx = 0, gs = 0, hx = 0, hs = 0;
      const T2* es_seg = es_s + ko;
#pragma unroll
      for (int q = 0; q < kSegMax; q += 4) {
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
  if (active) {
    T* B = (T*)p.B;
    const int n = p.n;
    const T cfl = (T)p.cflux, cfo = (T)p.cforce;
#pragma unroll
    for (int a = 0; a < 3; a++) B[a * n + k] = -cfl * (b[a] - cb[a]);
    if constexpr (FULL) {
      T* F = (T*)p.F;
#pragma unroll
      for (int a = 0; a < 3; a++) F[a * n + k] = cfo * (f[a] - cf[a]);
    }
  }
}

size_t ksf_smem(int kc, bool fp64) {
  const size_t e = fp64 ? 16 : 8;
  return (size_t)kSkTile * 3 * (kc + 1) * e + (size_t)kSkTile * (fp64 ? 32 : 16);
}

static int scatter_threads(int kc, bool fp64) {
  const size_t e = fp64 ? 16 : 8;
  for (int nt : {128, 64, 32})
    if ((size_t)(kc + 1) * nt * e + (size_t)kKChunk * e + (size_t)kKChunk / 4 * sizeof(KSeg) <= 200 * 1024)
      return nt;
  return 0;
}

size_t kscatter_smem(int kc, bool fp64) {
  const int nt = scatter_threads(kc, fp64);
  const size_t e = fp64 ? 16 : 8;
  return nt ? (size_t)(kc + 1) * nt * e + (size_t)kKChunk * e + (size_t)kKChunk / 4 * sizeof(KSeg) : 0;
}

template <typename T, int NT>
static void scatter_launch(cudaStream_t st, const KParams& p, bool full, size_t smem) {
  dim3 grid((p.n + NT - 1) / NT);
  if (full) {
    cudaFuncSetAttribute(k_kscatter<T, NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_kscatter<T, NT, true><<<grid, NT, smem, st>>>(p);
  } else {
    cudaFuncSetAttribute(k_kscatter<T, NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_kscatter<T, NT, false><<<grid, NT, smem, st>>>(p);
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
  k_sk_reduce<T><<<(p.nk + 255) / 256, 256, 0, st>>>(p);
  if (ev) cudaEventRecordWithFlags(ev[1], st, cudaEventRecordExternal);
  const int nt = scatter_threads(p.kc, fp64);
  const size_t sm2 = kscatter_smem(p.kc, fp64);
  if (nt == 128)
    scatter_launch<T, 128>(st, p, full, sm2);
  else if (nt == 64)
    scatter_launch<T, 64>(st, p, full, sm2);
  else
    scatter_launch<T, 32>(st, p, full, sm2);
  return 3;
}

int launch_kspace(cudaStream_t st, const KParams& p, bool full, bool fp64, cudaEvent_t* ev) {
  return fp64 ? kspace_t<double>(st, p, full, ev) : kspace_t<float>(st, p, full, ev);
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
