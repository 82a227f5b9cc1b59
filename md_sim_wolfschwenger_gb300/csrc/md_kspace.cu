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
// advanced by one complex multiply per k; each segment starts from per-
// particle tables X(n) = exp(2 pi i n x / L), n = 0..kc, that are evaluated
// directly (every 4th entry and n < 4) or as one product of two direct
// entries.  On the mixed path the table phases are reduced exactly in 32-bit
// fixed point before sincospif.
//
// Structure factor (k_sk): threads = segments, particles staged through
// shared-memory tiles of 32; FP32 sums per tile, compensated (Kahan) FP32
// across tiles, FP64 across particle chunks (k_sk_reduce).
// Scatter (k_kscatter): threads = particles, per-thread tables in shared
// memory; per segment FP32, blocks of 8 segments added with Kahan (mixed).
//
// Roofline: FP32 issue bound.  Algorithmic FLOPs per (k, particle): 14 for
// the structure factor, 12 for the field scatter, 22 for field + force.
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kSkThreads = 256;
constexpr int kSkTile = 32;
constexpr int kSegMax = 16;

// Table of exp(2 pi i n x) for n = 0..kc at out[n * stride].
template <typename T>
__device__ __forceinline__ void fill_table(typename V2<T>::t* out, int stride, int kc, unsigned sfix, double xb,
                                           double two_pi) {
  using T2 = typename V2<T>::t;
  for (int nn = 0; nn <= kc; nn++) {
    T2 v;
    if (nn < 4 || (nn & 3) == 0) {
      if constexpr (std::is_same<T, float>::value) {
        int ph = (int)((unsigned)nn * sfix);  // exact reduction mod 1 box
        float s, c;
        sincospif(2.0f * ((float)ph * 2.3283064365386963e-10f), &s, &c);
        v = make_float2(c, s);
      } else {
        double s, c;
        sincos(two_pi * (double)nn * xb, &s, &c);
        v = make_double2(c, s);
      }
    } else {
      T2 a = out[(nn & ~3) * stride], b = out[(nn & 3) * stride];
      T cr, ci;
      cmul<T>(a.x, a.y, b.x, b.y, cr, ci);
      v.x = cr;
      v.y = ci;
    }
    out[nn * stride] = v;
  }
}

template <typename T>
__device__ __forceinline__ void particle_coord(const SortedView& s, int k, int ax, unsigned& sfix, double& xb) {
  if constexpr (std::is_same<T, float>::value) {
    int4 q = s.xi[k];
    sfix = (unsigned)(ax == 0 ? q.x : (ax == 1 ? q.y : q.z));
    xb = 0.0;
  } else {
    double4_32a q = s.xd[k];
    xb = ax == 0 ? q.x : (ax == 1 ? q.y : q.z);
    sfix = 0;
  }
}

template <typename T>
__global__ void __launch_bounds__(kSkThreads) k_sk(KParams p) {
  using T2 = typename V2<T>::t;
  using T4 = typename V4<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K1 = p.kc + 1;
  T2* tab = (T2*)smem_raw;
  T4* mus = (T4*)(tab + kSkTile * 3 * K1);
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
  T sc[kSegMax], ss[kSegMax], cc[kSegMax], cs[kSegMax];
#pragma unroll
  for (int c = 0; c < kSegMax; c++) sc[c] = ss[c] = cc[c] = cs[c] = 0;

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
    T ac[kSegMax], as[kSegMax];
#pragma unroll
    for (int c = 0; c < kSegMax; c++) ac[c] = as[c] = 0;
    for (int pp = 0; pp < tn; pp++) {
      const T2* tb = tab + pp * 3 * K1;
      T2 X = tb[ax0], Y = tb[K1 + ay], Z = tb[2 * K1 + sg.nz], E = tb[1];
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
          ac[c + u] += w * pr;
          as[c + u] += w * pi;
          const T npr = pr * E.x - pi * E.y;
          pi = pr * E.y + pi * E.x;
          pr = npr;
          w += mu.x;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < kSegMax; c++) {
      if constexpr (std::is_same<T, float>::value) {
        float y = ac[c] - cc[c], t = sc[c] + y;
        cc[c] = (t - sc[c]) - y;
        sc[c] = t;
        y = as[c] - cs[c];
        t = ss[c] + y;
        cs[c] = (t - ss[c]) - y;
        ss[c] = t;
      } else {
        sc[c] += ac[c];
        ss[c] += as[c];
      }
    }
  }
  if (has) {
    const int ko = p.koff[sidx];
    double2* out = p.Spart + (size_t)chunk * p.nk + ko;
#pragma unroll
    for (int c = 0; c < kSegMax; c++)
      if (c < len) out[c] = make_double2((double)sc[c] - (double)cc[c], (double)ss[c] - (double)cs[c]);
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
    ((T2*)p.eS)[kk] = o;
  }
  if (blockIdx.x == 0 && threadIdx.x < 3) {
    double s = 0;
    for (int c = 0; c < p.nchunk; c++) s += p.musum_part[3 * c + threadIdx.x];
    p.musum[threadIdx.x] = s;
  }
}

template <typename T, int NT, bool FULL>
__global__ void __launch_bounds__(NT) k_kscatter(KParams p) {
  using T2 = typename V2<T>::t;
  using T4 = typename V4<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K1 = p.kc + 1;
  T2* tab = (T2*)smem_raw;  // [3 * K1][NT]
  const int tid = threadIdx.x;
  const int k = blockIdx.x * NT + tid;
  const bool active = k < p.n;
  const int kk = active ? k : p.n - 1;
  for (int ax = 0; ax < 3; ax++) {
    unsigned sf;
    double xb;
    particle_coord<T>(p.s, kk, ax, sf, xb);
    fill_table<T>(tab + ax * K1 * NT + tid, NT, p.kc, sf, xb, p.two_pi);
  }
  const T4 mu = ((const T4*)p.s.mu)[kk];
  const T2* eS = (const T2*)p.eS;
  const T2 E = tab[NT + tid];
  T b[3] = {0, 0, 0}, f[3] = {0, 0, 0}, cb[3] = {0, 0, 0}, cf[3] = {0, 0, 0};
  for (int s0 = 0; s0 < p.nseg; s0 += 8) {
    T bb[3] = {0, 0, 0}, fb[3] = {0, 0, 0};
    const int s1 = min(p.nseg, s0 + 8);
    for (int s = s0; s < s1; s++) {
      const KSeg sg = p.seg[s];
      const int ko = p.koff[s];
      const int ax0 = sg.nx0 < 0 ? -sg.nx0 : sg.nx0, ay = sg.ny < 0 ? -sg.ny : sg.ny;
      T2 X = tab[ax0 * NT + tid], Y = tab[(K1 + ay) * NT + tid], Z = tab[(2 * K1 + sg.nz) * NT + tid];
      if (sg.nx0 < 0) X.y = -X.y;
      if (sg.ny < 0) Y.y = -Y.y;
      T yr, yi, pr, pi;
      cmul<T>(Y.x, Y.y, Z.x, Z.y, yr, yi);
      cmul<T>(X.x, X.y, yr, yi, pr, pi);
      T nxf = (T)sg.nx0;
      T w = 0;
      if constexpr (FULL) w = nxf * mu.x + (T)sg.ny * mu.y + (T)sg.nz * mu.z;
      T gx = 0, gs = 0, hx = 0, hs = 0;
#pragma unroll
      for (int c = 0; c < kSegMax; c += 4) {
        if (c >= sg.len) break;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const T2 es = eS[ko + c + u];
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
      bb[0] += gx;
      bb[1] += gs * (T)sg.ny;
      bb[2] += gs * (T)sg.nz;
      if constexpr (FULL) {
        fb[0] += hx;
        fb[1] += hs * (T)sg.ny;
        fb[2] += hs * (T)sg.nz;
      }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if constexpr (std::is_same<T, float>::value) {
        float y = bb[a] - cb[a], t = b[a] + y;
        cb[a] = (t - b[a]) - y;
        b[a] = t;
        if constexpr (FULL) {
          y = fb[a] - cf[a];
          t = f[a] + y;
          cf[a] = (t - f[a]) - y;
          f[a] = t;
        }
      } else {
        b[a] += bb[a];
        if constexpr (FULL) f[a] += fb[a];
      }
    }
  }
  if (active) {
    T* B = (T*)p.B;
    const int n = p.n;
    const T cfl = (T)p.cflux, cfo = (T)p.cforce;
#pragma unroll
    for (int a = 0; a < 3; a++) B[a * n + k] = -cfl * b[a];
    if constexpr (FULL) {
      T* F = (T*)p.F;
#pragma unroll
      for (int a = 0; a < 3; a++) F[a * n + k] = cfo * f[a];
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
    if ((size_t)3 * (kc + 1) * nt * e <= 200 * 1024) return nt;
  return 0;
}

size_t kscatter_smem(int kc, bool fp64) {
  const int nt = scatter_threads(kc, fp64);
  return nt ? (size_t)3 * (kc + 1) * nt * (fp64 ? 16 : 8) : 0;
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
