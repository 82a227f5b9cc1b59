// md_place.cu -- initial placement on the GPU: random sequential addition
// (InitCoordsFromSketch, src/simulation.cpp:241-264) with a counter-based
// stream per particle, so that a parallel placement gives exactly the result
// of the sequential rule:
//
//   in placement order (the reference's index order, or largest first), each
//   particle takes the first attempt t = 0, 1, ... whose position overlaps no
//   particle placed before it (distance below the sum of the hydrodynamic
//   radii, plain distance inside the box as in the reference); attempt t of
//   particle i is drawn from Philox4x32-10 with counters {i, t} (the
//   reference draws every attempt from one sequential generator instead).
//
// One block works through the particles in batches of kRsaBatch: each thread
// skips its particle's attempts that overlap the earlier batches (a cell grid,
// cells no smaller than the largest contact distance, so a candidate meets
// only the 27 cells around it; each cell keeps up to kRsaSlots particle
// indices side by side, so a check issues its loads independently instead of
// walking a list); then one warp takes the batch
// in order and checks each candidate against the batch's particles accepted
// before it, drawing further attempts (checked against both) where one
// overlaps; then the batch enters the grid.  An attempt skipped in the first
// phase overlaps an earlier particle, so the sequential rule rejects it too.
// Distances are rounded operation by operation (no contraction), as in the
// restatement the tests compare with bit for bit.  GB300's FP64 rate is a
// small fraction of FP32, so each test first compares FP32 copies of the
// positions against the contact distance widened and narrowed by a bound on
// their rounding (4e-7 L, about twice the worst case of 2.1e-7 L: each
// coordinate within L/2 rounded to 24 bits, the difference rounded, three
// components), the squared thresholds loosened by a further 1e-4; only a pair
// inside that band takes the FP64 test, so every decision is the FP64 one.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "../../include/md_gb300.h"
#include "md_common.cuh"
#include "md_err.h"

namespace md {
namespace {

constexpr int kRsaBatch = 1024;  // particles per batch = threads of the block
constexpr int kRsaSlots = 64;   // particles a cell holds (a cell takes ~N / nc^3 on average)

struct RsaParams {
  int n;
  double L;
  uint64_t seed;
  long long max_tries;  // attempts of one particle
  unsigned long long budget;  // attempts of all particles (bounds the kernel's time)
  const double* rH;
  const int* order;  // placement order (null: index order)
  double* pos;       // [3][n], box centred at 0
  float4* pf;        // [n] FP32 copies (x, y, z, r) of the placed particles
  float ed;          // rounding bound of an FP32 distance (4e-7 L)
  int* cnt;          // [nc^3] particles in each cell
  int* slot;         // [nc^3][kRsaSlots] their indices
  int nc;
  double inv_cs, half;
  int* err;  // 1: a particle found no place within max_tries, or the budget ran out;
             // 2: a cell overflowed its slots
};

// Attempt t of particle i: three uniforms of 53 bits, coordinates
// (2u - 1)(L/2 - r_i).
__device__ __forceinline__ void rsa_cand(uint64_t seed, int i, long long t, double ext, double x[3]) {
  const uint32_t tl = (uint32_t)t, th = (uint32_t)((unsigned long long)t >> 32);
  const uint4 a = philox4x32_10(make_uint4((uint32_t)i, tl, th, 0xA5A5A5A5u), (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint4 b = philox4x32_10(make_uint4((uint32_t)i, tl, th, 0x5A5A5A5Au), (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t w[6] = {a.x, a.y, a.z, a.w, b.x, b.y};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const unsigned long long m = ((unsigned long long)w[2 * c] << 21) ^ (unsigned long long)(w[2 * c + 1] >> 11);
    const double u = (double)m * 1.1102230246251565e-16;  // 2^-53
    x[c] = __dmul_rn(__dsub_rn(__dmul_rn(2.0, u), 1.0), ext);
  }
}

// |x_j - x| < s, rounded as ((dx dx + dy dy) + dz dz) < s s
__device__ __forceinline__ bool rsa_overlap(double xj, double yj, double zj, const double x[3], double s) {
  const double dx = __dsub_rn(xj, x[0]), dy = __dsub_rn(yj, x[1]), dz = __dsub_rn(zj, x[2]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return r2 < __dmul_rn(s, s);
}

// Overlap through the FP32 filter: decided in FP32 outside the band
// (s -+ ed)^2 around the contact distance, by the FP64 test (xj, yj, zj from
// `exact`) inside it.
template <typename Exact>
__device__ __forceinline__ bool rsa_hit(const float4& jf, const float4& xf, float ed, Exact&& exact) {
  const float dx = jf.x - xf.x, dy = jf.y - xf.y, dz = jf.z - xf.z;
  const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  const float sf = jf.w + xf.w;
  const float sl = fmaxf(sf - ed, 0.f), lo = sl * sl, hi = (sf + ed) * (sf + ed);
  if (r2 < lo * 0.9999f) return true;
  if (r2 > hi * 1.0001f) return false;
  return exact();
}

__device__ __forceinline__ int rsa_cell(const RsaParams& p, double x) {
  const int k = (int)floor((x + p.half) * p.inv_cs);
  return min(p.nc - 1, max(0, k));
}

// Does the candidate overlap a particle in the grid (the earlier batches)?
__device__ __forceinline__ bool rsa_grid_overlap(const RsaParams& p, const double x[3], double ri) {
  const int cx = rsa_cell(p, x[0]), cy = rsa_cell(p, x[1]), cz = rsa_cell(p, x[2]), nc = p.nc, n = p.n;
  const float4 xf = make_float4((float)x[0], (float)x[1], (float)x[2], (float)ri);
  for (int dz = -1; dz <= 1; dz++) {
    const int uz = cz + dz;
    if (uz < 0 || uz >= nc) continue;
    for (int dy = -1; dy <= 1; dy++) {
      const int uy = cy + dy;
      if (uy < 0 || uy >= nc) continue;
      for (int dx = -1; dx <= 1; dx++) {
        const int ux = cx + dx;
        if (ux < 0 || ux >= nc) continue;
        const int c = (uz * nc + uy) * nc + ux;
        const int k = min(p.cnt[c], kRsaSlots);
        const int* sl = p.slot + (size_t)c * kRsaSlots;
        for (int q = 0; q < k; q++) {
          const int j = sl[q];
          if (rsa_hit(p.pf[j], xf, p.ed, [&] {
                return rsa_overlap(p.pos[j], p.pos[n + j], p.pos[2 * n + j], x, __dadd_rn(ri, p.rH[j]));
              }))
            return true;
        }
      }
    }
  }
  return false;
}

// First attempt from t0 on that is clear of the grid; max_tries if none.
__device__ __forceinline__ long long rsa_clear(const RsaParams& p, int i, long long t0, double ri, double x[3]) {
  const double ext = __dsub_rn(0.5 * p.L, ri);
  long long t = t0;
  for (; t < p.max_tries; t++) {
    rsa_cand(p.seed, i, t, ext, x);
    if (!rsa_grid_overlap(p, x, ri)) break;
  }
  return t;
}

// Shared memory of the block: the batch's candidates (FP64 and FP32 copies),
// their particles and attempts, the candidates redrawn in phase 2 and the
// flags of phase 1b.
struct RsaBatchMem {
  double x[kRsaBatch], y[kRsaBatch], z[kRsaBatch], r[kRsaBatch];
  float4 f[kRsaBatch];
  int i[kRsaBatch], t[kRsaBatch], redrawn[kRsaBatch];
  unsigned char flag[kRsaBatch];
};

// Surely apart in FP32 (outside the band of rsa_hit): no exact test needed.
__device__ __forceinline__ bool rsa_apart(const float4& jf, const float4& xf, float ed) {
  const float dx = jf.x - xf.x, dy = jf.y - xf.y, dz = jf.z - xf.z;
  const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  const float sf = jf.w + xf.w;
  return r2 > (sf + ed) * (sf + ed) * 1.0001f;
}

__global__ void __launch_bounds__(kRsaBatch) k_rsa(RsaParams p) {
  extern __shared__ __align__(16) unsigned char rsa_smem[];
  RsaBatchMem& B = *reinterpret_cast<RsaBatchMem*>(rsa_smem);
  __shared__ volatile int s_err;
  __shared__ unsigned long long s_tries;
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0) {
    s_err = 0;
    s_tries = 0;
  }
  __syncthreads();
  for (int b0 = 0; b0 < p.n; b0 += kRsaBatch) {
    const int m = min(kRsaBatch, p.n - b0);
    // 1. each particle's first attempt clear of the earlier batches
    if (tid < m) {
      const int i = p.order ? p.order[b0 + tid] : b0 + tid;
      const double ri = p.rH[i];
      double x[3];
      const long long t = rsa_clear(p, i, 0, ri, x);
      if (t >= p.max_tries) s_err = 1;
      atomicAdd(&s_tries, (unsigned long long)(t + 1));
      B.x[tid] = x[0];
      B.y[tid] = x[1];
      B.z[tid] = x[2];
      B.r[tid] = ri;
      B.f[tid] = make_float4((float)x[0], (float)x[1], (float)x[2], (float)ri);
      B.i[tid] = i;
      B.t[tid] = (int)t;
    }
    __syncthreads();
    if (s_err) break;
    // 1b. flag the candidates that may overlap an earlier candidate of the
    // batch (FP32, conservative: inside the rounding band counts as a flag)
    for (int q = tid; q < m; q += blockDim.x) {
      const float4 xf = B.f[q];
      unsigned char fl = 0;
      for (int j = 0; j < q; j++)
        if (!rsa_apart(B.f[j], xf, p.ed)) {
          fl = 1;
          break;
        }
      B.flag[q] = fl;
    }
    __syncthreads();
    // 2. in order: an unflagged candidate is clear of the batch as long as no
    // earlier one was redrawn; otherwise it meets the redrawn ones, and a
    // flagged or redrawn one meets every earlier batch-mate exactly
    if (tid < 32) {
      int nre = 0;
      for (int q = 0; q < m && !s_err; q++) {
        bool full = B.flag[q] != 0, again = false;
        if (!full && nre == 0) continue;
        for (;;) {
          const double x[3] = {B.x[q], B.y[q], B.z[q]};
          const double ri = B.r[q];
          const float4 xf = B.f[q];
          bool hit = false;
          if (full) {
            for (int j = lane; j < q && !hit; j += 32)
              hit = rsa_hit(B.f[j], xf, p.ed, [&] { return rsa_overlap(B.x[j], B.y[j], B.z[j], x, __dadd_rn(ri, B.r[j])); });
          } else {
            for (int k = lane; k < nre && !hit; k += 32) {
              const int j = B.redrawn[k];
              hit = rsa_hit(B.f[j], xf, p.ed, [&] { return rsa_overlap(B.x[j], B.y[j], B.z[j], x, __dadd_rn(ri, B.r[j])); });
            }
          }
          if (!__any_sync(kFull, hit)) break;
          if (lane == 0) {  // the next attempt clear of the grid; the loop checks the batch again
            double y[3];
            const long long t = rsa_clear(p, B.i[q], (long long)B.t[q] + 1, ri, y);
            s_tries += (unsigned long long)(t - B.t[q]);
            if (t >= p.max_tries || s_tries > p.budget) s_err = 1;
            B.x[q] = y[0];
            B.y[q] = y[1];
            B.z[q] = y[2];
            B.f[q] = make_float4((float)y[0], (float)y[1], (float)y[2], (float)ri);
            B.t[q] = (int)t;
            if (!again) B.redrawn[nre] = q;
          }
          if (!again) nre++;
          again = full = true;  // the new candidate meets every earlier batch-mate
          __syncwarp();
          if (s_err) break;
        }
      }
    }
    __syncthreads();
    if (tid == 0 && s_tries > p.budget) s_err = 1;
    __syncthreads();
    if (s_err) break;
    // 3. the batch enters the grid (the order within a cell does not matter)
    if (tid < m) {
      const int i = B.i[tid], n = p.n;
      const double x[3] = {B.x[tid], B.y[tid], B.z[tid]};
      p.pos[i] = x[0];
      p.pos[n + i] = x[1];
      p.pos[2 * n + i] = x[2];
      p.pf[i] = B.f[tid];
      const int c = (rsa_cell(p, x[2]) * p.nc + rsa_cell(p, x[1])) * p.nc + rsa_cell(p, x[0]);
      const int k = atomicAdd(&p.cnt[c], 1);
      if (k < kRsaSlots)
        p.slot[(size_t)c * kRsaSlots + k] = i;
      else
        s_err = 2;
    }
    __syncthreads();
  }
  if (tid == 0 && s_err) *p.err = s_err;
}

}  // namespace
}  // namespace md

extern "C" int md_place_rsa(int64_t n, double lBox, const double* rHydr, uint64_t seed, int largest_first,
                            double* pos) {
  using namespace md;
  if (!rHydr || !pos || n < 1 || n >= (int64_t)1 << 31 || !(lBox > 0))
    return set_err(nullptr, MD_ERR_INVALID, "md_place_rsa: bad arguments");
  double rmax = 0;
  for (int64_t i = 0; i < n; i++) {
    if (!(rHydr[i] > 0) || !(2.0 * rHydr[i] < lBox))
      return set_err(nullptr, MD_ERR_INVALID, "md_place_rsa: radius %lld not in (0, L/2)", (long long)i);
    rmax = std::max(rmax, rHydr[i]);
  }
  std::vector<int> order;
  if (largest_first) {
    order.resize((size_t)n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rHydr[a] > rHydr[b]; });
  }
  // cells no smaller than the largest contact distance; at most ~2N of them
  int nc = (int)std::floor(lBox / (2.0 * rmax));
  nc = std::max(1, std::min(nc, std::min(1024, (int)std::cbrt(2.0 * (double)n) + 1)));
  const size_t ncell = (size_t)nc * nc * nc, N = (size_t)n;
  RsaParams p{};
  p.n = (int)n;
  p.L = lBox;
  p.seed = seed;
  p.max_tries = 100000;  // attempts of one particle fit the batch's int
  p.budget = 100ull * (unsigned long long)n + 1000000ull;
  p.nc = nc;
  p.inv_cs = (double)nc / lBox;
  p.half = 0.5 * lBox;
  double *d_rH = nullptr, *d_pos = nullptr;
  float4* d_pf = nullptr;
  int *d_order = nullptr, *d_cnt = nullptr, *d_slot = nullptr, *d_err = nullptr;
  auto cleanup = [&] {
    for (void* q : {(void*)d_rH, (void*)d_pos, (void*)d_pf, (void*)d_order, (void*)d_cnt, (void*)d_slot, (void*)d_err})
      if (q) cudaFree(q);
  };
  cudaError_t e = cudaMalloc(&d_rH, 8 * N);
  if (e == cudaSuccess) e = cudaMalloc(&d_pos, 24 * N);
  if (e == cudaSuccess) e = cudaMalloc(&d_pf, 16 * N);
  if (e == cudaSuccess && largest_first) e = cudaMalloc(&d_order, 4 * N);
  if (e == cudaSuccess) e = cudaMalloc(&d_cnt, 4 * ncell);
  if (e == cudaSuccess) e = cudaMalloc(&d_slot, 4 * ncell * kRsaSlots);
  if (e == cudaSuccess) e = cudaMalloc(&d_err, 4);
  if (e != cudaSuccess) {
    cleanup();
    return set_err(nullptr, MD_ERR_NOMEM, "md_place_rsa: %s", cudaGetErrorString(e));
  }
  e = cudaMemcpy(d_rH, rHydr, 8 * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && largest_first) e = cudaMemcpy(d_order, order.data(), 4 * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d_cnt, 0, 4 * ncell);
  if (e == cudaSuccess) e = cudaMemset(d_err, 0, 4);
  p.rH = d_rH;
  p.order = d_order;
  p.pos = d_pos;
  p.pf = d_pf;
  p.ed = (float)(4e-7 * lBox);
  p.cnt = d_cnt;
  p.slot = d_slot;
  p.err = d_err;
  int herr = 0;
  if (e == cudaSuccess) {
    const int smem = (int)sizeof(RsaBatchMem);
    e = cudaFuncSetAttribute(k_rsa, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) k_rsa<<<1, kRsaBatch, smem>>>(p);
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && !herr) e = cudaMemcpy(pos, d_pos, 24 * N, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "md_place_rsa: %s", cudaGetErrorString(e));
  if (herr == 2)
    return set_err(nullptr, MD_ERR_UNSUPPORTED, "md_place_rsa: more than %d particles in one grid cell", kRsaSlots);
  if (herr) return set_err(nullptr, MD_ERR_INVALID, "md_place_rsa: no place found (volume fraction too high)");
  return MD_OK;
}
