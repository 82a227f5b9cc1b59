// md_post.cu -- post-processing on the device: the radial distribution
// function of the current frame, as the reference's analysis script computes
// it (mFiles/radial_dist_fun.m:19-66 of MD_Sim_Wolfschwenger): every pair
// i < j at its minimum-image distance (one wrap per axis, as the script),
// distances below contact clamped to 2 r_mag0, pairs closer than the range
// counted in `bins` equal bins, each count scaled by L^3 / (2 pi dr^3 N^2)
// / (k - 1/2)^2.  The script's inner loop stops at particle N - 1, leaving
// out the pairs with the last particle; include_last chooses between that
// and all pairs.
//
// Kernel: all pairs from the FP64 master positions; block (x, y) takes the
// particles i of tile x against the 256 particles j of tile y >= x, staged in
// shared memory; an FP32 pre-test in box units (with a margin) rejects the
// pairs far outside the range, the rest get their FP64 distance; pairs
// inside the range go to a per-block shared-memory histogram (integer
// atomics) added to the global counts at the end (deterministic integer
// sums).  O(N^2 / 2) FP32 pre-tests: a few ms at N = 32768, meant for
// analysis frames.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "md_ctx_internal.h"

namespace md {

constexpr int kRdfThreads = 256;
constexpr int kRdfMaxBins = 8192;

// Block (x, y): particles i of tile x against the particles j of tile y >= x.
__global__ void __launch_bounds__(kRdfThreads) k_rdf(int n, const double* __restrict__ pos, double L, double range2,
                                                     float range2_test, double rcont, double inv_bw, int bins,
                                                     int jmax, unsigned long long* __restrict__ counts) {
  if (blockIdx.y < blockIdx.x) return;
  extern __shared__ unsigned char smem_raw[];
  double* tile = (double*)smem_raw;                          // [3][kRdfThreads]
  float* tilef = (float*)(tile + 3 * kRdfThreads);           // [3][kRdfThreads] box units
  unsigned int* hist = (unsigned int*)(tilef + 3 * kRdfThreads);  // [bins]
  for (int b = threadIdx.x; b < bins; b += blockDim.x) hist[b] = 0;
  const float invL = (float)(1.0 / L);
  const int i = blockIdx.x * kRdfThreads + threadIdx.x;
  const int j0 = blockIdx.y * kRdfThreads, jl = j0 + threadIdx.x;
  if (jl < jmax) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
      tile[a * kRdfThreads + threadIdx.x] = pos[a * n + jl];
      tilef[a * kRdfThreads + threadIdx.x] = (float)pos[a * n + jl] * invL;
    }
  }
  __syncthreads();
  if (i < n) {
    const double xi = pos[i], yi = pos[n + i], zi = pos[2 * n + i];
    const float xf = (float)xi * invL, yf = (float)yi * invL, zf = (float)zi * invL;
    const double half = 0.5 * L;
    const int tn = min(kRdfThreads, jmax - j0);
    for (int t = 0; t < tn; t++) {
      if (j0 + t <= i) continue;
      // FP32 pre-test in box units with a margin, FP64 distance for the rest
      float fx = xf - tilef[t], fy = yf - tilef[kRdfThreads + t], fz = zf - tilef[2 * kRdfThreads + t];
      fx -= rintf(fx);
      fy -= rintf(fy);
      fz -= rintf(fz);
      if (fx * fx + fy * fy + fz * fz > range2_test) continue;
      double dx = xi - tile[t], dy = yi - tile[kRdfThreads + t], dz = zi - tile[2 * kRdfThreads + t];
      dx -= L * (double)(dx > half);
      dx += L * (double)(dx < -half);
      dy -= L * (double)(dy > half);
      dy += L * (double)(dy < -half);
      dz -= L * (double)(dz > half);
      dz += L * (double)(dz < -half);
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= range2) continue;
      double r = sqrt(r2);
      if (r < rcont) r = rcont;
      const int b = (int)floor(r * inv_bw);
      if (b >= 0 && b < bins) atomicAdd(&hist[b], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < bins; b += blockDim.x)
    if (hist[b]) atomicAdd(&counts[b], (unsigned long long)hist[b]);
}

}  // namespace md

extern "C" int md_rdf(md_ctx* c, int64_t bins, double range, double r_mag0, int include_last, double* g,
                      uint64_t* counts_out) {
  int st = check_ready(c, true);
  if (st) return st;
  if (bins < 1 || bins > md::kRdfMaxBins || !(range > 0) || !(r_mag0 > 0) || !g)
    return set_err(c, MD_ERR_INVALID, "md_rdf: bins must be 1..%d, range and r_mag0 positive", md::kRdfMaxBins);
  const int n = (int)c->n;
  if ((n + md::kRdfThreads - 1) / md::kRdfThreads > 65535)
    return set_err(c, MD_ERR_UNSUPPORTED, "md_rdf: at most %d particles", 65535 * md::kRdfThreads);
  const double L = c->L, bw = range / (double)bins;
  unsigned long long* d_counts = nullptr;
  if ((st = dalloc(c, &d_counts, sizeof(unsigned long long) * (size_t)bins))) return st;
  auto done = [&](int s) {
    dfree(c, d_counts);
    return s;
  };
  if (cudaMemsetAsync(d_counts, 0, sizeof(unsigned long long) * (size_t)bins, c->stream) != cudaSuccess)
    return done(set_err(c, MD_ERR_CUDA, "md_rdf: memset failed"));
  const size_t smem = (sizeof(double) + sizeof(float)) * 3 * md::kRdfThreads + sizeof(unsigned int) * (size_t)bins;
  cudaFuncSetAttribute(md::k_rdf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int jmax = include_last ? n : n - 1;
  const int nt = (n + md::kRdfThreads - 1) / md::kRdfThreads;
  const double rb = range / L * (1.0 + 1e-4) + 1e-6;  // box units, with a margin for the FP32 pre-test
  md::k_rdf<<<dim3(nt, nt), md::kRdfThreads, smem, c->stream>>>(n, c->pos, L, range * range, (float)(rb * rb),
                                                               2.0 * r_mag0, 1.0 / bw, (int)bins, jmax, d_counts);
  std::vector<unsigned long long> h((size_t)bins);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(h.data(), d_counts, sizeof(unsigned long long) * (size_t)bins, cudaMemcpyDeviceToHost,
                      c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return done(set_err(c, MD_ERR_CUDA, "md_rdf: kernel or copy failed"));
  // normalisation of the script: L^3 / (2 pi dr^3 N^2) / (k - 1/2)^2
  const double norm = L * L * L / (2.0 * c->cfg.my_pi * bw * bw * bw * (double)n * (double)n);
  for (int64_t k = 0; k < bins; k++) {
    const double kk = (double)k + 0.5;
    g[k] = (double)h[(size_t)k] * norm / (kk * kk);
    if (counts_out) counts_out[k] = h[(size_t)k];
  }
  return done(MD_OK);
}
