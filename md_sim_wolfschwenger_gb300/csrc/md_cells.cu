// md_cells.cu -- kernel (a): cell list as a counting sort of particle
// indices into cells, plus the sorted particle views used by the Ewald
// kernels.  Replaces the all-pairs enumeration of CompInteractVecs
// (src/interaction.cpp:88-137) as the neighbour search; the pair geometry
// itself (minimum image, cutoff, overlap clamp) is evaluated in md_real.cu.
//
// Determinism: counts are order-independent; the atomic scatter puts each
// cell's particles in arbitrary order, then one warp per cell sorts its
// segment by particle index.  The result equals a stable host counting sort
// (cells ascending, indices ascending inside a cell), bit for bit.
//
// The cell order is rebuilt together with the neighbour list (when some
// particle has moved more than half the list's skin); in between, the sorted
// views are refreshed every step from the particle-order state through the
// unchanged permutation.
//
// Roofline: HBM/L2 bound, ~60 B per particle of algorithmic traffic
// (pos 24 B read, cell id 4+4 B, sorted views 16+16+16 B written, index
// arrays 8 B) plus 8 B per cell.
#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

__device__ __forceinline__ int cell_coord(double xb, int ncx) {
  int c = (int)((xb + 0.5) * (double)ncx);
  return c < 0 ? 0 : (c >= ncx ? ncx - 1 : c);
}

// Box coordinate wrapped to [-0.5, 0.5).
__device__ __forceinline__ double wrap_box(double x, double invL) {
  double xb = x * invL;
  return xb - floor(xb + 0.5);
}

__device__ __forceinline__ bool skip(const StepFlags* f) { return f && !f->rebuild; }

// Start of a step: rebuild the cell order and the neighbour list if the host
// asked for it or some particle moved more than half the skin since the last
// build (box units).
__global__ void k_step_begin(StepFlags* f, float half_skin) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int rb = f->force || __uint_as_float(f->maxdisp) > half_skin;
  f->rebuild = rb;
  if (rb) {
    f->force = 0;
    f->maxdisp = 0u;
  }
}

__global__ void k_cell_assign(int n, const double* __restrict__ pos, double invL, int ncx, int* __restrict__ cellOf,
                              int* __restrict__ count, const StepFlags* flags) {
  if (skip(flags)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int cx = cell_coord(wrap_box(pos[i], invL), ncx);
  int cy = cell_coord(wrap_box(pos[n + i], invL), ncx);
  int cz = cell_coord(wrap_box(pos[2 * n + i], invL), ncx);
  int c = (cz * ncx + cy) * ncx + cx;
  cellOf[i] = c;
  if (count) atomicAdd(&count[c], 1);
}

// Exclusive scan of count[0..ncell) -> start[0..ncell]; count is zeroed so it
// can serve as the fill counter of the scatter.  One block of 1024 threads.
__global__ void __launch_bounds__(1024) k_cell_scan(int ncell, int* __restrict__ count, int* __restrict__ start,
                                                    const StepFlags* flags) {
  if (skip(flags)) return;
  __shared__ int wsum[32];
  const int t = threadIdx.x, nt = blockDim.x;
  const int per = (ncell + nt - 1) / nt;
  const int b = t * per, e = min(ncell, b + per);
  int local = 0;
  for (int c = b; c < e; c++) local += count[c];
  int lane = t & 31, w = t >> 5;
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    int v = lane < (nt >> 5) ? wsum[lane] : 0;
    int inc2 = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(kFull, inc2, o);
      if (lane >= o) inc2 += u;
    }
    wsum[lane] = inc2 - v;
  }
  __syncthreads();
  int run = wsum[w] + incl - local;
  for (int c = b; c < e; c++) {
    int v = count[c];
    start[c] = run;
    run += v;
    count[c] = 0;
  }
  if (t == nt - 1) start[ncell] = run;
}

__global__ void k_cell_scatter(int n, const int* __restrict__ cellOf, const int* __restrict__ start,
                               int* __restrict__ fill, int* __restrict__ tmp, const StepFlags* flags) {
  if (skip(flags)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cellOf[i];
  tmp[start[c] + atomicAdd(&fill[c], 1)] = i;
}

// One warp per cell: rank of each element = number of smaller indices in the
// segment (indices are distinct), so perm is the segment sorted ascending.
__global__ void k_cell_sort(int ncell, const int* __restrict__ start, const int* __restrict__ tmp,
                            int* __restrict__ perm, const StepFlags* flags) {
  if (skip(flags)) return;
  int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (c >= ncell) return;
  int s = start[c], e = start[c + 1], len = e - s;
  if (len <= 32) {
    int v = lane < len ? tmp[s + lane] : 0x7fffffff;
    int r = 0;
    for (int l = 0; l < len; l++) r += __shfl_sync(kFull, v, l) < v;
    if (lane < len) perm[s + r] = v;
    return;
  }
  for (int a = lane; a < len; a += 32) {
    int v = tmp[s + a], r = 0;
    for (int b = 0; b < len; b++) r += tmp[s + b] < v;
    perm[s + r] = v;
  }
}

__global__ void k_identity(int n, int* __restrict__ perm, const StepFlags* flags) {
  if (skip(flags)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[i] = i;
}

// Sorted views.  Fixed point: x_fix = round(x_box * 2^32) as a wrapping
// 32-bit integer, so x_fix[j] - x_fix[i] (mod 2^32) is the minimum-image
// difference in units of L / 2^32 (about 4e-16 m at L = 1.7 um).  On a
// rebuild the particle positions are recorded as the list's reference.
template <typename T>
__global__ void k_sorted_fill(int n, double invL, const double* __restrict__ pos, const double* __restrict__ mm,
                              const double* __restrict__ magMom_u, const double* __restrict__ rMag_u,
                              const int* __restrict__ cellOf, SortedView s, double* __restrict__ xbuild,
                              const StepFlags* flags) {
  using T4 = typename V4<T>::t;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int i = s.perm[k];
  const bool rb = !flags || flags->rebuild;
  const double px = pos[i], py = pos[n + i], pz = pos[2 * n + i];
  if (rb) {
    s.rank[i] = k;
    s.cell[k] = cellOf[i];
    if (xbuild) {
      xbuild[i] = px;
      xbuild[n + i] = py;
      xbuild[2 * n + i] = pz;
    }
  }
  double x = wrap_box(px, invL), y = wrap_box(py, invL), z = wrap_box(pz, invL);
  double rm = rMag_u[i];
  s.xf[k] = make_float4((float)x, (float)y, (float)z, (float)rm);
  if constexpr (std::is_same<T, float>::value) {
    const double sc = 4294967296.0;
    s.xi[k] = make_int4((int)(unsigned)(long long)llrint(x * sc), (int)(unsigned)(long long)llrint(y * sc),
                        (int)(unsigned)(long long)llrint(z * sc), i);
  } else {
    s.xd[k] = make_double4_32a(x, y, z, rm);
  }
  double mu = magMom_u[i];
  T4 m;
  m.x = (T)(mm[i] * mu);
  m.y = (T)(mm[n + i] * mu);
  m.z = (T)(mm[2 * n + i] * mu);
  m.w = (T)rm;
  ((T4*)s.mu)[k] = m;
}

// Moments for an explicit set of directions (CompDemagField input).
template <typename T>
__global__ void k_set_mu(int n, const double* __restrict__ mm, const double* __restrict__ magMom_u,
                         const double* __restrict__ rMag_u, SortedView s) {
  using T4 = typename V4<T>::t;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double mu = magMom_u[i];
  T4 m;
  m.x = (T)(mm[i] * mu);
  m.y = (T)(mm[n + i] * mu);
  m.z = (T)(mm[2 * n + i] * mu);
  m.w = (T)rMag_u[i];
  ((T4*)s.mu)[s.rank[i]] = m;
}

// After the caller replaced the positions: raise maxdisp by how far each
// particle now is from its position at the last build (box units), so the
// next step rebuilds only if the new state needs it.
__global__ void k_disp_check(int n, const double* __restrict__ pos, const double* __restrict__ xbuild, double L,
                             StepFlags* f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double d2 = 0;
  if (i < n)
    for (int a = 0; a < 3; a++) {
      double d = pos[a * n + i] - xbuild[a * n + i];
      d -= L * round(d / L);
      d2 += d * d;
    }
  float d = (float)(sqrt(d2) / L);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(kFull, d, o));
  if ((threadIdx.x & 31) == 0 && d > 0.f) atomicMax(&f->maxdisp, __float_as_uint(d));
}

int launch_disp_check(cudaStream_t st, int n, const double* pos, const double* xbuild, double L, StepFlags* flags) {
  k_disp_check<<<(n + 255) / 256, 256, 0, st>>>(n, pos, xbuild, L, flags);
  return 1;
}

int launch_step_begin(cudaStream_t st, StepFlags* flags, double half_skin) {
  k_step_begin<<<1, 32, 0, st>>>(flags, (float)half_skin);
  return 1;
}

int launch_cells(cudaStream_t st, int n, const double* pos, const double* mm, const double* magMom_u,
                 const double* rMag_u, double L, const CellGrid& g, int* cellOf, int* count, int* tmp,
                 const SortedView& s, bool fp64, double* xbuild, const StepFlags* flags) {
  const int tb = 256, nb = (n + tb - 1) / tb;
  int launches = 0;
  double invL = 1.0 / L;
  if (g.ncx == 1) {
    // all-pairs: one cell holding every particle in index order
    k_identity<<<nb, tb, 0, st>>>(n, s.perm, flags);
    k_cell_assign<<<nb, tb, 0, st>>>(n, pos, invL, 1, cellOf, nullptr, flags);
    launches += 2;
  } else {
    cudaMemsetAsync(count, 0, sizeof(int) * g.ncell, st);
    k_cell_assign<<<nb, tb, 0, st>>>(n, pos, invL, g.ncx, cellOf, count, flags);
    k_cell_scan<<<1, 1024, 0, st>>>(g.ncell, count, s.cell_start, flags);
    k_cell_scatter<<<nb, tb, 0, st>>>(n, cellOf, s.cell_start, count, tmp, flags);
    k_cell_sort<<<(g.ncell * 32 + 255) / 256, 256, 0, st>>>(g.ncell, s.cell_start, tmp, s.perm, flags);
    launches += 4;
  }
  if (fp64)
    k_sorted_fill<double><<<nb, tb, 0, st>>>(n, invL, pos, mm, magMom_u, rMag_u, cellOf, s, xbuild, flags);
  else
    k_sorted_fill<float><<<nb, tb, 0, st>>>(n, invL, pos, mm, magMom_u, rMag_u, cellOf, s, xbuild, flags);
  return launches + 1;
}

int launch_set_mu(cudaStream_t st, int n, const double* mm, const double* magMom_u, const double* rMag_u,
                  const SortedView& s, bool fp64) {
  const int tb = 256, nb = (n + tb - 1) / tb;
  if (fp64)
    k_set_mu<double><<<nb, tb, 0, st>>>(n, mm, magMom_u, rMag_u, s);
  else
    k_set_mu<float><<<nb, tb, 0, st>>>(n, mm, magMom_u, rMag_u, s);
  return 1;
}

}  // namespace md
