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
// Every kernel is a block body with two entry points: one system (parameters
// by value) and packed (a task table over several systems).
//
// Roofline: HBM/L2 bound, ~60 B per particle of algorithmic traffic
// (pos 24 B read, cell id 4+4 B, sorted views 16+16+16 B written, index
// arrays 8 B) plus 8 B per cell.
#include <map>
#include <mutex>

#include "md_common.cuh"
#include "md_kernels.h"

namespace md {

constexpr int kCellThreads = 256;

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
__device__ __forceinline__ void step_begin(StepFlags* f, float half_skin) {
  const int rb = f->force || __uint_as_float(f->maxdisp) > half_skin;
  f->rebuild = rb;
  if (rb) {
    f->force = 0;
    f->maxdisp = 0u;
  }
}

// Cell of each particle (all-pairs grid: identity order, one cell).
__device__ __forceinline__ void cell_assign(const CellParams& p, int bx) {
  if (skip(p.flags)) return;
  const int i = bx * kCellThreads + threadIdx.x, n = p.n;
  if (i >= n) return;
  const int ncx = p.grid.ncx;
  if (ncx == 1) {
    p.s.perm[i] = i;
    p.cellOf[i] = 0;
    return;
  }
  const int cx = cell_coord(wrap_box(p.pos[i], p.invL), ncx);
  const int cy = cell_coord(wrap_box(p.pos[n + i], p.invL), ncx);
  const int cz = cell_coord(wrap_box(p.pos[2 * n + i], p.invL), ncx);
  const int c = (cz * ncx + cy) * ncx + cx;
  p.cellOf[i] = c;
  atomicAdd(&p.count[c], 1);
}

// Exclusive scan of count[0..ncell) -> start[0..ncell]; count is zeroed so it
// can serve as the fill counter of the scatter.  One block of 1024 threads.
__device__ __forceinline__ void cell_scan(const CellParams& p) {
  if (skip(p.flags) || p.grid.ncx == 1) return;
  __shared__ int wsum[32];
  const int ncell = p.grid.ncell;
  int* count = p.count;
  int* start = p.s.cell_start;
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

__device__ __forceinline__ void cell_scatter(const CellParams& p, int bx) {
  if (skip(p.flags) || p.grid.ncx == 1) return;
  const int i = bx * kCellThreads + threadIdx.x;
  if (i >= p.n) return;
  const int c = p.cellOf[i];
  p.tmp[p.s.cell_start[c] + atomicAdd(&p.count[c], 1)] = i;
}

// One warp per cell: rank of each element = number of smaller indices in the
// segment (indices are distinct), so perm is the segment sorted ascending.
// The cell's fill counter is zeroed for the next build.
__device__ __forceinline__ void cell_sort(const CellParams& p, int bx) {
  if (skip(p.flags) || p.grid.ncx == 1) return;
  const int c = (bx * kCellThreads + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= p.grid.ncell) return;
  const int* tmp = p.tmp;
  int* perm = p.s.perm;
  const int s = p.s.cell_start[c], e = p.s.cell_start[c + 1], len = e - s;
  if (lane == 0) p.count[c] = 0;
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

// Sorted views.  Fixed point: x_fix = round(x_box * 2^32) as a wrapping
// 32-bit integer, so x_fix[j] - x_fix[i] (mod 2^32) is the minimum-image
// difference in units of L / 2^32 (about 4e-16 m at L = 1.7 um).  On a
// rebuild the particle positions are recorded as the list's reference.
template <typename T>
__device__ __forceinline__ void sorted_fill(const CellParams& p, int bx) {
  using T4 = typename V4<T>::t;
  const int k = bx * kCellThreads + threadIdx.x, n = p.n;
  if (k >= n) return;
  const SortedView& s = p.s;
  const int i = s.perm[k];
  const bool rb = !p.flags || p.flags->rebuild;
  const double px = p.pos[i], py = p.pos[n + i], pz = p.pos[2 * n + i];
  if (rb) {
    s.rank[i] = k;
    s.cell[k] = p.cellOf[i];
    if (p.xbuild) {
      p.xbuild[i] = px;
      p.xbuild[n + i] = py;
      p.xbuild[2 * n + i] = pz;
    }
  }
  const double x = wrap_box(px, p.invL), y = wrap_box(py, p.invL), z = wrap_box(pz, p.invL);
  const double rm = p.rMag_u[i];
  s.xf[k] = make_float4((float)x, (float)y, (float)z, (float)rm);
  if constexpr (std::is_same<T, float>::value) {
    const double sc = 4294967296.0;
    s.xi[k] = make_int4((int)(unsigned)(long long)llrint(x * sc), (int)(unsigned)(long long)llrint(y * sc),
                        (int)(unsigned)(long long)llrint(z * sc), i);
  } else {
    s.xd[k] = make_double4_32a(x, y, z, rm);
  }
  const double mu = p.magMom_u[i];
  T4 m;
  m.x = (T)(p.mm[i] * mu);
  m.y = (T)(p.mm[n + i] * mu);
  m.z = (T)(p.mm[2 * n + i] * mu);
  m.w = (T)rm;
  ((T4*)s.mu)[k] = m;
}

// ------------------------------------------------------------ one system

__global__ void k_step_begin(StepFlags* f, float half_skin) {
  if (threadIdx.x == 0 && blockIdx.x == 0) step_begin(f, half_skin);
}
__global__ void __launch_bounds__(kCellThreads) k_cell_assign(CellParams p) { cell_assign(p, blockIdx.x); }
__global__ void __launch_bounds__(1024) k_cell_scan(CellParams p) { cell_scan(p); }
__global__ void __launch_bounds__(kCellThreads) k_cell_scatter(CellParams p) { cell_scatter(p, blockIdx.x); }
__global__ void __launch_bounds__(kCellThreads) k_cell_sort(CellParams p) { cell_sort(p, blockIdx.x); }
template <typename T>
__global__ void __launch_bounds__(kCellThreads) k_sorted_fill(CellParams p) {
  sorted_fill<T>(p, blockIdx.x);
}

// ---------------------------------------------------------------- packed

// anyrb: raised when some system of the batch rebuilds its cell and
// neighbour lists this step; the packed list kernels return at once while it
// is clear (most steps), instead of claiming every task to find its system
// skips the work.  The step's last kernel clears it (k_obs_packed).
__global__ void k_step_begin_packed(const CellParams* __restrict__ ps, int R, unsigned* anyrb) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) {
    step_begin(ps[r].flags, ps[r].half_skin);
    if (ps[r].flags->rebuild) atomicOr(anyrb, 1u);
  }
}
// Packed kernels are persistent: their blocks stride over the task table,
// finishing one task before the next (the barrier keeps a task's shared
// memory until every thread of the block is done with it).
__global__ void __launch_bounds__(kCellThreads) k_cell_assign_packed(const CellParams* __restrict__ ps,
                                                                     const Task* __restrict__ tk, int ntask, WorkQ* wq,
                                                                     const unsigned* anyrb) {
  if (!__ldcg(anyrb)) return;  // the whole grid: no system rebuilds this step
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      cell_assign(ps[t.rep], t.blk);
  });
}
__global__ void __launch_bounds__(1024) k_cell_scan_packed(const CellParams* __restrict__ ps) {
  const CellParams p = ps[blockIdx.x];
  cell_scan(p);
}
__global__ void __launch_bounds__(kCellThreads) k_cell_scatter_packed(const CellParams* __restrict__ ps,
                                                                      const Task* __restrict__ tk, int ntask, WorkQ* wq,
    const unsigned* anyrb) {
  if (!__ldcg(anyrb)) return;
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      cell_scatter(ps[t.rep], t.blk);
  });
}
__global__ void __launch_bounds__(kCellThreads) k_cell_sort_packed(const CellParams* __restrict__ ps,
                                                                   const Task* __restrict__ tk, int ntask, WorkQ* wq,
    const unsigned* anyrb) {
  if (!__ldcg(anyrb)) return;
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      cell_sort(ps[t.rep], t.blk);
  });
}
template <typename T>
__global__ void __launch_bounds__(kCellThreads) k_sorted_fill_packed(const CellParams* __restrict__ ps,
                                                                     const Task* __restrict__ tk, int ntask, WorkQ* wq) {
  for_tasks<true>(tk, ntask, wq, [&](const Task& t) {
      sorted_fill<T>(ps[t.rep], t.blk);
  });
}

int persistent_grid(const void* fn, int threads, size_t smem, int ntask) {
  static std::mutex mu;
  static std::map<std::pair<const void*, std::pair<int, size_t>>, int> cache;
  int per = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(fn, std::make_pair(threads, smem));
    auto it = cache.find(key);
    if (it != cache.end()) {
      per = it->second;
    } else {
      int dev = 0, nsm = 0, occ = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 148;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem) != cudaSuccess || occ <= 0) {
        cudaGetLastError();
        occ = 1;
      }
      per = occ * nsm;
      cache[key] = per;
    }
  }
  return std::max(1, std::min(per, ntask));
}

// -------------------------------------------------------- other kernels

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

// md_step_io with host buffers that the device addresses directly
// (page-locked and mapped; on GB300 over NVLink-C2C): the state comes in
// through one kernel that also does k_disp_check's test (xbuild null: no
// list to test against), and goes out through one kernel, instead of three
// copies each way and a separate check.
__global__ void k_state_in(int n, const double* __restrict__ hpos, const double* __restrict__ hmm,
                           const double* __restrict__ hea, double* __restrict__ pos, double* __restrict__ mm,
                           double* __restrict__ ea, const double* __restrict__ xbuild, double L, StepFlags* f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double d2 = 0;
  if (i < n)
    for (int a = 0; a < 3; a++) {
      const size_t q = (size_t)a * n + i;
      const double x = hpos[q];
      pos[q] = x;
      mm[q] = hmm[q];
      ea[q] = hea[q];
      if (xbuild) {
        double d = x - xbuild[q];
        d -= L * round(d / L);
        d2 += d * d;
      }
    }
  if (!xbuild) return;  // uniform over the grid
  float d = (float)(sqrt(d2) / L);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(kFull, d, o));
  if ((threadIdx.x & 31) == 0 && d > 0.f) atomicMax(&f->maxdisp, __float_as_uint(d));
}

__global__ void k_state_out(int n, const double* __restrict__ pos, const double* __restrict__ mm,
                            const double* __restrict__ ea, double* __restrict__ hpos, double* __restrict__ hmm,
                            double* __restrict__ hea) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int a = 0; a < 3; a++) {
    const size_t q = (size_t)a * n + i;
    hpos[q] = pos[q];
    hmm[q] = mm[q];
    hea[q] = ea[q];
  }
}

// ------------------------------------------------------------- launchers

int launch_state_in(cudaStream_t st, int n, const double* hpos, const double* hmm, const double* hea, double* pos,
                    double* mm, double* ea, const double* xbuild, double L, StepFlags* flags) {
  k_state_in<<<(n + 255) / 256, 256, 0, st>>>(n, hpos, hmm, hea, pos, mm, ea, xbuild, L, flags);
  return 1;
}

int launch_state_out(cudaStream_t st, int n, const double* pos, const double* mm, const double* ea, double* hpos,
                     double* hmm, double* hea) {
  k_state_out<<<(n + 255) / 256, 256, 0, st>>>(n, pos, mm, ea, hpos, hmm, hea);
  return 1;
}

int cell_blocks(int n) { return (n + kCellThreads - 1) / kCellThreads; }
int cell_sort_blocks(const CellGrid& g) { return g.ncx == 1 ? 0 : (g.ncell * 32 + kCellThreads - 1) / kCellThreads; }

int launch_disp_check(cudaStream_t st, int n, const double* pos, const double* xbuild, double L, StepFlags* flags) {
  k_disp_check<<<(n + 255) / 256, 256, 0, st>>>(n, pos, xbuild, L, flags);
  return 1;
}

int launch_step_begin(cudaStream_t st, StepFlags* flags, double half_skin) {
  k_step_begin<<<1, 32, 0, st>>>(flags, (float)half_skin);
  return 1;
}

int launch_cells(cudaStream_t st, const CellParams& p, bool fp64) {
  const int nb = cell_blocks(p.n);
  int launches = 1;
  k_cell_assign<<<nb, kCellThreads, 0, st>>>(p);
  if (p.grid.ncx > 1) {
    k_cell_scan<<<1, 1024, 0, st>>>(p);
    k_cell_scatter<<<nb, kCellThreads, 0, st>>>(p);
    k_cell_sort<<<cell_sort_blocks(p.grid), kCellThreads, 0, st>>>(p);
    launches += 3;
  }
  if (fp64)
    k_sorted_fill<double><<<nb, kCellThreads, 0, st>>>(p);
  else
    k_sorted_fill<float><<<nb, kCellThreads, 0, st>>>(p);
  return launches + 1;
}

int launch_step_begin_packed(cudaStream_t st, const CellParams* ps, int R, unsigned* anyrb) {
  k_step_begin_packed<<<(R + 127) / 128, 128, 0, st>>>(ps, R, anyrb);
  return 1;
}

int launch_cells_packed(cudaStream_t st, const CellParams* ps, int R, const Packed& n256, const Packed& sort,
                        const unsigned* anyrb) {
  int l = 0;
  if (n256.n) {
    k_cell_assign_packed<<<persistent_grid((const void*)k_cell_assign_packed, kCellThreads, 0, n256.n), kCellThreads, 0, st>>>(ps, n256.tasks, n256.n, n256.wq, anyrb);
    l++;
  }
  k_cell_scan_packed<<<R, 1024, 0, st>>>(ps);
  l++;
  if (n256.n) {
    k_cell_scatter_packed<<<persistent_grid((const void*)k_cell_scatter_packed, kCellThreads, 0, n256.n), kCellThreads, 0, st>>>(ps, n256.tasks, n256.n, n256.wq, anyrb);
    l++;
  }
  if (sort.n) {
    k_cell_sort_packed<<<persistent_grid((const void*)k_cell_sort_packed, kCellThreads, 0, sort.n), kCellThreads, 0, st>>>(ps, sort.tasks, sort.n, sort.wq, anyrb);
    l++;
  }
  if (n256.n) {
    k_sorted_fill_packed<float><<<persistent_grid((const void*)k_sorted_fill_packed<float>, kCellThreads, 0, n256.n), kCellThreads, 0, st>>>(ps, n256.tasks, n256.n, n256.wq);
    l++;
  }
  return l;
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
