// md_noalloc.cu -- the Ewald structure factor without any device allocation.
//
// Some callers cannot call cudaMalloc: a host program whose framework owns
// all device memory through its own pool, a real-time loop that must not
// allocate after start-up, or a process running under a fixed device-memory
// budget.  For them this file computes the reciprocal-space structure factor
// S(n) = sum_j (n . mu_j) exp(2 pi i n . r_j / L) -- the quantity that
// CompDipInteractEwaldF / CompDipFieldEwaldF accumulate -- with caller-owned
// inputs and outputs and a fixed scratch area that lives in a file-scope
// __device__ array of this library (md_noalloc_scratch_bytes(): 2,430,592
// bytes for kc <= 16).  Every GPU that loads the library holds that array
// until the process exits.
//
// The array's name is a host-side stand-in in host code, not a device
// address.  Its device address is obtained once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on
// that device; make that first call before any stream capture.  Every call
// shares the one array, which keeps the contents of the last call, so calls
// whose work overlaps on the GPU (different streams, different host threads)
// race on it; serialise them.  The looked-up address is kept for the life
// of the process: after a cudaDeviceReset of that device the library's
// module (and the array) may be loaded elsewhere, so do not call this entry
// point on a device that was reset.
//
// A launch error is checked on each launch's own return code
// (cudaLaunchKernel), so an error left pending by the caller's earlier work
// is neither consumed nor reported here.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/md_gb300.h"
#include "md_common.cuh"

namespace {

// Number of k vectors of the reference's loops (interaction.cpp:438-450):
// nz = 0..kc, ny, nx = -kc..kc, 0 < |n|^2 <= kc^2.
constexpr int count_k(int kc) {
  int c = 0;
  for (int nz = 0; nz <= kc; nz++)
    for (int ny = -kc; ny <= kc; ny++)
      for (int nx = -kc; nx <= kc; nx++) {
        const int l = nx * nx + ny * ny + nz * nz;
        if (l > 0 && l <= kc * kc) c++;
      }
  return c;
}

constexpr int kMaxKc = MD_NOALLOC_MAX_KC;
constexpr int kChunks = 16;  // particle chunks; FP64 partial sums per chunk
constexpr int kMaxNk = count_k(kMaxKc);

struct Scratch {
  int4 klist[kMaxNk];                 // (nx, ny, nz, 0) in the reference's loop order
  double2 part[kChunks * kMaxNk];     // per-chunk partial sums (Sc, Ss)
};

static __device__ __align__(256) Scratch g_noalloc_scratch;

std::mutex g_mu;
Scratch* g_addr[64] = {};

// One thread writes the k list in loop order.
__global__ void k_noalloc_klist(Scratch* s, int kc) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int c = 0;
  for (int nz = 0; nz <= kc; nz++)
    for (int ny = -kc; ny <= kc; ny++)
      for (int nx = -kc; nx <= kc; nx++) {
        const int l = nx * nx + ny * ny + nz * nz;
        if (l > 0 && l <= kc * kc) s->klist[c++] = make_int4(nx, ny, nz, 0);
      }
}

// Partial sums over one particle chunk for each k (FP64, direct sincos of the
// full phase with the configuration's pi, as EvalSinCos's tables represent).
// Indices are 64-bit: 2 n + j exceeds INT_MAX for n above ~7e8.
__global__ void k_noalloc_partial(Scratch* s, const double* __restrict__ pos, const double* __restrict__ mom,
                                  long long n, int nk, double two_pi_over_L) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (k >= nk) return;
  const long long per = (n + kChunks - 1) / kChunks;
  const long long j0 = c * per, j1 = min(n, j0 + per);
  const int4 q = s->klist[k];
  const double nx = q.x, ny = q.y, nz = q.z;
  double sc = 0, ss = 0;
  for (long long j = j0; j < j1; j++) {
    const double ph = two_pi_over_L * (nx * pos[j] + ny * pos[n + j] + nz * pos[2 * n + j]);
    double sn, cs;
    sincos(ph, &sn, &cs);
    const double w = nx * mom[j] + ny * mom[n + j] + nz * mom[2 * n + j];
    sc += w * cs;
    ss += w * sn;
  }
  s->part[c * kMaxNk + k] = make_double2(sc, ss);  // written for every (c, k), also empty chunks
}

__global__ void k_noalloc_reduce(const Scratch* s, int nk, double* __restrict__ out5) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  double a = 0, b = 0;
  for (int c = 0; c < kChunks; c++) {
    const double2 v = s->part[c * kMaxNk + k];
    a += v.x;
    b += v.y;
  }
  const int4 q = s->klist[k];
  double* o = out5 + 5 * (size_t)k;
  o[0] = q.x;
  o[1] = q.y;
  o[2] = q.z;
  o[3] = a;
  o[4] = b;
}

}  // namespace

extern "C" size_t md_noalloc_scratch_bytes(void) { return sizeof(Scratch); }

extern "C" int md_structure_factor_noalloc(const double* pos, const double* mom, int64_t n, double lBox, int64_t kc,
                                           double my_pi, double* out5, int64_t* nk_out, void* stream) {
  if (!pos || !mom || !out5 || n < 1 || n > (1LL << 30) || !(lBox > 0) || !(my_pi > 0)) return MD_ERR_INVALID;
  if (kc < 1 || kc > kMaxKc) return MD_ERR_INVALID;  // beyond the compiled scratch size
  const int nk = count_k((int)kc);
  if (nk > kMaxNk) return MD_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return MD_ERR_NO_DEVICE;
  }
  Scratch* s;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        cudaGetLastError();
        return MD_ERR_CUDA;
      }
      g_addr[dev] = (Scratch*)ptr;
    }
    s = g_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  // each launch's own return code (a failed launch's error is then cleared
  // from the runtime's last-error state, which holds nothing of the caller's)
  auto launched = [](cudaError_t e) {
    if (e == cudaSuccess) return true;
    cudaGetLastError();
    return false;
  };
  int kci = (int)kc;
  void* a1[] = {&s, &kci};
  if (!launched(cudaLaunchKernel((const void*)k_noalloc_klist, dim3(1), dim3(1), a1, 0, st))) return MD_ERR_CUDA;
  long long nl = n;
  int nki = nk;
  double w = 2.0 * my_pi / lBox;
  void* a2[] = {&s, (void*)&pos, (void*)&mom, &nl, &nki, &w};
  if (!launched(cudaLaunchKernel((const void*)k_noalloc_partial, dim3((nk + 127) / 128, kChunks), dim3(128), a2, 0,
                                 st)))
    return MD_ERR_CUDA;
  const Scratch* cs = s;
  void* a3[] = {(void*)&cs, &nki, (void*)&out5};
  if (!launched(cudaLaunchKernel((const void*)k_noalloc_reduce, dim3((nk + 127) / 128), dim3(128), a3, 0, st)))
    return MD_ERR_CUDA;
  if (nk_out) *nk_out = nk;
  return MD_OK;
}
