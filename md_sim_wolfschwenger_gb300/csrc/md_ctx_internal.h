// md_ctx_internal.h -- the context behind the C ABI (include/md_gb300.h):
// host bookkeeping and the device buffers of one simulated system, plus the
// helpers shared by md_ctx.cu (one system) and md_batch.cu (packed systems).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/md_gb300.h"
#include "md_common.cuh"
#include "md_err.h"
#include "md_host.h"
#include "md_kernels.h"

namespace md {

// Device-resident scalars of one system.
struct DevScalars {
  double time;
  long long step;
  long long nrec;
  int err;
  unsigned done;  // blocks of the fused stage-2 + records kernel that finished (0 between launches)
  double musum[3];
  unsigned long long pairs;
  StepFlags flags;
  unsigned long long errmax;  // adaptive solvers: error norm of the attempt (double bits)
};

}  // namespace md

using namespace md;

// Named ranges for timeline tools (NVTX v3, header only; no-ops unless a
// tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

struct md_ctx {
  md_config cfg{};
  int64_t n = 0;
  int prec = MD_PREC_MIXED;
  int device = 0;
  cudaStream_t stream = nullptr;
  // second stream of the step: the k-space branch runs on it concurrently
  // with the real-space branch (fork/join events; captured into the graph)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev[2] = {}, join_ev[2] = {};
  std::string err;
  int err_status = 0;
  std::vector<void*> allocs;
  std::vector<size_t> alloc_bytes;  // size of each entry of allocs
  int64_t bytes = 0;

  // host state
  mdh::Props props;
  bool have_particles = false, have_state = false, have_ewald = false, have_geometry = false;
  double L = 0, alpha = 0, rc = 0;
  int64_t kc = 0;
  CellGrid grid{1, 1, 0};
  mdh::KList klist;
  int nchunk = 1, chunk = 0;
  int noise = MD_NOISE_PHILOX;
  uint64_t seed = 1;
  double cur_dt = -1;
  bool graph_valid = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t launches = 0, launches_per_step = 0;

  // device: master state & particle constants
  double *pos = nullptr, *mm = nullptr, *ea = nullptr, *truePos = nullptr, *posRef = nullptr;
  double *xi = nullptr, *tmpmm = nullptr, *Bout = nullptr, *Fout = nullptr;
  double *magMom_u = nullptr, *rMag_u = nullptr, *invZt = nullptr, *velEa1 = nullptr, *velEa2 = nullptr;
  double *sT = nullptr, *sB = nullptr, *sF = nullptr;
  // cells and sorted views
  int *cellOf = nullptr, *tmp = nullptr, *perm = nullptr, *rank = nullptr, *scell = nullptr;
  int *count = nullptr, *cell_start = nullptr;
  int ncell_cap = 0;
  float4* xf = nullptr;
  int4* xi4 = nullptr;
  double4_32a* xd = nullptr;
  void* mu = nullptr;
  // stage outputs (T)
  void *Br = nullptr, *Fr = nullptr, *ov = nullptr, *Bk = nullptr, *Fk = nullptr, *Br2 = nullptr, *Bk2 = nullptr;
  void *k1m = nullptr, *k1e = nullptr, *m2 = nullptr, *e2 = nullptr, *th = nullptr;
  // adaptive solvers (allocated on first use): stage slopes and coordinates
  void *rk_km[7] = {}, *rk_ke[7] = {}, *rk_cm = nullptr, *rk_ce = nullptr;
  double *Ppart = nullptr, *obs_part = nullptr;
  DevScalars* sc = nullptr;
  double* records = nullptr;
  long long rec_cap = 0;
  long long nrec_bound = 0;  // upper bound of the device's record count (ensure_records)
  // k space
  KSeg* kseg = nullptr;
  int* koff = nullptr;
  double* ek = nullptr;
  KSeg* rseg = nullptr;
  int* rowpos = nullptr;
  int2* chunks = nullptr;
  double2* Spart = nullptr;
  double* musum_part = nullptr;
  void* eS = nullptr;
  double2* Sfull = nullptr;
  void* ptab = nullptr;  // phase tables [3][kc+1][n]
  size_t ptab_cap = 0;
  size_t ksize_cap = 0, spart_cap = 0;
  int musum_cap = 0;
  // tensor-core k space (mixed path; md_ktc.cu): engine choice, k rows and
  // their buffers (tc_rows = 0 while the engine is off)
  int kengine = MD_KSPACE_AUTO;
  long long tc_wait = 2000000000LL;  // mbarrier wait limit of the tensor-core kernels (SM cycles)
  int tc_ring = -1, tc_waves = 1;     // structure-factor ring option and chunk-count multiplier (tuning)
  int tc_rows = 0;
  TcShape tcs{};
  int2* tc_row = nullptr;
  float4* tc_rowd = nullptr;  // scatter row descriptors
  int* tc_kmap = nullptr;
  float* tc_part = nullptr;
  float *tc_wfull = nullptr, *tc_wfield = nullptr;
  float* tc_bimg = nullptr;
  float2* tc_tblk = nullptr;
  // Verlet list (sorted indices) within rc + skin
  int *nbr = nullptr, *nbr_cnt = nullptr, *nbr_off = nullptr;
  long long nbr_cap = 0;
  double* xbuild = nullptr;
  // skin = skin_frac * rc.  Entries between rc and rc (1 + skin) cost a lane
  // each in both passes (~3 skin of the list); a Brownian step moves a
  // particle ~5 pm at dt = 1e-12 s, so even a 0.5 % skin (1 nm at rc = 400
  // nm) is crossed only after ~1e4 steps and rebuilds stay rare.
  double skin_frac = 0.005;
  bool list_valid = false;  // a build for the current particles, grid and skin exists
  // Strong pairs (mixed path, md_real.cu): list entries whose force weight
  // (|mu_i| |mu_j| / mu_min^2) (2 rHydr_min / r)^4 exceeds strong_theta are
  // evaluated in FP64; strong_w4sq is that threshold in kernel units
  // (squared, for |mu_i|^2 |mu_j|^2 > w4sq r^8; < 0: off).
  double kself[6] = {0, 0, 0, 0, 0, 0};  // k-space self-interaction matrix (IntParams::kself)
  double strong_theta = 3.0;
  float strong_w4sq = -1.f;
  int2* snbr = nullptr;
  int *snbr_cnt = nullptr, *snbr_off = nullptr;
  double* svals = nullptr;   // [9][scap] FP64 B, F, P terms per entry (full evaluation)
  double* svals2 = nullptr;  // [3][scap] FP64 B terms per entry (field-only evaluation)
  long long scap = 0;
  // profiling: events between the kernel segments of a step
  bool prof = false;
  cudaEvent_t ev[MD_NSEG + 1] = {};
};

// ------------------------------------------------------------ helpers

#define CK(ctx, call)                                                                              \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return set_err(ctx, MD_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                     __FILE__, __LINE__);                                                          \
  } while (0)

int dalloc_raw(md_ctx* c, void** p, size_t bytes);
template <typename P>
inline int dalloc(md_ctx* c, P** p, size_t bytes) {
  void* q = nullptr;
  const int st = dalloc_raw(c, &q, bytes);
  if (st == MD_OK) *p = (P*)q;
  return st;
}
void dfree(md_ctx* c, void* p);
bool fp64(const md_ctx* c);
size_t tsz(const md_ctx* c);
void invalidate_graph(md_ctx* c);
md::SortedView sorted_view(md_ctx* c);
double B_unit(const md_ctx* c);
double F_unit(const md_ctx* c);
md::CellParams cell_params(md_ctx* c);
md::RealParams real_params(md_ctx* c, void* B, void* F, void* ov);
md::KParams k_params(md_ctx* c, void* B, void* F);
md::IntParams int_params(md_ctx* c, double dt, const void* Br, const void* Bk);
md::ObsParams obs_params(md_ctx* c, double dt);
int check_ready(md_ctx* c, bool need_state);
int force_rebuild(md_ctx* c);
int alloc_nbr(md_ctx* c, long long cap);
// Strong-pair path: on for the mixed path without coating potentials and
// with a finite threshold; alloc_strong grows the strong list.
bool strong_active(const md_ctx* c);
int alloc_strong(md_ctx* c, long long cap);
void update_strong(md_ctx* c);
int check_overflow(md_ctx* c);
int ensure_records(md_ctx* c, int64_t extra);
int read_err_word(md_ctx* c);
// Thermal-noise scales for the step dt (DefThermFluct prefactors).
int prepare_dt(md_ctx* c, double dt);
