// md_batch.cu -- packed stepping of several independent systems (replicas of
// uneven N: field sweeps, seed ensembles, served requests).
//
// Each system keeps its own md_ctx (buffers, Ewald setup, device time, step
// counter, records).  A batch launches every kernel of the step ONCE for all
// of its systems: the grid of a packed launch is the concatenation of the
// systems' own grids, listed in a task table (system, local block), and each
// block reads its system's parameters from a device array.  The kernel bodies
// are those of the single-system path, so a system's trajectory is the same,
// bit for bit, alone or packed with others.  One step of the whole batch is
// captured once into a CUDA graph and replayed; the graph is re-captured
// only when the set of systems changes (the task tables and grid sizes
// change), and parameter arrays are re-uploaded when a system's buffers move
// (e.g. its neighbour list grew).
//
// Requirements: mixed precision, noise off or Philox (the uploaded-noise
// mode reads host data per step), same device as the batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "md_ctx_internal.h"
#include "md_kernels.h"

namespace {

struct Slot {
  md_ctx* ctx;
  int64_t id;
  int64_t left;  // steps still to run
  double dt;
  int status;    // MD_OK or the status of the last round (non-finite state)
};

}  // namespace

struct md_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t capacity = 0;
  std::vector<Slot> slots;
  int64_t next_id = 1;
  // packed state
  bool packed = false;        // tables, parameters and graph match `slots`
  bool params_dirty = false;  // parameters must be re-uploaded (graph still valid)
  std::vector<int> order;     // pack order (system index into slots)
  CellParams* d_cell = nullptr;
  RealParams *d_rfull = nullptr, *d_rfield = nullptr;
  KParams *d_kfull = nullptr, *d_kfield = nullptr;
  IntParams *d_i1 = nullptr, *d_i2 = nullptr;
  ObsParams* d_obs = nullptr;
  int* d_status = nullptr;
  Task* d_tasks = nullptr;  // task tables (expanded on the device from d_toff)
  size_t task_cap = 0;
  int* d_toff = nullptr;    // per-system first-task offsets of every table
  size_t toff_cap = 0;
  Packed n256{}, sort{}, real{}, pass{}, phase{}, sk{}, red{}, sc{};
  WorkQ* d_wq = nullptr;  // one work queue per task table (persistent packed launches)
  unsigned* d_anyrb = nullptr;  // some system rebuilds its lists this step (zeroed)
  // systems whose k space runs on the tensor cores (the context's engine):
  // operand prep, structure factor, reduction and scatter tables, and the
  // largest dynamic shared memory among them; the others take sk, red, sc
  Packed tprep{}, tsf{}, tred{}, tsc{};
  size_t tc_sf_smem = 0, tc_sc_smem = 0;
  int kcmax = 0, np = 64;
  bool coat = false;
  int64_t launches_per_step = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool running = false;  // a round was launched and not yet waited for
  int64_t round_steps = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_round_ms = 0;
  // k-space branch of the packed step, concurrent with the real-space branch
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev[2] = {}, join_ev[2] = {};
};

namespace {

void drop_graph(md_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  b->packed = false;
}

template <typename P>
int upload(P* d, const std::vector<P>& h, cudaStream_t st) {
  if (h.empty()) return MD_OK;
  cudaError_t e = cudaMemcpyAsync(d, h.data(), sizeof(P) * h.size(), cudaMemcpyHostToDevice, st);
  return e == cudaSuccess ? MD_OK : set_err(nullptr, MD_ERR_CUDA, "parameter upload: %s", cudaGetErrorString(e));
}

// Structure-factor chunking of a tensor-core system in a batch: the fewest
// chunks of <= 512 particles (the other systems of the batch fill the GPU;
// alone, md_step splits a small system into more, smaller chunks to fill it),
// a function of the system alone, so its sums do not depend on the mix.
TcShape batch_tc_shape(const md_ctx* c) {
  return kspace_tc_shape((int)c->kc, (int)c->n, c->tc_rows, 1, c->tc_ring, 1);
}

// Parameters of every system in pack order.
int upload_params(md_batch* b) {
  const size_t R = b->order.size();
  std::vector<CellParams> cell(R);
  std::vector<RealParams> rfull(R), rfield(R);
  std::vector<KParams> kfull(R), kfield(R);
  std::vector<IntParams> i1(R), i2(R);
  std::vector<ObsParams> obs(R);
  for (size_t r = 0; r < R; r++) {
    const Slot& s = b->slots[b->order[r]];
    md_ctx* c = s.ctx;
    cell[r] = cell_params(c);
    rfull[r] = real_params(c, c->Br, c->Fr, c->ov);
    rfull[r].npairs = nullptr;
    rfield[r] = real_params(c, c->Br2, nullptr, nullptr);
    kfull[r] = k_params(c, c->Bk, c->Fk);
    kfield[r] = k_params(c, c->Bk2, nullptr);
    if (c->tc_rows > 0) {
      // the context's buffers hold its own (more numerous) chunks' partials
      const TcShape bt = batch_tc_shape(c);
      kfull[r].tc_chunk = kfield[r].tc_chunk = bt.chunk;
      kfull[r].tc_nchunk = kfield[r].tc_nchunk = bt.nchunk;
    }
    i1[r] = int_params(c, s.dt, c->Br, c->Bk);
    i2[r] = int_params(c, s.dt, c->Br2, c->Bk2);
    // packed launches evaluate every pair in FP32 (no strong-pair kernels):
    // builds do not classify, and flagged entries of an earlier build count
    // as ordinary ones
    rfull[r].strong = rfield[r].strong = 0;
    i1[r].sv.off = i2[r].sv.off = nullptr;
    obs[r] = obs_params(c, s.dt);
    obs[r].status = b->d_status + r;
  }
  int st;
  if ((st = upload(b->d_cell, cell, b->stream))) return st;
  if ((st = upload(b->d_rfull, rfull, b->stream))) return st;
  if ((st = upload(b->d_rfield, rfield, b->stream))) return st;
  if ((st = upload(b->d_kfull, kfull, b->stream))) return st;
  if ((st = upload(b->d_kfield, kfield, b->stream))) return st;
  if ((st = upload(b->d_i1, i1, b->stream))) return st;
  if ((st = upload(b->d_i2, i2, b->stream))) return st;
  if ((st = upload(b->d_obs, obs, b->stream))) return st;
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "parameter upload: %s", cudaGetErrorString(e));
  b->params_dirty = false;
  return MD_OK;
}

// Task tables on the device from the per-system offsets (off[r] .. off[r+1]
// are system r's tasks): block (system, table) writes its system's entries.
// The host uploads R + 1 offsets per table instead of one entry per block.
constexpr int kMaxTables = 16;
struct ExpandArgs {
  int off_start[kMaxTables];  // first offset of each table in toff
  int task_base[kMaxTables];  // first entry of each table in tasks
};
__global__ void __launch_bounds__(256) k_expand_tasks(const int* __restrict__ toff, Task* __restrict__ tasks,
                                                      ExpandArgs a) {
  const int t = blockIdx.y, r = blockIdx.x;
  const int* off = toff + a.off_start[t];
  const int q0 = off[r], q1 = off[r + 1];
  Task* out = tasks + a.task_base[t];
  for (int q = q0 + (int)threadIdx.x; q < q1; q += blockDim.x) out[q] = Task{r, q - q0};
}

// Task tables, parameters and the captured step for the current systems.
int pack(md_batch* b) {
  drop_graph(b);
  const int R = (int)b->slots.size();
  b->order.resize(R);
  std::iota(b->order.begin(), b->order.end(), 0);
  // larger systems first: their blocks start first in every packed grid
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int x, int y) { return b->slots[x].ctx->n > b->slots[y].ctx->n; });
  // a system's k space runs on the tensor cores in the batch when it does
  // alone (tc_rows > 0: mixed precision, the tensor-core engine, kc within
  // the kernels' bounds), otherwise on the CUDA-core kernels
  auto on_tc = [](const md_ctx* c) { return c->tc_rows > 0; };
  b->kcmax = 0;
  b->coat = false;
  b->tc_sf_smem = b->tc_sc_smem = 0;
  bool any_simt = false;
  for (const Slot& s : b->slots) {
    if (on_tc(s.ctx)) {
      b->tc_sf_smem = std::max(b->tc_sf_smem, kspace_tc_sf_bytes(s.ctx->tcs, (int)s.ctx->kc));
      b->tc_sc_smem = std::max(b->tc_sc_smem, (size_t)s.ctx->tcs.scat_smem);
    } else {
      b->kcmax = std::max<int>(b->kcmax, (int)s.ctx->kc);
      any_simt = true;
    }
    b->coat = b->coat || s.ctx->cfg.ENABLE_COATING_POT;
  }
  b->np = scatter_particles(b->kcmax, false);
  if (any_simt && !b->np) return set_err(nullptr, MD_ERR_UNSUPPORTED, "kc too large for the packed k-space scatter");
  // task tables, one per kernel shape: R + 1 offsets each on the host
  std::vector<int> toff;
  ExpandArgs ex{};
  int ntab = 0;
  size_t ntask = 0;
  auto table = [&](Packed& pk, auto blocks_of) {
    if (ntab == kMaxTables) {  // a table beyond ExpandArgs' bounds: a build error, caught by every test
      pk.n = 0;
      pk.tasks = nullptr;
      return;
    }
    ex.off_start[ntab] = (int)toff.size();
    ex.task_base[ntab] = (int)ntask;
    ntab++;
    int cnt = 0;
    for (int r = 0; r < R; r++) {
      toff.push_back(cnt);
      cnt += blocks_of(b->slots[b->order[r]].ctx);
    }
    toff.push_back(cnt);
    pk.n = cnt;
    pk.tasks = reinterpret_cast<const Task*>(ntask);  // offset until the allocation
    ntask += (size_t)cnt;
  };
  table(b->n256, [](md_ctx* c) { return cell_blocks((int)c->n); });
  table(b->sort, [](md_ctx* c) { return cell_sort_blocks(c->grid); });
  table(b->real, [](md_ctx* c) { return real_blocks((int)c->n); });
  table(b->pass, [](md_ctx* c) { return real_pass_blocks((int)c->n); });
  table(b->phase, [](md_ctx* c) { return phase_blocks((int)c->n); });
  table(b->sk, [&](md_ctx* c) { return on_tc(c) ? 0 : sk_blocks(k_params(c, nullptr, nullptr)); });
  table(b->red, [&](md_ctx* c) { return on_tc(c) ? 0 : skred_blocks(k_params(c, nullptr, nullptr)); });
  const int np = b->np;
  table(b->sc, [&](md_ctx* c) { return on_tc(c) ? 0 : scatter_blocks(k_params(c, nullptr, nullptr), np); });
  // tensor-core systems: the blocks of their grids, the structure factor
  // with the batch chunking (batch_tc_shape)
  table(b->tprep, [&](md_ctx* c) { return on_tc(c) ? c->tcs.nsb : 0; });
  table(b->tsf, [&](md_ctx* c) {
    if (!on_tc(c)) return 0;
    const TcShape bt = batch_tc_shape(c);
    return bt.mt * bt.nchunk;
  });
  table(b->tred, [&](md_ctx* c) { return on_tc(c) ? c->tcs.mt * (2 * (int)c->kc + 1) : 0; });
  table(b->tsc, [&](md_ctx* c) { return on_tc(c) ? (int)((c->n + 127) / 128) : 0; });
  if (toff.size() > b->toff_cap) {
    if (b->d_toff) cudaFree(b->d_toff);
    b->d_toff = nullptr;
    b->toff_cap = 0;
    const size_t cap = toff.size() + toff.size() / 4 + 256;
    cudaError_t e = cudaMalloc(&b->d_toff, sizeof(int) * cap);
    if (e != cudaSuccess) return set_err(nullptr, MD_ERR_NOMEM, "task offsets: %s", cudaGetErrorString(e));
    b->toff_cap = cap;
  }
  if (ntask > b->task_cap) {
    if (b->d_tasks) cudaFree(b->d_tasks);
    b->d_tasks = nullptr;
    b->task_cap = 0;
    const size_t cap = ntask + ntask / 4 + 1024;
    cudaError_t e = cudaMalloc(&b->d_tasks, sizeof(Task) * cap);
    if (e != cudaSuccess) return set_err(nullptr, MD_ERR_NOMEM, "task table: %s", cudaGetErrorString(e));
    b->task_cap = cap;
  }
  for (Packed* pk : {&b->n256, &b->sort, &b->real, &b->pass, &b->phase, &b->sk, &b->red, &b->sc, &b->tprep, &b->tsf,
                     &b->tred, &b->tsc})
    pk->tasks = b->d_tasks + reinterpret_cast<size_t>(pk->tasks);
  if (!b->d_wq) {
    cudaError_t e = cudaMalloc(&b->d_wq, sizeof(WorkQ) * 8);
    if (e == cudaSuccess) e = cudaMemset(b->d_wq, 0, sizeof(WorkQ) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_anyrb, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(b->d_anyrb, 0, sizeof(unsigned));
    if (e != cudaSuccess) return set_err(nullptr, MD_ERR_NOMEM, "work queues: %s", cudaGetErrorString(e));
  }
  {
    // launches over one table run in stream order (never two at once), so a
    // queue per table suffices
    int q = 0;
    for (Packed* pk : {&b->n256, &b->sort, &b->real, &b->pass, &b->phase, &b->sk, &b->red, &b->sc}) pk->wq = b->d_wq + q++;
  }
  int st;
  if ((st = upload(b->d_toff, toff, b->stream))) return st;
  if (R > 0) {
    k_expand_tasks<<<dim3(R, ntab), 256, 0, b->stream>>>(b->d_toff, b->d_tasks, ex);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "task tables: %s", cudaGetErrorString(e));
  }
  if ((st = upload_params(b))) return st;
  if (R == 0) {
    b->packed = true;
    b->launches_per_step = 0;
    return MD_OK;
  }
  // capture one step of every system
  cudaStream_t s = b->stream;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
  int64_t l = 0;
  // the k-space branches run on the side stream, concurrently with the
  // real-space branches (parallel branches of the captured graph)
  cudaStream_t k = b->side;
  auto fork = [&](int q) {
    cudaEventRecord(b->fork_ev[q], s);
    cudaStreamWaitEvent(k, b->fork_ev[q], 0);
  };
  auto join = [&](int q) {
    cudaEventRecord(b->join_ev[q], k);
    cudaStreamWaitEvent(s, b->join_ev[q], 0);
  };
  l += launch_step_begin_packed(s, b->d_cell, R, b->d_anyrb);
  l += launch_cells_packed(s, b->d_cell, R, b->n256, b->sort, b->d_anyrb);
  fork(0);
  l += launch_phase_tables_packed(k, b->d_kfull, b->phase);
  l += launch_kspace_tc_prep_packed(k, b->d_kfull, b->tprep);
  l += launch_kspace_packed(k, b->d_kfull, b->sk, b->red, b->sc, true, b->kcmax, b->np);
  l += launch_kspace_tc_packed(k, b->d_kfull, b->tsf, b->tred, b->tsc, true, b->tc_sf_smem, b->tc_sc_smem);
  l += launch_nbr_packed(s, b->d_rfull, R, b->real, b->d_anyrb);
  l += launch_real_packed(s, b->d_rfull, b->real, b->pass, true, b->coat);
  join(0);
  l += launch_heun1_packed(s, b->d_i1, b->n256);
  fork(1);
  l += launch_kspace_packed(k, b->d_kfield, b->sk, b->red, b->sc, false, b->kcmax, b->np);
  l += launch_kspace_tc_packed(k, b->d_kfield, b->tsf, b->tred, b->tsc, false, b->tc_sf_smem, b->tc_sc_smem);
  l += launch_real_packed(s, b->d_rfield, b->real, b->pass, false, false);
  join(1);
  l += launch_heun2_packed(s, b->d_i2, b->n256);
  l += launch_obs_packed(s, b->d_obs, R, b->d_anyrb);
  e = cudaStreamEndCapture(s, &b->graph);
  if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->gexec, b->graph, 0);
  if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  b->launches_per_step = l;
  b->packed = true;
  return MD_OK;
}

Slot* find(md_batch* b, int64_t id) {
  for (Slot& s : b->slots)
    if (s.id == id) return &s;
  return nullptr;
}

template <typename P>
int alloc_array(P** p, size_t n) {
  cudaError_t e = cudaMalloc(p, sizeof(P) * std::max<size_t>(n, 1));
  return e == cudaSuccess ? MD_OK : set_err(nullptr, MD_ERR_NOMEM, "batch arrays: %s", cudaGetErrorString(e));
}

// Completes the launched round: per-system status (non-finite state, list
// overflow), step accounting.
int finish_round(md_batch* b) {
  if (!b->running) return MD_OK;
  b->running = false;
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "batch round: %s", cudaGetErrorString(e));
  cudaEventElapsedTime(&b->last_round_ms, b->ev0, b->ev1);
  const size_t R = b->order.size();
  std::vector<int> status(R);
  if (R) {
    e = cudaMemcpy(status.data(), b->d_status, sizeof(int) * R, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "batch status: %s", cudaGetErrorString(e));
  }
  int bad = MD_OK;
  for (size_t r = 0; r < R; r++) {
    Slot& s = b->slots[b->order[r]];
    s.left -= b->round_steps;
    s.ctx->have_geometry = true;
    s.ctx->list_valid = true;
    if (status[r] & 4) {
      // the neighbour list did not fit (results are correct): grow it
      const int64_t cap0 = s.ctx->nbr_cap;
      int st = check_overflow(s.ctx);
      if (st) return st;
      if (s.ctx->nbr_cap != cap0) b->params_dirty = true;
    }
    if (status[r] & ~4) {
      const int st = read_err_word(s.ctx);  // clears the word and records the message
      if (st) {
        s.status = st;
        if (!bad) bad = set_err(nullptr, st, "system %lld: non-finite state", (long long)s.id);
      }
    }
    if (status[r]) {
      // the fixes above went through the system's own stream
      e = cudaStreamSynchronize(s.ctx->stream);
      if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "batch status: %s", cudaGetErrorString(e));
    }
  }
  if (R) cudaMemset(b->d_status, 0, sizeof(int) * R);
  return bad;
}

}  // namespace

extern "C" {

int md_batch_create(int64_t capacity, md_batch** out) {
  if (!out || capacity < 1 || capacity > (1 << 20)) return set_err(nullptr, MD_ERR_INVALID, "bad batch capacity");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_err(nullptr, MD_ERR_NO_DEVICE, "no CUDA device visible");
  }
  md_batch* b = new md_batch();
  cudaGetDevice(&b->device);
  b->capacity = capacity;
  int st = MD_OK;
  auto fail = [&](int s) {
    md_batch_destroy(b);
    return s;
  };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
    return fail(set_err(nullptr, MD_ERR_CUDA, "batch stream/events"));
  for (int q = 0; q < 2; q++)
    if (cudaEventCreateWithFlags(&b->fork_ev[q], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join_ev[q], cudaEventDisableTiming) != cudaSuccess)
      return fail(set_err(nullptr, MD_ERR_CUDA, "batch events"));
  const size_t C = (size_t)capacity;
  if ((st = alloc_array(&b->d_cell, C)) || (st = alloc_array(&b->d_rfull, C)) || (st = alloc_array(&b->d_rfield, C)) ||
      (st = alloc_array(&b->d_kfull, C)) || (st = alloc_array(&b->d_kfield, C)) || (st = alloc_array(&b->d_i1, C)) ||
      (st = alloc_array(&b->d_i2, C)) || (st = alloc_array(&b->d_obs, C)) || (st = alloc_array(&b->d_status, C)))
    return fail(st);
  if (cudaMemset(b->d_status, 0, sizeof(int) * C) != cudaSuccess)
    return fail(set_err(nullptr, MD_ERR_CUDA, "batch status init"));
  *out = b;
  return MD_OK;
}

int md_batch_destroy(md_batch* b) {
  if (!b) return MD_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  void* arrays[] = {b->d_cell, b->d_rfull, b->d_rfield, b->d_kfull, b->d_kfield, b->d_i1, b->d_i2, b->d_obs,
                    b->d_status, b->d_tasks, b->d_toff, b->d_wq, b->d_anyrb};
  for (void* p : arrays)
    if (p) cudaFree(p);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  for (int q = 0; q < 2; q++) {
    if (b->fork_ev[q]) cudaEventDestroy(b->fork_ev[q]);
    if (b->join_ev[q]) cudaEventDestroy(b->join_ev[q]);
  }
  if (b->side) cudaStreamDestroy(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return MD_OK;
}

int md_batch_add(md_batch* b, md_ctx* c, int64_t nsteps, double dt, int64_t* id) {
  if (!b || !c) return set_err(nullptr, MD_ERR_INVALID, "null batch or context");
  if (b->running) return set_err(nullptr, MD_ERR_INVALID, "batch round in flight (md_batch_wait first)");
  if ((int64_t)b->slots.size() >= b->capacity) return set_err(nullptr, MD_ERR_NOMEM, "batch is full");
  if (nsteps < 0 || !(dt > 0)) return set_err(nullptr, MD_ERR_INVALID, "bad nsteps or dt");
  int st = check_ready(c, true);
  if (st) return st;
  if (c->prec != MD_PREC_MIXED) return set_err(c, MD_ERR_UNSUPPORTED, "packed stepping runs mixed precision only");
  if (c->noise == MD_NOISE_UPLOADED) return set_err(c, MD_ERR_UNSUPPORTED, "packed stepping: noise off or Philox");
  if (c->device != b->device) return set_err(c, MD_ERR_INVALID, "context and batch on different devices");
  for (const Slot& s : b->slots)
    if (s.ctx == c) return set_err(c, MD_ERR_INVALID, "context already in the batch");
  if (!scatter_particles((int)c->kc, false)) return set_err(c, MD_ERR_UNSUPPORTED, "kc too large");
  if ((st = prepare_dt(c, dt))) return st;
  if ((st = ensure_records(c, nsteps))) return st;
  CK(c, cudaStreamSynchronize(c->stream));
  Slot s{c, b->next_id++, nsteps, dt, MD_OK};
  b->slots.push_back(s);
  b->packed = false;
  if (id) *id = s.id;
  return MD_OK;
}

int md_batch_remove(md_batch* b, int64_t id) {
  if (!b) return set_err(nullptr, MD_ERR_INVALID, "null batch");
  if (b->running) return set_err(nullptr, MD_ERR_INVALID, "batch round in flight (md_batch_wait first)");
  for (size_t k = 0; k < b->slots.size(); k++)
    if (b->slots[k].id == id) {
      b->slots.erase(b->slots.begin() + k);
      b->packed = false;
      return MD_OK;
    }
  return set_err(nullptr, MD_ERR_INVALID, "no system %lld in the batch", (long long)id);
}

int md_batch_launch(md_batch* b, int64_t max_steps, int64_t* steps) {
  NvtxRange nv("md_batch_launch");
  if (!b || max_steps < 0) return set_err(nullptr, MD_ERR_INVALID, "bad arguments");
  if (b->running) return set_err(nullptr, MD_ERR_INVALID, "batch round in flight (md_batch_wait first)");
  int64_t k = max_steps;
  for (const Slot& s : b->slots) k = std::min(k, s.left);
  if (b->slots.empty()) k = 0;
  if (steps) *steps = k;
  if (k <= 0) return MD_OK;
  int st;
  if (!b->packed) {
    if ((st = pack(b))) return st;
  } else if (b->params_dirty) {
    if ((st = upload_params(b))) return st;
  }
  cudaEventRecord(b->ev0, b->stream);
  for (int64_t q = 0; q < k; q++) {
    cudaError_t e = cudaGraphLaunch(b->gexec, b->stream);
    if (e != cudaSuccess) return set_err(nullptr, MD_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
  }
  cudaEventRecord(b->ev1, b->stream);
  b->round_steps = k;
  b->running = true;
  return MD_OK;
}

int md_batch_wait(md_batch* b) {
  if (!b) return set_err(nullptr, MD_ERR_INVALID, "null batch");
  return finish_round(b);
}

int md_batch_run(md_batch* b, int64_t max_steps, int64_t* steps) {
  int st = md_batch_launch(b, max_steps, steps);
  if (st) return st;
  return finish_round(b);
}

int md_batch_remaining(const md_batch* b, int64_t id, int64_t* left, int* status) {
  if (!b) return set_err(nullptr, MD_ERR_INVALID, "null argument");
  Slot* s = find(const_cast<md_batch*>(b), id);
  if (!s) return set_err(nullptr, MD_ERR_INVALID, "no system %lld in the batch", (long long)id);
  if (left) *left = s->left;
  if (status) *status = s->status;
  return MD_OK;
}

int md_batch_info(const md_batch* b, int64_t* systems, int64_t* particles, int64_t* launches_per_step,
                  double* last_round_ms) {
  if (!b) return set_err(nullptr, MD_ERR_INVALID, "null batch");
  int64_t np = 0;
  for (const Slot& s : b->slots) np += s.ctx->n;
  if (systems) *systems = (int64_t)b->slots.size();
  if (particles) *particles = np;
  if (launches_per_step) *launches_per_step = b->launches_per_step;
  if (last_round_ms) *last_round_ms = b->last_round_ms;
  return MD_OK;
}

}  // extern "C"
