// Serving queue: continuous batching of ASD-POCS jobs on one GPU (host code).
//
// A worker thread owns every CUDA call.  Jobs are routed to the lane of
// their scan protocol -- identical sizes, geometry and view angles -- and
// wait there until a slot is free and the HBM budget has room for their
// state.  A lane owns the protocol's geometry (detector coordinates, view
// angles, ray tables, the residuals of its slots interleaved in groups of
// kShareSlots), computed once, so its backward step computes each chord once
// per voxel for a whole group of jobs.  Admission allocates the job's state
// (stream-ordered pool), uploads its data, resets its scalars and writes its
// descriptor into the lane's slot, all on the lane's stream, so it orders
// after the iterations already queued there.  A lane runs one ASD-POCS
// iteration of all its slots per launch sequence (empty slots point at
// scalars with done = 1 and exit at once), captured in a CUDA graph that is
// re-captured only when a job needs more TV steps than the captured one.
// After each iteration a tiny kernel gathers the slots' done flags into
// pinned memory; when the worker sees a job done it enqueues the copies of
// its results, empties the slot and frees the job's memory, again in stream
// order.  Lanes run on their own streams, so different protocols overlap on
// the device.  Every kernel computes an instance at its own sizes and
// reduces over its own blocks, so a job's result does not depend on the
// jobs sharing its launches.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "instance.h"

namespace asd {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
  long long id = 0;
  asdpocs_geometry g{};
  asdpocs_options o{};
  std::vector<double> phi;
  std::vector<float> P, m0, I0;  // host copies, dropped after upload
  std::vector<uint16_t> P16;     // the sinogram in FP16 / BF16 storage
  bool has_m0 = false, has_ref = false;
  bool cancel = false;  // asdpocs_server_cancel on a running job
  int state = ASDPOCS_JOB_QUEUED;
  Clock::time_point t_submit, t_admit, t_done;
  InstLayout lay{};
  char *dev = nullptr;
  int slot = -1;
  // results (one pinned block from the server's pool, filled by
  // stream-ordered copies): image, then RMSE, then the scalars
  void *pin = nullptr;
  size_t pin_cls = 0;
  float *img = nullptr;
  double *rmse = nullptr;
  Scalars *scal = nullptr;
  cudaEvent_t ev_done = nullptr;  // upload done, later results ready
};

struct Flight {
  cudaEvent_t ev = nullptr;
  int *flags = nullptr;            // pinned, one per slot
  std::vector<long long> owner;    // job id per slot when it was queued (0: none)
};

struct Lane {
  asdpocs_geometry g{};            // the protocol
  std::vector<double> phi;
  cudaStream_t st = nullptr;
  int S = 0;
  Inst *d_inst = nullptr;          // S descriptors
  int *d_flags = nullptr;          // S done flags
  Scalars *d_dead = nullptr;       // scalars of an empty slot (done = 1)
  char *geo = nullptr;             // the protocol's geometry block
  size_t geo_bytes = 0;
  int *chtab = nullptr;            // backward-step chord tables (2-D protocols)
  size_t chtab_bytes = 0;
  Inst tmpl{};                     // geometry of every slot
  std::vector<Inst> slot_desc;     // descriptor of each slot (host copy)
  std::vector<Job *> slot_job;
  int active = 0;
  std::deque<Job *> queue;
  std::vector<Job *> harvesting;
  std::deque<Flight> inflight;
  std::vector<Flight> spare;
  // captured iteration
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int gng = -1, gbatch = 0;  // TV steps and slots the graph covers
};

// Key of a job's lane: its sizes, geometry and angles, byte for byte.
std::string protocol_key(const asdpocs_geometry &g, const std::vector<double> &phi) {
  std::string k((const char *)&g, sizeof g);
  k.append((const char *)phi.data(), phi.size() * sizeof(double));
  return k;
}

// Pinned host blocks by power-of-two size class.  Blocks are allocated when
// a class runs dry and kept until the server is destroyed: page-locking and
// releasing host memory can stall every stream of the device, so neither
// happens while jobs run once the pool has warmed up.
struct PinnedPool {
  std::map<size_t, std::vector<void *>> spare;
  std::vector<void *> all;
  cudaError_t get(size_t bytes, void *&p, size_t &cls) {
    cls = 4096;
    while (cls < bytes) cls <<= 1;
    std::vector<void *> &v = spare[cls];
    if (!v.empty()) {
      p = v.back();
      v.pop_back();
      return cudaSuccess;
    }
    const cudaError_t e = cudaMallocHost(&p, cls);
    if (e == cudaSuccess) all.push_back(p);
    return e;
  }
  void put(void *p, size_t cls) {
    if (p) spare[cls].push_back(p);
  }
  void release() {
    for (void *p : all) cudaFreeHost(p);
    all.clear();
    spare.clear();
  }
};

}  // namespace
}  // namespace asd

struct asdpocs_server_s {
  int device = 0;
  asdpocs_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  bool stop = false;
  std::string error;  // set when the worker hit a CUDA error
  long long next_id = 1;
  std::map<long long, std::unique_ptr<asd::Job>> jobs;
  std::deque<asd::Job *> pending;  // not yet assigned to a lane
  std::map<std::string, std::unique_ptr<asd::Lane>> lanes;
  cudaMemPool_t pool = nullptr;  // the jobs' device memory
  cudaStream_t upload = nullptr; // admissions: allocation and data upload
  asd::PinnedPool pinned;        // the jobs' result blocks
  unsigned long long budget = 0, in_use = 0, peak = 0;
  unsigned long long chord_bytes = 0;  // the lanes' chord tables
};

namespace asd {
namespace {

#define SV_CUDA(call)                                 \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return fail(sv, e_, #call); \
  } while (0)

bool fail(asdpocs_server sv, cudaError_t e, const char *what) {
  if (sv->error.empty())
    sv->error = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

Dims inst_dims(const asdpocs_geometry &g) {
  return Dims{g.nx, g.ny, g.nz, g.na, g.nb};
}

// Slot s's descriptor when empty: the protocol's geometry with scalars that
// say done.  Slot 0 refreshes the shared 3-D ray-slope table every view.
Inst empty_slot(const Lane &L, int s) {
  Inst I = L.tmpl;
  I.s = L.d_dead;
  const size_t M = (size_t)L.g.na * L.g.nb;
  const size_t N = (size_t)L.g.nx * L.g.ny * L.g.nz;
  I.cor = L.tmpl.cor + (size_t)(s / kShareSlots) * M * kShareSlots + s % kShareSlots;
  I.cor_stride = kShareSlots;
  I.m_il = L.tmpl.m_il + (size_t)(s / kShareSlots) * N * kShareSlots;
  I.tabc_mode = s == 0 ? kTabcShared : kTabcNone;
  return I;
}

bool lane_create(asdpocs_server sv, Lane &L) {
  // slots: as configured, but the lane's interleaved images (4 bytes per
  // voxel and slot) within an eighth of the budget, in whole groups
  const size_t vox = (size_t)L.g.nx * L.g.ny * L.g.nz;
  const long long fit = (long long)(sv->budget / 8 / (vox * 4));
  L.S = (int)std::min<long long>(sv->cfg.slots_per_lane,
                                 std::max<long long>(kShareSlots, fit / kShareSlots * kShareSlots));
  const size_t M = (size_t)L.g.na * L.g.nb;
  const int groups = (L.S + kShareSlots - 1) / kShareSlots;
  SV_CUDA(cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking));
  SV_CUDA(cudaMalloc(&L.d_inst, sizeof(Inst) * L.S));
  SV_CUDA(cudaMalloc(&L.d_flags, sizeof(int) * L.S));
  SV_CUDA(cudaMalloc(&L.d_dead, sizeof(Scalars)));
  const size_t N = (size_t)L.g.nx * L.g.ny * L.g.nz;
  const InstLayout gl = layout_instance(L.g, 0, (size_t)groups * kShareSlots * M,
                                        kLayoutGeometry, (size_t)groups * kShareSlots * N);
  SV_CUDA(cudaMalloc(&L.geo, gl.bytes));
  L.geo_bytes = gl.bytes;  // outside the jobs' budget (bounded by the slots rule)
  SV_CUDA(cudaMemsetAsync(L.geo, 0, gl.bytes, L.st));
  Scalars dead_s;
  memset(&dead_s, 0, sizeof dead_s);
  dead_s.done = 1;
  SV_CUDA(cudaMemcpyAsync(L.d_dead, &dead_s, sizeof dead_s, cudaMemcpyHostToDevice,
                          L.st));
  memset(&L.tmpl, 0, sizeof L.tmpl);
  SV_CUDA(bind_geometry(L.tmpl, L.geo, gl, L.g, L.phi.data(), L.st));
  L.tmpl.m_il = (float *)(L.geo + gl.m_il);
  L.slot_desc.resize(L.S);
  for (int s = 0; s < L.S; s++) L.slot_desc[s] = empty_slot(L, s);
  SV_CUDA(cudaMemcpyAsync(L.d_inst, L.slot_desc.data(), sizeof(Inst) * L.S,
                          cudaMemcpyHostToDevice, L.st));
  // the protocol's ray tables and view flags, once, through slot 0
  SV_CUDA(launch_view_tables(L.d_inst, 1, inst_dims(L.g), L.g.nv, L.st));
  // and a 2-D protocol's backward-step chord tables: every lane's together
  // within a quarter of the budget (outside the jobs' share, like the
  // geometry block); without them the lane computes chords in every step
  const unsigned long long room =
      sv->budget / 4 > sv->chord_bytes ? sv->budget / 4 - sv->chord_bytes : 0;
  int K = 0;
  if (!getenv("ASDPOCS_NO_CHORD_TABLE"))
    SV_CUDA(build_chord_tables(L.d_inst, inst_dims(L.g), L.g.nv, (size_t)room, L.st,
                               &L.chtab, &K, &L.chtab_bytes));
  if (L.chtab) {
    sv->chord_bytes += L.chtab_bytes;
    L.tmpl.chtab = L.chtab;
    L.tmpl.chK = K;
    for (int s = 0; s < L.S; s++) L.slot_desc[s] = empty_slot(L, s);
    SV_CUDA(cudaMemcpyAsync(L.d_inst, L.slot_desc.data(), sizeof(Inst) * L.S,
                            cudaMemcpyHostToDevice, L.st));
  }
  L.slot_job.assign(L.S, nullptr);
  return true;
}

void lane_destroy(Lane &L) {
  if (L.st) cudaStreamSynchronize(L.st);
  for (Flight &f : L.inflight) {
    cudaEventDestroy(f.ev);
    cudaFreeHost(f.flags);
  }
  for (Flight &f : L.spare) {
    cudaEventDestroy(f.ev);
    cudaFreeHost(f.flags);
  }
  if (L.exec) cudaGraphExecDestroy(L.exec);
  if (L.graph) cudaGraphDestroy(L.graph);
  cudaFree(L.d_inst);
  cudaFree(L.d_flags);
  cudaFree(L.d_dead);
  cudaFree(L.geo);
  if (L.chtab) cudaFree(L.chtab);
  if (L.st) cudaStreamDestroy(L.st);
}

// Results of a finished job: stream-ordered copies, then the slot is
// emptied and the job's memory returned to the pool.
bool harvest(asdpocs_server sv, Lane &L, int s) {
  Job *J = L.slot_job[s];
  const size_t N = (size_t)J->g.nx * J->g.ny * J->g.nz;
  char *b = J->dev;
  SV_CUDA(cudaMemcpyAsync(J->img, b + J->lay.m_res, N * 4, cudaMemcpyDeviceToHost,
                          L.st));
  SV_CUDA(cudaMemcpyAsync(J->scal, b + J->lay.scal, sizeof(Scalars),
                          cudaMemcpyDeviceToHost, L.st));
  if (J->o.maxnumIter > 0)
    SV_CUDA(cudaMemcpyAsync(J->rmse, b + J->lay.rmse, (size_t)J->o.maxnumIter * 8,
                            cudaMemcpyDeviceToHost, L.st));
  SV_CUDA(cudaEventRecord(J->ev_done, L.st));
  L.slot_desc[s] = empty_slot(L, s);
  SV_CUDA(cudaMemcpyAsync(L.d_inst + s, &L.slot_desc[s], sizeof(Inst),
                          cudaMemcpyHostToDevice, L.st));
  SV_CUDA(cudaFreeAsync(J->dev, L.st));
  J->dev = nullptr;
  sv->in_use -= J->lay.bytes;
  L.slot_job[s] = nullptr;
  L.active--;
  L.harvesting.push_back(J);
  return true;
}

bool admit(asdpocs_server sv, Lane &L, int s, Job *J) {
  const size_t N = (size_t)J->g.nx * J->g.ny * J->g.nz;
  const size_t o_rmse = (N * 4 + 15) & ~(size_t)15;
  const size_t o_scal = o_rmse + (size_t)std::max(J->o.maxnumIter, 1) * 8;
  SV_CUDA(sv->pinned.get(o_scal + sizeof(Scalars), J->pin, J->pin_cls));
  J->img = (float *)J->pin;
  J->rmse = (double *)((char *)J->pin + o_rmse);
  J->scal = (Scalars *)((char *)J->pin + o_scal);
  SV_CUDA(cudaEventCreateWithFlags(&J->ev_done, cudaEventDisableTiming));
  // Allocation, upload and start state on the upload stream, which holds no
  // iterations: the pageable copies are staged and return at once instead of
  // waiting behind the lane's queued work.  The lane's stream then waits for
  // them before the slot's descriptor changes.
  SV_CUDA(cudaMallocFromPoolAsync((void **)&J->dev, J->lay.bytes, sv->pool, sv->upload));
  sv->in_use += J->lay.bytes;
  sv->peak = std::max(sv->peak, sv->in_use);
  char *b = J->dev;
  SV_CUDA(cudaMemsetAsync(b, 0, J->lay.bytes, sv->upload));
  Inst I = empty_slot(L, s);
  bind_state(I, b, J->lay);
  if (J->lay.p_fmt == ASDPOCS_STORE_F32)
    SV_CUDA(cudaMemcpyAsync(b + J->lay.P, J->P.data(), J->P.size() * 4,
                            cudaMemcpyHostToDevice, sv->upload));
  else
    SV_CUDA(cudaMemcpyAsync(b + J->lay.P, J->P16.data(), J->P16.size() * 2,
                            cudaMemcpyHostToDevice, sv->upload));
  if (J->has_m0)
    SV_CUDA(cudaMemcpyAsync(b + J->lay.m_k1, J->m0.data(), J->m0.size() * 4,
                            cudaMemcpyHostToDevice, sv->upload));
  if (J->has_ref)
    SV_CUDA(cudaMemcpyAsync(b + J->lay.I0, J->I0.data(), J->I0.size() * 4,
                            cudaMemcpyHostToDevice, sv->upload));
  SV_CUDA(reset_instance(I, initial_scalars(J->o, J->has_ref), sv->upload));
  SV_CUDA(cudaEventRecord(J->ev_done, sv->upload));
  SV_CUDA(cudaStreamWaitEvent(L.st, J->ev_done, 0));
  L.slot_desc[s] = I;
  SV_CUDA(cudaMemcpyAsync(L.d_inst + s, &L.slot_desc[s], sizeof I,
                          cudaMemcpyHostToDevice, L.st));
  std::vector<float>().swap(J->P);
  std::vector<uint16_t>().swap(J->P16);
  std::vector<float>().swap(J->m0);
  std::vector<float>().swap(J->I0);
  J->state = ASDPOCS_JOB_RUNNING;
  J->t_admit = Clock::now();
  J->slot = s;
  L.slot_job[s] = J;
  L.active++;
  return true;
}

bool launch_iteration(asdpocs_server sv, Lane &L) {
  int ng = 0, hw = 0;  // TV steps needed; slots up to the last occupied one
  for (int s = 0; s < L.S; s++)
    if (const Job *J = L.slot_job[s]) {
      ng = std::max(ng, J->o.numOfgradients);
      hw = s + 1;
    }
  if (!L.exec || ng > L.gng || hw > L.gbatch) {
    // capture for the most TV steps and slots seen so far (jobs with fewer
    // steps skip the rest; empty slots exit at once); admission fills the
    // lowest free slot, so the occupied ones stay packed
    ng = std::max(ng, L.gng);
    const int batch = std::min(L.S, std::max((hw + 3) & ~3, L.gbatch));
    if (L.exec) cudaGraphExecDestroy(L.exec);
    if (L.graph) cudaGraphDestroy(L.graph);
    L.exec = nullptr;
    L.graph = nullptr;
    SV_CUDA(cudaStreamBeginCapture(L.st, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e =
        enqueue_iteration(L.d_inst, batch, inst_dims(L.g), L.g.nv, ng, true, L.st);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(L.st, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail(sv, e, "capture of the lane iteration");
    }
    SV_CUDA(e2);
    L.graph = g;
    SV_CUDA(cudaGraphInstantiate(&L.exec, L.graph, 0));
    L.gng = ng;
    L.gbatch = batch;
  }
  Flight f;
  if (!L.spare.empty()) {
    f = std::move(L.spare.back());
    L.spare.pop_back();
  } else {
    SV_CUDA(cudaEventCreateWithFlags(&f.ev, cudaEventDisableTiming));
    SV_CUDA(cudaMallocHost(&f.flags, sizeof(int) * L.S));
  }
  f.owner.assign(L.S, 0);
  for (int s = 0; s < L.S; s++)
    if (L.slot_job[s]) f.owner[s] = L.slot_job[s]->id;
  SV_CUDA(cudaGraphLaunch(L.exec, L.st));
  SV_CUDA(launch_gather_done(L.d_inst, L.S, L.d_flags, L.st));
  SV_CUDA(cudaMemcpyAsync(f.flags, L.d_flags, sizeof(int) * L.S,
                          cudaMemcpyDeviceToHost, L.st));
  SV_CUDA(cudaEventRecord(f.ev, L.st));
  L.inflight.push_back(std::move(f));
  return true;
}

// A cancelled running job leaves slot s: the slot's descriptor is emptied and
// the job's memory freed, both in the order of the lane's stream (after the
// iterations already queued, which may still use it); no results are copied.
bool drop(asdpocs_server sv, Lane &L, int s) {
  Job *J = L.slot_job[s];
  L.slot_desc[s] = empty_slot(L, s);
  SV_CUDA(cudaMemcpyAsync(L.d_inst + s, &L.slot_desc[s], sizeof(Inst),
                          cudaMemcpyHostToDevice, L.st));
  SV_CUDA(cudaFreeAsync(J->dev, L.st));
  J->dev = nullptr;
  sv->in_use -= J->lay.bytes;
  L.slot_job[s] = nullptr;
  L.active--;
  J->state = ASDPOCS_JOB_CANCELLED;
  J->t_done = Clock::now();
  sv->cv_done.notify_all();
  return true;
}

// One pass over a lane; returns false on a CUDA error.  `progress` is set
// when something changed.
bool lane_step(asdpocs_server sv, Lane &L, bool &progress) {
  // finished result copies
  for (size_t i = 0; i < L.harvesting.size();) {
    Job *J = L.harvesting[i];
    const cudaError_t q = cudaEventQuery(J->ev_done);
    if (q == cudaErrorNotReady) {
      i++;
      continue;
    }
    SV_CUDA(q);
    J->state = ASDPOCS_JOB_DONE;
    J->t_done = Clock::now();
    L.harvesting.erase(L.harvesting.begin() + i);
    sv->cv_done.notify_all();
    progress = true;
  }
  // completed iterations: retire the jobs they finished
  while (!L.inflight.empty()) {
    Flight &f = L.inflight.front();
    const cudaError_t q = cudaEventQuery(f.ev);
    if (q == cudaErrorNotReady) break;
    SV_CUDA(q);
    for (int s = 0; s < L.S; s++) {
      // the flag belongs to the job that held the slot when the iteration
      // was queued; act on it only if that job still holds it
      const Job *J = L.slot_job[s];
      if (J && f.owner[s] == J->id && f.flags[s] && J->state == ASDPOCS_JOB_RUNNING)
        if (!harvest(sv, L, s)) return false;
    }
    L.spare.push_back(std::move(f));
    L.inflight.pop_front();
    progress = true;
  }
  // cancelled running jobs
  for (int s = 0; s < L.S; s++)
    if (Job *J = L.slot_job[s])
      if (J->cancel && J->state == ASDPOCS_JOB_RUNNING) {
        if (!drop(sv, L, s)) return false;
        progress = true;
      }
  // admissions (FIFO per lane, within the HBM budget)
  while (!L.queue.empty()) {
    Job *J = L.queue.front();
    int s = 0;
    while (s < L.S && L.slot_job[s]) s++;
    if (s == L.S || sv->in_use + J->lay.bytes > sv->budget) break;
    if (!admit(sv, L, s, J)) return false;
    L.queue.pop_front();
    progress = true;
  }
  while (L.active > 0 && (int)L.inflight.size() < sv->cfg.inflight) {
    if (!launch_iteration(sv, L)) return false;
    progress = true;
  }
  return true;
}

void worker_main(asdpocs_server sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  while (!sv->stop) {
    bool progress = false, ok = true;
    // route new jobs to their lanes
    while (!sv->pending.empty()) {
      Job *J = sv->pending.front();
      sv->pending.pop_front();
      const std::string key = protocol_key(J->g, J->phi);
      auto it = sv->lanes.find(key);
      if (it == sv->lanes.end()) {
        std::unique_ptr<Lane> L(new Lane);
        L->g = J->g;
        L->phi = J->phi;
        if (!lane_create(sv, *L)) {
          ok = false;
          sv->lanes[key] = std::move(L);
          break;
        }
        it = sv->lanes.emplace(key, std::move(L)).first;
      }
      it->second->queue.push_back(J);
      progress = true;
    }
    bool busy = false;
    for (auto &kv : sv->lanes) {
      if (!ok) break;
      ok = lane_step(sv, *kv.second, progress);
      busy = busy || kv.second->active > 0 || !kv.second->harvesting.empty() ||
             !kv.second->inflight.empty();
    }
    if (!ok) {
      for (auto &kv : sv->jobs)
        if (kv.second->state != ASDPOCS_JOB_DONE) kv.second->state = ASDPOCS_JOB_FAILED;
      sv->cv_done.notify_all();
      sv->cv_work.wait(lk, [&] { return sv->stop; });
      break;
    }
    if (!progress) {
      // GPU work outstanding: poll again shortly; idle: sleep until a submit
      if (busy)
        sv->cv_work.wait_for(lk, std::chrono::microseconds(50));
      else
        sv->cv_work.wait(lk, [&] { return sv->stop || !sv->pending.empty(); });
    }
  }
}

void release_job(asdpocs_server sv, Job *J) {
  sv->pinned.put(J->pin, J->pin_cls);
  if (J->ev_done) cudaEventDestroy(J->ev_done);
  J->pin = nullptr;
  J->img = nullptr;
  J->rmse = nullptr;
  J->scal = nullptr;
  J->ev_done = nullptr;
}

}  // namespace
}  // namespace asd

using namespace asd;

extern "C" {

void asdpocs_server_config_default(asdpocs_server_config *c) {
  if (!c) return;
  c->slots_per_lane = 32;
  c->hbm_budget_bytes = 0;
  c->inflight = 2;
}

int asdpocs_server_create(asdpocs_server *out, const asdpocs_server_config *cfg) {
  clear_error();
  if (!out) return set_error(ASDPOCS_ERR_ARG, "null server");
  *out = nullptr;
  asdpocs_server_config c;
  asdpocs_server_config_default(&c);
  if (cfg) c = *cfg;
  if (c.slots_per_lane <= 0 || c.inflight <= 0)
    return set_error(ASDPOCS_ERR_ARG, "slots_per_lane and inflight must be positive");
  int dev = 0;
  ASD_CUDA(cudaGetDevice(&dev));
  size_t free_b = 0, total_b = 0;
  ASD_CUDA(cudaMemGetInfo(&free_b, &total_b));
  asdpocs_server sv = new (std::nothrow) asdpocs_server_s;
  if (!sv) return set_error(ASDPOCS_ERR_NOMEM, "host allocation");
  sv->device = dev;
  sv->cfg = c;
  sv->budget = c.hbm_budget_bytes ? c.hbm_budget_bytes : free_b / 2;
  // a pool of our own that keeps freed blocks for the next admissions
  cudaMemPoolProps props;
  memset(&props, 0, sizeof props);
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaError_t e = cudaMemPoolCreate(&sv->pool, &props);
  if (e == cudaSuccess) {
    unsigned long long keep = sv->budget;
    e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sv->upload, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    delete sv;
    return cuda_status(e, "server setup");
  }
  sv->worker = std::thread(worker_main, sv);
  *out = sv;
  return 0;
}

int asdpocs_server_submit(asdpocs_server sv, const asdpocs_geometry *geom,
                          const double *phi_vec_deg, const asdpocs_options *opt,
                          const float *P, const float *m0, const float *I0,
                          long long *job) {
  clear_error();
  if (!sv || !geom || !phi_vec_deg || !P || !job)
    return set_error(ASDPOCS_ERR_ARG, "null argument");
  std::unique_ptr<Job> J(new (std::nothrow) Job);
  if (!J) return set_error(ASDPOCS_ERR_NOMEM, "host allocation");
  J->g = *geom;
  if (opt)
    J->o = *opt;
  else
    asdpocs_options_default(&J->o);
  if (int e = check_instance(J->g, J->o)) return e;
  if (J->o.ax_mode != ASDPOCS_AX_REFERENCE)
    return set_error(ASDPOCS_ERR_ARG,
                     "the serving queue runs the reference forward mode only; "
                     "run exact-mode jobs in a plan");
  const asdpocs_geometry &g = J->g;
  const size_t N = (size_t)g.nx * g.ny * g.nz;
  J->lay = layout_instance(g, J->o.maxnumIter, 0, kLayoutState, 0, J->o.sino_storage);
  if (J->lay.bytes > sv->budget)
    return set_error(ASDPOCS_ERR_NOMEM,
                     "job needs %zu bytes, over the server's HBM budget of %llu",
                     J->lay.bytes, sv->budget);
  J->phi.assign(phi_vec_deg, phi_vec_deg + g.nv);
  const size_t nP = (size_t)g.na * g.nb * g.nv;
  if (J->o.sino_storage == ASDPOCS_STORE_F32) {
    J->P.assign(P, P + nP);
  } else {  // rounded once here, uploaded at half the bytes
    J->P16.resize(nP);
    store_sinogram_host(P, J->P16.data(), nP, J->o.sino_storage);
  }
  if (m0) {
    J->m0.assign(m0, m0 + N);
    J->has_m0 = true;
  }
  if (I0) {
    J->I0.assign(I0, I0 + N);
    J->has_ref = true;
  }
  J->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(sv->mu);
  if (!sv->error.empty())
    return set_error(ASDPOCS_ERR_CUDA, "server failed: %s", sv->error.c_str());
  J->id = sv->next_id++;
  *job = J->id;
  sv->pending.push_back(J.get());
  sv->jobs[J->id] = std::move(J);
  sv->cv_work.notify_all();
  return 0;
}

int asdpocs_server_poll(asdpocs_server sv, long long job, int *state) {
  clear_error();
  if (!sv || !state) return set_error(ASDPOCS_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->jobs.find(job);
  if (it == sv->jobs.end()) return set_error(ASDPOCS_ERR_ARG, "unknown job %lld", job);
  *state = it->second->state;
  return 0;
}

int asdpocs_server_cancel(asdpocs_server sv, long long job) {
  clear_error();
  if (!sv) return set_error(ASDPOCS_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->jobs.find(job);
  if (it == sv->jobs.end()) return set_error(ASDPOCS_ERR_ARG, "unknown job %lld", job);
  Job *J = it->second.get();
  if (J->state == ASDPOCS_JOB_QUEUED) {
    // still on the server's pending list or in its lane's queue: drop it there
    auto p = std::find(sv->pending.begin(), sv->pending.end(), J);
    if (p != sv->pending.end()) {
      sv->pending.erase(p);
    } else {
      auto L = sv->lanes.find(protocol_key(J->g, J->phi));
      if (L != sv->lanes.end()) {
        auto q = std::find(L->second->queue.begin(), L->second->queue.end(), J);
        if (q != L->second->queue.end()) L->second->queue.erase(q);
      }
    }
    J->state = ASDPOCS_JOB_CANCELLED;
    J->t_done = Clock::now();
    sv->cv_done.notify_all();
    return 0;
  }
  if (J->state == ASDPOCS_JOB_RUNNING) {
    auto L = sv->lanes.find(protocol_key(J->g, J->phi));
    const bool in_slot = L != sv->lanes.end() && J->slot >= 0 &&
                         J->slot < (int)L->second->slot_job.size() &&
                         L->second->slot_job[J->slot] == J;
    if (in_slot) {
      J->cancel = true;  // the worker empties the slot
      sv->cv_work.notify_all();
      return 0;
    }
    return set_error(ASDPOCS_ERR_STATE, "job %lld is already copying out its results", job);
  }
  return set_error(ASDPOCS_ERR_STATE, "job %lld has finished", job);
}

int asdpocs_server_wait(asdpocs_server sv, long long job, float *m_res,
                        asdpocs_stats *st, double *rmse, asdpocs_job_times *t) {
  clear_error();
  if (!sv) return set_error(ASDPOCS_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->jobs.find(job);
  if (it == sv->jobs.end()) return set_error(ASDPOCS_ERR_ARG, "unknown job %lld", job);
  Job *J = it->second.get();
  sv->cv_done.wait(lk, [&] {
    return J->state == ASDPOCS_JOB_DONE || J->state == ASDPOCS_JOB_FAILED ||
           J->state == ASDPOCS_JOB_CANCELLED;
  });
  int rc = 0;
  if (J->state == ASDPOCS_JOB_CANCELLED) {
    rc = set_error(ASDPOCS_ERR_STATE, "job %lld was cancelled", job);
  } else if (J->state == ASDPOCS_JOB_FAILED) {
    rc = set_error(ASDPOCS_ERR_CUDA, "job failed: %s",
                   sv->error.empty() ? "server stopped" : sv->error.c_str());
  } else {
    const size_t N = (size_t)J->g.nx * J->g.ny * J->g.nz;
    if (m_res) memcpy(m_res, J->img, N * 4);
    const Scalars &s = *J->scal;
    if (st) {
      st->IterationNum = s.iterations;
      st->dataTolerance = s.dd2;
      st->alpha = s.alpha;
      st->beta = s.beta;
      st->dp = s.dp;
      st->dg = s.dg;
    }
    if (rmse && J->has_ref && J->o.maxnumIter > 0)
      memcpy(rmse, J->rmse, (size_t)J->o.maxnumIter * 8);
    if (t) {
      t->queued_ms = ms_between(J->t_submit, J->t_admit);
      t->run_ms = ms_between(J->t_admit, J->t_done);
      t->total_ms = ms_between(J->t_submit, J->t_done);
    }
  }
  release_job(sv, J);
  sv->jobs.erase(it);
  return rc;
}

int asdpocs_server_memory(asdpocs_server sv, unsigned long long *in_use,
                          unsigned long long *peak) {
  clear_error();
  if (!sv) return set_error(ASDPOCS_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(sv->mu);
  if (in_use) *in_use = sv->in_use;
  if (peak) *peak = sv->peak;
  return 0;
}

int asdpocs_server_destroy(asdpocs_server sv) {
  if (!sv) return 0;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  cudaSetDevice(sv->device);
  for (auto &kv : sv->jobs)
    if (kv.second->dev) {
      // still admitted: free in the order of its lane's stream
      auto L = sv->lanes.begin();
      for (; L != sv->lanes.end(); ++L)
        if (L->second->slot_job.size() > (size_t)kv.second->slot &&
            kv.second->slot >= 0 && L->second->slot_job[kv.second->slot] == kv.second.get())
          break;
      cudaFreeAsync(kv.second->dev, L != sv->lanes.end() ? L->second->st : 0);
    }
  for (auto &kv : sv->lanes) lane_destroy(*kv.second);
  for (auto &kv : sv->jobs) release_job(sv, kv.second.get());
  cudaDeviceSynchronize();
  sv->pinned.release();
  if (sv->upload) cudaStreamDestroy(sv->upload);
  if (sv->pool) cudaMemPoolDestroy(sv->pool);
  delete sv;
  return 0;
}

}  // extern "C"
