// dvm_server.cu -- request server for independent solves (dvm_server_* in include/dvm_gpu.h).
//
// Continuous batching: queued requests are admitted in arrival order whenever the sum of
// the admitted requests' device footprints stays within the budget and a slot is free;
// every admitted request keeps its f, CDFs and moments resident in its own context on its
// own stream and advances in turns of up to steps_per_turn steps, each turn one launch of a
// CUDA graph captured for that request. The graph is a device-side loop: a conditional
// while node whose body is one step (two where convection swaps f and f_conv) followed by
// a one-thread kernel that reads the step's convergence residual and continues the loop
// only while the residual is above the request's tolerance and the turn has steps left, so
// a request stops on the device at the step that converged. The turns of different
// requests run on different streams, so their kernels overlap on the device. After every
// turn the residual and the device step counter come back by asynchronous copies to pinned
// memory, polled with an event; the request is retired once the residual reaches its
// tolerance or its step limit is reached, its memory going back to the stream-ordered pool. Three host threads share the work so
// that the one issuing turns never waits on the others: a preparer admits requests (context,
// upload, graph capture), the worker polls and issues turns, a retirer downloads results and
// releases contexts. A request's result depends only on its own parameters,
// seed and step count, never on what else is in the mix.
//
// Preemption (dvm_server_set_preemption): a request that has run a given number of turns
// since its admission while another request waits is checkpointed to host memory
// (dvm_checkpoint_save: f, moments, the equilibrium cache and its CDF), its device memory
// and slot are released, and it is queued again behind the waiting requests. Readmitted, it
// continues from the checkpoint with its Philox step counter and collision total restored,
// so its result is that of an uninterrupted run.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/dvm_gpu.h"
#include "dvm_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

int cuda_st(cudaError_t e) {
  if (e == cudaSuccess) return DVM_OK;
  if (e == cudaErrorMemoryAllocation) return DVM_ERR_OOM;
  return DVM_ERR_CUDA;
}

struct Request {
  int64_t id = 0;
  dvm_params p{};
  std::vector<double> x, y, z, f0;
  int max_steps = 0;
  double tol = 0.0;
  size_t bytes = 0;
  Clock::time_point t_submit, t_admit, t_done;
  // while admitted
  dvm_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t* d_step = nullptr;
  long long* d_acc = nullptr;
  int* d_left = nullptr;    // steps the current turn may still take (the graph's loop)
  cudaGraphExec_t exec = nullptr;
  int quantum = 0;
  int body = 1;             // steps per pass of the graph's loop
  cudaEvent_t ev = nullptr;
  int slot = -1;
  bool inflight = false;
  int steps_done = 0;
  bool eager_tail = false;  // an odd last step was issued outside the graph
  int turns = 0;            // turns completed since the last admission
  // preemption
  int preempted = 0;                // times checkpointed and requeued
  bool parked = false;              // checkpointed, waiting to be readmitted
  std::vector<unsigned char> ckpt;  // the checkpoint while parked
  long long collisions_before = 0;  // collision total at the checkpoint
  // result
  int status = DVM_OK;
  int converged = 0;
  double residual = 0.0;
  long long collisions = 0;
  uint64_t device_bytes = 0;
  std::vector<double> props, f;
  bool done = false;
  bool handed = false;  // the worker gave it to the retirer

  dvm_vgrid vgrid() const {
    dvm_vgrid v;
    v.nx = static_cast<int32_t>(x.size());
    v.ny = static_cast<int32_t>(y.size());
    v.nz = static_cast<int32_t>(z.size());
    v.x = x.data();
    v.y = y.data();
    v.z = z.data();
    return v;
  }
  size_t ncells() const { return static_cast<size_t>(p.nx_space) * p.ny_space; }
  size_t nv() const { return x.size() * y.size() * z.size(); }
};

}  // namespace

struct dvm_server {
  uint64_t budget = 0;
  int max_active = 1;
  int quantum = 2;
  int device = 0;
  std::atomic<int> preempt_turns{0};  // 0: no preemption
  std::mutex mu;  // guards everything below but `active`
  std::condition_variable cv_work, cv_done, cv_prep, cv_retire;
  std::deque<std::shared_ptr<Request>> pending;   // submitted (or preempted), not admitted
  std::deque<std::shared_ptr<Request>> ready;     // admitted and prepared, for the worker
  std::deque<std::shared_ptr<Request>> finished;  // for the retirer
  std::map<int64_t, std::shared_ptr<Request>> all;
  std::vector<std::shared_ptr<Request>> active;   // worker thread only
  int64_t next_id = 1;
  bool stop = false;
  int live = 0;               // requests holding a slot (admission to retirement or parking)
  std::thread worker, preparer, retirer;
  double* h_slots = nullptr;  // pinned, one residual per slot
  uint32_t* h_steps = nullptr;  // pinned, the device step counter per slot
  int* h_left = nullptr;        // pinned, the turn length per slot (copied to d_left)
  std::vector<int> free_slots;
  uint64_t used = 0;
  // every thread ends once destruction was asked for and no request is left
  bool drained() const { return stop && pending.empty() && live == 0; }
  // statistics
  int64_t completed = 0;
  int peak_active = 0;
  uint64_t peak_bytes = 0;
};

namespace {

// One request step outside any graph: collision, convection, moments, step counter.
int eager_step(Request& r) {
  int st = dvm_compute_collision_integral(r.ctx, 0, nullptr);
  if (!st) st = dvm_compute_convection(r.ctx);
  if (!st) st = dvm_calculate_physical_properties(r.ctx);
  if (!st)
    st = cuda_st(dvm::launch_step_end(r.d_step, r.d_acc, dvm::ctx_total_samples(r.ctx),
                                      r.stream));
  return st;
}

// The loop's test after each pass: the turn's remaining steps go down by the pass, and the
// loop goes on while a whole pass still fits and the residual of the last step is above
// the tolerance (a NaN residual stops it too).
__global__ void k_turn_check(cudaGraphConditionalHandle h, const unsigned long long* residual,
                             double tol, int* left, int body) {
  const int l = *left - body;
  *left = l;
  const double res = __longlong_as_double(static_cast<long long>(*residual));
  cudaGraphSetConditional(h, (l >= body && res > tol) ? 1u : 0u);
}

// A turn as one graph: a conditional while node (its handle set to 1 at every launch)
// whose body, captured from the request's own stream, is r.body steps and the check.
int capture_turn(Request& r) {
  cudaGraph_t graph = nullptr;
  int st = cuda_st(cudaGraphCreate(&graph, 0));
  if (st) return st;
  cudaGraphConditionalHandle h;
  st = cuda_st(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (!st) st = cuda_st(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np));
  if (!st) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    st = cuda_st(cudaStreamBeginCaptureToGraph(r.stream, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeRelaxed));
    if (!st) {
      for (int s = 0; s < r.body && !st; ++s) st = eager_step(r);
      if (!st) {
        k_turn_check<<<1, 1, 0, r.stream>>>(h, dvm::ctx_residual(r.ctx), r.tol, r.d_left, r.body);
        st = cuda_st(cudaGetLastError());
      }
      cudaGraph_t out = nullptr;
      const int st2 = cuda_st(cudaStreamEndCapture(r.stream, &out));
      if (!st) st = st2;
    }
  }
  if (!st) st = cuda_st(cudaGraphInstantiate(&r.exec, graph, 0));
  cudaGraphDestroy(graph);
  return st;
}

int admit(dvm_server* sv, Request& r) {
  dvm_vgrid vg = r.vgrid();
  int st = dvm::ctx_create(&r.p, &vg, true, &r.ctx);
  if (st) return st;
  r.stream = dvm::ctx_stream(r.ctx);
  r.device_bytes = dvm::ctx_device_bytes(r.ctx);
  st = cuda_st(cudaMallocAsync(reinterpret_cast<void**>(&r.d_step), sizeof(uint32_t), r.stream));
  if (!st)
    st = cuda_st(cudaMallocAsync(reinterpret_cast<void**>(&r.d_acc), sizeof(long long), r.stream));
  if (!st)
    st = cuda_st(cudaMallocAsync(reinterpret_cast<void**>(&r.d_left), sizeof(int), r.stream));
  if (st) return st;
  cudaMemsetAsync(r.d_step, 0, sizeof(uint32_t), r.stream);
  cudaMemsetAsync(r.d_acc, 0, sizeof(long long), r.stream);
  dvm::ctx_set_step_dev(r.ctx, r.d_step);
  if (r.parked) {
    // resume: the checkpointed state, the step counter and the collision total
    uint64_t ntime = 0;
    st = dvm_checkpoint_load(r.ctx, r.ckpt.data(), r.ckpt.size(), &ntime);
    if (!st && ntime != static_cast<uint64_t>(r.steps_done)) st = DVM_ERR_PARAM;
    const uint32_t step = static_cast<uint32_t>(r.steps_done);
    if (!st)
      st = cuda_st(cudaMemcpyAsync(r.d_step, &step, sizeof(step), cudaMemcpyHostToDevice,
                                   r.stream));
    if (!st)
      st = cuda_st(cudaMemcpyAsync(r.d_acc, &r.collisions_before, sizeof(long long),
                                   cudaMemcpyHostToDevice, r.stream));
    if (!st) st = cuda_st(cudaStreamSynchronize(r.stream));
    if (st) return st;
    std::vector<unsigned char>().swap(r.ckpt);
    r.parked = false;
  } else {
    st = dvm_upload_f(r.ctx, r.f0.data());  // also computes the initial moments
    if (st) return st;
    std::vector<double>().swap(r.f0);
  }
  r.turns = 0;
  // two steps per pass of the loop when convection swaps f and f_conv (the graph then
  // leaves them where it found them); a turn is a whole number of passes
  r.body = (r.p.conv_method != DVM_CONV_NONE) ? 2 : 1;
  r.quantum = std::max(r.body, sv->quantum - sv->quantum % r.body);
  if (r.max_steps - r.steps_done < r.body) r.quantum = 0;  // eager steps only
  if (r.quantum > 0) st = capture_turn(r);
  if (!st) st = cuda_st(cudaEventCreateWithFlags(&r.ev, cudaEventDisableTiming));
  return st;
}

// Issues the next turn of a request: one launch of its graph (up to a turn's whole passes,
// fewer if the residual reaches the tolerance on the way), or a single eager step for a
// tail shorter than a pass (after which the graph is not launched again).
int issue(dvm_server* sv, Request& r) {
  const int left = r.max_steps - r.steps_done;
  int st = DVM_OK;
  if (r.quantum > 0 && !r.eager_tail && left >= r.body) {
    sv->h_left[r.slot] = std::min(r.quantum, left - left % r.body);
    st = cuda_st(cudaMemcpyAsync(r.d_left, sv->h_left + r.slot, sizeof(int),
                                 cudaMemcpyHostToDevice, r.stream));
    if (!st) st = cuda_st(cudaGraphLaunch(r.exec, r.stream));
  } else {
    r.eager_tail = true;
    st = eager_step(r);
  }
  if (!st)
    st = cuda_st(cudaMemcpyAsync(sv->h_slots + r.slot, dvm::ctx_residual(r.ctx), sizeof(double),
                                 cudaMemcpyDeviceToHost, r.stream));
  if (!st)
    st = cuda_st(cudaMemcpyAsync(sv->h_steps + r.slot, r.d_step, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, r.stream));
  if (!st) st = cuda_st(cudaEventRecord(r.ev, r.stream));
  if (!st) r.inflight = true;
  return st;
}

// Releases a request's graph, event, counters and context (after its stream is drained).
void release_device(Request& r) {
  cudaStreamSynchronize(r.stream);
  if (r.exec) cudaGraphExecDestroy(r.exec);
  if (r.ev) cudaEventDestroy(r.ev);
  if (r.d_step) cudaFreeAsync(r.d_step, r.stream);
  if (r.d_acc) cudaFreeAsync(r.d_acc, r.stream);
  if (r.d_left) cudaFreeAsync(r.d_left, r.stream);
  dvm::ctx_destroy(r.ctx);
  r.exec = nullptr;
  r.ev = nullptr;
  r.d_step = nullptr;
  r.d_acc = nullptr;
  r.d_left = nullptr;
  r.ctx = nullptr;
}

// Checkpoints an admitted request between turns and queues it again behind the waiting
// requests; returns nonzero (and leaves the request admitted) if the checkpoint fails.
int preempt(dvm_server* sv, Request& r) {
  uint64_t bytes = 0;
  int st = dvm_checkpoint_size(r.ctx, &bytes);
  if (st) return st;
  std::vector<unsigned char> buf(bytes);
  st = dvm_checkpoint_save(r.ctx, static_cast<uint64_t>(r.steps_done), buf.data(), bytes);
  long long acc = 0;
  if (!st)
    st = cuda_st(cudaMemcpyAsync(&acc, r.d_acc, sizeof(acc), cudaMemcpyDeviceToHost, r.stream));
  if (!st) st = cuda_st(cudaStreamSynchronize(r.stream));
  if (st) return st;
  release_device(r);
  r.ckpt.swap(buf);
  r.collisions_before = acc;
  r.parked = true;
  r.preempted++;
  r.eager_tail = false;
  r.quantum = 0;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (r.slot >= 0) sv->free_slots.push_back(r.slot);
    r.slot = -1;
    sv->used -= r.bytes;
    sv->live--;
    sv->pending.push_back(sv->all.at(r.id));
  }
  sv->cv_prep.notify_one();
  return DVM_OK;
}

// The retirer's part: results to the host, the context released, the slot given back.
void retire(dvm_server* sv, Request& r) {
  if (r.ctx) {
    if (r.status == DVM_OK) {
      r.props.resize(r.ncells() * DVM_NPROP);
      r.f.resize(r.ncells() * r.nv());
      int st = dvm_get_properties(r.ctx, r.props.data());
      if (!st) st = dvm_download_f(r.ctx, r.f.data());
      uint32_t err = 0;
      if (!st) st = dvm_get_error_word(r.ctx, &err);
      if (!st && err) st = DVM_ERR_NUMERIC;
      if (!st)
        st = cuda_st(cudaMemcpyAsync(&r.collisions, r.d_acc, sizeof(long long),
                                     cudaMemcpyDeviceToHost, r.stream));
      r.status = st;
    }
    release_device(r);
  }
  r.t_done = Clock::now();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (r.slot >= 0) sv->free_slots.push_back(r.slot);
    r.slot = -1;
    sv->used -= r.bytes;
    sv->live--;
    r.done = true;
    sv->completed++;
  }
  sv->cv_done.notify_all();
  sv->cv_prep.notify_one();
  sv->cv_work.notify_one();
  sv->cv_retire.notify_one();
}

// Hands a request that ended (or failed) to the retirer.
void finish(dvm_server* sv, const std::shared_ptr<Request>& r) {
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->finished.push_back(r);
  }
  sv->cv_retire.notify_one();
}

void preparer_loop(dvm_server* sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  for (;;) {
    sv->cv_prep.wait(lk, [&] {
      return sv->drained() ||
             (!sv->pending.empty() && !sv->free_slots.empty() &&
              sv->used + sv->pending.front()->bytes <= sv->budget);
    });
    if (sv->pending.empty()) {
      if (sv->drained()) break;
      continue;
    }
    std::shared_ptr<Request> r = sv->pending.front();
    sv->pending.pop_front();
    r->slot = sv->free_slots.back();
    sv->free_slots.pop_back();
    sv->used += r->bytes;
    sv->live++;
    sv->peak_active = std::max(sv->peak_active, sv->live);
    sv->peak_bytes = std::max(sv->peak_bytes, sv->used);
    lk.unlock();
    if (!r->parked) r->t_admit = Clock::now();  // the first admission
    r->status = admit(sv, *r);
    lk.lock();
    if (r->status) {
      sv->finished.push_back(r);
      sv->cv_retire.notify_one();
    } else {
      sv->ready.push_back(r);
      sv->cv_work.notify_one();
    }
  }
  lk.unlock();
  sv->cv_work.notify_all();
  sv->cv_retire.notify_all();
}

void retirer_loop(dvm_server* sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  for (;;) {
    sv->cv_retire.wait(lk, [&] { return !sv->finished.empty() || sv->drained(); });
    if (sv->finished.empty()) break;
    std::shared_ptr<Request> r = sv->finished.front();
    sv->finished.pop_front();
    lk.unlock();
    retire(sv, *r);
    lk.lock();
  }
  lk.unlock();
  sv->cv_work.notify_all();
  sv->cv_prep.notify_all();
}

void worker_loop(dvm_server* sv) {
  cudaSetDevice(sv->device);
  for (;;) {
    // take the prepared requests; with none running, wait for one (or for the end)
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      if (sv->active.empty())
        sv->cv_work.wait(lk, [&] { return !sv->ready.empty() || sv->drained(); });
      while (!sv->ready.empty()) {
        sv->active.push_back(sv->ready.front());
        sv->ready.pop_front();
      }
      if (sv->active.empty() && sv->drained()) break;
    }
    bool progress = false;
    for (auto& rp : sv->active) {
      Request& r = *rp;
      if (r.inflight) {
        const cudaError_t q = cudaEventQuery(r.ev);
        if (q == cudaErrorNotReady) continue;
        r.inflight = false;
        progress = true;
        if (q != cudaSuccess) {
          r.status = DVM_ERR_CUDA;
        } else {
          r.steps_done = static_cast<int>(sv->h_steps[r.slot]);
          r.residual = sv->h_slots[r.slot];
          if (r.residual <= r.tol) r.converged = 1;
        }
        if (r.status || r.converged || r.steps_done >= r.max_steps) {
          r.handed = true;
          finish(sv, rp);
          continue;
        }
        // preemption between turns, while another request waits
        const int pt = sv->preempt_turns.load();
        if (pt > 0 && ++r.turns >= pt && !r.eager_tail) {
          bool waiting;
          {
            std::lock_guard<std::mutex> lk(sv->mu);
            waiting = !sv->pending.empty();
          }
          if (waiting && preempt(sv, r) == DVM_OK) continue;
        }
      }
      if (!r.handed && !r.parked && !r.inflight) {
        r.status = issue(sv, r);
        if (r.status) {
          r.handed = true;
          finish(sv, rp);
        }
        progress = true;
      }
    }
    sv->active.erase(std::remove_if(sv->active.begin(), sv->active.end(),
                                    [](const std::shared_ptr<Request>& r) {
                                      return r->handed || r->parked;
                                    }),
                     sv->active.end());
    if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  sv->cv_prep.notify_all();
  sv->cv_retire.notify_all();
}

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

extern "C" {

int dvm_server_create(uint64_t hbm_budget_bytes, int max_active, int steps_per_turn,
                      dvm_server** out) {
  if (!out || hbm_budget_bytes == 0 || max_active < 1 || steps_per_turn < 1)
    return DVM_ERR_PARAM;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return DVM_ERR_NODEVICE;
  dvm_server* sv = new (std::nothrow) dvm_server();
  if (!sv) return DVM_ERR_OOM;
  sv->budget = hbm_budget_bytes;
  sv->max_active = max_active;
  sv->quantum = steps_per_turn;
  cudaGetDevice(&sv->device);
  if (cudaHostAlloc(reinterpret_cast<void**>(&sv->h_slots), sizeof(double) * max_active,
                    cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc(reinterpret_cast<void**>(&sv->h_steps), sizeof(uint32_t) * max_active,
                    cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc(reinterpret_cast<void**>(&sv->h_left), sizeof(int) * max_active,
                    cudaHostAllocDefault) != cudaSuccess) {
    if (sv->h_slots) cudaFreeHost(sv->h_slots);
    if (sv->h_steps) cudaFreeHost(sv->h_steps);
    delete sv;
    return DVM_ERR_OOM;
  }
  for (int i = max_active - 1; i >= 0; --i) sv->free_slots.push_back(i);
  // freed request memory stays in this process's stream-ordered pool for the next request
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, sv->device) == cudaSuccess) {
    uint64_t keep = hbm_budget_bytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  sv->worker = std::thread(worker_loop, sv);
  sv->preparer = std::thread(preparer_loop, sv);
  sv->retirer = std::thread(retirer_loop, sv);
  *out = sv;
  return DVM_OK;
}

int dvm_server_destroy(dvm_server* sv) {
  if (!sv) return DVM_ERR_PARAM;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  sv->cv_prep.notify_all();
  sv->cv_retire.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  if (sv->preparer.joinable()) sv->preparer.join();
  if (sv->retirer.joinable()) sv->retirer.join();
  cudaFreeHost(sv->h_slots);
  cudaFreeHost(sv->h_steps);
  cudaFreeHost(sv->h_left);
  delete sv;
  return DVM_OK;
}

int dvm_server_submit(dvm_server* sv, const dvm_params* params, const dvm_vgrid* vgrid,
                      const double* f0, int32_t max_steps, double residual_tol, int64_t* id) {
  if (!sv || !params || !vgrid || !f0 || !id || max_steps < 1) return DVM_ERR_PARAM;
  uint64_t bytes = 0;
  int st = dvm_footprint_bytes(params, vgrid, &bytes);
  if (st) return st;
  bytes += sizeof(uint32_t) + sizeof(long long);
  if (bytes > sv->budget) return DVM_ERR_TOO_LARGE;
  auto r = std::make_shared<Request>();
  r->t_submit = Clock::now();
  r->p = *params;
  r->x.assign(vgrid->x, vgrid->x + vgrid->nx);
  r->y.assign(vgrid->y, vgrid->y + vgrid->ny);
  r->z.assign(vgrid->z, vgrid->z + vgrid->nz);
  r->f0.assign(f0, f0 + r->ncells() * r->nv());
  r->max_steps = max_steps;
  r->tol = residual_tol;
  r->bytes = bytes;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) return DVM_ERR_PARAM;
    r->id = sv->next_id++;
    sv->all[r->id] = r;
    sv->pending.push_back(r);
  }
  sv->cv_prep.notify_one();
  *id = r->id;
  return DVM_OK;
}

int dvm_server_wait(dvm_server* sv, int64_t id, dvm_request_info* info) {
  if (!sv || !info) return DVM_ERR_PARAM;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return DVM_ERR_PARAM;
  std::shared_ptr<Request> r = it->second;
  sv->cv_done.wait(lk, [&] { return r->done; });
  std::memset(info, 0, sizeof(*info));
  info->status = r->status;
  info->converged = r->converged;
  info->steps = r->steps_done;
  info->residual = r->residual;
  info->queue_ms = ms_between(r->t_submit, r->t_admit);
  info->latency_ms = ms_between(r->t_submit, r->t_done);
  info->collisions = r->collisions;
  info->device_bytes = r->device_bytes;
  info->preempted = r->preempted;
  return DVM_OK;
}

int dvm_server_set_preemption(dvm_server* sv, int32_t turns) {
  if (!sv || turns < 0) return DVM_ERR_PARAM;
  sv->preempt_turns.store(turns);
  return DVM_OK;
}

int dvm_server_result(dvm_server* sv, int64_t id, double* props, double* f) {
  if (!sv) return DVM_ERR_PARAM;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->all.find(id);
  if (it == sv->all.end() || !it->second->done) return DVM_ERR_PARAM;
  Request& r = *it->second;
  if (r.status) return r.status;
  if (props) std::memcpy(props, r.props.data(), r.props.size() * sizeof(double));
  if (f) std::memcpy(f, r.f.data(), r.f.size() * sizeof(double));
  sv->all.erase(it);
  return DVM_OK;
}

int dvm_server_stats(dvm_server* sv, int64_t* completed, int32_t* peak_active,
                     uint64_t* peak_bytes) {
  if (!sv) return DVM_ERR_PARAM;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (completed) *completed = sv->completed;
  if (peak_active) *peak_active = sv->peak_active;
  if (peak_bytes) *peak_bytes = sv->peak_bytes;
  return DVM_OK;
}

}  // extern "C"
