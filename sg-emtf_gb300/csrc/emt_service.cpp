// emt_service.cpp -- service mode: batches of tasks that arrive over time,
// served concurrently on one GPU, over the library's public ABI.
//
// The reference's host scheduler (proposed model/SG-EMTF.cu:1836-1958)
// splits T tasks into BATCH_NUM batches at random points, lets each batch
// arrive after a random gap (0-100 ms), starts one host thread per task when
// its batch arrives (iter(), :1646), and reports the average response time
// (thread start - arrival), solve time (finish - arrival) and memory use
// (/proc/meminfo, :1757-1788).  Here a batch is one engine handle with its
// own non-blocking CUDA stream; a round launches the next epoch of every
// running batch whose previous epoch has completed (an event per batch, no
// host thread per task and no blocking wait), so the batches' epoch kernels
// overlap on the device.  Memory is the device's, from cudaMemGetInfo.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sgemtf.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Batch {
  std::vector<emt_task_desc> desc;
  std::vector<std::vector<double>> rot;  // deep copies of the caller's arrays
  std::vector<std::vector<float>> diag, shift;
  double arrival = 0.0, admit = -1.0, done = -1.0;
  int state = 0;  // 0 waiting, 1 running, 2 done, 3 failed
  int gens = 0;       // generations launched
  int completed = 0;  // generations seen complete
  bool inflight = false;
  emt_handle_t* h = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  std::vector<float> best;
  uint64_t evals = 0;
};

}  // namespace

struct emt_service {
  emt_config cfg{};
  int32_t generations = 0, epoch = 1;
  Clock::time_point t0;
  std::vector<Batch> batches;
  std::string err;
  double mem_max = 0.0, mem_sum = 0.0;
  int rounds = 0;

  double now() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(EMT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
};

namespace {

void release(Batch& b) {
  if (b.h) emt_destroy(b.h);
  if (b.ev) cudaEventDestroy(b.ev);
  if (b.stream) cudaStreamDestroy(b.stream);
  b.h = nullptr;
  b.ev = nullptr;
  b.stream = nullptr;
}

// A batch whose admission or launch failed: its handle, stream and event
// are released and it is not tried again; the failing call returns rc with
// the reason in the service's last error.
int give_up(emt_service* s, Batch& b, int id, int rc, const std::string& why) {
  const std::string m = "batch " + std::to_string(id) + ": " + why;
  if (b.stream) cudaStreamSynchronize(b.stream);
  release(b);
  b.inflight = false;
  b.state = 3;
  return s->fail(rc, m);
}

int admit(emt_service* s, Batch& b, int id) {
  emt_config c = s->cfg;
  c.seed = s->cfg.seed + (uint64_t)id;
  int rc = emt_create(&c, &b.h);
  if (rc) return give_up(s, b, id, rc, "emt_create failed");
  for (size_t t = 0; t < b.desc.size(); ++t) {  // point the copies at this batch's arrays
    b.desc[t].rotation_matrix = b.rot[t].empty() ? nullptr : b.rot[t].data();
    b.desc[t].diag = b.diag[t].empty() ? nullptr : b.diag[t].data();
    b.desc[t].shift = b.shift[t].empty() ? nullptr : b.shift[t].data();
  }
  if ((rc = emt_add_tasks(b.h, (int32_t)b.desc.size(), b.desc.data())))
    return give_up(s, b, id, rc, emt_last_error(b.h));
  cudaError_t e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming);
  if (e != cudaSuccess)
    return give_up(s, b, id, EMT_ERR_CUDA, std::string("batch stream: ") + cudaGetErrorString(e));
  if ((rc = emt_reset(b.h, b.stream))) return give_up(s, b, id, rc, emt_last_error(b.h));
  b.admit = s->now();
  b.state = 1;
  return EMT_OK;
}

// Launches the next epoch of a running batch whose previous one completed;
// retires it when its budget is done.  *launched is set when an epoch was
// queued.
int advance(emt_service* s, Batch& b, int id, bool* launched) {
  if (b.inflight) {
    const cudaError_t q = cudaEventQuery(b.ev);
    if (q == cudaErrorNotReady) return EMT_OK;
    if (q != cudaSuccess)
      return give_up(s, b, id, EMT_ERR_CUDA, std::string("batch epoch: ") + cudaGetErrorString(q));
    b.inflight = false;
    b.completed = b.gens;
  }
  int rc;
  if (b.gens < s->generations) {
    const int g = std::min(s->epoch, s->generations - b.gens);
    if ((rc = emt_run(b.h, g, b.stream))) return give_up(s, b, id, rc, emt_last_error(b.h));
    const cudaError_t e = cudaEventRecord(b.ev, b.stream);
    if (e != cudaSuccess)
      return give_up(s, b, id, EMT_ERR_CUDA, std::string("batch event: ") + cudaGetErrorString(e));
    b.gens += g;
    b.inflight = true;
    *launched = true;
    return EMT_OK;
  }
  b.best.resize(b.desc.size());
  if ((rc = emt_get_best_all(b.h, b.best.data()))) return give_up(s, b, id, rc, emt_last_error(b.h));
  emt_stats st;
  if ((rc = emt_get_stats(b.h, &st))) return give_up(s, b, id, rc, emt_last_error(b.h));
  b.evals = st.evaluations;
  b.done = s->now();
  b.state = 2;
  release(b);
  return EMT_OK;
}

}  // namespace

extern "C" {

EMT_API int emt_service_create(const emt_config* cfg, int32_t generations, int32_t epoch,
                               emt_service_t** out) {
  if (!cfg || !out || generations < 0 || epoch < 1) return EMT_ERR_INVALID_ARG;
  *out = nullptr;
  // the configuration is checked the way a batch's handle will check it
  emt_handle_t* probe = nullptr;
  const int rc = emt_create(cfg, &probe);
  if (rc) return rc;
  emt_destroy(probe);
  emt_service* s = new (std::nothrow) emt_service();
  if (!s) return EMT_ERR_OUT_OF_MEMORY;
  s->cfg = *cfg;
  s->generations = generations;
  s->epoch = epoch;
  s->t0 = Clock::now();
  *out = s;
  return EMT_OK;
}

EMT_API int emt_service_submit(emt_service_t* s, int32_t n, const emt_task_desc* tasks,
                               double arrival_ms, int32_t* batch) {
  if (!s) return EMT_ERR_INVALID_ARG;
  if (n < 1 || !tasks || !std::isfinite(arrival_ms))
    return s->fail(EMT_ERR_INVALID_ARG, "a batch needs tasks and a finite arrival time");
  for (int t = 0; t < n; ++t)
    if (tasks[t].dim < 1 || tasks[t].dim > EMT_MAX_FUSED_DIM)
      return s->fail(EMT_ERR_INVALID_ARG, "task " + std::to_string(t) +
                                              ": the service serves islands of D <= 128");
  try {  // the batch keeps copies of the caller's arrays
    Batch b;
    b.arrival = arrival_ms;
    b.desc.assign(tasks, tasks + n);
    b.rot.resize(n);
    b.diag.resize(n);
    b.shift.resize(n);
    for (int t = 0; t < n; ++t) {
      const emt_task_desc& d = tasks[t];
      const size_t D = (size_t)d.dim;
      if (d.rotation_matrix) b.rot[t].assign(d.rotation_matrix, d.rotation_matrix + D * D);
      if (d.diag) b.diag[t].assign(d.diag, d.diag + D);
      if (d.shift) b.shift[t].assign(d.shift, d.shift + D);
    }
    s->batches.push_back(std::move(b));
  } catch (const std::bad_alloc&) {
    return s->fail(EMT_ERR_OUT_OF_MEMORY, "host memory for the batch");
  }
  if (batch) *batch = (int32_t)s->batches.size() - 1;
  return EMT_OK;
}

EMT_API int emt_service_step(emt_service_t* s, int32_t* active) {
  if (!s) return EMT_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(s->cfg.device);
  if (e != cudaSuccess) return s->cuda_fail(e, "cudaSetDevice");
  const double t = s->now();
  int rc, left = 0;
  for (size_t i = 0; i < s->batches.size(); ++i) {
    Batch& b = s->batches[i];
    if (b.state == 0 && b.arrival <= t && (rc = admit(s, b, (int)i))) return rc;
    if (b.state == 1) {
      bool launched = false;
      if ((rc = advance(s, b, (int)i, &launched))) return rc;
    }
    left += b.state == 0 || b.state == 1;
  }
  size_t fr = 0, tot = 0;
  if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess) return s->cuda_fail(e, "cudaMemGetInfo");
  const double used = (double)(tot - fr) / (1024.0 * 1024.0);
  s->mem_max = std::max(s->mem_max, used);
  s->mem_sum += used;
  ++s->rounds;
  if (active) *active = left;
  return EMT_OK;
}

EMT_API int emt_service_drain(emt_service_t* s) {
  if (!s) return EMT_ERR_INVALID_ARG;
  for (;;) {
    int32_t left = 0;
    const int rc = emt_service_step(s, &left);
    if (rc) return rc;
    if (!left) return EMT_OK;
    bool running = false, waiting_launch = true;
    double next = INFINITY;
    for (const Batch& b : s->batches) {
      if (b.state == 1) {
        running = true;
        if (!b.inflight) waiting_launch = false;
      }
      if (b.state == 0) next = std::min(next, b.arrival);
    }
    if (!running && std::isfinite(next)) {  // idle until the next batch arrives
      const double wait = next - s->now();
      if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(wait));
    } else if (running && waiting_launch) {  // every running batch is busy on the device
      std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
  }
}

EMT_API int emt_service_batch(emt_service_t* s, int32_t batch, emt_service_batch_info* info,
                              float* best) {
  if (!s) return EMT_ERR_INVALID_ARG;
  if (batch < 0 || batch >= (int32_t)s->batches.size())
    return s->fail(EMT_ERR_INVALID_ARG, "no such batch");
  const Batch& b = s->batches[batch];
  if (info) {
    info->n_tasks = (int32_t)b.desc.size();
    info->state = b.state;
    info->generations = b.completed;
    info->reserved = 0;
    info->arrival_ms = b.arrival;
    info->admit_ms = b.admit;
    info->done_ms = b.done;
  }
  if (best) {
    if (b.state == 3) return s->fail(EMT_ERR_STATE, "the batch failed");
    if (b.state != 2) return s->fail(EMT_ERR_STATE, "the batch has not finished");
    std::copy(b.best.begin(), b.best.end(), best);
  }
  return EMT_OK;
}

EMT_API int emt_service_get_stats(emt_service_t* s, emt_service_stats* out) {
  if (!s || !out) return EMT_ERR_INVALID_ARG;
  *out = emt_service_stats{};
  out->batches_submitted = (int32_t)s->batches.size();
  double rs = 0.0, sl = 0.0;
  for (const Batch& b : s->batches) {
    if (b.state != 2) continue;
    const double n = (double)b.desc.size();
    ++out->batches_done;
    out->tasks_done += (int64_t)b.desc.size();
    rs += n * (b.admit - b.arrival);
    sl += n * (b.done - b.arrival);
    out->evaluations += b.evals;
  }
  if (out->tasks_done) {
    out->mean_response_ms = rs / (double)out->tasks_done;
    out->mean_solve_ms = sl / (double)out->tasks_done;
  }
  out->max_device_mem_mb = s->mem_max;
  out->mean_device_mem_mb = s->rounds ? s->mem_sum / s->rounds : 0.0;
  out->rounds = s->rounds;
  return EMT_OK;
}

EMT_API const char* emt_service_last_error(const emt_service_t* s) {
  return s ? s->err.c_str() : "null service";
}

EMT_API void emt_service_destroy(emt_service_t* s) {
  if (!s) return;
  for (Batch& b : s->batches) {
    if (b.stream) cudaStreamSynchronize(b.stream);
    release(b);
  }
  delete s;
}

}  // extern "C"
