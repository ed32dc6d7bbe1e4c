// pf_batch.cu -- continuous batching of independent jobs on one GPU.
//
// Each admitted job keeps its own device state.  A batch step is one CUDA
// graph over all live jobs (fused): each kernel of the coupled step runs once
// for the whole batch, over the CTAs of every job, a table of per-job CTA
// offsets (start[kernel][job]) and a table of per-job handles (BatchDesc)
// telling each CTA its job.  The graph is rebuilt when jobs join (admit),
// leave (retire) or detach.  A batch whose jobs cannot share the fused
// kernels (FP64, platelet boxes, cell-list Morse, mixed precision, or
// PFGPU_BATCH_FUSED=0) falls back to replaying every job's own step graph on
// its own streams.  Admission is against a device-memory budget using the
// job's exact allocation size.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "pf_internal.h"

using namespace pf;

extern "C" int pfgpu_job_enqueue(pfgpu_job* j, int nsteps);
extern "C" int pfgpu_job_batch_desc_(pfgpu_job* j, BatchDesc* d, int* precision, int* fast);

struct pfgpu_batch {
  size_t budget = 0, in_use = 0;
  struct Slot {
    pfgpu_job* job = nullptr;
    size_t bytes = 0;
    int status = PFGPU_OK;  // last step status (PFGPU_DONE: detached)
  };
  std::vector<Slot> slots;
  std::mutex mu;
  // fused step: plan over the live jobs (valid until the slots change)
  struct Fused {
    bool valid = false, usable = false;
    int precision = PF_PREC_FP32;
    bool fast = true;
    std::vector<int> order;  // slots in the plan
    BatchDesc* d_desc = nullptr;
    int* d_start = nullptr;  // [BK_COUNT][jobs + 1]
    int total[BK_COUNT] = {};
    size_t smem[BK_COUNT] = {};
    cudaStream_t st[5] = {};  // s0 (critical path), s1-s3 (forces), sL (lattice, low priority)
    cudaEvent_t ev[6] = {};
    cudaGraphExec_t graph = nullptr;
  } fused;
};

namespace {

void fused_release(pfgpu_batch::Fused& f) {
  if (f.graph) cudaGraphExecDestroy(f.graph);
  if (f.d_desc) cudaFree(f.d_desc);
  if (f.d_start) cudaFree(f.d_start);
  f.graph = nullptr;
  f.d_desc = nullptr;
  f.d_start = nullptr;
  f.valid = false;
  f.usable = false;
  f.order.clear();
}

#define BK_CK(call)                                                                      \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e_));  \
  } while (0)

// one fused coupled step of every job in the plan (the schedule of a single
// job's step, each kernel over the whole batch)
int fused_enqueue(pfgpu_batch::Fused& f) {
  cudaStream_t s0 = f.st[0], s1 = f.st[1], s2 = f.st[2], s3 = f.st[3], sL = f.st[4];
  cudaEvent_t fork = f.ev[0], flag = f.ev[1], evL = f.ev[2], ev1 = f.ev[3], ev2 = f.ev[4], ev3 = f.ev[5];
  const int nj = (int)f.order.size();
  auto launch = [&](int kind, cudaStream_t st) {
    return batch_launch(kind, f.d_desc, f.d_start + (size_t)kind * (nj + 1), nj, f.total[kind], f.smem[kind],
                        f.precision, f.fast, st);
  };
  BK_CK(cudaEventRecord(fork, s0));
  for (cudaStream_t st : {s1, s2, s3, sL}) BK_CK(cudaStreamWaitEvent(st, fork, 0));
  BK_CK(launch(BK_FLAG, s0));
  BK_CK(cudaEventRecord(flag, s0));
  BK_CK(cudaStreamWaitEvent(sL, flag, 0));
  BK_CK(launch(BK_MEMBRANE, s1));
  BK_CK(launch(BK_BOUNDS, s2));
  BK_CK(launch(BK_MORSE, s2));
  BK_CK(cudaEventRecord(ev2, s2));
  BK_CK(cudaStreamWaitEvent(s1, ev2, 0));
  BK_CK(launch(BK_SPREAD_ELEM, s1));
  BK_CK(launch(BK_BOND_PREP, s0));
  BK_CK(launch(BK_BOND_RESOLVE, s0));
  BK_CK(launch(BK_SPREAD_BOND, s0));
  BK_CK(launch(BK_FIBRIN, s3));
  BK_CK(launch(BK_SPREAD_FIB, s3));
  BK_CK(launch(BK_LBM_UNFLAGGED, sL));
  BK_CK(cudaEventRecord(evL, sL));
  BK_CK(cudaEventRecord(ev1, s1));
  BK_CK(cudaEventRecord(ev3, s3));
  for (cudaEvent_t e : {evL, ev1, ev3}) BK_CK(cudaStreamWaitEvent(s0, e, 0));
  BK_CK(launch(BK_LBM_FLAGGED, s0));
  BK_CK(launch(BK_MOMENTS, s0));
  BK_CK(launch(BK_INTERP, s0));
  return PFGPU_OK;
}

// (re)builds the fused plan over the live jobs; usable = false when a job
// cannot take part or the jobs disagree on precision / gather
int fused_plan(pfgpu_batch* b) {
  auto& f = b->fused;
  fused_release(f);
  f.valid = true;
  const char* env = getenv("PFGPU_BATCH_FUSED");
  if (env && strcmp(env, "0") == 0) return PFGPU_OK;
  std::vector<BatchDesc> descs;
  int prec = -1, fast = -1;
  for (size_t i = 0; i < b->slots.size(); ++i) {
    const auto& sl = b->slots[i];
    if (!sl.job || sl.status != PFGPU_OK) continue;
    BatchDesc d;
    int p = 0, fa = 0;
    if (!pfgpu_job_batch_desc_(sl.job, &d, &p, &fa) || !batch_supported(d)) return PFGPU_OK;
    if ((prec >= 0 && p != prec) || (fast >= 0 && fa != fast)) return PFGPU_OK;
    prec = p;
    fast = fa;
    descs.push_back(d);
    f.order.push_back((int)i);
  }
  if (descs.empty()) return PFGPU_OK;
  const int nj = (int)descs.size();
  int dev = 0, sms = 0;
  BK_CK(cudaGetDevice(&dev));
  BK_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  std::vector<int> start((size_t)BK_COUNT * (nj + 1), 0);
  for (int k = 0; k < BK_COUNT; ++k) {
    int acc = 0;
    size_t sm = 0;
    for (int j = 0; j < nj; ++j) {
      start[(size_t)k * (nj + 1) + j] = acc;
      acc += batch_ctas(descs[j], k, sms, nj);
      sm = std::max(sm, batch_smem(descs[j], k));
    }
    start[(size_t)k * (nj + 1) + nj] = acc;
    f.total[k] = acc;
    f.smem[k] = sm;
  }
  BK_CK(cudaMalloc(&f.d_desc, sizeof(BatchDesc) * nj));
  BK_CK(cudaMalloc(&f.d_start, sizeof(int) * start.size()));
  BK_CK(cudaMemcpy(f.d_desc, descs.data(), sizeof(BatchDesc) * nj, cudaMemcpyHostToDevice));
  BK_CK(cudaMemcpy(f.d_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
  if (!f.st[0]) {
    int lo = 0, hi = 0;
    BK_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int i = 0; i < 5; ++i) BK_CK(cudaStreamCreateWithPriority(&f.st[i], cudaStreamNonBlocking, i == 4 ? lo : hi));
    for (auto& e : f.ev) BK_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  f.precision = prec;
  f.fast = fast != 0;
  cudaGraph_t g = nullptr;
  BK_CK(cudaStreamBeginCapture(f.st[0], cudaStreamCaptureModeThreadLocal));
  const int rc = fused_enqueue(f);
  cudaError_t e = cudaStreamEndCapture(f.st[0], &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  BK_CK(e);
  e = cudaGraphInstantiate(&f.graph, g, 0);
  cudaGraphDestroy(g);
  BK_CK(e);
  f.usable = true;
  return PFGPU_OK;
}

}  // namespace

extern "C" {

int pfgpu_batch_create(size_t hbm_budget_bytes, pfgpu_batch** out) {
  if (!out) return report_error(PFGPU_ERR_INVALID, "out is NULL");
  pfgpu_batch* b = new pfgpu_batch();
  b->budget = hbm_budget_bytes;
  *out = b;
  return PFGPU_OK;
}

int pfgpu_batch_admit(pfgpu_batch* b, const pf_scene* scene, int precision, double fp16_scale, int* slot) {
  if (!b || !scene || !slot) return report_error(PFGPU_ERR_INVALID, "bad arguments");
  const size_t need = pfgpu_scene_device_bytes(scene, precision);
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->in_use + need > b->budget) return report_error(PFGPU_ERR_NOMEM, "job does not fit the batch budget");
  pfgpu_job* j = nullptr;
  const int rc = pfgpu_job_create(scene, precision, fp16_scale, &j);
  if (rc) return rc;
  const size_t bytes = pfgpu_job_device_bytes(j);
  int s = -1;
  for (size_t i = 0; i < b->slots.size(); ++i)
    if (!b->slots[i].job) { s = (int)i; break; }
  if (s < 0) {
    s = (int)b->slots.size();
    b->slots.emplace_back();
  }
  b->slots[s].job = j;
  b->slots[s].bytes = bytes;
  b->slots[s].status = PFGPU_OK;
  b->in_use += bytes;
  b->fused.valid = false;
  *slot = s;
  return PFGPU_OK;
}

// Advances every live job by nsteps; a detached job stops (its status reads
// PFGPU_DONE) and is left for the caller to retire.
int pfgpu_batch_step(pfgpu_batch* b, int nsteps) {
  if (!b || nsteps < 0) return report_error(PFGPU_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(b->mu);
  if (!b->fused.valid) {
    const int rc = fused_plan(b);
    if (rc) return rc;
  }
  if (b->fused.usable) {
    auto& f = b->fused;
    for (int i = 0; i < nsteps; ++i) BK_CK(cudaGraphLaunch(f.graph, f.st[0]));
    BK_CK(cudaStreamSynchronize(f.st[0]));
    int first_err = PFGPU_OK;
    bool changed = false;
    for (int i : f.order) {
      auto& s = b->slots[i];
      const int rc = pfgpu_job_sync(s.job);
      if (rc == PFGPU_DONE) {
        s.status = PFGPU_DONE;
        changed = true;
      } else if (rc && !first_err) {
        first_err = rc;
      }
    }
    if (changed) f.valid = false;  // detached jobs leave the fused step
    return first_err;
  }
  for (auto& s : b->slots)
    if (s.job && s.status == PFGPU_OK) {
      const int rc = pfgpu_job_enqueue(s.job, nsteps);
      if (rc) return rc;
    }
  int first_err = PFGPU_OK;
  for (auto& s : b->slots)
    if (s.job && s.status == PFGPU_OK) {
      const int rc = pfgpu_job_sync(s.job);
      if (rc == PFGPU_DONE) s.status = PFGPU_DONE;
      else if (rc && !first_err) first_err = rc;
    }
  return first_err;
}

int pfgpu_batch_status(pfgpu_batch* b, int slot) {
  if (!b) return report_error(PFGPU_ERR_INVALID, "bad batch");
  std::lock_guard<std::mutex> lk(b->mu);
  if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].job)
    return report_error(PFGPU_ERR_INVALID, "no job in this slot");
  return b->slots[slot].status;
}

int pfgpu_batch_retire(pfgpu_batch* b, int slot) {
  if (!b) return report_error(PFGPU_ERR_INVALID, "bad batch");
  std::lock_guard<std::mutex> lk(b->mu);
  if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].job)
    return report_error(PFGPU_ERR_INVALID, "no job in this slot");
  pfgpu_job_destroy(b->slots[slot].job);
  b->in_use -= b->slots[slot].bytes;
  b->slots[slot] = pfgpu_batch::Slot();
  b->fused.valid = false;
  return PFGPU_OK;
}

pfgpu_job* pfgpu_batch_job(pfgpu_batch* b, int slot) {
  if (!b) return nullptr;
  std::lock_guard<std::mutex> lk(b->mu);
  if (slot < 0 || slot >= (int)b->slots.size()) return nullptr;
  return b->slots[slot].job;
}

size_t pfgpu_batch_bytes_in_use(const pfgpu_batch* b) { return b ? b->in_use : 0; }

int pfgpu_batch_num_jobs(const pfgpu_batch* b) {
  if (!b) return 0;
  int n = 0;
  for (const auto& s : b->slots) n += s.job != nullptr;
  return n;
}

void pfgpu_batch_destroy(pfgpu_batch* b) {
  if (!b) return;
  fused_release(b->fused);
  for (cudaStream_t st : b->fused.st)
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t e : b->fused.ev)
    if (e) cudaEventDestroy(e);
  for (auto& s : b->slots)
    if (s.job) pfgpu_job_destroy(s.job);
  delete b;
}

}  // extern "C"
