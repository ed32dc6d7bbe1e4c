// pf_batch.cu -- continuous batching of independent jobs on one GPU.
//
// Each admitted job keeps its own device state.  A batch step is one CUDA
// graph over all live jobs (fused): each kernel of the coupled step runs once
// for the whole batch, over the CTAs of every job, a table of per-job CTA
// offsets (start[kernel][job]) and a table of per-job handles (BatchDesc)
// telling each CTA its job.  The graph is rebuilt when jobs join (admit),
// leave (retire) or detach.  The block and tile shapes of the fused kernels
// come from the autotuner (pf_tune.cu), which measures its candidates on the
// batch's own steps.  A batch whose jobs cannot share the fused kernels
// (FP64, platelet boxes, cell-list Morse, mixed precision, or
// PFGPU_BATCH_FUSED=0) falls back to replaying every job's own step graph on
// its own streams.  Admission is against a device-memory budget using the
// job's exact allocation size.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pf_internal.h"

using namespace pf;

extern "C" int pfgpu_job_enqueue(pfgpu_job* j, int nsteps);
extern "C" int pfgpu_job_batch_desc_(pfgpu_job* j, BatchDesc* d, int* precision, int* fast);
extern "C" int pfgpu_job_control_status_(const pfgpu_job* j, const Control* c);

namespace {
// every job's control block into one array (one copy to the host reads the
// status of the whole batch)
__global__ void gather_controls_k(const BatchDesc* d, int nj, Control* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nj) out[j] = *d[j].ctl;
}
}  // namespace

struct pfgpu_batch {
  size_t budget = 0, in_use = 0;
  struct Slot {
    pfgpu_job* job = nullptr;
    size_t bytes = 0;
    int status = PFGPU_OK;  // last step status (PFGPU_DONE: detached)
  };
  std::vector<Slot> slots;
  std::mutex mu;
  // shape forced by the caller (lbm_rows == 0: the autotuner picks)
  BatchTune forced = {0, 0, 0};
  // fused step: plan over the live jobs (valid until the slots change)
  struct Fused {
    bool valid = false, usable = false;
    int precision = PF_PREC_FP32;
    bool fast = true;
    std::vector<int> order;  // slots in the plan
    std::vector<BatchDesc> descs;
    int njobs = 0, sms = 0;
    long long nodes = 0;     // lattice nodes of all jobs (one step's node updates)
    BatchDesc* d_desc = nullptr;
    Control* d_ctl = nullptr;  // gathered control blocks (device) and their host copy
    Control* h_ctl = nullptr;
    // shapes with a CTA offset table on the device; `running` is the one
    // the step graph uses
    std::vector<BatchTune> shapes;
    std::vector<int> total;  // [shapes][BK_COUNT]
    int* d_start = nullptr;  // [kMaxShapes][BK_COUNT][jobs + 1]
    int running = 0;
    bool exploring = false;  // the autotuner is measuring this class
    std::string key;
    size_t smem[BK_COUNT] = {};
    cudaStream_t st[5] = {};  // s0 (critical path), s1-s3 (forces), sL (lattice, low priority)
    cudaEvent_t ev[6] = {};
    cudaGraphExec_t graph = nullptr;
  } fused;
  std::vector<cudaEvent_t> tev;  // timing events of the autotuner's trials
};

namespace {

constexpr int kTrialSteps = 2;  // steps per measured candidate (the faster counts)
constexpr int kMaxShapes = 48;  // offset tables a plan holds (a search measures fewer)

void fused_release(pfgpu_batch::Fused& f) {
  if (f.graph) cudaGraphExecDestroy(f.graph);
  if (f.d_desc) cudaFree(f.d_desc);
  if (f.d_start) cudaFree(f.d_start);
  if (f.d_ctl) cudaFree(f.d_ctl);
  if (f.h_ctl) cudaFreeHost(f.h_ctl);
  f.graph = nullptr;
  f.d_desc = nullptr;
  f.d_start = nullptr;
  f.d_ctl = nullptr;
  f.h_ctl = nullptr;
  f.valid = false;
  f.usable = false;
  f.exploring = false;
  f.running = 0;
  f.order.clear();
  f.descs.clear();
  f.shapes.clear();
  f.total.clear();
}

#define BK_CK(call)                                                                      \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e_));  \
  } while (0)

// one fused coupled step of every job in the plan (the schedule of a single
// job's step, each kernel over the whole batch) with shape `s` of the plan
int fused_enqueue(pfgpu_batch::Fused& f, int s) {
  cudaStream_t s0 = f.st[0], s1 = f.st[1], s2 = f.st[2], s3 = f.st[3], sL = f.st[4];
  cudaEvent_t fork = f.ev[0], flag = f.ev[1], evL = f.ev[2], ev1 = f.ev[3], ev2 = f.ev[4], ev3 = f.ev[5];
  const int nj = f.njobs;
  const int* start = f.d_start + (size_t)s * BK_COUNT * (nj + 1);
  const int* total = f.total.data() + (size_t)s * BK_COUNT;
  const BatchTune& t = f.shapes[s];
  auto launch = [&](int kind, cudaStream_t st) {
    return batch_launch(kind, f.d_desc, start + (size_t)kind * (nj + 1), nj, total[kind], f.smem[kind],
                        f.precision, f.fast, t, st);
  };
  BK_CK(cudaEventRecord(fork, s0));
  for (cudaStream_t st : {s1, s2, s3, sL}) BK_CK(cudaStreamWaitEvent(st, fork, 0));
  // the quiet lattice pass (bricks without force in the previous step)
  // needs no flag of this step: sL starts at the fork; the flagging lists
  // the bricks flagged in this step or the previous one for the flagged-
  // brick pass
  BK_CK(launch(BK_FLAG, s0));
  (void)flag;
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

// captures and instantiates the step graph of shape `s`
int fused_graph(pfgpu_batch::Fused& f, int s, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  BK_CK(cudaStreamBeginCapture(f.st[0], cudaStreamCaptureModeThreadLocal));
  const int rc = fused_enqueue(f, s);
  cudaError_t e = cudaStreamEndCapture(f.st[0], &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  BK_CK(e);
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  BK_CK(e);
  BK_CK(cudaGraphUpload(*out, f.st[0]));
  return PFGPU_OK;
}

bool tuning_enabled() {
  const char* env = getenv("PFGPU_BATCH_TUNE");
  return !(env && strcmp(env, "0") == 0);
}

// index of shape t in the plan, adding its CTA offset table (copied on s0,
// so it lands before any later launch reads it); -1 when the plan is full
int fused_shape(pfgpu_batch::Fused& f, const BatchTune& t) {
  for (size_t s = 0; s < f.shapes.size(); ++s)
    if (f.shapes[s].lbm_rows == t.lbm_rows && f.shapes[s].list_per_sm == t.list_per_sm &&
        f.shapes[s].marker_threads == t.marker_threads)
      return (int)s;
  if ((int)f.shapes.size() == kMaxShapes) return -1;
  const int nj = f.njobs;
  const size_t row = (size_t)nj + 1, s = f.shapes.size();
  std::vector<int> start(BK_COUNT * row, 0);
  for (int k = 0; k < BK_COUNT; ++k) {
    int* st = start.data() + k * row;
    int acc = 0;
    for (int j = 0; j < nj; ++j) {
      st[j] = acc;
      acc += batch_ctas(f.descs[j], k, f.sms, nj, t);
    }
    st[nj] = acc;
    f.total.push_back(acc);
  }
  const cudaError_t e = cudaMemcpyAsync(f.d_start + s * BK_COUNT * row, start.data(), sizeof(int) * start.size(),
                                        cudaMemcpyHostToDevice, f.st[0]);
  if (e != cudaSuccess) {
    f.total.resize(s * BK_COUNT);
    report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
    return -2;
  }
  f.shapes.push_back(t);
  return (int)s;
}

// makes shape t the running one (after the launches in flight)
int fused_switch(pfgpu_batch::Fused& f, const BatchTune& t) {
  const int s = fused_shape(f, t);
  if (s < 0) return s == -1 ? PFGPU_OK : PFGPU_ERR_CUDA;  // a full plan keeps its shape
  if (s == f.running && f.graph) return PFGPU_OK;
  cudaGraphExec_t g = nullptr;
  const int rc = fused_graph(f, s, &g);
  if (rc) return rc;
  BK_CK(cudaStreamSynchronize(f.st[0]));
  if (f.graph) cudaGraphExecDestroy(f.graph);
  f.graph = g;
  f.running = s;
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
  int prec = -1, fast = -1;
  long long nodes = 0, markers = 0;
  for (size_t i = 0; i < b->slots.size(); ++i) {
    const auto& sl = b->slots[i];
    if (!sl.job || sl.status != PFGPU_OK) continue;
    BatchDesc d;
    int p = 0, fa = 0;
    if (!pfgpu_job_batch_desc_(sl.job, &d, &p, &fa) || !batch_supported(d)) {
      fused_release(f);
      f.valid = true;
      return PFGPU_OK;
    }
    if ((prec >= 0 && p != prec) || (fast >= 0 && fa != fast)) {
      fused_release(f);
      f.valid = true;
      return PFGPU_OK;
    }
    prec = p;
    fast = fa;
    nodes += d.L.k.N;
    markers += (d.has_pl ? (long long)d.Pl.k.P * d.Pl.k.E : 0) + (d.has_fb ? d.Fb.M : 0);
    f.descs.push_back(d);
    f.order.push_back((int)i);
  }
  if (f.descs.empty()) return PFGPU_OK;
  const int nj = (int)f.descs.size();
  f.njobs = nj;
  f.nodes = nodes;
  f.precision = prec;
  f.fast = fast != 0;
  int dev = 0;
  BK_CK(cudaGetDevice(&dev));
  BK_CK(cudaDeviceGetAttribute(&f.sms, cudaDevAttrMultiProcessorCount, dev));
  for (int k = 0; k < BK_COUNT; ++k) {
    size_t sm = 0;
    for (int j = 0; j < nj; ++j) sm = std::max(sm, batch_smem(f.descs[j], k));
    f.smem[k] = sm;
  }
  BK_CK(cudaMalloc(&f.d_desc, sizeof(BatchDesc) * nj));
  BK_CK(cudaMalloc(&f.d_start, sizeof(int) * (size_t)kMaxShapes * BK_COUNT * (nj + 1)));
  BK_CK(cudaMemcpy(f.d_desc, f.descs.data(), sizeof(BatchDesc) * nj, cudaMemcpyHostToDevice));
  BK_CK(cudaMalloc(&f.d_ctl, sizeof(Control) * nj));
  BK_CK(cudaMallocHost(&f.h_ctl, sizeof(Control) * nj));
  if (!f.st[0]) {
    int lo = 0, hi = 0;
    BK_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int i = 0; i < 5; ++i) BK_CK(cudaStreamCreateWithPriority(&f.st[i], cudaStreamNonBlocking, i == 4 ? lo : hi));
    for (auto& e : f.ev) BK_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // the forced shape, the default (tuning off), or the class's best so far
  // (the search goes on while exploring)
  BatchTune t = kBatchTuneDefault;
  if (b->forced.lbm_rows > 0) {
    t = b->forced;
  } else if (tuning_enabled()) {
    f.key = tune_key(prec, fast != 0, nodes, nj, markers);
    f.exploring = !tune_best(f.key, &t);
  }
  const int rc = fused_switch(f, t);
  if (rc) return rc;
  f.usable = true;
  return PFGPU_OK;
}

// nsteps fused steps.  While the shape class is being explored, pairs of
// steps run candidate shapes from the autotuner (timed with events on s0),
// the other steps the running graph; the search's winner becomes the running
// shape.  Returns after the device work is done.
int fused_steps(pfgpu_batch* b, int nsteps) {
  auto& f = b->fused;
  struct Trial {
    int s;
    cudaGraphExec_t g;
    size_t ev;
  };
  std::vector<Trial> trials;
  std::vector<BatchTune> busy;
  size_t done = 0;
  int rc = PFGPU_OK;
  auto harvest = [&]() {
    const cudaError_t se = cudaStreamSynchronize(f.st[0]);
    if (!rc && se != cudaSuccess) rc = report_error(PFGPU_ERR_CUDA, cudaGetErrorString(se));
    for (; done < trials.size(); ++done) {
      const Trial& t = trials[done];
      float ms = INFINITY;
      for (int k = 0; k < kTrialSteps && !rc; ++k) {
        float m = 0;
        if (cudaEventElapsedTime(&m, b->tev[t.ev + k], b->tev[t.ev + k + 1]) == cudaSuccess) ms = std::min(ms, m);
      }
      if (!rc) tune_record(f.key, f.shapes[t.s], (float)(ms * 1e6 / (double)f.nodes));
      cudaGraphExecDestroy(t.g);
    }
    busy.clear();
  };
  for (int i = 0; i < nsteps && !rc;) {
    BatchTune t{};
    bool trial = false;
    if (f.exploring && nsteps - i >= kTrialSteps) {
      trial = tune_next(f.key, busy, &t);
      if (!trial && !busy.empty()) {
        harvest();
        trial = !rc && tune_next(f.key, busy, &t);
      }
      if (!trial && !rc) {
        // the search is over (or waits on nothing): run its best shape
        BatchTune best;
        if (tune_best(f.key, &best)) {
          rc = fused_switch(f, best);
          f.exploring = false;
        }
      }
    }
    const int s = trial ? fused_shape(f, t) : -1;
    if (s == -2) rc = PFGPU_ERR_CUDA;
    if (rc) break;
    if (s < 0) {
      if (trial) f.exploring = false;  // plan full: keep the running shape
      if (cudaGraphLaunch(f.graph, f.st[0]) != cudaSuccess) rc = report_error(PFGPU_ERR_CUDA, "graph launch");
      ++i;
      continue;
    }
    const size_t ev = trials.size() * (kTrialSteps + 1);
    while (!rc && b->tev.size() < ev + kTrialSteps + 1) {
      cudaEvent_t e = nullptr;
      const cudaError_t ce = cudaEventCreate(&e);
      if (ce != cudaSuccess) rc = report_error(PFGPU_ERR_CUDA, cudaGetErrorString(ce));
      else b->tev.push_back(e);
    }
    if (rc) break;
    cudaGraphExec_t g = nullptr;
    rc = fused_graph(f, s, &g);
    if (rc) break;
    trials.push_back({s, g, ev});
    busy.push_back(t);
    cudaError_t e = cudaEventRecord(b->tev[ev], f.st[0]);
    for (int k = 0; k < kTrialSteps && e == cudaSuccess; ++k) {
      e = cudaGraphLaunch(g, f.st[0]);
      if (e == cudaSuccess) e = cudaEventRecord(b->tev[ev + k + 1], f.st[0]);
    }
    if (e != cudaSuccess) rc = report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
    i += kTrialSteps;
  }
  harvest();
  if (!rc && f.exploring) {
    BatchTune best;
    if (tune_best(f.key, &best)) {
      rc = fused_switch(f, best);
      f.exploring = false;
    }
  }
  return rc;
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
    const int rc = fused_steps(b, nsteps);
    if (rc) return rc;
    const int nj = f.njobs;
    gather_controls_k<<<(nj + 127) / 128, 128, 0, f.st[0]>>>(f.d_desc, nj, f.d_ctl);
    BK_CK(cudaGetLastError());
    BK_CK(cudaMemcpyAsync(f.h_ctl, f.d_ctl, sizeof(Control) * nj, cudaMemcpyDeviceToHost, f.st[0]));
    BK_CK(cudaStreamSynchronize(f.st[0]));
    int first_err = PFGPU_OK;
    bool changed = false;
    for (int q = 0; q < nj; ++q) {
      auto& s = b->slots[f.order[q]];
      const int rc = pfgpu_job_control_status_(s.job, &f.h_ctl[q]);
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

// The job in `slot` stops by itself after step stop_step (0: never); its
// status turns PFGPU_DONE at the end of the batch step that reached it.
int pfgpu_batch_set_stop(pfgpu_batch* b, int slot, int64_t stop_step) {
  if (!b) return report_error(PFGPU_ERR_INVALID, "bad batch");
  std::lock_guard<std::mutex> lk(b->mu);
  if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].job)
    return report_error(PFGPU_ERR_INVALID, "no job in this slot");
  auto& s = b->slots[slot];
  int rc = pfgpu_job_set_stop(s.job, stop_step);
  if (rc) return rc;
  rc = pfgpu_job_sync(s.job);
  const int st = rc == PFGPU_DONE ? PFGPU_DONE : (rc ? s.status : PFGPU_OK);
  if (st != s.status) {
    s.status = st;
    b->fused.valid = false;
  }
  return rc == PFGPU_DONE ? PFGPU_OK : rc;
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

// The fused step's block and tile shapes: shape[0] groups of four bricks per CTA of
// the unflagged lattice pass, shape[1] CTAs per SM of the list and moments
// passes, shape[2] threads per CTA of the marker passes.  *state: 0 the
// autotuner is still measuring candidates (shape is the one running between
// trials), 1 tuned (or forced, or tuning off), -1 the batch does not use the
// fused step.  The plan is built first if the slots changed.
int pfgpu_batch_shape(pfgpu_batch* b, int shape[3], int* state) {
  if (!b || !shape || !state) return report_error(PFGPU_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(b->mu);
  if (!b->fused.valid) {
    const int rc = fused_plan(b);
    if (rc) return rc;
  }
  const auto& f = b->fused;
  if (!f.usable) {
    shape[0] = shape[1] = shape[2] = 0;
    *state = -1;
    return PFGPU_OK;
  }
  const BatchTune& t = f.shapes[f.running];
  shape[0] = t.lbm_rows;
  shape[1] = t.list_per_sm;
  shape[2] = t.marker_threads;
  *state = f.exploring ? 0 : 1;
  return PFGPU_OK;
}

// Forces the fused step's shapes (lbm_rows 0: back to the autotuner).
int pfgpu_batch_set_shape(pfgpu_batch* b, int lbm_rows, int list_per_sm, int marker_threads) {
  if (!b) return report_error(PFGPU_ERR_INVALID, "bad batch");
  if (lbm_rows != 0 && (lbm_rows < 1 || lbm_rows > 64 || list_per_sm < 1 || list_per_sm > 64 ||
                        marker_threads < 32 || marker_threads > kMarkerThreadsMax || marker_threads % 32))
    return report_error(PFGPU_ERR_INVALID, "shape out of range");
  std::lock_guard<std::mutex> lk(b->mu);
  b->forced = lbm_rows ? BatchTune{lbm_rows, list_per_sm, marker_threads} : BatchTune{0, 0, 0};
  b->fused.valid = false;
  return PFGPU_OK;
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
  for (cudaEvent_t e : b->tev) cudaEventDestroy(e);
  for (auto& s : b->slots)
    if (s.job) pfgpu_job_destroy(s.job);
  delete b;
}

}  // extern "C"
