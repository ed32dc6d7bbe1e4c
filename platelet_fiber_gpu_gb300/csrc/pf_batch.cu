// pf_batch.cu -- continuous batching of independent jobs on one GPU.
//
// Each admitted job keeps its own device state, streams and captured step
// graph; a batch step enqueues every live job's graphs back to back (each
// job on its own streams, so small lattices run side by side and fill the
// GPU together), then waits for all of them.  Jobs join (admit) and leave
// (retire) between batch steps; admission is against a device-memory budget
// using the job's exact allocation size.
#include <mutex>
#include <vector>

#include "pf_internal.h"

using namespace pf;

extern "C" int pfgpu_job_enqueue(pfgpu_job* j, int nsteps);

struct pfgpu_batch {
  size_t budget = 0, in_use = 0;
  struct Slot {
    pfgpu_job* job = nullptr;
    size_t bytes = 0;
    int status = PFGPU_OK;  // last step status (PFGPU_DONE: detached)
  };
  std::vector<Slot> slots;
  std::mutex mu;
};

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
  *slot = s;
  return PFGPU_OK;
}

// Advances every live job by nsteps; a detached job stops (its status reads
// PFGPU_DONE) and is left for the caller to retire.
int pfgpu_batch_step(pfgpu_batch* b, int nsteps) {
  if (!b || nsteps < 0) return report_error(PFGPU_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(b->mu);
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
  for (auto& s : b->slots)
    if (s.job) pfgpu_job_destroy(s.job);
  delete b;
}

}  // extern "C"
