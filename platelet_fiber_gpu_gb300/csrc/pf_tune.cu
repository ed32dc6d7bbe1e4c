// pf_tune.cu -- autotuner of the fused batch step's block and tile shapes.
//
// A shape (BatchTune) has three axes: groups of four bricks per CTA of the unflagged
// lattice pass, CTAs per SM of the near-region list and moments passes, and
// threads per CTA of the marker passes.  The search is coordinate descent:
// starting from the default shape, every value of one axis is measured with
// the other two held at the best shape so far, the best value is kept, and
// the next axis follows; two passes over the three axes.  A batch measures
// candidates online, on the steps it is asked to take (two steps each, the
// faster counts): every shape computes the same node and marker updates, so
// the steps are real work and the jobs advance as asked.  The figure of
// merit is device time per lattice-node update.  The search state is kept
// per shape class -- precision, gather kind and the log2 buckets of the
// batch's node count, job count and marker count -- in a process-wide table,
// so jobs joining and leaving a served batch resume the search instead of
// restarting it; finished classes are appended to a text file when
// PFGPU_TUNE_CACHE names one, and read back by later processes.
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "pf_internal.h"

namespace pf {

namespace {

constexpr int kPasses = 2;
const std::vector<int> kAxis[3] = {{1, 2, 4, 8, 16, 32, 64}, {2, 4, 8, 16, 32, 64}, {32, 64, 128, 256}};

using ShapeKey = std::array<int, 3>;
ShapeKey as_key(const BatchTune& t) { return {t.lbm_rows, t.list_per_sm, t.marker_threads}; }
BatchTune with_axis(BatchTune t, int axis, int v) {
  if (axis == 0) t.lbm_rows = v;
  else if (axis == 1) t.list_per_sm = v;
  else t.marker_threads = v;
  return t;
}

struct State {
  std::map<ShapeKey, float> ns;  // measured: device ns per node update
  BatchTune cur = kBatchTuneDefault;
  int axis = 0, pass = 0;
  bool done = false;
};

std::mutex g_mu;
std::map<std::string, State> g_table;
bool g_loaded = false;

int ilog2(long long v) {
  int r = 0;
  while (v > 1) {
    v >>= 1;
    ++r;
  }
  return r;
}

const char* cache_path() {
  const char* p = getenv("PFGPU_TUNE_CACHE");
  return p && *p ? p : nullptr;
}

// Lines "<class> <rows> <list_per_sm> <marker_threads> <ns per node>"; a
// later line for a class replaces an earlier one.
void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char* path = cache_path();
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char key[128];
  BatchTune t{};
  float ns = 0;
  while (fscanf(f, "%127s %d %d %d %f", key, &t.lbm_rows, &t.list_per_sm, &t.marker_threads, &ns) == 5) {
    if (t.lbm_rows < 1 || t.list_per_sm < 1 || t.marker_threads < 32 || t.marker_threads > kMarkerThreadsMax ||
        t.marker_threads % 32)
      continue;
    State& s = g_table[key];
    s.cur = t;
    s.ns[as_key(t)] = ns;
    s.done = true;
  }
  fclose(f);
}

void save_locked(const std::string& key, const State& s) {
  const char* path = cache_path();
  if (!path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  const auto it = s.ns.find(as_key(s.cur));
  fprintf(f, "%s %d %d %d %.6g\n", key.c_str(), s.cur.lbm_rows, s.cur.list_per_sm, s.cur.marker_threads,
          it == s.ns.end() ? 0.0 : (double)it->second);
  fclose(f);
}

// Moves the search on while the current axis is fully measured; returns the
// unmeasured candidates of the current axis (empty once done).
std::vector<BatchTune> pending_locked(const std::string& key, State& s) {
  while (!s.done) {
    std::vector<BatchTune> line, todo;
    for (int v : kAxis[s.axis]) line.push_back(with_axis(s.cur, s.axis, v));
    for (const BatchTune& t : line)
      if (!s.ns.count(as_key(t))) todo.push_back(t);
    if (!todo.empty()) return todo;
    BatchTune best = s.cur;
    float bn = INFINITY;
    for (const BatchTune& t : line) {
      const float n = s.ns[as_key(t)];
      if (n < bn) {
        bn = n;
        best = t;
      }
    }
    s.cur = best;
    if (++s.axis == 3) {
      s.axis = 0;
      if (++s.pass == kPasses) {
        s.done = true;
        save_locked(key, s);
      }
    }
  }
  return {};
}

}  // namespace

std::string tune_key(int precision, bool fast, long long nodes, int njobs, long long markers) {
  char buf[96];
  snprintf(buf, sizeof buf, "p%d.g%d.n%d.j%d.m%d", precision, fast ? 1 : 0, ilog2(nodes), ilog2(njobs),
           ilog2(markers + 1));
  return buf;
}

bool tune_best(const std::string& key, BatchTune* best) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  State& s = g_table[key];
  pending_locked(key, s);
  *best = s.cur;
  return s.done;
}

bool tune_next(const std::string& key, const std::vector<BatchTune>& busy, BatchTune* out) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  State& s = g_table[key];
  for (const BatchTune& t : pending_locked(key, s)) {
    bool in_flight = false;
    for (const BatchTune& b : busy) in_flight |= as_key(b) == as_key(t);
    if (!in_flight) {
      *out = t;
      return true;
    }
  }
  return false;
}

void tune_record(const std::string& key, const BatchTune& t, float ns_per_node) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  State& s = g_table[key];
  if (s.done) return;
  // a failed or non-finite measurement never wins
  s.ns[as_key(t)] = std::isfinite(ns_per_node) && ns_per_node > 0 ? ns_per_node : INFINITY;
  pending_locked(key, s);
}

}  // namespace pf

// Host hooks for testing the search without a GPU (not part of pfgpu.h):
// the next shape to measure for a class (returns 0 once the search is done,
// shape = the best), and recording a measurement.
extern "C" int pfgpu_tune_next_(const char* key, int shape[3]) {
  pf::BatchTune t{};
  const bool more = pf::tune_next(key, {}, &t);
  if (!more) pf::tune_best(key, &t);
  shape[0] = t.lbm_rows;
  shape[1] = t.list_per_sm;
  shape[2] = t.marker_threads;
  return more ? 1 : 0;
}
extern "C" void pfgpu_tune_record_(const char* key, const int shape[3], float ns_per_node) {
  pf::tune_record(key, pf::BatchTune{shape[0], shape[1], shape[2]}, ns_per_node);
}
