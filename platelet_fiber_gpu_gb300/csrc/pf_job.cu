// pf_job.cu -- job API of pfgpu.h: device-resident simulations built from a
// pf_scene, stepped by direct launches or by a captured CUDA graph.
//
// One coupled step (the reference's sem_invokeGPUKernel_Force followed by
// fluid_invokeGPUKernel, semLB.cu:303-531) is issued as:
//   fork  -> membrane forces | Morse forces | fibrin forces | receptor bonds
//   join  -> IBM spreading -> fused collide-stream -> moments of the active
//            bricks -> IBM interpolation + position update + cell binning
// The four force kernels write separate buffers, so they run concurrently.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pf_internal.h"

namespace pf {
size_t bond_scratch_bytes(int NR);
}

using namespace pf;

static thread_local std::string g_last_error;
static std::mutex g_err_mu;
static std::string g_last_error_global;

static int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error_global = msg;
  return code;
}

namespace pf {
int report_error(int code, const char* msg) { return set_error(code, msg); }
}  // namespace pf

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return set_error(e_ == cudaErrorMemoryAllocation ? PFGPU_ERR_NOMEM : PFGPU_ERR_CUDA,     \
                       std::string(#call) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

struct pfgpu_job {
  int precision = PF_PREC_FP64;
  Lattice L;
  Platelets Pl;
  Fibrin Fb;
  bool has_pl = false, has_fb = false;
  Control* ctl = nullptr;
  unsigned* done_blocks = nullptr;
  double* scratch4 = nullptr;
  // s0: flags, bonds, then the critical path after the forces (spreading,
  // flagged lattice pass, moments, interpolation); s1-s3: membrane, Morse,
  // fibrin; sL (low priority): the lattice pass over the force-free bricks
  cudaStream_t s0 = nullptr, s1 = nullptr, s2 = nullptr, s3 = nullptr, sL = nullptr, sF = nullptr;
  cudaEvent_t ev_fork = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr, ev_flag = nullptr, evL = nullptr,
              ev_far = nullptr, ev_list = nullptr, ev_q = nullptr;
  // pipelined schedule (PFGPU_PIPELINE=1): the far region of the next step
  // is updated during this step (far_ready: the far pass of the current step
  // is done)
  bool pipeline = false, far_ready = false;
  // quiet pass ahead (serial schedule): the quiet lattice pass of step t+1
  // runs beside step t's moments and interpolation, right after its
  // flagged-brick pass (quiet_ready: the current step's quiet pass is done)
  bool quiet_ahead = false, quiet_ready = false;
  // a quiet pass run ahead on sL that s0 has not waited for yet (the next
  // step's flagged-brick pass waits for it; quiet_join at the end of a
  // stepping call or graph capture)
  bool q_pending = false;
  // steps per captured graph (graphK), so that a step's force kernels
  // overlap the quiet pass run ahead by the step before (the graph's last
  // step joins it; 256x128x128 FP32: 0.2062 / 0.2060 / 0.2012 / 0.1998 ms
  // per step with 1 / 2 / 4 / 8 steps per graph).  Four: half the capture
  // time of eight, and step counts that are multiples of four need no
  // one-step graph
  int graph_k = 4;
  cudaGraphExec_t graphK = nullptr;
  cudaGraphExec_t graph = nullptr;
  double detach_rate = 0;
  uint64_t seed = 0;
  size_t bytes = 0;
  std::vector<void*> allocs;
  std::vector<size_t> alloc_bytes;  // size of each allocation (the state snapshot's layout)
  int launches_per_step = 0;
};

// Job buffers come from the device's stream-ordered memory pool, in order on
// the job's stream s0: the pool keeps up to kPoolKeepBytes of freed memory
// mapped, so a job created after another was destroyed (a served loop, a
// restart) reuses its memory instead of mapping new pages.  Every job-creation
// operation is queued on s0 (allocation, zero fill, uploads, the initial
// lattice), so host-side set-up overlaps the device work and one
// synchronisation ends the creation.
constexpr unsigned long long kPoolKeepBytes = 32ull << 30;
static void keep_pool_memory() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long keep = kPoolKeepBytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  done[dev] = true;
}

template <class T>
static cudaError_t dalloc(pfgpu_job* j, T** p, size_t count, bool zero = true) {
  size_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = sizeof(T);
  cudaError_t e = cudaMallocAsync((void**)p, bytes, j->s0);
  if (e == cudaSuccess) {
    j->allocs.push_back(*p);
    j->alloc_bytes.push_back(bytes);
    j->bytes += bytes;
    if (zero) e = cudaMemsetAsync(*p, 0, bytes, j->s0);
  }
  return e;
}
template <class T>
static cudaError_t dupload(pfgpu_job* j, T** p, const T* src, size_t count) {
  cudaError_t e = dalloc(j, p, count, !(src && count));
  if (e == cudaSuccess && src && count)
    e = cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, j->s0);
  return e;
}

static void destroy(pfgpu_job* j) {
  if (!j) return;
  if (j->graph) cudaGraphExecDestroy(j->graph);
  if (j->graphK) cudaGraphExecDestroy(j->graphK);
  if (j->s0) {
    cudaStreamSynchronize(j->s0);
    for (void* p : j->allocs) cudaFreeAsync(p, j->s0);
    cudaStreamSynchronize(j->s0);
  }
  cudaStream_t ss[6] = {j->s0, j->s1, j->s2, j->s3, j->sL, j->sF};
  for (cudaStream_t s : ss)
    if (s) cudaStreamDestroy(s);
  cudaEvent_t ee[9] = {j->ev_fork, j->ev1, j->ev2, j->ev3, j->ev_flag, j->evL, j->ev_far, j->ev_list, j->ev_q};
  for (cudaEvent_t e : ee)
    if (e) cudaEventDestroy(e);
  delete j;
}

// An address the device can read or write for caller memory: device and
// managed memory as given, pinned host memory through its mapping, and
// pageable host memory as given where the GPU walks the host's page tables
// (ATS over NVLink-C2C on Grace machines).  NULL otherwise, or when
// PFGPU_HOST_DIRECT=0: the data then goes through a device staging copy.
static void* device_view(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return const_cast<void*>(p);
  const char* env = getenv("PFGPU_HOST_DIRECT");
  if (env && strcmp(env, "0") == 0) return nullptr;
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  int dev = 0, pageable = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return pageable ? const_cast<void*>(p) : nullptr;
}

static size_t store_bytes(int precision) {
  return precision == PF_PREC_FP64 ? 8 : (precision == PF_PREC_FP32 ? 4 : 2);
}
static size_t real_bytes(int precision) { return precision == PF_PREC_FP64 ? 8 : 4; }

// lattice constants from the reference parameter table (float arithmetic where
// the reference does it in float)
static LatticeConst lattice_const(const pf_scene* s, double fp16_scale, int precision) {
  LatticeConst k{};
  k.nx = s->nx; k.ny = s->ny; k.nz = s->nz;
  k.nbx = (s->nx + kBrickX - 1) / kBrickX;
  k.nbricks = k.nbx * s->ny * s->nz;
  k.N = (long long)s->nx * s->ny * s->nz;
  for (int a = 0; a < 3; ++a) { k.bc[a] = s->bc[a]; k.ibm_wrap[a] = s->ibm_wrap[a]; }
  k.ibm_wrap[2] = 0;
  k.dxf = s->dx; k.dtf = s->dt;
  const float* mp = s->params;
  float c = s->dx / s->dt;
  c = c / mp[PF_P_UMAX];
  k.C = (double)c;
  k.omega = 1.0 / (double)mp[PF_P_TAU];
  const double Kd = (double)mp[PF_P_F0] / (double)mp[PF_P_RHO0] / (double)mp[PF_P_UMAX] * (double)mp[PF_P_UNIT];
  float kf = mp[PF_P_F0] / mp[PF_P_RHO0];
  kf = kf / mp[PF_P_UMAX];
  kf = kf * mp[PF_P_UNIT];
  k.kcoll = Kd * (double)s->dt / k.C;
  k.kmom = (double)kf * (double)s->dt / k.C;
  for (int a = 0; a < 3; ++a) k.body[a] = s->body_force[a];
  float uw = mp[PF_P_SHEAR] * (float)(s->nz - 1);
  uw = uw * s->dx;
  uw = uw / mp[PF_P_UMAX];
  k.uw = (double)uw / k.C;
  // FP16 stores q = (f - w) / (w * sigma); sigma defaults to eight times the
  // wall speed of a shear channel (or 0.05 lattice units otherwise)
  double sigma = fp16_scale;
  if (!(sigma > 0)) sigma = (s->bc[2] == PF_BC_ZOUHE_SHEAR && k.uw > 0) ? 8.0 * k.uw : 0.05;
  k.fp16_scale = precision == PF_PREC_FP16 ? sigma : 1.0;
  const double wc[3] = {1.0 / 3.0, 1.0 / 18.0, 1.0 / 36.0};
  for (int c = 0; c < 3; ++c) {
    k.hs[c] = (float)(wc[c] * k.fp16_scale);
    k.hinv[c] = 1.0f / k.hs[c];
  }
  k.isig = (float)(1.0 / k.fp16_scale);
  k.inv_dx = 1.0 / (double)k.dxf;
  k.Lx = (double)k.nx * (double)k.dxf;
  k.Ly = (double)k.ny * (double)k.dxf;
  // bounded device waits give up after 1 s; PFGPU_WAIT_LIMIT_NS shortens
  // the limit (0: give up at the first unfinished wait) so that tests can
  // run the give-up path
  k.wait_ns = 1000000000ull;
  if (const char* w = getenv("PFGPU_WAIT_LIMIT_NS")) k.wait_ns = strtoull(w, nullptr, 10);
  k.dtT = s->dt / mp[PF_P_T0];
  k.omega_f = (float)k.omega;
  k.kcoll_f = (float)k.kcoll;
  k.kmom_f = (float)k.kmom;
  for (int a = 0; a < 3; ++a) k.body_f[a] = (float)k.body[a];
  k.nobody = k.body_f[0] == 0.f && k.body_f[1] == 0.f && k.body_f[2] == 0.f;
  k.uw_f = (float)k.uw;
  return k;
}

static int validate(const pf_scene* s, int precision) {
  if (!s) return set_error(PFGPU_ERR_INVALID, "scene is NULL");
  if (s->nx < 1 || s->ny < 1 || s->nz < 1 || s->ny > 65535 || s->nz > 65535)
    return set_error(PFGPU_ERR_INVALID, "lattice dimensions out of range");
  if (precision < PF_PREC_FP64 || precision > PF_PREC_FP16) return set_error(PFGPU_ERR_INVALID, "bad precision");
  if (s->bc[0] == PF_BC_ZOUHE_SHEAR || s->bc[1] == PF_BC_ZOUHE_SHEAR)
    return set_error(PFGPU_ERR_UNSUPPORTED, "Zou/He shear walls are only supported on z");
  if (s->bc[2] == PF_BC_ZOUHE_SHEAR && (s->bc[0] == PF_BC_BOUNCEBACK || s->bc[1] == PF_BC_BOUNCEBACK))
    return set_error(PFGPU_ERR_UNSUPPORTED, "Zou/He z walls need periodic x and y");
  for (int a = 0; a < 3; ++a)
    if (s->bc[a] < PF_BC_PERIODIC || s->bc[a] > PF_BC_INOUT) return set_error(PFGPU_ERR_INVALID, "unknown boundary kind");
  if (s->bc[0] == PF_BC_INOUT || s->bc[2] == PF_BC_INOUT)
    return set_error(PFGPU_ERR_UNSUPPORTED, "the inflow/outflow planes are only supported on y");
  if (s->bc[1] == PF_BC_INOUT && (s->bc[2] != PF_BC_ZOUHE_SHEAR || s->bc[0] != PF_BC_PERIODIC || s->nx < 3 ||
                                  s->nz < 3 || s->ny < 2))
    return set_error(PFGPU_ERR_UNSUPPORTED, "inflow/outflow on y needs Zou/He shear walls on z, periodic x");
  if (s->n_platelets < 0 || s->n_elem < 0 || s->n_fib < 0 || s->n_rec < 0)
    return set_error(PFGPU_ERR_INVALID, "negative count");
  if (s->membrane_forces & ~(PF_MEM_ALL | PF_MEM_FEMBEND))
    return set_error(PFGPU_ERR_INVALID, "unknown membrane force bits");
  if (s->n_fib > 0) {
    if (s->fib_coupling != PF_FIBCPL_MARKER && s->fib_coupling != PF_FIBCPL_PENALTY)
      return set_error(PFGPU_ERR_INVALID, "unknown fibrin coupling");
    if (s->fib_coupling == PF_FIBCPL_PENALTY &&
        !(s->fib_node_mass > 0 && s->fib_gamma >= 0 && s->fib_kappa >= 0 && std::isfinite(s->fib_gamma) &&
          std::isfinite(s->fib_kappa) && std::isfinite(s->fib_node_mass)))
      return set_error(PFGPU_ERR_INVALID, "penalty coupling needs node mass > 0, gamma >= 0, kappa >= 0");
  }
  if (s->n_platelets > 0) {
    if (!s->X || !s->Y || !s->RY || !s->Z) return set_error(PFGPU_ERR_INVALID, "element positions missing");
    if (s->n_membrane > s->n_elem) return set_error(PFGPU_ERR_INVALID, "n_membrane > n_elem");
    if (s->n_tri > 0 && (!s->tri || !s->node_ntri || !s->ring || !s->S0 || !s->S0_all || !s->V0))
      return set_error(PFGPU_ERR_INVALID, "membrane topology missing");
    if (s->n_rec > 0 && (!s->rec_tri || !s->rec_r1 || !s->rec_r2 || s->n_tri == 0))
      return set_error(PFGPU_ERR_INVALID, "receptor arrays missing");
    if ((long long)s->n_platelets * s->n_rec > (1LL << 30)) return set_error(PFGPU_ERR_INVALID, "too many receptors");
  }
  if (s->n_fib > 0 && (!s->fib_X || !s->fib_Y || !s->fib_Z || !s->fib_fixed || !s->fib_ptr))
    return set_error(PFGPU_ERR_INVALID, "fibrin arrays missing");
  // every index a kernel dereferences is checked here, on the host
  if (s->n_platelets > 0 && s->n_elem > 0) {
    const int E = s->n_elem, Em = s->n_membrane, T = s->n_tri, NN = s->n_node;
    for (int t = 0; t < T; ++t)
      for (int i = 0; i < 6; ++i) {
        const int q = s->tri[6 * t + i];
        if (q < 0 || q >= NN || (i < 3 && q >= Em))
          return set_error(PFGPU_ERR_INVALID, "triangle index out of range");
      }
    for (int q = 0; q < NN; ++q)
      if (s->node_ntri[q] < 0 || s->node_ntri[q] > 10) return set_error(PFGPU_ERR_INVALID, "node_ntri out of range");
    if (T > 0)
      for (int v = 0; v < Em; ++v)
        for (int a = 0; a < s->node_ntri[v]; ++a) {
          const int r = s->ring[10 * v + a];
          if (r < 0 || r >= Em) return set_error(PFGPU_ERR_INVALID, "ring index out of range");
        }
    if (s->spring_ptr) {
      if (s->spring_ptr[0] != 0) return set_error(PFGPU_ERR_INVALID, "spring_ptr[0] != 0");
      for (int e = 0; e < E; ++e) {
        if (s->spring_ptr[e + 1] < s->spring_ptr[e]) return set_error(PFGPU_ERR_INVALID, "spring_ptr not monotone");
        for (int q = s->spring_ptr[e]; q < s->spring_ptr[e + 1]; ++q)
          if (s->spring_nbr[q] < 0 || s->spring_nbr[q] >= E)
            return set_error(PFGPU_ERR_INVALID, "spring neighbour out of range");
      }
    }
    const long long NR = (long long)s->n_platelets * s->n_rec;
    for (long long r = 0; r < NR; ++r)
      if (s->rec_tri[r] < 0 || s->rec_tri[r] >= T) return set_error(PFGPU_ERR_INVALID, "receptor triangle out of range");
  }
  if (s->n_fib > 0) {
    const int M = s->n_fib;
    if (s->fib_ptr[0] != 0) return set_error(PFGPU_ERR_INVALID, "fib_ptr[0] != 0");
    for (int m = 0; m < M; ++m) {
      if (s->fib_ptr[m + 1] < s->fib_ptr[m]) return set_error(PFGPU_ERR_INVALID, "fib_ptr not monotone");
      for (int q = s->fib_ptr[m]; q < s->fib_ptr[m + 1]; ++q)
        if (s->fib_nbr[q] < 0 || s->fib_nbr[q] >= M) return set_error(PFGPU_ERR_INVALID, "fibrin link out of range");
    }
  }
  return PFGPU_OK;
}

static int build_platelets(pfgpu_job* j, const pf_scene* s) {
  Platelets& P = j->Pl;
  PlateletConst& k = P.k;
  k.P = s->n_platelets; k.E = s->n_elem; k.Em = s->n_membrane; k.T = s->n_tri; k.NN = s->n_node;
  k.nrec = s->n_rec;
  k.mask = s->membrane_forces;
  const float* mp = s->params;
  k.kspring = mp[PF_P_KSPRING]; k.ks = mp[PF_P_KS]; k.kv = mp[PF_P_KV]; k.kbend = mp[PF_P_KBEND] * 1;
  k.f0 = mp[PF_P_F0]; k.kf0 = mp[PF_P_KF0]; k.kr0 = mp[PF_P_KR0]; k.numrec = mp[PF_P_NUMRECEPTORS];
  k.dxd = (double)s->dx; k.dtd = (double)s->dt; k.dxf = s->dx; k.dtf = s->dt; k.dtT = s->dt / mp[PF_P_T0];
  k.inv_f0 = 1.0 / (double)k.f0;
  k.bond_model = s->bond_model; k.p_on = s->p_on; k.p_off = s->p_off; k.seed = s->seed;
  k.morse = s->morse;
  for (int a = 0; a < 4; ++a) { k.morse_intra[a] = s->morse_intra[a]; k.morse_inter[a] = s->morse_inter[a]; }
  auto Fcut = [](const double* mp) {
    const double ex = std::exp(mp[1] * (mp[2] - mp[3]));
    return 2.0 * mp[1] * mp[0] * (ex * ex - ex);
  };
  k.morse_fc[0] = Fcut(s->morse_intra);
  k.morse_fc[1] = Fcut(s->morse_inter);
  k.nx = s->nx; k.ny = s->ny; k.nz = s->nz;
  const int n3[3] = {s->nx, s->ny, s->nz};
  const double rc = s->morse_intra[3] > s->morse_inter[3] ? s->morse_intra[3] : s->morse_inter[3];
  for (int a = 0; a < 3; ++a) {
    const double L = n3[a] * (double)s->dx;
    int nc = rc > 0 ? (int)std::floor(L / rc) : 1;
    if (nc < 1) nc = 1;
    k.ncell[a] = nc;
    k.cs[a] = L / nc;
    k.L[a] = L;
    k.wrap[a] = a < 2 ? s->ibm_wrap[a] : 0;
  }
  const size_t PE = (size_t)k.P * k.E;
  const size_t rb = real_bytes(j->precision);
  CK(dupload(j, &P.X, s->X, PE));
  CK(dupload(j, &P.Y, s->Y, PE));
  CK(dupload(j, &P.RY, s->RY, PE));
  CK(dupload(j, &P.Z, s->Z, PE));
  CK(dalloc(j, &P.V, 3 * PE));
  CK(dalloc(j, &P.Ftot, 3 * PE));
  CK(dalloc(j, (char**)&P.Fmem, 3 * PE * rb));
  CK(dalloc(j, &P.Fmorse, 3 * PE));
  CK(dalloc(j, (char**)&P.Fbond, 3 * PE * rb));
  // topology: triangles of each node in ascending order, and each vertex's
  // local index in them (gathers replace the reference's atomics)
  std::vector<int> node_tri((size_t)k.NN * 10, -1), vert_local((size_t)k.Em * 10, -1), fill(k.NN, 0);
  for (int t = 0; t < k.T; ++t)
    for (int i = 0; i < 6; ++i) {
      const int q = s->tri[6 * t + i];
      if (q < 0 || q >= k.NN) return set_error(PFGPU_ERR_INVALID, "triangle node index out of range");
      if (fill[q] >= 10) return set_error(PFGPU_ERR_INVALID, "more than 10 triangles share a node");
      node_tri[(size_t)q * 10 + fill[q]] = t;
      if (q < k.Em) vert_local[(size_t)q * 10 + fill[q]] = i;
      fill[q]++;
    }
  for (int q = 0; q < k.NN; ++q)
    if (fill[q] != s->node_ntri[q]) return set_error(PFGPU_ERR_INVALID, "node_ntri inconsistent with tri");
  CK(dupload(j, &P.tri, s->tri, (size_t)k.T * 6));
  CK(dupload(j, &P.node_ntri, s->node_ntri, (size_t)k.NN));
  CK(dupload(j, &P.node_tri, node_tri.data(), node_tri.size()));
  CK(dupload(j, &P.vert_local, vert_local.data(), vert_local.size()));
  CK(dupload(j, &P.ring, s->ring, (size_t)k.Em * 10));
  std::vector<int> sp_ptr(k.E + 1, 0);
  if (s->spring_ptr) sp_ptr.assign(s->spring_ptr, s->spring_ptr + k.E + 1);
  const int nsp = sp_ptr[k.E];
  CK(dupload(j, &P.sp_ptr, sp_ptr.data(), sp_ptr.size()));
  CK(dupload(j, &P.sp_nbr, s->spring_nbr, (size_t)nsp));
  CK(dupload(j, &P.sp_L0, s->spring_L0, (size_t)nsp));
  CK(dupload(j, &P.S0, s->S0, (size_t)k.P * k.T));
  CK(dupload(j, &P.S0_all, s->S0_all, (size_t)k.P));
  CK(dupload(j, &P.V0, s->V0, (size_t)k.P));
  CK(dalloc(j, (char**)&P.nN, (size_t)k.P * k.NN * 3 * rb));
  CK(dalloc(j, (char**)&P.nelem, (size_t)k.P * k.T * 3 * rb));
  CK(dalloc(j, (char**)&P.S, (size_t)k.P * k.T * rb));
  CK(dalloc(j, (char**)&P.km, (size_t)k.P * k.Em * rb));
  CK(dalloc(j, &P.SV, (size_t)k.P * 2));
  if (k.mask & PF_MEM_FEMBEND) {
    // the chain divides by S[vertex id] of the per-triangle area array
    if (k.Em > k.T) return set_error(PFGPU_ERR_INVALID, "FEM bending needs at least as many triangles as vertices");
    CK(dalloc(j, (char**)&P.fem, (size_t)k.P * ((size_t)k.NN * 12 + (size_t)k.T * 4) * rb));
  }
  // receptors and wall sites
  const size_t NR = (size_t)k.P * k.nrec;
  CK(dupload(j, &P.rec_tri, s->rec_tri, NR));
  CK(dupload(j, &P.r1, s->rec_r1, NR));
  CK(dupload(j, &P.r2, s->rec_r2, NR));
  std::vector<int> st(3 * NR, -1);
  if (s->rec_state) st.assign(s->rec_state, s->rec_state + 3 * NR);
  CK(dupload(j, &P.rec_state, st.data(), st.size()));
  std::vector<int> vw((size_t)4 * s->nx * s->ny, -1);
  if (s->vwf) vw.assign(s->vwf, s->vwf + vw.size());
  CK(dupload(j, &P.vwf, vw.data(), vw.size()));
  if (NR) CK(dalloc(j, (char**)&P.rec_tmp, bond_scratch_bytes((int)NR)));
  CK(dalloc(j, &P.bounds, (size_t)k.P * 4));
  CK(dalloc(j, (char**)&P.relpos, PE * 4 * rb));
  if (k.morse) {
    P.ncells = k.ncell[0] * k.ncell[1] * k.ncell[2];
    CK(dalloc(j, &P.bin_count, (size_t)P.ncells));
    CK(dalloc(j, (char**)&P.bin, (size_t)P.ncells * kBinCap * sizeof(float4) + (size_t)P.ncells * sizeof(int)));
  }
  return PFGPU_OK;
}

static int build_fibrin(pfgpu_job* j, const pf_scene* s) {
  Fibrin& F = j->Fb;
  F.M = s->n_fib;
  F.law = s->fib_law;
  F.k = s->fib_k;
  F.mass = s->fib_mass;
  const size_t M = (size_t)F.M;
  const int nl = s->fib_ptr[M];
  CK(dupload(j, &F.X, s->fib_X, M));
  CK(dupload(j, &F.Y, s->fib_Y, M));
  CK(dupload(j, &F.Z, s->fib_Z, M));
  CK(dalloc(j, &F.V, 3 * M));
  CK(dalloc(j, &F.F, 3 * M));
  CK(dupload(j, &F.fixed, s->fib_fixed, M));
  CK(dupload(j, &F.ptr, s->fib_ptr, M + 1));
  CK(dupload(j, &F.nbr, s->fib_nbr, (size_t)nl));
  CK(dupload(j, &F.L0, s->fib_L0, (size_t)nl));
  F.f0 = (double)s->params[PF_P_F0];
  F.coupling = s->fib_coupling;
  if (F.coupling == PF_FIBCPL_PENALTY) {
    F.gamma = s->fib_gamma;
    F.node_mass = s->fib_node_mass;
    F.kappa = s->fib_kappa;
    CK(dalloc(j, &F.Ffsi, 3 * M));
    CK(dalloc(j, &F.Fs, 3 * M));
  }
  return PFGPU_OK;
}

// One coupled step.  With markers:
//   fork -> s1 membrane | s2 Morse | s3 fibrin
//           s0 flag the force bricks of this step (from the marker
//              positions), then bonds
//           sL the lattice pass over the bricks without force in the
//              previous step (the quiet pass: it needs no flag of this step;
//              the few bricks that gain a force now are done again after
//              the spreading) -- with PFGPU_QUIET_AHEAD=0 only; by
//              default it runs ahead, below
//   join -> s0: spread, lattice pass over the bricks flagged in this step or
//       the previous one, moments there, interpolation + advance.
//   Quiet pass ahead (the default): the quiet pass of step t+1 needs only
//   step t's output, complete once step t's flagged-brick pass is done, so
//   it runs then on sL, beside step t's moments and interpolation, and the
//   next step's force kernels run alone.  Its parity and first-step flag
//   come from counters the flagged-brick pass sets (Control::qstep, qfirst,
//   qskip); a prologue runs it for the current step when no step before did
//   (quiet_ready).
// The force kernels are latency-bound and occupy few SMs; the memory-bound
// lattice pass fills the rest.  It runs at low stream priority, so the force
// kernels' blocks, enqueued first, are dispatched before its blocks take the
// SMs.
//
// Pipelined (PFGPU_PIPELINE=1): the lattice splits into the near region of a
// step -- bricks within one brick in x and two rows in y and z of a brick
// flagged in the previous step -- and the far region.  No far brick is
// flagged in this step or the previous one as long as no marker's base node
// moves more than one node per step (the flagging checks it), and no far
// node pulls from a flagged node of the previous step.  So the far region
// of step t+1 depends only on the unflagged passes of step t, and its pass
// runs beside step t's spreading, flagged-brick pass, moments and
// interpolation:
//   sL: lattice pass over the near, unflagged bricks of step t
//   sF: near region of step t+1 (from the flags of step t), then, after
//       the sL pass, the far pass of step t+1
// Before the first pipelined step (after creation or a profile run) the far
// pass of the current step runs alone (prologue), with its near region
// taken from the occupancy bits.  On the 256x128x128 channel the far pass,
// memory-bound, slows the latency-bound tail kernels it runs beside more
// than it saves, so the serial schedule is the default.
// Reduced precision spreads each force part as soon as it exists (membrane
// and Morse forces on s1, bond forces on s0, fibrin forces on s3), so after
// the join only the flagged-brick pass, the moments and the interpolation
// remain.
// Without markers: the lattice pass over everything, then the step close.
static int far_prologue(pfgpu_job* j) {
  if (!j->pipeline || j->far_ready || !(j->has_pl || j->has_fb)) return PFGPU_OK;
  CK(lattice_far_counter(j->ctl, 1, j->s0));
  CK(lattice_near(j->L, j->ctl, 1, j->s0));
  CK(lattice_step_part(j->L, j->ctl, 3, nullptr, 0, j->s0));
  CK(lattice_far_counter(j->ctl, 0, j->s0));
  j->far_ready = true;
  return PFGPU_OK;
}

// The quiet pass's step counters (and, run ahead, the pass itself) for the
// current step, when no flagged-brick pass of the step before set them:
// after creation, a restore, profiled steps or fused batch steps.
static int quiet_prologue(pfgpu_job* j) {
  if (j->pipeline || j->quiet_ready || !(j->has_pl || j->has_fb)) return PFGPU_OK;
  CK(lattice_quiet_prologue(j->ctl, j->s0));
  if (j->quiet_ahead) CK(lattice_step_part(j->L, j->ctl, 5, nullptr, 0, j->s0));
  j->quiet_ready = true;
  return PFGPU_OK;
}

static int quiet_join(pfgpu_job* j) {
  if (!j->q_pending) return PFGPU_OK;
  CK(cudaStreamWaitEvent(j->s0, j->ev_q, 0));
  j->q_pending = false;
  return PFGPU_OK;
}

// fibrin nodes the interpolation moves (markers); penalty-coupled nodes
// move with their own velocity
static Fibrin* marker_fibrin(Fibrin* Fb) { return Fb && Fb->coupling == PF_FIBCPL_MARKER ? Fb : nullptr; }

static int enqueue_step(pfgpu_job* j) {
  Platelets* Pl = j->has_pl ? &j->Pl : nullptr;
  Fibrin* Fb = j->has_fb ? &j->Fb : nullptr;
  const bool cells = Pl && Pl->k.morse && morse_uses_cells(Pl->k);
  int* bins = cells ? Pl->bin_count : nullptr;
  const int ncells = cells ? Pl->ncells : 0;
  int launches = 0;
  if (!Pl && !Fb) {
    CK(lattice_step_part(j->L, j->ctl, 0, nullptr, 0, j->s0));
    CK(interp_advance(j->L, Pl, Fb, j->ctl, j->detach_rate, j->seed, j->done_blocks, j->s0));
    j->launches_per_step = 2;
    return PFGPU_OK;
  }
  const bool pipe = j->pipeline;
  CK(cudaEventRecord(j->ev_fork, j->s0));
  CK(cudaStreamWaitEvent(j->s1, j->ev_fork, 0));
  CK(cudaStreamWaitEvent(j->s2, j->ev_fork, 0));
  CK(cudaStreamWaitEvent(j->s3, j->ev_fork, 0));
  // serial schedule: the lattice pass over the bricks without force in the
  // previous step starts at the fork, beside the flagging (part 5);
  // pipelined: the unflagged near bricks after the flags (part 4)
  const bool quiet = !pipe;
  const bool ahead = quiet && j->quiet_ahead;
  CK(flag_markers(j->L, Pl, Fb, j->ctl, j->s0, pipe, quiet));
  CK(cudaEventRecord(j->ev_flag, j->s0));
  CK(cudaStreamWaitEvent(j->sL, quiet ? j->ev_fork : j->ev_flag, 0));
  launches++;
  if (pipe) {
    CK(cudaStreamWaitEvent(j->sF, j->ev_flag, 0));
    CK(lattice_near(j->L, j->ctl, 0, j->sF));
    launches++;
  }
  // split: each force part is spread on its own stream as soon as it exists
  const bool split = spread_split(j->L);
  if (Pl) {
    CK(membrane_forces(*Pl, j->precision, j->ctl, j->s1));
    launches++;
    if (Pl->k.morse && Pl->k.P * Pl->k.E) {
      CK(morse_forces(*Pl, j->precision, j->ctl, j->s2));
      launches += 2;  // bounds + pairs, or bin sort + pairs
      CK(cudaEventRecord(j->ev2, j->s2));
      if (split) CK(cudaStreamWaitEvent(j->s1, j->ev2, 0));
    }
    if (split) {
      CK(spread_part(j->L, Pl, Fb, j->ctl, 0, j->s1));
      launches++;
    }
    if (Pl->k.nrec) {
      CK(bond_pass(*Pl, j->precision, j->ctl, j->s0));
      launches += 2;
      if (split) {
        CK(spread_part(j->L, Pl, Fb, j->ctl, 1, j->s0));
        launches++;
      }
    }
  }
  if (Fb) {
    CK(fibrin_forces(*Fb, j->precision, j->ctl, j->s3));
    launches++;
    if (split) {
      CK(spread_part(j->L, Pl, Fb, j->ctl, 2, j->s3));
      launches++;
    }
  }
  if (!ahead) {
    CK(lattice_step_part(j->L, j->ctl, pipe ? 4 : 5, nullptr, 0, j->sL));
    launches++;
  }
  CK(cudaEventRecord(j->evL, j->sL));
  if (pipe) {
    CK(cudaStreamWaitEvent(j->sF, j->evL, 0));
    CK(lattice_step_part(j->L, j->ctl, 3, nullptr, 0, j->sF));
    CK(lattice_far_counter(j->ctl, 0, j->sF));
    CK(cudaEventRecord(j->ev_far, j->sF));
    launches += 2;
  }
  CK(cudaEventRecord(j->ev1, j->s1));
  CK(cudaEventRecord(j->ev2, j->s2));
  CK(cudaEventRecord(j->ev3, j->s3));
  CK(cudaStreamWaitEvent(j->s0, j->evL, 0));
  if (j->q_pending) {
    // this step's quiet pass, run ahead by the step before
    CK(cudaStreamWaitEvent(j->s0, j->ev_q, 0));
    j->q_pending = false;
  }
  CK(cudaStreamWaitEvent(j->s0, j->ev1, 0));
  CK(cudaStreamWaitEvent(j->s0, j->ev2, 0));
  CK(cudaStreamWaitEvent(j->s0, j->ev3, 0));
  if (!split) {
    CK(spread_markers(j->L, Pl, Fb, j->ctl, j->s0));
    launches++;
  }
  CK(lattice_step_part(j->L, j->ctl, 2, bins, ncells, j->s0));
  launches++;
  if (ahead) {
    // the next step's quiet pass: it needs this step's output only
    CK(cudaEventRecord(j->ev_list, j->s0));
    CK(cudaStreamWaitEvent(j->sL, j->ev_list, 0));
    CK(lattice_step_part(j->L, j->ctl, 5, nullptr, 0, j->sL));
    CK(cudaEventRecord(j->ev_q, j->sL));
    launches++;
  }
  CK(lattice_moments_active(j->L, j->ctl, j->s0));
  launches++;
  if (Fb && Fb->coupling == PF_FIBCPL_PENALTY) {
    CK(fibrin_penalty_step(j->L, *Fb, j->precision, Pl ? (double)Pl->k.f0 : 1.0, j->ctl, j->s0));
    launches += 4;
  }
  CK(interp_advance(j->L, Pl, marker_fibrin(Fb), j->ctl, j->detach_rate, j->seed, j->done_blocks, j->s0));
  launches++;
  if (pipe) CK(cudaStreamWaitEvent(j->s0, j->ev_far, 0));
  if (ahead) j->q_pending = true;
  j->launches_per_step = launches;
  return PFGPU_OK;
}

// Same launches as enqueue_step, on one stream, with an event pair around
// each phase; the per-phase device times are summed over the steps.  "lbm"
// is both lattice passes (the flagged bricks' pass runs after the spreading).
static const char* kPhaseNames[] = {"flag",   "membrane", "morse", "fibrin", "bonds",
                                    "spread", "lbm",      "moments", "interp"};
constexpr int kNumPhases = 9;
static int profile_steps(pfgpu_job* j, int nsteps, double* ms) {
  Platelets* Pl = j->has_pl ? &j->Pl : nullptr;
  Fibrin* Fb = j->has_fb ? &j->Fb : nullptr;
  const int NPH = kNumPhases;
  std::vector<cudaEvent_t> ev((size_t)2 * NPH * nsteps, nullptr);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  cudaStream_t s = j->s0;
  auto rec = [&](int step, int ph, int end) { return cudaEventRecord(ev[((size_t)step * NPH + ph) * 2 + end], s); };
  const bool cells = Pl && Pl->k.morse && morse_uses_cells(Pl->k);
  const bool markers = Pl || Fb;
  for (int t = 0; t < nsteps; ++t) {
    CK(rec(t, 0, 0)); if (markers) CK(flag_markers(j->L, Pl, Fb, j->ctl, s, false, true)); CK(rec(t, 0, 1));
    CK(rec(t, 1, 0)); if (Pl) CK(membrane_forces(*Pl, j->precision, j->ctl, s)); CK(rec(t, 1, 1));
    CK(rec(t, 2, 0)); if (Pl && Pl->k.morse) CK(morse_forces(*Pl, j->precision, j->ctl, s)); CK(rec(t, 2, 1));
    CK(rec(t, 3, 0)); if (Fb) CK(fibrin_forces(*Fb, j->precision, j->ctl, s)); CK(rec(t, 3, 1));
    CK(rec(t, 4, 0)); if (Pl && Pl->k.nrec) CK(bond_pass(*Pl, j->precision, j->ctl, s)); CK(rec(t, 4, 1));
    CK(rec(t, 5, 0));
    if (markers && spread_split(j->L)) {
      for (int part = 0; part < 3; ++part) CK(spread_part(j->L, Pl, Fb, j->ctl, part, s));
    } else if (markers) {
      CK(spread_markers(j->L, Pl, Fb, j->ctl, s));
    }
    CK(rec(t, 5, 1));
    CK(rec(t, 6, 0));
    if (markers) {
      CK(lattice_quiet_prologue(j->ctl, s));
      CK(lattice_step_part(j->L, j->ctl, 5, nullptr, 0, s));
      CK(lattice_step_part(j->L, j->ctl, 2, cells ? Pl->bin_count : nullptr, cells ? Pl->ncells : 0, s));
    } else {
      CK(lattice_step_part(j->L, j->ctl, 0, nullptr, 0, s));
    }
    CK(rec(t, 6, 1));
    CK(rec(t, 7, 0)); if (markers) CK(lattice_moments_active(j->L, j->ctl, s)); CK(rec(t, 7, 1));
    CK(rec(t, 8, 0));
    if (Fb && Fb->coupling == PF_FIBCPL_PENALTY)
      CK(fibrin_penalty_step(j->L, *Fb, j->precision, Pl ? (double)Pl->k.f0 : 1.0, j->ctl, s));
    CK(interp_advance(j->L, Pl, marker_fibrin(Fb), j->ctl, j->detach_rate, j->seed, j->done_blocks, s));
    CK(rec(t, 8, 1));
  }
  CK(cudaStreamSynchronize(s));
  // these steps updated the whole lattice: the next pipelined step starts
  // with its own far pass, the next serial one with its own quiet pass
  j->far_ready = false;
  j->quiet_ready = false;
  for (int ph = 0; ph < NPH; ++ph) ms[ph] = 0;
  for (int t = 0; t < nsteps; ++t)
    for (int ph = 0; ph < NPH; ++ph) {
      float f = 0;
      CK(cudaEventElapsedTime(&f, ev[((size_t)t * NPH + ph) * 2], ev[((size_t)t * NPH + ph) * 2 + 1]));
      ms[ph] += f;
    }
  for (auto& e : ev) cudaEventDestroy(e);
  return PFGPU_OK;
}

static int control_status(const Control& c) {
  if (c.err) {
    char buf[128];
    snprintf(buf, sizeof buf, "device error bits 0x%x", c.err);
    return set_error(PFGPU_ERR_DEVICE, buf);
  }
  return c.done ? PFGPU_DONE : PFGPU_OK;
}
static int check_control(pfgpu_job* j) {
  Control c;
  CK(cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost));
  return control_status(c);
}

extern "C" {

size_t pfgpu_scene_device_bytes(const pf_scene* s, int precision) {
  if (!s) return 0;
  const size_t N = (size_t)s->nx * s->ny * s->nz;
  const size_t sb = store_bytes(precision), rb = real_bytes(precision);
  const size_t nbricks = (size_t)((s->nx + kBrickX - 1) / kBrickX) * s->ny * s->nz;
  size_t b = 2 * 19 * N * sb + 3 * N * 4 * rb + 6 * nbricks * 4 + 2 * nbricks;
  const size_t PE = (size_t)s->n_platelets * s->n_elem;
  b += PE * (4 * 8 + 6 * 8 + 3 * 8 + 6 * rb);
  b += (size_t)s->n_platelets * ((size_t)s->n_node * 3 + (size_t)s->n_tri * 4 + s->n_membrane) * rb;
  if (s->membrane_forces & PF_MEM_FEMBEND)
    b += (size_t)s->n_platelets * ((size_t)s->n_node * 12 + (size_t)s->n_tri * 4) * rb;
  const size_t NR = (size_t)s->n_platelets * s->n_rec;
  b += NR * 64 + 4 * (size_t)s->nx * s->ny * 4;
  if (s->morse) {
    const double rc = s->morse_intra[3] > s->morse_inter[3] ? s->morse_intra[3] : s->morse_inter[3];
    size_t nc = 1;
    const int n3[3] = {s->nx, s->ny, s->nz};
    for (int a = 0; a < 3; ++a) {
      int c = rc > 0 ? (int)std::floor(n3[a] * (double)s->dx / rc) : 1;
      nc *= (size_t)(c < 1 ? 1 : c);
    }
    b += nc * (kBinCap * 16 + 4);
  }
  b += (size_t)s->n_fib * 14 * 8;
  if (s->fib_coupling == PF_FIBCPL_PENALTY) b += (size_t)s->n_fib * 6 * 8;
  // topology tables (shared by the platelets), fibrin link lists, and the
  // small per-job buffers (control block, counters, bounds)
  if (s->n_platelets > 0 && s->n_elem > 0) {
    const size_t nsp = s->spring_ptr ? (size_t)s->spring_ptr[s->n_elem] : 0;
    b += (size_t)s->n_tri * 6 * 4 + (size_t)s->n_node * (4 + 40) + (size_t)s->n_membrane * 80 +
         ((size_t)s->n_elem + 1) * 4 + nsp * 12 + (size_t)s->n_platelets * ((size_t)s->n_tri * 8 + 64);
  }
  if (s->n_fib > 0) b += ((size_t)s->n_fib + 1) * 8 + (size_t)s->fib_ptr[s->n_fib] * 12;
  b += 64 * 1024;
  // transient staging of the caller's FP64 arrays, where the device cannot
  // read pageable host memory itself
  int dev = 0, pageable = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
    cudaGetLastError();
    pageable = 0;
  }
  if (!pageable) b += 19 * N * 8 + 4 * N * 8 + 3 * N * 8;
  return b;
}

int pfgpu_job_create(const pf_scene* s, int precision, double fp16_scale, pfgpu_job** out) {
  if (!out) return set_error(PFGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate(s, precision);
  if (rc) return rc;
  pfgpu_job* j = new pfgpu_job();
  j->precision = precision;
  j->detach_rate = s->detach_rate;
  j->seed = s->seed;
  auto fail = [&](int code) { destroy(j); return code; };
#define CKJ(call)                                                                               \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      set_error(e_ == cudaErrorMemoryAllocation ? PFGPU_ERR_NOMEM : PFGPU_ERR_CUDA,             \
                std::string(#call) + ": " + cudaGetErrorString(e_));                            \
      return fail(e_ == cudaErrorMemoryAllocation ? PFGPU_ERR_NOMEM : PFGPU_ERR_CUDA);          \
    }                                                                                           \
  } while (0)
  keep_pool_memory();
  int prio_low = 0, prio_high = 0;
  CKJ(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  CKJ(cudaStreamCreateWithPriority(&j->s0, cudaStreamNonBlocking, prio_high));
  CKJ(cudaStreamCreateWithPriority(&j->s1, cudaStreamNonBlocking, prio_high));
  CKJ(cudaStreamCreateWithPriority(&j->s2, cudaStreamNonBlocking, prio_high));
  CKJ(cudaStreamCreateWithPriority(&j->s3, cudaStreamNonBlocking, prio_high));
  CKJ(cudaStreamCreateWithPriority(&j->sL, cudaStreamNonBlocking, prio_low));
  CKJ(cudaStreamCreateWithPriority(&j->sF, cudaStreamNonBlocking, prio_low));
  CKJ(cudaEventCreateWithFlags(&j->ev_far, cudaEventDisableTiming));
  {
    const char* pl = getenv("PFGPU_PIPELINE");
    j->pipeline = pl && strcmp(pl, "1") == 0;
  }
  CKJ(cudaEventCreateWithFlags(&j->ev_flag, cudaEventDisableTiming));
  CKJ(cudaEventCreateWithFlags(&j->ev_list, cudaEventDisableTiming));
  CKJ(cudaEventCreateWithFlags(&j->ev_q, cudaEventDisableTiming));
  {
    // measured on the 256x128x128 channel with eight-step graphs: FP32
    // 0.2126 -> 0.1998 ms per step with the quiet pass ahead, FP16
    // 0.1822 -> 0.1755.  PFGPU_QUIET_AHEAD=0/1 overrides.
    const char* qa = getenv("PFGPU_QUIET_AHEAD");
    j->quiet_ahead = !j->pipeline && (qa ? strcmp(qa, "1") == 0 : true);
    const char* gk = getenv("PFGPU_GRAPH_STEPS");
    if (gk && atoi(gk) >= 1 && atoi(gk) <= 64) j->graph_k = atoi(gk);
  }
  CKJ(cudaEventCreateWithFlags(&j->evL, cudaEventDisableTiming));
  CKJ(cudaEventCreateWithFlags(&j->ev_fork, cudaEventDisableTiming));
  CKJ(cudaEventCreateWithFlags(&j->ev1, cudaEventDisableTiming));
  CKJ(cudaEventCreateWithFlags(&j->ev2, cudaEventDisableTiming));
  CKJ(cudaEventCreateWithFlags(&j->ev3, cudaEventDisableTiming));
  // lattice
  Lattice& L = j->L;
  L.precision = precision;
  L.k = lattice_const(s, fp16_scale, precision);
  {
    // PFGPU_IBM=boxes: FP32/FP16 platelet elements spread and interpolated
    // through per-platelet shared-memory node boxes (default: per marker,
    // which measured faster on the 50-platelet channel)
    const char* ibm = getenv("PFGPU_IBM");
    L.ibm_box = ibm && strcmp(ibm, "boxes") == 0;
    // PFGPU_SPREAD_LANES=1: one thread per marker in the reduced-precision
    // spreading (default four lanes per marker, measured faster)
    const char* sl = getenv("PFGPU_SPREAD_LANES");
    L.spread_lanes = sl && atoi(sl) == 1 ? 1 : 4;
  }
  const size_t N = (size_t)L.k.N;
  const size_t sb = store_bytes(precision), rb = real_bytes(precision);
  // populations: the initial-state pass writes every word of g[0], the
  // first step every word of g[1]
  CKJ(dalloc(j, (char**)&L.g[0], 19 * N * sb, false));
  CKJ(dalloc(j, (char**)&L.g[1], 19 * N * sb, false));
  CKJ(dalloc(j, (char**)&L.F[0], 4 * N * rb));
  CKJ(dalloc(j, (char**)&L.F[1], 4 * N * rb));
  CKJ(dalloc(j, (char**)&L.ubuf, 4 * N * rb));
  CKJ(dalloc(j, &L.flags[0], (size_t)L.k.nbricks));
  CKJ(dalloc(j, &L.flags[1], (size_t)L.k.nbricks));
  CKJ(dalloc(j, &L.list[0], (size_t)L.k.nbricks));
  CKJ(dalloc(j, &L.list[1], (size_t)L.k.nbricks));
  CKJ(dalloc(j, &L.mark, 2 * (size_t)L.k.nbricks));
  CKJ(dalloc(j, &L.near[0], (size_t)L.k.nbricks));
  CKJ(dalloc(j, &L.near[1], (size_t)L.k.nbricks));
  CKJ(dalloc(j, &j->ctl, 1));
  CKJ(dalloc(j, &j->done_blocks, 1));
  CKJ(dalloc(j, &j->scratch4, 4));
  Control c{};
  c.step = 0;
  c.done = 0;
  c.first = 1;
  c.qstep = 0;  // the quiet pass's counters describe the first step
  c.qfirst = 1;
  c.total_bond = 1;  // sem_initGPUKernel, semLB.cu:880
  CKJ(cudaMemcpyAsync(j->ctl, &c, sizeof c, cudaMemcpyHostToDevice, j->s0));
  if (s->n_platelets > 0 && s->n_elem > 0) {
    j->has_pl = true;
    rc = build_platelets(j, s);
    if (rc) return fail(rc);
    j->Pl.mem_items = membrane_items(j->Pl.k);
    CKJ(bin_elements(j->Pl, j->ctl, j->s0));
  }
  if (s->n_fib > 0) {
    j->has_fb = true;
    rc = build_fibrin(j, s);
    if (rc) return fail(rc);
  }
  // the initial lattice last: uploads from pageable host memory wait for the
  // stream, so the long initial-state pass goes after the small uploads
  {
    // initial populations: the scene's own, else the equilibrium of the
    // initial flow, built on the device in one pass that reads the caller's
    // arrays where they lie (no FP64 staging copy where the device can read
    // them: device, pinned or ATS-visible host memory)
    const float* mp = s->params;
    InitSource src{};
    src.zh = s->bc[2] == PF_BC_ZOUHE_SHEAR;
    std::vector<void*> staged;
    cudaError_t e = cudaSuccess;
    auto view = [&](const double* h, size_t count) -> const double* {
      if (!h || e != cudaSuccess) return nullptr;
      if (const void* v = device_view(h)) return static_cast<const double*>(v);
      void* d = nullptr;
      e = cudaMallocAsync(&d, count * sizeof(double), j->s0);
      if (e != cudaSuccess) return nullptr;
      staged.push_back(d);
      e = cudaMemcpyAsync(d, h, count * sizeof(double), cudaMemcpyHostToDevice, j->s0);
      return static_cast<const double*>(d);
    };
    src.F = view(s->F_init, 3 * N);
    if (s->f_init) {
      src.f = view(s->f_init, 19 * N);
      if (s->rho_init && s->u_init) {
        src.rho = view(s->rho_init, N);
        src.u = view(s->u_init, 3 * N);
      }
      float c = s->dx / s->dt;
      c = c / mp[PF_P_UMAX];
      float fq = mp[PF_P_F0] / mp[PF_P_RHO0];
      fq = fq / mp[PF_P_UMAX];
      fq = fq * mp[PF_P_UNIT];
      float uwf = mp[PF_P_SHEAR] * (float)(s->nz - 1);
      uwf = uwf * s->dx;
      uwf = uwf / mp[PF_P_UMAX];
      src.C = (double)c;
      src.Fo = (double)fq;
      src.dt = (double)s->dt;
      src.uw = (double)uwf;
    } else {
      src.u = view(s->u_init, 3 * N);
      src.rho = view(s->rho_init, N);
      src.shear = (double)mp[PF_P_SHEAR];
      src.umax = src.shear > 0 ? src.shear * (s->nz - 1) * (double)s->dx : (double)mp[PF_P_UMAX];
      src.dx = (double)s->dx;
      const float dxdt = s->dx / s->dt;
      src.C0 = (double)dxdt / src.umax;
      src.C02 = src.C0 * src.C0;
    }
    if (e == cudaSuccess) e = lattice_init(L, src, j->s0);
    if (e == cudaSuccess) e = lattice_configure(L);
    // the caller's arrays may be read by the device until the end of the
    // creation, which waits for s0; staging copies go back to the pool
    for (void* d : staged) cudaFreeAsync(d, j->s0);
    CKJ(e);
  }
  CKJ(mark_markers(j->L, j->has_pl ? &j->Pl : nullptr, j->has_fb ? &j->Fb : nullptr, j->s0));
  if (j->has_fb && j->Fb.coupling == PF_FIBCPL_PENALTY) CKJ(fibrin_penalty_init(j->L, j->Fb, j->s0));
  CKJ(cudaStreamSynchronize(j->s0));
  *out = j;
  return PFGPU_OK;
}

int pfgpu_job_step(pfgpu_job* j, int nsteps) {
  if (!j || nsteps < 0) return set_error(PFGPU_ERR_INVALID, "bad job or step count");
  if (nsteps > 0) {
    int rc = far_prologue(j);
    if (!rc) rc = quiet_prologue(j);
    if (rc) return rc;
  }
  for (int i = 0; i < nsteps; ++i) {
    int rc = enqueue_step(j);
    if (rc) return rc;
  }
  {
    int rc = quiet_join(j);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(j->s0));
  return check_control(j);
}

// A graph of k coupled steps (the last one's quiet pass run ahead joined
// at its end).
static int capture_steps(pfgpu_job* j, int k, cudaGraphExec_t* out) {
  {
    int rc = quiet_join(j);
    if (rc) return rc;
  }
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(j->s0, cudaStreamCaptureModeThreadLocal));
  int rc = PFGPU_OK;
  for (int i = 0; i < k && rc == PFGPU_OK; ++i) rc = enqueue_step(j);
  if (rc == PFGPU_OK) rc = quiet_join(j);
  j->q_pending = false;
  cudaError_t e = cudaStreamEndCapture(j->s0, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CK(e);
  // the kernels of one step, counted from the captured graph itself
  size_t nn = 0;
  e = cudaGraphGetNodes(g, nullptr, &nn);
  if (e == cudaSuccess && nn > 0) {
    std::vector<cudaGraphNode_t> nodes(nn);
    e = cudaGraphGetNodes(g, nodes.data(), &nn);
    int kernels = 0;
    for (size_t i = 0; e == cudaSuccess && i < nn; ++i) {
      cudaGraphNodeType t;
      e = cudaGraphNodeGetType(nodes[i], &t);
      if (e == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
    }
    if (e == cudaSuccess) j->launches_per_step = kernels / k;
  }
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    CK(e);
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  return PFGPU_OK;
}

int pfgpu_job_step_graph(pfgpu_job* j, int nsteps) {
  if (!j || nsteps < 0) return set_error(PFGPU_ERR_INVALID, "bad job or step count");
  // k-step graphs only where a step's quiet pass runs ahead of it, captured
  // on the first call (also with nsteps = 0); the one-step graph when a
  // call's step count leaves a remainder (or k = 1)
  const int k = j->quiet_ahead ? j->graph_k : 1;
  if (k > 1 && !j->graphK) {
    int rc = capture_steps(j, k, &j->graphK);
    if (rc) return rc;
  }
  if (!j->graph && (k == 1 || nsteps % k != 0)) {
    int rc = capture_steps(j, 1, &j->graph);
    if (rc) return rc;
  }
  if (nsteps > 0) {
    int rc = far_prologue(j);
    if (!rc) rc = quiet_prologue(j);
    if (rc) return rc;
  }
  int left = nsteps;
  if (k > 1)
    for (; left >= k; left -= k) CK(cudaGraphLaunch(j->graphK, j->s0));
  for (; left > 0; --left) CK(cudaGraphLaunch(j->graph, j->s0));
  CK(cudaStreamSynchronize(j->s0));
  return check_control(j);
}

int pfgpu_job_enqueue(pfgpu_job* j, int nsteps) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  if (!j->graph) {
    int rc = capture_steps(j, 1, &j->graph);
    if (rc) return rc;
  }
  if (nsteps > 0) {
    int rc = far_prologue(j);
    if (!rc) rc = quiet_prologue(j);
    if (rc) return rc;
  }
  for (int i = 0; i < nsteps; ++i) CK(cudaGraphLaunch(j->graph, j->s0));
  return PFGPU_OK;
}

int pfgpu_job_profile(pfgpu_job* j, int nsteps, double* ms_out) {
  if (!j || nsteps < 1 || !ms_out) return set_error(PFGPU_ERR_INVALID, "bad arguments");
  int rc = profile_steps(j, nsteps, ms_out);
  if (rc) return rc;
  return check_control(j);
}
const char* pfgpu_profile_phase_name(int i) { return (i >= 0 && i < kNumPhases) ? kPhaseNames[i] : ""; }
int pfgpu_profile_phase_count(void) { return kNumPhases; }

int pfgpu_job_sync(pfgpu_job* j) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  return check_control(j);
}

int pfgpu_job_set_stop(pfgpu_job* j, int64_t stop_step) {
  if (!j || stop_step < 0) return set_error(PFGPU_ERR_INVALID, "bad job or stop step");
  CK(cudaStreamSynchronize(j->s0));
  Control c;
  CK(cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost));
  c.stop = stop_step;
  // a job stopped at its old stop step runs on to a later one
  if (c.done == 2 && (stop_step == 0 || stop_step > c.step)) c.done = 0;
  if (c.done == 0 && stop_step > 0 && c.step >= stop_step) c.done = 2;
  CK(cudaMemcpy(j->ctl, &c, sizeof c, cudaMemcpyHostToDevice));
  return PFGPU_OK;
}

// status of a job from a copy of its control block (batch steps read all
// jobs' blocks with one copy)
int pfgpu_job_control_status_(const pfgpu_job* j, const Control* c) { return j ? control_status(*c) : PFGPU_ERR_INVALID; }

int64_t pfgpu_job_step_count(const pfgpu_job* j) {
  if (!j) return -1;
  Control c;
  if (cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return c.step;
}

int pfgpu_job_get_lattice(pfgpu_job* j, double* fIN, double* fOUT, double* rho, double* u, double* F) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  const size_t N = (size_t)j->L.k.N;
  Control c;
  CK(cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost));
  // the download kernel writes each array where it lies when the device can
  // reach it (device, pinned or ATS-visible host memory), else into a device
  // staging buffer copied back afterwards
  struct Out {
    double* host;
    size_t count;
    double* dev;
    bool staged;
  };
  Out o[5] = {{fIN, 19 * N, nullptr, false}, {fOUT, 19 * N, nullptr, false}, {rho, N, nullptr, false},
              {u, 3 * N, nullptr, false}, {F, 3 * N, nullptr, false}};
  cudaError_t e = cudaSuccess;
  for (auto& x : o) {
    if (!x.host || e != cudaSuccess) continue;
    x.dev = static_cast<double*>(device_view(x.host));
    if (!x.dev) {
      e = cudaMalloc(&x.dev, x.count * sizeof(double));
      x.staged = e == cudaSuccess;
    }
  }
  if (e == cudaSuccess) e = lattice_download(j->L, j->ctl, c.step, o[0].dev, o[1].dev, o[2].dev, o[3].dev, o[4].dev, j->s0);
  for (auto& x : o)
    if (e == cudaSuccess && x.staged)
      e = cudaMemcpyAsync(x.host, x.dev, x.count * sizeof(double), cudaMemcpyDeviceToHost, j->s0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(j->s0);
  for (auto& x : o)
    if (x.staged) cudaFree(x.dev);
  CK(e);
  return PFGPU_OK;
}

int pfgpu_job_get_fields(pfgpu_job* j, int stride, float* rho, float* ux, float* uy, float* uz, int dims[3]) {
  if (!j || stride < 1) return set_error(PFGPU_ERR_INVALID, "bad job or stride");
  const int mx = (j->L.k.nx + stride - 1) / stride, my = (j->L.k.ny + stride - 1) / stride,
            mz = (j->L.k.nz + stride - 1) / stride;
  if (dims) {
    dims[0] = mx;
    dims[1] = my;
    dims[2] = mz;
  }
  if (!rho && !ux) return PFGPU_OK;
  if (ux && (!uy || !uz)) return set_error(PFGPU_ERR_INVALID, "ux given without uy, uz");
  CK(cudaStreamSynchronize(j->s0));
  Control c;
  CK(cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost));
  const size_t M = (size_t)mx * my * mz;
  float* d = nullptr;
  CK(cudaMalloc(&d, 4 * M * sizeof(float)));
  cudaError_t e = lattice_fields(j->L, c.step, stride, rho ? d : nullptr, ux ? d + M : nullptr,
                                 ux ? d + 2 * M : nullptr, ux ? d + 3 * M : nullptr, j->s0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(j->s0);
  if (e == cudaSuccess && rho) e = cudaMemcpy(rho, d, M * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && ux) e = cudaMemcpy(ux, d + M, M * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && ux) e = cudaMemcpy(uy, d + 2 * M, M * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && ux) e = cudaMemcpy(uz, d + 3 * M, M * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CK(e);
  return PFGPU_OK;
}

int pfgpu_job_get_elements(pfgpu_job* j, double* X, double* Y, double* RY, double* Z, double* V, double* F) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  if (!j->has_pl) return PFGPU_OK;
  const size_t PE = (size_t)j->Pl.k.P * j->Pl.k.E;
  if (X) CK(cudaMemcpy(X, j->Pl.X, PE * 8, cudaMemcpyDeviceToHost));
  if (Y) CK(cudaMemcpy(Y, j->Pl.Y, PE * 8, cudaMemcpyDeviceToHost));
  if (RY) CK(cudaMemcpy(RY, j->Pl.RY, PE * 8, cudaMemcpyDeviceToHost));
  if (Z) CK(cudaMemcpy(Z, j->Pl.Z, PE * 8, cudaMemcpyDeviceToHost));
  if (V) CK(cudaMemcpy(V, j->Pl.V, 3 * PE * 8, cudaMemcpyDeviceToHost));
  if (F) CK(cudaMemcpy(F, j->Pl.Ftot, 3 * PE * 8, cudaMemcpyDeviceToHost));
  return PFGPU_OK;
}

int pfgpu_job_get_bonds(pfgpu_job* j, int* rec_state, int* vwf, int* total_bond) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  if (total_bond) {
    Control c;
    CK(cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost));
    *total_bond = c.total_bond;
  }
  if (!j->has_pl) return PFGPU_OK;
  const size_t NR = (size_t)j->Pl.k.P * j->Pl.k.nrec;
  if (rec_state && NR) CK(cudaMemcpy(rec_state, j->Pl.rec_state, 3 * NR * 4, cudaMemcpyDeviceToHost));
  if (vwf) CK(cudaMemcpy(vwf, j->Pl.vwf, (size_t)4 * j->L.k.nx * j->L.k.ny * 4, cudaMemcpyDeviceToHost));
  return PFGPU_OK;
}

int pfgpu_job_get_fibrin(pfgpu_job* j, double* X, double* Y, double* Z, double* V, double* F) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  if (!j->has_fb) return PFGPU_OK;
  const size_t M = (size_t)j->Fb.M;
  if (X) CK(cudaMemcpy(X, j->Fb.X, M * 8, cudaMemcpyDeviceToHost));
  if (Y) CK(cudaMemcpy(Y, j->Fb.Y, M * 8, cudaMemcpyDeviceToHost));
  if (Z) CK(cudaMemcpy(Z, j->Fb.Z, M * 8, cudaMemcpyDeviceToHost));
  if (V) CK(cudaMemcpy(V, j->Fb.V, 3 * M * 8, cudaMemcpyDeviceToHost));
  if (F) CK(cudaMemcpy(F, j->Fb.F, 3 * M * 8, cudaMemcpyDeviceToHost));
  return PFGPU_OK;
}

int pfgpu_job_get_membrane(pfgpu_job* j, double* S_V, double* km) {
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  if (!j->has_pl) return PFGPU_OK;
  const PlateletConst& k = j->Pl.k;
  if (S_V) CK(cudaMemcpy(S_V, j->Pl.SV, (size_t)k.P * 2 * 8, cudaMemcpyDeviceToHost));
  if (km) {
    const size_t n = (size_t)k.P * k.Em;
    if (j->precision == PF_PREC_FP64) {
      CK(cudaMemcpy(km, j->Pl.km, n * 8, cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> tmp(n);
      CK(cudaMemcpy(tmp.data(), j->Pl.km, n * 4, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n; ++i) km[i] = tmp[i];
    }
  }
  return PFGPU_OK;
}

int pfgpu_job_conservation(pfgpu_job* j, double out[4]) {
  if (!j || !out) return set_error(PFGPU_ERR_INVALID, "bad arguments");
  CK(cudaStreamSynchronize(j->s0));
  Control c;
  CK(cudaMemcpy(&c, j->ctl, sizeof c, cudaMemcpyDeviceToHost));
  CK(lattice_conservation(j->L, c.step, j->scratch4, j->s0));
  CK(cudaMemcpyAsync(out, j->scratch4, 4 * sizeof(double), cudaMemcpyDeviceToHost, j->s0));
  CK(cudaStreamSynchronize(j->s0));
  return PFGPU_OK;
}

size_t pfgpu_job_device_bytes(const pfgpu_job* j) { return j ? j->bytes : 0; }
int pfgpu_job_launches_per_step(const pfgpu_job* j) { return j ? j->launches_per_step : 0; }
// ------------------------------------------------------- state snapshots
// A snapshot is the byte image of every device buffer of the job, in
// allocation order, after a header: magic, format version, precision,
// buffer count and each buffer's size.  Buffers hold the whole state
// (populations of both parities, forces, moments, brick flags and lists,
// occupancy, element and fibrin state, bonds and vWF slots, the control
// block with the step counter and stop step), so a job restored from it
// continues exactly as the saved one would.  A job only accepts a snapshot
// of the same layout: created from the same scene sizes and precision.
namespace {
constexpr char kSnapMagic[8] = {'P', 'F', 'G', 'J', 'O', 'B', 'S', '1'};
constexpr uint32_t kSnapVersion = 1;
size_t snapshot_header_bytes(const pfgpu_job* j) { return 8 + 4 + 4 + 8 + 8 * j->allocs.size(); }
}  // namespace

size_t pfgpu_job_state_bytes(const pfgpu_job* j) {
  if (!j) return 0;
  size_t b = snapshot_header_bytes(j);
  for (size_t n : j->alloc_bytes) b += n;
  return b;
}

int pfgpu_job_save(pfgpu_job* j, void* buf, size_t bytes) {
  if (!j || !buf) return set_error(PFGPU_ERR_INVALID, "pfgpu_job_save: NULL job or buffer");
  if (bytes < pfgpu_job_state_bytes(j)) return set_error(PFGPU_ERR_INVALID, "pfgpu_job_save: buffer too small");
  CK(cudaStreamSynchronize(j->s0));
  unsigned char* p = static_cast<unsigned char*>(buf);
  std::memcpy(p, kSnapMagic, 8);
  const uint32_t ver = kSnapVersion, prec = (uint32_t)j->precision;
  const uint64_t n = j->allocs.size();
  std::memcpy(p + 8, &ver, 4);
  std::memcpy(p + 12, &prec, 4);
  std::memcpy(p + 16, &n, 8);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t b = j->alloc_bytes[i];
    std::memcpy(p + 24 + 8 * i, &b, 8);
  }
  size_t off = snapshot_header_bytes(j);
  for (size_t i = 0; i < n; ++i) {
    CK(cudaMemcpy(p + off, j->allocs[i], j->alloc_bytes[i], cudaMemcpyDeviceToHost));
    off += j->alloc_bytes[i];
  }
  return PFGPU_OK;
}

int pfgpu_job_restore(pfgpu_job* j, const void* buf, size_t bytes) {
  if (!j || !buf) return set_error(PFGPU_ERR_INVALID, "pfgpu_job_restore: NULL job or buffer");
  const unsigned char* p = static_cast<const unsigned char*>(buf);
  if (bytes < snapshot_header_bytes(j) || std::memcmp(p, kSnapMagic, 8) != 0)
    return set_error(PFGPU_ERR_INVALID, "pfgpu_job_restore: not a job snapshot");
  uint32_t ver = 0, prec = 0;
  uint64_t n = 0;
  std::memcpy(&ver, p + 8, 4);
  std::memcpy(&prec, p + 12, 4);
  std::memcpy(&n, p + 16, 8);
  if (ver != kSnapVersion) return set_error(PFGPU_ERR_INVALID, "pfgpu_job_restore: snapshot format version differs");
  if (prec != (uint32_t)j->precision || n != j->allocs.size())
    return set_error(PFGPU_ERR_INVALID, "pfgpu_job_restore: snapshot of a job of another precision or layout");
  for (size_t i = 0; i < n; ++i) {
    uint64_t b = 0;
    std::memcpy(&b, p + 24 + 8 * i, 8);
    if (b != j->alloc_bytes[i])
      return set_error(PFGPU_ERR_INVALID, "pfgpu_job_restore: snapshot of a job of other sizes");
  }
  if (bytes < pfgpu_job_state_bytes(j)) return set_error(PFGPU_ERR_INVALID, "pfgpu_job_restore: snapshot truncated");
  CK(cudaStreamSynchronize(j->s0));
  size_t off = snapshot_header_bytes(j);
  for (size_t i = 0; i < n; ++i) {
    CK(cudaMemcpy(j->allocs[i], p + off, j->alloc_bytes[i], cudaMemcpyHostToDevice));
    off += j->alloc_bytes[i];
  }
  j->far_ready = false;
  j->quiet_ready = false;
  return PFGPU_OK;
}

const char* pfgpu_job_lbm_kernel(const pfgpu_job* j) {
  if (!j) return "";
  return lattice_pass_name(j->L);
}
void pfgpu_job_destroy(pfgpu_job* j) {
  if (j && j->s0) cudaStreamSynchronize(j->s0);
  destroy(j);
}

const char* pfgpu_last_error(void) {
  if (!g_last_error.empty()) return g_last_error.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_last_error_global.c_str();
}
int pfgpu_version(void) { return 100; }

void* pfgpu_host_alloc(size_t bytes) {
  void* p = nullptr;
  const cudaError_t e = cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocMapped | cudaHostAllocPortable);
  if (e != cudaSuccess) {
    set_error(e == cudaErrorMemoryAllocation ? PFGPU_ERR_NOMEM : PFGPU_ERR_CUDA,
              std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    return nullptr;
  }
  return p;
}
void pfgpu_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

void pfgpu_receptor_uniforms(uint64_t seed, int64_t step, int64_t receptor, double out[2]) {
  receptor_uniforms(seed, step, receptor, out[0], out[1]);
}
double pfgpu_detach_uniform(uint64_t seed, int64_t step) { return detach_uniform(seed, step); }

// internal accessors for the batch and drop-in layers
cudaStream_t pfgpu_job_stream_(pfgpu_job* j) { return j->s0; }
// The job's handles for a fused batch step; returns 0 when the job cannot
// take part (FP64, platelet boxes, the pipelined schedule, cell-list Morse,
// or a platelet too large for the item-parallel membrane kernel).
int pfgpu_job_batch_desc_(pfgpu_job* j, BatchDesc* d, int* precision, int* fast) {
  if (j->precision == PF_PREC_FP64 || j->L.ibm_box || j->pipeline) return 0;
  if (j->has_pl && (!j->Pl.mem_items || (j->Pl.k.morse && morse_uses_cells(j->Pl.k)))) return 0;
  if (j->has_fb && j->Fb.coupling != PF_FIBCPL_MARKER) return 0;
  j->quiet_ready = false;  // fused steps run no quiet pass ahead
  d->L = j->L;
  d->Pl = j->has_pl ? j->Pl : Platelets();
  d->Fb = j->has_fb ? j->Fb : Fibrin();
  d->has_pl = j->has_pl;
  d->has_fb = j->has_fb;
  d->ctl = j->ctl;
  d->done_blocks = j->done_blocks;
  d->detach_rate = j->detach_rate;
  d->seed = j->seed;
  *precision = j->precision;
  *fast = fast_gather(j->L) ? 1 : 0;
  return 1;
}
void pfgpu_job_elem_dims_(const pfgpu_job* j, int* P, int* E, double* dt) {
  *P = j->has_pl ? j->Pl.k.P : 0;
  *E = j->has_pl ? j->Pl.k.E : 0;
  *dt = (double)j->L.k.dtf;
}
int pfgpu_job_control_(pfgpu_job* j, Control* out) {
  CK(cudaMemcpy(out, j->ctl, sizeof *out, cudaMemcpyDeviceToHost));
  return PFGPU_OK;
}

}  // extern "C"

int pfgpu_set_error_(int code, const char* msg) { return set_error(code, msg); }

extern "C" int pfgpu_job_get_cells(pfgpu_job* j, int* cell_of, int* counts, int* members, int* ncells3) {
  // Rebuilds the Morse cell lists from the current positions (binning +
  // per-cell sort by element id) and copies them out: the cell of every
  // element, the element count of every cell and each cell's members in
  // ascending element id ([ncells][count], packed in cell order).
  if (!j) return set_error(PFGPU_ERR_INVALID, "bad job");
  CK(cudaStreamSynchronize(j->s0));
  if (!j->has_pl || !j->Pl.k.morse) return set_error(PFGPU_ERR_UNSUPPORTED, "job has no Morse cell lists");
  Platelets& P = j->Pl;
  CK(bin_elements(P, j->ctl, j->s0));
  CK(sort_cell_bins(P, j->ctl, j->s0));
  CK(cudaStreamSynchronize(j->s0));
  const int nc = P.ncells, PE = P.k.P * P.k.E;
  std::vector<int> cnt(nc);
  std::vector<float4> bins((size_t)nc * kBinCap);
  CK(cudaMemcpy(cnt.data(), P.bin_count, nc * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(bins.data(), P.bin, bins.size() * sizeof(float4), cudaMemcpyDeviceToHost));
  size_t off = 0;
  for (int c = 0; c < nc; ++c) {
    const int n = cnt[c] < kBinCap ? cnt[c] : kBinCap;
    if (counts) counts[c] = cnt[c];
    for (int q = 0; q < n; ++q) {
      int g;
      std::memcpy(&g, &bins[(size_t)c * kBinCap + q].w, sizeof g);
      if (members) members[off] = g;
      if (cell_of && g >= 0 && g < PE) cell_of[g] = c;
      off++;
    }
  }
  if (ncells3) { ncells3[0] = P.k.ncell[0]; ncells3[1] = P.k.ncell[1]; ncells3[2] = P.k.ncell[2]; }
  return check_control(j);
}
