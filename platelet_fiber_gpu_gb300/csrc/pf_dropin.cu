// pf_dropin.cu -- the reference's C entry points (semLB.cu) over the job API.
//
// The reference driver (gpuSEM_LB.c) allocates a fluid, an SEM and a fibrin
// handle, uploads host arrays into each (fluid_initGPUKernel aFlag=1,
// sem_initGPUKernel, fiber_init_GPUKernel), then per step calls
// sem_invokeGPUKernel_Force (detach test + membrane forces) followed by
// fluid_invokeGPUKernel (bonds, spreading, lattice, interpolation, position
// update), and copies state back with fluid_initGPUKernel aFlag=0,
// sem_copyGPUKernel and fiber_copy_GPUKernel.
//
// Here the handles hold the uploaded host arrays in the job's scene layouts;
// the first fluid_invokeGPUKernel builds one pfgpu_job from the fluid handle,
// the SEM handle it is given and the fibrin handle attached to the fluid
// handle, and every invoke advances that job.  The copy calls read the job
// back into the reference's host layouts.  Functions return nothing, like the
// reference; failures are recorded for pfgpu_last_error().
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "pf_internal.h"

using namespace pf;

namespace {

std::mutex g_default_mu;
int g_default_precision = PF_PREC_FP64;
double g_default_fp16_scale = 0.0;

struct DropFluid;

struct DropFiber {
  int maxNodes = 0, maxLinks = 0, maxConn = 0;
  double dt = 0;
  int law = PF_FIB_HOOKE;
  double k = 0.5, mass = 1.0;
  std::vector<int> fixed, ptr, nbr;
  std::vector<double> X, Y, Z, L0;
  bool ready = false;
  DropFluid* fluid = nullptr;
};

struct DropSem {
  int maxCells = 0, maxElements = 0, SurfElem = 0, newnode = 0, R = 0;
  float dt = 0;
  double S0_all = 0, V0 = 0;
  float params[100] = {};
  int numOfCells = 0;
  int n_membrane = 0;
  std::vector<double> X, Y, RY, Z;  // [P][E]
  std::vector<int> tri, node_ntri, ring, sp_ptr, sp_nbr;
  std::vector<double> sp_L0, S0, S0all, V0v;
  std::vector<int> rec_tri, rec_state;  // [P][n_rec], [P][n_rec][3]
  std::vector<float> r1, r2;            // [P][n_rec]
  double gama = 0;
  bool ready = false, done = false;
  DropFluid* fluid = nullptr;
};

struct DropFluid {
  float dt = 0, dx = 0;
  int nx = 0, ny = 0, nz = 0;
  float params[100] = {};
  bool have_params = false, ready = false;
  std::vector<double> f, u, rho, F;  // [19][N], [3][N], [N], [3][N]
  std::vector<int> vwf;              // [4][ny][nx]
  int precision = PF_PREC_FP64;
  double fp16_scale = 0.0;
  DropFiber* fiber = nullptr;
  DropSem* sem = nullptr;
  pfgpu_job* job = nullptr;
};

size_t nodes(const DropFluid* g) { return (size_t)g->nx * g->ny * g->nz; }

// Builds the job from the handles (first invoke).  The receptor and detach
// uniforms come from the counter-based stream of `seed`.
int build_job(DropFluid* g, DropSem* s, uint64_t seed) {
  pf_scene sc;
  std::memset(&sc, 0, sizeof sc);
  sc.nx = g->nx; sc.ny = g->ny; sc.nz = g->nz;
  sc.dx = g->dx; sc.dt = g->dt;
  // the model parameter table is the one sem_allocGPUKernel uploads
  // (semLB.cu:855); a fluid-only run uses fluid_initGPUKernel's
  std::memcpy(sc.params, s ? s->params : g->params, sizeof sc.params);
  // the reference's channel: periodic x and y, Zou/He walls on z, IBM
  // y-periodic image (LB_kernel.cu:395-780, :1419-1642)
  sc.bc[0] = PF_BC_PERIODIC; sc.bc[1] = PF_BC_PERIODIC; sc.bc[2] = PF_BC_ZOUHE_SHEAR;
  sc.ibm_wrap[0] = 0; sc.ibm_wrap[1] = 1; sc.ibm_wrap[2] = 0;
  if (!g->ready) return report_error(PFGPU_ERR_INVALID, "fluid_invokeGPUKernel before fluid_initGPUKernel(aFlag=1)");
  sc.f_init = g->f.data();
  sc.u_init = g->u.data();
  sc.rho_init = g->rho.data();
  sc.F_init = g->F.data();
  sc.vwf = g->vwf.data();
  sc.seed = seed;
  if (s) {
    if (!s->ready) return report_error(PFGPU_ERR_INVALID, "fluid_invokeGPUKernel before sem_initGPUKernel");
    sc.n_platelets = s->numOfCells;
    sc.n_elem = s->maxElements;
    sc.n_membrane = s->n_membrane;
    sc.n_tri = s->SurfElem;
    sc.n_node = s->newnode;
    sc.tri = s->tri.data();
    sc.node_ntri = s->node_ntri.data();
    sc.ring = s->ring.data();
    sc.spring_ptr = s->sp_ptr.data();
    sc.spring_nbr = s->sp_nbr.data();
    sc.spring_L0 = s->sp_L0.data();
    sc.S0 = s->S0.data();
    sc.S0_all = s->S0all.data();
    sc.V0 = s->V0v.data();
    sc.X = s->X.data(); sc.Y = s->Y.data(); sc.RY = s->RY.data(); sc.Z = s->Z.data();
    sc.membrane_forces = PF_MEM_ALL;
    sc.n_rec = s->SurfElem * s->R;
    sc.rec_tri = s->rec_tri.data();
    sc.rec_r1 = s->r1.data();
    sc.rec_r2 = s->r2.data();
    sc.rec_state = s->rec_state.data();
    sc.bond_model = PF_BOND_BELL;
    sc.detach_rate = s->gama;
  }
  DropFiber* fb = g->fiber;
  if (fb && fb->ready) {
    sc.n_fib = fb->maxNodes;
    sc.fib_X = fb->X.data(); sc.fib_Y = fb->Y.data(); sc.fib_Z = fb->Z.data();
    sc.fib_fixed = fb->fixed.data();
    sc.fib_ptr = fb->ptr.data();
    sc.fib_nbr = fb->nbr.data();
    sc.fib_L0 = fb->L0.data();
    sc.fib_law = fb->law;
    sc.fib_k = fb->k;
    sc.fib_mass = fb->mass;
  }
  return pfgpu_job_create(&sc, g->precision, g->fp16_scale, &g->job);
}

}  // namespace

extern "C" {

int pfgpu_set_default_precision(int precision, double fp16_scale) {
  if (precision < PF_PREC_FP64 || precision > PF_PREC_FP16) return report_error(PFGPU_ERR_INVALID, "bad precision");
  std::lock_guard<std::mutex> lk(g_default_mu);
  g_default_precision = precision;
  g_default_fp16_scale = fp16_scale;
  return PFGPU_OK;
}

// ------------------------------------------------------------------ fluid
void* fluid_allocGPUKernel(void* model, float dt, float dx, int width, int height, int depth) {
  (void)model;
  if (width < 1 || height < 1 || depth < 3) {
    report_error(PFGPU_ERR_INVALID, "fluid_allocGPUKernel: bad lattice size");
    return nullptr;
  }
  DropFluid* g = new DropFluid();
  g->dt = dt; g->dx = dx; g->nx = width; g->ny = height; g->nz = depth;
  std::lock_guard<std::mutex> lk(g_default_mu);
  g->precision = g_default_precision;
  g->fp16_scale = g_default_fp16_scale;
  return g;
}

void fluid_initGPUKernel(void* model, void* gv, int aFlag, float* hostParameters, void** fIN, void** fOUT, void* ux,
                         void* uy, void* uz, void* rho, void* obstacle, void* Fx, void* Fy, void* Fz, void* vWFbond) {
  (void)model;
  (void)obstacle;  // the Zou/He planes are the only obstacles (reference bc kernels)
  DropFluid* g = static_cast<DropFluid*>(gv);
  if (!g) { report_error(PFGPU_ERR_INVALID, "fluid_initGPUKernel: NULL handle"); return; }
  const size_t N = nodes(g);
  if (aFlag) {
    if (hostParameters) { std::memcpy(g->params, hostParameters, sizeof g->params); g->have_params = true; }
    g->f.assign(19 * N, 0.0);
    for (int d = 0; d < 19; ++d)
      if (fIN && fIN[d]) std::memcpy(&g->f[d * N], fIN[d], N * sizeof(double));
    g->u.assign(3 * N, 0.0);
    g->rho.assign(N, 1.0);
    g->F.assign(3 * N, 0.0);
    if (ux) std::memcpy(&g->u[0], ux, N * sizeof(double));
    if (uy) std::memcpy(&g->u[N], uy, N * sizeof(double));
    if (uz) std::memcpy(&g->u[2 * N], uz, N * sizeof(double));
    if (rho) std::memcpy(g->rho.data(), rho, N * sizeof(double));
    if (Fx) std::memcpy(&g->F[0], Fx, N * sizeof(double));
    if (Fy) std::memcpy(&g->F[N], Fy, N * sizeof(double));
    if (Fz) std::memcpy(&g->F[2 * N], Fz, N * sizeof(double));
    g->vwf.assign((size_t)4 * g->nx * g->ny, -1);
    if (vWFbond) std::memcpy(g->vwf.data(), vWFbond, g->vwf.size() * sizeof(int));
    g->ready = true;
    if (g->job) {  // a new upload restarts the simulation
      pfgpu_job_destroy(g->job);
      g->job = nullptr;
    }
    return;
  }
  // download: the job's state, or the uploaded arrays before any step
  std::vector<double> f(19 * N), fo(19 * N), r(N), u(3 * N), F(3 * N);
  if (g->job) {
    if (pfgpu_job_get_lattice(g->job, f.data(), fo.data(), r.data(), u.data(), F.data()) != PFGPU_OK) return;
  } else if (g->ready) {
    f = g->f; fo = g->f; r = g->rho; u = g->u; F = g->F;
  } else {
    report_error(PFGPU_ERR_INVALID, "fluid_initGPUKernel(aFlag=0) before any upload");
    return;
  }
  for (int d = 0; d < 19; ++d) {
    if (fIN && fIN[d]) std::memcpy(fIN[d], &f[d * N], N * sizeof(double));
    if (fOUT && fOUT[d]) std::memcpy(fOUT[d], &fo[d * N], N * sizeof(double));
  }
  if (ux) std::memcpy(ux, &u[0], N * sizeof(double));
  if (uy) std::memcpy(uy, &u[N], N * sizeof(double));
  if (uz) std::memcpy(uz, &u[2 * N], N * sizeof(double));
  if (rho) std::memcpy(rho, r.data(), N * sizeof(double));
  if (Fx) std::memcpy(Fx, &F[0], N * sizeof(double));
  if (Fy) std::memcpy(Fy, &F[N], N * sizeof(double));
  if (Fz) std::memcpy(Fz, &F[2 * N], N * sizeof(double));
  if (vWFbond && g->job) {
    DropSem* s = g->sem;
    const size_t nr = s ? (size_t)s->numOfCells * s->SurfElem * s->R * 3 : 0;
    std::vector<int> st(nr > 0 ? nr : 3);
    int tot = 0;
    pfgpu_job_get_bonds(g->job, s ? st.data() : nullptr, static_cast<int*>(vWFbond), &tot);
  }
}

void fluid_invokeGPUKernel(void* model, void* gv, void* g_SEM, double* randNum, void* r, int timeSteps) {
  (void)model;
  (void)randNum;  // receptor uniforms come from the seeded counter-based stream
  DropFluid* g = static_cast<DropFluid*>(gv);
  DropSem* s = static_cast<DropSem*>(g_SEM);
  if (!g) { report_error(PFGPU_ERR_INVALID, "fluid_invokeGPUKernel: NULL handle"); return; }
  if (timeSteps < 0) { report_error(PFGPU_ERR_INVALID, "fluid_invokeGPUKernel: negative step count"); return; }
  if (!g->job) {
    g->sem = s;
    if (s) s->fluid = g;
    // r replaces the reference's gsl_rng*: a pfgpu_uniform_source whose seed
    // keys the stream; NULL takes the parameter table's SEED
    const pfgpu_uniform_source* src = static_cast<const pfgpu_uniform_source*>(r);
    const float* tab = s ? s->params : g->params;
    const uint64_t seed = src ? src->seed : (uint64_t)tab[PF_P_SEED];
    if (build_job(g, s, seed) != PFGPU_OK) return;
  }
  if (s && s->done) return;
  const int rc = pfgpu_job_step_graph(g->job, timeSteps);
  if (rc == PFGPU_DONE && s) s->done = true;
}

void fluid_releaseGPUKernel(void* model, void* gv) {
  (void)model;
  DropFluid* g = static_cast<DropFluid*>(gv);
  if (!g) return;
  if (g->job) pfgpu_job_destroy(g->job);
  if (g->sem && g->sem->fluid == g) g->sem->fluid = nullptr;
  if (g->fiber && g->fiber->fluid == g) g->fiber->fluid = nullptr;
  delete g;
}

int pfgpu_fluid_attach_fiber(void* gv, void* fgv, int law, double k, double mass) {
  DropFluid* g = static_cast<DropFluid*>(gv);
  DropFiber* fb = static_cast<DropFiber*>(fgv);
  if (!g || !fb) return report_error(PFGPU_ERR_INVALID, "pfgpu_fluid_attach_fiber: NULL handle");
  if (law != PF_FIB_HOOKE && law != PF_FIB_WLC) return report_error(PFGPU_ERR_INVALID, "bad fibrin law");
  if (g->job) return report_error(PFGPU_ERR_INVALID, "attach the fibrin handle before the first invoke");
  g->fiber = fb;
  fb->fluid = g;
  fb->law = law;
  fb->k = k;
  fb->mass = mass;
  return PFGPU_OK;
}

// ------------------------------------------------------------------ SEM
void* sem_allocGPUKernel(void* model, int maxCells, int maxElements, int SurfElem, int newnode,
                         int numReceptorsPerElem, float dt, double S0_all, float* hostSEMparameters) {
  (void)model;
  if (maxCells < 1 || maxElements < 1 || SurfElem < 1 || newnode < 1 || numReceptorsPerElem < 0) {
    report_error(PFGPU_ERR_INVALID, "sem_allocGPUKernel: bad sizes");
    return nullptr;
  }
  DropSem* s = new DropSem();
  s->maxCells = maxCells; s->maxElements = maxElements; s->SurfElem = SurfElem; s->newnode = newnode;
  s->R = numReceptorsPerElem; s->dt = dt; s->S0_all = S0_all;
  if (hostSEMparameters) std::memcpy(s->params, hostSEMparameters, sizeof s->params);
  return s;
}

void sem_initGPUKernel(void* model, void* gv, int numOfCells, int* numOfElements, int SurfElem,
                       int numReceptorsPerElem, void* hostX_Ref, void* hostY_Ref, void* hostZ_Ref, void* hostX,
                       void* hostY, void* hostRY, void* hostZ, void* hostVX, void* hostVY, void* hostVZ,
                       void* hostFX, void* hostFY, void* hostFZ, void* hostType, void* hostBonds, void* triElem,
                       void* receptor_r1, void* receptor_r2, void* node_share_Elem, void* N, void* node_nbrElemNum,
                       void* node_nbr_nodes, void* S0, double V0, void* receptBond, void* randNum) {
  (void)model; (void)numOfElements; (void)hostX_Ref; (void)hostY_Ref; (void)hostZ_Ref; (void)hostRY;
  (void)hostVX; (void)hostVY; (void)hostVZ; (void)hostFX; (void)hostFY; (void)hostFZ; (void)hostType;
  (void)node_share_Elem; (void)N; (void)randNum;
  DropSem* s = static_cast<DropSem*>(gv);
  if (!s) { report_error(PFGPU_ERR_INVALID, "sem_initGPUKernel: NULL handle"); return; }
  if (numOfCells < 1 || numOfCells > s->maxCells || SurfElem != s->SurfElem || numReceptorsPerElem != s->R) {
    report_error(PFGPU_ERR_INVALID, "sem_initGPUKernel: sizes differ from sem_allocGPUKernel");
    return;
  }
  if (!hostX || !hostY || !hostZ || !hostBonds || !triElem || !node_nbrElemNum || !node_nbr_nodes || !S0) {
    report_error(PFGPU_ERR_INVALID, "sem_initGPUKernel: missing array");
    return;
  }
  const int P = numOfCells, E = s->maxElements, C = s->maxCells, T = s->SurfElem, R = s->R;
  s->numOfCells = P;
  s->V0 = V0;
  // elements: host [maxElements][maxCells] (cell fastest, gpuSEM_LB.c:749-779)
  // -> platelet-major [P][E]; RY starts as Y (semLB.cu:914 copies hostY)
  const double* hx = static_cast<const double*>(hostX);
  const double* hy = static_cast<const double*>(hostY);
  const double* hz = static_cast<const double*>(hostZ);
  s->X.resize((size_t)P * E); s->Y.resize((size_t)P * E); s->RY.resize((size_t)P * E); s->Z.resize((size_t)P * E);
  for (int c = 0; c < P; ++c)
    for (int e = 0; e < E; ++e) {
      const size_t src = (size_t)e * C + c, dst = (size_t)c * E + e;
      s->X[dst] = hx[src]; s->Y[dst] = hy[src]; s->RY[dst] = hy[src]; s->Z[dst] = hz[src];
    }
  // mesh: triangles [T][6]; the vertices are the elements 0..n_membrane-1
  const int* tr = static_cast<const int*>(triElem);
  s->tri.assign(tr, tr + (size_t)T * 6);
  int nm = 0;
  for (int t = 0; t < T; ++t)
    for (int i = 0; i < 3; ++i) nm = std::max(nm, tr[6 * t + i] + 1);
  s->n_membrane = nm;
  const int* nn = static_cast<const int*>(node_nbrElemNum);
  s->node_ntri.assign(nn, nn + s->newnode);
  const int* rg = static_cast<const int*>(node_nbr_nodes);
  s->ring.assign(rg, rg + (size_t)nm * 10);
  // springs: the dense bond table's entries above 1e-6 (sem_kernel.cu:355-389)
  const double* bl = static_cast<const double*>(hostBonds);
  s->sp_ptr.assign(E + 1, 0);
  s->sp_nbr.clear();
  s->sp_L0.clear();
  for (int e = 0; e < E; ++e) {
    for (int q = 0; q < E; ++q) {
      const double b = bl[(size_t)e * E + q];
      if (b > 1e-6) { s->sp_nbr.push_back(q); s->sp_L0.push_back(b); }
    }
    s->sp_ptr[e + 1] = (int)s->sp_nbr.size();
  }
  // rest areas per triangle, rest area and volume: one platelet template
  const double* s0 = static_cast<const double*>(S0);
  s->S0.resize((size_t)P * T);
  for (int c = 0; c < P; ++c) std::memcpy(&s->S0[(size_t)c * T], s0, T * sizeof(double));
  s->S0all.assign(P, s->S0_all);
  s->V0v.assign(P, V0);
  // receptors: r1/r2 [T][R]; receptor id t*R + j; bonds [3][R][T] (i, j, count)
  const int nrec = T * R;
  s->rec_tri.resize((size_t)P * nrec);
  s->r1.resize((size_t)P * nrec);
  s->r2.resize((size_t)P * nrec);
  s->rec_state.resize((size_t)P * nrec * 3);
  const float* f1 = static_cast<const float*>(receptor_r1);
  const float* f2 = static_cast<const float*>(receptor_r2);
  const int* rb = static_cast<const int*>(receptBond);
  for (int c = 0; c < P; ++c)
    for (int t = 0; t < T; ++t)
      for (int j = 0; j < R; ++j) {
        const size_t rid = (size_t)c * nrec + (size_t)t * R + j;
        s->rec_tri[rid] = t;
        s->r1[rid] = f1 ? f1[(size_t)t * R + j] : 0.f;
        s->r2[rid] = f2 ? f2[(size_t)t * R + j] : 0.f;
        for (int k = 0; k < 3; ++k)
          s->rec_state[rid * 3 + k] = rb ? rb[((size_t)k * R + j) * T + t] : (k < 2 ? -1 : 0);
      }
  s->ready = true;
  s->done = false;
}

void sem_invokeGPUKernel_Force(void* model, void* gv, int timeSteps, int* done, int* totalT, void* r, double gama) {
  (void)model; (void)timeSteps; (void)r;
  DropSem* s = static_cast<DropSem*>(gv);
  if (!s) { report_error(PFGPU_ERR_INVALID, "sem_invokeGPUKernel_Force: NULL handle"); return; }
  // the membrane, Morse and bond forces of a step are computed inside the
  // job's step (fluid_invokeGPUKernel); here the detach bookkeeping of
  // semLB.cu:451-460: the detach probability per step, done, step counter
  s->gama = gama;
  if (s->done) {
    if (done) *done = 1;
    return;
  }
  if (totalT) (*totalT)++;
}

void sem_copyGPUKernel(void* model, void* gv, void* hostX, void* hostY, void* hostRY, void* hostZ, void* hostVX,
                       void* hostVY, void* hostVZ, void* hostFX, void* hostFY, void* hostFZ, int timeSteps) {
  (void)model; (void)timeSteps;
  DropSem* s = static_cast<DropSem*>(gv);
  if (!s) { report_error(PFGPU_ERR_INVALID, "sem_copyGPUKernel: NULL handle"); return; }
  const int P = s->numOfCells, E = s->maxElements, C = s->maxCells;
  const size_t PE = (size_t)P * E;
  std::vector<double> X(PE), Y(PE), RY(PE), Z(PE), V(3 * PE, 0.0), F(3 * PE, 0.0);
  if (s->fluid && s->fluid->job) {
    if (pfgpu_job_get_elements(s->fluid->job, X.data(), Y.data(), RY.data(), Z.data(), V.data(), F.data()) != PFGPU_OK)
      return;
  } else {
    X = s->X; Y = s->Y; RY = s->RY; Z = s->Z;
  }
  auto put = [&](void* dst, const double* src) {
    if (!dst) return;
    double* d = static_cast<double*>(dst);
    for (int c = 0; c < P; ++c)
      for (int e = 0; e < E; ++e) d[(size_t)e * C + c] = src[(size_t)c * E + e];
  };
  put(hostX, X.data()); put(hostY, Y.data()); put(hostRY, RY.data()); put(hostZ, Z.data());
  put(hostVX, &V[0]); put(hostVY, &V[PE]); put(hostVZ, &V[2 * PE]);
  put(hostFX, &F[0]); put(hostFY, &F[PE]); put(hostFZ, &F[2 * PE]);
}

void sem_releaseGPUKernel(void* model, void* gv) {
  (void)model;
  DropSem* s = static_cast<DropSem*>(gv);
  if (!s) return;
  if (s->fluid && s->fluid->sem == s) s->fluid->sem = nullptr;
  delete s;
}

// ------------------------------------------------------------------ fibrin
void* fiber_allocGPUKernel(void* model, int maxNodes, int maxLinks, int max_N_conn_at_Node, double dt,
                           double* hostParameters) {
  (void)model; (void)hostParameters;
  if (maxNodes < 1 || maxLinks < 0 || max_N_conn_at_Node < 1) {
    report_error(PFGPU_ERR_INVALID, "fiber_allocGPUKernel: bad sizes");
    return nullptr;
  }
  DropFiber* fb = new DropFiber();
  fb->maxNodes = maxNodes; fb->maxLinks = maxLinks; fb->maxConn = max_N_conn_at_Node; fb->dt = dt;
  return fb;
}

void fiber_init_GPUKernel(void* model, void* fgv, void* NodeType, void* N_Conn_at_Node, void* Link_at_Node,
                          void* lAdjVer, void* linkLengths, void* linkLengths0, void* linkThick, void* X, void* V_X,
                          void* X0, void* F_X, void* Y, void* Y0, void* V_Y, void* F_Y, void* Z, void* Z0,
                          void* V_Z, void* F_Z) {
  (void)model; (void)linkLengths; (void)linkThick; (void)V_X; (void)X0; (void)F_X; (void)Y0; (void)V_Y;
  (void)F_Y; (void)Z0; (void)V_Z; (void)F_Z;
  DropFiber* fb = static_cast<DropFiber*>(fgv);
  if (!fb) { report_error(PFGPU_ERR_INVALID, "fiber_init_GPUKernel: NULL handle"); return; }
  if (!NodeType || !N_Conn_at_Node || !Link_at_Node || !lAdjVer || !linkLengths0 || !X || !Y || !Z) {
    report_error(PFGPU_ERR_INVALID, "fiber_init_GPUKernel: missing array");
    return;
  }
  const int M = fb->maxNodes, L = fb->maxLinks, K = fb->maxConn;
  const int* type = static_cast<const int*>(NodeType);
  const int* nconn = static_cast<const int*>(N_Conn_at_Node);
  const int* lan = static_cast<const int*>(Link_at_Node);  // [M][K] link ids (pad -100, fiber.cpp:380-384)
  const int* adj = static_cast<const int*>(lAdjVer);       // [L][2] link end nodes
  const double* l0 = static_cast<const double*>(linkLengths0);
  fb->X.assign(static_cast<const double*>(X), static_cast<const double*>(X) + M);
  fb->Y.assign(static_cast<const double*>(Y), static_cast<const double*>(Y) + M);
  fb->Z.assign(static_cast<const double*>(Z), static_cast<const double*>(Z) + M);
  fb->fixed.resize(M);
  for (int m = 0; m < M; ++m) fb->fixed[m] = type[m] == 1 ? 1 : 0;  // NodeType 1: fixed node
  // per-node link lists -> CSR of (neighbour node, rest length)
  fb->ptr.assign(M + 1, 0);
  fb->nbr.clear();
  fb->L0.clear();
  for (int m = 0; m < M; ++m) {
    const int c = std::min(std::max(nconn[m], 0), K);
    for (int q = 0; q < c; ++q) {
      const int l = lan[(size_t)m * K + q];
      if (l < 0 || l >= L) continue;
      const int a = adj[2 * l], b = adj[2 * l + 1];
      const int other = a == m ? b : a;
      if (other < 0 || other >= M) continue;
      fb->nbr.push_back(other);
      fb->L0.push_back(l0[l]);
    }
    fb->ptr[m + 1] = (int)fb->nbr.size();
  }
  fb->ready = true;
}

void fiber_copy_GPUKernel(void* model, void* fgv, void* X, void* V_X, void* X0, void* F_X, void* Y, void* Y0,
                          void* V_Y, void* F_Y, void* Z, void* Z0, void* V_Z, void* F_Z) {
  (void)model; (void)X0; (void)Y0; (void)Z0;
  DropFiber* fb = static_cast<DropFiber*>(fgv);
  if (!fb) { report_error(PFGPU_ERR_INVALID, "fiber_copy_GPUKernel: NULL handle"); return; }
  const int M = fb->maxNodes;
  std::vector<double> x(M), y(M), z(M), v(3 * (size_t)M, 0.0), f(3 * (size_t)M, 0.0);
  if (fb->fluid && fb->fluid->job) {
    if (pfgpu_job_get_fibrin(fb->fluid->job, x.data(), y.data(), z.data(), v.data(), f.data()) != PFGPU_OK) return;
  } else {
    x = fb->X; y = fb->Y; z = fb->Z;
  }
  auto put = [&](void* dst, const double* src) {
    if (dst) std::memcpy(dst, src, (size_t)M * sizeof(double));
  };
  put(X, x.data()); put(Y, y.data()); put(Z, z.data());
  put(V_X, &v[0]); put(V_Y, &v[M]); put(V_Z, &v[2 * (size_t)M]);
  put(F_X, &f[0]); put(F_Y, &f[M]); put(F_Z, &f[2 * (size_t)M]);
}

void fiber_release_GPUKernel(void* model, void* fgv) {
  (void)model;
  DropFiber* fb = static_cast<DropFiber*>(fgv);
  if (!fb) return;
  if (fb->fluid && fb->fluid->fiber == fb) fb->fluid->fiber = nullptr;
  delete fb;
}

}  // extern "C"
