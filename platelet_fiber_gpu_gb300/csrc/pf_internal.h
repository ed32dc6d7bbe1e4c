// pf_internal.h -- device-resident state of one coupled simulation and the
// launchers of its kernels.
//
// Layout in HBM (one job):
//   populations   2 x Store[19][N]      ping-pong, shifted g = f - w, SoA
//   lattice force 2 x Real4[N]          reference force units, only bricks
//                                       flagged active are read or non-zero
//   brick flags   2 x uint32[nbricks]   + active-brick lists (one brick =
//                                       32 x-nodes of one (y,z) row), and
//                                       2 x uint32[nbricks] occupancy bits
//   u buffer      Real4[N]              (rho-1, u/C) at active bricks; before
//                                       the first step: the initial rho-1, u/C
//   elements      double X,Y,RY,Z,V,F   positions stay FP64
//   membrane/Morse/bond/fibrin forces   one buffer each (concurrent kernels)
//   Morse cell bins float4[ncells][512] (cell-relative position, id)
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pf_common.cuh"

namespace pf {

struct alignas(32) D4 {
  double x, y, z, w;
};
template <class R>
struct R4T;
template <>
struct R4T<float> {
  using type = float4;
};
template <>
struct R4T<double> {
  using type = D4;
};
template <class R>
using R4 = typename R4T<R>::type;

// ------------------------------------------------------------------ lattice
struct LatticeConst {
  int nx, ny, nz, nbx, nbricks;
  long long N;
  int bc[3];
  int ibm_wrap[3];
  float dxf, dtf;
  double inv_dx;      // 1 / (double)dxf, so kernels divide by no double per thread
  double Lx, Ly;      // (double)nx * dxf, (double)ny * dxf: periodic lengths of the position update
  double C;           // float-rounded dx/dt/UMAX
  double omega;       // 1/tau
  double kcoll;       // F0/rho0/UMAX*UNIT (double chain) * dt / C
  double kmom;        // F0/rho0/UMAX*UNIT (float chain) * dt / C
  double body[3];     // body force, reference units
  double uw;          // top-wall velocity / C
  double fp16_scale;  // sigma of the FP16 store
  float hs[3], hinv[3];  // w * sigma and 1 / (w * sigma) for w = 1/3, 1/18, 1/36 (FP16 store)
  float isig;            // 1 / sigma (FP16 store)
  unsigned long long wait_ns;  // limit of a bounded device wait (1 s; PFGPU_WAIT_LIMIT_NS for tests)
  float dtT;          // dt / T0 (float, sem_kernel.cu:2106): position update factor
  // the float roundings of omega, kcoll, kmom, body, uw: reduced-precision
  // kernels read these instead of converting from double per thread (FP64
  // conversions use the narrow FP64 pipe of this GPU)
  float omega_f, kcoll_f, kmom_f, body_f[3], uw_f;
  int nobody;  // the body force is zero (in its float rounding)
};

struct Lattice {
  int precision = PF_PREC_FP64;
  LatticeConst k{};
  void* g[2] = {nullptr, nullptr};
  void* F[2] = {nullptr, nullptr};
  void* ubuf = nullptr;
  unsigned* flags[2] = {nullptr, nullptr};
  int* list[2] = {nullptr, nullptr};
  // marker occupancy, one bit per node (one 32-bit word per brick), two
  // buffers by step parity: the position update marks the next step's
  // buffer, the flagging reads this step's, the flagged-brick pass clears it
  unsigned* mark = nullptr;
  // near region per step parity: bricks within one brick (x) and two rows
  // (y, z) of a force brick of the previous step; the rest (far) is updated
  // by the pipelined far pass while the previous step's tail runs
  unsigned char* near[2] = {nullptr, nullptr};
  // reduced precision: spread/interpolate platelet elements through shared
  // per-platelet node boxes (1) or per marker with global atomics (0)
  int ibm_box = 0;
  int spread_lanes = 4;  // reduced-precision spreading: threads per marker (1 or 4)
  size_t bytes = 0;
  // row-staged step: rows per tile, tiles in flight per CTA, persistent grid
  // (rows_stages == 0: the direct-gather kernel is used)
  int rows_rpt = 0, rows_stages = -1, rows_grid = 0, rows_ds = 0;
  size_t rows_smem = 0;
};

// ------------------------------------------------------------------ markers
struct PlateletConst {
  int P, E, Em, T, NN, nrec;
  int mask;
  float kspring, ks, kv, kbend, f0, kf0, kr0, numrec;
  double dxd, dtd;
  double inv_f0;  // 1 / (double)f0
  float dxf, dtf, dtT;
  int bond_model;
  double p_on, p_off;
  uint64_t seed;
  int morse;
  double morse_intra[4], morse_inter[4];
  double morse_fc[2];  // F(cutoff) of the intra / inter parameter sets (force shift)
  int ncell[3];
  double cs[3];
  double L[3];
  int wrap[3];
  int nx, ny, nz;
};

struct Platelets {
  PlateletConst k{};
  // state (FP64)
  double *X = nullptr, *Y = nullptr, *RY = nullptr, *Z = nullptr;
  double* V = nullptr;     // [3][PE]
  double* Ftot = nullptr;  // [3][PE] total element force of the last step
  void* Fmem = nullptr;    // Real[3][PE] membrane forces
  double* Fmorse = nullptr;  // [3][PE]
  void* Fbond = nullptr;   // Real[3][PE]
  // topology (template)
  int *tri = nullptr, *node_ntri = nullptr, *node_tri = nullptr, *vert_local = nullptr, *ring = nullptr;
  int *sp_ptr = nullptr, *sp_nbr = nullptr;
  double *sp_L0 = nullptr, *S0 = nullptr, *S0_all = nullptr, *V0 = nullptr;
  // membrane scratch (Real)
  void *nN = nullptr, *nelem = nullptr, *S = nullptr, *km = nullptr;
  double* SV = nullptr;  // [P][2]
  void* fem = nullptr;   // Real [P][NN*12 + T*4]: FEM bending chain (PF_MEM_FEMBEND only)
  bool mem_items = false;  // FP32 membrane through the item-parallel kernel
  // receptors
  int *rec_tri = nullptr, *rec_state = nullptr, *vwf = nullptr;
  float *r1 = nullptr, *r2 = nullptr;
  void* rec_tmp = nullptr;  // per-receptor scratch of the bond pass
  // Morse bins
  int* bin_count = nullptr;
  void* bin = nullptr;  // float4 [ncells][kBinCap]: cell-relative position, element id
  int ncells = 0;
  double* bounds = nullptr;  // [P][4] centroid and bounding radius (Morse culling)
  void* relpos = nullptr;    // Real4 [P*E] element positions relative to their centroid
  size_t bytes = 0;
};

struct Fibrin {
  int M = 0;
  int law = PF_FIB_HOOKE;
  double k = 0.5, mass = 1.0;
  double *X = nullptr, *Y = nullptr, *Z = nullptr, *V = nullptr, *F = nullptr;
  int *fixed = nullptr, *ptr = nullptr, *nbr = nullptr;
  double* L0 = nullptr;
  size_t bytes = 0;
  // penalty coupling (PF_FIBCPL_PENALTY): node force of the step in lattice
  // units [3][M], and its reaction in reference force units, spread in the
  // next step [3][M]
  int coupling = PF_FIBCPL_MARKER;
  double gamma = 0, node_mass = 1, kappa = 1;
  double f0 = 1;  // the reference's force unit F0 (link forces are in it)
  double *Ffsi = nullptr, *Fs = nullptr;
  // the force the lattice receives at the nodes: the link forces (markers)
  // or the penalty reaction
  const double* spread_force() const { return coupling == PF_FIBCPL_PENALTY ? Fs : F; }
};

// ------------------------------------------------------------------ batches
// One job of a fused batch step: copies of the job's lattice, platelet and
// fibrin handles (device pointers and constants), read by the batch kernels.
struct BatchDesc {
  Lattice L;
  Platelets Pl;
  Fibrin Fb;
  int has_pl, has_fb;
  Control* ctl;
  unsigned* done_blocks;
  double detach_rate;
  uint64_t seed;
};
// Kernels of a fused batch step; each runs over all jobs of the batch, a job
// owning the CTAs [start[j], start[j+1]) of the launch.
enum BatchKernel : int {
  BK_FLAG = 0, BK_LBM_UNFLAGGED, BK_MEMBRANE, BK_BOUNDS, BK_MORSE, BK_BOND_PREP, BK_BOND_RESOLVE, BK_FIBRIN,
  BK_SPREAD_ELEM, BK_SPREAD_BOND, BK_SPREAD_FIB, BK_LBM_FLAGGED, BK_MOMENTS, BK_INTERP, BK_COUNT
};
// Block and tile shapes of a fused batch step (picked by the batch autotuner)
struct BatchTune {
  int lbm_rows;        // groups of four bricks (kLbmBlock nodes) per CTA, unflagged lattice pass
  int list_per_sm;     // CTAs per SM (shared by the batch) of the near-region list and moments passes
  int marker_threads;  // threads per CTA of the spreading, fibrin and interpolation passes
};
constexpr BatchTune kBatchTuneDefault = {8, 8, 128};
constexpr int kMarkerThreadsMax = 256;
// Autotuner (pf_tune.cu), per shape class: the key of a batch's class; the
// best shape so far (true once the search is done); the next shape to
// measure that is not in `busy` (false: none until results come in, or
// done); a measurement in device ns per lattice-node update.
std::string tune_key(int precision, bool fast, long long nodes, int njobs, long long markers);
bool tune_best(const std::string& key, BatchTune* best);
bool tune_next(const std::string& key, const std::vector<BatchTune>& busy, BatchTune* out);
void tune_record(const std::string& key, const BatchTune& t, float ns_per_node);
// CTAs job `d` needs for kernel `kind` (0: the kernel has no work for it)
int batch_ctas(const BatchDesc& d, int kind, int sms, int njobs, const BatchTune& t);
// whether the batch kernels can take this job (row width of the flagging)
bool batch_supported(const BatchDesc& d);
// Block size and dynamic shared memory of a batch kernel
int batch_threads(int kind, const BatchTune& t);
size_t batch_smem(const BatchDesc& d, int kind);
// Launches one batch kernel over `total` CTAs; precision and fast gather are
// the batch's (all jobs share them).
cudaError_t batch_launch(int kind, const BatchDesc* descs, const int* start, int njobs, int total, size_t smem,
                         int precision, bool fast, const BatchTune& t, cudaStream_t st);
// the lattice part of batch_launch (pf_lattice.cu)
cudaError_t batch_launch_lattice(int kind, const BatchDesc* descs, const int* start, int njobs, int total,
                                 int precision, bool fast, int lbm_rows, cudaStream_t st);
bool fast_gather(const Lattice& L);

// ------------------------------------------------------------------ launchers
// All launchers enqueue on `st` and return the launch error.
// The initial state of a job: the caller's populations f [19][N] (with
// rho/u [N], [3][N] or their moments), or, with f NULL, the equilibrium of
// rest / u [3][N] / rho [N] / the Zou/He shear profile; F [3][N] the initial
// force.  Every pointer may be NULL where optional and must be readable by
// the device (device memory, pinned or device-accessible host memory).
struct InitSource {
  const double *f, *F, *rho, *u;
  int zh;                  // Zou/He shear walls on z
  double C, Fo, dt, uw;    // moments of f: lattice speed, force factor, dt, top wall velocity
  double shear, dx, umax, C0, C02;  // equilibrium of the shear profile
};
cudaError_t lattice_init(Lattice& L, const InitSource& src, cudaStream_t st);
// picks the row-staged or the direct-gather step kernel (host only; call
// before the first step and outside stream capture)
cudaError_t lattice_configure(Lattice& L);
// the kernels of the lattice passes this job runs (for reports)
const char* lattice_pass_name(const Lattice& L);
// part 0: the whole lattice; 1: bricks not flagged for this step's force
// (may run while the forces are computed); 2: the flagged bricks (after the
// spreading); 3: the far region of step far_step (near[] clear); 4: the
// unflagged bricks of the near region.  bin_count: Morse cell counters to
// clear (parts 0 and 2 only).
cudaError_t lattice_step_part(Lattice& L, Control* ctl, int part, int* bin_count, int ncells, cudaStream_t st);
// near region: from this step's flags into near[next parity] (from_mark 0),
// or from the occupancy bits into near[this parity] (from_mark 1)
cudaError_t lattice_near(Lattice& L, Control* ctl, int from_mark, cudaStream_t st);
// far pass counter: sync (far_step = step) or advance after a far pass
// sets the quiet pass (part 5) to compute the current step (before a quiet
// pass that no flagged-brick pass of the step before scheduled)
cudaError_t lattice_quiet_prologue(Control* ctl, cudaStream_t st);
cudaError_t lattice_far_counter(Control* ctl, int sync, cudaStream_t st);
cudaError_t lattice_moments_active(Lattice& L, Control* ctl, cudaStream_t st);
// density and velocity at every stride-th node (float [mz][my][mx] planes)
cudaError_t lattice_fields(Lattice& L, long long step, int stride, float* rho, float* ux, float* uy, float* uz,
                           cudaStream_t st);
// fIN [19][N], fOUT [19][N], rho [N], u [3][N], F [3][N] (double, device)
cudaError_t lattice_download(Lattice& L, Control* ctl, long long step, double* fIN, double* fOUT, double* rho,
                             double* u, double* F, cudaStream_t st);
cudaError_t lattice_conservation(Lattice& L, long long step, double* out4_dev, cudaStream_t st);

cudaError_t membrane_forces(Platelets& Pl, int precision, Control* ctl, cudaStream_t st);
cudaError_t morse_forces(Platelets& Pl, int precision, Control* ctl, cudaStream_t st);
cudaError_t fibrin_forces(Fibrin& Fb, int precision, Control* ctl, cudaStream_t st);
// Penalty coupling, after the step's moments and before the position update:
// the node forces from the flow at the nodes, then the damped kick-drift-kick
// with the link forces recomputed at the new positions (sets the nodes'
// occupancy bits of the next step).
cudaError_t fibrin_penalty_step(Lattice& L, Fibrin& Fb, int precision, double F0, Control* ctl, cudaStream_t st);
// initial node velocity of the penalty coupling: the flow at the node
cudaError_t fibrin_penalty_init(Lattice& L, Fibrin& Fb, cudaStream_t st);
cudaError_t bond_pass(Platelets& Pl, int precision, Control* ctl, cudaStream_t st);
// occupancy bits of the current marker positions (once, after an upload;
// the position update sets them for the following step)
cudaError_t mark_markers(Lattice& L, Platelets* Pl, Fibrin* Fb, cudaStream_t st);
// flags (and lists) the force bricks every marker's stencil can reach this
// step, before any force exists; spread_markers then only adds forces
// check_near: every flagged brick must lie in near[step parity] (pipelined
// schedule), else ERR_FAR_FLAGGED.  with_prev: the list of the flagged-brick
// pass also holds the bricks flagged in the previous step (the schedule whose
// lattice pass over the other bricks is the quiet pass, part 5)
cudaError_t flag_markers(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, cudaStream_t st,
                         bool check_near = false, bool with_prev = false);
cudaError_t spread_markers(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, cudaStream_t st);
// Reduced precision with per-marker spreading: each force part is spread
// as soon as it exists (part 0: element membrane + Morse forces, 1: bond
// forces, 2: fibrin forces) instead of spread_markers after all forces; the
// position update then writes the element force totals.
bool spread_split(const Lattice& L);
cudaError_t spread_part(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, int part, cudaStream_t st);
cudaError_t interp_advance(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, double detach_rate,
                           uint64_t seed, unsigned* done_blocks, cudaStream_t st);
cudaError_t bin_elements(Platelets& Pl, Control* ctl, cudaStream_t st);
cudaError_t membrane_forces_raw(const PlateletConst& k, int precision, const double* X, const double* Y,
                                const double* RY, const double* Z, const int* tri, const int* node_ntri,
                                const int* node_tri, const int* vert_local, const int* ring, const int* sp_ptr,
                                const int* sp_nbr, const double* sp_L0, const double* S0, const double* S0_all,
                                const double* V0, void* nN, void* nelem, void* S, void* km, double* SV, void* F,
                                Control* ctl, cudaStream_t st);
size_t bond_scratch_bytes(int NR);
bool morse_uses_cells(const PlateletConst& k);
cudaError_t sort_cell_bins(Platelets& Pl, Control* ctl, cudaStream_t st);

int membrane_threads();
// whether the FP32 membrane pass of these platelets runs item-parallel
// (shared-memory fit; PFGPU_MEMBRANE_PER_VERTEX=1 turns it off)
bool membrane_items(const PlateletConst& k);
// sets the message pfgpu_last_error returns; returns code
int report_error(int code, const char* msg);

}  // namespace pf
