/*
 * pfgpu.h -- C ABI of the GB300-native coupled platelet / fibrin / lattice-
 * Boltzmann step (libpfgpu.so).
 *
 * Two layers are exported:
 *
 *  1. Drop-in names with the reference's signatures (semLB.cu / GPUDefines.h):
 *     fluid_*GPUKernel, sem_*GPUKernel, fiber_*GPUKernel.  They take the same
 *     host array layouts as the reference driver (gpuSEM_LB.c) and return
 *     nothing, like the reference; a failure is recorded and can be read with
 *     pfgpu_last_error().  The gsl_rng* arguments of the reference are
 *     replaced by an opaque uniform source (pfgpu_uniform_source, may be NULL).
 *
 *  2. pfgpu_* functions that return a status code: the scene-based job API
 *     used by tests, the benchmark and the batch/serving layer.
 *
 * All pointers are host pointers unless a name says otherwise; every call is
 * synchronous with respect to the host buffers it reads or writes.
 */
#ifndef PFGPU_H
#define PFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status */
typedef enum pfgpu_status {
  PFGPU_OK = 0,
  PFGPU_ERR_INVALID = 1,      /* bad argument / inconsistent sizes */
  PFGPU_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  PFGPU_ERR_NOMEM = 3,        /* device allocation failed or budget exceeded */
  PFGPU_ERR_UNSUPPORTED = 4,  /* valid input the GPU path does not implement */
  PFGPU_ERR_DEVICE = 5,       /* a kernel reported an error status */
  PFGPU_DONE = 6              /* the platelet detached (reference semLB.cu:451-455) or the job reached its stop step */
} pfgpu_status;

/* ------------------------------------------------------------ scene */
/* PF_BC_INOUT (y only, with Zou/He shear walls on z and periodic x): the
 * velocity inlet at y=0 and outlet at y=ny-1 of the reference's
 * fluid3d_in_out_flow_boundary_kernel (LB_kernel.cu:78-392, commented out
 * there): the shear profile u = (0, uw z/(nz-1), 0) on both planes, Zou/He
 * unknowns on the interior of each plane, the equilibrium at unit density on
 * the plane's rows next to its edges (x = 1, nx-2; z = 1, nz-2).  Streaming
 * is periodic in y before the planes are rewritten, as the reference's is. */
enum { PF_BC_PERIODIC = 0, PF_BC_BOUNCEBACK = 1, PF_BC_ZOUHE_SHEAR = 2, PF_BC_INOUT = 3 };
enum { PF_PREC_FP64 = 0, PF_PREC_FP32 = 1, PF_PREC_FP16 = 2 };
enum { PF_BOND_BELL = 0, PF_BOND_CONSTANT = 1 };
enum { PF_FIB_HOOKE = 0, PF_FIB_WLC = 1 };
/* How fibrin nodes meet the fluid.  MARKER: immersed markers (link forces
 * spread into the lattice, nodes moved with the interpolated velocity).
 * PENALTY: the reference's fibrin FSI design (fiber_LB_Fsi_force /
 * Flow_vel_at_position, fiber.cpp:501-814, with the network's damped
 * kick-drift-kick, network.cpp:445-513,839-881): each node carries its own
 * velocity, the fluid pulls it with the penalty force kappa rho (u - V) and
 * receives the reaction. */
enum { PF_FIBCPL_MARKER = 0, PF_FIBCPL_PENALTY = 1 };
/* PF_MEM_ALL: the membrane chain the reference runs (semLB.cu:510-523).
 * PF_MEM_FEMBEND adds the reference's disabled FEM bending chain
 * (sem_calculate_K_kernel, sem_calculate_q_kernel, sem_bending_force_kernel,
 * sem_kernel.cu:1129-1497) in the slot its commented-out launches hold
 * (semLB.cu:518-520, between the curvature and the area/volume forces).
 * Single jobs only: the batch API and the no-allocation entry point refuse it. */
enum { PF_MEM_SPRING = 1, PF_MEM_WALL = 2, PF_MEM_AREAVOL = 4, PF_MEM_BEND = 8, PF_MEM_ALL = 15,
       PF_MEM_FEMBEND = 16 };

/* Indices into pf_scene.params: the reference's model parameter table
 * (sem_kernel.cu:58-76, filled at gpuSEM_LB.c:1206-1233). */
enum {
  PF_P_NUMRECEPTORS = 0, PF_P_SEED = 1, PF_P_KSPRING = 2, PF_P_KF0 = 3, PF_P_KR0 = 4,
  PF_P_SHEAR = 5, PF_P_RHO0 = 6, PF_P_L0 = 7, PF_P_T0 = 8, PF_P_M0 = 9, PF_P_F0 = 10,
  PF_P_UMAX = 11, PF_P_NU = 12, PF_P_TAU = 13, PF_P_P0 = 14, PF_P_CL = 15,
  PF_P_UNIT = 16, PF_P_KS = 17, PF_P_KV = 18, PF_P_KBEND = 19
};

/* Everything one coupled simulation needs.  Array layouts: lattice arrays are
 * [..][nz][ny][nx] (x fastest, the reference's dense host layout); platelet
 * arrays are platelet-major [n_platelets][...].  The triangulated membrane
 * topology is one template shared by all platelets: elements
 * 0..n_membrane-1 of each platelet are the mesh vertices, the rest are
 * cytoplasm elements. */
typedef struct pf_scene {
  /* lattice */
  int nx, ny, nz;
  float dx, dt;                 /* micron, second (float like the reference) */
  float params[100];            /* reference parameter table, PF_P_* */
  int bc[3];                    /* per axis: PF_BC_* (ZOUHE_SHEAR only on z) */
  int ibm_wrap[3];              /* per axis: 1 = IBM stencils and positions periodic */
  double body_force[3];         /* force added at every lattice node, reference force units */
  const double *f_init;         /* [19][nz][ny][nx] or NULL: equilibrium of rho=1, u_init */
  const double *u_init;         /* [3][nz][ny][nx] (units of UMAX) or NULL: reference shear profile
                                   gpuSEM_LB.c:1234-1243 when bc[2]==ZOUHE_SHEAR, else rest */
  const double *F_init;         /* [3][nz][ny][nx] lattice force of the step before the first, or NULL */
  const double *rho_init;       /* [nz][ny][nx] density the first collision uses (with u_init), or NULL.
                                   The reference's first collision reads the host rho/u arrays
                                   (fluid_initGPUKernel, semLB.cu:154-233), not moments of fIN. */

  /* platelets (SEM elements) */
  int n_platelets, n_elem, n_membrane, n_tri, n_node;
  const int *tri;               /* [n_tri][6]: 3 vertices, 3 edge-midpoint nodes (gpuSEM_LB.c:846-880) */
  const int *node_ntri;         /* [n_node] triangles sharing each node (node_nbrElemNum) */
  const int *ring;              /* [n_membrane][10] ring-ordered neighbour vertices (node_nbr_nodes) */
  const int *spring_ptr;        /* [n_elem+1] CSR of membrane springs (dense bondLengths > 1e-6) */
  const int *spring_nbr;        /* [spring_ptr[n_elem]] neighbour element, ascending per row */
  const double *spring_L0;      /* [spring_ptr[n_elem]] rest length */
  const double *S0;             /* [n_platelets][n_tri] rest triangle areas */
  const double *S0_all;         /* [n_platelets] rest membrane area */
  const double *V0;             /* [n_platelets] rest volume */
  const double *X, *Y, *RY, *Z; /* [n_platelets][n_elem] initial positions (Y wrapped, RY unwrapped) */
  int membrane_forces;          /* PF_MEM_* bitmask */

  /* receptors (GPIb-alpha) and vWF wall sites */
  int n_rec;                    /* receptors per platelet */
  const int *rec_tri;           /* [n_platelets][n_rec] triangle of each receptor */
  const float *rec_r1, *rec_r2; /* [n_platelets][n_rec] barycentric parameters */
  const int *rec_state;         /* [n_platelets][n_rec][3] (site i, site j, bonds) or NULL = unbound */
  const int *vwf;               /* [4][ny][nx] slot owners (-1 free) or NULL = all free */
  int bond_model;               /* PF_BOND_* */
  double p_on, p_off;           /* per-draw probabilities for PF_BOND_CONSTANT */

  /* Morse pair forces between elements (within and between platelets),
   * force-shifted at the cutoff: f = (F(r) - F(cutoff)) r_hat with
   * F(r) = 2 rho U0 [e^{2 rho (r_eq - r)} - e^{rho (r_eq - r)}] */
  int morse;                    /* 0 = off */
  double morse_intra[4];        /* U0, rho, r_eq, cutoff (same platelet) */
  double morse_inter[4];        /* U0, rho, r_eq, cutoff (different platelets) */

  /* fibrin network */
  int n_fib;
  const double *fib_X, *fib_Y, *fib_Z; /* [n_fib] */
  const int *fib_fixed;         /* [n_fib] 1 = node does not move (fiber.cpp:380-384) */
  const int *fib_ptr;           /* [n_fib+1] CSR of links at each node (Link_at_Node) */
  const int *fib_nbr;           /* other end node of each link slot */
  const double *fib_L0;         /* rest length of each link slot */
  int fib_law;                  /* PF_FIB_* */
  double fib_k;                 /* Hookean stiffness (nN/um) or WLC modulus */
  double fib_mass;              /* WLC mass divisor (fiber.cpp:730) */

  /* injected uniform stream and detachment */
  uint64_t seed;                /* Philox-4x32-10 key of the receptor/detach uniforms */
  double detach_rate;           /* gama of semLB.cu:451 (0 = never detach) */

  /* fibrin coupling (PF_FIBCPL_*; PENALTY only reads the three below) */
  int fib_coupling;
  double fib_gamma;             /* friction rate of the kick, per lattice step (0 = none) */
  double fib_node_mass;         /* node mass in lattice units (1 = the fluid in one lattice cell) */
  double fib_kappa;             /* penalty stiffness (1 = the reference's rho (u - V) / dt) */
} pf_scene;

/* ------------------------------------------------------------ job API */
typedef struct pfgpu_job pfgpu_job;

/* Creates a device-resident simulation on the current CUDA device.
 * precision: PF_PREC_*; fp16_scale: sigma of the FP16 store
 * q = (f - w)/(w sigma) (<= 0: eight times the shear wall speed in lattice
 * units, or 0.05), ignored for FP32/FP64. */
int pfgpu_job_create(const pf_scene *scene, int precision, double fp16_scale, pfgpu_job **out);
/* Runs nsteps coupled steps (SEM+Morse+fibrin forces, bonds, IBM spreading,
 * fused collide-stream, moments, IBM interpolation, position update).
 * Returns PFGPU_DONE if the platelet detached. */
int pfgpu_job_step(pfgpu_job *job, int nsteps);
/* Same, captured once in a CUDA graph and replayed (no host work per step). */
int pfgpu_job_step_graph(pfgpu_job *job, int nsteps);
int pfgpu_job_sync(pfgpu_job *job);
/* Enqueues nsteps replays of the step graph without waiting (pfgpu_job_sync
 * waits and reports PFGPU_DONE / device errors). */
int pfgpu_job_enqueue(pfgpu_job *job, int nsteps);
/* Runs nsteps steps serialised on one stream with CUDA events around each
 * phase and returns the summed device time per phase in ms (ms_out holds
 * pfgpu_profile_phase_count() entries): flag, membrane, morse, fibrin, bonds,
 * spread, lbm (both lattice passes), moments, interp. */
int pfgpu_job_profile(pfgpu_job *job, int nsteps, double *ms_out);
int pfgpu_profile_phase_count(void);
const char *pfgpu_profile_phase_name(int i);
/* Copies state back in scene layouts; any pointer may be NULL. */
int pfgpu_job_get_lattice(pfgpu_job *job, double *fIN, double *fOUT, double *rho, double *u /*[3][N]*/,
                          double *F /*[3][N]*/);
/* Density and velocity (the units of pfgpu_job_get_lattice's rho and u) at
 * every stride-th node in x, y and z, computed on the device: float arrays
 * [dims[2]][dims[1]][dims[0]], dims[i] = ceil(n_i / stride).  NULL arrays are
 * skipped (all NULL: only dims).  Feeds pfgpu_write_vti. */
int pfgpu_job_get_fields(pfgpu_job *job, int stride, float *rho, float *ux, float *uy, float *uz, int dims[3]);
int pfgpu_job_get_elements(pfgpu_job *job, double *X, double *Y, double *RY, double *Z,
                           double *V /*[3][P*E]*/, double *F /*[3][P*E]*/);
int pfgpu_job_get_bonds(pfgpu_job *job, int *rec_state /*[P][n_rec][3]*/, int *vwf /*[4][ny][nx]*/,
                        int *total_bond);
int pfgpu_job_get_fibrin(pfgpu_job *job, double *X, double *Y, double *Z, double *V /*[3][M]*/,
                         double *F /*[3][M]*/);
/* Per-platelet FP64 reductions of the last force pass: [P][2] (S_all, V) and
 * the membrane vertex mean curvature km [P][n_membrane]. */
int pfgpu_job_get_membrane(pfgpu_job *job, double *S_V, double *km);
/* Morse cell lists rebuilt from the current positions: cell of every element
 * [P*E], element count of every cell [ncells], members of each cell in
 * ascending element id packed in cell order, grid dimensions [3]. */
int pfgpu_job_get_cells(pfgpu_job *job, int *cell_of, int *counts, int *members, int *ncells3);
/* FP64 conservation sums over the lattice: mass and x/y/z momentum. */
int pfgpu_job_conservation(pfgpu_job *job, double out[4]);
int64_t pfgpu_job_step_count(const pfgpu_job *job);
/* The job stops by itself after completing step stop_step (0: never): later
 * steps do nothing and pfgpu_job_sync returns PFGPU_DONE, as after a
 * detachment.  A stop step at or before the current step stops it at once; a
 * later one lets a job stopped this way run on. */
int pfgpu_job_set_stop(pfgpu_job *job, int64_t stop_step);
size_t pfgpu_job_device_bytes(const pfgpu_job *job);
/* State snapshots, for checkpoint / resume, preemption and migration of
 * served jobs (the reference keeps its state on the host between the copy
 * calls, semLB.cu:154-296, 979-1000).  pfgpu_job_save writes the job's whole
 * device state (every population, force and flag buffer, element, fibrin and
 * bond state, the control block with the step counter) into `buf`, which
 * holds pfgpu_job_state_bytes(job) bytes; pfgpu_job_restore loads a snapshot
 * into a job created from a scene of the same sizes and precision and
 * rejects any other with PFGPU_ERR_INVALID.  Both wait for the job's work. */
size_t pfgpu_job_state_bytes(const pfgpu_job *job);
int pfgpu_job_save(pfgpu_job *job, void *buf, size_t bytes);
int pfgpu_job_restore(pfgpu_job *job, const void *buf, size_t bytes);
/* Kernel launches one coupled step issues: after a graph step, the kernel
 * nodes of the captured step graph per step; after a direct step, the
 * launches that step made. */
int pfgpu_job_launches_per_step(const pfgpu_job *job);
/* Which collide-stream kernels the job runs: "lbm_rows_k" (rows staged
 * through shared memory by bulk asynchronous copies; needs nx *
 * sizeof(population) to be a multiple of 16 bytes), "lbm_vec_k+lbm_list_k"
 * (FP32/FP16 without bounce-back faces: several x-nodes per thread with
 * vector loads, the force bricks one node per thread) or
 * "lbm_step_k+lbm_list_k" (one node per thread). */
const char *pfgpu_job_lbm_kernel(const pfgpu_job *job);

/* ---- element output dumps ----------------------------------------------
 * The reference driver's element files, written from a job's state
 * (replaces the fopen/fwrite/fprintf blocks of gpuSEM_LB.c:1327-1336,
 * 1376-1407, 1464-1494 and 1533): in `dir`, cellsPos.data, cellsVel.data,
 * cellsForce.data (per element x, y, z, z -- RY for the position's y, the
 * last value repeated "for alignment in the octal dump"), the three
 * "Timestep ElemID X Y Z" ASCII tables and cellsPauseTime.dat (appended).
 * PFGPU_OUT_FP64 writes doubles as the reference does; PFGPU_OUT_FP32 writes
 * floats, the 16-byte records convBtoXYZ.py reads through `od -f`. */
enum { PFGPU_OUT_FP64 = 0, PFGPU_OUT_FP32 = 1 };
typedef struct pfgpu_output pfgpu_output;
/* Opens the files and writes the initial frame (timestep 0 tables; all
 * three binary files). */
int pfgpu_output_open(pfgpu_job *job, const char *dir, int mode, pfgpu_output **out);
/* Appends one frame at the job's current step: positions to cellsPos.data
 * and a row per element to each table (gpuSEM_LB.c:1464-1494). */
int pfgpu_output_frame(pfgpu_output *out);
/* The same files from the caller's host arrays, as the reference driver
 * writes them after sem_copyGPUKernel: X, RY, Z [P * E] and V, F [3][P * E]
 * (platelet-major, the job API's layout); each frame names its step. */
int pfgpu_output_open_arrays(const char *dir, int mode, int P, int E, double dt, const double *X, const double *RY,
                             const double *Z, const double *V, const double *F, pfgpu_output **out);
int pfgpu_output_frame_arrays(pfgpu_output *out, long long step, const double *X, const double *RY, const double *Z,
                              const double *V, const double *F);
/* Appends "<step * dt>, <seed>" to cellsPauseTime.dat (gpuSEM_LB.c:1533)
 * and closes the files (step: the job's, or the last frame's). */
int pfgpu_output_close(pfgpu_output *out, int seed);
/* The reference driver's writeVTK (gpuSEM_LB.c:1631-1709, outputSave at
 * :1618): <directory>/<filename>_<t, 7 digits>.vti, VTK ImageData with ASCII
 * Float32 "Density" and 3-component "Velocity" point data, "%.4e " per value
 * and one line per x row; host arrays [nz][ny][nx].  `spacing` is the node
 * stride of downsampled fields (1: the reference's Spacing "1 1 1").  The
 * directory is created if missing.  Host-only. */
int pfgpu_write_vti(int t, int nx, int ny, int nz, int spacing, const float *rho, int write_rho, const float *ux,
                    const float *uy, const float *uz, int write_vel, const char *directory, const char *filename);
void pfgpu_job_destroy(pfgpu_job *job);

/* Device bytes a job with this scene and precision would allocate. */
size_t pfgpu_scene_device_bytes(const pf_scene *scene, int precision);

/* ------------------------------------------------------------ host input */
/* The reference driver's inputs, read and built on the host (no CUDA call):
 * the parameter file (ParReader, gpuSEM_LB.c:148-343), the NEU surface mesh
 * (NEUReader, gpuSEM_LB.c:345-404) and the membrane topology built from it
 * (gpuSEM_LB.c:846-1055), with CSR tables instead of the dense bondLengths
 * table and the [node][10] arrays.  Errors return PFGPU_ERR_INVALID with the
 * reason in pfgpu_last_error (the reference prints and exits). */
typedef struct pf_parameter_file {
  char pdb_path[256], psf_path[256], neu_path[256];
  float dx, dt, sim_time;                  /* DELTA_X, DELTA_T, SIM_TIME */
  int out_freq, max_cell, max_elem, surf_elem;  /* OUT_FREQ, MAX_CELL, MAX_ELEM, SURF_ELEM */
  /* HostParam: [0] RECEPTOR, [1] RANDOM_SEED, [2] K_SPRING, [3] Kf0 (not in
   * the file), [4] Kr0, [5] SHEAR_RATE, [6] INIT_RHO */
  float host_param[7];
} pf_parameter_file;
int pfgpu_read_parameter_file(const char *path, pf_parameter_file *out);
int pfgpu_neu_counts(const char *path, int *n_sce, int *n_tri);
/* X, Y, Z [n_sce]; tri3 [n_tri][3] 0-based; bond CSR of the triangle edges:
 * bond_ptr [n_sce + 1], bond_nbr / bond_len [6 n_tri] (ascending neighbour). */
int pfgpu_read_neu(const char *path, double *X, double *Y, double *Z, int *tri3, int *bond_ptr, int *bond_nbr,
                   double *bond_len);
/* tri6 [n_tri][6] (vertices, then the virtual edge nodes), node_ptr
 * [n_vert + 3 n_tri + 1] / node_tri [6 n_tri] (triangles of each node; a
 * vertex's in ring order), ring [3 n_tri] (vertex i's ordered neighbours at
 * ring[node_ptr[i] + j]), normals [3 (n_vert + 3 n_tri)], S0 [n_tri], the
 * total rest area and the volume; *n_nodes: vertices + virtual nodes. */
int pfgpu_build_topology(int n_vert, int n_tri, const int *tri3, const double *X, const double *Y, const double *Z,
                         int *tri6, int *n_nodes, int *node_ptr, int *node_tri, int *ring, double *normals,
                         double *S0, double *S0_all, double *V0);

/* ------------------------------------------------------------ batch API */
/* Continuous batching of independent jobs on one GPU: each admitted job keeps
 * its own device state.  A batch step of FP32 or FP16 jobs is one captured
 * graph in which each kernel of the coupled step runs once over the CTAs of
 * every job (a per-job CTA offset table); its block and tile shapes are picked
 * by an autotuner that measures candidate shapes on the batch's own steps
 * (PFGPU_BATCH_TUNE=0: fixed defaults; PFGPU_TUNE_CACHE=path: results kept in
 * a text file).  Other batches replay each job's own step graph on the job's
 * streams.  Jobs join and leave between batch steps; admission is checked
 * against a device-memory budget. */
typedef struct pfgpu_batch pfgpu_batch;
int pfgpu_batch_create(size_t hbm_budget_bytes, pfgpu_batch **out);
/* Admits a job if it fits the budget; returns PFGPU_ERR_NOMEM otherwise.
 * *slot receives the job's id within the batch. */
int pfgpu_batch_admit(pfgpu_batch *b, const pf_scene *scene, int precision, double fp16_scale, int *slot);
/* nsteps steps of every live job; a job whose platelet detached stops and its
 * status turns PFGPU_DONE (retire it). */
int pfgpu_batch_step(pfgpu_batch *b, int nsteps);
int pfgpu_batch_status(pfgpu_batch *b, int slot);
/* pfgpu_job_set_stop for the job in `slot`: a served job is admitted with the
 * step count it asked for and leaves the fused step when it reaches it, so a
 * batch step can run a whole chunk of steps whatever the other jobs need. */
int pfgpu_batch_set_stop(pfgpu_batch *b, int slot, int64_t stop_step);
int pfgpu_batch_retire(pfgpu_batch *b, int slot);
pfgpu_job *pfgpu_batch_job(pfgpu_batch *b, int slot);
/* The fused step's shapes: shape[0] groups of four bricks per CTA of the unflagged
 * lattice pass, shape[1] CTAs per SM of the near-region list and moments
 * passes, shape[2] threads per CTA of the marker passes.  *state: 0 still
 * tuning, 1 fixed (tuned, forced or tuning off), -1 no fused step. */
int pfgpu_batch_shape(pfgpu_batch *b, int shape[3], int *state);
/* Forces the fused step's shapes; lbm_rows = 0 hands them back to the tuner. */
int pfgpu_batch_set_shape(pfgpu_batch *b, int lbm_rows, int list_per_sm, int marker_threads);
size_t pfgpu_batch_bytes_in_use(const pfgpu_batch *b);
int pfgpu_batch_num_jobs(const pfgpu_batch *b);
void pfgpu_batch_destroy(pfgpu_batch *b);

/* ------------------------------------------------------------ misc */
/* ---- membrane pass without allocation ------------------------------------
 * No counterpart in the reference (its membrane pass runs inside
 * sem_invokeGPUKernel_Force on buffers sem_allocGPUKernel allocated).
 * The membrane forces of n_platelets platelets -- springs on RY, wall
 * repulsion, area/volume penalty, bending: the pass pfgpu_job_step runs --
 * computed from caller-owned device arrays into F_out, for callers that may
 * not allocate device memory while they run (a solver loop with a fixed
 * memory budget, code between a custom allocator's arena set-up and use).
 * It calls no cudaMalloc/cudaFree or other allocating routine: its scratch
 * (node triangle lists, normals, strains, curvatures) is a fixed static
 * device array of PFGPU_NOALLOC_SCRATCH_BYTES, and a call that needs more
 * (about P * (12 n_node + 16 n_tri + 4 n_membrane) bytes in FP32, twice that
 * in FP64, plus 80 n_node) returns PFGPU_ERR_INVALID with the sizes in
 * pfgpu_last_error().
 * - The first call on a device looks up the scratch's address
 *   (cudaGetSymbolAddress with that device current); make it before any
 *   stream capture.
 * - The scratch is shared: calls that overlap in time, on any streams or
 *   host threads, race on it.  Serialise them.
 * - Nothing needs to start at zero: each call zeroes the scratch's control
 *   word on `stream` and writes every other scratch word before reading it.
 * - The topology is checked on the device, where the call cannot wait for
 *   it: a triangle index outside the nodes, node_ntri outside 0..10 or
 *   unequal to the node's count in tri, a ring or spring entry out of range
 *   leaves F_out, S_V_out and km_out unwritten, and
 *   pfgpu_membrane_noalloc_status(stream) then returns PFGPU_ERR_INVALID.
 *   Call it after the pass when the inputs are not known to be consistent.
 * - The cached address belongs to the device's primary context: after a
 *   cudaDeviceReset on that device it is stale, so make no further call on
 *   that device in the process.
 * Inputs use the pf_scene layouts (device pointers); F_out is [3][P*n_elem]
 * in units of F0, double for PF_PREC_FP64 and float otherwise; S_V_out
 * ([P][2]: area, volume) and km_out ([P][n_membrane]: mean curvature, the
 * real type of F_out) may be NULL.  Asynchronous on `stream` (a
 * cudaStream_t, NULL for the default stream). */
#define PFGPU_NOALLOC_SCRATCH_BYTES (8u << 20)
typedef struct {
  int n_platelets, n_elem, n_membrane, n_tri, n_node;
  int precision;       /* PF_PREC_* */
  int membrane_forces; /* PF_MEM_* mask */
  float kspring, ks, kv, kbend, f0; /* reference parameters (float) */
  const double *X, *Y, *RY, *Z;     /* [P * n_elem] */
  const int *tri;                   /* [n_tri][6] */
  const int *node_ntri;             /* [n_node] */
  const int *ring;                  /* [n_membrane][10] */
  const int *spring_ptr;            /* [n_elem + 1] */
  const int *spring_nbr;            /* [spring_ptr[n_elem]] */
  const double *spring_L0;          /* [spring_ptr[n_elem]] */
  const double *S0;                 /* [P][n_tri] */
  const double *S0_all, *V0;        /* [P] */
  void *F_out;                      /* [3][P * n_elem] */
  double *S_V_out;                  /* [P][2] or NULL */
  void *km_out;                     /* [P][n_membrane] or NULL */
} pf_membrane_args;
int pfgpu_membrane_forces_noalloc(const pf_membrane_args *args, void *stream);
size_t pfgpu_membrane_noalloc_scratch_bytes(void);
/* Waits for `stream` and reports the last pass on the current device:
 * PFGPU_OK, or PFGPU_ERR_INVALID for rejected inputs (F_out unwritten) or a
 * platelet too large for the pass.  Allocates nothing. */
int pfgpu_membrane_noalloc_status(void *stream);

const char *pfgpu_last_error(void);
int pfgpu_version(void);
/* Pinned, device-mapped host memory for a caller's arrays (no counterpart in
 * the reference, whose driver malloc's its host arrays).  Job creation and
 * the lattice download read and write caller arrays where they lie whenever
 * the device can reach them -- pinned memory like this, or any host memory
 * on machines whose GPU walks the host page tables (Grace, NVLink-C2C) --
 * instead of staging them through device copies.  NULL on failure. */
void *pfgpu_host_alloc(size_t bytes);
void pfgpu_host_free(void *p);
/* Philox-4x32-10 uniforms of the receptor stream (step, receptor) -> (u1, u2),
 * the same values the device draws; for tests and drivers. */
void pfgpu_receptor_uniforms(uint64_t seed, int64_t step, int64_t receptor, double out[2]);
double pfgpu_detach_uniform(uint64_t seed, int64_t step);

/* Opaque replacement for the reference's gsl_rng* arguments. */
typedef struct pfgpu_uniform_source {
  uint64_t seed;
} pfgpu_uniform_source;

/* ------------------------------------------------------------ drop-in names
 * Signatures of semLB.cu:111, :154, :303, :534 (fluid), :749, :865, :441,
 * :979, :1005 (SEM), :562, :609, :669, :708 (fibrin); host array layouts of
 * gpuSEM_LB.c. */
void *fluid_allocGPUKernel(void *model, float dt, float dx, int width, int height, int depth);
void fluid_initGPUKernel(void *model, void *g, int aFlag, float *hostParameters, void **fIN, void **fOUT,
                         void *ux, void *uy, void *uz, void *rho, void *obstacle, void *Fx, void *Fy,
                         void *Fz, void *vWFbond);
void fluid_invokeGPUKernel(void *model, void *g, void *g_SEM, double *randNum, void *r, int timeSteps);
void fluid_releaseGPUKernel(void *model, void *g);

void *sem_allocGPUKernel(void *model, int maxCells, int maxElements, int SurfElem, int newnode,
                         int numReceptorsPerElem, float dt, double S0_all, float *hostSEMparameters);
/* node_share_Elem and N are accepted and not read: the node -> triangle
 * lists are built from triElem, and nodal normals are recomputed from the
 * positions each step.  The reference uploads both (semLB.cu:939-943) but
 * its kernels read neither outside commented-out code (sem_kernel.cu:743,
 * 856, 1513). */
void sem_initGPUKernel(void *model, void *g, int numOfCells, int *numOfElements, int SurfElem,
                       int numReceptorsPerElem, void *hostX_Ref, void *hostY_Ref, void *hostZ_Ref,
                       void *hostX, void *hostY, void *hostRY, void *hostZ, void *hostVX, void *hostVY,
                       void *hostVZ, void *hostFX, void *hostFY, void *hostFZ, void *hostType,
                       void *hostBonds, void *triElem, void *receptor_r1, void *receptor_r2,
                       void *node_share_Elem, void *N, void *node_nbrElemNum, void *node_nbr_nodes,
                       void *S0, double V0, void *receptBond, void *randNum);
void sem_invokeGPUKernel_Force(void *model, void *g, int timeSteps, int *done, int *totalT, void *r,
                               double gama);
void sem_copyGPUKernel(void *model, void *g, void *hostX, void *hostY, void *hostRY, void *hostZ,
                       void *hostVX, void *hostVY, void *hostVZ, void *hostFX, void *hostFY,
                       void *hostFZ, int timeSteps);
void sem_releaseGPUKernel(void *model, void *g);

void *fiber_allocGPUKernel(void *model, int maxNodes, int maxLinks, int max_N_conn_at_Node, double dt,
                           double *hostParameters);
void fiber_init_GPUKernel(void *model, void *fg, void *NodeType, void *N_Conn_at_Node, void *Link_at_Node,
                          void *lAdjVer, void *linkLengths, void *linkLengths0, void *linkThick, void *X,
                          void *V_X, void *X0, void *F_X, void *Y, void *Y0, void *V_Y, void *F_Y, void *Z,
                          void *Z0, void *V_Z, void *F_Z);
void fiber_copy_GPUKernel(void *model, void *fg, void *X, void *V_X, void *X0, void *F_X, void *Y, void *Y0,
                          void *V_Y, void *F_Y, void *Z, void *Z0, void *V_Z, void *F_Z);
void fiber_release_GPUKernel(void *model, void *fg);

/* Additions to the drop-in layer (no reference counterpart): couple a fibrin
 * handle to a fluid handle so fluid_invokeGPUKernel spreads its spring forces
 * and advects its nodes; select the fibrin force law. */
int pfgpu_fluid_attach_fiber(void *g, void *fg, int law, double k, double mass);
/* Precision of fluid handles created by later fluid_allocGPUKernel calls
 * (default PF_PREC_FP64, the reference's arithmetic). */
int pfgpu_set_default_precision(int precision, double fp16_scale);

#ifdef __cplusplus
}
#endif
#endif
