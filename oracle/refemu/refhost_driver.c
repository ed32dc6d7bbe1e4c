/*
 * refhost_driver.c -- the reference driver's host code (gpuSEM_LB.c,
 * included from the reference tree at build time) compiled for the CPU, with
 * its GPU entry points replaced by stubs that record what the driver hands
 * them.  It pins this repository's host restatements to the reference's own
 * code: the parameter-file and NEU readers (ParReader, NEUReader, called
 * directly), the topology build (gpuSEM_LB.c:846-1055, whose tables the
 * driver passes to sem_initGPUKernel), the element dumps of the step loop
 * (:1327-1336, 1376-1407, 1464-1494, 1533) and writeVTK (:1631-1709).
 *
 * ORACLE TEST INFRASTRUCTURE ONLY: built by oracle/refemu/build_refemu.sh into
 * oracle/_ref/ where the reference tree is present; never shipped or linked by
 * the product.  Substitutions, each needed to run the driver without a GPU:
 *   1. exit() returns, so the driver runs past its debugging exits
 *      (gpuSEM_LB.c:1288 after the fibrin set-up, and the one inside the step
 *      loop) -- the inputs given here take no error path;
 *   2. GSL's generator is a stand-in (stub/gsl/gsl_rng.h);
 *   3. sem_invokeGPUKernel_Force counts steps and reports `done` after the
 *      requested number; sem_copyGPUKernel fills the element arrays with
 *      refhost_pattern(), so every frame the driver writes is known;
 *      init_fibrin_network returns an empty network.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <gsl/gsl_rng.h>

int cudaSetDevice(int d);
int cudaGetDevice(int *d);

static void refhost_exit(int code) { (void)code; }
#define exit(c) refhost_exit(c)
#define main refhost_driver_main
#include "gpuSEM_LB.c"
#undef exit
#undef main

/* ----------------------------------------------------------- GSL stand-in */
static const gsl_rng_type g_type = {2};
const gsl_rng_type *gsl_rng_ranlxs2 = &g_type;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  (void)T;
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof *r);
  return r;
}
void gsl_rng_set(gsl_rng *r, unsigned long int seed) { r->s = 0x9E3779B97F4A7C15ull * (seed + 1); }
double gsl_rng_uniform(gsl_rng *r) {
  unsigned long long z = (r->s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
void gsl_rng_free(gsl_rng *r) { free(r); }
int cudaSetDevice(int d) { (void)d; return 0; }
int cudaGetDevice(int *d) { *d = 0; return 0; }

/* ------------------------------------------------------------ the records */
static int g_steps_wanted = 1, g_steps = 0;
static int g_dims[6]; /* maxCells, maxElements, SurfElem, newnode, R, numOfCells */
static double g_S0_all, g_V0;
static int *g_tri, *g_share, *g_nbrnum, *g_nbrnodes;
static double *g_N, *g_S0, *g_bonds, *g_elem[10];
static float *g_r1, *g_r2;

static void *dup_bytes(const void *p, size_t n) {
  void *q = malloc(n ? n : 1);
  if (p && n) memcpy(q, p, n);
  return q;
}

/* the element value the copy stub writes at (element i, cell j, step t,
 * field k: X, Y, RY, Z, VX, VY, VZ, FX, FY, FZ) */
double refhost_pattern(int i, int j, int t, int k) {
  return 1.0 + 0.001 * i + 0.25 * j + 1e-5 * t + 0.125 * k + 1e-9 * (double)(i * 7 % 13);
}

/* ----------------------------------------------------- GPU entry points */
void *fluid_allocGPUKernel(void *model, float dt, float dx, int width, int height, int depth) {
  (void)model; (void)dt; (void)dx; (void)width; (void)height; (void)depth;
  return calloc(1, 16);
}
void fluid_initGPUKernel(void *model, void *g, int aFlag, float *hostLBparameters, void **fIN, void **fOUT, void *ux,
                         void *uy, void *uz, void *rho, void *obstacle, void *Fx, void *Fy, void *Fz, void *vWFbond) {
  (void)model; (void)g; (void)aFlag; (void)hostLBparameters; (void)fIN; (void)fOUT; (void)ux; (void)uy; (void)uz;
  (void)rho; (void)obstacle; (void)Fx; (void)Fy; (void)Fz; (void)vWFbond;
}
void fluid_invokeGPUKernel(void *model, void *g, void *g_SEM, double *randNum, gsl_rng *r, int timeSteps) {
  (void)model; (void)g; (void)g_SEM; (void)randNum; (void)r; (void)timeSteps;
}
void fluid_releaseGPUKernel(void *model, void *g) { (void)model; free(g); }

void *sem_allocGPUKernel(void *model, int maxCells, int maxElements, int SurfElem, int newnode,
                         int numReceptorsPerElem, float dt, double S0_all, float *hostSEMparameters) {
  (void)model; (void)dt; (void)hostSEMparameters;
  g_dims[0] = maxCells; g_dims[1] = maxElements; g_dims[2] = SurfElem; g_dims[3] = newnode;
  g_dims[4] = numReceptorsPerElem;
  g_S0_all = S0_all;
  return calloc(1, 16);
}
void sem_initGPUKernel(void *model, void *g, int numOfCells, int *numOfElements, int SurfElem,
                       int numReceptorsPerElem, void *hostX_Ref, void *hostY_Ref, void *hostZ_Ref, void *hostX,
                       void *hostY, void *hostRY, void *hostZ, void *hostVX, void *hostVY, void *hostVZ,
                       void *hostFX, void *hostFY, void *hostFZ, void *hostType, void *hostBonds, void *triElem,
                       void *receptor_r1, void *receptor_r2, void *node_share_Elem, void *N, void *node_nbrElemNum,
                       void *node_nbr_nodes, void *S0, double V0, void *receptBond, void *randNum) {
  (void)model; (void)g; (void)numOfElements; (void)hostX_Ref; (void)hostY_Ref; (void)hostZ_Ref; (void)hostType;
  (void)receptBond; (void)randNum;
  const size_t C = (size_t)g_dims[0], E = (size_t)g_dims[1], T = (size_t)SurfElem, NN = (size_t)g_dims[3];
  const size_t R = (size_t)numReceptorsPerElem;
  g_dims[5] = numOfCells;
  g_V0 = V0;
  g_tri = (int *)dup_bytes(triElem, T * 6 * sizeof(int));
  g_share = (int *)dup_bytes(node_share_Elem, NN * 10 * sizeof(int));
  g_N = (double *)dup_bytes(N, NN * 3 * sizeof(double));
  g_nbrnum = (int *)dup_bytes(node_nbrElemNum, E * sizeof(int));
  g_nbrnodes = (int *)dup_bytes(node_nbr_nodes, E * 10 * sizeof(int));
  g_S0 = (double *)dup_bytes(S0, T * sizeof(double));
  g_bonds = (double *)dup_bytes(hostBonds, E * E * sizeof(double));
  g_r1 = (float *)dup_bytes(receptor_r1, T * R * sizeof(float));
  g_r2 = (float *)dup_bytes(receptor_r2, T * R * sizeof(float));
  void *el[10] = {hostX, hostY, hostRY, hostZ, hostVX, hostVY, hostVZ, hostFX, hostFY, hostFZ};
  for (int k = 0; k < 10; ++k) g_elem[k] = (double *)dup_bytes(el[k], E * C * sizeof(double));
}
void sem_invokeGPUKernel_Force(void *model, void *g, int timeSteps, int *done, int *totalT, gsl_rng *r,
                               double gama) {
  (void)model; (void)g; (void)r; (void)gama;
  *totalT += timeSteps;
  g_steps = *totalT;
  if (*totalT >= g_steps_wanted) *done = 1;
}
void sem_copyGPUKernel(void *model, void *g, void *hostX, void *hostY, void *hostRY, void *hostZ, void *hostVX,
                       void *hostVY, void *hostVZ, void *hostFX, void *hostFY, void *hostFZ, int timeSteps) {
  (void)model; (void)g; (void)timeSteps;
  const int C = g_dims[0], E = g_dims[1];
  double *a[10] = {(double *)hostX, (double *)hostY, (double *)hostRY, (double *)hostZ, (double *)hostVX,
                   (double *)hostVY, (double *)hostVZ, (double *)hostFX, (double *)hostFY, (double *)hostFZ};
  for (int k = 0; k < 10; ++k)
    for (int i = 0; i < E; ++i)
      for (int j = 0; j < C; ++j) a[k][(size_t)i * C + j] = refhost_pattern(i, j, g_steps, k);
}
void sem_releaseGPUKernel(void *model, void *g) { (void)model; free(g); }
void *fiber_allocGPUKernel(void *model, int maxNodes, int maxLinks, int maxConn, double dt, double *p) {
  (void)model; (void)maxNodes; (void)maxLinks; (void)maxConn; (void)dt; (void)p;
  return NULL;
}
tmp_fiber_GPUgrids *init_fibrin_network(double dt) {
  tmp_fiber_GPUgrids *f = (tmp_fiber_GPUgrids *)calloc(1, sizeof *f);
  f->dt = dt;
  return f;
}

/* ------------------------------------------------------------ harness API */
/* Runs runGPUSimulation(seed) in `workdir` (which holds Input/ and Output/)
 * for `steps` coupled steps; returns the step count reached. */
int refhost_run(const char *workdir, int seed, int steps) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd)) return -1;
  if (chdir(workdir) != 0) return -1;
  g_steps_wanted = steps;
  g_steps = 0;
  runGPUSimulation(seed);
  if (chdir(cwd) != 0) return -1;
  return g_steps;
}
void refhost_dims(int out[6]) { memcpy(out, g_dims, sizeof g_dims); }
double refhost_S0_all(void) { return g_S0_all; }
double refhost_V0(void) { return g_V0; }
const int *refhost_tri(void) { return g_tri; }
const int *refhost_node_share(void) { return g_share; }
const double *refhost_normals(void) { return g_N; }
const int *refhost_ring_count(void) { return g_nbrnum; }
const int *refhost_ring(void) { return g_nbrnodes; }
const double *refhost_S0(void) { return g_S0; }
const double *refhost_bond_lengths(void) { return g_bonds; }
const double *refhost_elem(int k) { return (k >= 0 && k < 10) ? g_elem[k] : NULL; }
const float *refhost_r(int which) { return which ? g_r2 : g_r1; }
/* writeVTK of the driver (static there): float fields [nz][ny][nx] */
void refhost_write_vtk(int t, int nx, int ny, int nz, float *rho, float *ux, float *uy, float *uz, char *dir,
                       char *name) {
  writeVTK(t, nx, ny, nz, rho, 1, ux, uy, uz, 1, dir, name);
}
