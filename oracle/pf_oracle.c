/*
 * pf_oracle.c -- CPU FP64 restatement of the reference's per-timestep
 * coupled path (lattice Boltzmann + immersed boundary + subcellular-element
 * membrane + receptor bonds + position update), plus the Morse pair forces,
 * fibrin spring forces and half-way bounce-back walls that the benchmark
 * workloads add.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY: the tests compare the CUDA path with
 * it, and the benchmark times it as the CPU baseline.  The product library
 * never links it.
 *
 * The step follows the reference's launch order (gpuSEM_LB.c:1441-1442 calls
 * sem_invokeGPUKernel_Force, semLB.cu:441-531, then fluid_invokeGPUKernel,
 * semLB.cu:303-438).  Each routine names the kernel whose per-thread body it
 * restates.  The reference's mixed float/double arithmetic is kept where it
 * changes results: model parameters are float (semLB.cu:46), the lattice
 * speed C is computed in float (LB_kernel.cu:1117,1212), the spreading kernel
 * forms node coordinates as int*float (LB_kernel.cu:1437,1474), and the
 * moving-plate boundary keeps C, Nzx, Nzy in float (LB_kernel.cu:623-624).
 *
 * Semantics this restatement fixes where the reference is racy or undefined
 * (the CUDA path implements the same ones):
 *  - receptor threads read totalBond before any thread of the same step adds
 *    to it (sem_kernel.cu:1764 vs :2069), i.e. avaiBond = NUMOFRECEPTORS - 0;
 *  - vWF slot claims/releases are resolved in ascending receptor id order
 *    (the order a serial schedule of sem_kernel.cu:1750-2083 gives);
 *  - a receptor that drops from 2 bonds to 1 keeps its wall site (the
 *    reference erases it, sem_kernel.cu:1937-1942, and then indexes
 *    vWFbond[-1] on the next step);
 *  - wall-site indices outside the lattice wrap periodically for the slot
 *    table (the reference indexes out of bounds).
 */
#include "pf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D3Q19 velocity set in the reference's ordering (LB_kernel.cu:40-47); the
 * ordering is part of the fIN[19] host layout at the boundary. */
static const double W19[19] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                               1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
static const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0};
static const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1};
static const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1};
static int OPP[19];

#define PI_REF 3.141592653589793
#define BOND_THRESHOLD 0.078 /* sem_kernel.cu:79 */
#define K_RECEPT_VWF 10.0    /* sem_kernel.cu:84 */
#define KBT_BOND 4.05        /* sem_kernel.cu:82 */

static int g_threads = 1;
void pfo_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int pfo_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------ Philox */
/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two
 * 32x32->64 multiplies with the published multipliers and Weyl key bumps. */
void pfo_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
static double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}
void pfo_receptor_uniforms(uint64_t seed, int64_t step, int64_t receptor, double out[2]) {
  uint32_t ctr[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), (uint32_t)receptor,
                     (uint32_t)((uint64_t)receptor >> 32) ^ 0x52454350u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  pfo_philox4x32(ctr, key, o);
  out[0] = u53(o[0], o[1]);
  out[1] = u53(o[2], o[3]);
}
double pfo_detach_uniform(uint64_t seed, int64_t step) {
  uint32_t ctr[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), 0xFFFFFFFFu, 0x44455443u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  pfo_philox4x32(ctr, key, o);
  return u53(o[0], o[1]);
}

/* ------------------------------------------------------------------ state */
struct pfo_sim {
  pf_scene sc;
  int nx, ny, nz;
  size_t N;
  float dx, dt;
  float mp[100];
  int brute;
  double *fIN, *fOUT, *rho, *ux, *uy, *uz, *Fx, *Fy, *Fz;
  /* platelets */
  int P, E, Em, T, NN;
  int *tri, *node_ntri, *ring, *sp_ptr, *sp_nbr;
  double *sp_L0, *S0, *S0_all, *V0;
  double *X, *Y, *RY, *Z, *VX, *VY, *VZ, *FX, *FY, *FZ;
  double *nodeN, *Kapa, *km, *S, *nelem, *SV;
  /* receptors */
  int nrec;
  int *rec_tri, *rec_state, *vwf;
  float *r1, *r2;
  int total_bond;
  /* Morse cell list */
  int ncell[3];
  double cs[3];
  int *cell_of, *cell_start, *cell_order;
  /* fibrin */
  int M;
  double *fX, *fY, *fZ, *fVX, *fVY, *fVZ, *fFX, *fFY, *fFZ, *fL0;
  int *ffix, *fptr, *fnbr;
  double *fsX, *fsY, *fsZ; /* penalty coupling: lattice force on each node this step */
  long long step;
  int done;
};

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) abort();
  return p;
}
static void *xdup(const void *src, size_t bytes) {
  void *p = xcalloc(bytes ? bytes : 1, 1);
  if (src && bytes) memcpy(p, src, bytes);
  return p;
}

/* float-rounded lattice speed C = dx/dt/UMAX (LB_kernel.cu:1117,1212) */
static double lattice_C(const pfo_sim *s) {
  float dxf = s->dx, dtf = s->dt, umax = s->mp[PF_P_UMAX];
  float c = dxf / dtf;
  c = c / umax;
  return (double)c;
}

void pfo_feq(double rho, const double u[3], double C, double out[19]) {
  double C2 = C * C, C4 = C2 * C2;
  for (int d = 0; d < 19; ++d) {
    double e0 = CX[d] * C, e1 = CY[d] * C, e2 = CZ[d] * C;
    double cu = 3.0 * (e0 * u[0] + e1 * u[1] + e2 * u[2]);
    out[d] = rho * W19[d] *
             (1.0 + cu / C2 + 0.5 * cu * cu / C4 - 1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / C2);
  }
}

double pfo_ibm_phi(double r) { return 0.25 * (1.0 + cos(0.5 * PI_REF * r)); }

static int zouhe(const pfo_sim *s) { return s->sc.bc[2] == PF_BC_ZOUHE_SHEAR; }
static int penalty(const pfo_sim *s) { return s->sc.fib_coupling == PF_FIBCPL_PENALTY; }

/* wall velocity of the moving plate in units of UMAX (LB_kernel.cu:640) */
static double top_wall_uy(const pfo_sim *s) {
  float v = s->mp[PF_P_SHEAR] * (float)(s->nz - 1);
  v = v * s->dx;
  v = v / s->mp[PF_P_UMAX];
  return (double)v;
}

static void fib_flow_at(const pfo_sim *s, double x, double y, double z, double u[3], double *rho);

/* ------------------------------------------------------------------ create */
pfo_sim *pfo_create(const pf_scene *sc, int ibm_bruteforce) {
  for (int d = 0; d < 19; ++d)
    for (int e = 0; e < 19; ++e)
      if (CX[e] == -CX[d] && CY[e] == -CY[d] && CZ[e] == -CZ[d]) OPP[d] = e;
  pfo_sim *s = (pfo_sim *)xcalloc(1, sizeof *s);
  s->sc = *sc;
  s->brute = ibm_bruteforce;
  s->nx = sc->nx; s->ny = sc->ny; s->nz = sc->nz;
  s->N = (size_t)s->nx * s->ny * s->nz;
  s->dx = sc->dx; s->dt = sc->dt;
  memcpy(s->mp, sc->params, sizeof s->mp);
  size_t N = s->N;
  s->fIN = (double *)xcalloc(19 * N, sizeof(double));
  s->fOUT = (double *)xcalloc(19 * N, sizeof(double));
  s->rho = (double *)xcalloc(N, sizeof(double));
  s->ux = (double *)xcalloc(N, sizeof(double));
  s->uy = (double *)xcalloc(N, sizeof(double));
  s->uz = (double *)xcalloc(N, sizeof(double));
  s->Fx = (double *)xcalloc(N, sizeof(double));
  s->Fy = (double *)xcalloc(N, sizeof(double));
  s->Fz = (double *)xcalloc(N, sizeof(double));
  double C = lattice_C(s);
  /* Initial state.  Populations: given, or the reference driver's shear-flow
   * equilibrium (gpuSEM_LB.c:1206-1258), which forms C with a double UMAX.
   * Density/velocity of the first collision: the given rho_init/u_init (the
   * host arrays fluid_initGPUKernel uploads), else the values the
   * equilibrium was built from, else moments of f_init. */
  const int have_ru = sc->rho_init && sc->u_init;
  if (sc->f_init) {
    memcpy(s->fIN, sc->f_init, 19 * N * sizeof(double));
  } else {
    double shear = (double)s->mp[PF_P_SHEAR];
    double umax_d = shear > 0 ? shear * (s->nz - 1) * (double)s->dx : (double)s->mp[PF_P_UMAX];
    float dxdt = s->dx / s->dt;
    double C0 = (double)dxdt / umax_d, C02 = C0 * C0;
    for (int k = 0; k < s->nz; ++k)
      for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
          size_t n = (size_t)i + (size_t)s->nx * (j + (size_t)s->ny * k);
          double u[3] = {0, 0, 0}, r = 1.0;
          if (sc->u_init) {
            u[0] = sc->u_init[n]; u[1] = sc->u_init[N + n]; u[2] = sc->u_init[2 * N + n];
          } else if (zouhe(s)) {
            u[1] = shear * k * (double)s->dx / umax_d;
          }
          if (sc->rho_init) r = sc->rho_init[n];
          for (int d = 0; d < 19; ++d) {
            double cu = 3.0 * (CX[d] * u[0] + CY[d] * u[1] + CZ[d] * u[2]);
            s->fIN[d * N + n] = r * W19[d] * (1.0 + cu / C0 + 0.5 * cu * cu / C02 -
                                              1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / C02);
          }
          if (!have_ru) {
            s->rho[n] = r; s->ux[n] = u[0]; s->uy[n] = u[1]; s->uz[n] = u[2];
          }
        }
  }
  if (sc->F_init) {
    memcpy(s->Fx, sc->F_init, N * sizeof(double));
    memcpy(s->Fy, sc->F_init + N, N * sizeof(double));
    memcpy(s->Fz, sc->F_init + 2 * N, N * sizeof(double));
  }
  if (have_ru) {
    memcpy(s->rho, sc->rho_init, N * sizeof(double));
    memcpy(s->ux, sc->u_init, N * sizeof(double));
    memcpy(s->uy, sc->u_init + N, N * sizeof(double));
    memcpy(s->uz, sc->u_init + 2 * N, N * sizeof(double));
  } else if (sc->f_init) {
    /* moments of fIN with the half-force term (LB_kernel.cu:1108-1199); the
     * Zou/He planes hold the prescribed velocity */
    float fq = s->mp[PF_P_F0] / s->mp[PF_P_RHO0];
    fq = fq / s->mp[PF_P_UMAX];
    fq = fq * s->mp[PF_P_UNIT];
    double F_over = (double)fq;
    for (size_t n = 0; n < N; ++n) {
      double r = 0, a = 0, b = 0, c = 0;
      for (int d = 0; d < 19; ++d) {
        double f = s->fIN[d * N + n];
        r += f; a += CX[d] * f; b += CY[d] * f; c += CZ[d] * f;
      }
      s->rho[n] = r;
      s->ux[n] = (a * C + 0.5 * F_over * s->Fx[n] * (double)s->dt) / r;
      s->uy[n] = (b * C + 0.5 * F_over * s->Fy[n] * (double)s->dt) / r;
      s->uz[n] = (c * C + 0.5 * F_over * s->Fz[n] * (double)s->dt) / r;
      if (zouhe(s)) {
        int k = (int)(n / ((size_t)s->nx * s->ny));
        if (k == 0 || k == s->nz - 1) {
          s->ux[n] = 0; s->uz[n] = 0;
          s->uy[n] = (k == 0) ? 0.0 : top_wall_uy(s);
        }
      }
    }
  }

  /* platelets */
  s->P = sc->n_platelets; s->E = sc->n_elem; s->Em = sc->n_membrane; s->T = sc->n_tri; s->NN = sc->n_node;
  size_t PE = (size_t)s->P * s->E;
  s->tri = (int *)xdup(sc->tri, (size_t)s->T * 6 * sizeof(int));
  s->node_ntri = (int *)xdup(sc->node_ntri, (size_t)s->NN * sizeof(int));
  s->ring = (int *)xdup(sc->ring, (size_t)s->Em * 10 * sizeof(int));
  s->sp_ptr = (int *)xdup(sc->spring_ptr, (size_t)(s->E + 1) * sizeof(int));
  int nsp = (sc->spring_ptr && s->E > 0) ? sc->spring_ptr[s->E] : 0;
  if (!sc->spring_ptr) s->sp_ptr = (int *)xcalloc(s->E + 1, sizeof(int));
  s->sp_nbr = (int *)xdup(sc->spring_nbr, (size_t)nsp * sizeof(int));
  s->sp_L0 = (double *)xdup(sc->spring_L0, (size_t)nsp * sizeof(double));
  s->S0 = (double *)xdup(sc->S0, (size_t)s->P * s->T * sizeof(double));
  s->S0_all = (double *)xdup(sc->S0_all, (size_t)s->P * sizeof(double));
  s->V0 = (double *)xdup(sc->V0, (size_t)s->P * sizeof(double));
  s->X = (double *)xdup(sc->X, PE * sizeof(double));
  s->Y = (double *)xdup(sc->Y, PE * sizeof(double));
  s->RY = (double *)xdup(sc->RY, PE * sizeof(double));
  s->Z = (double *)xdup(sc->Z, PE * sizeof(double));
  s->VX = (double *)xcalloc(PE, sizeof(double));
  s->VY = (double *)xcalloc(PE, sizeof(double));
  s->VZ = (double *)xcalloc(PE, sizeof(double));
  s->FX = (double *)xcalloc(PE, sizeof(double));
  s->FY = (double *)xcalloc(PE, sizeof(double));
  s->FZ = (double *)xcalloc(PE, sizeof(double));
  s->nodeN = (double *)xcalloc((size_t)s->P * s->NN * 3, sizeof(double));
  s->Kapa = (double *)xcalloc((size_t)s->P * s->NN * 9, sizeof(double));
  s->km = (double *)xcalloc((size_t)s->P * s->NN, sizeof(double));
  s->S = (double *)xcalloc((size_t)s->P * s->T, sizeof(double));
  s->nelem = (double *)xcalloc((size_t)s->P * s->T * 3, sizeof(double));
  s->SV = (double *)xcalloc((size_t)s->P * 2, sizeof(double));

  /* receptors */
  s->nrec = sc->n_rec;
  size_t PR = (size_t)s->P * s->nrec;
  s->rec_tri = (int *)xdup(sc->rec_tri, PR * sizeof(int));
  s->r1 = (float *)xdup(sc->rec_r1, PR * sizeof(float));
  s->r2 = (float *)xdup(sc->rec_r2, PR * sizeof(float));
  s->rec_state = (int *)xcalloc(PR * 3, sizeof(int));
  if (sc->rec_state)
    memcpy(s->rec_state, sc->rec_state, PR * 3 * sizeof(int));
  else
    for (size_t r = 0; r < PR; ++r) {
      s->rec_state[3 * r] = -1; s->rec_state[3 * r + 1] = -1; s->rec_state[3 * r + 2] = -1;
    }
  s->vwf = (int *)xcalloc((size_t)4 * s->ny * s->nx, sizeof(int));
  if (sc->vwf)
    memcpy(s->vwf, sc->vwf, (size_t)4 * s->ny * s->nx * sizeof(int));
  else
    for (size_t q = 0; q < (size_t)4 * s->ny * s->nx; ++q) s->vwf[q] = -1;
  s->total_bond = 1; /* sem_initGPUKernel sets totalBond = 1 (semLB.cu:880) */

  /* Morse cell grid: cells of edge >= the largest cutoff over the lattice box */
  {
    double rc = sc->morse_intra[3] > sc->morse_inter[3] ? sc->morse_intra[3] : sc->morse_inter[3];
    int n3[3] = {s->nx, s->ny, s->nz};
    for (int a = 0; a < 3; ++a) {
      double L = n3[a] * (double)s->dx;
      int nc = (rc > 0) ? (int)floor(L / rc) : 1;
      if (nc < 1) nc = 1;
      s->ncell[a] = nc;
      s->cs[a] = L / nc;
    }
    size_t nct = (size_t)s->ncell[0] * s->ncell[1] * s->ncell[2];
    s->cell_of = (int *)xcalloc(PE, sizeof(int));
    s->cell_start = (int *)xcalloc(nct + 1, sizeof(int));
    s->cell_order = (int *)xcalloc(PE, sizeof(int));
  }

  /* fibrin */
  s->M = sc->n_fib;
  size_t M = (size_t)s->M;
  s->fX = (double *)xdup(sc->fib_X, M * sizeof(double));
  s->fY = (double *)xdup(sc->fib_Y, M * sizeof(double));
  s->fZ = (double *)xdup(sc->fib_Z, M * sizeof(double));
  s->fVX = (double *)xcalloc(M, sizeof(double));
  s->fVY = (double *)xcalloc(M, sizeof(double));
  s->fVZ = (double *)xcalloc(M, sizeof(double));
  s->fFX = (double *)xcalloc(M, sizeof(double));
  s->fFY = (double *)xcalloc(M, sizeof(double));
  s->fFZ = (double *)xcalloc(M, sizeof(double));
  s->ffix = (int *)xdup(sc->fib_fixed, M * sizeof(int));
  s->fptr = (int *)xdup(sc->fib_ptr, (M + 1) * sizeof(int));
  if (!sc->fib_ptr) s->fptr = (int *)xcalloc(M + 1, sizeof(int));
  int nfl = (sc->fib_ptr && M) ? sc->fib_ptr[M] : 0;
  s->fnbr = (int *)xdup(sc->fib_nbr, (size_t)nfl * sizeof(int));
  s->fL0 = (double *)xdup(sc->fib_L0, (size_t)nfl * sizeof(double));
  s->fsX = (double *)xcalloc(M, sizeof(double));
  s->fsY = (double *)xcalloc(M, sizeof(double));
  s->fsZ = (double *)xcalloc(M, sizeof(double));
  if (sc->fib_coupling == PF_FIBCPL_PENALTY)
    for (int m = 0; m < s->M; ++m) {
      /* initial node velocity: the flow's at the node (cpu_init_fiber_LB,
       * fiber.cpp:815-910, interpolates it trilinearly; here with the
       * coupling's own stencil); fixed nodes rest */
      if (s->ffix[m]) continue;
      double u[3], r;
      fib_flow_at(s, s->fX[m], s->fY[m], s->fZ[m], u, &r);
      s->fVX[m] = u[0]; s->fVY[m] = u[1]; s->fVZ[m] = u[2];
    }
  return s;
}

void pfo_destroy(pfo_sim *s) {
  if (!s) return;
  void *p[] = {s->fIN, s->fOUT, s->rho, s->ux, s->uy, s->uz, s->Fx, s->Fy, s->Fz, s->tri, s->node_ntri,
               s->ring, s->sp_ptr, s->sp_nbr, s->sp_L0, s->S0, s->S0_all, s->V0, s->X, s->Y, s->RY,
               s->Z, s->VX, s->VY, s->VZ, s->FX, s->FY, s->FZ, s->nodeN, s->Kapa, s->km, s->S,
               s->nelem, s->SV, s->rec_tri, s->rec_state, s->vwf, s->r1, s->r2, s->cell_of,
               s->cell_start, s->cell_order, s->fX, s->fY, s->fZ, s->fVX, s->fVY, s->fVZ, s->fFX,
               s->fFY, s->fFZ, s->fL0, s->ffix, s->fptr, s->fnbr, s->fsX, s->fsY, s->fsZ};
  for (size_t i = 0; i < sizeof p / sizeof p[0]; ++i) free(p[i]);
  free(s);
}

/* ================================================================ SEM */
/* Gaussian elimination with partial pivoting on a 3x4 augmented matrix,
 * normalising each pivot row (sem_kernel.cu:249-284). */
static void gauss_3x4(double g[3][4]) {
  int i = 0, j = 0;
  while (i < 3 && j < 3) {
    int maxi = i;
    for (int k = i + 1; k < 3; ++k)
      if (fabs(g[k][j]) > fabs(g[maxi][j])) maxi = k;
    if (g[maxi][j] != 0) {
      double piv = 0;
      for (int k = j; k < 4; ++k) {
        double t = g[i][k];
        g[i][k] = g[maxi][k];
        g[maxi][k] = t;
        if (k == j) piv = g[i][j];
        g[i][k] /= piv;
      }
      for (int k = i + 1; k < 3; ++k) {
        double f = g[k][j];
        for (int l = j; l < 4; ++l) g[k][l] -= f * g[i][l];
      }
      i++;
    }
    j++;
  }
}
/* Row i of A solves [a1; a3; a5] x = [a2_i; a4_i; a6_i] (sem_kernel.cu:286-311). */
static void solve_rows(double A[3][3], const double a1[3], const double a2[3], const double a3[3],
                       const double a4[3], const double a5[3], const double a6[3]) {
  for (int i = 0; i < 3; ++i) {
    double g[3][4];
    for (int j = 0; j < 3; ++j) { g[0][j] = a1[j]; g[1][j] = a3[j]; g[2][j] = a5[j]; }
    g[0][3] = a2[i]; g[1][3] = a4[i]; g[2][3] = a6[i];
    gauss_3x4(g);
    A[i][2] = g[2][3];
    A[i][1] = g[1][3] - A[i][2] * g[1][2];
    A[i][0] = g[0][3] - A[i][2] * g[0][2] - A[i][1] * g[0][1];
  }
}

/* Quadratic (6-node) triangle: derivatives of the shape functions
 * N0=(1-s-t)(1-2s-2t), N1=s(2s-1), N2=t(2t-1), N3=4s(1-s-t), N4=4t(1-s-t),
 * N5=4st at the 6 nodes (s,t) = (0,0),(1,0),(0,1),(.5,0),(0,.5),(.5,.5). */
static const double QN_ST[6][2] = {{0, 0}, {1, 0}, {0, 1}, {0.5, 0}, {0, 0.5}, {0.5, 0.5}};
static void p2_grad(double s_, double t_, double dNds[6], double dNdt[6]) {
  dNds[0] = 4 * s_ + 4 * t_ - 3; dNdt[0] = 4 * t_ + 4 * s_ - 3;
  dNds[1] = 4 * s_ - 1;          dNdt[1] = 0;
  dNds[2] = 0;                   dNdt[2] = 4 * t_ - 1;
  dNds[3] = -8 * s_ - 4 * t_ + 4; dNdt[3] = -4 * s_;
  dNds[4] = -4 * t_;             dNdt[4] = -8 * t_ - 4 * s_ + 4;
  dNds[5] = 4 * t_;              dNdt[5] = 4 * s_;
}

static double nrm3(double a, double b, double c) { return sqrt(a * a + b * b + c * c); }

/* The reference's disabled FEM bending chain, in the slot of its
 * commented-out launches (semLB.cu:518-520): after the curvature tensors
 * (divided by the node's triangle count and symmetrised, as
 * sem_calculate_m_kernel leaves them) and before the area/volume forces.
 *  1. sem_calculate_K_kernel (sem_kernel.cu:1129-1235): per triangle and
 *     each of its 6 nodes i, for each column l of the curvature tensors, the
 *     3x3 system rows (dx/ds, dx/dt, n_i) with right-hand sides
 *     (dKapa_l/ds, dKapa_l/dt, 0) is solved; row k of the solution, entry j,
 *     is added to K[node i][j][k][l].
 *  2. sem_calculate_q_kernel (:1237-1306): K divided by the node's triangle
 *     count, traceK_i = sum_j K[j][j][i], q_j = sum_i traceK_i (I - n n)_ij.
 *  3. sem_bending_force_kernel (:1308-1497): per triangle, edge tangents t
 *     and the in-plane normals b = t x n at the 6 nodes, line loads
 *     f = (b . q) n, Simpson's rule along the three sides; the total goes to
 *     each of the 3 vertices divided by S[vertex id] and F0.  S is the
 *     per-triangle area array, so the divisor is the area of the triangle
 *     whose index equals the vertex id: kept as the reference wrote it. */
static void fem_bending(pfo_sim *s, int p, const double *X, const double *Y, const double *Z, const double *nN,
                        const double *Kp, const double *S, double *FX, double *FY, double *FZ, double F0) {
  const int T = s->T, NN = s->NN;
  double *K = (double *)xcalloc((size_t)NN * 27, sizeof(double));
  double *q = (double *)xcalloc((size_t)NN * 3, sizeof(double));
  (void)p;
  for (int t = 0; t < T; ++t) {
    const int *nd = s->tri + 6 * t;
    double c[6][3];
    for (int i = 0; i < 3; ++i) { c[i][0] = X[nd[i]]; c[i][1] = Y[nd[i]]; c[i][2] = Z[nd[i]]; }
    for (int i = 0; i < 3; ++i) {
      c[3][i] = 0.5 * (c[0][i] + c[1][i]);
      c[4][i] = 0.5 * (c[0][i] + c[2][i]);
      c[5][i] = 0.5 * (c[1][i] + c[2][i]);
    }
    for (int i = 0; i < 6; ++i) {
      double gs[6], gt[6];
      p2_grad(QN_ST[i][0], QN_ST[i][1], gs, gt);
      for (int l = 0; l < 3; ++l) {
        double a1[3], a2[3], a3[3], a4[3], a5[3], a6[3], Ke[3][3];
        for (int j = 0; j < 3; ++j) {
          a1[j] = c[0][j] * gs[0] + c[1][j] * gs[1] + c[2][j] * gs[2] + c[3][j] * gs[3] + c[4][j] * gs[4] +
                  c[5][j] * gs[5];
          a3[j] = c[0][j] * gt[0] + c[1][j] * gt[1] + c[2][j] * gt[2] + c[3][j] * gt[3] + c[4][j] * gt[4] +
                  c[5][j] * gt[5];
          a2[j] = 0;
          a4[j] = 0;
          for (int m = 0; m < 6; ++m) a2[j] += Kp[9 * nd[m] + j * 3 + l] * gs[m];
          for (int m = 0; m < 6; ++m) a4[j] += Kp[9 * nd[m] + j * 3 + l] * gt[m];
          a5[j] = nN[3 * nd[i] + j];
          a6[j] = 0;
        }
        solve_rows(Ke, a1, a2, a3, a4, a5, a6);
        double *kr = K + 27 * nd[i];
        for (int k = 0; k < 3; ++k)
          for (int j = 0; j < 3; ++j) kr[j * 9 + k * 3 + l] += Ke[k][j];
      }
    }
  }
  for (int v = 0; v < NN; ++v) {
    double *kr = K + 27 * v;
    const double *n = nN + 3 * v;
    const int cnt = s->node_ntri[v];
    if (cnt <= 0) continue;
    for (int m = 0; m < 27; ++m) kr[m] /= cnt;
    for (int i = 0; i < 3; ++i) {
      const double tr = kr[i] + kr[12 + i] + kr[24 + i];
      for (int j = 0; j < 3; ++j) q[3 * v + j] += tr * ((i == j ? 1.0 : 0.0) - n[i] * n[j]);
    }
  }
  for (int t = 0; t < T; ++t) {
    const int *nd = s->tri + 6 * t;
    double c[3][3], nv[6][3], tv[6][3], L[3], b[6][6], f[6][6], F[3];
    for (int i = 0; i < 3; ++i) { c[i][0] = X[nd[i]]; c[i][1] = Y[nd[i]]; c[i][2] = Z[nd[i]]; }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 3; ++j) nv[i][j] = nN[3 * nd[i] + j];
    for (int j = 0; j < 3; ++j) {
      tv[0][j] = c[0][j] - c[1][j];
      tv[1][j] = c[1][j] - c[2][j];
      tv[2][j] = c[2][j] - c[0][j];
    }
    for (int i = 0; i < 3; ++i) L[i] = nrm3(tv[i][0], tv[i][1], tv[i][2]);
    for (int j = 0; j < 3; ++j) {
      tv[3][j] = tv[0][j] / L[0];
      tv[4][j] = tv[2][j] / L[2];
      tv[5][j] = tv[1][j] / L[1];
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) tv[i][j] /= L[i];
    /* b_i = t_i x n_i at every node; the vertices also along the other side
     * that meets them (t2 at vertex 0, t0 at vertex 1, t1 at vertex 2) */
    static const int other[3] = {2, 0, 1};
    for (int i = 0; i < 6; ++i) {
      b[i][0] = tv[i][1] * nv[i][2] - tv[i][2] * nv[i][1];
      b[i][1] = tv[i][2] * nv[i][0] - tv[i][0] * nv[i][2];
      b[i][2] = tv[i][0] * nv[i][1] - tv[i][1] * nv[i][0];
      const double nb = nrm3(b[i][0], b[i][1], b[i][2]);
      for (int j = 0; j < 3; ++j) b[i][j] /= nb;
    }
    for (int i = 0; i < 3; ++i) {
      const double *o = tv[other[i]];
      b[i][3] = o[1] * nv[i][2] - o[2] * nv[i][1];
      b[i][4] = o[2] * nv[i][0] - o[0] * nv[i][2];
      b[i][5] = o[0] * nv[i][1] - o[1] * nv[i][0];
      const double nb = nrm3(b[i][3], b[i][4], b[i][5]);
      for (int j = 3; j < 6; ++j) b[i][j] /= nb;
    }
    for (int i = 0; i < 6; ++i) {
      const double *qq = q + 3 * nd[i];
      const double bq = b[i][0] * qq[0] + b[i][1] * qq[1] + b[i][2] * qq[2];
      const double bq2 = i < 3 ? b[i][3] * qq[0] + b[i][4] * qq[1] + b[i][5] * qq[2] : 0.0;
      for (int j = 0; j < 3; ++j) {
        f[i][j] = bq * nv[i][j];
        if (i < 3) f[i][j + 3] = bq2 * nv[i][j];
      }
    }
    for (int j = 0; j < 3; ++j)
      F[j] = 0.5 * ((1 / 3.0 * (f[0][j] + f[1][j + 3]) + 4.0 / 3.0 * f[3][j]) * L[0] +
                    (1 / 3.0 * (f[1][j] + f[2][j + 3]) + 4.0 / 3.0 * f[5][j]) * L[1] +
                    (1 / 3.0 * (f[2][j] + f[0][j + 3]) + 4.0 / 3.0 * f[4][j]) * L[2]);
    for (int i = 0; i < 3; ++i) {
      const double Sv = S[nd[i]];
      FX[nd[i]] += F[0] / Sv / F0;
      FY[nd[i]] += F[1] / Sv / F0;
      FZ[nd[i]] += F[2] / Sv / F0;
    }
  }
  free(K);
  free(q);
}

/* One platelet's membrane force pass: sem_Force_kernel (:320-513),
 * sem_calculate_A_kernel (:724-872), sem_surface_tension_kernel (:874-948),
 * sem_calculate_Kapa_kernel (:950-1055), sem_calculate_m_kernel (:1057-1128),
 * sem_ForceAreaVol_kernel (:1640-1749), sem_Laplace_Kapa_kernel (:1499-1638),
 * in that order; forces in units of F0. */
static void membrane_forces(pfo_sim *s, int p) {
  const int E = s->E, T = s->T, NN = s->NN, Em = s->Em;
  double *X = s->X + (size_t)p * E, *Y = s->Y + (size_t)p * E, *RY = s->RY + (size_t)p * E;
  double *Z = s->Z + (size_t)p * E;
  double *FX = s->FX + (size_t)p * E, *FY = s->FY + (size_t)p * E, *FZ = s->FZ + (size_t)p * E;
  double *nN = s->nodeN + (size_t)p * NN * 3, *Kp = s->Kapa + (size_t)p * NN * 9;
  double *km = s->km + (size_t)p * NN, *S = s->S + (size_t)p * T, *ne = s->nelem + (size_t)p * T * 3;
  const double F0 = (double)s->mp[PF_P_F0];
  const int mask = s->sc.membrane_forces;
  memset(nN, 0, (size_t)NN * 3 * sizeof(double));
  memset(Kp, 0, (size_t)NN * 9 * sizeof(double));
  double S_all = 0, V = 0;

  /* springs on RY (sem_kernel.cu:355-389); element 0 then adds the wall
   * repulsion on the lowest element (:409-430) */
  for (int e = 0; e < E; ++e) {
    if (mask & PF_MEM_SPRING)
      for (int q = s->sp_ptr[e]; q < s->sp_ptr[e + 1]; ++q) {
        int nb = s->sp_nbr[q];
        double L0 = s->sp_L0[q];
        double d1 = X[nb] - X[e], d2 = RY[nb] - RY[e], d3 = Z[nb] - Z[e];
        double r = nrm3(d1, d2, d3);
        double w = r - L0;
        double fc = (double)s->mp[PF_P_KSPRING] * w / r;
        FX[e] += fc * d1 / 1.0 / F0;
        FY[e] += fc * d2 / 1.0 / F0;
        FZ[e] += fc * d3 / 1.0 / F0;
      }
    if (e == 0 && (mask & PF_MEM_WALL)) {
      double dmin = Z[0];
      int idx = 0;
      for (int i = 1; i < E; ++i)
        if (Z[i] < dmin) { dmin = Z[i]; idx = i; }
      if (dmin <= 0.02) {
        double rep = 5e-4 * 2000 * exp(-2000 * dmin) / (1 - exp(-2000 * dmin));
        FZ[idx] += rep / F0;
      }
    }
  }
  if (!(mask & (PF_MEM_AREAVOL | PF_MEM_BEND | PF_MEM_FEMBEND))) {
    s->SV[2 * p] = 0; s->SV[2 * p + 1] = 0;
    return;
  }
  /* areas, element normals, global area and volume, nodal normal sums */
  for (int t = 0; t < T; ++t) {
    const int *nd = s->tri + 6 * t;
    double c[3][3];
    for (int i = 0; i < 3; ++i) { c[i][0] = X[nd[i]]; c[i][1] = Y[nd[i]]; c[i][2] = Z[nd[i]]; }
    double cc[3], e12[3], e13[3], n[3];
    for (int i = 0; i < 3; ++i) cc[i] = 1 / 3.0 * (c[0][i] + c[1][i] + c[2][i]);
    for (int i = 0; i < 3; ++i) { e12[i] = c[1][i] - c[0][i]; e13[i] = c[2][i] - c[0][i]; }
    n[0] = e12[1] * e13[2] - e12[2] * e13[1];
    n[1] = e12[2] * e13[0] - e12[0] * e13[2];
    n[2] = e12[0] * e13[1] - e12[1] * e13[0];
    double nn = nrm3(n[0], n[1], n[2]);
    n[0] /= -nn; n[1] /= -nn; n[2] /= -nn;
    S[t] = 0.5 * nn;
    S_all += S[t];
    V += 1 / 3.0 * (cc[0] * n[0] + cc[1] * n[1] + cc[2] * n[2]) * S[t];
    for (int i = 0; i < 3; ++i) ne[3 * t + i] = n[i];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 3; ++j) nN[3 * nd[i] + j] += n[j];
  }
  for (int q = 0; q < NN; ++q) {
    double *r = nN + 3 * q;
    int cnt = s->node_ntri[q];
    if (cnt <= 0) continue;
    for (int i = 0; i < 3; ++i) r[i] /= cnt;
    double nn = nrm3(r[0], r[1], r[2]);
    for (int i = 0; i < 3; ++i) r[i] /= nn;
  }
  /* curvature tensor by the 6-node triangle, accumulated at all 6 nodes */
  for (int t = 0; t < T; ++t) {
    const int *nd = s->tri + 6 * t;
    double c[6][3], nv[6][3];
    for (int i = 0; i < 3; ++i) { c[i][0] = X[nd[i]]; c[i][1] = Y[nd[i]]; c[i][2] = Z[nd[i]]; }
    for (int i = 0; i < 3; ++i) {
      c[3][i] = 0.5 * (c[0][i] + c[1][i]);
      c[4][i] = 0.5 * (c[0][i] + c[2][i]);
      c[5][i] = 0.5 * (c[1][i] + c[2][i]);
    }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 3; ++j) nv[i][j] = nN[3 * nd[i] + j];
    for (int i = 0; i < 6; ++i) {
      double gs[6], gt[6], a1[3], a2[3], a3[3], a4[3], a5[3], a6[3], K[3][3];
      p2_grad(QN_ST[i][0], QN_ST[i][1], gs, gt);
      for (int j = 0; j < 3; ++j) {
        a1[j] = c[0][j] * gs[0] + c[1][j] * gs[1] + c[2][j] * gs[2] + c[3][j] * gs[3] + c[4][j] * gs[4] +
                c[5][j] * gs[5];
        a2[j] = nv[0][j] * gs[0] + nv[1][j] * gs[1] + nv[2][j] * gs[2] + nv[3][j] * gs[3] +
                nv[4][j] * gs[4] + nv[5][j] * gs[5];
        a3[j] = c[0][j] * gt[0] + c[1][j] * gt[1] + c[2][j] * gt[2] + c[3][j] * gt[3] + c[4][j] * gt[4] +
                c[5][j] * gt[5];
        a4[j] = nv[0][j] * gt[0] + nv[1][j] * gt[1] + nv[2][j] * gt[2] + nv[3][j] * gt[3] +
                nv[4][j] * gt[4] + nv[5][j] * gt[5];
        a5[j] = nv[i][j];
        a6[j] = 0;
      }
      solve_rows(K, a1, a2, a3, a4, a5, a6);
      double *kr = Kp + 9 * nd[i];
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) kr[k * 3 + l] += K[l][k];
    }
  }
  for (int q = 0; q < NN; ++q) {
    double *kr = Kp + 9 * q, K[3][3];
    int cnt = s->node_ntri[q];
    if (cnt <= 0) { km[q] = 0; continue; }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) { kr[i * 3 + j] /= cnt; K[i][j] = kr[i * 3 + j]; }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) kr[i * 3 + j] = 0.5 * (K[i][j] + K[j][i]);
    km[q] = 0.5 * (kr[0] + kr[4] + kr[8]);
  }
  s->SV[2 * p] = S_all;
  s->SV[2 * p + 1] = V;
  if (mask & PF_MEM_FEMBEND) fem_bending(s, p, X, Y, Z, nN, Kp, S, FX, FY, FZ, F0);
  /* area and volume penalty forces */
  if (mask & PF_MEM_AREAVOL) {
    const double Ks = (double)s->mp[PF_P_KS], Kv = (double)s->mp[PF_P_KV];
    const double S0_all = s->S0_all[p], V0 = s->V0[p];
    for (int t = 0; t < T; ++t) {
      const int *nd = s->tri + 6 * t;
      double c[3][3], L[3][3], cc[3], n[3], dS[3][3], dV[3][3], F[3];
      for (int i = 0; i < 3; ++i) { c[i][0] = X[nd[i]]; c[i][1] = Y[nd[i]]; c[i][2] = Z[nd[i]]; }
      double S0e = s->S0[(size_t)p * T + t], Se = S[t];
      for (int i = 0; i < 3; ++i) {
        L[0][i] = c[1][i] - c[2][i];
        L[1][i] = c[2][i] - c[0][i];
        L[2][i] = c[0][i] - c[1][i];
        cc[i] = 1 / 3.0 * (c[0][i] + c[1][i] + c[2][i]);
        n[i] = ne[3 * t + i];
      }
      for (int i = 0; i < 3; ++i) {
        dS[i][0] = -0.5 * (L[i][1] * n[2] - L[i][2] * n[1]);
        dS[i][1] = -0.5 * (L[i][2] * n[0] - L[i][0] * n[2]);
        dS[i][2] = -0.5 * (L[i][0] * n[1] - L[i][1] * n[0]);
        for (int j = 0; j < 3; ++j) F[j] = -Ks * ((Se - S0e) / S0e + (S_all - S0_all) / S0_all) * dS[i][j];
        FX[nd[i]] += F[0] / F0; FY[nd[i]] += F[1] / F0; FZ[nd[i]] += F[2] / F0;
      }
      dV[0][0] = -L[1][1] * L[0][2] / 3.0 + L[1][2] * L[0][1] / 3.0 - L[0][2] * cc[1] + L[0][1] * cc[2];
      dV[0][1] = -L[1][2] * L[0][0] / 3.0 + L[1][0] * L[0][2] / 3.0 + L[0][2] * cc[0] - L[0][0] * cc[2];
      dV[0][2] = -L[1][0] * L[0][1] / 3.0 + L[1][1] * L[0][0] / 3.0 - L[0][1] * cc[0] + L[0][0] * cc[1];
      dV[1][0] = -L[1][1] * L[0][2] / 3.0 + L[1][2] * L[0][1] / 3.0 - L[1][2] * cc[1] + L[1][1] * cc[2];
      dV[1][1] = -L[1][2] * L[0][0] / 3.0 + L[1][0] * L[0][2] / 3.0 + L[1][2] * cc[0] - L[1][0] * cc[2];
      dV[1][2] = -L[1][0] * L[0][1] / 3.0 + L[1][1] * L[0][0] / 3.0 - L[1][1] * cc[0] + L[1][0] * cc[1];
      dV[2][0] = -L[1][1] * L[0][2] / 3.0 + L[1][2] * L[0][1] / 3.0 - L[2][2] * cc[1] + L[2][1] * cc[2];
      dV[2][1] = -L[1][2] * L[0][0] / 3.0 + L[1][0] * L[0][2] / 3.0 + L[2][2] * cc[0] - L[2][0] * cc[2];
      dV[2][2] = -L[1][0] * L[0][1] / 3.0 + L[1][1] * L[0][0] / 3.0 - L[2][1] * cc[0] + L[2][0] * cc[1];
      for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) F[j] = -Kv * (V - V0) / V0 * dV[i][j] / 6.0;
        FX[nd[i]] += F[0] / F0; FY[nd[i]] += F[1] / F0; FZ[nd[i]] += F[2] / F0;
      }
    }
  }
  /* bending: cotangent Laplacian of the mean curvature over the vertex ring */
  if (mask & PF_MEM_BEND) {
    const float Kb = s->mp[PF_P_KBEND] * 1;
    for (int i = 0; i < Em; ++i) {
      int cnt = s->node_ntri[i];
      const int *rg = s->ring + 10 * i;
      double xi[3] = {X[i], Y[i], Z[i]}, ni[3] = {nN[3 * i], nN[3 * i + 1], nN[3 * i + 2]};
      double Ai = 0, sum = 0;
      for (int a = 0; a < cnt; ++a) {
        int jn = rg[a], jp = rg[a == 0 ? cnt - 1 : a - 1], jx = rg[a == cnt - 1 ? 0 : a + 1];
        double xj[3] = {X[jn], Y[jn], Z[jn]}, x1[3] = {X[jp], Y[jp], Z[jp]}, x2[3] = {X[jx], Y[jx], Z[jx]};
        double ri1[3], r1j[3], rij[3], ri2[3], r2j[3], cij[3], ci2[3], c2j[3], ce[3];
        for (int k = 0; k < 3; ++k) {
          ri1[k] = xi[k] - x1[k]; r1j[k] = x1[k] - xj[k]; rij[k] = xi[k] - xj[k];
          ri2[k] = xi[k] - x2[k]; r2j[k] = x2[k] - xj[k];
          cij[k] = 0.5 * (xi[k] + xj[k]); ci2[k] = 0.5 * (xi[k] + x2[k]); c2j[k] = 0.5 * (x2[k] + xj[k]);
        }
        double ai = rij[0] * ri2[0] + rij[1] * ri2[1] + rij[2] * ri2[2];
        double a2 = -(ri2[0] * r2j[0] + ri2[1] * r2j[1] + ri2[2] * r2j[2]);
        double aj = rij[0] * r2j[0] + rij[1] * r2j[1] + rij[2] * r2j[2];
        double a1 = -(r1j[0] * ri1[0] + r1j[1] * ri1[1] + r1j[2] * ri1[2]);
        if (ai < 0) {
          for (int k = 0; k < 3; ++k) ce[k] = c2j[k];
        } else if (a2 < 0) {
          for (int k = 0; k < 3; ++k) ce[k] = cij[k];
        } else if (aj < 0) {
          for (int k = 0; k < 3; ++k) ce[k] = ci2[k];
        } else {
          double g[3][4] = {{0}};
          for (int k = 0; k < 3; ++k) {
            g[0][k] = rij[k]; g[1][k] = ri2[k];
            g[0][3] += cij[k] * rij[k]; g[1][3] += ci2[k] * ri2[k];
          }
          g[2][0] = (xj[1] - xi[1]) * (x2[2] - xi[2]) - (xj[2] - xi[2]) * (x2[1] - xi[1]);
          g[2][1] = (xj[2] - xi[2]) * (x2[0] - xi[0]) - (xj[0] - xi[0]) * (x2[2] - xi[2]);
          g[2][2] = (xj[0] - xi[0]) * (x2[1] - xi[1]) - (xj[1] - xi[1]) * (x2[0] - xi[0]);
          g[2][3] = g[2][0] * xi[0] + g[2][1] * xi[1] + g[2][2] * xi[2];
          gauss_3x4(g);
          ce[2] = g[2][3];
          ce[1] = g[1][3] - ce[2] * g[1][2];
          ce[0] = g[0][3] - ce[2] * g[0][2] - ce[1] * g[0][1];
        }
        double L1 = nrm3(xi[0] - cij[0], xi[1] - cij[1], xi[2] - cij[2]);
        double L2 = nrm3(ce[0] - cij[0], ce[1] - cij[1], ce[2] - cij[2]);
        double L3 = nrm3(xi[0] - ce[0], xi[1] - ce[1], xi[2] - ce[2]);
        double Pe = 0.5 * (L1 + L2 + L3);
        Ai += sqrt(Pe * (Pe - L1) * (Pe - L2) * (Pe - L3));
        L1 = nrm3(xi[0] - ci2[0], xi[1] - ci2[1], xi[2] - ci2[2]);
        L2 = nrm3(ce[0] - ci2[0], ce[1] - ci2[1], ce[2] - ci2[2]);
        Pe = 0.5 * (L1 + L2 + L3);
        Ai += sqrt(Pe * (Pe - L1) * (Pe - L2) * (Pe - L3));
        double alpha = 1 / tan(acos(a1 / (nrm3(xi[0] - x1[0], xi[1] - x1[1], xi[2] - x1[2]) *
                                          nrm3(x1[0] - xj[0], x1[1] - xj[1], x1[2] - xj[2]))));
        double beta = 1 / tan(acos(a2 / (nrm3(xi[0] - x2[0], xi[1] - x2[1], xi[2] - x2[2]) *
                                         nrm3(x2[0] - xj[0], x2[1] - xj[1], x2[2] - xj[2]))));
        sum += 0.5 * (alpha + beta) * (km[jn] - km[i]);
      }
      FX[i] += (double)Kb / Ai * sum * ni[0] / F0;
      FY[i] += (double)Kb / Ai * sum * ni[1] / F0;
      FZ[i] += (double)Kb / Ai * sum * ni[2] / F0;
    }
  }
}

/* ---------------------------------------------------------------- Morse */
static void build_cells(pfo_sim *s) {
  size_t PE = (size_t)s->P * s->E;
  int n3[3] = {s->nx, s->ny, s->nz};
  size_t nct = (size_t)s->ncell[0] * s->ncell[1] * s->ncell[2];
  memset(s->cell_start, 0, (nct + 1) * sizeof(int));
  for (size_t g = 0; g < PE; ++g) {
    double pos[3] = {s->X[g], s->Y[g], s->Z[g]};
    int c[3];
    for (int a = 0; a < 3; ++a) {
      double L = n3[a] * (double)s->dx, x = pos[a];
      if (s->sc.ibm_wrap[a]) x -= L * floor(x / L);
      int ci = (int)floor(x / s->cs[a]);
      if (ci < 0) ci = 0;
      if (ci >= s->ncell[a]) ci = s->ncell[a] - 1;
      c[a] = ci;
    }
    int cid = c[0] + s->ncell[0] * (c[1] + s->ncell[1] * c[2]);
    s->cell_of[g] = cid;
    s->cell_start[cid + 1]++;
  }
  for (size_t q = 0; q < nct; ++q) s->cell_start[q + 1] += s->cell_start[q];
  int *fill = (int *)xcalloc(nct, sizeof(int));
  for (size_t g = 0; g < PE; ++g) {
    int cid = s->cell_of[g];
    s->cell_order[s->cell_start[cid] + fill[cid]++] = (int)g;
  }
  free(fill);
}

/* Force-shifted Morse pair force for 0 < r < cutoff:
 *   F(r) = 2 rho U0 [e^{2rho(req-r)} - e^{rho(req-r)}]   (-dV/dr of
 *   V(r) = U0[e^{2rho(req-r)} - 2 e^{rho(req-r)}]),
 *   f_i += (F(r) - F(cutoff)) (xi - xj)/r,
 * so the force is continuous at the cutoff (a plain truncation jumps there,
 * and pairs sitting at the cutoff then decide the result by rounding). */
static double morse_F(const double *mp, double r) {
  double ex = exp(mp[1] * (mp[2] - r));
  return 2.0 * mp[1] * mp[0] * (ex * ex - ex);
}
static void morse_forces(pfo_sim *s) {
  build_cells(s);
  const int E = s->E;
  size_t PE = (size_t)s->P * E;
  const double F0 = (double)s->mp[PF_P_F0];
  double L3[3] = {s->nx * (double)s->dx, s->ny * (double)s->dx, s->nz * (double)s->dx};
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64)
  for (long long g = 0; g < (long long)PE; ++g) {
    int cid = s->cell_of[g];
    int c0 = cid % s->ncell[0], c1 = (cid / s->ncell[0]) % s->ncell[1], c2 = cid / (s->ncell[0] * s->ncell[1]);
    int pg = (int)(g / E);
    double xi = s->X[g], yi = s->Y[g], zi = s->Z[g];
    double fx = 0, fy = 0, fz = 0;
    int seen[27], nseen = 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dxo = -1; dxo <= 1; ++dxo) {
          int cc[3] = {c0 + dxo, c1 + dy, c2 + dz}, ok = 1;
          for (int a = 0; a < 3; ++a) {
            if (cc[a] < 0 || cc[a] >= s->ncell[a]) {
              if (s->sc.ibm_wrap[a]) cc[a] = (cc[a] + s->ncell[a]) % s->ncell[a];
              else ok = 0;
            }
          }
          if (!ok) continue;
          int nc = cc[0] + s->ncell[0] * (cc[1] + s->ncell[1] * cc[2]);
          int dup = 0;
          for (int q = 0; q < nseen; ++q) dup |= (seen[q] == nc);
          if (dup) continue;
          seen[nseen++] = nc;
          for (int q = s->cell_start[nc]; q < s->cell_start[nc + 1]; ++q) {
            int h = s->cell_order[q];
            if (h == g) continue;
            double d[3] = {xi - s->X[h], yi - s->Y[h], zi - s->Z[h]};
            for (int a = 0; a < 3; ++a)
              if (s->sc.ibm_wrap[a]) d[a] -= L3[a] * floor(d[a] / L3[a] + 0.5);
            double r = nrm3(d[0], d[1], d[2]);
            const double *mp = (h / E == pg) ? s->sc.morse_intra : s->sc.morse_inter;
            if (!(r < mp[3]) || r <= 0) continue;
            double f = (morse_F(mp, r) - morse_F(mp, mp[3])) / r;
            fx += f * d[0]; fy += f * d[1]; fz += f * d[2];
          }
        }
    s->FX[g] += fx / F0; s->FY[g] += fy / F0; s->FZ[g] += fz / F0;
  }
}

/* ---------------------------------------------------------------- fibrin */
/* Per-node gather over the node's links (fiber.cpp:647-706): F_ni -= wf *
 * (x_ni - x_other)/len with wf the worm-like-chain law of fiber.cpp:710-733
 * or the Hookean k (len - len0). */
static double wlc_force(double l0, double l, double mass) {
  const double kB = 1.3806503 * 1e-8, mTemp = 10, En = kB * mTemp;
  double CC = En / l0;
  double tl = 1.0 - (l - l0) / l0;
  double IP1 = 0.25 * 1.0 / (tl * tl) - 0.25 + (l - l0) / l0;
  return -CC * IP1 / mass;
}
double pfo_wlc_force(double l0, double l, double mass) { return wlc_force(l0, l, mass); }
static void fibrin_forces(pfo_sim *s) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ni = 0; ni < s->M; ++ni) {
    double fx = 0, fy = 0, fz = 0;
    for (int q = s->fptr[ni]; q < s->fptr[ni + 1]; ++q) {
      int o = s->fnbr[q];
      double d0 = s->fX[ni] - s->fX[o], d1 = s->fY[ni] - s->fY[o], d2 = s->fZ[ni] - s->fZ[o];
      double len = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
      if (len < 1.0e-13) continue;
      double wf = (s->sc.fib_law == PF_FIB_WLC) ? wlc_force(s->fL0[q], len, s->sc.fib_mass)
                                                : s->sc.fib_k * (len - s->fL0[q]);
      fx -= wf * d0 / len; fy -= wf * d1 / len; fz -= wf * d2 / len;
    }
    s->fFX[ni] = fx; s->fFY[ni] = fy; s->fFZ[ni] = fz;
  }
}

/* ---------------------------------------------------------------- bonds */
static int wrapi(int a, int n) { int r = a % n; return r < 0 ? r + n : r; }

/* sem_platelet_wall_kernel (sem_kernel.cu:1750-2083), receptors in id order */
static void receptor_bonds(pfo_sim *s) {
  const double dt = (double)s->dt, dx = (double)s->dx, F0 = (double)s->mp[PF_P_F0];
  const int avai = (int)(s->mp[PF_P_NUMRECEPTORS] - 0); /* totalBond read before any add */
  int total = 0;
  const int nx = s->nx, ny = s->ny;
  for (int p = 0; p < s->P; ++p) {
    const size_t eo = (size_t)p * s->E;
    for (int k = 0; k < s->nrec; ++k) {
      const size_t rid = (size_t)p * s->nrec + k;
      const int id = (int)rid;
      int *st = s->rec_state + 3 * rid;
      const int *nd = s->tri + 6 * s->rec_tri[rid];
      double c[3][3];
      for (int i = 0; i < 3; ++i) {
        c[i][0] = s->X[eo + nd[i]]; c[i][1] = s->Y[eo + nd[i]]; c[i][2] = s->Z[eo + nd[i]];
      }
      float r1 = s->r1[rid], r2 = s->r2[rid];
      float wa = 1 - r1, wb = r1 * (1 - r2), wc = r1 * r2;
      double rz = wa * c[0][2] + wb * c[1][2] + wc * c[2][2];
      int bond = st[2] > -1 ? st[2] : 0;
      if (rz > BOND_THRESHOLD && bond == 0) continue;
      double rx = wa * c[0][0] + wb * c[1][0] + wc * c[2][0];
      double ry = wa * c[0][1] + wb * c[1][1] + wc * c[2][1];
      int si, sj;
      if (bond) { si = st[0]; sj = st[1]; }
      else { si = (int)(rx / dx + 0.5); sj = (int)(ry / dx + 0.5); }
      double d1 = rx - si * dx, d2 = ry - sj * dx, d3 = rz;
      double dr = nrm3(d1, d2, d3);
      double w = fabs(BOND_THRESHOLD - dr);
      double fc = K_RECEPT_VWF * w;
      double aon, aoff;
      if (s->sc.bond_model == PF_BOND_BELL) {
        double Kf = (double)s->mp[PF_P_KF0] * exp(fc * (0.00071 - 0.5 * w) / KBT_BOND) * avai;
        double Kr = (double)s->mp[PF_P_KR0] * exp(0.00071 * fc / KBT_BOND) * avai;
        aon = 1 - exp(-Kf * dt);
        aoff = 1 - exp(-Kr * dt);
      } else {
        aon = s->sc.p_on;
        aoff = s->sc.p_off;
      }
      double u[2];
      pfo_receptor_uniforms(s->sc.seed, s->step, (int64_t)rid, u);
      int *slot0 = s->vwf;
      size_t plane = (size_t)nx * ny;
#define SLOT(kk, ii, jj) slot0[(size_t)(kk)*plane + (size_t)wrapi(jj, ny) * nx + wrapi(ii, nx)]
      /* claim one slot at the nearest site; returns 1 on success */
#define CLAIM()                                                              \
  do {                                                                       \
    si = (int)(rx / dx + 0.5); sj = (int)(ry / dx + 0.5);                    \
    for (int kk = 0; kk < 4; ++kk)                                           \
      if (SLOT(kk, si, sj) == -1) { SLOT(kk, si, sj) = id; bond++; st[0] = si; st[1] = sj; claimed = 1; break; } \
  } while (0)
#define RELEASE()                                                            \
  do {                                                                       \
    for (int kk = 0; kk < 4; ++kk)                                           \
      if (SLOT(kk, si, sj) == id) { SLOT(kk, si, sj) = -1; bond--; released = 1; break; } \
    if (released && bond == 0) { st[0] = -1; st[1] = -1; }                   \
  } while (0)
      int claimed = 0, released = 0;
      if (bond == 0) {
        if (u[0] < aon) CLAIM();
        claimed = 0;
        if (u[1] < aon) CLAIM();
      } else if (bond == 1) {
        if (u[0] < aoff) {
          RELEASE();
          if (u[1] < aon && rz < BOND_THRESHOLD) { claimed = 0; CLAIM(); }
        } else if (u[1] < aoff && rz < BOND_THRESHOLD) {
          RELEASE();
        }
      } else if (bond == 2) {
        if (u[0] < aoff) RELEASE();
        released = 0;
        if (u[1] < aoff) RELEASE();
      }
#undef CLAIM
#undef RELEASE
#undef SLOT
      (void)claimed;
      if (bond) {
        d1 = rx - si * dx; d2 = ry - sj * dx; d3 = rz;
        dr = nrm3(d1, d2, d3);
        double wt = BOND_THRESHOLD - dr;
        double fcb = K_RECEPT_VWF * wt * bond / dr;
        double fX = fcb * d1, fY = fcb * d2, fZ = fcb * d3, drv[3];
        for (int m = 0; m < 3; ++m) drv[m] = nrm3(rx - c[m][0], ry - c[m][1], rz - c[m][2]);
        double sum = 1.0 / drv[0] + 1.0 / drv[1] + 1.0 / drv[2];
        for (int m = 0; m < 3; ++m) {
          s->FX[eo + nd[m]] += fX * 1.0 / drv[m] / sum / F0;
          s->FY[eo + nd[m]] += fY * 1.0 / drv[m] / sum / F0;
          s->FZ[eo + nd[m]] += fZ * 1.0 / drv[m] / sum / F0;
        }
        st[2] = bond;
        total += bond;
      } else {
        st[2] = -1;
      }
    }
  }
  s->total_bond = total;
}

/* ---------------------------------------------------------------- IBM */
typedef struct { int node; double w; } stw;
/* Nodes of one axis within 2dx of coordinate x with their cosine weights.
 * spread=1 forms node coordinates as int*float (LB_kernel.cu:1474),
 * spread=0 as int*double (LB_kernel.cu:1581). */
static int axis_stencil(double x, float dxf, int n, int wrap, int spread, stw out[5]) {
  double dxd = (double)dxf;
  double thr = (double)(2 * dxf);
  int base = (int)floor(x / dxd);
  int cnt = 0;
  for (int ii = base - 2; ii <= base + 2; ++ii) {
    double xn = spread ? (double)((float)ii * dxf) : ii * dxd;
    if (fabs(x - xn) >= thr) continue;
    int node = ii;
    if (ii < 0 || ii >= n) {
      if (!wrap) continue;
      node = wrapi(ii, n);
    }
    out[cnt].node = node;
    out[cnt].w = 0.25 * (1.0 + cos(0.5 * PI_REF * (x - xn) / dxd));
    cnt++;
  }
  return cnt;
}

static void spread_marker(pfo_sim *s, double x, double y, double z, double fx, double fy, double fz) {
  stw ax[5], ay[5], az[5];
  int nxs = axis_stencil(x, s->dx, s->nx, s->sc.ibm_wrap[0], 1, ax);
  int nys = axis_stencil(y, s->dx, s->ny, s->sc.ibm_wrap[1], 1, ay);
  int nzs = axis_stencil(z, s->dx, s->nz, 0, 1, az);
  for (int c = 0; c < nzs; ++c)
    for (int b = 0; b < nys; ++b)
      for (int a = 0; a < nxs; ++a) {
        double delta = ax[a].w * ay[b].w * az[c].w;
        size_t n = (size_t)ax[a].node + (size_t)s->nx * (ay[b].node + (size_t)s->ny * az[c].node);
        s->Fx[n] += fx * delta; s->Fy[n] += fy * delta; s->Fz[n] += fz * delta;
      }
}
static void interp_marker(const pfo_sim *s, double x, double y, double z, double *vx, double *vy, double *vz) {
  stw ax[5], ay[5], az[5];
  int nxs = axis_stencil(x, s->dx, s->nx, s->sc.ibm_wrap[0], 0, ax);
  int nys = axis_stencil(y, s->dx, s->ny, s->sc.ibm_wrap[1], 0, ay);
  int nzs = axis_stencil(z, s->dx, s->nz, 0, 0, az);
  double a0 = 0, a1 = 0, a2 = 0;
  for (int c = 0; c < nzs; ++c)
    for (int b = 0; b < nys; ++b)
      for (int a = 0; a < nxs; ++a) {
        double delta = ax[a].w * ay[b].w * az[c].w;
        size_t n = (size_t)ax[a].node + (size_t)s->nx * (ay[b].node + (size_t)s->ny * az[c].node);
        a0 += s->ux[n] * delta; a1 += s->uy[n] * delta; a2 += s->uz[n] * delta;
      }
  *vx = a0; *vy = a1; *vz = a2;
}

/* ------------------------------------------------ fibrin penalty coupling */
/* Flow_vel_at_position (fiber.cpp:753-814): flow velocity and density at a
 * fibrin node, summed over the stencil with the IBM kernel
 * phi(r) = (1 + cos(pi r / 2)) / 4, |r| < 2 (r in lattice spacings), nodes
 * of the Zou/He wall planes (the obstacle nodes there) skipped, weights not
 * renormalised.  The text's DH1D (fiber.cpp:82-103) is that kernel with two
 * slips, fixed here: its non-zero branch computes the value without
 * returning it, and its callers pass distances already divided by dx. */
static void fib_flow_at(const pfo_sim *s, double x, double y, double z, double u[3], double *rho) {
  stw ax[5], ay[5], az[5];
  int nxs = axis_stencil(x, s->dx, s->nx, s->sc.ibm_wrap[0], 0, ax);
  int nys = axis_stencil(y, s->dx, s->ny, s->sc.ibm_wrap[1], 0, ay);
  int nzs = axis_stencil(z, s->dx, s->nz, 0, 0, az);
  const int walls = zouhe(s);
  double a0 = 0, a1 = 0, a2 = 0, r = 0;
  for (int c = 0; c < nzs; ++c) {
    if (walls && (az[c].node == 0 || az[c].node == s->nz - 1)) continue;
    for (int b = 0; b < nys; ++b)
      for (int a = 0; a < nxs; ++a) {
        double delta = ax[a].w * ay[b].w * az[c].w;
        size_t n = (size_t)ax[a].node + (size_t)s->nx * (ay[b].node + (size_t)s->ny * az[c].node);
        a0 += s->ux[n] * delta; a1 += s->uy[n] * delta; a2 += s->uz[n] * delta;
        r += s->rho[n] * delta;
      }
  }
  u[0] = a0; u[1] = a1; u[2] = a2;
  *rho = r;
}

/* reference nodal force -> lattice force: F0/rho0/UMAX*1e12 * dt / C */
static double fib_force_scale(const pfo_sim *s) {
  const double Kd = (double)s->mp[PF_P_F0] / (double)s->mp[PF_P_RHO0] / (double)s->mp[PF_P_UMAX] *
                    (double)s->mp[PF_P_UNIT];
  return Kd * (double)s->dt / lattice_C(s);
}

/* fiber_LB_Fsi_force (fiber.cpp:501-600): the penalty force
 * kappa rho (u - V) / dt on each node (lattice units; u and V in units of
 * UMAX, so divided by C) from the flow of this step's moments at the node.
 * The fluid receives the reaction in the next step's force (spread then,
 * at the node's position then): fibrin_penalty_spread.  The text adds
 * +rho (u - V)/dt to the fluid populations, which pushes the fluid away from
 * the node's velocity; the reaction (momentum exchange) is used here. */
static void fibrin_penalty(pfo_sim *s) {
  const double C = lattice_C(s), kap = s->sc.fib_kappa;
  for (int m = 0; m < s->M; ++m) {
    double u[3], r;
    fib_flow_at(s, s->fX[m], s->fY[m], s->fZ[m], u, &r);
    s->fsX[m] = kap * r * (u[0] - s->fVX[m]) / C;
    s->fsY[m] = kap * r * (u[1] - s->fVY[m]) / C;
    s->fsZ[m] = kap * r * (u[2] - s->fVZ[m]) / C;
  }
}
/* the previous step's penalty reaction onto the lattice force, with the
 * marker stencil, in reference force units (lattice force / scale) */
static void fibrin_penalty_spread(pfo_sim *s) {
  const double kc = fib_force_scale(s);
  for (int m = 0; m < s->M; ++m)
    spread_marker(s, s->fX[m], s->fY[m], s->fZ[m], -s->fsX[m] / kc, -s->fsY[m] / kc, -s->fsZ[m] / kc);
}

/* network::solverkick (network.cpp:839-881) over half a lattice step:
 * v <- e^{-gamma/2} v + a (1 - e^{-gamma/2}) / gamma (a/2 for gamma = 0),
 * a = (link force + penalty force) / node mass in lattice units; fixed
 * nodes rest. */
static void fibrin_kick(pfo_sim *s) {
  const double C = lattice_C(s), kc = fib_force_scale(s), F0 = (double)s->mp[PF_P_F0];
  const double g = s->sc.fib_gamma, mass = s->sc.fib_node_mass;
  const double vdt = exp(-0.5 * g), fdt = g > 0 ? (1.0 - vdt) / g : 0.5;
  double *V[3] = {s->fVX, s->fVY, s->fVZ}, *F[3] = {s->fFX, s->fFY, s->fFZ}, *P[3] = {s->fsX, s->fsY, s->fsZ};
  for (int m = 0; m < s->M; ++m)
    for (int a = 0; a < 3; ++a) {
      if (s->ffix[m]) { V[a][m] = 0; continue; }
      const double acc = (F[a][m] / F0 * kc + P[a][m]) / mass;
      V[a][m] = (vdt * (V[a][m] / C) + acc * fdt) * C;
    }
}

/* network::Solve (network.cpp:445-513): kick, drift of the free nodes, link
 * forces at the new positions, kick (the penalty force held over the step) */
static void fibrin_integrate(pfo_sim *s) {
  float dtT = s->dt / s->mp[PF_P_T0];
  double Lx = s->nx * (double)s->dx, Ly = s->ny * (double)s->dx;
  fibrin_kick(s);
  for (int m = 0; m < s->M; ++m) {
    if (s->ffix[m]) continue;
    s->fX[m] += s->fVX[m] * dtT;
    if (s->sc.ibm_wrap[0]) {
      if (s->fX[m] > Lx) s->fX[m] -= Lx;
      else if (s->fX[m] < 0) s->fX[m] += Lx;
    }
    s->fY[m] += s->fVY[m] * dtT;
    if (s->sc.ibm_wrap[1]) {
      if (s->fY[m] > Ly) s->fY[m] -= Ly;
      else if (s->fY[m] < 0) s->fY[m] += Ly;
    }
    s->fZ[m] += s->fVZ[m] * dtT;
  }
  fibrin_forces(s);
  fibrin_kick(s);
}

/* Node-centric loops of fluid3d_force_distribute_kernel and
 * fluid3d_velocity_distribute_kernel (LB_kernel.cu:1419-1642), including the
 * y-image pass for j<2 || j>ly-2; only for the reference's axis set
 * (x and z bounded, y periodic). */
static void brute_pass(pfo_sim *s, int spread) {
  const float dxf = s->dx;
  const double dxd = (double)dxf;
  const int nm = s->P * s->E;
  for (int k = 0; k < s->nz; ++k)
    for (int j0 = 0; j0 < s->ny; ++j0)
      for (int i = 0; i < s->nx; ++i) {
        size_t n = (size_t)i + (size_t)s->nx * (j0 + (size_t)s->ny * k);
        int passes = (j0 < 2 || j0 > s->ny - 2) ? 2 : 1;
        for (int pass = 0; pass < passes; ++pass) {
          int j = j0;
          if (pass == 1) j = (j0 < 2) ? j0 + s->ny : j0 - s->ny;
          for (int m = 0; m < nm; ++m) {
            double x = s->X[m], y = s->Y[m], z = s->Z[m];
            double thr, xi, yj, zk;
            if (spread) {
              thr = (double)(2 * dxf);
              xi = (double)(i * dxf); yj = (double)(j * dxf); zk = (double)(k * dxf);
            } else {
              thr = 2 * dxd;
              xi = i * dxd; yj = j * dxd; zk = k * dxd;
            }
            if (fabs(x - xi) >= thr) continue;
            if (fabs(y - yj) >= thr) continue;
            if (fabs(z - zk) >= thr) continue;
            double delta = (0.25 * (1.0 + cos(0.5 * PI_REF * (x - xi) / dxd))) *
                           (0.25 * (1.0 + cos(0.5 * PI_REF * (y - yj) / dxd))) *
                           (0.25 * (1.0 + cos(0.5 * PI_REF * (z - zk) / dxd)));
            if (spread) {
              s->Fx[n] += s->FX[m] * delta; s->Fy[n] += s->FY[m] * delta; s->Fz[n] += s->FZ[m] * delta;
            } else {
              s->VX[m] += s->ux[n] * delta; s->VY[m] += s->uy[n] * delta; s->VZ[m] += s->uz[n] * delta;
            }
          }
        }
      }
}
static int brute_ok(const pfo_sim *s) {
  return s->brute && !s->sc.ibm_wrap[0] && s->sc.ibm_wrap[1] && s->M == 0;
}

/* ---------------------------------------------------------------- lattice */
/* fluid3d_collision_kernel (LB_kernel.cu:1203-1304) */
static void collide(pfo_sim *s) {
  const size_t N = s->N;
  const double C = lattice_C(s), C2 = C * C, C4 = C2 * C2;
  const double tau = (double)s->mp[PF_P_TAU];
  const double F0 = (double)s->mp[PF_P_F0], R0 = (double)s->mp[PF_P_RHO0], UM = (double)s->mp[PF_P_UMAX];
  const double UF = (double)s->mp[PF_P_UNIT], dtd = (double)s->dt;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    size_t n = (size_t)nn;
    double rho = s->rho[n], u[3] = {s->ux[n], s->uy[n], s->uz[n]};
    double F[3] = {s->Fx[n], s->Fy[n], s->Fz[n]}, uF[3][3];
    for (int l = 0; l < 3; ++l)
      for (int m = 0; m < 3; ++m) uF[l][m] = u[l] * F[m] + F[l] * u[m];
    for (int d = 0; d < 19; ++d) {
      double e[3] = {CX[d] * C, CY[d] * C, CZ[d] * C}, ee[3][3], sum = 0;
      double cu = 3.0 * (e[0] * u[0] + e[1] * u[1] + e[2] * u[2]);
      for (int l = 0; l < 3; ++l)
        for (int m = 0; m < 3; ++m) ee[l][m] = (l == m) ? e[l] * e[m] - C2 / 3.0 : e[l] * e[m];
      for (int l = 0; l < 3; ++l)
        for (int m = 0; m < 3; ++m) sum += uF[l][m] * ee[m][l];
      double fEQ = rho * W19[d] * (1.0 + cu / C2 + 0.5 * cu * cu / C4 - 1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / C2);
      double fin = s->fIN[d * N + n];
      double fdt = W19[d] * (1.0 - 0.5 / tau) * (3.0 * (e[0] * F[0] + e[1] * F[1] + e[2] * F[2]) / C2 + 4.5 * sum / C4) * dtd;
      s->fOUT[d * N + n] = fin - (1.0 / tau) * (fin - fEQ) + F0 * fdt / R0 / UM * UF;
    }
  }
}

/* fluid3d_stream_kernel (LB_kernel.cu:1312-1359): periodic pull; on a
 * bounce-back axis a population entering through the face is the node's own
 * post-collision opposite population (half-way bounce-back, the pairing of
 * LB_kernel.cu:1070-1106 with :1362-1414 for a wall half a spacing outside). */
static void stream(pfo_sim *s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const size_t N = s->N;
  const int bbx = s->sc.bc[0] == PF_BC_BOUNCEBACK, bby = s->sc.bc[1] == PF_BC_BOUNCEBACK,
            bbz = s->sc.bc[2] == PF_BC_BOUNCEBACK;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t n = (size_t)i + (size_t)nx * (j + (size_t)ny * k);
        for (int d = 0; d < 19; ++d) {
          int si = i - CX[d], sj = j - CY[d], sk = k - CZ[d];
          int out = (bbx && (si < 0 || si >= nx)) || (bby && (sj < 0 || sj >= ny)) || (bbz && (sk < 0 || sk >= nz));
          if (out) {
            s->fIN[d * N + n] = s->fOUT[OPP[d] * N + n];
            continue;
          }
          if (si < 0) si = nx - 1;
          if (sj < 0) sj = ny - 1;
          if (sk < 0) sk = nz - 1;
          if (si == nx) si = 0;
          if (sj == ny) sj = 0;
          if (sk == nz) sk = 0;
          s->fIN[d * N + n] = s->fOUT[d * N + (size_t)si + (size_t)nx * (sj + (size_t)ny * sk)];
        }
      }
}

/* fluid3d_noslip_boundary_kernel (LB_kernel.cu:395-600) at z=0 and
 * fluid3d_moving_plate_boundary_kernel (:602-780) at z=lz-1 */
static void zouhe_bc(pfo_sim *s) {
  const size_t N = s->N;
  const int nx = s->nx, ny = s->ny, top = s->nz - 1;
  const double C = lattice_C(s);
  double *f = s->fIN;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      size_t n = (size_t)i + (size_t)nx * j;
#define FI(d) f[(size_t)(d)*N + n]
      s->ux[n] = 0.0; s->uy[n] = 0.0; s->uz[n] = 0.0;
      double rho = 1.0 / (1.0 - s->uz[n] / C) *
                   (FI(1) + FI(2) + FI(3) + FI(4) + FI(7) + FI(8) + FI(11) + FI(12) + FI(0) +
                    2.0 * (FI(6) + FI(10) + FI(14) + FI(16) + FI(18)));
      s->rho[n] = rho;
      double ux = s->ux[n], uy = s->uy[n], uz = s->uz[n];
      double Nzx = 0.5 * (FI(1) + FI(7) + FI(8) - FI(2) - FI(11) - FI(12)) - 1.0 / 3.0 * rho * ux / C;
      double Nzy = 0.5 * (FI(3) + FI(7) + FI(11) - FI(4) - FI(8) - FI(12)) - 1.0 / 3.0 * rho * uy / C;
      FI(5) = FI(6) + 1.0 / 3.0 * rho * uz / C;
      FI(9) = FI(14) + 1.0 / 6.0 * rho * (uz + ux) / C - Nzx;
      FI(13) = FI(10) + 1.0 / 6.0 * rho * (uz - ux) / C + Nzx;
      FI(15) = FI(18) + 1.0 / 6.0 * rho * (uz + uy) / C - Nzy;
      FI(17) = FI(16) + 1.0 / 6.0 * rho * (uz - uy) / C + Nzy;
#undef FI
    }
  {
    float Cf = (float)C;
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t n = (size_t)i + (size_t)nx * (j + (size_t)ny * top);
#define FI(d) f[(size_t)(d)*N + n]
        s->ux[n] = 0.0; s->uy[n] = top_wall_uy(s); s->uz[n] = 0.0;
        double rho = 1.0 / (1.0 + s->uz[n] / Cf) *
                     (FI(1) + FI(2) + FI(3) + FI(4) + FI(7) + FI(11) + FI(12) + FI(8) + FI(0) +
                      2.0 * (FI(5) + FI(9) + FI(13) + FI(15) + FI(17)));
        s->rho[n] = rho;
        double ux = s->ux[n], uy = s->uy[n], uz = s->uz[n];
        float Nzx = (float)(0.5 * (FI(1) + FI(7) + FI(8) - FI(2) - FI(11) - FI(12)) - 1.0 / 3.0 * rho * ux / Cf);
        float Nzy = (float)(0.5 * (FI(3) + FI(7) + FI(11) - FI(4) - FI(8) - FI(12)) - 1.0 / 3.0 * rho * uy / Cf);
        FI(6) = FI(5) - 1.0 / 3.0 * rho * uz / Cf;
        FI(10) = FI(13) + 1.0 / 6.0 * rho * (-uz + ux) / Cf - Nzx;
        FI(14) = FI(9) + 1.0 / 6.0 * rho * (-uz - ux) / Cf + Nzx;
        FI(16) = FI(17) + 1.0 / 6.0 * rho * (-uz + uy) / Cf - Nzy;
        FI(18) = FI(15) + 1.0 / 6.0 * rho * (-uz - uy) / Cf + Nzy;
#undef FI
      }
  }
}

/* The velocity inlet (y=0) and outlet (y=ly-1) of
 * fluid3d_in_out_flow_boundary_kernel (LB_kernel.cu:78-392, commented out in
 * the reference; its launch slot is after the wall kernels and before the
 * moments, semLB.cu:412-418).  Interior nodes of the two planes only
 * (0 < i < lx-1, 0 < k < lz-1); the prescribed velocity is the shear
 * profile (0, uw k/(lz-1), 0).  Rows next to the plane's edges
 * (i = 1, lx-2; k = 1, lz-2) are reset to the equilibrium at INIT_RHO = 1
 * (:120-153); the others get Zou/He unknowns (:155-246 inlet, :289-389
 * outlet).  Corrected slips of the text: the inlet's f11 is built from f8
 * (the text reads f9), and the outlet computes its own Nyx, Nyz (the text
 * uses variables set only on the inlet branch).  The moments pass then
 * recomputes density and velocity there (these nodes are not obstacles). */
static void inout_bc(pfo_sim *s) {
  const size_t N = s->N;
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double C = lattice_C(s), uw = top_wall_uy(s);
  double *f = s->fIN;
  for (int k = 1; k < nz - 1; ++k)
    for (int side = 0; side < 2; ++side) {
      const int j = side ? ny - 1 : 0;
      for (int i = 1; i < nx - 1; ++i) {
        size_t n = (size_t)i + (size_t)nx * (j + (size_t)ny * k);
#define FI(d) f[(size_t)(d)*N + n]
        const double ux = 0.0, uy = uw * k / (nz - 1), uz = 0.0;
        if (i == 1 || i == nx - 2 || k == 1 || k == nz - 2) {
          for (int d = 0; d < 19; ++d) {
            double cu = 3.0 * (CX[d] * ux + CY[d] * uy + CZ[d] * uz);
            FI(d) = 1.0 * W19[d] * (1.0 + cu / C + 0.5 * cu * cu / (C * C) -
                                    1.5 * (ux * ux + uy * uy + uz * uz) / (C * C));
          }
          continue;
        }
        const double inplane = FI(1) + FI(2) + FI(5) + FI(6) + FI(9) + FI(10) + FI(13) + FI(14) + FI(0);
        if (side == 0) {
          double rho = 1.0 / (1.0 - uy / C) * (inplane + 2.0 * (FI(4) + FI(8) + FI(12) + FI(17) + FI(18)));
          double Nyx = 0.5 * (FI(1) + FI(9) + FI(10) - FI(2) - FI(13) - FI(14)) - 1.0 / 3.0 * rho * ux / C;
          double Nyz = 0.5 * (FI(5) + FI(9) + FI(13) - FI(6) - FI(10) - FI(14)) - 1.0 / 3.0 * rho * uz / C;
          FI(3) = FI(4) + 1.0 / 3.0 * rho * uy / C;
          FI(7) = FI(12) + 1.0 / 6.0 * rho * (uy + ux) / C - Nyx;
          FI(11) = FI(8) + 1.0 / 6.0 * rho * (uy - ux) / C + Nyx;
          FI(15) = FI(18) + 1.0 / 6.0 * rho * (uy + uz) / C - Nyz;
          FI(16) = FI(17) + 1.0 / 6.0 * rho * (uy - uz) / C + Nyz;
        } else {
          double rho = 1.0 / (1.0 + uy / C) * (inplane + 2.0 * (FI(3) + FI(7) + FI(11) + FI(15) + FI(16)));
          double Nyx = 0.5 * (FI(1) + FI(9) + FI(10) - FI(2) - FI(13) - FI(14)) - 1.0 / 3.0 * rho * ux / C;
          double Nyz = 0.5 * (FI(5) + FI(9) + FI(13) - FI(6) - FI(10) - FI(14)) - 1.0 / 3.0 * rho * uz / C;
          FI(4) = FI(3) - 1.0 / 3.0 * rho * uy / C;
          FI(12) = FI(7) + 1.0 / 6.0 * rho * (-uy - ux) / C + Nyx;
          FI(8) = FI(11) + 1.0 / 6.0 * rho * (-uy + ux) / C - Nyx;
          FI(18) = FI(15) + 1.0 / 6.0 * rho * (-uy - uz) / C + Nyz;
          FI(17) = FI(16) + 1.0 / 6.0 * rho * (-uy + uz) / C - Nyz;
        }
#undef FI
      }
    }
}

/* fluid3d_velocity_density_kernel (LB_kernel.cu:1108-1199); the Zou/He
 * planes are obstacle nodes there (gpuSEM_LB.c:1150-1156) and keep the
 * boundary values. */
static void moments(pfo_sim *s) {
  const size_t N = s->N, plane = (size_t)s->nx * s->ny;
  const double C = lattice_C(s), dtd = (double)s->dt;
  float fq = s->mp[PF_P_F0] / s->mp[PF_P_RHO0];
  fq = fq / s->mp[PF_P_UMAX];
  fq = fq * s->mp[PF_P_UNIT];
  const double F_over = (double)fq;
  const int zh = zouhe(s);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    size_t n = (size_t)nn;
    if (zh) {
      size_t k = n / plane;
      if (k == 0 || k == (size_t)s->nz - 1) continue;
    }
    double r = 0, a = 0, b = 0, c = 0;
    for (int d = 0; d < 19; ++d) {
      double f = s->fIN[d * N + n];
      r += f; a += CX[d] * f; b += CY[d] * f; c += CZ[d] * f;
    }
    s->rho[n] = r;
    s->ux[n] = (a * C + 0.5 * F_over * s->Fx[n] * dtd) / r;
    s->uy[n] = (b * C + 0.5 * F_over * s->Fy[n] * dtd) / r;
    s->uz[n] = (c * C + 0.5 * F_over * s->Fz[n] * dtd) / r;
  }
}

/* ---------------------------------------------------------------- step */
static void advance_positions(pfo_sim *s) {
  float dtT = s->dt / s->mp[PF_P_T0];
  double Lx = s->nx * (double)s->dx, Ly = s->ny * (double)s->dx;
  size_t PE = (size_t)s->P * s->E;
  for (size_t g = 0; g < PE; ++g) {
    s->X[g] += s->VX[g] * dtT;
    if (s->sc.ibm_wrap[0]) {
      if (s->X[g] > Lx) s->X[g] -= Lx;
      else if (s->X[g] < 0) s->X[g] += Lx;
    }
    s->Y[g] += s->VY[g] * dtT;
    if (s->sc.ibm_wrap[1]) {
      if (s->Y[g] > Ly) s->Y[g] -= Ly;
      else if (s->Y[g] < 0) s->Y[g] += Ly;
    }
    s->RY[g] += s->VY[g] * dtT;
    s->Z[g] += s->VZ[g] * dtT;
  }
  for (int m = 0; m < s->M && !penalty(s); ++m) {
    if (s->ffix[m]) continue;
    s->fX[m] += s->fVX[m] * dtT;
    if (s->sc.ibm_wrap[0]) {
      if (s->fX[m] > Lx) s->fX[m] -= Lx;
      else if (s->fX[m] < 0) s->fX[m] += Lx;
    }
    s->fY[m] += s->fVY[m] * dtT;
    if (s->sc.ibm_wrap[1]) {
      if (s->fY[m] > Ly) s->fY[m] -= Ly;
      else if (s->fY[m] < 0) s->fY[m] += Ly;
    }
    s->fZ[m] += s->fVZ[m] * dtT;
  }
}

int pfo_step(pfo_sim *s, int nsteps) {
  const size_t N = s->N, PE = (size_t)s->P * s->E;
  for (int it = 0; it < nsteps; ++it) {
    if (s->done) return 1;
    /* detach test (semLB.cu:451-455) with the injected uniform */
    if (s->sc.detach_rate > 0 && s->total_bond == 0 &&
        pfo_detach_uniform(s->sc.seed, s->step) < s->sc.detach_rate) {
      s->done = 1;
      return 1;
    }
    /* SEM force pass (semLB.cu:467-523) + Morse + fibrin springs */
    memset(s->FX, 0, PE * sizeof(double));
    memset(s->FY, 0, PE * sizeof(double));
    memset(s->FZ, 0, PE * sizeof(double));
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 1)
    for (int p = 0; p < s->P; ++p) membrane_forces(s, p);
    if (s->sc.morse && PE) morse_forces(s);
    if (s->M) fibrin_forces(s);
    /* fluid step (semLB.cu:326-431) */
    memset(s->Fx, 0, N * sizeof(double));
    memset(s->Fy, 0, N * sizeof(double));
    memset(s->Fz, 0, N * sizeof(double));
    memset(s->VX, 0, PE * sizeof(double));
    memset(s->VY, 0, PE * sizeof(double));
    memset(s->VZ, 0, PE * sizeof(double));
    if (s->nrec) receptor_bonds(s);
    else s->total_bond = 0;
    if (brute_ok(s)) {
      brute_pass(s, 1);
    } else {
      for (size_t g = 0; g < PE; ++g) spread_marker(s, s->X[g], s->Y[g], s->Z[g], s->FX[g], s->FY[g], s->FZ[g]);
    }
    if (penalty(s)) {
      fibrin_penalty_spread(s);
    } else {
      const double F0 = (double)s->mp[PF_P_F0];
      for (int m = 0; m < s->M; ++m)
        spread_marker(s, s->fX[m], s->fY[m], s->fZ[m], s->fFX[m] / F0, s->fFY[m] / F0, s->fFZ[m] / F0);
    }
    if (s->sc.body_force[0] != 0 || s->sc.body_force[1] != 0 || s->sc.body_force[2] != 0)
      for (size_t n = 0; n < N; ++n) {
        s->Fx[n] += s->sc.body_force[0]; s->Fy[n] += s->sc.body_force[1]; s->Fz[n] += s->sc.body_force[2];
      }
    collide(s);
    stream(s);
    if (zouhe(s)) zouhe_bc(s);
    if (s->sc.bc[1] == PF_BC_INOUT) inout_bc(s);
    moments(s);
    if (brute_ok(s)) {
      brute_pass(s, 0);
    } else {
#pragma omp parallel for num_threads(g_threads) schedule(static)
      for (long long g = 0; g < (long long)PE; ++g)
        interp_marker(s, s->X[g], s->Y[g], s->Z[g], &s->VX[g], &s->VY[g], &s->VZ[g]);
    }
    if (!penalty(s)) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int m = 0; m < s->M; ++m) interp_marker(s, s->fX[m], s->fY[m], s->fZ[m], &s->fVX[m], &s->fVY[m], &s->fVZ[m]);
    }
    advance_positions(s);
    if (penalty(s)) {
      fibrin_penalty(s);
      fibrin_integrate(s);
    }
    s->step++;
  }
  return s->done;
}

/* ---------------------------------------------------------------- getters */
void pfo_get_lattice(const pfo_sim *s, double *fIN, double *fOUT, double *rho, double *u, double *F) {
  size_t N = s->N;
  if (fIN) memcpy(fIN, s->fIN, 19 * N * sizeof(double));
  if (fOUT) memcpy(fOUT, s->fOUT, 19 * N * sizeof(double));
  if (rho) memcpy(rho, s->rho, N * sizeof(double));
  if (u) {
    memcpy(u, s->ux, N * sizeof(double));
    memcpy(u + N, s->uy, N * sizeof(double));
    memcpy(u + 2 * N, s->uz, N * sizeof(double));
  }
  if (F) {
    memcpy(F, s->Fx, N * sizeof(double));
    memcpy(F + N, s->Fy, N * sizeof(double));
    memcpy(F + 2 * N, s->Fz, N * sizeof(double));
  }
}
void pfo_get_elements(const pfo_sim *s, double *X, double *Y, double *RY, double *Z, double *V, double *F) {
  size_t PE = (size_t)s->P * s->E;
  if (X) memcpy(X, s->X, PE * sizeof(double));
  if (Y) memcpy(Y, s->Y, PE * sizeof(double));
  if (RY) memcpy(RY, s->RY, PE * sizeof(double));
  if (Z) memcpy(Z, s->Z, PE * sizeof(double));
  if (V) {
    memcpy(V, s->VX, PE * sizeof(double));
    memcpy(V + PE, s->VY, PE * sizeof(double));
    memcpy(V + 2 * PE, s->VZ, PE * sizeof(double));
  }
  if (F) {
    memcpy(F, s->FX, PE * sizeof(double));
    memcpy(F + PE, s->FY, PE * sizeof(double));
    memcpy(F + 2 * PE, s->FZ, PE * sizeof(double));
  }
}
void pfo_get_bonds(const pfo_sim *s, int *rec_state, int *vwf, int *total_bond) {
  if (rec_state) memcpy(rec_state, s->rec_state, (size_t)s->P * s->nrec * 3 * sizeof(int));
  if (vwf) memcpy(vwf, s->vwf, (size_t)4 * s->ny * s->nx * sizeof(int));
  if (total_bond) *total_bond = s->total_bond;
}
void pfo_get_fibrin(const pfo_sim *s, double *X, double *Y, double *Z, double *V, double *F) {
  size_t M = (size_t)s->M;
  if (X) memcpy(X, s->fX, M * sizeof(double));
  if (Y) memcpy(Y, s->fY, M * sizeof(double));
  if (Z) memcpy(Z, s->fZ, M * sizeof(double));
  if (V) {
    memcpy(V, s->fVX, M * sizeof(double));
    memcpy(V + M, s->fVY, M * sizeof(double));
    memcpy(V + 2 * M, s->fVZ, M * sizeof(double));
  }
  if (F) {
    memcpy(F, s->fFX, M * sizeof(double));
    memcpy(F + M, s->fFY, M * sizeof(double));
    memcpy(F + 2 * M, s->fFZ, M * sizeof(double));
  }
}
void pfo_get_membrane(const pfo_sim *s, double *S_V, double *km) {
  if (S_V) memcpy(S_V, s->SV, (size_t)s->P * 2 * sizeof(double));
  if (km)
    for (int p = 0; p < s->P; ++p)
      memcpy(km + (size_t)p * s->Em, s->km + (size_t)p * s->NN, (size_t)s->Em * sizeof(double));
}
void pfo_conservation(const pfo_sim *s, double out[4]) {
  double m = 0, a = 0, b = 0, c = 0;
  for (size_t n = 0; n < s->N; ++n)
    for (int d = 0; d < 19; ++d) {
      double f = s->fIN[d * s->N + n];
      m += f; a += CX[d] * f; b += CY[d] * f; c += CZ[d] * f;
    }
  out[0] = m; out[1] = a; out[2] = b; out[3] = c;
}
int pfo_get_cells(const pfo_sim *s, int *cell_of, int *order, int *ncells) {
  size_t PE = (size_t)s->P * s->E;
  if (cell_of) memcpy(cell_of, s->cell_of, PE * sizeof(int));
  if (order) memcpy(order, s->cell_order, PE * sizeof(int));
  if (ncells) { ncells[0] = s->ncell[0]; ncells[1] = s->ncell[1]; ncells[2] = s->ncell[2]; }
  return (int)PE;
}
long long pfo_step_count(const pfo_sim *s) { return s->step; }
