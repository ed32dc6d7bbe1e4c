/*
 * refemu.cpp -- runs the reference's own CUDA kernels (LB_kernel.cu,
 * sem_kernel.cu, included verbatim from the reference tree at build time)
 * on the CPU through cuda_emu.h, in the per-step launch order of
 * semLB.cu:303-531, to produce golden vectors for the oracle.
 *
 * ORACLE TEST INFRASTRUCTURE ONLY: built by oracle/refemu/build_refemu.sh into
 * oracle/_ref/ in the development container; never shipped or linked by the
 * product.  The host-side step loop below restates semLB.cu's
 * fluid_invokeGPUKernel (:303-438) and sem_invokeGPUKernel_Force (:441-531)
 * with three documented substitutions:
 *   1. randNum is overwritten every step from a caller-supplied array
 *      (the injected uniform stream) instead of the GSL refill of :348-365;
 *   2. the per-step detach test (:451-455) is not evaluated;
 *   3. atomicAdd into totalBond is deferred to the end of the launch, i.e. the
 *      schedule in which every receptor thread reads totalBond
 *      (sem_kernel.cu:1764) before any thread adds to it (:2069).
 * Device structs are the host structs themselves (no devImage copies).
 */
#include "cuda_emu.h"

dim3 threadIdx, blockIdx, blockDim, gridDim;
int *g_emu_deferred_addr = nullptr;
long long g_emu_deferred_sum = 0;

__constant__ float model_Parameters[100];

extern "C" {
#define X_a 64
#define Y_a 1
#include "GPUDefines.h"

/* Field names and types match the reference's fluid grid struct
 * (semLB.cu:53-75) because the included kernels access it by name. */
typedef struct _fluid_GPUgrids {
  float dt;
  float dx;
  int width;
  int height;
  int depth;
  size_t pitch;
  cudaExtent iextent;
  cudaExtent fextent;
  cudaExtent dextent;
  cudaPitchedPtr fIN[19];
  cudaPitchedPtr fOUT[19];
  cudaPitchedPtr ux;
  cudaPitchedPtr uy;
  cudaPitchedPtr uz;
  cudaPitchedPtr obst;
  cudaPitchedPtr rho;
  cudaPitchedPtr Fx;
  cudaPitchedPtr Fy;
  cudaPitchedPtr Fz;
  cudaPitchedPtr vWFbond;
  void *deviceStruct;
} fluid_GPUgrids;

#define printf(...) ((void)0)
#include "sem_kernel.cu"
#include "LB_kernel.cu"
#undef printf
}

/* ---------------------------------------------------------------- launch */
template <typename F>
static void launch(dim3 grid, dim3 block, F body) {
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = dim3(bx, by, bz);
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx) {
              threadIdx = dim3(tx, ty, tz);
              body();
            }
      }
}

/* ------------------------------------------------------------ allocation */
static size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
static const size_t kPitchAlign = 512; /* cudaMallocPitch-like row pitch */

static cudaPitchedPtr alloc3d(size_t row_bytes, size_t h, size_t d) {
  cudaPitchedPtr p;
  p.pitch = round_up(row_bytes, kPitchAlign);
  p.xsize = row_bytes;
  p.ysize = h;
  p.ptr = calloc(p.pitch * h * d + kPitchAlign, 1);
  return p;
}

extern "C" {

/* Everything the emulated run needs, in the reference's dense host layouts
 * (gpuSEM_LB.c:1101-1166 for the lattice, :749-779 and :1091-1100 for the
 * SEM arrays).  Outputs overwrite the in/out arrays at the end. */
typedef struct refemu_case {
  int lx, ly, lz;
  float dx, dt;
  float params[100];           /* hostSEMparameters[0..99] */
  double *fIN;                 /* [19][lz][ly][lx], in/out */
  double *fOUT;                /* [19][lz][ly][lx], out */
  double *ux, *uy, *uz, *rho;  /* [lz][ly][lx], in/out */
  float *obst;                 /* [lz][ly][lx], in */
  double *Fx, *Fy, *Fz;        /* [lz][ly][lx], in/out */
  int *vWF;                    /* [4][ly][lx], in/out */
  int maxE, surf, newnode, R;
  double *X, *Y, *RY, *Z;      /* [maxE] (maxCells = 1), in/out */
  double *VX, *VY, *VZ;        /* [maxE] out */
  double *FX, *FY, *FZ;        /* [maxE] out */
  double *bondLengths;         /* [maxE][maxE] */
  int *triElem;                /* [surf][6] */
  float *r1, *r2;              /* [surf][R] */
  int *node_nbrElemNum;        /* [newnode] */
  int *node_nbr_nodes;         /* [maxE][10] */
  double *Nref;                /* [newnode][3] */
  double *S0;                  /* [surf] */
  double S0_all, V0;
  int *receptBond;             /* [3][R][surf], in/out */
  int nsteps;
  const double *uniforms;      /* [nsteps][2][R][surf] */
  int *totalBond_per_step;     /* [nsteps], out */
  double *traj;                /* [nsteps][3][maxE] element X,Y,Z after each step, out (may be null) */
  double *km_out;              /* [newnode] out (may be null) */
  double *S_all_V_out;         /* [nsteps][2] out (may be null) */
  int first_lost_site_step;    /* out: first step after which a bonded receptor has site -1, or -1 */
  int fem_bend;                /* in: also launch the FEM bending chain the reference comments out */
} refemu_case;

int refemu_run(refemu_case *c) {
  const int lx = c->lx, ly = c->ly, lz = c->lz;
  const size_t N = (size_t)lx * ly * lz;
  c->first_lost_site_step = -1;

  /* model parameters: the constant array of sem_allocGPUKernel (semLB.cu:854) */
  std::memcpy(model_Parameters, c->params, sizeof model_Parameters);

  /* ---- fluid grids (fluid_allocGPUKernel, semLB.cu:111-150) */
  fluid_GPUgrids fg;
  std::memset(&fg, 0, sizeof fg);
  fg.dt = c->dt;
  fg.dx = c->dx;
  fg.width = lx;
  fg.height = ly;
  fg.depth = lz;
  for (int d = 0; d < 19; ++d) {
    fg.fIN[d] = alloc3d(lx * sizeof(double), ly, lz);
    fg.fOUT[d] = alloc3d(lx * sizeof(double), ly, lz);
  }
  fg.ux = alloc3d(lx * sizeof(double), ly, lz);
  fg.uy = alloc3d(lx * sizeof(double), ly, lz);
  fg.uz = alloc3d(lx * sizeof(double), ly, lz);
  fg.rho = alloc3d(lx * sizeof(double), ly, lz);
  fg.Fx = alloc3d(lx * sizeof(double), ly, lz);
  fg.Fy = alloc3d(lx * sizeof(double), ly, lz);
  fg.Fz = alloc3d(lx * sizeof(double), ly, lz);
  fg.obst = alloc3d(lx * sizeof(float), ly, lz);
  /* slot table with a zeroed guard region in front: the reference indexes
   * vWFbond[k][-1][-1] for a receptor whose stored site was erased
   * (sem_kernel.cu:1937-1942 then :1818-1820); such runs are flagged through
   * first_lost_site_step and not used as golden vectors */
  fg.vWFbond = alloc3d(lx * sizeof(int), ly, 4);
  void *vwf_block = fg.vWFbond.ptr;
  {
    size_t guard = 2 * fg.vWFbond.pitch + kPitchAlign;
    size_t bytes = fg.vWFbond.pitch * ly * 4 + kPitchAlign;
    char *blk = (char *)calloc(guard + bytes, 1);
    free(vwf_block);
    vwf_block = blk;
    fg.vWFbond.ptr = blk + guard;
  }
  fg.deviceStruct = &fg;

  auto put3 = [&](cudaPitchedPtr p, const void *src, size_t esz, int depth) {
    for (int k = 0; k < depth; ++k)
      for (int j = 0; j < ly; ++j)
        std::memcpy((char *)p.ptr + (k * (size_t)ly + j) * p.pitch,
                    (const char *)src + ((size_t)k * ly + j) * lx * esz, lx * esz);
  };
  auto get3 = [&](cudaPitchedPtr p, void *dst, size_t esz, int depth) {
    for (int k = 0; k < depth; ++k)
      for (int j = 0; j < ly; ++j)
        std::memcpy((char *)dst + ((size_t)k * ly + j) * lx * esz,
                    (const char *)p.ptr + (k * (size_t)ly + j) * p.pitch, lx * esz);
  };
  for (int d = 0; d < 19; ++d) put3(fg.fIN[d], c->fIN + d * N, sizeof(double), lz);
  put3(fg.ux, c->ux, sizeof(double), lz);
  put3(fg.uy, c->uy, sizeof(double), lz);
  put3(fg.uz, c->uz, sizeof(double), lz);
  put3(fg.rho, c->rho, sizeof(double), lz);
  put3(fg.Fx, c->Fx, sizeof(double), lz);
  put3(fg.Fy, c->Fy, sizeof(double), lz);
  put3(fg.Fz, c->Fz, sizeof(double), lz);
  put3(fg.obst, c->obst, sizeof(float), lz);
  put3(fg.vWFbond, c->vWF, sizeof(int), 4);

  /* ---- SEM grids (sem_allocGPUKernel / sem_initGPUKernel, semLB.cu:749-977) */
  const int maxE = c->maxE, surf = c->surf, newnode = c->newnode, R = c->R;
  sem_GPUgrids sg;
  std::memset(&sg, 0, sizeof sg);
  sg.maxCells = 1;
  sg.numOfCells = 1;
  sg.maxElements = maxE;
  sg.SurfElem = surf;
  sg.newnodeNum = newnode;
  sg.numReceptorsPerElem = R;
  sg.dt = c->dt;
  sg.S0_all = c->S0_all;
  sg.V0 = c->V0;
  sg.totalBond = 1;
  const size_t pitch = kPitchAlign;
  sg.pitch = pitch;
  sg.bondpitch = round_up(maxE * sizeof(double), kPitchAlign);
  int numOfElements = maxE;
  sg.numOfElements = &numOfElements;
  auto rows = [&](int n) { return (char *)calloc((size_t)n * pitch + pitch, 1); };
  sg.elementType = (int *)rows(maxE);
  sg.triElem = (int *)rows(surf);
  sg.receptor_r1 = (float *)rows(surf);
  sg.receptor_r2 = (float *)rows(surf);
  sg.X_Ref = (double *)rows(maxE);
  sg.X = (double *)rows(maxE);
  sg.V_X = (double *)rows(maxE);
  sg.F_X = (double *)rows(maxE);
  sg.Y_Ref = (double *)rows(maxE);
  sg.Y = (double *)rows(maxE);
  sg.RY = (double *)rows(maxE);
  sg.V_Y = (double *)rows(maxE);
  sg.F_Y = (double *)rows(maxE);
  sg.Z_Ref = (double *)rows(maxE);
  sg.Z = (double *)rows(maxE);
  sg.V_Z = (double *)rows(maxE);
  sg.F_Z = (double *)rows(maxE);
  sg.node_share_Elem = (int *)rows(newnode);
  sg.N = (double *)rows(newnode);
  sg.n = (double *)rows(newnode);
  sg.q = (double *)rows(newnode);
  sg.A = (double *)rows(newnode);
  sg.tau = (double *)rows(newnode);
  sg.Kapa = (double *)rows(newnode);
  sg.km = (double *)rows(newnode);
  sg.K = (double *)rows(newnode);
  sg.nelem = (double *)rows(surf);
  sg.Laplace_km = (double *)rows(maxE);
  sg.node_nbrNodes = (int *)rows(maxE);
  sg.node_nbrElemNum = (int *)calloc(newnode, sizeof(int));
  sg.S0 = (double *)calloc(surf, sizeof(double));
  sg.S = (double *)calloc(surf, sizeof(double));
  sg.bondLengths = (double *)calloc((size_t)maxE * sg.bondpitch + kPitchAlign, 1);
  sg.receptBond.pitch = round_up(surf * sizeof(int), kPitchAlign);
  sg.receptBond.ptr = calloc(sg.receptBond.pitch * R * 3 + kPitchAlign, 1);
  sg.randNum.pitch = round_up(surf * sizeof(double), kPitchAlign);
  sg.randNum.ptr = calloc(sg.randNum.pitch * R * 2 + kPitchAlign, 1);
  sg.devImage = &sg;

  auto rowd = [&](double *base, int r) { return (double *)((char *)base + (size_t)r * pitch); };
  auto rowi = [&](int *base, int r) { return (int *)((char *)base + (size_t)r * pitch); };
  for (int e = 0; e < maxE; ++e) {
    rowd(sg.X, e)[0] = c->X[e];
    rowd(sg.X_Ref, e)[0] = c->X[e];
    rowd(sg.Y, e)[0] = c->Y[e];
    rowd(sg.Y_Ref, e)[0] = c->Y[e];
    rowd(sg.RY, e)[0] = c->RY[e];
    rowd(sg.Z, e)[0] = c->Z[e];
    rowd(sg.Z_Ref, e)[0] = c->Z[e];
    for (int k = 0; k < 10; ++k) rowi(sg.node_nbrNodes, e)[k] = c->node_nbr_nodes[e * 10 + k];
    std::memcpy((char *)sg.bondLengths + (size_t)e * sg.bondpitch, c->bondLengths + (size_t)e * maxE,
                maxE * sizeof(double));
  }
  for (int t = 0; t < surf; ++t) {
    for (int k = 0; k < 6; ++k) rowi(sg.triElem, t)[k] = c->triElem[t * 6 + k];
    for (int r = 0; r < R; ++r) {
      ((float *)((char *)sg.receptor_r1 + (size_t)t * pitch))[r] = c->r1[t * R + r];
      ((float *)((char *)sg.receptor_r2 + (size_t)t * pitch))[r] = c->r2[t * R + r];
    }
    sg.S0[t] = c->S0[t];
  }
  for (int n = 0; n < newnode; ++n) {
    sg.node_nbrElemNum[n] = c->node_nbrElemNum[n];
    for (int k = 0; k < 3; ++k) rowd(sg.N, n)[k] = c->Nref[n * 3 + k];
  }
  for (int s = 0; s < 3; ++s)
    for (int r = 0; r < R; ++r)
      std::memcpy((char *)sg.receptBond.ptr + ((size_t)s * R + r) * sg.receptBond.pitch,
                  c->receptBond + ((size_t)s * R + r) * surf, surf * sizeof(int));

  /* ---- per-step loop: semLB.cu:441-531 then :303-438 */
  const int bankDepth = 16;
  const int zBanks = (lz + bankDepth - 1) / bankDepth;
  dim3 tpb3(32, 1, bankDepth);
  dim3 bpg3((lx + 31) / 32, ly, 1);
  const int bpgSEM = (maxE + 31) / 32;
  const int bpgFEM = (surf + 31) / 32;
  const int bpgNode = (newnode + 31) / 32;
  auto zero_rows = [&](double *base, int nrows, size_t bytes) {
    for (int r = 0; r < nrows; ++r) std::memset((char *)base + (size_t)r * pitch, 0, bytes);
  };
  for (int t = 0; t < c->nsteps; ++t) {
    /* sem_invokeGPUKernel_Force body */
    sg.S_all = 0;
    sg.V = 0;
    sg.totalBond = 0;
    std::memset(sg.S, 0, surf * sizeof(double));
    zero_rows(sg.F_X, maxE, sizeof(double));
    zero_rows(sg.F_Y, maxE, sizeof(double));
    zero_rows(sg.F_Z, maxE, sizeof(double));
    zero_rows(sg.n, newnode, 3 * sizeof(double));
    zero_rows(sg.nelem, surf, 3 * sizeof(double));
    zero_rows(sg.q, newnode, 3 * sizeof(double));
    zero_rows(sg.A, newnode, 9 * sizeof(double));
    zero_rows(sg.tau, newnode, 9 * sizeof(double));
    zero_rows(sg.Kapa, newnode, 9 * sizeof(double));
    zero_rows(sg.K, newnode, 27 * sizeof(double));
    zero_rows(sg.Laplace_km, maxE, sizeof(double));
    void *gs = sg.devImage;
    launch(dim3(bpgSEM), dim3(32), [&] { sem_Force_kernel(gs); });
    launch(dim3(bpgFEM), dim3(32), [&] { sem_calculate_A_kernel(gs); });
    launch(dim3(bpgNode), dim3(32), [&] { sem_surface_tension_kernel(gs); });
    launch(dim3(bpgFEM), dim3(32), [&] { sem_calculate_Kapa_kernel(gs); });
    launch(dim3(bpgNode), dim3(32), [&] { sem_calculate_m_kernel(gs); });
    if (c->fem_bend) {
      /* the three launches commented out at semLB.cu:518-520, in their slot */
      launch(dim3(bpgFEM), dim3(32), [&] { sem_calculate_K_kernel(gs); });
      launch(dim3(bpgNode), dim3(32), [&] { sem_calculate_q_kernel(gs); });
      launch(dim3(bpgFEM), dim3(32), [&] { sem_bending_force_kernel(gs); });
    }
    launch(dim3(bpgFEM), dim3(32), [&] { sem_ForceAreaVol_kernel(gs); });
    launch(dim3(bpgSEM), dim3(32), [&] { sem_Laplace_Kapa_kernel(gs); });
    if (c->S_all_V_out) {
      c->S_all_V_out[2 * t] = sg.S_all;
      c->S_all_V_out[2 * t + 1] = sg.V;
    }

    /* fluid_invokeGPUKernel body */
    for (int k = 0; k < lz; ++k)
      for (int j = 0; j < ly; ++j) {
        std::memset((char *)fg.Fx.ptr + ((size_t)k * ly + j) * fg.Fx.pitch, 0, lx * sizeof(double));
        std::memset((char *)fg.Fy.ptr + ((size_t)k * ly + j) * fg.Fy.pitch, 0, lx * sizeof(double));
        std::memset((char *)fg.Fz.ptr + ((size_t)k * ly + j) * fg.Fz.pitch, 0, lx * sizeof(double));
      }
    zero_rows(sg.V_X, maxE, sizeof(double));
    zero_rows(sg.V_Y, maxE, sizeof(double));
    zero_rows(sg.V_Z, maxE, sizeof(double));
    const double *u = c->uniforms + (size_t)t * 2 * R * surf;
    for (int s = 0; s < 2; ++s)
      for (int r = 0; r < R; ++r)
        std::memcpy((char *)sg.randNum.ptr + ((size_t)s * R + r) * sg.randNum.pitch,
                    u + ((size_t)s * R + r) * surf, surf * sizeof(double));
    void *gf = fg.deviceStruct;
    g_emu_deferred_addr = &sg.totalBond;
    g_emu_deferred_sum = 0;
    launch(dim3(surf), dim3(R), [&] { sem_platelet_wall_kernel(gf, gs); });
    g_emu_deferred_addr = nullptr;
    sg.totalBond += (int)g_emu_deferred_sum;
    for (int b = 0; b < zBanks; ++b)
      launch(bpg3, tpb3, [&] { fluid3d_force_distribute_kernel(gf, gs, b); });
    for (int b = 0; b < zBanks; ++b) launch(bpg3, tpb3, [&] { fluid3d_collision_kernel(gf, b); });
    for (int b = 0; b < zBanks; ++b) launch(bpg3, tpb3, [&] { fluid3d_stream_kernel(gf, b); });
    for (int b = 0; b < zBanks; ++b) launch(bpg3, tpb3, [&] { fluid3d_noslip_boundary_kernel(gf, b); });
    for (int b = 0; b < zBanks; ++b)
      launch(bpg3, tpb3, [&] { fluid3d_moving_plate_boundary_kernel(gf, b); });
    for (int b = 0; b < zBanks; ++b) launch(bpg3, tpb3, [&] { fluid3d_velocity_density_kernel(gf, b); });
    for (int b = 0; b < zBanks; ++b)
      launch(bpg3, tpb3, [&] { fluid3d_velocity_distribute_kernel(gf, gs, b); });
    launch(dim3(bpgSEM), dim3(32), [&] { sem_update_position_kernel(gf, gs); });
    c->totalBond_per_step[t] = sg.totalBond;
    if (c->first_lost_site_step < 0) {
      for (int r = 0; r < R && c->first_lost_site_step < 0; ++r)
        for (int tt = 0; tt < surf; ++tt) {
          int *b0 = (int *)((char *)sg.receptBond.ptr + (size_t)r * sg.receptBond.pitch);
          int *b2 = (int *)((char *)sg.receptBond.ptr + ((size_t)2 * R + r) * sg.receptBond.pitch);
          if (b2[tt] >= 1 && b0[tt] < 0) { c->first_lost_site_step = t; break; }
        }
    }
    if (c->traj) {
      for (int e = 0; e < maxE; ++e) {
        c->traj[((size_t)t * 3 + 0) * maxE + e] = rowd(sg.X, e)[0];
        c->traj[((size_t)t * 3 + 1) * maxE + e] = rowd(sg.Y, e)[0];
        c->traj[((size_t)t * 3 + 2) * maxE + e] = rowd(sg.Z, e)[0];
      }
    }
  }

  /* ---- outputs (fluid_initGPUKernel aFlag=0, sem_copyGPUKernel) */
  for (int d = 0; d < 19; ++d) {
    get3(fg.fIN[d], c->fIN + d * N, sizeof(double), lz);
    get3(fg.fOUT[d], c->fOUT + d * N, sizeof(double), lz);
  }
  get3(fg.ux, c->ux, sizeof(double), lz);
  get3(fg.uy, c->uy, sizeof(double), lz);
  get3(fg.uz, c->uz, sizeof(double), lz);
  get3(fg.rho, c->rho, sizeof(double), lz);
  get3(fg.Fx, c->Fx, sizeof(double), lz);
  get3(fg.Fy, c->Fy, sizeof(double), lz);
  get3(fg.Fz, c->Fz, sizeof(double), lz);
  get3(fg.vWFbond, c->vWF, sizeof(int), 4);
  for (int e = 0; e < maxE; ++e) {
    c->X[e] = rowd(sg.X, e)[0];
    c->Y[e] = rowd(sg.Y, e)[0];
    c->RY[e] = rowd(sg.RY, e)[0];
    c->Z[e] = rowd(sg.Z, e)[0];
    c->VX[e] = rowd(sg.V_X, e)[0];
    c->VY[e] = rowd(sg.V_Y, e)[0];
    c->VZ[e] = rowd(sg.V_Z, e)[0];
    c->FX[e] = rowd(sg.F_X, e)[0];
    c->FY[e] = rowd(sg.F_Y, e)[0];
    c->FZ[e] = rowd(sg.F_Z, e)[0];
  }
  if (c->km_out)
    for (int n = 0; n < newnode; ++n) c->km_out[n] = rowd(sg.km, n)[0];
  for (int s = 0; s < 3; ++s)
    for (int r = 0; r < R; ++r)
      std::memcpy(c->receptBond + ((size_t)s * R + r) * surf,
                  (char *)sg.receptBond.ptr + ((size_t)s * R + r) * sg.receptBond.pitch, surf * sizeof(int));

  /* release */
  for (int d = 0; d < 19; ++d) {
    free(fg.fIN[d].ptr);
    free(fg.fOUT[d].ptr);
  }
  free(fg.ux.ptr); free(fg.uy.ptr); free(fg.uz.ptr); free(fg.rho.ptr);
  free(fg.Fx.ptr); free(fg.Fy.ptr); free(fg.Fz.ptr); free(fg.obst.ptr); free(vwf_block);
  void *frees[] = {sg.elementType, sg.triElem, sg.receptor_r1, sg.receptor_r2, sg.X_Ref, sg.X, sg.V_X,
                   sg.F_X, sg.Y_Ref, sg.Y, sg.RY, sg.V_Y, sg.F_Y, sg.Z_Ref, sg.Z, sg.V_Z, sg.F_Z,
                   sg.node_share_Elem, sg.N, sg.n, sg.q, sg.A, sg.tau, sg.Kapa, sg.km, sg.K, sg.nelem,
                   sg.Laplace_km, sg.node_nbrNodes, sg.node_nbrElemNum, sg.S0, sg.S, sg.bondLengths,
                   sg.receptBond.ptr, sg.randNum.ptr};
  for (void *p : frees) free(p);
  return 0;
}

} /* extern "C" */
