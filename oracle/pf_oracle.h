/*
 * pf_oracle.h -- CPU FP64 restatement of the reference's coupled step.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Tests and the smoke check compare the
 * CUDA path with it, the benchmark's CPU-baseline leg times it; the product
 * never links it.
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H

#include "pfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pfo_sim pfo_sim;

/* ibm_bruteforce: 1 = node-centric O(N*E) spreading/interpolation exactly as
 * LB_kernel.cu:1419-1642 iterates; 0 = element-centric 4x4x4 stencils (same
 * sums, different summation order). */
pfo_sim *pfo_create(const pf_scene *scene, int ibm_bruteforce);
void pfo_destroy(pfo_sim *s);
/* Runs nsteps coupled steps; returns 1 if the platelet detached, else 0. */
int pfo_step(pfo_sim *s, int nsteps);
/* Number of OpenMP threads the lattice loops use (1 = serial). */
void pfo_set_threads(int n);
int pfo_get_threads(void);

void pfo_get_lattice(const pfo_sim *s, double *fIN, double *fOUT, double *rho, double *u, double *F);
void pfo_get_elements(const pfo_sim *s, double *X, double *Y, double *RY, double *Z, double *V, double *F);
void pfo_get_bonds(const pfo_sim *s, int *rec_state, int *vwf, int *total_bond);
void pfo_get_fibrin(const pfo_sim *s, double *X, double *Y, double *Z, double *V, double *F);
void pfo_get_membrane(const pfo_sim *s, double *S_V, double *km);
void pfo_conservation(const pfo_sim *s, double out[4]);
/* Cell list of the last Morse pass: per element its cell id, and the
 * cell-sorted element order. */
int pfo_get_cells(const pfo_sim *s, int *cell_of, int *order, int *ncells);
long long pfo_step_count(const pfo_sim *s);

/* Philox-4x32-10 uniforms of the injected receptor/detach streams. */
void pfo_receptor_uniforms(uint64_t seed, int64_t step, int64_t receptor, double out[2]);
double pfo_detach_uniform(uint64_t seed, int64_t step);
/* the worm-like-chain link force law (fiber.cpp:710-733) */
double pfo_wlc_force(double l0, double l, double mass);
void pfo_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Single-operator entry points used by known-answer tests. */
double pfo_ibm_phi(double r);
void pfo_feq(double rho, const double u[3], double C, double out[19]);

#ifdef __cplusplus
}
#endif
#endif
